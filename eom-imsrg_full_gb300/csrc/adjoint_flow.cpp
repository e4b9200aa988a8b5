// adjoint_flow.cpp -- entry points of the reverse-mode derivatives.
//
// imsrg_gpu_magnus_decouple_adjoint runs the Magnus flow of magnus_decouple
// (IMSRG_MAGNUS.f90:15-128, White generator) exactly as
// imsrg_gpu_magnus_decouple does, keeping every series term in device memory:
// per step k the Magnus terms A_1 = eta(HS_k-1), A_i = [Omega_k-1, A_i-1]
// of MAGNUS_EXPAND (:622-693) and the BCH terms B_n = [Omega_k, B_n-1],
// B_0 = H, of BCH_EXPAND (:149-234).  Then one backward sweep from E0(s):
//   BCH:     HS_k = sum_n B_n / n!   ->  Bbar_N = HSbar / N!,
//            Omegabar += d<Bbar_n, [Omega_k, B_n-1]>/dOmega,
//            Bbar_n-1 = HSbar / (n-1)! + d<Bbar_n, [Omega_k, B_n-1]>/dB_n-1,
//            Hbar += Bbar_0;
//   Euler:   Omega_k = Omega_k-1 + ds DG_k  ->  DGbar = ds Omegabar;
//   Magnus:  DG_k = sum_i c_i A_i  ->  the same recursion with coefficients
//            c_i and with_e0 = 0 (the Magnus terms carry no E0);
//   White:   eta_k-1 = N / D of HS_k-1  ->  HSbar_k-1 (Hbar at k = 1).
// The series keep the forward flow's term counts and stops (the reference's
// norm tests are discrete decisions, constant under differentiation).
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace {

using imsrg::cuda_status;

const double kCof[7] = {1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5};

int chk(const imsrg_op *op) { return (op && op->b && op->d) ? IMSRG_OK : IMSRG_ERR_INVALID; }

// Device copies of the flow's series terms, in chunks of kChunk operators
// (one allocation per chunk), freed with the recorder.
struct Store {
  static constexpr int kChunk = 64;
  std::vector<double *> chunks;
  int used = kChunk;  // operators taken from the last chunk
  long n = 0;         // doubles per operator (padded to 32 for alignment)
  ~Store() {
    for (double *p : chunks) cudaFree(p);
  }
  int keep(imsrg_basis *b, const double *src, long nf, double **out) {
    if (used == kChunk) {
      double *p = nullptr;
      IMSRG_CUDA_TRY(cudaMalloc((void **)&p, (size_t)kChunk * n * sizeof(double)));
      chunks.push_back(p);
      used = 0;
    }
    double *p = chunks.back() + (long)used++ * n;
    IMSRG_CUDA_TRY(cudaMemcpyAsync(p, src, nf * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    *out = p;
    return IMSRG_OK;
  }
};

struct StepRecord {
  double *omega_prev = nullptr, *hs_prev = nullptr, *omega = nullptr;
  std::vector<double *> A;     // A_1 (eta) .. A_m+1
  std::vector<double *> B;     // B_1 .. B_N
  std::vector<double> bcoef;   // 1/n! as the forward accumulated it
};

int read_dev(imsrg_basis *b, const double *d, double *out) {
  IMSRG_CUDA_TRY(cudaMemcpyAsync(b->h_scal, d, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  IMSRG_TRY(imsrg::ozaki_check_error(b));
  *out = b->h_scal[0];
  return IMSRG_OK;
}

int norm_dev(imsrg_basis *b, const double *d, double *out) {
  IMSRG_TRY(imsrg::launch_norm(b, d, b->scal));
  return read_dev(b, b->scal, out);
}

// x = a x + c y (in place)
int axpy(imsrg_basis *b, double *x, double a, const double *y, double c) {
  return imsrg::launch_axpby(b, x, a, y, c, x);
}

}  // namespace

extern "C" {

int imsrg_gpu_commutator_adjoint(const imsrg_op_t *X, const imsrg_op_t *Cbar, int herm_Y, int with_e0,
                                 imsrg_op_t *Ybar) {
  IMSRG_TRY(chk(X));
  IMSRG_TRY(chk(Cbar));
  IMSRG_TRY(chk(Ybar));
  if (X->b != Cbar->b || X->b != Ybar->b) return IMSRG_ERR_MISMATCH;
  if (herm_Y != 1 && herm_Y != -1) return IMSRG_ERR_INVALID;
  if (Ybar == X || Ybar == Cbar) return IMSRG_ERR_INVALID;
  Ybar->herm = herm_Y;
  return imsrg::commutator_adjoint_dev(X->b, X->d, X->herm, Cbar->d, herm_Y, with_e0 ? 1 : 0, Ybar->d);
}

int imsrg_gpu_white_adjoint(const imsrg_op_t *H, const imsrg_op_t *ETAbar, imsrg_op_t *Hbar) {
  IMSRG_TRY(chk(H));
  IMSRG_TRY(chk(ETAbar));
  IMSRG_TRY(chk(Hbar));
  if (H->b != ETAbar->b || H->b != Hbar->b) return IMSRG_ERR_MISMATCH;
  if (Hbar == H || Hbar == ETAbar) return IMSRG_ERR_INVALID;
  imsrg_basis *b = H->b;
  IMSRG_TRY(imsrg::adjoint_prepare(b));
  IMSRG_CUDA_TRY(cudaMemsetAsync(Hbar->d, 0, b->nfull * sizeof(double), b->stream));
  Hbar->herm = H->herm;
  return imsrg::launch_white_adjoint(b, H->d, H->herm, ETAbar->d, Hbar->d, imsrg::adjoint_monob(b));
}

int imsrg_gpu_op_dot(const imsrg_op_t *A, const imsrg_op_t *B, double *out) {
  IMSRG_TRY(chk(A));
  IMSRG_TRY(chk(B));
  if (A->b != B->b) return IMSRG_ERR_MISMATCH;
  if (!out) return IMSRG_ERR_INVALID;
  return imsrg::dot_dev(A->b, A->d, B->d, A->b->nfull, out);
}

int imsrg_gpu_magnus_decouple_adjoint(imsrg_op_t *HS, imsrg_op_t *G, imsrg_op_t *Hbar, double s_max, double ds,
                                      int max_steps, int precision, int ndir, const imsrg_op_t *const *dirs,
                                      double *grad, double *trace, int *steps_out, int *ncomm) {
  IMSRG_TRY(chk(HS));
  IMSRG_TRY(chk(G));
  imsrg_basis *b = HS->b;
  if (G->b != b) return IMSRG_ERR_MISMATCH;
  if (Hbar) {
    IMSRG_TRY(chk(Hbar));
    if (Hbar->b != b) return IMSRG_ERR_MISMATCH;
  }
  if (ndir < 0 || (ndir > 0 && (!dirs || !grad))) return IMSRG_ERR_INVALID;
  for (int j = 0; j < ndir; j++) {
    IMSRG_TRY(chk(dirs[j]));
    if (dirs[j]->b != b) return IMSRG_ERR_MISMATCH;
  }
  if (ds <= 0.0 || max_steps < 0) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  IMSRG_TRY(imsrg::adjoint_prepare(b));
  const long nf = b->nfull;
  const size_t nb = nf * sizeof(double);
  cudaStream_t st = b->stream;
  imsrg_op *H0, *DG, *X0, *X1;
  IMSRG_TRY(imsrg::flow_tmp_ops(b, &H0, &DG, &X0, &X1));
  imsrg_op *X[2] = {X0, X1};
  Store store;
  store.n = (nf + 31) / 32 * 32;
  std::vector<StepRecord> rec;

  // --- forward: magnus_decouple with the White generator, recorded ---------
  IMSRG_CUDA_TRY(cudaMemsetAsync(G->d, 0, nb, st));
  IMSRG_CUDA_TRY(cudaMemsetAsync(DG->d, 0, nb, st));
  G->herm = -1;
  DG->herm = -1;
  IMSRG_TRY(imsrg::launch_white(b, HS->d, HS->herm, DG->d));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(H0->d, HS->d, nb, cudaMemcpyDeviceToDevice, st));
  H0->herm = HS->herm;
  if (H0->herm != 1) return IMSRG_ERR_INVALID;  // the flow evolves a Hamiltonian
  double s = 0.0, e0 = 0.0, emp2 = 0.0;
  IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
  IMSRG_TRY(read_dev(b, HS->d, &e0));
  double crit = std::fabs(emp2);
  auto row = [&](int k) {
    if (!trace) return;
    double *t = trace + 5 * k;
    t[0] = k;
    t[1] = s;
    t[2] = e0;
    t[3] = e0 + emp2;
    t[4] = crit;
  };
  row(0);
  int steps = 0, nct = 0;
  const double conv = 1e-6;
  while (crit > 1e-6 && s < s_max - 1e-12 && steps < max_steps) {
    steps++;
    StepRecord r;
    IMSRG_TRY(store.keep(b, G->d, nf, &r.omega_prev));
    IMSRG_TRY(store.keep(b, HS->d, nf, &r.hs_prev));
    double *a1 = nullptr;
    IMSRG_TRY(store.keep(b, DG->d, nf, &a1));
    r.A.push_back(a1);
    // MAGNUS_EXPAND (the sequence of imsrg_gpu_magnus_expand)
    {
      double advals[8] = {0};
      IMSRG_CUDA_TRY(cudaMemcpyAsync(X[0]->d, DG->d, nb, cudaMemcpyDeviceToDevice, st));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(X[1]->d, DG->d, sizeof(double), cudaMemcpyDeviceToDevice, st));
      X[0]->herm = X[1]->herm = DG->herm;
      IMSRG_TRY(norm_dev(b, X[0]->d, &advals[1]));
      double fullnorm = 0.0;
      IMSRG_TRY(norm_dev(b, G->d, &fullnorm));
      if (!(fullnorm < 1e-9)) {
        int q = 1, cur = 0;
        for (int i = 2; i <= 7; i++) {
          const double adnorm = advals[i - q];
          q = (std::fabs(kCof[i - 1]) > 1e-6) ? 1 : 2;
          if (std::fabs(adnorm / fullnorm) < conv) break;
          imsrg_op *AD = X[cur], *INT2 = X[1 - cur];
          const int h = -G->herm * AD->herm;
          INT2->herm = h;
          IMSRG_TRY(imsrg::commutator_dev(b, G->d, G->herm, AD->d, AD->herm, INT2->d, h, precision, 0));
          nct++;
          IMSRG_TRY(imsrg::launch_axpby(b, DG->d, 1.0, INT2->d, kCof[i - 1], DG->d));
          double nrm = 0.0;
          IMSRG_TRY(norm_dev(b, INT2->d, &nrm));
          if (!std::isfinite(nrm)) return IMSRG_ERR_NONFINITE;
          advals[i] = nrm * std::fabs(kCof[i - 1]);
          double *ai = nullptr;
          IMSRG_TRY(store.keep(b, INT2->d, nf, &ai));
          r.A.push_back(ai);
          cur = 1 - cur;
        }
      }
    }
    // euler_step
    IMSRG_TRY(imsrg::launch_axpby(b, G->d, 1.0, DG->d, ds, G->d));
    s += ds;
    IMSRG_TRY(store.keep(b, G->d, nf, &r.omega));
    // BCH_EXPAND (the sequence of imsrg_gpu_bch_expand)
    {
      HS->herm = H0->herm;
      IMSRG_CUDA_TRY(cudaMemcpyAsync(HS->d, H0->d, nb, cudaMemcpyDeviceToDevice, st));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(X[0]->d, H0->d, nb, cudaMemcpyDeviceToDevice, st));
      X[0]->herm = H0->herm;
      double coef = 1.0;
      int cur = 0, iw;
      for (iw = 2; iw <= 40; iw++) {
        coef = coef / (iw - 1.0);
        imsrg_op *AD = X[cur], *INT2 = X[1 - cur];
        const int h = -G->herm * AD->herm;
        INT2->herm = h;
        IMSRG_TRY(imsrg::commutator_dev(b, G->d, G->herm, AD->d, AD->herm, INT2->d, h, precision, 1));
        nct++;
        IMSRG_TRY(imsrg::launch_axpby(b, HS->d, 1.0, INT2->d, coef, HS->d));
        double nrm = 0.0;
        IMSRG_TRY(norm_dev(b, INT2->d, &nrm));
        if (!std::isfinite(nrm)) return IMSRG_ERR_NONFINITE;
        double *bn = nullptr;
        IMSRG_TRY(store.keep(b, INT2->d, nf, &bn));
        r.B.push_back(bn);
        r.bcoef.push_back(coef);
        cur = 1 - cur;
        if (nrm * coef < conv) break;
      }
      if (iw > 40) {
        if (steps_out) *steps_out = steps;
        if (ncomm) *ncomm = nct;
        return IMSRG_ERR_NOT_CONVERGED;
      }
    }
    rec.push_back(std::move(r));
    IMSRG_TRY(imsrg::launch_white(b, HS->d, HS->herm, DG->d));
    IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
    IMSRG_TRY(read_dev(b, HS->d, &e0));
    if (!std::isfinite(e0) || !std::isfinite(emp2)) return IMSRG_ERR_NONFINITE;
    crit = std::fabs(emp2);
    row(steps);
  }
  if (steps_out) *steps_out = steps;
  if (ncomm) *ncomm = nct;

  // --- backward sweep from E0(s) -------------------------------------------
  imsrg_op *H0b, *HSb, *Ob, *DGb, *Sb, *T1;
  IMSRG_TRY(imsrg::work_op(b, 17, &H0b));
  IMSRG_TRY(imsrg::work_op(b, 18, &HSb));
  IMSRG_TRY(imsrg::work_op(b, 19, &Ob));
  IMSRG_TRY(imsrg::work_op(b, 20, &DGb));
  IMSRG_TRY(imsrg::work_op(b, 21, &Sb));
  IMSRG_TRY(imsrg::work_op(b, 22, &T1));
  double *monob = imsrg::adjoint_monob(b);
  const double one = 1.0;
  IMSRG_CUDA_TRY(cudaMemsetAsync(H0b->d, 0, nb, st));
  IMSRG_CUDA_TRY(cudaMemsetAsync(HSb->d, 0, nb, st));
  IMSRG_CUDA_TRY(cudaMemsetAsync(Ob->d, 0, nb, st));
  // the derivative of E0(s) = HS(s)[0]
  IMSRG_CUDA_TRY(cudaMemcpyAsync(HSb->d, &one, sizeof(double), cudaMemcpyHostToDevice, st));
  if (rec.empty()) IMSRG_CUDA_TRY(cudaMemcpyAsync(H0b->d, HSb->d, nb, cudaMemcpyDeviceToDevice, st));
  for (int k = (int)rec.size() - 1; k >= 0; k--) {
    const StepRecord &r = rec[k];
    // BCH_EXPAND backwards (B_n herm +1, Omega herm -1, with E0)
    const int N = (int)r.B.size();
    IMSRG_TRY(imsrg::launch_axpby(b, HSb->d, r.bcoef[N - 1], HSb->d, 0.0, Sb->d));
    for (int n = N; n >= 1; n--) {
      const double *Bprev = n >= 2 ? r.B[n - 2] : H0->d;
      IMSRG_TRY(imsrg::commutator_adjoint_dev(b, Bprev, 1, Sb->d, -1, 1, T1->d));
      IMSRG_TRY(axpy(b, Ob->d, 1.0, T1->d, -1.0));
      IMSRG_TRY(imsrg::commutator_adjoint_dev(b, r.omega, -1, Sb->d, 1, 1, T1->d));
      IMSRG_TRY(imsrg::launch_axpby(b, T1->d, 1.0, HSb->d, n >= 2 ? r.bcoef[n - 2] : 1.0, Sb->d));
    }
    IMSRG_TRY(axpy(b, H0b->d, 1.0, Sb->d, 1.0));
    // euler_step backwards
    IMSRG_TRY(imsrg::launch_axpby(b, Ob->d, ds, Ob->d, 0.0, DGb->d));
    // MAGNUS_EXPAND backwards (all herm -1, no E0)
    const int M = (int)r.A.size();  // A_1 .. A_M
    IMSRG_TRY(imsrg::launch_axpby(b, DGb->d, kCof[M - 1], DGb->d, 0.0, Sb->d));
    for (int i = M; i >= 2; i--) {
      IMSRG_TRY(imsrg::commutator_adjoint_dev(b, r.A[i - 2], -1, Sb->d, -1, 0, T1->d));
      IMSRG_TRY(axpy(b, Ob->d, 1.0, T1->d, -1.0));
      IMSRG_TRY(imsrg::commutator_adjoint_dev(b, r.omega_prev, -1, Sb->d, -1, 0, T1->d));
      IMSRG_TRY(imsrg::launch_axpby(b, T1->d, 1.0, DGb->d, kCof[i - 2], Sb->d));
    }
    // the White generator of HS_k-1 (H itself at the first step)
    if (k == 0) {
      IMSRG_TRY(imsrg::launch_white_adjoint(b, H0->d, 1, Sb->d, H0b->d, monob));
    } else {
      IMSRG_CUDA_TRY(cudaMemsetAsync(HSb->d, 0, nb, st));
      IMSRG_TRY(imsrg::launch_white_adjoint(b, r.hs_prev, 1, Sb->d, HSb->d, monob));
    }
  }
  for (int j = 0; j < ndir; j++) IMSRG_TRY(imsrg::dot_dev(b, H0b->d, dirs[j]->d, nf, &grad[j]));
  if (Hbar) {
    IMSRG_CUDA_TRY(cudaMemcpyAsync(Hbar->d, H0b->d, nb, cudaMemcpyDeviceToDevice, st));
    Hbar->herm = 1;
  }
  IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
  return IMSRG_OK;
}

}  // extern "C"
