// adjoint.cu -- reverse-mode derivatives: the adjoint of the commutator and of
// the Magnus flow.
//
// The commutator RES = [X, Y] (the sequence of IMSRG_MAGNUS.f90:207-219,
// commutators.f90:10-925) is bilinear.  For a fixed X its adjoint with
// respect to Y is the transposed linear map
//     Ybar = d<Cbar, [X, Y]> / dY,
// built here by transposing every piece of the forward kernels
// (kernels_comm.cu) on the same host-built gather lists, one kernel per
// piece, in the reverse order of the forward data flow:
//   1. two-body assembly^T: the ladder epilogue of 222_pp_hh hands Cbar to
//      W1bar / W2bar, the 222_ph recoupling to Zbar, the commutator_122
//      insertions to Ybar (two- and one-body), the 220 energy to Ybar's pphh;
//   2. one-body assembly^T: commutator_111 / 121 to Ybar, 221 to W1bar/W2bar;
//   3. 110^T: the energy's particle-hole sum to Ybar's fph;
//   4. recoupling inputs^T: Zbar to WCCbar;
//   5. every dense product transposed as one grouped FP64 launch: the twelve
//      ladder products of each block into Ybar's two-body arrays, and
//      RCCbar = WCCbar^T LCC per cross-coupled block;
//   6. Pandya transform^T (calculate_cross_coupled, cross_coupled.f90:
//      1190-1300): RCCbar back to Ybar.
// The adjoint with respect to X follows from antisymmetry, [X, Y] = -[Y, X]:
//     d<Cbar, [X, Y]> / dX = -(the adjoint above with the roles swapped).
// The gather lists become scatters, added with FP64 atomics: the adjoint's
// results agree run to run to rounding, not bit for bit (the forward
// commutator stays atomic-free and bit-reproducible).
//
// The flow's adjoint (imsrg_gpu_magnus_decouple_adjoint) records one Magnus
// flow (the host-driven sequence of magnus_decouple, IMSRG_MAGNUS.f90:15-128,
// with MAGNUS_EXPAND :622-693, euler_step :756-766, BCH_EXPAND :149-234 and
// build_gs_white, generators.f90:4-106) with every series term kept in device
// memory, then sweeps back from E0(s) through each step: BCH terms, the Euler
// step, the Magnus terms and the White generator.  One backward sweep gives
// the gradient of E0(s) with respect to every element of the input
// Hamiltonian, so dE0/dc_k for H(c) = T + sum_k c_k V_k is one dot product
// per parameter.  The reference has no derivative code; its checks are
// central finite differences of the flow.
#include <cmath>
#include <cstring>
#include <vector>

#include "device.cuh"

namespace imsrg {

namespace {

// ---------------------------------------------------------------------------
// Grouped FP64 products of the adjoint: C += sum_t alpha_t op(A_t) op(B_t),
// each term with its own contraction length (the transposed ladder products
// of one output array read different intermediates).  64 x 64 tiles laid out
// as the forward's k_gemm_fp64: warp w owns columns 8w .. 8w + 7 and skips
// its products when they lie past N; a short last K chunk runs only its k.
// ---------------------------------------------------------------------------
struct AdjTerm {
  int a_src, b_src, ta, tb;
  long a_off, b_off;
  int lda, ldb, K;
  double coef;
  int use_hl, use_hr;
};

constexpr int kAdjTerms = 6;
struct AdjProb {
  int M, N, nterms, c_dst;
  long c_off;
  int ldc, tile0, tiles_m, tiles;
  AdjTerm t[kAdjTerms];
};

// operands: X (the fixed operator), W1bar, W2bar, WCCbar, LCC; outputs: Ybar, RCCbar
enum { AS_X = 0, AS_W1 = 1, AS_W2 = 2, AS_WCC = 3, AS_LCC = 4, AD_Y = 0, AD_RCC = 1 };
struct AdjOps {
  const double *src[5];
  double *dst[2];
};

constexpr int BM = 64, BN = 64, BK = 16;

__global__ void __launch_bounds__(256) k_gemm_adj(const AdjProb *__restrict__ probs, int nprobs, AdjOps ops, int hL,
                                                  int hR) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tile = blockIdx.x;
  int lo = 0, hi = nprobs;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (probs[mid].tile0 <= tile) lo = mid + 1;
    else hi = mid;
  }
  const AdjProb &P = probs[lo - 1];
  const int lt = tile - P.tile0;
  const int m0 = (lt % P.tiles_m) * BM, n0 = (lt / P.tiles_m) * BN;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const bool live = n0 + 8 * (tid >> 5) < P.N;  // warp-uniform: the warp's eight columns 4 ty + j
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  for (int it = 0; it < P.nterms; it++) {
    const AdjTerm &Tm = P.t[it];
    const double *A = ops.src[Tm.a_src] + Tm.a_off;
    const double *B = ops.src[Tm.b_src] + Tm.b_off;
    const double alpha = Tm.coef * (Tm.use_hl ? hL : 1) * (Tm.use_hr ? hR : 1);
    double part[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) part[i][j] = 0.0;
    for (int k0 = 0; k0 < Tm.K; k0 += BK) {
#pragma unroll
      for (int l = 0; l < 4; l++) {
        int m, k;
        if (!Tm.ta) { m = tid & 63; k = (tid >> 6) + 4 * l; }
        else { k = tid & 15; m = (tid >> 4) + 16 * l; }
        const int gm = m0 + m, gk = k0 + k;
        double v = 0.0;
        if (gm < P.M && gk < Tm.K) v = Tm.ta ? A[gk + (long)gm * Tm.lda] : A[gm + (long)gk * Tm.lda];
        As[k][m] = v;
      }
#pragma unroll
      for (int l = 0; l < 4; l++) {
        int n, k;
        if (!Tm.tb) { k = tid & 15; n = (tid >> 4) + 16 * l; }
        else { n = tid & 63; k = (tid >> 6) + 4 * l; }
        const int gn = n0 + n, gk = k0 + k;
        double v = 0.0;
        if (gn < P.N && gk < Tm.K) v = Tm.tb ? B[gn + (long)gk * Tm.ldb] : B[gk + (long)gn * Tm.ldb];
        Bs[k][n] = v;
      }
      __syncthreads();
      const int kn = live ? min(BK, Tm.K - k0) : 0;
#pragma unroll
      for (int k = 0; k < BK; k++) {
        if (k < kn) {
          double a[4], bv[4];
#pragma unroll
          for (int i = 0; i < 4; i++) a[i] = As[k][tx + 16 * i];
#pragma unroll
          for (int j = 0; j < 4; j++) bv[j] = Bs[k][4 * ty + j];
#pragma unroll
          for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) part[i][j] = fma(a[i], bv[j], part[i][j]);
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] += alpha * part[i][j];
  }
  double *Cp = ops.dst[P.c_dst] + P.c_off;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int gn = n0 + 4 * ty + j;
    if (gn >= P.N) continue;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int gm = m0 + tx + 16 * i;
      if (gm < P.M) Cp[gm + (long)gn * P.ldc] += acc[i][j];
    }
  }
}

// ---------------------------------------------------------------------------
// 1. Two-body assembly^T, one thread per element head (k_assemble_2body's
//    sequence read backwards).  Forward, per head:
//      t0 = s122 * nd;  t1 = diag ? -t0 (herm(RES) < 0) : t0;
//      t2 = t1 + W1[e] - W2[e] - [square] (+-)(W1[em] - W2[em]) + sm;
//      RES[e] = diag ? +-t2 : t2;  RES[em] = herm(RES) t2 (square, off-diagonal)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_adj_asm2(DevTables T, const double *__restrict__ X, int hL, int hR,
                                                  const double *__restrict__ Cb, int hRES, int with220,
                                                  double *Yb, double *W1b, double *W2b, double *Zb) {
  const long w = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= T.n_asm2) return;
  const Asm2Head h = T.asm2_head[w];
  const unsigned meta = h.meta;
  const int nL = hL < 0, nR = hR < 0, nres = hRES < 0, npm = (hL * hR) < 0;
  const bool diag = (meta >> 20) & 1, square = (meta >> 21) & 1;
  const long e = h.e, em = h.em;
  double tb = diag ? dflip(Cb[e], nres) : Cb[e];
  if (square && !diag) tb += dflip(Cb[em], nres);
  // ladder epilogue of 222_pp_hh (each W index belongs to one head)
  if (square) {
    const double m = dflip(tb, npm);
    if (diag) {
      W1b[e] += tb - m;
      W2b[e] += m - tb;
    } else {
      W1b[e] += tb;
      W2b[e] -= tb;
      W1b[em] -= m;
      W2b[em] += m;
    }
  } else {
    W1b[e] += tb;
    W2b[e] -= tb;
  }
  const int nd = (meta >> 18) & 3;
  // 222_ph recoupling: sm = c (+-sum_J' {6j} Z_in + sum_J' {6j} Z_out)
  if ((meta >> 15) & 1) {
    const int n_in = (meta >> 5) & 31, n_out = (meta >> 10) & 31;
    const double c = nd ? (nd == 1 ? .70710678118 : .70710678118 * .70710678118) : 1.0;
    const double s2 = tb * c, s1 = dflip(s2, (meta >> 16) & 1);
    const double *six1 = T.six + h.six1, *six2 = T.six + h.six2;
    double *z = Zb + h.zs;
    for (int k = 0; k < n_in; k++) atomicAdd(z + k, s1 * six1[k]);
    for (int k = 0; k < n_out; k++) atomicAdd(z + n_in + k, s2 * six2[k]);
  }
  // commutator_122: s122 = sum fL vR + fR vL over the element's terms, where
  // (L, R) = (X, Y) and only the Y factors vary
  double u = diag ? dflip(tb, nres) : tb;
  if (nd) u = u * (nd == 1 ? 0.7071067811865476 : 0.5);
  const unsigned long long *tm = T.asm2_terms + h.start;
  const int n122 = meta & 31;
  for (int k = 0; k < n122; k++) {
    const unsigned long long v = tm[k];
    const long vi = (long)(v & 0xFFFFFFFull), fi = (long)((v >> 28) & 0xFFFFFull);
    const int sg = (int)(v >> 48) & 1, nsq = (int)(v >> 49) & 3, tr = (int)(v >> 51) & 1, ftr = (int)(v >> 52) & 1;
    const double c = nsq ? (nsq == 1 ? IMSRG_SQRT2 : 2.0000000000000004) : 1.0;
    const double fL = dflip(X[fi], (ftr & nL) ^ sg);
    const double vL = dflip(X[vi], tr & nL) * c;
    atomicAdd(Yb + vi, dflip(u * fL * c, tr & nR));
    atomicAdd(Yb + fi, dflip(u * vL, (ftr & nR) ^ sg ^ 1));
  }
  // commutator_220 (E0 = ... - 2 herm_R sum (2J+1) L_pphh R_pphh)
  if (with220 && ((meta >> 22) & 1)) atomicAdd(Yb + e, -2.0 * hR * (h.J2 + 1.0) * Cb[0] * X[e]);
}

// ---------------------------------------------------------------------------
// 2. One-body assembly^T over k_assemble_1body's work split (an allowed
//    upper-triangle element per CTA, every other element per warp).  Forward:
//      x = c0 v0 + c1 v1 + c2 v2 + c3 v3 + [allowed] (rj v4 + c5 v5)
//    with v0..v3 the commutator_111 dot products, v4 the 121 sums, v5 the 221
//    sums; RES[p, q] = x and, for allowed square elements, RES[q, p] = herm x.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_adj_1body(DevTables T, const double *X, int hL, int hR,
                                                   const double *__restrict__ Cb, int hRES, double *Yb,
                                                   double *W1b, double *W2b) {
  const int A = T.A, P = T.P;
  const double *Lhh = X + T.off_fhh, *Lph = X + T.off_fph, *Lpp = X + T.off_fpp;
  double *Rhh = Yb + T.off_fhh, *Rph = Yb + T.off_fph, *Rpp = Yb + T.off_fpp;
  const int nheavy = T.n_asm1_heavy;
  const bool whole = (int)blockIdx.x < nheavy;
  long e;
  int tid, nt;
  if (whole) {
    e = T.asm1_heavy[blockIdx.x];
    tid = threadIdx.x;
    nt = blockDim.x;
  } else {
    const int li = ((int)blockIdx.x - nheavy) * 4 + (int)(threadIdx.x >> 5);
    if (li >= T.n_asm1_light) return;
    e = T.asm1_light[li];
    tid = threadIdx.x & 31;
    nt = 32;
  }
  const long nA2 = (long)A * A, nPA = (long)P * A;
  int type, p, q, pk, qk;
  if (e < nA2) {
    type = 0;
    p = (int)(e % A);
    q = (int)(e / A);
    pk = T.hole_orb[p];
    qk = T.hole_orb[q];
  } else if (e < nA2 + nPA) {
    type = 1;
    p = (int)((e - nA2) % P);
    q = (int)((e - nA2) / P);
    pk = T.part_orb[p];
    qk = T.hole_orb[q];
  } else {
    type = 2;
    p = (int)((e - nA2 - nPA) % P);
    q = (int)((e - nA2 - nPA) / P);
    pk = T.part_orb[p];
    qk = T.part_orb[q];
  }
  const bool allowed = T.orb[pk].x == T.orb[qk].x && T.orb[pk].y == T.orb[qk].y && T.orb[pk].z == T.orb[qk].z;
  const long base = type == 0 ? T.off_fhh : type == 1 ? T.off_fph : T.off_fpp;
  const int ld = type == 0 ? A : P;
  double xb = Cb[base + p + (long)q * ld];
  if (allowed && type != 1 && p != q) xb += hRES * Cb[base + q + (long)p * ld];
  if (xb == 0.0) return;
  double c0 = 1.0, c1 = 1.0, c2 = -1.0, c3 = -1.0;
  if (type == 0) {
    c1 = hL;
    c2 = -(double)(hL * hR);
    c3 = -hR;
  } else if (type == 2) {
    c0 = hR;
    c2 = -hL;
    c3 = -(double)(hR * hL);
  }
  const double b0 = c0 * xb, b1 = c1 * xb, b2 = c2 * xb, b3 = c3 * xb;
  // commutator_111 (commutators.f90:36-80), the Y factor of each product
  if (type == 0) {
    for (int k = tid; k < A; k += nt) {
      atomicAdd(Rhh + k + (long)q * A, b0 * Lhh[p + (long)k * A]);
      atomicAdd(Rhh + k + (long)p * A, b2 * Lhh[q + (long)k * A]);
    }
    for (int k = tid; k < P; k += nt) {
      atomicAdd(Rph + k + (long)q * P, b1 * Lph[k + (long)p * P]);
      atomicAdd(Rph + k + (long)p * P, b3 * Lph[k + (long)q * P]);
    }
  } else if (type == 1) {
    for (int k = tid; k < A; k += nt) {
      atomicAdd(Rhh + k + (long)q * A, b0 * Lph[p + (long)k * P]);
      atomicAdd(Rph + p + (long)k * P, b2 * Lhh[k + (long)q * A]);
    }
    for (int k = tid; k < P; k += nt) {
      atomicAdd(Rph + k + (long)q * P, b1 * Lpp[p + (long)k * P]);
      atomicAdd(Rpp + p + (long)k * P, b3 * Lph[k + (long)q * P]);
    }
  } else {
    for (int k = tid; k < A; k += nt) {
      atomicAdd(Rph + q + (long)k * P, b0 * Lph[p + (long)k * P]);
      atomicAdd(Rph + p + (long)k * P, b2 * Lph[q + (long)k * P]);
    }
    for (int k = tid; k < P; k += nt) {
      atomicAdd(Rpp + k + (long)q * P, b1 * Lpp[p + (long)k * P]);
      atomicAdd(Rpp + k + (long)p * P, b3 * Lpp[q + (long)k * P]);
    }
  }
  if (!allowed) return;
  // commutator_121 (:83-280) and 221 (:435-578) terms
  const double rj = 1.0 / (T.orb[pk].x + 1.0);
  const double u4 = rj * xb, u5 = ((type != 1 && p == q) ? hRES * rj : rj) * xb;
  const int st = T.obt_start[e], n = T.obt_count[e];
  const int nL = hL < 0, nR = hR < 0, npm = hL * hR > 0;
  for (int k = tid; k < n; k += nt) {
    const OneBodyTerm t = T.obt[st + k];
    const int kind = t.meta & 3;
    if (kind < 2) {
      const int tr = (t.meta >> 2) & 1, ph = t.meta >> 8;
      const double lv = dflip(X[t.idx], tr & nL) * t.coef;
      const double lph = Lph[ph];
      if (kind == 0) {  // L_ai (herm_L R) - R_ai (herm_R L) at <a p|i q>
        atomicAdd(Yb + t.idx, dflip(u4 * dflip(lph, nL) * t.coef, tr & nR));
        atomicAdd(Rph + ph, -dflip(u4 * lv, nR));
      } else {  // -L_ai R + R_ai L at <i p|a q>
        atomicAdd(Yb + t.idx, -dflip(u4 * lph * t.coef, tr & nR));
        atomicAdd(Rph + ph, u4 * lv);
      }
    } else {
      double *Wb = (t.meta & 8) ? W2b : W1b;
      const double w = u5 * t.coef;
      atomicAdd(Wb + t.idx, kind == 3 ? dflip(w, npm) : w);
    }
  }
}

// 3. commutator_110^T: E0 += sum_ai (2j_i+1) (L_ai R_ai herm_L - R_ai L_ai herm_R)
__global__ void k_adj_e0(DevTables T, const double *__restrict__ X, int hL, int hR, const double *__restrict__ Cb,
                         double *Yb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= T.P * T.A) return;
  const int ji = T.orb[T.hole_orb[k / T.P]].x;
  atomicAdd(Yb + T.off_fph + k, Cb[0] * (double)(hL - hR) * (ji + 1) * X[T.off_fph + k]);
}

// 4. Recoupling inputs^T: Z = herm_L (W(x1,y1) + e W(x2,y2)) - herm_R (e W(y2,x2) + W(y1,x1))
__global__ void __launch_bounds__(256) k_adj_ph(DevTables T, const double *__restrict__ Zb, int hL, int hR,
                                                double *WCCb) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.n_ph) return;
  const double z = Zb[t];
  if (z == 0.0) return;
  const PhTerm p = T.ph_terms[t];
  const unsigned long long u = p.rows;
  const unsigned x1 = (unsigned)(u & 0xFFFF), y1 = (unsigned)((u >> 16) & 0xFFFF);
  const unsigned x2 = (unsigned)((u >> 32) & 0xFFFF), y2 = (unsigned)(u >> 48);
  const int rl = T.cc_rlen[p.qx];
  double *W = WCCb + T.wcc_off[p.qx];
  const double a = dflip(z, hL < 0), c = -dflip(z, hR < 0);
  if (x1 != 0xFFFFu && y1 != 0xFFFFu) {
    atomicAdd(W + x1 + (long)y1 * rl, a);
    atomicAdd(W + y1 + (long)x1 * rl, c);
  }
  if (x2 != 0xFFFFu && y2 != 0xFFFFu) {
    atomicAdd(W + x2 + (long)y2 * rl, dflip(a, p.nph));
    atomicAdd(W + y2 + (long)x2 * rl, dflip(c, p.nph));
  }
}

// 6. Pandya transform^T: RCC[e] = sum_k coef_k (herm_R if transposed) R[idx_k]
__global__ void __launch_bounds__(256) k_adj_cc(DevTables T, const double *__restrict__ RCCb, int hR, double *Yb) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= T.cc_total) return;
  const double r = RCCb[e];
  if (r == 0.0) return;
  const int nR = hR < 0;
  for (int k = T.cct_start[e]; k < T.cct_start[e + 1]; k++) {
    const int ix = T.cct_idx[k];
    const int tr = (int)((unsigned)ix >> 31), idx = ix & 0x7fffffff;
    atomicAdd(Yb + idx, T.cct_coef[k] * dflip(r, tr & nR));
  }
}

// Fixed-order dot product: per-CTA partials, then one CTA sums them in order.
constexpr int DOT_CTAS = 256, DOT_THREADS = 256;
__global__ void __launch_bounds__(DOT_THREADS) k_dot_partial(const double *__restrict__ x,
                                                             const double *__restrict__ y, long n, double *part) {
  __shared__ double sh[DOT_THREADS / 32];
  double s = 0.0;
  for (long i = (long)blockIdx.x * DOT_THREADS + threadIdx.x; i < n; i += (long)DOT_CTAS * DOT_THREADS)
    s = fma(x[i], y[i], s);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < DOT_THREADS / 32; k++) t += sh[k];
    part[blockIdx.x] = t;
  }
}

__global__ void k_dot_final(const double *__restrict__ part, double *out) {
  double t = 0.0;
  for (int k = 0; k < DOT_CTAS; k++) t += part[k];
  *out = t;
}

}  // namespace

// Per-basis state of the adjoint (allocated on first use).
struct AdjState {
  double *w1b = nullptr, *w2b = nullptr, *rccb = nullptr, *wccb = nullptr, *zb = nullptr;
  double *monob = nullptr, *part = nullptr, *dot = nullptr, *h_dot = nullptr;
  AdjProb *d_probs = nullptr;
  int nprobs = 0, ntiles = 0;
};

namespace {

AdjState *adj_of(imsrg_basis *b) { return (AdjState *)b->adjoint; }

int adj_alloc(imsrg_basis *b, long n, double **out) {
  void *p = nullptr;
  IMSRG_CUDA_TRY(cudaMalloc(&p, (size_t)std::max(n, 1L) * sizeof(double)));
  b->dev_allocs.push_back(p);
  *out = (double *)p;
  return IMSRG_OK;
}

AdjTerm aterm(int a, long aoff, int lda, int ta, int bsrc, long boff, int ldb, int tb, int K, double coef,
              int hl = 0, int hr = 0) {
  AdjTerm t{};
  t.a_src = a;
  t.a_off = aoff;
  t.lda = lda;
  t.ta = ta;
  t.b_src = bsrc;
  t.b_off = boff;
  t.ldb = ldb;
  t.tb = tb;
  t.K = K;
  t.coef = coef;
  t.use_hl = hl;
  t.use_hr = hr;
  return t;
}

// The transposes of the forward products (basis.cpp's problem list, with
// R the variable): for each forward term alpha op(A) op(R) the adjoint adds
// alpha op(A)^T Wbar into Rbar, for alpha op(R) op(B) it adds alpha Wbar
// op(B)^T; the terms that land on one array of one block are one problem.
std::vector<AdjProb> adjoint_problems(const imsrg_basis *b) {
  std::vector<AdjProb> out;
  auto add = [&](int M, int N, int dst, long off, int ldc, std::initializer_list<AdjTerm> ts) {
    if (M <= 0 || N <= 0) return;
    AdjProb p{};
    p.M = M;
    p.N = N;
    p.c_dst = dst;
    p.c_off = off;
    p.ldc = ldc;
    for (const AdjTerm &t : ts)
      if (t.K > 0) p.t[p.nterms++] = t;
    if (p.nterms) out.push_back(p);
  };
  for (int qb = 0; qb < b->nblocks; qb++) {
    const int np = b->npp[qb], nb = b->nph[qb], nh = b->nhh[qb];
    auto G = [&](int g) { return b->gam_off[qb * 6 + g - 1]; };
    // pppp: W1_pppp = L1 R1, W1_pphh = -R1 L3, W1_ppph = -R1 L2
    add(np, np, AD_Y, G(1), np,
        {aterm(AS_X, G(1), np, 1, AS_W1, G(1), np, 0, np, 1.0), aterm(AS_W1, G(3), np, 0, AS_X, G(3), np, 1, nh, -1.0),
         aterm(AS_W1, G(2), np, 0, AS_X, G(2), np, 1, nb, -1.0)});
    // hhhh: W2_hhhh = L5 R5, W2_pphh = L3 R5, W2_phhh = L6 R5
    add(nh, nh, AD_Y, G(5), nh,
        {aterm(AS_X, G(5), nh, 1, AS_W2, G(5), nh, 0, nh, 1.0), aterm(AS_X, G(3), np, 1, AS_W2, G(3), np, 0, np, 1.0),
         aterm(AS_X, G(6), nb, 1, AS_W2, G(6), nb, 0, nb, 1.0)});
    // pphh: W1_hhhh = hL L3^T R3, W2_pppp = hR L3 R3^T, W1_pphh = L1 R3,
    // W2_pphh = -R3 L5, W1_phhh = hL L2^T R3, W2_ppph = -hL R3 L6^T
    add(np, nh, AD_Y, G(3), np,
        {aterm(AS_X, G(3), np, 0, AS_W1, G(5), nh, 0, nh, 1.0, 1, 0),
         aterm(AS_W2, G(1), np, 1, AS_X, G(3), np, 0, np, 1.0, 0, 1),
         aterm(AS_X, G(1), np, 1, AS_W1, G(3), np, 0, np, 1.0),
         aterm(AS_W2, G(3), np, 0, AS_X, G(5), nh, 1, nh, -1.0),
         aterm(AS_X, G(2), np, 0, AS_W1, G(6), nb, 0, nb, 1.0, 1, 0),
         aterm(AS_W2, G(2), np, 0, AS_X, G(6), nb, 0, nb, -1.0, 1, 0)});
    // ppph: W1_phph = hL L2^T R2, W1_ppph = L1 R2, W1_phhh = -hR R2^T L3
    add(np, nb, AD_Y, G(2), np,
        {aterm(AS_X, G(2), np, 0, AS_W1, G(4), nb, 0, nb, 1.0, 1, 0),
         aterm(AS_X, G(1), np, 1, AS_W1, G(2), np, 0, np, 1.0),
         aterm(AS_X, G(3), np, 0, AS_W1, G(6), nb, 1, nh, -1.0, 0, 1)});
    // phhh: W2_phph = hR L6 R6^T, W2_phhh = -R6 L5, W2_ppph = hR L3 R6^T
    add(nb, nh, AD_Y, G(6), nb,
        {aterm(AS_W2, G(4), nb, 1, AS_X, G(6), nb, 0, nb, 1.0, 0, 1),
         aterm(AS_W2, G(6), nb, 0, AS_X, G(5), nh, 1, nh, -1.0),
         aterm(AS_W2, G(2), np, 1, AS_X, G(3), np, 0, np, 1.0, 0, 1)});
  }
  // WCC = LCC RCC^T per cross-coupled block: RCCbar = WCCbar^T LCC
  for (int q1 = 0; q1 < b->ccblocks; q1++) {
    const int r = b->cc_rlen[q1], nb = b->cc_nph[q1];
    add(r, nb, AD_RCC, b->cc_off[q1], r, {aterm(AS_WCC, b->wcc_off[q1], r, 1, AS_LCC, b->cc_off[q1], r, 0, r, 1.0)});
  }
  int tiles = 0;
  for (AdjProb &p : out) {
    p.tiles_m = (p.M + BM - 1) / BM;
    p.tiles = p.tiles_m * ((p.N + BN - 1) / BN);
    p.tile0 = tiles;
    tiles += p.tiles;
  }
  return out;
}

}  // namespace

int adjoint_prepare(imsrg_basis *b) {
  if (b->adjoint) return IMSRG_OK;
  AdjState *a = new AdjState();
  b->adjoint = a;
  IMSRG_TRY(adj_alloc(b, b->nfull, &a->w1b));
  IMSRG_TRY(adj_alloc(b, b->nfull, &a->w2b));
  IMSRG_TRY(adj_alloc(b, b->cc_total, &a->rccb));
  IMSRG_TRY(adj_alloc(b, b->wcc_total, &a->wccb));
  IMSRG_TRY(adj_alloc(b, b->T.n_ph, &a->zb));
  IMSRG_TRY(adj_alloc(b, (long)b->norb * b->norb, &a->monob));
  IMSRG_TRY(adj_alloc(b, DOT_CTAS, &a->part));
  IMSRG_TRY(adj_alloc(b, 1, &a->dot));
  IMSRG_CUDA_TRY(cudaMallocHost((void **)&a->h_dot, sizeof(double)));
  std::vector<AdjProb> probs = adjoint_problems(b);
  a->nprobs = (int)probs.size();
  a->ntiles = probs.empty() ? 0 : probs.back().tile0 + probs.back().tiles;
  if (a->nprobs) {
    void *p = nullptr;
    IMSRG_CUDA_TRY(cudaMalloc(&p, probs.size() * sizeof(AdjProb)));
    b->dev_allocs.push_back(p);
    a->d_probs = (AdjProb *)p;
    IMSRG_CUDA_TRY(cudaMemcpy(a->d_probs, probs.data(), probs.size() * sizeof(AdjProb), cudaMemcpyHostToDevice));
  }
  return IMSRG_OK;
}

void adjoint_free(imsrg_basis *b) {
  AdjState *a = adj_of(b);
  if (!a) return;
  if (a->h_dot) cudaFreeHost(a->h_dot);
  delete a;  // device buffers are in b->dev_allocs
  b->adjoint = nullptr;
}

// Yb = d<Cb, [X, Y]> / dY for herm(X) = hX, herm(Y) = hY; with_e0 = 0: the
// commutator leaves RES E0 alone (as MAGNUS_EXPAND's do), so Cb[0] is ignored.
int commutator_adjoint_dev(imsrg_basis *b, const double *X, int hX, const double *Cb, int hY, int with_e0,
                           double *Yb) {
  IMSRG_TRY(adjoint_prepare(b));
  AdjState *a = adj_of(b);
  cudaStream_t st = b->stream;
  const int hL = hX, hR = hY, hRES = -hX * hY;
  const size_t nf = b->nfull * sizeof(double);
  IMSRG_CUDA_TRY(cudaMemsetAsync(Yb, 0, nf, st));
  IMSRG_CUDA_TRY(cudaMemsetAsync(a->w1b, 0, nf, st));
  IMSRG_CUDA_TRY(cudaMemsetAsync(a->w2b, 0, nf, st));
  if (b->T.n_ph) IMSRG_CUDA_TRY(cudaMemsetAsync(a->zb, 0, b->T.n_ph * sizeof(double), st));
  if (b->cc_total) IMSRG_CUDA_TRY(cudaMemsetAsync(a->rccb, 0, b->cc_total * sizeof(double), st));
  if (b->wcc_total) IMSRG_CUDA_TRY(cudaMemsetAsync(a->wccb, 0, b->wcc_total * sizeof(double), st));
  // LCC = Pandya transform of X (the fixed factor of RCCbar = WCCbar^T LCC)
  IMSRG_TRY(launch_cc_forward(b, X, hX, X, hX, nullptr, 0, 0, 1, st));
  ProfScope ps(b, IMSRG_KERNEL_OPS, st);
  const int with220 = with_e0 && hL * hR == -1;
  if (b->T.n_asm2 > 0)
    k_adj_asm2<<<(unsigned)((b->T.n_asm2 + 127) / 128), 128, 0, st>>>(b->T, X, hL, hR, Cb, hRES, with220, Yb,
                                                                       a->w1b, a->w2b, a->zb);
  const int grid1 = b->T.n_asm1_heavy + (b->T.n_asm1_light + 3) / 4;
  if (grid1 > 0) k_adj_1body<<<grid1, 128, 0, st>>>(b->T, X, hL, hR, Cb, hRES, Yb, a->w1b, a->w2b);
  if (with_e0 && b->P * b->A > 0)
    k_adj_e0<<<(b->P * b->A + 255) / 256, 256, 0, st>>>(b->T, X, hL, hR, Cb, Yb);
  if (b->T.n_ph > 0)
    k_adj_ph<<<(unsigned)((b->T.n_ph + 255) / 256), 256, 0, st>>>(b->T, a->zb, hL, hR, a->wccb);
  if (a->ntiles > 0) {
    AdjOps ops{};
    ops.src[AS_X] = X;
    ops.src[AS_W1] = a->w1b;
    ops.src[AS_W2] = a->w2b;
    ops.src[AS_WCC] = a->wccb;
    ops.src[AS_LCC] = b->lcc;
    ops.dst[AD_Y] = Yb;
    ops.dst[AD_RCC] = a->rccb;
    k_gemm_adj<<<a->ntiles, 256, 0, st>>>(a->d_probs, a->nprobs, ops, hL, hR);
  }
  if (b->cc_total > 0)
    k_adj_cc<<<(unsigned)((b->cc_total + 255) / 256), 256, 0, st>>>(b->T, a->rccb, hR, Yb);
  b->launches += 6;
  return cuda_status(cudaGetLastError());
}

// <x, y> over n doubles in a fixed order, into host memory.
int dot_dev(imsrg_basis *b, const double *x, const double *y, long n, double *out) {
  IMSRG_TRY(adjoint_prepare(b));
  AdjState *a = adj_of(b);
  k_dot_partial<<<DOT_CTAS, DOT_THREADS, 0, b->stream>>>(x, y, n, a->part);
  k_dot_final<<<1, 1, 0, b->stream>>>(a->part, a->dot);
  b->launches += 2;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(a->h_dot, a->dot, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  *out = *a->h_dot;
  return IMSRG_OK;
}

double *adjoint_monob(imsrg_basis *b) { return adj_of(b) ? adj_of(b)->monob : nullptr; }

}  // namespace imsrg
