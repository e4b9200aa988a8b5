// ode.cu -- the Shampine-Gordon ODE solver on the device and the ODE flow of
// the Hamiltonian (the reference's alternative to the Magnus flow).
//
// Restates decouple_hamiltonian (im-SRG/IMSRG_ODE.f90:9-178) with its
// derivative dHds (:416-463), and the solver it calls (im-SRG/adams_ode.f90:
// ODE :33-247, DE :249-595, STEP :597-1230, INTRP :1232-1357): the published
// variable-order (1-12), variable-step Adams PECE method with local
// extrapolation of Shampine and Gordon (1975).  The solver's state -- the
// packed operator y (the reference's vectorize order, neq doubles), the
// weights, the predictor and the 16 modified-divided-difference columns phi --
// stays on the device; every neq-long vector operation of a step is one fused
// element-wise kernel, and its weighted sums of squares are per-CTA partials
// summed on the host in a fixed order (deterministic).  The host keeps the
// solver's scalar recurrences (psi, alpha, beta, sigma, g, v, w), the order
// and step-size control, exactly as the published method states them.
#include <cmath>
#include <cstring>
#include <vector>

#include "device.cuh"

namespace imsrg {

namespace {

constexpr int ODE_THREADS = 256;
constexpr int ODE_CTAS = 304;  // two per SM; also the number of partial sums

// Constants of STEP's error estimates (adams_ode.f90:772-780), as published.
const double kGstr[13] = {0.50,   0.0833,  0.0417,  0.0264,  0.0188,  0.0143, 0.0114,
                          0.00936, 0.00789, 0.00679, 0.00592, 0.00524, 0.00468};
const double kTwo[13] = {2.0,   4.0,   8.0,   16.0,   32.0,   64.0,  128.0,
                         256.0, 512.0, 1024.0, 2048.0, 4096.0, 8192.0};
constexpr int kMaxNum = 500;  // DE's step budget per call (adams_ode.f90:404)

// Column i (1-based as in the method's statement) of phi.
__device__ __forceinline__ double *col(double *phi, long n, int i) { return phi + (long)(i - 1) * n; }
__device__ __forceinline__ const double *col(const double *phi, long n, int i) { return phi + (long)(i - 1) * n; }

struct PredictCoef {
  double beta[12], g[13], h;
  int k, ns, nornd;
};

__global__ void __launch_bounds__(ODE_THREADS) k_ode_wt(const double *__restrict__ y, double *__restrict__ wt, long n,
                                                        double releps, double abseps) {
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x)
    wt[l] = releps * fabs(y[l]) + abseps;
}

// Up to three weighted sums of squares in one pass: sum_l ((sum_t c[j][t]
// v[j][t][l]) / wt[l])^2, one partial per CTA (grid-stride, fixed order).
struct SumSq {
  const double *v[3][3];
  double c[3][3];
  int nsum;
};

__global__ void __launch_bounds__(ODE_THREADS) k_ode_sumsq(SumSq s, const double *__restrict__ wt, long n,
                                                           double *part) {
  __shared__ double sh[3][ODE_THREADS / 32];
  double acc[3] = {0.0, 0.0, 0.0};
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x) {
    const double w = wt[l];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (j >= s.nsum) break;
      double x = 0.0;
#pragma unroll
      for (int t = 0; t < 3; t++)
        if (s.v[j][t]) x += s.c[j][t] * s.v[j][t][l];
      x /= w;
      acc[j] += x * x;
    }
  }
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const double v = warp_sum(acc[j]);
    if ((threadIdx.x & 31) == 0) sh[j][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < ODE_THREADS / 32; w++) t += sh[threadIdx.x][w];
    part[blockIdx.x * 3 + threadIdx.x] = t;
  }
}

// STEP's predictor (adams_ode.f90, "predict a solution p"): phi_i *= beta_i
// (i > ns), shift columns k+1 -> k+2, p = sum_i g_i phi_i while forming
// phi_i += phi_(i+1), then p = y + h p (with the rounding-error compensation
// in columns 15/16 when nornd is off).
__global__ void __launch_bounds__(ODE_THREADS) k_ode_predict(double *phi, const double *__restrict__ y,
                                                             double *__restrict__ p, long n, PredictCoef c) {
  const int k = c.k, kp1 = k + 1, kp2 = k + 2;
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x) {
    for (int i = c.ns + 1; i <= k; i++) col(phi, n, i)[l] = c.beta[i - 1] * col(phi, n, i)[l];
    col(phi, n, kp2)[l] = col(phi, n, kp1)[l];
    col(phi, n, kp1)[l] = 0.0;
    double acc = 0.0, nxt = 0.0;  // nxt = phi_(i+1) of the loop below (phi_(k+1) = 0)
    for (int j = 1; j <= k; j++) {
      const int i = kp1 - j;
      const double pi = col(phi, n, i)[l];
      acc = acc + pi * c.g[i - 1];
      const double upd = pi + nxt;
      col(phi, n, i)[l] = upd;
      nxt = upd;
    }
    const double yl = y[l];
    if (!c.nornd) {
      const double tau = c.h * acc - col(phi, n, 15)[l];
      const double pl = yl + tau;
      p[l] = pl;
      col(phi, n, 16)[l] = (pl - yl) - tau;
    } else {
      p[l] = yl + c.h * acc;
    }
  }
}

// A rejected step restores the differences: phi_i = (phi_i - phi_(i+1)) / beta_i, i = 1..k.
__global__ void __launch_bounds__(ODE_THREADS) k_ode_restore(double *phi, long n, PredictCoef c) {
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x)
    for (int i = 1; i <= c.k; i++) col(phi, n, i)[l] = (col(phi, n, i)[l] - col(phi, n, i + 1)[l]) / c.beta[i - 1];
}

// The corrector: y = p + h g_(k+1) (yp - phi_1) (compensated when nornd is off).
__global__ void __launch_bounds__(ODE_THREADS) k_ode_correct(double *phi, const double *__restrict__ p,
                                                             const double *__restrict__ yp, double *__restrict__ y,
                                                             long n, double hg, int nornd) {
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x) {
    const double pl = p[l];
    if (!nornd) {
      const double rho = hg * (yp[l] - col(phi, n, 1)[l]) - col(phi, n, 16)[l];
      const double yl = pl + rho;
      y[l] = yl;
      col(phi, n, 15)[l] = (yl - pl) - rho;
    } else {
      y[l] = pl + hg * (yp[l] - col(phi, n, 1)[l]);
    }
  }
}

// After the final evaluation: phi_(k+1) = yp - phi_1, phi_(k+2) = phi_(k+1) -
// phi_(k+2), phi_i += phi_(k+1) for i = 1..k.
__global__ void __launch_bounds__(ODE_THREADS) k_ode_update(double *phi, const double *__restrict__ yp, long n, int k) {
  const int kp1 = k + 1, kp2 = k + 2;
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x) {
    const double d = yp[l] - col(phi, n, 1)[l];
    col(phi, n, kp1)[l] = d;
    col(phi, n, kp2)[l] = d - col(phi, n, kp2)[l];
    for (int i = 1; i <= k; i++) col(phi, n, i)[l] = col(phi, n, i)[l] + d;
  }
}

struct IntrpCoef {
  double g[13], rho[13], hi;
  int ki;
};

// INTRP: yout = y + hi sum_i g_i phi_i, ypout = sum_i rho_i phi_i (i = ki .. 1).
__global__ void __launch_bounds__(ODE_THREADS) k_ode_intrp(const double *phi, const double *__restrict__ y,
                                                           double *__restrict__ yout, double *__restrict__ ypout,
                                                           long n, IntrpCoef c) {
  for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (long)gridDim.x * blockDim.x) {
    double a = 0.0, b = 0.0;
    for (int j = 1; j <= c.ki; j++) {
      const int i = c.ki + 1 - j;
      const double v = col(phi, n, i)[l];
      a = a + c.g[i - 1] * v;
      b = b + c.rho[i - 1] * v;
    }
    yout[l] = y[l] + c.hi * a;
    ypout[l] = b;
  }
}

// The solver: device vectors and the method's scalar state.
struct DevSg {
  imsrg_basis *b = nullptr;
  long n = 0;
  int generator = IMSRG_GEN_WHITE, precision = IMSRG_PREC_FP64;
  imsrg_op *HSop = nullptr, *DHop = nullptr;  // flat work operators of the derivative
  double *mem = nullptr;
  double *yy = nullptr, *wt = nullptr, *p = nullptr, *yp = nullptr, *ypout = nullptr, *phi = nullptr;
  double *part = nullptr;  // ODE_CTAS x 3 partial sums
  double *h_part = nullptr;
  long nfev = 0;
  double alpha[12] = {}, beta[12] = {}, sig[13] = {}, v[12] = {}, w[12] = {}, g[13] = {}, psi[12] = {};
  double x = 0, h = 0, hold = 0, told = 0, delsgn = 0;
  bool start = false, phase1 = false, nornd = false;
  int ns = 0, k = 0, kold = 0, isnold = 0;

  int init(imsrg_basis *bb) {
    b = bb;
    n = b->neq;
    IMSRG_TRY(work_op(b, 15, &HSop));
    IMSRG_TRY(work_op(b, 16, &DHop));
    IMSRG_CUDA_TRY(cudaMalloc((void **)&mem, (size_t)(5 + 16) * n * sizeof(double) + ODE_CTAS * 3 * sizeof(double)));
    IMSRG_CUDA_TRY(cudaMemsetAsync(mem, 0, (size_t)(5 + 16) * n * sizeof(double), b->stream));
    yy = mem;
    wt = yy + n;
    p = wt + n;
    yp = p + n;
    ypout = yp + n;
    phi = ypout + n;
    part = phi + 16 * n;
    IMSRG_CUDA_TRY(cudaMallocHost((void **)&h_part, ODE_CTAS * 3 * sizeof(double)));
    return IMSRG_OK;
  }
  void release() {
    if (mem) cudaFree(mem);
    if (h_part) cudaFreeHost(h_part);
    mem = nullptr;
    h_part = nullptr;
  }
  double *phicol(int i) { return phi + (long)(i - 1) * n; }
  unsigned grid() const { return (unsigned)std::min<long>((n + ODE_THREADS - 1) / ODE_THREADS, ODE_CTAS); }

  // yp = dHds(y): unpack, generator, commutator, pack (IMSRG_ODE.f90:416-463)
  int f(const double *y, double *out) {
    nfev++;
    HSop->herm = 1;
    IMSRG_TRY(launch_unpack(b, y, 1, HSop->d));
    IMSRG_TRY(dhds_dev(b, HSop->d, 1, DHop->d, generator, precision));
    return launch_pack(b, DHop->d, out);
  }
  // weighted sums of squares (up to three), summed on the host in CTA order
  int sumsq(const SumSq &s, double *out) {
    k_ode_sumsq<<<ODE_CTAS, ODE_THREADS, 0, b->stream>>>(s, wt, n, part);
    b->launches++;
    IMSRG_CUDA_TRY(cudaGetLastError());
    IMSRG_CUDA_TRY(cudaMemcpyAsync(h_part, part, ODE_CTAS * 3 * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    IMSRG_TRY(ozaki_check_error(b));
    for (int j = 0; j < s.nsum; j++) {
      double t = 0.0;
      for (int c = 0; c < ODE_CTAS; c++) t += h_part[c * 3 + j];
      out[j] = t;
    }
    return IMSRG_OK;
  }
  int sumsq1(const double *a, double ca, const double *bb, double cb, const double *c, double cc, double *out) {
    SumSq s{};
    s.nsum = 1;
    s.v[0][0] = a;
    s.c[0][0] = ca;
    s.v[0][1] = bb;
    s.c[0][1] = cb;
    s.v[0][2] = c;
    s.c[0][2] = cc;
    return sumsq(s, out);
  }

  // STEP (adams_ode.f90:597-1230).  *crash set when h or eps had to be
  // raised (eps updated in place).
  int step(double &eps, bool *crash) {
    const double twou = 2.0 * 2.220446049250313e-16, fouru = 2.0 * twou;
    *crash = true;
    if (std::fabs(h) < fouru * std::fabs(x)) {
      h = std::copysign(fouru * std::fabs(x), h);
      return IMSRG_OK;
    }
    const double p5eps = 0.5 * eps;
    double s2;
    IMSRG_TRY(sumsq1(yy, 1.0, nullptr, 0, nullptr, 0, &s2));
    const double round = twou * std::sqrt(s2);
    if (p5eps < round) {
      eps = 2.0 * round * (1.0 + fouru);
      return IMSRG_OK;
    }
    *crash = false;
    g[0] = 1.0;
    g[1] = 0.5;
    sig[0] = 1.0;
    if (start) {
      IMSRG_TRY(f(yy, yp));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(phicol(1), yp, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaMemsetAsync(phicol(2), 0, n * sizeof(double), b->stream));
      double t2;
      IMSRG_TRY(sumsq1(yp, 1.0, nullptr, 0, nullptr, 0, &t2));
      const double total = std::sqrt(t2);
      double absh = std::fabs(h);
      if (eps < 16.0 * total * h * h) absh = 0.25 * std::sqrt(eps / total);
      h = std::copysign(std::max(absh, fouru * std::fabs(x)), h);
      hold = 0.0;
      k = 1;
      kold = 0;
      start = false;
      phase1 = true;
      nornd = true;
      if (p5eps <= 100.0 * round) {
        nornd = false;
        IMSRG_CUDA_TRY(cudaMemsetAsync(phicol(15), 0, n * sizeof(double), b->stream));
      }
    }
    int ifail = 0;
    int knew = 0;
    double erk = 0, erkm1 = 0, absh = 0;
    for (;;) {
      const int kp1 = k + 1, kp2 = k + 2, km1 = k - 1, km2 = k - 2;
      if (h != hold) ns = 0;
      if (ns <= kold) ns++;
      const int nsp1 = ns + 1;
      if (ns <= k) {
        beta[ns - 1] = 1.0;
        alpha[ns - 1] = 1.0 / ns;
        double temp1 = h * ns;
        sig[nsp1 - 1] = 1.0;
        for (int i = nsp1; i <= k; i++) {
          const double temp2 = psi[i - 2];
          psi[i - 2] = temp1;
          beta[i - 1] = beta[i - 2] * psi[i - 2] / temp2;
          temp1 = temp2 + h;
          alpha[i - 1] = h / temp1;
          sig[i] = i * alpha[i - 1] * sig[i - 1];
        }
        psi[k - 1] = temp1;
        if (ns <= 1) {
          for (int iq = 1; iq <= k; iq++) {
            v[iq - 1] = 1.0 / (double)(iq * (iq + 1));
            w[iq - 1] = v[iq - 1];
          }
        } else {
          if (kold < k) {
            v[k - 1] = 1.0 / (double)(k * kp1);
            for (int j = 1; j <= ns - 2; j++) {
              const int i = k - j;
              v[i - 1] = v[i - 1] - alpha[j] * v[i];
            }
          }
          for (int iq = 1; iq <= kp1 - ns; iq++) {
            v[iq - 1] = v[iq - 1] - alpha[ns - 1] * v[iq];
            w[iq - 1] = v[iq - 1];
          }
          g[nsp1 - 1] = w[0];
        }
        for (int i = ns + 2; i <= kp1; i++) {
          for (int iq = 1; iq <= kp2 - i; iq++) w[iq - 1] = w[iq - 1] - alpha[i - 2] * w[iq];
          g[i - 1] = w[0];
        }
      }
      PredictCoef pc{};
      std::memcpy(pc.beta, beta, sizeof(beta));
      std::memcpy(pc.g, g, sizeof(g));
      pc.h = h;
      pc.k = k;
      pc.ns = ns;
      pc.nornd = nornd;
      k_ode_predict<<<grid(), ODE_THREADS, 0, b->stream>>>(phi, yy, p, n, pc);
      b->launches++;
      IMSRG_CUDA_TRY(cudaGetLastError());
      const double xold = x;
      x = x + h;
      absh = std::fabs(h);
      IMSRG_TRY(f(p, yp));
      // erkm2, erkm1 and erk in one pass
      SumSq s{};
      s.nsum = 3;
      s.v[0][0] = yp;
      s.c[0][0] = 1.0;
      s.v[0][1] = phicol(1);
      s.c[0][1] = -1.0;
      if (km2 >= 0) {
        s.v[1][0] = phicol(k);
        s.c[1][0] = 1.0;
        s.v[1][1] = yp;
        s.c[1][1] = 1.0;
        s.v[1][2] = phicol(1);
        s.c[1][2] = -1.0;
      }
      if (km2 > 0) {
        s.v[2][0] = phicol(km1);
        s.c[2][0] = 1.0;
        s.v[2][1] = yp;
        s.c[2][1] = 1.0;
        s.v[2][2] = phicol(1);
        s.c[2][2] = -1.0;
      }
      double sums[3];
      IMSRG_TRY(sumsq(s, sums));
      double erkm2 = 0.0;
      erkm1 = 0.0;
      if (km2 > 0) erkm2 = absh * sig[km1 - 1] * kGstr[km2 - 1] * std::sqrt(sums[2]);
      if (km2 >= 0) erkm1 = absh * sig[k - 1] * kGstr[km1 - 1] * std::sqrt(sums[1]);
      const double serk = std::sqrt(sums[0]);
      const double err = absh * serk * (g[k - 1] - g[kp1 - 1]);
      erk = absh * serk * sig[kp1 - 1] * kGstr[k - 1];
      knew = k;
      if (km2 > 0) {
        if (std::max(erkm1, erkm2) <= erk) knew = km1;
      } else if (km2 == 0) {
        if (erkm1 <= 0.5 * erk) knew = km1;
      }
      if (!std::isfinite(err)) return IMSRG_ERR_NONFINITE;
      if (err <= eps) break;
      // rejected: restore the differences, shrink h, maybe lower the order
      phase1 = false;
      x = xold;
      k_ode_restore<<<grid(), ODE_THREADS, 0, b->stream>>>(phi, n, pc);
      b->launches++;
      IMSRG_CUDA_TRY(cudaGetLastError());
      for (int i = 2; i <= k; i++) psi[i - 2] = psi[i - 1] - h;
      ifail++;
      double temp2 = 0.5;
      if (ifail > 3 && p5eps < 0.25 * erk) temp2 = std::sqrt(p5eps / erk);
      if (ifail >= 3) knew = 1;
      h = temp2 * h;
      k = knew;
      if (std::fabs(h) < fouru * std::fabs(x)) {
        *crash = true;
        h = std::copysign(fouru * std::fabs(x), h);
        eps = eps + eps;
        return IMSRG_OK;
      }
    }
    const int kp1 = k + 1, kp2 = k + 2, km1 = k - 1;
    kold = k;
    hold = h;
    k_ode_correct<<<grid(), ODE_THREADS, 0, b->stream>>>(phi, p, yp, yy, n, h * g[kp1 - 1], nornd);
    b->launches++;
    IMSRG_CUDA_TRY(cudaGetLastError());
    IMSRG_TRY(f(yy, yp));
    k_ode_update<<<grid(), ODE_THREADS, 0, b->stream>>>(phi, yp, n, k);
    b->launches++;
    IMSRG_CUDA_TRY(cudaGetLastError());
    double erkp1 = 0.0;
    if (knew == km1 || k == 12) phase1 = false;
    if (phase1) {
      k = kp1;
      erk = erkp1;
    } else if (knew == km1) {
      k = km1;
      erk = erkm1;
    } else if (kp1 <= ns) {
      double s3;
      IMSRG_TRY(sumsq1(phicol(kp2), 1.0, nullptr, 0, nullptr, 0, &s3));
      erkp1 = absh * kGstr[kp1 - 1] * std::sqrt(s3);
      if (k == 1) {
        if (erkp1 < 0.5 * erk) {
          k = kp1;
          erk = erkp1;
        }
      } else if (erkm1 <= std::min(erk, erkp1)) {
        k = km1;
        erk = erkm1;
      } else if (erkp1 < erk && k < 12) {
        k = kp1;
        erk = erkp1;
      }
    }
    double hnew = h + h;
    if (!phase1) {
      if (p5eps < erk * kTwo[k]) {
        hnew = h;
        if (p5eps < erk) {
          const double r = std::pow(p5eps / erk, 1.0 / (double)(k + 1));
          hnew = absh * std::max(0.5, std::min(0.9, r));
          hnew = std::copysign(std::max(hnew, fouru * std::fabs(x)), h);
        }
      }
    }
    h = hnew;
    return IMSRG_OK;
  }

  // INTRP (adams_ode.f90:1232-1357) into yout
  int intrp(double xout, double *yout) {
    IntrpCoef c{};
    const double hi = xout - x;
    const int ki = kold + 1;
    double ww[14] = {};
    for (int i = 1; i <= ki; i++) ww[i - 1] = 1.0 / i;
    c.g[0] = 1.0;
    c.rho[0] = 1.0;
    double term = 0.0;
    for (int j = 2; j <= ki; j++) {
      const double psijm1 = psi[j - 2];
      const double gamma = (hi + term) / psijm1;
      const double eta = hi / psijm1;
      for (int i = 1; i <= ki + 1 - j; i++) ww[i - 1] = gamma * ww[i - 1] - eta * ww[i];
      c.g[j - 1] = ww[0];
      c.rho[j - 1] = gamma * c.rho[j - 2];
      term = psijm1;
    }
    c.hi = hi;
    c.ki = ki;
    k_ode_intrp<<<grid(), ODE_THREADS, 0, b->stream>>>(phi, yy, yout, ypout, n, c);
    b->launches++;
    return cuda_status(cudaGetLastError());
  }

  // DE (adams_ode.f90:249-595) for a positive IFLAG (the flow driver's use):
  // advances from t to tout, the result in y (device, packed).
  int de(double *y, double &t, double tout, double &relerr, double &abserr, int &iflag) {
    const double fouru = 4.0 * 2.220446049250313e-16;
    if (t == tout || relerr < 0.0 || abserr < 0.0) {
      iflag = 6;
      return IMSRG_OK;
    }
    double eps = std::max(relerr, abserr);
    if (eps <= 0.0 || iflag <= 0) {
      iflag = 6;
      return IMSRG_OK;
    }
    const int isn = 1;
    if (iflag != 1 && (t != told || iflag < 2 || iflag > 5)) {
      iflag = 6;
      return IMSRG_OK;
    }
    const double del = tout - t, absdel = std::fabs(del);
    const double tend = t + 10.0 * del;
    int nostep = 0, kle4 = 0;
    bool stiff = false;
    const double releps = relerr / eps, abseps = abserr / eps;
    if (iflag == 1 || isnold < 0 || delsgn * del <= 0.0) {
      start = true;
      x = t;
      IMSRG_CUDA_TRY(cudaMemcpyAsync(yy, y, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
      delsgn = std::copysign(1.0, del);
      h = std::copysign(std::max(std::fabs(tout - x), fouru * std::fabs(x)), tout - x);
    }
    for (;;) {
      if (absdel <= std::fabs(x - t)) {
        IMSRG_TRY(intrp(tout, y));
        iflag = 2;
        t = told = tout;
        isnold = isn;
        return IMSRG_OK;
      }
      if (kMaxNum <= nostep) {
        iflag = stiff ? 5 : 4;
        IMSRG_CUDA_TRY(cudaMemcpyAsync(y, yy, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
        t = told = x;
        isnold = 1;
        return IMSRG_OK;
      }
      h = std::copysign(std::min(std::fabs(h), std::fabs(tend - x)), h);
      k_ode_wt<<<grid(), ODE_THREADS, 0, b->stream>>>(yy, wt, n, releps, abseps);
      b->launches++;
      IMSRG_CUDA_TRY(cudaGetLastError());
      bool crash = false;
      IMSRG_TRY(step(eps, &crash));
      if (crash) {
        iflag = 3;
        relerr = eps * releps;
        abserr = eps * abseps;
        IMSRG_CUDA_TRY(cudaMemcpyAsync(y, yy, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
        t = told = x;
        isnold = 1;
        return IMSRG_OK;
      }
      nostep++;
      kle4++;
      if (kold > 4) kle4 = 0;
      if (kle4 >= 50) stiff = true;
    }
  }
};

}  // namespace

}  // namespace imsrg

extern "C" {

int imsrg_gpu_ode_decouple(imsrg_op_t *HS, int generator, int precision, double ds, double s_max, int max_steps,
                           double relerr, double abserr, double *trace, int *steps_out, long *nfev) {
  using namespace imsrg;
  if (!HS || !HS->b || !HS->d || !trace || max_steps < 0 || !(ds > 0.0)) return IMSRG_ERR_INVALID;
  if (generator != IMSRG_GEN_WHITE && generator != IMSRG_GEN_ATAN && generator != IMSRG_GEN_W2)
    return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  if (HS->herm != 1) return IMSRG_ERR_INVALID;
  imsrg_basis *b = HS->b;
  const double conv_crit = 1e-6;  // IMSRG_ODE.f90:15
  DevSg sg;
  sg.generator = generator;
  sg.precision = precision;
  int st = sg.init(b);
  double *y = nullptr;
  if (st == IMSRG_OK) st = cuda_status(cudaMalloc((void **)&y, b->neq * sizeof(double)));
  double s = 0.0;
  int steps = 0, iflag = 1;
  double emp2 = 0.0, e0 = 0.0;
  auto scalars = [&]() -> int {  // E0 and mbpt2 of HS
    IMSRG_TRY(launch_mbpt2(b, HS->d, 1, b->scal));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(b->scal + 1, HS->d, sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(b->h_scal, b->scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    emp2 = b->h_scal[0];
    e0 = b->h_scal[1];
    return (std::isfinite(emp2) && std::isfinite(e0)) ? IMSRG_OK : IMSRG_ERR_NONFINITE;
  };
  if (st == IMSRG_OK) st = scalars();
  if (st == IMSRG_OK) {
    double *row = trace;
    row[0] = 0;
    row[1] = s;
    row[2] = e0;
    row[3] = e0 + emp2;
    row[4] = std::fabs(emp2);
  }
  while (st == IMSRG_OK && steps < max_steps) {
    st = launch_pack(b, HS->d, y);  // vectorize(H, cur_vec)
    if (st != IMSRG_OK) break;
    st = sg.de(y, s, s + ds, relerr, abserr, iflag);
    if (st != IMSRG_OK) break;
    if (iflag == 6) {
      st = IMSRG_ERR_INVALID;
      break;
    }
    st = launch_unpack(b, y, 1, HS->d);  // repackage(H, cur_vec)
    if (st != IMSRG_OK) break;
    steps++;
    st = scalars();
    if (st != IMSRG_OK) break;
    double *row = trace + 5 * (long)steps;
    row[0] = steps;
    row[1] = s;
    row[2] = e0;
    row[3] = e0 + emp2;
    row[4] = std::fabs(emp2);
    if (std::fabs(emp2) < conv_crit || (s_max > 0.0 && s >= s_max - 1e-12)) break;
  }
  if (steps_out) *steps_out = steps;
  if (nfev) *nfev = sg.nfev;
  cudaStreamSynchronize(b->stream);
  sg.release();
  if (y) cudaFree(y);
  return st;
}

}  // extern "C"
