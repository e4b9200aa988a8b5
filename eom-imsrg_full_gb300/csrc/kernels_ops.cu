// kernels_ops.cu -- operator arithmetic, norms, mbpt2, the White generator and
// the packed-layout conversions, all on the basis stream.
//
// Reference routines (n-parzuchowski/EOM-IMSRG_FULL, im-SRG/):
//   add_sq_op        basic_IMSRG.f90:3450-3478
//   mat_frob_norm    basic_IMSRG.f90:3921-3952
//   mbpt2            basic_IMSRG.f90:4030-4064
//   build_gs_white   generators.f90:4-106 (twobody_monopole basic_IMSRG.f90:2031-2046)
//   vectorize        basic_IMSRG.f90:3794-3854, repackage :3857-3918
// Reductions use fixed-order partial sums (no atomics): results are
// bit-reproducible.
#include "device.cuh"

namespace imsrg {

namespace {

// C = ax A + bx B; bx_dev, when given, supplies bx from device memory (the
// graph-captured flow), with the same arithmetic as the scalar form.
// a ax + b bx with its roundings spelled out, shared by every kernel that
// updates a series sum, so the host-driven and graph-captured flows agree bit
// for bit whatever the compiler would contract
__device__ __forceinline__ double axpby_elem(double a, double ax, double b, double bx) {
  return __fma_rn(b, bx, __dmul_rn(a, ax));
}

__global__ void k_axpby(const double *__restrict__ A, double ax, const double *__restrict__ B, double bx,
                        const double *bx_dev, double *__restrict__ C, long n) {
  if (bx_dev) bx = *bx_dev;
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long stride = (long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) C[i] = axpby_elem(A[i], ax, B[i], bx);
}

// sum of squares of one chunk, times its weight
__global__ void __launch_bounds__(256) k_norm_partial(const double *__restrict__ op, const NormChunk *chunks,
                                                      double *partials) {
  __shared__ double sh[32];
  NormChunk c = chunks[blockIdx.x];
  double s = 0.0;
  for (int i = threadIdx.x; i < c.len; i += blockDim.x) {
    double x = op[c.start + i];
    s = fma(x, x, s);
  }
  s = block_sum_ops(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s * c.weight;
}

// One Magnus or BCH series term's bookkeeping in one pass over the new term
// B: C = A + bx B (the sum), X0 = B (the next term's operand, when X0 is set)
// and B's mat_frob_norm partials, chunk by chunk in k_norm_partial's order
// (so k_final_sum gives the same norm bit for bit).  E0 (index 0) lies
// outside the norm chunks and is updated by one thread.
__global__ void __launch_bounds__(256) k_series_update(const double *A, const double *__restrict__ B,
                                                       const double *bx_dev, double *C, double *X0,
                                                       const NormChunk *chunks, double *partials) {
  __shared__ double sh[32];
  const double bx = *bx_dev;
  const NormChunk c = chunks[blockIdx.x];
  double s = 0.0;
  for (int i = threadIdx.x; i < c.len; i += blockDim.x) {
    const long k = c.start + i;
    const double x = B[k];
    C[k] = axpby_elem(A[k], 1.0, x, bx);
    if (X0) X0[k] = x;
    s = fma(x, x, s);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    C[0] = axpby_elem(A[0], 1.0, B[0], bx);
    if (X0) X0[0] = B[0];
  }
  s = block_sum_ops(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s * c.weight;
}

__global__ void __launch_bounds__(256) k_final_sum(const double *partials, int n, double *out, int take_sqrt) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partials[i];
  s = block_sum_ops(s, sh);
  if (threadIdx.x == 0) *out = take_sqrt ? sqrt(s) : s;
}

// mbpt2: one CTA per block q; partial = (2J+1) * sum Gamma_pphh^2 / eden
__global__ void __launch_bounds__(256) k_mbpt2_partial(DevTables T, const double *__restrict__ H, int herm,
                                                       double *partials) {
  __shared__ double sh[32];
  int q = blockIdx.x;
  int np = T.gam_n1[q * 6 + 2], nh = T.gam_n2[q * 6 + 2];
  long o = T.gam_off[q * 6 + 2];
  const int *qp = T.qn + T.qn_start[q * 3 + 0];
  const int *qh = T.qn + T.qn_start[q * 3 + 2];
  double s = 0.0;
  for (int k = threadIdx.x; k < np * nh; k += blockDim.x) {
    int II = k % np, JJ = k / np;
    int i = qp[2 * II], j = qp[2 * II + 1], kk = qh[2 * JJ], l = qh[2 * JJ + 1];
    double fi = f_elem(T, H, herm, i, i), fj = f_elem(T, H, herm, j, j);
    double fk = f_elem(T, H, herm, kk, kk), fl = f_elem(T, H, herm, l, l);
    double eden = fk + fl - fi - fj;
    double x = H[o + k];
    s += x * x / eden;
  }
  s = block_sum_ops(s, sh);
  if (threadIdx.x == 0) partials[q] = (T.blk_J2[q] + 1.0) * s;
}

// twobody_monopole(a, b) for every ordered orbit pair
__global__ void k_monopole(DevTables T, const double *__restrict__ H, int herm, double *mono) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.norb * T.norb) return;
  int a = t / T.norb, b = t % T.norb;
  int ja = T.orb[a].x, jb = T.orb[b].x;
  double sm = 0.0;
  for (int JT = abs(ja - jb); JT <= ja + jb; JT += 2) sm += (JT + 1) * v_elem(T, H, herm, a, b, a, b, JT);
  mono[t] = sm / (ja + 1.0) / (jb + 1.0);
}

// Element t of the White generator's support (fph elements first, then the
// pphh arrays of all blocks): its flat index, and its energy denominator
// (generators.f90:18-95) evaluated on operator X -- linear in X, with X's
// monopole table.  Returns -1 for an fph element of mismatched (l,j,tz),
// which the reference leaves at zero.
__device__ long white_den(const DevTables &T, const double *__restrict__ X, int herm, const double *__restrict__ mono,
                          long t, double *den) {
  const long nph1 = (long)T.P * T.A;
  if (t < nph1) {
    const int a = (int)(t % T.P), i = (int)(t / T.P);
    const int ak = T.part_orb[a], ik = T.hole_orb[i];
    const int4 oa = T.orb[ak], oi = T.orb[ik];
    if (!(oa.x == oi.x && oa.y == oi.y && oa.z == oi.z)) return -1;
    const int ji = oi.x;
    double Eden = 0.0;
    for (int JT = 0; JT <= 2 * ji; JT += 2) Eden = Eden - (JT + 1) * v_elem(T, X, herm, ak, ik, ak, ik, JT);
    Eden = Eden / (ji + 1.0) / (ji + 1.0);
    Eden = Eden + X[T.off_fpp + a + (long)a * T.P] - X[T.off_fhh + i + (long)i * T.A];
    *den = Eden;
    return T.off_fph + t;
  }
  t -= nph1;
  // two-body: walk the pphh arrays of all blocks
  for (int q = 0; q < T.nblocks; q++) {
    const int s = q * 6 + 2;
    const long n = (long)T.gam_n1[s] * T.gam_n2[s];
    if (t >= n) {
      t -= n;
      continue;
    }
    const int np = T.gam_n1[s];
    const int IX = (int)(t % np), JX = (int)(t / np);
    const int *qp = T.qn + T.qn_start[q * 3 + 0] + 2 * IX;
    const int *qh = T.qn + T.qn_start[q * 3 + 2] + 2 * JX;
    const int a = qp[0], b = qp[1], i = qh[0], j = qh[1];
    const int N = T.norb;
    double Eden = 0.0;
    Eden = Eden + mono[a * N + b];
    Eden = Eden + mono[i * N + j];
    Eden = Eden - mono[a * N + i];
    Eden = Eden - mono[a * N + j];
    Eden = Eden - mono[i * N + b];
    Eden = Eden - mono[j * N + b];
    Eden = Eden + f_elem(T, X, herm, a, a) + f_elem(T, X, herm, b, b) - f_elem(T, X, herm, i, i) -
           f_elem(T, X, herm, j, j);
    *den = Eden;
    return T.gam_off[s] + t;
  }
  return -2;
}

// ETA one-body (fph) and two-body (pphh) elements; everything else was zeroed.
// Denominators from Hden (and its monopoles), numerators from Hnum:
//   White (generators.f90:4-106)          eta = N / D
//   atan, atanxx (generators.f90:162-376)  eta = atan(2 N / D) * 0.5
__global__ void __launch_bounds__(256) k_generator(DevTables T, const double *__restrict__ Hden, int herm,
                                                   const double *__restrict__ mono,
                                                   const double *__restrict__ Hnum, int use_atan, double *ETA) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double den = 1.0;
  const long e = white_den(T, Hden, herm, mono, t, &den);
  if (e == -1) ETA[T.off_fph + t] = 0.0;
  else if (e >= 0) ETA[e] = use_atan ? atan(2 * Hnum[e] / den) * 0.5 : Hnum[e] / den;
}

// Tangent of the White generator along dH: eta = N / D with N and D linear in
// H, so d eta = (dN - eta dD) / D.
__global__ void __launch_bounds__(256) k_white_tangent(DevTables T, const double *__restrict__ H,
                                                       const double *__restrict__ dH, int herm,
                                                       const double *__restrict__ mono,
                                                       const double *__restrict__ dmono, double *dETA) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double den = 1.0, dden = 0.0;
  const long e = white_den(T, H, herm, mono, t, &den);
  if (e == -1) {
    dETA[T.off_fph + t] = 0.0;
  } else if (e >= 0) {
    white_den(T, dH, herm, dmono, t, &dden);
    const double eta = H[e] / den;
    dETA[e] = (dH[e] - eta * dden) / den;
  }
}

// Adjoint of the White generator (reverse mode): given ETAb, the gradient of a
// scalar with respect to ETA = White(H), add its gradient with respect to H
// into Hb.  eta = N / D with N = H[e] and D linear in H (white_den), so
// Hb[e] += etab / D and D's adjoint Db = -etab eta / D flows back through
// white_den's linear map: one-body diagonals directly, the particle-hole
// diagonals of fph denominators through their J sums, and the pphh
// denominators' six monopoles through the table monob (k_white_adjoint2 takes
// it back to the two-body diagonals).  FP64 atomics: the order of the
// additions varies, so results agree to rounding, not bit for bit.
__device__ __forceinline__ void v_scatter(const DevTables &T, double *Hb, int herm, int a, int b, int c, int d,
                                          int J2, double w) {
  const VLoc l = v_loc(T, a, b, c, d, J2);
  if (l.idx < 0) return;
  double x = dflip(w, l.neg ^ (l.trans & (herm < 0)));
  if (l.nsq) x = x * (l.nsq == 1 ? IMSRG_SQRT2 : 2.0000000000000004);
  atomicAdd(Hb + l.idx, x);
}

__device__ __forceinline__ long fdiag(const DevTables &T, int a) {
  const int pa = T.orbpos[a];
  return T.orb[a].w ? T.off_fhh + pa + (long)pa * T.A : T.off_fpp + pa + (long)pa * T.P;
}

__global__ void __launch_bounds__(256) k_white_adjoint1(DevTables T, const double *__restrict__ H, int herm,
                                                        const double *__restrict__ mono,
                                                        const double *__restrict__ etab, double *Hb,
                                                        double *monob) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double den = 1.0;
  const long e = white_den(T, H, herm, mono, t, &den);
  if (e < 0) return;
  const double gb = etab[e];
  if (gb == 0.0) return;
  const double eta = H[e] / den;
  atomicAdd(Hb + e, gb / den);
  const double db = -gb * eta / den;
  const long nph1 = (long)T.P * T.A;
  if (t < nph1) {
    const int a = (int)(t % T.P), i = (int)(t / T.P);
    const int ak = T.part_orb[a], ik = T.hole_orb[i];
    const int ji = T.orb[ik].x;
    atomicAdd(Hb + T.off_fpp + a + (long)a * T.P, db);
    atomicAdd(Hb + T.off_fhh + i + (long)i * T.A, -db);
    for (int JT = 0; JT <= 2 * ji; JT += 2)
      v_scatter(T, Hb, herm, ak, ik, ak, ik, JT, -db * (JT + 1) / (ji + 1.0) / (ji + 1.0));
    return;
  }
  // pphh element: recover its orbits as white_den walked them
  long u = t - nph1;
  for (int q = 0; q < T.nblocks; q++) {
    const int s = q * 6 + 2;
    const long n = (long)T.gam_n1[s] * T.gam_n2[s];
    if (u >= n) {
      u -= n;
      continue;
    }
    const int np = T.gam_n1[s];
    const int *qp = T.qn + T.qn_start[q * 3 + 0] + 2 * (int)(u % np);
    const int *qh = T.qn + T.qn_start[q * 3 + 2] + 2 * (int)(u / np);
    const int a = qp[0], b = qp[1], i = qh[0], j = qh[1], N = T.norb;
    atomicAdd(monob + a * N + b, db);
    atomicAdd(monob + i * N + j, db);
    atomicAdd(monob + a * N + i, -db);
    atomicAdd(monob + a * N + j, -db);
    atomicAdd(monob + i * N + b, -db);
    atomicAdd(monob + j * N + b, -db);
    atomicAdd(Hb + fdiag(T, a), db);
    atomicAdd(Hb + fdiag(T, b), db);
    atomicAdd(Hb + fdiag(T, i), -db);
    atomicAdd(Hb + fdiag(T, j), -db);
    return;
  }
}

// monopole table adjoint -> the two-body diagonals <ab|V|ab>_J (k_monopole's
// transpose)
__global__ void k_white_adjoint2(DevTables T, int herm, const double *__restrict__ monob, double *Hb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.norb * T.norb) return;
  const double mb = monob[t];
  if (mb == 0.0) return;
  const int a = t / T.norb, b = t % T.norb;
  const int ja = T.orb[a].x, jb = T.orb[b].x;
  for (int JT = abs(ja - jb); JT <= ja + jb; JT += 2)
    v_scatter(T, Hb, herm, a, b, a, b, JT, mb * (JT + 1) / (ja + 1.0) / (jb + 1.0));
}

// normal_order (basic_IMSRG.f90:2375-2506) from T (the operator before
// normal ordering) into H.  Threads [0, A*A + P*A + P*P) take one one-body
// element each (upper triangles of fhh and fpp, mirrored; fph whole):
//   f_ab + sum_{i hole} sum_J (2J+1)/(2j_a+1) <a i|V|b i>_J  for (l,j,tz)-equal a, b.
// The last CTA forms E0 = (2 sum_i (2j_i+1) f_ii + sum_{ij holes} sum_J (2J+1) <ij|V|ij>_J) / 2.
__global__ void __launch_bounds__(256) k_normal_order(DevTables T, const double *__restrict__ Tin, int herm,
                                                      double *H, int nel) {
  __shared__ double sh[8];
  const int A = T.A, P = T.P;
  if ((int)blockIdx.x == (int)gridDim.x - 1) {
    // E0: hole diagonal one-body, then hole-hole monopoles (fixed order)
    double sm = 0.0;
    for (int k = threadIdx.x; k < A * A; k += blockDim.x) {
      const int i = T.hole_orb[k % A], j = T.hole_orb[k / A];
      double v = 0.0;
      if (k % A == k / A) v += 2.0 * f_elem(T, Tin, herm, i, i) * (T.orb[i].x + 1);
      const int ji = T.orb[i].x, jj = T.orb[j].x;
      for (int JT = abs(ji - jj); JT <= ji + jj; JT += 2) v += v_elem(T, Tin, herm, i, j, i, j, JT) * (JT + 1);
      sm += v;
    }
    sm = block_sum_ops(sm, sh);
    if (threadIdx.x == 0) H[0] = sm * 0.5;
    return;
  }
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nel) return;
  int ax, bx, pass, a, b;
  if (t < A * A) {
    pass = 0;
    a = t % A;
    b = t / A;
    ax = T.hole_orb[a];
    bx = T.hole_orb[b];
  } else if (t < A * A + P * A) {
    pass = 1;
    a = (t - A * A) % P;
    b = (t - A * A) / P;
    ax = T.part_orb[a];
    bx = T.hole_orb[b];
  } else {
    pass = 2;
    a = (t - A * A - P * A) % P;
    b = (t - A * A - P * A) / P;
    ax = T.part_orb[a];
    bx = T.part_orb[b];
  }
  if (pass != 1 && b < a) return;  // mirrored from the upper triangle
  const int4 oa = T.orb[ax], ob = T.orb[bx];
  if (oa.x != ob.x || oa.y != ob.y || oa.z != ob.z) return;  // the reference leaves these untouched
  double s = 0.0;
  for (int i = 0; i < A; i++) {
    const int ix = T.hole_orb[i];
    const int ji = T.orb[ix].x;
    for (int JT = abs(ji - oa.x); JT <= ji + oa.x; JT += 2)
      s += (JT + 1.0) / (oa.x + 1) * v_elem(T, Tin, herm, ax, ix, bx, ix, JT);
  }
  const double v = f_elem(T, Tin, herm, ax, bx) + s;
  if (pass == 0) {
    H[T.off_fhh + a + (long)b * A] = v;
    H[T.off_fhh + b + (long)a * A] = v;
  } else if (pass == 1) {
    H[T.off_fph + a + (long)b * P] = v;
  } else {
    H[T.off_fpp + a + (long)b * P] = v;
    H[T.off_fpp + b + (long)a * P] = v;
  }
}

__global__ void k_pack(const double *__restrict__ flat, const long *__restrict__ src, double *packed, long n) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    packed[k] = flat[src[k]];
}

__global__ void k_unpack(const double *__restrict__ packed, const long *__restrict__ src,
                         const long *__restrict__ mirror, int herm, double *flat, long n) {
  long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double v = packed[k];
  flat[src[k]] = v;
  if (mirror[k] >= 0) flat[mirror[k]] = v * herm;
}

__global__ void k_check_finite(const double *__restrict__ op, long n, int *flag) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long stride = (long)gridDim.x * blockDim.x;
  int bad = 0;
  for (; i < n; i += stride)
    if (!isfinite(op[i])) bad = 1;
  if (__syncthreads_or(bad) && threadIdx.x == 0) *flag = 1;
}

}  // namespace

int launch_axpby(imsrg_basis *b, const double *A, double ax, const double *B, double bx, double *C) {
  long n = b->nfull;
  int grid = (int)std::min<long>((n + 255) / 256, 152 * 8);
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  k_axpby<<<grid, 256, 0, b->stream>>>(A, ax, B, bx, nullptr, C, n);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_axpby_dev(imsrg_basis *b, const double *A, double ax, const double *B, const double *bx, double *C) {
  long n = b->nfull;
  int grid = (int)std::min<long>((n + 255) / 256, 152 * 8);
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  k_axpby<<<grid, 256, 0, b->stream>>>(A, ax, B, 0.0, bx, C, n);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_series_update(imsrg_basis *b, double *S, const double *X1, const double *coef_dev, double *X0,
                         double *d_norm) {
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  k_series_update<<<b->nchunks, 256, 0, b->stream>>>(S, X1, coef_dev, S, X0, b->d_chunks, b->partials);
  b->launches++;
  if (d_norm) {
    k_final_sum<<<1, 256, 0, b->stream>>>(b->partials, b->nchunks, d_norm, 1);
    b->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int launch_norm(imsrg_basis *b, const double *op, double *d_out) {
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  k_norm_partial<<<b->nchunks, 256, 0, b->stream>>>(op, b->d_chunks, b->partials);
  k_final_sum<<<1, 256, 0, b->stream>>>(b->partials, b->nchunks, d_out, 1);
  b->launches += 2;
  return cuda_status(cudaGetLastError());
}

int launch_mbpt2(imsrg_basis *b, const double *H, int herm, double *d_out) {
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  k_mbpt2_partial<<<b->nblocks, 256, 0, b->stream>>>(b->T, H, herm, b->partials);
  k_final_sum<<<1, 256, 0, b->stream>>>(b->partials, b->nblocks, d_out, 0);
  b->launches += 2;
  return cuda_status(cudaGetLastError());
}

int launch_generator(imsrg_basis *b, const double *Hden, int hH, const double *Hnum, int use_atan, double *ETA) {
  double *mono = b->mono;
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  IMSRG_CUDA_TRY(cudaMemsetAsync(ETA + 1, 0, (b->nfull - 1) * sizeof(double), b->stream));
  int nn = b->norb * b->norb;
  k_monopole<<<(nn + 127) / 128, 128, 0, b->stream>>>(b->T, Hden, hH, mono);
  long n3 = 0;
  for (int q = 0; q < b->nblocks; q++) n3 += (long)b->gam_n1[q * 6 + 2] * b->gam_n2[q * 6 + 2];
  long n = (long)b->P * b->A + n3;
  if (n > 0)
    k_generator<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(b->T, Hden, hH, mono, Hnum, use_atan, ETA);
  b->launches += 2;
  return cuda_status(cudaGetLastError());
}

int launch_white(imsrg_basis *b, const double *H, int hH, double *ETA) {
  return launch_generator(b, H, hH, H, 0, ETA);
}

int launch_white_tangent(imsrg_basis *b, const double *H, const double *dH, int hH, double *dETA) {
  double *mono = b->mono, *dmono = b->mono + (long)b->norb * b->norb;
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  IMSRG_CUDA_TRY(cudaMemsetAsync(dETA, 0, b->nfull * sizeof(double), b->stream));
  int nn = b->norb * b->norb;
  k_monopole<<<(nn + 127) / 128, 128, 0, b->stream>>>(b->T, H, hH, mono);
  k_monopole<<<(nn + 127) / 128, 128, 0, b->stream>>>(b->T, dH, hH, dmono);
  long n3 = 0;
  for (int q = 0; q < b->nblocks; q++) n3 += (long)b->gam_n1[q * 6 + 2] * b->gam_n2[q * 6 + 2];
  long n = (long)b->P * b->A + n3;
  if (n > 0)
    k_white_tangent<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(b->T, H, dH, hH, mono, dmono, dETA);
  b->launches += 3;
  return cuda_status(cudaGetLastError());
}

int launch_white_adjoint(imsrg_basis *b, const double *H, int hH, const double *ETAb, double *Hb, double *monob) {
  double *mono = b->mono;
  const int nn = b->norb * b->norb;
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  IMSRG_CUDA_TRY(cudaMemsetAsync(monob, 0, nn * sizeof(double), b->stream));
  k_monopole<<<(nn + 127) / 128, 128, 0, b->stream>>>(b->T, H, hH, mono);
  long n3 = 0;
  for (int q = 0; q < b->nblocks; q++) n3 += (long)b->gam_n1[q * 6 + 2] * b->gam_n2[q * 6 + 2];
  const long n = (long)b->P * b->A + n3;
  if (n > 0)
    k_white_adjoint1<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(b->T, H, hH, mono, ETAb, Hb, monob);
  k_white_adjoint2<<<(nn + 127) / 128, 128, 0, b->stream>>>(b->T, hH, monob, Hb);
  b->launches += 3;
  return cuda_status(cudaGetLastError());
}

int launch_pack(imsrg_basis *b, const double *flat, double *packed, cudaStream_t st, bool to_host) {
  if (!st) st = b->stream;
  // into host memory over the link: one CTA per SM writes fastest (more CTAs
  // measured slower: 95 against 134 GB/s for 3.9 MB)
  const long grid = to_host ? b->num_sms : (b->neq + 255) / 256;
  k_pack<<<(unsigned)std::max<long>(grid, 1), 256, 0, st>>>(flat, b->d_pack_src, packed, b->neq);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_unpack(imsrg_basis *b, const double *packed, int herm, double *flat, cudaStream_t st) {
  if (!st) st = b->stream;
  k_unpack<<<(unsigned)((b->neq + 255) / 256), 256, 0, st>>>(packed, b->d_pack_src, b->d_pack_mirror, herm, flat,
                                                              b->neq);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_normal_order(imsrg_basis *b, const double *Tin, int herm, double *H) {
  const int nel = b->A * b->A + b->P * b->A + b->P * b->P;
  ProfScope ps(b, IMSRG_KERNEL_OPS);
  k_normal_order<<<(nel + 255) / 256 + 1, 256, 0, b->stream>>>(b->T, Tin, herm, H, nel);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_check_finite(imsrg_basis *b, const double *op, int *d_flag) {
  IMSRG_CUDA_TRY(cudaMemsetAsync(d_flag, 0, sizeof(int), b->stream));
  k_check_finite<<<152 * 4, 256, 0, b->stream>>>(op, b->nfull, d_flag);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

}  // namespace imsrg
