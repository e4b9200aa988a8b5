// kernels_comm.cu -- FP64 kernels of one scalar-scalar commutator [L, R].
//
// One commutator is four launches on the basis stream:
//   1. cc_forward      Pandya transform of L and R into LCC, RCC
//                      (calculate_cross_coupled, cross_coupled.f90:1190-1300)
//   2. gemm_fp64       every dense contraction as one grouped GEMM: the 12
//                      ladder products per (2J,Tz,parity) block of
//                      commutator_222_pp_hh (commutators.f90:596-766) and the
//                      WCC = LCC RCC^T products of commutator_222_ph (:792-802)
//                      (the split-precision path replaces this launch)
//   3. assemble_2body  every two-body element of RES in one pass: the
//                      one-body insertions of commutator_122 (:283-396), the
//                      antisymmetrised ladder epilogue of 222_pp_hh
//                      (:658-764) and the inverse Pandya recoupling of
//                      222_ph (:804-923); RES is written once
//   4. assemble_1body  every one-body element: commutator_111 (:36-80),
//                      121 (:83-280) and 221 (:435-578), plus E0 from
//                      110 + 220 (:10-33, :399-432)
// No float atomics: every reduction has a fixed order, so results are
// bit-reproducible run to run.
#include "device.cuh"

namespace imsrg {

namespace {

__device__ __forceinline__ int upper_bound_l(const long *a, int n, long x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// 1. Pandya transform: CCX(r(a,b), nb(p,h)) of cross_coupled.f90:1247-1291.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_cc_forward(DevTables T, const double *L, int hL, const double *R, int hR,
                                                    double *LCC, double *RCC) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * T.cc_total) return;
  int which = t >= T.cc_total;
  long e = which ? t - T.cc_total : t;
  const double *op = which ? R : L;
  int herm = which ? hR : hL;
  double *out = which ? RCC : LCC;
  int q1 = upper_bound_l(T.cc_off, T.ccblocks, e) - 1;
  // skip empty blocks that share this offset
  while (q1 + 1 < T.ccblocks && T.cc_off[q1 + 1] <= e) q1++;
  int rlen = T.cc_rlen[q1];
  long loc = e - T.cc_off[q1];
  int r = (int)(loc % rlen), nb = (int)(loc / rlen);
  int ab = T.cc_rowpair[T.cc_rowstart[q1] + r];
  int ph = T.cc_colpair[T.cc_colstart[q1] + nb];
  int a = ab >> 16, b = ab & 0xffff, p = ph >> 16, h = ph & 0xffff;
  int4 oa = T.orb[a], ob = T.orb[b], op_ = T.orb[p], oh = T.orb[h];
  int JC = T.cc_J2[q1];
  double x = 0.0;
  if (((oa.y + oh.y) & 1) == ((ob.y + op_.y) & 1) && (oa.z + oh.z) == (ob.z + op_.z)) {
    int jp = op_.x, jh = oh.x, ja = oa.x, jb = ob.x;
    int Jmin = max(abs(jp - jb), abs(ja - jh));
    int Jmax = min(jp + jb, ja + jh);
    double sm = 0.0;
    // sum_J (-1)^J (2J+1) {jp jh J'; ja jb J} V^J_{hapb}: one DFMA per J
    for (int JT = Jmin; JT <= Jmax; JT += 2)
      sm = fma(dflip(sixj_w(T, jp, jh, JC, ja, jb, JT), JT >> 1), v_elem(T, op, herm, h, a, p, b, JT), sm);
    x = dflip(sm, (jh + jb + JC) >> 1) * T.sqrt_j21[JC >> 1];
  }
  out[e] = x;
}

// ---------------------------------------------------------------------------
// 2. Grouped FP64 GEMM: C = sum_t alpha_t op(A_t) op(B_t), 64x64 tiles.
// ---------------------------------------------------------------------------
constexpr int BM = 64, BN = 64, BK = 16;

__global__ void __launch_bounds__(256) k_gemm_fp64(const GemmProb *__restrict__ probs, int nprobs, Operands ops,
                                                   int hL, int hR) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  int tile = blockIdx.x;
  // find problem: last p with tile0 <= tile
  int lo = 0, hi = nprobs;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (probs[mid].tile0 <= tile) lo = mid + 1;
    else hi = mid;
  }
  const GemmProb &P = probs[lo - 1];
  int lt = tile - P.tile0;
  int m0 = (lt % P.tiles_m) * BM, n0 = (lt / P.tiles_m) * BN;
  int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  for (int it = 0; it < P.nterms; it++) {
    const GemmTerm &Tm = P.t[it];
    const double *A = ops.src[Tm.a_src] + Tm.a_off;
    const double *B = ops.src[Tm.b_src] + Tm.b_off;
    double alpha = Tm.coef * (Tm.use_hl ? hL : 1) * (Tm.use_hr ? hR : 1);
    double part[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) part[i][j] = 0.0;
    for (int k0 = 0; k0 < P.K; k0 += BK) {
      // A tile: op(A)(m, k), m in [m0, m0+64), k in [k0, k0+16)
#pragma unroll
      for (int l = 0; l < 4; l++) {
        int m, k;
        if (!Tm.ta) { m = tid & 63; k = (tid >> 6) + 4 * l; }
        else { k = tid & 15; m = (tid >> 4) + 16 * l; }
        int gm = m0 + m, gk = k0 + k;
        double v = 0.0;
        if (gm < P.M && gk < P.K) v = Tm.ta ? A[gk + (long)gm * Tm.lda] : A[gm + (long)gk * Tm.lda];
        As[k][m] = v;
      }
      // B tile: op(B)(k, n)
#pragma unroll
      for (int l = 0; l < 4; l++) {
        int n, k;
        if (!Tm.tb) { k = tid & 15; n = (tid >> 4) + 16 * l; }
        else { n = tid & 63; k = (tid >> 6) + 4 * l; }
        int gn = n0 + n, gk = k0 + k;
        double v = 0.0;
        if (gn < P.N && gk < P.K) v = Tm.tb ? B[gn + (long)gk * Tm.ldb] : B[gk + (long)gn * Tm.ldb];
        Bs[k][n] = v;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < BK; k++) {
        double a[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; i++) a[i] = As[k][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; j++) bv[j] = Bs[k][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) part[i][j] = fma(a[i], bv[j], part[i][j]);
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
    int gn = n0 + ty + 16 * j;
    if (gn >= P.N) continue;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      int gm = m0 + tx + 16 * i;
      if (gm < P.M) Cp[gm + (long)gn * P.ldc] = acc[i][j];
    }
  }
}

// ---------------------------------------------------------------------------
// 3. Two-body assembly.
// ---------------------------------------------------------------------------
// One-body insertions of commutator_122 for element <ab|..|cd> at J2: each
// term resolves the location once and reads it from R and from L (the
// reference's v_elem / v_same pair), two DFMAs per term.
__device__ __forceinline__ double c122(const DevTables &T, const double *L, int hL, const double *R, int hR, int a,
                                       int b, int c, int d, int J2) {
  double sm = 0.0;
  int s = T.ljt_start[a], n = T.ljt_count[a];
  for (int k = 0; k < n; k++) {
    int i = T.ljt_list[s + k];
    VLoc vl = v_loc(T, i, b, c, d, J2);
    sm = fma(f_elem(T, L, hL, a, i), v_read(R, hR, vl), sm);
    sm = fma(-f_elem(T, R, hR, a, i), v_read(L, hL, vl), sm);
  }
  s = T.ljt_start[b];
  n = T.ljt_count[b];
  for (int k = 0; k < n; k++) {
    int i = T.ljt_list[s + k];
    VLoc vl = v_loc(T, a, i, c, d, J2);
    sm = fma(f_elem(T, L, hL, b, i), v_read(R, hR, vl), sm);
    sm = fma(-f_elem(T, R, hR, b, i), v_read(L, hL, vl), sm);
  }
  s = T.ljt_start[c];
  n = T.ljt_count[c];
  for (int k = 0; k < n; k++) {
    int i = T.ljt_list[s + k];
    VLoc vl = v_loc(T, a, b, i, d, J2);
    sm = fma(-f_elem(T, L, hL, i, c), v_read(R, hR, vl), sm);
    sm = fma(f_elem(T, R, hR, i, c), v_read(L, hL, vl), sm);
  }
  s = T.ljt_start[d];
  n = T.ljt_count[d];
  for (int k = 0; k < n; k++) {
    int i = T.ljt_list[s + k];
    VLoc vl = v_loc(T, a, b, c, i, J2);
    sm = fma(-f_elem(T, L, hL, i, d), v_read(R, hR, vl), sm);
    sm = fma(f_elem(T, R, hR, i, d), v_read(L, hL, vl), sm);
  }
  // / sqrt(1 + delta_ab) / sqrt(1 + delta_cd)
  int nd = (a == b) + (c == d);
  if (nd) sm = sm * (nd == 1 ? 0.7071067811865476 : 0.5);
  return sm;
}

__device__ __forceinline__ double wcc_at(const DevTables &T, const double *W, int qx, int r, int c) {
  if (r < 0 || c < 0) return 0.0;  // unreachable for number-conserving blocks; guards the gather
  return W[T.wcc_off[qx] + r + (long)c * T.cc_rlen[qx]];
}
__device__ __forceinline__ int cc_r(const DevTables &T, int q1, int i, int j) {
  return T.cc_row[((long)q1 * T.norb + i) * T.norb + j];
}

// Inverse Pandya recoupling of commutator_222_ph (commutators.f90:855-910).
// The +-1 factors (herm, phases) become sign flips of the 6j symbol, leaving
// four DFMAs per J'.  Returns false where the reference's Tz/parity 'cycle'
// would skip the update.
__device__ __forceinline__ bool c222ph(const DevTables &T, const double *W, int hL, int hR, int i, int j, int k,
                                       int l, int Jtot, double *out) {
  int4 oi = T.orb[i], oj = T.orb[j], ok = T.orb[k], ol = T.orb[l];
  int ji = oi.x, jj = oj.x, jk = ok.x, jl = ol.x;
  int JTM = T.jtm;
  int nL = hL < 0, nR = hR < 0;
  double sm = 0.0;
  int jmin = max(abs(jj - jl), abs(ji - jk));
  int jmax = min(jj + jl, ji + jk);
  int Tz = abs(oi.z - ok.z) / 2;
  if (abs(ol.z - oj.z) != Tz * 2) return false;
  int PAR = (oi.y + ok.y) & 1;
  if (((ol.y + oj.y) & 1) != PAR) return false;
  int nph = ((ji + jj + jk + jl) >> 1) & 1;
  // 'inside' terms enter with -(-1)^((jl+jk+J)/2)
  int n2 = (((jl + jk + Jtot) >> 1) + 1) & 1;
  for (int JP = jmin; JP <= jmax; JP += 2) {
    int qx = JP / 2 + Tz * (JTM + 1) + 2 * PAR * (JTM + 1);
    int rjl = cc_r(T, qx, j, l), rik = cc_r(T, qx, i, k);
    int gjl = cc_r(T, qx, l, j), gik = cc_r(T, qx, k, i);
    double s6 = sixj(T, ji, jj, Jtot, jl, jk, JP);
    double c1 = dflip(s6, n2 ^ nL), c4 = dflip(s6, n2 ^ nR ^ 1);
    sm = fma(c1, wcc_at(T, W, qx, gik, rjl), sm);
    sm = fma(dflip(c1, nph), wcc_at(T, W, qx, gjl, rik), sm);
    sm = fma(dflip(c4, nph), wcc_at(T, W, qx, rik, gjl), sm);
    sm = fma(c4, wcc_at(T, W, qx, rjl, gik), sm);
  }
  Tz = abs(oi.z - ol.z) / 2;
  if (abs(ok.z - oj.z) != Tz * 2) return false;
  PAR = (oi.y + ol.y) & 1;
  if (((ok.y + oj.y) & 1) != PAR) return false;
  jmin = max(abs(ji - jl), abs(jj - jk));
  jmax = min(ji + jl, jj + jk);
  for (int JP = jmin; JP <= jmax; JP += 2) {
    int qx = JP / 2 + Tz * (JTM + 1) + 2 * PAR * (JTM + 1);
    int ril = cc_r(T, qx, i, l), rjk = cc_r(T, qx, j, k);
    int gil = cc_r(T, qx, l, i), gjk = cc_r(T, qx, k, j);
    double s6 = sixj(T, ji, jj, Jtot, jk, jl, JP);
    double c1 = dflip(s6, nL), c4 = dflip(s6, nR ^ 1);
    sm = fma(c1, wcc_at(T, W, qx, gil, rjk), sm);
    sm = fma(dflip(c1, nph), wcc_at(T, W, qx, gjk, ril), sm);
    sm = fma(dflip(c4, nph), wcc_at(T, W, qx, ril, gjk), sm);
    sm = fma(c4, wcc_at(T, W, qx, rjk, gil), sm);
  }
  *out = sm;
  return true;
}

__global__ void __launch_bounds__(256) k_assemble_2body(DevTables T, const double *L, int hL, const double *R, int hR,
                                                        const double *W1, const double *W2, const double *WCC,
                                                        double *RES, int hRES, long off2b) {
  long e = off2b + (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= T.nfull) return;
  int s = upper_bound_l(T.gam_off, T.nblocks * 6, e) - 1;
  int q = s / 6, g = s % 6;
  int n1 = T.gam_n1[s];
  long loc = e - T.gam_off[s];
  int IX = (int)(loc % n1), JX = (int)(loc / n1);
  bool square = (g == 0 || g == 3 || g == 4);
  if (square && IX > JX) return;
  // row / column pair categories: sea1 = (1,1,1,2,3,2), sea2 = (1,2,3,2,3,3)
  const int c1tab[6] = {0, 0, 0, 1, 2, 1}, c2tab[6] = {0, 1, 2, 1, 2, 2};
  const int *qr = T.qn + T.qn_start[q * 3 + c1tab[g]] + 2 * IX;
  const int *qc = T.qn + T.qn_start[q * 3 + c2tab[g]] + 2 * JX;
  int a = qr[0], b = qr[1], c = qc[0], d = qc[1];
  int J2 = T.blk_J2[q];
  int nres = hRES < 0, npm = (hL * hR) < 0;
  double t = c122(T, L, hL, R, hR, a, b, c, d, J2);
  long em = T.gam_off[s] + JX + (long)IX * n1;  // mirror (JX, IX) of a square array
  bool diag = square && IX == JX;
  if (diag) t = dflip(t, nres);
  t = t + W1[e];
  t = t - W2[e];
  if (square) t = t - dflip(W1[em] - W2[em], npm);
  double sm;
  if (c222ph(T, WCC, hL, hR, a, b, c, d, J2, &sm)) {
    // the reference's truncated 1/sqrt(2) literal for identical orbits
    int nd = (a == b) + (c == d);
    if (nd) sm = sm * (nd == 1 ? .70710678118 : .70710678118 * .70710678118);
    t = t + sm;
  }
  if (diag) {
    RES[e] = dflip(t, nres);
  } else {
    RES[e] = t;
    if (square) RES[em] = dflip(t, nres);
  }
}

// ---------------------------------------------------------------------------
// 4. One-body assembly (one warp per element) and E0 (last CTA).
// ---------------------------------------------------------------------------
// inner (a,i) sum of commutator_121 (commutators.f90:117-150) for orbits pk,qk
__device__ double c121_warp(const DevTables &T, const double *L, int hL, const double *R, int hR, int pk, int qk,
                            int lane) {
  int jq = T.orb[qk].x;
  double sm = 0.0;
  for (int k = lane; k < T.n_ph_pairs; k += 32) {
    int a = T.ph_pairs[2 * k], i = T.ph_pairs[2 * k + 1];
    int ak = T.part_orb[a], ik = T.hole_orb[i];
    int ji = T.orb[ik].x;
    double smx = 0, smy = 0, smx2 = 0, smy2 = 0;
    for (int JT = abs(ji - jq); JT <= ji + jq; JT += 2) {
      VLoc v1 = v_loc(T, ak, pk, ik, qk, JT);
      smx += v_read(R, hR, v1) * (JT + 1);
      smx2 += v_read(L, hL, v1) * (JT + 1);
      VLoc v2 = v_loc(T, ik, pk, ak, qk, JT);
      smy += v_read(R, hR, v2) * (JT + 1);
      smy2 += v_read(L, hL, v2) * (JT + 1);
    }
    double lph = L[T.off_fph + a + (long)i * T.P], rph = R[T.off_fph + a + (long)i * T.P];
    sm += lph * (hL * smx - smy) - rph * (hR * smx2 - smy2);
  }
  return warp_sum(sm);
}

// sum of commutator_221 (commutators.f90:470-486) for orbits ik, jk
__device__ double c221_warp(const DevTables &T, const double *W1, const double *W2, int pm, int ik, int jk,
                            bool with_pm, int lane) {
  int ji = T.orb[ik].x;
  double sm = 0.0;
  for (int c = lane; c < T.norb; c += 32) {
    int jc = T.orb[c].x;
    const double *W = T.orb[c].w ? W1 : W2;
    for (int JT = abs(jc - ji); JT <= jc + ji; JT += 2) {
      double v = v_elem(T, W, 1, c, ik, c, jk, JT);
      if (with_pm) v = v - pm * v_elem(T, W, 1, c, jk, c, ik, JT);
      sm += v * (JT + 1);
    }
  }
  return warp_sum(sm);
}

__device__ double dot_warp(const double *x, long sx, const double *y, long sy, int n, int lane) {
  double s = 0.0;
  for (int k = lane; k < n; k += 32) s = fma(x[k * sx], y[k * sy], s);
  return warp_sum(s);
}

__device__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(256) k_assemble_1body(DevTables T, const double *L, int hL, const double *R, int hR,
                                                        const double *W1, const double *W2, double *RES, int hRES,
                                                        int with_e0, int n_elem_blocks) {
  __shared__ double sh[32];
  int A = T.A, P = T.P;
  const double *Lhh = L + T.off_fhh, *Lph = L + T.off_fph, *Lpp = L + T.off_fpp;
  const double *Rhh = R + T.off_fhh, *Rph = R + T.off_fph, *Rpp = R + T.off_fpp;
  if ((int)blockIdx.x == n_elem_blocks) {
    if (!with_e0) return;
    // E0 = commutator_110 + commutator_220
    double s110 = 0.0;
    for (int k = threadIdx.x; k < P * A; k += blockDim.x) {
      int ji = T.orb[T.hole_orb[k / P]].x;
      s110 += (Lph[k] * Rph[k] * hL - Rph[k] * Lph[k] * hR) * (ji + 1);
    }
    double e110 = block_sum(s110, sh);
    double s220 = 0.0;
    if (hL * hR == -1) {
      for (int q = 0; q < T.nblocks; q++) {
        long o = T.gam_off[q * 6 + 2];
        int n = T.gam_n1[q * 6 + 2] * T.gam_n2[q * 6 + 2];
        double w = T.blk_J2[q] + 1;
        for (int k = threadIdx.x; k < n; k += blockDim.x) s220 -= L[o + k] * R[o + k] * hR * w;
      }
    }
    double e220 = block_sum(s220, sh) * 2.0;
    if (threadIdx.x == 0) RES[0] = e110 + e220;
    return;
  }
  int lane = threadIdx.x & 31;
  long e = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  long nA2 = (long)A * A, nPA = (long)P * A, nP2 = (long)P * P;
  if (e >= nA2 + nPA + nP2) return;
  const int *hole_orb = T.hole_orb, *part_orb = T.part_orb;
  if (e < nA2) {
    int p = (int)(e % A), q = (int)(e / A);
    int pk = hole_orb[p], qk = hole_orb[q];
    bool allowed = T.orb[pk].x == T.orb[qk].x && T.orb[pk].y == T.orb[qk].y && T.orb[pk].z == T.orb[qk].z;
    if (allowed && p > q) return;
    // th1 = Lhh Rhh, th2 = Lph^T Rph (commutators.f90:56-59)
    double th1pq = dot_warp(Lhh + p, A, Rhh + (long)q * A, 1, A, lane);
    double th2pq = dot_warp(Lph + (long)p * P, 1, Rph + (long)q * P, 1, P, lane);
    double th1qp = dot_warp(Lhh + q, A, Rhh + (long)p * A, 1, A, lane);
    double th2qp = dot_warp(Lph + (long)q * P, 1, Rph + (long)p * P, 1, P, lane);
    double t = th1pq + th2pq * hL - (th1qp * hL + th2qp) * hR;
    if (allowed) {
      double s121 = c121_warp(T, L, hL, R, hR, pk, qk, lane) / (T.orb[pk].x + 1.0);
      double s221 = c221_warp(T, W1, W2, hL * hR, pk, qk, true, lane) / (T.orb[pk].x + 1.0);
      if (p == q) t = ((t + s121) * hRES + s221) * hRES;
      else t = (t + s121) + s221;
    }
    if (lane == 0) {
      RES[T.off_fhh + p + (long)q * A] = t;
      if (allowed && p != q) RES[T.off_fhh + q + (long)p * A] = t * hRES;
    }
  } else if (e < nA2 + nPA) {
    long e2 = e - nA2;
    int p = (int)(e2 % P), q = (int)(e2 / P);
    int pk = part_orb[p], qk = hole_orb[q];
    bool allowed = T.orb[pk].x == T.orb[qk].x && T.orb[pk].y == T.orb[qk].y && T.orb[pk].z == T.orb[qk].z;
    // RES%fph = (Lph Rhh + Lpp Rph) - Rph Lhh - Rpp Lph (commutators.f90:63-71)
    double tb1 = dot_warp(Lph + p, P, Rhh + (long)q * A, 1, A, lane);
    double tb2 = dot_warp(Lpp + p, P, Rph + (long)q * P, 1, P, lane);
    double tb1b = dot_warp(Rph + p, P, Lhh + (long)q * A, 1, A, lane);
    double tb2b = dot_warp(Rpp + p, P, Lph + (long)q * P, 1, P, lane);
    double t = tb1 + tb2;
    t = t - tb1b - tb2b;
    if (allowed) {
      double s121 = c121_warp(T, L, hL, R, hR, pk, qk, lane) / (T.orb[pk].x + 1.0);
      double s221 = c221_warp(T, W1, W2, hL * hR, pk, qk, false, lane) / (T.orb[pk].x + 1.0);
      t = (t + s121) + s221;
    }
    if (lane == 0) RES[T.off_fph + p + (long)q * P] = t;
  } else {
    long e3 = e - nA2 - nPA;
    int p = (int)(e3 % P), q = (int)(e3 / P);
    int pk = part_orb[p], qk = part_orb[q];
    bool allowed = T.orb[pk].x == T.orb[qk].x && T.orb[pk].y == T.orb[qk].y && T.orb[pk].z == T.orb[qk].z;
    if (allowed && p > q) return;
    // tp1 = Lph Rph^T, tp2 = Lpp Rpp (commutators.f90:75-78)
    double tp1pq = dot_warp(Lph + p, P, Rph + q, P, A, lane);
    double tp2pq = dot_warp(Lpp + p, P, Rpp + (long)q * P, 1, P, lane);
    double tp1qp = dot_warp(Lph + q, P, Rph + p, P, A, lane);
    double tp2qp = dot_warp(Lpp + q, P, Rpp + (long)p * P, 1, P, lane);
    double t = tp1pq * hR + tp2pq - (tp1qp + tp2qp * hR) * hL;
    if (allowed) {
      double s121 = c121_warp(T, L, hL, R, hR, pk, qk, lane) / (T.orb[pk].x + 1.0);
      double s221 = c221_warp(T, W1, W2, hL * hR, pk, qk, true, lane) / (T.orb[pk].x + 1.0);
      if (p == q) t = ((t + s121) * hRES + s221) * hRES;
      else t = (t + s121) + s221;
    }
    if (lane == 0) {
      RES[T.off_fpp + p + (long)q * P] = t;
      if (allowed && p != q) RES[T.off_fpp + q + (long)p * P] = t * hRES;
    }
  }
}

}  // namespace

int launch_cc_forward(imsrg_basis *b, const double *L, int hL, const double *R, int hR) {
  long n = 2 * b->cc_total;
  if (n == 0) return IMSRG_OK;
  ProfScope ps(b, IMSRG_KERNEL_CC_FORWARD);
  k_cc_forward<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(b->T, L, hL, R, hR, b->lcc, b->rcc);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_gemm_fp64(imsrg_basis *b, const double *L, int hL, const double *R, int hR) {
  if (b->ntiles == 0) return IMSRG_OK;
  Operands ops{};
  ops.src[SRC_L] = L;
  ops.src[SRC_R] = R;
  ops.src[SRC_W1] = b->w1;
  ops.src[SRC_W2] = b->w2;
  ops.src[SRC_LCC] = b->lcc;
  ops.src[SRC_RCC] = b->rcc;
  ops.src[SRC_WCC] = b->wcc;
  ops.dst[SRC_W1] = b->w1;
  ops.dst[SRC_W2] = b->w2;
  ops.dst[SRC_WCC] = b->wcc;
  ProfScope ps(b, IMSRG_KERNEL_GEMM_FP64);
  k_gemm_fp64<<<b->ntiles, 256, 0, b->stream>>>(b->d_probs, b->nprobs, ops, hL, hR);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_assemble_2body(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES) {
  long off2b = b->off_fpp + (long)b->P * b->P;
  long n = b->nfull - off2b;
  if (n <= 0) return IMSRG_OK;
  ProfScope ps(b, IMSRG_KERNEL_ASSEMBLE_2BODY);
  k_assemble_2body<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(b->T, L, hL, R, hR, b->w1, b->w2, b->wcc, RES,
                                                                      hRES, off2b);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_assemble_1body(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                          int with_e0) {
  long nel = (long)b->A * b->A + (long)b->P * b->A + (long)b->P * b->P;
  int nblk = (int)((nel + 7) / 8);
  ProfScope ps(b, IMSRG_KERNEL_ASSEMBLE_1BODY);
  k_assemble_1body<<<nblk + 1, 256, 0, b->stream>>>(b->T, L, hL, R, hR, b->w1, b->w2, RES, hRES, with_e0, nblk);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

// The four FP64 launches of one commutator with caller-chosen workspace and
// stream; used by the allocation-free entry point (noalloc.cu).  Allocates
// nothing and records no profiling events.
int launch_commutator_fp64_ws(imsrg_basis *b, const Workspace &ws, const double *L, int hL, const double *R, int hR,
                              double *RES, int hRES, int with_e0, cudaStream_t st) {
  long ncc = 2 * b->cc_total;
  if (ncc > 0) {
    k_cc_forward<<<(unsigned)((ncc + 255) / 256), 256, 0, st>>>(b->T, L, hL, R, hR, ws.lcc, ws.rcc);
    b->launches++;
  }
  if (b->ntiles > 0) {
    Operands ops{};
    ops.src[SRC_L] = L;
    ops.src[SRC_R] = R;
    ops.src[SRC_W1] = ws.w1;
    ops.src[SRC_W2] = ws.w2;
    ops.src[SRC_LCC] = ws.lcc;
    ops.src[SRC_RCC] = ws.rcc;
    ops.src[SRC_WCC] = ws.wcc;
    ops.dst[SRC_W1] = ws.w1;
    ops.dst[SRC_W2] = ws.w2;
    ops.dst[SRC_WCC] = ws.wcc;
    k_gemm_fp64<<<b->ntiles, 256, 0, st>>>(b->d_probs, b->nprobs, ops, hL, hR);
    b->launches++;
  }
  long off2b = b->off_fpp + (long)b->P * b->P;
  long n2 = b->nfull - off2b;
  if (n2 > 0) {
    k_assemble_2body<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(b->T, L, hL, R, hR, ws.w1, ws.w2, ws.wcc, RES,
                                                                   hRES, off2b);
    b->launches++;
  }
  long nel = (long)b->A * b->A + (long)b->P * b->A + (long)b->P * b->P;
  int nblk = (int)((nel + 7) / 8);
  k_assemble_1body<<<nblk + 1, 256, 0, st>>>(b->T, L, hL, R, hR, ws.w1, ws.w2, RES, hRES, with_e0, nblk);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

}  // namespace imsrg
