// kernels_comm.cu -- FP64 kernels of one scalar-scalar commutator [L, R].
//
// One commutator is these launches on the basis stream (4 on a side stream
// beside 3; 5 and the commutator_122 sums of 3 (k_asm2_122) on streams of
// their own from the start, beside 1 and 2):
//   1. cc_forward      Pandya transform of L and R into LCC, RCC
//                      (calculate_cross_coupled, cross_coupled.f90:1190-1300)
//   2. gemm_fp64       every dense contraction as one grouped GEMM: the 12
//                      ladder products per (2J,Tz,parity) block of
//                      commutator_222_pp_hh (commutators.f90:596-766) and the
//                      WCC = LCC RCC^T products of commutator_222_ph (:792-802)
//                      (the split-precision path replaces this launch)
//   3. ph_inputs +     every two-body element of RES in one pass: the
//      assemble_2body  one-body insertions of commutator_122 (:283-396), the
//                      antisymmetrised ladder epilogue of 222_pp_hh
//                      (:658-764) and the inverse Pandya recoupling of
//                      222_ph (:804-923); RES is written once
//   4. assemble_1body  every one-body element: commutator_111 (:36-80),
//                      121 (:83-280) and 221 (:435-578)
//   5. e0              E0 from 110 + 220 (:10-33, :399-432), which need only
//                      L and R
// No float atomics: every reduction has a fixed order, so results are
// bit-reproducible run to run.
#include "device.cuh"

namespace imsrg {

namespace {

// ---------------------------------------------------------------------------
// 1. Pandya transform: CCX(r(a,b), nb(p,h)) of cross_coupled.f90:1247-1291.
// ---------------------------------------------------------------------------
// exps != nullptr (split-precision path, ccf_packed): also the largest IEEE
// exponent of every LCC block (into exps[gL + block]) and RCC block (exps[gR +
// block]) for the digit slicing: lanes of a warp that share a block combine
// theirs, one integer atomicMax per block and warp (order-independent).
// SIDES: 1 = LCC only, 2 = RCC only, 3 = both from one pass over the gather
// list (the separate passes let the RCC half run while L is still arriving).
template <int SIDES>
__global__ void __launch_bounds__(256) k_cc_forward(DevTables T, const double *__restrict__ L, int hL,
                                                    const double *__restrict__ R, int hR, double *LCC, double *RCC,
                                                    int *exps, int gL, int gR) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int q1 = -1, xL = 0, xR = 0;
  if (t < T.cc_total) {
    const int v = T.ccf_order[t];  // elements grouped by term count
    const long e = T.ccf_packed ? (v & 0xFFFFFF) : v;
    if (T.ccf_packed) q1 = v >> 24;
    const int k0 = T.cct_start[e], k1 = T.cct_start[e + 1];
    const int nL = hL < 0, nR = hR < 0;
    double sl = 0.0, sr = 0.0;
    for (int k = k0; k < k1; k++) {
      const int ix = T.cct_idx[k];
      const int tr = (int)((unsigned)ix >> 31), idx = ix & 0x7fffffff;
      const double c = T.cct_coef[k];
      if (SIDES & 1) sl = fma(c, dflip(L[idx], tr & nL), sl);
      if (SIDES & 2) sr = fma(c, dflip(R[idx], tr & nR), sr);
    }
    if (SIDES & 1) {
      LCC[e] = sl;
      xL = (int)((__double_as_longlong(sl) >> 52) & 0x7FF);
    }
    if (SIDES & 2) {
      RCC[e] = sr;
      xR = (int)((__double_as_longlong(sr) >> 52) & 0x7FF);
    }
  }
  if (exps) {  // every lane of the warp takes part (no early exit above)
    const unsigned peers = __match_any_sync(0xffffffffu, q1);
    const int mL = __reduce_max_sync(peers, xL), mR = __reduce_max_sync(peers, xR);
    if (q1 >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1) {
      if (SIDES & 1) atomicMax(exps + gL + q1, mL);
      if (SIDES & 2) atomicMax(exps + gR + q1, mR);
    }
  }
}

// ---------------------------------------------------------------------------
// 2. Grouped FP64 GEMM: C = sum_t alpha_t op(A_t) op(B_t), one problem
//    list, tiles of 64 x 64 (4 x 4 outputs per thread: rows tx + 16 i,
//    columns 4 ty + j, so warp w owns columns 8w .. 8w + 7 and skips the
//    products when they all lie past N) or, for outputs of at most eight
//    columns, 256 x 8 (one row of eight outputs per thread; warps whose rows
//    all lie past M skip the products).  A last K chunk shorter than BK runs
//    only its valid k.
// ---------------------------------------------------------------------------
constexpr int BM = 64, BN = 64, BK = 16;
constexpr int TBM = 256, TBN = 8, TBK = 8;

template <bool ABS>
__device__ __forceinline__ void gemm_thin_tile(const GemmProb &P, int lt, const Operands &ops, int hL, int hR) {
  __shared__ double As[TBK][TBM];
  __shared__ double Bs[TBK][TBN];
  const int tid = threadIdx.x;
  const int m0 = lt * TBM;
  const bool live = m0 + (tid & ~31) < P.M;  // warp-uniform
  double acc[TBN];
#pragma unroll
  for (int j = 0; j < TBN; j++) acc[j] = 0.0;
  for (int it = 0; it < P.nterms; it++) {
    const GemmTerm &Tm = P.t[it];
    const double *A = ABS ? Tm.a_abs : ops.src[Tm.a_src] + Tm.a_off;
    const double *B = ABS ? Tm.b_abs : ops.src[Tm.b_src] + Tm.b_off;
    const double alpha = Tm.coef * (Tm.use_hl ? hL : 1) * (Tm.use_hr ? hR : 1);
    double part[TBN];
#pragma unroll
    for (int j = 0; j < TBN; j++) part[j] = 0.0;
    for (int k0 = 0; k0 < P.K; k0 += TBK) {
#pragma unroll
      for (int l = 0; l < TBK; l++) {
        const int idx = l * TBM + tid;
        int m, k;
        if (!Tm.ta) { m = idx % TBM; k = idx / TBM; }
        else { k = idx % TBK; m = idx / TBK; }
        const int gm = m0 + m, gk = k0 + k;
        double v = 0.0;
        if (gm < P.M && gk < P.K) v = Tm.ta ? A[gk + (long)gm * Tm.lda] : A[gm + (long)gk * Tm.lda];
        As[k][m] = v;
      }
      if (tid < TBK * TBN) {
        int n, k;
        if (!Tm.tb) { k = tid % TBK; n = tid / TBK; }
        else { n = tid % TBN; k = tid / TBN; }
        const int gk = k0 + k;
        double v = 0.0;
        if (n < P.N && gk < P.K) v = Tm.tb ? B[n + (long)gk * Tm.ldb] : B[gk + (long)n * Tm.ldb];
        Bs[k][n] = v;
      }
      __syncthreads();
      if (live) {
        const int kn = min(TBK, P.K - k0);
#pragma unroll
        for (int k = 0; k < TBK; k++) {
          if (k < kn) {
            const double a = As[k][tid];
#pragma unroll
            for (int j = 0; j < TBN; j++) part[j] = fma(a, Bs[k][j], part[j]);
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < TBN; j++) acc[j] += alpha * part[j];
  }
  const int gm = m0 + tid;
  if (gm >= P.M) return;
  double *Cp = ABS ? P.c_abs : ops.dst[P.c_dst] + P.c_off;
#pragma unroll
  for (int j = 0; j < TBN; j++)
    if (j < P.N) Cp[gm + (long)j * P.ldc] = acc[j];
}

// ABS: a merged list of several bases (absolute pointers, tiles of bases
// with act[inst] == 0 skipped)
template <bool ABS>
__global__ void __launch_bounds__(256) k_gemm_fp64(const GemmProb *__restrict__ probs, int nprobs, Operands ops,
                                                   int hL, int hR, const int *__restrict__ act) {
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
  if (ABS && act && !act[P.inst]) return;  // block-uniform
  int lt = tile - P.tile0;
  if (P.shape == 1) {  // block-uniform
    gemm_thin_tile<ABS>(P, lt, ops, hL, hR);
    return;
  }
  int m0 = (lt % P.tiles_m) * BM, n0 = (lt / P.tiles_m) * BN;
  int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const bool live = n0 + 8 * (tid >> 5) < P.N;  // warp-uniform: the warp's eight columns
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  for (int it = 0; it < P.nterms; it++) {
    const GemmTerm &Tm = P.t[it];
    const double *A = ABS ? Tm.a_abs : ops.src[Tm.a_src] + Tm.a_off;
    const double *B = ABS ? Tm.b_abs : ops.src[Tm.b_src] + Tm.b_off;
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
      const int kn = live ? min(BK, P.K - k0) : 0;
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
  double *Cp = ABS ? P.c_abs : ops.dst[P.c_dst] + P.c_off;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    int gn = n0 + 4 * ty + j;
    if (gn >= P.N) continue;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      int gm = m0 + tx + 16 * i;
      if (gm < P.M) Cp[gm + (long)gn * P.ldc] = acc[i][j];
    }
  }
}

// ---------------------------------------------------------------------------
// 3. Two-body assembly from the per-element gather lists (see Asm2Head).
// ---------------------------------------------------------------------------
// Cross-coupled W(r, c) of one WCC block, zero where a row is absent (not
// reached for number-conserving blocks; the guard keeps the read in bounds).
__device__ __forceinline__ double wcc_at(const double *W, int rlen, unsigned r, unsigned c) {
  if (r == 0xFFFFu || c == 0xFFFFu) return 0.0;
  return W[r + (long)c * rlen];
}

__device__ __forceinline__ long long wcc_at_int(const long long *W, int rlen, unsigned r, unsigned c) {
  if (r == 0xFFFFu || c == 0xFFFFu) return 0;
  return W[r + (long)c * rlen];
}

// Recoupling inputs Z of commutator_222_ph, one thread per PhTerm.  With
// exps == nullptr WCC holds FP64 (the FP64 path); otherwise it holds the
// split engine's exact int64 level sums, WCC = v 2^k per cross-coupled block
// (k = both block exponents - kshift, kshift = 7 x the highest level kept),
// and the four entries are combined exactly in int64 before one conversion.
__global__ void __launch_bounds__(256) k_ph_inputs(DevTables T, const double *__restrict__ WCC, int hL, int hR,
                                                   const int *__restrict__ exps, const int2 *__restrict__ ccg,
                                                   int kshift, double *__restrict__ Z) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.n_ph) return;
  const PhTerm p = T.ph_terms[t];
  const unsigned long long u = p.rows;
  const unsigned x1 = (unsigned)(u & 0xFFFF), y1 = (unsigned)((u >> 16) & 0xFFFF);
  const unsigned x2 = (unsigned)((u >> 32) & 0xFFFF), y2 = (unsigned)(u >> 48);
  const int rl = T.cc_rlen[p.qx];
  if (exps) {
    const long long *W = reinterpret_cast<const long long *>(WCC) + T.wcc_off[p.qx];
    const long long w2 = wcc_at_int(W, rl, x2, y2), w3 = wcc_at_int(W, rl, y2, x2);
    const long long a = wcc_at_int(W, rl, x1, y1) + (p.nph ? -w2 : w2);
    const long long c = (p.nph ? -w3 : w3) + wcc_at_int(W, rl, y1, x1);
    const long long z = (hL < 0 ? -a : a) - (hR < 0 ? -c : c);
    const int2 g = ccg[p.qx];
    const int k = (exps[g.x] - 1022) + (exps[g.y] - 1022) - kshift;
    // z 2^k: add k to the exponent field on the integer pipe when the result
    // stays normal (exactly ldexp's value), else ldexp
    double d = (double)z;
    unsigned long long bits = (unsigned long long)__double_as_longlong(d);
    const int E = (int)((bits >> 52) & 0x7FF);
    if (E != 0 && E + k > 0 && E + k < 2047) {
      bits += (unsigned long long)(long long)k << 52;
      d = __longlong_as_double((long long)bits);
    } else if (E != 0) {
      d = ldexp(d, k);
    }
    Z[t] = d;
    return;
  }
  const double *W = WCC + T.wcc_off[p.qx];
  const double a = wcc_at(W, rl, x1, y1) + dflip(wcc_at(W, rl, x2, y2), p.nph);
  const double c = dflip(wcc_at(W, rl, y2, x2), p.nph) + wcc_at(W, rl, y1, x1);
  Z[t] = dflip(a, hL < 0) - dflip(c, hR < 0);
}

// E0 = commutator_110 + commutator_220 (commutators.f90:10-33, 399-432) by one
// CTA of NT threads; the 220 sum arrives as the two-body kernel's per-CTA
// partials (e0p == nullptr: no 220 term).  Fixed order: strided per-thread
// sums, warp shuffles, then thread 0 adds the warp totals in index order.
// The partials were written by other CTAs, so they are read past L1.
constexpr int ENERGY_THREADS = 256;

template <int NT>
__device__ void energy_block(const DevTables &T, const double *L, int hL, const double *R, int hR, double *RES,
                             const double *e0p, int ne0p) {
  __shared__ double sh[2][NT / 32];
  const int A = T.A, P = T.P, tid = threadIdx.x;
  const double *Lph = L + T.off_fph, *Rph = R + T.off_fph;
  double v0 = 0.0, v1[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k = tid; k < P * A; k += NT) {
    int ji = T.orb[T.hole_orb[k / P]].x;
    v0 += (Lph[k] * Rph[k] * hL - Rph[k] * Lph[k] * hR) * (ji + 1);
  }
  if (e0p) {  // four independent chains, so the partials' loads overlap
    int k = tid;
    for (; k + 3 * NT < ne0p; k += 4 * NT) {
#pragma unroll
      for (int u = 0; u < 4; u++) v1[u] += __ldcg(e0p + k + u * NT);
    }
    for (; k < ne0p; k += NT) v1[0] += __ldcg(e0p + k);
  }
  v0 = warp_sum(v0);
  const double s1 = warp_sum((v1[0] + v1[1]) + (v1[2] + v1[3]));
  if ((tid & 31) == 0) {
    sh[0][tid >> 5] = v0;
    sh[1][tid >> 5] = s1;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, c = 0.0;
    for (int w = 0; w < NT / 32; w++) {
      a += sh[0][w];
      c += sh[1][w];
    }
    RES[0] = a + c * 2.0;
  }
}

// commutator_122 (commutators.f90:283-396) of one element: f_L V_R - f_R V_L
// over its leg terms (term k at tm[k * STRIDE])
template <int STRIDE>
__device__ __forceinline__ double sum122(const unsigned long long *tm, int n122, const double *L, int nL,
                                         const double *R, int nR) {
  double t = 0.0;
  for (int k = 0; k < n122; k++) {
    const unsigned long long u = tm[k * STRIDE];
    const long vi = (long)(u & 0xFFFFFFFull), fi = (long)((u >> 28) & 0xFFFFFull);
    const int sg = (int)(u >> 48) & 1, nsq = (int)(u >> 49) & 3, tr = (int)(u >> 51) & 1, ftr = (int)(u >> 52) & 1;
    double vR = dflip(R[vi], tr & nR), vL = dflip(L[vi], tr & nL);
    if (nsq) {
      const double c = nsq == 1 ? IMSRG_SQRT2 : 2.0000000000000004;
      vR = vR * c;
      vL = vL * c;
    }
    const double fL = dflip(L[fi], (ftr & nL) ^ sg), fR = dflip(R[fi], (ftr & nR) ^ sg ^ 1);
    t = fma(fL, vR, t);
    t = fma(fR, vL, t);
  }
  return t;
}

// The commutator_122 part of every two-body element (upper triangles), with
// the element's 1/sqrt(1 + delta) factors and the diagonal's sign, into RES:
// it needs only L and R, so it runs ahead of the products, and the assembly
// after them (k_assemble_2body<true>) starts from it.  One warp per 32
// elements of equal term count; term k of every lane is one coalesced load.
// The arithmetic is the assembly's own, so RES is bit-identical either way.
// (Packing the sqrt(2)-scaled (L, R) pairs first, for one 16-byte gather per
// term, measured slower here: the pack kernel took more of the shared front
// than it saved.)
__global__ void __launch_bounds__(ASM2_THREADS) k_asm2_122(DevTables T, const double *__restrict__ L, int hL,
                                                           const double *__restrict__ R, int hR, int hRES,
                                                           double *RES) {
  const int g = (int)(((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (g >= T.n_pre_warps) return;
  const unsigned pe = T.pre_el[(long)g * 32 + lane];
  if (pe >> 31) return;  // padding
  const Asm2PreWarp W = T.pre_warp[g];
  const unsigned long long *tm = T.pre_terms + W.base + lane;
  const int nL = hL < 0, nR = hR < 0;
  double t = sum122<32>(tm, W.n122, L, nL, R, nR);
  const int nd = (pe >> 28) & 3;
  if (nd) t = t * (nd == 1 ? 0.7071067811865476 : 0.5);
  if ((pe >> 30) & 1) t = dflip(t, hRES < 0);
  RES[pe & 0x0FFFFFFFu] = t;
}

// Every two-body element of RES once (upper triangles of square arrays, the
// mirror written alongside): the one-body insertions of commutator_122, the
// antisymmetrised ladder epilogue of 222_pp_hh (:658-764) and the 222_ph
// recoupling sum over J' of {6j} Z(J').  Thread t takes element w0 + t of the
// work order `heads` while below w1.  PRE: the 122 part is already in RES
// (k_asm2_122).  has220 (the allocation-free path, w0 = 0): each CTA leaves
// its commutator_220 partial in e0p for k_energy.
template <bool PRE>
__global__ void __launch_bounds__(ASM2_THREADS) k_assemble_2body(DevTables T, const double *__restrict__ L, int hL,
                                                                 const double *__restrict__ R, int hR,
                                                                 const double *__restrict__ W1,
                                                                 const double *__restrict__ W2,
                                                                 const double *__restrict__ Z, double *RES, int hRES,
                                                                 const Asm2Head *__restrict__ heads, long w0, long w1,
                                                                 int has220, double *e0p) {
  __shared__ double sh220[ASM2_THREADS / 32];
  const long w = w0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
  double e220 = 0.0;  // this element's commutator_220 term (pphh arrays only)
  if (w < w1) {
    const Asm2Head h = heads[w];
    const unsigned long long *tm = T.asm2_terms + h.start;
    const unsigned meta = h.meta;
    const int nL = hL < 0, nR = hR < 0, nres = hRES < 0, npm = (hL * hR) < 0;
    const int nd = (meta >> 18) & 3;
    const bool diag = (meta >> 20) & 1, square = (meta >> 21) & 1;
    const long e = h.e, em = h.em;
    double t;
    if (PRE) {
      t = RES[e];
    } else {
      t = sum122<1>(tm, meta & 31, L, nL, R, nR);
      // / sqrt(1 + delta_ab) / sqrt(1 + delta_cd)
      if (nd) t = t * (nd == 1 ? 0.7071067811865476 : 0.5);
      if (diag) t = dflip(t, nres);
    }
    t = t + W1[e];
    t = t - W2[e];
    if (square) t = t - dflip(W1[em] - W2[em], npm);
    if ((meta >> 15) & 1) {
      const int n_in = (meta >> 5) & 31, n_out = (meta >> 10) & 31;
      const double *z = Z + h.zs, *s1 = T.six + h.six1, *s2 = T.six + h.six2;
      double a1 = 0.0, a2 = 0.0;
      for (int k = 0; k < n_in; k++) a1 = fma(s1[k], z[k], a1);
      for (int k = 0; k < n_out; k++) a2 = fma(s2[k], z[n_in + k], a2);
      double sm = dflip(a1, (meta >> 16) & 1) + a2;
      // the reference's truncated 1/sqrt(2) literal for identical orbits
      if (nd) sm = sm * (nd == 1 ? .70710678118 : .70710678118 * .70710678118);
      t = t + sm;
    }
    if (diag) {
      RES[e] = dflip(t, nres);
    } else {
      RES[e] = t;
      if (square) RES[em] = dflip(t, nres);
    }
    // commutator_220 (commutators.f90:409-427): -(2J+1) L_pphh R_pphh herm_R
    if (has220 && ((meta >> 22) & 1)) e220 = -L[e] * R[e] * hR * (h.J2 + 1.0);
  }
  if (has220) {  // per-CTA partial in a fixed order
    e220 = warp_sum(e220);
    if ((threadIdx.x & 31) == 0) sh220[threadIdx.x >> 5] = e220;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t220 = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); k++) t220 += sh220[k];
      e0p[blockIdx.x] = t220;
    }
  }
}

// E0 for the allocation-free path: one CTA over the two-body kernel's partials.
__global__ void __launch_bounds__(ENERGY_THREADS) k_energy(DevTables T, const double *L, int hL, const double *R,
                                                           int hR, double *RES, const double *e0p, int ne0p) {
  energy_block<ENERGY_THREADS>(T, L, hL, R, hR, RES, e0p, ne0p);
}

// E0 = commutator_110 + commutator_220 (commutators.f90:10-33, 399-432)
// straight from L and R: the 220 sum needs only their pphh arrays, so E0 runs
// beside the assembly kernels instead of after them.  One CTA; warp w takes
// the (2J,Tz,pi) blocks w, w + 16, ... in turn; fixed summation order.
constexpr int E0_THREADS = 512;

__global__ void __launch_bounds__(E0_THREADS) k_e0(DevTables T, const double *__restrict__ L, int hL,
                                                   const double *__restrict__ R, int hR, double *RES, int has220) {
  __shared__ double sh[2][E0_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int A = T.A, P = T.P;
  const double *Lph = L + T.off_fph, *Rph = R + T.off_fph;
  double v0 = 0.0, c = 0.0;
  for (int k = tid; k < P * A; k += E0_THREADS) {
    const int ji = T.orb[T.hole_orb[k / P]].x;
    v0 += (Lph[k] * Rph[k] * hL - Rph[k] * Lph[k] * hR) * (ji + 1);
  }
  if (has220)
    for (int q = wid; q < T.nblocks; q += E0_THREADS / 32) {
      const int n = T.gam_n1[q * 6 + 2] * T.gam_n2[q * 6 + 2];
      const double *Lq = L + T.gam_off[q * 6 + 2], *Rq = R + T.gam_off[q * 6 + 2];
      double s = 0.0;
      for (int k = lane; k < n; k += 32) s = fma(Lq[k], Rq[k], s);
      c += (T.blk_J2[q] + 1.0) * warp_sum(s);
    }
  v0 = warp_sum(v0);
  if (lane == 0) {
    sh[0][wid] = v0;
    sh[1][wid] = c;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, cc = 0.0;
    for (int w = 0; w < E0_THREADS / 32; w++) {
      a += sh[0][w];
      cc += sh[1][w];
    }
    // 2 sum_q (2J+1) sum -L_pphh R_pphh herm_R
    RES[0] = a - 2.0 * hR * cc;
  }
}

// One-body assembly.  The (l,j,tz)-allowed upper-triangle elements carry the
// 121 and 221 gather lists (a few hundred independent terms each) and get a
// CTA of four warps; every other element only has the four commutator_111 dot
// products and gets one warp, four elements per CTA.  Each thread folds its
// partial dot products and gather sums into the element's final linear
// combination, so one reduction per element remains.
__global__ void __launch_bounds__(128) k_assemble_1body(DevTables T, const double *L, int hL, const double *R, int hR,
                                                        const double *W1, const double *W2, double *RES, int hRES) {
  __shared__ double sh[4][8];
  const int A = T.A, P = T.P;
  const double *Lhh = L + T.off_fhh, *Lph = L + T.off_fph, *Lpp = L + T.off_fpp;
  const double *Rhh = R + T.off_fhh, *Rph = R + T.off_fph, *Rpp = R + T.off_fpp;
  const int nheavy = T.n_asm1_heavy;
  const bool whole = (int)blockIdx.x < nheavy;  // block-uniform
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
  // commutator_111 (commutators.f90:36-80): four dot products
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (type == 0) {  // th1 = Lhh Rhh, th2 = Lph^T Rph
    for (int k = tid; k < A; k += nt) {
      v[0] = fma(Lhh[p + (long)k * A], Rhh[k + (long)q * A], v[0]);
      v[2] = fma(Lhh[q + (long)k * A], Rhh[k + (long)p * A], v[2]);
    }
    for (int k = tid; k < P; k += nt) {
      v[1] = fma(Lph[k + (long)p * P], Rph[k + (long)q * P], v[1]);
      v[3] = fma(Lph[k + (long)q * P], Rph[k + (long)p * P], v[3]);
    }
  } else if (type == 1) {  // Lph Rhh + Lpp Rph - Rph Lhh - Rpp Lph
    for (int k = tid; k < A; k += nt) {
      v[0] = fma(Lph[p + (long)k * P], Rhh[k + (long)q * A], v[0]);
      v[2] = fma(Rph[p + (long)k * P], Lhh[k + (long)q * A], v[2]);
    }
    for (int k = tid; k < P; k += nt) {
      v[1] = fma(Lpp[p + (long)k * P], Rph[k + (long)q * P], v[1]);
      v[3] = fma(Rpp[p + (long)k * P], Lph[k + (long)q * P], v[3]);
    }
  } else {  // tp1 = Lph Rph^T, tp2 = Lpp Rpp
    for (int k = tid; k < A; k += nt) {
      v[0] = fma(Lph[p + (long)k * P], Rph[q + (long)k * P], v[0]);
      v[2] = fma(Lph[q + (long)k * P], Rph[p + (long)k * P], v[2]);
    }
    for (int k = tid; k < P; k += nt) {
      v[1] = fma(Lpp[p + (long)k * P], Rpp[k + (long)q * P], v[1]);
      v[3] = fma(Lpp[q + (long)k * P], Rpp[k + (long)p * P], v[3]);
    }
  }
  // commutator_121 and commutator_221 sums from the gather list
  if (allowed) {
    const int st = T.obt_start[e], n = T.obt_count[e];
    const int nL = hL < 0, nR = hR < 0, npm = hL * hR > 0;
    for (int k = tid; k < n; k += nt) {
      const OneBodyTerm t = T.obt[st + k];
      const int kind = t.meta & 3;
      if (kind < 2) {
        const int tr = (t.meta >> 2) & 1, ph = t.meta >> 8;
        const double rv = dflip(R[t.idx], tr & nR) * t.coef;
        const double lv = dflip(L[t.idx], tr & nL) * t.coef;
        const double lph = Lph[ph], rph = Rph[ph];
        if (kind == 0) {  // L_ai (herm_L R) - R_ai (herm_R L) at <a p|i q>
          v[4] = fma(dflip(lph, nL), rv, v[4]);
          v[4] = fma(-dflip(rph, nR), lv, v[4]);
        } else {  // -L_ai R + R_ai L at <i p|a q>
          v[4] = fma(-lph, rv, v[4]);
          v[4] = fma(rph, lv, v[4]);
        }
      } else {
        const double *W = (t.meta & 8) ? W2 : W1;
        const double w = W[t.idx] * t.coef;
        v[5] += (kind == 3) ? dflip(w, npm) : w;  // the second 221 term enters with -herm_L herm_R
      }
    }
  }
  // the element is linear in the six sums:
  //   type 0: v0 + v1 hL - (v2 hL + v3) hR      type 1: v0 + v1 - v2 - v3
  //   type 2: v0 hR + v1 - (v2 + v3 hR) hL
  // plus (v4 + v5) / (2j_p + 1) on allowed elements, where a diagonal of fhh
  // or fpp takes v5 times herm(RES) (((t + s121) hRES + s221) hRES with hRES^2 = 1)
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
  double x = fma(c3, v[3], fma(c2, v[2], fma(c1, v[1], c0 * v[0])));
  if (allowed) {
    const double rj = 1.0 / (T.orb[pk].x + 1.0);
    const double c5 = (type != 1 && p == q) ? hRES * rj : rj;
    x = fma(c5, v[5], fma(rj, v[4], x));
  }
  x = warp_sum(x);
  if (whole) {
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][0] = x;
    __syncthreads();
    x = ((sh[0][0] + sh[1][0]) + sh[2][0]) + sh[3][0];
  }
  if (tid != 0) return;
  const long base = type == 0 ? T.off_fhh : type == 1 ? T.off_fph : T.off_fpp;
  const int ld = type == 0 ? A : P;
  RES[base + p + (long)q * ld] = x;
  if (allowed && type != 1 && p != q) RES[base + q + (long)p * ld] = x * hRES;
}

}  // namespace

int launch_cc_forward(imsrg_basis *b, const double *L, int hL, const double *R, int hR, int *exps, int gL, int gR,
                      int sides, cudaStream_t st) {
  long n = b->cc_total;
  if (n == 0) return IMSRG_OK;
  if (!st) st = b->stream;
  ProfScope ps(b, IMSRG_KERNEL_CC_FORWARD, st);
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (sides == 1)
    k_cc_forward<1><<<grid, 256, 0, st>>>(b->T, L, hL, R, hR, b->lcc, b->rcc, exps, gL, gR);
  else if (sides == 2)
    k_cc_forward<2><<<grid, 256, 0, st>>>(b->T, L, hL, R, hR, b->lcc, b->rcc, exps, gL, gR);
  else
    k_cc_forward<3><<<grid, 256, 0, st>>>(b->T, L, hL, R, hR, b->lcc, b->rcc, exps, gL, gR);
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
  k_gemm_fp64<false><<<b->ntiles, 256, 0, b->stream>>>(b->d_probs, b->nprobs, ops, hL, hR, nullptr);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int gemm_fp64_merged(imsrg_basis *const *bases, int n, const double *const *L, const double *const *R,
                     GemmProb **d_probs, int *nprobs, int *ntiles) {
  std::vector<GemmProb> all;
  int tiles = 0;
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bases[i];
    const double *src[7] = {L[i], R[i], b->w1, b->w2, b->lcc, b->rcc, b->wcc};
    double *dst[7] = {nullptr, nullptr, b->w1, b->w2, nullptr, nullptr, b->wcc};
    for (GemmProb p : b->probs) {
      for (int t = 0; t < p.nterms; t++) {
        p.t[t].a_abs = src[p.t[t].a_src] + p.t[t].a_off;
        p.t[t].b_abs = src[p.t[t].b_src] + p.t[t].b_off;
      }
      p.c_abs = dst[p.c_dst] + p.c_off;
      p.inst = i;
      p.tile0 = tiles;
      tiles += p.tiles;
      all.push_back(p);
    }
  }
  *d_probs = nullptr;
  *nprobs = (int)all.size();
  *ntiles = tiles;
  if (all.empty()) return IMSRG_OK;
  IMSRG_CUDA_TRY(cudaMalloc((void **)d_probs, all.size() * sizeof(GemmProb)));
  IMSRG_CUDA_TRY(cudaMemcpy(*d_probs, all.data(), all.size() * sizeof(GemmProb), cudaMemcpyHostToDevice));
  return IMSRG_OK;
}

int launch_gemm_fp64_merged(const GemmProb *d_probs, int nprobs, int ntiles, int hL, int hR, const int *act,
                            cudaStream_t st) {
  if (ntiles == 0) return IMSRG_OK;
  Operands ops{};
  k_gemm_fp64<true><<<ntiles, 256, 0, st>>>(d_probs, nprobs, ops, hL, hR, act);
  return cuda_status(cudaGetLastError());
}

int launch_ph_inputs(imsrg_basis *b, int hL, int hR, int precision) {
  const int *exps = nullptr;
  const int2 *ccg = nullptr;
  int kshift = 0;
  if (precision == IMSRG_PREC_OZAKI) IMSRG_TRY(ozaki_wcc_scale(b, &exps, &ccg, &kshift));
  if (b->T.n_ph > 0) {
    k_ph_inputs<<<(unsigned)((b->T.n_ph + 255) / 256), 256, 0, b->stream>>>(b->T, b->wcc, hL, hR, exps, ccg,
                                                                            kshift, b->zph);
    b->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int launch_asm2_range(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                      long w0, long w1, bool by_range) {
  const long n = w1 - w0;
  if (n > 0) {
    k_assemble_2body<true><<<(unsigned)((n + ASM2_THREADS - 1) / ASM2_THREADS), ASM2_THREADS, 0, b->stream>>>(
        b->T, L, hL, R, hR, b->w1, b->w2, b->zph, RES, hRES, by_range ? b->T.asm2_head_out : b->T.asm2_head, w0,
        w1, 0, nullptr);
    b->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int launch_asm2_122(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                    cudaStream_t st) {
  if (b->T.n_pre_warps == 0) return IMSRG_OK;
  ProfScope ps(b, IMSRG_KERNEL_ASSEMBLE_2BODY, st);
  const unsigned grid = (unsigned)(((long)b->T.n_pre_warps * 32 + ASM2_THREADS - 1) / ASM2_THREADS);
  k_asm2_122<<<grid, ASM2_THREADS, 0, st>>>(b->T, L, hL, R, hR, hRES, RES);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_e0(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, cudaStream_t st) {
  ProfScope ps(b, IMSRG_KERNEL_ASSEMBLE_1BODY, st);
  k_e0<<<1, E0_THREADS, 0, st>>>(b->T, L, hL, R, hR, RES, hL * hR == -1);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int launch_assemble_1body(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                          cudaStream_t st) {
  const int grid = b->T.n_asm1_heavy + (b->T.n_asm1_light + 3) / 4;
  if (grid == 0) return IMSRG_OK;
  ProfScope ps(b, IMSRG_KERNEL_ASSEMBLE_1BODY, st);
  k_assemble_1body<<<grid, 128, 0, st>>>(b->T, L, hL, R, hR, b->w1, b->w2, RES, hRES);
  b->launches++;
  return cuda_status(cudaGetLastError());
}


// The four FP64 launches of one commutator with caller-chosen workspace and
// stream; used by the allocation-free entry point (noalloc.cu).  Allocates
// nothing and records no profiling events.
int launch_commutator_fp64_ws(imsrg_basis *b, const Workspace &ws, const double *L, int hL, const double *R, int hR,
                              double *RES, int hRES, int with_e0, cudaStream_t st) {
  long ncc = b->cc_total;
  if (ncc > 0) {
    k_cc_forward<3><<<(unsigned)((ncc + 255) / 256), 256, 0, st>>>(b->T, L, hL, R, hR, ws.lcc, ws.rcc, nullptr, 0,
                                                                    0);
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
    k_gemm_fp64<false><<<b->ntiles, 256, 0, st>>>(b->d_probs, b->nprobs, ops, hL, hR, nullptr);
    b->launches++;
  }
  if (b->T.n_ph > 0) {
    k_ph_inputs<<<(unsigned)((b->T.n_ph + 255) / 256), 256, 0, st>>>(b->T, ws.wcc, hL, hR, nullptr, nullptr,
                                                                       0, ws.zph);
    b->launches++;
  }
  const long n2 = b->T.n_asm2;
  if (n2 > 0) {
    const int has220 = with_e0 && hL * hR == -1;
    k_assemble_2body<false><<<(unsigned)((n2 + ASM2_THREADS - 1) / ASM2_THREADS), ASM2_THREADS, 0, st>>>(
        b->T, L, hL, R, hR, ws.w1, ws.w2, ws.zph, RES, hRES, b->T.asm2_head, 0, n2, has220, ws.e0p);
    b->launches++;
  }
  const int grid1 = b->T.n_asm1_heavy + (b->T.n_asm1_light + 3) / 4;
  if (grid1 > 0) {
    k_assemble_1body<<<grid1, 128, 0, st>>>(b->T, L, hL, R, hR, ws.w1, ws.w2, RES, hRES);
    b->launches++;
  }
  if (with_e0) {
    const bool e220 = hL * hR == -1;
    k_energy<<<1, ENERGY_THREADS, 0, st>>>(b->T, L, hL, R, hR, RES, e220 ? ws.e0p : nullptr, asm2_ctas(b));
    b->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int preload_commutator_fp64_ws() {
  cudaFuncAttributes a;
  const void *fns[] = {(const void *)k_cc_forward<3>, (const void *)k_gemm_fp64<false>, (const void *)k_ph_inputs,
                       (const void *)k_assemble_2body<false>, (const void *)k_assemble_1body, (const void *)k_energy};
  for (const void *f : fns) {
    cudaError_t e = cudaFuncGetAttributes(&a, f);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return IMSRG_OK;
}

}  // namespace imsrg
