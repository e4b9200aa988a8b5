// ozaki.cu -- split-precision (Ozaki-style) contraction engine on tcgen05.
//
// Replaces the FP64 grouped GEMM of one commutator (the twelve ladder products
// per (2J,Tz,parity) block of commutator_222_pp_hh, commutators.f90:596-766,
// and WCC = LCC RCC^T of commutator_222_ph, :792-802) with BF16 tensor-core
// products whose FP32 accumulations are exact integers:
//
//   1. k_oz_exponents: one power-of-two scale per block: e with |x| < 2^e for
//      every element of the block (all six arrays of a (2J,Tz,parity) block of
//      L or R; one cross-coupled block of LCC or RCC).  Every product term of
//      a block multiplies one L array by one R array of that block, so all
//      terms of a problem share the scale 2^(eL + eR).
//   2. k_oz_slice: x = 2^(e-42) * sum_{s=1..6} d_s 128^(6-s) with signed
//      base-128 digits (|d_1| <= 128, |d_s| <= 64), extracted with integer
//      operations only, written as BF16 (exact) into "images" laid out in the
//      tcgen05 K-major canonical layout (8 x 16-byte core matrices, no
//      swizzle), once with the second index contiguous (R image) and once with
//      the first (C image), so every transposition of every use is K-major.
//   3. k_oz_mma: persistent kernel, one 128 x 64 output tile at a time.  A
//      producer thread streams the six A and six B digit planes of each
//      K = 16 step into shared memory with cp.async.bulk; one thread issues
//      the 21 tcgen05.mma products d_s x d_t with s + t <= 7 into six FP32
//      accumulators in TMEM (one per level l = s + t), negating A for terms
//      with coefficient -1; four epilogue warps read the levels back
//      (tcgen05.ld), combine them exactly in int64 and write FP64.
//
// Exactness: level l sums at most 2 terms x K products bounded by
// 2^12 (l + 1), so every FP32 accumulator holds an exact integer below 2^24
// while 2 K (l + 1) 2^12 < 2^24 (checked per problem when the plan is built).
// The result differs from the exact product only by the dropped levels
// (s + t >= 8) and the digit rounding: about 2^-42 K max|A| max|B|.
//
// Every mbarrier wait is bounded (about 2 s of %globaltimer); a timeout sets
// an error flag that the host reports as IMSRG_ERR_TIMEOUT.
#include <cuda_bf16.h>

#include <algorithm>
#include <map>

#include "device.cuh"

namespace imsrg {

namespace {

constexpr int OZ_S = 6;                      // digits (slices) per operand
constexpr int OZ_LMAX = OZ_S + 1;            // highest level kept
constexpr int OZ_NLEV = OZ_LMAX - 1;         // levels 2 .. 7
constexpr int TM = 128, TN = 64, TK = 16;
constexpr int STAGES = 4;
constexpr int A_SLICE_BYTES = TM * TK * 2;   // 4096
constexpr int B_SLICE_BYTES = TN * TK * 2;   // 2048
constexpr int STAGE_BYTES = OZ_S * (A_SLICE_BYTES + B_SLICE_BYTES);
constexpr int TMEM_COLS = 512;
constexpr int OZ_THREADS = 192;              // warp 0 producer, 1 MMA, 2-5 epilogue
constexpr unsigned long long WAIT_NS = 2000000000ull;

struct OzMatrix {
  int src;         // 0 L, 1 R, 2 LCC, 3 RCC
  int group;       // exponent group
  long off;        // element offset in the source buffer
  int n1, n2;      // column-major shape
  long img_r;      // byte offset of the R image (rows n1, K = n2) in the source's image buffer
  long img_c;      // byte offset of the C image (rows n2, K = n1)
  int rg_r, rg_c;  // row groups (of 8) of each image, padded to 16
  long plane_r, plane_c;  // bytes per digit plane
  int tile0;       // first 8x8 core tile of this matrix in the slicing grid
};

struct OzGroup {
  int src;
  long off, len;
};

struct OzTerm {
  const uint8_t *a_img, *b_img;
  long a_plane, b_plane;
  int a_rg, b_rg;
  int neg, use_hl, use_hr;
};

struct OzProb {
  int M, N, K, ksteps, nterms;
  OzTerm t[2];
  double *C;
  int ldc;
  int gA, gB;
  int tiles_m, tile0, tiles;
};

struct OzPlan {
  std::vector<OzMatrix> mats;
  std::vector<OzGroup> groups;
  std::vector<OzProb> probs;
  OzMatrix *d_mats = nullptr;
  OzGroup *d_groups = nullptr;
  OzProb *d_probs = nullptr;
  int *d_exps = nullptr;
  int *d_err = nullptr;
  uint8_t *img[4] = {nullptr, nullptr, nullptr, nullptr};
  long img_bytes[4] = {0, 0, 0, 0};
  int nmats = 0, ngroups = 0, nprobs = 0, ntiles = 0, ncore = 0;
  int grid = 0;
  bool ok = false;
};

// ---------------------------------------------------------------------------
// PTX helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Waits for the phase of the given parity to complete; gives up after WAIT_NS
// or when another role has aborted.  Returns true on success.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
  uint32_t addr = smem_u32(bar);
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255) == 0) {
      if (*abort_flag) return false;
      unsigned long long t = gtimer();
      if (it == 0) t0 = t;
      else if (t - t0 > WAIT_NS) return false;
    }
  }
}

__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(sdst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D F32, A and B BF16, both K-major.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N, int negA) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)negA << 13) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---------------------------------------------------------------------------
// 1. block exponents
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_oz_exponents(const OzGroup *groups, const double *L, const double *R,
                                                      const double *LCC, const double *RCC, int *exps) {
  __shared__ int sh[8];
  OzGroup g = groups[blockIdx.x];
  const double *src = g.src == 0 ? L : g.src == 1 ? R : g.src == 2 ? LCC : RCC;
  int m = 0;
  for (long i = threadIdx.x; i < g.len; i += blockDim.x) {
    int E = (int)((__double_as_longlong(src[g.off + i]) >> 52) & 0x7FF);
    m = max(m, E);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = max(m, sh[w]);
    exps[blockIdx.x] = m - 1022;  // |x| < 2^(E - 1022) for biased exponent E
  }
}

// ---------------------------------------------------------------------------
// 2. digit slicing, one 8 x 8 core tile per thread
// ---------------------------------------------------------------------------
__device__ __forceinline__ void digits6(double x, int e, int *d) {
  unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  int E = (int)((bits >> 52) & 0x7FF);
  int neg = (int)(bits >> 63);
  unsigned long long V = 0;
  if (E != 0) {
    unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    int rs = e + 1033 - E;  // V = round(|x| 2^(42 - e)), rs >= 11
    if (rs <= 63) V = (mant + (1ull << (rs - 1))) >> rs;
  }
#pragma unroll
  for (int s = OZ_S - 1; s >= 1; s--) {
    int u = (int)(V & 127);
    V >>= 7;
    if (u >= 64) {
      u -= 128;
      V += 1;
    }
    d[s] = neg ? -u : u;
  }
  d[0] = neg ? -(int)V : (int)V;
}

__device__ __forceinline__ uint16_t bf16_bits(int v) {
  __nv_bfloat16 h = __float2bfloat16_rn((float)v);
  return *reinterpret_cast<uint16_t *>(&h);
}

__global__ void __launch_bounds__(256) k_oz_slice(const OzMatrix *mats, int nmats, int ncore, const double *L,
                                                  const double *R, const double *LCC, const double *RCC,
                                                  const int *exps, uint8_t *imgL, uint8_t *imgR, uint8_t *imgLCC,
                                                  uint8_t *imgRCC) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncore) return;
  int lo = 0, hi = nmats;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (mats[mid].tile0 <= t) lo = mid + 1;
    else hi = mid;
  }
  const OzMatrix &m = mats[lo - 1];
  int lt = t - m.tile0;
  int RG = (m.n1 + 7) / 8;
  int rg = lt % RG, cg = lt / RG;
  const double *src = (m.src == 0 ? L : m.src == 1 ? R : m.src == 2 ? LCC : RCC) + m.off;
  uint8_t *img = m.src == 0 ? imgL : m.src == 1 ? imgR : m.src == 2 ? imgLCC : imgRCC;
  int e = exps[m.group];
  int r0 = rg * 8, c0 = cg * 8;
  // R image: core matrix (rg, cg) holds rows r0.., cols c0.. with columns contiguous
  long offR = m.img_r + ((long)((cg >> 1) * m.rg_r + rg) * 2 + (cg & 1)) * 128;
  // C image: core matrix (cg, rg) holds the transpose
  long offC = m.img_c + ((long)((rg >> 1) * m.rg_c + cg) * 2 + (rg & 1)) * 128;
  // pass 1, by columns of the tile: rows of the C image
  for (int j = 0; j < 8; j++) {
    uint16_t row[OZ_S][8];
    int c = c0 + j;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      int r = r0 + i;
      double x = (r < m.n1 && c < m.n2) ? src[r + (long)c * m.n1] : 0.0;
      int d[OZ_S];
      digits6(x, e, d);
#pragma unroll
      for (int s = 0; s < OZ_S; s++) row[s][i] = bf16_bits(d[s]);
    }
#pragma unroll
    for (int s = 0; s < OZ_S; s++) {
      uint4 v;
      v.x = row[s][0] | ((uint32_t)row[s][1] << 16);
      v.y = row[s][2] | ((uint32_t)row[s][3] << 16);
      v.z = row[s][4] | ((uint32_t)row[s][5] << 16);
      v.w = row[s][6] | ((uint32_t)row[s][7] << 16);
      *reinterpret_cast<uint4 *>(img + offC + s * m.plane_c + j * 16) = v;
    }
  }
  // pass 2, by rows of the tile: rows of the R image
  for (int i = 0; i < 8; i++) {
    uint16_t row[OZ_S][8];
    int r = r0 + i;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      int c = c0 + j;
      double x = (r < m.n1 && c < m.n2) ? src[r + (long)c * m.n1] : 0.0;
      int d[OZ_S];
      digits6(x, e, d);
#pragma unroll
      for (int s = 0; s < OZ_S; s++) row[s][j] = bf16_bits(d[s]);
    }
#pragma unroll
    for (int s = 0; s < OZ_S; s++) {
      uint4 v;
      v.x = row[s][0] | ((uint32_t)row[s][1] << 16);
      v.y = row[s][2] | ((uint32_t)row[s][3] << 16);
      v.z = row[s][4] | ((uint32_t)row[s][5] << 16);
      v.w = row[s][6] | ((uint32_t)row[s][7] << 16);
      *reinterpret_cast<uint4 *>(img + offR + s * m.plane_r + i * 16) = v;
    }
  }
}

// ---------------------------------------------------------------------------
// 3. tensor-core products and exact recombination
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_prob(const OzProb *probs, int nprobs, int tile) {
  int lo = 0, hi = nprobs;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (probs[mid].tile0 <= tile) lo = mid + 1;
    else hi = mid;
  }
  return lo - 1;
}

__global__ void __launch_bounds__(OZ_THREADS, 1) k_oz_mma(const OzProb *__restrict__ probs, int nprobs, int ntiles,
                                                          const int *__restrict__ exps, int hL, int hR, int *err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + STAGES * STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *acc_full = empty + STAGES;
  uint64_t *acc_empty = acc_full + 1;
  uint32_t *tmem_slot = (uint32_t *)(acc_empty + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 4);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // producer: digit planes of A and B for every K step
      int stage = 0;
      uint32_t phase = 0;
      for (int tile = blockIdx.x; tile < ntiles && !*abort_flag; tile += gridDim.x) {
        const OzProb &P = probs[find_prob(probs, nprobs, tile)];
        if (P.ksteps == 0) continue;
        int lt = tile - P.tile0;
        int tm = lt % P.tiles_m, tn = lt / P.tiles_m;
        for (int it = 0; it < P.nterms; it++) {
          const OzTerm &T = P.t[it];
          for (int kk = 0; kk < P.ksteps; kk++) {
            if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
              atomicExch(err, 1);
              *abort_flag = 1;
              break;
            }
            mbar_expect_tx(&full[stage], STAGE_BYTES);
            uint8_t *sa = smem + stage * STAGE_BYTES;
            uint8_t *sb = sa + OZ_S * A_SLICE_BYTES;
            const uint8_t *ga = T.a_img + ((long)kk * T.a_rg + tm * 16) * 256;
            const uint8_t *gb = T.b_img + ((long)kk * T.b_rg + tn * 8) * 256;
#pragma unroll
            for (int s = 0; s < OZ_S; s++) {
              bulk_g2s(sa + s * A_SLICE_BYTES, ga + s * T.a_plane, A_SLICE_BYTES, &full[stage]);
              bulk_g2s(sb + s * B_SLICE_BYTES, gb + s * T.b_plane, B_SLICE_BYTES, &full[stage]);
            }
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (*abort_flag) break;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      int stage = 0;
      uint32_t phase = 0, aphase = 0;
      for (int tile = blockIdx.x; tile < ntiles && !*abort_flag; tile += gridDim.x) {
        const OzProb &P = probs[find_prob(probs, nprobs, tile)];
        if (P.ksteps == 0) continue;
        if (!mbar_wait(acc_empty, aphase ^ 1, abort_flag)) {
          atomicExch(err, 2);
          *abort_flag = 1;
          break;
        }
        aphase ^= 1;
        tc_fence_after();
        uint32_t started = 0;
        for (int it = 0; it < P.nterms && !*abort_flag; it++) {
          const OzTerm &T = P.t[it];
          int neg = T.neg ^ (T.use_hl & (hL < 0)) ^ (T.use_hr & (hR < 0));
          uint32_t idesc = idesc_bf16(TM, TN, neg);
          for (int kk = 0; kk < P.ksteps; kk++) {
            if (!mbar_wait(&full[stage], phase, abort_flag)) {
              atomicExch(err, 3);
              *abort_flag = 1;
              break;
            }
            tc_fence_after();
            uint32_t sa = smem_u32(smem + stage * STAGE_BYTES);
            uint32_t sb = sa + OZ_S * A_SLICE_BYTES;
#pragma unroll
            for (int s = 0; s < OZ_S; s++) {
#pragma unroll
              for (int u = 0; u < OZ_S; u++) {
                int lvl = s + u + 2;  // digits are 1-based in the level count
                if (lvl > OZ_LMAX) continue;
                uint64_t ad = smem_desc(sa + s * A_SLICE_BYTES, 128, 256);
                uint64_t bd = smem_desc(sb + u * B_SLICE_BYTES, 128, 256);
                int acc = (started >> lvl) & 1;
                started |= 1u << lvl;
                mma_bf16(tmem + (uint32_t)((lvl - 2) * TN), ad, bd, idesc, acc);
              }
            }
            mma_commit(&empty[stage]);
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
        mma_commit(acc_full);
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lane quadrant = warp % 4
    int quad = warp & 3;
    int row = quad * 32 + lane;
    uint32_t aphase = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      const OzProb &P = probs[find_prob(probs, nprobs, tile)];
      int lt = tile - P.tile0;
      int m = (lt % P.tiles_m) * TM + row;
      int n0 = (lt / P.tiles_m) * TN;
      if (P.ksteps == 0) {
        if (m < P.M)
          for (int c = 0; c < TN && n0 + c < P.N; c++) P.C[m + (long)(n0 + c) * P.ldc] = 0.0;
        continue;
      }
      if (*abort_flag) break;
      if (!mbar_wait(acc_full, aphase, abort_flag)) {
        atomicExch(err, 4);
        *abort_flag = 1;
        break;
      }
      aphase ^= 1;
      tc_fence_after();
      int k = exps[P.gA] + exps[P.gB] - 7 * OZ_LMAX;  // result = v * 2^k
      for (int cc = 0; cc < TN; cc += 16) {
        uint32_t acc[OZ_NLEV][16];
#pragma unroll
        for (int l = 0; l < OZ_NLEV; l++)
          tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(l * TN + cc), acc[l]);
        tmem_ld_wait();
#pragma unroll
        for (int c = 0; c < 16; c++) {
          long long v = 0;
#pragma unroll
          for (int l = 0; l < OZ_NLEV; l++) {
            long long cl = (long long)__float2int_rn(__uint_as_float(acc[l][c]));
            v += cl << (7 * (OZ_LMAX - 2 - l));
          }
          double d = (double)v;
          // scale by 2^k: add k to the exponent field on the integer pipe
          unsigned long long bits = (unsigned long long)__double_as_longlong(d);
          int E = (int)((bits >> 52) & 0x7FF);
          if (E != 0 && E + k > 0 && E + k < 2047) {
            bits += (unsigned long long)(long long)k << 52;
            d = __longlong_as_double((long long)bits);
          } else if (E != 0) {
            d = ldexp(d, k);
          }
          int n = n0 + cc + c;
          if (m < P.M && n < P.N) P.C[m + (long)n * P.ldc] = d;
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

OzPlan *plan_of(imsrg_basis *b) { return (OzPlan *)b->ozaki; }

}  // namespace

int ozaki_prepare(imsrg_basis *b) {
  if (b->ozaki) return plan_of(b)->ok ? IMSRG_OK : IMSRG_ERR_INVALID;
  OzPlan *pl = new OzPlan();
  b->ozaki = pl;
  int dev = b->device, major = 0, minor = 0, nsm = 0;
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (major != 10) return IMSRG_ERR_INVALID;  // tcgen05 needs a Blackwell data-center part

  // matrices and exponent groups: L and R per (2J,Tz,parity) block, LCC and
  // RCC per cross-coupled block
  std::map<std::pair<int, long>, int> mat_of;  // (src, off) -> matrix index
  long imgb[4] = {0, 0, 0, 0};
  int ncore = 0;
  auto add_matrix = [&](int src, int group, long off, int n1, int n2) {
    if (n1 <= 0 || n2 <= 0) return;
    OzMatrix m{};
    m.src = src;
    m.group = group;
    m.off = off;
    m.n1 = n1;
    m.n2 = n2;
    m.rg_r = ((n1 + 127) / 128) * 16;
    m.rg_c = ((n2 + 127) / 128) * 16;
    int kc_r = (n2 + 15) / 16, kc_c = (n1 + 15) / 16;
    m.plane_r = (long)m.rg_r * kc_r * 256;
    m.plane_c = (long)m.rg_c * kc_c * 256;
    m.img_r = imgb[src];
    imgb[src] += OZ_S * m.plane_r;
    m.img_c = imgb[src];
    imgb[src] += OZ_S * m.plane_c;
    m.tile0 = ncore;
    ncore += ((n1 + 7) / 8) * ((n2 + 7) / 8);
    mat_of[{src, off}] = (int)pl->mats.size();
    pl->mats.push_back(m);
  };
  for (int src = 0; src < 2; src++)
    for (int q = 0; q < b->nblocks; q++) {
      int g = (int)pl->groups.size();
      long o0 = b->gam_off[q * 6], o1 = (q + 1 < b->nblocks) ? b->gam_off[q * 6 + 6] : b->nfull;
      pl->groups.push_back({src, o0, o1 - o0});
      for (int k = 0; k < 6; k++) add_matrix(src, g, b->gam_off[q * 6 + k], b->gam_n1[q * 6 + k], b->gam_n2[q * 6 + k]);
    }
  for (int src = 2; src < 4; src++)
    for (int q1 = 0; q1 < b->ccblocks; q1++) {
      int g = (int)pl->groups.size();
      long len = (long)b->cc_rlen[q1] * b->cc_nph[q1];
      pl->groups.push_back({src, b->cc_off[q1], len});
      add_matrix(src, g, b->cc_off[q1], b->cc_rlen[q1], b->cc_nph[q1]);
    }
  pl->ncore = ncore;

  // device buffers: images (zero padding stays zero), exponents, error flag
  for (int s = 0; s < 4; s++) {
    pl->img_bytes[s] = std::max<long>(imgb[s], 256);
    void *p = nullptr;
    IMSRG_CUDA_TRY(cudaMalloc(&p, pl->img_bytes[s]));
    IMSRG_CUDA_TRY(cudaMemset(p, 0, pl->img_bytes[s]));
    pl->img[s] = (uint8_t *)p;
  }

  // problems: the FP64 grouped-GEMM list mapped onto images
  auto img_of = [&](int gsrc) -> int {  // GemmTerm source id -> image source
    return gsrc == SRC_L ? 0 : gsrc == SRC_R ? 1 : gsrc == SRC_LCC ? 2 : gsrc == SRC_RCC ? 3 : -1;
  };
  int tiles = 0;
  for (const GemmProb &gp : b->probs) {
    OzProb p{};
    p.M = gp.M;
    p.N = gp.N;
    p.K = gp.K;
    p.ksteps = (gp.K + TK - 1) / TK;
    p.nterms = gp.nterms;
    double *dst = gp.c_dst == SRC_W1 ? b->w1 : gp.c_dst == SRC_W2 ? b->w2 : b->wcc;
    p.C = dst + gp.c_off;
    p.ldc = gp.ldc;
    for (int it = 0; it < gp.nterms; it++) {
      const GemmTerm &t = gp.t[it];
      int sa = img_of(t.a_src), sb = img_of(t.b_src);
      if (sa < 0 || sb < 0) return IMSRG_ERR_INVALID;
      auto ia = mat_of.find({sa, t.a_off}), ib = mat_of.find({sb, t.b_off});
      if (p.K > 0 && (ia == mat_of.end() || ib == mat_of.end())) return IMSRG_ERR_INVALID;
      OzTerm &o = p.t[it];
      if (p.K > 0) {
        const OzMatrix &A = pl->mats[ia->second], &B = pl->mats[ib->second];
        // K-major A: op(A) = A uses the R image (K = columns), A^T the C image
        o.a_img = pl->img[sa] + (t.ta ? A.img_c : A.img_r);
        o.a_plane = t.ta ? A.plane_c : A.plane_r;
        o.a_rg = t.ta ? A.rg_c : A.rg_r;
        // K-major B (stored N x K): op(B) = B uses the C image, B^T the R image
        o.b_img = pl->img[sb] + (t.tb ? B.img_r : B.img_c);
        o.b_plane = t.tb ? B.plane_r : B.plane_c;
        o.b_rg = t.tb ? B.rg_r : B.rg_c;
        if (it == 0) {
          p.gA = A.group;
          p.gB = B.group;
        }
      }
      o.neg = t.coef < 0;
      o.use_hl = t.use_hl;
      o.use_hr = t.use_hr;
    }
    // exactness bound of the FP32 level accumulators
    if ((double)p.nterms * p.K * (OZ_LMAX + 1) * 4096.0 >= 16777216.0) return IMSRG_ERR_INVALID;
    p.tiles_m = (p.M + TM - 1) / TM;
    p.tiles = p.tiles_m * ((p.N + TN - 1) / TN);
    p.tile0 = tiles;
    tiles += p.tiles;
    pl->probs.push_back(p);
  }
  pl->nmats = (int)pl->mats.size();
  pl->ngroups = (int)pl->groups.size();
  pl->nprobs = (int)pl->probs.size();
  pl->ntiles = tiles;
  pl->grid = std::min(nsm, std::max(tiles, 1));

  auto up = [&](const void *h, size_t bytes, void **d) -> int {
    IMSRG_CUDA_TRY(cudaMalloc(d, std::max<size_t>(bytes, 16)));
    if (bytes) IMSRG_CUDA_TRY(cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice));
    return IMSRG_OK;
  };
  IMSRG_TRY(up(pl->mats.data(), pl->mats.size() * sizeof(OzMatrix), (void **)&pl->d_mats));
  IMSRG_TRY(up(pl->groups.data(), pl->groups.size() * sizeof(OzGroup), (void **)&pl->d_groups));
  IMSRG_TRY(up(pl->probs.data(), pl->probs.size() * sizeof(OzProb), (void **)&pl->d_probs));
  IMSRG_CUDA_TRY(cudaMalloc((void **)&pl->d_exps, std::max(pl->ngroups, 1) * sizeof(int)));
  IMSRG_CUDA_TRY(cudaMalloc((void **)&pl->d_err, sizeof(int)));
  IMSRG_CUDA_TRY(cudaMemset(pl->d_err, 0, sizeof(int)));
  int smem = STAGES * STAGE_BYTES + 1024 + 256;
  IMSRG_CUDA_TRY(cudaFuncSetAttribute(k_oz_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  pl->ok = true;
  return IMSRG_OK;
}

int ozaki_gemm(imsrg_basis *b, const double *L, int hL, const double *R, int hR) {
  IMSRG_TRY(ozaki_prepare(b));
  OzPlan *pl = plan_of(b);
  {
    ProfScope ps(b, IMSRG_KERNEL_OZAKI_SLICE);
    k_oz_exponents<<<pl->ngroups, 256, 0, b->stream>>>(pl->d_groups, L, R, b->lcc, b->rcc, pl->d_exps);
    k_oz_slice<<<(pl->ncore + 127) / 128, 128, 0, b->stream>>>(pl->d_mats, pl->nmats, pl->ncore, L, R, b->lcc,
                                                                b->rcc, pl->d_exps, pl->img[0], pl->img[1],
                                                                pl->img[2], pl->img[3]);
    b->launches += 2;
  }
  IMSRG_CUDA_TRY(cudaGetLastError());
  {
    ProfScope ps(b, IMSRG_KERNEL_OZAKI_MMA);
    int smem = STAGES * STAGE_BYTES + 1024 + 256;
    k_oz_mma<<<pl->grid, OZ_THREADS, smem, b->stream>>>(pl->d_probs, pl->nprobs, pl->ntiles, pl->d_exps, hL, hR,
                                                       pl->d_err);
    b->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int ozaki_check_error(imsrg_basis *b) {
  OzPlan *pl = plan_of(b);
  if (!pl || !pl->d_err) return IMSRG_OK;
  int h = 0;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(&h, pl->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (h) {
    cudaMemsetAsync(pl->d_err, 0, sizeof(int), b->stream);
    return IMSRG_ERR_TIMEOUT;
  }
  return IMSRG_OK;
}

void ozaki_free(imsrg_basis *b) {
  OzPlan *pl = plan_of(b);
  if (!pl) return;
  for (int s = 0; s < 4; s++) cudaFree(pl->img[s]);
  cudaFree(pl->d_mats);
  cudaFree(pl->d_groups);
  cudaFree(pl->d_probs);
  cudaFree(pl->d_exps);
  cudaFree(pl->d_err);
  delete pl;
  b->ozaki = nullptr;
}

}  // namespace imsrg
