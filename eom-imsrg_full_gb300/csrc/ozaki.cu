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
//   3. k_oz_mma: persistent kernel, one 128 x TN output tile at a time.  A
//      producer thread streams the S A digit planes and S B planes of each
//      K = 16 step into shared memory with two TMA tensor loads (3-D boxes:
//      256-byte core matrix rows x row groups x planes, one per operand; one
//      request per plane measured 4.8 us slower per commutator at 12 instead
//      of 21 requests, whatever the bytes); one thread issues, per A plane
//      s, ONE tcgen05.mma of d_s against the B planes d_1 .. d_(S+1-s) side
//      by side (negating A for terms with coefficient -1) into the FP32
//      accumulators of levels l = s + t = s + 1 .. S + 1, side by side in
//      TMEM: S MMAs per K step.  The accumulators are double-buffered (two
//      sets of S x TN columns) so the epilogue warps read one tile
//      (tcgen05.ld), combine its levels in int64 and write FP64 while the
//      next tile's products run.  Each CTA takes a host-built list of
//      (problem, tile) slots, longest first under a cost model that an
//      autotuner picks by timing the kernel when the plan is built.
//
// Exactness: the level sums of levels 2..4 are bounded by 5 * 2^12 per
// product and term, so those accumulators hold exact integers below 2^24
// while nterms K 5 2^12 < 2^24 (a longer contraction runs in chunks whose
// int64 sums the epilogue adds).  The lower levels may round in FP32 there
// (relative 2^-24 of a quantity 2^-14 below the leading level).  The result
// differs from the exact product by the dropped levels (s + t > S + 1) and
// the digit rounding: about 2^-(7S) K max|A| max|B|.
//
// Every mbarrier wait is bounded (about 2 s of %globaltimer); a timeout sets
// an error flag that the host reports as IMSRG_ERR_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <map>

#include "device.cuh"

namespace imsrg {

namespace {

// S digits (slices) per operand, S = 6, 5 or 4.  Levels l = s + t up to
// S + 1 are kept, each in its own FP32 accumulator: a tile's S accumulators
// lie side by side in TMEM (level l at column (l - 2) x TN), as do the S B
// planes of a stage in shared memory, so the products of A plane s with B
// planes 1 .. S + 1 - s are ONE tcgen05.mma of width (S + 1 - s) x TN into
// the accumulators of levels s + 1 .. S + 1: S MMAs per K step.  (Fewer,
// wider MMAs: the tensor pipe pays a large fixed cost per instruction at
// these shapes.)  The tile width TN(S) keeps S x TN <= 256 (the widest MMA)
// with every level's block on a 32-column boundary: 64 for four digits, 32
// for five and six.
constexpr int OZ_SMAX = 8;
constexpr int TM = 128, TK = 16;
__host__ __device__ constexpr int oz_tn(int S) { return S <= 4 ? 64 : 32; }
// Seven and eight digits are the FP64-class settings: every level stays an
// exact integer (chunks of at most (2^24 - 1) / (TK (S + 2) 2^12) K steps:
// a level sums at most S products of 2^12 plus two of 2^13 with the leading
// digit), the level sums are combined in two int64 halves (7 (S - 1) + 24
// bits do not fit one) and converted once, and the WCC products are stored as
// FP64 like every other output.
__host__ __device__ constexpr bool oz_fp64_class(int S) { return S >= 7; }
// Largest chunk of a tile's K steps whose FP32 level sums stay exact for
// levels 2..4 (at most 5 x 2^12 per product term and K): steps x TK x 5 x
// 2^12 < 2^24; the lower levels may round there, below the truncation.
constexpr int kOzChunkSteps = (16777216 - 1) / (TK * 5 * 4096);
static_assert(kOzChunkSteps * TK * 5 * 4096 < 16777216, "chunk bound");
// pipeline stages: six, five where six would not fit (eight digits; oz_stages)
constexpr int STAGES = 6;
// Lines (8 elements each) per slicing CTA: small CTAs spread the ~100,000
// lines of a part evenly over the SMs (emax=6: with 256, the SMs were busy
// for 47% of the L slicing; 128 took the commutator from 159.6 to 156.5 us,
// 64 gave 159.5).
constexpr int SLICE_THREADS = 128;
constexpr int A_SLICE_BYTES = TM * TK * 2;   // 4096
__host__ __device__ constexpr int oz_b_slice_bytes(int S) { return oz_tn(S) * TK * 2; }
__host__ __device__ constexpr int oz_stage_bytes(int S) { return S * (A_SLICE_BYTES + oz_b_slice_bytes(S)); }
__host__ __device__ constexpr int oz_stages(int S) { return S >= 8 ? 5 : STAGES; }
__host__ __device__ constexpr int oz_mma_smem(int S) { return oz_stages(S) * oz_stage_bytes(S) + 1024 + 256; }
// K steps per accumulator chunk (see kOzChunkSteps and oz_fp64_class)
__host__ __device__ constexpr int oz_chunk_steps(int S) {
  return oz_fp64_class(S) ? (16777216 - 1) / (TK * (S + 2) * 4096) : kOzChunkSteps;
}
constexpr int TMEM_COLS = 512;
constexpr int ACC_BUF_COLS = 256;  // accumulator set b (double-buffered) starts at column 256 b
// epilogue warps: one per (TMEM lane quadrant, 16-column chunk of the tile)
__host__ __device__ constexpr int oz_epi_warps(int S) { return 4 * (oz_tn(S) / 16); }
// warp 0 producer, 1 MMA issuer, then the epilogue warps
__host__ __device__ constexpr int oz_threads(int S) { return 32 * (2 + oz_epi_warps(S)); }
static_assert(OZ_SMAX * 32 <= ACC_BUF_COLS && 4 * 64 <= ACC_BUF_COLS, "level accumulators of a set");
static_assert(oz_mma_smem(6) <= 227 * 1024 && oz_mma_smem(7) <= 227 * 1024 && oz_mma_smem(8) <= 227 * 1024,
              "stages");
constexpr unsigned long long WAIT_NS = 2000000000ull;

struct OzMatrix {
  int src;         // 0 L, 1 R, 2 LCC, 3 RCC
  int group;       // exponent group
  long off;        // element offset in the source buffer
  int n1, n2;      // column-major shape
  long img_r;      // byte offset of the R image (rows n1, K = n2), -1 when no problem reads it
  long img_c;      // byte offset of the C image (rows n2, K = n1), -1 when no problem reads it
  int rg_r, rg_c;  // row groups (of 8 rows) of each image
  long plane_r, plane_c;  // bytes per digit plane
  int np_r, np_c;         // digit planes stored (S)
  int line_r0, line_c0;   // first line of this matrix in the R / C slicing grids
};

// A contiguous chunk of one exponent group's elements.
struct OzChunk {
  int group, src;
  long off;
  int len;
};

struct OzTerm {
  const uint8_t *a_img, *b_img;
  long a_plane, b_plane;
  int a_rg, b_rg;
  int a_map, b_map;  // tensor maps of the A and B images (index into the plan's maps)
  int neg, use_hl, use_hr;
};

struct OzProb {
  int M, N, K, ksteps, nterms;
  // The (term, K step) sequence of a tile, term-major, runs in chunks of
  // kchunk steps, each into a fresh accumulator set: a chunk's FP32 level sums
  // stay exact integers (kchunk TK 5 2^12 < 2^24) and the epilogue adds the
  // chunks' int64 level sums exactly before the one conversion.
  int kchunk, nchunks;
  OzTerm t[2];
  double *C;
  int ldc;
  int gA, gB;
  int tiles_m, tile0, tiles;
  int raw;   // store the exact int64 level sum v (result = v 2^k) instead of FP64: the WCC products
  int inst;  // instance (basis) of a merged batch plan; its tiles run only while act[inst] (0 alone)
};

// Cost models of the CTA schedule tried by the autotuner (weights of K steps,
// of the epilogue's live outputs in 64ths of a tile, and a per-tile
// constant).  Model 1 balances K steps alone; the others charge a full
// tile's epilogue and each tile's fixed cost between a quarter and four K
// steps (with the per-level kernel a tile's epilogue costs about one to two
// K steps of products; weights of 10-40 per 64th, tried before, were 25-50 %
// slower).
struct SchedModel {
  int kw, ew, base;
};
constexpr int kNumSchedModels = 5;
constexpr SchedModel kSchedModels[kNumSchedModels] = {{16, 1, 16}, {4, 0, 1}, {32, 1, 16}, {8, 0, 8}, {64, 1, 16}};

struct OzPlan {
  int S = OZ_SMAX;  // digits per operand
  int chunk_steps = kOzChunkSteps;  // K steps per accumulator chunk (<= kOzChunkSteps)
  bool chunked = false;             // some problem runs in more than one chunk
  std::vector<OzMatrix> mats;
  std::vector<OzChunk> chunks;
  std::vector<OzProb> probs;
  OzMatrix *d_mats = nullptr;
  OzChunk *d_chunks = nullptr;
  OzProb *d_probs = nullptr;
  int2 *d_sched = nullptr;     // (problem, tile within the problem), grouped by CTA
  int *d_sched_off = nullptr;  // [grid + 1] start of each CTA's list
  int *d_exps = nullptr;       // per group: max biased exponent (e = value - 1022)
  int *d_err = nullptr;
  uint8_t *img[4] = {nullptr, nullptr, nullptr, nullptr};
  long img_bytes[4] = {0, 0, 0, 0};
  int nmats = 0, ngroups = 0, nchunks = 0, nprobs = 0, ntiles = 0;
  int lines_r = 0, lines_c = 0;
  // The operands fall in three parts that are sliced separately (and
  // concurrently): part 0 = L, part 1 = R (both available at once), part 2 =
  // LCC and RCC (after the Pandya transform).  Groups, chunks and image lines
  // are numbered part by part; part k owns [x_lo[k], x_lo[k + 1]).
  int group_lo[4] = {0, 0, 0, 0}, chunk_lo[4] = {0, 0, 0, 0}, linec_lo[4] = {0, 0, 0, 0}, liner_lo[4] = {0, 0, 0, 0};
  int *d_blk_mat = nullptr;  // slicing grids: matrix of each CTA's first line
  int2 *d_ccgroups = nullptr;  // [ccblocks]: exponent groups of LCC and RCC block q1
  int cblocks[3] = {0, 0, 0}, rblocks[3] = {0, 0, 0}, blk_off[3] = {0, 0, 0};
  int grid = 0;
  int tune_choice = 0;                   // the schedule model the autotuner kept
  double tune_us[kNumSchedModels] = {};  // its timings of each model
  bool tuned = false;
  std::vector<int> tile_ksteps, tile_live;  // per tile: K steps x terms, live outputs / 64
  std::vector<int2> tile_slot;
  std::vector<CUtensorMap> maps;     // TMA maps of the digit images, by role (see map_of)
  CUtensorMap *d_maps = nullptr;
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

// One 3-D TMA tile of a digit image into shared memory (x = 0: the 16-byte
// rule on the innermost coordinate always holds; rows past the image arrive
// as zeros).
__device__ __forceinline__ void tma_load_3d(void *sdst, const CUtensorMap *map, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(sdst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(y), "r"(z), "r"(smem_u32(bar))
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

// A tile element's level sums (integer-valued FP32 accumulators, below 2^31)
// combined exactly in int64, in units of level S + 1 (32-bit conversions: the
// conversion pipe, where a 64-bit one would take the FP64 pipe).
template <int S>
__device__ __forceinline__ long long oz_level_sum(const uint32_t (&acc)[S][16], int c) {
  long long v = 0;
#pragma unroll
  for (int l = 0; l < S; l++) v += (long long)__float2int_rn(__uint_as_float(acc[l][c])) << (7 * (S - 1 - l));
  return v;
}

// The same as one FP64 value, in units of level S + 1: one conversion of the
// exact int64 sum, or for seven and eight digits the sum's two halves (the
// levels at least 2^28 apart and the rest, each exact in int64 and below
// 2^53) converted exactly and added with one rounding.
template <int S>
__device__ __forceinline__ double oz_level_value(const uint32_t (&acc)[S][16], int c) {
  if constexpr (S <= 6) {
    return (double)oz_level_sum<S>(acc, c);
  } else {
    long long hi = 0, lo = 0;
#pragma unroll
    for (int l = 0; l < S; l++) {
      const long long a = (long long)__float2int_rn(__uint_as_float(acc[l][c]));
      const int sh = 7 * (S - 1 - l);
      if (sh >= 28) hi += a << (sh - 28);
      else lo += a << sh;
    }
    return fma((double)hi, 268435456.0, (double)lo);
  }
}

// d 2^k: k added to the exponent field on the integer pipe while the result
// stays normal (exactly ldexp's value), else ldexp
__device__ __forceinline__ double oz_scale(double d, int k) {
  unsigned long long bits = (unsigned long long)__double_as_longlong(d);
  const int E = (int)((bits >> 52) & 0x7FF);
  if (E != 0 && E + k > 0 && E + k < 2047) {
    bits += (unsigned long long)(long long)k << 52;
    return __longlong_as_double((long long)bits);
  }
  return E != 0 ? ldexp(d, k) : d;
}

// ---------------------------------------------------------------------------
// 1. block exponents: max biased exponent of each group (integer atomicMax,
//    order-independent, so the result is deterministic)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_oz_exponents(const OzChunk *chunks, const double *L, const double *R,
                                                      const double *LCC, const double *RCC, int *exps) {
  __shared__ int sh[8];
  OzChunk c = chunks[blockIdx.x];
  const double *src = (c.src == 0 ? L : c.src == 1 ? R : c.src == 2 ? LCC : RCC) + c.off;
  // chunks hold at most 4 x 256 elements: four independent loads per thread
  int m = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int i = threadIdx.x + k * 256;
    if (i < c.len) m = max(m, (int)((__double_as_longlong(src[i]) >> 52) & 0x7FF));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = max(m, sh[w]);
    atomicMax(&exps[c.group], m);
  }
}

// ---------------------------------------------------------------------------
// 2. digit slicing: one thread per 8-element line of a core matrix
// ---------------------------------------------------------------------------
// Digits of x with |x| < 2^e: x = 2^(e-7S) sum_{s} d_s 128^(S-1-s), d_0 first.
// One 64-bit shift rounds |x| to the 7S-bit integer V; the balanced base-128
// digits then come from its low 21 bits and the rest on the 32-bit integer
// pipe (S <= 6), or all on the 64-bit one (S = 7, 8: V has up to 56 bits).
template <int S>
__device__ __forceinline__ void digits(double x, int e, int *d) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((bits >> 52) & 0x7FF);
  const int neg = (int)(bits >> 63);
  unsigned long long V = 0;
  if (E != 0) {
    const unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    // V = round(|x| 2^(7S - e)): rs >= 53 - 7S (>= 11 for S <= 6, >= -3 for S = 8)
    const int rs = e + 1075 - 7 * S - E;
    if constexpr (S >= 8) {
      if (rs <= 0) V = mant << (-rs);  // exact: the 53-bit significand fits in 56 bits
      else if (rs <= 63) V = (mant + (1ull << (rs - 1))) >> rs;
    } else {
      if (rs <= 63) V = (mant + (1ull << (rs - 1))) >> rs;
    }
  }
  if constexpr (S >= 7) {
#pragma unroll
    for (int s = S - 1; s >= 1; s--) {
      int u = (int)(V & 127u);
      V >>= 7;
      if (u >= 64) {
        u -= 128;
        V += 1;
      }
      d[s] = neg ? -u : u;
    }
    d[0] = neg ? -(int)V : (int)V;
    return;
  }
  unsigned lo = (unsigned)(V & 0x1FFFFFu), hi = (unsigned)(V >> 21);
#pragma unroll
  for (int s = S - 1; s >= S - 3; s--) {
    int u = (int)(lo & 127u);
    lo >>= 7;
    if (u >= 64) {
      u -= 128;
      lo += 1;
    }
    d[s] = neg ? -u : u;
  }
  hi += lo;  // carry out of the low half
#pragma unroll
  for (int s = S - 4; s >= 1; s--) {
    int u = (int)(hi & 127u);
    hi >>= 7;
    if (u >= 64) {
      u -= 128;
      hi += 1;
    }
    d[s] = neg ? -u : u;
  }
  d[0] = neg ? -(int)hi : (int)hi;
}

// Threads of the first cblocks CTAs write C-image lines [c_lo, c_hi) (8
// consecutive rows of one column: one 16-byte row of a C core matrix per digit
// plane); the other CTAs write R-image lines [r_lo, r_hi) (8 consecutive
// columns of one row).  blk_mat[b] is the matrix of CTA b's first line.  Padding lines of the images are never
// written and stay zero.
template <int S>
__global__ void __launch_bounds__(SLICE_THREADS) k_oz_slice(const OzMatrix *__restrict__ mats, int nmats,
                                                  const int *__restrict__ blk_mat, int cblocks, int c_lo, int c_hi,
                                                  int r_lo, int r_hi, const double *L, const double *R, const double *LCC,
                                                  const double *RCC, const int *exps, uint8_t *imgL, uint8_t *imgR,
                                                  uint8_t *imgLCC, uint8_t *imgRCC) {
  // BF16 bit patterns of the digits -128..128 (exact), built once per CTA
  __shared__ uint32_t tab[257];
  for (int i = threadIdx.x; i < 257; i += blockDim.x) {
    __nv_bfloat16 h = __float2bfloat16_rn((float)(i - 128));
    tab[i] = *reinterpret_cast<uint16_t *>(&h);
  }
  __syncthreads();
  const bool cimg = (int)blockIdx.x < cblocks;
  const int t = (cimg ? c_lo : r_lo) + ((int)blockIdx.x - (cimg ? 0 : cblocks)) * blockDim.x + threadIdx.x;
  if (t >= (cimg ? c_hi : r_hi)) return;
  int mi = blk_mat[blockIdx.x];
  while (mi + 1 < nmats && (cimg ? mats[mi + 1].line_c0 : mats[mi + 1].line_r0) <= t) mi++;
  const OzMatrix &m = mats[mi];
  const double *src = (m.src == 0 ? L : m.src == 1 ? R : m.src == 2 ? LCC : RCC) + m.off;
  uint8_t *img = m.src == 0 ? imgL : m.src == 1 ? imgR : m.src == 2 ? imgLCC : imgRCC;
  const int e = exps[m.group] - 1022;
  double x[8];
  long off;
  long plane;
  if (cimg) {
    const int RG = (m.n1 + 7) >> 3;
    const int l = t - m.line_c0;
    const int rg = l % RG, c = l / RG;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int r = rg * 8 + i;
      x[i] = r < m.n1 ? src[r + (long)c * m.n1] : 0.0;
    }
    off = m.img_c + ((long)((rg >> 1) * m.rg_c + (c >> 3)) * 2 + (rg & 1)) * 128 + (c & 7) * 16;
    plane = m.plane_c;
  } else {
    const int l = t - m.line_r0;
    const int r = l % m.n1, cg = l / m.n1;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int c = cg * 8 + j;
      x[j] = c < m.n2 ? src[r + (long)c * m.n1] : 0.0;
    }
    off = m.img_r + ((long)((cg >> 1) * m.rg_r + (r >> 3)) * 2 + (cg & 1)) * 128 + (r & 7) * 16;
    plane = m.plane_r;
  }
  uint32_t h[8][S];  // BF16 bits of each digit
#pragma unroll
  for (int i = 0; i < 8; i++) {
    int d[S];
    digits<S>(x[i], e, d);
#pragma unroll
    for (int s = 0; s < S; s++) h[i][s] = tab[d[s] + 128];
  }
  // plane s: digit s of the 8 elements (16 bytes)
#pragma unroll
  for (int k = 0; k < S; k++) {
    uint32_t w4[4];
#pragma unroll
    for (int i = 0; i < 8; i += 2) w4[i >> 1] = h[i][k] | (h[i + 1][k] << 16);
    *reinterpret_cast<uint4 *>(img + off + k * plane) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
  }
}

// ---------------------------------------------------------------------------
// 3. tensor-core products and exact recombination
// ---------------------------------------------------------------------------

// CH: the plan has contractions in several chunks (see OzProb); without any,
// the chunk bookkeeping folds away at compile time.
template <int S, bool CH>
__global__ void __launch_bounds__(oz_threads(S), 1) k_oz_mma(const OzProb *__restrict__ probs, int nprobs,
                                                          const int2 *__restrict__ sched,
                                                          const int *__restrict__ sched_off,
                                                          const int *__restrict__ exps, int hL, int hR, int *err,
                                                          const CUtensorMap *__restrict__ maps,
                                                          const int *__restrict__ act) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int STAGE_BYTES = oz_stage_bytes(S), LMAX = S + 1, TN = oz_tn(S), STAGES = oz_stages(S);
  uint64_t *full = (uint64_t *)(smem + STAGES * STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *acc_full = empty + STAGES;   // [2]
  uint64_t *acc_empty = acc_full + 2;    // [2]
  uint32_t *tmem_slot = (uint32_t *)(acc_empty + 2);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's tiles (longest first, assigned on the host)
  const int t_begin = sched_off[blockIdx.x], t_end = sched_off[blockIdx.x + 1];

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], oz_epi_warps(S));
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // (every stage is written whole by its two TMA boxes before the MMAs read it)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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
      for (int ti = t_begin; ti < t_end && !*abort_flag; ti++) {
        const int2 slot = sched[ti];
        const OzProb &P = probs[slot.x];
        if (P.ksteps == 0 || (act && !act[P.inst])) continue;
        const int lt = slot.y;
        int tm = lt % P.tiles_m, tn = lt / P.tiles_m;
        for (int it = 0; it < P.nterms; it++) {
          const OzTerm &T = P.t[it];
          const CUtensorMap *amap = maps + T.a_map, *bmap = maps + T.b_map;
          for (int kk = 0; kk < P.ksteps; kk++) {  // the chunks only regroup these steps
            if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
              atomicExch(err, 1);
              *abort_flag = 1;
              break;
            }
            // two whole boxes: the row groups past the tile's operand rows
            // (next K step's rows, or zeros past the image) only reach
            // accumulator rows and columns that are never stored
            mbar_expect_tx(&full[stage], STAGE_BYTES);
            uint8_t *sa = smem + stage * STAGE_BYTES;
            uint8_t *sb = sa + S * A_SLICE_BYTES;
            tma_load_3d(sa, amap, kk * T.a_rg + tm * (TM / 8), 0, &full[stage]);
            tma_load_3d(sb, bmap, kk * T.b_rg + tn * (TN / 8), 0, &full[stage]);
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
      // MMA issuer: alternates between the two accumulator sets so the next
      // tile's products overlap the epilogue of the previous one
      int stage = 0, nt = 0;
      uint32_t phase = 0;
      for (int ti = t_begin; ti < t_end && !*abort_flag; ti++) {
        const OzProb &P = probs[sched[ti].x];
        if (P.ksteps == 0 || (act && !act[P.inst])) continue;
        const uint64_t desc0 = smem_desc(smem_u32(smem), 128, 256);
        const int kchunk = CH ? P.kchunk : 0x40000000;
        int left = 0;                          // steps left in the current chunk
        int total = P.nterms * P.ksteps;       // steps left in the tile
        uint32_t dbase = 0;
        bool first = true;  // first K step of a chunk overwrites the accumulators
        for (int it = 0; it < P.nterms && !*abort_flag; it++) {
          const OzTerm &T = P.t[it];
          int neg = T.neg ^ (T.use_hl & (hL < 0)) ^ (T.use_hr & (hR < 0));
          uint32_t idesc[S];  // A plane s: width (S - s) TN
#pragma unroll
          for (int s = 0; s < S; s++) idesc[s] = idesc_bf16(TM, (S - s) * TN, neg);
          for (int kk = 0; kk < P.ksteps; kk++) {
            if (left == 0) {  // a chunk starts: take the next accumulator set
              const int buf = nt & 1;
              const uint32_t use = (uint32_t)(nt >> 1);
              nt++;
              if (!mbar_wait(&acc_empty[buf], (use & 1) ^ 1, abort_flag)) {
                atomicExch(err, 2);
                *abort_flag = 1;
                break;
              }
              tc_fence_after();
              dbase = tmem + (uint32_t)(buf * ACC_BUF_COLS);
              first = true;
              left = kchunk;
            }
            if (!mbar_wait(&full[stage], phase, abort_flag)) {
              atomicExch(err, 3);
              *abort_flag = 1;
              break;
            }
            tc_fence_after();
            // descriptor start-address fields advance in 16-byte units
            const uint64_t da = desc0 + (uint64_t)((stage * STAGE_BYTES) >> 4);
            const uint64_t db = da + (uint64_t)((S * A_SLICE_BYTES) >> 4);
            // A plane s (0-based) times B planes 0 .. S - 1 - s (side by side
            // in the stage) is one MMA into the accumulators of levels s + 2
            // .. S + 1 (side by side in TMEM).  The first K step of a chunk
            // overwrites: plane 0's MMA covers every accumulator.
#pragma unroll
            for (int s = 0; s < S; s++)
              mma_bf16(dbase + (uint32_t)(s * TN), da + (uint64_t)(s * (A_SLICE_BYTES >> 4)), db, idesc[s],
                       (first && s == 0) ? 0 : 1);
            first = false;
            mma_commit(&empty[stage]);
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
            // a chunk ends: its accumulator set goes to the epilogue
            --left;
            --total;
            if (left == 0 || total == 0) mma_commit(&acc_full[(nt - 1) & 1]);
          }
        }
      }
    }
  } else {
    // epilogue warps 2..: TMEM lane quadrant = warp % 4 (the lanes a warp
    // may read), 16-column chunk = (warp - 2) / 4
    const int quad = warp & 3, chunk = (warp - 2) >> 2;
    const int row = quad * 32 + lane;
    int nt = 0;
    for (int ti = t_begin; ti < t_end; ti++) {
      const int2 slot = sched[ti];
      const OzProb &P = probs[slot.x];
      if (act && !act[P.inst]) continue;  // an instance whose series has stopped: its outputs stay
      const int lt = slot.y;
      // problem fields in registers: the stores below could alias the problem
      // table as far as the compiler knows, which would force a reload per column
      const int Mp = P.M, Np = P.N, ldc = P.ldc, ksteps = P.ksteps, gA = P.gA, gB = P.gB;
      const int nch = CH ? P.nchunks : 1, raw = P.raw;
      const int tiles_m = P.tiles_m;
      double *const Cbase = P.C;
      const int m0 = (lt % tiles_m) * TM;
      const int m = m0 + row;
      const int n0 = (lt / tiles_m) * TN + 16 * chunk;
      const bool row_ok = m < Mp;
      double *crow = Cbase + m;
      if (ksteps == 0) {
        if (row_ok)
          for (int c = 0; c < 16 && n0 + c < Np; c++) crow[(long)(n0 + c) * ldc] = 0.0;
        continue;
      }
      // warp-uniform: a piece entirely past M or N is neither read nor converted
      const bool live = m0 + quad * 32 < Mp && n0 < Np;
      // A tile in several chunks adds the chunks' exact level sums in the
      // output's own 8-byte slots (each thread owns its elements), as int64,
      // until the last chunk converts
      long long *irow = reinterpret_cast<long long *>(crow);
      for (int ch = 0; ch < nch; ch++) {
        const int buf = nt & 1;
        const uint32_t use = (uint32_t)(nt >> 1);
        nt++;
        if (*abort_flag || !mbar_wait(&acc_full[buf], use & 1, abort_flag)) {
          if (!*abort_flag) atomicExch(err, 4);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        uint32_t acc[S][16];
        if (live) {
#pragma unroll
          for (int l = 0; l < S; l++)
            tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * ACC_BUF_COLS + l * TN + 16 * chunk),
                      acc[l]);
        }
        tmem_ld_wait();
        // the accumulators are in registers: hand the TMEM set back to the MMA issuer
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[buf]);
        if (!live) continue;
        // the level sums in units of level S + 1 (hardware conversions:
        // measured faster here than assembling the double from integer bit
        // operations)
#define OZ_LEVEL_SUM(c) oz_level_sum<S>(acc, c)
        if (nch == 1 && !raw) {
          const int k = (exps[gA] - 1022) + (exps[gB] - 1022) - 7 * LMAX;  // result = v * 2^k
#pragma unroll
          for (int c = 0; c < 16; c++) {
            const double d = oz_scale(oz_level_value<S>(acc, c), k);
            const int n = n0 + c;
            if (row_ok && n < Np) crow[(long)n * ldc] = d;
          }
          continue;
        }
        if constexpr (oz_fp64_class(S)) {
          // a long contraction at seven or eight digits adds its chunks in
          // FP64 in the output's own slots, then scales once
#pragma unroll
          for (int c = 0; c < 16; c++) {
            double v = oz_level_value<S>(acc, c);
            const int n = n0 + c;
            if (row_ok && n < Np) {
              if (ch > 0) v += crow[(long)n * ldc];
              crow[(long)n * ldc] = v;
            }
          }
          if (ch < nch - 1 || !row_ok) continue;
          const int k = (exps[gA] - 1022) + (exps[gB] - 1022) - 7 * LMAX;
          for (int c = 0; c < 16 && n0 + c < Np; c++) crow[(long)(n0 + c) * ldc] = oz_scale(crow[(long)(n0 + c) * ldc], k);
        } else {
          // WCC keeps the exact level sum as an integer (the 222_ph recoupling
          // combines four entries of one block, which share 2^k, before its one
          // conversion to FP64); a long contraction adds its chunks there
#pragma unroll
          for (int c = 0; c < 16; c++) {
            long long v = OZ_LEVEL_SUM(c);
            const int n = n0 + c;
            if (row_ok && n < Np) {
              if (ch > 0) v += irow[(long)n * ldc];
              irow[(long)n * ldc] = v;
            }
          }
          if (raw || ch < nch - 1 || !row_ok) continue;
          // the last chunk of a long FP64 contraction: convert the summed integers
          const int k = (exps[gA] - 1022) + (exps[gB] - 1022) - 7 * LMAX;
          for (int c = 0; c < 16 && n0 + c < Np; c++)
            crow[(long)(n0 + c) * ldc] = oz_scale((double)irow[(long)(n0 + c) * ldc], k);
        }
#undef OZ_LEVEL_SUM
      }
      if (*abort_flag) break;
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

void launch_mma(int S, bool chunked, int grid, cudaStream_t st, const OzProb *probs, int nprobs, const int2 *sched,
                const int *sched_off, const int *exps, int hL, int hR, int *err, const CUtensorMap *maps,
                const int *act = nullptr) {
#define OZ_LAUNCH(SS, CC)                                                                                    \
  k_oz_mma<SS, CC><<<grid, oz_threads(SS), oz_mma_smem(SS), st>>>(probs, nprobs, sched, sched_off, exps, hL, hR, err, \
                                                              maps, act)
  switch (S) {
    case 4: if (chunked) OZ_LAUNCH(4, true); else OZ_LAUNCH(4, false); break;
    case 5: if (chunked) OZ_LAUNCH(5, true); else OZ_LAUNCH(5, false); break;
    case 6: if (chunked) OZ_LAUNCH(6, true); else OZ_LAUNCH(6, false); break;
    case 7: if (chunked) OZ_LAUNCH(7, true); else OZ_LAUNCH(7, false); break;
    default: if (chunked) OZ_LAUNCH(8, true); else OZ_LAUNCH(8, false); break;
  }
#undef OZ_LAUNCH
}

// CTA schedule: longest-processing-time-first assignment of tiles to the
// persistent CTAs under the cost model cost = kw * (K steps x terms) + ew *
// (live outputs / 64) + base.
void build_sched(const OzPlan *pl, const SchedModel &md, std::vector<int2> &sched, std::vector<int> &sched_off) {
  const int tiles = (int)pl->tile_slot.size();
  std::vector<long> cost(tiles);
  for (int i = 0; i < tiles; i++)
    cost[i] = (long)md.kw * pl->tile_ksteps[i] + (long)md.ew * pl->tile_live[i] + md.base;
  std::vector<int> order(tiles);
  for (int i = 0; i < tiles; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
  std::vector<long> load(pl->grid, 0);
  std::vector<std::vector<int>> lists(pl->grid);
  for (int t : order) {
    int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[best] += cost[t];
    lists[best].push_back(t);
  }
  sched.clear();
  sched_off.assign(pl->grid + 1, 0);
  for (int c = 0; c < pl->grid; c++) {
    sched_off[c] = (int)sched.size();
    for (int t : lists[c]) sched.push_back(pl->tile_slot[t]);
  }
  sched_off[pl->grid] = (int)sched.size();
}

int use_model(imsrg_basis *b, OzPlan *pl, int c) {
  std::vector<int2> sched;
  std::vector<int> sched_off;
  build_sched(pl, kSchedModels[c], sched, sched_off);
  IMSRG_CUDA_TRY(cudaMemcpyAsync(pl->d_sched, sched.data(), sched.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                 b->stream));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(pl->d_sched_off, sched_off.data(), sched_off.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

// Autotuning of the CTA schedule, on the first split-precision commutator
// that is not being captured into a graph: with that commutator's own digit
// images in place, every candidate cost model is timed on the real kernel
// (warm-up first, as clocks ramp on an idle GPU; then two interleaved passes,
// three launches each, a candidate's time being its fastest launch) and the
// fastest is kept.  The kernel is deterministic per tile, so the schedule
// never changes results.
int autotune(imsrg_basis *b, OzPlan *pl, int hL, int hR) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  IMSRG_CUDA_TRY(cudaEventCreate(&e0));
  IMSRG_CUDA_TRY(cudaEventCreate(&e1));
  auto launch_timed = [&](float *ms) -> int {
    IMSRG_CUDA_TRY(cudaEventRecord(e0, b->stream));
    launch_mma(pl->S, pl->chunked, pl->grid, b->stream, pl->d_probs, pl->nprobs, pl->d_sched, pl->d_sched_off, pl->d_exps, hL, hR,
               pl->d_err, pl->d_maps);
    b->launches++;
    IMSRG_CUDA_TRY(cudaEventRecord(e1, b->stream));
    IMSRG_CUDA_TRY(cudaEventSynchronize(e1));
    IMSRG_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
    return IMSRG_OK;
  };
  int s = IMSRG_OK;
  for (int w = 0; w < 8 && s == IMSRG_OK; w++) {
    float ms;
    s = launch_timed(&ms);
  }
  for (int c = 0; c < kNumSchedModels; c++) pl->tune_us[c] = 1e30;
  for (int pass = 0; pass < 2 && s == IMSRG_OK; pass++)
    for (int c = 0; c < kNumSchedModels && s == IMSRG_OK; c++) {
      s = use_model(b, pl, c);
      for (int rep = 0; rep < 3 && s == IMSRG_OK; rep++) {
        float ms = 0.f;
        s = launch_timed(&ms);
        pl->tune_us[c] = std::min(pl->tune_us[c], 1e3 * (double)ms);
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  IMSRG_TRY(s);
  int best = 0;
  for (int c = 1; c < kNumSchedModels; c++)
    if (pl->tune_us[c] < pl->tune_us[best]) best = c;
  pl->tune_choice = best;
  pl->tuned = true;
  return use_model(b, pl, best);
}

}  // namespace

int ozaki_prepare(imsrg_basis *b) {
  if (b->ozaki) return plan_of(b)->ok ? IMSRG_OK : IMSRG_ERR_INVALID;
  OzPlan *pl = new OzPlan();
  b->ozaki = pl;
  pl->S = b->split_digits;
  if (pl->S < 4 || pl->S > OZ_SMAX) return IMSRG_ERR_INVALID;
  pl->chunk_steps = oz_chunk_steps(pl->S);
  if (b->split_chunk_steps > 0) pl->chunk_steps = std::min(b->split_chunk_steps, oz_chunk_steps(pl->S));
  int dev = b->device, major = 0, nsm = 0;
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (major != 10) return IMSRG_ERR_INVALID;  // tcgen05 needs a Blackwell data-center part

  // matrices: L and R arrays per (2J,Tz,parity) block (one exponent group per
  // block), LCC and RCC per cross-coupled block (one group each)
  std::map<std::pair<int, long>, int> mat_of;  // (src, off) -> matrix index
  std::vector<OzChunk> &chunks = pl->chunks;
  int ngroups = 0;
  auto add_group = [&](int src, long off, long len) {
    int g = ngroups++;
    for (long s0 = 0; s0 < len; s0 += 1024) chunks.push_back({g, src, off + s0, (int)std::min<long>(1024, len - s0)});
    return g;
  };
  auto add_matrix = [&](int src, int group, long off, int n1, int n2) {
    if (n1 <= 0 || n2 <= 0) return;
    OzMatrix m{};
    m.src = src;
    m.group = group;
    m.off = off;
    m.n1 = n1;
    m.n2 = n2;
    m.img_r = m.img_c = -1;
    mat_of[{src, off}] = (int)pl->mats.size();
    pl->mats.push_back(m);
  };
  for (int src = 0; src < 2; src++) {
    pl->group_lo[src] = ngroups;
    pl->chunk_lo[src] = (int)chunks.size();
    for (int q = 0; q < b->nblocks; q++) {
      long o0 = b->gam_off[q * 6], o1 = (q + 1 < b->nblocks) ? b->gam_off[q * 6 + 6] : b->nfull;
      int g = add_group(src, o0, o1 - o0);
      for (int k = 0; k < 6; k++) add_matrix(src, g, b->gam_off[q * 6 + k], b->gam_n1[q * 6 + k], b->gam_n2[q * 6 + k]);
    }
  }
  pl->group_lo[2] = ngroups;
  pl->chunk_lo[2] = (int)chunks.size();
  for (int src = 2; src < 4; src++)
    for (int q1 = 0; q1 < b->ccblocks; q1++) {
      long len = (long)b->cc_rlen[q1] * b->cc_nph[q1];
      int g = add_group(src, b->cc_off[q1], len);
      add_matrix(src, g, b->cc_off[q1], b->cc_rlen[q1], b->cc_nph[q1]);
    }
  pl->ngroups = ngroups;
  pl->nchunks = (int)chunks.size();
  pl->group_lo[3] = ngroups;
  pl->chunk_lo[3] = (int)chunks.size();

  // which images each matrix needs: op(A) = X reads X's R image, X^T its C
  // image; op(B) = Y reads Y's C image, Y^T its R image.  An image read as a B
  // operand also carries the scaled tail planes.
  auto img_of = [&](int gsrc) -> int {
    return gsrc == SRC_L ? 0 : gsrc == SRC_R ? 1 : gsrc == SRC_LCC ? 2 : gsrc == SRC_RCC ? 3 : -1;
  };
  std::vector<int> role_r(pl->mats.size(), 0), role_c(pl->mats.size(), 0);  // 0 unused, 1 B, 2 A
  std::vector<int> b_role_r(pl->mats.size(), 0), b_role_c(pl->mats.size(), 0);  // read as a B operand
  for (const GemmProb &gp : b->probs) {
    if (gp.K <= 0) continue;
    for (int it = 0; it < gp.nterms; it++) {
      const GemmTerm &t = gp.t[it];
      int sa = img_of(t.a_src), sb = img_of(t.b_src);
      if (sa < 0 || sb < 0) return IMSRG_ERR_INVALID;
      auto ia = mat_of.find({sa, t.a_off}), ib = mat_of.find({sb, t.b_off});
      if (ia == mat_of.end() || ib == mat_of.end()) return IMSRG_ERR_INVALID;
      (t.ta ? role_c : role_r)[ia->second] = 2;
      int &rb = (t.tb ? role_r : role_c)[ib->second];
      rb = std::max(rb, 1);
      (t.tb ? b_role_r : b_role_c)[ib->second] = 1;
    }
  }
  long imgb[4] = {0, 0, 0, 0};
  int lines_r = 0, lines_c = 0;
  for (size_t i = 0; i < pl->mats.size(); i++) {
    OzMatrix &m = pl->mats[i];
    m.line_r0 = lines_r;
    m.line_c0 = lines_c;
    if (role_r[i]) {
      m.rg_r = (m.n1 + 7) / 8;
      m.plane_r = (long)m.rg_r * ((m.n2 + 15) / 16) * 256;
      m.np_r = pl->S;
      m.img_r = imgb[m.src];
      imgb[m.src] += m.np_r * m.plane_r;
      lines_r += ((m.n2 + 7) / 8) * m.n1;
    }
    if (role_c[i]) {
      m.rg_c = (m.n2 + 7) / 8;
      m.plane_c = (long)m.rg_c * ((m.n1 + 15) / 16) * 256;
      m.np_c = pl->S;
      m.img_c = imgb[m.src];
      imgb[m.src] += m.np_c * m.plane_c;
      lines_c += ((m.n1 + 7) / 8) * m.n2;
    }
  }
  pl->lines_r = lines_r;
  pl->lines_c = lines_c;
  // first lines of each part (matrices are ordered L, R, then LCC and RCC)
  for (int part = 0; part < 3; part++) {
    pl->linec_lo[part] = lines_c;
    pl->liner_lo[part] = lines_r;
    for (const OzMatrix &m : pl->mats)
      if ((part < 2 && m.src == part) || (part == 2 && m.src >= 2)) {
        pl->linec_lo[part] = m.line_c0;
        pl->liner_lo[part] = m.line_r0;
        break;
      }
  }
  pl->linec_lo[3] = lines_c;
  pl->liner_lo[3] = lines_r;
  // per part: the matrix of each CTA's first line (C lines, then R lines)
  std::vector<int> blk_mat;
  for (int part = 0; part < 3; part++) {
    const int c_lo = pl->linec_lo[part], c_hi = pl->linec_lo[part + 1];
    const int r_lo = pl->liner_lo[part], r_hi = pl->liner_lo[part + 1];
    pl->cblocks[part] = (c_hi - c_lo + SLICE_THREADS - 1) / SLICE_THREADS;
    pl->rblocks[part] = (r_hi - r_lo + SLICE_THREADS - 1) / SLICE_THREADS;
    pl->blk_off[part] = (int)blk_mat.size();
    for (int cimg = 1; cimg >= 0; cimg--) {
      const int nb = cimg ? pl->cblocks[part] : pl->rblocks[part];
      const int lo = cimg ? c_lo : r_lo;
      int mi = 0;
      auto l0 = [&](int k) { return cimg ? pl->mats[k].line_c0 : pl->mats[k].line_r0; };
      for (int bk = 0; bk < nb; bk++) {
        const int t0 = lo + bk * SLICE_THREADS;
        while (mi + 1 < (int)pl->mats.size() && l0(mi + 1) <= t0) mi++;
        blk_mat.push_back(mi);
      }
    }
  }
  for (int s = 0; s < 4; s++) {
    pl->img_bytes[s] = std::max<long>(imgb[s], 256);
    void *p = nullptr;
    IMSRG_CUDA_TRY(cudaMalloc(&p, pl->img_bytes[s]));
    IMSRG_CUDA_TRY(cudaMemset(p, 0, pl->img_bytes[s]));  // padding stays zero
    pl->img[s] = (uint8_t *)p;
  }

  // TMA maps of the images, one per (image, role): a digit image is planes x
  // (K steps x row groups) x 256-byte core-matrix rows; an A tile is the box
  // 16 row groups x 6 planes, a B tile 8 row groups x 15 planes.  The encoder
  // is the driver's cuTensorMapEncodeTiled, reached through the runtime.
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return IMSRG_ERR_CUDA;
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  std::map<std::pair<const uint8_t *, int>, int> map_index;
  auto map_of = [&](const uint8_t *img, long plane, int np, int brole, int *idx) -> int {
    auto it = map_index.find({img, brole});
    if (it != map_index.end()) {
      *idx = it->second;
      return IMSRG_OK;
    }
    const cuuint32_t box_planes = pl->S;
    if (plane <= 0 || plane % 256 || (long)np < (long)box_planes) return IMSRG_ERR_INVALID;
    CUtensorMap m;
    const cuuint64_t gdim[3] = {32, (cuuint64_t)(plane / 256), (cuuint64_t)np};
    const cuuint64_t gstride[2] = {256, (cuuint64_t)plane};
    const cuuint32_t box[3] = {32, (cuuint32_t)(brole ? oz_tn(pl->S) / 8 : TM / 8), box_planes};
    const cuuint32_t estride[3] = {1, 1, 1};
    if (encode(&m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, (void *)img, gdim, gstride, box, estride,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return IMSRG_ERR_INVALID;
    *idx = (int)pl->maps.size();
    pl->maps.push_back(m);
    map_index[{img, brole}] = *idx;
    return IMSRG_OK;
  };

  // problems: the FP64 grouped-GEMM list mapped onto images
  int tiles = 0;
  std::vector<int> &tile_ksteps = pl->tile_ksteps, &tile_live = pl->tile_live;
  std::vector<int2> &tile_slot = pl->tile_slot;  // (problem, tile within the problem) of each tile
  for (const GemmProb &gp : b->probs) {
    OzProb p{};
    p.M = gp.M;
    p.N = gp.N;
    p.K = gp.K;
    p.ksteps = (gp.K + TK - 1) / TK;
    p.nterms = gp.nterms;
    double *dst = gp.c_dst == SRC_W1 ? b->w1 : gp.c_dst == SRC_W2 ? b->w2 : b->wcc;
    p.C = dst + gp.c_off;
    p.raw = gp.c_dst == SRC_WCC && !oz_fp64_class(pl->S);
    p.ldc = gp.ldc;
    for (int it = 0; it < gp.nterms; it++) {
      const GemmTerm &t = gp.t[it];
      OzTerm &o = p.t[it];
      if (p.K > 0) {
        const OzMatrix &A = pl->mats[mat_of[{img_of(t.a_src), t.a_off}]];
        const OzMatrix &B = pl->mats[mat_of[{img_of(t.b_src), t.b_off}]];
        o.a_img = pl->img[A.src] + (t.ta ? A.img_c : A.img_r);
        o.a_plane = t.ta ? A.plane_c : A.plane_r;
        o.a_rg = t.ta ? A.rg_c : A.rg_r;
        o.b_img = pl->img[B.src] + (t.tb ? B.img_r : B.img_c);
        o.b_plane = t.tb ? B.plane_r : B.plane_c;
        o.b_rg = t.tb ? B.rg_r : B.rg_c;
        IMSRG_TRY(map_of(o.a_img, o.a_plane, t.ta ? A.np_c : A.np_r, 0, &o.a_map));
        IMSRG_TRY(map_of(o.b_img, o.b_plane, t.tb ? B.np_r : B.np_c, 1, &o.b_map));
        if (it == 0) {
          p.gA = A.group;
          p.gB = B.group;
        }
      }
      o.neg = t.coef < 0;
      o.use_hl = t.use_hl;
      o.use_hr = t.use_hr;
    }
    // exactness bound of the FP32 level accumulators (levels 2..4 are exact
    // integers while their sums stay below 2^24; each of their products adds
    // at most 5 x 2^12 per element): a chunk holds at most kOzChunkSteps steps of
    // TK, and longer contractions run in several chunks
    {
      const int steps = p.nterms * p.ksteps;
      const int lim = std::min(oz_chunk_steps(pl->S), std::max(1, pl->chunk_steps));
      p.kchunk = std::max(1, std::min(steps, lim));
      p.nchunks = steps > 0 ? (steps + p.kchunk - 1) / p.kchunk : 0;
      if (p.nchunks > 1) pl->chunked = true;
    }
    const int TN = oz_tn(pl->S);
    p.tiles_m = (p.M + TM - 1) / TM;
    p.tiles = p.tiles_m * ((p.N + TN - 1) / TN);
    p.tile0 = tiles;
    tiles += p.tiles;
    for (int k = 0; k < p.tiles; k++) {
      const int live_m = std::min(TM, p.M - (k % p.tiles_m) * TM), live_n = std::min(TN, p.N - (k / p.tiles_m) * TN);
      tile_ksteps.push_back(p.nterms * p.ksteps);
      tile_live.push_back((64 * live_m * live_n) / (TM * TN));
      tile_slot.push_back(make_int2((int)pl->probs.size(), k));
    }
    pl->probs.push_back(p);
  }
  pl->nmats = (int)pl->mats.size();
  pl->nprobs = (int)pl->probs.size();
  pl->ntiles = tiles;
  pl->grid = std::min(nsm, std::max(tiles, 1));

  std::vector<int2> sched;
  std::vector<int> sched_off;
  build_sched(pl, kSchedModels[0], sched, sched_off);

  auto up = [&](const void *h, size_t bytes, void **d) -> int {
    IMSRG_CUDA_TRY(cudaMalloc(d, std::max<size_t>(bytes, 16)));
    if (bytes) IMSRG_CUDA_TRY(cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice));
    return IMSRG_OK;
  };
  IMSRG_TRY(up(pl->mats.data(), pl->mats.size() * sizeof(OzMatrix), (void **)&pl->d_mats));
  IMSRG_TRY(up(chunks.data(), chunks.size() * sizeof(OzChunk), (void **)&pl->d_chunks));
  IMSRG_TRY(up(pl->probs.data(), pl->probs.size() * sizeof(OzProb), (void **)&pl->d_probs));
  IMSRG_TRY(up(sched.data(), sched.size() * sizeof(int2), (void **)&pl->d_sched));
  IMSRG_TRY(up(sched_off.data(), sched_off.size() * sizeof(int), (void **)&pl->d_sched_off));
  IMSRG_TRY(up(blk_mat.data(), blk_mat.size() * sizeof(int), (void **)&pl->d_blk_mat));
  // (cudaMalloc memory is 256-byte aligned: the 64-byte alignment of a tensor map holds)
  IMSRG_TRY(up(pl->maps.data(), pl->maps.size() * sizeof(CUtensorMap), (void **)&pl->d_maps));
  std::vector<int2> ccg(b->ccblocks);
  for (int q1 = 0; q1 < b->ccblocks; q1++)
    ccg[q1] = make_int2(pl->group_lo[2] + q1, pl->group_lo[2] + b->ccblocks + q1);
  IMSRG_TRY(up(ccg.data(), ccg.size() * sizeof(int2), (void **)&pl->d_ccgroups));
  IMSRG_CUDA_TRY(cudaMalloc((void **)&pl->d_exps, std::max(pl->ngroups, 1) * sizeof(int)));
  IMSRG_CUDA_TRY(cudaMalloc((void **)&pl->d_err, sizeof(int)));
  IMSRG_CUDA_TRY(cudaMemset(pl->d_err, 0, sizeof(int)));
  {
    const int sm = oz_mma_smem(pl->S);
    const void *by_s[5][2] = {{(const void *)k_oz_mma<4, false>, (const void *)k_oz_mma<4, true>},
                              {(const void *)k_oz_mma<5, false>, (const void *)k_oz_mma<5, true>},
                              {(const void *)k_oz_mma<6, false>, (const void *)k_oz_mma<6, true>},
                              {(const void *)k_oz_mma<7, false>, (const void *)k_oz_mma<7, true>},
                              {(const void *)k_oz_mma<8, false>, (const void *)k_oz_mma<8, true>}};
    const void *const *fn = by_s[pl->S - 4];
    for (int v = 0; v < 2; v++) IMSRG_CUDA_TRY(cudaFuncSetAttribute(fn[v], cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  }

  int herr = 0;
  IMSRG_CUDA_TRY(cudaMemcpy(&herr, pl->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return IMSRG_ERR_TIMEOUT;
  pl->ok = true;
  return IMSRG_OK;
}

int ozaki_cc_exponents(imsrg_basis *b, cudaStream_t st, int **exps, int *gL, int *gR) {
  OzPlan *pl = plan_of(b);
  *exps = nullptr;
  if (!pl || !pl->ok || !b->T.ccf_packed) return IMSRG_OK;
  const int g0 = pl->group_lo[2], g1 = pl->group_lo[3];
  if (g1 > g0) IMSRG_CUDA_TRY(cudaMemsetAsync(pl->d_exps + g0, 0, (g1 - g0) * sizeof(int), st));
  *exps = pl->d_exps;
  *gL = g0;
  *gR = g0 + b->ccblocks;
  return IMSRG_OK;
}

int ozaki_slice(imsrg_basis *b, const double *L, const double *R, int part, cudaStream_t st, bool exps_ready) {
  OzPlan *pl = plan_of(b);
  if (!pl) return IMSRG_ERR_INVALID;
  ProfScope ps(b, IMSRG_KERNEL_OZAKI_SLICE, st);
  if (part < 0 || part > 2) return IMSRG_ERR_INVALID;
  const int g0 = pl->group_lo[part], g1 = pl->group_lo[part + 1];
  const int k0 = pl->chunk_lo[part], k1 = pl->chunk_lo[part + 1];
  if (g1 > g0 && !exps_ready) IMSRG_CUDA_TRY(cudaMemsetAsync(pl->d_exps + g0, 0, (g1 - g0) * sizeof(int), st));
  if (k1 > k0 && !exps_ready) {
    k_oz_exponents<<<k1 - k0, 256, 0, st>>>(pl->d_chunks + k0, L, R, b->lcc, b->rcc, pl->d_exps);
    b->launches++;
  }
  const int nblk = pl->cblocks[part] + pl->rblocks[part];
  if (nblk) {
    (pl->S == 4 ? k_oz_slice<4> : pl->S == 5 ? k_oz_slice<5> : pl->S == 6 ? k_oz_slice<6> : pl->S == 7 ? k_oz_slice<7> : k_oz_slice<8>)<<<nblk, SLICE_THREADS, 0, st>>>(pl->d_mats, pl->nmats, pl->d_blk_mat + pl->blk_off[part], pl->cblocks[part],
                                     pl->linec_lo[part], pl->linec_lo[part + 1], pl->liner_lo[part],
                                     pl->liner_lo[part + 1], L, R, b->lcc, b->rcc, pl->d_exps, pl->img[0],
                                     pl->img[1], pl->img[2], pl->img[3]);
    b->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int ozaki_mma(imsrg_basis *b, int hL, int hR) {
  OzPlan *pl = plan_of(b);
  if (!pl) return IMSRG_ERR_INVALID;
  if (!pl->tuned) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    IMSRG_CUDA_TRY(cudaStreamIsCapturing(b->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone) IMSRG_TRY(autotune(b, pl, hL, hR));
  }
  ProfScope ps(b, IMSRG_KERNEL_OZAKI_MMA);
  launch_mma(pl->S, pl->chunked, pl->grid, b->stream, pl->d_probs, pl->nprobs, pl->d_sched, pl->d_sched_off, pl->d_exps, hL, hR,
             pl->d_err, pl->d_maps);
  b->launches++;
  return cuda_status(cudaGetLastError());
}

int ozaki_check_error(imsrg_basis *b) {
  OzPlan *pl = plan_of(b);
  if (!pl || !pl->d_err) return IMSRG_OK;
  return synchronize_checked(b);
}

// The engine's error flag comes back into a page-locked slot queued behind
// the work, so one stream synchronisation serves both.
int synchronize_checked(imsrg_basis *b) {
  OzPlan *pl = plan_of(b);
  int *slot = reinterpret_cast<int *>(b->h_scal + 63);
  *slot = 0;
  if (pl && pl->d_err)
    IMSRG_CUDA_TRY(cudaMemcpyAsync(slot, pl->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (*slot) {
    cudaMemsetAsync(pl->d_err, 0, sizeof(int), b->stream);
    return IMSRG_ERR_TIMEOUT;
  }
  return IMSRG_OK;
}

int ozaki_wcc_scale(imsrg_basis *b, const int **exps, const int2 **ccgroups, int *kshift) {
  OzPlan *pl = plan_of(b);
  if (!pl || !pl->ok) return IMSRG_ERR_INVALID;
  // FP64-class digit counts store WCC as FP64: the recoupling inputs read it so
  *exps = oz_fp64_class(pl->S) ? nullptr : pl->d_exps;
  *ccgroups = pl->d_ccgroups;
  *kshift = 7 * (pl->S + 1);
  return IMSRG_OK;
}

bool ozaki_tuned(imsrg_basis *b) {
  OzPlan *pl = plan_of(b);
  return pl && pl->ok && pl->tuned;
}

// Pins the CTA schedule to one cost model instead of timing them all (for
// runs whose event timings are distorted, e.g. under a profiler that
// serialises launches).  Timings read back as 0 for a pinned schedule.
int ozaki_set_schedule(imsrg_basis *b, int model) {
  if (model < 0 || model >= kNumSchedModels) return IMSRG_ERR_INVALID;
  IMSRG_TRY(ozaki_prepare(b));
  OzPlan *pl = plan_of(b);
  if (!pl || !pl->ok) return IMSRG_ERR_INVALID;
  IMSRG_TRY(use_model(b, pl, model));
  for (int c = 0; c < kNumSchedModels; c++) pl->tune_us[c] = 0.0;
  pl->tune_choice = model;
  pl->tuned = true;
  return IMSRG_OK;
}

int ozaki_schedule_info(imsrg_basis *b, int *choice, int *ncand, double *us, int max) {
  OzPlan *pl = plan_of(b);
  if (!pl || !pl->ok || !pl->tuned) return IMSRG_ERR_INVALID;
  if (choice) *choice = pl->tune_choice;
  if (ncand) *ncand = kNumSchedModels;
  if (us)
    for (int k = 0; k < kNumSchedModels && k < max; k++) us[k] = pl->tune_us[k];
  return IMSRG_OK;
}

// ---------------------------------------------------------------------------
// One persistent launch for the products of several bases.  Every problem
// keeps its own output pointer; its exponent groups and tensor maps are
// renumbered into merged arrays, and the tiles of all bases are assigned
// longest first over one grid.  Each basis's slicing still writes its own
// exponents; ozaki_batch_mma gathers them (one small copy per basis) before
// the launch.  Tiles compute exactly as in a basis's own launch, so results
// are bit-identical.
namespace {
struct OzBatch {
  std::vector<OzPlan *> plans;
  std::vector<int> exps_base;
  OzProb *d_probs = nullptr;
  int nprobs = 0, grid = 0, ngroups = 0;
  bool chunked = false;  // some merged problem runs in more than one chunk
  int2 *d_sched = nullptr;
  int *d_sched_off = nullptr, *d_exps = nullptr, *d_err = nullptr;
  CUtensorMap *d_maps = nullptr;
  ~OzBatch() {
    cudaFree(d_probs);
    cudaFree(d_sched);
    cudaFree(d_sched_off);
    cudaFree(d_exps);
    cudaFree(d_err);
    cudaFree(d_maps);
  }
};
}  // namespace

int ozaki_batch_create(imsrg_basis *const *bases, int n, void **out) {
  *out = nullptr;
  if (n <= 0) return IMSRG_ERR_INVALID;
  OzBatch *bt = new OzBatch();
  auto fail = [&](int s) {
    delete bt;
    return s;
  };
  OzPlan all;  // the merged tile list, for build_sched
  std::vector<OzProb> probs;
  std::vector<CUtensorMap> maps;
  int model = -1;
  for (int i = 0; i < n; i++) {
    const int s = ozaki_prepare(bases[i]);
    if (s != IMSRG_OK) return fail(s);
    OzPlan *pl = plan_of(bases[i]);
    if (!pl || !pl->ok || bases[i]->device != bases[0]->device) return fail(IMSRG_ERR_INVALID);
    bt->plans.push_back(pl);
    bt->chunked = bt->chunked || pl->chunked;
    if (pl->S != bt->plans[0]->S) return fail(IMSRG_ERR_INVALID);  // one digit count per merged launch
    bt->exps_base.push_back(bt->ngroups);
    const int p0 = (int)probs.size(), m0 = (int)maps.size();
    for (const OzProb &p : pl->probs) {
      OzProb q = p;
      q.inst = i;
      q.gA += bt->ngroups;
      q.gB += bt->ngroups;
      for (int t = 0; t < q.nterms; t++) {
        q.t[t].a_map += m0;
        q.t[t].b_map += m0;
      }
      probs.push_back(q);
    }
    for (size_t k = 0; k < pl->tile_slot.size(); k++) {
      all.tile_ksteps.push_back(pl->tile_ksteps[k]);
      all.tile_live.push_back(pl->tile_live[k]);
      all.tile_slot.push_back(make_int2(pl->tile_slot[k].x + p0, pl->tile_slot[k].y));
    }
    maps.insert(maps.end(), pl->maps.begin(), pl->maps.end());
    bt->ngroups += pl->ngroups;
    // the bases' own tuned cost model when they agree, else the one usually chosen
    const int m = pl->tuned ? pl->tune_choice : 1;
    model = (model < 0 || model == m) ? m : 1;
  }
  int nsm = 0;
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, bases[0]->device));
  all.grid = std::min(nsm, std::max((int)all.tile_slot.size(), 1));
  std::vector<int2> sched;
  std::vector<int> sched_off;
  build_sched(&all, kSchedModels[model < 0 ? 1 : model], sched, sched_off);
  bt->grid = all.grid;
  bt->nprobs = (int)probs.size();
  auto up = [&](const void *h, size_t bytes, void **d) -> int {
    IMSRG_CUDA_TRY(cudaMalloc(d, std::max<size_t>(bytes, 16)));
    if (bytes) IMSRG_CUDA_TRY(cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice));
    return IMSRG_OK;
  };
  int s = IMSRG_OK;
  if (s == IMSRG_OK) s = up(probs.data(), probs.size() * sizeof(OzProb), (void **)&bt->d_probs);
  if (s == IMSRG_OK) s = up(sched.data(), sched.size() * sizeof(int2), (void **)&bt->d_sched);
  if (s == IMSRG_OK) s = up(sched_off.data(), sched_off.size() * sizeof(int), (void **)&bt->d_sched_off);
  // (cudaMalloc memory is 256-byte aligned: the 64-byte alignment of a tensor map holds)
  if (s == IMSRG_OK) s = up(maps.data(), maps.size() * sizeof(CUtensorMap), (void **)&bt->d_maps);
  if (s == IMSRG_OK) s = cuda_status(cudaMalloc((void **)&bt->d_exps, std::max(bt->ngroups, 1) * sizeof(int)));
  const int zero = 0;
  if (s == IMSRG_OK) s = up(&zero, sizeof(int), (void **)&bt->d_err);
  if (s != IMSRG_OK) return fail(s);
  *out = bt;
  return IMSRG_OK;
}

int ozaki_batch_mma(void *batch, cudaStream_t st, int hL, int hR, const int *act) {
  OzBatch *bt = (OzBatch *)batch;
  if (!bt) return IMSRG_ERR_INVALID;
  for (size_t i = 0; i < bt->plans.size(); i++)
    if (bt->plans[i]->ngroups > 0)
      IMSRG_CUDA_TRY(cudaMemcpyAsync(bt->d_exps + bt->exps_base[i], bt->plans[i]->d_exps,
                                     bt->plans[i]->ngroups * sizeof(int), cudaMemcpyDeviceToDevice, st));
  launch_mma(bt->plans[0]->S, bt->chunked, bt->grid, st, bt->d_probs, bt->nprobs, bt->d_sched, bt->d_sched_off,
             bt->d_exps, hL, hR, bt->d_err, bt->d_maps, act);
  return cuda_status(cudaGetLastError());
}

int ozaki_batch_error(void *batch, cudaStream_t st) {
  OzBatch *bt = (OzBatch *)batch;
  if (!bt) return IMSRG_ERR_INVALID;
  int h = 0;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(&h, bt->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
  if (h) {
    cudaMemsetAsync(bt->d_err, 0, sizeof(int), st);
    return IMSRG_ERR_TIMEOUT;
  }
  return IMSRG_OK;
}

void ozaki_batch_free(void *batch) { delete (OzBatch *)batch; }

void ozaki_free(imsrg_basis *b) {
  OzPlan *pl = plan_of(b);
  if (!pl) return;
  for (int s = 0; s < 4; s++) cudaFree(pl->img[s]);
  cudaFree(pl->d_mats);
  cudaFree(pl->d_chunks);
  cudaFree(pl->d_probs);
  cudaFree(pl->d_sched);
  cudaFree(pl->d_sched_off);
  cudaFree(pl->d_blk_mat);
  cudaFree(pl->d_ccgroups);
  cudaFree(pl->d_exps);
  cudaFree(pl->d_maps);
  cudaFree(pl->d_err);
  delete pl;
  b->ozaki = nullptr;
}

}  // namespace imsrg
