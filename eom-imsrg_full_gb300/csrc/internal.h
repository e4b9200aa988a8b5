// internal.h -- shared declarations of the imsrg_gpu library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/imsrg_gpu.h"

namespace imsrg {

// Device-resident basis tables, passed by value to every kernel.  Orbits are
// 0-based here; angular momenta stay doubled as in the reference.
struct DevTables {
  int norb, A, P, nblocks, jtm, nJ, nj, ccblocks;
  long off_fhh, off_fph, off_fpp, nfull;
  const int4 *orb;         // x = jj, y = ll, z = itzp, w = con
  const int *orbpos;       // position among holes (con=1) or particles (0-based)
  const int *pairrow;      // [(a*norb+b)*nJ + J2/2], a<=b: row in its category, -1 if absent
  const long *gam_off;     // [q*6+g] (g 0-based) flat offset
  const int *gam_n1;       // [q*6+g]
  const int *gam_n2;       // [q*6+g]
  const int *blk_J2;       // [q]
  const int *qn;           // pair lists: qn[qn_start[q*3+c] + 2*IX + k], 0-based orbits
  const int *qn_start;     // [q*3+c], c = 0 pp, 1 ph, 2 hh
  const double *six;       // dense 6j table, see sixj_index()
  const double *six_w;     // (J6 + 1) * 6j, same index
  const double *sqrt_j21;  // sqrt(J2 + 1) for J2 = 0, 2, .. (index J2/2)
  const double *jp1;       // (double)(J2 + 1) for J2 = 0 .. 2*nJ (index J2)
  const int *ljt_start;    // [a]: start of orbits sharing (l,j,tz) with a
  const int *ljt_count;    // [a]
  const int *ljt_list;     // concatenated lists (0-based orbits, ascending)
  const int *cc_row;       // [(q1*norb+i)*norb+j] row (0-based) or -1
  const long *cc_off;      // [q1] offset of CCX(q1) (rlen x nph, column-major)
  const long *wcc_off;     // [q1] offset of WCC(q1) (rlen x rlen)
  const int *cc_rlen;      // [q1]
  const int *cc_nph;       // [q1]
  const int *cc_J2;        // [q1]
  const int *cc_rowpair;   // [cc_rowstart[q1] + r] = a*65536 + b
  const int *cc_rowstart;  // [q1]
  const int *cc_colpair;   // [cc_colstart[q1] + c] = p*65536 + h
  const int *cc_colstart;  // [q1]
  const int *ph_pairs;     // (l,j,tz)-allowed (particle pos, hole pos) pairs: [2*k], [2*k+1]
  int n_ph_pairs;
  const int *hole_orb;     // [hole position] -> orbit
  const int *part_orb;     // [particle position] -> orbit
  // Work orders: elements grouped by identical loop-trip signatures so the
  // lanes of a warp run the same FP64 instruction sequence (GB300 issues an
  // FP64 warp instruction at full cost whatever the active lanes).
  // Two-body elements (upper triangles only): asm2_head[w] is the w-th
  // element of the work order, its commutator_122 terms asm2_terms[head.start
  // ..]; the 222_ph recoupling inputs Z (one per orbit quadruple, channel and
  // J', shared by the quadruple's elements of every J) come from the ph_terms
  // list (see Asm2Head, PhTerm).  asm2_head_out holds the same heads grouped
  // by output range first (imsrg_basis::asm2_el), for copies of RES to the
  // host that run beside the assembly.
  const struct Asm2Head *asm2_head, *asm2_head_out;
  // [flat index] number of sqrt(2) normalisation factors v_elem applies to a
  // stored two-body element (identical-orbit row pair + identical-orbit
  // column pair: 0, 1 or 2)
  const unsigned char *vsq;
  const unsigned long long *asm2_terms;
  int n_asm2;
  const struct PhTerm *ph_terms;
  int n_ph;
  // The commutator_122 sums again, for the kernel that runs them ahead of the
  // products (k_asm2_122): warp g takes elements pre_el[32 g .. 32 g + 32),
  // all with pre_warp[g].n122 terms; term k of its lane l is
  // pre_terms[pre_warp[g].base + 32 k + l] (one coalesced load per term).
  // pre_el: bits 0-27 flat index, 28-29 identical orbit pairs, 30 diagonal;
  // 0xFFFFFFFF pads a warp.
  const struct Asm2PreWarp *pre_warp;
  const unsigned *pre_el;
  const unsigned long long *pre_terms;
  int n_pre_warps;
  const int *ccf_order;    // cross-coupled elements (bits 0-23), with their block in bits 24-30 if ccf_packed
  int n_ccf;
  int ccf_packed;
  // Gather lists of the Pandya transform: element e of every CC block is
  // sum_k cct_coef[k] * op[cct_idx[k] & 0x7fffffff] (bit 31: read transposed,
  // times herm), k in [cct_start[e], cct_start[e + 1]).
  const int *cct_start;
  const int *cct_idx;
  const double *cct_coef;
  // Gather lists of the one-body assembly (121 and 221 sums), per one-body
  // element in flat order: obt[obt_start[e] .. + obt_count[e]).
  const struct OneBodyTerm *obt;
  const int *obt_start;
  const int *obt_count;
  // One-body work split: elements with gather lists (a CTA each, longest
  // first) and the rest (a warp each); mirrored lower triangles are in neither.
  const int *asm1_heavy;
  int n_asm1_heavy;
  const int *asm1_light;
  int n_asm1_light;
  long cc_total, wcc_total;
};

// One term of a one-body sum.  kind 0/1: commutator_121 terms at the two
// locations <a p|i q> and <i p|a q> (idx into L and R, ph = fph offset of the
// (a,i) pair, trans = read transposed); kind 2/3: commutator_221 terms
// <c i|c j> and the -herm(L)herm(R) <c j|c i> term (idx into W1 or W2).
struct OneBodyTerm {
  int idx;
  int meta;     // bits 0-1 kind, bit 2 trans, bit 3 W2 (else W1), bits 8.. ph
  double coef;  // (2J+1) x phase x sqrt(2)^n
};

// One warp of the commutator_122 sums run ahead of the products (see
// DevTables::pre_warp).
struct __align__(16) Asm2PreWarp {
  long long base;  // first term of lane 0
  int n122;
  int pad;
};

// One J'-term of the inverse Pandya recoupling of commutator_222_ph
// (commutators.f90:855-910) for an orbit quadruple (a,b,c,d) and one exchange
// channel: the kernel forms
//   Z = herm_L (W(x1,y1) + e W(x2,y2)) - herm_R (e W(y2,x2) + W(y1,x1))
// from four cross-coupled rows (16 bits each in `rows`: x1, y1, x2, y2;
// 0xFFFF = absent) of WCC block qx, e = (-1)^((ja+jb+jc+jd)/2).  The
// reference's four products per J' become sum_J' {6j} Z(J') per element, with
// the inside channel's (-1)^n2(J) applied after the sum.
struct __align__(16) PhTerm {
  unsigned long long rows;
  int qx;
  int nph;  // the exponent of e
};

// One two-body element of the assembly kernel with its operator-independent
// gather list, resolved once per basis on the host: n122 commutator_122
// terms (:283-396) at asm2_terms[start ..]: bits 0-27 flat index of the
// two-body element V, bits 28-47 flat index of the one-body element f, bit 48
// sign (leg sign x pair-reordering phase), bits 49-50 number of sqrt(2)
// factors, bit 51 V read transposed, bit 52 f read transposed (each transposed
// read takes the operator's herm).  Its recoupling reads Z[zs .. zs + n_in)
// (inside channel) and Z[zs + n_in .. + n_out) (outside) against consecutive
// 6j-table entries from six1 and six2.
struct __align__(16) Asm2Head {
  int e;       // flat index of the element
  int em;      // flat index of its mirror (JX, IX) in a square array, else -1 (== e on the diagonal)
  int start;   // first commutator_122 term
  int zs;      // first recoupling input
  int six1;    // 6j-table index of the first J' of each channel
  int six2;
  unsigned meta;  // bits 0-4 n122, 5-9 n_in, 10-14 n_out, 15 recoupling applies,
                  // 16 inside phase n2, 18-19 identical orbit pairs, 20 diagonal,
                  // 21 square array, 22 pphh array
  int J2;
};

// One term alpha * op(A) * op(B) of a grouped GEMM problem.  Operand ids:
// 0 L, 1 R, 2 W1, 3 W2, 4 LCC, 5 RCC, 6 WCC.
struct GemmTerm {
  int a_src, b_src;
  int ta, tb;        // 1 = transposed
  long a_off, b_off;
  int lda, ldb;
  double coef;
  int use_hl, use_hr;  // multiply coef by herm(L) / herm(R)
  const double *a_abs, *b_abs;  // merged lists of several bases: the operands themselves
};

struct GemmProb {
  int M, N, K, nterms;
  GemmTerm t[2];
  int c_dst;
  long c_off;
  int ldc;
  int tile0;    // first tile id of this problem
  int tiles_m;  // tiles along M
  int tiles;    // tiles of this problem
  int shape;    // FP64 tile: 0 = 64 x 64, 1 = 256 x 8 (problems with N <= 8)
  double *c_abs;  // merged lists of several bases: the output itself
  int inst;       // merged lists: the basis the problem belongs to
};

struct Operands {
  const double *src[7];
  double *dst[7];
};

enum { SRC_L = 0, SRC_R = 1, SRC_W1 = 2, SRC_W2 = 3, SRC_LCC = 4, SRC_RCC = 5, SRC_WCC = 6 };

// Norm segments: chunks of the flat layout with weight 1 or 2.
struct NormChunk {
  long start;
  int len;
  int weight;
};

}  // namespace imsrg

struct imsrg_op;

namespace imsrg {
// Host operands of one commutator (flat layout, nfull doubles each).  pinned:
// all three are page-locked, so copies may run asynchronously beside kernels.
struct HostIO {
  const double *L, *R;
  double *RES;
  bool pinned = false;
  // packed (vectorize-order, neq doubles) host arrays when set: device staging
  // buffers the copies land in, unpacked into L and R on the device; RES is
  // packed into RESst before its one copy back
  double *Lst = nullptr, *Rst = nullptr, *RESst = nullptr;
  // packed page-locked host arrays the device can address (set by
  // commutator_dev): the unpack kernels read L and R, and the pack kernel
  // writes RES, over the host link directly, with no staging copies
  const double *Ldev = nullptr, *Rdev = nullptr;
  double *RESdev = nullptr;
};
// The two-body part of RES is assembled, and copied back to a page-locked host
// result, in this many address ranges, so that each range's copy runs beside
// the assembly of the next.  Two: the assembly is latency-bound and needs
// most of the GPU's warp slots, which a smaller range no longer fills (emax=6:
// 284 us per host-operand commutator with two ranges, 287 with four, 322
// with eight, 291 with one).
constexpr int kOutChunks = 2;
// fraction of the two-body part in the first range (its copy is the one that
// overlaps; the last range's copy is exposed).  Even is best at emax=6: 269
// us per host-operand call, 274 / 277 / 279 with 0.6 / 0.7 / 0.8 (a smaller
// last range fills the GPU less while it is assembled).
constexpr double kOutFirst = 0.5;
}  // namespace imsrg

namespace imsrg {
// Live kernel timing with CUDA events on the basis stream.
struct Profiler {
  bool on = false;
  struct Pending {
    int kind;
    cudaEvent_t start, stop;
  };
  std::vector<cudaEvent_t> pool;
  std::vector<Pending> pending;
  double ms[IMSRG_KERNEL_COUNT] = {};
  long n[IMSRG_KERNEL_COUNT] = {};
};
}  // namespace imsrg

struct imsrg_basis {
  // host copies
  int norb, A, P, nblocks, jtm, ccblocks;
  std::vector<int> nn, ll, jj, itzp, con;
  std::vector<int> holes, parts;  // 0-based orbit ids
  std::vector<int> npp, nph, nhh; // per block
  std::vector<long> gam_off;      // [q*6+g]
  std::vector<int> gam_n1, gam_n2;
  std::vector<std::vector<int>> qn;  // [q*3+c] pair list (0-based, 2 ints per pair)
  std::vector<int> cc_rlen, cc_nph, cc_J2;
  std::vector<int> pairrow;          // [(a * norb + b) * (jtm + 1) + J2 / 2] row of pair a <= b in its block
  std::vector<long> cc_off, wcc_off;
  long nfull = 0, neq = 0, cc_total = 0, wcc_total = 0;
  long off_fhh = 1, off_fph = 0, off_fpp = 0;

  // device
  imsrg::DevTables T{};
  std::vector<void *> dev_allocs;
  cudaStream_t stream = nullptr;      // where all work is enqueued
  cudaStream_t own_stream = nullptr;  // the library's own stream
  // Library streams for independent launches inside one commutator, forked
  // from and joined back into `stream` with events.
  // side3 runs E0 (one CTA) from the first fork to the end; side4 the
  // commutator_122 sums, which need only L and R, beside the Pandya transform,
  // the digit images and the products.
  cudaStream_t side = nullptr, side2 = nullptr, side3 = nullptr, side4 = nullptr;
  cudaEvent_t ev_pre = nullptr;    // the commutator_122 sums are in RES
  cudaEvent_t ev_rdev = nullptr;   // a packed host operand R is unpacked on the device
  cudaEvent_t ev_fork[2] = {nullptr, nullptr}, ev_join[2] = {nullptr, nullptr}, ev_join2 = nullptr;
  cudaEvent_t ev_join3 = nullptr;
  cudaEvent_t ev_hostL = nullptr;  // a host operand L has arrived (commutator_host)
  cudaEvent_t ev_hostR = nullptr;  // a host operand R has arrived
  cudaEvent_t ev_out[imsrg::kOutChunks] = {}, ev_outj = nullptr;  // chunked copy of RES to the host
  // Two-body work order by output range: elements asm2_el[c] .. asm2_el[c+1]
  // write only RES[asm2_addr[c] ..) (the mirror of a square-array element
  // lies at a lower address, so an element belongs to the range of its lower
  // write); RES[asm2_addr[c] .. asm2_addr[c+1]) is final once every range up
  // to c is assembled.
  long asm2_el[imsrg::kOutChunks + 1] = {}, asm2_addr[imsrg::kOutChunks + 1] = {};
  int device = 0;
  int num_sms = 1;  // multiprocessors of the device
  imsrg::Profiler prof;
  // commutator workspace
  double *w1 = nullptr, *w2 = nullptr, *lcc = nullptr, *rcc = nullptr, *wcc = nullptr;
  double *zph = nullptr;        // 222_ph recoupling inputs (T.n_ph)
  long off_2b = 0;              // first two-body index of the flat layout
  double *mono = nullptr;       // 2 x norb x norb monopole tables of the White generator (H, tangent dH)
  double *scal = nullptr;       // small device scratch for reductions (E0, norms)
  double *partials = nullptr;   // norm/mbpt2 partial sums
  double *h_scal = nullptr;     // pinned host mirror of scal
  int partials_len = 0;
  // grouped GEMM problems
  imsrg::GemmProb *d_probs = nullptr;
  int nprobs = 0, ntiles = 0;
  std::vector<imsrg::GemmProb> probs;
  // norm chunks
  imsrg::NormChunk *d_chunks = nullptr;
  int nchunks = 0;
  // packed layout map: packed index k -> flat index, and mirrored flat index (or -1)
  long *d_pack_src = nullptr, *d_pack_mirror = nullptr;
  // staging buffer (pinned) for Fortran-style uploads/downloads
  double *h_stage = nullptr;
  double *d_stage = nullptr;  // device staging for packed uploads
  // flow temporaries (allocated on first use)
  std::vector<imsrg_op *> tmp_ops;
  long launches = 0;
  // Ozaki split-precision engine state (allocated on first use)
  void *ozaki = nullptr;
  int split_digits = 6;  // digits per operand of the split engine (4 to 8), fixed once its plan exists
  int split_chunk_steps = 0;  // K steps per exact accumulator chunk (0: the largest exact one)
  // Reverse-mode (adjoint) workspace (adjoint.cu), allocated on first use
  void *adjoint = nullptr;
  // Graph of one Magnus flow step (graph.cu), built on first use
  void *flowgraph = nullptr;
  // Captured commutator launch sequences, one per argument set (api.cpp)
  struct CommGraph {
    const double *L, *R;
    double *RES;
    int hL, hR, hRES, precision, with_e0;
    imsrg::HostIO io;  // host operands copied in and out by the graph (all null if none)
    cudaGraphExec_t exec;
    long last_use;
    long nlaunch;  // library kernel launches in the sequence
  };
  std::vector<CommGraph> comm_graphs;
  long comm_calls = 0;
};

struct imsrg_op {
  imsrg_basis *b;
  double *d;  // nfull doubles on device
  int herm;
};

namespace imsrg {

int build_basis(imsrg_basis *b);            // host tables + device upload (basis.cpp)
// Where v_elem (basic_IMSRG.f90:1270-1385) finds <a b|V|c d>_J in the flat
// layout (idx -1: structurally zero) and how it modifies the stored value.
struct HLoc {
  long idx;   // flat index, -1 if structurally zero
  int neg;    // pair-reordering phase
  int nsq;    // sqrt(2) normalisation factors
  int trans;  // read transposed (times herm)
};
HLoc v_location(const imsrg_basis *b, int a, int bb, int c, int d, int J2);
// {a b c; d e f} with doubled arguments (host, exact Racah sum)
double sixj(int a, int b, int c, int d, int e, int f);
void free_basis_device(imsrg_basis *b);
int cuda_status(cudaError_t e);

// Threads per CTA of the two-body assembly; its commutator_220 partials are
// one per CTA.
constexpr int ASM2_THREADS = 128;
inline int asm2_ctas(const imsrg_basis *b) { return (b->T.n_asm2 + ASM2_THREADS - 1) / ASM2_THREADS; }

// launchers (kernels_*.cu); all enqueue on b->stream and bump b->launches
// Pandya transform into b->lcc, b->rcc; exps != nullptr: also the largest
// exponent of each LCC block q1 into exps[gL + q1] and RCC block into exps[gR + q1];
// sides 1 / 2 / 3: LCC only, RCC only, both; st = nullptr: the basis stream
int launch_cc_forward(imsrg_basis *b, const double *L, int hL, const double *R, int hR, int *exps = nullptr,
                      int gL = 0, int gR = 0, int sides = 3, cudaStream_t st = nullptr);
int launch_gemm_fp64(imsrg_basis *b, const double *L, int hL, const double *R, int hR);
// The FP64 products of several bases (operators L[i], R[i] of bases[i]) as one
// problem list with absolute pointers, uploaded to *d_probs (cudaFree it).
int gemm_fp64_merged(imsrg_basis *const *bases, int n, const double *const *L, const double *const *R,
                     GemmProb **d_probs, int *nprobs, int *ntiles);
// one launch of a merged list; act (optional, one int per basis): only the
// bases with act[i] != 0 take part
int launch_gemm_fp64_merged(const GemmProb *d_probs, int nprobs, int ntiles, int hL, int hR, const int *act,
                            cudaStream_t st);
// the two-body assembly: the recoupling inputs of 222_ph, then the elements
// [w0, w1) of the signature work order or of the order by output range, on
// top of launch_asm2_122's part in RES
int launch_ph_inputs(imsrg_basis *b, int hL, int hR, int precision);
// commutator_122 part of every two-body element into RES on stream st (the
// assembly after the products adds the rest)
int launch_asm2_122(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                    cudaStream_t st);
int launch_asm2_range(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                      long w0, long w1, bool by_range);
int launch_assemble_1body(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                          cudaStream_t st);
// E0 of [L, R] into RES[0] on stream st (independent of the assembly kernels)
int launch_e0(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, cudaStream_t st);
int launch_axpby(imsrg_basis *b, const double *A, double ax, const double *B, double bx, double *C);
int launch_axpby_dev(imsrg_basis *b, const double *A, double ax, const double *B, const double *bx, double *C);
// S += *coef_dev X1, X0 = X1 (unless X0 is null), *d_norm = mat_frob_norm(X1):
// one series term's bookkeeping in one pass over X1 (the same values as
// launch_axpby_dev, a copy and launch_norm).  d_norm null: the norm's
// partials stay in b->partials (b->nchunks of them) for a kernel that sums
// them with block_sum_ops in k_final_sum's order
int launch_series_update(imsrg_basis *b, double *S, const double *X1, const double *coef_dev, double *X0,
                         double *d_norm);
int launch_norm(imsrg_basis *b, const double *op, double *d_out);
int launch_mbpt2(imsrg_basis *b, const double *H, int herm, double *d_out);
int launch_white(imsrg_basis *b, const double *H, int hH, double *ETA);
int launch_generator(imsrg_basis *b, const double *Hden, int hH, const double *Hnum, int use_atan, double *ETA);
int launch_white_tangent(imsrg_basis *b, const double *H, const double *dH, int hH, double *dETA);
// Hb += (d White / d H)^T ETAb (reverse mode; monob: norb x norb scratch)
int launch_white_adjoint(imsrg_basis *b, const double *H, int hH, const double *ETAb, double *Hb, double *monob);
// (un)pack between the flat layout and vectorize order; `packed` may be
// device-addressable page-locked host memory (to_host: a grid sized for
// writes over the host link)
int launch_pack(imsrg_basis *b, const double *flat, double *packed, cudaStream_t st = nullptr, bool to_host = false);
int launch_unpack(imsrg_basis *b, const double *packed, int herm, double *flat, cudaStream_t st = nullptr);
int launch_check_finite(imsrg_basis *b, const double *op, int *d_flag);
int launch_normal_order(imsrg_basis *b, const double *Tin, int herm, double *H);

// Intermediates of one commutator: W1, W2 (flat operators), LCC, RCC (all
// cross-coupled blocks) and WCC.
struct Workspace {
  double *w1, *w2, *lcc, *rcc, *wcc, *zph;
  double *e0p;  // per-CTA commutator_220 partials of the two-body kernel
};
int launch_commutator_fp64_ws(imsrg_basis *b, const Workspace &ws, const double *L, int hL, const double *R, int hR,
                              double *RES, int hRES, int with_e0, cudaStream_t st);
// Loads the device code of every kernel launch_commutator_fp64_ws launches on
// the current device (with lazy module loading a kernel's module is otherwise
// loaded, and may allocate, at its first launch).
int preload_commutator_fp64_ws();

// Ozaki split-precision contraction engine (ozaki.cu)
int ozaki_prepare(imsrg_basis *b);  // plans and allocates the engine once; errors if unavailable
// part 0: exponents and digit images of L; part 1: of R; part 2: of LCC and
// RCC (after the Pandya transform).  ozaki_mma then runs every contraction.
// exps_ready: the part's block exponents are already in place (part 2: the
// Pandya transform reduced them, see ozaki_cc_exponents).
int ozaki_slice(imsrg_basis *b, const double *L, const double *R, int part, cudaStream_t st,
                bool exps_ready = false);
// Where the Pandya transform may leave the LCC/RCC block exponents (zeroed on
// st here): exps[gL + q1], exps[gR + q1]; *exps = nullptr if it cannot.
int ozaki_cc_exponents(imsrg_basis *b, cudaStream_t st, int **exps, int *gL, int *gR);
int ozaki_mma(imsrg_basis *b, int hL, int hR);
int ozaki_check_error(imsrg_basis *b);  // IMSRG_ERR_TIMEOUT if a bounded device wait gave up
// synchronise the basis stream and then check as ozaki_check_error, with one
// synchronisation (the flag is read back behind the work)
int synchronize_checked(imsrg_basis *b);
bool ozaki_tuned(imsrg_basis *b);       // the CTA schedule has been autotuned
// After a split-precision product WCC holds exact int64 level sums v with
// WCC = v 2^k, k = (exps[g.x] - 1022) + (exps[g.y] - 1022) - kshift for the
// groups g = ccgroups[q1] of cross-coupled block q1 (kshift = 7 (S + 1) for S
// digits: 49 with six, 42 with five).
int ozaki_wcc_scale(imsrg_basis *b, const int **exps, const int2 **ccgroups, int *kshift);
int ozaki_schedule_info(imsrg_basis *b, int *choice, int *ncand, double *us, int max);
int ozaki_set_schedule(imsrg_basis *b, int model);  // pin one cost model, no timing
void ozaki_free(imsrg_basis *b);
// The products of several bases as one persistent launch (a batch of
// independent commutators): ozaki_batch_create merges the bases' plans,
// ozaki_batch_mma gathers their block exponents and launches on st,
// ozaki_batch_error reads (and clears) the bounded-wait flag.
int ozaki_batch_create(imsrg_basis *const *bases, int n, void **out);
// act (optional, one int per basis): only the bases with act[i] != 0 take part
int ozaki_batch_mma(void *batch, cudaStream_t st, int hL, int hR, const int *act = nullptr);
int ozaki_batch_error(void *batch, cudaStream_t st);
void ozaki_batch_free(void *batch);

// Reverse mode (adjoint.cu): Yb = d<Cb, [X, Y]> / dY (herm(X) = hX,
// herm(Y) = hY; with_e0 = 0 ignores Cb[0]); FP64, overwrites Yb.
int adjoint_prepare(imsrg_basis *b);
void adjoint_free(imsrg_basis *b);
int commutator_adjoint_dev(imsrg_basis *b, const double *X, int hX, const double *Cb, int hY, int with_e0,
                           double *Yb);
int dot_dev(imsrg_basis *b, const double *x, const double *y, long n, double *out);  // fixed order
double *adjoint_monob(imsrg_basis *b);  // norb x norb scratch of the White adjoint

// Magnus flow step as a CUDA graph (graph.cu)
int flow_tmp_ops(imsrg_basis *b, imsrg_op **H0, imsrg_op **DG, imsrg_op **X0, imsrg_op **X1);  // api.cpp
// work operator k of the basis (created on first use; 15 and 16 belong to the ODE flow)
int work_op(imsrg_basis *b, int k, imsrg_op **out);
// dHds (IMSRG_ODE.f90:416-463): DH = [eta(HS), HS] with generator IMSRG_GEN_*
int dhds_dev(imsrg_basis *b, const double *HS, int hH, double *DH, int generator, int precision);
int flow_graph_begin(imsrg_op *HS, imsrg_op *G, int precision, double ds, double *e0, double *emp2);
int flow_graph_set_s(imsrg_basis *b, double s);  // a flow restarted at s
int flow_graph_launch(imsrg_basis *b);
int flow_graph_finish(imsrg_basis *b, double *s, double *e0, double *emp2, int *nc, int *status);
void flow_graph_free(imsrg_basis *b);
// Lockstep batched Magnus flows of the bases of one batch (graph.cu): each
// step one graph for all instances, the split products of all running series
// in one masked launch per term; the graph is cached in *cache (freed by
// batch_flow_free).
int batch_flow_run(imsrg_basis *const *bases, int n, void *oz, cudaStream_t st, void **cache,
                   imsrg_op *const *HS, imsrg_op *const *G, double s_max, double ds, int max_steps, int precision,
                   double *const *traces, int *steps, int *ncomm, int *status);
void batch_flow_free(void *cache);

// Records CUDA events around the launches of one kernel class while profiling
// is enabled (profile.cpp).
struct ProfScope {
  imsrg_basis *b;
  int kind;
  cudaEvent_t start = nullptr;
  cudaStream_t st = nullptr;
  ProfScope(imsrg_basis *b, int kind, cudaStream_t st = nullptr);
  ~ProfScope();
};
int profile_collect(imsrg_basis *b);
void profile_free(imsrg_basis *b);

// one full commutator (api.cpp); io != nullptr: L and R are first copied
// from io->L, io->R (host) and RES is copied to io->RES afterwards, all on the
// basis stream
int commutator_dev(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                   int precision, int with_e0, const HostIO *io = nullptr);
// parts of the launch sequence of one commutator (device operands for any
// part short of kPhaseAll)
constexpr int kPhaseFront = 1, kPhaseProducts = 2, kPhaseBack = 4, kPhaseAll = 7;
// with the phases: the E0 side stream joins at the end of the front phase (not
// in the back phase), so front and back can be captured into separate graphs
constexpr int kPhaseJoinE0Front = 8;
int commutator_launches(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                        int precision, int with_e0, const HostIO *io, int phases);

}  // namespace imsrg

#define IMSRG_CUDA_TRY(expr)                           \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return imsrg::cuda_status(_e); \
  } while (0)

#define IMSRG_TRY(expr)          \
  do {                           \
    int _s = (expr);             \
    if (_s != IMSRG_OK) return _s; \
  } while (0)
