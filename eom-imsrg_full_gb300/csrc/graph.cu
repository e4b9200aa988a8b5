// graph.cu -- the Magnus flow step as one CUDA graph with device-side loops.
//
// One step of magnus_decouple (IMSRG_MAGNUS.f90:15-128) is MAGNUS_EXPAND
// (:622-693), euler_step (:756-766), BCH_EXPAND (:149-234), then the White
// generator and the MBPT2 stop criterion.  The two series stop on norms of
// their latest term, which the host path reads back term by term.  Here the
// step is captured once per operator set into a graph whose series are
// conditional WHILE nodes: after each term a one-thread control kernel
// updates the series state in device memory (the FlowDev struct) and sets the
// loop's condition with cudaGraphSetConditional.  The host launches one graph
// per step and reads back only the step's scalars.
//
// The graph runs the same kernels in the same order on the same data as the
// host-driven path, so both give bit-identical operators.  The one structural
// difference: the host path alternates two commutator buffers, the graph
// copies the new term back into the input buffer (a graph body has fixed
// kernel arguments).
//
// Batched flows: independent instances (each with its own basis, hence its
// own workspace and streams) launch their step graphs back to back on their
// own streams, so their kernels overlap on the device; each instance's
// results equal its unbatched flow bit for bit.
#include <cmath>
#include <vector>

#include "device.cuh"
#include "internal.h"

namespace imsrg {

namespace {

// Truncated Bernoulli coefficients of IMSRG_MAGNUS.f90:648.
__constant__ double c_cof[7] = {1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5};
const double kConv = 1e-6;

struct FlowDev {
  double adv[8];   // the reference's advals: scaled norms of the Magnus terms
  double fullnorm; // norm of Omega
  double nrm;      // norm of the latest commutator
  double cof;      // coefficient of the current Magnus term
  double coef;     // 1/n! of the current BCH term
  double s, e0, emp2;
  int i, q;        // Magnus term index and the reference's look-back
  int iw;          // BCH term index
  int nc;          // commutators of this step
  int status;      // IMSRG_OK or the error of a series
  int pad;
};

// The pre-test of Magnus term i (IMSRG_MAGNUS.f90:660-674): stop when the
// previous (non-zero-coefficient) term is small against Omega.  Returns
// whether term i runs.
__device__ unsigned magnus_go(FlowDev *F) {
  unsigned go = 0;
  const int i = F->i;
  if (F->status == IMSRG_OK && i <= 7 && !(F->fullnorm < 1e-9)) {
    const double adnorm = F->adv[i - F->q];
    F->q = (fabs(c_cof[i - 1]) > 1e-6) ? 1 : 2;
    go = !(fabs(adnorm / F->fullnorm) < kConv);
    F->cof = c_cof[i - 1];
  }
  return go;
}

__device__ unsigned magnus_init_go(FlowDev *F) {
  F->adv[0] = 0.0;
  for (int k = 2; k < 8; k++) F->adv[k] = 0.0;
  F->i = 2;
  F->q = 1;
  F->nc = 0;
  F->status = IMSRG_OK;
  return magnus_go(F);
}

__device__ unsigned magnus_next_go(FlowDev *F) {
  F->nc++;
  const double nrm = F->nrm;
  if (!isfinite(nrm)) {
    F->status = IMSRG_ERR_NONFINITE;
    return 0;
  }
  F->adv[F->i] = nrm * fabs(c_cof[F->i - 1]);
  F->i++;
  return magnus_go(F);
}

__device__ unsigned bch_init_go(FlowDev *F, double ds) {
  F->s += ds;
  F->iw = 2;
  F->coef = 1.0;  // 1/(iw - 1)! at iw = 2
  return F->status == IMSRG_OK ? 1u : 0u;
}

// After BCH term iw (IMSRG_MAGNUS.f90:207-231): stop when |term| / n! < conv;
// 39 terms without convergence is the reference's 'clipping BCH'.
__device__ unsigned bch_next_go(FlowDev *F) {
  F->nc++;
  const double nrm = F->nrm;
  unsigned go = 1;
  if (!isfinite(nrm)) {
    F->status = IMSRG_ERR_NONFINITE;
    go = 0;
  } else if (nrm * F->coef < kConv) {
    go = 0;
  } else {
    F->iw++;
    if (F->iw > 40) {
      F->status = IMSRG_ERR_NOT_CONVERGED;
      go = 0;
    } else {
      F->coef = F->coef / (F->iw - 1.0);
    }
  }
  return go;
}

__global__ void k_magnus_init(FlowDev *F, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, magnus_init_go(F));
}

__global__ void k_bch_init(FlowDev *F, cudaGraphConditionalHandle h, double ds) {
  cudaGraphSetConditional(h, bch_init_go(F, ds));
}

// A series term's norm from its partials (k_final_sum's order, so the same
// bits) and the series' stop test in one launch.
template <bool MAGNUS>
__global__ void __launch_bounds__(256) k_norm_next(const double *partials, int n, FlowDev *F,
                                                   cudaGraphConditionalHandle h) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partials[i];
  s = block_sum_ops(s, sh);
  if (threadIdx.x == 0) {
    F->nrm = sqrt(s);
    cudaGraphSetConditional(h, MAGNUS ? magnus_next_go(F) : bch_next_go(F));
  }
}

__global__ void k_step_end(FlowDev *F, const double *HS) { F->e0 = HS[0]; }

}  // namespace

// Per-basis flow graph: one instantiated step graph for one operator set.
struct FlowGraph {
  FlowDev *d_state = nullptr;
  FlowDev *h_state = nullptr;  // pinned
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const double *key[4] = {nullptr, nullptr, nullptr, nullptr};
  int precision = -1;
  double ds = 0.0;
};

namespace {

FlowGraph *flow_of(imsrg_basis *b) { return (FlowGraph *)b->flowgraph; }

// Capture helpers: append the work that `fn` enqueues on b->stream to graph g
// after `deps`; return the frontier nodes (what the next work must follow).
template <typename Fn>
int capture(imsrg_basis *b, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, Fn fn,
            std::vector<cudaGraphNode_t> *frontier) {
  IMSRG_CUDA_TRY(cudaStreamBeginCaptureToGraph(b->stream, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                               deps.size(), cudaStreamCaptureModeThreadLocal));
  int s = fn();
  cudaStreamCaptureStatus st;
  const cudaGraphNode_t *fr = nullptr;
  size_t nfr = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(b->stream, &st, nullptr, nullptr, &fr, nullptr, &nfr);
  if (frontier && e == cudaSuccess) frontier->assign(fr, fr + nfr);
  cudaGraph_t out = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &out);
  if (s != IMSRG_OK) return s;
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(e2);
}

int add_while(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, cudaGraphConditionalHandle h,
              cudaGraphNode_t *node, cudaGraph_t *body) {
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  IMSRG_CUDA_TRY(cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p));
  *body = p.conditional.phGraph_out[0];
  return IMSRG_OK;
}

// Builds the step graph for HS, G (with the flow's work operators H0, DG, X0,
// X1).  Profiling is paused while capturing.
int build_step_graph(imsrg_basis *b, FlowGraph *fg, imsrg_op *HS, imsrg_op *G, imsrg_op *H0, imsrg_op *DG,
                     imsrg_op *X0, imsrg_op *X1, int precision, double ds) {
  FlowDev *F = fg->d_state;
  const long nb = b->nfull * (long)sizeof(double);
  cudaGraph_t g = nullptr;
  IMSRG_CUDA_TRY(cudaGraphCreate(&g, 0));
  fg->graph = g;
  cudaGraphConditionalHandle hM, hB;
  IMSRG_CUDA_TRY(cudaGraphConditionalHandleCreate(&hM, g, 0, 0));
  IMSRG_CUDA_TRY(cudaGraphConditionalHandleCreate(&hB, g, 0, 0));
  std::vector<cudaGraphNode_t> fr;
  // MAGNUS_EXPAND set-up: X0 = DG (and X1's E0 slot, which with_e0 = 0 keeps)
  IMSRG_TRY(capture(b, g, {}, [&]() -> int {
    IMSRG_CUDA_TRY(cudaMemcpyAsync(X0->d, DG->d, nb, cudaMemcpyDeviceToDevice, b->stream));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(X1->d, DG->d, sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    IMSRG_TRY(launch_norm(b, X0->d, &F->adv[1]));
    IMSRG_TRY(launch_norm(b, G->d, &F->fullnorm));
    k_magnus_init<<<1, 1, 0, b->stream>>>(F, hM);
    return cuda_status(cudaGetLastError());
  }, &fr));
  cudaGraphNode_t wm, wb;
  cudaGraph_t body;
  IMSRG_TRY(add_while(g, fr, hM, &wm, &body));
  // one Magnus term: X1 = [G, X0]; DG += cof X1; |X1|; X0 = X1
  IMSRG_TRY(capture(b, body, {}, [&]() -> int {
    IMSRG_TRY(commutator_dev(b, G->d, G->herm, X0->d, -1, X1->d, -G->herm * -1, precision, 0));
    IMSRG_TRY(launch_series_update(b, DG->d, X1->d, &F->cof, X0->d, nullptr));
    k_norm_next<true><<<1, 256, 0, b->stream>>>(b->partials, b->nchunks, F, hM);
    return cuda_status(cudaGetLastError());
  }, nullptr));
  // euler_step, then BCH_EXPAND set-up: HS = H0, X0 = H0
  IMSRG_TRY(capture(b, g, {wm}, [&]() -> int {
    IMSRG_TRY(launch_axpby(b, G->d, 1.0, DG->d, ds, G->d));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(HS->d, H0->d, nb, cudaMemcpyDeviceToDevice, b->stream));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(X0->d, H0->d, nb, cudaMemcpyDeviceToDevice, b->stream));
    k_bch_init<<<1, 1, 0, b->stream>>>(F, hB, ds);
    return cuda_status(cudaGetLastError());
  }, &fr));
  IMSRG_TRY(add_while(g, fr, hB, &wb, &body));
  // one BCH term: X1 = [G, X0] (with E0); HS += X1 / n!; |X1|; X0 = X1
  IMSRG_TRY(capture(b, body, {}, [&]() -> int {
    IMSRG_TRY(commutator_dev(b, G->d, G->herm, X0->d, H0->herm, X1->d, -G->herm * H0->herm, precision, 1));
    IMSRG_TRY(launch_series_update(b, HS->d, X1->d, &F->coef, X0->d, nullptr));
    k_norm_next<false><<<1, 256, 0, b->stream>>>(b->partials, b->nchunks, F, hB);
    return cuda_status(cudaGetLastError());
  }, nullptr));
  // next generator and the stop criterion
  IMSRG_TRY(capture(b, g, {wb}, [&]() -> int {
    IMSRG_TRY(launch_white(b, HS->d, HS->herm, DG->d));
    IMSRG_TRY(launch_mbpt2(b, HS->d, HS->herm, &F->emp2));
    k_step_end<<<1, 1, 0, b->stream>>>(F, HS->d);
    return cuda_status(cudaGetLastError());
  }, nullptr));
  IMSRG_CUDA_TRY(cudaGraphInstantiate(&fg->exec, g, 0));
  return IMSRG_OK;
}

}  // namespace

void flow_graph_free(imsrg_basis *b) {
  FlowGraph *fg = flow_of(b);
  if (!fg) return;
  if (fg->exec) cudaGraphExecDestroy(fg->exec);
  if (fg->graph) cudaGraphDestroy(fg->graph);
  if (fg->d_state) cudaFree(fg->d_state);
  if (fg->h_state) cudaFreeHost(fg->h_state);
  delete fg;
  b->flowgraph = nullptr;
}

// Sets up (or reuses) the step graph of HS, G and starts the flow: G = 0,
// DG = white(HS), H0 = HS.  Fills the step-0 scalars.
int flow_graph_begin(imsrg_op *HS, imsrg_op *G, int precision, double ds, double *e0, double *emp2) {
  imsrg_basis *b = HS->b;
  imsrg_op *H0, *DG, *X0, *X1;
  IMSRG_TRY(flow_tmp_ops(b, &H0, &DG, &X0, &X1));
  if (precision == IMSRG_PREC_OZAKI) IMSRG_TRY(ozaki_prepare(b));
  FlowGraph *fg = flow_of(b);
  const bool same = fg && fg->exec && fg->key[0] == HS->d && fg->key[1] == G->d && fg->precision == precision &&
                    fg->ds == ds;
  if (!same) {
    flow_graph_free(b);
    fg = new FlowGraph();
    b->flowgraph = fg;
    IMSRG_CUDA_TRY(cudaMalloc((void **)&fg->d_state, sizeof(FlowDev)));
    IMSRG_CUDA_TRY(cudaMemset(fg->d_state, 0, sizeof(FlowDev)));
    IMSRG_CUDA_TRY(cudaMallocHost((void **)&fg->h_state, sizeof(FlowDev)));
    const bool prof = b->prof.on;
    b->prof.on = false;
    G->herm = -1;
    DG->herm = -1;
    H0->herm = HS->herm;
    int s = build_step_graph(b, fg, HS, G, H0, DG, X0, X1, precision, ds);
    b->prof.on = prof;
    if (s != IMSRG_OK) {
      flow_graph_free(b);
      return s;
    }
    fg->key[0] = HS->d;
    fg->key[1] = G->d;
    fg->precision = precision;
    fg->ds = ds;
  }
  // the host path's start of magnus_decouple
  IMSRG_CUDA_TRY(cudaMemsetAsync(G->d, 0, b->nfull * sizeof(double), b->stream));
  IMSRG_CUDA_TRY(cudaMemsetAsync(DG->d, 0, b->nfull * sizeof(double), b->stream));
  G->herm = -1;
  DG->herm = -1;
  IMSRG_TRY(launch_white(b, HS->d, HS->herm, DG->d));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(H0->d, HS->d, b->nfull * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  H0->herm = HS->herm;
  IMSRG_TRY(launch_mbpt2(b, HS->d, HS->herm, &fg->d_state->emp2));
  k_step_end<<<1, 1, 0, b->stream>>>(fg->d_state, HS->d);
  IMSRG_CUDA_TRY(cudaMemsetAsync(&fg->d_state->s, 0, sizeof(double), b->stream));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(fg->h_state, fg->d_state, sizeof(FlowDev), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  *e0 = fg->h_state->e0;
  *emp2 = fg->h_state->emp2;
  return IMSRG_OK;
}

// Sets the flow parameter s of the step graph's state (a flow restarted from
// a checkpoint at s).
int flow_graph_set_s(imsrg_basis *b, double s) {
  FlowGraph *fg = flow_of(b);
  if (!fg) return IMSRG_ERR_INVALID;
  fg->h_state->s = s;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(&fg->d_state->s, &fg->h_state->s, sizeof(double), cudaMemcpyHostToDevice,
                                 b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return IMSRG_OK;
}

// Enqueues one step graph and the read-back of its scalars (no wait).
int flow_graph_launch(imsrg_basis *b) {
  FlowGraph *fg = flow_of(b);
  if (!fg || !fg->exec) return IMSRG_ERR_INVALID;
  IMSRG_CUDA_TRY(cudaGraphLaunch(fg->exec, b->stream));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(fg->h_state, fg->d_state, sizeof(FlowDev), cudaMemcpyDeviceToHost, b->stream));
  return IMSRG_OK;
}

// Waits for the step and returns its scalars.
int flow_graph_finish(imsrg_basis *b, double *s, double *e0, double *emp2, int *nc, int *status) {
  FlowGraph *fg = flow_of(b);
  if (!fg) return IMSRG_ERR_INVALID;
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  IMSRG_TRY(ozaki_check_error(b));
  const FlowDev &h = *fg->h_state;
  *s = h.s;
  *e0 = h.e0;
  *emp2 = h.emp2;
  *nc = h.nc;
  *status = h.status;
  return IMSRG_OK;
}

// ---------------------------------------------------------------------------
// Lockstep batched flows: n instances (each on its own basis, the bases of one
// imsrg_batch) advance one Magnus step per graph launch together.  The Magnus
// and BCH series are WHILE loops that run while any instance's series
// continues; in each iteration every instance's commutator is split into its
// part before the products (an IF node: the instance's series still runs),
// ONE launch of the products of all instances whose series runs (the split
// engine's persistent tensor-core kernel over the merged tile list, or the
// merged FP64 list; the others' tiles are skipped), and its part after the products
// (an IF node).  The set-up of the Magnus series, the Euler step with the BCH
// set-up, and the generator with the stop criterion are IF nodes too (the
// instance still flows).  Every instance runs the kernels of its unbatched
// step graph in the same order on the same data, and the merged launch
// computes each tile as the instance's own launch would, so each instance's
// flow equals its unbatched one bit for bit.
// ---------------------------------------------------------------------------
namespace {

__global__ void k_bm_init(FlowDev *F, int *go) { *go = (int)magnus_init_go(F); }
__global__ void k_bm_next(FlowDev *F, int *go) { *go = (int)magnus_next_go(F); }
__global__ void k_bb_init(FlowDev *F, int *go, double ds) { *go = (int)bch_init_go(F, ds); }
__global__ void k_bb_next(FlowDev *F, int *go) { *go = (int)bch_next_go(F); }

// h = 1 while any flowing instance's series continues
__global__ void k_b_any(const int *go, const int *flow, int n, cudaGraphConditionalHandle h) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (flow[i] && go[i]) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// One series term: instance i takes part while it flows and its series runs;
// act[i] masks the merged product launch, hs[k * n + i] (k < nh) gate its IF
// nodes.
__global__ void k_b_term(const int *go, const int *flow, int n, int *act, const cudaGraphConditionalHandle *hs,
                         int nh) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int g = flow[i] && go[i];
    act[i] = g;
    for (int k = 0; k < nh; k++) cudaGraphSetConditional(hs[k * n + i], g ? 1u : 0u);
  }
}

// the step's IF nodes of the flowing instances
__global__ void k_b_step(const int *flow, int n, const cudaGraphConditionalHandle *hs, int nh) {
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int k = 0; k < nh; k++) cudaGraphSetConditional(hs[k * n + i], flow[i] ? 1u : 0u);
}

int add_if(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, cudaGraphConditionalHandle h,
           cudaGraphNode_t *node, cudaGraph_t *body) {
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  IMSRG_CUDA_TRY(cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p));
  *body = p.conditional.phGraph_out[0];
  return IMSRG_OK;
}

// capture into graph g after deps, on stream st (the batch stream)
template <typename Fn>
int capture_st(cudaStream_t st, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, Fn fn,
               std::vector<cudaGraphNode_t> *frontier) {
  IMSRG_CUDA_TRY(cudaStreamBeginCaptureToGraph(st, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                               cudaStreamCaptureModeThreadLocal));
  int s = fn();
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t *fr = nullptr;
  size_t nfr = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &fr, nullptr, &nfr);
  if (frontier && e == cudaSuccess) frontier->assign(fr, fr + nfr);
  cudaGraph_t out = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(st, &out);
  if (s != IMSRG_OK) return s;
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(e2);
}

}  // namespace

struct BatchFlowGraph {
  int n = 0, precision = -1;
  double ds = 0.0;
  std::vector<const double *> key;
  FlowDev *d_state = nullptr, *h_state = nullptr;
  int *d_go = nullptr, *d_flow = nullptr, *d_act = nullptr, *h_flow = nullptr;
  cudaGraphConditionalHandle *d_h = nullptr;  // IF handles: 3n of the step, 2n per series body
  GemmProb *d_fp64 = nullptr;                 // FP64: the merged product list of [G_i, X0_i]
  int fp64_nprobs = 0, fp64_ntiles = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

void batch_flow_free(void *p) {
  BatchFlowGraph *f = (BatchFlowGraph *)p;
  if (!f) return;
  if (f->exec) cudaGraphExecDestroy(f->exec);
  if (f->graph) cudaGraphDestroy(f->graph);
  cudaFree(f->d_state);
  cudaFree(f->d_go);
  cudaFree(f->d_flow);
  cudaFree(f->d_act);
  cudaFree(f->d_h);
  cudaFree(f->d_fp64);
  if (f->h_state) cudaFreeHost(f->h_state);
  if (f->h_flow) cudaFreeHost(f->h_flow);
  delete f;
}

namespace {

// Builds the step graph of the instances HS[i], G[i] on bases[i].
int build_batch_graph(BatchFlowGraph *f, imsrg_basis *const *bases, void *oz, cudaStream_t st,
                      imsrg_op *const *HS, imsrg_op *const *G) {
  const int n = f->n, precision = f->precision;
  const double ds = f->ds;
  const bool ozp = precision == IMSRG_PREC_OZAKI;
  std::vector<imsrg_op *> H0(n), DG(n), X0(n), X1(n);
  for (int i = 0; i < n; i++) IMSRG_TRY(flow_tmp_ops(bases[i], &H0[i], &DG[i], &X0[i], &X1[i]));
  if (!ozp) {  // every series term is [G_i, X0_i]: one merged FP64 product list
    std::vector<const double *> Lp(n), Rp(n);
    for (int i = 0; i < n; i++) {
      Lp[i] = G[i]->d;
      Rp[i] = X0[i]->d;
    }
    IMSRG_TRY(gemm_fp64_merged(bases, n, Lp.data(), Rp.data(), &f->d_fp64, &f->fp64_nprobs, &f->fp64_ntiles));
  }
  cudaGraph_t g = nullptr;
  IMSRG_CUDA_TRY(cudaGraphCreate(&g, 0));
  f->graph = g;
  std::vector<cudaGraphConditionalHandle> h(3 * (size_t)n);
  cudaGraphConditionalHandle hM, hB;
  IMSRG_CUDA_TRY(cudaGraphConditionalHandleCreate(&hM, g, 0, 0));
  IMSRG_CUDA_TRY(cudaGraphConditionalHandleCreate(&hB, g, 0, 0));
  for (int k = 0; k < 3 * n; k++) IMSRG_CUDA_TRY(cudaGraphConditionalHandleCreate(&h[k], g, 0, 0));
  cudaGraphConditionalHandle *dh_step = f->d_h, *dh_m = f->d_h + 3 * n, *dh_b = f->d_h + 5 * n;
  IMSRG_CUDA_TRY(cudaMemcpy(dh_step, h.data(), 3 * n * sizeof(cudaGraphConditionalHandle), cudaMemcpyHostToDevice));
  std::vector<cudaGraphNode_t> fr, ifs;
  IMSRG_TRY(capture_st(st, g, {}, [&]() -> int {
    k_b_step<<<1, 128, 0, st>>>(f->d_flow, n, dh_step, 3);
    return cuda_status(cudaGetLastError());
  }, &fr));
  // MAGNUS_EXPAND set-up of each flowing instance
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bases[i];
    const size_t bytes = b->nfull * sizeof(double);
    FlowDev *F = f->d_state + i;
    cudaGraphNode_t node;
    cudaGraph_t body;
    IMSRG_TRY(add_if(g, fr, h[i], &node, &body));
    IMSRG_TRY(capture(b, body, {}, [&]() -> int {
      IMSRG_CUDA_TRY(cudaMemcpyAsync(X0[i]->d, DG[i]->d, bytes, cudaMemcpyDeviceToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(X1[i]->d, DG[i]->d, sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
      IMSRG_TRY(launch_norm(b, X0[i]->d, &F->adv[1]));
      IMSRG_TRY(launch_norm(b, G[i]->d, &F->fullnorm));
      k_bm_init<<<1, 1, 0, b->stream>>>(F, f->d_go + i);
      return cuda_status(cudaGetLastError());
    }, nullptr));
    ifs.push_back(node);
  }
  // one series loop: magnus (commutators without E0, DG += cof X1) or BCH
  // (with E0, HS += coef X1)
  auto series = [&](cudaGraphConditionalHandle hw, const std::vector<cudaGraphNode_t> &deps, bool magnus,
                    cudaGraphConditionalHandle *dh, cudaGraphNode_t *wnode) -> int {
    std::vector<cudaGraphNode_t> wfr;
    IMSRG_TRY(capture_st(st, g, deps, [&]() -> int {
      k_b_any<<<1, 128, 0, st>>>(f->d_go, f->d_flow, n, hw);
      return cuda_status(cudaGetLastError());
    }, &wfr));
    cudaGraph_t body;
    IMSRG_TRY(add_while(g, wfr, hw, wnode, &body));
    std::vector<cudaGraphConditionalHandle> hb(2 * (size_t)n);
    for (int k = 0; k < 2 * n; k++) IMSRG_CUDA_TRY(cudaGraphConditionalHandleCreate(&hb[k], body, 0, 0));
    IMSRG_CUDA_TRY(cudaMemcpy(dh, hb.data(), 2 * n * sizeof(cudaGraphConditionalHandle), cudaMemcpyHostToDevice));
    std::vector<cudaGraphNode_t> bfr, fronts, backs;
    IMSRG_TRY(capture_st(st, body, {}, [&]() -> int {
      k_b_term<<<1, 128, 0, st>>>(f->d_go, f->d_flow, n, f->d_act, dh, 2);
      return cuda_status(cudaGetLastError());
    }, &bfr));
    const int hX = magnus ? -1 : 1, hRES = magnus ? -1 : 1, with_e0 = magnus ? 0 : 1;
    const int fphase = kPhaseFront | kPhaseJoinE0Front;
    for (int i = 0; i < n; i++) {
      imsrg_basis *b = bases[i];
      cudaGraphNode_t node;
      cudaGraph_t ib;
      IMSRG_TRY(add_if(body, bfr, hb[i], &node, &ib));
      IMSRG_TRY(capture(b, ib, {}, [&]() -> int {
        return commutator_launches(b, G[i]->d, -1, X0[i]->d, hX, X1[i]->d, hRES, precision, with_e0, nullptr,
                                   fphase);
      }, nullptr));
      fronts.push_back(node);
    }
    std::vector<cudaGraphNode_t> mfr;
    IMSRG_TRY(capture_st(st, body, fronts, [&]() -> int {
      if (ozp) return ozaki_batch_mma(oz, st, -1, hX, f->d_act);
      return launch_gemm_fp64_merged(f->d_fp64, f->fp64_nprobs, f->fp64_ntiles, -1, hX, f->d_act, st);
    }, &mfr));
    for (int i = 0; i < n; i++) {
      imsrg_basis *b = bases[i];
      FlowDev *F = f->d_state + i;
      cudaGraphNode_t node;
      cudaGraph_t ib;
      IMSRG_TRY(add_if(body, mfr, hb[n + i], &node, &ib));
      IMSRG_TRY(capture(b, ib, {}, [&]() -> int {
        IMSRG_TRY(commutator_launches(b, G[i]->d, -1, X0[i]->d, hX, X1[i]->d, hRES, precision, with_e0, nullptr,
                                      kPhaseBack | kPhaseJoinE0Front));
        IMSRG_TRY(launch_series_update(b, magnus ? DG[i]->d : HS[i]->d, X1[i]->d, magnus ? &F->cof : &F->coef,
                                       X0[i]->d, &F->nrm));
        if (magnus) k_bm_next<<<1, 1, 0, b->stream>>>(F, f->d_go + i);
        else k_bb_next<<<1, 1, 0, b->stream>>>(F, f->d_go + i);
        return cuda_status(cudaGetLastError());
      }, nullptr));
      backs.push_back(node);
    }
    return capture_st(st, body, backs, [&]() -> int {
      k_b_any<<<1, 128, 0, st>>>(f->d_go, f->d_flow, n, hw);
      return cuda_status(cudaGetLastError());
    }, nullptr);
  };
  cudaGraphNode_t wm, wb;
  IMSRG_TRY(series(hM, ifs, true, dh_m, &wm));
  // euler_step, then the BCH_EXPAND set-up
  ifs.clear();
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bases[i];
    const size_t bytes = b->nfull * sizeof(double);
    FlowDev *F = f->d_state + i;
    cudaGraphNode_t node;
    cudaGraph_t body;
    IMSRG_TRY(add_if(g, {wm}, h[n + i], &node, &body));
    IMSRG_TRY(capture(b, body, {}, [&]() -> int {
      IMSRG_TRY(launch_axpby(b, G[i]->d, 1.0, DG[i]->d, ds, G[i]->d));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(HS[i]->d, H0[i]->d, bytes, cudaMemcpyDeviceToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(X0[i]->d, H0[i]->d, bytes, cudaMemcpyDeviceToDevice, b->stream));
      k_bb_init<<<1, 1, 0, b->stream>>>(F, f->d_go + i, ds);
      return cuda_status(cudaGetLastError());
    }, nullptr));
    ifs.push_back(node);
  }
  IMSRG_TRY(series(hB, ifs, false, dh_b, &wb));
  // the next generator and the stop criterion
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bases[i];
    FlowDev *F = f->d_state + i;
    cudaGraphNode_t node;
    cudaGraph_t body;
    IMSRG_TRY(add_if(g, {wb}, h[2 * n + i], &node, &body));
    IMSRG_TRY(capture(b, body, {}, [&]() -> int {
      IMSRG_TRY(launch_white(b, HS[i]->d, HS[i]->herm, DG[i]->d));
      IMSRG_TRY(launch_mbpt2(b, HS[i]->d, HS[i]->herm, &F->emp2));
      k_step_end<<<1, 1, 0, b->stream>>>(F, HS[i]->d);
      return cuda_status(cudaGetLastError());
    }, nullptr));
  }
  IMSRG_CUDA_TRY(cudaGraphInstantiate(&f->exec, g, 0));
  return IMSRG_OK;
}

}  // namespace

int batch_flow_run(imsrg_basis *const *bases, int n, void *oz, cudaStream_t st, void **cache,
                   imsrg_op *const *HS, imsrg_op *const *G, double s_max, double ds, int max_steps, int precision,
                   double *const *traces, int *steps_out, int *ncomm, int *status) {
  if (precision == IMSRG_PREC_OZAKI && !oz) return IMSRG_ERR_INVALID;
  BatchFlowGraph *f = (BatchFlowGraph *)*cache;
  std::vector<const double *> key;
  for (int i = 0; i < n; i++) {
    key.push_back(HS[i]->d);
    key.push_back(G[i]->d);
  }
  if (!(f && f->exec && f->key == key && f->precision == precision && f->ds == ds && f->n == n)) {
    batch_flow_free(f);
    *cache = nullptr;
    f = new BatchFlowGraph();
    *cache = f;
    f->n = n;
    f->precision = precision;
    f->ds = ds;
    f->key = key;
    IMSRG_CUDA_TRY(cudaMalloc((void **)&f->d_state, n * sizeof(FlowDev)));
    IMSRG_CUDA_TRY(cudaMemset(f->d_state, 0, n * sizeof(FlowDev)));
    IMSRG_CUDA_TRY(cudaMallocHost((void **)&f->h_state, n * sizeof(FlowDev)));
    IMSRG_CUDA_TRY(cudaMalloc((void **)&f->d_go, n * sizeof(int)));
    IMSRG_CUDA_TRY(cudaMalloc((void **)&f->d_flow, n * sizeof(int)));
    IMSRG_CUDA_TRY(cudaMalloc((void **)&f->d_act, n * sizeof(int)));
    IMSRG_CUDA_TRY(cudaMallocHost((void **)&f->h_flow, n * sizeof(int)));
    IMSRG_CUDA_TRY(cudaMalloc((void **)&f->d_h, 7 * n * sizeof(cudaGraphConditionalHandle)));
    std::vector<char> prof(n);
    for (int i = 0; i < n; i++) {
      G[i]->herm = -1;
      prof[i] = bases[i]->prof.on;
      bases[i]->prof.on = false;
    }
    const int s = build_batch_graph(f, bases, oz, st, HS, G);
    for (int i = 0; i < n; i++) bases[i]->prof.on = prof[i];
    if (s != IMSRG_OK) {
      batch_flow_free(f);
      *cache = nullptr;
      return s;
    }
  }
  // the start of magnus_decouple per instance (as flow_graph_begin)
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bases[i];
    imsrg_op *H0, *DG, *X0, *X1;
    IMSRG_TRY(flow_tmp_ops(b, &H0, &DG, &X0, &X1));
    IMSRG_CUDA_TRY(cudaMemsetAsync(G[i]->d, 0, b->nfull * sizeof(double), b->stream));
    IMSRG_CUDA_TRY(cudaMemsetAsync(DG->d, 0, b->nfull * sizeof(double), b->stream));
    G[i]->herm = -1;
    DG->herm = -1;
    IMSRG_TRY(launch_white(b, HS[i]->d, HS[i]->herm, DG->d));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(H0->d, HS[i]->d, b->nfull * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    H0->herm = HS[i]->herm;
    IMSRG_TRY(launch_mbpt2(b, HS[i]->d, HS[i]->herm, &f->d_state[i].emp2));
    k_step_end<<<1, 1, 0, b->stream>>>(f->d_state + i, HS[i]->d);
    IMSRG_CUDA_TRY(cudaMemsetAsync(&f->d_state[i].s, 0, sizeof(double), b->stream));
  }
  for (int i = 0; i < n; i++) IMSRG_CUDA_TRY(cudaStreamSynchronize(bases[i]->stream));
  IMSRG_CUDA_TRY(cudaMemcpy(f->h_state, f->d_state, n * sizeof(FlowDev), cudaMemcpyDeviceToHost));
  std::vector<double> sv(n, 0.0), crit(n, 0.0);
  std::vector<int> steps(n, 0), nct(n, 0), stat(n, IMSRG_OK);
  auto row = [&](int i, int k, double e0, double emp2) {
    if (!traces || !traces[i]) return;
    double *t = traces[i] + 5 * k;
    t[0] = k;
    t[1] = sv[i];
    t[2] = e0;
    t[3] = e0 + emp2;
    t[4] = std::fabs(emp2);
  };
  for (int i = 0; i < n; i++) {
    crit[i] = std::fabs(f->h_state[i].emp2);
    row(i, 0, f->h_state[i].e0, f->h_state[i].emp2);
  }
  auto active = [&](int i) {
    return stat[i] == IMSRG_OK && crit[i] > 1e-6 && sv[i] < s_max - 1e-12 && steps[i] < max_steps;
  };
  for (;;) {
    int nact = 0;
    for (int i = 0; i < n; i++) nact += (f->h_flow[i] = active(i) ? 1 : 0);
    if (!nact) break;
    IMSRG_CUDA_TRY(cudaMemcpyAsync(f->d_flow, f->h_flow, n * sizeof(int), cudaMemcpyHostToDevice, st));
    IMSRG_CUDA_TRY(cudaGraphLaunch(f->exec, st));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(f->h_state, f->d_state, n * sizeof(FlowDev), cudaMemcpyDeviceToHost, st));
    IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
    if (precision == IMSRG_PREC_OZAKI) IMSRG_TRY(ozaki_batch_error(oz, st));
    for (int i = 0; i < n; i++) {
      if (!f->h_flow[i]) continue;
      const FlowDev &hs = f->h_state[i];
      steps[i]++;
      nct[i] += hs.nc;
      sv[i] = hs.s;
      int st1 = hs.status;
      if (st1 == IMSRG_OK && (!std::isfinite(hs.e0) || !std::isfinite(hs.emp2))) st1 = IMSRG_ERR_NONFINITE;
      stat[i] = st1;
      crit[i] = std::fabs(hs.emp2);
      if (st1 == IMSRG_OK) row(i, steps[i], hs.e0, hs.emp2);
    }
  }
  int worst = IMSRG_OK;
  for (int i = 0; i < n; i++) {
    if (steps_out) steps_out[i] = steps[i];
    if (ncomm) ncomm[i] = nct[i];
    if (status) status[i] = stat[i];
    if (stat[i] != IMSRG_OK && worst == IMSRG_OK) worst = stat[i];
  }
  return worst;
}

}  // namespace imsrg
