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
// previous (non-zero-coefficient) term is small against Omega.
__device__ void magnus_check(FlowDev *F, cudaGraphConditionalHandle h) {
  unsigned go = 0;
  const int i = F->i;
  if (F->status == IMSRG_OK && i <= 7 && !(F->fullnorm < 1e-9)) {
    const double adnorm = F->adv[i - F->q];
    F->q = (fabs(c_cof[i - 1]) > 1e-6) ? 1 : 2;
    go = !(fabs(adnorm / F->fullnorm) < kConv);
    F->cof = c_cof[i - 1];
  }
  cudaGraphSetConditional(h, go);
}

__global__ void k_magnus_init(FlowDev *F, cudaGraphConditionalHandle h) {
  F->adv[0] = 0.0;
  for (int k = 2; k < 8; k++) F->adv[k] = 0.0;
  F->i = 2;
  F->q = 1;
  F->nc = 0;
  F->status = IMSRG_OK;
  magnus_check(F, h);
}

__global__ void k_magnus_next(FlowDev *F, cudaGraphConditionalHandle h) {
  F->nc++;
  const double nrm = F->nrm;
  if (!isfinite(nrm)) {
    F->status = IMSRG_ERR_NONFINITE;
    cudaGraphSetConditional(h, 0);
    return;
  }
  F->adv[F->i] = nrm * fabs(c_cof[F->i - 1]);
  F->i++;
  magnus_check(F, h);
}

__global__ void k_bch_init(FlowDev *F, cudaGraphConditionalHandle h, double ds) {
  F->s += ds;
  F->iw = 2;
  F->coef = 1.0;  // 1/(iw - 1)! at iw = 2
  cudaGraphSetConditional(h, F->status == IMSRG_OK ? 1u : 0u);
}

// After BCH term iw (IMSRG_MAGNUS.f90:207-231): stop when |term| / n! < conv;
// 39 terms without convergence is the reference's 'clipping BCH'.
__global__ void k_bch_next(FlowDev *F, cudaGraphConditionalHandle h) {
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
  cudaGraphSetConditional(h, go);
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
    IMSRG_TRY(launch_axpby_dev(b, DG->d, 1.0, X1->d, &F->cof, DG->d));
    IMSRG_TRY(launch_norm(b, X1->d, &F->nrm));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(X0->d, X1->d, nb, cudaMemcpyDeviceToDevice, b->stream));
    k_magnus_next<<<1, 1, 0, b->stream>>>(F, hM);
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
    IMSRG_TRY(launch_axpby_dev(b, HS->d, 1.0, X1->d, &F->coef, HS->d));
    IMSRG_TRY(launch_norm(b, X1->d, &F->nrm));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(X0->d, X1->d, nb, cudaMemcpyDeviceToDevice, b->stream));
    k_bch_next<<<1, 1, 0, b->stream>>>(F, hB);
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

}  // namespace imsrg
