// api.cpp -- the extern "C" entry points of include/imsrg_gpu.h and the host
// side of the Magnus flow.
//
// The flow drivers restate IMSRG_MAGNUS.f90 (n-parzuchowski/EOM-IMSRG_FULL,
// im-SRG/): MAGNUS_EXPAND (:622-693), BCH_EXPAND (:149-234), euler_step
// (:756-766) and magnus_decouple (:15-128).  Operators stay resident on the
// device; only the scalars that steer the series (norms, mbpt2, E0) are read
// back.  The reference allocates fresh work operators in every BCH/MAGNUS call
// (:164-174, :633-643); here they are allocated once per basis and reused, and
// the INT1/AD/INT2 copies become two alternating buffers.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "internal.h"

using imsrg::cuda_status;

namespace {

// Truncated Bernoulli coefficients of IMSRG_MAGNUS.f90:648, kept for parity.
const double kMagnusCof[7] = {1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5};

int check_op(const imsrg_op *op) { return (op && op->b && op->d) ? IMSRG_OK : IMSRG_ERR_INVALID; }

int read_scalar(imsrg_basis *b, const double *d, double *out) {
  IMSRG_CUDA_TRY(cudaMemcpyAsync(b->h_scal, d, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  IMSRG_TRY(imsrg::ozaki_check_error(b));
  *out = b->h_scal[0];
  return IMSRG_OK;
}

int op_norm(imsrg_basis *b, const double *d, double *out) {
  IMSRG_TRY(imsrg::launch_norm(b, d, b->scal));
  return read_scalar(b, b->scal, out);
}

int copy_dev(imsrg_basis *b, const double *src, double *dst, long n) {
  if (src == dst) return IMSRG_OK;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  return IMSRG_OK;
}

// Work operators of the flow, created on first use: 0,1 alternating
// commutator buffers, 2 the unevolved H, 3 the generator / dOmega.
int tmp_op(imsrg_basis *b, int k, imsrg_op **out) {
  while ((int)b->tmp_ops.size() <= k) {
    imsrg_op *op = nullptr;
    int s = imsrg_gpu_op_create(b, 1, &op);
    if (s != IMSRG_OK) return s;
    b->tmp_ops.push_back(op);
  }
  *out = b->tmp_ops[k];
  return IMSRG_OK;
}

// The generator of the flow from H into ETA (herm -1): build_gs_white
// (generators.f90:4-106), build_gs_atan (:162-266) or build_gs_w2 (:109-159:
// ETA = 1.5 atan(H) + 0.5 atanxx(H, [atan(H), H])).
int generator_dev(imsrg_basis *b, const double *H, int hH, double *ETA, int generator, int precision) {
  if (generator == IMSRG_GEN_WHITE) return imsrg::launch_white(b, H, hH, ETA);
  if (generator == IMSRG_GEN_ATAN) return imsrg::launch_generator(b, H, hH, H, 1, ETA);
  if (generator != IMSRG_GEN_W2) return IMSRG_ERR_INVALID;
  imsrg_op *E1, *H2, *E2;
  IMSRG_TRY(tmp_op(b, 9, &E1));
  IMSRG_TRY(tmp_op(b, 10, &H2));
  IMSRG_TRY(tmp_op(b, 11, &E2));
  IMSRG_CUDA_TRY(cudaMemsetAsync(E1->d, 0, sizeof(double), b->stream));
  IMSRG_CUDA_TRY(cudaMemsetAsync(E2->d, 0, sizeof(double), b->stream));
  IMSRG_TRY(imsrg::launch_generator(b, H, hH, H, 1, E1->d));
  E1->herm = E2->herm = -1;
  H2->herm = hH;
  IMSRG_TRY(imsrg::commutator_dev(b, E1->d, -1, H, hH, H2->d, hH, precision, 1));
  IMSRG_TRY(imsrg::launch_generator(b, H, hH, H2->d, 1, E2->d));
  return imsrg::launch_axpby(b, E1->d, 1.5, E2->d, 0.5, ETA);
}

}  // namespace

namespace imsrg {

int work_op(imsrg_basis *b, int k, imsrg_op **out) { return tmp_op(b, k, out); }

// dHds (IMSRG_ODE.f90:416-463) on device buffers: DH = [eta(HS), HS].
int dhds_dev(imsrg_basis *b, const double *HS, int hH, double *DH, int generator, int precision) {
  imsrg_op *ETA;
  IMSRG_TRY(tmp_op(b, 14, &ETA));
  IMSRG_CUDA_TRY(cudaMemsetAsync(ETA->d, 0, sizeof(double), b->stream));
  ETA->herm = -1;
  IMSRG_TRY(generator_dev(b, HS, hH, ETA->d, generator, precision));
  return commutator_dev(b, ETA->d, -1, HS, hH, DH, hH, precision, 1);
}

// The launch sequence of one commutator.  Independent launches run on the
// side streams, forked from and joined back into the basis stream with
// events, so the call stays one ordered unit on that stream.  `phases`
// selects the part before the products (kPhaseFront: E0, images, Pandya
// transform), the products (kPhaseProducts) and the part after them
// (kPhaseBack: assemblies, joins); a batch of commutators runs the products
// of all its bases in one launch between the two (device operands only).
int commutator_launches(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                        int precision, int with_e0, const HostIO *io, int phases) {
  const bool front = phases & kPhaseFront, prods = phases & kPhaseProducts, back = phases & kPhaseBack;
  if (io && phases != kPhaseAll) return IMSRG_ERR_INVALID;
  // While kernel timing is on, every launch goes to the basis stream in the
  // same order, so each kernel class's event pair times that kernel alone.
  const bool serial = b->prof.on;
  cudaStream_t side = serial ? b->stream : b->side, side2 = serial ? b->stream : b->side2;
  const size_t bytes = (size_t)b->nfull * sizeof(double);
  const bool oz = precision == IMSRG_PREC_OZAKI;
  // Page-locked host operands (outside profiling): R is copied first, so its
  // digit images and its half of the Pandya transform run on side2 while L is
  // in flight, and RES comes back by output range beside the two-body assembly.
  const bool overlap = io && io->pinned && !serial;
  // packed host arrays (vectorize order): copied into staging buffers and
  // unpacked on the device; RES packed before one copy back
  const bool packed = io && io->Lst;
  const size_t pbytes = (size_t)b->neq * sizeof(double);
  // packed page-locked operands the device addresses: no staging copies
  const bool direct = overlap && packed && io->Ldev && io->Rdev && io->RESdev;
  // the transform also reduces the LCC/RCC block exponents (split precision)
  int *cc_exps = nullptr, gL = 0, gR = 0;
  if (overlap) {
    if (oz) IMSRG_TRY(ozaki_cc_exponents(b, b->stream, &cc_exps, &gL, &gR));
    if (direct) {
      // the unpack kernels of R (side2) and L read the host arrays at once
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_hostR, b->stream));
      IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->side2, b->ev_hostR, 0));
      IMSRG_TRY(launch_unpack(b, io->Rdev, hR, const_cast<double *>(R), b->side2));
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_rdev, b->side2));  // R is on the device
      IMSRG_TRY(launch_unpack(b, io->Ldev, hL, const_cast<double *>(L), b->stream));
    } else if (packed) {
      IMSRG_CUDA_TRY(cudaMemcpyAsync(io->Rst, io->R, pbytes, cudaMemcpyHostToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_hostR, b->stream));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(io->Lst, io->L, pbytes, cudaMemcpyHostToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->side2, b->ev_hostR, 0));
      IMSRG_TRY(launch_unpack(b, io->Rst, hR, const_cast<double *>(R), b->side2));
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_rdev, b->side2));  // R is on the device
      IMSRG_TRY(launch_unpack(b, io->Lst, hL, const_cast<double *>(L), b->stream));
    } else {
      IMSRG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(R), io->R, bytes, cudaMemcpyHostToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_hostR, b->stream));
      IMSRG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(L), io->L, bytes, cudaMemcpyHostToDevice, b->stream));
      IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->side2, b->ev_hostR, 0));
    }
    if (oz) IMSRG_TRY(ozaki_slice(b, L, R, 1, b->side2));
    IMSRG_TRY(launch_cc_forward(b, L, hL, R, hR, cc_exps, gL, gR, 2, b->side2));
    IMSRG_CUDA_TRY(cudaEventRecord(b->ev_join2, b->side2));
  } else if (io && packed) {  // pageable packed host operands, one after the other
    IMSRG_CUDA_TRY(cudaMemcpyAsync(io->Lst, io->L, pbytes, cudaMemcpyHostToDevice, b->stream));
    IMSRG_TRY(launch_unpack(b, io->Lst, hL, const_cast<double *>(L), b->stream));
    IMSRG_CUDA_TRY(cudaEventRecord(b->ev_hostL, b->stream));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(io->Rst, io->R, pbytes, cudaMemcpyHostToDevice, b->stream));
    IMSRG_TRY(launch_unpack(b, io->Rst, hR, const_cast<double *>(R), b->stream));
  } else if (io) {  // pageable host operands: L first, so the digit images of L start while R is in flight
    IMSRG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(L), io->L, bytes, cudaMemcpyHostToDevice, b->stream));
    IMSRG_CUDA_TRY(cudaEventRecord(b->ev_hostL, b->stream));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(R), io->R, bytes, cudaMemcpyHostToDevice, b->stream));
  }
  auto fork = [&](int k) -> int {
    if (serial) return IMSRG_OK;
    IMSRG_CUDA_TRY(cudaEventRecord(b->ev_fork[k], b->stream));
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->side, (io && !overlap && k == 0) ? b->ev_hostL : b->ev_fork[k], 0));
    return IMSRG_OK;
  };
  auto join = [&](int k) -> int {
    if (serial) return IMSRG_OK;
    IMSRG_CUDA_TRY(cudaEventRecord(b->ev_join[k], b->side));
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_join[k], 0));
    return IMSRG_OK;
  };
  // E0 and the commutator_122 part of the two-body assembly need only L and
  // R: E0's single CTA runs on side3 and the 122 sums on side4 from here,
  // beside the Pandya transform, the slicing and the products.  E0 is joined at the end (after the one-body
  // assembly, where it ran before, it finished last: the one-body kernel runs
  // slowly beside the 3,769 CTAs of the two-body assembly), the 122 sums
  // before the rest of the two-body assembly.
  if (front) {
    if (serial) {
      if (with_e0) IMSRG_TRY(launch_e0(b, L, hL, R, hR, RES, b->stream));
      IMSRG_TRY(launch_asm2_122(b, L, hL, R, hR, RES, hRES, b->stream));
    } else {
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_fork[0], b->stream));
      for (cudaStream_t s : {b->side3, b->side4}) {
        IMSRG_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_fork[0], 0));
        if (overlap && packed) IMSRG_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_rdev, 0));
      }
      if (with_e0) {
        IMSRG_TRY(launch_e0(b, L, hL, R, hR, RES, b->side3));
        IMSRG_CUDA_TRY(cudaEventRecord(b->ev_join3, b->side3));
      }
      IMSRG_TRY(launch_asm2_122(b, L, hL, R, hR, RES, hRES, b->side4));
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_pre, b->side4));
    }
  }
  const bool e0_front = (phases & kPhaseJoinE0Front) != 0;
  auto join_e0 = [&]() -> int {
    if (with_e0 && !serial) IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_join3, 0));
    return IMSRG_OK;
  };
  auto join_pre = [&]() -> int {
    if (!serial) IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_pre, 0));
    return IMSRG_OK;
  };
  if (overlap) {  // R's half is under way on side2; L's half once L is in
    IMSRG_TRY(fork(0));
    if (oz) IMSRG_TRY(ozaki_slice(b, L, R, 0, side));
    IMSRG_TRY(launch_cc_forward(b, L, hL, R, hR, cc_exps, gL, gR, 1));
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_join2, 0));
    if (oz) {
      IMSRG_TRY(ozaki_slice(b, L, R, 2, b->stream, cc_exps != nullptr));
      IMSRG_TRY(join(0));
      IMSRG_TRY(ozaki_mma(b, hL, hR));
    } else {
      IMSRG_TRY(join(0));
      IMSRG_TRY(launch_gemm_fp64(b, L, hL, R, hR));
    }
  } else if (oz) {
    // digit images of L and of R on the two side streams, beside the Pandya
    // transform and the images of LCC and RCC
    if (front) {
      IMSRG_TRY(fork(0));
      if (!serial) IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->side2, b->ev_fork[0], 0));
      IMSRG_TRY(ozaki_slice(b, L, R, 0, side));
      IMSRG_TRY(ozaki_slice(b, L, R, 1, side2));
      IMSRG_TRY(ozaki_cc_exponents(b, b->stream, &cc_exps, &gL, &gR));
      IMSRG_TRY(launch_cc_forward(b, L, hL, R, hR, cc_exps, gL, gR));
      IMSRG_TRY(ozaki_slice(b, L, R, 2, b->stream, cc_exps != nullptr));
      IMSRG_TRY(join(0));
      if (!serial) {
        IMSRG_CUDA_TRY(cudaEventRecord(b->ev_join2, b->side2));
        IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_join2, 0));
      }
    }
    if (prods) IMSRG_TRY(ozaki_mma(b, hL, hR));
  } else {
    if (front) IMSRG_TRY(launch_cc_forward(b, L, hL, R, hR));
    if (prods) IMSRG_TRY(launch_gemm_fp64(b, L, hL, R, hR));
  }
  if (front && e0_front) {  // phases in separate graphs: join what the front forked
    IMSRG_TRY(join_e0());
    IMSRG_TRY(join_pre());
  }
  if (!back) return IMSRG_OK;
  // one-body assembly beside the two-body assembly
  IMSRG_TRY(fork(1));
  IMSRG_TRY(launch_assemble_1body(b, L, hL, R, hR, RES, hRES, side));
  if (overlap && !packed) {
    // two-body elements by output range; each range's copy to the host runs on
    // side2 beside the assembly of the next (see imsrg_basis::asm2_el)
    IMSRG_TRY(launch_ph_inputs(b, hL, hR, precision));
    if (!e0_front) IMSRG_TRY(join_pre());
    for (int c = 0; c < kOutChunks; c++) {
      IMSRG_TRY(launch_asm2_range(b, L, hL, R, hR, RES, hRES, b->asm2_el[c], b->asm2_el[c + 1], true));
      IMSRG_CUDA_TRY(cudaEventRecord(b->ev_out[c], b->stream));
      IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->side2, b->ev_out[c], 0));
      const long a0 = b->asm2_addr[c], a1 = b->asm2_addr[c + 1];
      if (a1 > a0)
        IMSRG_CUDA_TRY(cudaMemcpyAsync(io->RES + a0, RES + a0, (size_t)(a1 - a0) * sizeof(double),
                                       cudaMemcpyDeviceToHost, b->side2));
    }
    IMSRG_TRY(join(1));
    IMSRG_TRY(join_e0());
    // E0 and the one-body part
    IMSRG_CUDA_TRY(cudaMemcpyAsync(io->RES, RES, (size_t)b->asm2_addr[0] * sizeof(double), cudaMemcpyDeviceToHost,
                                   b->stream));
    IMSRG_CUDA_TRY(cudaEventRecord(b->ev_outj, b->side2));
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_outj, 0));
    return IMSRG_OK;
  }
  {
    ProfScope ps(b, IMSRG_KERNEL_ASSEMBLE_2BODY);
    IMSRG_TRY(launch_ph_inputs(b, hL, hR, precision));
    if (!e0_front) IMSRG_TRY(join_pre());
    IMSRG_TRY(launch_asm2_range(b, L, hL, R, hR, RES, hRES, 0, b->T.n_asm2, false));
  }
  IMSRG_TRY(join(1));
  if (!e0_front) IMSRG_TRY(join_e0());
  if (direct) {
    IMSRG_TRY(launch_pack(b, RES, io->RESdev, b->stream, true));
  } else if (io && packed) {
    IMSRG_TRY(launch_pack(b, RES, io->RESst, b->stream));
    IMSRG_CUDA_TRY(cudaMemcpyAsync(io->RES, io->RESst, pbytes, cudaMemcpyDeviceToHost, b->stream));
  } else if (io) {
    IMSRG_CUDA_TRY(cudaMemcpyAsync(io->RES, RES, bytes, cudaMemcpyDeviceToHost, b->stream));
  }
  return IMSRG_OK;
}

namespace {
constexpr size_t kCommGraphs = 8;
}

// One commutator.  Outside profiling and outside a caller's stream capture,
// the launch sequence of each argument set is captured once into a CUDA graph
// and replayed (one launch instead of ~12, and no host work per kernel); the
// graph runs the same kernels on the same data, so results are unchanged.
int commutator_dev(imsrg_basis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                   int precision, int with_e0, const HostIO *io) {
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  if (precision == IMSRG_PREC_OZAKI) IMSRG_TRY(ozaki_prepare(b));
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  IMSRG_CUDA_TRY(cudaStreamIsCapturing(b->stream, &cs));
  bool pinned = true;  // host copies enter a graph only from page-locked memory
  void *dev[3] = {nullptr, nullptr, nullptr};  // their device addresses, when mapped
  if (io) {
    const void *hp[3] = {io->L, io->R, io->RES};
    for (int k = 0; k < 3; k++) {
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, hp[k]) != cudaSuccess || a.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        pinned = false;
      } else {
        dev[k] = a.devicePointer;
      }
    }
  }
  HostIO hio{};
  if (io) {
    hio = *io;
    hio.pinned = pinned;
    if (pinned && hio.Lst) {
      hio.Ldev = (const double *)dev[0];
      hio.Rdev = (const double *)dev[1];
      hio.RESdev = (double *)dev[2];
    }
    io = &hio;
  }
  const bool graphable = !b->prof.on && cs == cudaStreamCaptureStatusNone && pinned &&
                         (precision != IMSRG_PREC_OZAKI || ozaki_tuned(b));
  if (!graphable) return commutator_launches(b, L, hL, R, hR, RES, hRES, precision, with_e0, io, kPhaseAll);
  const HostIO none{nullptr, nullptr, nullptr};
  const HostIO &key = io ? *io : none;
  b->comm_calls++;
  for (imsrg_basis::CommGraph &g : b->comm_graphs)
    if (g.L == L && g.R == R && g.RES == RES && g.hL == hL && g.hR == hR && g.hRES == hRES &&
        g.precision == precision && g.with_e0 == with_e0 && g.io.L == key.L && g.io.R == key.R &&
        g.io.RES == key.RES && g.io.Lst == key.Lst) {
      g.last_use = b->comm_calls;
      b->launches += g.nlaunch;
      return cuda_status(cudaGraphLaunch(g.exec, b->stream));
    }
  // capture the sequence of this argument set
  IMSRG_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const long launches0 = b->launches;
  int s = commutator_launches(b, L, hL, R, hR, RES, hRES, precision, with_e0, io, kPhaseAll);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  IMSRG_TRY(s);
  IMSRG_CUDA_TRY(e);
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  IMSRG_CUDA_TRY(e);
  if (b->comm_graphs.size() >= kCommGraphs) {  // evict the least recently used
    size_t lru = 0;
    for (size_t k = 1; k < b->comm_graphs.size(); k++)
      if (b->comm_graphs[k].last_use < b->comm_graphs[lru].last_use) lru = k;
    cudaGraphExecDestroy(b->comm_graphs[lru].exec);
    b->comm_graphs.erase(b->comm_graphs.begin() + lru);
  }
  b->comm_graphs.push_back({L, R, RES, hL, hR, hRES, precision, with_e0, key, exec, b->comm_calls,
                            b->launches - launches0});
  return cuda_status(cudaGraphLaunch(exec, b->stream));
}

int flow_tmp_ops(imsrg_basis *b, imsrg_op **H0, imsrg_op **DG, imsrg_op **X0, imsrg_op **X1) {
  IMSRG_TRY(tmp_op(b, 0, X0));
  IMSRG_TRY(tmp_op(b, 1, X1));
  IMSRG_TRY(tmp_op(b, 2, H0));
  IMSRG_TRY(tmp_op(b, 3, DG));
  return IMSRG_OK;
}

}  // namespace imsrg

extern "C" {

const char *imsrg_gpu_strerror(int s) {
  switch (s) {
    case IMSRG_OK: return "ok";
    case IMSRG_ERR_INVALID: return "invalid argument, shape or handle";
    case IMSRG_ERR_CUDA: return "CUDA runtime error";
    case IMSRG_ERR_OOM: return "device allocation failed";
    case IMSRG_ERR_NOT_CONVERGED: return "BCH series did not converge in 39 terms (clipping BCH)";
    case IMSRG_ERR_NONFINITE: return "non-finite value in a result";
    case IMSRG_ERR_TIMEOUT: return "a bounded device wait gave up";
    case IMSRG_ERR_MISMATCH: return "operators belong to different bases";
    case IMSRG_ERR_NO_DEVICE: return "no usable CUDA device";
    case IMSRG_ERR_TOO_LARGE: return "basis too large for a fixed-size table or workspace";
    case IMSRG_ERR_IO: return "file could not be written or read (or has the wrong length)";
    default: return "unknown status";
  }
}

int imsrg_gpu_basis_create(int norb, const int *nn, const int *ll, const int *jj, const int *itzp, const int *con,
                           imsrg_basis_t **out) {
  if (!out || norb <= 0 || norb > 4096 || !nn || !ll || !jj || !itzp || !con) return IMSRG_ERR_INVALID;
  *out = nullptr;
  int nholes = 0;
  for (int i = 0; i < norb; i++) {
    if (jj[i] <= 0 || jj[i] % 2 != 1 || ll[i] < 0 || nn[i] < 0) return IMSRG_ERR_INVALID;
    if (itzp[i] != 1 && itzp[i] != -1) return IMSRG_ERR_INVALID;
    if (con[i] != 0 && con[i] != 1) return IMSRG_ERR_INVALID;
    if (std::abs(2 * ll[i] - jj[i]) != 1) return IMSRG_ERR_INVALID;
    nholes += con[i];
  }
  if (nholes == 0 || nholes == norb) return IMSRG_ERR_INVALID;
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0) return IMSRG_ERR_NO_DEVICE;
  imsrg_basis *b = new (std::nothrow) imsrg_basis();
  if (!b) return IMSRG_ERR_OOM;
  b->norb = norb;
  b->nn.assign(nn, nn + norb);
  b->ll.assign(ll, ll + norb);
  b->jj.assign(jj, jj + norb);
  b->itzp.assign(itzp, itzp + norb);
  b->con.assign(con, con + norb);
  int s = imsrg::build_basis(b);
  if (s != IMSRG_OK) {
    imsrg::free_basis_device(b);
    delete b;
    return s;
  }
  *out = b;
  return IMSRG_OK;
}

int imsrg_gpu_basis_destroy(imsrg_basis_t *b) {
  if (!b) return IMSRG_ERR_INVALID;
  for (imsrg_op *op : b->tmp_ops) {
    cudaFree(op->d);
    delete op;
  }
  b->tmp_ops.clear();
  imsrg::free_basis_device(b);
  delete b;
  return IMSRG_OK;
}

int imsrg_gpu_basis_info(const imsrg_basis_t *b, imsrg_basis_info_t *info) {
  if (!b || !info) return IMSRG_ERR_INVALID;
  info->norb = b->norb;
  info->nholes = b->A;
  info->nparts = b->P;
  info->nblocks = b->nblocks;
  info->jtotal_max = b->jtm;
  info->ccblocks = b->ccblocks;
  info->nfull = b->nfull;
  info->neq = b->neq;
  info->cc_total = b->cc_total;
  info->wcc_total = b->wcc_total;
  return IMSRG_OK;
}

int imsrg_gpu_block_dims(const imsrg_basis_t *b, int q, int *npp, int *nph, int *nhh) {
  if (!b || q < 1 || q > b->nblocks) return IMSRG_ERR_INVALID;
  if (npp) *npp = b->npp[q - 1];
  if (nph) *nph = b->nph[q - 1];
  if (nhh) *nhh = b->nhh[q - 1];
  return IMSRG_OK;
}

int imsrg_gpu_synchronize(imsrg_basis_t *b) {
  if (!b) return IMSRG_ERR_INVALID;
  return imsrg::synchronize_checked(b);
}

int imsrg_gpu_launch_count(const imsrg_basis_t *b, long *count) {
  if (!b || !count) return IMSRG_ERR_INVALID;
  *count = b->launches;
  return IMSRG_OK;
}

int imsrg_gpu_op_create(imsrg_basis_t *b, int herm, imsrg_op_t **out) {
  if (!b || !out || (herm != 1 && herm != -1)) return IMSRG_ERR_INVALID;
  *out = nullptr;
  imsrg_op *op = new (std::nothrow) imsrg_op();
  if (!op) return IMSRG_ERR_OOM;
  op->b = b;
  op->herm = herm;
  cudaError_t ce = cudaMalloc(&op->d, b->nfull * sizeof(double));
  if (ce != cudaSuccess) {
    delete op;
    return cuda_status(ce);
  }
  ce = cudaMemsetAsync(op->d, 0, b->nfull * sizeof(double), b->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->stream);
  if (ce != cudaSuccess) {
    cudaFree(op->d);
    delete op;
    return cuda_status(ce);
  }
  *out = op;
  return IMSRG_OK;
}

int imsrg_gpu_op_destroy(imsrg_op_t *op) {
  if (!op) return IMSRG_ERR_INVALID;
  if (op->b) cudaStreamSynchronize(op->b->stream);
  cudaFree(op->d);
  delete op;
  return IMSRG_OK;
}

int imsrg_gpu_op_set_herm(imsrg_op_t *op, int herm) {
  IMSRG_TRY(check_op(op));
  if (herm != 1 && herm != -1) return IMSRG_ERR_INVALID;
  op->herm = herm;
  return IMSRG_OK;
}

int imsrg_gpu_op_get_herm(const imsrg_op_t *op, int *herm) {
  IMSRG_TRY(check_op(op));
  if (!herm) return IMSRG_ERR_INVALID;
  *herm = op->herm;
  return IMSRG_OK;
}

int imsrg_gpu_op_device_ptr(imsrg_op_t *op, double **dptr) {
  IMSRG_TRY(check_op(op));
  if (!dptr) return IMSRG_ERR_INVALID;
  *dptr = op->d;
  return IMSRG_OK;
}

int imsrg_gpu_op_upload_flat(imsrg_op_t *op, const double *flat) {
  IMSRG_TRY(check_op(op));
  if (!flat) return IMSRG_ERR_INVALID;
  imsrg_basis *b = op->b;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(op->d, flat, b->nfull * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

int imsrg_gpu_op_download_flat(const imsrg_op_t *op, double *flat) {
  IMSRG_TRY(check_op(op));
  if (!flat) return IMSRG_ERR_INVALID;
  imsrg_basis *b = op->b;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(flat, op->d, b->nfull * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

int imsrg_gpu_op_upload(imsrg_op_t *op, double e0, const double *fhh, const double *fph, const double *fpp,
                        const double *const *gam) {
  IMSRG_TRY(check_op(op));
  imsrg_basis *b = op->b;
  if ((b->A && !fhh) || (b->A * b->P && !fph) || (b->P && !fpp) || !gam) return IMSRG_ERR_INVALID;
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));  // h_stage may be in flight
  double *h = b->h_stage;
  h[0] = e0;
  std::memcpy(h + b->off_fhh, fhh, (size_t)b->A * b->A * sizeof(double));
  std::memcpy(h + b->off_fph, fph, (size_t)b->P * b->A * sizeof(double));
  std::memcpy(h + b->off_fpp, fpp, (size_t)b->P * b->P * sizeof(double));
  for (int k = 0; k < b->nblocks * 6; k++) {
    size_t n = (size_t)b->gam_n1[k] * b->gam_n2[k];
    if (n == 0) continue;
    if (!gam[k]) return IMSRG_ERR_INVALID;
    std::memcpy(h + b->gam_off[k], gam[k], n * sizeof(double));
  }
  IMSRG_CUDA_TRY(cudaMemcpyAsync(op->d, h, b->nfull * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

int imsrg_gpu_op_download(const imsrg_op_t *op, double *e0, double *fhh, double *fph, double *fpp,
                          double *const *gam) {
  IMSRG_TRY(check_op(op));
  imsrg_basis *b = op->b;
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  double *h = b->h_stage;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(h, op->d, b->nfull * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (e0) *e0 = h[0];
  if (fhh) std::memcpy(fhh, h + b->off_fhh, (size_t)b->A * b->A * sizeof(double));
  if (fph) std::memcpy(fph, h + b->off_fph, (size_t)b->P * b->A * sizeof(double));
  if (fpp) std::memcpy(fpp, h + b->off_fpp, (size_t)b->P * b->P * sizeof(double));
  if (gam) {
    for (int k = 0; k < b->nblocks * 6; k++) {
      size_t n = (size_t)b->gam_n1[k] * b->gam_n2[k];
      if (n == 0 || !gam[k]) continue;
      std::memcpy(gam[k], h + b->gam_off[k], n * sizeof(double));
    }
  }
  return IMSRG_OK;
}

int imsrg_gpu_op_upload_packed(imsrg_op_t *op, const double *packed) {
  IMSRG_TRY(check_op(op));
  if (!packed) return IMSRG_ERR_INVALID;
  imsrg_basis *b = op->b;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(b->d_stage, packed, b->neq * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  IMSRG_TRY(imsrg::launch_unpack(b, b->d_stage, op->herm, op->d));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

int imsrg_gpu_op_download_packed(const imsrg_op_t *op, double *packed) {
  IMSRG_TRY(check_op(op));
  if (!packed) return IMSRG_ERR_INVALID;
  imsrg_basis *b = op->b;
  IMSRG_TRY(imsrg::launch_pack(b, op->d, b->d_stage));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(packed, b->d_stage, b->neq * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

int imsrg_gpu_op_copy(const imsrg_op_t *src, imsrg_op_t *dst) {
  IMSRG_TRY(check_op(src));
  IMSRG_TRY(check_op(dst));
  if (src->b != dst->b) return IMSRG_ERR_MISMATCH;
  dst->herm = src->herm;
  return copy_dev(src->b, src->d, dst->d, src->b->nfull);
}

int imsrg_gpu_op_clear(imsrg_op_t *op) {
  IMSRG_TRY(check_op(op));
  IMSRG_CUDA_TRY(cudaMemsetAsync(op->d, 0, op->b->nfull * sizeof(double), op->b->stream));
  return IMSRG_OK;
}

int imsrg_gpu_op_add(const imsrg_op_t *A, double ax, const imsrg_op_t *B, double bx, imsrg_op_t *C) {
  IMSRG_TRY(check_op(A));
  IMSRG_TRY(check_op(B));
  IMSRG_TRY(check_op(C));
  if (A->b != B->b || A->b != C->b) return IMSRG_ERR_MISMATCH;
  return imsrg::launch_axpby(A->b, A->d, ax, B->d, bx, C->d);
}

int imsrg_gpu_op_norm(const imsrg_op_t *op, double *out) {
  IMSRG_TRY(check_op(op));
  if (!out) return IMSRG_ERR_INVALID;
  return op_norm(op->b, op->d, out);
}

int imsrg_gpu_op_mbpt2(const imsrg_op_t *H, double *out) {
  IMSRG_TRY(check_op(H));
  if (!out) return IMSRG_ERR_INVALID;
  imsrg_basis *b = H->b;
  IMSRG_TRY(imsrg::launch_mbpt2(b, H->d, H->herm, b->scal));
  return read_scalar(b, b->scal, out);
}

int imsrg_gpu_op_get_e0(const imsrg_op_t *op, double *e0) {
  IMSRG_TRY(check_op(op));
  if (!e0) return IMSRG_ERR_INVALID;
  return read_scalar(op->b, op->d, e0);
}

int imsrg_gpu_commutator(const imsrg_op_t *L, const imsrg_op_t *R, imsrg_op_t *RES, int precision, int with_e0) {
  IMSRG_TRY(check_op(L));
  IMSRG_TRY(check_op(R));
  IMSRG_TRY(check_op(RES));
  if (L->b != R->b || L->b != RES->b) return IMSRG_ERR_MISMATCH;
  if (RES == L || RES == R || RES->d == L->d || RES->d == R->d) return IMSRG_ERR_INVALID;
  int hRES = -L->herm * R->herm;
  RES->herm = hRES;
  return imsrg::commutator_dev(L->b, L->d, L->herm, R->d, R->herm, RES->d, hRES, precision, with_e0 ? 1 : 0);
}

int imsrg_gpu_commutator_host(imsrg_basis_t *b, const double *L, int herm_L, const double *R, int herm_R,
                              double *RES, int precision, int with_e0) {
  if (!b || !L || !R || !RES) return IMSRG_ERR_INVALID;
  if ((herm_L != 1 && herm_L != -1) || (herm_R != 1 && herm_R != -1)) return IMSRG_ERR_INVALID;
  const size_t bytes = (size_t)b->nfull * sizeof(double);
  auto overlap = [&](const void *x, const void *y) {
    const char *p = (const char *)x, *q = (const char *)y;
    return p < q + bytes && q < p + bytes;
  };
  if (overlap(RES, L) || overlap(RES, R)) return IMSRG_ERR_INVALID;
  imsrg_op *dL, *dR, *dRES;  // device copies of the operands (work operators 17-19)
  IMSRG_TRY(tmp_op(b, 17, &dL));
  IMSRG_TRY(tmp_op(b, 18, &dR));
  IMSRG_TRY(tmp_op(b, 19, &dRES));
  dL->herm = herm_L;
  dR->herm = herm_R;
  dRES->herm = -herm_L * herm_R;
  const imsrg::HostIO io{L, R, RES};
  IMSRG_TRY(imsrg::commutator_dev(b, dL->d, herm_L, dR->d, herm_R, dRES->d, dRES->herm, precision, with_e0 ? 1 : 0,
                                  &io));
  return imsrg::synchronize_checked(b);
}

int imsrg_gpu_commutator_host_packed(imsrg_basis_t *b, const double *L, int herm_L, const double *R, int herm_R,
                                     double *RES, int precision, int with_e0) {
  if (!b || !L || !R || !RES) return IMSRG_ERR_INVALID;
  if ((herm_L != 1 && herm_L != -1) || (herm_R != 1 && herm_R != -1)) return IMSRG_ERR_INVALID;
  const size_t bytes = (size_t)b->neq * sizeof(double);
  auto overlap = [&](const void *x, const void *y) {
    const char *p = (const char *)x, *q = (const char *)y;
    return p < q + bytes && q < p + bytes;
  };
  if (overlap(RES, L) || overlap(RES, R)) return IMSRG_ERR_INVALID;
  imsrg_op *dL, *dR, *dRES, *sL, *sR, *sRES;  // device operands (17-19) and packed staging (23-25)
  IMSRG_TRY(tmp_op(b, 17, &dL));
  IMSRG_TRY(tmp_op(b, 18, &dR));
  IMSRG_TRY(tmp_op(b, 19, &dRES));
  IMSRG_TRY(tmp_op(b, 23, &sL));
  IMSRG_TRY(tmp_op(b, 24, &sR));
  IMSRG_TRY(tmp_op(b, 25, &sRES));
  dL->herm = herm_L;
  dR->herm = herm_R;
  dRES->herm = -herm_L * herm_R;
  imsrg::HostIO io{L, R, RES};
  io.Lst = sL->d;
  io.Rst = sR->d;
  io.RESst = sRES->d;
  IMSRG_TRY(imsrg::commutator_dev(b, dL->d, herm_L, dR->d, herm_R, dRES->d, dRES->herm, precision, with_e0 ? 1 : 0,
                                  &io));
  return imsrg::synchronize_checked(b);
}

}  // extern "C"

// A batch of independent commutators, one per basis (imsrg_gpu_batch_*).
struct imsrg_batch {
  std::vector<imsrg_basis *> bases;
  void *oz = nullptr;  // the merged split-precision plan
  cudaStream_t st = nullptr;
  cudaEvent_t ev_start = nullptr, ev_mma = nullptr;
  std::vector<cudaEvent_t> ev_front, ev_back;
  struct Graph {
    std::vector<const void *> key;
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;  // one per argument set, least recently built dropped first
  void *flow = nullptr;       // the lockstep flow's step graph (graph.cu), built on first use
  // merged FP64 product lists, one per operand set (graphs replay them)
  struct Fp64List {
    std::vector<const void *> key;
    imsrg::GemmProb *d_probs;
    int nprobs, ntiles;
  };
  std::vector<Fp64List> fp64;
};

namespace {

void batch_release(imsrg_batch *bt) {
  imsrg::batch_flow_free(bt->flow);
  bt->flow = nullptr;
  for (imsrg_batch::Fp64List &l : bt->fp64) cudaFree(l.d_probs);
  bt->fp64.clear();
  for (imsrg_batch::Graph &g : bt->graphs) cudaGraphExecDestroy(g.exec);
  bt->graphs.clear();
  for (cudaEvent_t e : bt->ev_front) cudaEventDestroy(e);
  for (cudaEvent_t e : bt->ev_back) cudaEventDestroy(e);
  if (bt->ev_start) cudaEventDestroy(bt->ev_start);
  if (bt->ev_mma) cudaEventDestroy(bt->ev_mma);
  if (bt->st) cudaStreamDestroy(bt->st);
  imsrg::ozaki_batch_free(bt->oz);
  delete bt;
}

// The merged FP64 product list of the operand set (built on first use).
int batch_fp64_list(imsrg_batch *bt, imsrg_op_t *const *L, imsrg_op_t *const *R, imsrg_batch::Fp64List **out) {
  const int n = (int)bt->bases.size();
  std::vector<const void *> key;
  std::vector<const double *> dl(n), dr(n);
  for (int i = 0; i < n; i++) {
    key.push_back(L[i]->d);
    key.push_back(R[i]->d);
    dl[i] = L[i]->d;
    dr[i] = R[i]->d;
  }
  for (imsrg_batch::Fp64List &l : bt->fp64)
    if (l.key == key) {
      *out = &l;
      return IMSRG_OK;
    }
  imsrg_batch::Fp64List l{key, nullptr, 0, 0};
  IMSRG_TRY(imsrg::gemm_fp64_merged(bt->bases.data(), n, dl.data(), dr.data(), &l.d_probs, &l.nprobs, &l.ntiles));
  bt->fp64.push_back(l);
  *out = &bt->fp64.back();
  return IMSRG_OK;
}

// One step of the batch on the batch stream: every basis's part before the
// products on its own streams, the products of all bases in one launch (the
// split engine's merged plan, or the merged FP64 list), every basis's part
// after them, joined back into the batch stream.
int batch_sequence(imsrg_batch *bt, imsrg_op_t *const *L, imsrg_op_t *const *R, imsrg_op_t *const *RES,
                   int precision, int with_e0) {
  const int n = (int)bt->bases.size();
  const bool oz = precision == IMSRG_PREC_OZAKI;
  imsrg_batch::Fp64List *fl = nullptr;
  // (built, with an allocation, outside any capture: imsrg_gpu_batch_commutator
  // asks for it before it captures a new operand set)
  if (!oz) IMSRG_TRY(batch_fp64_list(bt, L, R, &fl));
  IMSRG_CUDA_TRY(cudaEventRecord(bt->ev_start, bt->st));
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bt->bases[i];
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, bt->ev_start, 0));
    IMSRG_TRY(imsrg::commutator_launches(b, L[i]->d, L[i]->herm, R[i]->d, R[i]->herm, RES[i]->d, RES[i]->herm,
                                         precision, with_e0, nullptr, imsrg::kPhaseFront));
    IMSRG_CUDA_TRY(cudaEventRecord(bt->ev_front[i], b->stream));
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(bt->st, bt->ev_front[i], 0));
  }
  if (oz) {
    IMSRG_TRY(imsrg::ozaki_batch_mma(bt->oz, bt->st, L[0]->herm, R[0]->herm));
  } else {
    IMSRG_TRY(imsrg::launch_gemm_fp64_merged(fl->d_probs, fl->nprobs, fl->ntiles, L[0]->herm, R[0]->herm, nullptr,
                                             bt->st));
  }
  for (imsrg_basis *b : bt->bases) b->launches++;
  IMSRG_CUDA_TRY(cudaEventRecord(bt->ev_mma, bt->st));
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = bt->bases[i];
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(b->stream, bt->ev_mma, 0));
    IMSRG_TRY(imsrg::commutator_launches(b, L[i]->d, L[i]->herm, R[i]->d, R[i]->herm, RES[i]->d, RES[i]->herm,
                                         precision, with_e0, nullptr, imsrg::kPhaseBack));
    IMSRG_CUDA_TRY(cudaEventRecord(bt->ev_back[i], b->stream));
    IMSRG_CUDA_TRY(cudaStreamWaitEvent(bt->st, bt->ev_back[i], 0));
  }
  return IMSRG_OK;
}

}  // namespace

extern "C" {

int imsrg_gpu_batch_create(int n, imsrg_basis_t *const *bases, imsrg_batch_t **out) {
  if (!out || n <= 0 || !bases) return IMSRG_ERR_INVALID;
  *out = nullptr;
  for (int i = 0; i < n; i++) {
    if (!bases[i]) return IMSRG_ERR_INVALID;
    for (int k = 0; k < i; k++)
      if (bases[k] == bases[i]) return IMSRG_ERR_INVALID;  // each basis once: its streams and workspace
  }
  imsrg_batch *bt = new imsrg_batch();
  bt->bases.assign(bases, bases + n);
  int s = IMSRG_OK;
  auto ev = [&](cudaEvent_t *e) {
    if (s == IMSRG_OK) s = imsrg::cuda_status(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  };
  IMSRG_CUDA_TRY(cudaSetDevice(bases[0]->device));
  s = imsrg::cuda_status(cudaStreamCreateWithFlags(&bt->st, cudaStreamNonBlocking));
  ev(&bt->ev_start);
  ev(&bt->ev_mma);
  bt->ev_front.assign(n, nullptr);
  bt->ev_back.assign(n, nullptr);
  for (int i = 0; i < n; i++) {
    ev(&bt->ev_front[i]);
    ev(&bt->ev_back[i]);
  }
  if (s == IMSRG_OK) s = imsrg::ozaki_batch_create(bt->bases.data(), n, &bt->oz);
  if (s != IMSRG_OK) {
    batch_release(bt);
    return s;
  }
  *out = bt;
  return IMSRG_OK;
}

int imsrg_gpu_batch_magnus_decouple(imsrg_batch_t *batch, imsrg_op_t *const *HS, imsrg_op_t *const *G,
                                    double s_max, double ds, int max_steps, int precision, double *const *traces,
                                    int *steps, int *ncomm, int *status) {
  if (!batch || !HS || !G || ds <= 0.0 || max_steps < 0) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  const int n = (int)batch->bases.size();
  for (int i = 0; i < n; i++) {
    IMSRG_TRY(check_op(HS[i]));
    IMSRG_TRY(check_op(G[i]));
    if (HS[i]->b != batch->bases[i] || G[i]->b != batch->bases[i]) return IMSRG_ERR_MISMATCH;
    if (HS[i]->herm != 1 || HS[i] == G[i]) return IMSRG_ERR_INVALID;
  }
  return imsrg::batch_flow_run(batch->bases.data(), n, batch->oz, batch->st, &batch->flow, HS, G, s_max, ds,
                               max_steps, precision, traces, steps, ncomm, status);
}

int imsrg_gpu_batch_destroy(imsrg_batch_t *batch) {
  if (!batch) return IMSRG_ERR_INVALID;
  cudaStreamSynchronize(batch->st);
  batch_release(batch);
  return IMSRG_OK;
}

int imsrg_gpu_batch_commutator(imsrg_batch_t *batch, imsrg_op_t *const *L, imsrg_op_t *const *R,
                               imsrg_op_t *const *RES, int precision, int with_e0) {
  if (!batch || !L || !R || !RES) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  const int n = (int)batch->bases.size();
  bool graphable = true;
  std::vector<const void *> key{(const void *)(long)precision, (const void *)(long)(with_e0 ? 1 : 0)};
  for (int i = 0; i < n; i++) {
    imsrg_basis *b = batch->bases[i];
    for (imsrg_op_t *op : {L[i], R[i], RES[i]}) {
      IMSRG_TRY(check_op(op));
      if (op->b != b) return IMSRG_ERR_MISMATCH;
    }
    if (RES[i] == L[i] || RES[i] == R[i]) return IMSRG_ERR_INVALID;
    // one launch takes one pair of Hermiticities
    if (L[i]->herm != L[0]->herm || R[i]->herm != R[0]->herm) return IMSRG_ERR_INVALID;
    RES[i]->herm = -L[i]->herm * R[i]->herm;
    graphable = graphable && !b->prof.on;
    key.push_back(L[i]->d);
    key.push_back(R[i]->d);
    key.push_back(RES[i]->d);
  }
  key.push_back((const void *)(long)L[0]->herm);
  key.push_back((const void *)(long)R[0]->herm);
  if (!graphable) {
    IMSRG_TRY(batch_sequence(batch, L, R, RES, precision, with_e0 ? 1 : 0));
  } else {
    cudaGraphExec_t exec = nullptr;
    for (const imsrg_batch::Graph &g : batch->graphs)
      if (g.key == key) exec = g.exec;
    if (!exec) {
      if (precision == IMSRG_PREC_FP64) {  // allocate the merged FP64 list before capturing
        imsrg_batch::Fp64List *fl = nullptr;
        IMSRG_TRY(batch_fp64_list(batch, L, R, &fl));
      }
      IMSRG_CUDA_TRY(cudaStreamBeginCapture(batch->st, cudaStreamCaptureModeThreadLocal));
      const int s = batch_sequence(batch, L, R, RES, precision, with_e0 ? 1 : 0);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(batch->st, &graph);
      IMSRG_TRY(s);
      IMSRG_CUDA_TRY(e);
      const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      IMSRG_CUDA_TRY(ei);
      if (batch->graphs.size() >= 4) {
        cudaGraphExecDestroy(batch->graphs.front().exec);
        batch->graphs.erase(batch->graphs.begin());
      }
      batch->graphs.push_back({key, exec});
    }
    IMSRG_CUDA_TRY(cudaGraphLaunch(exec, batch->st));
  }
  IMSRG_CUDA_TRY(cudaStreamSynchronize(batch->st));
  if (precision == IMSRG_PREC_OZAKI) IMSRG_TRY(imsrg::ozaki_batch_error(batch->oz, batch->st));
  return IMSRG_OK;
}

int imsrg_gpu_build_gs_white(const imsrg_op_t *H, imsrg_op_t *ETA) {
  IMSRG_TRY(check_op(H));
  IMSRG_TRY(check_op(ETA));
  if (H->b != ETA->b) return IMSRG_ERR_MISMATCH;
  if (H == ETA) return IMSRG_ERR_INVALID;
  ETA->herm = -1;
  return imsrg::launch_white(H->b, H->d, H->herm, ETA->d);
}

int imsrg_gpu_euler_step(imsrg_op_t *G, const imsrg_op_t *DG, double *s, double ds) {
  IMSRG_TRY(check_op(G));
  IMSRG_TRY(check_op(DG));
  if (G->b != DG->b) return IMSRG_ERR_MISMATCH;
  IMSRG_TRY(imsrg::launch_axpby(G->b, G->d, 1.0, DG->d, ds, G->d));
  if (s) *s = *s + ds;
  return IMSRG_OK;
}

int imsrg_gpu_magnus_expand(imsrg_op_t *DG, const imsrg_op_t *G, int precision, int *ncomm) {
  IMSRG_TRY(check_op(DG));
  IMSRG_TRY(check_op(G));
  if (DG->b != G->b) return IMSRG_ERR_MISMATCH;
  imsrg_basis *b = DG->b;
  const double conv = 1e-6;
  imsrg_op *X[2];
  IMSRG_TRY(tmp_op(b, 0, &X[0]));
  IMSRG_TRY(tmp_op(b, 1, &X[1]));
  int nc = 0;
  double advals[8] = {0};
  // INT2 = DG; the E0 of INT2 never changes inside the loop (no 110/220)
  IMSRG_TRY(copy_dev(b, DG->d, X[0]->d, b->nfull));
  IMSRG_TRY(copy_dev(b, DG->d, X[1]->d, 1));
  X[0]->herm = X[1]->herm = DG->herm;
  IMSRG_TRY(op_norm(b, X[0]->d, &advals[1]));
  double fullnorm = 0.0;
  IMSRG_TRY(op_norm(b, G->d, &fullnorm));
  if (fullnorm < 1e-9) {
    if (ncomm) *ncomm = 0;
    return IMSRG_OK;
  }
  int q = 1, cur = 0;
  for (int i = 2; i <= 7; i++) {
    double adnorm = advals[i - q];
    q = (std::fabs(kMagnusCof[i - 1]) > 1e-6) ? 1 : 2;
    if (std::fabs(adnorm / fullnorm) < conv) break;
    imsrg_op *AD = X[cur], *INT2 = X[1 - cur];
    int h = -G->herm * AD->herm;
    INT2->herm = h;
    IMSRG_TRY(imsrg::commutator_dev(b, G->d, G->herm, AD->d, AD->herm, INT2->d, h, precision, 0));
    nc++;
    IMSRG_TRY(imsrg::launch_axpby(b, DG->d, 1.0, INT2->d, kMagnusCof[i - 1], DG->d));
    double nrm = 0.0;
    IMSRG_TRY(op_norm(b, INT2->d, &nrm));
    if (!std::isfinite(nrm)) return IMSRG_ERR_NONFINITE;
    advals[i] = nrm * std::fabs(kMagnusCof[i - 1]);
    cur = 1 - cur;
  }
  if (ncomm) *ncomm = nc;
  return IMSRG_OK;
}

int imsrg_gpu_bch_expand(imsrg_op_t *HS, const imsrg_op_t *G, const imsrg_op_t *H, int precision, int *ncomm) {
  IMSRG_TRY(check_op(HS));
  IMSRG_TRY(check_op(G));
  IMSRG_TRY(check_op(H));
  if (HS->b != G->b || HS->b != H->b) return IMSRG_ERR_MISMATCH;
  imsrg_basis *b = HS->b;
  const double conv = 1e-6;
  imsrg_op *X[2];
  IMSRG_TRY(tmp_op(b, 0, &X[0]));
  IMSRG_TRY(tmp_op(b, 1, &X[1]));
  HS->herm = H->herm;
  IMSRG_TRY(copy_dev(b, H->d, HS->d, b->nfull));
  IMSRG_TRY(copy_dev(b, H->d, X[0]->d, b->nfull));
  X[0]->herm = H->herm;
  double coef = 1.0;
  int nc = 0, cur = 0, iw;
  for (iw = 2; iw <= 40; iw++) {
    coef = coef / (iw - 1.0);
    imsrg_op *AD = X[cur], *INT2 = X[1 - cur];
    int h = -G->herm * AD->herm;
    INT2->herm = h;
    IMSRG_TRY(imsrg::commutator_dev(b, G->d, G->herm, AD->d, AD->herm, INT2->d, h, precision, 1));
    nc++;
    IMSRG_TRY(imsrg::launch_axpby(b, HS->d, 1.0, INT2->d, coef, HS->d));
    double nrm = 0.0;
    IMSRG_TRY(op_norm(b, INT2->d, &nrm));
    if (!std::isfinite(nrm)) return IMSRG_ERR_NONFINITE;
    cur = 1 - cur;
    if (nrm * coef < conv) break;
  }
  if (ncomm) *ncomm = nc;
  return (iw > 40) ? IMSRG_ERR_NOT_CONVERGED : IMSRG_OK;
}

int imsrg_gpu_normal_order(imsrg_op_t *H) {
  IMSRG_TRY(check_op(H));
  imsrg_basis *b = H->b;
  imsrg_op *T;
  IMSRG_TRY(tmp_op(b, 12, &T));
  IMSRG_TRY(copy_dev(b, H->d, T->d, b->nfull));
  return imsrg::launch_normal_order(b, T->d, H->herm, H->d);
}

int imsrg_gpu_transform_bch(imsrg_op_t *Op, const imsrg_op_t *G, int precision, int *ncomm) {
  IMSRG_TRY(check_op(Op));
  IMSRG_TRY(check_op(G));
  if (Op->b != G->b) return IMSRG_ERR_MISMATCH;
  imsrg_op *E;
  IMSRG_TRY(tmp_op(Op->b, 13, &E));
  IMSRG_TRY(imsrg_gpu_bch_expand(E, G, Op, precision, ncomm));
  return imsrg_gpu_op_copy(E, Op);
}

int imsrg_gpu_dhds(const imsrg_op_t *HS, imsrg_op_t *DH, int generator, int precision) {
  IMSRG_TRY(check_op(HS));
  IMSRG_TRY(check_op(DH));
  if (HS->b != DH->b) return IMSRG_ERR_MISMATCH;
  if (HS == DH) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  DH->herm = HS->herm;
  return imsrg::dhds_dev(HS->b, HS->d, HS->herm, DH->d, generator, precision);
}

int imsrg_gpu_op_save(const imsrg_op_t *op, const char *path) {
  IMSRG_TRY(check_op(op));
  if (!path) return IMSRG_ERR_INVALID;
  std::vector<double> v(op->b->neq);
  IMSRG_TRY(imsrg_gpu_op_download_packed(op, v.data()));
  FILE *f = std::fopen(path, "wb");
  if (!f) return IMSRG_ERR_IO;
  const size_t n = std::fwrite(v.data(), sizeof(double), v.size(), f);
  const int c = std::fclose(f);
  return (n == v.size() && c == 0) ? IMSRG_OK : IMSRG_ERR_IO;
}

int imsrg_gpu_op_load(imsrg_op_t *op, const char *path) {
  IMSRG_TRY(check_op(op));
  if (!path) return IMSRG_ERR_INVALID;
  FILE *f = std::fopen(path, "rb");
  if (!f) return IMSRG_ERR_IO;
  std::vector<double> v(op->b->neq);
  const size_t n = std::fread(v.data(), sizeof(double), v.size(), f);
  const bool at_end = std::fgetc(f) == EOF;
  std::fclose(f);
  if (n != v.size() || !at_end) return IMSRG_ERR_IO;
  return imsrg_gpu_op_upload_packed(op, v.data());
}

int imsrg_gpu_checkpoint_name(const char *dir, const char *prefix, double s, char *out, int outlen) {
  if (!dir || !prefix || !out || outlen <= 0) return IMSRG_ERR_INVALID;
  // the run prefix up to its 'hw' field and two characters after it
  const char *hw = std::strstr(prefix, "hw");
  const size_t keep = hw ? std::min(std::strlen(prefix), (size_t)(hw - prefix) + 4) : std::strlen(prefix);
  // f6.3 of s, left-adjusted; a trailing 0 below s = 10 (the reference's
  // character(8) slot then holds '_s' and six characters)
  char num[32];
  std::snprintf(num, sizeof(num), "%6.3f", s);
  const char *p = num;
  while (*p == ' ') p++;
  const int len = std::snprintf(out, outlen, "%s%.*s_s%s%s.bin", dir, (int)keep, prefix, p, s < 10.0 ? "0" : "");
  return (len > 0 && len < outlen) ? IMSRG_OK : IMSRG_ERR_INVALID;
}

int imsrg_gpu_build_gs_atan(const imsrg_op_t *H, imsrg_op_t *ETA) {
  IMSRG_TRY(check_op(H));
  IMSRG_TRY(check_op(ETA));
  if (H->b != ETA->b) return IMSRG_ERR_MISMATCH;
  if (H == ETA) return IMSRG_ERR_INVALID;
  ETA->herm = -1;
  return generator_dev(H->b, H->d, H->herm, ETA->d, IMSRG_GEN_ATAN, IMSRG_PREC_FP64);
}

int imsrg_gpu_build_gs_w2(const imsrg_op_t *H, imsrg_op_t *ETA, int precision) {
  IMSRG_TRY(check_op(H));
  IMSRG_TRY(check_op(ETA));
  if (H->b != ETA->b) return IMSRG_ERR_MISMATCH;
  if (H == ETA) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  ETA->herm = -1;
  return generator_dev(H->b, H->d, H->herm, ETA->d, IMSRG_GEN_W2, precision);
}

int imsrg_gpu_magnus_decouple(imsrg_op_t *HS, imsrg_op_t *G, double s_max, double ds, int max_steps, int precision,
                              double *trace, int *steps_out, int *ncomm) {
  return imsrg_gpu_magnus_decouple_gen(HS, G, IMSRG_GEN_WHITE, s_max, ds, max_steps, precision, trace, steps_out,
                                       ncomm);
}

int imsrg_gpu_magnus_decouple_gen(imsrg_op_t *HS, imsrg_op_t *G, int generator, double s_max, double ds,
                                  int max_steps, int precision, double *trace, int *steps_out, int *ncomm) {
  if (generator != IMSRG_GEN_WHITE && generator != IMSRG_GEN_ATAN && generator != IMSRG_GEN_W2)
    return IMSRG_ERR_INVALID;
  IMSRG_TRY(check_op(HS));
  IMSRG_TRY(check_op(G));
  if (HS->b != G->b) return IMSRG_ERR_MISMATCH;
  if (ds <= 0.0 || max_steps < 0) return IMSRG_ERR_INVALID;
  imsrg_basis *b = HS->b;
  imsrg_op *H0, *DG;
  IMSRG_TRY(tmp_op(b, 2, &H0));
  IMSRG_TRY(tmp_op(b, 3, &DG));
  IMSRG_CUDA_TRY(cudaMemsetAsync(G->d, 0, b->nfull * sizeof(double), b->stream));
  IMSRG_CUDA_TRY(cudaMemsetAsync(DG->d, 0, b->nfull * sizeof(double), b->stream));
  G->herm = -1;
  DG->herm = -1;
  IMSRG_TRY(generator_dev(b, HS->d, HS->herm, DG->d, generator, precision));
  IMSRG_TRY(copy_dev(b, HS->d, H0->d, b->nfull));
  H0->herm = HS->herm;
  double s = 0.0, e0 = 0.0, emp2 = 0.0;
  IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
  IMSRG_TRY(read_scalar(b, HS->d, &e0));
  double crit = std::fabs(emp2);
  if (trace) {
    trace[0] = 0; trace[1] = s; trace[2] = e0; trace[3] = e0 + emp2; trace[4] = crit;
  }
  int steps = 0, nct = 0;
  while (crit > 1e-6 && s < s_max - 1e-12 && steps < max_steps) {
    steps++;
    int nm = 0, nb = 0;
    IMSRG_TRY(imsrg_gpu_magnus_expand(DG, G, precision, &nm));
    IMSRG_TRY(imsrg_gpu_euler_step(G, DG, &s, ds));
    int st = imsrg_gpu_bch_expand(HS, G, H0, precision, &nb);
    nct += nm + nb;
    if (st != IMSRG_OK) {
      if (steps_out) *steps_out = steps;
      if (ncomm) *ncomm = nct;
      return st;
    }
    IMSRG_TRY(generator_dev(b, HS->d, HS->herm, DG->d, generator, precision));
    IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
    IMSRG_TRY(read_scalar(b, HS->d, &e0));
    if (!std::isfinite(e0) || !std::isfinite(emp2)) return IMSRG_ERR_NONFINITE;
    crit = std::fabs(emp2);
    if (trace) {
      double *t = trace + 5 * steps;
      t[0] = steps; t[1] = s; t[2] = e0; t[3] = e0 + emp2; t[4] = crit;
    }
  }
  if (steps_out) *steps_out = steps;
  if (ncomm) *ncomm = nct;
  return IMSRG_OK;
}

// --- tangent-linear flow -------------------------------------------------
// The Magnus flow together with its derivative along one direction dH of the
// input Hamiltonian (forward mode): every nested commutator T_n = [G, T_n-1]
// carries dT_n = [dG, T_n-1] + [G, dT_n-1], the White generator its tangent,
// and the series keep the term counts and stops of the undifferentiated flow.
// dtrace rows: (step, s, dE0 along dH, 0, 0).
namespace {

int tangent_commutator(imsrg_basis *b, const imsrg_op *G, const imsrg_op *dG, const imsrg_op *A, const imsrg_op *dA,
                       imsrg_op *X, imsrg_op *dX, imsrg_op *T1, int precision, int with_e0) {
  const int h = -G->herm * A->herm;
  X->herm = dX->herm = T1->herm = h;
  IMSRG_TRY(imsrg::commutator_dev(b, G->d, G->herm, A->d, A->herm, X->d, h, precision, with_e0));
  IMSRG_TRY(imsrg::commutator_dev(b, dG->d, G->herm, A->d, A->herm, T1->d, h, precision, with_e0));
  IMSRG_TRY(imsrg::commutator_dev(b, G->d, G->herm, dA->d, A->herm, dX->d, h, precision, with_e0));
  return imsrg::launch_axpby(b, dX->d, 1.0, T1->d, 1.0, dX->d);
}

}  // namespace

int imsrg_gpu_magnus_decouple_tangent(imsrg_op_t *HS, imsrg_op_t *dHS, imsrg_op_t *G, imsrg_op_t *dG, double s_max,
                                      double ds, int max_steps, int precision, double *trace, double *dtrace,
                                      int *steps_out, int *ncomm) {
  IMSRG_TRY(check_op(HS));
  IMSRG_TRY(check_op(dHS));
  IMSRG_TRY(check_op(G));
  IMSRG_TRY(check_op(dG));
  imsrg_basis *b = HS->b;
  if (dHS->b != b || G->b != b || dG->b != b) return IMSRG_ERR_MISMATCH;
  if (ds <= 0.0 || max_steps < 0) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  imsrg_op *A, *X, *H0, *DG, *dH0, *dDG, *dA, *dX, *T1;
  IMSRG_TRY(tmp_op(b, 0, &A));
  IMSRG_TRY(tmp_op(b, 1, &X));
  IMSRG_TRY(tmp_op(b, 2, &H0));
  IMSRG_TRY(tmp_op(b, 3, &DG));
  IMSRG_TRY(tmp_op(b, 4, &dH0));
  IMSRG_TRY(tmp_op(b, 5, &dDG));
  IMSRG_TRY(tmp_op(b, 6, &dA));
  IMSRG_TRY(tmp_op(b, 7, &dX));
  IMSRG_TRY(tmp_op(b, 8, &T1));
  const long nf = b->nfull;
  const double conv = 1e-6;
  IMSRG_CUDA_TRY(cudaMemsetAsync(G->d, 0, nf * sizeof(double), b->stream));
  IMSRG_CUDA_TRY(cudaMemsetAsync(dG->d, 0, nf * sizeof(double), b->stream));
  G->herm = dG->herm = DG->herm = dDG->herm = -1;
  dHS->herm = HS->herm;
  IMSRG_TRY(imsrg::launch_white(b, HS->d, HS->herm, DG->d));
  IMSRG_TRY(imsrg::launch_white_tangent(b, HS->d, dHS->d, HS->herm, dDG->d));
  IMSRG_TRY(copy_dev(b, HS->d, H0->d, nf));
  IMSRG_TRY(copy_dev(b, dHS->d, dH0->d, nf));
  H0->herm = dH0->herm = HS->herm;
  double s = 0.0, e0 = 0.0, de0 = 0.0, emp2 = 0.0;
  IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
  IMSRG_TRY(read_scalar(b, HS->d, &e0));
  IMSRG_TRY(read_scalar(b, dHS->d, &de0));
  double crit = std::fabs(emp2);
  auto row = [&](int k) {
    if (trace) {
      double *t = trace + 5 * k;
      t[0] = k; t[1] = s; t[2] = e0; t[3] = e0 + emp2; t[4] = crit;
    }
    if (dtrace) {
      double *t = dtrace + 5 * k;
      t[0] = k; t[1] = s; t[2] = de0; t[3] = 0.0; t[4] = 0.0;
    }
  };
  row(0);
  int steps = 0, nct = 0;
  while (crit > 1e-6 && s < s_max - 1e-12 && steps < max_steps) {
    steps++;
    // MAGNUS_EXPAND and its tangent (IMSRG_MAGNUS.f90:622-693)
    double advals[8] = {0}, fullnorm = 0.0;
    IMSRG_TRY(copy_dev(b, DG->d, A->d, nf));
    IMSRG_TRY(copy_dev(b, DG->d, X->d, 1));
    IMSRG_TRY(copy_dev(b, dDG->d, dA->d, nf));
    IMSRG_TRY(copy_dev(b, dDG->d, dX->d, 1));
    IMSRG_CUDA_TRY(cudaMemsetAsync(T1->d, 0, sizeof(double), b->stream));
    A->herm = dA->herm = -1;
    IMSRG_TRY(op_norm(b, A->d, &advals[1]));
    IMSRG_TRY(op_norm(b, G->d, &fullnorm));
    if (!(fullnorm < 1e-9)) {
      int q = 1;
      for (int i = 2; i <= 7; i++) {
        double adnorm = advals[i - q];
        q = (std::fabs(kMagnusCof[i - 1]) > 1e-6) ? 1 : 2;
        if (std::fabs(adnorm / fullnorm) < conv) break;
        IMSRG_TRY(tangent_commutator(b, G, dG, A, dA, X, dX, T1, precision, 0));
        nct += 3;
        IMSRG_TRY(imsrg::launch_axpby(b, DG->d, 1.0, X->d, kMagnusCof[i - 1], DG->d));
        IMSRG_TRY(imsrg::launch_axpby(b, dDG->d, 1.0, dX->d, kMagnusCof[i - 1], dDG->d));
        double nrm = 0.0;
        IMSRG_TRY(op_norm(b, X->d, &nrm));
        if (!std::isfinite(nrm)) return IMSRG_ERR_NONFINITE;
        advals[i] = nrm * std::fabs(kMagnusCof[i - 1]);
        IMSRG_TRY(copy_dev(b, X->d, A->d, nf));
        IMSRG_TRY(copy_dev(b, dX->d, dA->d, nf));
      }
    }
    // euler_step
    IMSRG_TRY(imsrg::launch_axpby(b, G->d, 1.0, DG->d, ds, G->d));
    IMSRG_TRY(imsrg::launch_axpby(b, dG->d, 1.0, dDG->d, ds, dG->d));
    s += ds;
    // BCH_EXPAND and its tangent (IMSRG_MAGNUS.f90:149-234)
    IMSRG_TRY(copy_dev(b, H0->d, HS->d, nf));
    IMSRG_TRY(copy_dev(b, dH0->d, dHS->d, nf));
    IMSRG_TRY(copy_dev(b, H0->d, A->d, nf));
    IMSRG_TRY(copy_dev(b, dH0->d, dA->d, nf));
    A->herm = dA->herm = H0->herm;
    double coef = 1.0;
    int iw;
    for (iw = 2; iw <= 40; iw++) {
      coef = coef / (iw - 1.0);
      IMSRG_TRY(tangent_commutator(b, G, dG, A, dA, X, dX, T1, precision, 1));
      nct += 3;
      IMSRG_TRY(imsrg::launch_axpby(b, HS->d, 1.0, X->d, coef, HS->d));
      IMSRG_TRY(imsrg::launch_axpby(b, dHS->d, 1.0, dX->d, coef, dHS->d));
      double nrm = 0.0;
      IMSRG_TRY(op_norm(b, X->d, &nrm));
      if (!std::isfinite(nrm)) return IMSRG_ERR_NONFINITE;
      IMSRG_TRY(copy_dev(b, X->d, A->d, nf));
      IMSRG_TRY(copy_dev(b, dX->d, dA->d, nf));
      A->herm = dA->herm = X->herm;
      if (nrm * coef < conv) break;
    }
    if (iw > 40) {
      if (steps_out) *steps_out = steps;
      if (ncomm) *ncomm = nct;
      return IMSRG_ERR_NOT_CONVERGED;
    }
    IMSRG_TRY(imsrg::launch_white(b, HS->d, HS->herm, DG->d));
    IMSRG_TRY(imsrg::launch_white_tangent(b, HS->d, dHS->d, HS->herm, dDG->d));
    IMSRG_TRY(imsrg_gpu_op_mbpt2(HS, &emp2));
    IMSRG_TRY(read_scalar(b, HS->d, &e0));
    IMSRG_TRY(read_scalar(b, dHS->d, &de0));
    if (!std::isfinite(e0) || !std::isfinite(emp2) || !std::isfinite(de0)) return IMSRG_ERR_NONFINITE;
    crit = std::fabs(emp2);
    row(steps);
  }
  if (steps_out) *steps_out = steps;
  if (ncomm) *ncomm = nct;
  return IMSRG_OK;
}

int imsrg_gpu_magnus_decouple_batch(int n, imsrg_op_t *const *HS, imsrg_op_t *const *G, double s_max, double ds,
                                    int max_steps, int precision, double *const *traces, int *steps_out, int *ncomm,
                                    int *status) {
  if (n <= 0 || !HS || !G || ds <= 0.0 || max_steps < 0) return IMSRG_ERR_INVALID;
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_OZAKI) return IMSRG_ERR_INVALID;
  for (int i = 0; i < n; i++) {
    IMSRG_TRY(check_op(HS[i]));
    IMSRG_TRY(check_op(G[i]));
    if (HS[i]->b != G[i]->b) return IMSRG_ERR_MISMATCH;
    for (int j = 0; j < i; j++)
      if (HS[j]->b == HS[i]->b) return IMSRG_ERR_INVALID;  // instances need their own workspace
  }
  std::vector<double> s(n, 0.0), crit(n, 0.0);
  std::vector<int> steps(n, 0), nct(n, 0), st(n, IMSRG_OK);
  for (int i = 0; i < n; i++) {
    double e0 = 0.0, emp2 = 0.0;
    IMSRG_TRY(imsrg::flow_graph_begin(HS[i], G[i], precision, ds, &e0, &emp2));
    crit[i] = std::fabs(emp2);
    if (traces && traces[i]) {
      double *t = traces[i];
      t[0] = 0; t[1] = 0.0; t[2] = e0; t[3] = e0 + emp2; t[4] = crit[i];
    }
  }
  auto active = [&](int i) { return st[i] == IMSRG_OK && crit[i] > 1e-6 && s[i] < s_max - 1e-12 && steps[i] < max_steps; };
  for (;;) {
    int nact = 0;
    for (int i = 0; i < n; i++)
      if (active(i)) {
        IMSRG_TRY(imsrg::flow_graph_launch(HS[i]->b));
        nact++;
      }
    if (!nact) break;
    for (int i = 0; i < n; i++) {
      if (!active(i)) continue;
      double e0, emp2;
      int nc, stat;
      IMSRG_TRY(imsrg::flow_graph_finish(HS[i]->b, &s[i], &e0, &emp2, &nc, &stat));
      steps[i]++;
      nct[i] += nc;
      if (stat == IMSRG_OK && (!std::isfinite(e0) || !std::isfinite(emp2))) stat = IMSRG_ERR_NONFINITE;
      st[i] = stat;
      crit[i] = std::fabs(emp2);
      if (stat == IMSRG_OK && traces && traces[i]) {
        double *t = traces[i] + 5 * steps[i];
        t[0] = steps[i]; t[1] = s[i]; t[2] = e0; t[3] = e0 + emp2; t[4] = crit[i];
      }
    }
  }
  int worst = IMSRG_OK;
  for (int i = 0; i < n; i++) {
    if (steps_out) steps_out[i] = steps[i];
    if (ncomm) ncomm[i] = nct[i];
    if (status) status[i] = st[i];
    if (st[i] != IMSRG_OK && worst == IMSRG_OK) worst = st[i];
  }
  return worst;
}

int imsrg_gpu_magnus_decouple_graph(imsrg_op_t *HS, imsrg_op_t *G, double s_max, double ds, int max_steps,
                                    int precision, double *trace, int *steps_out, int *ncomm) {
  double *traces[1] = {trace};
  return imsrg_gpu_magnus_decouple_batch(1, &HS, &G, s_max, ds, max_steps, precision, traces, steps_out, ncomm,
                                         nullptr);
}

int imsrg_gpu_split_schedule(imsrg_basis_t *b, int *choice, int *ncand, double *us, int max) {
  if (!b) return IMSRG_ERR_INVALID;
  return imsrg::ozaki_schedule_info(b, choice, ncand, us, max);
}

int imsrg_gpu_split_digits_set(imsrg_basis_t *b, int digits) {
  if (!b || digits < 4 || digits > 8) return IMSRG_ERR_INVALID;
  if (b->ozaki) return digits == b->split_digits ? IMSRG_OK : IMSRG_ERR_INVALID;  // plan already built
  b->split_digits = digits;
  return IMSRG_OK;
}

int imsrg_gpu_split_chunk_set(imsrg_basis_t *b, int steps) {
  if (!b || steps < 0) return IMSRG_ERR_INVALID;
  if (b->ozaki) return steps == b->split_chunk_steps ? IMSRG_OK : IMSRG_ERR_INVALID;  // plan already built
  b->split_chunk_steps = steps;
  return IMSRG_OK;
}

int imsrg_gpu_split_schedule_set(imsrg_basis_t *b, int model) {
  if (!b) return IMSRG_ERR_INVALID;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  IMSRG_CUDA_TRY(cudaStreamIsCapturing(b->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return IMSRG_ERR_INVALID;
  return imsrg::ozaki_set_schedule(b, model);
}

}  // extern "C"
