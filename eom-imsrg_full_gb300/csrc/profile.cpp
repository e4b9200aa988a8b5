// profile.cpp -- live per-kernel timing with CUDA events on the basis stream.
#include "internal.h"

namespace imsrg {

namespace {
cudaEvent_t get_event(imsrg_basis *b) {
  Profiler &p = b->prof;
  if (!p.pool.empty()) {
    cudaEvent_t e = p.pool.back();
    p.pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}
}  // namespace

ProfScope::ProfScope(imsrg_basis *b_, int kind_, cudaStream_t st_) : b(b_), kind(kind_), st(st_ ? st_ : b_->stream) {
  if (!b->prof.on) return;
  start = get_event(b);
  if (start) cudaEventRecord(start, st);
}

ProfScope::~ProfScope() {
  if (!start) return;
  cudaEvent_t stop = get_event(b);
  if (!stop) {
    b->prof.pool.push_back(start);
    return;
  }
  cudaEventRecord(stop, st);
  b->prof.pending.push_back({kind, start, stop});
  if (b->prof.pending.size() > 8192) profile_collect(b);
}

int profile_collect(imsrg_basis *b) {
  Profiler &p = b->prof;
  if (p.pending.empty()) return IMSRG_OK;
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (const Profiler::Pending &q : p.pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, q.start, q.stop) == cudaSuccess) {
      p.ms[q.kind] += ms;
      p.n[q.kind] += 1;
    }
    p.pool.push_back(q.start);
    p.pool.push_back(q.stop);
  }
  p.pending.clear();
  return IMSRG_OK;
}

void profile_free(imsrg_basis *b) {
  Profiler &p = b->prof;
  for (const Profiler::Pending &q : p.pending) {
    cudaEventDestroy(q.start);
    cudaEventDestroy(q.stop);
  }
  for (cudaEvent_t e : p.pool) cudaEventDestroy(e);
  p.pending.clear();
  p.pool.clear();
}

}  // namespace imsrg

extern "C" {

int imsrg_gpu_profile_enable(imsrg_basis_t *b, int on) {
  if (!b) return IMSRG_ERR_INVALID;
  b->prof.on = on != 0;
  return IMSRG_OK;
}

int imsrg_gpu_profile_read(imsrg_basis_t *b, int kernel, double *ms, long *launches) {
  if (!b || kernel < 0 || kernel >= IMSRG_KERNEL_COUNT) return IMSRG_ERR_INVALID;
  IMSRG_TRY(imsrg::profile_collect(b));
  if (ms) *ms = b->prof.ms[kernel];
  if (launches) *launches = b->prof.n[kernel];
  return IMSRG_OK;
}

int imsrg_gpu_profile_reset(imsrg_basis_t *b) {
  if (!b) return IMSRG_ERR_INVALID;
  IMSRG_TRY(imsrg::profile_collect(b));
  for (int k = 0; k < IMSRG_KERNEL_COUNT; k++) {
    b->prof.ms[k] = 0.0;
    b->prof.n[k] = 0;
  }
  return IMSRG_OK;
}

int imsrg_gpu_basis_get_stream(imsrg_basis_t *b, void **stream) {
  if (!b || !stream) return IMSRG_ERR_INVALID;
  *stream = (void *)b->stream;
  return IMSRG_OK;
}

int imsrg_gpu_basis_set_stream(imsrg_basis_t *b, void *stream) {
  if (!b) return IMSRG_ERR_INVALID;
  IMSRG_TRY(imsrg::profile_collect(b));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;
  return IMSRG_OK;
}

}  // extern "C"
