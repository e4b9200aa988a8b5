// noalloc.cu -- the allocation-free FP64 commutator entry point.
//
// Some callers may not allocate device memory while they run (their memory is
// owned or capped by another allocator, or a cudaMalloc/cudaFree, which can
// synchronise the device, is not allowed where they call from).  For them the
// commutator's intermediates (W1, W2, LCC, RCC, WCC) live in one file-scope
// device array of fixed size instead of the basis workspace.  In host code
// g_noalloc_scratch is only a stand-in symbol, never a device address: its
// address is looked up with cudaGetSymbolAddress once per device, with that
// device current, and passed to the kernels.
#include <cstdint>
#include <mutex>

#include "internal.h"

namespace imsrg {
namespace {

// Every GPU that loads the library holds these 8 MiB until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[IMSRG_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.  The first call
// for a device is its set-up: it looks the address up and loads the device
// code of every kernel this path launches (with lazy module loading both
// would otherwise happen, and could allocate, inside a later call).
int scratch_address(int dev, double **out) {
  if (dev < 0 || dev >= kMaxDevices) return IMSRG_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    int s = preload_commutator_fp64_ws();
    if (s != IMSRG_OK) return s;
    g_scratch_ptr[dev] = (double *)p;
  }
  *out = g_scratch_ptr[dev];
  return IMSRG_OK;
}

// True when [a, a + n) and [b, b + n) share an element.
bool overlaps(const double *a, const double *b, long n) {
  const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b, len = (uintptr_t)n * sizeof(double);
  return x < y + len && y < x + len;
}

long round_up(long n) { return (n + 31) / 32 * 32; }

}  // namespace
}  // namespace imsrg

extern "C" int imsrg_gpu_commutator_noalloc(imsrg_basis_t *b, const double *d_L, int herm_L, const double *d_R,
                                            int herm_R, double *d_RES, int with_e0, void *stream) {
  using namespace imsrg;
  if (!b || !d_L || !d_R || !d_RES) return IMSRG_ERR_INVALID;
  if ((herm_L != 1 && herm_L != -1) || (herm_R != 1 && herm_R != -1)) return IMSRG_ERR_INVALID;
  if (overlaps(d_RES, d_L, b->nfull) || overlaps(d_RES, d_R, b->nfull)) return IMSRG_ERR_INVALID;
  long ne0p = round_up(imsrg::asm2_ctas(b));
  long need = 2 * round_up(b->nfull) + 2 * round_up(b->cc_total) + round_up(b->wcc_total) + round_up(b->T.n_ph) + ne0p;
  if (need > IMSRG_NOALLOC_SCRATCH_DOUBLES) return IMSRG_ERR_TOO_LARGE;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev != b->device) return IMSRG_ERR_INVALID;
  double *base = nullptr;
  int s = scratch_address(dev, &base);
  if (s != IMSRG_OK) return s;
  Workspace ws;
  ws.w1 = base;
  ws.w2 = ws.w1 + round_up(b->nfull);
  ws.lcc = ws.w2 + round_up(b->nfull);
  ws.rcc = ws.lcc + round_up(b->cc_total);
  ws.wcc = ws.rcc + round_up(b->cc_total);
  ws.zph = ws.wcc + round_up(b->wcc_total);
  ws.e0p = ws.zph + round_up(b->T.n_ph);
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  return launch_commutator_fp64_ws(b, ws, d_L, herm_L, d_R, herm_R, d_RES, -herm_L * herm_R, with_e0 ? 1 : 0, st);
}
