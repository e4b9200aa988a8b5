// ozaki.cu -- split-precision contraction engine (placeholder until the
// tcgen05 path lands: the precision mode reports itself as unavailable).
#include "internal.h"

namespace imsrg {

int ozaki_gemm(imsrg_basis *b, const double *L, int hL, const double *R, int hR) {
  (void)b; (void)L; (void)hL; (void)R; (void)hR;
  return IMSRG_ERR_INVALID;
}

void ozaki_free(imsrg_basis *b) { (void)b; }

}  // namespace imsrg
