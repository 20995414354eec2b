// bsg_fused_wide.cu -- instantiations of the probit colour kernel with the
// 16-subject whole-word step (four Philox calls per step, two resident
// blocks of 128 registers), one lane per voxel, Philox variates; with and
// without the beta_WM update.
#include "bsg_fused.cuh"

namespace bsg {
template <bool WMU>
static cudaError_t launch_wide(int P, int threads, const DatasetDev *ds, ChainDev *ch,
                               const BlockMap *map, int nblocks, int colour, cudaStream_t st,
                               bool pdl) {
  const Supplied sup{};
#define BSG_WIDE(PP)                                                                      \
  case PP:                                                                                \
    return launch_one<PP, 1, false, false, WMU, false, true>(nblocks, threads, st, pdl, ds, \
                                                              ch, map, colour, sup);
  switch (P) {
    BSG_WIDE(1)
    BSG_WIDE(2)
    BSG_WIDE(3)
    BSG_WIDE(4)
    BSG_WIDE(5)
    BSG_WIDE(6)
    BSG_WIDE(7)
    BSG_WIDE(8)
    default:
      return cudaErrorInvalidValue;
  }
#undef BSG_WIDE
}

cudaError_t launch_fused_wide(int P, int threads, bool wmu, const DatasetDev *ds,
                              ChainDev *ch, const BlockMap *map, int nblocks, int colour,
                              cudaStream_t st, bool pdl) {
  if (nblocks <= 0) return cudaSuccess;
  return wmu ? launch_wide<true>(P, threads, ds, ch, map, nblocks, colour, st, pdl)
             : launch_wide<false>(P, threads, ds, ch, map, nblocks, colour, st, pdl);
}
}  // namespace bsg
