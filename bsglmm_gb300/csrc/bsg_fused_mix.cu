// bsg_fused_mix.cu -- instantiations of the fused colour kernel for the
// t/logit links (two lanes per voxel, Philox variates): with X' Phi X in
// registers the kernel fits two 256-thread blocks per SM, and two lanes per
// voxel make the brain-sized grid about three full waves instead of 1.5.
#include "bsg_fused.cuh"

namespace bsg {
cudaError_t launch_fused_mix(int P, int threads, const DatasetDev *ds, ChainDev *ch,
                             const BlockMap *map, int nblocks, int colour,
                             cudaStream_t st, bool pdl) {
  if (nblocks <= 0) return cudaSuccess;
  const Supplied sup{};
  switch (P) {
    case 1: return launch_one<1, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 2: return launch_one<2, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 3: return launch_one<3, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 4: return launch_one<4, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 5: return launch_one<5, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 6: return launch_one<6, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 7: return launch_one<7, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 8: return launch_one<8, 2, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace bsg
