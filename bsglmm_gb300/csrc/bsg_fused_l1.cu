// bsg_fused_l1.cu -- instantiations of the fused colour kernel with 1
// lane(s) per voxel (one translation unit per tile width, built in
// parallel).
#include "bsg_fused.cuh"

namespace bsg {
cudaError_t launch_fused_l1(int P, int threads, bool supplied,
                            const DatasetDev *ds, ChainDev *ch,
                            const BlockMap *map, int nblocks, int colour,
                            const Supplied &sup, cudaStream_t st, bool pdl) {
  return launch_fused_lpv<1>(P, threads, supplied, ds, ch, map, nblocks,
                              colour, sup, st, pdl);
}
}  // namespace bsg
