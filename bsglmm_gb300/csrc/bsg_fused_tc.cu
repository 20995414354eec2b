// bsg_fused_tc.cu -- instantiations of the probit colour kernel with the
// X'Z contraction on the tensor cores (BF16x3 split, bsg_mma.cuh), one lane
// per voxel, Philox variates.
#include "bsg_fused.cuh"

namespace bsg {
cudaError_t launch_fused_tc(int P, int threads, const DatasetDev *ds, ChainDev *ch,
                            const BlockMap *map, int nblocks, int colour, cudaStream_t st,
                            bool pdl) {
  if (nblocks <= 0) return cudaSuccess;
  const Supplied sup{};
  switch (P) {
    case 1: return launch_one<1, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 2: return launch_one<2, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 3: return launch_one<3, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 4: return launch_one<4, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 5: return launch_one<5, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 6: return launch_one<6, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 7: return launch_one<7, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    case 8: return launch_one<8, 1, false, false, false, true>(nblocks, threads, st, pdl, ds, ch, map, colour, sup);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace bsg
