// bsg_fused_tc.cu -- instantiations of the probit colour kernel with the
// X'Z contraction on the tensor cores (BF16x3 split, bsg_mma.cuh), one lane
// per voxel, Philox variates.
#include "bsg_fused.cuh"

namespace bsg {
// The kernels' dynamic shared memory opt-in (the chunk's BF16 design slices
// and the warps' Z tiles exceed the default 48 KB with the static staging).
// Called on the host before any launch, outside stream capture.
cudaError_t prepare_fused_tc() {
  const cudaError_t e[8] = {prepare_tc<1>(), prepare_tc<2>(), prepare_tc<3>(), prepare_tc<4>(),
                            prepare_tc<5>(), prepare_tc<6>(), prepare_tc<7>(), prepare_tc<8>()};
  for (cudaError_t x : e)
    if (x != cudaSuccess) return x;
  return cudaSuccess;
}

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
