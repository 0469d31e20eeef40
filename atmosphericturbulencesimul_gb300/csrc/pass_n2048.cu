// Row-pass kernels for 2048 x 2048 grids.
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_2048(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<2048>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
