// Row-pass kernels for 512 x 512 grids.
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_512(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<512>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
