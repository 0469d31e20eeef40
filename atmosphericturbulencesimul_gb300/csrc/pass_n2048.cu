// Row-pass kernels for 2048 x 2048 grids (every tile configuration).
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_2048(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<2048>(var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_cfg_2048(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st)
{
    return launch_pass_nc<2048>(cfg, var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_half_2048(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                cudaStream_t st)
{
    return launch_pass_hn<2048>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
