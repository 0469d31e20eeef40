// Row-pass kernels for 1024 x 1024 grids (every tile configuration).
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_1024(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<1024>(var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_cfg_1024(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st)
{
    return launch_pass_nc<1024>(cfg, var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_half_1024(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                cudaStream_t st)
{
    return launch_pass_hn<1024>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
