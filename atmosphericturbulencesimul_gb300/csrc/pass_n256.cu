// Row-pass kernels for 256 x 256 grids (every tile configuration).
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_256(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<256>(var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_cfg_256(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st)
{
    return launch_pass_nc<256>(cfg, var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_half_256(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                cudaStream_t st)
{
    return launch_pass_hn<256>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
