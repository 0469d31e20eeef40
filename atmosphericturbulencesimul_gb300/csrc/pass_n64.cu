// Row-pass kernels for 64 x 64 grids (every tile configuration).
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_64(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<64>(var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_cfg_64(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st)
{
    return launch_pass_nc<64>(cfg, var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_half_64(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                cudaStream_t st)
{
    return launch_pass_hn<64>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
