// Row-pass kernels for 512 x 512 grids (every tile configuration).
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_512(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<512>(var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_cfg_512(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st)
{
    return launch_pass_nc<512>(cfg, var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_half_512(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                cudaStream_t st)
{
    return launch_pass_hn<512>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
