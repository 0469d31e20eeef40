// Row-pass kernels for 128 x 128 grids (every tile configuration).
#include "pass_impl.cuh"

namespace atmwfs {
cudaError_t launch_pass_128(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    return launch_pass_n<128>(var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_cfg_128(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st)
{
    return launch_pass_nc<128>(cfg, var, grid, a, maps, tw, st);
}

cudaError_t launch_pass_half_128(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                cudaStream_t st)
{
    return launch_pass_hn<128>(var, grid, a, maps, tw, st);
}
}  // namespace atmwfs
