// engine.cuh -- device-side data structures of the wavefront-series engine.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdlib>
#include <utility>

#include "atmwfs.h"
#include "fft_core.cuh"

namespace atmwfs {

// Programmatic dependent launch.  The kernels of a step are launched with
// programmatic stream serialization, so the CTAs of a kernel can be
// scheduled while its predecessor's last CTAs still run.  Every such kernel
// opens with pdl_gate(): griddepcontrol.wait returns once all its
// predecessor grids have completed and their memory is visible, and
// launch_dependents then lets its own successors be scheduled.  The gate
// comes before any global read and before any early return, so ordering
// stays transitive along a chain.  Launched without the attribute, both
// instructions return at once.
#if defined(__CUDACC__)
__device__ __forceinline__ void pdl_gate()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
#endif

// Grids of at most this many CTAs get the attribute: one CTA per SM.
// Such launches are bound by launch latency, which the early scheduling
// hides (a 256^2 single-frame step: 29.1 -> 25.0 us).  Larger grids are
// bound by throughput.  There, early-scheduled CTAs that wait resident take
// SM slots from the step's concurrent branches: a 7-layer 512^2 step went
// 0.107 -> 0.149 ms with the attribute on every launch.  ATMWFS_PDL=0 turns
// the attribute off.
inline int pdl_max_ctas()
{
    static const int n = [] {
        const char* e = getenv("ATMWFS_PDL");
        if (e && atoi(e) == 0) return 0;
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return sms;
    }();
    return n;
}

// Non-zero while the autotuner times its candidates: it times each
// configuration's launches back to back, and overlapped launches there would
// not predict the configuration's time inside a step.
inline int& pdl_hold()
{
    static int h = 0;
    return h;
}

// Launch k<<<grid, block, sm, st>>>(args...), with programmatic stream
// serialization when the grid is small (above); k must open with
// pdl_gate().
template <typename... P, typename... A>
cudaError_t launch_gated(void (*k)(P...), dim3 grid, dim3 block, size_t sm, cudaStream_t st, A&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = sm;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_hold() == 0 && (long)grid.x * grid.y * grid.z <= pdl_max_ctas() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

constexpr int kMaxLayers = 16;
// Fractional bits of the fixed-point science bin sums.  A bin is under 40
// pixels wide (nb = Wout / 20 rounded down, Wout >= 20), so it sums fewer
// than 1,600 unit phasors per step: |sum| < 2^11 and sum * 2^50 < 2^61 stays
// inside a signed 64-bit integer.
constexpr int kBinFrac = 50;

// Integer and fractional sample position of one layer window for one
// instance at one step, in the screen's own (untransposed) frame:
// pixel (ii, jj) of the window samples the screen at (ix + fx + ii, iy + fy + jj).
struct LayerPos {
    int ix, iy;
    float fx, fy;
};

// One (wavelength, direction, output-mode) instance.
struct InstDev {
    float2* fld[2];            // ping-pong N x N fields
    const float2* H;           // hop transfer tables, [P][N], 1-D, include 1/N
    const void* Hh;            // the same as N H in FP16 (__half2), for FP16 transforms
    float scoeff[kMaxLayers];  // per-layer phase multiplier
    float* out_pha;            // this instance's frame in output slot 0; slot k at + k * ostride
    float* out_amp;
    long ostride;              // floats between output slots (the frames of all instances)
    float* phisum;             // geometric phase sum of the crop [Nout*Nout] (k_phasum)
    // science scratch: [2][nb*nb] (re, im) sums in fixed point, units of
    // 2^-kBinFrac (integer sums are order-free, so the totals do not depend
    // on the order in which CTAs add their parts)
    unsigned long long* bins;
    float* peak;               // science scratch: unwrapped bin phase [nb*nb]
    const short* binx;         // bin index of each output coordinate [Nout]
    const short* binx0;        // first output coordinate of each bin [nb + 1]
    int N, Nout, off, nb;
    int mode;                  // kModeRef / kModeSci / kModePhase
    int ring;                  // output frames kept on the device
    int gidx;                  // global instance index (positions, scratch)
    // Bicubic windows of the screens at this step, shared by every instance
    // whose layer positions are identical (a window group: the wavelengths
    // of one direction): win[orient][layer] is wstride x wstride floats
    // (wstride = the largest grid of the group), row-major in the pass
    // orientation; this instance reads its top-left N x N.  Unit-scale
    // samples: the pass multiplies by scoeff.
    const float* win[2][kMaxLayers];
    int wstride;
    // Geometric phase sum by factoring: when every member of the window
    // group has one Scoeff for all its layers, the group's compensated layer
    // sum sum_l window_l is formed once per step (k_group_sum; (hi, lo) pairs,
    // wstride x wstride, pass coordinates) and this instance's phase sum is
    // scoeff[0] * (hi + lo).  Null: the per-instance sum in phisum.
    const float2* gsum;
};

// One window group's layer sum (k_group_sum): its L windows in the screen
// orientation, side x side, and the (hi, lo) output.
struct GroupSumJob {
    float2* out;
    const float* win[kMaxLayers];
    int side;
};

// One window of the per-step window kernel: layer `layer` of group leader
// `gidx` in orientation `orient`, written to `out` with row stride `stride`.
struct WinJob {
    float* out;
    int gidx, layer, orient, stride;
};

enum : int { kModeRef = 0, kModeSci = 1, kModePhase = 2 };

// Operation flags of a row pass.
enum : int {
    OP_LOAD = 1,       // read the field (else start from 1 + 0i)
    OP_PROP1 = 2,      // 1-D Fresnel propagation along the rows (table hop1)
    OP_GATHER = 4,     // apply the phase screens of layers [g_lo, g_hi)
    OP_PROP2 = 8,      // 1-D Fresnel propagation along the rows (table hop2)
    OP_STORE_T = 16,   // store transposed
    OP_EPI = 32,       // output epilogue (crop, phase sum, amplitude, phase)
    OP_FFT_FWD = 64,   // unit: forward 1-D FFT only
    OP_FFT_INV = 128,  // unit: inverse 1-D FFT only
    OP_PHASUM = 256,   // geometric phase sum of all layers (k_phasum)
    OP_WINDOWS = 512,  // per-step bicubic windows of the window groups (k_layer_windows)
};

constexpr int kVarFirst = OP_GATHER | OP_PROP2 | OP_STORE_T;
constexpr int kVarMid = OP_LOAD | OP_PROP1 | OP_GATHER | OP_PROP2 | OP_STORE_T;
constexpr int kVarLast = OP_LOAD | OP_PROP1 | OP_GATHER | OP_EPI;
constexpr int kVarSingle = OP_GATHER | OP_EPI;
constexpr int kVarUnitProp = OP_LOAD | OP_PROP2 | OP_STORE_T;
constexpr int kVarUnitFwd = OP_LOAD | OP_FFT_FWD | OP_STORE_T;
constexpr int kVarUnitInv = OP_LOAD | OP_FFT_INV | OP_STORE_T;
constexpr int kVarPhasum = OP_PHASUM;
constexpr int kVarWindows = OP_WINDOWS;

// Status bits written by kernels.
enum : unsigned {
    kStatTmaTimeout = 1u,
    kStatBadArg = 2u,
    kStatUnwrapTimeout = 4u,
};

struct PassArgs {
    const InstDev* inst;       // instances of this launch (blockIdx.y), or null (unit path)
    const LayerPos* pos;       // [poscap][ninst_total][L]
    const int* d_step;         // current step (device counter), may be null
    unsigned* d_status;        // error bits
    int L, ninst_total, poscap;
    int g_lo, g_hi;            // layers gathered by OP_GATHER
    int hop1, hop2;            // transfer table index for PROP1 / PROP2
    int src, dst;              // field buffer index
    int orient;                // 0: rows are screen rows; 1: rows are screen columns
    int row0;                  // first row handled by blockIdx.x == 0
    // unit path (inst == null)
    const float2* ext_in;
    float2* ext_out;
    const float2* H1;
    const float2* H2;
    // window kernel: its jobs (blockIdx.y)
    const WinJob* jobs;
};

// Tensor maps of the halo-padded screens: [orientation][layer].
struct TmaSet {
    CUtensorMap m[2][kMaxLayers];
};

// Padded screen geometry: Pad[yp][xp] = S[(yp - kPadY) mod M][(xp - kPadX) mod M]
// (and the transposed copy with the roles of the axes exchanged).
constexpr int kPadX = 4;
constexpr int kPadY = 1;
constexpr int kBoxW = 32;  // TMA box width (floats)

// Host-side launch entry of one row pass for grid size N (defined per N).
typedef cudaError_t (*PassLauncher)(int var, dim3 grid, const PassArgs& a, const TmaSet* maps,
                                    const float2* tw, cudaStream_t st);
// Same, for tile configuration `cfg` (see tile_cfg).
typedef cudaError_t (*PassLauncherCfg)(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps,
                                       const float2* tw, cudaStream_t st);

// Pass configurations compiled per grid size: the radix plan (Plan / Stages
// variant), rows per CTA, the minimum number of resident CTAs per SM the
// kernel is register-limited to, whether the screen tile overlays the
// exchange rows, and whether the hop transfer tables are staged in shared
// memory.  Configurations 0-2 use the default plan with the tables read
// through L1: 0 is the one-CTA-per-SM shape; 1 trades rows per tile for
// several resident CTAs per SM; 2 also overlays the tile on the exchange
// buffer, which cuts shared memory so that one more CTA fits per SM.
// Configurations 3 and 4 run the size's alternative radix plan (where it has
// one; rr = 0 elsewhere) in two tile shapes; configuration 5 is 1 with the
// transfer tables copied into shared memory by cp.async at kernel start.
// The engine's autotuner times every compiled configuration of a grid class
// at set-up and keeps the fastest.
struct TileCfg {
    int rr, minb;
    bool alias;
    int plan;
    bool hsm;
};
constexpr int kNumTileCfg = ATMWFS_NUM_TILE_CFG;
constexpr TileCfg tile_cfg(int N, int c)
{
    return c == 3 ? (N == 1024 ? TileCfg{4, 3, false, 1, false} : TileCfg{0, 0, false, 0, false})
         : c == 4 ? (N == 1024 ? TileCfg{2, 6, false, 1, false} : TileCfg{0, 0, false, 0, false})
         : c == 5 ? (N == 1024 ? TileCfg{4, 3, false, 0, true} : N == 512 ? TileCfg{8, 3, false, 0, true}
                                                                          : TileCfg{0, 0, false, 0, false})
         : c > 5  ? TileCfg{0, 0, false, 0, false}
         : N == 64    ? (c == 0 ? TileCfg{32, 1, false, 0, false} : c == 1 ? TileCfg{16, 2, false, 0, false} : TileCfg{16, 3, true, 0, false})
         : N == 128   ? (c == 0 ? TileCfg{32, 1, false, 0, false} : c == 1 ? TileCfg{16, 2, false, 0, false} : TileCfg{16, 3, true, 0, false})
         : N == 256   ? (c == 0 ? TileCfg{16, 1, false, 0, false} : c == 1 ? TileCfg{8, 3, false, 0, false} : TileCfg{8, 4, true, 0, false})
         : N == 512   ? (c == 0 ? TileCfg{16, 1, false, 0, false} : c == 1 ? TileCfg{8, 3, false, 0, false} : TileCfg{8, 4, true, 0, false})
         : N == 1024  ? (c == 0 ? TileCfg{8, 1, false, 0, false} : c == 1 ? TileCfg{4, 3, false, 0, false} : TileCfg{4, 4, true, 0, false})
         : N == 2048  ? (c == 0 ? TileCfg{4, 1, false, 0, false} : c == 1 ? TileCfg{2, 3, false, 0, false} : TileCfg{2, 3, true, 0, false})
                      : TileCfg{0, 0, false, 0, false};
}

// Threads of a phase-sum CTA and CTAs per instance of its launch.
constexpr int kPhasumThreads = 256;
inline int phasum_blocks(int Nout)
{
    const long items = (long)Nout * Nout / ((Nout % 4) == 0 ? 4 : 1);
    const long n = (items + kPhasumThreads - 1) / kPhasumThreads;
    return (int)(n < 1024 ? n : 1024);
}

// Rows per CTA of configuration 0 (unit operators).
inline int rows_per_cta(int N) { return tile_cfg(N, 0).rr; }

PassLauncher pass_launcher(int N);
PassLauncherCfg pass_launcher_cfg(int N);
// FP16-transform series passes (tile configuration 2); tw = FP16 twiddles
typedef cudaError_t (*PassLauncherHalf)(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw,
                                        cudaStream_t st);
PassLauncherHalf pass_launcher_half(int N);

}  // namespace atmwfs
