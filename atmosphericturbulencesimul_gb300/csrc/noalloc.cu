// noalloc.cu -- a Fresnel hop that allocates nothing.
//
// atmwfs_fresnel_dev() takes a temporary n x n field and a transfer table
// from the stream-ordered allocator on every call.  Some callers cannot do
// that: a real-time loop that feeds frames to an adaptive-optics controller
// must not call the CUDA allocator once it runs (an allocation or free can
// wait on the whole device and its duration is unbounded), and a host that
// hands all device memory to its own pool at start-up has nothing left to
// allocate from.  atmwfs_fresnel_noalloc() serves them from scratch arrays
// that live in this file for as long as the library is loaded.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "atmwfs.h"
#include "aux_kernels.cuh"

namespace atmwfs {
void set_error_message(const char* msg);
int twiddle_count(int N);
void twiddle_fill(int N, float2* out);
}

namespace {

using namespace atmwfs;

constexpr long kMaxN = ATMWFS_NOALLOC_MAX_N;
constexpr long kMaxTw = 2 * kMaxN;  // stage twiddle tables of the largest grid
constexpr int kMaxDevices = 64;
const double kPi = 3.14159265358979323846264338328;

// Scratch shared by every call on a device: the field after the first
// (transposed) pass, the 1-D transfer table and the twiddles of the call's
// size.  2 MiB + 12 KiB per device that loads the library, held until exit.
__device__ __align__(256) float2 g_field[kMaxN * kMaxN];
__device__ __align__(256) float2 g_table[kMaxN];
__device__ __align__(256) float2 g_twiddle[kMaxTw];

// Device addresses of the scratch arrays.  In host code the array names are
// host-side stand-ins, so the addresses are looked up once per device.
struct Scratch {
    float2* field = nullptr;
    float2* table = nullptr;
    float2* twiddle = nullptr;
    bool ready = false;
};
Scratch g_scratch[kMaxDevices];
std::mutex g_mu;

atmwfs_status err(atmwfs_status s, const char* msg)
{
    set_error_message(msg);
    return s;
}

atmwfs_status scratch_for_current_device(Scratch** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return err(ATMWFS_ERR_NODEVICE, "no current CUDA device");
    if (dev < 0 || dev >= kMaxDevices) return err(ATMWFS_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    Scratch& s = g_scratch[dev];
    if (!s.ready) {
        if (cudaGetSymbolAddress((void**)&s.field, g_field) != cudaSuccess ||
            cudaGetSymbolAddress((void**)&s.table, g_table) != cudaSuccess ||
            cudaGetSymbolAddress((void**)&s.twiddle, g_twiddle) != cudaSuccess)
            return err(ATMWFS_ERR_CUDA, "cudaGetSymbolAddress failed for the no-alloc scratch");
        s.ready = true;
    }
    *out = &s;
    return ATMWFS_OK;
}

}  // namespace

extern "C" atmwfs_status atmwfs_fresnel_noalloc(const void* in, void* out, long n, double dx, double z, double lambda,
                                                void* stream)
{
    if (!in || !out) return err(ATMWFS_ERR_INVALID, "null buffer");
    if (n < 64 || n > kMaxN || (n & (n - 1)) != 0) {
        char m[160];
        snprintf(m, sizeof m, "atmwfs_fresnel_noalloc: size %ld unsupported (power of two, 64..%ld: the static scratch holds %ld x %ld)",
                 n, kMaxN, kMaxN, kMaxN);
        return err(ATMWFS_ERR_INVALID, m);
    }
    Scratch* s = nullptr;
    atmwfs_status st = scratch_for_current_device(&s);
    if (st != ATMWFS_OK) return st;
    cudaStream_t cs = (cudaStream_t)stream;
    // transfer table and twiddles of this size, built on the stack (the same
    // formulas as the allocating path) and copied into the static arrays
    float2 h[kMaxN], tw[kMaxTw];
    const double coeff = kPi * z * lambda / (dx * (double)n) / (dx * (double)n);
    for (long k = 0; k < n; k++) {
        const long f = k < n / 2 ? k : k - n;
        double ang = -coeff * (double)(f * f);
        ang -= 2.0 * kPi * nearbyint(ang / (2.0 * kPi));
        h[k] = make_float2((float)(cos(ang) / n), (float)(sin(ang) / n));
    }
    const int ntw = twiddle_count((int)n);
    if (ntw > kMaxTw) return err(ATMWFS_ERR_INVALID, "twiddle tables exceed the static scratch");
    twiddle_fill((int)n, tw);
    // pageable sources: each copy is staged before the call returns
    if (cudaMemcpyAsync(s->table, h, sizeof(float2) * n, cudaMemcpyHostToDevice, cs) != cudaSuccess ||
        cudaMemcpyAsync(s->twiddle, tw, sizeof(float2) * ntw, cudaMemcpyHostToDevice, cs) != cudaSuccess)
        return err(ATMWFS_ERR_CUDA, "copy of the transfer table failed");
    const PassLauncher fn = pass_launcher((int)n);
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.H1 = s->table;
    a.H2 = s->table;
    a.ext_in = (const float2*)in;
    a.ext_out = s->field;
    const dim3 grid((unsigned)(n / rows_per_cta((int)n)), 1);
    cudaError_t e = fn(kVarUnitProp, grid, a, nullptr, s->twiddle, cs);
    if (e == cudaSuccess) {
        a.ext_in = s->field;
        a.ext_out = (float2*)out;
        e = fn(kVarUnitProp, grid, a, nullptr, s->twiddle, cs);
    }
    if (e != cudaSuccess) return err(ATMWFS_ERR_CUDA, cudaGetErrorString(e));
    return ATMWFS_OK;
}
