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
}

namespace {

using namespace atmwfs;

constexpr long kMaxN = ATMWFS_NOALLOC_MAX_N;
constexpr long kMaxTw = 2 * kMaxN;  // stage twiddle tables of the largest grid
constexpr int kMaxDevices = 64;
constexpr double kPi = 3.14159265358979323846264338328;

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

// One thread per entry of the call's tables, evaluated in double like the
// host tables of the allocating path:
//   table[k] = exp(-i c f_k^2) / n, f_k the centred frequency of unshifted
//   index k, the angle reduced to [-pi, pi] in double before the cosine and
//   sine (Fresnel_propagate_wavefront, WFpropagate.c:68-152);
//   twiddles: for each order (o = 0, 1) and stage st >= 1 of the size's plan,
//   tab[r * ns + k] = exp(-2 pi i k r / (ns R)) at offset tw_offset(o, st).
template <int N>
__global__ void k_noalloc_tables(double coeff)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < N) {
        const long f = j < N / 2 ? j : j - N;
        double ang = -coeff * (double)(f * f);
        ang -= 2.0 * kPi * nearbyint(ang / (2.0 * kPi));
        g_table[j] = make_float2((float)(cos(ang) / N), (float)(sin(ang) / N));
        return;
    }
    const int i = j - N;
    if (i >= tw_total<N>()) return;
    for (int o = 0; o < 2; o++)
        for (int st = 1; st < Stages<N>::S; st++) {
            const int base = tw_offset<N>(o, st);
            const int R = stage_radix<N>(st, o), ns = stage_ns<N>(st, o);
            if (i < base || i >= base + R * ns) continue;
            const int r = (i - base) / ns, k = (i - base) % ns;
            const double a = -2.0 * kPi * (double)(k * r) / (double)(ns * R);
            g_twiddle[i] = make_float2((float)cos(a), (float)sin(a));
            return;
        }
}

template <int N>
cudaError_t launch_tables_n(double coeff, cudaStream_t cs)
{
    if (tw_total<N>() > kMaxTw) return cudaErrorInvalidValue;  // the static twiddle array is too small
    const int total = N + tw_total<N>();
    k_noalloc_tables<N><<<(total + 255) / 256, 256, 0, cs>>>(coeff);
    return cudaGetLastError();
}

cudaError_t launch_tables(long n, double coeff, cudaStream_t cs)
{
    switch (n) {
        case 64: return launch_tables_n<64>(coeff, cs);
        case 128: return launch_tables_n<128>(coeff, cs);
        case 256: return launch_tables_n<256>(coeff, cs);
        case 512: return launch_tables_n<512>(coeff, cs);
        default: return cudaErrorInvalidValue;
    }
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
    // transfer table and twiddles of this size, written into the static
    // arrays by a kernel on the caller's stream: nothing is copied from host
    // memory, so the call does not wait for the stream to drain
    const double coeff = kPi * z * lambda / (dx * (double)n) / (dx * (double)n);
    cudaError_t e = launch_tables(n, coeff, cs);
    if (e != cudaSuccess) return err(ATMWFS_ERR_CUDA, cudaGetErrorString(e));
    const PassLauncher fn = pass_launcher((int)n);
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.H1 = s->table;
    a.H2 = s->table;
    a.ext_in = (const float2*)in;
    a.ext_out = s->field;
    const dim3 grid((unsigned)(n / rows_per_cta((int)n)), 1);
    e = fn(kVarUnitProp, grid, a, nullptr, s->twiddle, cs);
    if (e == cudaSuccess) {
        a.ext_in = s->field;
        a.ext_out = (float2*)out;
        e = fn(kVarUnitProp, grid, a, nullptr, s->twiddle, cs);
    }
    if (e != cudaSuccess) return err(ATMWFS_ERR_CUDA, cudaGetErrorString(e));
    return ATMWFS_OK;
}
