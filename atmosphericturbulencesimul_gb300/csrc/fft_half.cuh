// fft_half.cuh -- the Stockham stage loop of fft_core.cuh with the values,
// twiddles and exchange rows in FP16 (complex __half2, real part in .x).
// Forward transforms scale every stage by 1 / radix (an exact power of two)
// so that magnitudes stay near those of the input; the transfer table is
// then stored as N H (unit modulus) and the inverse runs unscaled, which
// gives the same propagation as the FP32 path.  Device code only.
#pragma once

#include <cuda_fp16.h>

#include "fft_core.cuh"

namespace atmwfs {

// Barrier of the threads that share one row's exchange buffer.  Thread
// tid works on row tid / T, so rows of T <= 32 threads lie inside one warp
// (a warp barrier suffices); rows of 64 threads use named barrier 1 + row.
// Callers keep a CTA barrier wherever another row's data aliases the buffer.
template <int T>
__device__ __forceinline__ void row_sync()
{
    static_assert(T <= 32 ? (32 % T == 0) : (T % 32 == 0 && T <= 64 * 4), "rows must tile warps");
    if constexpr (T <= 32) {
        __syncwarp();
    } else {
        const int id = 1 + (int)threadIdx.x / T;
        asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(T) : "memory");
    }
}

__device__ __forceinline__ __half2 hcmul(__half2 a, __half2 b) { return __hcmadd(a, b, __float2half2_rn(0.0f)); }

// d * exp(-2 pi i k / n) for a compile-time (after unrolling) k < n <= 32:
// every stage runs forward; an inverse transform is the conjugate of the
// forward transform of the conjugate.
__device__ __forceinline__ __half2 tw_fwd_h(__half2 d, int k, int n)
{
    if (k == 0) return d;
    const int j = k * (32 / n);
    if (j == 16) return __hneg2(d);
    if (j == 8) return __hmul2(__lowhigh2highlow(d), __floats2half2_rn(1.0f, -1.0f));   // (x, y) -> (y, -x)
    if (j == 24) return __hmul2(__lowhigh2highlow(d), __floats2half2_rn(-1.0f, 1.0f));  // (x, y) -> (-y, x)
    return hcmul(d, __floats2half2_rn(cos32(j), -sin32(j)));
}

__device__ __forceinline__ __half2 hconj(__half2 v) { return __hmul2(v, __floats2half2_rn(1.0f, -1.0f)); }

template <int R>
__device__ __forceinline__ void dft_fwd_h(__half2* v)
{
#pragma unroll
    for (int span = R / 2; span >= 1; span >>= 1) {
#pragma unroll
        for (int base = 0; base < R; base += 2 * span) {
#pragma unroll
            for (int k = 0; k < span; k++) {
                const __half2 a = v[base + k], b = v[base + k + span];
                v[base + k] = __hadd2(a, b);
                v[base + k + span] = tw_fwd_h(__hsub2(a, b), k, 2 * span);
            }
        }
    }
    __half2 t[R];
#pragma unroll
    for (int i = 0; i < R; i++) t[i] = v[i];
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = t[brev<R>(i)];
}

// One forward stage: stage twiddles, butterflies, and the 1 / R scaling of
// the forward transforms of a propagation.
template <int N, int T, int E, int R>
__device__ __forceinline__ void stage_h(__half2* v, int t, const __half2* __restrict__ tws, int ns, bool scale)
{
    if (ns > 1) {
#pragma unroll
        for (int w = 0; w < E / R; w++) {
            const int k = (t + T * w) & (ns - 1);
#pragma unroll
            for (int r = 1; r < R; r++) v[w * R + r] = hcmul(v[w * R + r], tws[r * ns + k]);
        }
    }
#pragma unroll
    for (int w = 0; w < E / R; w++) dft_fwd_h<R>(v + w * R);
    if (scale) {
        const __half2 s = __float2half2_rn(1.0f / R);
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = __hmul2(v[e], s);
    }
}

template <int N, int T, int E>
__device__ __forceinline__ void stage_compute_h(__half2* v, int t, const __half2* tw, int r, int ns, bool scale)
{
    if constexpr (has_radix<N>(32)) if (r == 32) { stage_h<N, T, E, 32>(v, t, tw, ns, scale); return; }
    if constexpr (has_radix<N>(16)) if (r == 16) { stage_h<N, T, E, 16>(v, t, tw, ns, scale); return; }
    if constexpr (has_radix<N>(8)) if (r == 8) { stage_h<N, T, E, 8>(v, t, tw, ns, scale); return; }
}

template <int N, int T, int E, int R>
__device__ __forceinline__ void store_h(const __half2* v, __half2* buf, int t, int ns)
{
#pragma unroll
    for (int w = 0; w < E / R; w++) {
        const int j = t + T * w;
        const int base = (j & ~(ns - 1)) * R + (j & (ns - 1));
#pragma unroll
        for (int q = 0; q < R; q++) buf[padi(base + q * ns)] = v[w * R + q];
    }
}

template <int N, int T, int E, int R>
__device__ __forceinline__ void load_h(__half2* v, const __half2* buf, int t)
{
#pragma unroll
    for (int w = 0; w < E / R; w++) {
        const int j = t + T * w;
#pragma unroll
        for (int r = 0; r < R; r++) v[w * R + r] = buf[padi(j + r * (N / R))];
    }
}

template <int N, int T, int E>
__device__ __forceinline__ void exchange_h(__half2* v, __half2* buf, int t, int rp, int nsp, int r)
{
    if constexpr (has_radix<N>(32)) if (rp == 32) store_h<N, T, E, 32>(v, buf, t, nsp);
    if constexpr (has_radix<N>(16)) if (rp == 16) store_h<N, T, E, 16>(v, buf, t, nsp);
    if constexpr (has_radix<N>(8)) if (rp == 8) store_h<N, T, E, 8>(v, buf, t, nsp);
    row_sync<T>();
    if constexpr (has_radix<N>(32)) if (r == 32) load_h<N, T, E, 32>(v, buf, t);
    if constexpr (has_radix<N>(16)) if (r == 16) load_h<N, T, E, 16>(v, buf, t);
    if constexpr (has_radix<N>(8)) if (r == 8) load_h<N, T, E, 8>(v, buf, t);
}

// Two-stage plans with compile-time radices, strides and exchange indices.
template <int N, int T, int E, int RA, int RB>
__device__ __forceinline__ void fft2_ct_h(__half2* v, __half2* xrow, int t, const __half2* __restrict__ tws1,
                                          bool scale)
{
    stage_h<N, T, E, RA>(v, t, nullptr, 1, scale);
    row_sync<T>();
    store_h<N, T, E, RA>(v, xrow, t, 1);
    row_sync<T>();
    load_h<N, T, E, RB>(v, xrow, t);
    stage_h<N, T, E, RB>(v, t, tws1, RA, scale);
}

// One transform of the row in FP16, all stages forward; `scale` applies
// 1 / radix per stage (the forward transform of a propagation).
template <int N, int T, int E>
__device__ __forceinline__ void fft_fwd_h(__half2* v, __half2* xrow, int t, const __half2* __restrict__ tw, int rev,
                                          bool scale)
{
    if constexpr (Stages<N>::S == 2) {
        constexpr int R0 = Stages<N>::R0, R1 = Stages<N>::R1;
        if constexpr (R0 == R1) {
            fft2_ct_h<N, T, E, R0, R1>(v, xrow, t, tw + tw_offset<N>(rev, 1), scale);
        } else {
            if (rev) fft2_ct_h<N, T, E, R1, R0>(v, xrow, t, tw + tw_offset<N>(1, 1), scale);
            else fft2_ct_h<N, T, E, R0, R1>(v, xrow, t, tw + tw_offset<N>(0, 1), scale);
        }
        return;
    }
    int ns = 1, rp = 0, nsp = 1;
#pragma unroll 1
    for (int st = 0; st < Stages<N>::S; st++) {
        const int r = stage_radix<N>(st, rev);
        if (st > 0) {
            row_sync<T>();
            exchange_h<N, T, E>(v, xrow, t, rp, nsp, r);
        }
        stage_compute_h<N, T, E>(v, t, tw + tw_offset<N>(rev, st), r, ns, scale);
        rp = r;
        nsp = ns;
        ns *= r;
    }
}

// 1-D Fresnel propagation of the row with FP16 transforms: the FP32 values
// are rounded once on entry and widened once on exit; h is N H in FP16.
// IFFT(H FFT(x)) = conj(FFT(conj(H FFT(x)))), the inner conjugation folded
// into the transfer multiply, the outer one into the widening.
template <int N, int T, int E>
__device__ __forceinline__ void prop_row_h(float2* v, float2* xrow, int t, const __half2* __restrict__ tw,
                                           const __half2* __restrict__ h)
{
    constexpr int RL = last_radix<N>();
    __half2 u[E];
#pragma unroll
    for (int e = 0; e < E; e++) u[e] = __floats2half2_rn(v[e].x, v[e].y);
    __half2* xr = reinterpret_cast<__half2*>(xrow);
    fft_fwd_h<N, T, E>(u, xr, t, tw, 0, true);
#pragma unroll
    for (int s = 0; s < E; s++) u[s] = hconj(hcmul(u[s], h[last_index<N, T, RL>(t, s)]));
    fft_fwd_h<N, T, E>(u, xr, t, tw, 1, false);
#pragma unroll
    for (int e = 0; e < E; e++) {
        const float2 f = __half22float2(u[e]);
        v[e] = make_float2(f.x, -f.y);
    }
}

}  // namespace atmwfs
