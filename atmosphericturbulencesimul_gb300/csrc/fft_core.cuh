// fft_core.cuh -- in-CTA Stockham FFT building blocks for the wavefront-series
// engine.  One transform of length N is spread over T threads that each hold
// E = N/T complex values in registers; each stage performs E/R radix-R
// butterflies per thread and stages exchange through shared memory.
//
// Every function here is __host__ __device__ so that the index arithmetic can
// be exercised by a thread-by-thread CPU emulation (tests/emul/).
//
// Conventions (those of FFTW, which the reference calls through FFT_do2dfft,
// src/fft/fft.c:1145-1296): unnormalised, X[k] = sum_n x[n] exp(D 2 pi i nk/N),
// D = -1 forward, D = +1 inverse.
#pragma once

#if defined(__CUDACC__)
#define AW_HD __host__ __device__ __forceinline__
#define AW_UNROLL _Pragma("unroll")
#else
// host-only build (CPU emulation): vector types come from the CUDA headers
#include <cuda_runtime.h>
#include <cmath>
#define AW_HD inline
#define AW_UNROLL
#endif

namespace atmwfs {

AW_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
AW_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
AW_HD float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
AW_HD float2 cmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }

// cos(2 pi j / 32) for j in [0, 8]
AW_HD constexpr float cos32_oct(int j)
{
    return j == 0 ? 1.0f
         : j == 1 ? 0.980785280403230449f
         : j == 2 ? 0.923879532511286756f
         : j == 3 ? 0.831469612302545237f
         : j == 4 ? 0.707106781186547524f
         : j == 5 ? 0.555570233019602225f
         : j == 6 ? 0.382683432365089772f
         : j == 7 ? 0.195090322016128268f
         : 0.0f;
}
AW_HD constexpr float cos32(int j)
{
    return (j & 31) <= 8 ? cos32_oct(j & 31)
         : (j & 31) <= 16 ? -cos32_oct(16 - (j & 31))
         : (j & 31) <= 24 ? -cos32_oct((j & 31) - 16)
         : cos32_oct(32 - (j & 31));
}
AW_HD constexpr float sin32(int j) { return cos32((j + 24) & 31); }

// d * exp(D 2 pi i k / n) for a compile-time (after unrolling) k < n <= 32
template <int D>
AW_HD float2 tw_const(float2 d, int k, int n)
{
    if (k == 0) return d;
    const int j = k * (32 / n);
    if (j == 8) return D < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
    if (j == 16) return make_float2(-d.x, -d.y);
    if (j == 24) return D < 0 ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
    const float c = cos32(j);
    const float s = D < 0 ? -sin32(j) : sin32(j);
    return make_float2(d.x * c - d.y * s, d.x * s + d.y * c);
}

template <int R>
AW_HD constexpr int brev(int i)
{
    int r = 0;
    for (int b = 1, o = R >> 1; b < R; b <<= 1, o >>= 1)
        if (i & b) r |= o;
    return r;
}

// In-register radix-R DFT, natural order in and out (radix-2 decimation in
// frequency followed by a compile-time bit-reversal relabelling).
template <int R, int D>
AW_HD void dft(float2* v)
{
    AW_UNROLL
    for (int span = R / 2; span >= 1; span >>= 1) {
        AW_UNROLL
        for (int base = 0; base < R; base += 2 * span) {
            AW_UNROLL
            for (int k = 0; k < span; k++) {
                const float2 a = v[base + k], b = v[base + k + span];
                v[base + k] = cadd(a, b);
                v[base + k + span] = tw_const<D>(csub(a, b), k, 2 * span);
            }
        }
    }
    float2 t[R];
    AW_UNROLL
    for (int i = 0; i < R; i++) t[i] = v[i];
    AW_UNROLL
    for (int i = 0; i < R; i++) v[i] = t[brev<R>(i)];
}

// Padded shared-memory index: one spare slot every 32 complex values keeps
// the stride-R scatters of early stages free of bank conflicts.
AW_HD constexpr int padi(int i) { return i + (i >> 5); }

// Row stride (complex values) of one transform in the exchange buffer:
// the smallest value >= padi(N) that is congruent to 2 modulo 16, so that the
// rows of a tile fall on distinct banks in the transposing read.
template <int N>
AW_HD constexpr int row_stride() { return padi(N) + ((2 - (padi(N) & 15)) + 16) % 16; }

// ---------------------------------------------------------------------------
// Stockham stage primitives.  Thread t of a transform owns the work items
// j_w = t + T w, w in [0, E/R).  Register slot v[w R + r].
//   load   : v[w R + r] = buf[j_w + r N/R]
//   twiddle: v[w R + r] *= W_N^(D (j_w mod Ns) r N/(Ns R))      (table tw[k] = exp(-2 pi i k/N))
//   dft    : radix-R DFT of each work item
//   store  : buf[(j_w / Ns) Ns R + (j_w mod Ns) + q Ns] = v[w R + q]
// After the last stage (Ns R = N) thread t holds X[j_w + q N/R].
// ---------------------------------------------------------------------------
template <int N, int T, int E, int R>
AW_HD void stage_load(float2* v, const float2* buf, int t)
{
    AW_UNROLL
    for (int w = 0; w < E / R; w++) {
        const int j = t + T * w;
        AW_UNROLL
        for (int r = 0; r < R; r++) v[w * R + r] = buf[padi(j + r * (N / R))];
    }
}

template <int N, int T, int E, int R, int NS, int D>
AW_HD void stage_twiddle(float2* v, int t, const float2* tw)
{
    if (NS == 1) return;
    AW_UNROLL
    for (int w = 0; w < E / R; w++) {
        const int k = (t + T * w) % NS;
        AW_UNROLL
        for (int r = 1; r < R; r++) {
            const float2 w0 = tw[k * r * (N / (NS * R))];
            v[w * R + r] = D < 0 ? cmul(v[w * R + r], w0) : cmulc(v[w * R + r], w0);
        }
    }
}

template <int E, int R, int D>
AW_HD void stage_dft(float2* v)
{
    AW_UNROLL
    for (int w = 0; w < E / R; w++) dft<R, D>(v + w * R);
}

template <int N, int T, int E, int R, int NS>
AW_HD void stage_store(const float2* v, float2* buf, int t)
{
    AW_UNROLL
    for (int w = 0; w < E / R; w++) {
        const int j = t + T * w;
        const int base = (j / NS) * NS * R + (j % NS);
        AW_UNROLL
        for (int q = 0; q < R; q++) buf[padi(base + q * NS)] = v[w * R + q];
    }
}

// Frequency (or output) index held in register slot s after the last stage
// of radix RL: k = j_w + q N/RL with w = s / RL, q = s % RL.
template <int N, int T, int RL>
AW_HD int last_index(int t, int s) { return t + T * (s / RL) + (s % RL) * (N / RL); }

// Radix plans.  Forward radices start with E (one work item per thread, so
// the coalesced global load x[t + e T] is already the first stage's layout);
// the inverse uses the reversed sequence so that it can start from the
// forward's output registers and ends in the same layout x[t + e T].
template <int N> struct Plan;
template <> struct Plan<64>   { static constexpr int E = 8,  T = 8;  };
template <> struct Plan<128>  { static constexpr int E = 16, T = 8;  };
template <> struct Plan<256>  { static constexpr int E = 16, T = 16; };
template <> struct Plan<512>  { static constexpr int E = 32, T = 16; };
template <> struct Plan<1024> { static constexpr int E = 32, T = 32; };
template <> struct Plan<2048> { static constexpr int E = 32, T = 64; };

template <int... Rs> struct Radices {};

template <int N> struct FwdRadices;
template <> struct FwdRadices<64>   { using type = Radices<8, 8>; };
template <> struct FwdRadices<128>  { using type = Radices<16, 8>; };
template <> struct FwdRadices<256>  { using type = Radices<16, 16>; };
template <> struct FwdRadices<512>  { using type = Radices<32, 16>; };
template <> struct FwdRadices<1024> { using type = Radices<32, 32>; };
template <> struct FwdRadices<2048> { using type = Radices<32, 8, 8>; };

template <int N> struct InvRadices;
template <> struct InvRadices<64>   { using type = Radices<8, 8>; };
template <> struct InvRadices<128>  { using type = Radices<8, 16>; };
template <> struct InvRadices<256>  { using type = Radices<16, 16>; };
template <> struct InvRadices<512>  { using type = Radices<16, 32>; };
template <> struct InvRadices<1024> { using type = Radices<32, 32>; };
template <> struct InvRadices<2048> { using type = Radices<8, 8, 32>; };

template <int R0, int... Rs> struct LastRadix { static constexpr int value = LastRadix<Rs...>::value; };
template <int R0> struct LastRadix<R0> { static constexpr int value = R0; };
template <int R0, int... Rs> struct FirstRadix { static constexpr int value = R0; };

}  // namespace atmwfs
