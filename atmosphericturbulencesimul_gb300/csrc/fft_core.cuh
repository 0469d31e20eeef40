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

// Complex add / subtract.  On sm_100 and later the (re, im) pair is one
// packed FP32x2 operation (per component the same IEEE rounding as the
// scalar form; a - b as the exact b * (-1) + a).  A translation unit whose
// kernels run faster with scalar butterflies defines AW_SCALAR_BUTTERFLY
// before including this header (the results are the same either way).
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && !defined(AW_SCALAR_BUTTERFLY)
#define AW_PACKED_BUTTERFLY 1
#endif
AW_HD float2 cadd(float2 a, float2 b)
{
#if defined(AW_PACKED_BUTTERFLY)
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
AW_HD float2 csub(float2 a, float2 b)
{
#if defined(AW_PACKED_BUTTERFLY)
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
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

// In-register radix-R DFT, natural order in and out: decimation in frequency
// taking the radix-2 levels two at a time (radix 2^2), then a last radix-2
// level when log2 R is odd, followed by a compile-time bit-reversal
// relabelling.  A pair of levels with span s works on x0..x3 = v[k + {0, s,
// 2s, 3s}] of each block of 4s:
//   c0 = x0 + x2, c1 = x1 + x3, c2 = (x0 - x2) + W4 (x1 - x3), c3 = (x0 - x2) - W4 (x1 - x3)
//   v[k] = c0 + c1,  v[k + s] = (c0 - c1) W^2k,  v[k + 2s] = c2 W^k,  v[k + 3s] = c3 W^3k
// with W = exp(D 2 pi i / 4s) and W4 = W^s = D i (a register swap): the same
// values, at the same places, as the two radix-2 levels (whose second level
// multiplies by W^k and W^(k + s) = W4 W^k), with three twiddle multiplies per
// group of four instead of four.
// Translation units built with scalar butterflies (AW_SCALAR_BUTTERFLY: the
// whole-row transforms of the large screens) keep the plain radix-2 levels,
// which measured faster there (8192^2: 0.98 against 1.10 ms).
template <int R, int D>
AW_HD void dft_radix2(float2* v)
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

template <int R, int D>
AW_HD void dft(float2* v)
{
#if defined(AW_SCALAR_BUTTERFLY)
    dft_radix2<R, D>(v);
    return;
#endif
    constexpr int L2 = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : R == 16 ? 4 : R == 32 ? 5 : 6;
    int span = R / 4;
    AW_UNROLL
    for (int lv = 0; lv + 1 < L2; lv += 2, span /= 4) {
        AW_UNROLL
        for (int base = 0; base < R; base += 4 * span) {
            AW_UNROLL
            for (int k = 0; k < span; k++) {
                const float2 x0 = v[base + k], x1 = v[base + k + span];
                const float2 x2 = v[base + k + 2 * span], x3 = v[base + k + 3 * span];
                const float2 c0 = cadd(x0, x2), c1 = cadd(x1, x3);
                const float2 d0 = csub(x0, x2), d1 = tw_const<D>(csub(x1, x3), 1, 4);
                v[base + k] = cadd(c0, c1);
                v[base + k + span] = tw_const<D>(csub(c0, c1), 2 * k, 4 * span);
                v[base + k + 2 * span] = tw_const<D>(cadd(d0, d1), k, 4 * span);
                v[base + k + 3 * span] = tw_const<D>(csub(d0, d1), 3 * k, 4 * span);
            }
        }
    }
    if constexpr ((L2 & 1) != 0) {
        // the last radix-2 level (span 1: no twiddles)
        AW_UNROLL
        for (int base = 0; base < R; base += 2) {
            const float2 a = v[base], b = v[base + 1];
            v[base] = cadd(a, b);
            v[base + 1] = csub(a, b);
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

// The same with the stride NS known at run time (ns is a power of two): the
// stage loop below runs every stage of every transform through one copy of
// the code of each radix.  The stages are always forward (compile-time
// butterfly constants, the +-i rotations free); an inverse transform is the
// conjugate of the forward transform of the conjugate.
// tws: the stage's twiddle table tws[r * ns + k] = exp(-2 pi i k r / (ns R))
// (see tw_offset), read with consecutive k across a warp.
template <int N, int T, int E, int R>
AW_HD void stage_twiddle_rt(float2* v, int t, const float2* tws, int ns)
{
    if (ns == 1) return;
    AW_UNROLL
    for (int w = 0; w < E / R; w++) {
        const int k = (t + T * w) & (ns - 1);
        AW_UNROLL
        for (int r = 1; r < R; r++) v[w * R + r] = cmul(v[w * R + r], tws[r * ns + k]);
    }
}

template <int E, int R>
AW_HD void stage_dft_rt(float2* v)
{
    AW_UNROLL
    for (int w = 0; w < E / R; w++) dft<R, -1>(v + w * R);
}

template <int E>
AW_HD void conj_all(float2* v)
{
    AW_UNROLL
    for (int e = 0; e < E; e++) v[e].y = -v[e].y;
}

template <int N, int T, int E, int R>
AW_HD void stage_store_rt(const float2* v, float2* buf, int t, int ns)
{
    AW_UNROLL
    for (int w = 0; w < E / R; w++) {
        const int j = t + T * w;
        const int base = (j & ~(ns - 1)) * R + (j & (ns - 1));
        AW_UNROLL
        for (int q = 0; q < R; q++) buf[padi(base + q * ns)] = v[w * R + q];
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
//
// A grid size can have more than one plan (V = 0 is the default; the engine's
// autotuner times the others as further configurations): V = 1 at 1024 is
// 16 x 8 x 8 with 16 values per thread and two warps per row -- one more
// exchange per transform than 32 x 32, but half the registers, so more
// warps per SM to hide the exchange and load latencies.
template <int N, int V = 0> struct Plan;
template <> struct Plan<64>   { static constexpr int E = 8,  T = 8;  };
template <> struct Plan<128>  { static constexpr int E = 16, T = 8;  };
template <> struct Plan<256>  { static constexpr int E = 16, T = 16; };
template <> struct Plan<512>  { static constexpr int E = 32, T = 16; };
template <> struct Plan<1024> { static constexpr int E = 32, T = 32; };
template <> struct Plan<2048> { static constexpr int E = 32, T = 64; };
template <> struct Plan<4096> { static constexpr int E = 16, T = 256; };
template <> struct Plan<8192> { static constexpr int E = 32, T = 256; };
template <> struct Plan<1024, 1> { static constexpr int E = 16, T = 64; };

// Radix sequence of the forward transform as a runtime-indexable table; the
// inverse of a propagation walks it backwards.
template <int N, int V = 0> struct Stages;
template <> struct Stages<64>   { static constexpr int S = 2, R0 = 8, R1 = 8, R2 = 0; };
template <> struct Stages<128>  { static constexpr int S = 2, R0 = 16, R1 = 8, R2 = 0; };
template <> struct Stages<256>  { static constexpr int S = 2, R0 = 16, R1 = 16, R2 = 0; };
template <> struct Stages<512>  { static constexpr int S = 2, R0 = 32, R1 = 16, R2 = 0; };
template <> struct Stages<1024> { static constexpr int S = 2, R0 = 32, R1 = 32, R2 = 0; };
template <> struct Stages<2048> { static constexpr int S = 3, R0 = 32, R1 = 8, R2 = 8; };
// whole-row plans of the large 2-D transforms (one CTA of 256 threads per row)
template <> struct Stages<4096> { static constexpr int S = 3, R0 = 16, R1 = 16, R2 = 16; };
template <> struct Stages<8192> { static constexpr int S = 3, R0 = 32, R1 = 16, R2 = 16; };
// alternative plans (see Plan)
template <> struct Stages<1024, 1> { static constexpr int S = 3, R0 = 16, R1 = 8, R2 = 8; };

template <int N, int V = 0>
AW_HD constexpr bool has_radix(int r)
{
    return Stages<N, V>::R0 == r || Stages<N, V>::R1 == r || Stages<N, V>::R2 == r;
}

// last radix of the forward sequence
template <int N, int V = 0>
AW_HD constexpr int last_radix() { return Stages<N, V>::S == 3 ? Stages<N, V>::R2 : Stages<N, V>::R1; }

// radix of stage st, forward order (rev = 0) or reversed (rev = 1)
template <int N, int V = 0>
AW_HD int stage_radix(int st, int rev)
{
    const int i = rev ? Stages<N, V>::S - 1 - st : st;
    return i == 0 ? Stages<N, V>::R0 : i == 1 ? Stages<N, V>::R1 : Stages<N, V>::R2;
}

// Stride (product of the earlier radices) of stage st in the given order.
template <int N, int V = 0>
AW_HD int stage_ns(int st, int rev)
{
    int ns = 1;
    for (int i = 0; i < st; i++) ns *= stage_radix<N, V>(i, rev);
    return ns;
}

// Twiddle tables: for each order (rev = 0, 1) and stage st >= 1 a table of
// R x ns entries tab[r * ns + k] = exp(-2 pi i k r / (ns R)); this gives the
// offset of table (rev, st) in the concatenation and the total size.
template <int N, int V = 0>
AW_HD int tw_offset(int rev, int st)
{
    int off = 0;
    for (int o = 0; o <= rev; o++)
        for (int i = 1; i < Stages<N, V>::S; i++) {
            if (o == rev && i == st) return off;
            off += stage_radix<N, V>(i, o) * stage_ns<N, V>(i, o);
        }
    return off;
}
template <int N, int V = 0>
AW_HD int tw_total() { return tw_offset<N, V>(1, Stages<N, V>::S); }

// Fill the concatenated stage tables (host side, double precision).
template <int N, int V = 0>
inline void build_twiddles(float2* out)
{
    for (int o = 0; o < 2; o++)
        for (int st = 1; st < Stages<N, V>::S; st++) {
            const int R = stage_radix<N, V>(st, o), ns = stage_ns<N, V>(st, o);
            float2* tab = out + tw_offset<N, V>(o, st);
            for (int r = 0; r < R; r++)
                for (int k = 0; k < ns; k++) {
                    const double a = -2.0 * 3.14159265358979323846264338328 * (double)(k * r) / (double)(ns * R);
                    tab[r * ns + k] = make_float2((float)cos(a), (float)sin(a));
                }
        }
}

// Stage body (twiddles + butterflies) of radix r and stride ns for one
// thread; a uniform branch selects the code of the radix.
template <int N, int T, int E, int V = 0>
AW_HD void stage_compute(float2* v, int t, const float2* tw, int r, int ns)
{
    if constexpr (has_radix<N, V>(32)) if (r == 32) { stage_twiddle_rt<N, T, E, 32>(v, t, tw, ns); stage_dft_rt<E, 32>(v); return; }
    if constexpr (has_radix<N, V>(16)) if (r == 16) { stage_twiddle_rt<N, T, E, 16>(v, t, tw, ns); stage_dft_rt<E, 16>(v); return; }
    if constexpr (has_radix<N, V>(8)) if (r == 8) { stage_twiddle_rt<N, T, E, 8>(v, t, tw, ns); stage_dft_rt<E, 8>(v); return; }
}

template <int N, int T, int E, int V = 0>
AW_HD void stage_exchange_store(const float2* v, float2* buf, int t, int r, int ns)
{
    if constexpr (has_radix<N, V>(32)) if (r == 32) { stage_store_rt<N, T, E, 32>(v, buf, t, ns); return; }
    if constexpr (has_radix<N, V>(16)) if (r == 16) { stage_store_rt<N, T, E, 16>(v, buf, t, ns); return; }
    if constexpr (has_radix<N, V>(8)) if (r == 8) { stage_store_rt<N, T, E, 8>(v, buf, t, ns); return; }
}

template <int N, int T, int E, int V = 0>
AW_HD void stage_exchange_load(float2* v, const float2* buf, int t, int r)
{
    if constexpr (has_radix<N, V>(32)) if (r == 32) { stage_load<N, T, E, 32>(v, buf, t); return; }
    if constexpr (has_radix<N, V>(16)) if (r == 16) { stage_load<N, T, E, 16>(v, buf, t); return; }
    if constexpr (has_radix<N, V>(8)) if (r == 8) { stage_load<N, T, E, 8>(v, buf, t); return; }
}

}  // namespace atmwfs
