// capi.cu -- C ABI of the wavefront-series engine: context set-up (the host
// part of make_AtmosphericTurbulence_wavefront_series,
// src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433-2560), the per-step
// launch graph, and the unit-level operators.
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "atmwfs.h"
#include "aux_kernels.cuh"
#include "atan_ff.cuh"

namespace atmwfs {

static const double kPi = 3.14159265358979323846264338328;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

static atmwfs_status fail(atmwfs_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

#define AW_CUDA(expr)                                                                                     \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return fail(ATMWFS_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                        \
    } while (0)

#define AW_TRY(expr)                            \
    do {                                        \
        atmwfs_status s_ = (expr);              \
        if (s_ != ATMWFS_OK) return s_;         \
    } while (0)

// Error message for entry points defined in other translation units.
void set_error_message(const char* msg) { g_err = msg ? msg : ""; }

PassLauncher pass_launcher(int N)
{
    switch (N) {
        case 64: return launch_pass_64;
        case 128: return launch_pass_128;
        case 256: return launch_pass_256;
        case 512: return launch_pass_512;
        case 1024: return launch_pass_1024;
        case 2048: return launch_pass_2048;
        default: return nullptr;
    }
}

PassLauncherCfg pass_launcher_cfg(int N)
{
    switch (N) {
        case 64: return launch_pass_cfg_64;
        case 128: return launch_pass_cfg_128;
        case 256: return launch_pass_cfg_256;
        case 512: return launch_pass_cfg_512;
        case 1024: return launch_pass_cfg_1024;
        case 2048: return launch_pass_cfg_2048;
        default: return nullptr;
    }
}

PassLauncherHalf pass_launcher_half(int N)
{
    switch (N) {
        case 64: return launch_pass_half_64;
        case 128: return launch_pass_half_128;
        case 256: return launch_pass_half_256;
        case 512: return launch_pass_half_512;
        case 1024: return launch_pass_half_1024;
        case 2048: return launch_pass_half_2048;
        default: return nullptr;
    }
}

static bool pow2_in(long n, long lo, long hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

// Concatenated stage twiddle tables of grid size N and radix plan V
// (build_twiddles).
static std::vector<float2> host_twiddles(int N, int V = 0)
{
    std::vector<float2> h;
    if (V == 1 && N == 1024) {
        h.resize(tw_total<1024, 1>());
        build_twiddles<1024, 1>(h.data());
        return h;
    }
    if (V != 0) return h;
    switch (N) {
        case 64: h.resize(tw_total<64>()); build_twiddles<64>(h.data()); break;
        case 128: h.resize(tw_total<128>()); build_twiddles<128>(h.data()); break;
        case 256: h.resize(tw_total<256>()); build_twiddles<256>(h.data()); break;
        case 512: h.resize(tw_total<512>()); build_twiddles<512>(h.data()); break;
        case 1024: h.resize(tw_total<1024>()); build_twiddles<1024>(h.data()); break;
        case 2048: h.resize(tw_total<2048>()); build_twiddles<2048>(h.data()); break;
        case 4096: h.resize(tw_total<4096>()); build_twiddles<4096>(h.data()); break;
        case 8192: h.resize(tw_total<8192>()); build_twiddles<8192>(h.data()); break;
        default: break;
    }
    return h;
}

// Size and contents of the tables without any allocation (used by the
// allocation-free entry point).
int twiddle_count(int N)
{
    switch (N) {
        case 64: return tw_total<64>();
        case 128: return tw_total<128>();
        case 256: return tw_total<256>();
        case 512: return tw_total<512>();
        case 1024: return tw_total<1024>();
        case 2048: return tw_total<2048>();
        default: return 0;
    }
}

void twiddle_fill(int N, float2* out)
{
    switch (N) {
        case 64: build_twiddles<64>(out); break;
        case 128: build_twiddles<128>(out); break;
        case 256: build_twiddles<256>(out); break;
        case 512: build_twiddles<512>(out); break;
        case 1024: build_twiddles<1024>(out); break;
        case 2048: build_twiddles<2048>(out); break;
        default: break;
    }
}

// Stage twiddle tables evaluated in double.  One copy per (device, N, radix
// plan) for the life of the process.
static const float2* twiddles(int N, int V = 0)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, float2*> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(dev, N * 4 + V);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const std::vector<float2> h = host_twiddles(N, V);
    if (h.empty()) return nullptr;
    float2* d = nullptr;
    if (cudaMalloc(&d, sizeof(float2) * h.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    cache[key] = d;
    return d;
}

const float2* stage_twiddles(int N) { return twiddles(N); }

// The same tables rounded to FP16 for the FP16-transform passes.
static const __half2* twiddles_half(int N)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, __half2*> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(dev, N);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const std::vector<float2> h = host_twiddles(N);
    std::vector<__half2> hh(h.size());
    for (size_t i = 0; i < h.size(); i++) hh[i] = __floats2half2_rn(h[i].x, h[i].y);
    __half2* d = nullptr;
    if (cudaMalloc(&d, sizeof(__half2) * hh.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, hh.data(), sizeof(__half2) * hh.size(), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    cache[key] = d;
    return d;
}

// 1-D Fresnel transfer table of one hop: H[k] = exp(-i c f_k^2) / N with
// c = pi z lambda / (dx N)^2 (WFpropagate.c:91) and f_k the centred
// frequency of unshifted index k (the permut() pair around the multiply,
// WFpropagate.c:75, 143).  The product over the two axes is the reference's
// exp(-i c ((i-N/2)^2 + (j-N/2)^2)) / N^2.  The angle is formed and reduced
// to [-pi, pi] in double before the float rounding.
static void transfer_table(float2* h, int N, double dx, double z, double lambda)
{
    const double coeff = kPi * z * lambda / (dx * (double)N) / (dx * (double)N);
    for (int k = 0; k < N; k++) {
        const long f = k < N / 2 ? k : k - N;
        double ang = -coeff * (double)(f * f);
        ang -= 2.0 * kPi * nearbyint(ang / (2.0 * kPi));
        h[k] = make_float2((float)(cos(ang) / N), (float)(sin(ang) / N));
    }
}

// ---------------------------------------------------------------------------
// super-layer grouping (AtmosphericTurbulence.c:2067-2132) and the layer ->
// super-layer index (:2135-2147; the reference's read past the end of the
// separator array is given the value +infinity, which leaves the result
// unchanged).  cn2 is normalised.
// ---------------------------------------------------------------------------
static int group_superlayers(const std::vector<double>& alt, const std::vector<double>& cn2, double bin,
                             std::vector<double>& salt, std::vector<int>& sidx)
{
    const int L = (int)alt.size();
    salt = alt;
    std::vector<double> scn2 = cn2;
    int S = L;
    for (;;) {
        double mind = alt[L - 1];
        int idx = 0;
        for (int i = 0; i < S - 1; i++) {
            const double v = salt[i + 1] - salt[i];
            if (v < mind) { mind = v; idx = i; }
        }
        if (mind > bin || S == 1) break;
        salt[idx] = (scn2[idx] * salt[idx] + scn2[idx + 1] * salt[idx + 1]) / (scn2[idx] + scn2[idx + 1]);
        scn2[idx] += scn2[idx + 1];
        for (int i = idx + 1; i < S - 1; i++) { salt[i] = salt[i + 1]; scn2[i] = scn2[i + 1]; }
        S--;
    }
    salt.resize(S);
    const int nsep = S - 1;
    std::vector<double> sep(nsep + 1);
    for (int i = 0; i < nsep; i++) sep[i] = 0.5 * (salt[i] + salt[i + 1]);
    sep[nsep] = INFINITY;
    sidx.assign(L, 0);
    for (int l = 0; l < L; l++) {
        int idx = 0;
        for (int i = 0; i < nsep; i++)
            if (sep[i] < alt[l] && sep[i + 1] > alt[l]) idx = i + 1;
        if (nsep > 0 && alt[l] > sep[nsep - 1]) idx = nsep;
        sidx[l] = idx;
    }
    return S;
}

// Propagation planes: runs of layers with one super-layer index met while
// walking from the top layer down (:2649-2692); hop k goes from plane k to
// plane k + 1 over (salt[upper] - salt[lower]) / cos(zenith).  Without
// amplitude or Fresnel propagation all layers share one plane.
static void build_planes(const std::vector<double>& salt, const std::vector<int>& sidx, int amplitude, int fresnel,
                         float zangle, std::vector<int>& lo, std::vector<int>& hi, std::vector<double>& hop)
{
    const int L = (int)sidx.size();
    lo.clear(); hi.clear(); hop.clear();
    if (amplitude && fresnel) {
        int h = L;
        for (int l = L - 1; l >= 0; l--) {
            if (l == 0 || sidx[l - 1] != sidx[l]) {
                lo.push_back(l);
                hi.push_back(h);
                if (l > 0) hop.push_back((salt[sidx[l]] - salt[sidx[l - 1]]) / cos((double)zangle));
                h = l;
            }
        }
    } else {
        lo.push_back(0);
        hi.push_back(L);
    }
}

struct Class {
    int N = 0, Nout = 0, RR = 0;
    int cfg = 0;               // tile configuration (tile_cfg), chosen by the autotuner
    std::vector<int> members;  // global instance indices
    int base = 0;              // first slot in the class-ordered InstDev array
    // this class's science instances: entries [sci0, sci0 + nsci) of the
    // context's science list, their largest bin grid and crop
    int sci0 = 0, nsci = 0, maxnb = 0, maxnout = 0;
    TmaSet maps[kNumTileCfg];  // per configuration: the box height is RR + 3
    double tuned_ms[kNumTileCfg] = {};
    // windows of the groups whose side is this class's N (the class that
    // owns the TMA maps of that size computes them), tile configuration 0
    std::vector<WinJob> jobs;
    WinJob* d_jobs = nullptr;
    // layer sums of the same groups (those with a factoring Scoeff), and
    // whether any member still needs its own phase sum (k_phasum)
    std::vector<GroupSumJob> gjobs;
    GroupSumJob* d_gjobs = nullptr;
    bool need_phasum = true;
};

}  // namespace atmwfs

using namespace atmwfs;

struct atmwfs_ctx {
    // configuration
    int L = 0, ninst = 0, ring = 1;
    bool fp16 = false;                   // FP16 transforms in the series passes
    long M = 0;
    float pupil = 0, zangle = 0, tstep = 0;
    int amplitude = 1, fresnel = 1, realtime = 0;
    double rtfactor = 1.0;
    std::vector<double> alt, cn2, speed, dir;
    std::vector<atmwfs_instance> inst;
    std::vector<std::vector<float>> scoeff;
    std::vector<std::vector<double>> roff;
    // planes: runs of layers with one super-layer index, top first
    std::vector<double> salt;
    std::vector<int> sidx;
    std::vector<int> plane_lo, plane_hi;  // layers [lo, hi)
    std::vector<double> hop_z;            // hop i: plane i -> plane i + 1
    std::vector<std::vector<double>> hop_n;  // per instance: air index of each hop (1 = vacuum lambda)
    // frozen-flow state [inst * L + layer]
    std::vector<double> xpos, ypos, xpos0, ypos0, vx, vy;
    std::vector<long> xcnt, ycnt;
    long steps = 0;
    // device
    cudaStream_t st = nullptr;
    int Nmax = 0, Wp = 0, Hp = 0;
    std::vector<float*> d_screen;        // raw M x M per layer
    std::vector<float*> d_pad[2];        // padded copies per layer and orientation
    std::vector<char> loaded;
    bool normalized = false, committed = false;
    std::vector<Class> classes;
    // window groups: instances whose layer positions are identical at every
    // step (same start positions and offsets) share the per-step bicubic
    // windows of the screens; group g has side wg[g] (its largest grid)
    std::vector<int> group_of;           // global instance -> group
    std::vector<int> group_leader, wg;
    std::vector<float*> d_win[2];        // [orient][group * L + layer], or null
    // per group: its layer sum (k_group_sum) when every member's Scoeff is
    // the same for all layers, else null
    std::vector<float2*> d_gsum;
    std::vector<InstDev> hinst;          // class order
    std::vector<int> slot_of;            // global index -> class-order slot
    InstDev* d_inst = nullptr;
    std::vector<void*> allocs;
    size_t frame_floats = 0;
    std::vector<size_t> frame_off;       // per global instance
    float* d_out_pha = nullptr;          // [ring][frame_floats]
    float* d_out_amp = nullptr;
    int* d_step = nullptr;
    unsigned* d_status = nullptr;
    int* d_iters = nullptr;
    int* d_sci = nullptr;
    float2* d_atan_tab = nullptr;  // atan(k / 1024) pairs of the science unwrap
    int nsci = 0, maxnb = 0, maxnout = 0;
    LayerPos* d_pos = nullptr;
    int poscap = 256;
    LayerPos* h_pos[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec = nullptr;
    int step_kernels = 0;                // kernel nodes of the captured step graph
    // graph branches: one stream per grid class, one for the phase sums
    std::vector<cudaStream_t> cls_st;
    cudaStream_t sum_st = nullptr;
    std::vector<cudaEvent_t> gev;
    // copies to the caller's sink: their own stream, so that step g + 1
    // computes while step g's frames leave; per device ring slot, the event
    // after the step that wrote it and the event after its copy
    cudaStream_t out_st = nullptr;
    std::vector<cudaEvent_t> ev_written, ev_copied;
};

namespace {

atmwfs_status dalloc(atmwfs_ctx* c, void** p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(ATMWFS_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    c->allocs.push_back(*p);
    return ATMWFS_OK;
}

// Start positions, wind, source and refraction offsets (:2152-2197).
void init_positions(atmwfs_ctx* c)
{
    const int L = c->L;
    const size_t n = (size_t)c->ninst * L;
    c->xpos.assign(n, 0); c->ypos.assign(n, 0); c->xpos0.assign(n, 0); c->ypos0.assign(n, 0);
    c->vx.assign(n, 0); c->vy.assign(n, 0); c->xcnt.assign(n, 0); c->ycnt.assign(n, 0);
    const float dx = c->pupil;  // PUPIL_SCALE / pfactor with pfactor = 1, a float
    for (int i = 0; i < c->ninst; i++)
        for (int l = 0; l < L; l++) {
            const size_t k = (size_t)i * L + l;
            const atmwfs_instance& I = c->inst[i];
            c->xpos[k] = 0.05 * c->M;
            c->ypos[k] = 0.05 * c->M;
            c->ypos[k] += c->roff[i][l] / dx;
            c->xpos[k] += I.src_x * c->alt[l] / dx;
            c->ypos[k] += I.src_y * c->alt[l] / dx;
            c->xpos0[k] = I.src_x * c->alt[l] / dx;
            c->ypos0[k] = I.src_y * c->alt[l] / dx;
            c->vx[k] = c->speed[l] * cos(c->dir[l]) / dx;
            c->vy[k] = c->speed[l] * sin(c->dir[l]) / dx;
        }
}

// Window groups: instances with bit-identical start positions and source
// offsets on every layer move identically at every step (the same updates
// from the same values), so their bicubic windows are the same samples.
void make_groups(atmwfs_ctx* c)
{
    const int L = c->L;
    c->group_of.assign(c->ninst, -1);
    c->group_leader.clear();
    c->wg.clear();
    for (int i = 0; i < c->ninst; i++) {
        for (size_t g = 0; g < c->group_leader.size() && c->group_of[i] < 0; g++) {
            const int j = c->group_leader[g];
            bool same = true;
            for (int l = 0; l < L && same; l++) {
                const size_t a = (size_t)i * L + l, b = (size_t)j * L + l;
                same = c->xpos[a] == c->xpos[b] && c->ypos[a] == c->ypos[b] && c->xpos0[a] == c->xpos0[b] &&
                       c->ypos0[a] == c->ypos0[b];
            }
            if (same) c->group_of[i] = (int)g;
        }
        if (c->group_of[i] < 0) {
            c->group_of[i] = (int)c->group_leader.size();
            c->group_leader.push_back(i);
            c->wg.push_back(0);
        }
        int& w = c->wg[c->group_of[i]];
        w = std::max(w, (int)c->inst[i].wf_raw_size);
    }
}

// One step of the frozen-flow update of every layer of every instance
// (:2700-2756) and the per-window sample origin (the reference evaluates
// fmod(pos + ii, M) per pixel; at ii = 0 this gives the window origin).
void advance_positions(atmwfs_ctx* c, double tnow, LayerPos* out)
{
    const double Md = (double)c->M;
    const size_t n = (size_t)c->ninst * c->L;
    for (size_t k = 0; k < n; k++) {
        if (c->realtime) {
            c->xpos[k] = c->xpos0[k] + c->vx[k] * tnow + 1.0 * c->xcnt[k] * Md;
            c->ypos[k] = c->ypos0[k] + c->vy[k] * tnow + 1.0 * c->ycnt[k] * Md;
        } else {
            c->xpos[k] += c->vx[k] * c->tstep;
            c->ypos[k] += c->vy[k] * c->tstep;
        }
        while (c->xpos[k] < 0) { c->xpos[k] += Md; c->xcnt[k]++; }
        while (c->xpos[k] > Md) { c->xpos[k] -= Md; c->xcnt[k]--; }
        while (c->ypos[k] < 0) { c->ypos[k] += Md; c->ycnt[k]++; }
        while (c->ypos[k] > Md) { c->ypos[k] -= Md; c->ycnt[k]--; }
        const double fxm = fmod(c->xpos[k], Md), fym = fmod(c->ypos[k], Md);
        LayerPos p;
        p.ix = (int)(long)fxm;
        p.iy = (int)(long)fym;
        p.fx = (float)(fxm - (double)p.ix);
        p.fy = (float)(fym - (double)p.iy);
        out[k] = p;
    }
}

atmwfs_status make_tma_map(CUtensorMap* m, float* base, int Wp, int Hp, int box_rows)
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
            return fail(ATMWFS_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    cuuint64_t dims[2] = {(cuuint64_t)Wp, (cuuint64_t)Hp};
    cuuint64_t strides[1] = {(cuuint64_t)Wp * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kBoxW, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(ATMWFS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return ATMWFS_OK;
}

// Orientation of pass k (1-based) of Q = P + 1 passes: the last pass is in
// the screen's own orientation.
int pass_orient(int k, int Q) { return (Q - k) & 1; }

// The window kernel over jobs [j0, j1) of class cl (the windows of the
// groups whose side is cl's grid); optionally report its algorithmic bytes.
atmwfs_status launch_windows(atmwfs_ctx* c, Class& cl, int j0, int j1, double* bytes, cudaStream_t st)
{
    if (bytes) *bytes = 0;
    if (j1 <= j0) return ATMWFS_OK;
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.pos = c->d_pos;
    a.d_step = c->d_step;
    a.d_status = c->d_status;
    a.L = c->L;
    a.ninst_total = c->ninst;
    a.poscap = c->poscap;
    a.jobs = cl.d_jobs + j0;
    const int RR0 = tile_cfg(cl.N, 0).rr;
    // screen tiles in (RR0 + 3 rows of the padded width) and windows out
    if (bytes) *bytes = (4.0 * (RR0 + 3) / RR0 + 4.0) * (double)cl.N * cl.N * (j1 - j0);
    AW_CUDA(pass_launcher_cfg(cl.N)(0, kVarWindows, dim3(cl.N / RR0, (unsigned)(j1 - j0)), a, &cl.maps[0], nullptr, st));
    return ATMWFS_OK;
}

// Launch pass k (1-based) for grid class cl; optionally report the
// algorithmic bytes of the launch.
atmwfs_status launch_pass(atmwfs_ctx* c, int k, Class& cl, double* bytes, cudaStream_t st)
{
    const int Q = (int)c->plane_lo.size();
    const int P = Q - 1;
    if (k == 0) {
        // geometric phase sums: the layer sums of the window groups this class
        // computes (instances whose Scoeff factors out), then the per-instance
        // sums of the others (k_phasum), from the step's windows
        double b = 0;
        if (!cl.gjobs.empty()) {
            AW_CUDA(group_sums(cl.d_gjobs, (int)cl.gjobs.size(), c->L, cl.N, st));
            b += (4.0 * c->L + 8.0) * (double)cl.N * cl.N * cl.gjobs.size();
        }
        if (!cl.need_phasum) {
            if (bytes) *bytes = b;
            return ATMWFS_OK;
        }
        PassArgs a;
        memset(&a, 0, sizeof a);
        a.inst = c->d_inst + cl.base;
        a.d_step = c->d_step;
        a.d_status = c->d_status;
        a.L = c->L;
        a.ninst_total = c->ninst;
        a.poscap = c->poscap;
        int own = 0;
        for (int i : cl.members) own += c->d_gsum[c->group_of[i]] == nullptr;
        if (bytes) *bytes = b + (4.0 * c->L + 4.0) * cl.Nout * cl.Nout * own;
        AW_CUDA(pass_launcher_cfg(cl.N)(0, kVarPhasum, dim3(phasum_blocks(cl.Nout), (unsigned)cl.members.size()), a,
                                        nullptr, nullptr, st));
        return ATMWFS_OK;
    }
    if (k == Q + 2) {
        // the science unwrap and the final 2 pi multiples of every science
        // instance of the context (diagnostics only)
        if (bytes) *bytes = 0;
        if (c->nsci > 0) {
            AW_CUDA(unwrap_bins(c->d_inst, c->d_sci, c->nsci, c->maxnb, c->d_status, c->d_iters, c->d_atan_tab, st));
            AW_CUDA(sci_apply(c->d_inst, c->d_sci, c->nsci, c->maxnout, c->d_step, st));
        }
        return ATMWFS_OK;
    }
    if (k == Q + 1) {
        // the step's windows of the groups this class computes
        if (bytes) *bytes = 0;
        if (cl.jobs.empty()) return ATMWFS_OK;
        return launch_windows(c, cl, 0, (int)cl.jobs.size(), bytes, st);
    }
    {
        {
            PassArgs a;
            memset(&a, 0, sizeof a);
            a.inst = c->d_inst + cl.base;
            a.pos = c->d_pos;
            a.d_step = c->d_step;
            a.d_status = c->d_status;
            a.L = c->L;
            a.ninst_total = c->ninst;
            a.poscap = c->poscap;
            a.g_lo = c->plane_lo[k - 1];
            a.g_hi = c->plane_hi[k - 1];
            a.hop1 = k - 2;
            a.hop2 = k - 1;
            a.src = k & 1;
            a.dst = (k + 1) & 1;
            a.orient = pass_orient(k, Q);
            int var;
            (void)P;
            if (Q == 1) var = kVarSingle;
            else if (k == 1) var = kVarFirst;
            else if (k == Q) var = kVarLast;
            else var = kVarMid;
            int rows = cl.N;
            a.row0 = 0;
            if (var == kVarLast || var == kVarSingle) {
                const int off = (cl.N - cl.Nout) / 2;
                a.row0 = off / cl.RR * cl.RR;
                rows = (off + cl.Nout - a.row0 + cl.RR - 1) / cl.RR * cl.RR;
            }
            dim3 grid(rows / cl.RR, (unsigned)cl.members.size());
            if (bytes) {
                // field read / transposed write (8 B/px each), the window rows
                // of every gathered layer (4 B/px), outputs
                const double px = (double)cl.N * cl.N, npx = (double)rows * cl.N, cnt = (double)cl.members.size();
                const int ng = a.g_hi - a.g_lo;
                double b = 0;
                if (var & OP_LOAD) b += 8.0 * npx;
                if (var & OP_STORE_T) b += 8.0 * px;
                b += 4.0 * npx * ng;
                if (var & OP_EPI) b += (double)cl.Nout * cl.Nout * 12.0;  // phase sum in, pha + amp out
                *bytes = b * cnt;
            }
            if (c->fp16 && var != kVarSingle)
                AW_CUDA(pass_launcher_half(cl.N)(var, grid, a, &cl.maps[cl.cfg], twiddles_half(cl.N), st));
            else
                AW_CUDA(pass_launcher_cfg(cl.N)(cl.cfg, var, grid, a, &cl.maps[cl.cfg],
                                                twiddles(cl.N, tile_cfg(cl.N, cl.cfg).plan), st));
        }
    }
    return ATMWFS_OK;
}

// One step.  The screen windows of every window group come first; then the
// graph forks: the phase sums (independent of the field) on their own
// branch, every grid class's chain of passes on its own branch; the last pass
// of each class waits for the phase sums; everything joins before the
// science unwrap.
atmwfs_status launch_step(atmwfs_ctx* c)
{
    const int Q = (int)c->plane_lo.size();
    const int nc = (int)c->classes.size();
    cudaEvent_t fork = c->gev[0], sums = c->gev[1];
    // the step's screen windows, read by the phase sums and by every pass
    // (launching those of the later passes beside the first pass measured no
    // faster: the transforms keep every SM's registers busy)
    for (Class& cl : c->classes) AW_TRY(launch_windows(c, cl, 0, (int)cl.jobs.size(), nullptr, c->st));
    AW_CUDA(cudaEventRecord(fork, c->st));
    AW_CUDA(cudaStreamWaitEvent(c->sum_st, fork, 0));
    for (Class& cl : c->classes) AW_TRY(launch_pass(c, 0, cl, nullptr, c->sum_st));
    AW_CUDA(cudaEventRecord(sums, c->sum_st));
    for (int ci = 0; ci < nc; ci++) {
        cudaStream_t cs = c->cls_st[ci];
        AW_CUDA(cudaStreamWaitEvent(cs, fork, 0));
        for (int k = 1; k <= Q; k++) {
            if (k == Q) AW_CUDA(cudaStreamWaitEvent(cs, sums, 0));
            AW_TRY(launch_pass(c, k, c->classes[ci], nullptr, cs));
        }
        // the class's science unwrap and apply on its own branch: a class that
        // finishes early unwraps beside the passes of the larger grids
        const Class& cl = c->classes[ci];
        if (cl.nsci > 0) {
            AW_CUDA(unwrap_bins(c->d_inst, c->d_sci + cl.sci0, cl.nsci, cl.maxnb, c->d_status, c->d_iters,
                                c->d_atan_tab, cs));
            AW_CUDA(sci_apply(c->d_inst, c->d_sci + cl.sci0, cl.nsci, cl.maxnout, c->d_step, cs));
        }
        AW_CUDA(cudaEventRecord(c->gev[2 + ci], cs));
        AW_CUDA(cudaStreamWaitEvent(c->st, c->gev[2 + ci], 0));
    }
    AW_CUDA(step_advance(c->d_step, c->st));
    return ATMWFS_OK;
}

atmwfs_status check_status(atmwfs_ctx* c);

// Zero the science bins on the engine stream: a last pass launched outside a
// step (timing, tuning) adds its bin sums, which the next step's unwrap
// would otherwise read.
atmwfs_status clear_bins(atmwfs_ctx* c)
{
    for (const InstDev& d : c->hinst)
        if (d.bins) AW_CUDA(cudaMemsetAsync(d.bins, 0, sizeof(*d.bins) * 2 * (d.nb * d.nb > 0 ? d.nb * d.nb : 1), c->st));
    return ATMWFS_OK;
}

// Project autotuner: for every grid class time the representative pass
// (a middle pass when there is one) in each configuration compiled for its
// size -- radix plan and tile shape (tile_cfg) -- and keep the fastest.
// ATMWFS_TILE_CFG=<k> forces configuration k (ignored where the size has
// none); ATMWFS_TILE_CFG=<N>:<k>[,<N>:<k>...] forces it for the listed grid
// sizes only and tunes the others.  Science bins are cleared afterwards (a
// timed last pass accumulates into them).
int forced_cfg(const char* force, int N)
{
    if (!force || !*force) return -1;
    if (!strchr(force, ':')) return atoi(force);
    for (const char* p = force; p && *p;) {
        char* end = nullptr;
        const long n = strtol(p, &end, 10);
        if (end && *end == ':' && n == N) return atoi(end + 1);
        p = strchr(p, ',');
        if (p) p++;
    }
    return -1;
}

atmwfs_status autotune(atmwfs_ctx* c)
{
    const int Q = (int)c->plane_lo.size();
    const char* force = getenv("ATMWFS_TILE_CFG");
    const int k = Q >= 3 ? 2 : 1;
    // the candidates are timed with plain launches (see pdl_hold)
    struct Hold {
        Hold() { pdl_hold() = 1; }
        ~Hold() { pdl_hold() = 0; }
    } hold;
    cudaEvent_t e0, e1;
    AW_CUDA(cudaEventCreate(&e0));
    AW_CUDA(cudaEventCreate(&e1));
    atmwfs_status s = ATMWFS_OK;
    for (Class& cl : c->classes) {
        if (c->fp16) {
            cl.cfg = 2;  // the FP16-transform passes are compiled for configuration 2
        } else if (forced_cfg(force, cl.N) >= 0) {
            const int g = forced_cfg(force, cl.N);
            cl.cfg = (g < kNumTileCfg && tile_cfg(cl.N, g).rr > 0) ? g : 0;
        } else {
            // two interleaved rounds over the configurations; each keeps its
            // fastest reading, so one disturbed reading does not decide
            for (int g = 0; g < kNumTileCfg; g++) cl.tuned_ms[g] = 1e30f;
            for (int round = 0; round < 2 && s == ATMWFS_OK; round++) {
                for (int g = 0; g < kNumTileCfg && s == ATMWFS_OK; g++) {
                    if (tile_cfg(cl.N, g).rr == 0) continue;  // not compiled at this size
                    cl.cfg = g;
                    cl.RR = tile_cfg(cl.N, g).rr;
                    s = launch_pass(c, k, cl, nullptr, c->st);
                    if (s != ATMWFS_OK) break;
                    cudaEventRecord(e0, c->st);
                    for (int r = 0; r < 3 && s == ATMWFS_OK; r++) s = launch_pass(c, k, cl, nullptr, c->st);
                    cudaEventRecord(e1, c->st);
                    float ms = 0;
                    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                        s = fail(ATMWFS_ERR_CUDA, "autotune timing failed");
                    if (ms / 3 < cl.tuned_ms[g]) cl.tuned_ms[g] = ms / 3;
                }
            }
            int bg = 0;
            for (int g = 1; g < kNumTileCfg; g++)
                if (cl.tuned_ms[g] < cl.tuned_ms[bg]) bg = g;
            for (int g = 0; g < kNumTileCfg; g++)
                if (tile_cfg(cl.N, g).rr == 0) cl.tuned_ms[g] = 0;
            cl.cfg = bg;
        }
        cl.RR = tile_cfg(cl.N, cl.cfg).rr;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != ATMWFS_OK) return s;
    AW_TRY(clear_bins(c));
    AW_CUDA(cudaStreamSynchronize(c->st));
    return check_status(c);
}

atmwfs_status commit(atmwfs_ctx* c)
{
    if (c->committed) return ATMWFS_OK;
    for (int l = 0; l < c->L; l++)
        if (!c->loaded[l]) return fail(ATMWFS_ERR_STATE, "screen of layer %d not loaded", l);
    const int Q = (int)c->plane_lo.size();
    // orientations needed: 0 for every layer (last pass sums all layers),
    // 1 for the layers gathered by passes in the transposed orientation
    std::vector<char> need1(c->L, 0);
    for (int k = 1; k <= Q; k++)
        if (pass_orient(k, Q) == 1)
            for (int l = c->plane_lo[k - 1]; l < c->plane_hi[k - 1]; l++) need1[l] = 1;
    const size_t padn = (size_t)c->Wp * c->Hp;
    for (int l = 0; l < c->L; l++) {
        for (int o = 0; o < 2; o++) {
            if (o == 1 && !need1[l]) continue;
            if (!c->d_pad[o][l]) AW_TRY(dalloc(c, (void**)&c->d_pad[o][l], padn * sizeof(float)));
            AW_CUDA(pad_screen(c->d_screen[l], (int)c->M, c->d_pad[o][l], c->Wp, c->Hp, o, c->st));
        }
    }
    // windows: the screen orientation of every layer (phase sums, passes in
    // that orientation), the transposed one of the layers gathered by
    // transposed passes
    const int G = (int)c->group_leader.size();
    for (int o = 0; o < 2; o++) c->d_win[o].resize((size_t)G * c->L, nullptr);
    for (int g = 0; g < G; g++)
        for (int o = 0; o < 2; o++)
            for (int l = 0; l < c->L; l++) {
                if (o == 1 && !need1[l]) continue;
                float*& w = c->d_win[o][(size_t)g * c->L + l];
                if (!w) {
                    const size_t bytes = sizeof(float) * (size_t)c->wg[g] * c->wg[g];
                    AW_TRY(dalloc(c, (void**)&w, bytes));
                    AW_CUDA(cudaMemsetAsync(w, 0, bytes, c->st));
                }
            }
    for (Class& cl : c->classes) {
        cl.jobs.clear();
        bool owner = true;  // the first class of each size computes its groups' windows
        for (const Class& other : c->classes) {
            if (&other == &cl) break;
            if (other.N == cl.N) owner = false;
        }
        if (!owner) continue;
        for (int g = 0; g < G; g++) {
            if (c->wg[g] != cl.N) continue;
            for (int o = 0; o < 2; o++)
                for (int l = 0; l < c->L; l++)
                    if (float* w = c->d_win[o][(size_t)g * c->L + l])
                        cl.jobs.push_back(WinJob{w, c->group_leader[g], l, o, c->wg[g]});
        }
        if (cl.jobs.empty()) continue;
        if (!cl.d_jobs) AW_TRY(dalloc(c, (void**)&cl.d_jobs, sizeof(WinJob) * cl.jobs.size()));
        AW_CUDA(cudaMemcpyAsync(cl.d_jobs, cl.jobs.data(), sizeof(WinJob) * cl.jobs.size(), cudaMemcpyHostToDevice, c->st));
    }
    // Phase-sum factoring per group (ATMWFS_GROUP_PHASE_SUM=0 turns it off):
    // every member's Scoeff equal on all layers (bit for bit)
    const char* gps = getenv("ATMWFS_GROUP_PHASE_SUM");
    const bool factor = !(gps && atoi(gps) == 0);
    c->d_gsum.resize(G, nullptr);
    for (int g = 0; g < G; g++) {
        bool ok = factor && c->L <= kMaxLayers;
        for (int i = 0; i < c->ninst && ok; i++)
            if (c->group_of[i] == g)
                for (int l = 1; l < c->L && ok; l++) ok = c->scoeff[i][l] == c->scoeff[i][0];
        if (ok && !c->d_gsum[g]) AW_TRY(dalloc(c, (void**)&c->d_gsum[g], sizeof(float2) * (size_t)c->wg[g] * c->wg[g]));
    }
    for (Class& cl : c->classes) {
        cl.gjobs.clear();
        for (const WinJob& j : cl.jobs) {
            const int g = c->group_of[j.gidx];
            if (j.orient != 0 || j.layer != 0 || !c->d_gsum[g]) continue;
            GroupSumJob gj;
            memset(&gj, 0, sizeof gj);
            gj.out = c->d_gsum[g];
            gj.side = c->wg[g];
            for (int l = 0; l < c->L; l++) gj.win[l] = c->d_win[0][(size_t)g * c->L + l];
            cl.gjobs.push_back(gj);
        }
        cl.need_phasum = false;
        for (int i : cl.members) cl.need_phasum = cl.need_phasum || !c->d_gsum[c->group_of[i]];
        if (cl.gjobs.empty()) continue;
        if (!cl.d_gjobs) AW_TRY(dalloc(c, (void**)&cl.d_gjobs, sizeof(GroupSumJob) * cl.gjobs.size()));
        AW_CUDA(cudaMemcpyAsync(cl.d_gjobs, cl.gjobs.data(), sizeof(GroupSumJob) * cl.gjobs.size(),
                                cudaMemcpyHostToDevice, c->st));
    }
    for (InstDev& d : c->hinst) {
        const int g = c->group_of[d.gidx];
        d.gsum = c->d_gsum[g];
        d.wstride = c->wg[g];
        for (int o = 0; o < 2; o++)
            for (int l = 0; l < c->L; l++) d.win[o][l] = c->d_win[o][(size_t)g * c->L + l];
    }
    AW_CUDA(cudaMemcpyAsync(c->d_inst, c->hinst.data(), sizeof(InstDev) * c->hinst.size(), cudaMemcpyHostToDevice, c->st));
    for (Class& cl : c->classes) {
        memset(cl.maps, 0, sizeof cl.maps);
        for (int g = 0; g < kNumTileCfg; g++)
            for (int o = 0; o < 2; o++)
                for (int l = 0; l < c->L; l++)
                    if (c->d_pad[o][l] && tile_cfg(cl.N, g).rr > 0)
                        AW_TRY(make_tma_map(&cl.maps[g].m[o][l], c->d_pad[o][l], c->Wp, c->Hp, tile_cfg(cl.N, g).rr + 3));
    }
    AW_CUDA(cudaStreamSynchronize(c->st));
    AW_TRY(autotune(c));
    // capture one step
    cudaGraph_t g = nullptr;
    AW_CUDA(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed));
    atmwfs_status s = launch_step(c);
    cudaError_t ec = cudaStreamEndCapture(c->st, &g);
    if (s != ATMWFS_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    AW_CUDA(ec);
    {
        size_t nn = 0;
        AW_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        AW_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
        c->step_kernels = 0;
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType ty;
            AW_CUDA(cudaGraphNodeGetType(nd, &ty));
            c->step_kernels += ty == cudaGraphNodeTypeKernel;
        }
    }
    AW_CUDA(cudaGraphInstantiate(&c->gexec, g, 0));
    cudaGraphDestroy(g);
    c->committed = true;
    return ATMWFS_OK;
}

atmwfs_status check_status(atmwfs_ctx* c)
{
    unsigned st = 0;
    AW_CUDA(cudaMemcpyAsync(&st, c->d_status, sizeof st, cudaMemcpyDeviceToHost, c->st));
    AW_CUDA(cudaStreamSynchronize(c->st));
    if (st & kStatTmaTimeout) return fail(ATMWFS_ERR_TIMEOUT, "a screen tile load did not complete within 1 s");
    if (st) return fail(ATMWFS_ERR_CUDA, "device status 0x%x", st);
    return ATMWFS_OK;
}

}  // namespace

extern "C" {

const char* atmwfs_last_error(void) { return g_err.c_str(); }

atmwfs_status atmwfs_create(const atmwfs_params* p, atmwfs_ctx** out)
{
    if (!p || !out) return fail(ATMWFS_ERR_INVALID, "null argument");
    *out = nullptr;
    if (p->nlayers < 1 || p->nlayers > kMaxLayers) return fail(ATMWFS_ERR_INVALID, "nlayers must be 1..%d", kMaxLayers);
    if (!p->alt || !p->cn2 || !p->speed || !p->dir) return fail(ATMWFS_ERR_INVALID, "profile arrays missing");
    if (!pow2_in(p->master_size, 64, 1 << 16)) return fail(ATMWFS_ERR_INVALID, "master_size must be a power of two >= 64");
    if (p->ninst < 1 || !p->inst) return fail(ATMWFS_ERR_INVALID, "no instances");
    if (!(p->pupil_scale > 0)) return fail(ATMWFS_ERR_INVALID, "pupil_scale must be > 0");
    for (int i = 0; i < p->ninst; i++) {
        const atmwfs_instance& I = p->inst[i];
        if (!pow2_in(I.wf_raw_size, 64, 2048)) return fail(ATMWFS_ERR_INVALID, "instance %d: wf_raw_size must be a power of two in 64..2048", i);
        if (I.wf_size < 1 || I.wf_size > I.wf_raw_size) return fail(ATMWFS_ERR_INVALID, "instance %d: wf_size must be 1..wf_raw_size", i);
        if (I.mode < 0 || I.mode > 2) return fail(ATMWFS_ERR_INVALID, "instance %d: bad mode", i);
        if (!(I.lambda > 0)) return fail(ATMWFS_ERR_INVALID, "instance %d: lambda must be > 0", i);
    }
    // the arguments are checked before any CUDA call
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(ATMWFS_ERR_NODEVICE, "no CUDA device");
    atmwfs_ctx* c = new atmwfs_ctx();
    c->L = p->nlayers;
    c->ninst = p->ninst;
    c->ring = p->ring < 1 ? 1 : p->ring;
    c->fp16 = p->fft_fp16 != 0;
    c->M = p->master_size;
    c->pupil = p->pupil_scale;
    c->zangle = p->zangle;
    c->tstep = p->time_step;
    c->amplitude = p->amplitude;
    c->fresnel = p->amplitude ? p->fresnel : 0;  // :1395-1402
    c->realtime = p->realtime;
    c->rtfactor = p->realtime_factor;
    c->alt.assign(p->alt, p->alt + c->L);
    c->cn2.assign(p->cn2, p->cn2 + c->L);
    c->speed.assign(p->speed, p->speed + c->L);
    c->dir.assign(p->dir, p->dir + c->L);
    // Cn2 normalised to a sum of 1 (:2009-2015)
    double tot = 0.0;
    for (double v : c->cn2) tot += v;
    if (!(tot > 0)) { delete c; return fail(ATMWFS_ERR_INVALID, "sum of cn2 must be > 0"); }
    for (double& v : c->cn2) v *= 1.0 / tot;
    c->inst.assign(p->inst, p->inst + c->ninst);
    c->scoeff.resize(c->ninst);
    c->roff.resize(c->ninst);
    for (int i = 0; i < c->ninst; i++) {
        c->scoeff[i].assign(c->L, 1.0f);
        c->roff[i].assign(c->L, 0.0);
        if (p->inst[i].scoeff) c->scoeff[i].assign(p->inst[i].scoeff, p->inst[i].scoeff + c->L);
        if (p->inst[i].roffset) c->roff[i].assign(p->inst[i].roffset, p->inst[i].roffset + c->L);
        c->inst[i].scoeff = nullptr;
        c->inst[i].roffset = nullptr;
        if (c->inst[i].mode == ATMWFS_MODE_PHASE && c->amplitude) c->inst[i].mode = ATMWFS_MODE_REF;
        if (!c->amplitude) c->inst[i].mode = ATMWFS_MODE_PHASE;
    }
    group_superlayers(c->alt, c->cn2, p->fresnel_bin, c->salt, c->sidx);
    build_planes(c->salt, c->sidx, c->amplitude, c->fresnel, c->zangle, c->plane_lo, c->plane_hi, c->hop_z);
    const int P = (int)c->hop_z.size();
    c->hop_n.assign(c->ninst, std::vector<double>(P, 1.0));
    for (int i = 0; i < c->ninst; i++) {
        if (p->inst[i].hop_n)
            for (int k = 0; k < P; k++) {
                const double n = p->inst[i].hop_n[k];
                if (!(n >= 1.0 && n < 2.0)) {
                    delete c;
                    return fail(ATMWFS_ERR_INVALID, "instance %d: hop_n[%d] must be in [1, 2)", i, k);
                }
                c->hop_n[i][k] = n;
            }
        c->inst[i].hop_n = nullptr;
    }
    init_positions(c);
    make_groups(c);

    atmwfs_status s = ATMWFS_OK;
#define CK(x)                                  \
    do {                                       \
        s = (x);                               \
        if (s != ATMWFS_OK) goto fail_out;     \
    } while (0)
#define CKC(x)                                                                                            \
    do {                                                                                                  \
        cudaError_t e_ = (x);                                                                             \
        if (e_ != cudaSuccess) {                                                                          \
            s = fail(ATMWFS_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));                        \
            goto fail_out;                                                                                \
        }                                                                                                 \
    } while (0)
    {
        CKC(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
        c->d_screen.assign(c->L, nullptr);
        c->d_pad[0].assign(c->L, nullptr);
        c->d_pad[1].assign(c->L, nullptr);
        c->loaded.assign(c->L, 0);
        // classes by (N, Nout)
        for (int i = 0; i < c->ninst; i++) {
            const int N = (int)c->inst[i].wf_raw_size, No = (int)c->inst[i].wf_size;
            Class* cl = nullptr;
            for (Class& x : c->classes)
                if (x.N == N && x.Nout == No) cl = &x;
            if (!cl) {
                c->classes.push_back(Class());
                cl = &c->classes.back();
                cl->N = N;
                cl->Nout = No;
                cl->cfg = 0;
                cl->RR = tile_cfg(N, 0).rr;
            }
            cl->members.push_back(i);
            c->Nmax = c->Nmax > N ? c->Nmax : N;
        }
        c->Wp = (int)c->M + c->Nmax + 64;
        c->Hp = (int)c->M + c->Nmax + 8;
        // output frame layout: instance i at frame_off[i] inside one step's frame block
        c->frame_off.assign(c->ninst, 0);
        for (int i = 0; i < c->ninst; i++) {
            c->frame_off[i] = c->frame_floats;
            c->frame_floats += (size_t)c->inst[i].wf_size * c->inst[i].wf_size;
        }
        CK(dalloc(c, (void**)&c->d_out_pha, sizeof(float) * c->frame_floats * c->ring));
        CK(dalloc(c, (void**)&c->d_out_amp, sizeof(float) * c->frame_floats * c->ring));
        c->slot_of.assign(c->ninst, 0);
        std::vector<int> sci;
        int slot = 0;
        for (Class& cl : c->classes) {
            cl.base = slot;
            for (int i : cl.members) {
                const atmwfs_instance& I = c->inst[i];
                InstDev d;
                memset(&d, 0, sizeof d);
                const int N = cl.N, No = cl.Nout;
                d.N = N;
                d.Nout = No;
                d.off = (N - No) / 2;
                d.mode = I.mode;
                d.ring = c->ring;
                d.gidx = i;
                for (int l = 0; l < c->L; l++) d.scoeff[l] = c->scoeff[i][l];
                for (int b = 0; b < 2; b++) CK(dalloc(c, (void**)&d.fld[b], sizeof(float2) * (size_t)N * N));
                if (P > 0) {
                    std::vector<float2> h((size_t)P * N);
                    for (int hh = 0; hh < P; hh++)
                        transfer_table(h.data() + (size_t)hh * N, N, (double)c->pupil, c->hop_z[hh],
                                       I.lambda / c->hop_n[i][hh]);
                    float2* dh = nullptr;
                    CK(dalloc(c, (void**)&dh, sizeof(float2) * h.size()));
                    CKC(cudaMemcpy(dh, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice));
                    d.H = dh;
                    if (c->fp16) {
                        // N H (unit modulus) for the FP16 transforms
                        std::vector<__half2> hh(h.size());
                        for (size_t q = 0; q < h.size(); q++) hh[q] = __floats2half2_rn(h[q].x * N, h[q].y * N);
                        __half2* dhh = nullptr;
                        CK(dalloc(c, (void**)&dhh, sizeof(__half2) * hh.size()));
                        CKC(cudaMemcpy(dhh, hh.data(), sizeof(__half2) * hh.size(), cudaMemcpyHostToDevice));
                        d.Hh = dhh;
                    }
                }
                // the ring holds the frames of all instances contiguously per slot
                d.out_pha = c->d_out_pha + c->frame_off[i];
                d.out_amp = c->d_out_amp + c->frame_off[i];
                d.ostride = (long)c->frame_floats;
                CK(dalloc(c, (void**)&d.phisum, sizeof(float) * (size_t)No * No));
                if (I.mode == ATMWFS_MODE_SCI) {
                    d.nb = No / 20;
                    const int nb2 = d.nb * d.nb > 0 ? d.nb * d.nb : 1;
                    CK(dalloc(c, (void**)&d.bins, sizeof(*d.bins) * 2 * nb2));
                    CKC(cudaMemset(d.bins, 0, sizeof(*d.bins) * 2 * nb2));
                    CK(dalloc(c, (void**)&d.peak, sizeof(float) * nb2));
                    // bin of each output coordinate, as the reference computes it
                    // (long)(1.0 * ii / Wout * nb), and the first coordinate of each bin
                    std::vector<short> bx(No), b0(d.nb + 2, (short)No);
                    for (int ii = 0; ii < No; ii++) bx[ii] = (short)(long)(1.0 * ii / No * d.nb);
                    for (int ii = No - 1; ii >= 0; ii--) b0[bx[ii]] = (short)ii;
                    for (int ib = d.nb - 1; ib >= 0; ib--)
                        if (b0[ib] > b0[ib + 1]) b0[ib] = b0[ib + 1];
                    short* dbx = nullptr;
                    CK(dalloc(c, (void**)&dbx, sizeof(short) * (No + d.nb + 2)));
                    CKC(cudaMemcpy(dbx, bx.data(), sizeof(short) * No, cudaMemcpyHostToDevice));
                    CKC(cudaMemcpy(dbx + No, b0.data(), sizeof(short) * (d.nb + 2), cudaMemcpyHostToDevice));
                    d.binx = dbx;
                    d.binx0 = dbx + No;
                    if (cl.nsci == 0) cl.sci0 = (int)sci.size();
                    sci.push_back(slot);
                    cl.nsci++;
                    cl.maxnb = cl.maxnb > d.nb ? cl.maxnb : d.nb;
                    cl.maxnout = cl.maxnout > No ? cl.maxnout : No;
                    c->maxnb = c->maxnb > d.nb ? c->maxnb : d.nb;
                    c->maxnout = c->maxnout > No ? c->maxnout : No;
                }
                c->hinst.push_back(d);
                c->slot_of[i] = slot;
                slot++;
            }
        }
        CK(dalloc(c, (void**)&c->d_inst, sizeof(InstDev) * c->hinst.size()));
        CKC(cudaMemcpy(c->d_inst, c->hinst.data(), sizeof(InstDev) * c->hinst.size(), cudaMemcpyHostToDevice));
        c->nsci = (int)sci.size();
        if (c->nsci) {
            CK(dalloc(c, (void**)&c->d_sci, sizeof(int) * sci.size()));
            CKC(cudaMemcpy(c->d_sci, sci.data(), sizeof(int) * sci.size(), cudaMemcpyHostToDevice));
            std::vector<float2> tab(kAtanTabN + 1);
            atan_table_host(tab.data());
            CK(dalloc(c, (void**)&c->d_atan_tab, sizeof(float2) * tab.size()));
            CKC(cudaMemcpy(c->d_atan_tab, tab.data(), sizeof(float2) * tab.size(), cudaMemcpyHostToDevice));
        }
        CK(dalloc(c, (void**)&c->d_step, sizeof(int)));
        CKC(cudaMemset(c->d_step, 0, sizeof(int)));
        CK(dalloc(c, (void**)&c->d_status, sizeof(unsigned)));
        CKC(cudaMemset(c->d_status, 0, sizeof(unsigned)));
        CK(dalloc(c, (void**)&c->d_iters, sizeof(int) * c->ninst * 0 + sizeof(int) * (c->hinst.size() + 1)));
        const size_t posn = (size_t)c->poscap * c->ninst * c->L;
        CK(dalloc(c, (void**)&c->d_pos, sizeof(LayerPos) * posn));
        CKC(cudaMemset(c->d_pos, 0, sizeof(LayerPos) * posn));
        for (int b = 0; b < 2; b++) {
            CKC(cudaHostAlloc((void**)&c->h_pos[b], sizeof(LayerPos) * posn, cudaHostAllocDefault));
            CKC(cudaEventCreateWithFlags(&c->ev[b], cudaEventDisableTiming));
        }
        for (int b = 0; b < 2; b++) CKC(cudaEventRecord(c->ev[b], c->st));
        for (const Class& cl : c->classes) {
            // the tables of every radix plan the autotuner may pick
            for (int g = 0; g < kNumTileCfg; g++) {
                if (tile_cfg(cl.N, g).rr == 0) continue;
                if (!twiddles(cl.N, tile_cfg(cl.N, g).plan)) {
                    s = fail(ATMWFS_ERR_NOMEM, "twiddle table allocation failed");
                    goto fail_out;
                }
            }
        }
        CKC(cudaStreamCreateWithFlags(&c->sum_st, cudaStreamNonBlocking));
        c->cls_st.assign(c->classes.size(), nullptr);
        for (auto& cs : c->cls_st) CKC(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        c->gev.assign(2 + c->classes.size(), nullptr);
        for (auto& e : c->gev) CKC(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
#undef CK
#undef CKC
    *out = c;
    return ATMWFS_OK;
fail_out:
    atmwfs_destroy(c);
    return s;
}

void atmwfs_destroy(atmwfs_ctx* c)
{
    if (!c) return;
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    for (void* p : c->allocs) cudaFree(p);
    for (int b = 0; b < 2; b++) {
        if (c->h_pos[b]) cudaFreeHost(c->h_pos[b]);
        if (c->ev[b]) cudaEventDestroy(c->ev[b]);
    }
    for (auto cs : c->cls_st)
        if (cs) cudaStreamDestroy(cs);
    if (c->sum_st) cudaStreamDestroy(c->sum_st);
    for (auto e : c->gev)
        if (e) cudaEventDestroy(e);
    if (c->out_st) {
        cudaStreamSynchronize(c->out_st);
        cudaStreamDestroy(c->out_st);
    }
    for (auto e : c->ev_written)
        if (e) cudaEventDestroy(e);
    for (auto e : c->ev_copied)
        if (e) cudaEventDestroy(e);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
}

static atmwfs_status load_common(atmwfs_ctx* c, int layer, const float* src, long M, cudaMemcpyKind kind)
{
    if (!c || !src) return fail(ATMWFS_ERR_INVALID, "null argument");
    if (layer < 0 || layer >= c->L) return fail(ATMWFS_ERR_INVALID, "layer %d out of range", layer);
    if (M != c->M) return fail(ATMWFS_ERR_INVALID, "screen size %ld differs from master_size %ld", M, c->M);
    if (c->normalized) return fail(ATMWFS_ERR_STATE, "screens already normalised");
    if (!c->d_screen[layer]) AW_TRY(dalloc(c, (void**)&c->d_screen[layer], sizeof(float) * (size_t)M * M));
    AW_CUDA(cudaMemcpyAsync(c->d_screen[layer], src, sizeof(float) * (size_t)M * M, kind, c->st));
    AW_CUDA(cudaStreamSynchronize(c->st));
    c->loaded[layer] = 1;
    c->committed = false;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    return ATMWFS_OK;
}

atmwfs_status atmwfs_load_screen(atmwfs_ctx* c, int layer, const float* host, long M)
{
    return load_common(c, layer, host, M, cudaMemcpyHostToDevice);
}

atmwfs_status atmwfs_load_screen_dev(atmwfs_ctx* c, int layer, const float* dev, long M)
{
    return load_common(c, layer, dev, M, cudaMemcpyDeviceToDevice);
}

atmwfs_status atmwfs_read_screen(atmwfs_ctx* c, int layer, float* host)
{
    if (!c || !host) return fail(ATMWFS_ERR_INVALID, "null argument");
    if (layer < 0 || layer >= c->L) return fail(ATMWFS_ERR_INVALID, "layer %d out of range", layer);
    if (!c->loaded[layer]) return fail(ATMWFS_ERR_STATE, "screen of layer %d not loaded", layer);
    AW_CUDA(cudaMemcpyAsync(host, c->d_screen[layer], sizeof(float) * (size_t)c->M * c->M, cudaMemcpyDeviceToHost,
                            c->st));
    AW_CUDA(cudaStreamSynchronize(c->st));
    return ATMWFS_OK;
}

atmwfs_status atmwfs_normalize_screens(atmwfs_ctx* c, float lambda_ref, float seeing, double* r0_pix)
{
    return atmwfs_normalize_screens_ext(c, lambda_ref, seeing, nullptr, 0, r0_pix);
}

atmwfs_status atmwfs_normalize_screens_ext(atmwfs_ctx* c, float lambda_ref, float seeing, const float* const* extra,
                                           long nextra, double* r0_pix)
{
    if (!c) return fail(ATMWFS_ERR_INVALID, "null context");
    if (nextra < 0 || (nextra > 0 && !extra)) return fail(ATMWFS_ERR_INVALID, "bad extra screens");
    for (long e = 0; e < nextra; e++)
        if (!extra[e]) return fail(ATMWFS_ERR_INVALID, "extra screen %ld is null", e);
    for (int l = 0; l < c->L; l++)
        if (!c->loaded[l]) return fail(ATMWFS_ERR_STATE, "screen of layer %d not loaded", l);
    const int dpix = 50;
    if (c->M <= dpix) return fail(ATMWFS_ERR_INVALID, "master_size must exceed 50 pixels");
    // every master screen, layers first (ID_TM[0..NBMASTERS-1], :2246-2276)
    const size_t M2 = (size_t)c->M * c->M;
    const long nm = c->L + nextra;
    std::vector<float*> scr(c->d_screen.begin(), c->d_screen.begin() + c->L);
    double* acc = nullptr;
    float* ext = nullptr;
    atmwfs_status s = ATMWFS_OK;
    if (cudaMalloc(&acc, sizeof(double) * nm) != cudaSuccess ||
        (nextra > 0 && cudaMalloc(&ext, sizeof(float) * M2 * nextra) != cudaSuccess))
        s = fail(ATMWFS_ERR_NOMEM, "cudaMalloc failed");
    for (long e = 0; e < nextra && s == ATMWFS_OK; e++) {
        scr.push_back(ext + M2 * e);
        if (cudaMemcpyAsync(ext + M2 * e, extra[e], sizeof(float) * M2, cudaMemcpyHostToDevice, c->st) != cudaSuccess)
            s = fail(ATMWFS_ERR_CUDA, "copy of extra screen %ld failed", e);
    }
    auto measure = [&](double* r0) -> atmwfs_status {
        AW_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * nm, c->st));
        for (long k = 0; k < nm; k++) AW_CUDA(lag_sumsq(scr[k], (int)c->M, dpix, acc + k, c->st));
        std::vector<double> h(nm);
        AW_CUDA(cudaMemcpyAsync(h.data(), acc, sizeof(double) * nm, cudaMemcpyDeviceToHost, c->st));
        AW_CUDA(cudaStreamSynchronize(c->st));
        const double cnt = (double)(c->M - dpix) * (double)c->M;
        double tot = 0.0;
        for (long k = 0; k < nm; k++) tot += 1.0 * dpix * pow((h[k] / cnt) / 6.88, -3.0 / 5.0);
        *r0 = tot / nm;
        return ATMWFS_OK;
    };
    double r0a = 0, r0b = 0;
    if (s == ATMWFS_OK) s = measure(&r0a);
    if (s == ATMWFS_OK) {
        // r0 target (:2278-2285): lambda / seeing[rad] / pixel scale
        const double target = lambda_ref / (seeing / 3600.0 / 180.0 * kPi) / c->pupil * 1;
        const double tmp1 = pow(r0a / target, 5.0 / 6.0);
        for (long k = 0; k < nm && s == ATMWFS_OK; k++)
            if (scale_screen(scr[k], c->M * c->M, tmp1, c->st) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "scale failed");
        if (s == ATMWFS_OK) s = measure(&r0b);
        // per-layer weight sqrt(Cn2 / cos(zenith)) (:2340-2363)
        for (int l = 0; l < c->L && s == ATMWFS_OK; l++)
            if (scale_screen(c->d_screen[l], c->M * c->M, sqrt(c->cn2[l] / cos((double)c->zangle)), c->st) != cudaSuccess)
                s = fail(ATMWFS_ERR_CUDA, "scale failed");
    }
    cudaStreamSynchronize(c->st);
    cudaFree(acc);
    if (ext) cudaFree(ext);
    if (s != ATMWFS_OK) return s;
    if (r0_pix) { r0_pix[0] = r0a; r0_pix[1] = r0b; }
    c->normalized = true;
    c->committed = false;
    return ATMWFS_OK;
}

atmwfs_status atmwfs_run(atmwfs_ctx* c, long nsteps, const atmwfs_sink* sink)
{
    if (!c) return fail(ATMWFS_ERR_INVALID, "null context");
    if (nsteps < 0) return fail(ATMWFS_ERR_INVALID, "nsteps < 0");
    AW_TRY(commit(c));
    const size_t per = (size_t)c->ninst * c->L;
    const bool copies = sink && (sink->pha || sink->amp);
    if (copies && !c->out_st) {
        // the copy stream has the highest priority: its few CTAs take the
        // next free SM slots ahead of the queued pass and phase-sum CTAs, so a
        // step's frames leave while the next step computes
        int lo = 0, hi = 0;
        AW_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        AW_CUDA(cudaStreamCreateWithPriority(&c->out_st, cudaStreamNonBlocking, hi));
        c->ev_written.assign(c->ring, nullptr);
        c->ev_copied.assign(c->ring, nullptr);
        for (long r = 0; r < c->ring; r++) {
            AW_CUDA(cudaEventCreateWithFlags(&c->ev_written[r], cudaEventDisableTiming));
            AW_CUDA(cudaEventCreateWithFlags(&c->ev_copied[r], cudaEventDisableTiming));
        }
    }
    // copy kernel when the sink is pinned host or device memory on 16-byte
    // boundaries (frames are a multiple of four floats); else the copy engine
    bool by_kernel = copies && c->frame_floats % 4 == 0;
    float* dev_sink[2] = {nullptr, nullptr};  // the sink as the device addresses it
    for (int o = 0; o < 2 && by_kernel; o++) {
        float* p = o == 0 ? sink->pha : sink->amp;
        if (!p) continue;
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
            cudaGetLastError();
            by_kernel = false;
            continue;
        }
        const bool reachable = pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeHost ||
                               pa.type == cudaMemoryTypeManaged;
        dev_sink[o] = static_cast<float*>(pa.devicePointer);
        if (!reachable || !dev_sink[o] || (reinterpret_cast<uintptr_t>(dev_sink[o]) & 15) != 0) by_kernel = false;
    }
    long s = 0;
    int b = 0;
    while (s < nsteps) {
        const long g0 = c->steps;
        long chunk = nsteps - s;
        if (chunk > c->poscap) chunk = c->poscap;
        AW_CUDA(cudaEventSynchronize(c->ev[b]));
        for (long i = 0; i < chunk; i++) {
            double tnow = 0.0;
            if (c->realtime) {
                struct timespec ts;
                clock_gettime(CLOCK_REALTIME, &ts);
                tnow = (1.0 * ts.tv_sec + 1.0e-9 * ts.tv_nsec) * c->rtfactor;
            }
            advance_positions(c, tnow, c->h_pos[b] + (size_t)i * per);
            c->steps++;
        }
        // upload into ring slots g0 .. g0 + chunk - 1 (mod poscap)
        const long s0 = g0 % c->poscap;
        const long n1 = chunk < c->poscap - s0 ? chunk : c->poscap - s0;
        AW_CUDA(cudaMemcpyAsync(c->d_pos + s0 * per, c->h_pos[b], sizeof(LayerPos) * per * n1, cudaMemcpyHostToDevice, c->st));
        if (chunk > n1)
            AW_CUDA(cudaMemcpyAsync(c->d_pos, c->h_pos[b] + n1 * per, sizeof(LayerPos) * per * (chunk - n1),
                                    cudaMemcpyHostToDevice, c->st));
        AW_CUDA(cudaEventRecord(c->ev[b], c->st));
        for (long i = 0; i < chunk; i++) {
            const long slot = (g0 + i) % c->ring;
            // the slot is free once its previous copy is done (a no-op for a
            // slot never copied); with ring >= 2 this copy overlaps the next step
            if (copies) AW_CUDA(cudaStreamWaitEvent(c->st, c->ev_copied[slot], 0));
            AW_CUDA(cudaGraphLaunch(c->gexec, c->st));
            if (copies) {
                AW_CUDA(cudaEventRecord(c->ev_written[slot], c->st));
                AW_CUDA(cudaStreamWaitEvent(c->out_st, c->ev_written[slot], 0));
                const long hs = sink->nslots > 0 ? (s + i) % sink->nslots : (s + i);
                const size_t ff = c->frame_floats;
                if (by_kernel) {
                    auto f4 = [](const float* q) { return reinterpret_cast<const float4*>(q); };
                    auto h4 = [&](float* q) { return q ? reinterpret_cast<float4*>(q + (size_t)hs * ff) : nullptr; };
                    AW_CUDA(copy_out(f4(c->d_out_pha + slot * ff), h4(dev_sink[0]), (long)(ff / 4),
                                     f4(c->d_out_amp + slot * ff), h4(dev_sink[1]), (long)(ff / 4), c->out_st));
                } else {
                    if (sink->pha)
                        AW_CUDA(cudaMemcpyAsync(sink->pha + (size_t)hs * ff, c->d_out_pha + slot * ff, sizeof(float) * ff,
                                                cudaMemcpyDefault, c->out_st));
                    if (sink->amp)
                        AW_CUDA(cudaMemcpyAsync(sink->amp + (size_t)hs * ff, c->d_out_amp + slot * ff, sizeof(float) * ff,
                                                cudaMemcpyDefault, c->out_st));
                }
                AW_CUDA(cudaEventRecord(c->ev_copied[slot], c->out_st));
            }
        }
        s += chunk;
        b ^= 1;
    }
    // the caller's buffers hold every frame on return
    if (copies) AW_CUDA(cudaStreamSynchronize(c->out_st));
    return check_status(c);
}

atmwfs_status atmwfs_advance(atmwfs_ctx* c, long nsteps)
{
    if (!c) return fail(ATMWFS_ERR_INVALID, "null context");
    if (nsteps < 0) return fail(ATMWFS_ERR_INVALID, "nsteps < 0");
    AW_TRY(commit(c));
    const size_t per = (size_t)c->ninst * c->L;
    for (long s = 0; s < nsteps; s++) {
        // one step at a time: the host slot is reused once its copy is done
        AW_CUDA(cudaEventSynchronize(c->ev[0]));
        double tnow = 0.0;
        if (c->realtime) {
            struct timespec ts;
            clock_gettime(CLOCK_REALTIME, &ts);
            tnow = (1.0 * ts.tv_sec + 1.0e-9 * ts.tv_nsec) * c->rtfactor;
        }
        const long g = c->steps;
        advance_positions(c, tnow, c->h_pos[0]);
        c->steps++;
        AW_CUDA(cudaMemcpyAsync(c->d_pos + (g % c->poscap) * per, c->h_pos[0], sizeof(LayerPos) * per,
                                cudaMemcpyHostToDevice, c->st));
        AW_CUDA(cudaEventRecord(c->ev[0], c->st));
        AW_CUDA(step_advance(c->d_step, c->st));
    }
    AW_CUDA(cudaStreamSynchronize(c->st));
    return ATMWFS_OK;
}

atmwfs_status atmwfs_windows_dev(atmwfs_ctx* c, int i, float* out, void* stream)
{
    if (!c || !out || i < 0 || i >= c->ninst) return fail(ATMWFS_ERR_INVALID, "bad instance or buffer");
    if (c->steps == 0) return fail(ATMWFS_ERR_STATE, "no step computed yet");
    std::vector<float> sc(c->L);
    for (int l = 0; l < c->L; l++) sc[l] = c->scoeff[i][l];
    AW_CUDA(windows(c->d_screen.data(), sc.data(), c->L, (int)c->M, c->d_pos, c->poscap, c->ninst, i, c->d_step,
                    (int)c->inst[i].wf_raw_size, out, stream ? (cudaStream_t)stream : c->st));
    return ATMWFS_OK;
}

atmwfs_status atmwfs_frame_dev(atmwfs_ctx* c, int i, const float** pha, const float** amp)
{
    if (!c || i < 0 || i >= c->ninst) return fail(ATMWFS_ERR_INVALID, "bad instance");
    if (c->steps == 0) return fail(ATMWFS_ERR_STATE, "no frame computed yet");
    const long slot = (c->steps - 1) % c->ring;
    if (pha) *pha = c->d_out_pha + slot * c->frame_floats + c->frame_off[i];
    if (amp) *amp = c->d_out_amp + slot * c->frame_floats + c->frame_off[i];
    return ATMWFS_OK;
}

atmwfs_status atmwfs_layer_planes(const double* alt, const double* cn2, int L, double fresnel_bin, int amplitude,
                                  int fresnel, float zangle, int* nsuper, double* salt, int* sidx, int* nplanes,
                                  int* plane_lo, int* plane_hi, double* hop_z)
{
    if (!alt || !cn2 || L < 1) return fail(ATMWFS_ERR_INVALID, "bad profile");
    std::vector<double> a(alt, alt + L), c2(cn2, cn2 + L), sa;
    double tot = 0.0;
    for (double v : c2) tot += v;
    if (!(tot > 0)) return fail(ATMWFS_ERR_INVALID, "sum of cn2 must be > 0");
    for (double& v : c2) v *= 1.0 / tot;
    std::vector<int> si, lo, hi;
    std::vector<double> hz;
    const int S = group_superlayers(a, c2, fresnel_bin, sa, si);
    build_planes(sa, si, amplitude, amplitude ? fresnel : 0, zangle, lo, hi, hz);
    if (nsuper) *nsuper = S;
    for (int i = 0; i < S && salt; i++) salt[i] = sa[i];
    for (int l = 0; l < L && sidx; l++) sidx[l] = si[l];
    if (nplanes) *nplanes = (int)lo.size();
    for (size_t k = 0; k < lo.size(); k++) {
        if (plane_lo) plane_lo[k] = lo[k];
        if (plane_hi) plane_hi[k] = hi[k];
        if (hop_z && k < hz.size()) hop_z[k] = hz[k];
    }
    return ATMWFS_OK;
}

atmwfs_status atmwfs_class_info(const atmwfs_ctx* c, int ci, int* n, int* nout, int* count, int* rows_per_cta,
                                double* tuned_ms)
{
    if (!c || ci < 0 || ci >= (int)c->classes.size()) return fail(ATMWFS_ERR_INVALID, "bad class");
    const Class& cl = c->classes[ci];
    if (n) *n = cl.N;
    if (nout) *nout = cl.Nout;
    if (count) *count = (int)cl.members.size();
    if (rows_per_cta) *rows_per_cta = cl.RR;
    for (int g = 0; g < kNumTileCfg && tuned_ms; g++) tuned_ms[g] = cl.tuned_ms[g];
    return ATMWFS_OK;
}

atmwfs_status atmwfs_class_plan(const atmwfs_ctx* c, int ci, int* cfg, int* radices)
{
    if (!c || ci < 0 || ci >= (int)c->classes.size()) return fail(ATMWFS_ERR_INVALID, "bad class");
    const Class& cl = c->classes[ci];
    if (cfg) *cfg = cl.cfg;
    if (radices) {
        const int V = tile_cfg(cl.N, cl.cfg).plan;
        int r[3] = {0, 0, 0};
        switch (cl.N * 4 + V) {
#define AW_PLAN(NN, VV)                                                                      \
    case NN * 4 + VV:                                                                        \
        r[0] = Stages<NN, VV>::R0;                                                           \
        r[1] = Stages<NN, VV>::R1;                                                           \
        r[2] = Stages<NN, VV>::R2;                                                           \
        break;
            AW_PLAN(64, 0)
            AW_PLAN(128, 0)
            AW_PLAN(256, 0)
            AW_PLAN(512, 0)
            AW_PLAN(1024, 0)
            AW_PLAN(1024, 1)
            AW_PLAN(2048, 0)
#undef AW_PLAN
            default: break;
        }
        for (int i = 0; i < 3; i++) radices[i] = r[i];
    }
    return ATMWFS_OK;
}

void* atmwfs_stream(atmwfs_ctx* c) { return c ? (void*)c->st : nullptr; }

int atmwfs_step_kernels(const atmwfs_ctx* c) { return c ? c->step_kernels : 0; }

int atmwfs_num_classes(const atmwfs_ctx* c) { return c ? (int)c->classes.size() : 0; }

atmwfs_status atmwfs_time_pass(atmwfs_ctx* c, int k, int ci, int reps, double* ms, double* bytes, int* n, int* count)
{
    if (!c || ci < 0 || ci >= (int)c->classes.size()) return fail(ATMWFS_ERR_INVALID, "bad class");
    if (k < 0 || k > (int)c->plane_lo.size() + 2 || reps < 1) return fail(ATMWFS_ERR_INVALID, "bad pass");
    AW_TRY(commit(c));
    Class& cl = c->classes[ci];
    cudaEvent_t e0, e1;
    AW_CUDA(cudaEventCreate(&e0));
    AW_CUDA(cudaEventCreate(&e1));
    double b = 0;
    atmwfs_status s = launch_pass(c, k, cl, &b, c->st);  // warm-up
    if (s == ATMWFS_OK) {
        cudaEventRecord(e0, c->st);
        for (int r = 0; r < reps && s == ATMWFS_OK; r++) s = launch_pass(c, k, cl, nullptr, c->st);
        cudaEventRecord(e1, c->st);
    }
    float t = 0;
    if (s == ATMWFS_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != ATMWFS_OK) return s;
    if (k == (int)c->plane_lo.size() || k == (int)c->plane_lo.size() + 2)
        AW_TRY(clear_bins(c));  // the last pass accumulated science bins, the unwrap read them
    if (ms) *ms = t / reps;
    if (bytes) *bytes = b;
    if (n) *n = cl.N;
    if (count) *count = (int)cl.members.size();
    return check_status(c);
}

size_t atmwfs_frame_offset(const atmwfs_ctx* c, int i) { return (c && i >= 0 && i < c->ninst) ? c->frame_off[i] : 0; }
size_t atmwfs_frame_floats(const atmwfs_ctx* c) { return c ? c->frame_floats : 0; }

long atmwfs_steps_done(const atmwfs_ctx* c) { return c ? c->steps : -1; }

int atmwfs_num_planes(const atmwfs_ctx* c) { return c ? (int)c->plane_lo.size() : 0; }

atmwfs_status atmwfs_plane_info(const atmwfs_ctx* c, int* lo, int* hi, double* z)
{
    if (!c) return fail(ATMWFS_ERR_INVALID, "null context");
    for (size_t k = 0; k < c->plane_lo.size(); k++) {
        if (lo) lo[k] = c->plane_lo[k];
        if (hi) hi[k] = c->plane_hi[k];
        if (z && k < c->hop_z.size()) z[k] = c->hop_z[k];
    }
    return ATMWFS_OK;
}

atmwfs_status atmwfs_positions(const atmwfs_ctx* c, int i, double* x, double* y)
{
    if (!c || i < 0 || i >= c->ninst) return fail(ATMWFS_ERR_INVALID, "bad instance");
    for (int l = 0; l < c->L; l++) {
        if (x) x[l] = c->xpos[(size_t)i * c->L + l];
        if (y) y[l] = c->ypos[(size_t)i * c->L + l];
    }
    return ATMWFS_OK;
}

int atmwfs_last_iters(atmwfs_ctx* c, int i)
{
    if (!c || i < 0 || i >= c->ninst || !c->d_iters) return -1;
    int v = -1;
    cudaMemcpy(&v, c->d_iters + c->slot_of[i], sizeof(int), cudaMemcpyDeviceToHost);
    return v;
}

// ---------------------------------------------------------------------------
// unit operators
// ---------------------------------------------------------------------------
static atmwfs_status two_pass(const void* in, void* out, long n, int var, const float2* H, cudaStream_t st)
{
    const PassLauncher fn = pass_launcher((int)n);
    if (!fn) return fail(ATMWFS_ERR_INVALID, "size %ld unsupported (power of two 64..2048)", n);
    const float2* tw = twiddles((int)n);
    if (!tw) return fail(ATMWFS_ERR_NOMEM, "twiddle allocation failed");
    float2* tmp = nullptr;
    AW_CUDA(cudaMallocAsync((void**)&tmp, sizeof(float2) * n * n, st));
    const int RR = rows_per_cta((int)n);
    PassArgs a;
    memset(&a, 0, sizeof a);
    a.H1 = H;
    a.H2 = H;
    a.ext_in = (const float2*)in;
    a.ext_out = tmp;
    cudaError_t e = fn(var, dim3((unsigned)(n / RR), 1), a, nullptr, tw, st);
    if (e == cudaSuccess) {
        a.ext_in = tmp;
        a.ext_out = (float2*)out;
        e = fn(var, dim3((unsigned)(n / RR), 1), a, nullptr, tw, st);
    }
    cudaFreeAsync(tmp, st);
    AW_CUDA(e);
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fresnel_dev(const void* in, void* out, long n, double dx, double z, double lambda, void* stream)
{
    if (!in || !out) return fail(ATMWFS_ERR_INVALID, "null buffer");
    if (!pow2_in(n, 64, 2048)) return fail(ATMWFS_ERR_INVALID, "size %ld unsupported (power of two 64..2048)", n);
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float2> h(n);
    transfer_table(h.data(), (int)n, dx, z, lambda);
    float2* dh = nullptr;
    AW_CUDA(cudaMallocAsync((void**)&dh, sizeof(float2) * n, st));
    cudaError_t e = cudaMemcpyAsync(dh, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, st);
    atmwfs_status s = e == cudaSuccess ? two_pass(in, out, n, kVarUnitProp, dh, st)
                                       : fail(ATMWFS_ERR_CUDA, "copy failed: %s", cudaGetErrorString(e));
    cudaFreeAsync(dh, st);
    // the host table must outlive the asynchronous copy
    cudaStreamSynchronize(st);
    return s;
}

atmwfs_status atmwfs_fft2d_dev(const void* in, void* out, long n, int sign, void* stream)
{
    if (!in || !out) return fail(ATMWFS_ERR_INVALID, "null buffer");
    if (sign != -1 && sign != 1) return fail(ATMWFS_ERR_INVALID, "sign must be -1 or +1");
    if (fft2d_large_supported(n)) {
        cudaStream_t st = (cudaStream_t)stream;
        float2* tmp = nullptr;
        AW_CUDA(cudaMallocAsync((void**)&tmp, sizeof(float2) * n * n, st));
        const cudaError_t e = fft2d_large((const float2*)in, (float2*)out, tmp, (int)n, sign, st);
        cudaFreeAsync(tmp, st);
        AW_CUDA(e);
        return ATMWFS_OK;
    }
    return two_pass(in, out, n, sign < 0 ? kVarUnitFwd : kVarUnitInv, nullptr, (cudaStream_t)stream);
}

static atmwfs_status fft_thunk(const void* in, void* out, long n, void* st, const void* arg);

static atmwfs_status host_unit(const float* in, float* out, long n,
                               atmwfs_status (*fn)(const void*, void*, long, void*, const void*), const void* arg)
{
    if (!in || !out) return fail(ATMWFS_ERR_INVALID, "null buffer");
    const bool big = fn == fft_thunk && fft2d_large_supported(n);
    if (!pow2_in(n, 64, 2048) && !big)
        return fail(ATMWFS_ERR_INVALID, "size %ld unsupported (power of two 64..2048%s)", n,
                    fn == fft_thunk ? ", 4096 or 8192" : "");
    const size_t bytes = sizeof(float2) * n * n;
    void *din = nullptr, *dout = nullptr;
    AW_CUDA(cudaMalloc(&din, bytes));
    if (cudaMalloc(&dout, bytes) != cudaSuccess) {
        cudaFree(din);
        return fail(ATMWFS_ERR_NOMEM, "cudaMalloc failed");
    }
    atmwfs_status s = ATMWFS_OK;
    if (cudaMemcpy(din, in, bytes, cudaMemcpyHostToDevice) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "H2D failed");
    if (s == ATMWFS_OK) s = fn(din, dout, n, nullptr, arg);
    if (s == ATMWFS_OK && cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "D2H failed");
    cudaFree(din);
    cudaFree(dout);
    return s;
}

struct FresnelArg { double dx, z, lambda; };

static atmwfs_status fresnel_thunk(const void* in, void* out, long n, void* st, const void* arg)
{
    const FresnelArg* f = (const FresnelArg*)arg;
    return atmwfs_fresnel_dev(in, out, n, f->dx, f->z, f->lambda, st);
}

static atmwfs_status fft_thunk(const void* in, void* out, long n, void* st, const void* arg)
{
    atmwfs_status s = atmwfs_fft2d_dev(in, out, n, *(const int*)arg, st);
    if (s == ATMWFS_OK && cudaStreamSynchronize((cudaStream_t)st) != cudaSuccess) return fail(ATMWFS_ERR_CUDA, "sync failed");
    return s;
}

atmwfs_status atmwfs_fresnel(const float* in, float* out, long n, double dx, double z, double lambda)
{
    FresnelArg f = {dx, z, lambda};
    return host_unit(in, out, n, fresnel_thunk, &f);
}

atmwfs_status atmwfs_fft2d(const float* in, float* out, long n, int sign)
{
    if (sign != -1 && sign != 1) return fail(ATMWFS_ERR_INVALID, "sign must be -1 or +1");
    return host_unit(in, out, n, fft_thunk, &sign);
}

atmwfs_status atmwfs_master_screen(uint64_t seed, uint32_t stream, long M, double outer_pix, double inner_pix,
                                   float* out1, float* out2, double* cfit)
{
    if (!pow2_in(M, 64, 8192)) return fail(ATMWFS_ERR_INVALID, "M=%ld unsupported (power of two 64..8192)", M);
    if (!(outer_pix > 0) || !(inner_pix > 0)) return fail(ATMWFS_ERR_INVALID, "scales must be > 0");
    const size_t n = (size_t)M * M;
    float2 *C = nullptr, *F = nullptr;
    double* acc = nullptr;
    float *o1 = nullptr, *o2 = nullptr;
    atmwfs_status s = ATMWFS_OK;
    cudaStream_t st = nullptr;
    if (cudaMalloc(&C, n * sizeof(float2)) != cudaSuccess || cudaMalloc(&F, n * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&acc, 8 * sizeof(double)) != cudaSuccess || cudaMalloc(&o1, n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&o2, n * sizeof(float)) != cudaSuccess) {
        s = fail(ATMWFS_ERR_NOMEM, "cudaMalloc failed");
    }
    // f0 = M / L0pix, fi = (5.92 / 2 pi) M / l0pix (:679-680)
    const double fo = 1.0 * M / outer_pix;
    const double fi = (5.92 / (2.0 * kPi)) * M / inner_pix;
    double C12[2] = {0, 0};
    if (s == ATMWFS_OK && screen_spectrum(seed, stream, (int)M, fo, fi, C, st) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "spectrum kernel failed");
    if (s == ATMWFS_OK) s = atmwfs_fft2d_dev(C, F, M, -1, st);
    if (s == ATMWFS_OK && cudaMemset(acc, 0, 8 * sizeof(double)) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "memset failed");
    if (s == ATMWFS_OK && strf_lags(F, (int)M, acc, st) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "strf kernel failed");
    double h[8];
    if (s == ATMWFS_OK && cudaMemcpy(h, acc, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "D2H failed");
    if (s == ATMWFS_OK) {
        // C = 10^(mean over lags (1..2)^2 of log10 D - 5/3 log10 r)  (:795-816)
        for (int part = 0; part < 2; part++) {
            double v = 0.0;
            for (int q = 0; q < 4; q++) {
                const int lx = 1 + (q & 1), ly = 1 + (q >> 1);
                const double D = h[part * 4 + q] / (double)n;
                v += log10(D) - 5.0 / 3.0 * log10(sqrt((double)(lx * lx + ly * ly)));
            }
            C12[part] = pow(10.0, v / 4.0);
        }
        if (split_scale(F, (long)n, 1.0 / sqrt(C12[0]), 1.0 / sqrt(C12[1]), o1, o2, st) != cudaSuccess)
            s = fail(ATMWFS_ERR_CUDA, "scale kernel failed");
    }
    if (s == ATMWFS_OK && out1 && cudaMemcpy(out1, o1, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "D2H failed");
    if (s == ATMWFS_OK && out2 && cudaMemcpy(out2, o2, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) s = fail(ATMWFS_ERR_CUDA, "D2H failed");
    if (s == ATMWFS_OK && cfit) { cfit[0] = C12[0]; cfit[1] = C12[1]; }
    cudaFree(C); cudaFree(F); cudaFree(acc); cudaFree(o1); cudaFree(o2);
    return s;
}

}  // extern "C"
