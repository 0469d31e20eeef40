// refract.cu -- atmospheric refraction by ray tracing
// (AtmosphereModel_RefractionPath, src/AtmosphereModel/AtmosphereModel.c:4215-4291).
//
// A ray leaves the site at zenith angle alpha and advances in 20 m steps
// over a spherical Earth; at each step the local zenith angle follows
// Snell's law between the refractive indices of consecutive points, and the
// flux is attenuated by the local absorption.  The launch angle is iterated
// until the exit angle at 99 km equals the requested zenith angle; the
// refraction is the difference of the two.
//
// atmwfs_refraction_path is the host form with model callbacks (a drop-in
// for the reference's call); atmwfs_refraction_table runs one ray per GPU
// thread in FP64 for every (wavelength, zenith angle) pair of a table
// model.  The path geometry needs FP64: the altitude is the difference of
// two numbers near the Earth radius.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "atmwfs.h"
#include "atmwfs_mkwfs.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

constexpr double kLstep = 20.0;          // beam distance step [m]
constexpr double kRe = 6371000.0;        // Earth radius [m]
constexpr double kHtop = 99000.0;        // exit altitude [m]
constexpr int kMaxIter = 20;
constexpr double kTolArcsec = 0.00001;
constexpr long kMaxSteps = 1000000;      // per pass: a ray that never climbs is an error
constexpr double kPi = 3.14159265358979323846264338328;

// The reference's table read (stdAtmModel_N, AtmosphereModel.c:3240-3250):
// index (long)(alt / dh) capped at ntab - 2, float fraction clamped to [0, 1].
__host__ __device__ inline void table_pos(float alt, double dh, long ntab, long& i, float& f)
{
    i = (long)(alt / dh);
    if (i > ntab - 3) i = ntab - 2;
    if (i < 0) i = 0;
    f = (float)(1.0 * alt / dh - i);
    if (f < 0) f = 0.0f;
    if (f > 1.0f) f = 1.0f;
}

struct Ray {
    double refraction_arcsec, transmission;
    int ok;
};

// The caller's model callbacks (host only).
struct CallbackModel {
    atmwfs_refractivity_fn N;
    atmwfs_absorption_fn K;
    void* user;
    __host__ __device__ float n(float alt, float lam) const
    {
#ifdef __CUDA_ARCH__
        return 0.0f;
#else
        return N(alt, lam, user);
#endif
    }
    __host__ __device__ double k(float alt, float lam) const
    {
#ifdef __CUDA_ARCH__
        return 0.0;
#else
        return K ? K(alt, lam, user) : 0.0;
#endif
    }
};

// A table model of one wavelength (nodes k * dh).
struct TableModel {
    const float* N;
    const double* K;
    long ntab;
    double dh;
    __host__ __device__ float n(float alt, float) const
    {
        long i;
        float f;
        table_pos(alt, dh, ntab, i, f);
        return (float)((1.0 - f) * N[i] + f * N[i + 1]);
    }
    __host__ __device__ double k(float alt, float) const
    {
        if (!K) return 0.0;
        long i;
        float f;
        table_pos(alt, dh, ntab, i, f);
        return (1.0 - f) * K[i] + f * K[i + 1];
    }
};

// One ray; m.n(h, lambda) = N as float, m.k(h, lambda) = absorption
// coefficient.  The arithmetic is the reference's, statement by statement.
template <class Model>
__host__ __device__ Ray trace(double lambda, double Zangle, double site, const Model& m, FILE* path)
{
    double Zangle0 = Zangle, offsetangle = 0.0, errV = 100000.0, flux = 1.0, alpha = Zangle0;
    int iter = 0;
    Ray r{0.0, 1.0, 1};
    while (iter < kMaxIter && errV > kTolArcsec) {
        double x0 = 0.0, y0 = 0.0, h1 = 0.0;
        alpha = Zangle0;
        double n0 = 1.0 + m.n((float)site, (float)lambda);
        flux = 1.0;
        long steps = 0;
        while (h1 < kHtop) {
            if (++steps > kMaxSteps) {
                r.ok = 0;
                return r;
            }
            const double x1 = x0 + kLstep * sin(alpha);
            const double y1 = y0 + kLstep * cos(alpha);
            h1 = sqrt(x1 * x1 + (y1 + site + kRe) * (y1 + site + kRe)) - kRe;
            const double n1 = 1.0 + m.n((float)h1, (float)lambda);
            const double alphae = atan2(x1, y1 + site + kRe);
            flux *= exp(-kLstep * m.k((float)h1, (float)lambda));
            const double alpha0 = alpha - alphae;
            const double alpha1 = asin(n0 * sin(alpha0) / n1);
            alpha = alpha1 + alphae;
            n0 = n1;
            x0 = x1;
            y0 = y1;
#ifndef __CUDA_ARCH__
            if (path)
                fprintf(path, "%10.3f %10.3f %10.3f  %12.9f  %20g    %20g   %20g\n", h1, x0, y0, alpha, alpha - Zangle,
                        (alpha - Zangle) / kPi * 180.0 * 3600.0, y0 * tan(Zangle) - x0);
#endif
        }
        offsetangle = alpha - Zangle;
        Zangle0 -= offsetangle;
        errV = fabs(offsetangle / kPi * 180.0 * 3600.0);
        iter++;
#ifndef __CUDA_ARCH__
        if (path && iter < kMaxIter && errV > kTolArcsec) {   // only the last pass stays in the file
            fflush(path);
            if (freopen(nullptr, "w", path) == nullptr) path = nullptr;
        }
#endif
    }
    r.refraction_arcsec = (Zangle - Zangle0) / kPi * 180.0 * 3600.0;
    r.transmission = flux;
    return r;
}

__global__ void k_refraction(const double* __restrict__ lambdas, int nl, const double* __restrict__ zangles, int nz,
                             double site, const float* __restrict__ Ntab, const double* __restrict__ Ktab, long ntab,
                             double dh, double* __restrict__ refr, double* __restrict__ trans, int* __restrict__ bad)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl * nz) return;
    const int li = t / nz, zi = t % nz;
    const TableModel m{Ntab + (size_t)li * ntab, Ktab ? Ktab + (size_t)li * ntab : nullptr, ntab, dh};
    const Ray r = trace(lambdas[li], zangles[zi], site, m, nullptr);
    refr[t] = r.refraction_arcsec;
    trans[t] = r.transmission;
    if (!r.ok) atomicExch(bad, 1);
}

atmwfs_status fail(atmwfs_status s, const char* msg)
{
    atmwfs::set_error_message(msg);
    return s;
}

}  // namespace

extern "C" {

atmwfs_status atmwfs_refraction_path(double lambda, double zangle, double site_alt, atmwfs_refractivity_fn N,
                                     atmwfs_absorption_fn K, void* user, const char* path_file,
                                     double* refraction_arcsec, double* transmission)
{
    if (!N) return fail(ATMWFS_ERR_INVALID, "refraction_path: no refractivity model");
    if (!(zangle >= 0.0 && zangle < 0.5 * kPi)) return fail(ATMWFS_ERR_INVALID, "refraction_path: zenith angle out of [0, pi/2)");
    FILE* fp = nullptr;
    if (path_file && !(fp = fopen(path_file, "w"))) return fail(ATMWFS_ERR_IO, "refraction_path: cannot write the path file");
    const CallbackModel m{N, K, user};
    const Ray r = trace(lambda, zangle, site_alt, m, fp);
    if (fp) fclose(fp);
    if (!r.ok) return fail(ATMWFS_ERR_INVALID, "refraction_path: the ray does not reach 99 km");
    if (refraction_arcsec) *refraction_arcsec = r.refraction_arcsec;
    if (transmission) *transmission = r.transmission;
    return ATMWFS_OK;
}

atmwfs_status atmwfs_refraction_table(const double* lambdas, long nlambda, const double* zangles, long nzangle,
                                      double site_alt, const float* Ntab, const double* Ktab, long ntab, double dh,
                                      double* refraction_arcsec, double* transmission)
{
    if (!lambdas || !zangles || !Ntab || !refraction_arcsec || nlambda < 1 || nzangle < 1 || ntab < 3 || !(dh > 0))
        return fail(ATMWFS_ERR_INVALID, "refraction_table: bad arguments");
    if (nlambda * nzangle > (1L << 24)) return fail(ATMWFS_ERR_INVALID, "refraction_table: too many rays");
    for (long z = 0; z < nzangle; z++)
        if (!(zangles[z] >= 0.0 && zangles[z] < 0.5 * kPi))
            return fail(ATMWFS_ERR_INVALID, "refraction_table: zenith angle out of [0, pi/2)");
    const long nr = nlambda * nzangle;
    double *dl = nullptr, *dz = nullptr, *dK = nullptr, *dr = nullptr, *dt = nullptr;
    float* dN = nullptr;
    int* dbad = nullptr;
    std::vector<double> tr(nr);
    auto cleanup = [&]() {
        cudaFree(dl); cudaFree(dz); cudaFree(dN); cudaFree(dK); cudaFree(dr); cudaFree(dt); cudaFree(dbad);
    };
    auto cu = [&](cudaError_t e) -> bool { return e == cudaSuccess; };
    bool ok = cu(cudaMalloc(&dl, sizeof(double) * nlambda)) && cu(cudaMalloc(&dz, sizeof(double) * nzangle)) &&
              cu(cudaMalloc(&dN, sizeof(float) * nlambda * ntab)) && cu(cudaMalloc(&dr, sizeof(double) * nr)) &&
              cu(cudaMalloc(&dt, sizeof(double) * nr)) && cu(cudaMalloc(&dbad, sizeof(int))) &&
              (!Ktab || cu(cudaMalloc(&dK, sizeof(double) * nlambda * ntab)));
    if (!ok) {
        cleanup();
        return fail(ATMWFS_ERR_NOMEM, "refraction_table: device allocation failed");
    }
    int bad = 0;
    ok = cu(cudaMemcpy(dl, lambdas, sizeof(double) * nlambda, cudaMemcpyHostToDevice)) &&
         cu(cudaMemcpy(dz, zangles, sizeof(double) * nzangle, cudaMemcpyHostToDevice)) &&
         cu(cudaMemcpy(dN, Ntab, sizeof(float) * nlambda * ntab, cudaMemcpyHostToDevice)) &&
         (!Ktab || cu(cudaMemcpy(dK, Ktab, sizeof(double) * nlambda * ntab, cudaMemcpyHostToDevice))) &&
         cu(cudaMemset(dbad, 0, sizeof(int)));
    if (ok) {
        // one warp per block: FP64 throughput per SM is low on this part, so
        // the rays are spread over as many SMs as there are warps of rays
        k_refraction<<<(unsigned)((nr + 31) / 32), 32>>>(dl, (int)nlambda, dz, (int)nzangle, site_alt, dN, dK, ntab, dh,
                                                           dr, dt, dbad);
        ok = cu(cudaGetLastError()) &&
             cu(cudaMemcpy(refraction_arcsec, dr, sizeof(double) * nr, cudaMemcpyDeviceToHost)) &&
             cu(cudaMemcpy(tr.data(), dt, sizeof(double) * nr, cudaMemcpyDeviceToHost)) &&
             cu(cudaMemcpy(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost));
    }
    cleanup();
    if (!ok) return fail(ATMWFS_ERR_CUDA, "refraction_table: CUDA call failed");
    if (bad) return fail(ATMWFS_ERR_INVALID, "refraction_table: a ray does not reach 99 km");
    if (transmission)
        for (long i = 0; i < nr; i++) transmission[i] = tr[i];
    return ATMWFS_OK;
}

atmwfs_status atmwfs_refraction_table_host(const double* lambdas, long nlambda, const double* zangles, long nzangle,
                                           double site_alt, const float* Ntab, const double* Ktab, long ntab, double dh,
                                           int threads, double* refraction_arcsec, double* transmission)
{
    if (!lambdas || !zangles || !Ntab || !refraction_arcsec || nlambda < 1 || nzangle < 1 || ntab < 3 || !(dh > 0))
        return fail(ATMWFS_ERR_INVALID, "refraction_table_host: bad arguments");
    for (long z = 0; z < nzangle; z++)
        if (!(zangles[z] >= 0.0 && zangles[z] < 0.5 * kPi))
            return fail(ATMWFS_ERR_INVALID, "refraction_table_host: zenith angle out of [0, pi/2)");
    const long nr = nlambda * nzangle;
    const int nt = std::max(1, std::min<int>(threads > 0 ? threads : (int)std::thread::hardware_concurrency(), (int)nr));
    std::atomic<long> next(0);
    std::atomic<int> bad(0);
    auto work = [&]() {
        for (long t; (t = next.fetch_add(1)) < nr;) {
            const long li = t / nzangle, zi = t % nzangle;
            const TableModel m{Ntab + (size_t)li * ntab, Ktab ? Ktab + (size_t)li * ntab : nullptr, ntab, dh};
            const Ray r = trace(lambdas[li], zangles[zi], site_alt, m, nullptr);
            refraction_arcsec[t] = r.refraction_arcsec;
            if (transmission) transmission[t] = r.transmission;
            if (!r.ok) bad = 1;
        }
    };
    std::vector<std::thread> pool;
    for (int i = 1; i < nt; i++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    if (bad) return fail(ATMWFS_ERR_INVALID, "refraction_table_host: a ray does not reach 99 km");
    return ATMWFS_OK;
}

}  // extern "C"
