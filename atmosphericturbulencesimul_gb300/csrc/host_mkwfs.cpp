// host_mkwfs.cpp -- the series command on top of the GPU engine: the
// reference's make_AtmosphericTurbulence_wavefront_series()
// (src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433-4455) as a host
// driver that reads the same files, feeds atmwfs_run() and writes the same
// FITS cubes and shared-memory streams.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "atmwfs.h"
#include "atmwfs_fno.h"
#include "atmwfs_mkwfs.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

atmwfs_status err(atmwfs_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    atmwfs::set_error_message(buf);
    return s;
}

#define MK_TRY(x)                                      \
    do {                                               \
        const atmwfs_status s_ = (x);                  \
        if (s_ != ATMWFS_OK) return s_;                \
    } while (0)

bool file_exists(const std::string& name)
{
    FILE* f = fopen(name.c_str(), "r");
    if (!f) return false;
    fclose(f);
    return true;
}

// `touch`: create the file if absent, else update its times (:4362-4375)
atmwfs_status touch(const std::string& name)
{
    const int fd = open(name.c_str(), O_WRONLY | O_CREAT, 0666);
    if (fd < 0) return err(ATMWFS_ERR_IO, "cannot touch \"%s\"", name.c_str());
    futimens(fd, nullptr);
    close(fd);
    return ATMWFS_OK;
}

std::string fmt(const char* f, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof buf, f, ap);
    va_end(ap);
    return buf;
}

// Dry standard air (Ciddor 1996, eq. 1; sigma in 1/um) thinned with an 8 km
// exponential scale height: the refractivity used when the caller brings
// no atmosphere model.
float builtin_refractivity(float alt, float lambda, void*)
{
    double s2 = 1.0 / ((double)lambda * 1e6);
    s2 *= s2;
    const double nas = 1e-8 * (5792105.0 / (238.0185 - s2) + 167917.0 / (57.362 - s2));
    return (float)(nas * exp(-(double)alt / 8000.0));
}

atmwfs_status write_cube(const std::string& name, const std::vector<float>& cube, long w, long nframes, long precision)
{
    const long ax[3] = {w, w, nframes};
    if (precision == 0) return atmwfs_fits_write(name.c_str(), cube.data(), -32, 3, ax);
    std::vector<double> d(cube.begin(), cube.end());
    return atmwfs_fits_write(name.c_str(), d.data(), -64, 3, ax);
}

struct Resources {
    atmwfs_ctx* ctx = nullptr;
    atmwfs_shm* shm[4] = {nullptr, nullptr, nullptr, nullptr};
    atmwfs_fno* fno = nullptr;
    std::vector<void*> dev;
    ~Resources()
    {
        for (atmwfs_shm* s : shm)
            if (s) atmwfs_shm_close(s);
        for (void* p : dev) cudaFree(p);
        if (fno) atmwfs_fno_destroy(fno);
        if (ctx) atmwfs_destroy(ctx);
    }
    float* alloc(size_t n)
    {
        void* p = nullptr;
        if (cudaMalloc(&p, n * sizeof(float)) != cudaSuccess) return nullptr;
        dev.push_back(p);
        return (float*)p;
    }
};

// Surrogate frame: windows of every instance -> network -> amplitude and
// phase (phi + arg(1 + D)), cropped to Wout into the host frame block.
struct SurrogateStep {
    float *win, *lam, *in, *phi, *out, *amp, *pha;
};

atmwfs_status surrogate_frame(Resources& R, const SurrogateStep& b, int ni, int L, long W, long Wout, const long* off,
                              float* hpha, float* hamp)
{
    const long P = W * W;
    MK_TRY(atmwfs_advance(R.ctx, 1));
    for (int i = 0; i < ni; i++) MK_TRY(atmwfs_windows_dev(R.ctx, i, b.win + (size_t)i * L * P, nullptr));
    void* st = atmwfs_stream(R.ctx);
    MK_TRY(atmwfs_fno_prepare(b.win, b.lam, ni, L, (int)W, b.in, b.phi, st));
    MK_TRY(atmwfs_fno_forward(R.fno, b.in, b.out, ni, st));
    MK_TRY(atmwfs_fno_assemble(b.out, b.phi, ni, (int)W, b.amp, b.pha, st));
    const long c0 = (W - Wout) / 2;
    for (int i = 0; i < ni; i++) {
        const size_t src = (size_t)i * P + (size_t)c0 * W + c0;
        if (cudaMemcpy2DAsync(hpha + off[i], Wout * sizeof(float), b.pha + src, W * sizeof(float), Wout * sizeof(float),
                              Wout, cudaMemcpyDeviceToHost, (cudaStream_t)st) != cudaSuccess ||
            cudaMemcpy2DAsync(hamp + off[i], Wout * sizeof(float), b.amp + src, W * sizeof(float), Wout * sizeof(float),
                              Wout, cudaMemcpyDeviceToHost, (cudaStream_t)st) != cudaSuccess)
            return err(ATMWFS_ERR_CUDA, "surrogate frame copy failed");
    }
    if (cudaStreamSynchronize((cudaStream_t)st) != cudaSuccess) return err(ATMWFS_ERR_CUDA, "surrogate frame failed");
    return ATMWFS_OK;
}

}  // namespace

extern "C" atmwfs_status atmwfs_mkwfs(const char* conf_file, float slambda_um, long precision,
                                      const atmwfs_mkwfs_opts* o)
{
    atmwfs_mkwfs_opts opts;
    memset(&opts, 0, sizeof opts);
    if (o) opts = *o;
    if (precision != 0 && precision != 1) return err(ATMWFS_ERR_INVALID, "precision must be 0 (float) or 1 (double)");
    if (!(slambda_um > 0)) return err(ATMWFS_ERR_INVALID, "science wavelength must be > 0");
    atmwfs_conf cf;
    MK_TRY(atmwfs_conf_load(conf_file, &cf));
    const double SLAMBDA = 1.0e-6 * slambda_um;                       // :1623
    const long W = cf.wf_raw_size, Wout = cf.wfsize, M = cf.master_size;
    if (W < 1 || Wout < 1 || Wout > W) return err(ATMWFS_ERR_INVALID, "WF_RAW_SIZE %ld / WFsize %ld", W, Wout);
    const long ratio = W / Wout;                                       // :1855-1870
    if (ratio != 1 && ratio != 2 && ratio != 4 && ratio != 8)
        return err(ATMWFS_ERR_INVALID, "unknown contraction factor (WF_RAW_SIZE / WFsize = %ld)", ratio);
    const long nframes = (long)(1.0 * cf.time_span / cf.wftime_step + 0.5);   // :1876
    if (nframes < 1) return err(ATMWFS_ERR_INVALID, "TIME_SPAN / WFTIME_STEP gives %ld frames", nframes);
    if (M < 64) return err(ATMWFS_ERR_INVALID, "MASTER_SIZE %ld", M);
    const bool verbose = opts.verbose != 0;

    // master screen files already present (:1925-1945)
    const char sfx = precision == 0 ? 'f' : 'd';
    auto master_name = [&](long i) { return fmt("t%03ld_%ld_%c.fits", i, M, sfx); };
    long nmasters = 0;
    while (file_exists(master_name(nmasters))) nmasters++;

    // profile (:1946-2015)
    long L = 0;
    MK_TRY(atmwfs_profile_read(cf.prof_file, (double)cf.site_alt, nullptr, 0, &L));
    if (L < 1) return err(ATMWFS_ERR_INVALID, "no layer in profile \"%s\"", cf.prof_file);
    std::vector<double> prof((size_t)L * 8);
    MK_TRY(atmwfs_profile_read(cf.prof_file, (double)cf.site_alt, prof.data(), L, &L));
    std::vector<double> alt(L), cn2(L), spd(L), dir(L), outer(L), inner(L);
    for (long l = 0; l < L; l++) {
        alt[l] = prof[l * 8 + 0];
        cn2[l] = prof[l * 8 + 1];
        spd[l] = prof[l * 8 + 2];
        dir[l] = prof[l * 8 + 3];
        outer[l] = prof[l * 8 + 4];
        inner[l] = prof[l * 8 + 5];
    }
    if (nmasters < L) nmasters = L;                                    // :2205-2206

    // load, or synthesise and save, every master screen (:2207-2226)
    const size_t M2 = (size_t)M * M;
    std::vector<std::vector<float>> screens(nmasters);
    for (long i = 0; i < nmasters; i++) {
        screens[i].resize(M2);
        const std::string fn = master_name(i);
        if (file_exists(fn)) {
            int nax = 0;
            long ax[3];
            MK_TRY(atmwfs_fits_read_f32(fn.c_str(), nullptr, 0, &nax, ax));
            if (nax != 2 || ax[0] != M || ax[1] != M)
                return err(ATMWFS_ERR_INVALID, "\"%s\" is %ld x %ld, MASTER_SIZE is %ld", fn.c_str(), ax[0], ax[1], M);
            MK_TRY(atmwfs_fits_read_f32(fn.c_str(), screens[i].data(), (long)M2, &nax, ax));
        } else {
            if (verbose) printf("CREATING %s   (%f - %f)\n", fn.c_str(), outer[i] / cf.pupil_scale, inner[i] / cf.pupil_scale);
            std::vector<float> second(M2);
            double cfit[2];
            MK_TRY(atmwfs_master_screen(opts.seed, (uint32_t)i, M, outer[i] / cf.pupil_scale, inner[i] / cf.pupil_scale,
                                        screens[i].data(), second.data(), cfit));
            const long ax[2] = {M, M};
            if (precision == 0) {
                MK_TRY(atmwfs_fits_write(fn.c_str(), screens[i].data(), -32, 2, ax));
            } else {
                std::vector<double> d(screens[i].begin(), screens[i].end());
                MK_TRY(atmwfs_fits_write(fn.c_str(), d.data(), -64, 2, ax));
            }
        }
    }

    // chromatic phase scaling and refraction offsets per layer
    const atmwfs_refractivity_fn N = opts.refractivity ? opts.refractivity : builtin_refractivity;
    void* user = opts.refractivity ? opts.refractivity_user : nullptr;
    std::vector<double> scoeff(L), roff(L);
    for (long l = 0; l < L; l++) {
        if (opts.scoeff) {
            scoeff[l] = opts.scoeff[l];
        } else {                                                       // :2661-2663
            const double Nl = N((float)alt[l], cf.lambda, user);
            const double Ns = N((float)alt[l], (float)SLAMBDA, user);
            scoeff[l] = cf.lambda / SLAMBDA * Ns / Nl;
        }
        if (opts.roffset) {
            roff[l] = opts.roffset[l];
        } else {                                                       // :2159-2183
            const double sz = sin(cf.zangle);
            double off[2] = {0.0, 0.0};
            if (sz != 0.0)
                for (int w = 0; w < 2; w++)
                    for (double h = cf.site_alt; h < alt[l]; h += 1.0) {
                        const double n = 1.0 + N((float)h, w == 0 ? cf.lambda : (float)SLAMBDA, user);
                        double t = sz / sqrt(n * n - sz * sz);
                        t -= sz / sqrt(1.0 - sz * sz);
                        off[w] += t;
                    }
            roff[l] = off[1] - off[0];
        }
    }

    // instances: the reference wavelength (files or stream) and the science one
    const bool amp = cf.wavefront_amplitude == 1;
    const bool ref_on = cf.wfoutput == 1 || cf.shm_output == 1;
    const bool sci_on = cf.make_swavefront == 1;
    std::vector<float> sc_f(L);
    for (long l = 0; l < L; l++) sc_f[l] = (float)scoeff[l];
    atmwfs_instance inst[2];
    memset(inst, 0, sizeof inst);
    int ni = 0, iref = -1, isci = -1;
    if (ref_on) {
        // one set of window positions serves both wavelengths, so the
        // reference wavelength also carries the refraction offsets (:2183)
        inst[ni] = atmwfs_instance{(double)cf.lambda, amp ? ATMWFS_MODE_REF : ATMWFS_MODE_PHASE, cf.source_xpos,
                                   cf.source_ypos, W, Wout, nullptr, roff.data()};
        iref = ni++;
    }
    if (sci_on) {
        inst[ni] = atmwfs_instance{SLAMBDA, amp ? ATMWFS_MODE_SCI : ATMWFS_MODE_PHASE, cf.source_xpos, cf.source_ypos,
                                   W, Wout, sc_f.data(), roff.data()};
        isci = ni++;
    }

    // optional lambda / n hops: the air index at the middle of each hop, at
    // the instance's wavelength (the reference propagates with the vacuum
    // wavelength, WFpropagate.c:91)
    std::vector<double> hop_n[2];
    if (opts.fresnel_air_index) {
        std::vector<double> salt(L), hz(L > 1 ? L - 1 : 1);
        std::vector<int> sidx(L), plo(L), phi(L);
        int ns = 0, npl = 0;
        MK_TRY(atmwfs_layer_planes(alt.data(), cn2.data(), (int)L, cf.fresnel_propagation_bin,
                                   cf.wavefront_amplitude == 1, cf.fresnel_propagation, cf.zangle, &ns, salt.data(),
                                   sidx.data(), &npl, plo.data(), phi.data(), hz.data()));
        for (int k = 0; k < ni; k++)
            for (int h = 0; h + 1 < npl; h++) {
                const double mid = 0.5 * (salt[sidx[plo[h]]] + salt[sidx[plo[h + 1]]]);
                hop_n[k].push_back(1.0 + N((float)mid, (float)inst[k].lambda, user));
            }
        for (int k = 0; k < ni; k++) inst[k].hop_n = hop_n[k].empty() ? nullptr : hop_n[k].data();
    }

    Resources R;
    std::vector<float> hpha, hamp;
    long ff = 0, off_ref = 0, off_sci = 0;
    const bool stepwise = cf.realtime == 1 || cf.shm_output == 1 || cf.shm_soutput == 1 || cf.waitforsem == 1 ||
                          cf.simtdelay > 0;
    if (ni > 0) {
        atmwfs_params p;
        memset(&p, 0, sizeof p);
        p.nlayers = (int)L;
        p.alt = alt.data();
        p.cn2 = cn2.data();
        p.speed = spd.data();
        p.dir = dir.data();
        p.fresnel_bin = cf.fresnel_propagation_bin;
        p.zangle = cf.zangle;
        p.pupil_scale = cf.pupil_scale;
        p.time_step = cf.wftime_step;
        p.master_size = M;
        p.amplitude = amp ? 1 : 0;
        p.fresnel = cf.fresnel_propagation;
        p.realtime = cf.realtime;
        p.realtime_factor = cf.realtime_factor;
        p.ninst = ni;
        p.inst = inst;
        p.ring = 2;
        MK_TRY(atmwfs_create(&p, &R.ctx));
        for (long l = 0; l < L; l++) MK_TRY(atmwfs_load_screen(R.ctx, (int)l, screens[l].data(), M));
        std::vector<const float*> extra;
        for (long i = L; i < nmasters; i++) extra.push_back(screens[i].data());
        double r0[2];
        MK_TRY(atmwfs_normalize_screens_ext(R.ctx, cf.lambda, cf.seeing, extra.data(), (long)extra.size(), r0));
        if (verbose) printf("r0 = %g pix -> %g pix\n", r0[0], r0[1]);
        ff = atmwfs_frame_floats(R.ctx);
        if (iref >= 0) off_ref = atmwfs_frame_offset(R.ctx, iref);
        if (isci >= 0) off_sci = atmwfs_frame_offset(R.ctx, isci);
        hpha.resize((size_t)ff * nframes);
        hamp.resize((size_t)ff * nframes);
        // learned surrogate in real-time mode (SURROGATE_MODEL, a keyword of
        // this engine): it stands in for the propagation when the model fits
        // the run; otherwise the plain path runs
        char mpath[200];
        if (cf.realtime == 1 && atmwfs_conf_read(conf_file ? conf_file : "WFsim.conf", "SURROGATE_MODEL", mpath,
                                                 sizeof mpath) == 1) {
            atmwfs_fno* f = nullptr;
            atmwfs_fno_cfg fc;
            if (atmwfs_fno_load(mpath, &f) == ATMWFS_OK && atmwfs_fno_get_cfg(f, &fc) == ATMWFS_OK && fc.grid == W &&
                fc.nin == L + 1 && fc.nout == 2 && amp) {
                R.fno = f;
            } else {
                if (f) atmwfs_fno_destroy(f);
                if (verbose) printf("surrogate \"%s\" does not fit this run: plain propagation\n", mpath);
            }
        }
    }
    SurrogateStep sb{};
    long offs[2] = {off_ref, off_sci};
    if (R.fno) {
        const size_t P = (size_t)W * W;
        sb.win = R.alloc((size_t)ni * L * P);
        sb.lam = R.alloc(ni);
        sb.in = R.alloc((size_t)ni * (L + 1) * P);
        sb.phi = R.alloc((size_t)ni * P);
        sb.out = R.alloc((size_t)ni * 2 * P);
        sb.amp = R.alloc((size_t)ni * P);
        sb.pha = R.alloc((size_t)ni * P);
        if (!sb.win || !sb.lam || !sb.in || !sb.phi || !sb.out || !sb.amp || !sb.pha)
            return err(ATMWFS_ERR_NOMEM, "surrogate buffers");
        float lams[2];
        for (int i = 0; i < ni; i++) lams[i] = (float)inst[i].lambda;
        if (cudaMemcpy(sb.lam, lams, sizeof(float) * ni, cudaMemcpyHostToDevice) != cudaSuccess)
            return err(ATMWFS_ERR_CUDA, "surrogate wavelength copy");
        if (iref < 0) offs[0] = off_sci;  // instance order: the science instance comes first
        if (verbose) printf("real-time frames from the surrogate model\n");
    }
    screens.clear();

    // shared-memory streams (:2425-2483)
    const int dtype = precision == 0 ? 3 : 4;
    if (cf.shm_output == 1) {
        MK_TRY(atmwfs_shm_create("atmwfpha", Wout, Wout, dtype, &R.shm[0]));
        MK_TRY(atmwfs_shm_create("atmwfamp", Wout, Wout, dtype, &R.shm[1]));
    }
    if (cf.shm_soutput == 1) {
        MK_TRY(atmwfs_shm_create((std::string(cf.shm_sprefix) + "pha").c_str(), Wout, Wout, dtype, &R.shm[2]));
        MK_TRY(atmwfs_shm_create((std::string(cf.shm_sprefix) + "amp").c_str(), Wout, Wout, dtype, &R.shm[3]));
    }
    // stream scale of the science phase (:4287-4300)
    double coeff = 1.0;
    if (cf.shm_soutputm == 1) coeff = SLAMBDA / 2.0 / M_PI;
    if (cf.shm_soutputm == 2) coeff = SLAMBDA / 2.0 / M_PI * 1e6;
    const size_t fr = (size_t)Wout * Wout;
    std::vector<double> dbuf(fr);
    std::vector<float> fbuf(fr);
    auto stream = [&](atmwfs_shm* s, const float* src, double k, int bump) -> atmwfs_status {
        if (!s) return ATMWFS_OK;
        if (dtype == 3) {
            for (size_t i = 0; i < fr; i++) fbuf[i] = (float)(src[i] * k);
            return atmwfs_shm_write(s, fbuf.data(), bump);
        }
        for (size_t i = 0; i < fr; i++) dbuf[i] = src[i] * k;
        return atmwfs_shm_write(s, dbuf.data(), bump);
    };

    const long lam_pm = (long)(1.0e12 * SLAMBDA + 0.5);
    long start = 0;                                                    // :2489-2511
    if (cf.skip_existing == 1)
        while (file_exists(fmt("%s%08ld.%09ld.pha.fits", cf.swf_file_prefix, start, lam_pm))) start++;

    std::vector<float> cube((size_t)fr * nframes);
    auto gather = [&](const std::vector<float>& src, long off) {
        for (long f = 0; f < nframes; f++)
            memcpy(&cube[(size_t)f * fr], &src[(size_t)f * ff + off], sizeof(float) * fr);
    };
    for (long tspan = start; tspan < cf.nb_tspan; tspan++) {
        if (ni > 0) {
            if (stepwise) {
                for (long f = 0; f < nframes; f++) {
                    if (cf.simtdelay > 0) usleep((useconds_t)cf.simtdelay);
                    if (cf.waitforsem == 1) MK_TRY(atmwfs_shm_semwait(cf.waitsemimname, 0, opts.semwait_timeout));
                    atmwfs_sink sk{hpha.data() + (size_t)f * ff, hamp.data() + (size_t)f * ff, 1};
                    if (R.fno)
                        MK_TRY(surrogate_frame(R, sb, ni, (int)L, W, Wout, offs, sk.pha, sk.amp));
                    else
                        MK_TRY(atmwfs_run(R.ctx, 1, &sk));
                    if (iref >= 0) {
                        MK_TRY(stream(R.shm[0], sk.pha + off_ref, 1.0, 0));
                        MK_TRY(stream(R.shm[1], sk.amp + off_ref, 1.0, 0));
                    }
                    if (isci >= 0) {
                        MK_TRY(stream(R.shm[2], sk.pha + off_sci, coeff, 1));
                        MK_TRY(stream(R.shm[3], sk.amp + off_sci, 1.0, 1));
                    }
                }
            } else {
                atmwfs_sink sk{hpha.data(), hamp.data(), nframes};
                MK_TRY(atmwfs_run(R.ctx, nframes, &sk));
            }
        }
        if (verbose) printf("time span %ld / %ld: %ld frames\n", tspan, cf.nb_tspan, nframes);
        // reference-wavelength files, named with the science wavelength (:4349-4376)
        const std::string rp = fmt("%s%08ld.%09ld.pha.fits", cf.wf_file_prefix, tspan, lam_pm);
        const std::string ra = fmt("%s%08ld.%09ld.amp.fits", cf.wf_file_prefix, tspan, lam_pm);
        if (cf.wfoutput == 1) {
            gather(hpha, off_ref);
            MK_TRY(write_cube("!" + rp, cube, Wout, nframes, precision));
            if (amp) {
                gather(hamp, off_ref);
                MK_TRY(write_cube("!" + ra, cube, Wout, nframes, precision));
            }
        } else if (cf.wfoutput == 0) {
            MK_TRY(touch(rp));
            if (amp) MK_TRY(touch(ra));
        }
        if (sci_on && cf.swf_write2disk == 1) {                        // :4380-4400
            gather(hpha, off_sci);
            MK_TRY(write_cube("!" + fmt("%s%08ld.%09ld.pha.fits", cf.swf_file_prefix, tspan, lam_pm), cube, Wout,
                              nframes, precision));
            if (amp) {
                gather(hamp, off_sci);
                MK_TRY(write_cube("!" + fmt("%s%08ld.%09ld.amp.fits", cf.swf_file_prefix, tspan, lam_pm), cube, Wout,
                                  nframes, precision));
            }
        }
    }
    return ATMWFS_OK;
}
