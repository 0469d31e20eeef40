// host_hv.cpp -- Hufnagel-Valley turbulence profile file, the input of the
// series command that the reference's mkHVturbprof command writes.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "atmwfs_mkwfs.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

const double kPi = 3.14159265358979323846264338328;

// Hufnagel-Valley Cn2(h) with the wind term scaled by (v / 27 m/s)^2 and a
// ground layer of strength A decaying over 100 m above the site.
double hv_cn2(double h, double wspeed, double A, double sitealt)
{
    return 5.94e-53 * pow(wspeed / 27.0, 2.0) * pow(h, 10.0) * exp(-h / 1000.0) + 2.7e-16 * exp(-h / 1500.0) +
           A * exp(-(h - sitealt) / 100.0);
}

}  // namespace

extern "C" atmwfs_status atmwfs_make_hv_profile(double wspeed, double r0, double sitealt, long nlayers,
                                                const char* outfile, double* seeing)
{
    if (!outfile || nlayers < 2 || !(r0 > 0) || !(sitealt < 30000.0)) {
        atmwfs::set_error_message("atmwfs_make_hv_profile: bad arguments (nlayers >= 2, r0 > 0, site below 30 km)");
        return ATMWFS_ERR_INVALID;
    }
    const double hmax = 30000.0, lambda = 0.55e-6, A0 = 1.7e-14;
    double hstep = 1.0, Acoeff = 1.0, Astep = 1.0, A = A0, CN2sum = 0.0, r0val = 0.0;
    // ground-layer strength: 30 multiplicative bisection steps on r0 at 550 nm
    for (int iter = 0; iter < 30; iter++) {
        A = A0 * Acoeff;
        CN2sum = 0.0;
        for (double h = sitealt; h < hmax; h += hstep) CN2sum += hv_cn2(h, wspeed, A, sitealt) / hstep;
        r0val = 1.0 / pow(0.423 * pow(2.0 * kPi / lambda, 2.0) * CN2sum, 3.0 / 5.0);
        if (r0val > r0) Acoeff *= 1.0 + Astep;
        else Acoeff /= 1.0 + Astep;
        Astep *= 0.8;
    }
    const double see = (lambda / r0val) / kPi * 180.0 * 3600.0;
    if (seeing) *seeing = see;
    FILE* fp = fopen("conf_turb.txt", "w");
    if (!fp) {
        atmwfs::set_error_message("cannot create conf_turb.txt");
        return ATMWFS_ERR_IO;
    }
    fprintf(fp, "%f\n", see);
    fclose(fp);
    // layers at quadratically spaced altitudes; each 1 m slice's Cn2 goes to
    // the nearest layer in sqrt-altitude
    std::vector<double> lh(nlayers), frac(nlayers, 0.0);
    for (long k = 0; k < nlayers; k++) lh[k] = sitealt + pow(1.0 * k / (nlayers - 1), 2.0) * (hmax - sitealt);
    hstep = 1.0;
    for (double h = sitealt; h < hmax; h += hstep) {
        const long k = (long)(sqrt((h - sitealt) / (hmax - sitealt)) * (1.0 * nlayers - 1.0) + 0.5);
        frac[k] += hv_cn2(h, wspeed, A, sitealt);
    }
    fp = fopen(outfile, "w");
    if (!fp) {
        atmwfs::set_error_message("cannot create the profile file");
        return ATMWFS_ERR_IO;
    }
    fprintf(fp, "# altitude(m)   relativeCN2     speed(m/s)   direction(rad) outerscale[m] innerscale[m] sigmaWsp[m/s] Lwind[m]\n");
    fprintf(fp, "\n");
    for (long k = 0; k < nlayers; k++) {
        frac[k] /= CN2sum;
        const double l0 = 0.008 + 0.072 * pow(lh[k] / 20000.0, 1.6);
        const double L0 = lh[k] < 14000.0 ? pow(10.0, 2.0 - 0.9 * (lh[k] / 14000.0))
                                          : pow(10.0, 1.1 + 0.3 * (lh[k] - 14000.0) / 6000.0);
        const double ws = wspeed * (0.3 + 0.8 * sqrt(1.0 * k / (1.0 + nlayers)));
        fprintf(fp, "%12f  %12f  %12f  %12f  %12f  %12f  %12f  %12f\n", lh[k], frac[k], ws, 2.0 * kPi * k / (1.0 + nlayers),
                L0, l0, 0.1 * ws, 500.0);
    }
    if (fclose(fp) != 0) {
        atmwfs::set_error_message("write of the profile file failed");
        return ATMWFS_ERR_IO;
    }
    return ATMWFS_OK;
}
