// host_conf.cpp -- the configuration file (WFsim.conf) and the turbulence
// profile, read with the reference's token rules so that every file the
// reference accepts yields the same values here.
#include <cctype>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "atmwfs_mkwfs.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

// fgets() buffer sizes of the reference readers: lines longer than this are
// read as several lines, as there.
constexpr int kConfLine = 1000;     // COREMOD_tools.c:603, 633
constexpr int kProfLine = 2000;     // AtmosphericTurbulence.c:1955, 1979

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

// The first `want` whitespace-separated tokens of a line (sscanf "%s"
// semantics: isspace() separates, nothing is assigned past the last token).
int tokens(const char* line, std::string* out, int want)
{
    int n = 0;
    const unsigned char* p = (const unsigned char*)line;
    while (n < want) {
        while (*p && isspace(*p)) p++;
        if (!*p) break;
        const unsigned char* q = p;
        while (*q && !isspace(*q)) q++;
        out[n++].assign((const char*)p, (size_t)(q - p));
        p = q;
    }
    return n;
}

void copy_out(char* dst, long cap, const std::string& s)
{
    if (!dst || cap <= 0) return;
    const size_t n = s.size() < (size_t)(cap - 1) ? s.size() : (size_t)(cap - 1);
    memcpy(dst, s.data(), n);
    dst[n] = '\0';
}

}  // namespace

extern "C" int atmwfs_conf_read(const char* conf_file, const char* keyword, char* content, long cap)
{
    if (!conf_file || !keyword) {
        err(ATMWFS_ERR_INVALID, "null argument");
        return -1;
    }
    FILE* fp = fopen(conf_file, "r");
    if (!fp) {
        err(ATMWFS_ERR_IO, "cannot open file \"%s\"", conf_file);
        return -1;
    }
    // keyw / cont carry over between lines, as the reference's locals do
    // when sscanf assigns fewer than two tokens
    std::string tok[2];
    std::string value = "---";
    int read = 0;
    char line[kConfLine];
    while (fgets(line, sizeof line, fp)) {
        tokens(line, tok, 2);
        if (tok[0] == keyword) {
            value = tok[1];
            read = 1;
        }
    }
    fclose(fp);
    if (!read) value = "-";
    copy_out(content, cap, value);
    return read;
}

extern "C" int atmwfs_conf_exists(const char* conf_file, const char* keyword)
{
    if (!conf_file || !keyword) {
        err(ATMWFS_ERR_INVALID, "null argument");
        return -1;
    }
    FILE* fp = fopen(conf_file, "r");
    if (!fp) {
        err(ATMWFS_ERR_IO, "cannot open file \"%s\"", conf_file);
        return -1;
    }
    std::string tok[1];
    int read = 0;
    char line[kConfLine];
    while (!read && fgets(line, sizeof line, fp)) {
        tokens(line, tok, 1);
        if (tok[0] == keyword) read = 1;
    }
    fclose(fp);
    return read;
}

extern "C" atmwfs_status atmwfs_conf_load(const char* conf_file, atmwfs_conf* c)
{
    if (!c) return err(ATMWFS_ERR_INVALID, "null conf");
    const char* f = conf_file ? conf_file : "WFsim.conf";
    FILE* probe = fopen(f, "r");
    if (!probe) return err(ATMWFS_ERR_IO, "cannot open file \"%s\"", f);
    fclose(probe);
    memset(c, 0, sizeof *c);
    // initial values of the globals (AtmosphericTurbulence.c:104-160)
    c->wfoutput = 1;
    c->realtime_factor = 1.0;
    char v[200];
    auto get = [&](const char* k) -> const char* {
        atmwfs_conf_read(f, k, v, sizeof v);
        return v;
    };
    auto has = [&](const char* k) { return atmwfs_conf_exists(f, k) == 1; };
    // same order and conversions as AtmosphericTurbulence_ReadConf (:1233-1427)
    c->lambda = (float)(atof(get("TURBULENCE_REF_WAVEL")) * 0.000001);
    c->seeing = (float)atof(get("TURBULENCE_SEEING"));
    atmwfs_conf_read(f, "TURBULENCE_PROF_FILE", c->prof_file, sizeof c->prof_file);
    c->zangle = (float)atof(get("ZENITH_ANGLE"));
    c->source_xpos = (float)atof(get("SOURCE_XPOS"));
    c->source_ypos = (float)atof(get("SOURCE_YPOS"));
    if (has("WFOUTPUT")) c->wfoutput = atoi(get("WFOUTPUT"));
    atmwfs_conf_read(f, "WF_FILE_PREFIX", c->wf_file_prefix, sizeof c->wf_file_prefix);
    if (has("SHM_OUTPUT")) c->shm_output = atoi(get("SHM_OUTPUT"));
    c->make_swavefront = atoi(get("MAKE_SWAVEFRONT"));
    c->swf_write2disk = atoi(get("SWF_WRITE2DISK"));
    atmwfs_conf_read(f, "SWF_FILE_PREFIX", c->swf_file_prefix, sizeof c->swf_file_prefix);
    if (has("SHM_SOUTPUT")) c->shm_soutput = atoi(get("SHM_SOUTPUT"));
    atmwfs_conf_read(f, "SHM_SPREFIX", c->shm_sprefix, sizeof c->shm_sprefix);
    c->shm_soutputm = atoi(get("SHM_SOUTPUTM"));
    c->pupil_scale = (float)atof(get("PUPIL_SCALE"));
    c->wfsize = atol(get("WFsize"));
    c->realtime = atoi(get("REALTIME"));
    c->realtime_factor = atof(get("REALTIMEFACTOR"));
    c->wftime_step = (float)atof(get("WFTIME_STEP"));
    c->time_span = (float)atof(get("TIME_SPAN"));
    c->nb_tspan = atol(get("NB_TSPAN"));
    c->simtdelay = atol(get("SIMTDELAY"));
    c->waitforsem = atoi(get("WAITFORSEM"));
    atmwfs_conf_read(f, "WAITSEMIMNAME", c->waitsemimname, sizeof c->waitsemimname);
    c->skip_existing = has("SKIP_EXISTING") ? 1 : 0;
    c->wf_raw_size = atol(get("WF_RAW_SIZE"));
    c->master_size = atol(get("MASTER_SIZE"));
    c->wavefront_amplitude = atoi(get("WAVEFRONT_AMPLITUDE"));
    c->fresnel_propagation = c->wavefront_amplitude == 1 ? atoi(get("FRESNEL_PROPAGATION")) : 0;
    c->fresnel_propagation_bin = (float)atof(get("FRESNEL_PROPAGATION_BIN"));
    // the atmosphere model's site altitude (AtmosphereModel.c:3907-3909)
    c->site_alt = (float)atof(get("SITE_ALT"));
    return ATMWFS_OK;
}

extern "C" atmwfs_status atmwfs_profile_read(const char* path, double site_alt, double* layers, long cap,
                                             long* nlayers)
{
    if (!path || !nlayers) return err(ATMWFS_ERR_INVALID, "null argument");
    FILE* fp = fopen(path, "r");
    if (!fp) return err(ATMWFS_ERR_IO, "Cannot open turbulence profile file \"%s\"", path);
    // `word` and the eight values persist between lines, as the reference's
    // locals do when sscanf assigns nothing (blank lines) or fewer values
    std::string word[1];
    double fl[8];
    bool have_fl[8] = {false, false, false, false, false, false, false, false};
    long n = 0;
    char line[kProfLine];
    atmwfs_status st = ATMWFS_OK;
    while (fgets(line, sizeof line, fp)) {
        tokens(line, word, 1);
        if (word[0].empty() || !isdigit((unsigned char)word[0][0])) continue;
        // sscanf("%lf" x 8): stops at the first field that does not convert
        const char* p = line;
        for (int k = 0; k < 8; k++) {
            char* end = nullptr;
            const double x = strtod(p, &end);
            if (end == p) break;
            fl[k] = x;
            have_fl[k] = true;
            p = end;
        }
        bool complete = true;
        for (bool h : have_fl) complete = complete && h;
        if (!complete) {
            st = err(ATMWFS_ERR_INVALID, "profile line %ld has fewer than 8 numbers and no previous line to fill them", n);
            break;
        }
        if (!(fl[0] > site_alt - 0.1)) {
            st = err(ATMWFS_ERR_INVALID, "profile layer at %g m is not above the site altitude %g m", fl[0], site_alt);
            break;
        }
        if (layers && n < cap)
            for (int k = 0; k < 8; k++) layers[n * 8 + k] = fl[k];
        n++;
    }
    fclose(fp);
    if (st != ATMWFS_OK) return st;
    *nlayers = n;
    return ATMWFS_OK;
}
