// host_fits.cpp -- primary-HDU FITS images: the wavefront cubes and master
// screens the series command writes and reads.  FITS stores big-endian
// values in 2880-byte blocks after a header of 80-character cards.
#include <cerrno>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "atmwfs_mkwfs.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

constexpr size_t kBlock = 2880;

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

void card(std::string& h, const char* key, const char* value)
{
    char c[81];
    snprintf(c, sizeof c, "%-8.8s= %20s", key, value);
    std::string s(c);
    s.resize(80, ' ');
    h += s;
}

// big-endian <-> host, byte by byte (no reliance on the host's order)
void put_be(unsigned char* dst, const unsigned char* src, int size)
{
    const uint16_t probe = 1;
    const bool little = *(const unsigned char*)&probe == 1;
    for (int i = 0; i < size; i++) dst[i] = little ? src[size - 1 - i] : src[i];
}

}  // namespace

extern "C" atmwfs_status atmwfs_fits_write(const char* name, const void* data, int bitpix, int naxis, const long* naxes)
{
    if (!name || !data || !naxes) return err(ATMWFS_ERR_INVALID, "null argument");
    if (bitpix != -32 && bitpix != -64) return err(ATMWFS_ERR_INVALID, "BITPIX %d unsupported (-32 or -64)", bitpix);
    if (naxis < 1 || naxis > 3) return err(ATMWFS_ERR_INVALID, "NAXIS %d unsupported (1..3)", naxis);
    size_t n = 1;
    for (int i = 0; i < naxis; i++) {
        if (naxes[i] < 1) return err(ATMWFS_ERR_INVALID, "NAXIS%d = %ld", i + 1, naxes[i]);
        n *= (size_t)naxes[i];
    }
    const bool overwrite = name[0] == '!';
    const char* path = overwrite ? name + 1 : name;
    if (!overwrite) {
        FILE* t = fopen(path, "rb");
        if (t) {
            fclose(t);
            return err(ATMWFS_ERR_IO, "file \"%s\" exists (prefix the name with '!' to overwrite)", path);
        }
    }
    std::string h;
    char v[32];
    card(h, "SIMPLE", "T");
    snprintf(v, sizeof v, "%d", bitpix);
    card(h, "BITPIX", v);
    snprintf(v, sizeof v, "%d", naxis);
    card(h, "NAXIS", v);
    for (int i = 0; i < naxis; i++) {
        char k[16];
        snprintf(k, sizeof k, "NAXIS%d", i + 1);
        snprintf(v, sizeof v, "%ld", naxes[i]);
        card(h, k, v);
    }
    card(h, "EXTEND", "T");
    std::string end = "END";
    end.resize(80, ' ');
    h += end;
    h.resize((h.size() + kBlock - 1) / kBlock * kBlock, ' ');
    FILE* fp = fopen(path, "wb");
    if (!fp) return err(ATMWFS_ERR_IO, "cannot create \"%s\": %s", path, strerror(errno));
    bool ok = fwrite(h.data(), 1, h.size(), fp) == h.size();
    const int es = bitpix == -32 ? 4 : 8;
    std::vector<unsigned char> buf(kBlock * 64);
    const unsigned char* src = (const unsigned char*)data;
    size_t done = 0;
    while (ok && done < n) {
        const size_t m = (buf.size() / es) < (n - done) ? buf.size() / es : n - done;
        for (size_t i = 0; i < m; i++) put_be(&buf[i * es], src + (done + i) * es, es);
        ok = fwrite(buf.data(), es, m, fp) == m;
        done += m;
    }
    const size_t pad = (kBlock - (n * es) % kBlock) % kBlock;
    if (ok && pad) {
        std::vector<unsigned char> z(pad, 0);
        ok = fwrite(z.data(), 1, pad, fp) == pad;
    }
    if (fclose(fp) != 0) ok = false;
    if (!ok) return err(ATMWFS_ERR_IO, "write to \"%s\" failed", path);
    return ATMWFS_OK;
}

extern "C" atmwfs_status atmwfs_fits_read_f32(const char* name, float* out, long cap, int* naxis_out, long* naxes_out)
{
    if (!name) return err(ATMWFS_ERR_INVALID, "null name");
    FILE* fp = fopen(name, "rb");
    if (!fp) return err(ATMWFS_ERR_IO, "cannot open \"%s\"", name);
    int bitpix = 0, naxis = -1;
    long naxes[3] = {1, 1, 1};
    double bscale = 1.0, bzero = 0.0;
    bool end = false;
    std::vector<char> block(kBlock);
    while (!end) {
        if (fread(block.data(), 1, kBlock, fp) != kBlock) {
            fclose(fp);
            return err(ATMWFS_ERR_IO, "\"%s\": truncated FITS header", name);
        }
        for (size_t o = 0; o < kBlock && !end; o += 80) {
            const char* c = block.data() + o;
            std::string key(c, 8);
            while (!key.empty() && key.back() == ' ') key.pop_back();
            if (key == "END") {
                end = true;
                break;
            }
            if (c[8] != '=') continue;
            std::string val(c + 10, 70);
            const size_t slash = val.find('/');
            if (slash != std::string::npos) val.resize(slash);
            const char* s = val.c_str();
            if (key == "BITPIX") bitpix = atoi(s);
            else if (key == "NAXIS") naxis = atoi(s);
            else if (key == "NAXIS1") naxes[0] = atol(s);
            else if (key == "NAXIS2") naxes[1] = atol(s);
            else if (key == "NAXIS3") naxes[2] = atol(s);
            else if (key == "BSCALE") bscale = atof(s);
            else if (key == "BZERO") bzero = atof(s);
        }
    }
    int es = 0;
    switch (bitpix) {
        case 8: es = 1; break;
        case 16: es = 2; break;
        case 32: case -32: es = 4; break;
        case 64: case -64: es = 8; break;
        default:
            fclose(fp);
            return err(ATMWFS_ERR_INVALID, "\"%s\": BITPIX %d unsupported", name, bitpix);
    }
    if (naxis < 1 || naxis > 3) {
        fclose(fp);
        return err(ATMWFS_ERR_INVALID, "\"%s\": NAXIS %d unsupported (1..3)", name, naxis);
    }
    const size_t n = (size_t)naxes[0] * naxes[1] * naxes[2];
    if (naxis_out) *naxis_out = naxis;
    if (naxes_out)
        for (int i = 0; i < 3; i++) naxes_out[i] = naxes[i];
    if (!out) {
        fclose(fp);
        return ATMWFS_OK;
    }
    if ((long)n > cap) {
        fclose(fp);
        return err(ATMWFS_ERR_INVALID, "\"%s\": %zu values exceed the buffer (%ld)", name, n, cap);
    }
    std::vector<unsigned char> raw(n * es);
    if (fread(raw.data(), 1, raw.size(), fp) != raw.size()) {
        fclose(fp);
        return err(ATMWFS_ERR_IO, "\"%s\": truncated data", name);
    }
    fclose(fp);
    for (size_t i = 0; i < n; i++) {
        unsigned char b[8];
        put_be(b, &raw[i * es], es);
        double x = 0.0;
        switch (bitpix) {
            case 8: x = raw[i]; break;
            case 16: { int16_t t; memcpy(&t, b, 2); x = t; } break;
            case 32: { int32_t t; memcpy(&t, b, 4); x = t; } break;
            case 64: { int64_t t; memcpy(&t, b, 8); x = (double)t; } break;
            case -32: { float t; memcpy(&t, b, 4); x = t; } break;
            case -64: { double t; memcpy(&t, b, 8); x = t; } break;
        }
        out[i] = (bscale == 1.0 && bzero == 0.0) ? (float)x : (float)(x * bscale + bzero);
    }
    return ATMWFS_OK;
}
