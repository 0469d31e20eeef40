/*
 * shim_fitsio.c -- primary-HDU FITS image I/O with the cfitsio calling
 * convention used by the reference's src/COREMOD_iofits/COREMOD_iofits.c.
 * Part of the checker build of the reference (oracle/ref); cfitsio itself is
 * not installed.  Supports BITPIX 8/16/32/-32/-64 images and the keyword
 * reads the reference performs.
 */
#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fitsio.h"

struct atmref_fits {
    FILE *fp;
    int writing;
    char *hdr;        /* header cards (reading) */
    long hdr_len;
    long data_off;
    int bitpix, naxis;
    long naxes[8];
    double bscale, bzero;
    long written;     /* bytes of data written */
};

static int set(int *status, int v) { *status = v; return v; }

static const char *find_card(const fitsfile *f, const char *key)
{
    size_t kl = strlen(key);
    for (long o = 0; o + 80 <= f->hdr_len; o += 80) {
        const char *c = f->hdr + o;
        if (strncmp(c, key, kl) == 0 && (c[kl] == ' ' || c[kl] == '=') && kl <= 8) return c;
        if (strncmp(c, "END     ", 8) == 0) break;
    }
    return NULL;
}

static void card_value(const char *c, char *val, char *comment)
{
    char buf[81];
    memcpy(buf, c + 10, 70);
    buf[70] = 0;
    char *s = buf;
    while (*s == ' ') s++;
    if (*s == '\'') {
        char *e = strchr(s + 1, '\'');
        if (e) *e = 0;
        strcpy(val, s + 1);
        if (comment) comment[0] = 0;
        return;
    }
    char *slash = strchr(s, '/');
    if (comment) {
        if (slash) { strncpy(comment, slash + 1, 72); comment[72] = 0; }
        else comment[0] = 0;
    }
    if (slash) *slash = 0;
    size_t n = strlen(s);
    while (n > 0 && s[n - 1] == ' ') s[--n] = 0;
    strcpy(val, s);
}

int fits_open_file(fitsfile **pf, const char *name, int mode, int *status)
{
    (void)mode;
    if (*status) return *status;
    FILE *fp = fopen(name, "rb");
    if (!fp) return set(status, FILE_NOT_OPENED);
    fitsfile *f = calloc(1, sizeof *f);
    f->fp = fp;
    f->bscale = 1.0;
    char block[2880];
    int done = 0;
    while (!done && fread(block, 1, 2880, fp) == 2880) {
        f->hdr = realloc(f->hdr, f->hdr_len + 2880);
        memcpy(f->hdr + f->hdr_len, block, 2880);
        f->hdr_len += 2880;
        for (int o = 0; o < 2880; o += 80)
            if (strncmp(block + o, "END     ", 8) == 0 || strncmp(block + o, "END\0", 4) == 0) done = 1;
    }
    if (!done) { fclose(fp); free(f->hdr); free(f); return set(status, FILE_NOT_OPENED); }
    f->data_off = f->hdr_len;
    char v[81];
    const char *c;
    if ((c = find_card(f, "BITPIX"))) { card_value(c, v, NULL); f->bitpix = atoi(v); }
    if ((c = find_card(f, "NAXIS"))) { card_value(c, v, NULL); f->naxis = atoi(v); }
    for (int i = 0; i < f->naxis && i < 8; i++) {
        char k[16];
        snprintf(k, sizeof k, "NAXIS%d", i + 1);
        if ((c = find_card(f, k))) { card_value(c, v, NULL); f->naxes[i] = atol(v); }
    }
    if ((c = find_card(f, "BSCALE"))) { card_value(c, v, NULL); f->bscale = atof(v); }
    if ((c = find_card(f, "BZERO"))) { card_value(c, v, NULL); f->bzero = atof(v); }
    *pf = f;
    return 0;
}

int fits_read_keyword(fitsfile *f, const char *key, char *value, char *comment, int *status)
{
    if (*status) return *status;
    const char *c = find_card(f, key);
    if (!c) return set(status, KEY_NO_EXIST);
    card_value(c, value, comment);
    return 0;
}

int fits_read_key(fitsfile *f, int datatype, const char *key, void *value, char *comment, int *status)
{
    if (*status) return *status;
    char v[81];
    if (fits_read_keyword(f, key, v, comment, status)) return *status;
    switch (datatype) {
        case TLONG: *(long *)value = atol(v); break;
        case TINT: *(int *)value = atoi(v); break;
        case TSHORT: *(short *)value = (short)atoi(v); break;
        case TFLOAT: *(float *)value = (float)atof(v); break;
        case TDOUBLE: *(double *)value = atof(v); break;
        case TSTRING: strcpy((char *)value, v); break;
        default: *(long *)value = atol(v); break;
    }
    return 0;
}

int fits_set_bscale(fitsfile *f, double scale, double zero, int *status)
{
    if (*status) return *status;
    f->bscale = scale;
    f->bzero = zero;
    return 0;
}

static int bpe(int bitpix) { return abs(bitpix) / 8; }

static double get_be(const unsigned char *p, int bitpix)
{
    uint64_t u = 0;
    int n = bpe(bitpix);
    for (int i = 0; i < n; i++) u = (u << 8) | p[i];
    switch (bitpix) {
        case 8: return (double)(uint8_t)u;
        case 16: return (double)(int16_t)u;
        case 32: return (double)(int32_t)u;
        case 64: return (double)(int64_t)u;
        case -32: { uint32_t w = (uint32_t)u; float x; memcpy(&x, &w, 4); return x; }
        case -64: { double x; memcpy(&x, &u, 8); return x; }
    }
    return 0;
}

static void put_be(unsigned char *p, int bitpix, double v)
{
    uint64_t u = 0;
    switch (bitpix) {
        case 8: u = (uint8_t)(long)v; break;
        case 16: u = (uint16_t)(int16_t)(long)v; break;
        case 32: u = (uint32_t)(int32_t)(long)v; break;
        case 64: u = (uint64_t)(int64_t)v; break;
        case -32: { float x = (float)v; uint32_t w; memcpy(&w, &x, 4); u = w; break; }
        case -64: memcpy(&u, &v, 8); break;
    }
    int n = bpe(bitpix);
    for (int i = n - 1; i >= 0; i--) { p[i] = (unsigned char)(u & 0xff); u >>= 8; }
}

static void store(void *array, int datatype, long i, double v)
{
    switch (datatype) {
        case TFLOAT: ((float *)array)[i] = (float)v; break;
        case TDOUBLE: ((double *)array)[i] = v; break;
        case TUSHORT: ((unsigned short *)array)[i] = (unsigned short)v; break;
        case TSHORT: ((short *)array)[i] = (short)v; break;
        case TINT: ((int *)array)[i] = (int)v; break;
        case TLONG: ((long *)array)[i] = (long)v; break;
        case TBYTE: ((unsigned char *)array)[i] = (unsigned char)v; break;
    }
}

static double load(const void *array, int datatype, long i)
{
    switch (datatype) {
        case TFLOAT: return ((const float *)array)[i];
        case TDOUBLE: return ((const double *)array)[i];
        case TUSHORT: return ((const unsigned short *)array)[i];
        case TSHORT: return ((const short *)array)[i];
        case TINT: return ((const int *)array)[i];
        case TLONG: return (double)((const long *)array)[i];
        case TBYTE: return ((const unsigned char *)array)[i];
    }
    return 0;
}

int fits_read_img(fitsfile *f, int datatype, long firstelem, long nelem, void *nulval, void *array, int *anynul,
                  int *status)
{
    (void)nulval;
    if (*status) return *status;
    if (anynul) *anynul = 0;
    const int n = bpe(f->bitpix);
    unsigned char *buf = malloc((size_t)nelem * n);
    fseek(f->fp, f->data_off + (firstelem - 1) * n, SEEK_SET);
    if ((long)fread(buf, n, nelem, f->fp) != nelem) { free(buf); return set(status, 107); }
    const int scaled = f->bitpix > 0;
    for (long i = 0; i < nelem; i++) {
        double v = get_be(buf + i * n, f->bitpix);
        if (scaled) v = v * f->bscale + f->bzero;
        store(array, datatype, i, v);
    }
    free(buf);
    return 0;
}

int fits_create_file(fitsfile **pf, const char *name, int *status)
{
    if (*status) return *status;
    int overwrite = name[0] == '!';
    const char *path = overwrite ? name + 1 : name;
    if (!overwrite) {
        FILE *t = fopen(path, "rb");
        if (t) { fclose(t); return set(status, FILE_NOT_CREATED); }
    }
    FILE *fp = fopen(path, "wb");
    if (!fp) return set(status, FILE_NOT_CREATED);
    fitsfile *f = calloc(1, sizeof *f);
    f->fp = fp;
    f->writing = 1;
    f->bscale = 1.0;
    *pf = f;
    return 0;
}

static void card(char *blk, int *pos, const char *fmt, ...)
    __attribute__((format(printf, 3, 4)));
#include <stdarg.h>
static void card(char *blk, int *pos, const char *fmt, ...)
{
    char c[128];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c, sizeof c, fmt, ap);
    va_end(ap);
    size_t n = strlen(c);
    memset(blk + *pos, ' ', 80);
    memcpy(blk + *pos, c, n > 80 ? 80 : n);
    *pos += 80;
}

int fits_create_img(fitsfile *f, int bitpix, int naxis, long *naxes, int *status)
{
    if (*status) return *status;
    f->bitpix = bitpix;
    f->naxis = naxis;
    char blk[2880 * 2];
    memset(blk, ' ', sizeof blk);
    int pos = 0;
    card(blk, &pos, "SIMPLE  = %20s / file does conform to FITS standard", "T");
    card(blk, &pos, "BITPIX  = %20d / number of bits per data pixel", bitpix);
    card(blk, &pos, "NAXIS   = %20d / number of data axes", naxis);
    for (int i = 0; i < naxis; i++) {
        f->naxes[i] = naxes[i];
        card(blk, &pos, "NAXIS%-3d= %20ld / length of data axis %d", i + 1, naxes[i], i + 1);
    }
    card(blk, &pos, "EXTEND  = %20s / FITS dataset may contain extensions", "T");
    card(blk, &pos, "END");
    long len = (pos + 2879) / 2880 * 2880;
    fwrite(blk, 1, (size_t)len, f->fp);
    f->data_off = len;
    return 0;
}

int fits_write_img(fitsfile *f, int datatype, long firstelem, long nelem, void *array, int *status)
{
    if (*status) return *status;
    const int n = bpe(f->bitpix);
    unsigned char *buf = malloc((size_t)nelem * n);
    for (long i = 0; i < nelem; i++) put_be(buf + i * n, f->bitpix, load(array, datatype, i));
    fseek(f->fp, f->data_off + (firstelem - 1) * n, SEEK_SET);
    fwrite(buf, n, (size_t)nelem, f->fp);
    free(buf);
    long end = (firstelem - 1 + nelem) * n;
    if (end > f->written) f->written = end;
    return 0;
}

int fits_close_file(fitsfile *f, int *status)
{
    if (!f) return *status;
    if (f->writing) {
        long pad = (2880 - f->written % 2880) % 2880;
        if (pad) {
            fseek(f->fp, f->data_off + f->written, SEEK_SET);
            char z[2880];
            memset(z, 0, sizeof z);
            fwrite(z, 1, (size_t)pad, f->fp);
        }
    }
    fclose(f->fp);
    free(f->hdr);
    free(f);
    return *status;
}

void fits_get_errstatus(int status, char *text) { snprintf(text, FLEN_STATUS, "fits shim status %d", status); }

void fits_report_error(FILE *stream, int status)
{
    if (status) fprintf(stream, "fits shim status %d\n", status);
}
