/* fitsio.h -- declarations of the cfitsio subset the reference calls
 * (src/COREMOD_iofits/COREMOD_iofits.c); implemented by shim_fitsio.c
 * (primary-HDU images only).  Checker build only. */
#ifndef ATMREF_FITSIO_SHIM_H
#define ATMREF_FITSIO_SHIM_H
#include <stdio.h>
typedef struct atmref_fits fitsfile;
#define READONLY 0
#define READWRITE 1
#define TBIT 1
#define TBYTE 11
#define TLOGICAL 14
#define TSTRING 16
#define TUSHORT 20
#define TSHORT 21
#define TINT 31
#define TLONG 41
#define TFLOAT 42
#define TDOUBLE 82
#define TCOMPLEX 83
#define TDBLCOMPLEX 163
#define BYTE_IMG 8
#define SHORT_IMG 16
#define USHORT_IMG 20
#define LONG_IMG 32
#define FLOAT_IMG (-32)
#define DOUBLE_IMG (-64)
#define FLEN_FILENAME 1025
#define FLEN_KEYWORD 75
#define FLEN_CARD 81
#define FLEN_VALUE 71
#define FLEN_COMMENT 73
#define FLEN_ERRMSG 81
#define FLEN_STATUS 31
#define KEY_NO_EXIST 202
#define FILE_NOT_OPENED 104
#define FILE_NOT_CREATED 105
int fits_open_file(fitsfile** f, const char* name, int mode, int* status);
int fits_close_file(fitsfile* f, int* status);
int fits_create_file(fitsfile** f, const char* name, int* status);
int fits_create_img(fitsfile* f, int bitpix, int naxis, long* naxes, int* status);
int fits_read_key(fitsfile* f, int datatype, const char* key, void* value, char* comment, int* status);
int fits_read_keyword(fitsfile* f, const char* key, char* value, char* comment, int* status);
int fits_set_bscale(fitsfile* f, double scale, double zero, int* status);
int fits_read_img(fitsfile* f, int datatype, long firstelem, long nelem, void* nulval, void* array, int* anynul,
                  int* status);
int fits_write_img(fitsfile* f, int datatype, long firstelem, long nelem, void* array, int* status);
void fits_get_errstatus(int status, char* text);
void fits_report_error(FILE* stream, int status);
#endif
