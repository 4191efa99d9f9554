/* fitsio.h -- a stand-in for the CFITSIO calls the reference makes, so that
 * its FITS loaders (ImagePixelData::load_data_fits, load_mask_fits,
 * load_noise_map_fits, QLens::load_psf_fits) can be compiled and run to make
 * golden vectors.  Test infrastructure only.  Reading covers primary and
 * IMAGE-extension HDUs of BITPIX 8/16/32/64/-32/-64 with BSCALE/BZERO;
 * the writing calls fail with a non-zero status.  Only names and signatures
 * follow CFITSIO's public interface; the code is this repository's own. */
#pragma once
#include <cstdio>

struct shim_fitsfile;
typedef struct shim_fitsfile fitsfile;

#define READONLY 0
#define READWRITE 1
#define FLEN_CARD 81
#define TDOUBLE 82
#define DOUBLE_IMG (-64)
#define FLOAT_IMG (-32)

int fits_open_file(fitsfile** fptr, const char* name, int mode, int* status);
int fits_movabs_hdu(fitsfile* fptr, int hdunum, int* exttype, int* status);
int fits_get_hdrspace(fitsfile* fptr, int* nexist, int* nmore, int* status);
int fits_read_record(fitsfile* fptr, int nrec, char* card, int* status);
int fits_get_img_param(fitsfile* fptr, int maxdim, int* bitpix, int* naxis, long* naxes, int* status);
int fits_read_pix(fitsfile* fptr, int datatype, long* firstpix, long nelem, void* nulval, void* array, int* anynul,
                  int* status);
int fits_close_file(fitsfile* fptr, int* status);
void fits_report_error(FILE* stream, int status);
int fits_create_file(fitsfile** fptr, const char* name, int* status);
int fits_create_img(fitsfile* fptr, int bitpix, int naxis, long* naxes, int* status);
int fits_write_key(fitsfile* fptr, int datatype, const char* keyname, void* value, const char* comment, int* status);
int fits_write_pix(fitsfile* fptr, int datatype, long* firstpix, long nelem, void* array, int* status);
int fits_write_comment(fitsfile* fptr, const char* comment, int* status);
