// fitsio_shim.cpp -- the reading half of the CFITSIO stand-in declared in
// fitsio.h (test infrastructure: it lets the reference's own FITS loaders run
// to make golden vectors).  Written independently of the library's reader
// (qlens_gb300/csrc/fits.cpp) so that the two check each other.
#include "fitsio.h"
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

struct shim_fitsfile {
    std::vector<unsigned char> bytes;
    std::vector<size_t> hdr_start, data_start;   // per HDU
    std::vector<int> ncards;
    int cur = 0;                                 // current HDU, 0-based
};

static const int BAD = 104;   // a non-zero status ("could not open")

static long card_int(const unsigned char* c)  // integer value of a card
{
    char buf[72];
    memcpy(buf, c + 10, 70);
    buf[70] = 0;
    return strtol(buf, nullptr, 10);
}

static double card_real(const unsigned char* c)
{
    char buf[72];
    memcpy(buf, c + 10, 70);
    buf[70] = 0;
    for (char* p = buf; *p; p++) if (*p == 'D') *p = 'E';
    return strtod(buf, nullptr);
}

static bool key_is(const unsigned char* c, const char* k)
{
    size_t n = strlen(k);
    if (memcmp(c, k, n) != 0) return false;
    for (size_t i = n; i < 8; i++) if (c[i] != ' ') return false;
    return true;
}

int fits_open_file(fitsfile** fptr, const char* name, int, int* status)
{
    if (*status) return *status;
    FILE* f = fopen(name, "rb");
    if (!f) return *status = BAD;
    shim_fitsfile* s = new shim_fitsfile;
    int ch;
    while ((ch = fgetc(f)) != EOF) s->bytes.push_back((unsigned char)ch);
    fclose(f);
    size_t off = 0;
    while (off + 2880 <= s->bytes.size()) {
        size_t h = off;
        int n = 0;
        long bitpix = 0, naxis = 0, pc = 0, gc = 1, prod = 1;
        bool end = false;
        while (!end && off + 2880 <= s->bytes.size()) {
            for (int k = 0; k < 36; k++) {
                const unsigned char* c = &s->bytes[off + 80 * k];
                if (key_is(c, "END")) { end = true; break; }
                n++;
                if (key_is(c, "BITPIX")) bitpix = card_int(c);
                else if (key_is(c, "NAXIS")) naxis = card_int(c);
                else if (memcmp(c, "NAXIS", 5) == 0 && c[5] >= '1' && c[5] <= '9') prod *= card_int(c);
                else if (key_is(c, "PCOUNT")) pc = card_int(c);
                else if (key_is(c, "GCOUNT")) gc = card_int(c);
            }
            off += 2880;
        }
        if (!end) break;
        s->hdr_start.push_back(h);
        s->ncards.push_back(n);
        s->data_start.push_back(off);
        long nbytes = (naxis > 0) ? labs(bitpix) / 8 * gc * (pc + prod) : 0;
        off += (size_t)((nbytes + 2879) / 2880) * 2880;
    }
    if (s->hdr_start.empty()) { delete s; return *status = BAD; }
    *fptr = s;
    return 0;
}

int fits_movabs_hdu(fitsfile* f, int hdunum, int* exttype, int* status)
{
    if (*status) return *status;
    if (hdunum < 1 || hdunum > (int)f->hdr_start.size()) return *status = 107;
    f->cur = hdunum - 1;
    if (exttype) *exttype = 0;
    return 0;
}

int fits_get_hdrspace(fitsfile* f, int* nexist, int* nmore, int* status)
{
    if (*status) return *status;
    if (nexist) *nexist = f->ncards[f->cur];
    if (nmore) *nmore = 0;
    return 0;
}

int fits_read_record(fitsfile* f, int nrec, char* card, int* status)
{
    if (*status) return *status;
    if (nrec < 1 || nrec > f->ncards[f->cur]) return *status = 203;
    memcpy(card, &f->bytes[f->hdr_start[f->cur] + 80 * (nrec - 1)], 80);
    card[80] = 0;
    for (int i = 79; i >= 0 && card[i] == ' '; i--) card[i] = 0;   // trailing blanks dropped
    return 0;
}

struct ImgHdr { long bitpix = 0, naxis = 0, n[9] = {1, 1, 1, 1, 1, 1, 1, 1, 1}; double bscale = 1, bzero = 0; };

static ImgHdr img_hdr(fitsfile* f)
{
    ImgHdr h;
    const unsigned char* c0 = &f->bytes[f->hdr_start[f->cur]];
    for (int k = 0; k < f->ncards[f->cur]; k++) {
        const unsigned char* c = c0 + 80 * k;
        if (key_is(c, "BITPIX")) h.bitpix = card_int(c);
        else if (key_is(c, "NAXIS")) h.naxis = card_int(c);
        else if (memcmp(c, "NAXIS", 5) == 0 && c[5] >= '1' && c[5] <= '9' && c[6] == ' ') h.n[c[5] - '1'] = card_int(c);
        else if (key_is(c, "BSCALE")) h.bscale = card_real(c);
        else if (key_is(c, "BZERO")) h.bzero = card_real(c);
    }
    return h;
}

int fits_get_img_param(fitsfile* f, int maxdim, int* bitpix, int* naxis, long* naxes, int* status)
{
    if (*status) return *status;
    ImgHdr h = img_hdr(f);
    *bitpix = (int)h.bitpix;
    *naxis = (int)h.naxis;
    for (int a = 0; a < maxdim && a < h.naxis; a++) naxes[a] = h.n[a];
    return 0;
}

int fits_read_pix(fitsfile* f, int datatype, long* firstpix, long nelem, void*, void* array, int* anynul, int* status)
{
    if (*status) return *status;
    if (datatype != TDOUBLE) return *status = 410;
    ImgHdr h = img_hdr(f);
    const long nb = labs(h.bitpix) / 8;
    long first = firstpix[0] - 1, stride = 1;
    for (int a = 1; a < h.naxis; a++) {
        stride *= h.n[a - 1];
        first += (firstpix[a] - 1) * stride;
    }
    double* out = (double*)array;
    const size_t base = f->data_start[f->cur];
    for (long e = 0; e < nelem; e++) {
        size_t at = base + (size_t)(first + e) * nb;
        if (at + nb > f->bytes.size()) return *status = 108;
        uint64_t u = 0;
        for (long b = 0; b < nb; b++) u = u * 256u + f->bytes[at + b];
        double v;
        if (h.bitpix == 8) v = (double)u;
        else if (h.bitpix == 16) v = (double)(int16_t)(uint16_t)u;
        else if (h.bitpix == 32) v = (double)(int32_t)(uint32_t)u;
        else if (h.bitpix == 64) v = (double)(int64_t)u;
        else if (h.bitpix == -32) { uint32_t w = (uint32_t)u; float x; memcpy(&x, &w, 4); v = x; }
        else { double x; memcpy(&x, &u, 8); v = x; }
        out[e] = (h.bscale == 1.0 && h.bzero == 0.0) ? v : h.bzero + h.bscale * v;
    }
    if (anynul) *anynul = 0;
    return 0;
}

int fits_close_file(fitsfile* f, int* status)
{
    delete f;
    return *status;
}

void fits_report_error(FILE* stream, int status) { fprintf(stream, "FITS stand-in: status %d\n", status); }

int fits_create_file(fitsfile**, const char*, int* status) { return *status ? *status : (*status = 105); }
int fits_create_img(fitsfile*, int, int, long*, int* status) { return *status ? *status : (*status = 105); }
int fits_write_key(fitsfile*, int, const char*, void*, const char*, int* status) { return *status ? *status : (*status = 105); }
int fits_write_pix(fitsfile*, int, long*, long, void*, int* status) { return *status ? *status : (*status = 105); }
int fits_write_comment(fitsfile*, const char*, int* status) { return *status ? *status : (*status = 105); }
