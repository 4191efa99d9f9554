// fits.cpp -- FITS image input for the pixel-likelihood data: the image
// surface brightness, the pixel mask, the noise map and the PSF.
//
// The reference reads these through CFITSIO (ImagePixelData::load_data_fits,
// load_mask_fits, load_noise_map_fits, QLens::load_psf_fits;
// pixelgrid.cpp:6016-6283, 6344-6430, 6512-6650, 6737-6870).  This is a
// self-contained reader of the FITS standard's image HDUs (FITS 4.0: 2880-byte
// blocks of 80-character cards, big-endian pixels of BITPIX 8, 16, 32, 64,
// -32 or -64, physical value = BZERO + BSCALE * stored value), followed by the
// reference's own handling of what it read: the header keywords it looks for,
// the pixel grid it lays over the image, the centring of a smaller mask and
// the PSF's threshold crop and normalisation.
//
// Pixel (i, j) -- i along FITS axis 1, j along axis 2, both from 0 -- goes to
// out[i * ny + j], the library's image layout.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>
#include "qlpix.h"

namespace qlpix {
void set_error(const char* fmt, const char* a, int code);
}

namespace {

constexpr size_t BLOCK = 2880, CARD = 80;

struct Hdu {
    std::vector<std::string> cards;   // header cards before END
    int bitpix = 0, naxis = 0;
    long naxes[3] = {1, 1, 1};
    double bscale = 1.0, bzero = 0.0;
    bool image = false;               // primary array or IMAGE extension
    size_t data_off = 0, data_bytes = 0;
};

std::string keyword(const std::string& c) {
    std::string k = c.substr(0, 8);
    while (!k.empty() && k.back() == ' ') k.pop_back();
    return k;
}

// value field of a "KEYWORD = value / comment" card (columns 11-80), without
// the comment; empty when the card has no value indicator
std::string value_of(const std::string& c)
{
    if (c.size() < 10 || c[8] != '=' || c[9] != ' ') return std::string();
    std::string v = c.substr(10);
    if (!v.empty()) {
        size_t s = v.find_first_not_of(' ');
        if (s != std::string::npos && v[s] == '\'') {
            size_t e = v.find('\'', s + 1);
            return v.substr(s, e == std::string::npos ? std::string::npos : e - s + 1);
        }
        size_t sl = v.find('/');
        if (sl != std::string::npos) v = v.substr(0, sl);
    }
    size_t a = v.find_first_not_of(' '), b = v.find_last_not_of(' ');
    return (a == std::string::npos) ? std::string() : v.substr(a, b - a + 1);
}

bool num(const std::string& s, double* out)
{
    if (s.empty()) return false;
    std::string t = s;
    for (char& ch : t) if (ch == 'D' || ch == 'd') ch = 'E';      // Fortran exponent
    char* end = nullptr;
    const double v = strtod(t.c_str(), &end);
    if (end == t.c_str()) return false;
    *out = v;
    return true;
}

int parse(const std::vector<unsigned char>& f, std::vector<Hdu>& hdus, int want)
{
    size_t off = 0;
    while (off + BLOCK <= f.size() && (int)hdus.size() < want) {
        Hdu h;
        bool end = false;
        while (!end) {
            if (off + BLOCK > f.size()) return QLP_ERR_ARG;
            for (size_t k = 0; k < BLOCK / CARD; k++) {
                std::string c((const char*)&f[off + k * CARD], CARD);
                if (keyword(c) == "END") { end = true; break; }
                h.cards.push_back(c);
            }
            off += BLOCK;
        }
        long pcount = 0, gcount = 1;
        bool first = hdus.empty(), simple = false;
        std::string xt;
        for (const std::string& c : h.cards) {
            const std::string k = keyword(c), v = value_of(c);
            double d = 0;
            if (k == "SIMPLE") simple = (v == "T");
            else if (k == "XTENSION") xt = v;
            else if (k == "BITPIX" && num(v, &d)) h.bitpix = (int)d;
            else if (k == "NAXIS" && num(v, &d)) h.naxis = (int)d;
            else if (k.size() > 5 && k.compare(0, 5, "NAXIS") == 0 && num(v, &d)) {
                const int ax = atoi(k.c_str() + 5);
                if (ax >= 1 && ax <= 3) h.naxes[ax - 1] = (long)d;
            } else if (k == "PCOUNT" && num(v, &d)) pcount = (long)d;
            else if (k == "GCOUNT" && num(v, &d)) gcount = (long)d;
            else if (k == "BSCALE" && num(v, &d)) h.bscale = d;
            else if (k == "BZERO" && num(v, &d)) h.bzero = d;
        }
        if (first && !simple) return QLP_ERR_ARG;
        h.image = first || xt == "'IMAGE   '" || xt == "'IMAGE'";
        const int b = h.bitpix;
        if (b != 8 && b != 16 && b != 32 && b != 64 && b != -32 && b != -64) return QLP_ERR_ARG;
        if (h.naxis < 0 || h.naxis > 999) return QLP_ERR_ARG;
        size_t n = 0;
        if (h.naxis > 0) {
            n = 1;
            for (int a = 1; a <= h.naxis; a++) {
                long na = 1;
                if (a <= 3) na = h.naxes[a - 1];
                else {   // axes past the third only size the data unit
                    for (const std::string& c : h.cards) {
                        double d;
                        if (keyword(c) == "NAXIS" + std::to_string(a) && num(value_of(c), &d)) na = (long)d;
                    }
                }
                if (na < 0) return QLP_ERR_ARG;
                n *= (size_t)na;
            }
        }
        h.data_bytes = (size_t)(std::abs(b) / 8) * (size_t)gcount * ((size_t)pcount + n);
        if (h.naxis == 0) h.data_bytes = 0;
        h.data_off = off;
        off += (h.data_bytes + BLOCK - 1) / BLOCK * BLOCK;
        hdus.push_back(h);
    }
    return ((int)hdus.size() >= want) ? QLP_OK : QLP_ERR_ARG;
}

double stored(const unsigned char* p, int bitpix)
{
    uint64_t u = 0;
    const int nb = std::abs(bitpix) / 8;
    for (int k = 0; k < nb; k++) u = (u << 8) | p[k];        // big-endian
    switch (bitpix) {
    case 8: return (double)(unsigned)u;
    case 16: return (double)(int16_t)(uint16_t)u;
    case 32: return (double)(int32_t)(uint32_t)u;
    case 64: return (double)(int64_t)u;
    case -32: { uint32_t w = (uint32_t)u; float x; memcpy(&x, &w, 4); return (double)x; }
    default: { double x; memcpy(&x, &u, 8); return x; }
    }
}

bool slurp(const char* path, std::vector<unsigned char>& f)
{
    FILE* fp = fopen(path, "rb");
    if (!fp) return false;
    unsigned char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), fp)) > 0) f.insert(f.end(), buf, buf + n);
    fclose(fp);
    return true;
}

// The 2-D image of HDU hdu (1 = primary): its first two axes, as the
// reference reads it (fits_get_img_param with two dimensions, then one
// fits_read_pix row per axis-2 index: pixelgrid.cpp:6133-6241).
int read_image(const char* path, int hdu, std::vector<double>& pix, int* nx, int* ny, Hdu* hout)
{
    if (!path || hdu < 1) return QLP_ERR_ARG;
    std::vector<unsigned char> f;
    if (!slurp(path, f)) {
        qlpix::set_error("%s (%d)", "cannot open FITS file", 0);
        return QLP_ERR_ARG;
    }
    std::vector<Hdu> hdus;
    if (parse(f, hdus, hdu) != QLP_OK) {
        qlpix::set_error("%s (%d)", "not a readable FITS file or no such HDU", hdu);
        return QLP_ERR_ARG;
    }
    const Hdu& h = hdus[hdu - 1];
    if (!h.image || h.naxis == 0) {
        qlpix::set_error("%s (%d)", "HDU holds no image (only 1D or 2D images are supported)", hdu);
        return QLP_ERR_ARG;
    }
    const long n1 = h.naxes[0], n2 = (h.naxis >= 2) ? h.naxes[1] : 1;
    if (n1 < 1 || n2 < 1 || n1 * n2 > (1L << 30)) return QLP_ERR_ARG;
    const size_t bpp = (size_t)(std::abs(h.bitpix) / 8);
    if (h.data_off + (size_t)n1 * n2 * bpp > f.size()) {
        qlpix::set_error("%s (%d)", "FITS data unit is truncated", hdu);
        return QLP_ERR_ARG;
    }
    pix.assign((size_t)n1 * n2, 0.0);
    const bool scaled = !(h.bscale == 1.0 && h.bzero == 0.0);
    for (long j = 0; j < n2; j++)
        for (long i = 0; i < n1; i++) {
            const double s = stored(&f[h.data_off + ((size_t)j * n1 + i) * bpp], h.bitpix);
            pix[(size_t)i * n2 + j] = scaled ? h.bzero + h.bscale * s : s;
        }
    *nx = (int)n1;
    *ny = (int)n2;
    if (hout) *hout = h;
    return QLP_OK;
}

// The header keywords QLens reads from a data image, in its order of tests
// (pixelgrid.cpp:6059-6116): a card holding "ql: " or "mk: " opens a run of
// COMMENT cards (model description, parameter markers) that ends the scan at
// its first non-COMMENT card; otherwise a card holding "PXSIZE ", "PXNOISE ",
// "PSFSIG ", "ZSRC " or "ZLENS " gives that value, read from column 12 on.
void scan_keys(const Hdu& h, qlp_fits_info* info)
{
    memset(info, 0, sizeof(*info));
    info->bitpix = h.bitpix;
    info->naxis = h.naxis;
    bool in_ql = false, in_mk = false;
    auto has = [](const std::string& c, const char* s) { return c.find(s) != std::string::npos; };
    auto val = [](const std::string& c) { return c.size() > 11 ? strtod(c.c_str() + 11, nullptr) : 0.0; };
    for (const std::string& c : h.cards) {
        if (in_ql) {
            if (!has(c, "COMMENT")) break;
            if (has(c, "mk: ") || has(c, "MK: ")) { in_mk = true; in_ql = false; }
        } else if (in_mk) {
            if (!has(c, "COMMENT")) break;
        } else if (has(c, "ql: ") || has(c, "QL: ")) {
            in_ql = true;
        } else if (has(c, "mk: ") || has(c, "MK: ")) {
            in_mk = true;
        } else if (has(c, "PXSIZE ")) {
            info->pxsize = val(c); info->has_pxsize = 1;
        } else if (has(c, "PXNOISE ")) {
            info->pxnoise = val(c); info->has_pxnoise = 1;
        } else if (has(c, "PSFSIG ")) {
            info->psfsig = val(c); info->has_psfsig = 1;
        } else if (has(c, "ZSRC ")) {
            info->zsrc = val(c); info->has_zsrc = 1;
        } else if (has(c, "ZLENS ")) {
            info->zlens = val(c); info->has_zlens = 1;
        }
    }
}

}  // namespace

extern "C" {

int qlp_fits_read_image(const char* path, int hdu, double* pix, long cap, int* nx, int* ny, qlp_fits_info* info)
{
    if (!nx || !ny) return QLP_ERR_ARG;
    std::vector<double> p;
    Hdu h;
    int e = read_image(path, hdu, p, nx, ny, &h);
    if (e != QLP_OK) return e;
    if (info) scan_keys(h, info);
    if (!pix) return QLP_OK;                         // sizes only
    if (cap < (long)p.size()) return QLP_ERR_ARG;
    memcpy(pix, p.data(), p.size() * sizeof(double));
    return QLP_OK;
}

int qlp_load_data_fits(const char* path, int hdu, double pixel_size, double xmin, double xmax, double ymin,
                       double ymax, double* xvals, double* yvals, double* data, long cap, int* nx, int* ny,
                       qlp_fits_info* info)
{
    if (!nx || !ny) return QLP_ERR_ARG;
    std::vector<double> p;
    Hdu h;
    int e = read_image(path, hdu, p, nx, ny, &h);
    if (e != QLP_OK) return e;
    qlp_fits_info inf;
    scan_keys(h, &inf);
    if (info) *info = inf;
    if (!xvals && !yvals && !data) return QLP_OK;   // sizes only
    if (!xvals || !yvals || !data || cap < (long)p.size()) return QLP_ERR_ARG;
    // the pixel grid (pixelgrid.cpp:6187-6206): a PXSIZE card, else the
    // caller's pixel size, gives square pixels centred on the origin; without
    // either the image spans [xmin, xmax] x [ymin, ymax].  Edges accumulate
    // the step, as the reference's loop does.
    const int npx = *nx, npy = *ny;
    double ps = inf.has_pxsize ? inf.pxsize : pixel_size;
    double xstep, ystep;
    if (inf.has_pxsize || pixel_size > 0) {
        xstep = ystep = ps;
        xmax = 0.5 * npx * ps;
        ymax = 0.5 * npy * ps;
        xmin = -xmax;
        ymin = -ymax;
    } else {
        if (!(xmax > xmin && ymax > ymin)) {
            qlpix::set_error("%s (%d)", "no pixel size in the file or the call, and no image bounds", 0);
            return QLP_ERR_ARG;
        }
        xstep = (xmax - xmin) / npx;
        ystep = (ymax - ymin) / npy;
    }
    double x = xmin, y = ymin;
    for (int i = 0; i <= npx; i++, x += xstep) xvals[i] = x;
    for (int j = 0; j <= npy; j++, y += ystep) yvals[j] = y;
    memcpy(data, p.data(), p.size() * sizeof(double));
    return QLP_OK;
}

int qlp_load_mask_fits(const char* path, int nx, int ny, int add, unsigned char* mask, int* n_in_mask)
{
    if (!mask || nx < 1 || ny < 1) return QLP_ERR_ARG;
    std::vector<double> p;
    int mx = 0, my = 0;
    int e = read_image(path, 1, p, &mx, &my, nullptr);
    if (e != QLP_OK) return e;
    // a smaller mask is centred on the image (pixelgrid.cpp:6542-6551); a
    // larger one is an error
    int ox = 0, oy = 0;
    if (mx != nx || my != ny) {
        if (mx < nx && my < ny) {
            ox = (nx - mx) / 2;
            oy = (ny - my) / 2;
        } else {
            qlpix::set_error("%s (%d)", "mask file has more pixels than the image along x and/or y", 0);
            return QLP_ERR_ARG;
        }
    }
    // zero unsets a pixel (unless adding), anything else sets it; pixels the
    // file does not cover keep their state (pixelgrid.cpp:6618-6630).  The
    // count returned is of every set pixel of the result.
    for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++) {
            unsigned char& m = mask[(size_t)(i + ox) * ny + (j + oy)];
            if (p[(size_t)i * my + j] == 0.0) {
                if (!add) m = 0;
            } else {
                m = 1;
            }
        }
    if (n_in_mask) {
        int n = 0;
        for (long k = 0; k < (long)nx * ny; k++) n += mask[k] ? 1 : 0;
        *n_in_mask = n;
    }
    return QLP_OK;
}

int qlp_load_noise_map_fits(const char* path, int hdu, int nx, int ny, double* covinv, double* noise_min)
{
    if (!covinv || nx < 1 || ny < 1) return QLP_ERR_ARG;
    std::vector<double> p;
    int mx = 0, my = 0;
    int e = read_image(path, hdu, p, &mx, &my, nullptr);
    if (e != QLP_OK) return e;
    if (mx != nx || my != ny) {
        qlpix::set_error("%s (%d)", "noise map does not match the image's pixel counts", 0);
        return QLP_ERR_ARG;
    }
    // C^-1 = 1 / sigma^2 per pixel; the smallest sigma is the background
    // noise (pixelgrid.cpp:6398-6418)
    double mn = 1e30;
    for (size_t k = 0; k < p.size(); k++) {
        covinv[k] = 1.0 / (p[k] * p[k]);
        if (p[k] < mn) mn = p[k];
    }
    if (noise_min) *noise_min = mn;
    return QLP_OK;
}

int qlp_load_psf_fits(const char* path, double threshold, double* psf, long cap, int* pnx, int* pny)
{
    if (!pnx || !pny) return QLP_ERR_ARG;
    std::vector<double> p;
    int nx = 0, ny = 0;
    int e = read_image(path, 1, p, &nx, &ny, nullptr);
    if (e != QLP_OK) return e;
    // QLens::load_psf_fits (pixelgrid.cpp:6806-6857): the box around the
    // central pixel (nx/2, ny/2) that holds every pixel above threshold x
    // peak, made symmetric about the centre with half-widths
    // (extent + 1) / 2, then normalised to unit sum
    double peak = -1e30;
    for (double v : p) if (v > peak) peak = v;
    const int imid = nx / 2, jmid = ny / 2;
    int imin = imid, imax = imid, jmin = jmid, jmax = jmid;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            if (p[(size_t)i * ny + j] > threshold * peak) {
                if (i < imin) imin = i;
                if (i > imax) imax = i;
                if (j < jmin) jmin = j;
                if (j > jmax) jmax = j;
            }
    const int hx = (imax - imin + 1) / 2, hy = (jmax - jmin + 1) / 2;
    const int onx = 2 * hx + 1, ony = 2 * hy + 1;
    if (imid - hx < 0 || imid + hx >= nx || jmid - hy < 0 || jmid + hy >= ny) {
        // an even-sized PSF whose signal reaches its far edge: the
        // reference's symmetric box would read past the array
        qlpix::set_error("%s (%d)", "PSF above threshold reaches past the symmetric box about the centre", 0);
        return QLP_ERR_ARG;
    }
    *pnx = onx;
    *pny = ony;
    if (!psf) return QLP_OK;                         // sizes only
    if (cap < (long)onx * ony) return QLP_ERR_ARG;
    double norm = 0;
    for (int a = 0; a < onx; a++)
        for (int b = 0; b < ony; b++) norm += p[(size_t)(imid - hx + a) * ny + (jmid - hy + b)];
    for (int a = 0; a < onx; a++)
        for (int b = 0; b < ony; b++)
            psf[(size_t)a * ony + b] = p[(size_t)(imid - hx + a) * ny + (jmid - hy + b)] / norm;
    return QLP_OK;
}

}  // extern "C"
