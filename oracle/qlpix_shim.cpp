// The QLens-side shim of INTEGRATION.md as a compilable unit, and a check
// that it builds and links against the unmodified reference objects and
// libqlpix (test infrastructure: built by oracle/Makefile.ref into
// oracle/_ref/qlpix_shim_check; tests/test_shim.py runs it).
//
// qlpix_invert() is what a QLens maintainer would call at the top of the
// Cartesian branch of QLens::invert_image_surface_brightness_map
// (lens.cpp:12431) for inversion_method=dense, interpolating ray tracing,
// curvature regularisation and split image pixels: it builds one qlp_ctx from
// the QLens members the reference's own branch reads -- the image pixel data,
// mask, noise, PSF matrix, source-grid settings and lens list -- and returns
// -2 log(evidence) with chisq0, as the reference's entry point does.
//
// Usage: qlpix_shim_check <script.in>
//   exit 0 and "no device" when the library refuses for want of a GPU
//   (QLP_ERR_NO_DEVICE: there is no CPU fallback), exit 0 and the two values
//   when a GPU evaluated it and agrees with the reference within 1e-6, else 1.
#include <cmath>
#include <cstdio>
#include <complex>
#include <fstream>
#include <iomanip>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>
#include <omp.h>
#include <unistd.h>

#define private public
#define protected public
#include "qlens.h"
#include "pixelgrid.h"
#include "profile.h"
#undef private
#undef protected
#include "../include/qlpix.h"

// QLens's lens list -> the library's lens list, in the 'lens' command's
// parameter order (LensProfile::get_parameters gives angles in degrees).
static bool qlpix_lenses(QLens& q, std::vector<qlp_lens>& out)
{
    out.clear();
    for (int k = 0; k < q.nlens; k++) {
        LensProfile* lp = q.lens_list[k];
        double p[32] = {0};
        lp->get_parameters(p);
        qlp_lens l = {};
        l.plane = q.lens_redshift_idx[k];
        int np = 0;
        if (lp->lenstype == sple_LENS) { l.type = QLP_LENS_SPLE; np = 7; }
        else if (lp->lenstype == SHEAR) { l.type = QLP_LENS_SHEAR; np = 4; }
        else if (lp->lenstype == nfw) {
            np = 6;
            l.type = (lp->parameter_mode == 1) ? QLP_LENS_NFW_M200_C
                     : (lp->parameter_mode == 2) ? QLP_LENS_NFW_M200_RS : QLP_LENS_NFW;
            l.sigma_cr = lp->sigma_cr;
            l.kpc_to_arcsec = lp->kpc_to_arcsec;
            l.critical_density = q.cosmo.critical_density(lp->zlens);
        } else {
            return false;                  // a lens model the library does not carry
        }
        for (int i = 0; i < np; i++) l.p[i] = p[i];
        out.push_back(l);
    }
    return true;
}

int qlpix_invert(QLens& q, qlp_ctx*& ctx, double& chisq0, double& m2logev)
{
    int st = QLP_OK;
    if (ctx == nullptr) {
        ImagePixelData* d = q.image_pixel_data;
        const int mk = q.assigned_mask ? q.assigned_mask[0] : 0;
        std::vector<double> sb, cov;
        std::vector<unsigned char> msk;
        for (int i = 0; i < d->npixels_x; i++)
            for (int j = 0; j < d->npixels_y; j++) {
                sb.push_back(d->surface_brightness[i][j]);
                cov.push_back(q.use_noise_map ? d->covinv_map[i][j] : 0.0);
                msk.push_back(d->in_mask[mk][i][j] ? 1 : 0);
            }
        std::vector<double> psf;
        for (int i = 0; i < q.psf_npixels_x; i++)
            for (int j = 0; j < q.psf_npixels_y; j++) psf.push_back(q.psf_matrix[i][j]);
        qlp_image im = {d->npixels_x, d->npixels_y, d->xvals, d->yvals, sb.data(),
                        q.use_noise_map ? cov.data() : nullptr, q.background_pixel_noise, msk.data()};
        qlp_psf ps = {q.psf_npixels_x, q.psf_npixels_y, psf.data()};
        qlp_srcgrid_opts o;
        qlp_srcgrid_defaults(&o);
        o.nsplit = q.default_imgpixel_nsplit;
        o.npixels_x = q.srcgrid_npixels_x;
        o.npixels_y = q.srcgrid_npixels_y;
        o.auto_sourcegrid = q.auto_sourcegrid ? 1 : 0;
        o.xmin = q.sourcegrid_xmin; o.xmax = q.sourcegrid_xmax;
        o.ymin = q.sourcegrid_ymin; o.ymax = q.sourcegrid_ymax;
        o.limit_xmin = q.sourcegrid_limit_xmin; o.limit_xmax = q.sourcegrid_limit_xmax;
        o.limit_ymin = q.sourcegrid_limit_ymin; o.limit_ymax = q.sourcegrid_limit_ymax;
        o.noise_threshold = q.noise_threshold;
        o.regularization = 1;
        double lam = 0;                                      // the script's 'regparam' (its source object)
        if (q.n_pixellated_src > 0) q.srcgrids[0]->get_specific_parameter("regparam", lam);
        o.regparam = lam;
        ctx = qlp_create(&im, &ps, &o, 0, &st);
        if (!ctx) return st;
        std::vector<qlp_lens> ls;
        if (!qlpix_lenses(q, ls)) return QLP_ERR_ARG;
        qlp_planes pl = {};
        pl.n_planes = 1;
        pl.zfac[0] = 1.0;
        if ((st = qlp_set_lens_model(ctx, ls.data(), (int)ls.size(), &pl)) != QLP_OK) return st;
    }
    qlp_result r;
    st = qlp_eval(ctx, nullptr, 0.0, &r);
    chisq0 = r.chisq0;
    m2logev = r.m2logev;
    return st;
}

int main(int argc, char** argv)
{
    if (argc < 2) { fprintf(stderr, "usage: %s script.in\n", argv[0]); return 2; }
    int nthreads = 1;
    #pragma omp parallel
    {
        #pragma omp master
        nthreads = omp_get_num_threads();
    }
    Grid::allocate_multithreaded_variables(nthreads);
    SourcePixel::allocate_multithreaded_variables(nthreads);
    DelaunayGrid::allocate_multithreaded_variables(nthreads);
    ImagePixelGrid::allocate_multithreaded_variables(nthreads);
    QLens::allocate_multithreaded_variables(nthreads);
    QLens lens;
    lens.set_mpi_params(0, 1);
    lens.set_verbal_mode(false);
    lens.set_quit_after_error(true);
    lens.set_suppress_plots(true);
    if (!lens.open_script_file(argv[1])) { fprintf(stderr, "cannot open script %s\n", argv[1]); return 2; }
    lens.set_quit_after_reading_file(true);
    lens.process_commands(true);
    if (lens.image_pixel_data == nullptr) { fprintf(stderr, "script loaded no image data\n"); return 2; }
    if (lens.n_lens_redshifts != 1) { fprintf(stderr, "the shim check runs single-plane scripts\n"); return 2; }

    qlp_ctx* ctx = nullptr;
    double chisq0 = 0, m2 = 0;
    const int st = qlpix_invert(lens, ctx, chisq0, m2);
    // (the process ends with _exit: QLens's destructor is not part of the check)
    if (st == QLP_ERR_NO_DEVICE) {
        printf("no device: qlp_create refused (%s)\n", qlp_last_error());
        fflush(stdout);
        _exit(0);
    }
    if (st != QLP_OK) { printf("qlpix status %d: %s\n", st, qlp_last_error()); fflush(stdout); _exit(1); }
    double chisq0_ref = 0;
    const double m2_ref = lens.invert_surface_brightness_map_from_data(chisq0_ref, false, true);
    qlp_destroy(ctx);
    const double rel = fabs(m2 - m2_ref) / fabs(m2_ref);
    printf("qlpix -2logev %.10f reference %.10f rel %.2e\n", m2, m2_ref, rel);
    fflush(stdout);
    _exit(rel < 1e-6 ? 0 : 1);
}
