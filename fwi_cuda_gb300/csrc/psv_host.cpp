// psv_host.cpp -- host-side preprocessing and file formats of the engine.
//
// FP64 restatements of the reference's setup code (src/h_preproc_PSV.cpp,
// src/h_holbergcoeff.cpp, src/h_checkfd_ssg_elastic.cpp) and readers /
// writers of its binary files (src/h_io_PSV.cpp).  Compiled with
// -ffp-contract=off so the profiles are bitwise equal to the reference's.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fwi_psv.h"
#include "psv_checkpoint.hpp"
#include "psv_internal.h"

namespace {
// The reference's PI (include/h_globvar.hpp:39); CPML, wavelet and taper use it.
constexpr double REF_PI = 3.14159265;

// Holberg (1987) staggered-grid coefficients in the layout of the DENISE code
// family, which the reference also uses (src/h_holbergcoeff.cpp:25-75): row =
// maximum relative group-velocity error (0 Taylor, 1: 0.1 %, 2: 0.5 %,
// 3: 1 %, 4: 3 %), entry 0 = minimum points per wavelength, 1..6 = weights.
const double kHolberg[5][6][7] = {
    {{23.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0},
     {8.0, 9.0 / 8.0, -1.0 / 24.0, 0.0, 0.0, 0.0, 0.0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0.0, 0.0, 0.0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0.0, 0.0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0,
      35.0 / 294912.0, 0.0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0, -5445.0 / 1835008.0,
      847.0 / 2359296.0, -63.0 / 2883584.0}},
    {{49.7, 1.0010, 0.0, 0.0, 0.0, 0.0, 0.0},
     {8.32, 1.1382, -0.046414, 0.0, 0.0, 0.0, 0.0},
     {4.77, 1.1965, -0.078804, 0.0081781, 0.0, 0.0, 0.0},
     {3.69, 1.2257, -0.099537, 0.018063, -0.0026274, 0.0, 0.0},
     {3.19, 1.2415, -0.11231, 0.026191, -0.0064682, 0.001191, 0.0},
     {2.91, 1.2508, -0.12034, 0.032131, -0.010142, 0.0029857, -0.00066667}},
    {{22.2, 1.0050, 0.0, 0.0, 0.0, 0.0, 0.0},
     {5.65, 1.1534, -0.052806, 0.0, 0.0, 0.0, 0.0},
     {3.74, 1.2111, -0.088313, 0.011768, 0.0, 0.0, 0.0},
     {3.11, 1.2367, -0.10815, 0.023113, -0.0046905, 0.0, 0.0},
     {2.80, 1.2496, -0.11921, 0.031130, -0.0093272, 0.0025161, 0.0},
     {2.62, 1.2568, -0.12573, 0.036423, -0.013132, 0.0047484, -0.0015979}},
    {{15.8, 1.0100, 0.0, 0.0, 0.0, 0.0, 0.0},
     {4.80, 1.1640, -0.057991, 0.0, 0.0, 0.0, 0.0},
     {3.39, 1.2192, -0.094070, 0.014608, 0.0, 0.0, 0.0},
     {2.90, 1.2422, -0.11269, 0.026140, -0.0064054, 0.0, 0.0},
     {2.65, 1.2534, -0.12257, 0.033755, -0.011081, 0.0036784, 0.0},
     {2.51, 1.2596, -0.12825, 0.038550, -0.014763, 0.0058619, -0.0024538}},
    {{9.16, 1.0300, 0.0, 0.0, 0.0, 0.0, 0.0},
     {3.47, 1.1876, -0.072518, 0.0, 0.0, 0.0, 0.0},
     {2.91, 1.2341, -0.10569, 0.022589, 0.0, 0.0, 0.0},
     {2.61, 1.2516, -0.12085, 0.032236, -0.011459, 0.0, 0.0},
     {2.45, 1.2596, -0.12829, 0.038533, -0.014681, 0.0072580, 0.0},
     {2.36, 1.2640, -0.13239, 0.042217, -0.017803, 0.0081959, -0.0051848}},
};

// One side of the CPML profile (cpml_PSV, src/h_preproc_PSV.cpp:134-194 and
// :199-261; the two sides differ only in the abscissa).
void cpml_point(int i, bool low, double xorigin, double thickness, double d0, double npower,
                double k_max, double alpha_max, double dt, double dh, double *a, double *b,
                double *K, double *a_half, double *b_half, double *K_half)
{
    double d = 0, d_half = 0, alpha_prime = 0.0, alpha_prime_half = 0.0, x;
    const double xval = dh * (double)i;
    x = low ? xorigin - xval : xval - xorigin;
    if (x >= 0) {
        const double xn = x / thickness;
        d = d0 * pow(xn, npower);
        K[i] = 1.0 + (k_max - 1.0) * pow(xn, npower);
        alpha_prime = alpha_max * (1.0 - xn);
    }
    x = low ? xorigin - (xval + dh / 2.0) : (xval + dh / 2.0) - xorigin;
    if (x >= 0) {
        const double xn = x / thickness;
        d_half = d0 * pow(xn, npower);
        K_half[i] = 1.0 + (k_max - 1.0) * pow(xn, npower);
        alpha_prime_half = alpha_max * (1.0 - xn);
    }
    if (alpha_prime < 0.0) alpha_prime = 0.0;
    if (alpha_prime_half < 0.0) alpha_prime_half = 0.0;
    b[i] = exp(-(d / K[i] + alpha_prime) * dt);
    b_half[i] = exp(-(d_half / K_half[i] + alpha_prime_half) * dt);
    if (fabs(d) > 1.0e-6) a[i] = d * (b[i] - 1.0) / (K[i] * (d + K[i] * alpha_prime));
    if (fabs(d_half) > 1.0e-6)
        a_half[i] = d_half * (b_half[i] - 1.0) / (K_half[i] * (d_half + K_half[i] * alpha_prime_half));
}
}  // namespace

extern "C" int psv_holbergcoeff(int fdorder, int maxrelerror, double *hc7)
{
    if (!hc7 || fdorder < 2 || fdorder > 12 || (fdorder & 1) || maxrelerror < 0 || maxrelerror > 4)
        return psv::fail(PSV_ERR_ARG, "holbergcoeff: fdorder must be even in [2, 12], maxrelerror in [0, 4]");
    const int nl = fdorder / 2 - 1;
    for (int i = 0; i <= 6; i++) hc7[i] = kHolberg[maxrelerror][nl][i];
    return PSV_OK;
}

extern "C" int psv_cpml_PSV(double *a, double *b, double *K, double *a_half, double *b_half,
                            double *K_half, double npower, double damp_v_PML, double rcoef,
                            double k_max_PML, double freq, int npml_h1, int npml_h2, int fpad,
                            int nh, double dt, double dh)
{
    if (!a || !b || !K || !a_half || !b_half || !K_half || nh <= 0)
        return psv::fail(PSV_ERR_ARG, "cpml_PSV: null array or nh <= 0");
    if (npml_h1 < 0 || npml_h2 < 0 || fpad < 0 || npml_h1 + fpad >= nh ||
        nh - fpad - npml_h2 - 1 < 0)
        return psv::fail(PSV_ERR_ARG, "cpml_PSV: PML layers do not fit the axis");
    const double alpha_max_PML = 2.0 * REF_PI * (freq / 2.0);
    for (int ih = 0; ih < nh; ih++) {
        a[ih] = 0.0; a_half[ih] = 0.0;
        b[ih] = 1.0; b_half[ih] = 1.0;
        K[ih] = 1.0; K_half[ih] = 1.0;
    }
    if (npml_h1) {
        const double thickness = npml_h1 * dh;
        const double d0 = -(npower + 1) * damp_v_PML * log(rcoef) / (2.0 * thickness);
        for (int i = fpad; i <= npml_h1 + fpad; i++)
            cpml_point(i, true, thickness, thickness, d0, npower, k_max_PML, alpha_max_PML, dt, dh,
                       a, b, K, a_half, b_half, K_half);
    }
    if (npml_h2) {
        const double thickness = npml_h2 * dh;
        const double xorigin = dh * (nh - fpad - npml_h2 - 1);
        const double d0 = -(npower + 1) * damp_v_PML * log(rcoef) / (2.0 * thickness);
        for (int i = nh - fpad - npml_h2 - 1; i < nh - fpad; i++)
            cpml_point(i, false, xorigin, thickness, d0, npower, k_max_PML, alpha_max_PML, dt, dh,
                       a, b, K, a_half, b_half, K_half);
    }
    return PSV_OK;
}

extern "C" int psv_wavelet(double *signal, int nt, double dt, double amp, double fc, double ts,
                           int shape)
{
    if (!signal || nt < 0) return psv::fail(PSV_ERR_ARG, "wavelet: null signal or nt < 0");
    if (shape != 1) return psv::fail(PSV_ERR_UNSUPPORTED, "wavelet: only shape 1 (Ricker) exists");
    const double fci = 1.0 / fc;
    for (int it = 0; it < nt; it++) {
        const double t = it * dt;
        const double tau = REF_PI * (t - 1.5 * fci - ts) / (1.5 * fci);
        signal[it] = amp * (1.0 - 2.0 * tau * tau) * exp(-2.0 * tau * tau);
    }
    return PSV_OK;
}

extern "C" int psv_checkfd_ssg_elastic(int nz, int nx, double dh, double dt, double ts, int fw,
                                       const double *rho, const double *lam, const double *mu,
                                       const double *hc7, double *out4)
{
    if (!rho || !lam || !mu || !hc7 || !out4 || nz <= 1 || nx <= 1)
        return psv::fail(PSV_ERR_ARG, "checkfd: null array or empty grid");
    double cmax_p = 0.0, cmin_p = 1e9, cmax_s = 0.0, cmin_s = 1e9;
    const int i2 = std::min(nx - fw, nx - 1), j2 = std::min(nz - fw, nz - 1);
    for (int i = 1 + fw; i <= i2; i++)
        for (int j = 1; j <= j2; j++) {
            const size_t k = (size_t)j * nx + i;
            if (fabs(mu[k]) < 1.0e-9) continue;
            double c = sqrt(mu[k] / rho[k]);
            cmax_s = std::max(cmax_s, c);
            cmin_s = std::min(cmin_s, c);
            c = sqrt((lam[k] + 2.0 * mu[k]) / rho[k]);
            cmax_p = std::max(cmax_p, c);
            cmin_p = std::min(cmin_p, c);
        }
    const double cmax = cmax_s > cmax_p ? cmax_s : cmax_p;
    const double cmin = cmin_s < cmin_p ? cmin_s : cmin_p;
    const double gamma =
        fabs(hc7[1]) + fabs(hc7[2]) + fabs(hc7[3]) + fabs(hc7[4]) + fabs(hc7[5]) + fabs(hc7[6]);
    out4[0] = dh / (sqrt(2.0) * gamma * cmax);
    out4[1] = cmin / (12.0 * (2.0 * ts));
    out4[2] = cmax;
    out4[3] = cmin;
    if ((fw > nx - fw) || (fw > nz - fw))
        return psv::fail(PSV_ERR_ARG, "checkfd: absorbing frame wider than the domain");
    if (dt > out4[0]) return psv::fail(PSV_ERR_CFL, "checkfd: dt above the stability limit");
    return PSV_OK;
}

// ---------------------------------------------------------------------------
// Step-length search (src/cpu/n_step_length_PSV.cpp:13-209, 461-518).
// ---------------------------------------------------------------------------
extern "C" double psv_calc_opt_step(const double *L2, const double *sl)
{
    double A[3][3], b[3], x[3];
    for (int i = 0; i < 3; i++) {
        A[i][2] = sl[i] * sl[i];
        A[i][1] = sl[i];
        A[i][0] = 1.0;
        b[i] = L2[i];
    }
    for (int k = 0; k < 2; k++)  // Gauss elimination, no pivoting (n_solvelin.hpp:28-35)
        for (int r = k; r < 2; r++) {
            const double a = A[r + 1][k] / A[k][k];
            for (int m = 0; m < 3; m++) A[r + 1][m] = A[r + 1][m] - a * A[k][m];
            b[r + 1] = b[r + 1] - a * b[k];
        }
    for (int k = 2; k >= 0; k--) {
        double c = b[k];
        for (int m = 2; m > k; m--) c = c - A[k][m] * x[m];
        x[k] = c / A[k][k];
    }
    double opteps = -x[1] / (2.0 * x[2]);
    if (opteps > sl[2]) opteps = sl[2];
    if (opteps < 0.0) opteps = sl[1];
    if (L2[1] < L2[0] && L2[2] < L2[1]) opteps = sl[2];
    return opteps;
}

extern "C" int psv_step_length(double *est_io, double L2_0, psv_trial_fn trial, void *ctx,
                               int *ntrials, double *tlog, int max_trials)
{
    if (!est_io || !trial) return psv::fail(PSV_ERR_ARG, "step_length: null estimate or trial");
    // A misfit that is not a number (a NaN gradient: a shot whose sources
    // never fire, nt = 1) makes every comparison below false, and the
    // reference's search never ends; here it fails instead.
    if (std::isnan(L2_0)) {
        if (ntrials) *ntrials = 0;
        return psv::fail(PSV_ERR_STEP_SEARCH, "step length search: misfit is not a number");
    }
    const double scalefac = 2.0, stepmax_1 = 30, stepmax_2 = 4;
    double L2_test[3] = {L2_0, 0.0, 0.0}, sl[3] = {0.0, 0.0, 0.0};
    unsigned step1 = 0, step2 = 0, itests = 1, iteste = 1, countstep = 0;
    double est = *est_io;
    int n = 0;
    while ((step2 != 1) || (step1 != 1)) {
        for (unsigned itest = itests; itest <= iteste; itest++) {
            double L2t = 0;
            const int rc = trial(est, &L2t, ctx);
            if (rc != PSV_OK) {
                if (ntrials) *ntrials = n;
                return rc;
            }
            L2_test[itest] = L2t;
            sl[itest] = est;
            sl[0] = 0.0;
            if (tlog && n < max_trials) {
                tlog[2 * n] = est;
                tlog[2 * n + 1] = L2t;
            }
            n++;
            if (std::isnan(L2t)) {
                if (ntrials) *ntrials = n;
                return psv::fail(PSV_ERR_STEP_SEARCH,
                                 "step length search: trial misfit is not a number");
            }
        }
        if ((step1 == 0) && (L2_test[0] <= L2_test[1])) {  // no decrease yet: halve
            est = est / scalefac;
            countstep++;
        }
        if ((step1 == 1) && (L2_test[1] < L2_test[2])) {  // bracketed
            sl[2] = est;
            step2 = 1;
        }
        if ((step1 == 1) && (L2_test[1] >= L2_test[2])) {  // still decreasing: grow
            sl[2] = est;
            est = est + (est / scalefac);
            countstep++;
        }
        if ((step1 == 0) && (L2_test[0] > L2_test[1])) {  // first decrease
            sl[1] = est;
            step1 = 1;
            iteste = 2;
            itests = 2;
            countstep = 0;
            est = est + (est / scalefac);
        }
        if ((step1 == 0) && (countstep > stepmax_1)) {
            if (ntrials) *ntrials = n;
            return psv::fail(PSV_ERR_STEP_SEARCH, "step length search failed (31 halvings without a decrease)");
        }
        if ((step1 == 1) && (countstep > stepmax_2)) {
            step1 = 1;
            step2 = 1;
        }
    }
    if (step1 == 1) est = psv_calc_opt_step(L2_test, sl);
    if (ntrials) *ntrials = n;
    *est_io = est;
    return PSV_OK;
}

extern "C" int psv_gauss_filter_kernel(int hfs, double *k)
{
    if (!k) return psv::fail(PSV_ERR_ARG, "gauss_filter_kernel: null filter");
    hfs = std::abs(hfs);
    if (hfs < 2) return psv::fail(PSV_ERR_ARG, "gauss_filter_kernel: hfs must be at least 2");
    const int n = 2 * hfs + 1;
    const double sigma = (double)(hfs / 2);  // the reference's integer division
    const double q = 2.0 * sigma * sigma;
    double sum = 0.0;
    for (int ii = -hfs; ii <= hfs; ii++)  // x offset outer, as the reference sums
        for (int jj = -hfs; jj <= hfs; jj++) {
            const double v = std::exp(-((ii * ii) / q) - ((jj * jj) / q));
            k[(size_t)(jj + hfs) * n + ii + hfs] = v;
            sum += v;
        }
    for (int i = 0; i < n * n; i++) k[i] /= sum;
    return PSV_OK;
}

extern "C" int psv_checkpoint_schedule(int nseg, int slots, int *actions, int cap, int *nactions,
                                       long long *advances)
{
    if (nseg < 1 || slots < 1) return psv::fail(PSV_ERR_ARG, "need nseg >= 1 and slots >= 1");
    if (psv::ck_min_advances(nseg, std::min(slots, nseg)) > psv::CK_MAX_ADVANCES)
        return psv::fail(PSV_ERR_ARG, "checkpoint schedule: more than 2^26 segment advances; "
                                      "give more slots");
    const psv::CkSchedule c = psv::ck_schedule(nseg, std::min(slots, nseg));
    const int n = (int)(c.fwd.size() + c.bwd.size());
    if (nactions) *nactions = n;
    if (advances) *advances = c.advances;
    if (!actions) return PSV_OK;
    if (cap < n) return psv::fail(PSV_ERR_ARG, "action buffer too small");
    int k = 0;
    for (const auto *v : {&c.fwd, &c.bwd})
        for (const psv::CkAction &x : *v) {
            actions[3 * k] = x.op;
            actions[3 * k + 1] = x.seg;
            actions[3 * k + 2] = x.slot;
            k++;
        }
    return PSV_OK;
}

// ---------------------------------------------------------------------------
// Binary files of the reference (src/h_io_PSV.cpp, scripts/pre_proc_fwi.py:240-276).
// ---------------------------------------------------------------------------
namespace psv {

static bool read_exact(FILE *f, void *dst, size_t bytes)
{
    return fread(dst, 1, bytes, f) == bytes;
}

int read_inputs(const std::string &dir, RefInputs &in)
{
    const std::string b = dir + "/bin/";
    FILE *f = fopen((b + "metaint.bin").c_str(), "rb");
    if (!f) return fail(PSV_ERR_IO, "cannot open bin/metaint.bin");
    int32_t v[37];
    const bool ok = read_exact(f, v, sizeof(v));
    fclose(f);
    if (!ok) return fail(PSV_ERR_IO, "bin/metaint.bin: short read (expects 37 int32)");
    // read_input_metaint, src/h_io_PSV.cpp:40-102: 8 flags then 29 integers.
    in.gpu_code = v[0] != 0; in.surf = v[1] != 0; in.pml_z = v[2] != 0; in.pml_x = v[3] != 0;
    in.accu_save = v[4] != 0; in.seismo_save = v[5] != 0; in.fwinv = v[6] != 0;
    in.rtf_meas_true = v[7] != 0;
    int *dst[] = {&in.nt, &in.nz, &in.nx, &in.snap_t1, &in.snap_t2, &in.snap_z1, &in.snap_z2,
                  &in.snap_x1, &in.snap_x2, &in.snap_dt, &in.snap_dz, &in.snap_dx, &in.taper[0],
                  &in.taper[1], &in.taper[2], &in.taper[3], &in.taper[4], &in.taper[5],
                  &in.taper[6], &in.taper[7], &in.nsrc, &in.nrec, &in.nshot, &in.stf_type,
                  &in.rtf_type, &in.fdorder, &in.fpad, &in.mat_save_interval, &in.mat_grid};
    for (int k = 0; k < 29; k++) *dst[k] = v[8 + k];
    if (in.nt <= 0 || in.nz <= 2 || in.nx <= 2 || in.nsrc < 0 || in.nrec < 0 || in.nshot <= 0)
        return fail(PSV_ERR_IO, "bin/metaint.bin: invalid sizes");

    // read_input_int_array, :109-164.
    f = fopen((b + "intarray.bin").c_str(), "rb");
    if (!f) return fail(PSV_ERR_IO, "cannot open bin/intarray.bin");
    int32_t h[8];
    bool ok2 = read_exact(f, h, sizeof(h));
    for (int k = 0; k < 4; k++) { in.npml[k] = h[k]; in.isurf[k] = h[4 + k]; }
    in.z_src.resize(in.nsrc); in.x_src.resize(in.nsrc); in.src_shot_to_fire.resize(in.nsrc);
    in.z_rec.resize(in.nrec); in.x_rec.resize(in.nrec);
    ok2 = ok2 && read_exact(f, in.z_src.data(), 4 * (size_t)in.nsrc) &&
          read_exact(f, in.x_src.data(), 4 * (size_t)in.nsrc) &&
          read_exact(f, in.src_shot_to_fire.data(), 4 * (size_t)in.nsrc) &&
          read_exact(f, in.z_rec.data(), 4 * (size_t)in.nrec) &&
          read_exact(f, in.x_rec.data(), 4 * (size_t)in.nrec);
    fclose(f);
    if (!ok2) return fail(PSV_ERR_IO, "bin/intarray.bin: short read");

    // read_inp_metafloat, :167-199.
    f = fopen((b + "metafloat.bin").c_str(), "rb");
    if (!f) return fail(PSV_ERR_IO, "cannot open bin/metafloat.bin");
    double m[11];
    ok2 = read_exact(f, m, sizeof(m));
    fclose(f);
    if (!ok2) return fail(PSV_ERR_IO, "bin/metafloat.bin: short read (expects 11 float64)");
    in.dt = m[0]; in.dz = m[1]; in.dx = m[2]; in.npower = m[3]; in.damp_v_pml = m[4];
    in.rcoef = m[5]; in.k_max_pml = m[6]; in.freq_pml = m[7]; in.scalar_lam = m[8];
    in.scalar_mu = m[9]; in.scalar_rho = m[10];

    const size_t n = (size_t)in.nz * in.nx;
    in.lam.assign(n, in.scalar_lam); in.mu.assign(n, in.scalar_mu); in.rho.assign(n, in.scalar_rho);
    if (in.mat_grid) {  // read_material_array, :201-242; else mat_stag_PSV
        f = fopen((b + "mat.bin").c_str(), "rb");
        if (!f) return fail(PSV_ERR_IO, "cannot open bin/mat.bin");
        ok2 = read_exact(f, in.lam.data(), 8 * n) && read_exact(f, in.mu.data(), 8 * n) &&
              read_exact(f, in.rho.data(), 8 * n);
        fclose(f);
        if (!ok2) return fail(PSV_ERR_IO, "bin/mat.bin: short read");
    }
    if (in.fwinv) {  // read_seismo, :320-345: io/shot{i}_rtf_u{z,x}.bin, [nrec][nt]
        if (!in.rtf_meas_true)
            return fail(PSV_ERR_ARG, "FWI requested without field measurements (rtf_meas_true = 0)");
        const size_t nr = (size_t)in.nrec * in.nt;
        in.rtf_z_true.resize(nr * in.nshot);
        in.rtf_x_true.resize(nr * in.nshot);
        for (int s = 0; s < in.nshot; s++) {
            const std::string pz = dir + "/io/shot" + std::to_string(s) + "_rtf_uz.bin";
            const std::string px = dir + "/io/shot" + std::to_string(s) + "_rtf_ux.bin";
            FILE *fz = fopen(pz.c_str(), "rb"), *fx = fopen(px.c_str(), "rb");
            bool okz = fz && fx && read_exact(fz, in.rtf_z_true.data() + s * nr, 8 * nr) &&
                       read_exact(fx, in.rtf_x_true.data() + s * nr, 8 * nr);
            if (fz) fclose(fz);
            if (fx) fclose(fx);
            if (!okz) return fail(PSV_ERR_IO, "cannot read " + pz + " / " + px);
        }
    }
    return PSV_OK;
}

int write_f64(const std::string &path, const double *data, size_t n)
{
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return fail(PSV_ERR_IO, "cannot open " + path + " for writing");
    const bool ok = fwrite(data, 8, n, f) == n;
    fclose(f);
    return ok ? PSV_OK : fail(PSV_ERR_IO, "short write to " + path);
}

}  // namespace psv
