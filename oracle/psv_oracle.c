/*
 * psv_oracle.c -- FP64 CPU restatement of the reference P/SV path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Only tests/, the smoke check and
 * the CPU-baseline leg of bench.py load this library; the product path never
 * does.
 *
 * Each function follows one reference function (Mohammad-debug/FWI_CUDA) and
 * cites it.  The loop nests, their OpenMP placement and the FP64 operation
 * order follow the reference, so this file doubles as a faithful CPU
 * baseline: sdiff2 and update_v2 stay serial as in the reference
 * (src/cpu/n_kernel_lib_PSV.cpp:224,253).  Build with -ffp-contract=off.
 */
#include "psv_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(iz, ix, nx) ((size_t)(iz) * (size_t)(nx) + (size_t)(ix))

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* ------------------------------------------------------------------------ */
/* Host preprocessing                                                       */
/* ------------------------------------------------------------------------ */

/* Holberg (1987) staggered-grid coefficients as tabulated by the DENISE code
 * family; the reference holds the same published table
 * (src/h_holbergcoeff.cpp:25-75).  Row = maximum relative group-velocity
 * error (0 Taylor, 1: 0.1 %, 2: 0.5 %, 3: 1 %, 4: 3 %); column 0 = minimum
 * points per wavelength, columns 1..6 = coefficients. */
static const double holberg_table[5][6][7] = {
    {{23.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0},
     {8.0, 9.0 / 8.0, -1.0 / 24.0, 0.0, 0.0, 0.0, 0.0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0.0, 0.0, 0.0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0.0, 0.0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0,
      35.0 / 294912.0, 0.0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0,
      -5445.0 / 1835008.0, 847.0 / 2359296.0, -63.0 / 2883584.0}},
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

/* holbergcoeff, src/h_holbergcoeff.cpp:21-80 (row = FDORDER/2 - 1, all 7 columns). */
void orc_holbergcoeff(int fdorder, int maxrelerror, double *hc7)
{
    int nl = fdorder / 2 - 1;
    for (int i = 0; i <= 6; i++) hc7[i] = holberg_table[maxrelerror][nl][i];
}

/* cpml_PSV, src/h_preproc_PSV.cpp:112-263: 1D CPML profiles for one axis. */
void orc_cpml_PSV(double *a, double *b, double *K, double *a_half, double *b_half, double *K_half,
                  double npower, double damp_v_PML, double rcoef, double k_max_PML, double freq,
                  int npml_h1, int npml_h2, int fpad, int nh, double dt, double dh)
{
    const double alpha_max_PML = 2.0 * ORC_PI * (freq / 2.0);
    double thickness_PML, xorigin_PML, xval, abscissa_in_PML, abscissa_normalized;
    double d0, d, d_half, alpha_prime, alpha_prime_half;

    for (int ih = 0; ih < nh; ih++) { /* :126-130 */
        a[ih] = 0.0; a_half[ih] = 0.0;
        b[ih] = 1.0; b_half[ih] = 1.0;
        K[ih] = 1.0; K_half[ih] = 1.0;
    }
    if (npml_h1) { /* :134-194, low side */
        thickness_PML = npml_h1 * dh;
        xorigin_PML = thickness_PML;
        d0 = -(npower + 1) * damp_v_PML * log(rcoef) / (2.0 * thickness_PML);
        for (int i = fpad; i <= npml_h1 + fpad; i++) {
            abscissa_normalized = 0.0;
            d = 0; d_half = 0;
            alpha_prime = 0.0; alpha_prime_half = 0.0;
            xval = dh * (double)i;
            abscissa_in_PML = xorigin_PML - xval;
            if (abscissa_in_PML >= 0) {
                abscissa_normalized = abscissa_in_PML / thickness_PML;
                d = d0 * pow(abscissa_normalized, npower);
                K[i] = 1.0 + (k_max_PML - 1.0) * pow(abscissa_normalized, npower);
                alpha_prime = alpha_max_PML * (1.0 - abscissa_normalized);
            }
            abscissa_in_PML = xorigin_PML - (xval + dh / 2.0);
            if (abscissa_in_PML >= 0) {
                abscissa_normalized = abscissa_in_PML / thickness_PML;
                d_half = d0 * pow(abscissa_normalized, npower);
                K_half[i] = 1.0 + (k_max_PML - 1.0) * pow(abscissa_normalized, npower);
                alpha_prime_half = alpha_max_PML * (1.0 - abscissa_normalized);
            }
            if (alpha_prime < 0.0) alpha_prime = 0.0;
            if (alpha_prime_half < 0.0) alpha_prime_half = 0.0;
            b[i] = exp(-(d / K[i] + alpha_prime) * dt);
            b_half[i] = exp(-(d_half / K_half[i] + alpha_prime_half) * dt);
            if (fabs(d) > 1.0e-6) a[i] = d * (b[i] - 1.0) / (K[i] * (d + K[i] * alpha_prime));
            if (fabs(d_half) > 1.0e-6)
                a_half[i] = d_half * (b_half[i] - 1.0) /
                            (K_half[i] * (d_half + K_half[i] * alpha_prime_half));
        }
    }
    if (npml_h2) { /* :199-261, high side */
        thickness_PML = npml_h2 * dh;
        xorigin_PML = dh * (nh - fpad - npml_h2 - 1);
        d0 = -(npower + 1) * damp_v_PML * log(rcoef) / (2.0 * thickness_PML);
        for (int i = nh - fpad - npml_h2 - 1; i < nh - fpad; i++) {
            abscissa_normalized = 0.0;
            d = 0; d_half = 0;
            alpha_prime = 0.0; alpha_prime_half = 0.0;
            xval = dh * (double)i;
            abscissa_in_PML = xval - xorigin_PML;
            if (abscissa_in_PML >= 0) {
                abscissa_normalized = abscissa_in_PML / thickness_PML;
                d = d0 * pow(abscissa_normalized, npower);
                K[i] = 1.0 + (k_max_PML - 1.0) * pow(abscissa_normalized, npower);
                alpha_prime = alpha_max_PML * (1.0 - abscissa_normalized);
            }
            abscissa_in_PML = (xval + dh / 2.0) - xorigin_PML;
            if (abscissa_in_PML >= 0) {
                abscissa_normalized = abscissa_in_PML / thickness_PML;
                d_half = d0 * pow(abscissa_normalized, npower);
                K_half[i] = 1.0 + (k_max_PML - 1.0) * pow(abscissa_normalized, npower);
                alpha_prime_half = alpha_max_PML * (1.0 - abscissa_normalized);
            }
            if (alpha_prime < 0.0) alpha_prime = 0.0;
            if (alpha_prime_half < 0.0) alpha_prime_half = 0.0;
            b[i] = exp(-(d / K[i] + alpha_prime) * dt);
            b_half[i] = exp(-(d_half / K_half[i] + alpha_prime_half) * dt);
            if (fabs(d) > 1.0e-6) a[i] = d * (b[i] - 1.0) / (K[i] * (d + K[i] * alpha_prime));
            if (fabs(d_half) > 1.0e-6)
                a_half[i] = d_half * (b_half[i] - 1.0) /
                            (K_half[i] * (d_half + K_half[i] * alpha_prime_half));
        }
    }
}

/* wavelet, src/h_preproc_PSV.cpp:267-286 (shape 1 = Ricker). */
void orc_wavelet(double *signal, int nt, double dt, double amp, double fc, double ts, int shape)
{
    const double fci = 1.0 / fc;
    if (shape != 1) return;
    for (int it = 0; it < nt; it++) {
        double t = it * dt;
        double tau = ORC_PI * (t - 1.5 * fci - ts) / (1.5 * fci);
        signal[it] = amp * (1.0 - 2.0 * tau * tau) * exp(-2.0 * tau * tau);
    }
}

/* checkfd_ssg_elastic, src/h_checkfd_ssg_elastic.cpp:14-144.  The reference
 * scans j in [1, nz-fw] and i in [1+fw, nx-fw] inclusive, which reads one
 * row/column past the array when fw == 0; this restatement clamps the scan to
 * the array. */
int orc_checkfd_ssg_elastic(int nz, int nx, double dh, double dt, double ts, int fw,
                            const double *rho, const double *lam, const double *mu,
                            const double *hc, double *out)
{
    double cmax_p = 0.0, cmin_p = 1e9, cmax_s = 0.0, cmin_s = 1e9, c;
    int i1 = 1 + fw, i2 = nx - fw, j1 = 1, j2 = nz - fw;
    if (i2 > nx - 1) i2 = nx - 1;
    if (j2 > nz - 1) j2 = nz - 1;
    for (int i = i1; i <= i2; i++)
        for (int j = j1; j <= j2; j++) {
            double u = mu[IDX(j, i, nx)];
            if (fabs(u) < 1.0e-9) continue;
            c = sqrt(u / rho[IDX(j, i, nx)]);
            if (cmax_s < c) cmax_s = c;
            if (cmin_s > c) cmin_s = c;
            c = sqrt((lam[IDX(j, i, nx)] + 2.0 * u) / rho[IDX(j, i, nx)]);
            if (cmax_p < c) cmax_p = c;
            if (cmin_p > c) cmin_p = c;
        }
    double cmax = cmax_s > cmax_p ? cmax_s : cmax_p;
    double cmin = cmin_s < cmin_p ? cmin_s : cmin_p;
    double fmax = 2.0 * ts;
    double gamma = fabs(hc[1]) + fabs(hc[2]) + fabs(hc[3]) + fabs(hc[4]) + fabs(hc[5]) + fabs(hc[6]);
    out[0] = dh / (sqrt(2) * gamma * cmax);
    out[1] = cmin / (12.0 * fmax);
    out[2] = cmax;
    out[3] = cmin;
    return (fw > nx - fw) || (fw > nz - fw);
}

/* ------------------------------------------------------------------------ */
/* Kernel library                                                           */
/* ------------------------------------------------------------------------ */

/* mat_av2, src/cpu/n_kernel_lib_PSV.cpp:853-922.  Keeps the reference's
 * rho_xp vacuum check that writes rho_zp (:894-897).  Cells of the last
 * row/column, left unset by the reference, are zero here. */
void orc_mat_av2(const double *lam, const double *mu, const double *rho,
                 double *mu_zx, double *rho_zp, double *rho_xp, double *C3, int nz, int nx)
{
    double C_lam = 0.0, C_mu = 0.0, C_rho = 0.0;
    for (int ix = 0; ix < nx; ix++) {
        mu_zx[IDX(nz - 1, ix, nx)] = 0.0;
        rho_zp[IDX(nz - 1, ix, nx)] = 0.0;
        rho_xp[IDX(nz - 1, ix, nx)] = 0.0;
    }
    for (int iz = 0; iz < nz; iz++) {
        mu_zx[IDX(iz, nx - 1, nx)] = 0.0;
        rho_zp[IDX(iz, nx - 1, nx)] = 0.0;
        rho_xp[IDX(iz, nx - 1, nx)] = 0.0;
    }
#pragma omp parallel for collapse(2) reduction(+ : C_lam, C_mu, C_rho)
    for (int iz = 0; iz < nz - 1; iz++) {
        for (int ix = 0; ix < nx - 1; ix++) {
            const double m00 = mu[IDX(iz, ix, nx)], m01 = mu[IDX(iz, ix + 1, nx)];
            const double m10 = mu[IDX(iz + 1, ix, nx)], m11 = mu[IDX(iz + 1, ix + 1, nx)];
            double v = 4.0 / ((1.0 / m00) + (1.0 / m01) + (1.0 / m10) + (1.0 / m11));
            if ((m00 == 0.0) || (m01 == 0.0) || (m10 == 0.0) || (m11 == 0.0)) v = 0.0;
            mu_zx[IDX(iz, ix, nx)] = v;

            const double r00 = rho[IDX(iz, ix, nx)], r10 = rho[IDX(iz + 1, ix, nx)];
            const double r01 = rho[IDX(iz, ix + 1, nx)];
            rho_zp[IDX(iz, ix, nx)] = 1.0 / (0.5 * (r00 + r10));
            rho_xp[IDX(iz, ix, nx)] = 1.0 / (0.5 * (r00 + r01));
            if ((r00 < 1e-4) && (r10 < 1e-4)) rho_zp[IDX(iz, ix, nx)] = 0.0;
            if ((r00 < 1e-4) && (r01 < 1e-4)) rho_zp[IDX(iz, ix, nx)] = 0.0;

            C_lam += lam[IDX(iz, ix, nx)];
            C_mu += m00;
            C_rho += r00;
        }
    }
    C3[0] = C_lam / ((nz - 1) * (nx - 1));
    C3[1] = C_mu / ((nz - 1) * (nx - 1));
    C3[2] = C_rho / ((nz - 1) * (nx - 1));
}

/* adjsrc2, src/cpu/n_kernel_lib_PSV.cpp:579-626 (rtf_type 0): residual
 * mod - true into a_stf (may alias the model arrays) and the L2 misfit. */
double orc_adjsrc2(double *a_stf_uz, double *a_stf_ux, const double *rtf_uz_true,
                   const double *rtf_ux_true, const double *rtf_uz_mod, const double *rtf_ux_mod,
                   double dt, int nseis, int nt)
{
    double L2 = 0;
    for (int is = 0; is < nseis; is++) {
        for (int it = 0; it < nt; it++) {
            size_t k = IDX(is, it, nt);
            a_stf_uz[k] = rtf_uz_mod[k] - rtf_uz_true[k];
            a_stf_ux[k] = rtf_ux_mod[k] - rtf_ux_true[k];
            L2 += 0.5 * dt * (a_stf_uz[k] * a_stf_uz[k]) + 0.5 * dt * (a_stf_ux[k] * a_stf_ux[k]);
        }
    }
    return L2;
}

/* interpol_grad2, src/cpu/n_kernel_lib_PSV.cpp:628-693. */
void orc_interpol_grad2(double *grad, const double *grad_shot, int nx, int snap_z1, int snap_z2,
                        int snap_x1, int snap_x2, int snap_dz, int snap_dx)
{
    const int snap_nx = 1 + (snap_x2 - snap_x1) / snap_dx;
    int jz = 0;
    for (int iz = snap_z1; iz <= snap_z2; iz += snap_dz) {
        int jx = 0;
        for (int ix = snap_x1; ix <= snap_x2; ix += snap_dx) {
            grad[IDX(iz, ix, nx)] = grad_shot[IDX(jz, jx, snap_nx)];
            jx++;
        }
        jz++;
    }
    if (snap_dx > 1) {
        for (int iz = snap_z1; iz < snap_z2; iz += snap_dz)
            for (int ix = snap_x1; ix < snap_x2; ix += snap_dx) {
                double t = (grad[IDX(iz, ix + snap_dx, nx)] - grad[IDX(iz, ix, nx)]) / snap_dx;
                for (int kx = 1; kx < snap_dx; kx++)
                    grad[IDX(iz, ix + kx, nx)] = grad[IDX(iz, ix, nx)] + t * kx;
            }
    }
    if (snap_dz > 1) {
        for (int iz = snap_z1; iz < snap_z2; iz += snap_dz)
            for (int ix = snap_x1; ix < snap_x2; ix++) {
                double t = (grad[IDX(iz + snap_dz, ix, nx)] - grad[IDX(iz, ix, nx)]) / snap_dz;
                for (int kz = 1; kz < snap_dz; kz++)
                    grad[IDX(iz + kz, ix, nx)] = grad[IDX(iz, ix, nx)] + t * kz;
            }
    }
}

/* energy_weights2, src/cpu/n_kernel_lib_PSV.cpp:696-757.  max_out3 receives
 * max_We and the maxima of the two input energies (print-only there). */
void orc_energy_weights2(double *We, const double *We_adj, int nx, int snap_z1, int snap_z2,
                         int snap_x1, int snap_x2, double *max_out3)
{
    double max_We = 0, max_w1 = 0, max_w2 = 0;
    const double epsilon_We = 0.005;
#pragma omp parallel for collapse(2) reduction(max : max_w1, max_w2)
    for (int iz = snap_z1; iz < snap_z2; iz++)
        for (int ix = snap_x1; ix < snap_x2; ix++) {
            size_t k = IDX(iz, ix, nx);
            if (We[k] > max_w1) max_w1 = We[k];
            if (We_adj[k] > max_w2) max_w2 = We_adj[k];
            We[k] = sqrt(We[k] * We_adj[k]);
        }
#pragma omp parallel for collapse(2) reduction(max : max_We)
    for (int iz = snap_z1; iz < snap_z2; iz++)
        for (int ix = snap_x1; ix < snap_x2; ix++)
            if (We[IDX(iz, ix, nx)] > max_We) max_We = We[IDX(iz, ix, nx)];
    for (int iz = snap_z1; iz < snap_z2; iz++)
        for (int ix = snap_x1; ix < snap_x2; ix++) We[IDX(iz, ix, nx)] += epsilon_We * max_We;
    if (max_out3) {
        max_out3[0] = max_We;
        max_out3[1] = max_w1;
        max_out3[2] = max_w2;
    }
}

/* scale_grad_E2, src/cpu/n_kernel_lib_PSV.cpp:760-783. */
void orc_scale_grad_E2(double *grad, const double *grad_shot, double mat_av, const double *We,
                       int nx, int snap_z1, int snap_z2, int snap_x1, int snap_x2)
{
    if (!(mat_av > 0)) return;
#pragma omp parallel for collapse(2)
    for (int iz = snap_z1; iz < snap_z2; iz++)
        for (int ix = snap_x1; ix < snap_x2; ix++) {
            size_t k = IDX(iz, ix, nx);
            grad[k] += grad_shot[k] / (We[k] * mat_av * mat_av);
        }
}

/* update_mat2, src/cpu/n_kernel_lib_PSV.cpp:785-832. */
void orc_update_mat2(double *mat, const double *mat_old, const double *grad_mat, double mat_max,
                     double mat_min, double step_length, int nz, int nx)
{
    double grad_max = 0.0, mat_array_max = 0.0;
    const size_t n = (size_t)nz * nx;
#pragma omp parallel for reduction(max : grad_max, mat_array_max)
    for (size_t k = 0; k < n; k++) {
        double g = fabs(grad_mat[k]), m = fabs(mat_old[k]);
        if (g > grad_max) grad_max = g;
        if (m > mat_array_max) mat_array_max = m;
    }
    if (mat_array_max < mat_max) mat_array_max = mat_max;
    const double step_factor = mat_array_max / grad_max;
    for (size_t k = 0; k < n; k++) {
        double v = mat_old[k] + step_length * step_factor * grad_mat[k];
        if (v > mat_max) v = mat_max;
        if (v < mat_min) v = mat_min;
        mat[k] = v;
    }
}

/* taper2, src/cpu/n_kernel_lib_PSV.cpp:942-1010 (Tukey taper; horizontal then vertical). */
void orc_taper2(double *A, int nz, int nx, int snap_z1, int snap_z2, int snap_x1, int snap_x2,
                const int *t8)
{
    const int taper_t1 = t8[0], taper_t2 = t8[1], taper_b1 = t8[2], taper_b2 = t8[3];
    const int taper_l1 = t8[4], taper_l2 = t8[5], taper_r1 = t8[6], taper_r2 = t8[7];
    const int taper_l = taper_l2 - taper_l1, taper_r = taper_r1 - taper_r2;
    const int taper_t = taper_t2 - taper_t1, taper_b = taper_b1 - taper_b2;
#pragma omp parallel for collapse(2)
    for (int iz = 0; iz < nz; iz++)
        for (int ix = 0; ix < nx; ix++) {
            double *p = &A[IDX(iz, ix, nx)];
            if (ix >= snap_x1 && ix < taper_l1) *p *= 0.0;
            else if (ix >= taper_l1 && ix < taper_l2)
                *p *= 0.5 * (1.0 - cos(ORC_PI * (ix - taper_l1) / taper_l));
            else if (ix > taper_r2 && ix < taper_r1)
                *p *= 0.5 * (1.0 - cos(ORC_PI * (taper_r1 - ix) / taper_r));
            else if (ix >= taper_r1 && ix <= snap_x2) *p *= 0.0;
        }
#pragma omp parallel for collapse(2)
    for (int ix = 0; ix < nx; ix++)
        for (int iz = 0; iz < nz; iz++) {
            double *p = &A[IDX(iz, ix, nx)];
            if (iz >= snap_z1 && iz < taper_t1) *p *= 0.0;
            else if (iz >= taper_t1 && iz < taper_t2)
                *p *= 0.5 * (1.0 - cos(ORC_PI * (iz - taper_t1) / taper_t));
            else if (iz > taper_b2 && iz < taper_b1)
                *p *= 0.5 * (1.0 - cos(ORC_PI * (taper_b1 - iz) / taper_b));
            else if (iz >= taper_b1 && iz <= snap_z2) *p *= 0.0;
        }
}

/* gauss_filter_kernel, src/cpu/n_kernel_lib_PSV.cpp:1012-1050: (2 hfs + 1)^2
 * weights exp(-(i^2 / q) - (j^2 / q)), q = 2 sigma^2, sigma = hfs / 2 in
 * integer arithmetic as the reference writes it, normalised by their sum
 * (accumulated with the x offset outer).  Row jj + hfs, column ii + hfs.
 * hfs < 2 is rejected (-1): the reference's sigma is 0 there and its
 * weights are NaN. */
int orc_gauss_filter_kernel(int hfs, double *k)
{
    if (hfs < 0) hfs = -hfs;
    if (hfs < 2) return -1;
    const int n = 2 * hfs + 1;
    const double sigma = (double)(hfs / 2);
    const double q = 2.0 * sigma * sigma;
    double sum = 0.0;
    for (int ii = -hfs; ii <= hfs; ii++)
        for (int jj = -hfs; jj <= hfs; jj++) {
            const double v = exp(-((ii * ii) / q) - ((jj * jj) / q));
            k[(size_t)(jj + hfs) * n + ii + hfs] = v;
            sum += v;
        }
    for (int i = 0; i < n * n; i++) k[i] /= sum;
    return 0;
}

/* apply_gauss_filter, src/cpu/n_kernel_lib_PSV.cpp:1053-1084: points
 * [hfs, nz - hfs - 1) x [hfs, nx - hfs - 1) take the filtered value of a copy
 * of mat (rows outer, filter row jj outer, column ii inner); the others keep
 * theirs.  The sum is a double: the reference accumulates into an int,
 * which truncates every partial sum (gradients become 0, moduli overflow). */
void orc_apply_gauss_filter(double *mat, int nz, int nx, const double *filt, int hfs)
{
    const int n = 2 * hfs + 1;
    double *tmp = zalloc((size_t)nz * nx);
    memcpy(tmp, mat, sizeof(double) * (size_t)nz * nx);
    for (int iz = hfs; iz < nz - hfs - 1; iz++)
        for (int ix = hfs; ix < nx - hfs - 1; ix++) {
            double conv = 0.0;
            for (int jj = 0; jj < n; jj++)
                for (int ii = 0; ii < n; ii++)
                    conv += tmp[IDX(iz + jj - hfs, ix + ii - hfs, nx)] * filt[(size_t)jj * n + ii];
            mat[IDX(iz, ix, nx)] = conv;
        }
    free(tmp);
}

/* PCG_PSV, src/cpu/n_PCG_PSV.cpp:13-44 (Fletcher-Reeves): beta = |grad|^2 /
 * |old|^2, negative beta -> 0; old <- -grad; dir <- -grad + beta dir;
 * grad <- dir.  When |old|^2 = 0 (the first call, old starts at zero) beta
 * is 0: the reference divides by zero there and its direction is NaN. */
void orc_PCG_PSV(double *dir, double *old, double *grad, int nz, int nx)
{
    const size_t n = (size_t)nz * nx;
    double bi = 0.0, bj = 0.0;
    for (size_t i = 0; i < n; i++) {
        bi += grad[i] * grad[i];
        bj += old[i] * old[i];
        old[i] = -grad[i];
    }
    double beta = bj > 0.0 ? bi / bj : 0.0;
    beta = beta > 0 ? beta : 0.0;
    for (size_t i = 0; i < n; i++) {
        dir[i] = -grad[i] + beta * dir[i];
        grad[i] = dir[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Time-loop building blocks                                                */
/* ------------------------------------------------------------------------ */

static int stencil_terms(const orc_grid *g)
{
    return g->stencil == ORC_STENCIL_HOLBERG ? g->fdorder / 2 : 1;
}

/* vdiff2, src/cpu/n_kernel_lib_PSV.cpp:100-131.  Term k of the Holberg form
 * spans rows iz+k-1 / iz-k (backward) or iz+k / iz-k+1 (forward); k = 1 is
 * the reference's 2-point difference with the same rounding. */
static void vdiff2(const orc_grid *g, double *vz_z, double *vx_z, double *vz_x, double *vx_x,
                   const double *vz, const double *vx, int nz1, int nz2, int nx1, int nx2)
{
    const int nx = g->nx, ns = stencil_terms(g);
    const double dxi = 1.0 / g->dx, dzi = 1.0 / g->dz;
    const double *hc = g->hc;
    const long sz = nx;
#pragma omp parallel for collapse(2)
    for (int iz = nz1; iz < nz2; iz++)
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(iz, ix, nx);
            double a = dzi * hc[1] * (vz[i] - vz[i - sz]);
            double b = dzi * hc[1] * (vx[i + sz] - vx[i]);
            double c = dxi * hc[1] * (vz[i + 1] - vz[i]);
            double d = dxi * hc[1] * (vx[i] - vx[i - 1]);
            for (int k = 2; k <= ns; k++) {
                a += dzi * hc[k] * (vz[i + (k - 1) * sz] - vz[i - k * sz]);
                b += dzi * hc[k] * (vx[i + k * sz] - vx[i - (k - 1) * sz]);
                c += dxi * hc[k] * (vz[i + k] - vz[i - (k - 1)]);
                d += dxi * hc[k] * (vx[i + (k - 1)] - vx[i - k]);
            }
            vz_z[i] = a; vx_z[i] = b; vz_x[i] = c; vx_x[i] = d;
        }
}

/* pml_diff2, src/cpu/n_kernel_lib_PSV.cpp:134-178. */
static void pml_diff2(const orc_grid *g, double *dz_z, double *dx_z, double *dz_x, double *dx_x,
                      double *mem_z_z, double *mem_x_z, double *mem_z_x, double *mem_x_x,
                      int nz1, int nz2, int nx1, int nx2)
{
    const int nx = g->nx, pml_z = g->pml_z, pml_x = g->pml_x;
#pragma omp parallel for collapse(2)
    for (int iz = nz1; iz < nz2; iz++)
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(iz, ix, nx);
            if (pml_z) {
                mem_z_z[i] = g->b_z[iz] * mem_z_z[i] + g->a_z[iz] * dz_z[i];
                mem_x_z[i] = g->b_half_z[iz] * mem_x_z[i] + g->a_half_z[iz] * dx_z[i];
                dz_z[i] = dz_z[i] / g->K_z[iz] + mem_z_z[i];
                dx_z[i] = dx_z[i] / g->K_half_z[iz] + mem_x_z[i];
            }
            if (pml_x) {
                mem_x_x[i] = g->b_x[ix] * mem_x_x[i] + g->a_x[ix] * dx_x[i];
                mem_z_x[i] = g->b_half_x[ix] * mem_z_x[i] + g->a_half_x[ix] * dz_x[i];
                dx_x[i] = dx_x[i] / g->K_x[ix] + mem_x_x[i];
                dz_x[i] = dz_x[i] / g->K_half_x[ix] + mem_z_x[i];
            }
        }
}

/* update_s2, src/cpu/n_kernel_lib_PSV.cpp:181-205. */
static void update_s2(const orc_grid *g, double *szz, double *szx, double *sxx,
                      const double *vz_z, const double *vx_z, const double *vz_x,
                      const double *vx_x, const double *lam, const double *mu,
                      const double *mu_zx, int nz1, int nz2, int nx1, int nx2)
{
    const int nx = g->nx;
    const double dt = g->dt;
#pragma omp parallel for collapse(2)
    for (int iz = nz1; iz < nz2; iz++)
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(iz, ix, nx);
            szz[i] += dt * (lam[i] * (vx_x[i] + vz_z[i]) + (2.0 * mu[i] * vz_z[i]));
            szx[i] += dt * mu_zx[i] * (vz_x[i] + vx_z[i]);
            sxx[i] += dt * (lam[i] * (vx_x[i] + vz_z[i]) + (2.0 * mu[i] * vx_x[i]));
        }
}

/* surf_mirror, src/cpu/n_kernel_lib_PSV.cpp:272-395 (top, bottom, left, right in that order). */
static void surf_mirror(const orc_grid *g, double *szz, double *szx, double *sxx,
                        const double *vz_z, const double *vx_x, const double *lam,
                        const double *mu, int nz1, int nz2, int nx1, int nx2)
{
    const int nx = g->nx;
    const double dt = g->dt;
    const int *surf = g->isurf;
    if (surf[0] > 0) {
        const int is = surf[0];
#pragma omp parallel for
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(is, ix, nx);
            szz[i] = 0.0;
            szx[i] = 0.0;
            sxx[i] = 4.0 * dt * vx_x[i] * (lam[i] * mu[i] + mu[i] * mu[i]) / (lam[i] + 2.0 * mu[i]);
            for (int sz = 1; sz < is - nz1 + 1; sz++) {
                szx[IDX(is - sz, ix, nx)] = -szx[IDX(is + sz, ix, nx)];
                szz[IDX(is - sz, ix, nx)] = -szz[IDX(is + sz, ix, nx)];
            }
        }
    }
    if (surf[1] > 0) {
        const int is = surf[1];
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(is, ix, nx);
            szz[i] = 0.0;
            szx[i] = 0.0;
            sxx[i] = 4.0 * dt * vx_x[i] * (lam[i] * mu[i] + mu[i] * mu[i]) / (lam[i] + 2.0 * mu[i]);
            for (int sz = 1; sz <= nz2 - is; sz++) {
                szx[IDX(is + sz, ix, nx)] = -szx[IDX(is - sz, ix, nx)];
                szz[IDX(is + sz, ix, nx)] = -szz[IDX(is - sz, ix, nx)];
            }
        }
    }
    if (surf[2] > 0) {
        const int is = surf[2];
        for (int iz = nz1; iz < nz2; iz++) {
            const size_t i = IDX(iz, is, nx);
            sxx[i] = 0.0;
            szx[i] = 0.0;
            szz[i] = 4.0 * dt * vz_z[i] * (lam[i] * mu[i] + mu[i] * mu[i]) / (lam[i] + 2.0 * mu[i]);
            for (int sx = 1; sx < is - nx1 + 1; sx++) {
                szx[IDX(iz, is - sx, nx)] = -szx[IDX(iz, is + sx, nx)];
                sxx[IDX(iz, is - sx, nx)] = -sxx[IDX(iz, is + sx, nx)];
            }
        }
    }
    if (surf[3] > 0) {
        const int is = surf[3];
        for (int iz = nz1; iz < nz2; iz++) {
            const size_t i = IDX(iz, is, nx);
            sxx[i] = 0.0;
            szx[i] = 0.0;
            szz[i] = 4.0 * dt * vz_z[i] * (lam[i] * mu[i] + mu[i] * mu[i]) / (lam[i] + 2.0 * mu[i]);
            for (int sx = 1; sx <= nx2 - is; sx++) {
                szx[IDX(iz, is + sx, nx)] = -szx[IDX(iz, is - sx, nx)];
                sxx[IDX(iz, is + sx, nx)] = -sxx[IDX(iz, is - sx, nx)];
            }
        }
    }
}

/* sdiff2, src/cpu/n_kernel_lib_PSV.cpp:207-236 (serial, as there). */
static void sdiff2(const orc_grid *g, double *szz_z, double *szx_z, double *szx_x, double *sxx_x,
                   const double *szz, const double *szx, const double *sxx, int nz1, int nz2,
                   int nx1, int nx2)
{
    const int nx = g->nx, ns = stencil_terms(g);
    const double dxi = 1.0 / g->dx, dzi = 1.0 / g->dz;
    const double *hc = g->hc;
    const long sz = nx;
    for (int iz = nz1; iz < nz2; iz++)
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(iz, ix, nx);
            double a = dzi * hc[1] * (szz[i + sz] - szz[i]);
            double b = dzi * hc[1] * (szx[i] - szx[i - sz]);
            double c = dxi * hc[1] * (szx[i] - szx[i - 1]);
            double d = dxi * hc[1] * (sxx[i + 1] - sxx[i]);
            for (int k = 2; k <= ns; k++) {
                a += dzi * hc[k] * (szz[i + k * sz] - szz[i - (k - 1) * sz]);
                b += dzi * hc[k] * (szx[i + (k - 1) * sz] - szx[i - k * sz]);
                c += dxi * hc[k] * (szx[i + (k - 1)] - szx[i - k]);
                d += dxi * hc[k] * (sxx[i + k] - sxx[i - (k - 1)]);
            }
            szz_z[i] = a; szx_z[i] = b; szx_x[i] = c; sxx_x[i] = d;
        }
}

/* update_v2, src/cpu/n_kernel_lib_PSV.cpp:239-270 (serial, as there). */
static void update_v2(const orc_grid *g, double *vz, double *vx, double *uz, double *ux,
                      double *We, const double *szz_z, const double *szx_z, const double *szx_x,
                      const double *sxx_x, const double *rho_zp, const double *rho_xp, int nz1,
                      int nz2, int nx1, int nx2)
{
    const int nx = g->nx;
    const double dt = g->dt;
    for (int iz = nz1; iz < nz2; iz++)
        for (int ix = nx1; ix < nx2; ix++) {
            const size_t i = IDX(iz, ix, nx);
            uz[i] += dt * vz[i];
            ux[i] += dt * vx[i];
            vz[i] += dt * rho_zp[i] * (szx_x[i] + szz_z[i]);
            vx[i] += dt * rho_xp[i] * (sxx_x[i] + szx_z[i]);
            We[i] += vx[i] * vx[i] + vz[i] * vz[i];
        }
}

/* vsrc2, src/cpu/n_kernel_lib_PSV.cpp:487-536. */
static void vsrc2(const orc_grid *g, double *vz, double *vx, const double *rho_zp,
                  const double *rho_xp, int nsrc, int stf_type, const double *stf_z,
                  const double *stf_x, const int *z_src, const int *x_src,
                  const int *src_shot_to_fire, int ishot, int it)
{
    const int nx = g->nx, nt = g->nt;
    const double dt = g->dt, dz = g->dz, dx = g->dx;
    for (int is = 0; is < nsrc; is++) {
        if (src_shot_to_fire[is] != ishot) continue;
        const size_t i = IDX(z_src[is], x_src[is], nx);
        const size_t s = IDX(is, it, nt);
        if (stf_type == 0) {
            vz[i] += dt * rho_zp[i] * stf_z[s] / (dz * dx);
            vx[i] += dt * rho_xp[i] * stf_x[s] / (dz * dx);
        } else if (stf_type == 1) {
            vz[i] += stf_z[s];
            vx[i] += stf_x[s];
        }
    }
}

/* urec2, src/cpu/n_kernel_lib_PSV.cpp:538-576: displacement = running sum. */
static void urec2(const orc_grid *g, int rtf_type, double *rtf_uz, double *rtf_ux,
                  const double *vz, const double *vx, int nrec, const int *rz, const int *rx,
                  int it)
{
    const int nx = g->nx, nt = g->nt;
    const double dt = g->dt, dz = g->dz, dx = g->dx;
    if (rtf_type != 0) return;
    for (int ir = 0; ir < nrec; ir++) {
        const size_t i = IDX(rz[ir], rx[ir], nx);
        const size_t k = IDX(ir, it, nt);
        if (it == 0) {
            rtf_uz[k] = dt * vz[i] / (dz * dx);
            rtf_ux[k] = dt * vx[i] / (dz * dx);
        } else {
            rtf_uz[k] = rtf_uz[k - 1] + dt * vz[i] / (dz * dx);
            rtf_ux[k] = rtf_ux[k - 1] + dt * vx[i] / (dz * dx);
        }
    }
}

static void snap_dims(const orc_grid *g, int *snap_nt, int *snap_nz, int *snap_nx)
{
    *snap_nt = 1 + (g->nt - 1) / g->snap_dt;
    *snap_nz = 1 + (g->snap_z2 - g->snap_z1) / g->snap_dz;
    *snap_nx = 1 + (g->snap_x2 - g->snap_x1) / g->snap_dx;
}

/* gard_fwd_storage2, src/cpu/n_kernel_lib_PSV.cpp:398-436. */
static void gard_fwd_storage2(const orc_grid *g, double *accu_vz, double *accu_vx,
                              double *accu_szz, double *accu_szx, double *accu_sxx,
                              const double *vz, const double *vx, const double *szz,
                              const double *szx, const double *sxx, int itf)
{
    int snap_nt, snap_nz, snap_nx;
    snap_dims(g, &snap_nt, &snap_nz, &snap_nx);
    const int nx = g->nx;
    const double dt = g->dt;
    const size_t base = (size_t)itf * snap_nz * snap_nx;
#pragma omp parallel for
    for (int jz = 0; jz < snap_nz; jz++) {
        const int iz = g->snap_z1 + jz * g->snap_dz;
        for (int jx = 0; jx < snap_nx; jx++) {
            const int ix = g->snap_x1 + jx * g->snap_dx;
            const size_t s = base + IDX(jz, jx, snap_nx), i = IDX(iz, ix, nx);
            accu_sxx[s] = sxx[i];
            accu_szx[s] = szx[i];
            accu_szz[s] = szz[i];
            accu_vx[s] = vx[i] / dt;
            accu_vz[s] = vz[i] / dt;
        }
    }
}

/* fwi_grad2, src/cpu/n_kernel_lib_PSV.cpp:439-484 (CPU sign -=, or the CUDA
 * path's += when grad_sign > 0). */
static void fwi_grad2(const orc_grid *g, double *grad_lam, double *grad_mu, double *grad_rho,
                      const double *accu_vz, const double *accu_vx, const double *accu_szz,
                      const double *accu_szx, const double *accu_sxx, const double *uz,
                      const double *ux, const double *szz, const double *szx, const double *sxx,
                      const double *lam, const double *mu, int tf)
{
    int snap_nt, snap_nz, snap_nx;
    snap_dims(g, &snap_nt, &snap_nz, &snap_nx);
    const int nx = g->nx, snap_dt = g->snap_dt;
    const double dt = g->dt;
    const size_t base = (size_t)tf * snap_nz * snap_nx;
#pragma omp parallel for
    for (int jz = 0; jz < snap_nz; jz++) {
        const int iz = g->snap_z1 + jz * g->snap_dz;
        for (int jx = 0; jx < snap_nx; jx++) {
            const int ix = g->snap_x1 + jx * g->snap_dx;
            const size_t s = base + IDX(jz, jx, snap_nx), i = IDX(iz, ix, nx);
            const size_t q = IDX(jz, jx, snap_nx);
            const double lm = lam[i] + mu[i];
            double s1 = 0.25 * (accu_szz[s] + accu_sxx[s]) * (szz[i] + sxx[i]) / (lm * lm);
            double s2 = 0.25 * (accu_szz[s] - accu_sxx[s]) * (szz[i] - sxx[i]) / (mu[i] * mu[i]);
            double s3 = (accu_szx[s] * szx[i]) / (mu[i] * mu[i]);
            double s4 = ux[i] * accu_vx[s] + uz[i] * accu_vz[s];
            if (g->grad_sign > 0) {
                grad_lam[q] += snap_dt * dt * s1;
                grad_mu[q] += snap_dt * dt * (s3 + s1 + s2);
                grad_rho[q] += snap_dt * dt * s4;
            } else {
                grad_lam[q] -= snap_dt * dt * s1;
                grad_mu[q] -= snap_dt * dt * (s3 + s1 + s2);
                grad_rho[q] -= snap_dt * dt * s4;
            }
        }
    }
}

/* kernel_PSV, src/cpu/n_kernel_PSV.cpp:20-213.  The derivative and CPML
 * memory arrays the reference passes in are internal here. */
void orc_kernel_PSV(const orc_grid *g, int ishot,
                    double *vz, double *vx, double *uz, double *ux,
                    double *szz, double *szx, double *sxx, double *We,
                    const double *lam, const double *mu, const double *mu_zx,
                    const double *rho_zp, const double *rho_xp,
                    int grad, double *grad_lam, double *grad_mu, double *grad_rho,
                    int nsrc, int stf_type, const double *stf_z, const double *stf_x,
                    const int *z_src, const int *x_src, const int *src_shot_to_fire,
                    int nrec, int rtf_type, double *rtf_uz, double *rtf_ux,
                    const int *z_rec, const int *x_rec,
                    int accu, double *accu_vz, double *accu_vx,
                    double *accu_szz, double *accu_szx, double *accu_sxx)
{
    const int nt = g->nt, nz = g->nz, nx = g->nx;
    const size_t n = (size_t)nz * nx;
    const int fpad = g->fdorder / 2;
    const int nz1 = fpad, nz2 = nz - fpad, nx1 = fpad, nx2 = nx - fpad; /* :70-71 */

    double *dz_z = zalloc(n), *dx_z = zalloc(n), *dz_x = zalloc(n), *dx_x = zalloc(n);
    double *m[8];
    for (int k = 0; k < 8; k++) m[k] = zalloc(n); /* reset_PML_memory2, :76-82 */
    double *mem_vz_z = m[0], *mem_vx_z = m[1], *mem_szz_z = m[2], *mem_szx_z = m[3];
    double *mem_vz_x = m[4], *mem_vx_x = m[5], *mem_szx_x = m[6], *mem_sxx_x = m[7];

    /* reset_sv2, :74 */
    memset(vz, 0, n * sizeof(double)); memset(vx, 0, n * sizeof(double));
    memset(uz, 0, n * sizeof(double)); memset(ux, 0, n * sizeof(double));
    memset(szz, 0, n * sizeof(double)); memset(szx, 0, n * sizeof(double));
    memset(sxx, 0, n * sizeof(double)); memset(We, 0, n * sizeof(double));

    if (grad) { /* reset_grad_shot2, :84-88 */
        int snap_nt, snap_nz, snap_nx;
        snap_dims(g, &snap_nt, &snap_nz, &snap_nx);
        const size_t ns = (size_t)snap_nz * snap_nx;
        memset(grad_lam, 0, ns * sizeof(double));
        memset(grad_mu, 0, ns * sizeof(double));
        memset(grad_rho, 0, ns * sizeof(double));
    }

    for (int jt = 0; jt < nt; jt++) { /* :90-210 */
        const int it = grad ? nt - jt - 1 : jt;

        vdiff2(g, dz_z, dx_z, dz_x, dx_x, vz, vx, nz1, nz2, nx1, nx2);
        if (g->pml_z || g->pml_x)
            pml_diff2(g, dz_z, dx_z, dz_x, dx_x, mem_vz_z, mem_vx_z, mem_vz_x, mem_vx_x, nz1,
                      nz2, nx1, nx2);
        update_s2(g, szz, szx, sxx, dz_z, dx_z, dz_x, dx_x, lam, mu, mu_zx, nz1, nz2, nx1, nx2);
        if (g->surf) surf_mirror(g, szz, szx, sxx, dz_z, dx_x, lam, mu, nz1, nz2, nx1, nx2);

        sdiff2(g, dz_z, dx_z, dz_x, dx_x, szz, szx, sxx, nz1, nz2, nx1, nx2);
        if (g->pml_z || g->pml_x)
            pml_diff2(g, dz_z, dx_z, dz_x, dx_x, mem_szz_z, mem_szx_z, mem_szx_x, mem_sxx_x,
                      nz1, nz2, nx1, nx2);
        update_v2(g, vz, vx, uz, ux, We, dz_z, dx_z, dz_x, dx_x, rho_zp, rho_xp, nz1, nz2, nx1,
                  nx2);

        if (nsrc)
            vsrc2(g, vz, vx, rho_zp, rho_xp, nsrc, stf_type, stf_z, stf_x, z_src, x_src,
                  src_shot_to_fire, ishot, it);
        if (nrec && !grad) urec2(g, rtf_type, rtf_uz, rtf_ux, vz, vx, nrec, z_rec, x_rec, it);

        if (!(it % g->snap_dt)) {
            const int tf = it / g->snap_dt;
            if (accu)
                gard_fwd_storage2(g, accu_vz, accu_vx, accu_szz, accu_szx, accu_sxx, vz, vx, szz,
                                  szx, sxx, tf);
            if (grad)
                fwi_grad2(g, grad_lam, grad_mu, grad_rho, accu_vz, accu_vx, accu_szz, accu_szx,
                          accu_sxx, uz, ux, szz, szx, sxx, lam, mu, tf);
        }
    }
    free(dz_z); free(dx_z); free(dz_x); free(dx_x);
    for (int k = 0; k < 8; k++) free(m[k]);
}

/* ------------------------------------------------------------------------ */
/* Line search                                                              */
/* ------------------------------------------------------------------------ */

/* calc_opt_step, src/cpu/n_step_length_PSV.cpp:461-518: vertex of the
 * parabola through (sl[i], L2[i]) with the reference's clamps.  The 3x3
 * system A x = b (A[i] = [1, sl, sl^2]) is solved by Gauss elimination
 * without pivoting, as the reference's solvelin intends
 * (include/cpu/n_solvelin.hpp:28-35), with back-substitution over k = 2..0. */
double orc_calc_opt_step(const double *L2, const double *sl)
{
    double A[3][3], b[3], x[3];
    for (int i = 0; i < 3; i++) {
        A[i][2] = sl[i] * sl[i];
        A[i][1] = sl[i];
        A[i][0] = 1.0;
        b[i] = L2[i];
    }
    for (int k = 0; k < 2; k++)
        for (int n = k; n < 2; n++) {
            double a = A[n + 1][k] / A[k][k];
            for (int m = 0; m < 3; m++) A[n + 1][m] = A[n + 1][m] - a * A[k][m];
            b[n + 1] = b[n + 1] - a * b[k];
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

/* ------------------------------------------------------------------------ */
/* Drivers                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t n, nsnap, nhist;
    double *vz, *vx, *uz, *ux, *szz, *szx, *sxx, *We, *We_adj;
    double *mu_zx, *rho_zp, *rho_xp;
    double *accu[5];
    double *rtf_uz, *rtf_ux;
    double *gl, *gm, *gr;
    int *rec_shot;
} work_t;

static void work_alloc(work_t *w, const orc_grid *g, const orc_shots *s, int need_hist)
{
    int snap_nt, snap_nz, snap_nx;
    snap_dims(g, &snap_nt, &snap_nz, &snap_nx);
    memset(w, 0, sizeof(*w));
    w->n = (size_t)g->nz * g->nx;
    w->nsnap = (size_t)snap_nz * snap_nx;
    w->nhist = (size_t)snap_nt * w->nsnap;
    w->vz = zalloc(w->n); w->vx = zalloc(w->n); w->uz = zalloc(w->n); w->ux = zalloc(w->n);
    w->szz = zalloc(w->n); w->szx = zalloc(w->n); w->sxx = zalloc(w->n);
    w->We = zalloc(w->n); w->We_adj = zalloc(w->n);
    w->mu_zx = zalloc(w->n); w->rho_zp = zalloc(w->n); w->rho_xp = zalloc(w->n);
    for (int k = 0; k < 5; k++) w->accu[k] = need_hist ? zalloc(w->nhist) : zalloc(1);
    w->rtf_uz = zalloc((size_t)s->nrec * g->nt);
    w->rtf_ux = zalloc((size_t)s->nrec * g->nt);
    w->gl = zalloc(w->nsnap); w->gm = zalloc(w->nsnap); w->gr = zalloc(w->nsnap);
    w->rec_shot = (int *)calloc(s->nrec ? s->nrec : 1, sizeof(int));
}

static void work_free(work_t *w)
{
    double *p[] = {w->vz, w->vx, w->uz, w->ux, w->szz, w->szx, w->sxx, w->We, w->We_adj,
                   w->mu_zx, w->rho_zp, w->rho_xp, w->accu[0], w->accu[1], w->accu[2],
                   w->accu[3], w->accu[4], w->rtf_uz, w->rtf_ux, w->gl, w->gm, w->gr};
    for (size_t k = 0; k < sizeof(p) / sizeof(p[0]); k++) free(p[k]);
    free(w->rec_shot);
}

static void run_forward(const orc_grid *g, const orc_shots *s, work_t *w, int ishot,
                        const double *lam, const double *mu, int accu)
{
    orc_kernel_PSV(g, ishot, w->vz, w->vx, w->uz, w->ux, w->szz, w->szx, w->sxx, w->We, lam, mu,
                   w->mu_zx, w->rho_zp, w->rho_xp, 0, w->gl, w->gm, w->gr, s->nsrc, s->stf_type,
                   s->stf_z, s->stf_x, s->z_src, s->x_src, s->src_shot_to_fire, s->nrec,
                   s->rtf_type, w->rtf_uz, w->rtf_ux, s->z_rec, s->x_rec, accu, w->accu[0],
                   w->accu[1], w->accu[2], w->accu[3], w->accu[4]);
}

/* Adjoint call of simulate_fwi_PSV, :336-356: all receivers fire this shot's
 * residuals as displacement sources (stf_type = rtf_type). */
static void run_adjoint(const orc_grid *g, const orc_shots *s, work_t *w, int ishot,
                        const double *lam, const double *mu)
{
    for (int ir = 0; ir < s->nrec; ir++) w->rec_shot[ir] = ishot;
    orc_kernel_PSV(g, ishot, w->vz, w->vx, w->uz, w->ux, w->szz, w->szx, w->sxx, w->We_adj, lam,
                   mu, w->mu_zx, w->rho_zp, w->rho_xp, 1, w->gl, w->gm, w->gr, s->nrec,
                   s->rtf_type, w->rtf_uz, w->rtf_ux, s->z_rec, s->x_rec, w->rec_shot, s->nrec,
                   s->rtf_type, w->rtf_uz, w->rtf_ux, s->z_rec, s->x_rec, 0, w->accu[0],
                   w->accu[1], w->accu[2], w->accu[3], w->accu[4]);
}

void orc_simulate_fwd(const orc_grid *g, const orc_shots *s, const double *lam,
                      const double *mu, const double *rho, double *rtf_uz_out, double *rtf_ux_out)
{
    work_t w;
    double C[3];
    work_alloc(&w, g, s, 0);
    orc_mat_av2(lam, mu, rho, w.mu_zx, w.rho_zp, w.rho_xp, C, g->nz, g->nx);
    const size_t nr = (size_t)s->nrec * g->nt;
    for (int ishot = 0; ishot < s->nshot; ishot++) {
        run_forward(g, s, &w, ishot, lam, mu, 0);
        memcpy(rtf_uz_out + ishot * nr, w.rtf_uz, nr * sizeof(double));
        memcpy(rtf_ux_out + ishot * nr, w.rtf_ux, nr * sizeof(double));
    }
    work_free(&w);
}

double orc_shot_gradient(const orc_grid *g, const orc_shots *s, int ishot,
                         const double *lam, const double *mu, const double *rho,
                         const double *rtf_uz_true, const double *rtf_ux_true,
                         double *grad_lam_shot, double *grad_mu_shot, double *grad_rho_shot,
                         double *We, double *We_adj, double *rtf_uz_mod, double *rtf_ux_mod)
{
    work_t w;
    double C[3];
    work_alloc(&w, g, s, 1);
    orc_mat_av2(lam, mu, rho, w.mu_zx, w.rho_zp, w.rho_xp, C, g->nz, g->nx);
    run_forward(g, s, &w, ishot, lam, mu, 1);
    const size_t nr = (size_t)s->nrec * g->nt;
    if (rtf_uz_mod) memcpy(rtf_uz_mod, w.rtf_uz, nr * sizeof(double));
    if (rtf_ux_mod) memcpy(rtf_ux_mod, w.rtf_ux, nr * sizeof(double));
    const double L2 = orc_adjsrc2(w.rtf_uz, w.rtf_ux, rtf_uz_true + ishot * nr,
                                  rtf_ux_true + ishot * nr, w.rtf_uz, w.rtf_ux, g->dt, s->nrec,
                                  g->nt);
    run_adjoint(g, s, &w, ishot, lam, mu);
    memcpy(grad_lam_shot, w.gl, w.nsnap * sizeof(double));
    memcpy(grad_mu_shot, w.gm, w.nsnap * sizeof(double));
    memcpy(grad_rho_shot, w.gr, w.nsnap * sizeof(double));
    if (We) memcpy(We, w.We, w.n * sizeof(double));
    if (We_adj) memcpy(We_adj, w.We_adj, w.n * sizeof(double));
    work_free(&w);
    return L2;
}

#define TRIAL_LOG_MAX 64

/* step_length_PSV, src/cpu/n_step_length_PSV.cpp:13-209 (update_param 0,
 * all shots per trial). */
static int step_length(const orc_grid *g, const orc_shots *s, work_t *w, double *est,
                       double L2_0, double *lam, double *mu, double *rho, const double *lam_copy,
                       const double *mu_copy, const double *rho_copy, const double *gl,
                       const double *gm, const double *gr, const double *rtf_z_true,
                       const double *rtf_x_true, int *ntrial, double *tlog)
{
    const double step_factor_rho = 0.5, scalefac = 2.0, stepmax_1 = 30, stepmax_2 = 4;
    double L2_test[3] = {L2_0, 0.0, 0.0}, sl[3] = {0.0, 0.0, 0.0}, C[3];
    unsigned int step1 = 0, step2 = 0, itests = 1, iteste = 1, countstep = 0;
    const size_t nr = (size_t)s->nrec * g->nt;
    double est_step_length = *est;
    *ntrial = 0;
    /* NaN misfits (a NaN gradient) make every comparison false and the
     * reference's loop endless; the engine fails there, so does this. */
    if (isnan(L2_0)) return -1;
    while ((step2 != 1) || (step1 != 1)) {
        double L2_tmp = 0;
        for (unsigned int itest = itests; itest <= iteste; itest++) {
            orc_update_mat2(lam, lam_copy, gl, 4.8e+10, 0.0, est_step_length, g->nz, g->nx);
            orc_update_mat2(mu, mu_copy, gm, 2.7e+10, 0.0, est_step_length, g->nz, g->nx);
            orc_update_mat2(rho, rho_copy, gr, 3000.0, 1.5, step_factor_rho * est_step_length,
                            g->nz, g->nx);
            orc_mat_av2(lam, mu, rho, w->mu_zx, w->rho_zp, w->rho_xp, C, g->nz, g->nx);
            L2_tmp = 0;
            for (int ishot = 0; ishot < s->nshot; ishot++) {
                run_forward(g, s, w, ishot, lam, mu, 0);
                L2_tmp += orc_adjsrc2(w->rtf_uz, w->rtf_ux, rtf_z_true + ishot * nr,
                                      rtf_x_true + ishot * nr, w->rtf_uz, w->rtf_ux, g->dt,
                                      s->nrec, g->nt);
            }
            L2_test[itest] = L2_tmp;
            sl[itest] = est_step_length;
            sl[0] = 0.0;
            if (*ntrial < TRIAL_LOG_MAX && tlog) {
                tlog[2 * *ntrial] = est_step_length;
                tlog[2 * *ntrial + 1] = L2_tmp;
            }
            (*ntrial)++;
            if (isnan(L2_tmp)) return -1;
        }
        if ((step1 == 0) && (L2_test[0] <= L2_test[1])) {
            est_step_length = est_step_length / scalefac;
            countstep++;
        }
        if ((step1 == 1) && (L2_test[1] < L2_test[2])) {
            sl[2] = est_step_length;
            step2 = 1;
        }
        if ((step1 == 1) && (L2_test[1] >= L2_test[2])) {
            sl[2] = est_step_length;
            est_step_length = est_step_length + (est_step_length / scalefac);
            countstep++;
        }
        if ((step1 == 0) && (L2_test[0] > L2_test[1])) {
            sl[1] = est_step_length;
            step1 = 1;
            iteste = 2;
            itests = 2;
            countstep = 0;
            est_step_length = est_step_length + (est_step_length / scalefac);
        }
        if ((step1 == 0) && (countstep > stepmax_1)) return -1; /* :173-178 exits */
        if ((step1 == 1) && (countstep > stepmax_2)) {
            step1 = 1;
            step2 = 1;
        }
    }
    if (step1 == 1) est_step_length = orc_calc_opt_step(L2_test, sl);
    *est = est_step_length;
    return 0;
}

int orc_step_length_cb(double *est_io, double L2_0, orc_trial_fn fn, void *ctx, int *ntrial,
                       double *tlog)
{
    const double scalefac = 2.0, stepmax_1 = 30, stepmax_2 = 4;
    double L2_test[3] = {L2_0, 0.0, 0.0}, sl[3] = {0.0, 0.0, 0.0};
    unsigned int step1 = 0, step2 = 0, itests = 1, iteste = 1, countstep = 0;
    double est_step_length = *est_io;
    *ntrial = 0;
    if (isnan(L2_0)) return -1; /* as in step_length above */
    while ((step2 != 1) || (step1 != 1)) {
        for (unsigned int itest = itests; itest <= iteste; itest++) {
            const double L2_tmp = fn(est_step_length, ctx);
            L2_test[itest] = L2_tmp;
            sl[itest] = est_step_length;
            sl[0] = 0.0;
            if (*ntrial < TRIAL_LOG_MAX && tlog) {
                tlog[2 * *ntrial] = est_step_length;
                tlog[2 * *ntrial + 1] = L2_tmp;
            }
            (*ntrial)++;
            if (isnan(L2_tmp)) return -1;
        }
        if ((step1 == 0) && (L2_test[0] <= L2_test[1])) {
            est_step_length = est_step_length / scalefac;
            countstep++;
        }
        if ((step1 == 1) && (L2_test[1] < L2_test[2])) {
            sl[2] = est_step_length;
            step2 = 1;
        }
        if ((step1 == 1) && (L2_test[1] >= L2_test[2])) {
            sl[2] = est_step_length;
            est_step_length = est_step_length + (est_step_length / scalefac);
            countstep++;
        }
        if ((step1 == 0) && (L2_test[0] > L2_test[1])) {
            sl[1] = est_step_length;
            step1 = 1;
            iteste = 2;
            itests = 2;
            countstep = 0;
            est_step_length = est_step_length + (est_step_length / scalefac);
        }
        if ((step1 == 0) && (countstep > stepmax_1)) return -1;
        if ((step1 == 1) && (countstep > stepmax_2)) {
            step1 = 1;
            step2 = 1;
        }
    }
    if (step1 == 1) est_step_length = orc_calc_opt_step(L2_test, sl);
    *est_io = est_step_length;
    return 0;
}

int orc_simulate_fwi(const orc_grid *g, const orc_shots *s, double *lam, double *mu, double *rho,
                     const double *rtf_z_true, const double *rtf_x_true, const int *taper8,
                     int niter, double step0, double *grad_lam, double *grad_mu, double *grad_rho,
                     double *L2_out, double *step_out, int *trials_out, double *trial_log)
{
    const int nz = g->nz, nx = g->nx;
    work_t w;
    work_alloc(&w, g, s, 1);
    const size_t n = w.n, nr = (size_t)s->nrec * g->nt;
    double *lam_copy = zalloc(n), *mu_copy = zalloc(n), *rho_copy = zalloc(n);
    double C[3];
    double step = step0; /* :243 */
    int rc = 0;
    for (int iterstep = 0; iterstep < niter; iterstep++) {
        double L2 = 0.0;
        memcpy(lam_copy, lam, n * sizeof(double)); /* copy_mat, :263 */
        memcpy(mu_copy, mu, n * sizeof(double));
        memcpy(rho_copy, rho, n * sizeof(double));
        orc_mat_av2(lam, mu, rho, w.mu_zx, w.rho_zp, w.rho_xp, C, nz, nx); /* :266 */
        for (int ishot = 0; ishot < s->nshot; ishot++) {
            run_forward(g, s, &w, ishot, lam, mu, 1);                     /* :279-290 */
            L2 += orc_adjsrc2(w.rtf_uz, w.rtf_ux, rtf_z_true + ishot * nr, /* :320 */
                              rtf_x_true + ishot * nr, w.rtf_uz, w.rtf_ux, g->dt, s->nrec,
                              g->nt);
            run_adjoint(g, s, &w, ishot, lam, mu);                         /* :344-356 */
            orc_energy_weights2(w.We, w.We_adj, nx, g->snap_z1, g->snap_z2, g->snap_x1,
                                g->snap_x2, NULL);                         /* :385 */
            const double *gs[3] = {w.gl, w.gm, w.gr};
            double *gg[3] = {grad_lam, grad_mu, grad_rho};
            for (int p = 0; p < 3; p++) { /* :394-417 */
                orc_interpol_grad2(w.We_adj, gs[p], nx, g->snap_z1, g->snap_z2, g->snap_x1,
                                   g->snap_x2, g->snap_dz, g->snap_dx);
                orc_scale_grad_E2(gg[p], w.We_adj, C[p], w.We, nx, g->snap_z1, g->snap_z2,
                                  g->snap_x1, g->snap_x2);
            }
        }
        L2_out[iterstep] = L2;
        orc_taper2(grad_lam, nz, nx, g->snap_z1, g->snap_z2, g->snap_x1, g->snap_x2, taper8);
        orc_taper2(grad_mu, nz, nx, g->snap_z1, g->snap_z2, g->snap_x1, g->snap_x2, taper8);
        orc_taper2(grad_rho, nz, nx, g->snap_z1, g->snap_z2, g->snap_x1, g->snap_x2, taper8);
        int ntrial = 0;
        rc = step_length(g, s, &w, &step, L2, lam, mu, rho, lam_copy, mu_copy, rho_copy,
                         grad_lam, grad_mu, grad_rho, rtf_z_true, rtf_x_true, &ntrial,
                         trial_log ? trial_log + (size_t)iterstep * 2 * TRIAL_LOG_MAX : NULL);
        if (trials_out) trials_out[iterstep] = ntrial;
        if (rc) break;
        step_out[iterstep] = step;
        orc_update_mat2(lam, lam_copy, grad_lam, 4.8e+10, 0.0, step, nz, nx); /* :542-546 */
        orc_update_mat2(mu, mu_copy, grad_mu, 2.7e+10, 0.0, step, nz, nx);
        orc_update_mat2(rho, rho_copy, grad_rho, 3000.0, 1.25, 0.5 * step, nz, nx);
    }
    free(lam_copy); free(mu_copy); free(rho_copy);
    work_free(&w);
    return rc;
}
