/*
 * psv_oracle.h -- FP64 CPU restatement of the reference P/SV path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is used by the
 * tests, by the smoke check and by the CPU-baseline leg of bench.py, never by
 * the product path (fwi_cuda_gb300/), which has no CPU fallback.
 *
 * Every function restates one function of the reference
 * (Mohammad-debug/FWI_CUDA, CPU path under src/cpu and src/h_*.cpp) and cites
 * the file:line it follows.  Arithmetic is FP64 with the same operation
 * order as the reference so that, compiled without FMA contraction, results
 * agree bit for bit with the reference compiled the same way.
 *
 * Arrays are flat and row-major: a field is [nz][nx] (index iz*nx+ix), a
 * time function is [n][nt], a snapshot history is [snap_nt][snap_nz][snap_nx]
 * (the reference's allocate_array layouts, include/cpu/n_contiguous_arrays.hpp:7-66).
 *
 * One addition beyond the reference: stencil = ORC_STENCIL_HOLBERG evaluates
 * the full 2N-point staggered Holberg derivative (N = fdorder/2) instead of
 * the reference's 2-point difference scaled by hc[1]
 * (src/cpu/n_kernel_lib_PSV.cpp:125-128,230-233).  ORC_STENCIL_REFERENCE is
 * the reference as written.
 */
#ifndef PSV_ORACLE_H
#define PSV_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PI 3.14159265 /* include/cpu/n_globvar.hpp:15 -- the reference's PI */

#define ORC_STENCIL_REFERENCE 0
#define ORC_STENCIL_HOLBERG 1

/* Grid, boundary and snapshot geometry shared by every kernel call. */
typedef struct {
    int nt, nz, nx;
    double dt, dx, dz;
    int surf;      /* free surface present (h_simulate_PSV.cpp:36) */
    int isurf[4];  /* 0 top, 1 bottom, 2 left, 3 right; 0 = none */
    double hc[7];  /* Holberg coefficients (h_holbergcoeff.cpp:21) */
    int fdorder;
    int stencil;   /* ORC_STENCIL_REFERENCE or ORC_STENCIL_HOLBERG */
    int pml_z, pml_x;
    const double *a_z, *b_z, *K_z, *a_half_z, *b_half_z, *K_half_z; /* [nz] */
    const double *a_x, *b_x, *K_x, *a_half_x, *b_half_x, *K_half_x; /* [nx] */
    int snap_z1, snap_z2, snap_x1, snap_x2, snap_dt, snap_dz, snap_dx;
    /* Sign of the imaging condition: -1 (or 0) = the reference's CPU path
     * (grad -= ..., src/cpu/n_kernel_lib_PSV.cpp:477-479); +1 = its CUDA path
     * (grad += ..., src/cuda/d_kernel_lib_PSV.cu:838-840). */
    int grad_sign;
} orc_grid;

/* Sources / receivers of a survey (h_simulate_PSV.cpp:46-56). */
typedef struct {
    int nshot, nsrc, nrec, stf_type, rtf_type;
    const int *z_src, *x_src, *src_shot_to_fire; /* [nsrc] */
    const double *stf_z, *stf_x;                  /* [nsrc][nt] */
    const int *z_rec, *x_rec;                     /* [nrec] */
} orc_shots;

void orc_set_threads(int n);

/* ---- host preprocessing (src/h_*.cpp) ---- */
void orc_holbergcoeff(int fdorder, int maxrelerror, double *hc7);
void orc_cpml_PSV(double *a, double *b, double *K, double *a_half, double *b_half, double *K_half,
                  double npower, double damp_v_PML, double rcoef, double k_max_PML, double freq,
                  int npml_h1, int npml_h2, int fpad, int nh, double dt, double dh);
void orc_wavelet(double *signal, int nt, double dt, double amp, double fc, double ts, int shape);
/* out[0]=dtstab, out[1]=dhstab, out[2]=cmax, out[3]=cmin; returns 1 when the
 * absorbing frame is wider than the domain (the reference exits there). */
int orc_checkfd_ssg_elastic(int nz, int nx, double dh, double dt, double ts, int fw,
                            const double *rho, const double *lam, const double *mu,
                            const double *hc, double *out);

/* ---- kernel library (src/cpu/n_kernel_lib_PSV.cpp) ---- */
void orc_mat_av2(const double *lam, const double *mu, const double *rho,
                 double *mu_zx, double *rho_zp, double *rho_xp, double *C3, int nz, int nx);
double orc_adjsrc2(double *a_stf_uz, double *a_stf_ux, const double *rtf_uz_true,
                   const double *rtf_ux_true, const double *rtf_uz_mod, const double *rtf_ux_mod,
                   double dt, int nseis, int nt);
void orc_interpol_grad2(double *grad, const double *grad_shot, int nx, int snap_z1, int snap_z2,
                        int snap_x1, int snap_x2, int snap_dz, int snap_dx);
void orc_energy_weights2(double *We, const double *We_adj, int nx, int snap_z1, int snap_z2,
                         int snap_x1, int snap_x2, double *max_out3);
void orc_scale_grad_E2(double *grad, const double *grad_shot, double mat_av, const double *We,
                       int nx, int snap_z1, int snap_z2, int snap_x1, int snap_x2);
void orc_update_mat2(double *mat, const double *mat_old, const double *grad_mat, double mat_max,
                     double mat_min, double step_length, int nz, int nx);
int orc_gauss_filter_kernel(int hfs, double *k);
void orc_apply_gauss_filter(double *mat, int nz, int nx, const double *filt, int hfs);
void orc_PCG_PSV(double *dir, double *old, double *grad, int nz, int nx);
void orc_taper2(double *A, int nz, int nx, int snap_z1, int snap_z2, int snap_x1, int snap_x2,
                const int *taper8 /* t1 t2 b1 b2 l1 l2 r1 r2 */);

/* ---- the per-shot time loop (src/cpu/n_kernel_PSV.cpp:20-213) ---- */
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
                    double *accu_szz, double *accu_szx, double *accu_sxx);

/* ---- line search (src/cpu/n_step_length_PSV.cpp:461-518) ---- */
/* Parabola vertex with a correct 3x3 Gauss solve (the reference's
 * back-substitution, include/cpu/n_solvelin.hpp:37-42, indexes past the end). */
double orc_calc_opt_step(const double *L2, const double *sl);

/* step_length_PSV's control flow (src/cpu/n_step_length_PSV.cpp:83-208)
 * with the trial forwards replaced by a callback returning L2(step). */
typedef double (*orc_trial_fn)(double step, void *ctx);
int orc_step_length_cb(double *est, double L2_0, orc_trial_fn fn, void *ctx, int *ntrial,
                       double *tlog);

/* ---- drivers (src/cpu/n_simulate_PSV.cpp) ---- */
/* Forward modelling of all shots (simulate_fwd_PSV, :18-149): receiver
 * displacements out [nshot][nrec][nt] x2. */
void orc_simulate_fwd(const orc_grid *g, const orc_shots *s, const double *lam,
                      const double *mu, const double *rho, double *rtf_uz_out, double *rtf_ux_out);

/* One shot's forward + residual + adjoint (simulate_fwi_PSV :279-356): the
 * per-shot snapped gradients, the forward and adjoint energies, and the L2
 * misfit.  Material averages are computed inside (mat_av2). */
double orc_shot_gradient(const orc_grid *g, const orc_shots *s, int ishot,
                         const double *lam, const double *mu, const double *rho,
                         const double *rtf_uz_true, const double *rtf_ux_true,
                         double *grad_lam_shot, double *grad_mu_shot, double *grad_rho_shot,
                         double *We, double *We_adj, double *rtf_uz_mod, double *rtf_ux_mod);

/* niter FWI iterations (simulate_fwi_PSV :153-597 with step_length_PSV
 * n_step_length_PSV.cpp:13-209).  lam/mu/rho are updated in place.  grad_*
 * are the global gradients, carried in and out (the reference never resets
 * them, :260).  Logs: L2[niter], step[niter], trials[niter] (trial forwards
 * per iteration), trial_log[niter][64][2] (alpha, L2 of each trial).
 * Returns 0, or -1 when the step search fails (the reference exits). */
int orc_simulate_fwi(const orc_grid *g, const orc_shots *s, double *lam, double *mu, double *rho,
                     const double *rtf_z_true, const double *rtf_x_true, const int *taper8,
                     int niter, double step0, double *grad_lam, double *grad_mu, double *grad_rho,
                     double *L2_out, double *step_out, int *trials_out, double *trial_log);

#ifdef __cplusplus
}
#endif
#endif
