// psv_fwi.cuh -- model-side kernels: material averages and scaled
// coefficients, misfit, gradient preconditioning and model update.  These
// run once per shot or per iteration and are memory-bound elementwise or
// reduction passes; model, gradients and traces stay FP64 as in the
// reference, only the per-step coefficients are in the wavefield precision.
#pragma once

#include <cuda_runtime.h>

namespace psv {

// Inputs of mat_av2 + coefficient scaling for one model.
template <typename T>
struct CoeffParams {
    int nz, nx, pitch;
    double dt, kimg;                 // kimg = snap_dt * dt
    double gscale;                   // power of two applied to g1, g2
    const double *lam, *mu, *rho;    // [nz][nx]; rho may be null when avg given
    const double *mu_zx, *rho_zp, *rho_xp;  // given averages [nz][nx] or null
    T *c_lam, *c_l2m, *c_muzx, *c_rz, *c_rx, *g1, *g2;  // [nz][pitch]
    int st, sb, sl, sr;
    T *fs_top, *fs_bot, *fs_left, *fs_right;
};

// Interpolation / scaling of one batch of snapped shot gradients into the
// global gradients (interpol_grad2 + energy_weights2 + scale_grad_E2).
template <typename T>
struct ScaleParams {
    int nz, nx, pitch;
    int z1, z2, x1, x2, sdz, sdx;        // snapshot window
    int snx_pitch;
    long long snap_plane;
    const T *gshot;                      // [batch][3][snz][snx_pitch]
    long long gshot_shot_stride;
    const T *fld;                        // [batch][NFIELD][nz][pitch] (We, We_adj)
    long long plane, shot_stride;
    const double *wmax;                  // [batch] max of sqrt(We We_adj) over the window
    const double *fscale, *ascale;       // [nshot] forward / adjoint amplitude scales
    int s0;                              // global index of batch shot 0
    double gun[3];                       // unscale of the g1/g2-weighted planes (1/gscale) and of rho (1)
    double C[3];                         // scalar averages C_lam, C_mu, C_rho
    double *grad[3];                     // [nz][nx] global gradients
    int nbatch;
};

template <typename T> cudaError_t launch_coeffs(const CoeffParams<T> &c, cudaStream_t st);
template <typename T>
cudaError_t launch_energy_max(const T *fld, long long plane, long long shot_stride, int pitch,
                              int z1, int z2, int x1, int x2, int nbatch, double *wmax,
                              cudaStream_t st);
template <typename T> cudaError_t launch_scale(const ScaleParams<T> &s, cudaStream_t st);

// Per-shot max |residual| (bit patterns into rmax_bits[shot], zeroed here)
// and the adjoint amplitude scale 2^-round(log2(rmax * inj)) of each shot.
cudaError_t launch_adjoint_scale(const double *res_z, const double *res_x, long long n_per_shot,
                                 int nshot, double inj, unsigned long long *rmax_bits,
                                 double *ascale, cudaStream_t st);

// Deterministic FP64 sums: partial sums by a fixed grid, then one block.
cudaError_t launch_model_sums(const double *lam, const double *mu, const double *rho, int nz,
                              int nx, double *partial, double *out3, cudaStream_t st);
// Blocks of the first stage of the deterministic reductions: launch_adjsrc
// writes kRedBlocks partial sums per shot, launch_model_sums 3 * kRedBlocks.
constexpr int kRedBlocks = 256;

// Residual res = mod - true (skipped when res_z is null) and L2 of nshot
// shots, traces [shot][nt][nrec]; L2 of each shot into out[shot].  partial
// needs nshot * kRedBlocks doubles.
cudaError_t launch_adjsrc(const double *mod_z, const double *mod_x, const double *true_z,
                          const double *true_x, double *res_z, double *res_x,
                          long long n_per_shot, int nshot, double dt, double *partial,
                          double *out, cudaStream_t st);
cudaError_t launch_taper(double *A, int nz, int nx, const double *tx, const double *tz,
                         cudaStream_t st);
// update_mat2: max|grad|, max|old| then the clamped update.
cudaError_t launch_update_mat(double *mat, const double *old, const double *grad, int n,
                              double mat_max, double mat_min, double step,
                              unsigned long long *maxbits2, cudaStream_t st);

// apply_gauss_filter on nplanes planes of nz x nx values (row pitch `pitch`,
// plane stride `plane`): dst at [hfs, nz - hfs - 1) x [hfs, nx - hfs - 1)
// takes the (2 hfs + 1)^2 weighted sum of src in FP64 (filter row outer,
// column inner); dst elsewhere is left alone.  filt is on the device.
template <typename T>
cudaError_t launch_gauss_filter(const T *src, T *dst, long long plane, int pitch, int nz, int nx,
                                int nplanes, const double *filt, int hfs, cudaStream_t st);
// PCG_PSV on n values: beta = |g|^2 / |old|^2 (0 when |old|^2 = 0, clipped
// at 0), old <- -g, dir <- -g + beta dir, g <- dir.  part needs
// 2 * PCG_BLOCKS doubles.
constexpr int PCG_BLOCKS = 304;
cudaError_t launch_pcg(double *dir, double *old, double *g, long long n, double *part,
                       cudaStream_t st);

}  // namespace psv
