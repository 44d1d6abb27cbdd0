/*
 * fwi_psv.h -- C ABI of the GB300 P/SV finite-difference engine.
 *
 * The engine replaces the time loop of Mohammad-debug/FWI_CUDA (kernel_PSV,
 * include/cpu/n_kernel_PSV.hpp:8-43, and its CUDA twin kernel_PSV_GPU,
 * include/cuda/d_kernel_PSV.cuh:9-44) and the shot/FWI drivers that call it
 * (simulate_fwd_PSV / simulate_fwi_PSV, include/cpu/n_simulate_PSV.hpp:23-44;
 * step_length_PSV, include/cpu/n_step_length_PSV.hpp:17).  Wavefields live on
 * one GB300 in FP32 (or FP64 on request); every array crossing this boundary
 * is a caller-owned HOST array in FP64 with the reference's row-major layout:
 *   field          [nz][nx]
 *   time function  [n][nt]           (stf, one shot's seismograms)
 *   survey traces  [nshot][nrec][nt]  (rtf_*_true, allocate_array(...,nshot,nrec,nt))
 *   snapshot       [snap_nt][snap_nz][snap_nx]
 *
 * Conventions (the reference prints and calls exit(0) on errors,
 * include/cuda/d_globvar.cuh:23-29; this ABI never exits):
 *   - every function returns a psv_status; psv_last_error() gives the text;
 *   - no host memory is retained after a call returns;
 *   - a plan is used by one host thread at a time; plans are independent;
 *   - there is no CPU fallback: without a usable GPU calls return
 *     PSV_ERR_CUDA.
 */
#ifndef FWI_PSV_H
#define FWI_PSV_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PSV_OK = 0,
    PSV_ERR_ARG = 1,          /* invalid or inconsistent argument */
    PSV_ERR_CFL = 2,          /* time step above the stability limit */
    PSV_ERR_OOM = 3,          /* device memory or HBM budget exceeded */
    PSV_ERR_CUDA = 4,         /* CUDA runtime error / no device */
    PSV_ERR_UNSUPPORTED = 5,  /* valid for the reference, not implemented here */
    PSV_ERR_TIMEOUT = 6,      /* a bounded device wait gave up */
    PSV_ERR_STEP_SEARCH = 7,  /* step-length search failed (reference: exit(0)) */
    PSV_ERR_IO = 8            /* file missing / short read / write failed */
} psv_status;

#define PSV_STENCIL_REFERENCE 0 /* reference: 2-point difference x hc[1], pad fdorder/2 */
#define PSV_STENCIL_HOLBERG 1   /* full 2N-point staggered Holberg stencil, N = fdorder/2 */

#define PSV_STORE_AUTO 0        /* full history when it fits the budget, else CHECKPOINT,
                                   else BINOMIAL */
#define PSV_STORE_FULL 1        /* every snapshot kept in HBM (the reference's accu_*) */
#define PSV_STORE_CHECKPOINT 2  /* a state at every segment start + one recomputed forward */
#define PSV_STORE_BINOMIAL 3    /* fewer state slots than segments, placed by Griewank's
                                   binomial schedule (more recomputation, less memory) */

/* Time-step kernel families (psv_options.kernel_family). */
#define PSV_KERNELS_DIRECT 1    /* per-thread loads of the stencil neighbours */
#define PSV_KERNELS_TMA 2       /* tiles staged in shared memory by TMA tensor copies (FP32) */
#define PSV_KERNELS_VEC4 3      /* four columns per thread, 128-bit loads and stores (FP32) */
#define PSV_KERNELS_FUSED 4     /* one launch per time step: stress of a tile and its halo,
                                   then its velocities, from shared memory (FP32) */
#define PSV_KERNELS_MARCH 5     /* one launch per time step: each CTA marches down a strip of
                                   columns, stress then velocity row by row, stencil windows
                                   in registers, rows staged ahead by cp.async (FP32) */

/* Size limits (PSV_ERR_UNSUPPORTED above them).  The reference has none
 * besides memory; here grid rows and shots map to CUDA grid dimensions and
 * the time-step kernels address one shot's field planes with 32-bit offsets:
 * nz x (nx padded to 128 bytes) x planes, 14 planes in FP32 (the second
 * velocity / stress copy of the FUSED family included), 9 in FP64. */
#define PSV_MAX_NZ 65535
#define PSV_MAX_SHOTS 65535
#define PSV_MAX_SHOT_ELEMS 2147483647LL

const char *psv_error_string(int status);
/* Message of the last failing call on this host thread. */
const char *psv_last_error(void);
/* 1 when a CUDA device is usable, else 0. */
int psv_device_available(void);

/* ------------------------------------------------------------------------ */
/* Host preprocessing (FP64, bitwise equal to the reference's formulas).     */
/* ------------------------------------------------------------------------ */

/* Replaces holbergcoeff, include/h_holbergcoeff.hpp:23 (hc7 has 7 entries). */
int psv_holbergcoeff(int fdorder, int maxrelerror, double *hc7);

/* Replaces cpml_PSV, include/h_preproc_PSV.hpp:41-44 (arrays of length nh). */
int psv_cpml_PSV(double *a, double *b, double *K, double *a_half, double *b_half,
                 double *K_half, double npower, double damp_v_PML, double rcoef,
                 double k_max_PML, double freq, int npml_h1, int npml_h2, int fpad, int nh,
                 double dt, double dh);

/* Replaces wavelet, include/h_preproc_PSV.hpp:48 (shape 1 = Ricker). */
int psv_wavelet(double *signal, int nt, double dt, double amp, double fc, double ts, int shape);

/* Replaces checkfd_ssg_elastic, include/h_checkfd_ssg_elastic.hpp:16.
 * out4 = {dtstab, dhstab, cmax, cmin}.  Returns PSV_ERR_CFL when dt > dtstab,
 * PSV_ERR_ARG when the absorbing frame fw exceeds the domain (where the
 * reference exits), else PSV_OK. */
int psv_checkfd_ssg_elastic(int nz, int nx, double dh, double dt, double ts, int fw,
                            const double *rho, const double *lam, const double *mu,
                            const double *hc7, double *out4);

/* ------------------------------------------------------------------------ */
/* Survey description                                                         */
/* ------------------------------------------------------------------------ */

typedef struct psv_grid {
    int nt, nz, nx;
    double dt, dx, dz;
    int fdorder;         /* 2, 4, 6 or 8 */
    int stencil;         /* PSV_STENCIL_* */
    int surf;            /* free surface present */
    int isurf[4];        /* 0 top, 1 bottom, 2 left, 3 right; 0 = none */
    double hc[7];        /* psv_holbergcoeff output */
    int pml_z, pml_x;
    /* CPML profiles (psv_cpml_PSV output): [nz] for *_z, [nx] for *_x.
     * Ignored (may be NULL) when the axis has no PML. */
    const double *a_z, *b_z, *K_z, *a_half_z, *b_half_z, *K_half_z;
    const double *a_x, *b_x, *K_x, *a_half_x, *b_half_x, *K_half_x;
    /* Snapshot / gradient window, inclusive, and subsampling. */
    int snap_z1, snap_z2, snap_x1, snap_x2, snap_dt, snap_dz, snap_dx;
    /* Tukey taper of the gradient: t1 t2 b1 b2 l1 l2 r1 r2 (taper2). */
    int taper[8];
    /* Sign of the imaging condition.  <= 0: the reference's CPU path,
     * grad -= ... (src/cpu/n_kernel_lib_PSV.cpp:477-479); > 0: its CUDA path,
     * grad += ... (src/cuda/d_kernel_lib_PSV.cu:838-840).  The two differ by
     * an exact negation of every gradient. */
    int imaging_sign;
} psv_grid;

typedef struct psv_shots {
    int nshot, nsrc, nrec;
    int stf_type;                /* 0 displacement, 1 velocity (vsrc2) */
    int rtf_type;                /* 0 displacement (urec2) */
    const int *z_src, *x_src;    /* [nsrc] grid indices */
    const int *src_shot_to_fire; /* [nsrc] shot index that fires each source */
    const double *stf_z, *stf_x; /* [nsrc][nt] */
    const int *z_rec, *x_rec;    /* [nrec] */
} psv_shots;

typedef struct psv_options {
    int precision;              /* 32 (default) or 64 */
    int storage;                /* PSV_STORE_* */
    double hbm_budget_gb;       /* device memory the plan may use; 0 = 180 */
    int checkpoint_interval;    /* CHECKPOINT / BINOMIAL storage: steps per segment, 0 = auto
                                   (balanced for CHECKPOINT, snap_dt for BINOMIAL) */
    int max_batch;              /* shots per launch; 0 = all shots of the survey */
    int use_graphs;             /* capture the time loop in CUDA graphs (default 1) */
    int block_x, block_y;       /* thread-block shape of the stencil kernels (block_x = 32;
                                   MARCH family: block_y = warps per CTA, 2 or 4); 0 = default */
    int rows_per_thread;        /* rows each thread marches: direct family 1, 2, 4 (negative:
                                   warp-shuffle variant); TMA family 2, 4, 8; VEC4 family
                                   1, 2, 4; FUSED family: tile rows 16 or 32; MARCH family:
                                   rows each CTA marches, 32, 64 or 128; 0 = default */
    int kernel_family;          /* time-step kernels: 0 = any (the autotuner chooses),
                                   PSV_KERNELS_DIRECT, _TMA, _VEC4, _FUSED or _MARCH (the
                                   last four FP32 only; FUSED needs no free surface but a top
                                   one, MARCH none or a top one on the first interior row) */
    int autotune;               /* 1 (default): time the kernel candidates (family, tile
                                   shape and, for the direct family, the chain count) on the
                                   first gradient and keep the fastest (psv_plan_autotune);
                                   0: use block_y / rows_per_thread / chains as given */
    int checkpoint_slots;       /* BINOMIAL storage: state slots per shot (segment 0's
                                   included); 0 = the fewest with at most two forward
                                   repetitions, fewer if the budget holds fewer */
    int smooth_hfs;             /* >= 2: Gaussian smoothing (half size hfs) of every shot's
                                   gradients before the energy preconditioning, where the
                                   reference's commented-out apply_gauss_filter calls sit
                                   (src/cpu/n_simulate_PSV.cpp:377-379); 0 = off */
    int pcg;                    /* 1: psv_fwi_iteration turns the global gradients into
                                   Fletcher-Reeves directions before the taper (the
                                   reference's commented-out PCG_PSV calls, :433-435) */
    int chains;                 /* direct family: the batch's shots split into 1, 2 or 4
                                   groups whose time loops run on their own streams (each
                                   group's launches fill the others' kernel boundaries;
                                   checkpointed passes join them around every state copy);
                                   0 = the autotuner picks */
    int adjoint;                /* PSV_ADJOINT_REFERENCE (default): the reference's imaging
                                   condition (fwi_grad2) with its energy preconditioning;
                                   PSV_ADJOINT_EXACT: the derivative of L2 itself (see below) */
} psv_options;

/* Adjoint modes (psv_options.adjoint).  EXACT has no counterpart in the
 * reference: psv_gradient then accumulates -imaging_sign * dL2/dm (m = lam,
 * mu, rho on every cell, no energy preconditioning) into the global
 * gradients, computed by the hand-transposed discrete adjoint of the whole
 * time loop (CPML, free surface, staggered averages, sources and receivers
 * included), the same orientation the reference mode's imaging term has.
 * FP64 plans only, no or a top free surface, displacement receivers
 * (rtf_type 0); the forward stores 8 planes per step and shot, so it is for
 * verification-sized grids (PSV_ERR_OOM beyond the budget).  Per-shot
 * imaging terms (psv_plan_get_shot_gradient) do not exist in this mode. */
#define PSV_ADJOINT_REFERENCE 0
#define PSV_ADJOINT_EXACT 1

void psv_options_default(psv_options *opt);

typedef struct psv_plan psv_plan;

/* Allocates the device state of a survey (wavefields of max_batch shots,
 * snapshot storage or checkpoints, materials, traces).  The grid/shots
 * arrays are copied; the caller may free them afterwards. */
int psv_plan_create(const psv_grid *grid, const psv_shots *shots, const psv_options *opt,
                    psv_plan **out);
int psv_plan_destroy(psv_plan *plan);
/* Bytes of device memory the plan holds. */
long long psv_plan_device_bytes(const psv_plan *plan);

/* Sets lam/mu/rho [nz][nx] (host FP64) and derives the staggered averages
 * and scaled coefficients on the device (mat_av2, n_kernel_lib_PSV.hpp:170). */
int psv_plan_set_model(psv_plan *plan, const double *lam, const double *mu, const double *rho);
int psv_plan_get_model(psv_plan *plan, double *lam, double *mu, double *rho);
/* Observed traces rtf_*_true [nshot][nrec][nt] (read_seismo, h_io_PSV.hpp:34). */
int psv_plan_set_observed(psv_plan *plan, const double *rtf_uz_true, const double *rtf_ux_true);

/* Forward modelling of every shot (simulate_fwd_PSV's shot loop,
 * n_simulate_PSV.hpp:23): receiver displacements [nshot][nrec][nt]. */
int psv_forward(psv_plan *plan, double *rtf_uz, double *rtf_ux);

/* One FWI gradient over every shot, in the reference's order
 * (simulate_fwi_PSV's shot loop, src/cpu/n_simulate_PSV.cpp:270-419):
 * forward with snapshots, residual and L2 (adjsrc2), time-reversed adjoint
 * with the imaging condition, energy weights, interpolation and scaling
 * added into the plan's global gradients.  The global gradients are NOT
 * reset (the reference never resets them, :260); see psv_reset_gradient.
 * L2 = sum over shots.  grad_* (host [nz][nx], may be NULL) receive the
 * global gradients after the call. */
int psv_gradient(psv_plan *plan, double *L2, double *grad_lam, double *grad_mu,
                 double *grad_rho);

/* Several surveys at once (uneven grid sizes, time-step counts and stencil
 * orders: one plan each, all created on the calling thread's current
 * device).  Runs psv_forward / psv_gradient of every plan concurrently, each
 * on its plan's own stream and host thread, so the GPU overlaps the surveys'
 * time loops; one call, not one kernel launch.  Plans still due an autotune
 * are tuned one after another first, so their timings are not disturbed.
 * The same plan may not appear twice.  forward: uz[k], ux[k] as in
 * psv_forward for plan k (entries may be NULL); gradient: L2[k] per plan
 * (may be NULL), the global gradients stay on each plan (psv_get_gradient).
 * The first failing plan's status is returned, its message prefixed with its
 * index.  No counterpart in the reference (one survey per program run). */
int psv_multi_forward(psv_plan *const *plans, int nplans, double *const *rtf_uz,
                      double *const *rtf_ux);
int psv_multi_gradient(psv_plan *const *plans, int nplans, double *L2);

/* Joint passes: up to 8 surveys (one plan each, all of one precision)
 * stepped in ONE stress launch and ONE velocity launch per time step, whose
 * blocks cover every shot of every survey still running.  Grid sizes,
 * stencil orders (mixed in one launch), shot counts and step counts may
 * differ; a survey leaves the launches after its last step.  Plans whose
 * shots take several batches (max_batch, HBM budget) run batch by batch:
 * the joint launches cover batch b of every plan that has one.  Each pass
 * of each batch is one CUDA graph, captured by the first call and replayed
 * by the later ones.
 *   psv_joint_create: the plans and the tile shape of the joint launches
 *     (rows_per_thread 1 or 2, FP64: 1; blocks of 32 x block_y threads,
 *     block_y 1..8), or rows_per_thread 0: the first psv_joint_forward
 *     times the first steps (up to 24) of the joint loop for each of a few
 *     shapes and keeps the fastest.  Every psv_joint_forward sets each plan
 *     to the direct kernel family with the joint shape (psv_plan_shape
 *     reports it; the plan's own passes then use it too).
 *   psv_joint_shape: the joint shape (0, 0 while an autotune is pending).
 *   psv_joint_forward: psv_forward of every plan (uz[k], ux[k] as there;
 *     NULL arrays or entries skip the download); *ms (may be NULL) gets the
 *     device time of the joint time loop.  The operations per grid point are
 *     those of each plan's own psv_forward with the same tile shape; the
 *     joint kernels' compiled multiply-add contraction may differ, so traces
 *     agree to rounding (FP32 relative L2 ~1e-8), not bit for bit.  One
 *     joint pass runs at a time per process (the survey tables are in
 *     constant memory).
 *   psv_joint_gradient: psv_gradient of every plan (with its observed
 *     traces; any storage: full history, two-level or binomial
 *     checkpoints): the gradient forward pass of all surveys in one launch
 *     pair per joint step, residuals and adjoint sources per plan, then the
 *     adjoint pass of all surveys in one launch pair per joint step, each
 *     survey at its own step of its own sequence (time-reversed adjoint
 *     steps, and with checkpoints its schedule's recomputed segments, the
 *     state copies enqueued between the launches), preconditioning per
 *     plan.  L2[k] per plan (may be NULL); the global gradients stay on
 *     each plan (psv_get_gradient); *ms (may be NULL) the device time of
 *     the two joint passes.  Gradients agree with each plan's own
 *     psv_gradient with the same tile shape to rounding.
 *     PSV_ERR_UNSUPPORTED for the exact adjoint.
 *   psv_joint_launches: kernel launches of the last psv_joint_forward or
 *     psv_joint_gradient (two per joint step; 0 before the first call).
 * Errors: PSV_ERR_ARG (more than 8 plans, mixed precisions, a plan twice,
 * no model or no observed traces).  No counterpart in the reference (one
 * survey per program run). */
typedef struct psv_joint psv_joint;
int psv_joint_create(psv_plan *const *plans, int nplans, int rows_per_thread, int block_y,
                     psv_joint **out);
int psv_joint_forward(psv_joint *joint, double *const *rtf_uz, double *const *rtf_ux, double *ms);
int psv_joint_gradient(psv_joint *joint, double *L2, double *ms);
long long psv_joint_launches(const psv_joint *joint);
int psv_joint_shape(const psv_joint *joint, int *rows_per_thread, int *block_y);
int psv_joint_destroy(psv_joint *joint);

int psv_reset_gradient(psv_plan *plan);
int psv_get_gradient(psv_plan *plan, double *grad_lam, double *grad_mu, double *grad_rho);
int psv_set_gradient(psv_plan *plan, const double *grad_lam, const double *grad_mu,
                     const double *grad_rho);

/* Per-shot outputs of the last psv_gradient for shot ishot: snapped shot
 * gradients [snap_nz][snap_nx] (kernel_PSV's grad_*), forward / adjoint
 * energies We, We_adj [nz][nx] (before energy_weights2), modelled traces
 * [nrec][nt] and the shot's L2.  Any pointer may be NULL. */
int psv_get_shot_gradient(psv_plan *plan, int ishot, double *grad_lam_shot,
                          double *grad_mu_shot, double *grad_rho_shot, double *We,
                          double *We_adj, double *rtf_uz, double *rtf_ux, double *L2);

/* One FWI iteration (src/cpu/n_simulate_PSV.cpp:249-576): copy_mat, the
 * gradient above, taper2, step_length_PSV with trial forwards of every
 * shot, and update_mat2 of lam, mu, rho.  *step is the step-length estimate
 * carried between iterations (in: estimate, out: accepted step).  Outputs:
 * the iteration's L2, the number of trial forward passes and their (alpha,
 * L2) pairs in trial_log[2*k] (room for max_trials entries; may be NULL).
 * On PSV_ERR_STEP_SEARCH (where the reference exits, or loops for ever on a
 * NaN misfit) the plan's model is the last trial's; psv_plan_set_model
 * replaces it. */
int psv_fwi_iteration(psv_plan *plan, double *step, double *L2, int *ntrials,
                      double *trial_log, int max_trials);

/* adjsrc2 (include/cpu/n_kernel_lib_PSV.hpp:139) for nshot shots at once on
 * the GPU: residuals res = mod - true and L2[s] = sum over the shot's traces
 * of dt/2 (r_z^2 + r_x^2).  Host arrays [nshot][nrec][nt]; res_* may alias
 * mod_* (the reference overwrites its model traces, n_simulate_PSV.cpp:320)
 * or be NULL.  The sum runs in a fixed order (deterministic). */
int psv_misfit(const double *mod_z, const double *mod_x, const double *true_z,
               const double *true_x, double *res_z, double *res_x, int nshot, int nrec, int nt,
               double dt, double *L2);

/* psv_misfit for callers that cannot allocate device memory.  No counterpart
 * in the reference.  Some callers may not call cudaMalloc: code whose GPU
 * memory is owned by a framework allocator or a fixed pool (an allocation of
 * its own would bypass the owner's accounting and could fail once the pool
 * holds the device's memory), or a latency-bound loop that must not pay for
 * cudaMalloc/cudaFree or fragment the heap.  They pass DEVICE
 * pointers for every input and output (traces [nshot][nrec][nt], residuals
 * optional as a pair, d_L2[nshot]); the only scratch, the reduction's partial
 * sums, lives in a fixed device array inside the library (2 MiB, held by each
 * GPU that loads the library until exit), so nshot is limited to
 * PSV_MISFIT_NOALLOC_MAX_SHOTS (larger values return PSV_ERR_ARG).  Work is
 * enqueued on `stream` (a cudaStream_t, NULL = default stream) and not
 * synchronised.  The first call on a device looks up the array's device
 * address (once per device, with that device current): make that first call
 * before any stream capture.  All calls share the array, so calls that
 * overlap on the GPU (different streams, or several devices' threads
 * enqueueing concurrently on one device) race; order them on one stream.
 * Results equal psv_misfit's. */
#define PSV_MISFIT_NOALLOC_MAX_SHOTS 1024
int psv_misfit_noalloc(const double *d_mod_z, const double *d_mod_x, const double *d_true_z,
                       const double *d_true_x, double *d_res_z, double *d_res_x, int nshot,
                       int nrec, int nt, double dt, double *d_L2, void *stream);

/* Trial evaluation used by the step-length search: L2 misfit of the model
 * updated with step length `step`.  Returns a psv_status. */
typedef int (*psv_trial_fn)(double step, double *L2, void *ctx);

/* Control flow of step_length_PSV (src/cpu/n_step_length_PSV.cpp:53-209):
 * halve the estimate until a trial lowers L2 below L2_0, then grow it by
 * 1.5 until a trial misfit rises again (at most 4 growths), then take the
 * parabola vertex (psv_calc_opt_step).  *est is the starting estimate in and
 * the accepted step out.  Trials are logged as (step, L2) pairs in tlog.
 * Returns PSV_ERR_STEP_SEARCH after 31 halvings without a decrease, and
 * when L2_0 or a trial's L2 is NaN (a NaN gradient; the reference's loop
 * never ends there). */
int psv_step_length(double *est, double L2_0, psv_trial_fn trial, void *ctx, int *ntrials,
                    double *tlog, int max_trials);

/* calc_opt_step (include/cpu/n_step_length_PSV.hpp:58): vertex of the
 * parabola through (sl[i], L2[i]) with the reference's clamps, solved with a
 * correct 3x3 elimination (the reference's solvelin back-substitution reads
 * past its arrays, include/cpu/n_solvelin.hpp:37-42). */
double psv_calc_opt_step(const double *L2, const double *sl);

/* Optional preconditioners (dead code in the reference, available here):
 *   psv_gauss_filter_kernel: gauss_filter_kernel (src/cpu/n_kernel_lib_PSV.cpp:1012):
 *     filter[(2 hfs + 1)^2], row = z offset + hfs, column = x offset + hfs,
 *     sigma = hfs / 2 in integer arithmetic as the reference computes it;
 *     hfs < 2 is PSV_ERR_ARG (the reference's weights are NaN there).  Host only.
 *   psv_apply_gauss_filter: apply_gauss_filter (:1053) on a host [nz][nx] array,
 *     in place, on the device; the filtered sums are FP64 (the reference
 *     accumulates into an int, truncating every partial sum).
 *   psv_PCG_PSV: PCG_PSV (src/cpu/n_PCG_PSV.cpp:13), Fletcher-Reeves, on host
 *     [nz][nx] arrays updated in place, on the device; beta = 0 when |old|^2 = 0
 *     (the reference divides by zero on its first call). */
int psv_gauss_filter_kernel(int hfs, double *filter);
int psv_apply_gauss_filter(double *mat, int nz, int nx, int hfs);
int psv_PCG_PSV(double *dir, double *old, double *grad, int nz, int nx);

/* The pieces of psv_fwi_iteration, for drivers that split the shots of a
 * survey over several plans / GPUs and reduce between them:
 *   psv_save_model      copy_mat: the model trials and the update start from
 *                       (src/cpu/n_simulate_PSV.cpp:263);
 *   psv_taper_gradient  taper2 of the three global gradients (:443-450);
 *   psv_trial_misfit    one trial of step_length_PSV: update_mat2 of the saved
 *                       model by `step` (rho by step/2, floor 1.5), forward of
 *                       this plan's shots, their summed L2
 *                       (src/cpu/n_step_length_PSV.cpp:87-123);
 *   psv_update_model    the final update_mat2 x3 (:542-546).
 * A distributed iteration: save, gradient, all-reduce the gradients and L2,
 * psv_set_gradient, taper, psv_step_length with trials whose L2 is
 * all-reduced, update. */
int psv_save_model(psv_plan *plan);
int psv_taper_gradient(psv_plan *plan);
/* PCG_PSV on the plan's three global gradients with the plan's direction
 * state (zero before the first call), as psv_PCG_PSV. */
int psv_pcg_gradient(psv_plan *plan);
int psv_trial_misfit(psv_plan *plan, double step, double *L2);
int psv_update_model(psv_plan *plan, double step);

/* Event-timed device milliseconds of the last forward / gradient /
 * iteration call, split: [0] forward, [1] adjoint (incl. recompute), [2]
 * everything else. */
int psv_last_timing(const psv_plan *plan, double *ms3);

/* Time-step kernel autotuner: times every candidate (kernel family, rows
 * per thread, block height) over nsteps forward + nsteps adjoint steps
 * (CUDA events) and keeps the fastest.  Results are cached per (grid,
 * stencil order, batch, precision, requested family) for the process.
 * Needs a model and observed traces (it runs the kernels on them); leaves
 * the wavefields undefined.  Outputs the chosen shape (any pointer may be
 * NULL). */
int psv_plan_autotune(psv_plan *plan, int nsteps, int *kernel_family, int *rows_per_thread,
                      int *block_y);
/* The time-step kernels the plan launches now: family (PSV_KERNELS_*), rows
 * per thread (FUSED: tile rows, MARCH: rows a CTA marches) and block height
 * (TMA: 4, FUSED: 0, MARCH: warps per CTA); any pointer may be NULL. */
int psv_plan_shape(const psv_plan *plan, int *kernel_family, int *rows_per_thread, int *block_y);
/* Shot groups (streams) the plan's time loops run in: 1, 2 or 4. */
int psv_plan_chains(const psv_plan *plan, int *chains);
/* The plan's snapshot storage: PSV_STORE_FULL, _CHECKPOINT or _BINOMIAL
 * (never AUTO), steps per segment and state slots per shot (0 for FULL),
 * and the segment advances the adjoint pass recomputes beyond the one
 * recomputation of each segment (0 unless BINOMIAL).  Any pointer may be
 * NULL.  Replaces the accu_* allocation in the reference's
 * simulate_fwi_PSV (src/cpu/n_simulate_PSV.cpp). */
int psv_plan_storage(const psv_plan *plan, int *storage, int *segment_steps, int *slots,
                     long long *advances);
/* Griewank's binomial checkpoint schedule for nseg segments and `slots`
 * state slots (host only, no device): writes up to `cap` actions as
 * (op, segment, slot) triples into `actions` -- first the forward pass's
 * saves (op 1), then the adjoint pass (2 restore, 3 advance, 4 save the
 * working state, 5 recompute + reverse a segment) -- and their count into
 * *nactions, and the advances into *advances.  PSV_ERR_ARG if cap is too
 * small (the counts are still written), and for a schedule of more than
 * 2^26 advances (every advance is an action; plan creation refuses those
 * with PSV_ERR_UNSUPPORTED). */
int psv_checkpoint_schedule(int nseg, int slots, int *actions, int cap, int *nactions,
                            long long *advances);

/* The CUDA stream every call of this plan runs on (a cudaStream_t), for
 * callers that time or order work against it. */
void *psv_plan_stream(const psv_plan *plan);
/* Number of kernels this plan has launched so far (graph replays count
 * their kernel nodes). */
long long psv_plan_kernel_launches(const psv_plan *plan);
/* Event-timed profile of the time-step kernels: nsteps forward steps then
 * nsteps adjoint steps of the first batch, each kernel bracketed by CUDA
 * events on the plan's stream.  ms6 = mean milliseconds per launch of
 * {stress, velocity, 0} forward, then the same adjoint (sources and
 * receivers run inside the velocity kernel; slots 2 and 5 stay 0).
 * Needs a model and observed traces; leaves the wavefields undefined. */
int psv_profile_kernels(psv_plan *plan, int nsteps, double *ms6);

/* ------------------------------------------------------------------------ */
/* Reference-shaped drop-ins                                                  */
/* ------------------------------------------------------------------------ */

/* kernel_PSV / kernel_PSV_GPU (include/cpu/n_kernel_PSV.hpp:8-43,
 * include/cuda/d_kernel_PSV.cuh:9-44): the same arguments in the same
 * order, with flat host arrays.  One shot, nt steps, forward (grad = 0) or
 * time-reversed adjoint (grad = 1).  On return the host arrays hold what the
 * reference leaves in them: final wavefields, energies, the CPML memories
 * (when non-NULL), receiver traces (forward), the snapshot history (accu),
 * the snapped shot gradients (grad).  dz_z..dx_x are the reference's
 * internal derivative scratch arrays: accepted and ignored (may be NULL).
 * stencil selects PSV_STENCIL_*; precision 32 or 64. */
int psv_kernel_PSV(int ishot, int nt, int nz, int nx, double dt, double dx, double dz,
                   int surf, const int *isurf, const double *hc, int fdorder,
                   double *vz, double *vx, double *uz, double *ux,
                   double *szz, double *szx, double *sxx, double *We,
                   double *dz_z, double *dx_z, double *dz_x, double *dx_x,
                   const double *lam, const double *mu, const double *mu_zx,
                   const double *rho_zp, const double *rho_xp,
                   int grad, double *grad_lam, double *grad_mu, double *grad_rho,
                   int pml_z, const double *a_z, const double *b_z, const double *K_z,
                   const double *a_half_z, const double *b_half_z, const double *K_half_z,
                   int pml_x, const double *a_x, const double *b_x, const double *K_x,
                   const double *a_half_x, const double *b_half_x, const double *K_half_x,
                   double *mem_vz_z, double *mem_vx_z, double *mem_szz_z, double *mem_szx_z,
                   double *mem_vz_x, double *mem_vx_x, double *mem_szx_x, double *mem_sxx_x,
                   int nsrc, int stf_type, const double *stf_z, const double *stf_x,
                   const int *z_src, const int *x_src, const int *src_shot_to_fire,
                   int nrec, int rtf_type, double *rtf_uz, double *rtf_ux,
                   const int *z_rec, const int *x_rec,
                   int accu, double *accu_vz, double *accu_vx,
                   double *accu_szz, double *accu_szx, double *accu_sxx,
                   int snap_z1, int snap_z2, int snap_x1, int snap_x2,
                   int snap_dt, int snap_dz, int snap_dx, int stencil, int precision);

/* simulate_PSV (include/h_simulate_PSV.hpp:23) run on the GPU: reads
 * workdir/bin/metaint.bin, intarray.bin, metafloat.bin, mat.bin (and
 * workdir/io/shot{i}_rtf_u{z,x}.bin for FWI), builds the CPML profiles,
 * Holberg coefficients and Ricker wavelets as the reference does
 * (src/h_simulate_PSV.cpp:99-185), then runs forward modelling (writing
 * bin/shot{i}_rtf_u{z,x}.bin and, with accu_save, bin/shot{i}_{vz,vx,szz,szx,sxx}.bin)
 * or FWI (writing bin/iter{n}_mat.bin every mat_save_interval iterations).
 * max_iter caps the FWI iterations (the reference's cap is 1000 with an
 * early stop after 25, src/cpu/n_simulate_PSV.cpp:240,576-581; 0 = that).
 * imaging_sign has the meaning of the grid field of that name (the files
 * carry no such field; <= 0 is the reference's CPU path). */
int psv_simulate_PSV(const char *workdir, int max_iter, int imaging_sign, const psv_options *opt);

#ifdef __cplusplus
}
#endif
#endif
