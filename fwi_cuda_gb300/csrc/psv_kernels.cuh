// psv_kernels.cuh -- sm_103a kernels of the P/SV velocity-stress time loop.
//
// One time step of the reference loop (src/cpu/n_kernel_PSV.cpp:90-210) is
// two launches here instead of eight full-grid passes:
//   k_stress    vdiff2 + pml_diff2 + update_s2 + surf_mirror   (:107-128)
//   k_velocity  sdiff2 + pml_diff2 + update_v2, fused with the snapshot
//               store gard_fwd_storage2 (forward) or the imaging condition
//               fwi_grad2 (adjoint)                             (:138-150,191-206),
//               and vsrc2 + urec2 for the sources and receivers of each
//               block's tile                                    (:164-175)
// Derivatives never leave registers, CPML memories exist only on the
// absorbing strips, and every shot of a batch is one blockIdx.z slice.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace psv {

// Planes of one shot's wavefield block [NFIELD][nz][pitch].
enum { F_VZ = 0, F_VX, F_SZZ, F_SZX, F_SXX, F_UZ, F_UX, F_WE, F_WEA, NFIELD };
// FP32 plans also hold a second copy of vz vx szz szx sxx at planes
// NFIELD .. NFIELD + 4 for the fused time step, which reads one copy and
// writes the other (ping-pong by step parity).
constexpr int NFIELD_PP = NFIELD + 5;
// z-strip CPML memories (rows outside [pz0, pz1)): mem_vz_z, mem_vx_z, mem_szz_z, mem_szx_z.
enum { MZ_VZ = 0, MZ_VX, MZ_SZZ, MZ_SZX, NMZ };
// x-strip CPML memories (columns outside [px0, px1)): mem_vz_x, mem_vx_x, mem_szx_x, mem_sxx_x.
enum { MX_VZ = 0, MX_VX, MX_SZX, MX_SXX, NMX };
// FP32 plans: second copies of the memories the stress update reads at
// halo points (mem_vz_z, mem_vx_z at planes NMZ, NMZ + 1; mem_vz_x, mem_vx_x
// at NMX, NMX + 1), ping-ponged by the fused time step.
constexpr int NMZ_PP = NMZ + 2, NMX_PP = NMX + 2;
// Snapshot planes of one stored step: accu_szz, accu_szx, accu_sxx, accu_vz, accu_vx.
enum { H_SZZ = 0, H_SZX, H_SXX, H_VZ, H_VX, NHIST };
// Velocity-kernel modes: forward with the energy We; forward without it
// (trial and modelling runs); forward that also integrates the displacement
// u (the reference always does, the engine only needs it in the drop-in);
// time-reversed adjoint (u, We_adj and the imaging condition).
enum { MODE_FWD = 0, MODE_FWD_NOWE = 1, MODE_FWD_U = 2, MODE_ADJ = 3 };

template <typename T>
struct StepParams {
    int nz, nx, pitch;
    int nz1, nz2, nx1, nx2;  // interior [fpad, n - fpad)
    long long plane;         // nz * pitch
    long long shot_stride;   // NFIELD * plane
    T *fld;                  // [batch][NFIELD][nz][pitch]
    T cz[4], cx[4];          // hc[k] / dz, hc[k] / dx
    T dt, inv_dt;
    T kimg;                  // snap_dt * dt (fwi_grad2 weight)
    int pml_z, pml_x;
    int pz0, pz1, px0, px1;  // identity (non-CPML) row / column ranges
    int mx_pitch;            // row pitch of the x-strip memories
    long long mz_plane, mz_shot_stride, mx_plane, mx_shot_stride;
    T *memz, *memx;
    const T *a_z, *b_z, *ki_z, *ah_z, *bh_z, *khi_z;  // [nz], ki = 1/K
    const T *a_x, *b_x, *ki_x, *ah_x, *bh_x, *khi_x;  // [nx]
    // dt-scaled coefficients, [nz][pitch]: dt*lam, dt*(lam+2mu), dt*mu_zx,
    // dt*rho_zp, dt*rho_xp, and the imaging factors g1 = snap_dt*dt/4/(lam+mu)^2,
    // g2 = snap_dt*dt/mu^2.
    const T *c_lam, *c_l2m, *c_muzx, *c_rz, *c_rx, *g1, *g2;
    // Free surfaces (0 = none) and their sxx / szz factors 4dt(lam mu + mu^2)/(lam + 2mu).
    int st, sb, sl, sr;
    const T *fs_top, *fs_bot;    // [nx]
    const T *fs_left, *fs_right; // [nz]
    // Snapshot window, storage [batch][slot][NHIST][snz][snx_pitch] and shot gradients.
    int snap_z1, snap_z2, snap_x1, snap_x2, snap_dz, snap_dx;
    int snz, snx, snx_pitch;
    long long snap_plane, hist_slot_stride, hist_shot_stride;
    T *hist;
    T *gshot;                  // [batch][3][snz][snx_pitch] (grad_lam, grad_mu, grad_rho)
    long long gshot_shot_stride;
    const int *ctl;            // device [2]: global index of batch shot 0, shots in this batch
    int *err;                  // device error word (nonzero: a bounded wait gave up)
    int nbatch;                // shots per launch (grid extent in shots)
    int pp_planes;             // planes from the first to the second vz..sxx copy (0: none)
};

// Block coordinates of the grid-stepping kernels: blockIdx.z = shot of the
// batch, so x-adjacent tiles of one shot run together and share their halo
// rows and columns through L1/L2.  (Making the shot the fastest index, so
// the shots of one tile share the coefficients instead, measured 10-15 %
// slower on L2-resident grids and no faster on HBM-bound ones for these
// kernels; the persistent TMA kernels do order their tiles that way.)
struct BlockPos {
    int bz, bx, by, ntx;  // shot of the batch, tile column, tile row, tile columns
};
__device__ __forceinline__ BlockPos block_pos(int)
{
    return {(int)blockIdx.z, (int)blockIdx.x, (int)blockIdx.y, (int)gridDim.x};
}

// Source injection and receiver recording of one step for every shot of a batch.
template <typename T>
struct SrcRecParams {
    const int *src_off;         // [nshot + 1] CSR offsets (global shot index)
    const int *src_pos;         // [nsrc_total] iz * pitch + ix
    const int *src_col;         // [nsrc_total] column in the time-function array
    const int *src_snap;        // [nsrc_total] snapshot cell jz*snx_pitch+jx or -1
    const double *stf_z, *stf_x;  // [*][nt][ncol], row it
    long long stf_shot_stride;    // 0 when all shots share the array
    int stf_ncol;
    int stf_type;                 // 0: v += dt rho^-1 s/(dz dx); 1: v += s
    double inv_dzdx;
    int nrec;
    const int *rec_pos;           // [nrec]
    double *rtf_z, *rtf_x;        // [nshot][nt][nrec] or null (adjoint)
    long long rtf_shot_stride;
    double dt_d, dzdx;
    int nt;
    // Power-of-two range scaling (exact in floating point): injected
    // amplitudes are multiplied by amp_scale[shot]; recorded displacements by
    // rec_unscale[shot] = 1 / amp_scale[shot].  Keeps FP32 wavefields of
    // physical-unit surveys away from the denormal range.
    const double *amp_scale, *rec_unscale;  // [nshot]
    // Sources and receivers by tile of the velocity kernel (32 columns x tz
    // rows), so the block that owns a cell injects / records it:
    //   src_kind 0: the shot's sources, t_src_off[shot][ntiles + 1] into
    //               t_src_k (entries index src_pos / src_col / src_snap);
    //   src_kind 1: every receiver fires its column of the stf array;
    //   src_kind -1: nothing is injected.
    int src_kind, ntiles;
    const int *t_src_off, *t_src_k;
    const int *t_rec_off, *t_rec_r;  // [ntiles + 1] into receiver indices
};

// Rows per thread of the stencil kernels: 1, 2 or 4 (FP32); negative values
// select the warp-shuffle variant with |r| rows.  FP64 always uses 1.
template <typename T> inline int rpt_ok(int r)
{
    if (sizeof(T) == 8) return 1;
    return (r == 1 || r == 2 || r == 4 || r == -2 || r == -4) ? r : 1;
}

}  // namespace psv
