// psv_exact.cu -- exact discrete adjoint of the FP64 time loop (the
// `adjoint = PSV_ADJOINT_EXACT` plan option): dL2/dlam, dL2/dmu, dL2/drho of
// the misfit the engine computes, L2 = 1/2 dt sum (u_mod - u_obs)^2
// (adjsrc2, src/cpu/n_kernel_lib_PSV.cpp:579-626), to rounding.
//
// The reference's gradient (fwi_grad2, :439-484) runs the forward operator
// backwards in time and images with point estimates; its CPML, free surface,
// staggered material averages and leapfrog staggering make it differ from
// the derivative of the discrete misfit.  Here every operation of one
// forward step (n_kernel_PSV.cpp:90-210) is transposed by hand, in reverse
// order:
//   forward step n                        adjoint step n (reverse time)
//   d  = D v^n          (vdiff2)          v-bar   += D^T d-bar
//   d' = CPML(d), psi   (pml_diff2)       d-bar    = CPML^T(d'-bar), psi-bar
//   sigma^{n+1} = sigma^n + M(m) d'       d'-bar   = M^T sigma-bar,
//     surface row, mirror (surf_mirror)     grad M += sigma-bar d', surface/mirror
//   e  = E sigma^{n+1}  (sdiff2)          sigma-bar += E^T e-bar
//   e' = CPML(e), phi   (pml_diff2)       e-bar    = CPML^T(e'-bar), phi-bar
//   v^{n+1} = v^n + B(m) e' (update_v2)   e'-bar   = B^T v-bar, grad B += v-bar e'
//   v^{n+1}[src] += B s(n)  (vsrc2)       grad B[src] += v-bar s(n)
//   R(n) = R(n-1) + dt v^{n+1}[rec]/dzdx  v-bar[rec] += dt/dzdx sum_{n'>=n} dL/dR(n')
//     (urec2)
// The forward pass stores d' and e' of every step (8 planes per step and
// shot), the adjoint pass carries v-bar, sigma-bar and the adjoint CPML
// memories and accumulates the derivatives of L2 with respect to the
// dt-scaled coefficients dt lam, dt (lam + 2 mu), dt mu_zx, dt / rho_z,
// dt / rho_x and the surface factor; a last kernel applies the chain rule
// through mat_av2's harmonic and arithmetic averages (:853-922) and the
// surface factor 4 dt (lam mu + mu^2) / (lam + 2 mu).
//
// Free surface: none or a top one (mirrored rows included); the plan
// refuses the others in this mode.  Sources and receivers: force sources
// (stf_type 0 scales by dt / rho, type 1 injects the time function), every
// receiver records displacement (rtf_type 0).  No range scaling: FP64.
#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"

namespace psv {
namespace {

using P64 = StepParams<double>;
using Q64 = SrcRecParams<double>;

__device__ __forceinline__ bool grid_point(const P64 &p, int &iz, int &ix, int &bz)
{
    ix = blockIdx.x * blockDim.x + threadIdx.x;
    iz = blockIdx.y * blockDim.y + threadIdx.y;
    bz = blockIdx.z;
    return ix < p.nx && iz < p.nz && bz < p.ctl[1];
}
__device__ __forceinline__ bool interior(const P64 &p, int iz, int ix)
{
    return iz >= p.nz1 && iz < p.nz2 && ix >= p.nx1 && ix < p.nx2;
}
// value of plane a at (iz, ix), zero outside the grid
__device__ __forceinline__ double at0(const P64 &p, const double *a, int iz, int ix)
{
    return (iz >= 0 && iz < p.nz && ix >= 0 && ix < p.nx) ? a[(long long)iz * p.pitch + ix] : 0.0;
}

// ---------------------------------------------------------------- forward
// Stress update of stress_point (psv_kernels_impl.cuh) that also stores the
// CPML-corrected velocity derivatives d' (vz_z, vx_z, vz_x, vx_x).
template <int NS>
__global__ void k_exact_stress(const P64 p, ExactBufs X, const int n)
{
    int iz, ix, bz;
    if (!grid_point(p, iz, ix, bz) || !interior(p, iz, ix)) return;
    double *f = p.fld + (long long)bz * p.shot_stride;
    const double *vz = f + F_VZ * p.plane, *vx = f + F_VX * p.plane;
    const double oz = at0(p, vz, iz, ix), ox = at0(p, vx, iz, ix);
    double vz_z = p.cz[0] * (oz - at0(p, vz, iz - 1, ix));
    double vx_z = p.cz[0] * (at0(p, vx, iz + 1, ix) - ox);
    double vz_x = p.cx[0] * (at0(p, vz, iz, ix + 1) - oz);
    double vx_x = p.cx[0] * (ox - at0(p, vx, iz, ix - 1));
#pragma unroll
    for (int k = 2; k <= NS; k++) {
        vz_z += p.cz[k - 1] * (at0(p, vz, iz + k - 1, ix) - at0(p, vz, iz - k, ix));
        vx_z += p.cz[k - 1] * (at0(p, vx, iz + k, ix) - at0(p, vx, iz - k + 1, ix));
        vz_x += p.cx[k - 1] * (at0(p, vz, iz, ix + k) - at0(p, vz, iz, ix - (k - 1)));
        vx_x += p.cx[k - 1] * (at0(p, vx, iz, ix + k - 1) - at0(p, vx, iz, ix - k));
    }
    const long long i = (long long)iz * p.pitch + ix;
    cpml_stress(p, bz, iz, ix, vz_z, vx_z, vz_x, vx_x);
    double *S = X.store + (long long)n * X.step_stride + (long long)bz * 8 * p.plane + i;
    S[0] = vz_z; S[p.plane] = vx_z; S[2 * p.plane] = vz_x; S[3 * p.plane] = vx_x;
    double *szz = f + F_SZZ * p.plane, *szx = f + F_SZX * p.plane, *sxx = f + F_SXX * p.plane;
    stress_finish(p, szz, szx, sxx, iz, ix, i, szz[i], szx[i], sxx[i], p.c_lam[i], p.c_l2m[i],
                  p.c_muzx[i], vz_z, vx_z, vz_x, vx_x);
}

// Velocity update of velocity_point that also stores the CPML-corrected
// stress derivatives e' (szz_z, szx_z, szx_x, sxx_x).
template <int NS>
__global__ void k_exact_velocity(const P64 p, ExactBufs X, const int n)
{
    int iz, ix, bz;
    if (!grid_point(p, iz, ix, bz) || !interior(p, iz, ix)) return;
    double *f = p.fld + (long long)bz * p.shot_stride;
    const double *szz = f + F_SZZ * p.plane, *szx = f + F_SZX * p.plane, *sxx = f + F_SXX * p.plane;
    const double ozz = at0(p, szz, iz, ix), ozx = at0(p, szx, iz, ix), oxx = at0(p, sxx, iz, ix);
    double szz_z = p.cz[0] * (at0(p, szz, iz + 1, ix) - ozz);
    double szx_z = p.cz[0] * (ozx - at0(p, szx, iz - 1, ix));
    double szx_x = p.cx[0] * (ozx - at0(p, szx, iz, ix - 1));
    double sxx_x = p.cx[0] * (at0(p, sxx, iz, ix + 1) - oxx);
#pragma unroll
    for (int k = 2; k <= NS; k++) {
        szz_z += p.cz[k - 1] * (at0(p, szz, iz + k, ix) - at0(p, szz, iz - k + 1, ix));
        szx_z += p.cz[k - 1] * (at0(p, szx, iz + k - 1, ix) - at0(p, szx, iz - k, ix));
        szx_x += p.cx[k - 1] * (at0(p, szx, iz, ix + k - 1) - at0(p, szx, iz, ix - k));
        sxx_x += p.cx[k - 1] * (at0(p, sxx, iz, ix + k) - at0(p, sxx, iz, ix - (k - 1)));
    }
    cpml_velocity(p, bz, iz, ix, szz_z, szx_z, szx_x, sxx_x);
    const long long i = (long long)iz * p.pitch + ix;
    double *S = X.store + (long long)n * X.step_stride + (long long)bz * 8 * p.plane + i;
    S[4 * p.plane] = szz_z; S[5 * p.plane] = szx_z; S[6 * p.plane] = szx_x; S[7 * p.plane] = sxx_x;
    double vzn, vxn, uzn, uxn;
    velocity_finish<double, MODE_FWD_NOWE>(p, f, i, f[F_VZ * p.plane + i], f[F_VX * p.plane + i],
                                           0.0, 0.0, 0.0, p.c_rz[i], p.c_rx[i], szz_z, szx_z,
                                           szx_x, sxx_x, vzn, vxn, uzn, uxn);
}

// vsrc2: the step's sources of every shot of the batch (no range scaling).
__global__ void k_exact_inject(const P64 p, const Q64 q, const int n)
{
    const int bz = blockIdx.y;
    if (bz >= p.ctl[1]) return;
    const int shot = p.ctl[0] + bz;
    const int k = q.src_off[shot] + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= q.src_off[shot + 1]) return;
    double *f = p.fld + (long long)bz * p.shot_stride;
    const int pos = q.src_pos[k], col = q.src_col[k];
    const double sz = q.stf_z[(long long)n * q.stf_ncol + col];
    const double sx = q.stf_x[(long long)n * q.stf_ncol + col];
    const double az = q.stf_type == 0 ? p.c_rz[pos] * (sz * q.inv_dzdx) : sz;
    const double ax = q.stf_type == 0 ? p.c_rx[pos] * (sx * q.inv_dzdx) : sx;
    atomicAdd(&f[F_VZ * p.plane + pos], az);
    atomicAdd(&f[F_VX * p.plane + pos], ax);
}

// urec2: running-sum displacement at the receivers.
__global__ void k_exact_record(const P64 p, const Q64 q, const int n)
{
    const int bz = blockIdx.y, r = blockIdx.x * blockDim.x + threadIdx.x;
    if (bz >= p.ctl[1] || r >= q.nrec) return;
    const int shot = p.ctl[0] + bz;
    const double *f = p.fld + (long long)bz * p.shot_stride;
    const int pos = q.rec_pos[r];
    double *rz = q.rtf_z + shot * q.rtf_shot_stride, *rx = q.rtf_x + shot * q.rtf_shot_stride;
    const long long row = (long long)n * q.nrec;
    const double pz = n ? rz[row - q.nrec + r] : 0.0, px = n ? rx[row - q.nrec + r] : 0.0;
    rz[row + r] = pz + (q.dt_d * f[F_VZ * p.plane + pos]) / q.dzdx;
    rx[row + r] = px + (q.dt_d * f[F_VX * p.plane + pos]) / q.dzdx;
}

// --------------------------------------------------------------- adjoint
// dL2/dR(n) = dt res(n) and R(n) enters every later R: the adjoint of the
// running sum is the reverse cumulative sum; scaled by dt / dzdx it is what
// the receivers add to v-bar at step n.  In place on the residual traces.
__global__ void k_exact_revsum(double *res_z, double *res_x, int nt, int nrec, long long stride,
                               double dt, double gain, int nbatch)
{
    const int b = blockIdx.y, r = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbatch || r >= nrec) return;
    double *az = res_z + b * stride, *ax = res_x + b * stride;
    double sz = 0.0, sx = 0.0;
    for (int n = nt - 1; n >= 0; n--) {
        const long long k = (long long)n * nrec + r;
        sz += dt * az[k];
        sx += dt * ax[k];
        az[k] = gain * sz;
        ax[k] = gain * sx;
    }
}

__device__ __forceinline__ double *wplane(const ExactBufs &X, const P64 &p, int bz, int k)
{
    return X.work + ((long long)bz * EXACT_WORK_PLANES + k) * p.plane;
}

// Receivers: v-bar[rec] += dt / dzdx * sum_{n' >= n} dt res(n').
__global__ void k_exact_adj_record(const P64 p, const Q64 q, ExactBufs X, const int n)
{
    const int bz = blockIdx.y, r = blockIdx.x * blockDim.x + threadIdx.x;
    if (bz >= p.ctl[1] || r >= q.nrec) return;
    const int shot = p.ctl[0] + bz;
    const int pos = q.rec_pos[r];
    const long long k = shot * q.rtf_shot_stride + (long long)n * q.nrec + r;
    atomicAdd(wplane(X, p, bz, EX_VBZ) + pos, X.rsum_z[k]);
    atomicAdd(wplane(X, p, bz, EX_VBX) + pos, X.rsum_x[k]);
}

// Sources: d L2 / d(dt / rho) at the source cells (stf_type 0).
__global__ void k_exact_adj_source(const P64 p, const Q64 q, ExactBufs X, const int n)
{
    const int bz = blockIdx.y;
    if (bz >= p.ctl[1] || q.stf_type != 0) return;
    const int shot = p.ctl[0] + bz;
    const int k = q.src_off[shot] + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= q.src_off[shot + 1]) return;
    const int pos = q.src_pos[k], col = q.src_col[k];
    const double sz = q.stf_z[(long long)n * q.stf_ncol + col] * q.inv_dzdx;
    const double sx = q.stf_x[(long long)n * q.stf_ncol + col] * q.inv_dzdx;
    atomicAdd(wplane(X, p, bz, EX_GRZ) + pos, wplane(X, p, bz, EX_VBZ)[pos] * sz);
    atomicAdd(wplane(X, p, bz, EX_GRX) + pos, wplane(X, p, bz, EX_VBX)[pos] * sx);
}

// Transpose of one CPML recursion: forward psi' = b psi + a d, d' = d / K + psi';
// adjoint with the carried memory Q (= b times the later total adjoint of psi'):
// T = Q + d'-bar, d-bar = d'-bar / K + a T, Q <- b T.
__device__ __forceinline__ double cpml_adj(double *Q, double dpb, double a, double b, double ki)
{
    const double T = *Q + dpb;
    *Q = b * T;
    return ki * dpb + a * T;
}

// Transpose of update_v2 + pml_diff2 of the velocity side at every point:
// e-bar from v-bar, gradients of dt / rho_z and dt / rho_x.
__global__ void k_exact_adj_velocity(const P64 p, ExactBufs X, const int n)
{
    int iz, ix, bz;
    if (!grid_point(p, iz, ix, bz)) return;
    const long long i = (long long)iz * p.pitch + ix;
    double *eb = wplane(X, p, bz, EX_EB);
    double e1 = 0.0, e2 = 0.0, e3 = 0.0, e4 = 0.0;
    if (interior(p, iz, ix)) {
        const double vbz = wplane(X, p, bz, EX_VBZ)[i], vbx = wplane(X, p, bz, EX_VBX)[i];
        const double *S = X.store + (long long)n * X.step_stride + (long long)bz * 8 * p.plane + i;
        const double szz_z = S[4 * p.plane], szx_z = S[5 * p.plane];
        const double szx_x = S[6 * p.plane], sxx_x = S[7 * p.plane];
        wplane(X, p, bz, EX_GRZ)[i] += vbz * (szx_x + szz_z);
        wplane(X, p, bz, EX_GRX)[i] += vbx * (sxx_x + szx_z);
        e1 = e3 = p.c_rz[i] * vbz;
        e2 = e4 = p.c_rx[i] * vbx;
        if (iz < p.pz0 || iz >= p.pz1) {
            const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
            double *m = X.qz + (long long)bz * p.mz_shot_stride + (long long)rr * p.pitch + ix;
            e1 = cpml_adj(m + MZ_SZZ * p.mz_plane, e1, p.a_z[iz], p.b_z[iz], p.ki_z[iz]);
            e2 = cpml_adj(m + MZ_SZX * p.mz_plane, e2, p.ah_z[iz], p.bh_z[iz], p.khi_z[iz]);
        }
        if (ix < p.px0 || ix >= p.px1) {
            const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
            double *m = X.qx + (long long)bz * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
            e4 = cpml_adj(m + MX_SXX * p.mx_plane, e4, p.a_x[ix], p.b_x[ix], p.ki_x[ix]);
            e3 = cpml_adj(m + MX_SZX * p.mx_plane, e3, p.ah_x[ix], p.bh_x[ix], p.khi_x[ix]);
        }
    }
    eb[i] = e1; eb[p.plane + i] = e2; eb[2 * p.plane + i] = e3; eb[3 * p.plane + i] = e4;
}

// sigma-bar += E^T e-bar (gather form of sdiff2's transpose).
template <int NS>
__global__ void k_exact_adj_sigma(const P64 p, ExactBufs X, const int sin)
{
    int iz, ix, bz;
    if (!grid_point(p, iz, ix, bz)) return;
    const long long i = (long long)iz * p.pitch + ix;
    const double *e1 = wplane(X, p, bz, EX_EB), *e2 = e1 + p.plane, *e3 = e2 + p.plane;
    const double *e4 = e3 + p.plane;
    double gzz = 0.0, gzx = 0.0, gxx = 0.0;
#pragma unroll
    for (int k = 1; k <= NS; k++) {
        const double cz = p.cz[k - 1], cx = p.cx[k - 1];
        gzz += cz * (at0(p, e1, iz - k, ix) - at0(p, e1, iz + k - 1, ix));
        gzx += cz * (at0(p, e2, iz - k + 1, ix) - at0(p, e2, iz + k, ix));
        gzx += cx * (at0(p, e3, iz, ix - k + 1) - at0(p, e3, iz, ix + k));
        gxx += cx * (at0(p, e4, iz, ix - k) - at0(p, e4, iz, ix + k - 1));
    }
    double *sb = wplane(X, p, bz, sin);
    sb[i] += gzz;
    sb[p.plane + i] += gzx;
    sb[2 * p.plane + i] += gxx;
}

// Transpose of update_s2 + surf_mirror + pml_diff2 of the stress side:
// d-bar, gradients of dt lam, dt (lam + 2 mu), dt mu_zx and the surface
// factor; sigma-bar of the step's input into copy sout.
__global__ void k_exact_adj_stress(const P64 p, ExactBufs X, const int n, const int sin,
                                   const int sout)
{
    int iz, ix, bz;
    if (!grid_point(p, iz, ix, bz)) return;
    const long long i = (long long)iz * p.pitch + ix, PL = p.plane;
    const double *sb = wplane(X, p, bz, sin);
    double *so = wplane(X, p, bz, sout);
    double *db = wplane(X, p, bz, EX_DB);
    if (!interior(p, iz, ix)) {  // never updated: sigma-bar carries
        so[i] = sb[i]; so[PL + i] = sb[PL + i]; so[2 * PL + i] = sb[2 * PL + i];
        db[i] = db[PL + i] = db[2 * PL + i] = db[3 * PL + i] = 0.0;
        return;
    }
    const double *S = X.store + (long long)n * X.step_stride + (long long)bz * 8 * PL + i;
    const double d1 = S[0], d2 = S[PL], d3 = S[2 * PL], d4 = S[3 * PL];
    double zz = sb[i], zx = sb[PL + i], xx = sb[2 * PL + i];
    double b1, b2, b3, b4;
    if (p.st && iz == p.st) {  // szz = szx = 0, sxx = fs vx_x: no dependence on the old stresses
        b4 = p.fs_top[ix] * xx;
        b1 = b2 = b3 = 0.0;
        atomicAdd(wplane(X, p, bz, EX_GFS) + ix, xx * d4);
        zz = zx = xx = 0.0;
        so[i] = 0.0; so[PL + i] = 0.0; so[2 * PL + i] = 0.0;
    } else {
        if (p.st && iz < p.st) {  // mirrored rows: their updated szz, szx are overwritten
            zz = 0.0;
            zx = 0.0;
        } else if (p.st && iz <= 2 * p.st - p.nz1) {  // image rows feed the mirrored rows
            const long long j = (long long)(2 * p.st - iz) * p.pitch + ix;
            zz -= sb[j];
            zx -= sb[PL + j];
        }
        const double c2 = p.c_l2m[i], cl = p.c_lam[i], cm = p.c_muzx[i];
        b1 = c2 * zz + cl * xx;
        b4 = cl * zz + c2 * xx;
        b2 = b3 = cm * zx;
        wplane(X, p, bz, EX_GC2)[i] += zz * d1 + xx * d4;
        wplane(X, p, bz, EX_GCL)[i] += zz * d4 + xx * d1;
        wplane(X, p, bz, EX_GCM)[i] += zx * (d3 + d2);
        so[i] = zz; so[PL + i] = zx; so[2 * PL + i] = xx;
    }
    if (iz < p.pz0 || iz >= p.pz1) {
        const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
        double *m = X.qz + (long long)bz * p.mz_shot_stride + (long long)rr * p.pitch + ix;
        b1 = cpml_adj(m + MZ_VZ * p.mz_plane, b1, p.a_z[iz], p.b_z[iz], p.ki_z[iz]);
        b2 = cpml_adj(m + MZ_VX * p.mz_plane, b2, p.ah_z[iz], p.bh_z[iz], p.khi_z[iz]);
    }
    if (ix < p.px0 || ix >= p.px1) {
        const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
        double *m = X.qx + (long long)bz * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
        b4 = cpml_adj(m + MX_VX * p.mx_plane, b4, p.a_x[ix], p.b_x[ix], p.ki_x[ix]);
        b3 = cpml_adj(m + MX_VZ * p.mx_plane, b3, p.ah_x[ix], p.bh_x[ix], p.khi_x[ix]);
    }
    db[i] = b1; db[PL + i] = b2; db[2 * PL + i] = b3; db[3 * PL + i] = b4;
}

// v-bar += D^T d-bar (gather form of vdiff2's transpose).
template <int NS>
__global__ void k_exact_adj_v(const P64 p, ExactBufs X)
{
    int iz, ix, bz;
    if (!grid_point(p, iz, ix, bz)) return;
    const long long i = (long long)iz * p.pitch + ix;
    const double *d1 = wplane(X, p, bz, EX_DB), *d2 = d1 + p.plane, *d3 = d2 + p.plane;
    const double *d4 = d3 + p.plane;
    double gz = 0.0, gx = 0.0;
#pragma unroll
    for (int k = 1; k <= NS; k++) {
        const double cz = p.cz[k - 1], cx = p.cx[k - 1];
        gz += cz * (at0(p, d1, iz - k + 1, ix) - at0(p, d1, iz + k, ix));
        gz += cx * (at0(p, d3, iz, ix - k) - at0(p, d3, iz, ix + k - 1));
        gx += cz * (at0(p, d2, iz - k, ix) - at0(p, d2, iz + k - 1, ix));
        gx += cx * (at0(p, d4, iz, ix - k + 1) - at0(p, d4, iz, ix + k));
    }
    wplane(X, p, bz, EX_VBZ)[i] += gz;
    wplane(X, p, bz, EX_VBX)[i] += gx;
}

// Chain rule from the dt-scaled coefficients to lam, mu, rho (mat_av2,
// src/cpu/n_kernel_lib_PSV.cpp:853-898, and the surface factor), summed over
// the batch's shots into the global gradients with factor `sign`.
__global__ void k_exact_chain(const P64 p, ExactBufs X, const double *lam, const double *mu,
                              const double *rho, double *gl, double *gm, double *gr, double dt,
                              double sign)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, iz = blockIdx.y * blockDim.y + threadIdx.y;
    const int nz = p.nz, nx = p.nx;
    if (ix >= nx || iz >= nz) return;
    const long long k = (long long)iz * nx + ix;
    double sl = 0.0, sm = 0.0, sr = 0.0;
    for (int bz = 0; bz < p.ctl[1]; bz++) {
        auto G = [&](int plane, int z, int x) {
            return wplane(X, p, bz, plane)[(long long)z * p.pitch + x];
        };
        const long long i = (long long)iz * p.pitch + ix;
        sl += dt * (G(EX_GCL, iz, ix) + G(EX_GC2, iz, ix));
        sm += 2.0 * dt * G(EX_GC2, iz, ix);
        (void)i;
        // mu_zx at (z, x) = 4 / sum of 1/mu over its four cells, for z < nz - 1, x < nx - 1
        for (int dz = -1; dz <= 0; dz++)
            for (int dx = -1; dx <= 0; dx++) {
                const int z = iz + dz, x = ix + dx;
                if (z < 0 || x < 0 || z >= nz - 1 || x >= nx - 1) continue;
                const long long c = (long long)z * nx + x;
                const double m00 = mu[c], m01 = mu[c + 1], m10 = mu[c + nx], m11 = mu[c + nx + 1];
                if (m00 == 0.0 || m01 == 0.0 || m10 == 0.0 || m11 == 0.0) continue;
                const double mz = 4.0 / ((1.0 / m00) + (1.0 / m01) + (1.0 / m10) + (1.0 / m11));
                sm += dt * G(EX_GCM, z, x) * mz * mz / (4.0 * mu[k] * mu[k]);
            }
        // rho_zp at (z, x) = 1 / (rho(z, x) + rho(z + 1, x)) * 2, rho_xp with (z, x + 1)
        for (int dz = -1; dz <= 0; dz++) {
            const int z = iz + dz;
            if (z < 0 || z >= nz - 1 || ix >= nx - 1) continue;
            const long long c = (long long)z * nx + ix;
            const double r00 = rho[c], r10 = rho[c + nx], r01 = rho[c + 1];
            if ((r00 < 1e-4 && r10 < 1e-4) || (r00 < 1e-4 && r01 < 1e-4)) continue;
            const double rz = 1.0 / (0.5 * (r00 + r10));
            sr += dt * G(EX_GRZ, z, ix) * (-0.5 * rz * rz);
        }
        for (int dx = -1; dx <= 0; dx++) {
            const int x = ix + dx;
            if (x < 0 || x >= nx - 1 || iz >= nz - 1) continue;
            const long long c = (long long)iz * nx + x;
            const double rx = 1.0 / (0.5 * (rho[c] + rho[c + 1]));
            sr += dt * G(EX_GRX, iz, x) * (-0.5 * rx * rx);
        }
        if (p.st && iz == p.st) {  // fs = 4 dt (lam mu + mu^2) / (lam + 2 mu)
            const double l = lam[k], m = mu[k], d = l + 2.0 * m;
            const double g = wplane(X, p, bz, EX_GFS)[ix];
            sl += g * 4.0 * dt * m * m / (d * d);
            sm += g * 4.0 * dt * (l * l + 2.0 * l * m + 2.0 * m * m) / (d * d);
        }
    }
    gl[k] += sign * sl;
    gm[k] += sign * sm;
    gr[k] += sign * sr;
}

template <int NS>
cudaError_t fwd_step_ns(const P64 &p, const ExactBufs &X, int n, int nbatch, cudaStream_t st)
{
    const dim3 b(32, 8), g((p.nx + 31) / 32, (p.nz + 7) / 8, nbatch);
    k_exact_stress<NS><<<g, b, 0, st>>>(p, X, n);
    k_exact_velocity<NS><<<g, b, 0, st>>>(p, X, n);
    return cudaGetLastError();
}

template <int NS>
cudaError_t adj_step_ns(const P64 &p, const Q64 &q, const ExactBufs &X, int n, int sin, int sout,
                        int nbatch, int maxsrc, cudaStream_t st)
{
    const dim3 b(32, 8), g((p.nx + 31) / 32, (p.nz + 7) / 8, nbatch);
    if (q.nrec) k_exact_adj_record<<<dim3((q.nrec + 127) / 128, nbatch), 128, 0, st>>>(p, q, X, n);
    if (maxsrc) k_exact_adj_source<<<dim3((maxsrc + 127) / 128, nbatch), 128, 0, st>>>(p, q, X, n);
    k_exact_adj_velocity<<<g, b, 0, st>>>(p, X, n);
    k_exact_adj_sigma<NS><<<g, b, 0, st>>>(p, X, sin);
    k_exact_adj_stress<<<g, b, 0, st>>>(p, X, n, sin, sout);
    k_exact_adj_v<NS><<<g, b, 0, st>>>(p, X);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_exact_forward_step(const StepParams<double> &p, const SrcRecParams<double> &q,
                                      const ExactBufs &X, int ns, int n, int nbatch, int maxsrc,
                                      cudaStream_t st)
{
    cudaError_t e;
    switch (ns) {
    case 1: e = fwd_step_ns<1>(p, X, n, nbatch, st); break;
    case 2: e = fwd_step_ns<2>(p, X, n, nbatch, st); break;
    case 3: e = fwd_step_ns<3>(p, X, n, nbatch, st); break;
    case 4: e = fwd_step_ns<4>(p, X, n, nbatch, st); break;
    default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    if (maxsrc) k_exact_inject<<<dim3((maxsrc + 127) / 128, nbatch), 128, 0, st>>>(p, q, n);
    if (q.nrec) k_exact_record<<<dim3((q.nrec + 127) / 128, nbatch), 128, 0, st>>>(p, q, n);
    return cudaGetLastError();
}

cudaError_t launch_exact_revsum(double *res_z, double *res_x, int nt, int nrec, long long stride,
                                double dt, double gain, int nbatch, cudaStream_t st)
{
    if (!nrec) return cudaSuccess;
    k_exact_revsum<<<dim3((nrec + 127) / 128, nbatch), 128, 0, st>>>(res_z, res_x, nt, nrec,
                                                                    stride, dt, gain, nbatch);
    return cudaGetLastError();
}

cudaError_t launch_exact_adjoint_step(const StepParams<double> &p, const SrcRecParams<double> &q,
                                      const ExactBufs &X, int ns, int n, int sin, int sout,
                                      int nbatch, int maxsrc, cudaStream_t st)
{
    switch (ns) {
    case 1: return adj_step_ns<1>(p, q, X, n, sin, sout, nbatch, maxsrc, st);
    case 2: return adj_step_ns<2>(p, q, X, n, sin, sout, nbatch, maxsrc, st);
    case 3: return adj_step_ns<3>(p, q, X, n, sin, sout, nbatch, maxsrc, st);
    case 4: return adj_step_ns<4>(p, q, X, n, sin, sout, nbatch, maxsrc, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_exact_chain(const StepParams<double> &p, const ExactBufs &X, const double *lam,
                               const double *mu, const double *rho, double *gl, double *gm,
                               double *gr, double dt, double sign, cudaStream_t st)
{
    const dim3 b(32, 8), g((p.nx + 31) / 32, (p.nz + 7) / 8);
    k_exact_chain<<<g, b, 0, st>>>(p, X, lam, mu, rho, gl, gm, gr, dt, sign);
    return cudaGetLastError();
}

}  // namespace psv
