// psv_kernels_impl.cuh -- bodies of the time-step kernels, instantiated for
// float and double by psv_kernels_f32.cu / psv_kernels_f64.cu.
#pragma once

#include "psv_kernels.cuh"

namespace psv {

// ---------------------------------------------------------------------------
// Stress step: vdiff2 + pml_diff2 + update_s2 + surf_mirror
// (src/cpu/n_kernel_lib_PSV.cpp:100-131, 134-178, 181-205, 272-395).
//
// One thread per interior point.  The free-surface mirror is done by the
// thread that owns the image row/column: it writes the negated new stress
// to the mirrored cell, while the mirrored cell's own thread skips writing
// the mirrored components.  Every cell therefore has exactly one writer and
// the result equals the reference's update-then-mirror sequence for a top
// and/or bottom surface, or a left and/or right surface.
// ---------------------------------------------------------------------------
template <typename T, int NS>
__global__ void __launch_bounds__(256) k_stress(const StepParams<T> p)
{
    const int ix = p.nx1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = p.nz1 + blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= p.nx2 || iz >= p.nz2 || (int)blockIdx.z >= p.ctl[1]) return;
    const long long P = p.pitch;
    T *f = p.fld + (long long)blockIdx.z * p.shot_stride;
    const T *__restrict__ vz = f + F_VZ * p.plane;
    const T *__restrict__ vx = f + F_VX * p.plane;
    T *szz = f + F_SZZ * p.plane;
    T *szx = f + F_SZX * p.plane;
    T *sxx = f + F_SXX * p.plane;
    const long long i = (long long)iz * P + ix;

    // Staggered derivatives; term 1 is the reference's 2-point difference.
    T vz_z = p.cz[0] * (vz[i] - vz[i - P]);
    T vx_z = p.cz[0] * (vx[i + P] - vx[i]);
    T vz_x = p.cx[0] * (vz[i + 1] - vz[i]);
    T vx_x = p.cx[0] * (vx[i] - vx[i - 1]);
#pragma unroll
    for (int k = 2; k <= NS; k++) {
        vz_z += p.cz[k - 1] * (vz[i + (k - 1) * P] - vz[i - k * P]);
        vx_z += p.cz[k - 1] * (vx[i + k * P] - vx[i - (k - 1) * P]);
        vz_x += p.cx[k - 1] * (vz[i + k] - vz[i - (k - 1)]);
        vx_x += p.cx[k - 1] * (vx[i + (k - 1)] - vx[i - k]);
    }

    // CPML recursion, only on the absorbing strips (a = 0, b = K = 1 elsewhere).
    if (iz < p.pz0 || iz >= p.pz1) {
        const int r = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
        T *m = p.memz + (long long)blockIdx.z * p.mz_shot_stride + (long long)r * P + ix;
        const T m0 = p.b_z[iz] * m[MZ_VZ * p.mz_plane] + p.a_z[iz] * vz_z;
        const T m1 = p.bh_z[iz] * m[MZ_VX * p.mz_plane] + p.ah_z[iz] * vx_z;
        m[MZ_VZ * p.mz_plane] = m0;
        m[MZ_VX * p.mz_plane] = m1;
        vz_z = vz_z * p.ki_z[iz] + m0;
        vx_z = vx_z * p.khi_z[iz] + m1;
    }
    if (ix < p.px0 || ix >= p.px1) {
        const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
        T *m = p.memx + (long long)blockIdx.z * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
        const T m0 = p.b_x[ix] * m[MX_VX * p.mx_plane] + p.a_x[ix] * vx_x;
        const T m1 = p.bh_x[ix] * m[MX_VZ * p.mx_plane] + p.ah_x[ix] * vz_x;
        m[MX_VX * p.mx_plane] = m0;
        m[MX_VZ * p.mx_plane] = m1;
        vx_x = vx_x * p.ki_x[ix] + m0;
        vz_x = vz_x * p.khi_x[ix] + m1;
    }

    const T cl = p.c_lam[i], c2 = p.c_l2m[i];
    T nzz = szz[i] + (c2 * vz_z + cl * vx_x);
    T nxx = sxx[i] + (cl * vz_z + c2 * vx_x);
    T nzx = szx[i] + p.c_muzx[i] * (vz_x + vx_z);

    bool wzz = true, wzx = true, wxx = true;
    if (p.st) {  // top: rows [nz1, st) mirror rows (st, 2 st - nz1]
        if (iz == p.st) {
            nzz = T(0); nzx = T(0);
            nxx = p.fs_top[ix] * vx_x;
        } else if (iz < p.st) {
            wzz = false; wzx = false;
        } else if (iz <= 2 * p.st - p.nz1) {
            const long long j = (long long)(2 * p.st - iz) * P + ix;
            szz[j] = -nzz; szx[j] = -nzx;
        }
    }
    if (p.sb) {  // bottom: rows (sb, nz2] mirror rows [2 sb - nz2, sb)
        if (iz == p.sb) {
            nzz = T(0); nzx = T(0);
            nxx = p.fs_bot[ix] * vx_x;
        } else if (iz > p.sb) {
            wzz = false; wzx = false;
        } else if (iz >= 2 * p.sb - p.nz2) {
            const long long j = (long long)(2 * p.sb - iz) * P + ix;
            szz[j] = -nzz; szx[j] = -nzx;
        }
    }
    if (p.sl) {  // left: columns [nx1, sl) mirror columns (sl, 2 sl - nx1]
        if (ix == p.sl) {
            nxx = T(0); nzx = T(0);
            nzz = p.fs_left[iz] * vz_z;
        } else if (ix < p.sl) {
            wzx = false; wxx = false;
        } else if (ix <= 2 * p.sl - p.nx1) {
            const long long j = (long long)iz * P + (2 * p.sl - ix);
            szx[j] = -nzx; sxx[j] = -nxx;
        }
    }
    if (p.sr) {  // right: columns (sr, nx2] mirror columns [2 sr - nx2, sr)
        if (ix == p.sr) {
            nxx = T(0); nzx = T(0);
            nzz = p.fs_right[iz] * vz_z;
        } else if (ix > p.sr) {
            wzx = false; wxx = false;
        } else if (ix >= 2 * p.sr - p.nx2) {
            const long long j = (long long)iz * P + (2 * p.sr - ix);
            szx[j] = -nzx; sxx[j] = -nxx;
        }
    }
    if (wzz) szz[i] = nzz;
    if (wzx) szx[i] = nzx;
    if (wxx) sxx[i] = nxx;
}

// ---------------------------------------------------------------------------
// Velocity step: sdiff2 + pml_diff2 + update_v2 (src/cpu/n_kernel_lib_PSV.cpp:
// 207-270, 134-178), fused with the step's snapshot work:
//   forward modes: gard_fwd_storage2 (:398-436) into `slot`;
//   MODE_ADJ: u += dt v, and fwi_grad2 (:439-484, CPU sign) against `slot`.
// Launched over the whole grid: cells outside the interior only take part in
// the snapshot / imaging work (their fields are never updated).
// ---------------------------------------------------------------------------
template <typename T, int NS, int MODE>
__global__ void __launch_bounds__(256) k_velocity(const StepParams<T> p, const int slot)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= p.nx || iz >= p.nz || (int)blockIdx.z >= p.ctl[1]) return;
    const long long P = p.pitch;
    T *f = p.fld + (long long)blockIdx.z * p.shot_stride;
    const T *__restrict__ szz = f + F_SZZ * p.plane;
    const T *__restrict__ szx = f + F_SZX * p.plane;
    const T *__restrict__ sxx = f + F_SXX * p.plane;
    T *vz = f + F_VZ * p.plane;
    T *vx = f + F_VX * p.plane;
    const long long i = (long long)iz * P + ix;
    const bool inner = iz >= p.nz1 && iz < p.nz2 && ix >= p.nx1 && ix < p.nx2;

    T vzn, vxn, uzn = T(0), uxn = T(0);
    if (inner) {
        T szz_z = p.cz[0] * (szz[i + P] - szz[i]);
        T szx_z = p.cz[0] * (szx[i] - szx[i - P]);
        T szx_x = p.cx[0] * (szx[i] - szx[i - 1]);
        T sxx_x = p.cx[0] * (sxx[i + 1] - sxx[i]);
#pragma unroll
        for (int k = 2; k <= NS; k++) {
            szz_z += p.cz[k - 1] * (szz[i + k * P] - szz[i - (k - 1) * P]);
            szx_z += p.cz[k - 1] * (szx[i + (k - 1) * P] - szx[i - k * P]);
            szx_x += p.cx[k - 1] * (szx[i + (k - 1)] - szx[i - k]);
            sxx_x += p.cx[k - 1] * (sxx[i + k] - sxx[i - (k - 1)]);
        }
        if (iz < p.pz0 || iz >= p.pz1) {
            const int r = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
            T *m = p.memz + (long long)blockIdx.z * p.mz_shot_stride + (long long)r * P + ix;
            const T m0 = p.b_z[iz] * m[MZ_SZZ * p.mz_plane] + p.a_z[iz] * szz_z;
            const T m1 = p.bh_z[iz] * m[MZ_SZX * p.mz_plane] + p.ah_z[iz] * szx_z;
            m[MZ_SZZ * p.mz_plane] = m0;
            m[MZ_SZX * p.mz_plane] = m1;
            szz_z = szz_z * p.ki_z[iz] + m0;
            szx_z = szx_z * p.khi_z[iz] + m1;
        }
        if (ix < p.px0 || ix >= p.px1) {
            const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
            T *m = p.memx + (long long)blockIdx.z * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
            const T m0 = p.b_x[ix] * m[MX_SXX * p.mx_plane] + p.a_x[ix] * sxx_x;
            const T m1 = p.bh_x[ix] * m[MX_SZX * p.mx_plane] + p.ah_x[ix] * szx_x;
            m[MX_SXX * p.mx_plane] = m0;
            m[MX_SZX * p.mx_plane] = m1;
            sxx_x = sxx_x * p.ki_x[ix] + m0;
            szx_x = szx_x * p.khi_x[ix] + m1;
        }
        const T vzo = vz[i], vxo = vx[i];
        if (MODE == MODE_ADJ || MODE == MODE_FWD_U) {
            T *uz = f + F_UZ * p.plane;
            T *ux = f + F_UX * p.plane;
            uzn = uz[i] + p.dt * vzo;
            uxn = ux[i] + p.dt * vxo;
            uz[i] = uzn;
            ux[i] = uxn;
        }
        vzn = vzo + p.c_rz[i] * (szx_x + szz_z);
        vxn = vxo + p.c_rx[i] * (sxx_x + szx_z);
        vz[i] = vzn;
        vx[i] = vxn;
        if (MODE != MODE_FWD_NOWE) {
            T *we = f + (MODE == MODE_ADJ ? F_WEA : F_WE) * p.plane;
            we[i] += vxn * vxn + vzn * vzn;
        }
    } else {
        vzn = vz[i];
        vxn = vx[i];
        if (MODE == MODE_ADJ || MODE == MODE_FWD_U) {
            uzn = f[F_UZ * p.plane + i];
            uxn = f[F_UX * p.plane + i];
        }
    }

    if (slot < 0) return;
    const int dzr = iz - p.snap_z1, dxr = ix - p.snap_x1;
    if (dzr < 0 || iz > p.snap_z2 || dxr < 0 || ix > p.snap_x2) return;
    if (dzr % p.snap_dz || dxr % p.snap_dx) return;
    const long long q = (long long)(dzr / p.snap_dz) * p.snx_pitch + dxr / p.snap_dx;
    const long long sp = p.snap_plane;
    T *h = p.hist + (long long)blockIdx.z * p.hist_shot_stride + (long long)slot * p.hist_slot_stride + q;
    if (MODE != MODE_ADJ) {
        h[H_SZZ * sp] = szz[i];
        h[H_SZX * sp] = szx[i];
        h[H_SXX * sp] = sxx[i];
        h[H_VZ * sp] = vzn * p.inv_dt;
        h[H_VX * sp] = vxn * p.inv_dt;
    } else {
        const T fzz = h[H_SZZ * sp], fzx = h[H_SZX * sp], fxx = h[H_SXX * sp];
        const T fvz = h[H_VZ * sp], fvx = h[H_VX * sp];
        const T azz = szz[i], azx = szx[i], axx = sxx[i];
        const T s1 = p.g1[i] * ((fzz + fxx) * (azz + axx));
        const T s23 = p.g2[i] * (fzx * azx + T(0.25) * ((fzz - fxx) * (azz - axx)));
        T *g = p.gshot + (long long)blockIdx.z * p.gshot_shot_stride + q;
        g[0] -= s1;
        g[sp] -= s23 + s1;
        g[2 * sp] -= p.kimg * (uxn * fvx + uzn * fvz);
    }
}

// ---------------------------------------------------------------------------
// Sources and receivers: vsrc2 + urec2 (src/cpu/n_kernel_lib_PSV.cpp:487-576).
// One block per shot.  Sources are added atomically (several may share a
// cell); receivers read the velocities after all injections and extend the
// FP64 running sum of displacement; the step's snapshot of a source cell is
// rewritten with the post-injection velocity (the reference stores after
// vsrc2).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_srcrec(const StepParams<T> p, const SrcRecParams<T> q,
                                                const int it, const int slot)
{
    const int b = blockIdx.x;
    if (b >= p.ctl[1]) return;
    const int shot = p.ctl[0] + b;
    T *f = p.fld + (long long)b * p.shot_stride;
    T *vz = f + F_VZ * p.plane;
    T *vx = f + F_VX * p.plane;
    const int k0 = q.src_off[shot], k1 = q.src_off[shot + 1];
    const double *sz = q.stf_z + shot * q.stf_shot_stride + (long long)it * q.stf_ncol;
    const double *sx = q.stf_x + shot * q.stf_shot_stride + (long long)it * q.stf_ncol;
    const double sc = q.amp_scale[shot];
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const int pos = q.src_pos[k], col = q.src_col[k];
        T az, ax;
        if (q.stf_type == 0) {
            az = p.c_rz[pos] * (T)(sz[col] * sc * q.inv_dzdx);
            ax = p.c_rx[pos] * (T)(sx[col] * sc * q.inv_dzdx);
        } else {
            az = (T)(sz[col] * sc);
            ax = (T)(sx[col] * sc);
        }
        atomicAdd(&vz[pos], az);
        atomicAdd(&vx[pos], ax);
    }
    __syncthreads();
    if (q.rtf_z) {
        double *rz = q.rtf_z + shot * q.rtf_shot_stride;
        double *rx = q.rtf_x + shot * q.rtf_shot_stride;
        const double ru = q.rec_unscale[shot];
        const long long row = (long long)it * q.nrec;
        for (int r = threadIdx.x; r < q.nrec; r += blockDim.x) {
            const int pos = q.rec_pos[r];
            const double pz = it ? rz[row - q.nrec + r] : 0.0;
            const double px = it ? rx[row - q.nrec + r] : 0.0;
            rz[row + r] = pz + ((q.dt_d * (double)vz[pos]) / q.dzdx) * ru;
            rx[row + r] = px + ((q.dt_d * (double)vx[pos]) / q.dzdx) * ru;
        }
    }
    if (slot >= 0) {
        T *h = p.hist + (long long)b * p.hist_shot_stride + (long long)slot * p.hist_slot_stride;
        for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            const int c = q.src_snap[k];
            if (c < 0) continue;
            const int pos = q.src_pos[k];
            h[H_VZ * p.snap_plane + c] = vz[pos] * p.inv_dt;
            h[H_VX * p.snap_plane + c] = vx[pos] * p.inv_dt;
        }
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
template <typename T>
cudaError_t launch_stress(const StepParams<T> &p, int ns, dim3 block, int nbatch, cudaStream_t st)
{
    dim3 grid((p.nx2 - p.nx1 + block.x - 1) / block.x, (p.nz2 - p.nz1 + block.y - 1) / block.y,
              nbatch);
    switch (ns) {
    case 1: k_stress<T, 1><<<grid, block, 0, st>>>(p); break;
    case 2: k_stress<T, 2><<<grid, block, 0, st>>>(p); break;
    case 3: k_stress<T, 3><<<grid, block, 0, st>>>(p); break;
    case 4: k_stress<T, 4><<<grid, block, 0, st>>>(p); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T, int NS>
static cudaError_t launch_velocity_ns(const StepParams<T> &p, int mode, int slot, dim3 grid,
                                      dim3 block, cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: k_velocity<T, NS, MODE_FWD><<<grid, block, 0, st>>>(p, slot); break;
    case MODE_FWD_NOWE: k_velocity<T, NS, MODE_FWD_NOWE><<<grid, block, 0, st>>>(p, slot); break;
    case MODE_FWD_U: k_velocity<T, NS, MODE_FWD_U><<<grid, block, 0, st>>>(p, slot); break;
    case MODE_ADJ: k_velocity<T, NS, MODE_ADJ><<<grid, block, 0, st>>>(p, slot); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_velocity(const StepParams<T> &p, int ns, int mode, int slot, dim3 block,
                            int nbatch, cudaStream_t st)
{
    dim3 grid((p.nx + block.x - 1) / block.x, (p.nz + block.y - 1) / block.y, nbatch);
    switch (ns) {
    case 1: return launch_velocity_ns<T, 1>(p, mode, slot, grid, block, st);
    case 2: return launch_velocity_ns<T, 2>(p, mode, slot, grid, block, st);
    case 3: return launch_velocity_ns<T, 3>(p, mode, slot, grid, block, st);
    case 4: return launch_velocity_ns<T, 4>(p, mode, slot, grid, block, st);
    default: return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_srcrec(const StepParams<T> &p, const SrcRecParams<T> &q, int it, int slot,
                          int nbatch, cudaStream_t st)
{
    k_srcrec<T><<<nbatch, 256, 0, st>>>(p, q, it, slot);
    return cudaGetLastError();
}

#define PSV_INSTANTIATE_STEP(T)                                                                 \
    template cudaError_t launch_stress<T>(const StepParams<T> &, int, dim3, int, cudaStream_t); \
    template cudaError_t launch_velocity<T>(const StepParams<T> &, int, int, int, dim3, int,    \
                                            cudaStream_t);                                      \
    template cudaError_t launch_srcrec<T>(const StepParams<T> &, const SrcRecParams<T> &, int,  \
                                          int, int, cudaStream_t);

}  // namespace psv
