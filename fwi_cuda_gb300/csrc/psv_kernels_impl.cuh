// psv_kernels_impl.cuh -- bodies of the time-step kernels, instantiated for
// float and double by psv_kernels_f32.cu / psv_kernels_f64.cu.
//
// Thread mapping (both kernels): a block is 32 x BY threads; one warp covers
// 32 consecutive columns, and each thread marches RPT consecutive rows of its
// column.  The vertical stencil window of a field (RPT + 2N - 1 values) is
// loaded once into registers, so a thread issues independent loads up front
// and reuses each value for up to 2N rows; horizontal neighbours come from
// the adjacent lanes by warp shuffle, only the N lanes at each warp edge read
// memory for them.
#pragma once

#include "psv_kernels.cuh"

namespace psv {

// Value at column ix + d of the row: with SH, from lane + d by shuffle (all
// 32 lanes must call) and from memory only when that lane is outside the
// warp; without SH, a plain (L1-cached) load.
template <bool SH, typename T>
__device__ __forceinline__ T xnb(T own, int d, const T *__restrict__ row, int ix, int nx,
                                 bool rowok)
{
    if constexpr (SH) {
        const int src = (int)threadIdx.x + d;
        T v = __shfl_sync(0xffffffffu, own, src & 31);
        if (src < 0 || src > 31) {
            const int c = ix + d;
            v = (rowok && c >= 0 && c < nx) ? row[c] : T(0);
        }
        return v;
    } else {
        const int c = ix + d;
        return (rowok && c >= 0 && c < nx) ? row[c] : T(0);
    }
}

// ---------------------------------------------------------------------------
// Stress step: vdiff2 + pml_diff2 + update_s2 + surf_mirror
// (src/cpu/n_kernel_lib_PSV.cpp:100-131, 134-178, 181-205, 272-395).
//
// Interior points only.  The free-surface mirror is done by the thread that
// owns the image row/column: it writes the negated new stress to the mirrored
// cell, while the mirrored cell's own thread skips writing the mirrored
// components.  Every cell has exactly one writer and the result equals the
// reference's update-then-mirror sequence for a top and/or bottom surface, or
// a left and/or right surface.
// ---------------------------------------------------------------------------
template <typename T, int NS, int RPT, bool SH>
__global__ void __launch_bounds__(256) k_stress(const StepParams<T> p)
{
    if ((int)blockIdx.z >= p.ctl[1]) return;
    const int ix = p.nx1 + blockIdx.x * 32 + threadIdx.x;
    const int zb = p.nz1 + (blockIdx.y * blockDim.y + threadIdx.y) * RPT;
    if (zb >= p.nz2) return;  // uniform across the warp; no block barrier follows
    const long long P = p.pitch;
    T *f = p.fld + (long long)blockIdx.z * p.shot_stride;
    const T *__restrict__ vz = f + F_VZ * p.plane;
    const T *__restrict__ vx = f + F_VX * p.plane;
    T *szz = f + F_SZZ * p.plane;
    T *szx = f + F_SZX * p.plane;
    T *sxx = f + F_SXX * p.plane;
    const bool colin = ix < p.nx2, colok = ix < p.nx;

    // wz[j] = vz[zb - N + j], wx[j] = vx[zb - N + 1 + j]
    constexpr int W = RPT + 2 * NS - 1;
    T wz[W], wx[W];
#pragma unroll
    for (int j = 0; j < W; j++) {
        const int rz = zb - NS + j, rx = zb - NS + 1 + j;  // >= 0: zb >= fpad >= N
        wz[j] = (colok && rz < p.nz) ? vz[(long long)rz * P + ix] : T(0);
        wx[j] = (colok && rx < p.nz) ? vx[(long long)rx * P + ix] : T(0);
    }

#pragma unroll
    for (int r = 0; r < RPT; r++) {
        const int iz = zb + r;
        const bool rowload = iz < p.nz;
        const long long rowoff = (long long)(rowload ? iz : 0) * P;
        const T *vzr = vz + rowoff, *vxr = vx + rowoff;
        // staggered derivatives; term 1 is the reference's 2-point difference
        const T oz = wz[r + NS], ox = wx[r + NS - 1];
        T vz_z = p.cz[0] * (oz - wz[r + NS - 1]);
        T vx_z = p.cz[0] * (wx[r + NS] - ox);
        T vz_x = p.cx[0] * (xnb<SH>(oz, 1, vzr, ix, p.nx, rowload) - oz);
        T vx_x = p.cx[0] * (ox - xnb<SH>(ox, -1, vxr, ix, p.nx, rowload));
#pragma unroll
        for (int k = 2; k <= NS; k++) {
            vz_z += p.cz[k - 1] * (wz[r + NS + k - 1] - wz[r + NS - k]);
            vx_z += p.cz[k - 1] * (wx[r + NS + k - 1] - wx[r + NS - k]);
            vz_x += p.cx[k - 1] * (xnb<SH>(oz, k, vzr, ix, p.nx, rowload) -
                                   xnb<SH>(oz, -(k - 1), vzr, ix, p.nx, rowload));
            vx_x += p.cx[k - 1] * (xnb<SH>(ox, k - 1, vxr, ix, p.nx, rowload) -
                                   xnb<SH>(ox, -k, vxr, ix, p.nx, rowload));
        }
        if (iz >= p.nz2 || !colin) continue;
        const long long i = (long long)iz * P + ix;

        // CPML recursion, only on the absorbing strips (a = 0, b = K = 1 elsewhere)
        if (iz < p.pz0 || iz >= p.pz1) {
            const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
            T *m = p.memz + (long long)blockIdx.z * p.mz_shot_stride + (long long)rr * P + ix;
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
}

// ---------------------------------------------------------------------------
// Velocity step: sdiff2 + pml_diff2 + update_v2 (src/cpu/n_kernel_lib_PSV.cpp:
// 207-270, 134-178), fused with the step's remaining work:
//   forward modes: gard_fwd_storage2 (:398-436) into `slot`;
//   MODE_ADJ: u += dt v, and fwi_grad2 (:439-484, CPU sign) against `slot`;
//   epilogue: vsrc2 + urec2 (:487-576) for the sources / receivers of the
//   block's tile, after all of the tile's velocities are written.
// Covers the whole grid: cells outside the interior only take part in the
// snapshot / imaging work (their fields are never updated).
// ---------------------------------------------------------------------------
template <typename T, int NS, int MODE, int RPT, bool SH>
__global__ void __launch_bounds__(256) k_velocity(const StepParams<T> p, const SrcRecParams<T> q,
                                                  const int it, const int slot)
{
    if ((int)blockIdx.z >= p.ctl[1]) return;  // whole block
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int zb = (blockIdx.y * blockDim.y + threadIdx.y) * RPT;
    const long long P = p.pitch;
    T *f = p.fld + (long long)blockIdx.z * p.shot_stride;
    const T *__restrict__ szz = f + F_SZZ * p.plane;
    const T *__restrict__ szx = f + F_SZX * p.plane;
    const T *__restrict__ sxx = f + F_SXX * p.plane;
    T *vz = f + F_VZ * p.plane;
    T *vx = f + F_VX * p.plane;
    const bool colok = ix < p.nx;
    const bool colin = ix >= p.nx1 && ix < p.nx2;
    const long long sp = p.snap_plane;

    if (zb < p.nz) {  // warp-uniform
        // wzz[j] = szz[zb - N + 1 + j], wzx[j] = szx[zb - N + j]
        constexpr int W = RPT + 2 * NS - 1;
        T wzz[W], wzx[W], wxx[RPT];
#pragma unroll
        for (int j = 0; j < W; j++) {
            const int ra = zb - NS + 1 + j, rb = zb - NS + j;
            wzz[j] = (colok && ra >= 0 && ra < p.nz) ? szz[(long long)ra * P + ix] : T(0);
            wzx[j] = (colok && rb >= 0 && rb < p.nz) ? szx[(long long)rb * P + ix] : T(0);
        }
#pragma unroll
        for (int r = 0; r < RPT; r++) {
            const int iz = zb + r;
            wxx[r] = (colok && iz < p.nz) ? sxx[(long long)iz * P + ix] : T(0);
        }

#pragma unroll
        for (int r = 0; r < RPT; r++) {
            const int iz = zb + r;
            const bool rowload = iz < p.nz;
            const long long rowoff = (long long)(rowload ? iz : 0) * P;
            const T *szxr = szx + rowoff, *sxxr = sxx + rowoff;
            const T ozz = wzz[r + NS - 1], ozx = wzx[r + NS], oxx = wxx[r];
            T szz_z = p.cz[0] * (wzz[r + NS] - ozz);
            T szx_z = p.cz[0] * (ozx - wzx[r + NS - 1]);
            T szx_x = p.cx[0] * (ozx - xnb<SH>(ozx, -1, szxr, ix, p.nx, rowload));
            T sxx_x = p.cx[0] * (xnb<SH>(oxx, 1, sxxr, ix, p.nx, rowload) - oxx);
#pragma unroll
            for (int k = 2; k <= NS; k++) {
                szz_z += p.cz[k - 1] * (wzz[r + NS + k - 1] - wzz[r + NS - k]);
                szx_z += p.cz[k - 1] * (wzx[r + NS + k - 1] - wzx[r + NS - k]);
                szx_x += p.cx[k - 1] * (xnb<SH>(ozx, k - 1, szxr, ix, p.nx, rowload) -
                                        xnb<SH>(ozx, -k, szxr, ix, p.nx, rowload));
                sxx_x += p.cx[k - 1] * (xnb<SH>(oxx, k, sxxr, ix, p.nx, rowload) -
                                        xnb<SH>(oxx, -(k - 1), sxxr, ix, p.nx, rowload));
            }
            if (!rowload || !colok) continue;
            const long long i = (long long)iz * P + ix;
            const bool inner = colin && iz >= p.nz1 && iz < p.nz2;
            T vzn, vxn, uzn = T(0), uxn = T(0);
            if (inner) {
                if (iz < p.pz0 || iz >= p.pz1) {
                    const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
                    T *m = p.memz + (long long)blockIdx.z * p.mz_shot_stride + (long long)rr * P + ix;
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
            if (slot < 0) continue;
            const int dzr = iz - p.snap_z1, dxr = ix - p.snap_x1;
            if (dzr < 0 || iz > p.snap_z2 || dxr < 0 || ix > p.snap_x2) continue;
            if (dzr % p.snap_dz || dxr % p.snap_dx) continue;
            const long long qq = (long long)(dzr / p.snap_dz) * p.snx_pitch + dxr / p.snap_dx;
            T *h = p.hist + (long long)blockIdx.z * p.hist_shot_stride + (long long)slot * p.hist_slot_stride + qq;
            if (MODE != MODE_ADJ) {
                h[H_SZZ * sp] = ozz;
                h[H_SZX * sp] = ozx;
                h[H_SXX * sp] = oxx;
                h[H_VZ * sp] = vzn * p.inv_dt;
                h[H_VX * sp] = vxn * p.inv_dt;
            } else {
                const T fzz = h[H_SZZ * sp], fzx = h[H_SZX * sp], fxx = h[H_SXX * sp];
                const T fvz = h[H_VZ * sp], fvx = h[H_VX * sp];
                const T s1 = p.g1[i] * ((fzz + fxx) * (ozz + oxx));
                const T s23 = p.g2[i] * (fzx * ozx + T(0.25) * ((fzz - fxx) * (ozz - oxx)));
                T *g = p.gshot + (long long)blockIdx.z * p.gshot_shot_stride + qq;
                g[0] -= s1;
                g[sp] -= s23 + s1;
                g[2 * sp] -= p.kimg * (uxn * fvx + uzn * fvz);
            }
        }
    }

    // ---- epilogue: sources and receivers of this tile (vsrc2, urec2) ----
    if (q.src_kind < 0 && !q.rtf_z) return;  // uniform: kernel argument
    const int tile = blockIdx.y * gridDim.x + blockIdx.x;
    const int shot = p.ctl[0] + blockIdx.z;
    const int tid = threadIdx.y * 32 + threadIdx.x, nth = 32 * blockDim.y;
    int k0 = 0, k1 = 0;
    if (q.src_kind == 0) {
        const int *off = q.t_src_off + (long long)shot * (q.ntiles + 1);
        k0 = off[tile];
        k1 = off[tile + 1];
    } else if (q.src_kind == 1) {
        k0 = q.t_rec_off[tile];
        k1 = q.t_rec_off[tile + 1];
    }
    const bool recs = q.rtf_z && q.t_rec_off[tile] < q.t_rec_off[tile + 1];
    if (k0 == k1 && !recs) return;  // uniform over the block
    __syncthreads();  // the tile's velocities are written
    const double sc = q.amp_scale[shot];
    const double *sz = q.stf_z + shot * q.stf_shot_stride + (long long)it * q.stf_ncol;
    const double *sx = q.stf_x + shot * q.stf_shot_stride + (long long)it * q.stf_ncol;
    for (int k = k0 + tid; k < k1; k += nth) {
        int pos, col;
        if (q.src_kind == 0) {
            const int j = q.t_src_k[k];
            pos = q.src_pos[j];
            col = q.src_col[j];
        } else {
            const int rr = q.t_rec_r[k];
            pos = q.rec_pos[rr];
            col = rr;
        }
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
    if (recs) {
        double *rz = q.rtf_z + shot * q.rtf_shot_stride;
        double *rx = q.rtf_x + shot * q.rtf_shot_stride;
        const double ru = q.rec_unscale[shot];
        const long long row = (long long)it * q.nrec;
        for (int k = q.t_rec_off[tile] + tid; k < q.t_rec_off[tile + 1]; k += nth) {
            const int rr = q.t_rec_r[k];
            const int pos = q.rec_pos[rr];
            const double pz = it ? rz[row - q.nrec + rr] : 0.0;
            const double px = it ? rx[row - q.nrec + rr] : 0.0;
            rz[row + rr] = pz + ((q.dt_d * (double)vz[pos]) / q.dzdx) * ru;
            rx[row + rr] = px + ((q.dt_d * (double)vx[pos]) / q.dzdx) * ru;
        }
    }
    if (slot >= 0 && q.src_kind == 0 && MODE != MODE_ADJ) {  // snapshot holds post-injection v
        T *h = p.hist + (long long)blockIdx.z * p.hist_shot_stride + (long long)slot * p.hist_slot_stride;
        for (int k = k0 + tid; k < k1; k += nth) {
            const int j = q.t_src_k[k];
            const int c = q.src_snap[j];
            if (c < 0) continue;
            const int pos = q.src_pos[j];
            h[H_VZ * sp + c] = vz[pos] * p.inv_dt;
            h[H_VX * sp + c] = vx[pos] * p.inv_dt;
        }
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers.  rpt (rows per thread) 1, 2 or 4; rpt < 0 selects the
// shuffle variant with |rpt| rows.  FP64 uses 1 row, plain loads.
// ---------------------------------------------------------------------------

template <typename T, int NS>
static cudaError_t launch_stress_ns(const StepParams<T> &p, int rpt, dim3 block, int nbatch,
                                    cudaStream_t st)
{
    const int rows = p.nz2 - p.nz1, cols = p.nx2 - p.nx1, ar = rpt < 0 ? -rpt : rpt;
    dim3 grid((cols + 31) / 32, (rows + block.y * ar - 1) / (block.y * ar), nbatch);
    if constexpr (sizeof(T) == 8) {
        k_stress<T, NS, 1, false><<<grid, block, 0, st>>>(p);
    } else {
        switch (rpt) {
        case 2: k_stress<T, NS, 2, false><<<grid, block, 0, st>>>(p); break;
        case 4: k_stress<T, NS, 4, false><<<grid, block, 0, st>>>(p); break;
        case -2: k_stress<T, NS, 2, true><<<grid, block, 0, st>>>(p); break;
        case -4: k_stress<T, NS, 4, true><<<grid, block, 0, st>>>(p); break;
        default: k_stress<T, NS, 1, false><<<grid, block, 0, st>>>(p); break;
        }
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_stress(const StepParams<T> &p, int ns, int rpt, dim3 block, int nbatch,
                          cudaStream_t st)
{
    rpt = rpt_ok<T>(rpt);
    switch (ns) {
    case 1: return launch_stress_ns<T, 1>(p, rpt, block, nbatch, st);
    case 2: return launch_stress_ns<T, 2>(p, rpt, block, nbatch, st);
    case 3: return launch_stress_ns<T, 3>(p, rpt, block, nbatch, st);
    case 4: return launch_stress_ns<T, 4>(p, rpt, block, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <typename T, int NS, int MODE>
static cudaError_t launch_velocity_m(const StepParams<T> &p, const SrcRecParams<T> &q, int it,
                                     int slot, int rpt, dim3 block, int nbatch, cudaStream_t st)
{
    const int ar = rpt < 0 ? -rpt : rpt;
    dim3 grid((p.nx + 31) / 32, (p.nz + block.y * ar - 1) / (block.y * ar), nbatch);
    if constexpr (sizeof(T) == 8) {
        k_velocity<T, NS, MODE, 1, false><<<grid, block, 0, st>>>(p, q, it, slot);
    } else {
        switch (rpt) {
        case 2: k_velocity<T, NS, MODE, 2, false><<<grid, block, 0, st>>>(p, q, it, slot); break;
        case 4: k_velocity<T, NS, MODE, 4, false><<<grid, block, 0, st>>>(p, q, it, slot); break;
        case -2: k_velocity<T, NS, MODE, 2, true><<<grid, block, 0, st>>>(p, q, it, slot); break;
        case -4: k_velocity<T, NS, MODE, 4, true><<<grid, block, 0, st>>>(p, q, it, slot); break;
        default: k_velocity<T, NS, MODE, 1, false><<<grid, block, 0, st>>>(p, q, it, slot); break;
        }
    }
    return cudaGetLastError();
}

template <typename T, int NS>
static cudaError_t launch_velocity_ns(const StepParams<T> &p, const SrcRecParams<T> &q, int mode,
                                      int it, int slot, int rpt, dim3 block, int nbatch,
                                      cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: return launch_velocity_m<T, NS, MODE_FWD>(p, q, it, slot, rpt, block, nbatch, st);
    case MODE_FWD_NOWE: return launch_velocity_m<T, NS, MODE_FWD_NOWE>(p, q, it, slot, rpt, block, nbatch, st);
    case MODE_FWD_U: return launch_velocity_m<T, NS, MODE_FWD_U>(p, q, it, slot, rpt, block, nbatch, st);
    case MODE_ADJ: return launch_velocity_m<T, NS, MODE_ADJ>(p, q, it, slot, rpt, block, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_velocity(const StepParams<T> &p, const SrcRecParams<T> &q, int ns, int mode,
                            int it, int slot, int rpt, dim3 block, int nbatch, cudaStream_t st)
{
    rpt = rpt_ok<T>(rpt);
    switch (ns) {
    case 1: return launch_velocity_ns<T, 1>(p, q, mode, it, slot, rpt, block, nbatch, st);
    case 2: return launch_velocity_ns<T, 2>(p, q, mode, it, slot, rpt, block, nbatch, st);
    case 3: return launch_velocity_ns<T, 3>(p, q, mode, it, slot, rpt, block, nbatch, st);
    case 4: return launch_velocity_ns<T, 4>(p, q, mode, it, slot, rpt, block, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

#define PSV_INSTANTIATE_STEP(T)                                                                     \
    template cudaError_t launch_stress<T>(const StepParams<T> &, int, int, dim3, int, cudaStream_t); \
    template cudaError_t launch_velocity<T>(const StepParams<T> &, const SrcRecParams<T> &, int,    \
                                            int, int, int, int, dim3, int, cudaStream_t);

}  // namespace psv
