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
// Per-point pieces shared by the direct-load kernels below and the TMA tile
// kernels (psv_tiled.cu), so both compute the same floating-point operations.
// ---------------------------------------------------------------------------

// pml_diff2 on the velocity derivatives of a stress update
// (src/cpu/n_kernel_lib_PSV.cpp:134-178), only on the absorbing strips
// (a = 0, b = K = 1 elsewhere).
template <typename T>
__device__ __forceinline__ void cpml_stress(const StepParams<T> &p, int shot, int iz, int ix,
                                            T &vz_z, T &vx_z, T &vz_x, T &vx_x)
{
    if (iz < p.pz0 || iz >= p.pz1) {
        const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
        T *m = p.memz + (long long)shot * p.mz_shot_stride + (long long)rr * p.pitch + ix;
        const T m0 = p.b_z[iz] * m[MZ_VZ * p.mz_plane] + p.a_z[iz] * vz_z;
        const T m1 = p.bh_z[iz] * m[MZ_VX * p.mz_plane] + p.ah_z[iz] * vx_z;
        m[MZ_VZ * p.mz_plane] = m0;
        m[MZ_VX * p.mz_plane] = m1;
        vz_z = vz_z * p.ki_z[iz] + m0;
        vx_z = vx_z * p.khi_z[iz] + m1;
    }
    if (ix < p.px0 || ix >= p.px1) {
        const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
        T *m = p.memx + (long long)shot * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
        const T m0 = p.b_x[ix] * m[MX_VX * p.mx_plane] + p.a_x[ix] * vx_x;
        const T m1 = p.bh_x[ix] * m[MX_VZ * p.mx_plane] + p.ah_x[ix] * vz_x;
        m[MX_VX * p.mx_plane] = m0;
        m[MX_VZ * p.mx_plane] = m1;
        vx_x = vx_x * p.ki_x[ix] + m0;
        vz_x = vz_x * p.khi_x[ix] + m1;
    }
}

// cpml_stress with ping-ponged memories (the fused families, FP32): reads
// copy `par`, and the owner of the point writes copy 1 - par (halo points
// only read).
__device__ __forceinline__ void cpml_stress_pp(const StepParams<float> &p, int shot, int iz, int ix,
                                               float &vz_z, float &vx_z, float &vz_x, float &vx_x,
                                               int par, bool own)
{
    static_assert(NMZ == NMX, "second copies at the same plane offset");
    const int ro = par ? NMZ : 0, wo = par ? 0 : NMZ;
    if (iz < p.pz0 || iz >= p.pz1) {
        const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
        float *m = p.memz + (long long)shot * p.mz_shot_stride + (long long)rr * p.pitch + ix;
        const float m0 = p.b_z[iz] * m[(MZ_VZ + ro) * p.mz_plane] + p.a_z[iz] * vz_z;
        const float m1 = p.bh_z[iz] * m[(MZ_VX + ro) * p.mz_plane] + p.ah_z[iz] * vx_z;
        if (own) {
            m[(MZ_VZ + wo) * p.mz_plane] = m0;
            m[(MZ_VX + wo) * p.mz_plane] = m1;
        }
        vz_z = vz_z * p.ki_z[iz] + m0;
        vx_z = vx_z * p.khi_z[iz] + m1;
    }
    if (ix < p.px0 || ix >= p.px1) {
        const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
        float *m = p.memx + (long long)shot * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
        const float m0 = p.b_x[ix] * m[(MX_VX + ro) * p.mx_plane] + p.a_x[ix] * vx_x;
        const float m1 = p.bh_x[ix] * m[(MX_VZ + ro) * p.mx_plane] + p.ah_x[ix] * vz_x;
        if (own) {
            m[(MX_VX + wo) * p.mx_plane] = m0;
            m[(MX_VZ + wo) * p.mx_plane] = m1;
        }
        vx_x = vx_x * p.ki_x[ix] + m0;
        vz_x = vz_x * p.khi_x[ix] + m1;
    }
}

// update_s2 + surf_mirror (src/cpu/n_kernel_lib_PSV.cpp:181-205, 272-395) of
// interior point (iz, ix) from its old stresses o*, the dt-scaled
// coefficients and the (CPML-corrected) derivatives.  The thread that owns
// an image row/column writes the negated new stress into the mirrored cell;
// the mirrored cell's own thread skips those components, so every cell has
// one writer and the result equals the reference's update-then-mirror
// sequence for a top and/or bottom surface, or a left and/or right surface.
template <typename T>
__device__ __forceinline__ void stress_finish(const StepParams<T> &p, T *szz, T *szx, T *sxx,
                                              int iz, int ix, long long i, T ozz, T ozx, T oxx,
                                              T cl, T c2, T cm, T vz_z, T vx_z, T vz_x, T vx_x)
{
    const long long P = p.pitch;
    T nzz = ozz + (c2 * vz_z + cl * vx_x);
    T nxx = oxx + (cl * vz_z + c2 * vx_x);
    T nzx = ozx + cm * (vz_x + vx_z);
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

// pml_diff2 on the stress derivatives of a velocity update.
template <typename T>
__device__ __forceinline__ void cpml_velocity(const StepParams<T> &p, int shot, int iz, int ix,
                                              T &szz_z, T &szx_z, T &szx_x, T &sxx_x)
{
    if (iz < p.pz0 || iz >= p.pz1) {
        const int rr = iz < p.pz0 ? iz : iz - p.pz1 + p.pz0;
        T *m = p.memz + (long long)shot * p.mz_shot_stride + (long long)rr * p.pitch + ix;
        const T m0 = p.b_z[iz] * m[MZ_SZZ * p.mz_plane] + p.a_z[iz] * szz_z;
        const T m1 = p.bh_z[iz] * m[MZ_SZX * p.mz_plane] + p.ah_z[iz] * szx_z;
        m[MZ_SZZ * p.mz_plane] = m0;
        m[MZ_SZX * p.mz_plane] = m1;
        szz_z = szz_z * p.ki_z[iz] + m0;
        szx_z = szx_z * p.khi_z[iz] + m1;
    }
    if (ix < p.px0 || ix >= p.px1) {
        const int c = ix < p.px0 ? ix : ix - p.px1 + p.px0;
        T *m = p.memx + (long long)shot * p.mx_shot_stride + (long long)iz * p.mx_pitch + c;
        const T m0 = p.b_x[ix] * m[MX_SXX * p.mx_plane] + p.a_x[ix] * sxx_x;
        const T m1 = p.bh_x[ix] * m[MX_SZX * p.mx_plane] + p.ah_x[ix] * szx_x;
        m[MX_SXX * p.mx_plane] = m0;
        m[MX_SZX * p.mx_plane] = m1;
        sxx_x = sxx_x * p.ki_x[ix] + m0;
        szx_x = szx_x * p.khi_x[ix] + m1;
    }
}

// The snapshot history (read by the adjoint thousands of launches after
// the forward wrote it) and the shot gradients (revisited every snap_dt
// steps) are touched once per imaging step: streaming (evict-first) loads
// and stores keep their lines from evicting the wavefields, which the next
// launch reads again from L2.
template <typename T>
__device__ __forceinline__ T ld_once(const T *a) { return __ldcs(a); }
template <typename T>
__device__ __forceinline__ void st_once(T *a, T v) { __stcs(a, v); }

// gard_fwd_storage2 (forward: store the step's snapshot into `slot`) or
// fwi_grad2 (adjoint: image against snapshot `slot`, CPU sign) at point
// (iz, ix) of the snapshot window (src/cpu/n_kernel_lib_PSV.cpp:398-484).
template <typename T, int MODE>
__device__ __forceinline__ void snapshot_point(const StepParams<T> &p, int shot, int iz, int ix,
                                               long long i, int slot, T ozz, T ozx, T oxx, T vzn,
                                               T vxn, T uzn, T uxn)
{
    const int dzr = iz - p.snap_z1, dxr = ix - p.snap_x1;
    if (dzr < 0 || iz > p.snap_z2 || dxr < 0 || ix > p.snap_x2) return;
    if (dzr % p.snap_dz || dxr % p.snap_dx) return;
    const long long sp = p.snap_plane;
    const long long qq = (long long)(dzr / p.snap_dz) * p.snx_pitch + dxr / p.snap_dx;
    T *h = p.hist + (long long)shot * p.hist_shot_stride + (long long)slot * p.hist_slot_stride + qq;
    if (MODE != MODE_ADJ) {
        st_once(h + H_SZZ * sp, ozz);
        st_once(h + H_SZX * sp, ozx);
        st_once(h + H_SXX * sp, oxx);
        st_once(h + H_VZ * sp, vzn * p.inv_dt);
        st_once(h + H_VX * sp, vxn * p.inv_dt);
    } else {
        const T fzz = ld_once(h + H_SZZ * sp), fzx = ld_once(h + H_SZX * sp);
        const T fxx = ld_once(h + H_SXX * sp);
        const T fvz = ld_once(h + H_VZ * sp), fvx = ld_once(h + H_VX * sp);
        const T s1 = p.g1[i] * ((fzz + fxx) * (ozz + oxx));
        const T s23 = p.g2[i] * (fzx * ozx + T(0.25) * ((fzz - fxx) * (ozz - oxx)));
        T *g = p.gshot + (long long)shot * p.gshot_shot_stride + qq;
        st_once(g, ld_once(g) - s1);
        st_once(g + sp, ld_once(g + sp) - (s23 + s1));
        st_once(g + 2 * sp, ld_once(g + 2 * sp) - p.kimg * (uxn * fvx + uzn * fvz));
    }
}

// fwi_grad2 of one point split in two: image_preload issues the point's
// history, shot-gradient and imaging-factor loads (they come from HBM) as
// early as the caller wants; image_apply then performs snapshot_point's
// adjoint operations with them.
template <typename T>
struct ImagePre {
    T h[5], g[3], g1, g2;
    long long qq;
    bool in;
};
template <typename T>
__device__ __forceinline__ ImagePre<T> image_preload(const StepParams<T> &p, int bz, int iz, int ix,
                                                     long long i, int slot)
{
    ImagePre<T> e{};
    const int dzr = iz - p.snap_z1, dxr = ix - p.snap_x1;
    e.in = !(dzr < 0 || iz > p.snap_z2 || dxr < 0 || ix > p.snap_x2) && !(dzr % p.snap_dz) &&
           !(dxr % p.snap_dx);
    if (!e.in) return e;
    const long long sp = p.snap_plane;
    e.qq = (long long)(dzr / p.snap_dz) * p.snx_pitch + dxr / p.snap_dx;
    const T *h = p.hist + (long long)bz * p.hist_shot_stride + (long long)slot * p.hist_slot_stride + e.qq;
    const T *g = p.gshot + (long long)bz * p.gshot_shot_stride + e.qq;
    e.h[0] = ld_once(h + H_SZZ * sp); e.h[1] = ld_once(h + H_SZX * sp);
    e.h[2] = ld_once(h + H_SXX * sp);
    e.h[3] = ld_once(h + H_VZ * sp); e.h[4] = ld_once(h + H_VX * sp);
    e.g[0] = ld_once(g); e.g[1] = ld_once(g + sp); e.g[2] = ld_once(g + 2 * sp);
    e.g1 = p.g1[i];
    e.g2 = p.g2[i];
    return e;
}
template <typename T>
__device__ __forceinline__ void image_apply(const StepParams<T> &p, int bz, const ImagePre<T> &e,
                                            T ozz, T ozx, T oxx, T uzn, T uxn)
{
    if (!e.in) return;
    const long long sp = p.snap_plane;
    const T fzz = e.h[0], fzx = e.h[1], fxx = e.h[2], fvz = e.h[3], fvx = e.h[4];
    const T s1 = e.g1 * ((fzz + fxx) * (ozz + oxx));
    const T s23 = e.g2 * (fzx * ozx + T(0.25) * ((fzz - fxx) * (ozz - oxx)));
    T *g = p.gshot + (long long)bz * p.gshot_shot_stride + e.qq;
    st_once(g, e.g[0] - s1);
    st_once(g + sp, e.g[1] - (s23 + s1));
    st_once(g + 2 * sp, e.g[2] - p.kimg * (uxn * fvx + uzn * fvz));
}

// update_v2 (src/cpu/n_kernel_lib_PSV.cpp:243-270) of interior point i from
// its old velocities, plus the displacement integration (adjoint and the
// drop-in forward) and the energy sum We / We_adj from the old u / We
// values; stores and returns the new values.  The new velocities go to the
// planes of `fv` when given (the fused step's write copy), else of f.
template <typename T, int MODE>
__device__ __forceinline__ void velocity_finish(const StepParams<T> &p, T *f, long long i, T vzo,
                                                T vxo, T uzo, T uxo, T weo, T crz, T crx,
                                                T szz_z, T szx_z, T szx_x, T sxx_x, T &vzn,
                                                T &vxn, T &uzn, T &uxn, T *fv = nullptr)
{
    if (MODE == MODE_ADJ || MODE == MODE_FWD_U) {
        uzn = uzo + p.dt * vzo;
        uxn = uxo + p.dt * vxo;
        f[F_UZ * p.plane + i] = uzn;
        f[F_UX * p.plane + i] = uxn;
    }
    vzn = vzo + crz * (szx_x + szz_z);
    vxn = vxo + crx * (sxx_x + szx_z);
    T *vb = fv ? fv : f;
    vb[F_VZ * p.plane + i] = vzn;
    vb[F_VX * p.plane + i] = vxn;
    if (MODE != MODE_FWD_NOWE)
        f[(MODE == MODE_ADJ ? F_WEA : F_WE) * p.plane + i] = weo + (vxn * vxn + vzn * vzn);
}

// Entries of one tile in the per-tile source / receiver index: sources to
// inject [k0, k1) (index into t_src_k or t_rec_r, per src_kind) and
// receivers to record [r0, r1) (empty when the pass records nothing).
struct TileSR {
    int k0, k1, r0, r1;
};
template <typename T>
__device__ __forceinline__ TileSR tile_srcrec(const StepParams<T> &p, const SrcRecParams<T> &q,
                                              int tile, int bz)
{
    TileSR s{0, 0, 0, 0};
    if (q.src_kind == 0) {
        const int *off = q.t_src_off + (long long)(p.ctl[0] + bz) * (q.ntiles + 1);
        s.k0 = off[tile];
        s.k1 = off[tile + 1];
    } else if (q.src_kind == 1) {
        s.k0 = q.t_rec_off[tile];
        s.k1 = q.t_rec_off[tile + 1];
    }
    if (q.rtf_z) {
        s.r0 = q.t_rec_off[tile];
        s.r1 = q.t_rec_off[tile + 1];
    }
    return s;
}

// vsrc2 + urec2 (src/cpu/n_kernel_lib_PSV.cpp:487-576) for the sources and
// receivers of one tile of the velocity kernel, after the tile's velocities
// are written; then the snapshot fix-up of source cells (the stored
// velocity is the post-injection one).  Called by every thread of the block
// with the tile's index entries `e`.
template <typename T, int MODE>
__device__ __forceinline__ void srcrec_apply(const StepParams<T> &p, const SrcRecParams<T> &q,
                                             int it, int slot, int bz, TileSR e, int tid, int nth,
                                             T *fbase = nullptr)
{
    const int k0 = e.k0, k1 = e.k1;
    const bool recs = e.r0 < e.r1;
    if (k0 == k1 && !recs) return;  // uniform over the block
    const int shot = p.ctl[0] + bz;
    T *f = (fbase ? fbase : p.fld) + (long long)bz * p.shot_stride;  // planes holding the new v
    T *vz = f + F_VZ * p.plane;
    T *vx = f + F_VX * p.plane;
    const long long sp = p.snap_plane;
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
        for (int k = e.r0 + tid; k < e.r1; k += nth) {
            const int rr = q.t_rec_r[k];
            const int pos = q.rec_pos[rr];
            const double pz = it ? rz[row - q.nrec + rr] : 0.0;
            const double px = it ? rx[row - q.nrec + rr] : 0.0;
            rz[row + rr] = pz + ((q.dt_d * (double)vz[pos]) / q.dzdx) * ru;
            rx[row + rr] = px + ((q.dt_d * (double)vx[pos]) / q.dzdx) * ru;
        }
    }
    if (slot >= 0 && q.src_kind == 0 && MODE != MODE_ADJ) {  // snapshot holds post-injection v
        T *h = p.hist + (long long)bz * p.hist_shot_stride + (long long)slot * p.hist_slot_stride;
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

// srcrec_apply for tile `tile` of batch shot bz.
template <typename T, int MODE>
__device__ __forceinline__ void srcrec_tile(const StepParams<T> &p, const SrcRecParams<T> &q,
                                            int it, int slot, int tile, int bz, int tid, int nth)
{
    if (q.src_kind < 0 && !q.rtf_z) return;  // uniform: kernel argument
    srcrec_apply<T, MODE>(p, q, it, slot, bz, tile_srcrec(p, q, tile, bz), tid, nth);
}

// Rows [z0, z1) x columns [x0, x1) lie inside the interior, away from the
// CPML strips: the velocity update there is a plain stencil.
template <typename T>
__device__ __forceinline__ bool inner_box(const StepParams<T> &p, int z0, int z1, int x0, int x1)
{
    return z0 >= p.nz1 && z1 <= p.nz2 && x0 >= p.nx1 && x1 <= p.nx2 && p.plane < (1LL << 29);
}

// Rows [z0, z1) x columns [x0, x1) have no CPML memory work.
template <typename T>
__device__ __forceinline__ bool cpml_free_box(const StepParams<T> &p, int z0, int z1, int x0, int x1)
{
    return z0 >= p.pz0 && z1 <= p.pz1 && x0 >= p.px0 && x1 <= p.px1;
}

// Rows [z0, z1) x columns [x0, x1) lie inside the interior (every stencil
// neighbour inside the grid, 32-bit offsets suffice), away from the CPML
// strips: the velocity update there is a plain stencil.
template <typename T>
__device__ __forceinline__ bool plain_box(const StepParams<T> &p, int z0, int z1, int x0, int x1)
{
    return inner_box(p, z0, z1, x0, x1) && cpml_free_box(p, z0, z1, x0, x1);
}

// Interior box the stress update may treat without free-surface work: away
// from every free-surface row and the rows / columns it mirrors (no cell of
// the box is written by another thread's mirror, none of its threads writes
// a mirror).  CPML strips allowed.
template <typename T>
__device__ __forceinline__ bool inner_stress_box(const StepParams<T> &p, int z0, int z1, int x0,
                                                 int x1)
{
    bool ok = inner_box(p, z0, z1, x0, x1);
    if (p.st) ok = ok && z0 > 2 * p.st - p.nz1;
    if (p.sb) ok = ok && z1 - 1 < 2 * p.sb - p.nz2;
    if (p.sl) ok = ok && x0 > 2 * p.sl - p.nx1;
    if (p.sr) ok = ok && x1 - 1 < 2 * p.sr - p.nx2;
    return ok;
}

// ... and without CPML work: the plain stress stencil.
template <typename T>
__device__ __forceinline__ bool plain_stress_box(const StepParams<T> &p, int z0, int z1, int x0,
                                                 int x1)
{
    return inner_stress_box(p, z0, z1, x0, x1) && cpml_free_box(p, z0, z1, x0, x1);
}

// Value of field plane `a` at (iz, ix), zero outside the grid (the values the
// reference's padded arrays hold there).
// CK = false: the caller guarantees (iz, ix) inside the grid (stencil
// neighbours of interior points are), so the load is unchecked.
template <typename T, bool CK = true>
__device__ __forceinline__ T at(const StepParams<T> &p, const T *a, int iz, int ix)
{
    if constexpr (!CK) return a[(long long)iz * p.pitch + ix];
    return (iz >= 0 && iz < p.nz && ix >= 0 && ix < p.nx) ? a[(long long)iz * p.pitch + ix] : T(0);
}

// Whole stress update of interior point (iz, ix) of batch shot bz, the same
// operations as the kernels' unrolled windows.  CK: loads checked against
// the grid (false only where every neighbour is known to be inside).
template <typename T, int NS, bool CK = true>
__device__ __forceinline__ void stress_point(const StepParams<T> &p, int bz, int iz, int ix)
{
    T *f = p.fld + (long long)bz * p.shot_stride;
    const T *vz = f + F_VZ * p.plane, *vx = f + F_VX * p.plane;
    const T oz = at<T, CK>(p, vz, iz, ix), ox = at<T, CK>(p, vx, iz, ix);
    T vz_z = p.cz[0] * (oz - at<T, CK>(p, vz, iz - 1, ix));
    T vx_z = p.cz[0] * (at<T, CK>(p, vx, iz + 1, ix) - ox);
    T vz_x = p.cx[0] * (at<T, CK>(p, vz, iz, ix + 1) - oz);
    T vx_x = p.cx[0] * (ox - at<T, CK>(p, vx, iz, ix - 1));
#pragma unroll
    for (int k = 2; k <= NS; k++) {
        vz_z += p.cz[k - 1] * (at<T, CK>(p, vz, iz + k - 1, ix) - at<T, CK>(p, vz, iz - k, ix));
        vx_z += p.cz[k - 1] * (at<T, CK>(p, vx, iz + k, ix) - at<T, CK>(p, vx, iz - k + 1, ix));
        vz_x += p.cx[k - 1] * (at<T, CK>(p, vz, iz, ix + k) - at<T, CK>(p, vz, iz, ix - (k - 1)));
        vx_x += p.cx[k - 1] * (at<T, CK>(p, vx, iz, ix + k - 1) - at<T, CK>(p, vx, iz, ix - k));
    }
    const long long i = (long long)iz * p.pitch + ix;
    T *szz = f + F_SZZ * p.plane, *szx = f + F_SZX * p.plane, *sxx = f + F_SXX * p.plane;
    cpml_stress(p, bz, iz, ix, vz_z, vx_z, vz_x, vx_x);
    stress_finish(p, szz, szx, sxx, iz, ix, i, szz[i], szx[i], sxx[i], p.c_lam[i], p.c_l2m[i],
                  p.c_muzx[i], vz_z, vx_z, vz_x, vx_x);
}

// Whole velocity step of grid point (iz, ix) with checked loads: update when
// it is interior, then the snapshot store / imaging of `slot`.
template <typename T, int NS, int MODE, bool CK = true>
__device__ __forceinline__ void velocity_point(const StepParams<T> &p, int bz, int iz, int ix,
                                               int slot)
{
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    T *f = p.fld + (long long)bz * p.shot_stride;
    const T *szz = f + F_SZZ * p.plane, *szx = f + F_SZX * p.plane, *sxx = f + F_SXX * p.plane;
    const T ozz = at<T, CK>(p, szz, iz, ix), ozx = at<T, CK>(p, szx, iz, ix), oxx = at<T, CK>(p, sxx, iz, ix);
    const long long i = (long long)iz * p.pitch + ix;
    T vzn = f[F_VZ * p.plane + i], vxn = f[F_VX * p.plane + i];
    T uzn = U ? f[F_UZ * p.plane + i] : T(0), uxn = U ? f[F_UX * p.plane + i] : T(0);
    if (iz >= p.nz1 && iz < p.nz2 && ix >= p.nx1 && ix < p.nx2) {
        T szz_z = p.cz[0] * (at<T, CK>(p, szz, iz + 1, ix) - ozz);
        T szx_z = p.cz[0] * (ozx - at<T, CK>(p, szx, iz - 1, ix));
        T szx_x = p.cx[0] * (ozx - at<T, CK>(p, szx, iz, ix - 1));
        T sxx_x = p.cx[0] * (at<T, CK>(p, sxx, iz, ix + 1) - oxx);
#pragma unroll
        for (int k = 2; k <= NS; k++) {
            szz_z += p.cz[k - 1] * (at<T, CK>(p, szz, iz + k, ix) - at<T, CK>(p, szz, iz - k + 1, ix));
            szx_z += p.cz[k - 1] * (at<T, CK>(p, szx, iz + k - 1, ix) - at<T, CK>(p, szx, iz - k, ix));
            szx_x += p.cx[k - 1] * (at<T, CK>(p, szx, iz, ix + k - 1) - at<T, CK>(p, szx, iz, ix - k));
            sxx_x += p.cx[k - 1] * (at<T, CK>(p, sxx, iz, ix + k) - at<T, CK>(p, sxx, iz, ix - (k - 1)));
        }
        cpml_velocity(p, bz, iz, ix, szz_z, szx_z, szx_x, sxx_x);
        const T weo = MODE != MODE_FWD_NOWE ? f[(MODE == MODE_ADJ ? F_WEA : F_WE) * p.plane + i] : T(0);
        velocity_finish<T, MODE>(p, f, i, vzn, vxn, uzn, uxn, weo, p.c_rz[i], p.c_rx[i], szz_z,
                                 szx_z, szx_x, sxx_x, vzn, vxn, uzn, uxn);
    }
    if (slot >= 0)
        snapshot_point<T, MODE>(p, bz, iz, ix, i, slot, ozz, ozx, oxx, vzn, vxn, uzn, uxn);
}

// Stress update of rows zb .. zb + RPT - 1 of column ix of a block lying in
// the interior, away from the free surfaces and the rows / columns they
// mirror: unchecked loads with 32-bit offsets (stencil neighbours are inside
// the grid).  CPML: the block touches an absorbing strip, and the points in
// it apply pml_diff2 (cpml_stress skips the others).
template <typename T, int NS, int RPT, bool CPML>
__device__ __forceinline__ void stress_rows_inner(const StepParams<T> &p, T *f, int bz, int zb,
                                                  int ix)
{
    const int P = p.pitch, pl = (int)p.plane, i0 = zb * P + ix;
    const T *__restrict__ vzc = f + F_VZ * pl + i0;
    const T *__restrict__ vxc = f + F_VX * pl + i0;
    T *__restrict__ szz = f + F_SZZ * pl;
    constexpr int W = RPT + 2 * NS - 1;
    T wz[W], wx[W];  // wz[j] = vz[zb - N + j], wx[j] = vx[zb - N + 1 + j]
#pragma unroll
    for (int j = 0; j < W; j++) {
        wz[j] = vzc[(j - NS) * P];
        wx[j] = vxc[(j - NS + 1) * P];
    }
#pragma unroll
    for (int r = 0; r < RPT; r++) {
        const T *vzr = vzc + r * P, *vxr = vxc + r * P;
        const T oz = wz[r + NS], ox = wx[r + NS - 1];
        T vz_z = p.cz[0] * (oz - wz[r + NS - 1]);
        T vx_z = p.cz[0] * (wx[r + NS] - ox);
        T vz_x = p.cx[0] * (vzr[1] - oz);
        T vx_x = p.cx[0] * (ox - vxr[-1]);
#pragma unroll
        for (int k = 2; k <= NS; k++) {
            vz_z += p.cz[k - 1] * (wz[r + NS + k - 1] - wz[r + NS - k]);
            vx_z += p.cz[k - 1] * (wx[r + NS + k - 1] - wx[r + NS - k]);
            vz_x += p.cx[k - 1] * (vzr[k] - vzr[-(k - 1)]);
            vx_x += p.cx[k - 1] * (vxr[k - 1] - vxr[-k]);
        }
        if constexpr (CPML) cpml_stress(p, bz, zb + r, ix, vz_z, vx_z, vz_x, vx_x);
        const int i = i0 + r * P;
        const T cl = p.c_lam[i], c2 = p.c_l2m[i], cm = p.c_muzx[i];
        const T ozz = szz[i], ozx = szz[i + pl], oxx = szz[i + 2 * pl];
        szz[i] = ozz + (c2 * vz_z + cl * vx_x);
        szz[i + 2 * pl] = oxx + (cl * vz_z + c2 * vx_x);
        szz[i + pl] = ozx + cm * (vz_x + vx_z);
    }
}

// ---------------------------------------------------------------------------
// Stress step, direct loads: vdiff2 + pml_diff2 + update_s2 + surf_mirror
// (src/cpu/n_kernel_lib_PSV.cpp:100-131, 134-205, 272-395).  Interior points
// only.  stress_block is one block's work (block bp of a grid over the
// interior, 32 x blockDim.y threads); k_stress runs it over one survey's
// batch, k_joint_stress over several surveys (psv_joint.cu).
// ---------------------------------------------------------------------------
template <typename T, int NS, int RPT, bool SH>
__device__ __forceinline__ void stress_block(const StepParams<T> &p, const BlockPos bp)
{
    if (bp.bz >= p.ctl[1]) return;
    const int ix = p.nx1 + bp.bx * 32 + threadIdx.x;
    const int zb = p.nz1 + (bp.by * blockDim.y + threadIdx.y) * RPT;
    if (zb >= p.nz2) return;  // uniform across the warp; no block barrier follows
    T *f = p.fld + (long long)bp.bz * p.shot_stride;
    {
        const int bz0 = p.nz1 + bp.by * blockDim.y * RPT, bx0 = p.nx1 + bp.bx * 32;
        const int bz1 = bz0 + (int)blockDim.y * RPT, bx1 = bx0 + 32;
        if (plain_stress_box(p, bz0, bz1, bx0, bx1)) {
            // no bounds, CPML or surface work: 32-bit offsets, unpredicated loads
            stress_rows_inner<T, NS, RPT, false>(p, f, bp.bz, zb, ix);
            return;
        }
        if (inner_stress_box(p, bz0, bz1, bx0, bx1)) {  // CPML strip, no bounds or surface work
            stress_rows_inner<T, NS, RPT, true>(p, f, bp.bz, zb, ix);
            return;
        }
    }
    const long long P = p.pitch;
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
        cpml_stress(p, bp.bz, iz, ix, vz_z, vx_z, vz_x, vx_x);
        stress_finish(p, szz, szx, sxx, iz, ix, i, szz[i], szx[i], sxx[i], p.c_lam[i], p.c_l2m[i],
                      p.c_muzx[i], vz_z, vx_z, vz_x, vx_x);
    }
}

template <typename T, int NS, int RPT, bool SH>
__global__ void __launch_bounds__(256) k_stress(const StepParams<T> p)
{
    stress_block<T, NS, RPT, SH>(p, block_pos(p.nbatch));
}

// Velocity update (with the step's snapshot store / imaging) of rows
// zb .. zb + RPT - 1 of column ix of a block lying in the interior:
// unchecked loads with 32-bit offsets, imaging loads issued first.  CPML:
// the block touches an absorbing strip, and the points in it apply
// pml_diff2 (cpml_velocity skips the others).
template <typename T, int NS, int MODE, int RPT, bool CPML>
__device__ __forceinline__ void velocity_rows_inner(const StepParams<T> &p, T *f, int bz, int zb,
                                                    int ix, int slot)
{
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    const int P = p.pitch, pl = (int)p.plane, i0 = zb * P + ix;
    const T *__restrict__ zzc = f + F_SZZ * pl + i0;
    const T *__restrict__ zxc = f + F_SZX * pl + i0;
    const T *__restrict__ xxc = f + F_SXX * pl + i0;
    constexpr int W = RPT + 2 * NS - 1;
    const bool image = MODE == MODE_ADJ && slot >= 0;
    ImagePre<T> pre[RPT];  // imaging loads first: their latency overlaps the stencil loads
#pragma unroll
    for (int r = 0; r < RPT; r++)
        if (image) pre[r] = image_preload(p, bz, zb + r, ix, i0 + r * P, slot);
    T wzz[W], wzx[W];  // wzz[j] = szz[zb - N + 1 + j], wzx[j] = szx[zb - N + j]
#pragma unroll
    for (int j = 0; j < W; j++) {
        wzz[j] = zzc[(j - NS + 1) * P];
        wzx[j] = zxc[(j - NS) * P];
    }
#pragma unroll
    for (int r = 0; r < RPT; r++) {
        const T *zxr = zxc + r * P, *xxr = xxc + r * P;
        const T ozz = wzz[r + NS - 1], ozx = wzx[r + NS], oxx = xxr[0];
        T szz_z = p.cz[0] * (wzz[r + NS] - ozz);
        T szx_z = p.cz[0] * (ozx - wzx[r + NS - 1]);
        T szx_x = p.cx[0] * (ozx - zxr[-1]);
        T sxx_x = p.cx[0] * (xxr[1] - oxx);
#pragma unroll
        for (int k = 2; k <= NS; k++) {
            szz_z += p.cz[k - 1] * (wzz[r + NS + k - 1] - wzz[r + NS - k]);
            szx_z += p.cz[k - 1] * (wzx[r + NS + k - 1] - wzx[r + NS - k]);
            szx_x += p.cx[k - 1] * (zxr[k - 1] - zxr[-k]);
            sxx_x += p.cx[k - 1] * (xxr[k] - xxr[-(k - 1)]);
        }
        if constexpr (CPML) cpml_velocity(p, bz, zb + r, ix, szz_z, szx_z, szx_x, sxx_x);
        const int i = i0 + r * P;
        const T uzo = U ? f[F_UZ * pl + i] : T(0), uxo = U ? f[F_UX * pl + i] : T(0);
        const T weo = MODE != MODE_FWD_NOWE ? f[(MODE == MODE_ADJ ? F_WEA : F_WE) * pl + i] : T(0);
        T vzn, vxn, uzn = T(0), uxn = T(0);
        velocity_finish<T, MODE>(p, f, i, f[F_VZ * pl + i], f[F_VX * pl + i], uzo, uxo, weo,
                                 p.c_rz[i], p.c_rx[i], szz_z, szx_z, szx_x, sxx_x, vzn, vxn,
                                 uzn, uxn);
        if (image)
            image_apply(p, bz, pre[r], ozz, ozx, oxx, uzn, uxn);
        else if (slot >= 0)
            snapshot_point<T, MODE>(p, bz, zb + r, ix, i, slot, ozz, ozx, oxx,
                                    vzn, vxn, uzn, uxn);
    }
}

// ---------------------------------------------------------------------------
// Velocity step, direct loads: sdiff2 + pml_diff2 + update_v2
// (src/cpu/n_kernel_lib_PSV.cpp:207-270, 134-178), fused with the step's
// remaining work:
//   forward modes: gard_fwd_storage2 (:398-436) into `slot`;
//   MODE_ADJ: u += dt v, and fwi_grad2 (:439-484, CPU sign) against `slot`;
//   epilogue: vsrc2 + urec2 (:487-576) for the sources / receivers of the
//   block's tile, after all of the tile's velocities are written.
// Covers the whole grid: cells outside the interior only take part in the
// snapshot / imaging work (their fields are never updated).  velocity_block
// is one block's work (block bp of a grid over the whole nz x nx plane);
// k_velocity runs it over one survey's batch, k_joint_velocity over several
// surveys (psv_joint.cu).
// ---------------------------------------------------------------------------
template <typename T, int NS, int MODE, int RPT, bool SH>
__device__ __forceinline__ void velocity_block(const StepParams<T> &p, const SrcRecParams<T> &q,
                                               const int it, const int slot, const BlockPos bp)
{
    if (bp.bz >= p.ctl[1]) return;  // whole block
    const int ix = bp.bx * 32 + threadIdx.x;
    const int zb = (bp.by * blockDim.y + threadIdx.y) * RPT;
    const long long P = p.pitch;
    T *f = p.fld + (long long)bp.bz * p.shot_stride;
    const T *__restrict__ szz = f + F_SZZ * p.plane;
    const T *__restrict__ szx = f + F_SZX * p.plane;
    const T *__restrict__ sxx = f + F_SXX * p.plane;
    const bool colok = ix < p.nx;
    const bool colin = ix >= p.nx1 && ix < p.nx2;
    const int bz0 = bp.by * blockDim.y * RPT, bx0 = bp.bx * 32;
    const bool plain = plain_box(p, bz0, bz0 + (int)blockDim.y * RPT, bx0, bx0 + 32);

    if (plain) {  // interior, no CPML: 32-bit offsets, unpredicated loads
        velocity_rows_inner<T, NS, MODE, RPT, false>(p, f, bp.bz, zb, ix, slot);
    } else if (inner_box(p, bz0, bz0 + (int)blockDim.y * RPT, bx0, bx0 + 32)) {  // + CPML
        velocity_rows_inner<T, NS, MODE, RPT, true>(p, f, bp.bz, zb, ix, slot);
    } else if (zb < p.nz) {  // warp-uniform
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
                cpml_velocity(p, bp.bz, iz, ix, szz_z, szx_z, szx_x, sxx_x);
                constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
                const T uzo = U ? f[F_UZ * p.plane + i] : T(0);
                const T uxo = U ? f[F_UX * p.plane + i] : T(0);
                const T weo = MODE != MODE_FWD_NOWE
                                  ? f[(MODE == MODE_ADJ ? F_WEA : F_WE) * p.plane + i]
                                  : T(0);
                velocity_finish<T, MODE>(p, f, i, f[F_VZ * p.plane + i], f[F_VX * p.plane + i],
                                         uzo, uxo, weo, p.c_rz[i], p.c_rx[i], szz_z, szx_z, szx_x,
                                         sxx_x, vzn, vxn, uzn, uxn);
            } else {
                vzn = f[F_VZ * p.plane + i];
                vxn = f[F_VX * p.plane + i];
                if (MODE == MODE_ADJ || MODE == MODE_FWD_U) {
                    uzn = f[F_UZ * p.plane + i];
                    uxn = f[F_UX * p.plane + i];
                }
            }
            if (slot >= 0)
                snapshot_point<T, MODE>(p, bp.bz, iz, ix, i, slot, ozz, ozx, oxx, vzn,
                                        vxn, uzn, uxn);
        }
    }
    srcrec_tile<T, MODE>(p, q, it, slot, bp.by * bp.ntx + bp.bx, bp.bz,
                         threadIdx.y * 32 + threadIdx.x, 32 * blockDim.y);
}

template <typename T, int NS, int MODE, int RPT, bool SH>
__global__ void __launch_bounds__(256) k_velocity(const StepParams<T> p, const SrcRecParams<T> q,
                                                  const int it, const int slot)
{
    velocity_block<T, NS, MODE, RPT, SH>(p, q, it, slot, block_pos(p.nbatch));
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
