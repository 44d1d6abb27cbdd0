// psv_vec.cu -- FP32 time-step kernels with four columns per thread.
//
// A block is 32 x BY threads and covers 128 columns x BY R rows of one shot
// (origin on a multiple of 128 columns, so every thread's columns
// x .. x + 3 form one 16-byte aligned float4 of each row: the row pitch is a
// multiple of 32 floats).  Inside the CPML-free interior, away from free
// surfaces, a thread
//   - keeps the vertical stencil window of its four columns in float4
//     registers (R + 2 NS - 1 rows per differentiated field),
//   - takes the horizontal neighbours from the float4 quads left and right
//     of its own,
//   - reads and writes its own values and coefficients as float4,
// so one 128-bit load serves four grid points and the per-thread set-up is
// shared by 4 R points.  Threads in the CPML strips run the per-point code
// of psv_kernels_impl.cuh with unchecked loads (every neighbour of an
// interior point lies inside the grid); only threads whose points touch the
// grid frame or a free surface check each load.
// Both paths perform the same floating-point operations as the direct
// kernels for every point.
#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"

namespace psv {

namespace {

constexpr int VW = 128;  // block columns

__device__ __forceinline__ float4 ld4(const float *a) { return *reinterpret_cast<const float4 *>(a); }
__device__ __forceinline__ void st4(float *a, float4 v) { *reinterpret_cast<float4 *>(a) = v; }
__device__ __forceinline__ float c4(const float4 &v, int c)
{
    return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}

// Columns x - 4 .. x + 7 of one row as L | C | R quads; q(c) for c in
// [-4, 8) (compile-time after unrolling).
struct Row12 {
    float4 l, c, r;
    __device__ __forceinline__ float q(int k) const
    {
        return k < 0 ? c4(l, k + 4) : k < 4 ? c4(c, k) : c4(r, k - 4);
    }
};

}  // namespace

// ---------------------------------------------------------------------------
// Stress step: vdiff2 + pml_diff2 + update_s2 + surf_mirror
// (src/cpu/n_kernel_lib_PSV.cpp:100-205, 272-395).
// ---------------------------------------------------------------------------
template <int NS, int R>
__global__ void __launch_bounds__(256) k_stress_v4(const StepParams<float> p)
{
    const BlockPos bp = block_pos(p.nbatch);
    const int bz = bp.bz;
    if (bz >= p.ctl[1]) return;
    const int BY = blockDim.y;
    const int x0 = bp.bx * VW, zb0 = bp.by * BY * R;
    const int x = x0 + 4 * threadIdx.x, zb = zb0 + threadIdx.y * R;
    float *f = p.fld + (long long)bz * p.shot_stride;
    // per thread: the threads whose 4 x R points touch the frame or a free
    // surface take the checked path, CPML-strip threads the unchecked one
    if (!inner_stress_box(p, zb, zb + R, x, x + 4)) {
#pragma unroll 1
        for (int r = 0; r < R; r++) {
            const int iz = zb + r;
            if (iz < p.nz1 || iz >= p.nz2) continue;
#pragma unroll 1
            for (int c = 0; c < 4; c++)
                if (x + c >= p.nx1 && x + c < p.nx2) stress_point<float, NS>(p, bz, iz, x + c);
        }
        return;
    }
    if (!cpml_free_box(p, zb, zb + R, x, x + 4)) {  // CPML strips: unchecked point path
#pragma unroll 1
        for (int r = 0; r < R; r++)
#pragma unroll 1
            for (int c = 0; c < 4; c++) stress_point<float, NS, false>(p, bz, zb + r, x + c);
        return;
    }
    const int P = p.pitch, pl = (int)p.plane;
    const float *vz = f + F_VZ * pl, *vx = f + F_VX * pl;
    float *sg = f + F_SZZ * pl;  // szz; szx at + pl, sxx at + 2 pl
    constexpr int W = R + 2 * NS - 1;
    float4 wz[W], wx[W];  // wz[j] = vz[zb - N + j], wx[j] = vx[zb - N + 1 + j] (columns x..x+3)
#pragma unroll
    for (int j = 0; j < W; j++) {
        wz[j] = ld4(vz + (zb - NS + j) * P + x);
        wx[j] = ld4(vx + (zb - NS + 1 + j) * P + x);
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int i = (zb + r) * P + x;
        Row12 az, ax;  // vz needs columns -(N-1) .. +N, vx -N .. +N-1
        az.c = wz[r + NS];
        az.l = NS >= 2 ? ld4(vz + i - 4) : make_float4(0.f, 0.f, 0.f, 0.f);
        az.r = ld4(vz + i + 4);
        ax.c = wx[r + NS - 1];
        ax.l = ld4(vx + i - 4);
        ax.r = NS >= 2 ? ld4(vx + i + 4) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 ozz = ld4(sg + i), ozx = ld4(sg + pl + i), oxx = ld4(sg + 2 * pl + i);
        const float4 cl = ld4(p.c_lam + i), c2 = ld4(p.c_l2m + i), cm = ld4(p.c_muzx + i);
        float nzz[4], nzx[4], nxx[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const float oz = az.q(c), ox = ax.q(c);
            float vz_z = p.cz[0] * (oz - c4(wz[r + NS - 1], c));
            float vx_z = p.cz[0] * (c4(wx[r + NS], c) - ox);
            float vz_x = p.cx[0] * (az.q(c + 1) - oz);
            float vx_x = p.cx[0] * (ox - ax.q(c - 1));
#pragma unroll
            for (int k = 2; k <= NS; k++) {
                vz_z += p.cz[k - 1] * (c4(wz[r + NS + k - 1], c) - c4(wz[r + NS - k], c));
                vx_z += p.cz[k - 1] * (c4(wx[r + NS + k - 1], c) - c4(wx[r + NS - k], c));
                vz_x += p.cx[k - 1] * (az.q(c + k) - az.q(c - (k - 1)));
                vx_x += p.cx[k - 1] * (ax.q(c + k - 1) - ax.q(c - k));
            }
            nzz[c] = c4(ozz, c) + (c4(c2, c) * vz_z + c4(cl, c) * vx_x);
            nxx[c] = c4(oxx, c) + (c4(cl, c) * vz_z + c4(c2, c) * vx_x);
            nzx[c] = c4(ozx, c) + c4(cm, c) * (vz_x + vx_z);
        }
        st4(sg + i, make_float4(nzz[0], nzz[1], nzz[2], nzz[3]));
        st4(sg + pl + i, make_float4(nzx[0], nzx[1], nzx[2], nzx[3]));
        st4(sg + 2 * pl + i, make_float4(nxx[0], nxx[1], nxx[2], nxx[3]));
    }
}

// ---------------------------------------------------------------------------
// Velocity step: sdiff2 + pml_diff2 + update_v2, snapshot store / imaging,
// then vsrc2 + urec2 for the block's tile (src/cpu/n_kernel_lib_PSV.cpp:
// 207-270, 398-576).  Covers the whole grid.
// ---------------------------------------------------------------------------
template <int NS, int MODE, int R>
__global__ void __launch_bounds__(256) k_velocity_v4(const StepParams<float> p,
                                                     const SrcRecParams<float> q, const int it,
                                                     const int slot)
{
    const BlockPos bp = block_pos(p.nbatch);
    const int bz = bp.bz;
    if (bz >= p.ctl[1]) return;  // whole block
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    constexpr bool WE = MODE != MODE_FWD_NOWE;
    const int BY = blockDim.y;
    const int x0 = bp.bx * VW, zb0 = bp.by * BY * R;
    const int x = x0 + 4 * threadIdx.x, zb = zb0 + threadIdx.y * R;
    float *f = p.fld + (long long)bz * p.shot_stride;
    if (!inner_box(p, zb, zb + R, x, x + 4)) {  // per thread, as in the stress step
#pragma unroll 1
        for (int r = 0; r < R; r++) {
            const int iz = zb + r;
            if (iz >= p.nz) continue;
#pragma unroll 1
            for (int c = 0; c < 4; c++)
                if (x + c < p.nx) velocity_point<float, NS, MODE>(p, bz, iz, x + c, slot);
        }
    } else if (!cpml_free_box(p, zb, zb + R, x, x + 4)) {  // CPML strips: unchecked points
#pragma unroll 1
        for (int r = 0; r < R; r++)
#pragma unroll 1
            for (int c = 0; c < 4; c++)
                velocity_point<float, NS, MODE, false>(p, bz, zb + r, x + c, slot);
    } else {
        const int P = p.pitch, pl = (int)p.plane;
        const float *szz = f + F_SZZ * pl, *szx = f + F_SZX * pl, *sxx = f + F_SXX * pl;
        constexpr int W = R + 2 * NS - 1;
        float4 wzz[W], wzx[W];  // wzz[j] = szz[zb - N + 1 + j], wzx[j] = szx[zb - N + j]
#pragma unroll
        for (int j = 0; j < W; j++) {
            wzz[j] = ld4(szz + (zb - NS + 1 + j) * P + x);
            wzx[j] = ld4(szx + (zb - NS + j) * P + x);
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = (zb + r) * P + x;
            Row12 bx, cx;  // szx needs columns -N .. +N-1, sxx -(N-1) .. +N
            bx.c = wzx[r + NS];
            bx.l = ld4(szx + i - 4);
            bx.r = NS >= 2 ? ld4(szx + i + 4) : make_float4(0.f, 0.f, 0.f, 0.f);
            cx.c = ld4(sxx + i);
            cx.l = NS >= 2 ? ld4(sxx + i - 4) : make_float4(0.f, 0.f, 0.f, 0.f);
            cx.r = ld4(sxx + i + 4);
            const float4 vzo = ld4(f + F_VZ * pl + i), vxo = ld4(f + F_VX * pl + i);
            const float4 crz = ld4(p.c_rz + i), crx = ld4(p.c_rx + i);
            const float4 uzo = U ? ld4(f + F_UZ * pl + i) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 uxo = U ? ld4(f + F_UX * pl + i) : make_float4(0.f, 0.f, 0.f, 0.f);
            float *wep = f + (MODE == MODE_ADJ ? F_WEA : F_WE) * pl + i;
            const float4 weo = WE ? ld4(wep) : make_float4(0.f, 0.f, 0.f, 0.f);
            float vzn[4], vxn[4], uzn[4], uxn[4], wen[4], ozz[4], ozx[4], oxx[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                ozz[c] = c4(wzz[r + NS - 1], c);
                ozx[c] = bx.q(c);
                oxx[c] = cx.q(c);
                float szz_z = p.cz[0] * (c4(wzz[r + NS], c) - ozz[c]);
                float szx_z = p.cz[0] * (ozx[c] - c4(wzx[r + NS - 1], c));
                float szx_x = p.cx[0] * (ozx[c] - bx.q(c - 1));
                float sxx_x = p.cx[0] * (cx.q(c + 1) - oxx[c]);
#pragma unroll
                for (int k = 2; k <= NS; k++) {
                    szz_z += p.cz[k - 1] * (c4(wzz[r + NS + k - 1], c) - c4(wzz[r + NS - k], c));
                    szx_z += p.cz[k - 1] * (c4(wzx[r + NS + k - 1], c) - c4(wzx[r + NS - k], c));
                    szx_x += p.cx[k - 1] * (bx.q(c + k - 1) - bx.q(c - k));
                    sxx_x += p.cx[k - 1] * (cx.q(c + k) - cx.q(c - (k - 1)));
                }
                // update_v2 (+ u, We) as in velocity_finish
                uzn[c] = U ? c4(uzo, c) + p.dt * c4(vzo, c) : 0.f;
                uxn[c] = U ? c4(uxo, c) + p.dt * c4(vxo, c) : 0.f;
                vzn[c] = c4(vzo, c) + c4(crz, c) * (szx_x + szz_z);
                vxn[c] = c4(vxo, c) + c4(crx, c) * (sxx_x + szx_z);
                wen[c] = c4(weo, c) + (vxn[c] * vxn[c] + vzn[c] * vzn[c]);
            }
            if (U) {
                st4(f + F_UZ * pl + i, make_float4(uzn[0], uzn[1], uzn[2], uzn[3]));
                st4(f + F_UX * pl + i, make_float4(uxn[0], uxn[1], uxn[2], uxn[3]));
            }
            st4(f + F_VZ * pl + i, make_float4(vzn[0], vzn[1], vzn[2], vzn[3]));
            st4(f + F_VX * pl + i, make_float4(vxn[0], vxn[1], vxn[2], vxn[3]));
            if (WE) st4(wep, make_float4(wen[0], wen[1], wen[2], wen[3]));
            if (slot >= 0)
#pragma unroll
                for (int c = 0; c < 4; c++)
                    snapshot_point<float, MODE>(p, bz, zb + r, x + c, i + c, slot, ozz[c], ozx[c],
                                                oxx[c], vzn[c], vxn[c], uzn[c], uxn[c]);
        }
    }
    srcrec_tile<float, MODE>(p, q, it, slot, bp.by * bp.ntx + bp.bx, bz,
                             threadIdx.y * 32 + threadIdx.x, 32 * BY);
}

// ---------------------------------------------------------------------------
// Launchers: rpt in {1, 2, 4} rows per thread, block 32 x by.
// ---------------------------------------------------------------------------
namespace {

template <int NS, int R>
cudaError_t stress_v4_rn(const StepParams<float> &p, int by, int nbatch, cudaStream_t st)
{
    dim3 grid((p.nx + VW - 1) / VW, (p.nz + by * R - 1) / (by * R), nbatch);
    k_stress_v4<NS, R><<<grid, dim3(32, by), 0, st>>>(p);
    return cudaGetLastError();
}

template <int NS>
cudaError_t stress_v4_n(const StepParams<float> &p, int rpt, int by, int nbatch, cudaStream_t st)
{
    switch (rpt) {
    case 1: return stress_v4_rn<NS, 1>(p, by, nbatch, st);
    case 2: return stress_v4_rn<NS, 2>(p, by, nbatch, st);
    case 4: return stress_v4_rn<NS, 4>(p, by, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int NS, int MODE, int R>
cudaError_t velocity_v4_rmn(const StepParams<float> &p, const SrcRecParams<float> &q, int it,
                            int slot, int by, int nbatch, cudaStream_t st)
{
    dim3 grid((p.nx + VW - 1) / VW, (p.nz + by * R - 1) / (by * R), nbatch);
    k_velocity_v4<NS, MODE, R><<<grid, dim3(32, by), 0, st>>>(p, q, it, slot);
    return cudaGetLastError();
}

template <int NS, int MODE>
cudaError_t velocity_v4_mn(const StepParams<float> &p, const SrcRecParams<float> &q, int it,
                           int slot, int rpt, int by, int nbatch, cudaStream_t st)
{
    switch (rpt) {
    case 1: return velocity_v4_rmn<NS, MODE, 1>(p, q, it, slot, by, nbatch, st);
    case 2: return velocity_v4_rmn<NS, MODE, 2>(p, q, it, slot, by, nbatch, st);
    case 4: return velocity_v4_rmn<NS, MODE, 4>(p, q, it, slot, by, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int NS>
cudaError_t velocity_v4_n(const StepParams<float> &p, const SrcRecParams<float> &q, int mode,
                          int it, int slot, int rpt, int by, int nbatch, cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: return velocity_v4_mn<NS, MODE_FWD>(p, q, it, slot, rpt, by, nbatch, st);
    case MODE_FWD_NOWE: return velocity_v4_mn<NS, MODE_FWD_NOWE>(p, q, it, slot, rpt, by, nbatch, st);
    case MODE_FWD_U: return velocity_v4_mn<NS, MODE_FWD_U>(p, q, it, slot, rpt, by, nbatch, st);
    case MODE_ADJ: return velocity_v4_mn<NS, MODE_ADJ>(p, q, it, slot, rpt, by, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_stress_v4(const StepParams<float> &p, int ns, int rpt, int by, int nbatch,
                             cudaStream_t st)
{
    if (by < 1 || by > 8 || p.pitch % 4) return cudaErrorInvalidValue;
    switch (ns) {
    case 1: return stress_v4_n<1>(p, rpt, by, nbatch, st);
    case 2: return stress_v4_n<2>(p, rpt, by, nbatch, st);
    case 3: return stress_v4_n<3>(p, rpt, by, nbatch, st);
    case 4: return stress_v4_n<4>(p, rpt, by, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_velocity_v4(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                               int mode, int it, int slot, int rpt, int by, int nbatch,
                               cudaStream_t st)
{
    if (by < 1 || by > 8 || p.pitch % 4) return cudaErrorInvalidValue;
    switch (ns) {
    case 1: return velocity_v4_n<1>(p, q, mode, it, slot, rpt, by, nbatch, st);
    case 2: return velocity_v4_n<2>(p, q, mode, it, slot, rpt, by, nbatch, st);
    case 3: return velocity_v4_n<3>(p, q, mode, it, slot, rpt, by, nbatch, st);
    case 4: return velocity_v4_n<4>(p, q, mode, it, slot, rpt, by, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace psv
