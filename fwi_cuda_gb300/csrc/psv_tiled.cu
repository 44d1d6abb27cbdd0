// psv_tiled.cu -- FP32 time-step kernels that stream tiles through shared
// memory with TMA tensor copies, software-pipelined.
//
// Tiles are TW = 64 columns x TZ = 4 R rows of one shot.  A launch is
// persistent: each CTA walks the tiles t = blockIdx.x, + gridDim.x, ... and
// keeps S = 2 stages in flight, so the copies of its next tile overlap the
// arithmetic of the current one.  A stage holds, as one
// cp.async.bulk.tensor box each,
//   - the fields the step differentiates (v for the stress step, sigma for
//     the velocity step): TZ + 2 NS rows x 72 columns from (z0 - NS, x0 - 4).
//     x0 is a multiple of 64, so the box's first column sits on a 16-byte
//     boundary; the tensor map's zero fill supplies cells outside the grid,
//     the values the direct kernels substitute;
//   - the tile's own old values and dt-scaled coefficients (64 x TZ boxes).
// Its mbarrier completes on the boxes' transaction bytes.  The 256 threads
// are 8 warps: warp w covers columns (w & 1) * 32 + lane and rows
// (w >> 1) * R .. + R - 1, holding each column's vertical stencil window in
// registers.  Tiles inside the CPML-free interior and away from free
// surfaces ("plain" tiles) take a branch-free update; the others use the
// per-point code shared with the direct kernels (psv_kernels_impl.cuh).
//
// Every wait on a copy is bounded: after ~1 s without completion the block
// records error code 1 in StepParams::err and returns; the host turns that
// into PSV_ERR_CUDA.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"
#include "psv_tma.cuh"

namespace psv {

namespace {

constexpr int TW = 64;             // tile columns
constexpr int HX = 4;              // columns staged left and right of the tile
constexpr int SW = TW + 2 * HX;    // staged row length (floats)
constexpr int NTHREADS = 256;
constexpr int NSTAGE = 2;          // tiles in flight per CTA

__host__ __device__ constexpr int halo_rows(int ns, int r) { return 4 * r + 2 * ns; }
__host__ __device__ constexpr int halo_plane(int ns, int r) { return (halo_rows(ns, r) * SW + 31) / 32 * 32; }
__host__ __device__ constexpr int own_plane(int r) { return TW * 4 * r; }

// Floats of one stage: nh halo planes and no own planes.
__host__ __device__ constexpr int stage_floats(int nh, int no, int ns, int r)
{
    return nh * halo_plane(ns, r) + no * own_plane(r);
}

// Dynamic shared memory of a launch: NSTAGE stages, 128-byte aligned (TMA
// destination rule), then one mbarrier and one 32-byte tile record per stage.
__host__ __device__ constexpr int pipe_smem_bytes(int nh, int no, int ns, int r)
{
    return NSTAGE * stage_floats(nh, no, ns, r) * 4 + 128 + (8 + 32) * NSTAGE;
}

// Own planes the velocity step stages, per mode (after vz vx crz crx): We or
// We_adj, then uz ux for the displacement modes, then g1 g2 when it images.
template <int MODE> __host__ __device__ constexpr int vel_own_planes(bool image)
{
    return 4 + (MODE != MODE_FWD_NOWE ? 1 : 0) + (MODE == MODE_ADJ || MODE == MODE_FWD_U ? 2 : 0) +
           (MODE == MODE_ADJ && image ? 2 : 0);
}

// All threads wait (bounded) for stage barrier `bar` to complete phase
// `parity`; true in every thread iff all of them saw it.  On a timeout the
// block records error code 1 for the host.
__device__ __forceinline__ bool wait_stage(uint32_t bar, uint32_t parity, int *err)
{
    const bool ok = mbar_wait(bar, parity);
    const bool all = __syncthreads_and(ok) != 0;
    if (!all && threadIdx.x == 0) atomicExch(err, 1);
    return all;
}

// Coefficient planes of StepParams::c_lam .. g2 in the coefficient tensor.
enum { C_LAM = 0, C_L2M, C_MUZX, C_RZ, C_RX, C_G1, C_G2 };

// Tile t of a launch: shot bz of the batch, origin (z0, x0), whether it is a
// plain tile, and its source / receiver index entries.  The shot varies
// fastest (t = spatial tile * nvalid + shot), so the tiles of one place for
// all shots are processed together and share its coefficients through L2.
// Thread 0 fills the record when it issues the tile's copies; the others
// read it from shared memory after the stage barrier (one set of integer
// divisions and index loads per tile, not per thread).
struct Tile {
    int bz, z0, x0, plain;
    TileSR sr;
};
static_assert(sizeof(Tile) == 32, "tile record size");
__device__ __forceinline__ Tile tile_of(int t, int ntx, int nvalid, int tz)
{
    const int r = t / nvalid;
    return {t % nvalid, (r / ntx) * tz, (r % ntx) * TW, 0, {0, 0, 0, 0}};
}

// ------------------------------------------------------------------ stress
template <int NS, int R>
__device__ __forceinline__ void stress_issue(const TileMaps &m, float *st, uint32_t b, const Tile &T,
                                             int pps)
{
    constexpr int HP = halo_plane(NS, R), OP = own_plane(R), HR = halo_rows(NS, R);
    float *own = st + 2 * HP;
    const int pb = T.bz * pps, x0 = T.x0, z0 = T.z0;
    mbar_expect_tx(b, (uint32_t)(2 * HR * SW * 4 + 6 * OP * 4));
    tma_load(smem_u32(st), &m.halo, x0 - HX, z0 - NS, pb + F_VZ, b);
    tma_load(smem_u32(st + HP), &m.halo, x0 - HX, z0 - NS, pb + F_VX, b);
    tma_load(smem_u32(own), &m.own, x0, z0, pb + F_SZZ, b);
    tma_load(smem_u32(own + OP), &m.own, x0, z0, pb + F_SZX, b);
    tma_load(smem_u32(own + 2 * OP), &m.own, x0, z0, pb + F_SXX, b);
    tma_load(smem_u32(own + 3 * OP), &m.coef, x0, z0, C_LAM, b);
    tma_load(smem_u32(own + 4 * OP), &m.coef, x0, z0, C_L2M, b);
    tma_load(smem_u32(own + 5 * OP), &m.coef, x0, z0, C_MUZX, b);
}

// vdiff2 + pml_diff2 + update_s2 + surf_mirror (src/cpu/n_kernel_lib_PSV.cpp:
// 100-205, 272-395) of one staged tile: halo'd vz, vx; the tile's szz, szx,
// sxx and dt*lam, dt*(lam+2mu), dt*mu_zx.
template <int NS, int R>
__device__ __forceinline__ void stress_tile(const StepParams<float> &p, const float *st,
                                            const Tile &T)
{
    constexpr int HP = halo_plane(NS, R), OP = own_plane(R);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lc = (w & 1) * 32 + lane, lr0 = (w >> 1) * R;
    const int x0 = T.x0, z0 = T.z0, ix = x0 + lc;
    const bool plain = T.plain;  // interior, no CPML, no free-surface row or mirror image

    // derivatives of the thread's R rows, from shared memory only
    float dzz[R], dzx[R], dxz[R], dxx[R];  // vz_z, vz_x, vx_z, vx_x
    {
        constexpr int W = R + 2 * NS - 1;
        const float *cz = st + lr0 * SW + HX + lc;  // staged row lr0 = tile row lr0 - NS
        float wz[W], wx[W];  // wz[j] = vz[row lr0 - NS + j], wx[j] = vx[row lr0 - NS + 1 + j]
#pragma unroll
        for (int j = 0; j < W; j++) {
            wz[j] = cz[j * SW];
            wx[j] = cz[HP + (j + 1) * SW];
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const float *az = cz + (r + NS) * SW, *ax = az + HP;
            const float oz = wz[r + NS], ox = wx[r + NS - 1];
            float vz_z = p.cz[0] * (oz - wz[r + NS - 1]);
            float vx_z = p.cz[0] * (wx[r + NS] - ox);
            float vz_x = p.cx[0] * (az[1] - oz);
            float vx_x = p.cx[0] * (ox - ax[-1]);
#pragma unroll
            for (int k = 2; k <= NS; k++) {
                vz_z += p.cz[k - 1] * (wz[r + NS + k - 1] - wz[r + NS - k]);
                vx_z += p.cz[k - 1] * (wx[r + NS + k - 1] - wx[r + NS - k]);
                vz_x += p.cx[k - 1] * (az[k] - az[-(k - 1)]);
                vx_x += p.cx[k - 1] * (ax[k - 1] - ax[-k]);
            }
            dzz[r] = vz_z; dzx[r] = vz_x; dxz[r] = vx_z; dxx[r] = vx_x;
        }
    }
    const float *o = st + 2 * HP + lr0 * TW + lc;
    float *f = p.fld + (long long)T.bz * p.shot_stride;
    if (plain) {
        const int P = p.pitch, pl = (int)p.plane;
        float *szz = f + F_SZZ * p.plane;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = (z0 + lr0 + r) * P + ix;
            const int k = r * TW;
            const float cl = o[k + 3 * OP], c2 = o[k + 4 * OP], cm = o[k + 5 * OP];
            szz[i] = o[k] + (c2 * dzz[r] + cl * dxx[r]);
            szz[i + 2 * pl] = o[k + 2 * OP] + (cl * dzz[r] + c2 * dxx[r]);
            szz[i + pl] = o[k + OP] + cm * (dzx[r] + dxz[r]);
        }
        return;
    }
    const long long P = p.pitch;
    float *szz = f + F_SZZ * p.plane, *szx = f + F_SZX * p.plane, *sxx = f + F_SXX * p.plane;
    const bool colin = ix >= p.nx1 && ix < p.nx2;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int iz = z0 + lr0 + r;
        if (!colin || iz < p.nz1 || iz >= p.nz2) continue;
        const long long i = (long long)iz * P + ix;
        const int k = r * TW;
        float vz_z = dzz[r], vx_z = dxz[r], vz_x = dzx[r], vx_x = dxx[r];
        cpml_stress(p, T.bz, iz, ix, vz_z, vx_z, vz_x, vx_x);
        stress_finish(p, szz, szx, sxx, iz, ix, i, o[k], o[k + OP], o[k + 2 * OP], o[k + 3 * OP],
                      o[k + 4 * OP], o[k + 5 * OP], vz_z, vx_z, vz_x, vx_x);
    }
}

// ---------------------------------------------------------------- velocity
template <int NS, int MODE, int R>
__device__ __forceinline__ void velocity_issue(const TileMaps &m, float *st, uint32_t b,
                                               const Tile &T, int pps, bool image)
{
    constexpr int HP = halo_plane(NS, R), OP = own_plane(R), HR = halo_rows(NS, R);
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    constexpr bool WE = MODE != MODE_FWD_NOWE;
    constexpr int K_WE = 4, K_U = WE ? 5 : 4, K_G = K_U + (U ? 2 : 0);
    float *own = st + 3 * HP;  // vz vx crz crx [we] [uz ux] [g1 g2]
    const int pb = T.bz * pps, x0 = T.x0, z0 = T.z0;
    mbar_expect_tx(b, (uint32_t)(3 * HR * SW * 4 + vel_own_planes<MODE>(image) * OP * 4));
    tma_load(smem_u32(st), &m.halo, x0 - HX, z0 - NS, pb + F_SZZ, b);
    tma_load(smem_u32(st + HP), &m.halo, x0 - HX, z0 - NS, pb + F_SZX, b);
    tma_load(smem_u32(st + 2 * HP), &m.halo, x0 - HX, z0 - NS, pb + F_SXX, b);
    tma_load(smem_u32(own), &m.own, x0, z0, pb + F_VZ, b);
    tma_load(smem_u32(own + OP), &m.own, x0, z0, pb + F_VX, b);
    tma_load(smem_u32(own + 2 * OP), &m.coef, x0, z0, C_RZ, b);
    tma_load(smem_u32(own + 3 * OP), &m.coef, x0, z0, C_RX, b);
    if (WE)
        tma_load(smem_u32(own + K_WE * OP), &m.own, x0, z0, pb + (MODE == MODE_ADJ ? F_WEA : F_WE), b);
    if (U) {
        tma_load(smem_u32(own + K_U * OP), &m.own, x0, z0, pb + F_UZ, b);
        tma_load(smem_u32(own + (K_U + 1) * OP), &m.own, x0, z0, pb + F_UX, b);
    }
    if (image) {
        tma_load(smem_u32(own + K_G * OP), &m.coef, x0, z0, C_G1, b);
        tma_load(smem_u32(own + (K_G + 1) * OP), &m.coef, x0, z0, C_G2, b);
    }
}

// sdiff2 + pml_diff2 + update_v2, snapshot store / imaging
// (src/cpu/n_kernel_lib_PSV.cpp:207-270, 398-484) of one staged tile:
// halo'd szz, szx, sxx and the tile's own planes.  Cells outside the
// interior only take part in the snapshot / imaging work.
template <int NS, int MODE, int R>
__device__ __forceinline__ void velocity_tile(const StepParams<float> &p, const float *st,
                                              const Tile &T, int slot)
{
    constexpr int HP = halo_plane(NS, R), OP = own_plane(R);
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    constexpr bool WE = MODE != MODE_FWD_NOWE;
    constexpr int K_WE = 4, K_U = WE ? 5 : 4, K_G = K_U + (U ? 2 : 0);
    const bool image = MODE == MODE_ADJ && slot >= 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lc = (w & 1) * 32 + lane, lr0 = (w >> 1) * R;
    const int x0 = T.x0, z0 = T.z0, ix = x0 + lc;
    const bool plain = T.plain;  // interior, no CPML

    // Imaging steps: issue the history and shot-gradient loads of all R rows
    // first (they come from HBM), so their latency overlaps the stencil work.
    float hv[R][5], gv[R][3];
    long long qq[R];
    bool win[R];
    const long long sp = p.snap_plane;
#pragma unroll
    for (int r = 0; r < R; r++) {
        win[r] = false;
        qq[r] = 0;
        if (!image) continue;
        const int iz = z0 + lr0 + r, dzr = iz - p.snap_z1, dxr = ix - p.snap_x1;
        win[r] = !(dzr < 0 || iz > p.snap_z2 || dxr < 0 || ix > p.snap_x2) &&
                 !(dzr % p.snap_dz) && !(dxr % p.snap_dx);
        if (!win[r]) continue;
        qq[r] = (long long)(dzr / p.snap_dz) * p.snx_pitch + dxr / p.snap_dx;
        const float *h = p.hist + (long long)T.bz * p.hist_shot_stride +
                         (long long)slot * p.hist_slot_stride + qq[r];
        const float *g = p.gshot + (long long)T.bz * p.gshot_shot_stride + qq[r];
        hv[r][0] = h[H_SZZ * sp]; hv[r][1] = h[H_SZX * sp]; hv[r][2] = h[H_SXX * sp];
        hv[r][3] = h[H_VZ * sp]; hv[r][4] = h[H_VX * sp];
        gv[r][0] = g[0]; gv[r][1] = g[sp]; gv[r][2] = g[2 * sp];
    }

    float ozz[R], ozx[R], oxx[R], dzz[R], dzxz[R], dzxx[R], dxxx[R];
    {
        constexpr int W = R + 2 * NS - 1;
        const float *c0 = st + lr0 * SW + HX + lc;  // staged row lr0 = tile row lr0 - NS
        float wzz[W], wzx[W];  // wzz[j] = szz[row lr0 - NS + 1 + j], wzx[j] = szx[row lr0 - NS + j]
#pragma unroll
        for (int j = 0; j < W; j++) {
            wzz[j] = c0[(j + 1) * SW];
            wzx[j] = c0[HP + j * SW];
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const float *b = c0 + HP + (r + NS) * SW, *c = b + HP;
            ozz[r] = wzz[r + NS - 1];
            ozx[r] = wzx[r + NS];
            oxx[r] = c[0];
            float szz_z = p.cz[0] * (wzz[r + NS] - ozz[r]);
            float szx_z = p.cz[0] * (ozx[r] - wzx[r + NS - 1]);
            float szx_x = p.cx[0] * (ozx[r] - b[-1]);
            float sxx_x = p.cx[0] * (c[1] - oxx[r]);
#pragma unroll
            for (int k = 2; k <= NS; k++) {
                szz_z += p.cz[k - 1] * (wzz[r + NS + k - 1] - wzz[r + NS - k]);
                szx_z += p.cz[k - 1] * (wzx[r + NS + k - 1] - wzx[r + NS - k]);
                szx_x += p.cx[k - 1] * (b[k - 1] - b[-k]);
                sxx_x += p.cx[k - 1] * (c[k] - c[-(k - 1)]);
            }
            dzz[r] = szz_z; dzxz[r] = szx_z; dzxx[r] = szx_x; dxxx[r] = sxx_x;
        }
    }
    const float *o = st + 3 * HP + lr0 * TW + lc;
    float *f = p.fld + (long long)T.bz * p.shot_stride;
    const long long P = p.pitch;
    const bool colok = ix < p.nx, colin = ix >= p.nx1 && ix < p.nx2;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int iz = z0 + lr0 + r;
        const int k = r * TW;
        const float vzo = o[k], vxo = o[k + OP];
        const float uzo = U ? o[k + K_U * OP] : 0.f, uxo = U ? o[k + (K_U + 1) * OP] : 0.f;
        float vzn = vzo, vxn = vxo, uzn = uzo, uxn = uxo;
        if (!plain && (!colok || iz >= p.nz)) continue;
        const long long i = (long long)iz * P + ix;
        if (plain) {
            velocity_finish<float, MODE>(p, f, i, vzo, vxo, uzo, uxo, WE ? o[k + K_WE * OP] : 0.f,
                                         o[k + 2 * OP], o[k + 3 * OP], dzz[r], dzxz[r], dzxx[r],
                                         dxxx[r], vzn, vxn, uzn, uxn);
        } else if (colin && iz >= p.nz1 && iz < p.nz2) {
            float szz_z = dzz[r], szx_z = dzxz[r], szx_x = dzxx[r], sxx_x = dxxx[r];
            cpml_velocity(p, T.bz, iz, ix, szz_z, szx_z, szx_x, sxx_x);
            velocity_finish<float, MODE>(p, f, i, vzo, vxo, uzo, uxo, WE ? o[k + K_WE * OP] : 0.f,
                                         o[k + 2 * OP], o[k + 3 * OP], szz_z, szx_z, szx_x, sxx_x,
                                         vzn, vxn, uzn, uxn);
        }
        if (slot < 0) continue;
        if (image) {  // fwi_grad2 with the staged imaging factors and preloaded history
            if (!win[r]) continue;
            const float fzz = hv[r][0], fzx = hv[r][1], fxx = hv[r][2];
            const float fvz = hv[r][3], fvx = hv[r][4];
            const float s1 = o[k + K_G * OP] * ((fzz + fxx) * (ozz[r] + oxx[r]));
            const float s23 = o[k + (K_G + 1) * OP] *
                              (fzx * ozx[r] + 0.25f * ((fzz - fxx) * (ozz[r] - oxx[r])));
            float *g = p.gshot + (long long)T.bz * p.gshot_shot_stride + qq[r];
            g[0] = gv[r][0] - s1;
            g[sp] = gv[r][1] - (s23 + s1);
            g[2 * sp] = gv[r][2] - p.kimg * (uxn * fvx + uzn * fvz);
        } else {
            snapshot_point<float, MODE>(p, T.bz, iz, ix, i, slot, ozz[r], ozx[r], oxx[r], vzn, vxn,
                                        uzn, uxn);
        }
    }
}

// Barriers of the NSTAGE stages: initialised by thread 0 before any copy.
__device__ __forceinline__ uint32_t stage_bar(float *stages, int sfl, int s)
{
    return smem_u32(reinterpret_cast<uint64_t *>(stages + NSTAGE * sfl) + s);
}

// Tile records of the NSTAGE stages (after the barriers).
__device__ __forceinline__ Tile *stage_tile(float *stages, int sfl, int s)
{
    return reinterpret_cast<Tile *>(reinterpret_cast<uint64_t *>(stages + NSTAGE * sfl) + NSTAGE) + s;
}

template <int R>
__device__ __forceinline__ Tile stress_record(const StepParams<float> &p, int t, int ntx)
{
    Tile T = tile_of(t, ntx, p.ctl[1], 4 * R);
    T.plain = plain_stress_box(p, T.z0, T.z0 + 4 * R, T.x0, T.x0 + TW);
    return T;
}

template <int R>
__device__ __forceinline__ Tile velocity_record(const StepParams<float> &p,
                                                const SrcRecParams<float> &q, int t, int ntx)
{
    Tile T = tile_of(t, ntx, p.ctl[1], 4 * R);
    T.plain = plain_box(p, T.z0, T.z0 + 4 * R, T.x0, T.x0 + TW);
    if (q.src_kind >= 0 || q.rtf_z)
        T.sr = tile_srcrec(p, q, (T.z0 / (4 * R)) * ntx + T.x0 / TW, T.bz);
    return T;
}

}  // namespace

// ---------------------------------------------------------------------------
// Persistent stress step over all tiles of the batch (NS stencil terms, R
// rows per thread).
// ---------------------------------------------------------------------------
template <int NS, int R>
__global__ void __launch_bounds__(NTHREADS) k_stress_tma(const StepParams<float> p,
                                                         const __grid_constant__ TileMaps m)
{
    constexpr int TZ = 4 * R, SF = stage_floats(2, 6, NS, R);
    extern __shared__ __align__(128) unsigned char smraw[];
    float *stg = align128(smraw);
    const int ntx = (p.nx + TW - 1) / TW, ntz = (p.nz + TZ - 1) / TZ;
    const int ntile = ntx * ntz * p.ctl[1];
    const int pps = (int)(p.shot_stride / p.plane);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSTAGE; s++) mbar_init(stage_bar(stg, SF, s), 1);
        fence_init();
        for (int s = 0; s < NSTAGE; s++) {
            const int t = blockIdx.x + s * gridDim.x;
            if (t < ntile) {
                const Tile T = stress_record<R>(p, t, ntx);
                *stage_tile(stg, SF, s) = T;
                stress_issue<NS, R>(m, stg + s * SF, stage_bar(stg, SF, s), T, pps);
            }
        }
    }
    __syncthreads();  // barriers and records initialised before anyone reads them
    for (int k = 0;; k++) {
        const int t = blockIdx.x + k * gridDim.x;
        if (t >= ntile) break;
        const int s = k % NSTAGE;
        if (!wait_stage(stage_bar(stg, SF, s), (k / NSTAGE) & 1, p.err)) return;
        const Tile T = *stage_tile(stg, SF, s);
        stress_tile<NS, R>(p, stg + s * SF, T);
        __syncthreads();  // stage s and its record are read
        const int tn = t + NSTAGE * gridDim.x;
        if (threadIdx.x == 0 && tn < ntile) {
            const Tile Tn = stress_record<R>(p, tn, ntx);
            *stage_tile(stg, SF, s) = Tn;
            fence_async_smem();
            stress_issue<NS, R>(m, stg + s * SF, stage_bar(stg, SF, s), Tn, pps);
        }
    }
}

// ---------------------------------------------------------------------------
// Persistent velocity step over all tiles of the batch, each followed by
// vsrc2 + urec2 (src/cpu/n_kernel_lib_PSV.cpp:487-576) for the tile's
// sources and receivers.
// ---------------------------------------------------------------------------
// Register budget: four CTAs per SM for the forward modes at 2 rows per
// thread (no spills, measured 7 % faster on HBM-bound grids), three
// otherwise (the adjoint and taller tiles spill at four).
template <int NS, int MODE, int R>
__global__ void __launch_bounds__(NTHREADS, (MODE == MODE_ADJ || R > 2) ? 3 : 4) k_velocity_tma(const StepParams<float> p,
                                                           const SrcRecParams<float> q,
                                                           const int it, const int slot,
                                                           const __grid_constant__ TileMaps m)
{
    constexpr int TZ = 4 * R, SF = stage_floats(3, vel_own_planes<MODE>(true), NS, R);
    extern __shared__ __align__(128) unsigned char smraw[];
    float *stg = align128(smraw);
    const int ntx = (p.nx + TW - 1) / TW, ntz = (p.nz + TZ - 1) / TZ;
    const int ntile = ntx * ntz * p.ctl[1];
    const int pps = (int)(p.shot_stride / p.plane);
    const bool image = MODE == MODE_ADJ && slot >= 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSTAGE; s++) mbar_init(stage_bar(stg, SF, s), 1);
        fence_init();
        for (int s = 0; s < NSTAGE; s++) {
            const int t = blockIdx.x + s * gridDim.x;
            if (t < ntile) {
                const Tile T = velocity_record<R>(p, q, t, ntx);
                *stage_tile(stg, SF, s) = T;
                velocity_issue<NS, MODE, R>(m, stg + s * SF, stage_bar(stg, SF, s), T, pps, image);
            }
        }
    }
    __syncthreads();  // barriers and records initialised before anyone reads them
    for (int k = 0;; k++) {
        const int t = blockIdx.x + k * gridDim.x;
        if (t >= ntile) break;
        const int s = k % NSTAGE;
        if (!wait_stage(stage_bar(stg, SF, s), (k / NSTAGE) & 1, p.err)) return;
        const Tile T = *stage_tile(stg, SF, s);
        velocity_tile<NS, MODE, R>(p, stg + s * SF, T, slot);
        __syncthreads();  // stage s and its record are read; the tile's velocities are written
        const int tn = t + NSTAGE * gridDim.x;
        if (threadIdx.x == 0 && tn < ntile) {
            const Tile Tn = velocity_record<R>(p, q, tn, ntx);
            *stage_tile(stg, SF, s) = Tn;
            fence_async_smem();
            velocity_issue<NS, MODE, R>(m, stg + s * SF, stage_bar(stg, SF, s), Tn, pps, image);
        }
        srcrec_apply<float, MODE>(p, q, it, slot, T.bz, T.sr, (int)threadIdx.x, NTHREADS);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        (void)cudaGetLastError();
    });
    return encode;
}

}  // namespace

// 3-D map (column, row, plane) over nplanes planes of nz x nx floats with
// row pitch `pitch` and plane stride `plane` elements; box bx x by x 1,
// zero fill outside.
int encode3(CUtensorMap *map, const float *base, int nx, int nz, int pitch, long long plane,
            int nplanes, int bx, int by)
{
    auto encode = encoder();
    if (!encode) return fail(PSV_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dim[3] = {(cuuint64_t)nx, (cuuint64_t)nz, (cuuint64_t)nplanes};
    const cuuint64_t stride[2] = {(cuuint64_t)pitch * 4, (cuuint64_t)plane * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)base, dim, stride, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(PSV_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return PSV_OK;
}

int encode_tile_maps(TileMaps *m, const float *fld, int nfplanes, const float *coef, int nx, int nz,
                     int pitch, long long plane, int ns, int rpt)
{
    if (ns < 1 || ns > HX) return fail(PSV_ERR_UNSUPPORTED, "TMA tiles: stencil half-width above 4");
    if (rpt != 2 && rpt != 4 && rpt != 8) return fail(PSV_ERR_ARG, "TMA tiles: rows per thread 2, 4 or 8");
    if (pitch % 4 || ((uintptr_t)fld | (uintptr_t)coef) % 16)
        return fail(PSV_ERR_ARG, "TMA tiles: misaligned field block");
    PSV_TRY(encode3(&m->halo, fld, nx, nz, pitch, plane, nfplanes, SW, halo_rows(ns, rpt)));
    PSV_TRY(encode3(&m->own, fld, nx, nz, pitch, plane, nfplanes, TW, 4 * rpt));
    PSV_TRY(encode3(&m->coef, coef, nx, nz, pitch, plane, 7, TW, 4 * rpt));
    return PSV_OK;
}

namespace {

// Occupancy of one tile-kernel instantiation (shared-memory opt-in first).
struct Occupancy {
    cudaError_t e;
    int per_sm;
};
template <typename K> Occupancy occupancy(K kernel, int smem)
{
    Occupancy r{cudaSuccess, 0};
    if (smem > 48 * 1024)
        r.e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (r.e == cudaSuccess)
        r.e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r.per_sm, kernel, NTHREADS, smem);
    return r;
}

// Persistent grid: as many CTAs as fit on the GPU at once, at most one per tile.
cudaError_t pipe_grid(const Occupancy &o, int ntile, int *grid)
{
    if (o.e != cudaSuccess) return o.e;
    if (o.per_sm < 1) return cudaErrorInvalidConfiguration;
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    *grid = std::max(1, std::min(ntile, nsm * o.per_sm));
    return cudaSuccess;
}

template <int NS, int R>
cudaError_t stress_rn(const StepParams<float> &p, const TileMaps &m, int nbatch, cudaStream_t st)
{
    constexpr int smem = pipe_smem_bytes(2, 6, NS, R);
    const int ntile = ((p.nx + TW - 1) / TW) * ((p.nz + 4 * R - 1) / (4 * R)) * nbatch;
    static const Occupancy occ = occupancy(k_stress_tma<NS, R>, smem);  // per instantiation
    int grid = 0;
    const cudaError_t e = pipe_grid(occ, ntile, &grid);
    if (e != cudaSuccess) return e;
    k_stress_tma<NS, R><<<grid, NTHREADS, smem, st>>>(p, m);
    return cudaGetLastError();
}

template <int NS>
cudaError_t stress_n(const StepParams<float> &p, const TileMaps &m, int rpt, int nbatch,
                     cudaStream_t st)
{
    switch (rpt) {
    case 2: return stress_rn<NS, 2>(p, m, nbatch, st);
    case 4: return stress_rn<NS, 4>(p, m, nbatch, st);
    case 8: return stress_rn<NS, 8>(p, m, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int NS, int MODE, int R>
cudaError_t velocity_rmn(const StepParams<float> &p, const SrcRecParams<float> &q,
                         const TileMaps &m, int it, int slot, int nbatch, cudaStream_t st)
{
    constexpr int smem = pipe_smem_bytes(3, vel_own_planes<MODE>(true), NS, R);
    const int ntile = ((p.nx + TW - 1) / TW) * ((p.nz + 4 * R - 1) / (4 * R)) * nbatch;
    static const Occupancy occ = occupancy(k_velocity_tma<NS, MODE, R>, smem);  // per instantiation
    int grid = 0;
    const cudaError_t e = pipe_grid(occ, ntile, &grid);
    if (e != cudaSuccess) return e;
    k_velocity_tma<NS, MODE, R><<<grid, NTHREADS, smem, st>>>(p, q, it, slot, m);
    return cudaGetLastError();
}

template <int NS, int MODE>
cudaError_t velocity_mn(const StepParams<float> &p, const SrcRecParams<float> &q,
                        const TileMaps &m, int it, int slot, int rpt, int nbatch, cudaStream_t st)
{
    switch (rpt) {
    case 2: return velocity_rmn<NS, MODE, 2>(p, q, m, it, slot, nbatch, st);
    case 4: return velocity_rmn<NS, MODE, 4>(p, q, m, it, slot, nbatch, st);
    case 8: return velocity_rmn<NS, MODE, 8>(p, q, m, it, slot, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int NS>
cudaError_t velocity_n(const StepParams<float> &p, const SrcRecParams<float> &q,
                       const TileMaps &m, int mode, int it, int slot, int rpt, int nbatch,
                       cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: return velocity_mn<NS, MODE_FWD>(p, q, m, it, slot, rpt, nbatch, st);
    case MODE_FWD_NOWE: return velocity_mn<NS, MODE_FWD_NOWE>(p, q, m, it, slot, rpt, nbatch, st);
    case MODE_FWD_U: return velocity_mn<NS, MODE_FWD_U>(p, q, m, it, slot, rpt, nbatch, st);
    case MODE_ADJ: return velocity_mn<NS, MODE_ADJ>(p, q, m, it, slot, rpt, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_stress_tma(const StepParams<float> &p, const TileMaps &m, int ns, int rpt,
                              int nbatch, cudaStream_t st)
{
    switch (ns) {
    case 1: return stress_n<1>(p, m, rpt, nbatch, st);
    case 2: return stress_n<2>(p, m, rpt, nbatch, st);
    case 3: return stress_n<3>(p, m, rpt, nbatch, st);
    case 4: return stress_n<4>(p, m, rpt, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_velocity_tma(const StepParams<float> &p, const SrcRecParams<float> &q,
                                const TileMaps &m, int ns, int mode, int it, int slot, int rpt,
                                int nbatch, cudaStream_t st)
{
    switch (ns) {
    case 1: return velocity_n<1>(p, q, m, mode, it, slot, rpt, nbatch, st);
    case 2: return velocity_n<2>(p, q, m, mode, it, slot, rpt, nbatch, st);
    case 3: return velocity_n<3>(p, q, m, mode, it, slot, rpt, nbatch, st);
    case 4: return velocity_n<4>(p, q, m, mode, it, slot, rpt, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace psv
