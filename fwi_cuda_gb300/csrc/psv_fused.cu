// psv_fused.cu -- the fused time step (FP32): one launch per step of the
// reference loop (src/cpu/n_kernel_PSV.cpp:90-210) instead of a stress and
// a velocity launch.
//
// A CTA owns a tile of 64 columns x TZ rows of one shot.  It stages the old
// velocities of the tile plus a 2N halo and the old stresses plus an N halo
// in shared memory (cp.async, zero-filled outside the grid), recomputes the
// stress update (vdiff2 + pml_diff2 + update_s2 + surf_mirror, :107-128) on
// the tile and its N halo, then the velocity update (sdiff2 + pml_diff2 +
// update_v2, :138-150) of the tile from the new stresses in shared memory,
// with the step's snapshot store (gard_fwd_storage2) or imaging (fwi_grad2)
// and the tile's sources and receivers (vsrc2, urec2).  The new stresses go
// to HBM once and are not read back within the step.
//
// A CTA's halo is another CTA's tile, so it must read old values there
// while the owner writes new ones.  The old and new v, sigma and the
// stress-side CPML memories therefore live in two copies, ping-ponged by the
// step's parity `par` (read copy par, write copy 1 - par); the velocity-side
// CPML memories, u and We are touched by their owner only and stay in place.
// Halo stresses are recomputed with the same per-point operations as the
// owner's, so every copy of a value is bit-identical.
//
// Free surface: only a top surface (the rows above it mirror the rows
// below, within the first tile row's stress region); bottom, left and right
// surfaces use the two-launch families (fused_supported).
#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"

namespace psv {
namespace {

constexpr int FTX = 64;   // tile columns
constexpr int FNT = 256;  // threads per CTA

template <int NS, int TZ>
struct FusedGeo {
    static constexpr int SZR = TZ + 2 * NS;   // stress rows the velocity update reads
    static constexpr int RS = NS <= 2 ? 6 : 8;  // stress rows per work item
    static constexpr int SG = (SZR + RS - 1) / RS;  // work items a column
    static constexpr int SRA = SG * RS;       // stress rows staged and computed (>= SZR)
    static constexpr int SXC = FTX + 2 * NS;  // stress columns
    static constexpr int VZR = SRA + 2 * NS;  // velocity rows staged
    static constexpr int VXC = FTX + 4 * NS;  // velocity columns staged
    static constexpr int RV = TZ / 4;         // velocity rows per work item, 4 items a column
    // floats per cp.async: the staged regions start at columns x0 - 2N and
    // x0 - N (x0 a multiple of 64), which fixes their alignment
    static constexpr int CV = (2 * NS) % 4 == 0 ? 4 : 2;
    static constexpr int CS = NS % 4 == 0 ? 4 : NS % 2 == 0 ? 2 : 1;
    static constexpr int SMEM = (2 * VZR * VXC + 3 * SRA * SXC) * 4;
    // CTAs per SM the register budget targets: what the shared memory allows
    // (228 KB, 1 KB reserved per CTA), at most 4 for 16-row tiles and 3 for
    // 32-row tiles (measured best: 64 registers spill too much in the latter)
    static constexpr int MAXB = TZ == 16 ? 4 : 3;
    static constexpr int MINB = (233472 / (SMEM + 1024)) < MAXB ? (233472 / (SMEM + 1024)) : MAXB;
    static_assert(4 * FTX == FNT && TZ % 4 == 0 && MINB >= 1, "work split");
    static_assert(VXC % CV == 0 && SXC % CS == 0 && (2 * VZR * VXC) % 4 == 0 && (SRA * SXC) % CS == 0,
                  "cp.async alignment of the staged rows");
};

template <int CH>
__device__ __forceinline__ void cp_async(float *dst, const float *src, bool in)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    if constexpr (CH == 4)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src),
                     "r"(in ? 16 : 0) : "memory");
    else if constexpr (CH == 2)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src),
                     "r"(in ? 8 : 0) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src),
                     "r"(in ? 4 : 0) : "memory");
}

// Shared-memory planes of one CTA.
struct FusedSmem {
    float *vz, *vx, *zz, *zx, *xx;
};

// Stress update of the tile and its N halo into the staged stresses.
// PLAIN: the whole stress region lies in the CPML-free interior, away from
// the free surface and its mirrored rows (no per-point checks, coefficient
// loads issued before the arithmetic, 32-bit offsets).
template <int NS, int TZ, bool PLAIN>
__device__ __forceinline__ void fused_stress(const StepParams<float> &p, const FusedSmem &m, int bz,
                                             int x0, int z0, int tid, int par)
{
    using G = FusedGeo<NS, TZ>;
    for (int item = tid; item < G::SG * G::SXC; item += FNT) {
        const int g = item / G::SXC, c = item - g * G::SXC;
        const int r0 = g * G::RS;
        const int ix = x0 - NS + c;
        constexpr int W = G::RS + 2 * NS - 1;
        // wz[j] = vz at grid row (z0 - N + r0) - N + j, wx[j] = vx at that row + 1
        float wz[W], wx[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
            wz[j] = m.vz[(r0 + j) * G::VXC + c + NS];
            wx[j] = m.vx[(r0 + 1 + j) * G::VXC + c + NS];
        }
        float cl[PLAIN ? G::RS : 1], c2[PLAIN ? G::RS : 1], cm[PLAIN ? G::RS : 1];
        if constexpr (PLAIN) {
            const int i0 = (z0 - NS + r0) * p.pitch + ix;
#pragma unroll
            for (int r = 0; r < G::RS; r++) {
                cl[r] = p.c_lam[i0 + r * p.pitch];
                c2[r] = p.c_l2m[i0 + r * p.pitch];
                cm[r] = p.c_muzx[i0 + r * p.pitch];
            }
        }
        const bool colin = PLAIN || (ix >= p.nx1 && ix < p.nx2);
        const bool ownc = ix >= x0 && ix < x0 + FTX;
#pragma unroll
        for (int r = 0; r < G::RS; r++) {
            const int sr = r0 + r, iz = z0 - NS + sr;
            const int vr = (sr + NS) * G::VXC + c + NS;  // (iz, ix) in the staged velocities
            const float oz = wz[r + NS], ox = wx[r + NS - 1];
            float vz_z = p.cz[0] * (oz - wz[r + NS - 1]);
            float vx_z = p.cz[0] * (wx[r + NS] - ox);
            float vz_x = p.cx[0] * (m.vz[vr + 1] - oz);
            float vx_x = p.cx[0] * (ox - m.vx[vr - 1]);
#pragma unroll
            for (int k = 2; k <= NS; k++) {
                vz_z += p.cz[k - 1] * (wz[r + NS + k - 1] - wz[r + NS - k]);
                vx_z += p.cz[k - 1] * (wx[r + NS + k - 1] - wx[r + NS - k]);
                vz_x += p.cx[k - 1] * (m.vz[vr + k] - m.vz[vr - (k - 1)]);
                vx_x += p.cx[k - 1] * (m.vx[vr + k - 1] - m.vx[vr - k]);
            }
            const int si = sr * G::SXC + c;
            if constexpr (PLAIN) {
                m.zz[si] = m.zz[si] + (c2[r] * vz_z + cl[r] * vx_x);
                m.xx[si] = m.xx[si] + (cl[r] * vz_z + c2[r] * vx_x);
                m.zx[si] = m.zx[si] + cm[r] * (vz_x + vx_z);
                continue;
            }
            if (!colin || iz < p.nz1 || iz >= p.nz2) continue;
            const long long i = (long long)iz * p.pitch + ix;
            cpml_stress_pp(p, bz, iz, ix, vz_z, vx_z, vz_x, vx_x, par,
                           ownc && iz >= z0 && iz < z0 + TZ);
            const float ccl = p.c_lam[i], cc2 = p.c_l2m[i], ccm = p.c_muzx[i];
            const float ozz = m.zz[si], ozx = m.zx[si], oxx = m.xx[si];
            // update_s2 and the surface row of surf_mirror (stress_finish's operations)
            float nzz = ozz + (cc2 * vz_z + ccl * vx_x);
            float nxx = oxx + (ccl * vz_z + cc2 * vx_x);
            float nzx = ozx + ccm * (vz_x + vx_z);
            if (p.st) {
                if (iz == p.st) {
                    nzz = 0.f;
                    nzx = 0.f;
                    nxx = p.fs_top[ix] * vx_x;
                } else if (iz < p.st) {  // mirrored below
                    nzz = ozz;
                    nzx = ozx;
                }
            }
            m.zz[si] = nzz;
            m.zx[si] = nzx;
            m.xx[si] = nxx;
        }
    }
}

// Velocity update of the tile from the new stresses, the write-back of the
// tile's new v and sigma, and the snapshot store / imaging of `slot`.
// PLAIN: every tile point is interior and CPML-free.
template <int NS, int MODE, int TZ, bool PLAIN>
__device__ __forceinline__ void fused_velocity(const StepParams<float> &p, const FusedSmem &m,
                                               int bz, int x0, int z0, int tid, int slot,
                                               float *f, float *fw)
{
    using G = FusedGeo<NS, TZ>;
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    const long long PL = p.plane;
    const int g = tid / FTX, c = tid - g * FTX;
    const int r0 = g * G::RV;
    const int ix = x0 + c;
    if (!PLAIN && ix >= p.nx) return;
    constexpr int W = G::RV + 2 * NS - 1;
    // wzz[j] = szz at tile row r0 - N + 1 + j, wzx[j] = szx at tile row r0 - N + j
    float wzz[W], wzx[W];
#pragma unroll
    for (int j = 0; j < W; j++) {
        wzz[j] = m.zz[(r0 + 1 + j) * G::SXC + c + NS];
        wzx[j] = m.zx[(r0 + j) * G::SXC + c + NS];
    }
    const bool image = MODE == MODE_ADJ && slot >= 0;
    const bool colin = PLAIN || (ix >= p.nx1 && ix < p.nx2);
#pragma unroll
    for (int r = 0; r < G::RV; r++) {
        const int iz = z0 + r0 + r;
        if (!PLAIN && iz >= p.nz) break;
        const long long i = (long long)iz * p.pitch + ix;
        ImagePre<float> pre{};
        if (image) pre = image_preload(p, bz, iz, ix, i, slot);
        const int ss = (r0 + r + NS) * G::SXC + c + NS;  // (iz, ix) in the stresses
        const float ozz = wzz[r + NS - 1], ozx = wzx[r + NS], oxx = m.xx[ss];
        const int vi = (r0 + r + 2 * NS) * G::VXC + c + 2 * NS;
        float vzn = m.vz[vi], vxn = m.vx[vi], uzn = 0.f, uxn = 0.f;
        if (PLAIN || (colin && iz >= p.nz1 && iz < p.nz2)) {
            float szz_z = p.cz[0] * (wzz[r + NS] - ozz);
            float szx_z = p.cz[0] * (ozx - wzx[r + NS - 1]);
            float szx_x = p.cx[0] * (ozx - m.zx[ss - 1]);
            float sxx_x = p.cx[0] * (m.xx[ss + 1] - oxx);
#pragma unroll
            for (int k = 2; k <= NS; k++) {
                szz_z += p.cz[k - 1] * (wzz[r + NS + k - 1] - wzz[r + NS - k]);
                szx_z += p.cz[k - 1] * (wzx[r + NS + k - 1] - wzx[r + NS - k]);
                szx_x += p.cx[k - 1] * (m.zx[ss + k - 1] - m.zx[ss - k]);
                sxx_x += p.cx[k - 1] * (m.xx[ss + k] - m.xx[ss - (k - 1)]);
            }
            if (!PLAIN) cpml_velocity(p, bz, iz, ix, szz_z, szx_z, szx_x, sxx_x);
            const float uzo = U ? f[F_UZ * PL + i] : 0.f, uxo = U ? f[F_UX * PL + i] : 0.f;
            const float weo =
                MODE != MODE_FWD_NOWE ? f[(MODE == MODE_ADJ ? F_WEA : F_WE) * PL + i] : 0.f;
            velocity_finish<float, MODE>(p, f, i, vzn, vxn, uzo, uxo, weo, p.c_rz[i], p.c_rx[i],
                                         szz_z, szx_z, szx_x, sxx_x, vzn, vxn, uzn, uxn, fw);
        } else {  // not updated: carry the old values into the write copy
            if (U) {
                uzn = f[F_UZ * PL + i];
                uxn = f[F_UX * PL + i];
            }
            fw[F_VZ * PL + i] = vzn;
            fw[F_VX * PL + i] = vxn;
        }
        fw[F_SZZ * PL + i] = ozz;
        fw[F_SZX * PL + i] = ozx;
        fw[F_SXX * PL + i] = oxx;
        if (image)
            image_apply(p, bz, pre, ozz, ozx, oxx, uzn, uxn);
        else if (slot >= 0)
            snapshot_point<float, MODE>(p, bz, iz, ix, i, slot, ozz, ozx, oxx, vzn, vxn, uzn, uxn);
    }
}

template <int NS, int MODE, int TZ>
__global__ void __launch_bounds__(FNT, (FusedGeo<NS, TZ>::MINB))
    k_step_fused(const StepParams<float> p, const SrcRecParams<float> q, const int it,
                 const int slot, const int par)
{
    using G = FusedGeo<NS, TZ>;
    extern __shared__ __align__(16) float fsm[];
    FusedSmem m;
    m.vz = fsm;
    m.vx = fsm + G::VZR * G::VXC;
    m.zz = m.vx + G::VZR * G::VXC;
    m.zx = m.zz + G::SRA * G::SXC;
    m.xx = m.zx + G::SRA * G::SXC;
    const int bz = blockIdx.z;
    if (bz >= p.ctl[1]) return;  // whole block
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * FTX, z0 = blockIdx.y * TZ;
    const long long P = p.pitch, PL = p.plane;
    float *f = p.fld + (long long)bz * p.shot_stride;  // u, We, We_adj planes
    const int rd = par ? p.pp_planes : 0, wr = par ? 0 : p.pp_planes;
    const float *fr = f + rd * PL;  // old vz vx szz szx sxx
    float *fw = f + wr * PL;        // new

    // ---- stage the old fields
    {
        constexpr int CPR = G::VXC / G::CV;
        for (int k = tid; k < G::VZR * CPR; k += FNT) {
            const int r = k / CPR, c = (k - r * CPR) * G::CV;
            const int iz = z0 - 2 * NS + r, ix = x0 - 2 * NS + c;
            const bool in = iz >= 0 && iz < p.nz && ix >= 0 && ix + G::CV <= p.pitch;
            const long long gi = in ? (long long)iz * P + ix : 0;
            cp_async<G::CV>(m.vz + r * G::VXC + c, fr + F_VZ * PL + gi, in);
            cp_async<G::CV>(m.vx + r * G::VXC + c, fr + F_VX * PL + gi, in);
        }
    }
    {
        constexpr int CPR = G::SXC / G::CS;
        for (int k = tid; k < G::SRA * CPR; k += FNT) {
            const int r = k / CPR, c = (k - r * CPR) * G::CS;
            const int iz = z0 - NS + r, ix = x0 - NS + c;
            const bool in = iz >= 0 && iz < p.nz && ix >= 0 && ix + G::CS <= p.pitch;
            const long long gi = in ? (long long)iz * P + ix : 0;
            cp_async<G::CS>(m.zz + r * G::SXC + c, fr + F_SZZ * PL + gi, in);
            cp_async<G::CS>(m.zx + r * G::SXC + c, fr + F_SZX * PL + gi, in);
            cp_async<G::CS>(m.xx + r * G::SXC + c, fr + F_SXX * PL + gi, in);
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();

    // block-uniform: the stress region (and so the tile) is plain
    const bool plain = plain_stress_box(p, z0 - NS, z0 - NS + G::SRA, x0 - NS, x0 + FTX + NS);
    if (plain)
        fused_stress<NS, TZ, true>(p, m, bz, x0, z0, tid, par);
    else
        fused_stress<NS, TZ, false>(p, m, bz, x0, z0, tid, par);
    if (p.st && z0 - NS < p.st) {  // block-uniform: the first tile row
        __syncthreads();
        // rows [nz1, st) at interior columns: minus the new stress of row 2 st - iz
        const int ra = max(p.nz1, z0 - NS) - (z0 - NS), rb = p.st - (z0 - NS);
        for (int k = tid; k < (rb - ra) * G::SXC; k += FNT) {
            const int sr = ra + k / G::SXC, c = k % G::SXC;
            const int ix = x0 - NS + c, iz = z0 - NS + sr;
            if (ix < p.nx1 || ix >= p.nx2) continue;
            const int si = sr * G::SXC + c, sj = (sr + 2 * (p.st - iz)) * G::SXC + c;
            m.zz[si] = -m.zz[sj];
            m.zx[si] = -m.zx[sj];
        }
    }
    __syncthreads();

    if (plain)
        fused_velocity<NS, MODE, TZ, true>(p, m, bz, x0, z0, tid, slot, f, fw);
    else
        fused_velocity<NS, MODE, TZ, false>(p, m, bz, x0, z0, tid, slot, f, fw);
    if (q.src_kind < 0 && !q.rtf_z) return;  // uniform: kernel argument
    srcrec_apply<float, MODE>(p, q, it, slot, bz,
                              tile_srcrec(p, q, (int)(blockIdx.y * gridDim.x + blockIdx.x), bz),
                              tid, FNT, p.fld + wr * PL);
}

template <int NS, int MODE, int TZ>
cudaError_t launch_fused_m(const StepParams<float> &p, const SrcRecParams<float> &q, int it,
                           int slot, int par, int nbatch, cudaStream_t st)
{
    using G = FusedGeo<NS, TZ>;
    static cudaError_t attr = cudaFuncSetAttribute(
        k_step_fused<NS, MODE, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
    if (attr != cudaSuccess) return attr;
    const dim3 grid((p.nx + FTX - 1) / FTX, (p.nz + TZ - 1) / TZ, nbatch);
    k_step_fused<NS, MODE, TZ><<<grid, FNT, G::SMEM, st>>>(p, q, it, slot, par);
    return cudaGetLastError();
}

template <int NS, int TZ>
cudaError_t launch_fused_ns(const StepParams<float> &p, const SrcRecParams<float> &q, int mode,
                            int it, int slot, int par, int nbatch, cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: return launch_fused_m<NS, MODE_FWD, TZ>(p, q, it, slot, par, nbatch, st);
    case MODE_FWD_NOWE: return launch_fused_m<NS, MODE_FWD_NOWE, TZ>(p, q, it, slot, par, nbatch, st);
    case MODE_FWD_U: return launch_fused_m<NS, MODE_FWD_U, TZ>(p, q, it, slot, par, nbatch, st);
    case MODE_ADJ: return launch_fused_m<NS, MODE_ADJ, TZ>(p, q, it, slot, par, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int TZ>
cudaError_t launch_fused_tz(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                            int mode, int it, int slot, int par, int nbatch, cudaStream_t st)
{
    switch (ns) {
    case 1: return launch_fused_ns<1, TZ>(p, q, mode, it, slot, par, nbatch, st);
    case 2: return launch_fused_ns<2, TZ>(p, q, mode, it, slot, par, nbatch, st);
    case 3: return launch_fused_ns<3, TZ>(p, q, mode, it, slot, par, nbatch, st);
    case 4: return launch_fused_ns<4, TZ>(p, q, mode, it, slot, par, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool fused_supported(int ns, int tz, int st, int sb, int sl, int sr, int nz1)
{
    if (tz != 16 && tz != 32) return false;
    if (sb || sl || sr) return false;
    // the first tile row's stress region holds every mirrored row and its
    // image; the second tile row's holds none
    return !st || (st + ns <= tz && 2 * st - nz1 <= tz + ns - 1);
}

cudaError_t launch_step_fused(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                              int mode, int it, int slot, int par, int tz, int nbatch,
                              cudaStream_t st)
{
    if (!p.pp_planes) return cudaErrorInvalidValue;
    if (tz == 16) return launch_fused_tz<16>(p, q, ns, mode, it, slot, par, nbatch, st);
    if (tz == 32) return launch_fused_tz<32>(p, q, ns, mode, it, slot, par, nbatch, st);
    return cudaErrorInvalidValue;
}

}  // namespace psv
