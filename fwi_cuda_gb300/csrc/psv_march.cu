// psv_march.cu -- the fused time step as a vertical march (FP32): one
// launch per step of the reference loop (src/cpu/n_kernel_PSV.cpp:90-210),
// each CTA walking down a strip of columns.
//
// A CTA of NT threads owns W = NT - 2N columns [x0, x0 + W) and L rows
// [z0, z0 + L) of one shot (N = fdorder / 2).  Thread t handles column
// xs + t (xs = x0 - N) of a window NT columns wide.  Iteration k computes
// the stress update (vdiff2 + pml_diff2 + update_s2 + the surface row of
// surf_mirror, :107-128) of row s = z0 - N + k on the whole window -- the
// owned columns and an N halo on each side -- and then, N rows behind, the
// velocity update (sdiff2 + pml_diff2 + update_v2, :138-150) of row
// q = s - N on the owned columns, with the step's snapshot store
// (gard_fwd_storage2) or imaging (fwi_grad2).  The tile's sources and
// receivers (vsrc2, urec2) follow the march.  Rows z0 - N .. z0 - 1 and
// z0 + L .. z0 + L + N - 1 of stress are recomputed halo rows, the only
// vertical overlap between CTAs.
//
// Memory traffic: every field a step touches crosses HBM once per owned
// point (old v and sigma read, new v and sigma written, coefficients, We,
// u), plus the halo columns and rows, which the neighbouring CTAs read too
// (mostly L2 hits).  The vertical stencil windows of old v (for the stress
// derivatives) and of new sigma (for the velocity derivatives) live in
// registers and shift by one row per iteration; horizontal neighbours come
// from shared memory: a ring of staged old-v rows and a ring of the last
// N + 1 new szx / sxx rows.  Everything the march reads from HBM is staged
// MD rows ahead with cp.async into shared-memory rings (zero-filled outside
// the grid), one commit group per iteration, so each CTA keeps MD rows of
// loads in flight.
//
// A CTA's halo is another CTA's interior, so v, sigma and the stress-side
// CPML memories are read from copy `par` and written to copy 1 - par, as in
// the tile-fused step (psv_fused.cu); halo stresses are recomputed with the
// owner's operations, so every copy of a value is bit identical.
//
// Free surface: none, or a top surface on the first interior row (it
// mirrors no interior row); other placements use the two-launch families
// (march_supported).
#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"

namespace psv {
namespace {

constexpr int MD = 3;  // iterations staged ahead (cp.async groups in flight)

template <int NS, int NT, int MODE>
struct MarchGeo {
    static constexpr int W = NT - 2 * NS;             // owned columns
    static constexpr int VC = (NT + 2 * NS + 3 + 3) / 4 * 4;  // staged v columns (4-aligned start)
    static constexpr int SC = NT + 4;                 // staged own-column planes (4-aligned start)
    static constexpr int RV = NS + MD + 1;            // v rows ring
    static constexpr int RS = MD + 1;                 // stress-side rows ring
    static constexpr int NQ = (MODE == MODE_ADJ || MODE == MODE_FWD_U) ? 5 : MODE == MODE_FWD ? 3 : 2;
    static constexpr int RN = NS + 1;                 // new-stress rows ring
    static constexpr int SMEM = (RV * 2 * VC + RS * 6 * SC + RS * NQ * SC + RN * 2 * SC) * 4;
    static constexpr int MINB = NT == 128 ? 5 : 10;   // CTAs per SM the register budget targets
    static_assert(2 * NS <= RV, "the prologue rows fit the v ring");
    static_assert(VC % 4 == 0 && SC % 4 == 0, "16-byte rows");
};

__device__ __forceinline__ void cp16(float *dst, const float *src, bool in)
{
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src),
                 "r"(in ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// floor(a / 4) * 4 for a >= -16
__device__ __forceinline__ int floor4(int a) { return ((a + 16) & ~3) - 16; }

template <int NS, int NT, int MODE>
struct March {
    using G = MarchGeo<NS, NT, MODE>;
    const StepParams<float> &p;
    float *vr, *sr, *qr, *nr;  // rings: v rows, stress-side rows, velocity-side rows, new stress
    const float *fr;           // read copy of v, sigma (this shot)
    float *f;                  // u, We, We_adj planes (this shot)
    int x0, z0, L, xva, xsa, tid;

    __device__ __forceinline__ float *vrow(int j, int plane) const
    {
        return vr + ((j % G::RV) * 2 + plane) * G::VC;
    }
    __device__ __forceinline__ float *srow(int k, int plane) const
    {
        return sr + ((k % G::RS) * 6 + plane) * G::SC;
    }
    __device__ __forceinline__ float *qrow(int k, int plane) const
    {
        return qr + ((k % G::RS) * G::NQ + plane) * G::SC;
    }
    __device__ __forceinline__ float *nrow(int k, int plane) const
    {
        return nr + ((k % G::RN) * 2 + plane) * G::SC;
    }

    // cp.async of `planes` rows of the 4-aligned window starting at column c0
    // (cols columns) of grid row z into consecutive shared rows of stride sc.
    // Source planes: n0 planes from b0, then n1 from b1, then the rest from
    // b2, each group `plane` elements apart.
    __device__ __forceinline__ void stage_rows(float *dst, int sc, int cols, int c0, int z,
                                               int planes, const float *b0, int n0,
                                               const float *b1, int n1, const float *b2) const
    {
        const int nch = cols / 4;
        const bool zin = z >= 0 && z < p.nz;
        const long long rowoff = zin ? (long long)z * p.pitch : 0;
        for (int k = tid; k < planes * nch; k += NT) {
            const int pl = k / nch, ch = k - pl * nch;
            const int c = c0 + 4 * ch;
            const bool in = zin && c >= 0 && c + 4 <= p.pitch;
            const float *src = pl < n0        ? b0 + pl * p.plane
                               : pl < n0 + n1 ? b1 + (pl - n0) * p.plane
                                              : b2 + (pl - n0 - n1) * p.plane;
            cp16(dst + pl * sc + 4 * ch, src + (in ? rowoff + c : 0), in);
        }
    }

    // v row j of the march (grid row z0 - 2N + j).
    __device__ __forceinline__ void stage_v(int j) const
    {
        stage_rows(vrow(j, 0), G::VC, G::VC, xva, z0 - 2 * NS + j, 2, fr + F_VZ * p.plane, 2,
                   nullptr, 0, nullptr);
    }

    // Everything iteration k reads from HBM: v row 2N + k, the stress-side
    // row of stress row s = z0 - N + k (old szz szx sxx, dt lam, dt (lam +
    // 2 mu), dt mu_zx), the velocity-side row of velocity row
    // q = z0 - 2N + k while q is a row of the tile (dt / rho_z, dt / rho_x,
    // We or We_adj, uz, ux as the mode needs).  One commit group.
    __device__ __forceinline__ void stage(int k) const
    {
        const int K = L + 2 * NS;
        if (k < K) {
            stage_v(2 * NS + k);
            stage_rows(srow(k, 0), G::SC, G::SC, xsa, z0 - NS + k, 6, fr + F_SZZ * p.plane, 3,
                       p.c_lam, 3, nullptr);
            if (k >= 2 * NS)
                stage_rows(qrow(k, 0), G::SC, G::SC, xsa, z0 - 2 * NS + k, G::NQ, p.c_rz, 2,
                           f + (MODE == MODE_ADJ ? F_WEA : F_WE) * p.plane, 1, f + F_UZ * p.plane);
        }
        cp_commit();
    }
};

template <int NS, int NT, int MODE>
__global__ void __launch_bounds__(NT, (MarchGeo<NS, NT, MODE>::MINB))
    k_step_march(const StepParams<float> p, const SrcRecParams<float> q, const int it,
                 const int slot, const int par, const int L)
{
    using G = MarchGeo<NS, NT, MODE>;
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    extern __shared__ __align__(16) float msm[];
    const int bz = blockIdx.z;
    if (bz >= p.ctl[1]) return;  // whole block
    const int tid = threadIdx.x;
    const long long PL = p.plane, P = p.pitch;
    float *f = p.fld + (long long)bz * p.shot_stride;
    const int rd = par ? p.pp_planes : 0, wr = par ? 0 : p.pp_planes;
    float *fw = f + wr * PL;  // new v, sigma

    March<NS, NT, MODE> m{p};
    m.vr = msm;
    m.sr = m.vr + G::RV * 2 * G::VC;
    m.qr = m.sr + G::RS * 6 * G::SC;
    m.nr = m.qr + G::RS * G::NQ * G::SC;
    m.fr = f + rd * PL;
    m.f = f;
    m.x0 = blockIdx.x * G::W;
    m.z0 = blockIdx.y * L;
    m.L = L;
    const int xs = m.x0 - NS;               // window column of thread 0
    m.xva = floor4(xs - NS);                // staged v columns start here
    m.xsa = floor4(xs);                     // staged own-column planes start here
    m.tid = tid;
    const int ov = xs - m.xva;              // shared index of the thread's column in a v row
    const int os = xs - m.xsa;              // ... in an own-column row
    const int ix = xs + tid;
    const int z0 = m.z0;
    const bool own_c = tid >= NS && tid < NS + G::W && ix < p.nx;
    const bool col_in = ix >= p.nx1 && ix < p.nx2;
    // block-uniform: every window column interior and CPML-free (stress),
    // every owned column (velocity)
    const int cx0 = max(p.nx1, p.px0), cx1 = min(p.nx2, p.px1);
    const int rz0 = max(p.nz1, p.pz0), rz1 = min(p.nz2, p.pz1);
    const bool cols_plain_s = xs >= cx0 && xs + NT <= cx1;
    const bool cols_plain_v = m.x0 >= cx0 && m.x0 + G::W <= cx1;
    const int K = L + 2 * NS;

    // ---- prologue: v rows j = 0 .. 2N - 1 fill the vertical windows
    float wvz[2 * NS], wvx[2 * NS + 1];  // vz rows s-N .. s+N-1, vx rows s-N .. s+N
    float wzz[2 * NS], wzx[2 * NS + 1];  // new szz rows s-2N+1 .. s, szx rows s-2N .. s
    for (int j = 0; j < 2 * NS; j++) m.stage_v(j);
    cp_commit();
    cp_wait<0>();
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 2 * NS; j++) {
        if (j < 2 * NS - 1) wvz[j + 1] = m.vrow(j, 0)[tid + ov];
        wvx[j + 1] = m.vrow(j, 1)[tid + ov];
    }
#pragma unroll
    for (int j = 0; j < 2 * NS; j++) wzz[j] = 0.f;
#pragma unroll
    for (int j = 0; j <= 2 * NS; j++) wzx[j] = 0.f;
    __syncthreads();  // window reads done before the ring slots are restaged
#pragma unroll
    for (int k = 0; k < MD; k++) m.stage(k);

    for (int k = 0; k < K; k++) {
        cp_wait<MD - 1>();
        __syncthreads();  // iteration k's rows are in; iteration k - 1's reads are done
        m.stage(k + MD);
        const int s = z0 - NS + k;          // stress row
        const int qz = s - NS;              // velocity row
        const bool vel = k >= 2 * NS && qz < p.nz && own_c;
        const bool image = MODE == MODE_ADJ && slot >= 0;
        ImagePre<float> pre{};
        if (image && vel) pre = image_preload(p, bz, qz, ix, (long long)qz * P + ix, slot);

        // ---- vertical windows shift by a row
#pragma unroll
        for (int j = 0; j < 2 * NS - 1; j++) wvz[j] = wvz[j + 1];
#pragma unroll
        for (int j = 0; j < 2 * NS; j++) wvx[j] = wvx[j + 1];
        wvz[2 * NS - 1] = m.vrow(2 * NS + k - 1, 0)[tid + ov];
        wvx[2 * NS] = m.vrow(2 * NS + k, 1)[tid + ov];

        // ---- stress update of row s on the window
        {
            const float *svz = m.vrow(NS + k, 0) + tid + ov;  // row s, this column
            const float *svx = m.vrow(NS + k, 1) + tid + ov;
            const float ozz = m.srow(k, 0)[tid + os], ozx = m.srow(k, 1)[tid + os];
            const float oxx = m.srow(k, 2)[tid + os];
            float nzz = ozz, nzx = ozx, nxx = oxx;
            const bool row_in = s >= p.nz1 && s < p.nz2;
            if (row_in && col_in) {
                const float oz = wvz[NS], ox = wvx[NS];
                float vz_z = p.cz[0] * (oz - wvz[NS - 1]);
                float vx_z = p.cz[0] * (wvx[NS + 1] - ox);
                float vz_x = p.cx[0] * (svz[1] - oz);
                float vx_x = p.cx[0] * (ox - svx[-1]);
#pragma unroll
                for (int kk = 2; kk <= NS; kk++) {
                    vz_z += p.cz[kk - 1] * (wvz[NS + kk - 1] - wvz[NS - kk]);
                    vx_z += p.cz[kk - 1] * (wvx[NS + kk] - wvx[NS - kk + 1]);
                    vz_x += p.cx[kk - 1] * (svz[kk] - svz[-(kk - 1)]);
                    vx_x += p.cx[kk - 1] * (svx[kk - 1] - svx[-kk]);
                }
                const bool plain = cols_plain_s && s >= rz0 && s < rz1;  // block-uniform
                if (!plain)
                    cpml_stress_pp(p, bz, s, ix, vz_z, vx_z, vz_x, vx_x, par,
                                     own_c && s >= z0 && s < z0 + L);
                const float cl = m.srow(k, 3)[tid + os], c2 = m.srow(k, 4)[tid + os];
                const float cm = m.srow(k, 5)[tid + os];
                nzz = ozz + (c2 * vz_z + cl * vx_x);
                nxx = oxx + (cl * vz_z + c2 * vx_x);
                nzx = ozx + cm * (vz_x + vx_z);
                if (p.st && s == p.st) {
                    nzz = 0.f;
                    nzx = 0.f;
                    nxx = p.fs_top[ix] * vx_x;
                }
            }
            if (own_c && s >= z0 && s < z0 + L && s < p.nz) {
                const long long i = (long long)s * P + ix;
                fw[F_SZZ * PL + i] = nzz;
                fw[F_SZX * PL + i] = nzx;
                fw[F_SXX * PL + i] = nxx;
            }
#pragma unroll
            for (int j = 0; j < 2 * NS - 1; j++) wzz[j] = wzz[j + 1];
#pragma unroll
            for (int j = 0; j < 2 * NS; j++) wzx[j] = wzx[j + 1];
            wzz[2 * NS - 1] = nzz;
            wzx[2 * NS] = nzx;
            m.nrow(k, 0)[tid] = nzx;
            m.nrow(k, 1)[tid] = nxx;
        }
        __syncthreads();  // new stresses of row s visible

        // ---- velocity update of row qz on the owned columns
        if (vel) {
            const long long i = (long long)qz * P + ix;
            const float *nzxr = m.nrow(k - NS, 0) + tid;  // row qz, this column
            const float *nxxr = m.nrow(k - NS, 1) + tid;
            const float ozz = wzz[NS - 1], ozx = wzx[NS], oxx = nxxr[0];
            const float vzo = wvz[0], vxo = wvx[0];
            float vzn = vzo, vxn = vxo, uzn = 0.f, uxn = 0.f;
            const float uzo = U ? m.qrow(k, 3)[tid + os] : 0.f;
            const float uxo = U ? m.qrow(k, 4)[tid + os] : 0.f;
            if (qz >= p.nz1 && qz < p.nz2 && col_in) {
                float szz_z = p.cz[0] * (wzz[NS] - ozz);
                float szx_z = p.cz[0] * (ozx - wzx[NS - 1]);
                float szx_x = p.cx[0] * (ozx - nzxr[-1]);
                float sxx_x = p.cx[0] * (nxxr[1] - oxx);
#pragma unroll
                for (int kk = 2; kk <= NS; kk++) {
                    szz_z += p.cz[kk - 1] * (wzz[NS + kk - 1] - wzz[NS - kk]);
                    szx_z += p.cz[kk - 1] * (wzx[NS + kk - 1] - wzx[NS - kk]);
                    szx_x += p.cx[kk - 1] * (nzxr[kk - 1] - nzxr[-kk]);
                    sxx_x += p.cx[kk - 1] * (nxxr[kk] - nxxr[-(kk - 1)]);
                }
                const bool plain = cols_plain_v && qz >= rz0 && qz < rz1;
                if (!plain) cpml_velocity(p, bz, qz, ix, szz_z, szx_z, szx_x, sxx_x);
                const float weo = MODE != MODE_FWD_NOWE ? m.qrow(k, 2)[tid + os] : 0.f;
                velocity_finish<float, MODE>(p, f, i, vzo, vxo, uzo, uxo, weo,
                                             m.qrow(k, 0)[tid + os], m.qrow(k, 1)[tid + os],
                                             szz_z, szx_z, szx_x, sxx_x, vzn, vxn, uzn, uxn, fw);
            } else {  // not updated: carry the old values into the write copy
                uzn = uzo;
                uxn = uxo;
                fw[F_VZ * PL + i] = vzo;
                fw[F_VX * PL + i] = vxo;
            }
            if (image)
                image_apply(p, bz, pre, ozz, ozx, oxx, uzn, uxn);
            else if (slot >= 0)
                snapshot_point<float, MODE>(p, bz, qz, ix, i, slot, ozz, ozx, oxx, vzn, vxn, uzn,
                                            uxn);
        }
    }
    cp_wait<0>();  // the trailing (empty) groups
    if (q.src_kind < 0 && !q.rtf_z) return;  // uniform: kernel argument
    srcrec_apply<float, MODE>(p, q, it, slot, bz,
                              tile_srcrec(p, q, (int)(blockIdx.y * gridDim.x + blockIdx.x), bz),
                              tid, NT, p.fld + wr * PL);
}

template <int NS, int NT, int MODE>
cudaError_t launch_march_m(const StepParams<float> &p, const SrcRecParams<float> &q, int it,
                           int slot, int par, int L, int nbatch, cudaStream_t st)
{
    using G = MarchGeo<NS, NT, MODE>;
    static cudaError_t attr = cudaFuncSetAttribute(
        k_step_march<NS, NT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
    if (attr != cudaSuccess) return attr;
    const dim3 grid((p.nx + G::W - 1) / G::W, (p.nz + L - 1) / L, nbatch);
    k_step_march<NS, NT, MODE><<<grid, NT, G::SMEM, st>>>(p, q, it, slot, par, L);
    return cudaGetLastError();
}

template <int NS, int NT>
cudaError_t launch_march_ns(const StepParams<float> &p, const SrcRecParams<float> &q, int mode,
                            int it, int slot, int par, int L, int nbatch, cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: return launch_march_m<NS, NT, MODE_FWD>(p, q, it, slot, par, L, nbatch, st);
    case MODE_FWD_NOWE: return launch_march_m<NS, NT, MODE_FWD_NOWE>(p, q, it, slot, par, L, nbatch, st);
    case MODE_FWD_U: return launch_march_m<NS, NT, MODE_FWD_U>(p, q, it, slot, par, L, nbatch, st);
    case MODE_ADJ: return launch_march_m<NS, NT, MODE_ADJ>(p, q, it, slot, par, L, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int NT>
cudaError_t launch_march_nt(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                            int mode, int it, int slot, int par, int L, int nbatch, cudaStream_t st)
{
    switch (ns) {
    case 1: return launch_march_ns<1, NT>(p, q, mode, it, slot, par, L, nbatch, st);
    case 2: return launch_march_ns<2, NT>(p, q, mode, it, slot, par, L, nbatch, st);
    case 3: return launch_march_ns<3, NT>(p, q, mode, it, slot, par, L, nbatch, st);
    case 4: return launch_march_ns<4, NT>(p, q, mode, it, slot, par, L, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool march_supported(int ns, int rows, int warps, int st, int sb, int sl, int sr, int nz1)
{
    if (rows != 32 && rows != 64 && rows != 128) return false;
    if (warps != 2 && warps != 4) return false;
    if (ns < 1 || ns > 4) return false;
    if (sb || sl || sr) return false;
    return !st || st == nz1;  // a top surface that mirrors no interior row
}

int march_tile_width(int ns, int warps) { return 32 * warps - 2 * ns; }

cudaError_t launch_step_march(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                              int mode, int it, int slot, int par, int rows, int warps, int nbatch,
                              cudaStream_t st)
{
    if (!p.pp_planes) return cudaErrorInvalidValue;
    if (warps == 4) return launch_march_nt<128>(p, q, ns, mode, it, slot, par, rows, nbatch, st);
    if (warps == 2) return launch_march_nt<64>(p, q, ns, mode, it, slot, par, rows, nbatch, st);
    return cudaErrorInvalidValue;
}

}  // namespace psv
