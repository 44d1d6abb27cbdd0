// psv_march.cu -- the fused time step as a vertical march (FP32): one
// launch per step of the reference loop (src/cpu/n_kernel_PSV.cpp:90-210),
// each CTA walking down a strip of columns.
//
// A CTA owns W = 128 - 2N columns [x0, x0 + W) and L rows [z0, z0 + L) of
// one shot (N = fdorder / 2).  Its 256 threads are two row groups of 128
// columns: thread (g, t) handles column xs + t (xs = x0 - N) of a window 128
// columns wide.  Iteration k takes R rows: the stress update (vdiff2 +
// pml_diff2 + update_s2 + the free-surface row of surf_mirror, :107-128) of
// rows s_k .. s_k + R - 1 (s_k = z0 - N + k R) on the whole window -- the
// owned columns and an N halo on each side -- and then, N rows behind, the
// velocity update (sdiff2 + pml_diff2 + update_v2, :138-150) of rows
// s_k - N .. s_k - N + R - 1 on the owned columns, with the step's snapshot
// store (gard_fwd_storage2) or imaging (fwi_grad2); each row group takes R / 2
// of the R rows.  The tile's sources and receivers (vsrc2, urec2) follow the
// march.  Stress rows z0 - N .. z0 - 1 and z0 + L .. z0 + L + N - 1 are
// recomputed halo rows, the only vertical overlap between CTAs.
//
// Data movement:
//  - old v (both planes; every neighbour the stress stencil reads) arrives by
//    TMA tensor copies of R rows x (128 + 2N + 4) columns per stage into a
//    ring of stages, one mbarrier each, issued ahead by thread 0;
//  - the new stresses go to a shared ring of the last 2N + R rows (the
//    velocity stencil's neighbours) and, for owned points, to HBM once;
//  - each thread's own old stresses, coefficients, We and u are plain
//    coalesced loads issued one iteration ahead into registers.
//  Every field crosses HBM once per owned point plus the halo; the grid is
//  ordered with the shot fastest (blockIdx.x), so the shots of one strip run
//  together and read its coefficients from HBM once.
//
// A CTA's halo is another CTA's interior, so v, sigma and the stress-side
// CPML memories are read from copy `par` and written to copy 1 - par, as in
// the tile-fused step (psv_fused.cu); halo stresses are recomputed with the
// owner's operations, so every copy of a value is bit identical.
//
// Every mbarrier wait is bounded: after ~1 s the block records error code 1
// in StepParams::err and returns; the host turns that into PSV_ERR_CUDA.
//
// Free surface: none, or a top surface on the first interior row (it
// mirrors no interior row); other placements use the two-launch families
// (march_supported).
#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"
#include "psv_tma.cuh"

namespace psv {
namespace {

constexpr int MNT = 128;  // window columns
constexpr int MRG = 2;    // row groups
constexpr int MTHREADS = MNT * MRG;

__host__ __device__ constexpr int pow2_at_least(int n) { return n <= 1 ? 1 : 2 * pow2_at_least((n + 1) / 2); }
__host__ __device__ constexpr int march_box_width(int ns) { return (MNT + 2 * ns + 3 + 15) / 16 * 16; }

template <int NS, int R>
struct MGeo {
    static constexpr int W = MNT - 2 * NS;                     // owned columns
    static constexpr int BW = march_box_width(NS);             // staged v columns (>= MNT + 2N + 3)
    static constexpr int RPT = R / MRG;                        // rows per thread per phase
    static constexpr int VS = (R + 2 * NS + R - 1) / R - 1;    // v stages beyond the first an iteration reads
    static constexpr int VR = pow2_at_least(VS + 2);           // v ring stages (at least one in flight)
    static constexpr int RV = VR * R;                          // v ring rows
    static constexpr int SN = pow2_at_least(2 * NS + R);       // new-stress ring rows
    static constexpr int SMEM = (2 * RV * BW + 3 * SN * MNT) * 4 + VR * 8 + 128;
    static_assert(R % MRG == 0, "row groups split a stage");
    static_assert((R * BW * 4) % 128 == 0, "each staged box starts on a 128-byte boundary");
};

template <int NS, int MODE, int R>
__global__ void __launch_bounds__(MTHREADS, 2)
    k_step_march(const StepParams<float> p, const SrcRecParams<float> q,
                 const __grid_constant__ MarchMaps mm, const int it, const int slot,
                 const int par, const int L)
{
    using G = MGeo<NS, R>;
    constexpr bool U = MODE == MODE_ADJ || MODE == MODE_FWD_U;
    constexpr bool WE = MODE != MODE_FWD_NOWE;
    extern __shared__ __align__(16) unsigned char msm_raw[];
    float *vring = align128(msm_raw);                 // [2][RV][BW]: old vz, vx rows
    float *nring = vring + 2 * G::RV * G::BW;         // [3][SN][MNT]: new szz, szx, sxx rows
    uint64_t *bars = reinterpret_cast<uint64_t *>(nring + 3 * G::SN * MNT);

    const int bz = blockIdx.x;  // shot of the batch (fastest)
    if (bz >= p.ctl[1]) return;  // whole block
    const int tid = threadIdx.x, t = tid % MNT, g = tid / MNT;
    // 32-bit offsets: a shot's field block holds fewer than 2^31 elements
    const int PL = (int)p.plane, P = p.pitch;
    float *f = p.fld + (long long)bz * p.shot_stride;
    const int rd = par ? p.pp_planes : 0, wr = par ? 0 : p.pp_planes;
    const float *fr = f + rd * PL;  // old v, sigma
    float *fw = f + wr * PL;        // new
    const int pps = (int)(p.shot_stride / PL);  // planes per shot in the tensor map
    const CUtensorMap *vmap = &mm.fld;

    const int x0 = blockIdx.y * G::W, z0 = blockIdx.z * L;
    const int xs = x0 - NS;                        // window column of t = 0
    const int xva = ((xs - NS + 16) & ~3) - 16;    // first staged v column (16-byte aligned)
    const int ov = xs - xva;                       // staged index of the thread's column
    const int ix = xs + t;
    const int zb = z0 - 2 * NS;                    // v row of stage 0, row 0
    const int K = (L + 2 * NS + R - 1) / R;        // iterations
    const int nstage = K + G::VS;                  // v stages the march reads
    const bool own_c = t >= NS && t < NS + G::W && ix < p.nx;
    const bool col_ok = ix >= 0 && ix < p.nx;
    const bool col_in = ix >= p.nx1 && ix < p.nx2;
    const int cx0 = max(p.nx1, p.px0), cx1 = min(p.nx2, p.px1);
    const int rz0 = max(p.nz1, p.pz0), rz1 = min(p.nz2, p.pz1);
    const bool cols_plain_s = xs >= cx0 && xs + MNT <= cx1;  // block-uniform
    const bool cols_plain_v = x0 >= cx0 && x0 + G::W <= cx1;

    auto issue_v = [&](int j) {  // v stage j: rows zb + j R .. + R - 1, both planes
        const int s = j % G::VR;
        const uint32_t bar = smem_u32(bars + s);
        mbar_expect_tx(bar, (uint32_t)(2 * R * G::BW * 4));
        float *dst = vring + s * R * G::BW;
        tma_load(smem_u32(dst), vmap, xva, zb + j * R, bz * pps + rd + F_VZ, bar);
        tma_load(smem_u32(dst + G::RV * G::BW), vmap, xva, zb + j * R, bz * pps + rd + F_VX, bar);
    };
    if (tid == 0) {
        for (int s = 0; s < G::VR; s++) mbar_init(smem_u32(bars + s), 1);
        fence_init();
    }
    __syncthreads();
    if (tid == 0)
        for (int j = 0; j < min(G::VR, nstage); j++) issue_v(j);

    // the thread's column in row r (>= zb) of the staged vz plane; the vx
    // plane follows at + RV BW
    const float *vcol = vring + t + ov;
    auto vrow = [&](int r) -> const float * { return vcol + ((r - zb) & (G::RV - 1)) * G::BW; };
    // the thread's column in row r of the new-stress ring (plane 0 szz;
    // szx, sxx follow at + SN MNT, + 2 SN MNT).  Rows below z0 - N are only
    // read for velocity rows outside the tile, which are skipped.
    float *ncol = nring + t;
    auto nrow = [&](int r) -> float * { return ncol + ((r - (z0 - NS)) & (G::SN - 1)) * MNT; };
    constexpr int VXO = G::RV * G::BW, NXO = G::SN * MNT;

    // Own-column values, loaded one iteration ahead: stress side (old szz,
    // szx, sxx, dt lam, dt (lam + 2 mu), dt mu_zx) of the group's stress rows,
    // velocity side (dt / rho_z, dt / rho_x, We or We_adj, uz, ux) of its
    // velocity rows.
    float so[G::RPT][6], vo[G::RPT][5];
    auto load_own = [&](int k, float (&a)[G::RPT][6], float (&b)[G::RPT][5]) {
#pragma unroll
        for (int i = 0; i < G::RPT; i++) {
            const int s = z0 - NS + k * R + g * G::RPT + i;
            const bool in = col_ok && s >= 0 && s < p.nz;
            const int o = in ? s * P + ix : 0;
            a[i][0] = in ? fr[F_SZZ * PL + o] : 0.f;
            a[i][1] = in ? fr[F_SZX * PL + o] : 0.f;
            a[i][2] = in ? fr[F_SXX * PL + o] : 0.f;
            a[i][3] = in ? __ldg(p.c_lam + o) : 0.f;
            a[i][4] = in ? __ldg(p.c_l2m + o) : 0.f;
            a[i][5] = in ? __ldg(p.c_muzx + o) : 0.f;
            const int qz = s - NS;
            const bool vin = own_c && qz >= z0 && qz < z0 + L && qz < p.nz;
            const int oq = vin ? qz * P + ix : 0;
            b[i][0] = vin ? __ldg(p.c_rz + oq) : 0.f;
            b[i][1] = vin ? __ldg(p.c_rx + oq) : 0.f;
            b[i][2] = (vin && WE) ? f[(MODE == MODE_ADJ ? F_WEA : F_WE) * PL + oq] : 0.f;
            b[i][3] = (vin && U) ? f[F_UZ * PL + oq] : 0.f;
            b[i][4] = (vin && U) ? f[F_UX * PL + oq] : 0.f;
        }
    };
    float so_n[G::RPT][6], vo_n[G::RPT][5];
    load_own(0, so, vo);

    for (int k = 0; k < K; k++) {
        if (k + 1 < K) load_own(k + 1, so_n, vo_n);
        // stages k .. k + VS are in (every earlier one was waited for already)
        bool ok = true;
        for (int j = (k == 0 ? 0 : k + G::VS); j <= k + G::VS && j < nstage; j++) {
            const bool w = mbar_wait(smem_u32(bars + j % G::VR), (uint32_t)((j / G::VR) & 1));
            ok = __syncthreads_and(w) != 0;
            if (!ok) break;
        }
        if (!ok) {
            if (tid == 0) atomicExch(p.err, 1);
            return;
        }

        // ---- stress rows of this thread's group, whole window
        const int sg = z0 - NS + k * R + g * G::RPT;  // first row
        {
            constexpr int WV = G::RPT + 2 * NS - 1;
            float wz[WV], wx[WV];  // wz[j] = vz row sg - N + j, wx[j] = vx row sg - N + 1 + j
#pragma unroll
            for (int j = 0; j < WV; j++) {
                wz[j] = vrow(sg - NS + j)[0];
                wx[j] = vrow(sg - NS + 1 + j)[VXO];
            }
#pragma unroll
            for (int i = 0; i < G::RPT; i++) {
                const int s = sg + i;
                float nzz = so[i][0], nzx = so[i][1], nxx = so[i][2];
                if (s >= p.nz1 && s < p.nz2 && col_in) {
                    const float oz = wz[i + NS], ox = wx[i + NS - 1];
                    const float *hz = vrow(s), *hx = hz + VXO;
                    float vz_z = p.cz[0] * (oz - wz[i + NS - 1]);
                    float vx_z = p.cz[0] * (wx[i + NS] - ox);
                    float vz_x = p.cx[0] * (hz[1] - oz);
                    float vx_x = p.cx[0] * (ox - hx[-1]);
#pragma unroll
                    for (int kk = 2; kk <= NS; kk++) {
                        vz_z += p.cz[kk - 1] * (wz[i + NS + kk - 1] - wz[i + NS - kk]);
                        vx_z += p.cz[kk - 1] * (wx[i + NS + kk - 1] - wx[i + NS - kk]);
                        vz_x += p.cx[kk - 1] * (hz[kk] - hz[-(kk - 1)]);
                        vx_x += p.cx[kk - 1] * (hx[kk - 1] - hx[-kk]);
                    }
                    if (!(cols_plain_s && s >= rz0 && s < rz1))
                        cpml_stress_pp(p, bz, s, ix, vz_z, vx_z, vz_x, vx_x, par,
                                       own_c && s >= z0 && s < z0 + L);
                    const float cl = so[i][3], c2 = so[i][4], cm = so[i][5];
                    nzz = so[i][0] + (c2 * vz_z + cl * vx_x);
                    nxx = so[i][2] + (cl * vz_z + c2 * vx_x);
                    nzx = so[i][1] + cm * (vz_x + vx_z);
                    if (p.st && s == p.st) {
                        nzz = 0.f;
                        nzx = 0.f;
                        nxx = p.fs_top[ix] * vx_x;
                    }
                }
                if (own_c && s >= z0 && s < z0 + L && s < p.nz) {
                    const int o = s * P + ix;
                    fw[F_SZZ * PL + o] = nzz;
                    fw[F_SZX * PL + o] = nzx;
                    fw[F_SXX * PL + o] = nxx;
                }
                float *nr = nrow(s);
                nr[0] = nzz;
                nr[NXO] = nzx;
                nr[2 * NXO] = nxx;
            }
        }
        __syncthreads();  // the iteration's new stresses are in the ring

        // ---- velocity rows of this thread's group, owned columns
        const int qg = sg - NS;
        if (own_c && qg + G::RPT > z0) {  // some velocity row of the group lies in the tile
            constexpr int WS = G::RPT + 2 * NS - 1;
            float wzz[WS], wzx[WS];  // wzz[j] = szz row qg - N + 1 + j, wzx[j] = szx row qg - N + j
#pragma unroll
            for (int j = 0; j < WS; j++) {
                wzz[j] = nrow(qg - NS + 1 + j)[0];
                wzx[j] = nrow(qg - NS + j)[NXO];
            }
            const bool image = MODE == MODE_ADJ && slot >= 0;
#pragma unroll
            for (int i = 0; i < G::RPT; i++) {
                const int qz = qg + i;
                if (qz < z0 || qz >= z0 + L || qz >= p.nz) continue;
                const int o = qz * P + ix;
                ImagePre<float> pre{};
                if (image) pre = image_preload(p, bz, qz, ix, o, slot);
                const float *nzx = nrow(qz) + NXO, *nxx = nzx + NXO;
                const float ozz = wzz[i + NS - 1], ozx = wzx[i + NS], oxx = nxx[0];
                const float *vq = vrow(qz);
                const float vzo = vq[0], vxo = vq[VXO];
                float vzn = vzo, vxn = vxo, uzn = vo[i][3], uxn = vo[i][4];
                if (qz >= p.nz1 && qz < p.nz2 && col_in) {
                    float szz_z = p.cz[0] * (wzz[i + NS] - ozz);
                    float szx_z = p.cz[0] * (ozx - wzx[i + NS - 1]);
                    float szx_x = p.cx[0] * (ozx - nzx[-1]);
                    float sxx_x = p.cx[0] * (nxx[1] - oxx);
#pragma unroll
                    for (int kk = 2; kk <= NS; kk++) {
                        szz_z += p.cz[kk - 1] * (wzz[i + NS + kk - 1] - wzz[i + NS - kk]);
                        szx_z += p.cz[kk - 1] * (wzx[i + NS + kk - 1] - wzx[i + NS - kk]);
                        szx_x += p.cx[kk - 1] * (nzx[kk - 1] - nzx[-kk]);
                        sxx_x += p.cx[kk - 1] * (nxx[kk] - nxx[-(kk - 1)]);
                    }
                    if (!(cols_plain_v && qz >= rz0 && qz < rz1))
                        cpml_velocity(p, bz, qz, ix, szz_z, szx_z, szx_x, sxx_x);
                    velocity_finish<float, MODE>(p, f, o, vzo, vxo, vo[i][3], vo[i][4], vo[i][2],
                                                 vo[i][0], vo[i][1], szz_z, szx_z, szx_x, sxx_x,
                                                 vzn, vxn, uzn, uxn, fw);
                } else {  // not updated: carry the old values into the write copy
                    fw[F_VZ * PL + o] = vzo;
                    fw[F_VX * PL + o] = vxo;
                }
                if (image)
                    image_apply(p, bz, pre, ozz, ozx, oxx, uzn, uxn);
                else if (slot >= 0)
                    snapshot_point<float, MODE>(p, bz, qz, ix, o, slot, ozz, ozx, oxx, vzn, vxn,
                                                uzn, uxn);
            }
        }
        __syncthreads();  // stage k's ring slot and the oldest new-stress rows are free
        if (tid == 0 && k + G::VR < nstage) {
            fence_async_smem();
            issue_v(k + G::VR);
        }
        if (k + 1 < K) {
#pragma unroll
            for (int i = 0; i < G::RPT; i++) {
#pragma unroll
                for (int c = 0; c < 6; c++) so[i][c] = so_n[i][c];
#pragma unroll
                for (int c = 0; c < 5; c++) vo[i][c] = vo_n[i][c];
            }
        }
    }
    if (q.src_kind < 0 && !q.rtf_z) return;  // uniform: kernel argument
    srcrec_apply<float, MODE>(p, q, it, slot, bz,
                              tile_srcrec(p, q, (int)(blockIdx.z * gridDim.y + blockIdx.y), bz),
                              tid, MTHREADS, p.fld + wr * PL);
}

template <int NS, int MODE, int R>
cudaError_t launch_march_m(const StepParams<float> &p, const SrcRecParams<float> &q,
                           const MarchMaps &mm, int it, int slot, int par, int L, int nbatch,
                           cudaStream_t st)
{
    using G = MGeo<NS, R>;
    static cudaError_t attr = cudaFuncSetAttribute(
        k_step_march<NS, MODE, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
    if (attr != cudaSuccess) return attr;
    const dim3 grid(nbatch, (p.nx + G::W - 1) / G::W, (p.nz + L - 1) / L);
    k_step_march<NS, MODE, R><<<grid, MTHREADS, G::SMEM, st>>>(p, q, mm, it, slot, par, L);
    return cudaGetLastError();
}

template <int NS, int R>
cudaError_t launch_march_ns(const StepParams<float> &p, const SrcRecParams<float> &q,
                            const MarchMaps &mm, int mode, int it, int slot, int par, int L,
                            int nbatch, cudaStream_t st)
{
    switch (mode) {
    case MODE_FWD: return launch_march_m<NS, MODE_FWD, R>(p, q, mm, it, slot, par, L, nbatch, st);
    case MODE_FWD_NOWE: return launch_march_m<NS, MODE_FWD_NOWE, R>(p, q, mm, it, slot, par, L, nbatch, st);
    case MODE_FWD_U: return launch_march_m<NS, MODE_FWD_U, R>(p, q, mm, it, slot, par, L, nbatch, st);
    case MODE_ADJ: return launch_march_m<NS, MODE_ADJ, R>(p, q, mm, it, slot, par, L, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int R>
cudaError_t launch_march_r(const StepParams<float> &p, const SrcRecParams<float> &q,
                           const MarchMaps &mm, int ns, int mode, int it, int slot, int par, int L,
                           int nbatch, cudaStream_t st)
{
    switch (ns) {
    case 1: return launch_march_ns<1, R>(p, q, mm, mode, it, slot, par, L, nbatch, st);
    case 2: return launch_march_ns<2, R>(p, q, mm, mode, it, slot, par, L, nbatch, st);
    case 3: return launch_march_ns<3, R>(p, q, mm, mode, it, slot, par, L, nbatch, st);
    case 4: return launch_march_ns<4, R>(p, q, mm, mode, it, slot, par, L, nbatch, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool march_supported(int ns, int rows, int stage, int st, int sb, int sl, int sr, int nz1)
{
    if (rows != 32 && rows != 64 && rows != 128) return false;
    if (stage != 2 && stage != 4) return false;
    if (ns < 1 || ns > 4) return false;
    if (sb || sl || sr) return false;
    return !st || st == nz1;  // a top surface that mirrors no interior row
}

int march_tile_width(int ns, int) { return MNT - 2 * ns; }

int encode_march_maps(MarchMaps *m, const float *fld, int nfplanes, int nx, int nz, int pitch,
                      long long plane, int ns, int stage)
{
    if (pitch % 4 || ((uintptr_t)fld) % 16) return fail(PSV_ERR_ARG, "march: misaligned field block");
    return encode3(&m->fld, fld, nx, nz, pitch, plane, nfplanes, march_box_width(ns), stage);
}

cudaError_t launch_step_march(const StepParams<float> &p, const SrcRecParams<float> &q,
                              const MarchMaps &mm, int ns, int mode, int it, int slot, int par,
                              int rows, int stage, int nbatch, cudaStream_t st)
{
    if (!p.pp_planes) return cudaErrorInvalidValue;
    if (stage == 4) return launch_march_r<4>(p, q, mm, ns, mode, it, slot, par, rows, nbatch, st);
    if (stage == 2) return launch_march_r<2>(p, q, mm, ns, mode, it, slot, par, rows, nbatch, st);
    return cudaErrorInvalidValue;
}

}  // namespace psv
