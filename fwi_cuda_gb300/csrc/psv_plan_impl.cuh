// psv_plan_impl.cuh -- Plan<T>: device layout, time loop and FWI drivers.
// Instantiated for float (psv_plan_f32.cu) and double (psv_plan_f64.cu).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "psv_checkpoint.hpp"
#include "psv_plan.cuh"

namespace psv {

inline int round_up(int v, int a) { return (v + a - 1) / a * a; }

// Process-wide cache of autotuned tile shapes: (nz, nx, stencil terms, batch,
// element size, requested family) -> (family, rows per thread, block height).
using TuneKey = std::tuple<int, int, int, int, int, int>;
inline std::map<TuneKey, std::tuple<int, int, int>> &tune_cache()
{
    static std::map<TuneKey, std::tuple<int, int, int>> m;
    return m;
}
// ... and the chain count the autotuner chose for that key.
inline std::map<TuneKey, int> &chain_cache()
{
    static std::map<TuneKey, int> m;
    return m;
}
inline std::mutex &tune_mutex()
{
    static std::mutex m;
    return m;
}

// Which time loop a pass runs.
enum PassKind {
    PASS_FWD_STORE = 0,  // gradient forward: We + snapshots (kernel_PSV accu = true)
    PASS_FWD_PLAIN = 1,  // modelling / step-length trials: traces only
    PASS_ADJ_RES = 2,    // adjoint fired by the residuals at the receivers
    PASS_FWD_U = 3,      // drop-in forward: u, We, optional snapshots (no graph)
    PASS_ADJ_GIVEN = 4,  // drop-in adjoint with the caller's sources (no graph)
    NPASS = 5
};

template <typename T>
class Plan final : public PlanIface {
public:
    Survey sv;
    psv_options opt;
    int B = 1, nbatch = 1;
    int pitch = 0, mx_pitch = 0, snx_pitch = 0, nzs = 0, nxs = 0;
    long long plane = 0, shot_stride = 0, mz_shot = 0, mx_shot = 0, hist_shot = 0, gshot_shot = 0;
    long long ntr = 0;  // nt * nrec
    size_t total = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {};
    int *h_ctl = nullptr;
    DevMem fld, memz, memx, hist, gshot, coef, prof, fsb;
    DevMem model, stf, traces, red, taperb, ctl, scales;
    DevMem f_off, f_pos, f_col, f_snap, a_off, a_pos, a_col, a_snap, rec_pos;
    DevMem t_src_off, t_src_k, t_rec_off, t_rec_r;  // per-tile source / receiver index
    int rpt = 1;                                     // rows per thread (< 0: shuffle variant)
    int fam = PSV_KERNELS_DIRECT;                    // kernel family of the time step
    TileMaps tmap{}, tmap2{};                        // tensor maps of fld / fld2 (TMA family)
    MarchMaps mmap{}, mmap2{};                       // tensor maps of fld / fld2 (MARCH family)
    int *h_err = nullptr;                            // pinned copy of the device error word
    std::vector<int> h_f_off;                        // host copy of the per-shot source lists
    // Checkpointed storage: nck state slots at starts of K-step segments
    // (where the schedule puts them), a working state (5 field planes + CPML
    // strips) and a segment snapshot buffer.  nck = nseg: a state at every
    // segment start (two-level); nck < nseg: binomial schedule.
    bool ckpt = false;
    int store_kind = PSV_STORE_FULL;
    int K = 0, nseg = 0, nck = 0, nslots = 0;
    long long ck_state = 0;  // elements of one shot's checkpointed state
    CkSchedule sched;
    std::vector<int> fwd_slot;  // per segment: slot the forward pass saves into, or -1
    // Optional preconditioners: smoothing scratch and filter; Fletcher-Reeves
    // state (dir, old for lam, mu, rho) and reduction partials.
    DevMem gtmp, gfilt, pcgbuf, pcgpart;
    DevMem ex_store, ex_work, ex_q;  // exact adjoint: per-step derivatives, work planes, memories
    DevMem ck, fld2, memz2, memx2;
    StepParams<T> sp{}, sp2{};
    SrcRecParams<T> qf{}, qa{}, qk{}, qr{};
    cudaGraphExec_t gx[NPASS] = {};
    double C[3] = {0, 0, 0};
    double inj = 1.0;     // dt/(dz dx) * max(1/rho): injection gain of a displacement source
    double gscale = 1.0;  // power of two on the imaging factors g1, g2
    std::vector<double> L2_shot;
    int last_s0 = -1, last_n = 0, last_batch_s0 = 0;
    double t_ms[3] = {0, 0, 0};
    bool have_model = false, have_obs = false, store_flag = false;
    bool tuned = false;
    long long nlaunch = 0;          // kernels launched (graph nodes counted per replay)
    long long gx_nodes[NPASS] = {}; // kernels in each captured pass
    dim3 blk{32, 8, 1};
    // Chained schedule (direct family): the batch split into `chains` groups
    // of slots whose time loops run on their own (captured) streams, so one
    // group's launches fill the kernel boundaries of the others.
    static constexpr int MAXCH = 4;
    int chains = 1;
    cudaStream_t stc[MAXCH] = {};
    cudaEvent_t evf = nullptr, evj[MAXCH] = {};
    DevMem ctl2;            // [MAXCH][2]: global shot of the group's slot 0, shots
    int *h_ctl2 = nullptr;  // pinned [nbatch][MAXCH][2]

    ~Plan() override
    {
        if (evf) cudaEventDestroy(evf);
        for (int k = 0; k < MAXCH; k++) {
            if (evj[k]) cudaEventDestroy(evj[k]);
            if (stc[k]) cudaStreamDestroy(stc[k]);
        }
        if (h_ctl2) cudaFreeHost(h_ctl2);
        for (auto &g : gx)
            if (g) cudaGraphExecDestroy(g);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (h_err) cudaFreeHost(h_err);
        if (st) cudaStreamDestroy(st);
    }

    long long device_bytes() const override { return (long long)total; }

    double *dm(int k) const { return model.as<double>() + (size_t)k * sv.g.nz * sv.g.nx; }
    double *lam() const { return dm(0); }
    double *mu() const { return dm(1); }
    double *rho() const { return dm(2); }
    double *lamc() const { return dm(3); }
    double *muc() const { return dm(4); }
    double *rhoc() const { return dm(5); }
    double *grad(int k) const { return dm(6 + k); }
    double *avg(int k) const { return dm(9 + k); }
    double *tr(int k) const { return traces.as<double>() + (size_t)k * sv.s.nshot * ntr; }
    // traces: 0 rtf_z 1 rtf_x 2 obs_z 3 obs_x 4 res_z 5 res_x (all [shot][nt][nrec])
    double *partial() const { return red.as<double>(); }
    double *L2dev() const { return red.as<double>() + (size_t)256 * std::max(3, sv.s.nshot); }
    double *cavg() const { return L2dev() + sv.s.nshot; }
    double *wmax() const { return cavg() + 3; }
    unsigned long long *maxbits() const { return (unsigned long long *)(wmax() + B); }
    // scales: fscale[nshot] funscale[nshot] ascale[nshot] rmax_bits[nshot]
    double *fscale() const { return scales.as<double>(); }
    double *funscale() const { return fscale() + sv.s.nshot; }
    double *ascale() const { return fscale() + 2 * sv.s.nshot; }
    int ntiles = 0;
    std::vector<int> src_list_col;  // source index of each entry of the per-shot lists
    unsigned long long *rmax() const { return (unsigned long long *)(fscale() + 3 * sv.s.nshot); }

    // ---------------------------------------------------------------- setup
    int init(const Survey &s_, const psv_options &o)
    {
        sv = s_;
        opt = o;
        const psv_grid &g = sv.g;
        const int nz = g.nz, nx = g.nx, nshot = sv.s.nshot, nrec = sv.s.nrec;
        const int al = 128 / (int)sizeof(T);
        if (opt.kernel_family < 0 || opt.kernel_family > PSV_KERNELS_MARCH)
            return fail(PSV_ERR_ARG, "kernel_family must be 0, 1, 2, 3, 4 or 5");
        if (opt.kernel_family >= PSV_KERNELS_TMA && sizeof(T) != 4)
            return fail(PSV_ERR_UNSUPPORTED, "TMA, VEC4, FUSED and MARCH kernels are FP32 only");
        if (opt.chains != 0 && opt.chains != 1 && opt.chains != 2 && opt.chains != 4)
            return fail(PSV_ERR_ARG, "chains must be 0 (autotuned), 1, 2 or 4");
        if (opt.smooth_hfs < 0 || opt.smooth_hfs == 1)
            return fail(PSV_ERR_ARG, "smooth_hfs must be 0 (off) or at least 2");
        if (opt.block_y > 0 && opt.block_y <= 8) blk = dim3(32, opt.block_y, 1);
        if (opt.block_y > 0 || opt.rows_per_thread) opt.autotune = 0;  // explicit shape wins
        if (opt.kernel_family == PSV_KERNELS_TMA) {
            fam = PSV_KERNELS_TMA;
            rpt = tma_rpt(opt.rows_per_thread ? opt.rows_per_thread : 4);
        } else if (opt.kernel_family == PSV_KERNELS_VEC4) {
            fam = PSV_KERNELS_VEC4;
            rpt = v4_rpt(opt.rows_per_thread ? opt.rows_per_thread : 1);
            if (opt.block_y <= 0) blk = dim3(32, 4, 1);
        } else if (opt.kernel_family == PSV_KERNELS_FUSED) {
            fam = PSV_KERNELS_FUSED;
            rpt = fused_tz(opt.rows_per_thread ? opt.rows_per_thread : 32);
            if (!fused_ok(rpt))
                return fail(PSV_ERR_UNSUPPORTED, "fused time step: only a top free surface, within "
                                                 "the first tile row");
        } else if (opt.kernel_family == PSV_KERNELS_MARCH) {
            fam = PSV_KERNELS_MARCH;
            rpt = march_rows(opt.rows_per_thread ? opt.rows_per_thread : 64);
            blk = dim3(32, march_stage(opt.block_y > 0 ? opt.block_y : 4), 1);
            if (!march_ok(rpt, (int)blk.y))
                return fail(PSV_ERR_UNSUPPORTED, "march time step: no free surface or a top one on "
                                                 "the first interior row only");
        } else {
            rpt = rpt_ok<T>(opt.rows_per_thread ? opt.rows_per_thread : 1);
            if (opt.block_y <= 0) blk = dim3(32, 4, 1);
        }
        if (opt.adjoint != PSV_ADJOINT_REFERENCE && opt.adjoint != PSV_ADJOINT_EXACT)
            return fail(PSV_ERR_ARG, "adjoint must be PSV_ADJOINT_REFERENCE or PSV_ADJOINT_EXACT");
        if (opt.adjoint == PSV_ADJOINT_EXACT) {
            if (sizeof(T) != 8) return fail(PSV_ERR_UNSUPPORTED, "exact adjoint: FP64 plans only");
            if (sv.sb || sv.sl || sv.sr)
                return fail(PSV_ERR_UNSUPPORTED, "exact adjoint: no free surface or a top one only");
            if (sv.s.rtf_type != 0 || sv.s.nrec == 0)
                return fail(PSV_ERR_UNSUPPORTED, "exact adjoint: displacement receivers (rtf_type 0) needed");
        }
        pitch = round_up(nx, al);
        plane = (long long)nz * pitch;
        shot_stride = (long long)nfield() * plane;
        // The time-step kernels address one shot's field planes with 32-bit
        // offsets.
        if (shot_stride > PSV_MAX_SHOT_ELEMS)
            return fail(PSV_ERR_UNSUPPORTED, "grid too large: one shot's field planes exceed "
                                             "2^31 - 1 elements (nz x padded nx x " +
                                                 std::to_string(nfield()) + " planes)");
        nzs = g.pml_z ? sv.pz0 + (nz - sv.pz1) : 0;
        nxs = g.pml_x ? sv.px0 + (nx - sv.px1) : 0;
        mx_pitch = nxs ? round_up(nxs, al) : 0;
        mz_shot = (long long)(sizeof(T) == 4 ? NMZ_PP : NMZ) * nzs * pitch;
        mx_shot = (long long)(sizeof(T) == 4 ? NMX_PP : NMX) * nz * mx_pitch;
        snx_pitch = round_up(sv.snx, al);
        const long long snap_plane = (long long)sv.snz * snx_pitch;
        hist_shot = (long long)sv.snt * NHIST * snap_plane;
        gshot_shot = 3 * snap_plane;
        ntr = (long long)g.nt * nrec;

        const double budget = (opt.hbm_budget_gb > 0 ? opt.hbm_budget_gb : 180.0) * 1e9;
        const double per_shot = (double)(shot_stride + mz_shot + mx_shot + gshot_shot) * sizeof(T);
        const double per_hist = (double)hist_shot * sizeof(T);
        const double shared = 7.0 * plane * sizeof(T) + 12.0 * nz * nx * 8 + 6.0 * nshot * ntr * 8;
        // checkpointed alternative: K minimising nt/K states + K/snap_dt snapshots
        ck_state = 5 * plane + mz_shot + mx_shot;
        const double snap5 = (double)NHIST * snap_plane, sdt = g.snap_dt;
        const bool binomial = opt.storage == PSV_STORE_BINOMIAL;
        auto segments = [&](int k) {
            K = std::min(std::max(k, 1), g.nt);
            nseg = (g.nt + K - 1) / K;
            nslots = (K + g.snap_dt - 1) / g.snap_dt + 1;
        };
        segments(opt.checkpoint_interval > 0 ? opt.checkpoint_interval
                 : binomial ? g.snap_dt
                            : (int)std::max(1.0, std::round(std::sqrt(g.nt * (double)ck_state * sdt / snap5))));
        auto per_ck = [&](int slots) {
            return ((double)slots * ck_state + (double)ck_state + (double)nslots * snap5) * sizeof(T);
        };
        auto fit = [&](double extra) {
            int b = opt.max_batch > 0 ? std::min(opt.max_batch, nshot) : nshot;
            while (b > 1 && shared + b * (per_shot + extra) > budget) b--;
            return shared + b * (per_shot + extra) <= budget ? b : 0;
        };
        const int b_full = fit(per_hist);
        int b_ck = binomial ? 0 : fit(per_ck(nseg));
        nck = nseg;
        if (opt.storage == PSV_STORE_FULL) {
            if (!b_full) return fail(PSV_ERR_OOM, "full snapshot history of one shot exceeds the HBM budget");
            B = b_full;
        } else if (opt.storage == PSV_STORE_CHECKPOINT) {
            if (!b_ck) return fail(PSV_ERR_OOM, "checkpoints of one shot exceed the HBM budget");
            ckpt = true;
            B = b_ck;
        } else if (!binomial && (b_full || b_ck)) {
            ckpt = b_ck > b_full;
            B = ckpt ? b_ck : b_full;
        } else {
            // binomial: the slots asked for, else the fewest giving at most two
            // forward repetitions (C(S + 2, 2) >= nseg), at the largest batch
            // that holds them; with less room, one shot and every slot that fits
            if (!binomial && opt.checkpoint_interval <= 0) segments(g.snap_dt);
            int S = opt.checkpoint_slots > 0 ? opt.checkpoint_slots : 1;
            if (opt.checkpoint_slots <= 0)
                while (S < nseg && ck_reps(nseg, S) > 2) S++;
            S = std::min(S, nseg);
            B = fit(per_ck(S));
            if (!B && opt.checkpoint_slots <= 0) {
                while (S > 2 && !fit(per_ck(S))) S--;
                B = fit(per_ck(S));
            }
            if (!B) return fail(PSV_ERR_OOM, "binomial checkpoints of one shot exceed the HBM budget");
            ckpt = true;
            nck = S;
        }
        if (ckpt) {
            store_kind = nck < nseg ? PSV_STORE_BINOMIAL : PSV_STORE_CHECKPOINT;
            if (ck_min_advances(nseg, nck) > CK_MAX_ADVANCES)
                return fail(PSV_ERR_UNSUPPORTED, "binomial checkpoints: more than 2^26 segment "
                                                 "advances; give more checkpoint_slots or a "
                                                 "longer checkpoint_interval");
            sched = ck_schedule(nseg, nck);
            fwd_slot.assign((size_t)nseg, -1);
            for (const CkAction &x : sched.fwd) fwd_slot[(size_t)x.seg] = x.slot;
        }
        if (ckpt) hist_shot = (long long)nslots * NHIST * snap_plane;
        nbatch = (nshot + B - 1) / B;

        PSV_CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        for (auto &e : ev) PSV_CU(cudaEventCreate(&e));
        PSV_CU(cudaMallocHost(&h_ctl, sizeof(int) * 2 * nbatch));
        PSV_CU(cudaMallocHost(&h_err, sizeof(int)));
        PSV_CU(cudaEventCreateWithFlags(&evf, cudaEventDisableTiming));
        for (int k = 1; k < MAXCH; k++) PSV_CU(cudaStreamCreateWithFlags(&stc[k], cudaStreamNonBlocking));
        for (int k = 0; k < MAXCH; k++) PSV_CU(cudaEventCreateWithFlags(&evj[k], cudaEventDisableTiming));
        stc[0] = nullptr;  // chain 0 runs on the plan's stream
        PSV_CU(cudaMallocHost(&h_ctl2, sizeof(int) * 2 * MAXCH * nbatch));
        chains = opt.chains == 2 || opt.chains == 4 ? opt.chains : 1;
        PSV_TRY(set_chains(chains));
        *h_err = 0;
        for (int b = 0; b < nbatch; b++) {
            h_ctl[2 * b] = b * B;
            h_ctl[2 * b + 1] = std::min(B, nshot - b * B);
        }

        PSV_TRY(fld.alloc((size_t)B * shot_stride * sizeof(T), total));
        PSV_TRY(memz.alloc((size_t)B * mz_shot * sizeof(T), total));
        PSV_TRY(memx.alloc((size_t)B * mx_shot * sizeof(T), total));
        PSV_TRY(gshot.alloc((size_t)B * gshot_shot * sizeof(T), total));
        PSV_TRY(coef.alloc((size_t)7 * plane * sizeof(T), total));
        const int nmax = std::max(nz, nx);
        PSV_TRY(prof.alloc((size_t)12 * nmax * sizeof(T), total));
        PSV_TRY(fsb.alloc((size_t)(2 * nx + 2 * nz) * sizeof(T), total));
        PSV_TRY(model.alloc((size_t)12 * nz * nx * 8, total));
        PSV_TRY(traces.alloc((size_t)6 * nshot * ntr * 8 + 8, total));
        PSV_TRY(red.alloc(((size_t)256 * std::max(3, nshot) + nshot + 3 + B + 2) * 8, total));
        PSV_TRY(taperb.alloc((size_t)(nx + nz) * 8, total));
        PSV_TRY(ctl.alloc(4 * sizeof(int), total));
        PSV_TRY(ctl2.alloc(2 * MAXCH * sizeof(int), total));
        PSV_CU(cudaMemsetAsync(ctl2.p, 0, 2 * MAXCH * sizeof(int), st));
        PSV_CU(cudaMemsetAsync(ctl.p, 0, 4 * sizeof(int), st));
        PSV_TRY(scales.alloc((size_t)4 * nshot * 8, total));
        {
            std::vector<double> one((size_t)3 * nshot, 1.0);
            PSV_CU(cudaMemcpyAsync(scales.p, one.data(), one.size() * 8, cudaMemcpyHostToDevice, st));
        }
        PSV_CU(cudaMemsetAsync(model.p, 0, model.bytes, st));
        PSV_CU(cudaMemsetAsync(fld.p, 0, fld.bytes, st));
        PSV_CU(cudaMemsetAsync(coef.p, 0, coef.bytes, st));
        PSV_CU(cudaMemsetAsync(fsb.p, 0, fsb.bytes, st));
        PSV_CU(cudaMemsetAsync(traces.p, 0, traces.bytes, st));
        PSV_CU(cudaMemcpyAsync(ctl.p, h_ctl, 2 * sizeof(int), cudaMemcpyHostToDevice, st));

        PSV_TRY(upload_profiles());
        PSV_TRY(upload_sources());
        PSV_TRY(upload_taper());
        fill_params();
        PSV_TRY(encode_maps());
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    static int tma_rpt(int r) { return (r == 2 || r == 4 || r == 8) ? r : 4; }
    static int fused_tz(int r) { return (r == 16 || r == 32) ? r : 32; }
    bool fused_ok(int tz) const
    {
        return sizeof(T) == 4 && fused_supported(sv.ns, tz, sv.st, sv.sb, sv.sl, sv.sr, sv.nz1);
    }
    // Field planes per shot: FP32 plans hold the second vz..sxx copy of the
    // fused step; the working (recompute) state has 5 planes, 10 in FP32.
    static constexpr int nfield() { return sizeof(T) == 4 ? NFIELD_PP : NFIELD; }
    static constexpr int nwork() { return sizeof(T) == 4 ? 10 : 5; }
    static int march_rows(int r) { return (r == 32 || r == 64 || r == 128) ? r : 64; }
    static int march_stage(int w) { return (w == 2 || w == 4) ? w : 4; }
    bool march_ok(int rows, int warps) const
    {
        return sizeof(T) == 4 &&
               march_supported(sv.ns, rows, warps, sv.st, sv.sb, sv.sl, sv.sr, sv.nz1);
    }
    // One launch per step, v and sigma ping-ponged (FUSED tiles or MARCH strips).
    bool fused() const { return fam == PSV_KERNELS_FUSED || fam == PSV_KERNELS_MARCH; }
    // Copy of v and sigma a step reads: step k of a pass reads copy k & 1
    // (the fused family ping-pongs; the others update in place, copy 0).
    int par(int k) const { return fused() ? (k & 1) : 0; }
    static int v4_rpt(int r) { return (r == 1 || r == 2 || r == 4) ? r : 1; }

    // Tensor maps of the field blocks for the TMA family (rebuilt when the
    // tile height or a field buffer changes).
    int encode_maps()
    {
        if constexpr (sizeof(T) == 4) {
            const psv_grid &g = sv.g;
            if (fam == PSV_KERNELS_MARCH) {
                PSV_TRY(encode_march_maps(&mmap, fld.as<float>(), (int)(B * nfield()), g.nx, g.nz,
                                          pitch, plane, sv.ns, (int)blk.y));
                if (fld2.p)
                    PSV_TRY(encode_march_maps(&mmap2, fld2.as<float>(), B * nwork(), g.nx, g.nz,
                                              pitch, plane, sv.ns, (int)blk.y));
                return PSV_OK;
            }
            if (fam != PSV_KERNELS_TMA) return PSV_OK;
            PSV_TRY(encode_tile_maps(&tmap, fld.as<float>(), (int)(B * nfield()), coef.as<float>(),
                                     g.nx, g.nz, pitch, plane, sv.ns, rpt));
            if (fld2.p)
                PSV_TRY(encode_tile_maps(&tmap2, fld2.as<float>(), B * nwork(), coef.as<float>(), g.nx,
                                         g.nz, pitch, plane, sv.ns, rpt));
        }
        return PSV_OK;
    }

    // One stress / velocity launch of the current kernel family; `second`
    // selects the checkpoint recompute state.
    cudaError_t ks(const StepParams<T> &s, bool second, int nb = 0, cudaStream_t sm = nullptr)
    {
        if (nb) return launch_stress<T>(s, sv.ns, rpt, blk, nb, sm);  // a chain: direct family
        if constexpr (sizeof(T) == 4) {
            if (fam == PSV_KERNELS_TMA)
                return launch_stress_tma(s, second ? tmap2 : tmap, sv.ns, rpt, B, st);
            if (fam == PSV_KERNELS_VEC4) return launch_stress_v4(s, sv.ns, rpt, (int)blk.y, B, st);
        }
        (void)second;
        return launch_stress<T>(s, sv.ns, rpt, blk, B, st);
    }
    cudaError_t kv(const StepParams<T> &s, const SrcRecParams<T> &q, int mode, int it, int slot,
                   bool second, int nb = 0, cudaStream_t sm = nullptr)
    {
        if (nb) return launch_velocity<T>(s, q, sv.ns, mode, it, slot, rpt, blk, nb, sm);
        if constexpr (sizeof(T) == 4) {
            if (fam == PSV_KERNELS_TMA)
                return launch_velocity_tma(s, q, second ? tmap2 : tmap, sv.ns, mode, it, slot, rpt,
                                           B, st);
            if (fam == PSV_KERNELS_VEC4)
                return launch_velocity_v4(s, q, sv.ns, mode, it, slot, rpt, (int)blk.y, B, st);
        }
        (void)second;
        return launch_velocity<T>(s, q, sv.ns, mode, it, slot, rpt, blk, B, st);
    }

    // One time step: the family's stress and velocity launches, or the fused
    // launch reading copy `pr` of v and sigma and writing the other.
    cudaError_t step(const StepParams<T> &s, const SrcRecParams<T> &q, int mode, int it, int slot,
                     bool second, int pr)
    {
        if constexpr (sizeof(T) == 4)
            if (fam == PSV_KERNELS_MARCH)
                return launch_step_march(s, q, second ? mmap2 : mmap, sv.ns, mode, it, slot, pr, rpt,
                                         (int)blk.y, B, st);
            else if (fused())
                return launch_step_fused(s, q, sv.ns, mode, it, slot, pr, rpt, B, st);
        cudaError_t e = ks(s, second);
        if (e != cudaSuccess) return e;
        return kv(s, q, mode, it, slot, second);
    }
    long long lps() const { return fused() ? 1 : 2; }  // launches per step

    // Parameters of chain k (slots [k h, k h + h), h = ceil(B / chains)):
    // base pointers moved to the chain's first slot, its own control block.
    StepParams<T> chain_view(const StepParams<T> &s, int k) const
    {
        StepParams<T> v = s;
        v.ctl = ctl2.as<int>() + 2 * k;
        const long long o = (long long)k * ((B + chains - 1) / chains);
        v.fld += o * s.shot_stride;
        if (v.memz) v.memz += o * s.mz_shot_stride;
        if (v.memx) v.memx += o * s.mx_shot_stride;
        if (v.hist) v.hist += o * s.hist_shot_stride;
        if (v.gshot) v.gshot += o * s.gshot_shot_stride;
        return v;
    }
    int chain_n(int k) const
    {
        const int h = (B + chains - 1) / chains;
        return std::max(0, std::min(h, B - k * h));
    }
    // Chains apply to the direct family's passes; checkpointed passes join
    // them around every copy of the batch's states.
    bool chained() const { return chains > 1 && fam == PSV_KERNELS_DIRECT; }
    cudaStream_t chain_stream(int k) const { return k ? stc[k] : st; }

    // The time loop of one pass over chains: fork from the plan's stream,
    // each chain's steps on its stream, join.
    // Steps it of state s over the chains (fork from the plan's stream, each
    // group's steps on its stream, join): its[j] for j < nstep, snapshot slot
    // slot_of(it).
    template <typename ItFn, typename SlotFn>
    int chained_steps(const StepParams<T> &s, const SrcRecParams<T> &q, int mode, int nstep,
                      ItFn it_of, SlotFn slot_of, bool second, long long &nk)
    {
        StepParams<T> v[MAXCH];
        for (int k = 0; k < chains; k++) v[k] = chain_view(s, k);
        PSV_CU(cudaEventRecord(evf, st));
        for (int k = 1; k < chains; k++) PSV_CU(cudaStreamWaitEvent(stc[k], evf, 0));
        for (int j = 0; j < nstep; j++) {
            const int it = it_of(j), slot = slot_of(it);
            for (int k = 0; k < chains; k++) {
                const int n = chain_n(k);
                if (n <= 0) continue;
                PSV_CU(ks(v[k], second, n, chain_stream(k)));
                PSV_CU(kv(v[k], q, mode, it, slot, second, n, chain_stream(k)));
                nk += 2;
            }
        }
        for (int k = 1; k < chains; k++) {
            PSV_CU(cudaEventRecord(evj[k], stc[k]));
            PSV_CU(cudaStreamWaitEvent(st, evj[k], 0));
        }
        return PSV_OK;
    }

    int enqueue_chained(const SrcRecParams<T> &q, int mode, bool adj, bool store, long long &nk,
                        int nsteps = -1)
    {
        const int nt = sv.g.nt, sdt = sv.g.snap_dt, ring = ckpt ? nslots : sv.snt;
        return chained_steps(
            sp, q, mode, nsteps < 0 ? nt : nsteps, [&](int j) { return adj ? nt - 1 - j : j; },
            [&](int it) { return (!(it % sdt) && (store || adj)) ? (it / sdt) % ring : -1; }, false,
            nk);
    }

    // Wait for the stream, then fail if a time-step kernel gave up a bounded
    // wait (device error word).
    int sync_check()
    {
        PSV_CU(cudaMemcpyAsync(h_err, ctl.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
        PSV_CU(cudaStreamSynchronize(st));
        if (*h_err) {
            *h_err = 0;
            PSV_CU(cudaMemsetAsync(ctl.as<int>() + 2, 0, sizeof(int), st));
            PSV_CU(cudaStreamSynchronize(st));
            return fail(PSV_ERR_CUDA, "time-step kernel: a tile copy did not complete in time");
        }
        return PSV_OK;
    }

    int upload_profiles()
    {
        const int nz = sv.g.nz, nx = sv.g.nx, nmax = std::max(nz, nx);
        std::vector<T> h((size_t)12 * nmax, T(0));
        for (int a = 0; a < 12; a++) {
            const bool zaxis = a < 6;
            const int n = zaxis ? nz : nx;
            const bool on = zaxis ? sv.g.pml_z : sv.g.pml_x;
            const int kind = a % 6;  // a b K a_half b_half K_half
            for (int i = 0; i < n; i++) {
                double v;
                if (on) v = sv.prof[a][i];
                else v = (kind == 1 || kind == 2 || kind == 4 || kind == 5) ? 1.0 : 0.0;
                if (kind == 2 || kind == 5) v = 1.0 / v;  // store 1/K
                h[(size_t)a * nmax + i] = (T)v;
            }
        }
        PSV_CU(cudaMemcpyAsync(prof.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    // Forward sources grouped by the shot that fires them (vsrc2's
    // src_shot_to_fire test), the adjoint's receivers per shot, receiver cells.
    int upload_sources()
    {
        const int nshot = sv.s.nshot, nsrc = sv.s.nsrc, nrec = sv.s.nrec, nt = sv.g.nt;
        std::vector<int> off(nshot + 1, 0), pos, col, snap;
        for (int s = 0; s < nshot; s++) {
            for (int is = 0; is < nsrc; is++)
                if (sv.fire[is] == s) {
                    pos.push_back(sv.z_src[is] * pitch + sv.x_src[is]);
                    col.push_back(is);
                    snap.push_back(snap_cell(sv.z_src[is], sv.x_src[is]));
                }
            off[s + 1] = (int)pos.size();
        }
        h_f_off = off;
        PSV_TRY(put(f_off, off));
        PSV_TRY(put(f_pos, pos));
        src_list_col = col;
        PSV_TRY(put(f_col, col));
        PSV_TRY(put(f_snap, snap));
        std::vector<int> aoff(nshot + 1), apos, acol, asnap, rpos(nrec);
        for (int r = 0; r < nrec; r++) rpos[r] = sv.z_rec[r] * pitch + sv.x_rec[r];
        for (int s = 0; s < nshot; s++) {
            aoff[s] = s * nrec;
            for (int r = 0; r < nrec; r++) {
                apos.push_back(rpos[r]);
                acol.push_back(r);
                asnap.push_back(-1);
            }
        }
        aoff[nshot] = nshot * nrec;
        PSV_TRY(put(a_off, aoff));
        PSV_TRY(put(a_pos, apos));
        PSV_TRY(put(a_col, acol));
        PSV_TRY(put(a_snap, asnap));
        PSV_TRY(put(rec_pos, rpos));
        PSV_TRY(build_tile_index());
        // stf [nsrc][nt] -> [nt][nsrc]
        std::vector<double> h((size_t)2 * nt * std::max(nsrc, 1), 0.0);
        for (int is = 0; is < nsrc; is++)
            for (int it = 0; it < nt; it++) {
                h[(size_t)it * nsrc + is] = sv.stf_z[(size_t)is * nt + it];
                h[(size_t)nt * nsrc + (size_t)it * nsrc + is] = sv.stf_x[(size_t)is * nt + it];
            }
        PSV_TRY(stf.alloc(h.size() * 8, total));
        PSV_CU(cudaMemcpyAsync(stf.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    // Sources and receivers bucketed by the velocity kernel's tiles (direct
    // family: 32 columns x blk.y * |rpt| rows; TMA: 64 x 4 rpt; VEC4: 128 x
    // blk.y * rpt; FUSED: 64 x rpt; MARCH: 32 blk.y - fdorder x rpt), so each
    // block finds its own.
    int build_tile_index()
    {
        const int nshot = sv.s.nshot, nrec = sv.s.nrec;
        const bool tma = fam == PSV_KERNELS_TMA, v4 = fam == PSV_KERNELS_VEC4;
        const bool mr = fam == PSV_KERNELS_MARCH;
        const int tw = mr ? march_tile_width(sv.ns, (int)blk.y) : tma || fused() ? 64 : v4 ? 128 : 32;
        const int tz = tma ? 4 * rpt : fused() ? rpt : (int)blk.y * (rpt < 0 ? -rpt : rpt);
        const int ntx = (sv.g.nx + tw - 1) / tw, ntz = (sv.g.nz + tz - 1) / tz;
        const int nt_ = ntx * ntz;
        auto tile_of = [&](int z, int x) { return (z / tz) * ntx + x / tw; };
        std::vector<int> soff((size_t)nshot * (nt_ + 1), 0), sk;
        std::vector<std::vector<int>> b(nt_);
        for (int s_ = 0; s_ < nshot; s_++) {
            for (auto &v : b) v.clear();
            for (int j = h_f_off[s_]; j < h_f_off[s_ + 1]; j++) {
                const int is = src_list_col[j];
                b[tile_of(sv.z_src[is], sv.x_src[is])].push_back(j);
            }
            int *o = &soff[(size_t)s_ * (nt_ + 1)];
            for (int t = 0; t < nt_; t++) {
                o[t] = (int)sk.size();
                sk.insert(sk.end(), b[t].begin(), b[t].end());
            }
            o[nt_] = (int)sk.size();
        }
        std::vector<int> roff(nt_ + 1, 0), rr;
        for (auto &v : b) v.clear();
        for (int r = 0; r < nrec; r++) b[tile_of(sv.z_rec[r], sv.x_rec[r])].push_back(r);
        for (int t = 0; t < nt_; t++) {
            roff[t] = (int)rr.size();
            rr.insert(rr.end(), b[t].begin(), b[t].end());
        }
        roff[nt_] = (int)rr.size();
        ntiles = nt_;
        PSV_TRY(put(t_src_off, soff));
        PSV_TRY(put(t_src_k, sk));
        PSV_TRY(put(t_rec_off, roff));
        PSV_TRY(put(t_rec_r, rr));
        return PSV_OK;
    }

    int snap_cell(int iz, int ix) const
    {
        const psv_grid &g = sv.g;
        const int dz = iz - g.snap_z1, dx = ix - g.snap_x1;
        if (dz < 0 || iz > g.snap_z2 || dx < 0 || ix > g.snap_x2) return -1;
        if (dz % g.snap_dz || dx % g.snap_dx) return -1;
        return (dz / g.snap_dz) * snx_pitch + dx / g.snap_dx;
    }

    template <typename V> int put(DevMem &m, const std::vector<V> &v)
    {
        PSV_TRY(m.alloc(std::max<size_t>(v.size(), 1) * sizeof(V), total));
        if (!v.empty())
            PSV_CU(cudaMemcpyAsync(m.p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    // taper2's horizontal and vertical factors (src/cpu/n_kernel_lib_PSV.cpp:949-1009).
    int upload_taper()
    {
        const psv_grid &g = sv.g;
        const int nz = g.nz, nx = g.nx;
        const int t1 = g.taper[0], t2 = g.taper[1], b1 = g.taper[2], b2 = g.taper[3];
        const int l1 = g.taper[4], l2 = g.taper[5], r1 = g.taper[6], r2 = g.taper[7];
        const int tl = l2 - l1, trr = r1 - r2, tt = t2 - t1, tb = b1 - b2;
        const double PI_REF = 3.14159265;
        std::vector<double> h((size_t)nx + nz, 1.0);
        for (int ix = 0; ix < nx; ix++) {
            double f = 1.0;
            if (ix >= g.snap_x1 && ix < l1) f = 0.0;
            else if (ix >= l1 && ix < l2) f = 0.5 * (1.0 - cos(PI_REF * (ix - l1) / tl));
            else if (ix > r2 && ix < r1) f = 0.5 * (1.0 - cos(PI_REF * (r1 - ix) / trr));
            else if (ix >= r1 && ix <= g.snap_x2) f = 0.0;
            h[ix] = f;
        }
        for (int iz = 0; iz < nz; iz++) {
            double f = 1.0;
            if (iz >= g.snap_z1 && iz < t1) f = 0.0;
            else if (iz >= t1 && iz < t2) f = 0.5 * (1.0 - cos(PI_REF * (iz - t1) / tt));
            else if (iz > b2 && iz < b1) f = 0.5 * (1.0 - cos(PI_REF * (b1 - iz) / tb));
            else if (iz >= b1 && iz <= g.snap_z2) f = 0.0;
            h[(size_t)nx + iz] = f;
        }
        PSV_CU(cudaMemcpyAsync(taperb.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    void fill_params()
    {
        const psv_grid &g = sv.g;
        const int nz = g.nz, nx = g.nx, nmax = std::max(nz, nx);
        StepParams<T> &p = sp;
        p = StepParams<T>{};
        p.nz = nz; p.nx = nx; p.pitch = pitch;
        p.nz1 = sv.nz1; p.nz2 = sv.nz2; p.nx1 = sv.nx1; p.nx2 = sv.nx2;
        p.plane = plane; p.shot_stride = shot_stride;
        p.fld = fld.as<T>();
        const double dzi = 1.0 / g.dz, dxi = 1.0 / g.dx;
        for (int k = 0; k < 4; k++) {
            p.cz[k] = k < sv.ns ? (T)(dzi * g.hc[k + 1]) : T(0);
            p.cx[k] = k < sv.ns ? (T)(dxi * g.hc[k + 1]) : T(0);
        }
        p.dt = (T)g.dt;
        p.inv_dt = (T)(1.0 / g.dt);
        p.kimg = (T)(g.snap_dt * g.dt);
        p.pml_z = g.pml_z; p.pml_x = g.pml_x;
        p.pz0 = g.pml_z ? sv.pz0 : 0; p.pz1 = g.pml_z ? sv.pz1 : nz;
        p.px0 = g.pml_x ? sv.px0 : 0; p.px1 = g.pml_x ? sv.px1 : nx;
        p.mx_pitch = mx_pitch;
        p.mz_plane = (long long)nzs * pitch; p.mz_shot_stride = mz_shot;
        p.mx_plane = (long long)nz * mx_pitch; p.mx_shot_stride = mx_shot;
        p.memz = memz.as<T>(); p.memx = memx.as<T>();
        const T *pr = prof.as<T>();
        p.a_z = pr + 0 * nmax; p.b_z = pr + 1 * nmax; p.ki_z = pr + 2 * nmax;
        p.ah_z = pr + 3 * nmax; p.bh_z = pr + 4 * nmax; p.khi_z = pr + 5 * nmax;
        p.a_x = pr + 6 * nmax; p.b_x = pr + 7 * nmax; p.ki_x = pr + 8 * nmax;
        p.ah_x = pr + 9 * nmax; p.bh_x = pr + 10 * nmax; p.khi_x = pr + 11 * nmax;
        T *c = coef.as<T>();
        p.c_lam = c; p.c_l2m = c + plane; p.c_muzx = c + 2 * plane; p.c_rz = c + 3 * plane;
        p.c_rx = c + 4 * plane; p.g1 = c + 5 * plane; p.g2 = c + 6 * plane;
        p.st = sv.st; p.sb = sv.sb; p.sl = sv.sl; p.sr = sv.sr;
        T *fs = fsb.as<T>();
        p.fs_top = fs; p.fs_bot = fs + nx; p.fs_left = fs + 2 * nx; p.fs_right = fs + 2 * nx + nz;
        p.snap_z1 = g.snap_z1; p.snap_z2 = g.snap_z2; p.snap_x1 = g.snap_x1; p.snap_x2 = g.snap_x2;
        p.snap_dz = g.snap_dz; p.snap_dx = g.snap_dx;
        p.snz = sv.snz; p.snx = sv.snx; p.snx_pitch = snx_pitch;
        p.snap_plane = (long long)sv.snz * snx_pitch;
        p.hist_slot_stride = NHIST * p.snap_plane;
        p.hist_shot_stride = hist_shot;
        p.hist = hist.as<T>();
        p.gshot = gshot.as<T>();
        p.gshot_shot_stride = gshot_shot;
        p.ctl = ctl.as<int>();
        p.err = ctl.as<int>() + 2;
        p.nbatch = B;

        SrcRecParams<T> q{};
        q.src_off = f_off.as<int>(); q.src_pos = f_pos.as<int>(); q.src_col = f_col.as<int>();
        q.src_snap = f_snap.as<int>();
        q.stf_z = stf.as<double>();
        q.stf_x = stf.as<double>() + (size_t)g.nt * sv.s.nsrc;
        q.stf_shot_stride = 0; q.stf_ncol = sv.s.nsrc; q.stf_type = sv.s.stf_type;
        q.inv_dzdx = 1.0 / (g.dz * g.dx);
        q.nrec = sv.s.nrec; q.rec_pos = rec_pos.as<int>();
        q.rtf_z = sv.s.rtf_type == 0 ? tr(0) : nullptr;
        q.rtf_x = sv.s.rtf_type == 0 ? tr(1) : nullptr;
        q.rtf_shot_stride = ntr;
        q.dt_d = g.dt; q.dzdx = g.dz * g.dx; q.nt = g.nt;
        q.amp_scale = fscale(); q.rec_unscale = funscale();
        q.src_kind = 0; q.ntiles = ntiles;
        q.t_src_off = t_src_off.as<int>(); q.t_src_k = t_src_k.as<int>();
        q.t_rec_off = t_rec_off.as<int>(); q.t_rec_r = t_rec_r.as<int>();
        qf = q;
        qk = q;  // drop-in adjoint: the caller's sources, no recording
        qk.rtf_z = qk.rtf_x = nullptr;
        qa = q;  // FWI adjoint: residuals fired at the receivers (adjoint call, n_simulate_PSV.cpp:344-356)
        qa.src_off = a_off.as<int>(); qa.src_pos = a_pos.as<int>(); qa.src_col = a_col.as<int>();
        qa.src_snap = a_snap.as<int>();
        qa.stf_z = tr(4); qa.stf_x = tr(5);
        qa.stf_shot_stride = ntr; qa.stf_ncol = sv.s.nrec; qa.stf_type = sv.s.rtf_type;
        qa.rtf_z = qa.rtf_x = nullptr;
        qa.amp_scale = ascale();
        qa.src_kind = 1;
        qr = qf;  // recomputed forward: sources and snapshot fix-ups, no recording
        qr.rtf_z = qr.rtf_x = nullptr;
        sp.pp_planes = sizeof(T) == 4 ? NFIELD : 0;
        sp2 = sp;  // recompute state: 5 planes per shot (10 in FP32) and its own CPML strips
        sp2.shot_stride = nwork() * plane;
        sp2.pp_planes = sizeof(T) == 4 ? 5 : 0;
    }

    int ensure_hist()
    {
        if (hist.p || hist_shot == 0) return PSV_OK;
        PSV_TRY(hist.alloc((size_t)B * hist_shot * sizeof(T), total));
        sp.hist = hist.as<T>();
        if (ckpt) {
            PSV_TRY(ck.alloc((size_t)nck * B * ck_state * sizeof(T), total));
            PSV_TRY(fld2.alloc((size_t)B * nwork() * plane * sizeof(T), total));
            PSV_TRY(memz2.alloc((size_t)B * mz_shot * sizeof(T), total));
            PSV_TRY(memx2.alloc((size_t)B * mx_shot * sizeof(T), total));
            // padding columns are read by the fused step's staging copies
            PSV_CU(cudaMemsetAsync(fld2.p, 0, fld2.bytes, st));
            sp2.fld = fld2.as<T>();
            sp2.memz = memz2.as<T>();
            sp2.memx = memx2.as<T>();
        }
        sp2.hist = hist.as<T>();
        PSV_TRY(encode_maps());
        drop_graphs();
        return PSV_OK;
    }

    // Copy the batch's forward state between checkpoint slot j and the main
    // state (CK_SAVE_MAIN) or the working state (CK_SAVE_WORK, CK_RESTORE),
    // taking v and sigma from / to copy pr.  The CPML strips are copied
    // whole (both copies of the ping-ponged memories).
    int ck_copy(int j, int op, int pr, cudaStream_t cs = nullptr)
    {
        const cudaStream_t st = cs ? cs : this->st;
        T *c = ck.as<T>() + (size_t)j * B * ck_state;
        const size_t cp = (size_t)ck_state * sizeof(T);
        const bool main = op == CK_SAVE_MAIN, save = op != CK_RESTORE;
        T *f = main ? fld.as<T>() + (size_t)pr * sp.pp_planes * plane
                    : fld2.as<T>() + (size_t)pr * sp2.pp_planes * plane;
        const size_t fp = (size_t)(main ? shot_stride : nwork() * plane) * sizeof(T);
        T *mz = main ? memz.as<T>() : memz2.as<T>();
        T *mx = main ? memx.as<T>() : memx2.as<T>();
        const size_t w = (size_t)5 * plane * sizeof(T);
        if (save) PSV_CU(cudaMemcpy2DAsync(c, cp, f, fp, w, B, cudaMemcpyDeviceToDevice, st));
        else PSV_CU(cudaMemcpy2DAsync(f, fp, c, cp, w, B, cudaMemcpyDeviceToDevice, st));
        if (mz_shot) {
            const size_t zw = (size_t)mz_shot * sizeof(T);
            if (save) PSV_CU(cudaMemcpy2DAsync(c + 5 * plane, cp, mz, zw, zw, B, cudaMemcpyDeviceToDevice, st));
            else PSV_CU(cudaMemcpy2DAsync(mz, zw, c + 5 * plane, cp, zw, B, cudaMemcpyDeviceToDevice, st));
        }
        if (mx_shot) {
            const size_t xw = (size_t)mx_shot * sizeof(T);
            T *cx = c + 5 * plane + mz_shot;
            if (save) PSV_CU(cudaMemcpy2DAsync(cx, cp, mx, xw, xw, B, cudaMemcpyDeviceToDevice, st));
            else PSV_CU(cudaMemcpy2DAsync(mx, xw, cx, cp, xw, B, cudaMemcpyDeviceToDevice, st));
        }
        return PSV_OK;
    }

    // The adjoint pass of a checkpointed plan: the schedule's actions in
    // order; returns the time-step launches enqueued through nk.
    int run_schedule(long long &nk)
    {
        const int nt = sv.g.nt, sdt = sv.g.snap_dt;
        for (const CkAction &x : sched.bwd) {
            const int a = x.seg * K, e = std::min(a + K, nt);
            // the working state of forward step it is copy par(it) (as in the
            // forward pass); adjoint step it is step nt - 1 - it of its pass
            if (x.op == CK_RESTORE || x.op == CK_SAVE_WORK) {
                PSV_TRY(ck_copy(x.slot, x.op, par(a)));
            } else if (x.op == CK_ADVANCE && chained()) {
                PSV_TRY(chained_steps(
                    sp2, qr, MODE_FWD_NOWE, e - a, [&](int j) { return a + j; },
                    [](int) { return -1; }, true, nk));
            } else if (x.op == CK_ADVANCE) {
                for (int it = a; it < e; it++)
                    PSV_CU(step(sp2, qr, MODE_FWD_NOWE, it, -1, true, par(it)));
                nk += lps() * (e - a);
            } else if (x.op == CK_REVERSE && chained()) {
                const int base = (a + sdt - 1) / sdt, last = (e - 1) / sdt * sdt;
                auto slot_of = [&](int it) { return !(it % sdt) ? it / sdt - base : -1; };
                PSV_TRY(chained_steps(
                    sp2, qr, MODE_FWD_NOWE, std::max(last - a + 1, 0),
                    [&](int j) { return a + j; }, slot_of, true, nk));
                PSV_TRY(chained_steps(
                    sp, qa, MODE_ADJ, e - a, [&](int j) { return e - 1 - j; }, slot_of, false,
                    nk));
            } else if (x.op == CK_REVERSE) {
                // recompute up to the segment's last snapshot step into the
                // segment buffer, then the segment's adjoint steps
                const int base = (a + sdt - 1) / sdt, last = (e - 1) / sdt * sdt;
                for (int it = a; it <= last; it++) {
                    const int slot = !(it % sdt) ? it / sdt - base : -1;
                    PSV_CU(step(sp2, qr, MODE_FWD_NOWE, it, slot, true, par(it)));
                }
                for (int it = e - 1; it >= a; it--) {
                    const int slot = !(it % sdt) ? it / sdt - base : -1;
                    PSV_CU(step(sp, qa, MODE_ADJ, it, slot, false, par(nt - 1 - it)));
                }
                nk += lps() * (std::max(last - a + 1, 0) + e - a);
            }
        }
        return PSV_OK;
    }

    void drop_graphs()
    {
        for (auto &g : gx)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    }

    // ----------------------------------------------------------- time loop
    int enqueue(int kind)
    {
        const int nt = sv.g.nt, sdt = sv.g.snap_dt;
        const bool adj = kind == PASS_ADJ_RES || kind == PASS_ADJ_GIVEN;
        const bool store = kind == PASS_FWD_STORE || (kind == PASS_FWD_U && store_flag);
        const int mode = kind == PASS_FWD_STORE ? MODE_FWD
                         : kind == PASS_FWD_PLAIN ? MODE_FWD_NOWE
                         : kind == PASS_FWD_U ? MODE_FWD_U : MODE_ADJ;
        const SrcRecParams<T> &q = kind == PASS_ADJ_RES ? qa : kind == PASS_ADJ_GIVEN ? qk : qf;
        T *f = fld.as<T>();
        const long long n0 = nlaunch;
        // reset_sv2 / reset_PML_memory2 / reset_grad_shot2 (n_kernel_PSV.cpp:74-88)
        if (fused())  // the second copy of v and sigma
            PSV_CU(launch_zero_planes<T>(f, shot_stride, (long long)NFIELD * plane, 5 * plane, B, st));
        if (mode == MODE_ADJ) {
            PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, 7 * plane, B, st));
            PSV_CU(launch_zero_planes<T>(f, shot_stride, F_WEA * plane, plane, B, st));
            PSV_CU(launch_zero_planes<T>(gshot.as<T>(), gshot_shot, 0, gshot_shot, B, st));
        } else if (mode == MODE_FWD_U) {
            PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, 8 * plane, B, st));
        } else {
            PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, 5 * plane, B, st));
            if (mode == MODE_FWD)
                PSV_CU(launch_zero_planes<T>(f, shot_stride, F_WE * plane, plane, B, st));
        }
        PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
        PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
        long long nk = (mode == MODE_ADJ ? 5 : mode == MODE_FWD ? 4 : 3);
        if (ckpt && kind == PASS_FWD_STORE && chained()) {
            // one segment at a time: its state saved, then its steps on the chains
            for (int a = 0; a < nt; a += K) {
                if (fwd_slot[(size_t)(a / K)] >= 0)
                    PSV_TRY(ck_copy(fwd_slot[(size_t)(a / K)], CK_SAVE_MAIN, par(a)));
                PSV_TRY(chained_steps(
                    sp, qf, mode, std::min(K, nt - a), [&](int j) { return a + j; },
                    [](int) { return -1; }, false, nk));
            }
        } else if (ckpt && kind == PASS_FWD_STORE) {
            // forward saving the schedule's states at the starts of their segments
            for (int it = 0; it < nt; it++) {
                if (!(it % K) && fwd_slot[(size_t)(it / K)] >= 0)
                    PSV_TRY(ck_copy(fwd_slot[(size_t)(it / K)], CK_SAVE_MAIN, par(it)));
                PSV_CU(step(sp, qf, mode, it, -1, false, par(it)));
            }
            nk += lps() * nt;
        } else if (ckpt && kind == PASS_ADJ_RES) {
            PSV_TRY(run_schedule(nk));
        } else if (chained()) {
            PSV_TRY(enqueue_chained(q, mode, adj, store, nk));
        } else {
            for (int jt = 0; jt < nt; jt++) {
                const int it = adj ? nt - 1 - jt : jt;
                const bool snap = !(it % sdt);
                PSV_CU(step(sp, q, mode, it, (snap && (store || adj)) ? it / sdt : -1, false, par(jt)));
            }
            nk += lps() * nt;
        }
        nlaunch = n0 + nk;
        return PSV_OK;
    }

    int run_pass(int kind)
    {
        const bool graphable = kind == PASS_FWD_STORE || kind == PASS_FWD_PLAIN || kind == PASS_ADJ_RES;
        if (!opt.use_graphs || !graphable) return enqueue(kind);
        if (!gx[kind]) {
            cudaGraph_t graph = nullptr;
            PSV_CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const long long n0 = nlaunch;
            const int s = enqueue(kind);
            gx_nodes[kind] = nlaunch - n0;
            nlaunch = n0;
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            if (s != PSV_OK) {
                if (graph) cudaGraphDestroy(graph);
                return s;
            }
            if (e != cudaSuccess) return fail(PSV_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&gx[kind], graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                gx[kind] = nullptr;
                return fail(PSV_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            }
        }
        PSV_CU(cudaGraphLaunch(gx[kind], st));
        nlaunch += gx_nodes[kind];
        return PSV_OK;
    }

    // Group sizes of `k` chains over the batch slots (ceil(B / k) slots each,
    // the last ones possibly short or empty) and their control blocks.
    int set_chains(int k)
    {
        chains = std::max(1, std::min(k, (int)MAXCH));
        while (chains > B) chains /= 2;  // 4 -> 2 -> 1: at least one shot a group
        const int h = (B + chains - 1) / chains;
        for (int b = 0; b < nbatch; b++) {
            const int n = std::min(B, sv.s.nshot - b * B);
            for (int c = 0; c < MAXCH; c++) {
                h_ctl2[(b * MAXCH + c) * 2] = b * B + c * h;
                h_ctl2[(b * MAXCH + c) * 2 + 1] = c < chains ? std::max(0, std::min(h, n - c * h)) : 0;
            }
        }
        drop_graphs();
        return PSV_OK;
    }

    int set_batch(int b)
    {
        PSV_CU(cudaMemcpyAsync(ctl.p, h_ctl + 2 * b, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(ctl2.p, h_ctl2 + 2 * MAXCH * b, 2 * MAXCH * sizeof(int),
                               cudaMemcpyHostToDevice, st));
        return PSV_OK;
    }

    // --------------------------------------------------------------- model
    int coefficients(bool sums, bool given_avg)
    {
        CoeffParams<T> c{};
        c.nz = sv.g.nz; c.nx = sv.g.nx; c.pitch = pitch;
        c.dt = sv.g.dt; c.kimg = (double)sv.g.snap_dt * sv.g.dt; c.gscale = gscale;
        c.lam = lam(); c.mu = mu(); c.rho = rho();
        if (given_avg) { c.mu_zx = avg(0); c.rho_zp = avg(1); c.rho_xp = avg(2); }
        c.c_lam = (T *)sp.c_lam; c.c_l2m = (T *)sp.c_l2m; c.c_muzx = (T *)sp.c_muzx;
        c.c_rz = (T *)sp.c_rz; c.c_rx = (T *)sp.c_rx; c.g1 = (T *)sp.g1; c.g2 = (T *)sp.g2;
        c.st = sv.st; c.sb = sv.sb; c.sl = sv.sl; c.sr = sv.sr;
        c.fs_top = (T *)sp.fs_top; c.fs_bot = (T *)sp.fs_bot;
        c.fs_left = (T *)sp.fs_left; c.fs_right = (T *)sp.fs_right;
        PSV_CU(launch_coeffs<T>(c, st));
        if (sums) {
            PSV_CU(launch_model_sums(lam(), mu(), rho(), sv.g.nz, sv.g.nx, partial(), cavg(), st));
            double h[3];
            PSV_CU(cudaMemcpyAsync(h, cavg(), sizeof(h), cudaMemcpyDeviceToHost, st));
            PSV_CU(cudaStreamSynchronize(st));
            const double cnt = (double)((sv.g.nz - 1) * (sv.g.nx - 1));
            for (int k = 0; k < 3; k++) C[k] = h[k] / cnt;
        }
        return PSV_OK;
    }

    static double pow2_near(double x) { return (x > 0 && std::isfinite(x)) ? std::exp2(-std::rint(std::log2(x))) : 1.0; }

    // Range scales from a host model: forward source gain (exact powers of two).
    void model_scales(const double *l, const double *m, double inv_rho_max)
    {
        const psv_grid &g = sv.g;
        const size_t n = (size_t)g.nz * g.nx;
        inj = g.dt / (g.dz * g.dx) * inv_rho_max;
        double amax = 0.0;
        for (double v : sv.stf_z) amax = std::max(amax, std::fabs(v));
        for (double v : sv.stf_x) amax = std::max(amax, std::fabs(v));
        const double sf = pow2_near(sv.s.stf_type == 0 ? amax * inj : amax);
        // imaging factor: g1 * (dt (lam + 2 mu) / dz)^2 ~ 1 with unit-scaled fields
        double g1max = 0.0, cmax = 0.0;
        const double kimg = (double)g.snap_dt * g.dt;
        for (size_t k = 0; k < n; k++) {
            const double lm = l[k] + m[k];
            if (lm > 0) g1max = std::max(g1max, kimg * 0.25 / (lm * lm));
            cmax = std::max(cmax, g.dt * (l[k] + 2.0 * m[k]) / std::min(g.dz, g.dx));
        }
        gscale = pow2_near(g1max * cmax * cmax);
        std::vector<double> h((size_t)2 * sv.s.nshot);
        for (int s_ = 0; s_ < sv.s.nshot; s_++) { h[s_] = sf; h[sv.s.nshot + s_] = 1.0 / sf; }
        cudaMemcpyAsync(fscale(), h.data(), h.size() * 8, cudaMemcpyHostToDevice, st);
    }

    int set_model(const double *l, const double *m, const double *r) override
    {
        const size_t n = (size_t)sv.g.nz * sv.g.nx;
        double rmin = 0.0;
        for (size_t k = 0; k < n; k++)
            if (r[k] > 1e-4 && (rmin == 0.0 || r[k] < rmin)) rmin = r[k];
        model_scales(l, m, rmin > 0 ? 1.0 / rmin : 1.0);
        PSV_CU(cudaMemcpyAsync(lam(), l, n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(mu(), m, n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(rho(), r, n * 8, cudaMemcpyHostToDevice, st));
        PSV_TRY(coefficients(true, false));
        have_model = true;
        return PSV_OK;
    }

    int get_model(double *l, double *m, double *r) override
    {
        const size_t n = (size_t)sv.g.nz * sv.g.nx;
        if (l) PSV_CU(cudaMemcpyAsync(l, lam(), n * 8, cudaMemcpyDeviceToHost, st));
        if (m) PSV_CU(cudaMemcpyAsync(m, mu(), n * 8, cudaMemcpyDeviceToHost, st));
        if (r) PSV_CU(cudaMemcpyAsync(r, rho(), n * 8, cudaMemcpyDeviceToHost, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    // Host traces [nshot][nrec][nt] <-> device [nshot][nt][nrec] through the
    // residual buffer used as staging.
    int upload_traces(double *dst, const double *src)
    {
        const int nshot = sv.s.nshot;
        PSV_CU(cudaMemcpyAsync(tr(4), src, (size_t)nshot * ntr * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(launch_transpose(tr(4), dst, sv.s.nrec, sv.g.nt, nshot, st));
        return PSV_OK;
    }

    int download_traces(double *dst, const double *src, int s0, int n)
    {
        PSV_CU(launch_transpose(src + (size_t)s0 * ntr, tr(5), sv.g.nt, sv.s.nrec, n, st));
        PSV_CU(cudaMemcpyAsync(dst, tr(5), (size_t)n * ntr * 8, cudaMemcpyDeviceToHost, st));
        return PSV_OK;
    }

    int set_observed(const double *uz, const double *ux) override
    {
        if (sv.s.nrec == 0) return fail(PSV_ERR_ARG, "survey has no receivers");
        PSV_TRY(upload_traces(tr(2), uz));
        PSV_TRY(upload_traces(tr(3), ux));
        PSV_CU(cudaStreamSynchronize(st));
        have_obs = true;
        return PSV_OK;
    }

    // ------------------------------------------------------------ drivers
    int forward(double *uz, double *ux) override
    {
        if (!have_model) return fail(PSV_ERR_ARG, "forward: no model set");
        PSV_CU(cudaEventRecord(ev[0], st));
        for (int b = 0; b < nbatch; b++) {
            PSV_TRY(set_batch(b));
            PSV_TRY(run_pass(PASS_FWD_PLAIN));
        }
        PSV_CU(cudaEventRecord(ev[1], st));
        if (uz && sv.s.nrec) PSV_TRY(download_traces(uz, tr(0), 0, sv.s.nshot));
        if (ux && sv.s.nrec) PSV_TRY(download_traces(ux, tr(1), 0, sv.s.nshot));
        PSV_TRY(sync_check());
        float ms = 0;
        PSV_CU(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        t_ms[0] = ms; t_ms[1] = 0; t_ms[2] = 0;
        return PSV_OK;
    }

    // Forward + residual + adjoint + preconditioning of every shot
    // (src/cpu/n_simulate_PSV.cpp:270-419), batch by batch in shot order.
    int gradient(double *L2) override
    {
        if (!have_model || !have_obs) return fail(PSV_ERR_ARG, "gradient: model and observed traces required");
        if (opt.adjoint == PSV_ADJOINT_EXACT) return exact_gradient(L2);
        PSV_TRY(ensure_hist());
        PSV_TRY(maybe_autotune());
        PSV_TRY(coefficients(true, false));
        const int nshot = sv.s.nshot;
        double tf = 0, ta = 0, to = 0;
        for (int b = 0; b < nbatch; b++) {
            const int s0 = b * B, n = std::min(B, nshot - s0);
            PSV_TRY(set_batch(b));
            last_batch_s0 = s0;
            PSV_CU(cudaEventRecord(ev[0], st));
            PSV_TRY(run_pass(PASS_FWD_STORE));
            PSV_CU(cudaEventRecord(ev[1], st));
            PSV_CU(launch_adjsrc(tr(0) + s0 * ntr, tr(1) + s0 * ntr, tr(2) + s0 * ntr,
                                 tr(3) + s0 * ntr, tr(4) + s0 * ntr, tr(5) + s0 * ntr, ntr, n,
                                 sv.g.dt, partial(), L2dev() + s0, st));
            PSV_CU(launch_adjoint_scale(tr(4) + s0 * ntr, tr(5) + s0 * ntr, ntr, n, inj,
                                        rmax() + s0, ascale() + s0, st));
            PSV_CU(cudaEventRecord(ev[2], st));
            PSV_TRY(run_pass(PASS_ADJ_RES));
            PSV_CU(cudaEventRecord(ev[3], st));
            if (opt.smooth_hfs >= 2) PSV_TRY(smooth_shot_gradients(n));
            PSV_TRY(precondition(n));
            PSV_TRY(sync_check());
            float a, c, d;
            PSV_CU(cudaEventElapsedTime(&a, ev[0], ev[1]));
            PSV_CU(cudaEventElapsedTime(&c, ev[1], ev[2]));
            PSV_CU(cudaEventElapsedTime(&d, ev[2], ev[3]));
            tf += a; to += c; ta += d;
            last_s0 = s0;
            last_n = n;
        }
        L2_shot.assign(nshot, 0.0);
        PSV_CU(cudaMemcpy(L2_shot.data(), L2dev(), nshot * 8, cudaMemcpyDeviceToHost));
        double s = 0.0;
        for (int i = 0; i < nshot; i++) s += L2_shot[i];
        if (L2) *L2 = s;
        t_ms[0] = tf; t_ms[1] = ta; t_ms[2] = to;
        return PSV_OK;
    }

    // apply_gauss_filter of the n batch shots' gradient planes (the
    // reference's commented-out calls, n_simulate_PSV.cpp:377-379).
    int smooth_shot_gradients(int n)
    {
        const int hfs = opt.smooth_hfs;
        if (!gfilt.p) {
            std::vector<double> k((size_t)(2 * hfs + 1) * (2 * hfs + 1));
            PSV_TRY(psv_gauss_filter_kernel(hfs, k.data()));
            PSV_TRY(gfilt.alloc(k.size() * sizeof(double), total));
            PSV_CU(cudaMemcpy(gfilt.p, k.data(), k.size() * sizeof(double), cudaMemcpyHostToDevice));
            PSV_TRY(gtmp.alloc((size_t)B * gshot_shot * sizeof(T), total));
        }
        const size_t bytes = (size_t)n * gshot_shot * sizeof(T);
        PSV_CU(cudaMemcpyAsync(gtmp.p, gshot.p, bytes, cudaMemcpyDeviceToDevice, st));
        PSV_CU(launch_gauss_filter<T>(gtmp.as<T>(), gshot.as<T>(), sp.snap_plane, snx_pitch, sv.snz,
                                      sv.snx, 3 * n, gfilt.as<double>(), hfs, st));
        return PSV_OK;
    }

    // PCG_PSV x3 on the global gradients (n_simulate_PSV.cpp:433-435).
    int pcg_gradient() override
    {
        const long long n = (long long)sv.g.nz * sv.g.nx;
        if (!pcgbuf.p) {
            PSV_TRY(pcgbuf.alloc((size_t)6 * n * sizeof(double), total));
            PSV_TRY(pcgpart.alloc(2 * PCG_BLOCKS * sizeof(double), total));
            PSV_CU(cudaMemsetAsync(pcgbuf.p, 0, pcgbuf.bytes, st));
        }
        double *d = pcgbuf.as<double>();
        for (int k = 0; k < 3; k++)
            PSV_CU(launch_pcg(d + (size_t)k * n, d + (size_t)(3 + k) * n, grad(k), n,
                              pcgpart.as<double>(), st));
        return PSV_OK;
    }

    // energy_weights2 + interpol_grad2 + scale_grad_E2 (n_simulate_PSV.cpp:385-417).
    int precondition(int n)
    {
        const psv_grid &g = sv.g;
        PSV_CU(cudaMemsetAsync(wmax(), 0, B * 8, st));
        PSV_CU(launch_energy_max<T>(fld.as<T>(), plane, shot_stride, pitch, g.snap_z1, g.snap_z2,
                                    g.snap_x1, g.snap_x2, n, wmax(), st));
        ScaleParams<T> s{};
        s.nz = g.nz; s.nx = g.nx; s.pitch = pitch;
        s.z1 = g.snap_z1; s.z2 = g.snap_z2; s.x1 = g.snap_x1; s.x2 = g.snap_x2;
        s.sdz = g.snap_dz; s.sdx = g.snap_dx; s.snx_pitch = snx_pitch;
        s.snap_plane = sp.snap_plane;
        s.gshot = gshot.as<T>(); s.gshot_shot_stride = gshot_shot;
        s.fld = fld.as<T>(); s.plane = plane; s.shot_stride = shot_stride;
        s.wmax = wmax();
        s.fscale = fscale(); s.ascale = ascale(); s.s0 = last_batch_s0;
        const double sg = sv.g.imaging_sign > 0 ? -1.0 : 1.0;  // kernels accumulate the CPU sign
        s.gun[0] = s.gun[1] = sg / gscale; s.gun[2] = sg;
        for (int k = 0; k < 3; k++) { s.C[k] = C[k]; s.grad[k] = grad(k); }
        s.nbatch = n;
        PSV_CU(launch_scale<T>(s, st));
        return PSV_OK;
    }

    // Exact discrete adjoint (psv_exact.cu): a forward pass storing the
    // CPML-corrected derivatives of every step, residual and L2 (adjsrc2), the
    // transposed steps in reverse time, then the chain rule into the global
    // gradients as -imaging_sign * dL2/dm.  Batch by batch in shot order, one
    // launch sequence per step (no graphs: verification-sized grids).
    int exact_gradient(double *L2)
    {
        if constexpr (sizeof(T) != 8) {
            (void)L2;
            return fail(PSV_ERR_UNSUPPORTED, "exact adjoint: FP64 plans only");
        } else {
            const psv_grid &g = sv.g;
            const int nt = g.nt, nshot = sv.s.nshot;
            PSV_TRY(coefficients(true, false));
            const size_t store_b = (size_t)nt * B * 8 * plane * sizeof(double);
            const size_t work_b = (size_t)B * EXACT_WORK_PLANES * plane * sizeof(double);
            const size_t q_b = (size_t)B * (mz_shot + mx_shot) * sizeof(double);
            if (!ex_store.p) {
                const double budget = (opt.hbm_budget_gb > 0 ? opt.hbm_budget_gb : 180.0) * 1e9;
                if ((double)total + store_b + work_b + q_b > budget)
                    return fail(PSV_ERR_OOM, "exact adjoint: the per-step derivatives (" +
                                                 std::to_string(store_b >> 20) + " MiB) exceed the "
                                                 "HBM budget; use fewer steps, shots per batch or "
                                                 "a smaller grid");
                PSV_TRY(ex_store.alloc(store_b, total));
                PSV_TRY(ex_work.alloc(work_b, total));
                PSV_TRY(ex_q.alloc(std::max<size_t>(q_b, 8), total));
            }
            ExactBufs X{};
            X.store = ex_store.as<double>();
            X.step_stride = (long long)B * 8 * plane;
            X.work = ex_work.as<double>();
            X.qz = ex_q.as<double>();
            X.qx = ex_q.as<double>() + (size_t)B * mz_shot;
            X.rsum_z = tr(4);
            X.rsum_x = tr(5);
            int maxsrc = 0;
            for (int s_ = 0; s_ < nshot; s_++) maxsrc = std::max(maxsrc, h_f_off[s_ + 1] - h_f_off[s_]);
            const double sign = sv.g.imaging_sign > 0 ? -1.0 : 1.0;
            double tf = 0, ta = 0;
            for (int b = 0; b < nbatch; b++) {
                const int s0 = b * B, n = std::min(B, nshot - s0);
                PSV_TRY(set_batch(b));
                PSV_CU(cudaEventRecord(ev[0], st));
                PSV_CU(launch_zero_planes<T>(fld.as<T>(), shot_stride, 0, shot_stride, B, st));
                PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
                PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
                for (int it = 0; it < nt; it++) {
                    PSV_CU(launch_exact_forward_step(sp, qf, X, sv.ns, it, B, maxsrc, st));
                    nlaunch += 2 + (maxsrc ? 1 : 0) + 1;
                }
                PSV_CU(cudaEventRecord(ev[1], st));
                PSV_CU(launch_adjsrc(tr(0) + s0 * ntr, tr(1) + s0 * ntr, tr(2) + s0 * ntr,
                                     tr(3) + s0 * ntr, tr(4) + s0 * ntr, tr(5) + s0 * ntr, ntr, n,
                                     g.dt, partial(), L2dev() + s0, st));
                PSV_CU(launch_exact_revsum(tr(4) + s0 * ntr, tr(5) + s0 * ntr, nt, sv.s.nrec, ntr,
                                           g.dt, g.dt / (g.dz * g.dx), n, st));
                PSV_CU(cudaMemsetAsync(ex_work.p, 0, work_b, st));
                PSV_CU(cudaMemsetAsync(ex_q.p, 0, ex_q.bytes, st));
                int sin = EX_SB0, sout = EX_SB1;
                for (int it = nt - 1; it >= 0; it--) {
                    PSV_CU(launch_exact_adjoint_step(sp, qf, X, sv.ns, it, sin, sout, B, maxsrc, st));
                    nlaunch += 4 + 1 + (maxsrc ? 1 : 0);
                    std::swap(sin, sout);
                }
                PSV_CU(launch_exact_chain(sp, X, lam(), mu(), rho(), grad(0), grad(1), grad(2), g.dt,
                                          sign, st));
                PSV_CU(cudaEventRecord(ev[2], st));
                PSV_TRY(sync_check());
                float a, c;
                PSV_CU(cudaEventElapsedTime(&a, ev[0], ev[1]));
                PSV_CU(cudaEventElapsedTime(&c, ev[1], ev[2]));
                tf += a;
                ta += c;
                last_s0 = s0;
                last_n = n;
            }
            L2_shot.assign(nshot, 0.0);
            PSV_CU(cudaMemcpy(L2_shot.data(), L2dev(), nshot * 8, cudaMemcpyDeviceToHost));
            double s = 0.0;
            for (int i = 0; i < nshot; i++) s += L2_shot[i];
            if (L2) *L2 = s;
            t_ms[0] = tf; t_ms[1] = ta; t_ms[2] = 0;
            return PSV_OK;
        }
    }

    int get_gradient(double *gl, double *gm, double *gr) override
    {
        const size_t n = (size_t)sv.g.nz * sv.g.nx;
        double *o[3] = {gl, gm, gr};
        for (int k = 0; k < 3; k++)
            if (o[k]) PSV_CU(cudaMemcpyAsync(o[k], grad(k), n * 8, cudaMemcpyDeviceToHost, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    int set_gradient(const double *gl, const double *gm, const double *gr) override
    {
        const size_t n = (size_t)sv.g.nz * sv.g.nx;
        const double *in[3] = {gl, gm, gr};
        for (int k = 0; k < 3; k++)
            if (in[k]) PSV_CU(cudaMemcpyAsync(grad(k), in[k], n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    int reset_gradient() override
    {
        PSV_CU(cudaMemsetAsync(grad(0), 0, (size_t)3 * sv.g.nz * sv.g.nx * 8, st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    int get_shot(int ishot, double *gl, double *gm, double *gr, double *We, double *WeA,
                 double *uz, double *ux, double *L2) override
    {
        if (opt.adjoint == PSV_ADJOINT_EXACT)
            return fail(PSV_ERR_UNSUPPORTED, "get_shot_gradient: the exact adjoint has no per-shot "
                                             "imaging terms");
        if (ishot < last_s0 || ishot >= last_s0 + last_n)
            return fail(PSV_ERR_ARG, "get_shot_gradient: shot not in the last gradient batch");
        const int b = ishot - last_s0;
        const psv_grid &g = sv.g;
        double sf = 1, sa = 1;
        PSV_CU(cudaMemcpy(&sf, fscale() + ishot, 8, cudaMemcpyDeviceToHost));
        PSV_CU(cudaMemcpy(&sa, ascale() + ishot, 8, cudaMemcpyDeviceToHost));
        const double sg = sv.g.imaging_sign > 0 ? -1.0 : 1.0;
        const double gun[3] = {sg / (gscale * sf * sa), sg / (gscale * sf * sa), sg / (sf * sa)};
        std::vector<T> h((size_t)gshot_shot);
        PSV_CU(cudaMemcpy(h.data(), gshot.as<T>() + b * gshot_shot, h.size() * sizeof(T),
                          cudaMemcpyDeviceToHost));
        double *o[3] = {gl, gm, gr};
        for (int k = 0; k < 3; k++)
            if (o[k])
                for (int jz = 0; jz < sv.snz; jz++)
                    for (int jx = 0; jx < sv.snx; jx++)
                        o[k][(size_t)jz * sv.snx + jx] =
                            (double)h[k * sp.snap_plane + (size_t)jz * snx_pitch + jx] * gun[k];
        double *w[2] = {We, WeA};
        const int wp[2] = {F_WE, F_WEA};
        const double wun[2] = {1.0 / (sf * sf), 1.0 / (sa * sa)};
        std::vector<T> pl((size_t)plane);
        for (int k = 0; k < 2; k++) {
            if (!w[k]) continue;
            PSV_CU(cudaMemcpy(pl.data(), fld.as<T>() + b * shot_stride + wp[k] * plane,
                              plane * sizeof(T), cudaMemcpyDeviceToHost));
            for (int iz = 0; iz < g.nz; iz++)
                for (int ix = 0; ix < g.nx; ix++)
                    w[k][(size_t)iz * g.nx + ix] = (double)pl[(size_t)iz * pitch + ix] * wun[k];
        }
        if (uz) PSV_TRY(download_traces(uz, tr(0), ishot, 1));
        if (ux) PSV_TRY(download_traces(ux, tr(1), ishot, 1));
        PSV_CU(cudaStreamSynchronize(st));
        if (L2) *L2 = L2_shot.empty() ? 0.0 : L2_shot[ishot];
        return PSV_OK;
    }

    // ---------------------------------------------------------- FWI step
    // Trial forward of every shot for a candidate step (step_length_PSV's
    // inner loop, src/cpu/n_step_length_PSV.cpp:87-123).
    int trial(double est, double *L2)
    {
        const int n = sv.g.nz * sv.g.nx;
        unsigned long long *mb = maxbits();
        PSV_CU(launch_update_mat(lam(), lamc(), grad(0), n, 4.8e+10, 0.0, est, mb, st));
        PSV_CU(launch_update_mat(mu(), muc(), grad(1), n, 2.7e+10, 0.0, est, mb, st));
        PSV_CU(launch_update_mat(rho(), rhoc(), grad(2), n, 3000.0, 1.5, 0.5 * est, mb, st));
        PSV_TRY(coefficients(false, false));
        for (int b = 0; b < nbatch; b++) {
            const int s0 = b * B, nb = std::min(B, sv.s.nshot - s0);
            PSV_TRY(set_batch(b));
            PSV_TRY(run_pass(PASS_FWD_PLAIN));
            PSV_CU(launch_adjsrc(tr(0) + s0 * ntr, tr(1) + s0 * ntr, tr(2) + s0 * ntr,
                                 tr(3) + s0 * ntr, nullptr, nullptr, ntr, nb, sv.g.dt, partial(),
                                 L2dev() + s0, st));
        }
        std::vector<double> h(sv.s.nshot);
        PSV_CU(cudaMemcpyAsync(h.data(), L2dev(), h.size() * 8, cudaMemcpyDeviceToHost, st));
        PSV_TRY(sync_check());
        double s = 0.0;
        for (double v : h) s += v;
        *L2 = s;
        return PSV_OK;
    }

    // copy_mat (n_simulate_PSV.cpp:263): the model the trials and the update start from.
    int save_model() override
    {
        const size_t n = (size_t)sv.g.nz * sv.g.nx;
        PSV_CU(cudaMemcpyAsync(lamc(), lam(), n * 8, cudaMemcpyDeviceToDevice, st));
        PSV_CU(cudaMemcpyAsync(muc(), mu(), n * 8, cudaMemcpyDeviceToDevice, st));
        PSV_CU(cudaMemcpyAsync(rhoc(), rho(), n * 8, cudaMemcpyDeviceToDevice, st));
        return PSV_OK;
    }

    // taper2 x3 (n_simulate_PSV.cpp:443-450).
    int taper_gradient() override
    {
        for (int k = 0; k < 3; k++)
            PSV_CU(launch_taper(grad(k), sv.g.nz, sv.g.nx, taperb.as<double>(),
                                taperb.as<double>() + sv.g.nx, st));
        return PSV_OK;
    }

    // update_mat2 x3 from the saved model (n_simulate_PSV.cpp:542-546).
    int update_model(double step) override
    {
        const int ni = sv.g.nz * sv.g.nx;
        PSV_CU(launch_update_mat(lam(), lamc(), grad(0), ni, 4.8e+10, 0.0, step, maxbits(), st));
        PSV_CU(launch_update_mat(mu(), muc(), grad(1), ni, 2.7e+10, 0.0, step, maxbits(), st));
        PSV_CU(launch_update_mat(rho(), rhoc(), grad(2), ni, 3000.0, 1.25, 0.5 * step, maxbits(), st));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    int trial_misfit(double step, double *L2) override
    {
        if (!have_model || !have_obs) return fail(PSV_ERR_ARG, "trial: model and observed traces required");
        return trial(step, L2);
    }

    int fwi_iteration(double *step, double *L2out, int *ntrials, double *tlog, int maxt) override
    {
        if (!have_model || !have_obs) return fail(PSV_ERR_ARG, "fwi_iteration: model and observed traces required");
        PSV_TRY(save_model());
        double L2 = 0;
        PSV_TRY(gradient(&L2));
        if (L2out) *L2out = L2;
        PSV_CU(cudaEventRecord(ev[0], st));
        if (opt.pcg) PSV_TRY(pcg_gradient());
        PSV_TRY(taper_gradient());
        // step_length_PSV (src/cpu/n_step_length_PSV.cpp:53-209), update_param 0.
        double est = *step;
        auto fn = [](double a, double *L, void *ctx) -> int {
            return static_cast<Plan<T> *>(ctx)->trial(a, L);
        };
        const int rc = psv_step_length(&est, L2, fn, this, ntrials, tlog, maxt);
        if (rc != PSV_OK) return rc;
        *step = est;
        PSV_TRY(update_model(est));
        PSV_CU(cudaEventRecord(ev[1], st));
        PSV_CU(cudaStreamSynchronize(st));
        float ms = 0;
        PSV_CU(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        t_ms[2] += ms;
        return PSV_OK;
    }

    int timing(double *ms3) const override
    {
        for (int k = 0; k < 3; k++) ms3[k] = t_ms[k];
        return PSV_OK;
    }

    // Switch the stencil kernels' tile shape (rebuilds the per-tile source
    // index, drops captured graphs).
    int set_shape(int f, int r, int by)
    {
        if (f >= PSV_KERNELS_TMA && sizeof(T) != 4) f = PSV_KERNELS_DIRECT;
        if (f == PSV_KERNELS_FUSED && !fused_ok(fused_tz(r))) f = PSV_KERNELS_DIRECT;
        if (f == PSV_KERNELS_MARCH && !march_ok(march_rows(r), march_stage(by))) f = PSV_KERNELS_DIRECT;
        r = f == PSV_KERNELS_TMA     ? tma_rpt(r)
            : f == PSV_KERNELS_VEC4  ? v4_rpt(r)
            : f == PSV_KERNELS_FUSED ? fused_tz(r)
            : f == PSV_KERNELS_MARCH ? march_rows(r)
                                     : rpt_ok<T>(r);
        if (f == PSV_KERNELS_TMA) by = 4;
        if (f == PSV_KERNELS_FUSED) by = (int)blk.y;  // unused
        if (f == PSV_KERNELS_MARCH) by = march_stage(by);
        if (f != PSV_KERNELS_MARCH && (by < 1 || by > 8)) by = 4;
        if (f == fam && r == rpt && (int)blk.y == by) return PSV_OK;
        fam = f;
        rpt = r;
        blk = dim3(32, by, 1);
        PSV_TRY(build_tile_index());
        qf.t_src_off = qr.t_src_off = qk.t_src_off = qa.t_src_off = t_src_off.as<int>();
        qf.t_src_k = qr.t_src_k = qk.t_src_k = qa.t_src_k = t_src_k.as<int>();
        qf.t_rec_off = qr.t_rec_off = qk.t_rec_off = qa.t_rec_off = t_rec_off.as<int>();
        qf.t_rec_r = qr.t_rec_r = qk.t_rec_r = qa.t_rec_r = t_rec_r.as<int>();
        qf.ntiles = qr.ntiles = qk.ntiles = qa.ntiles = ntiles;
        PSV_TRY(encode_maps());
        drop_graphs();
        return PSV_OK;
    }

    int autotune(int nsteps, int *out_fam, int *out_rpt, int *out_by) override
    {
        const TuneKey key{sv.g.nz, sv.g.nx, sv.ns, B, (int)sizeof(T), opt.kernel_family};
        auto report = [&] {
            if (out_fam) *out_fam = fam;
            if (out_rpt) *out_rpt = rpt;
            if (out_by) *out_by = (int)blk.y;
        };
        {
            std::lock_guard<std::mutex> lk(tune_mutex());
            auto it = tune_cache().find(key);
            if (it != tune_cache().end()) {
                PSV_TRY(set_shape(std::get<0>(it->second), std::get<1>(it->second),
                                  std::get<2>(it->second)));
                if (opt.chains == 0) PSV_TRY(set_chains(chain_cache()[key]));
                tuned = true;
                report();
                return PSV_OK;
            }
        }
        // candidates: direct loads (rows per thread x block height), TMA tiles (rows per thread)
        std::vector<std::tuple<int, int, int>> cand;
        if (opt.kernel_family == 0 || opt.kernel_family == PSV_KERNELS_DIRECT) {
            const int r32[] = {1, 2, 4, -2, -4};
            for (int r : r32) {
                if (sizeof(T) == 8 && r != 1) continue;
                for (int by : {2, 4, 8}) cand.emplace_back(PSV_KERNELS_DIRECT, r, by);
            }
        }
        if (sizeof(T) == 4 && (opt.kernel_family == 0 || opt.kernel_family == PSV_KERNELS_TMA))
            for (int r : {2, 4, 8}) cand.emplace_back(PSV_KERNELS_TMA, r, 4);
        if (sizeof(T) == 4 && (opt.kernel_family == 0 || opt.kernel_family == PSV_KERNELS_VEC4))
            for (int r : {1, 2, 4})
                for (int by : {2, 4, 8}) cand.emplace_back(PSV_KERNELS_VEC4, r, by);
        if (opt.kernel_family == 0 || opt.kernel_family == PSV_KERNELS_FUSED)
            for (int tz : {16, 32})
                if (fused_ok(tz)) cand.emplace_back(PSV_KERNELS_FUSED, tz, (int)blk.y);
        if (opt.kernel_family == 0 || opt.kernel_family == PSV_KERNELS_MARCH)
            for (int rows : {32, 64, 128})
                for (int w : {2, 4})
                    if (march_ok(rows, w)) cand.emplace_back(PSV_KERNELS_MARCH, rows, w);
        // 1) every candidate, launch by launch with CUDA events
        std::vector<std::pair<double, std::tuple<int, int, int>>> timed;
        for (auto &c : cand) {
            PSV_TRY(set_shape(std::get<0>(c), std::get<1>(c), std::get<2>(c)));
            double ms[6];
            PSV_TRY(profile(nsteps, ms));
            timed.emplace_back(ms[0] + ms[1] + ms[3] + ms[4], std::make_tuple(fam, rpt, (int)blk.y));
        }
        std::sort(timed.begin(), timed.end(),
                  [](const auto &a, const auto &b) { return a.first < b.first; });
        // 2) the three fastest again as graph-replayed bursts of forward +
        // adjoint steps, the way the passes run, with 1, 2 and 4 chains for
        // the direct family (chaining can reorder them)
        std::tuple<int, int, int> pick = timed.empty() ? std::make_tuple(fam, rpt, (int)blk.y)
                                                       : timed.front().second;
        int ck = chains;
        double tb = 1e30;
        for (size_t i = 0; i < std::min<size_t>(3, timed.size()); i++) {
            const auto &sh = timed[i].second;
            PSV_TRY(set_shape(std::get<0>(sh), std::get<1>(sh), std::get<2>(sh)));
            const bool chainable = opt.chains == 0 && fam == PSV_KERNELS_DIRECT && B >= 2;
            for (int k : {1, 2, 4}) {
                if (chainable ? k > B : k != 1) continue;
                double t = 0;
                PSV_TRY(time_chains(nsteps, chainable ? k : chains, &t));
                if (t < tb) {
                    tb = t;
                    pick = sh;
                    ck = chainable ? k : chains;
                }
            }
        }
        PSV_TRY(set_shape(std::get<0>(pick), std::get<1>(pick), std::get<2>(pick)));
        PSV_TRY(set_chains(ck));
        {
            std::lock_guard<std::mutex> lk(tune_mutex());
            tune_cache()[key] = pick;
            chain_cache()[key] = ck;
        }
        tuned = true;
        report();
        return PSV_OK;
    }

    int chain_count() const override { return chained() ? chains : 1; }

    void storage(int *kind, int *segment_steps, int *slots, long long *advances) const override
    {
        if (kind) *kind = store_kind;
        if (segment_steps) *segment_steps = ckpt ? K : 0;
        if (slots) *slots = ckpt ? nck : 0;
        if (advances) *advances = ckpt ? sched.advances : 0;
    }

    void shape(int *f, int *r, int *by) const override
    {
        if (f) *f = fam;
        if (r) *r = rpt;
        if (by) *by = fam == PSV_KERNELS_TMA ? 4 : fam == PSV_KERNELS_FUSED ? 0 : (int)blk.y;
    }

    int prepare() override
    {
        if (!have_model || !have_obs) return PSV_OK;
        PSV_TRY(ensure_hist());
        return maybe_autotune();
    }

    int batches() const override { return nbatch; }

    int joint_begin(int r, int by, int batch, void *entry, size_t bytes,
                    std::vector<JointOp> *ops) override
    {
        if (bytes != sizeof(JointSurvey<T>))
            return fail(PSV_ERR_ARG, "joint launch: every plan of one precision");
        if (!have_model) return fail(PSV_ERR_ARG, "joint launch: a plan has no model");
        if (batch < 0 || batch >= nbatch) return fail(PSV_ERR_ARG, "joint launch: no such shot batch");
        PSV_TRY(set_shape(PSV_KERNELS_DIRECT, r, by));
        if (fam != PSV_KERNELS_DIRECT || rpt != r || (int)blk.y != by)
            return fail(PSV_ERR_ARG, "joint launch: unsupported tile shape");
        PSV_TRY(set_batch(batch));
        // reset_sv2 / reset_PML_memory2 (n_kernel_PSV.cpp:74-88), as the plain forward pass
        T *f = fld.as<T>();
        PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, 5 * plane, B, st));
        PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
        PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
        joint_entry(entry, r, by);
        ops->clear();
        for (int it = 0; it < sv.g.nt; it++) ops->push_back(joint_step(0, 0, MODE_FWD_NOWE, it, -1));
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    int joint_end(double *uz, double *ux) override
    {
        if (uz && sv.s.nrec) PSV_TRY(download_traces(uz, tr(0), 0, sv.s.nshot));
        if (ux && sv.s.nrec) PSV_TRY(download_traces(ux, tr(1), 0, sv.s.nshot));
        return sync_check();
    }

    static JointOp joint_step(int state, int qsel, int mode, int it, int slot)
    {
        return JointOp{0, joint_flags(state, qsel, mode), it, slot, 0, 0, 0};
    }

    void joint_entry(void *entry, int r, int by) const
    {
        JointSurvey<T> &e = *static_cast<JointSurvey<T> *>(entry);
        e.p = sp;
        e.p2 = sp2;
        e.q[0] = qf;
        e.q[1] = qr;
        e.q[2] = qa;
        e.ops = nullptr;
        e.nops = 0;
        e.ns = sv.ns;
        e.nb = B;
        const int tz = by * r;
        e.sx = (sv.nx2 - sv.nx1 + 31) / 32;
        e.sy = (sv.nz2 - sv.nz1 + tz - 1) / tz;
        e.vx = (sv.g.nx + 31) / 32;
        e.vy = (sv.g.nz + tz - 1) / tz;
    }

    int joint_ck_copy(int slot, int op, int par, void *stream) override
    {
        return ck_copy(slot, op, par, (cudaStream_t)stream);
    }

    // The operations of the gradient's forward pass (enqueue, PASS_FWD_STORE):
    // steps with snapshots, or with checkpoint saves at segment starts.
    void joint_forward_ops(std::vector<JointOp> *ops) const
    {
        const int nt = sv.g.nt, sdt = sv.g.snap_dt;
        ops->clear();
        for (int it = 0; it < nt; it++) {
            if (ckpt && !(it % K) && fwd_slot[(size_t)(it / K)] >= 0)
                ops->push_back(JointOp{1, 0, 0, 0, fwd_slot[(size_t)(it / K)], CK_SAVE_MAIN, par(it)});
            const int slot = !ckpt && !(it % sdt) ? it / sdt : -1;
            ops->push_back(joint_step(0, 0, MODE_FWD, it, slot));
        }
    }

    // The operations of the adjoint pass (enqueue, PASS_ADJ_RES): reversed
    // steps with imaging, or the checkpoint schedule (run_schedule).
    void joint_adjoint_ops(std::vector<JointOp> *ops) const
    {
        const int nt = sv.g.nt, sdt = sv.g.snap_dt;
        ops->clear();
        if (!ckpt) {
            for (int jt = 0; jt < nt; jt++) {
                const int it = nt - 1 - jt;
                ops->push_back(joint_step(0, 2, MODE_ADJ, it, !(it % sdt) ? it / sdt : -1));
            }
            return;
        }
        for (const CkAction &x : sched.bwd) {
            const int a = x.seg * K, e = std::min(a + K, nt);
            if (x.op == CK_RESTORE || x.op == CK_SAVE_WORK) {
                ops->push_back(JointOp{1, 0, 0, 0, x.slot, x.op, par(a)});
            } else if (x.op == CK_ADVANCE) {
                for (int it = a; it < e; it++) ops->push_back(joint_step(1, 1, MODE_FWD_NOWE, it, -1));
            } else if (x.op == CK_REVERSE) {
                const int base = (a + sdt - 1) / sdt, last = (e - 1) / sdt * sdt;
                for (int it = a; it <= last; it++)
                    ops->push_back(joint_step(1, 1, MODE_FWD_NOWE, it, !(it % sdt) ? it / sdt - base : -1));
                for (int it = e - 1; it >= a; it--)
                    ops->push_back(joint_step(0, 2, MODE_ADJ, it, !(it % sdt) ? it / sdt - base : -1));
            }
        }
    }

    int joint_gradient_phase(int phase, int r, int by, int batch, void *entry, size_t bytes,
                             double *L2, std::vector<JointOp> *ops) override
    {
        T *f = fld.as<T>();
        const int s0 = batch * B, n = std::min(B, sv.s.nshot - s0);
        if (phase == 0) {
            if (bytes != sizeof(JointSurvey<T>))
                return fail(PSV_ERR_ARG, "joint launch: every plan of one precision");
            if (!have_model || !have_obs)
                return fail(PSV_ERR_ARG, "joint gradient: a plan without model or observed traces");
            if (opt.adjoint == PSV_ADJOINT_EXACT)
                return fail(PSV_ERR_UNSUPPORTED, "joint gradient: the reference-mode adjoint only");
            if (batch < 0 || batch >= nbatch) return fail(PSV_ERR_ARG, "joint launch: no such shot batch");
            if (batch == 0) {
                PSV_TRY(ensure_hist());
                PSV_TRY(coefficients(true, false));
            }
            PSV_TRY(set_shape(PSV_KERNELS_DIRECT, r, by));
            if (fam != PSV_KERNELS_DIRECT || rpt != r || (int)blk.y != by)
                return fail(PSV_ERR_ARG, "joint launch: unsupported tile shape");
            PSV_TRY(set_batch(batch));
            last_batch_s0 = s0;
            // the gradient forward pass's resets (enqueue, MODE_FWD)
            PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, 5 * plane, B, st));
            PSV_CU(launch_zero_planes<T>(f, shot_stride, F_WE * plane, plane, B, st));
            PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
            PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
            joint_entry(entry, r, by);
            joint_forward_ops(ops);
        } else if (phase == 1) {
            // residuals, L2 and adjoint sources (as gradient()), then the
            // adjoint pass's resets (enqueue, MODE_ADJ)
            PSV_CU(launch_adjsrc(tr(0) + s0 * ntr, tr(1) + s0 * ntr, tr(2) + s0 * ntr,
                                 tr(3) + s0 * ntr, tr(4) + s0 * ntr, tr(5) + s0 * ntr, ntr, n,
                                 sv.g.dt, partial(), L2dev() + s0, st));
            PSV_CU(launch_adjoint_scale(tr(4) + s0 * ntr, tr(5) + s0 * ntr, ntr, n, inj,
                                        rmax() + s0, ascale() + s0, st));
            PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, 7 * plane, B, st));
            PSV_CU(launch_zero_planes<T>(f, shot_stride, F_WEA * plane, plane, B, st));
            PSV_CU(launch_zero_planes<T>(gshot.as<T>(), gshot_shot, 0, gshot_shot, B, st));
            PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
            PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
            joint_entry(entry, r, by);
            joint_adjoint_ops(ops);
        } else {
            if (opt.smooth_hfs >= 2) PSV_TRY(smooth_shot_gradients(n));
            PSV_TRY(precondition(n));
            PSV_TRY(sync_check());
            last_s0 = s0;
            last_n = n;
            if (batch + 1 < nbatch) return PSV_OK;  // L2 after the last batch
            const int nshot = sv.s.nshot;
            L2_shot.assign(nshot, 0.0);
            PSV_CU(cudaMemcpy(L2_shot.data(), L2dev(), nshot * 8, cudaMemcpyDeviceToHost));
            double s = 0.0;
            for (int i = 0; i < nshot; i++) s += L2_shot[i];
            if (L2) *L2 = s;
            return PSV_OK;
        }
        PSV_CU(cudaStreamSynchronize(st));
        return PSV_OK;
    }

    int maybe_autotune()
    {
        if (tuned || !opt.autotune || !have_model || !have_obs) return PSV_OK;
        return autotune(std::min(24, sv.g.nt), nullptr, nullptr, nullptr);
    }

    void *stream() const override { return (void *)st; }
    int precision() const override { return (int)sizeof(T) * 8; }
    long long launches() const override { return nlaunch; }

    // Per-kernel event timing of nsteps forward then nsteps adjoint steps.
    // Device milliseconds of nsteps forward + nsteps adjoint steps of the
    // current shape with k chains (the autotuner's chain choice), replayed
    // as a CUDA graph like the passes themselves (direct launches would time
    // the host's launch rate instead).
    int time_chains(int nsteps, int k, double *ms)
    {
        PSV_TRY(set_chains(k));
        PSV_TRY(set_batch(0));
        T *f = fld.as<T>();
        PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, shot_stride, B, st));
        PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
        PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
        PSV_CU(cudaStreamSynchronize(st));
        long long nk = 0;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        PSV_CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = burst(nsteps, nk);
        const cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (rc != PSV_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return fail(PSV_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return fail(PSV_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        cudaError_t e = cudaGraphLaunch(exec, st);  // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(ev[0], st);
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
        if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaGraphExecDestroy(exec);
        if (e != cudaSuccess) return fail(PSV_ERR_CUDA, cudaGetErrorString(e));
        PSV_TRY(sync_check());
        float t = 0;
        PSV_CU(cudaEventElapsedTime(&t, ev[0], ev[1]));
        *ms = t;
        nlaunch += 2 * nk;
        return PSV_OK;
    }

    // nsteps forward and nsteps adjoint steps of the current schedule.
    int burst(int nsteps, long long &nk)
    {
        for (int pass = 0; pass < 2; pass++) {
            const bool adj = pass == 1;
            const SrcRecParams<T> &q = adj ? qa : qf;
            const int mode = adj ? MODE_ADJ : MODE_FWD;
            if (chained()) {
                PSV_TRY(enqueue_chained(q, mode, adj, true, nk, nsteps));
            } else {
                const int nt = sv.g.nt, sdt = sv.g.snap_dt;
                for (int j = 0; j < nsteps; j++) {
                    const int it = adj ? nt - 1 - j : j;
                    const int slot = !(it % sdt) ? (it / sdt) % (ckpt ? nslots : sv.snt) : -1;
                    PSV_CU(step(sp, q, mode, it, slot, false, par(j)));
                    nk += lps();
                }
            }
        }
        return PSV_OK;
    }

    int profile(int nsteps, double *ms6) override
    {
        if (!have_model || !have_obs) return fail(PSV_ERR_ARG, "profile: model and observed traces required");
        if (nsteps <= 0 || nsteps > sv.g.nt) return fail(PSV_ERR_ARG, "profile: nsteps must be in [1, nt]");
        PSV_TRY(ensure_hist());
        PSV_TRY(coefficients(true, false));
        PSV_TRY(set_batch(0));
        std::vector<cudaEvent_t> e((size_t)8 * nsteps, nullptr);
        for (auto &x : e) PSV_CU(cudaEventCreate(&x));
        const int nt = sv.g.nt, sdt = sv.g.snap_dt;
        T *f = fld.as<T>();
        PSV_CU(launch_zero_planes<T>(f, shot_stride, 0, shot_stride, B, st));
        PSV_CU(launch_zero_planes<T>(memz.as<T>(), mz_shot, 0, mz_shot, B, st));
        PSV_CU(launch_zero_planes<T>(memx.as<T>(), mx_shot, 0, mx_shot, B, st));
        int rc = PSV_OK;
        for (int pass = 0; pass < 2 && rc == PSV_OK; pass++) {
            const bool adj = pass == 1;
            const SrcRecParams<T> &q = adj ? qa : qf;
            for (int j = 0; j < nsteps; j++) {
                const int it = adj ? nt - 1 - j : j;
                const int slot = !(it % sdt) ? (it / sdt) % (ckpt ? nslots : sv.snt) : -1;
                cudaEvent_t *E = &e[(size_t)(pass * nsteps + j) * 4];
                // fused family: the whole step is timed in the velocity slot
                cudaEventRecord(E[0], st);
                cudaError_t c = fused() ? cudaSuccess : ks(sp, false);
                cudaEventRecord(E[1], st);
                if (c == cudaSuccess)
                    c = fused() ? step(sp, q, adj ? MODE_ADJ : MODE_FWD, it, slot, false, par(j))
                                : kv(sp, q, adj ? MODE_ADJ : MODE_FWD, it, slot, false);
                cudaEventRecord(E[2], st);
                cudaEventRecord(E[3], st);
                if (c != cudaSuccess) { rc = fail(PSV_ERR_CUDA, cudaGetErrorString(c)); break; }
                nlaunch += lps();
            }
        }
        if (rc == PSV_OK) rc = sync_check();
        for (int k = 0; k < 6; k++) ms6[k] = 0.0;
        if (rc == PSV_OK)
            for (int pass = 0; pass < 2; pass++)
                for (int j = 0; j < nsteps; j++) {
                    cudaEvent_t *E = &e[(size_t)(pass * nsteps + j) * 4];
                    for (int k = 0; k < 3; k++) {
                        float ms = 0;
                        cudaEventElapsedTime(&ms, E[k], E[k + 1]);
                        ms6[pass * 3 + k] += ms / nsteps;
                    }
                }
        for (auto &x : e) cudaEventDestroy(x);
        return rc;
    }

    // ------------------------------------------------------- drop-in call
    int kernel_call(const double *l, const double *m, const double *mzx, const double *rzp,
                    const double *rxp, int ishot, int grad_, int accu, double *const *accu_io,
                    double *const *fields_out, double *const *mem_out, double *rtf_uz,
                    double *rtf_ux, double *const *grad_out) override
    {
        (void)ishot;
        const psv_grid &g = sv.g;
        const int nz = g.nz, nx = g.nx;
        const size_t n = (size_t)nz * nx;
        PSV_CU(cudaMemcpyAsync(lam(), l, n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(mu(), m, n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(avg(0), mzx, n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(avg(1), rzp, n * 8, cudaMemcpyHostToDevice, st));
        PSV_CU(cudaMemcpyAsync(avg(2), rxp, n * 8, cudaMemcpyHostToDevice, st));
        double rzmax = 0.0;
        for (size_t k = 0; k < n; k++) rzmax = std::max(rzmax, std::max(std::fabs(rzp[k]), std::fabs(rxp[k])));
        model_scales(l, m, rzmax > 0 ? rzmax : 1.0);
        double sc = 1.0;  // amplitude scale of this call's wavefields
        PSV_CU(cudaMemcpy(&sc, fscale(), 8, cudaMemcpyDeviceToHost));
        if (grad_) {  // adjoint sources are the caller's: same rule as the forward gain
            const double h2[2] = {sc, 1.0 / sc};
            PSV_CU(cudaMemcpy(ascale(), h2, 8, cudaMemcpyHostToDevice));
            qk.amp_scale = ascale();
        }
        PSV_TRY(coefficients(false, true));
        PSV_TRY(set_batch(0));
        const long long snp = sp.snap_plane;
        const double un = 1.0 / sc;
        if (grad_ || accu) PSV_TRY(ensure_hist());
        if (grad_) {  // forward history in (gard_fwd_storage2 layout [snap_nt][snap_nz][snap_nx])
            std::vector<T> h((size_t)hist_shot, T(0));
            const int map[5] = {H_VZ, H_VX, H_SZZ, H_SZX, H_SXX};
            for (int k = 0; k < 5; k++)
                for (int t = 0; t < sv.snt; t++)
                    for (int jz = 0; jz < sv.snz; jz++)
                        for (int jx = 0; jx < sv.snx; jx++)
                            h[(size_t)t * NHIST * snp + map[k] * snp + (size_t)jz * snx_pitch + jx] =
                                (T)accu_io[k][((size_t)t * sv.snz + jz) * sv.snx + jx];
            PSV_CU(cudaMemcpyAsync(hist.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
            PSV_CU(cudaStreamSynchronize(st));
            PSV_TRY(run_pass(PASS_ADJ_GIVEN));
        } else {
            store_flag = accu != 0;
            PSV_TRY(run_pass(PASS_FWD_U));
            store_flag = false;
        }
        PSV_TRY(sync_check());
        // wavefields: vz vx uz ux szz szx sxx We
        std::vector<T> pl((size_t)shot_stride);
        PSV_CU(cudaMemcpy(pl.data(), fld.p, pl.size() * sizeof(T), cudaMemcpyDeviceToHost));
        // the pass's last step wrote copy par(nt) of v, sigma and the
        // stress-side CPML memories
        const int fp = par(g.nt), vo = fp * sp.pp_planes;
        const int fmap[8] = {F_VZ + vo, F_VX + vo, F_UZ, F_UX, F_SZZ + vo, F_SZX + vo, F_SXX + vo,
                             grad_ ? F_WEA : F_WE};
        for (int k = 0; k < 8; k++)
            if (fields_out[k])
                for (int iz = 0; iz < nz; iz++)
                    for (int ix = 0; ix < nx; ix++)
                        fields_out[k][(size_t)iz * nx + ix] =
                            (double)pl[fmap[k] * plane + (size_t)iz * pitch + ix] * (k == 7 ? un * un : un);
        // CPML memories: mem_vz_z mem_vx_z mem_szz_z mem_szx_z mem_vz_x mem_vx_x mem_szx_x mem_sxx_x
        std::vector<T> mz((size_t)std::max<long long>(mz_shot, 1)), mxv((size_t)std::max<long long>(mx_shot, 1));
        if (mz_shot) PSV_CU(cudaMemcpy(mz.data(), memz.p, mz_shot * sizeof(T), cudaMemcpyDeviceToHost));
        if (mx_shot) PSV_CU(cudaMemcpy(mxv.data(), memx.p, mx_shot * sizeof(T), cudaMemcpyDeviceToHost));
        for (int k = 0; k < 8; k++) {
            if (!mem_out[k]) continue;
            std::fill(mem_out[k], mem_out[k] + n, 0.0);
            for (int iz = 0; iz < nz; iz++)
                for (int ix = 0; ix < nx; ix++) {
                    if (k < 4 && nzs && (iz < sv.pz0 || iz >= sv.pz1)) {
                        const int r = iz < sv.pz0 ? iz : iz - sv.pz1 + sv.pz0;
                        const int pl = k + (k == MZ_VZ || k == MZ_VX ? fp * NMZ : 0);
                        mem_out[k][(size_t)iz * nx + ix] = (double)mz[(size_t)pl * nzs * pitch + (size_t)r * pitch + ix] * un;
                    } else if (k >= 4 && nxs && (ix < sv.px0 || ix >= sv.px1)) {
                        const int c = ix < sv.px0 ? ix : ix - sv.px1 + sv.px0;
                        const int pl = (k - 4) + (k - 4 == MX_VZ || k - 4 == MX_VX ? fp * NMX : 0);
                        mem_out[k][(size_t)iz * nx + ix] =
                            (double)mxv[(size_t)pl * nz * mx_pitch + (size_t)iz * mx_pitch + c] * un;
                    }
                }
        }
        const int nrec = sv.s.nrec, nt = g.nt;
        if (!grad_ && nrec && (rtf_uz || rtf_ux)) {
            std::vector<double> a((size_t)ntr), b((size_t)ntr);
            PSV_CU(cudaMemcpy(a.data(), tr(0), ntr * 8, cudaMemcpyDeviceToHost));
            PSV_CU(cudaMemcpy(b.data(), tr(1), ntr * 8, cudaMemcpyDeviceToHost));
            for (int r = 0; r < nrec; r++)
                for (int t = 0; t < nt; t++) {
                    if (rtf_uz) rtf_uz[(size_t)r * nt + t] = a[(size_t)t * nrec + r];
                    if (rtf_ux) rtf_ux[(size_t)r * nt + t] = b[(size_t)t * nrec + r];
                }
        }
        if (!grad_ && accu) {
            std::vector<T> h((size_t)hist_shot);
            PSV_CU(cudaMemcpy(h.data(), hist.p, h.size() * sizeof(T), cudaMemcpyDeviceToHost));
            const int map[5] = {H_VZ, H_VX, H_SZZ, H_SZX, H_SXX};
            for (int k = 0; k < 5; k++)
                if (accu_io[k])
                    for (int t = 0; t < sv.snt; t++)
                        for (int jz = 0; jz < sv.snz; jz++)
                            for (int jx = 0; jx < sv.snx; jx++)
                                accu_io[k][((size_t)t * sv.snz + jz) * sv.snx + jx] =
                                    (double)h[(size_t)t * NHIST * snp + map[k] * snp + (size_t)jz * snx_pitch + jx] * un;
        }
        if (grad_) {
            std::vector<T> h((size_t)gshot_shot);
            PSV_CU(cudaMemcpy(h.data(), gshot.p, h.size() * sizeof(T), cudaMemcpyDeviceToHost));
            for (int k = 0; k < 3; k++)
                if (grad_out[k])
                    for (int jz = 0; jz < sv.snz; jz++)
                        for (int jx = 0; jx < sv.snx; jx++)
                            grad_out[k][(size_t)jz * sv.snx + jx] =
                                (double)h[k * snp + (size_t)jz * snx_pitch + jx] * (k < 2 ? un / gscale : un) *
                                (g.imaging_sign > 0 ? -1.0 : 1.0);
        }
        return PSV_OK;
    }
};

template <typename T>
std::unique_ptr<PlanIface> make_plan_t(const Survey &sv, const psv_options &opt, int &status)
{
    std::unique_ptr<Plan<T>> p(new Plan<T>());
    status = p->init(sv, opt);
    if (status != PSV_OK) return nullptr;
    return std::unique_ptr<PlanIface>(p.release());
}

}  // namespace psv
