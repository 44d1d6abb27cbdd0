// psv_joint.cu -- forward modelling and FWI gradients of several surveys in
// one launch per half-step.
//
// A joint pass steps up to JOINT_MAX surveys (one plan each: any grid size,
// stencil order, step count and shot count) together: every joint step is
// one stress launch and one velocity launch whose blocks cover every shot of
// every survey still running.  The survey entries (JointSurvey: the plans'
// own step and source / receiver parameters) sit in constant memory; a
// launch carries only its joint step index and the segment it belongs to.
// Block b of a launch belongs to the survey whose first block is the last one
// <= b (a block-uniform scan of at most JOINT_MAX entries), reads that
// survey's step descriptor for the joint step (which state, which sources,
// velocity mode, the survey's own time step and snapshot slot) and runs the
// direct family's block body for the survey's stencil order
// (stress_block / velocity_block, psv_kernels_impl.cuh): each survey gets
// the operations of its own plan's direct launches.  The survey's parameters
// are read from constant memory instead of kernel arguments, and the
// compiler may contract multiply-adds differently in this context, so FP32
// results agree with the plan's own to rounding (not always bit for bit).
//
// A pass is each survey's list of operations (PlanIface::joint_begin,
// joint_gradient_phase): time steps, and for checkpointed gradients the
// schedule's state copies between them.  Joint step k runs every survey's
// k-th time step, after the copies its list puts before that step (enqueued
// per survey, ahead of the launch pair).  Uneven lists: the surveys sorted
// by step count split the joint steps into segments; segment g holds the
// surveys with more than its first step (their order and first blocks in
// c_seg[g]), and a survey leaves the launches after its last step.  Each
// pass (forward modelling, gradient forward, adjoint) is one CUDA graph,
// captured once per joint object and replayed.  Residuals, adjoint sources
// and preconditioning run per plan between and after the gradient passes.
#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>

#include "psv_kernels_impl.cuh"
#include "psv_plan.cuh"

namespace psv {

namespace {

// Segment tables: for each segment, its surveys (index into the entry table)
// and their first blocks in the stress and velocity grids.
struct JointSeg {
    int n;                  // surveys in the segment
    int idx[JOINT_MAX];     // entry of the j-th survey
    int s0[JOINT_MAX];      // its first stress block
    int v0[JOINT_MAX];      // its first velocity block
};

__constant__ JointSurvey<float> c_joint_f[JOINT_MAX];
__constant__ JointSurvey<double> c_joint_d[JOINT_MAX];
__constant__ JointSeg c_seg[JOINT_MAX];

template <typename T> __device__ __forceinline__ const JointSurvey<T> &joint_entry(int k);
template <> __device__ __forceinline__ const JointSurvey<float> &joint_entry<float>(int k)
{
    return c_joint_f[k];
}
template <> __device__ __forceinline__ const JointSurvey<double> &joint_entry<double>(int k)
{
    return c_joint_d[k];
}

// Position j in segment g of the survey owning block b (first blocks `first`).
__device__ __forceinline__ int joint_slot(const int *first, int n, int b)
{
    int j = 0;
#pragma unroll
    for (int k = 1; k < JOINT_MAX; k++)
        if (k < n && b >= first[k]) j = k;
    return j;
}

// Block b of a survey's grid of gx x gy blocks per shot: (shot, column, row).
__device__ __forceinline__ BlockPos joint_pos(int b, int gx, int gy)
{
    return {b / (gx * gy), b % gx, (b / gx) % gy, gx};
}

// The block bodies of stencil half-widths 1 .. NSMAX (2 or 4: the widest
// among the joint surveys), so surveys of orders up to 4 do not pay the
// registers of the order-8 body.
template <typename T, int RPT, int NSMAX>
__global__ void __launch_bounds__(256) k_joint_stress(const int g, const int k)
{
    const JointSeg &sg = c_seg[g];
    const int j = joint_slot(sg.s0, sg.n, (int)blockIdx.x);
    const JointSurvey<T> &e = joint_entry<T>(sg.idx[j]);
    const BlockPos bp = joint_pos((int)blockIdx.x - sg.s0[j], e.sx, e.sy);
    const int4 d = __ldg(e.ops + k);
    const StepParams<T> &p = (d.x & 1) ? e.p2 : e.p;
    if constexpr (NSMAX >= 4) {
        if (e.ns == 4) return stress_block<T, 4, RPT, false>(p, bp);
        if (e.ns == 3) return stress_block<T, 3, RPT, false>(p, bp);
    }
    if (e.ns == 2) return stress_block<T, 2, RPT, false>(p, bp);
    stress_block<T, 1, RPT, false>(p, bp);
}

template <typename T, int RPT, int NSMAX, int MODE>
__device__ __forceinline__ void joint_velocity_ns(int ns, const StepParams<T> &p,
                                                  const SrcRecParams<T> &q, int it, int slot,
                                                  const BlockPos bp)
{
    if constexpr (NSMAX >= 4) {
        if (ns == 4) return velocity_block<T, 4, MODE, RPT, false>(p, q, it, slot, bp);
        if (ns == 3) return velocity_block<T, 3, MODE, RPT, false>(p, q, it, slot, bp);
    }
    if (ns == 2) return velocity_block<T, 2, MODE, RPT, false>(p, q, it, slot, bp);
    velocity_block<T, 1, MODE, RPT, false>(p, q, it, slot, bp);
}

// Velocity step of joint step k.  MSEL: the one velocity mode of every
// survey's descriptor in the pass (MODE_FWD_NOWE forward modelling, MODE_FWD
// gradient forward, MODE_ADJ adjoint without checkpoints), or JOINT_MIXED:
// each survey's descriptor picks it (checkpointed adjoint passes, where
// recomputed segments run beside adjoint steps).
constexpr int JOINT_MIXED = -1;
template <typename T, int RPT, int NSMAX, int MSEL>
__global__ void __launch_bounds__(256) k_joint_velocity(const int g, const int k)
{
    const JointSeg &sg = c_seg[g];
    const int j = joint_slot(sg.v0, sg.n, (int)blockIdx.x);
    const JointSurvey<T> &e = joint_entry<T>(sg.idx[j]);
    const BlockPos bp = joint_pos((int)blockIdx.x - sg.v0[j], e.vx, e.vy);
    const int4 d = __ldg(e.ops + k);
    const StepParams<T> &p = (d.x & 1) ? e.p2 : e.p;
    const SrcRecParams<T> &q = e.q[(d.x >> 1) & 3];
    if constexpr (MSEL != JOINT_MIXED) {
        joint_velocity_ns<T, RPT, NSMAX, MSEL>(e.ns, p, q, d.y, d.z, bp);
    } else {
        const int mode = d.x >> 3;
        if (mode == MODE_ADJ) return joint_velocity_ns<T, RPT, NSMAX, MODE_ADJ>(e.ns, p, q, d.y, d.z, bp);
        if (mode == MODE_FWD) return joint_velocity_ns<T, RPT, NSMAX, MODE_FWD>(e.ns, p, q, d.y, d.z, bp);
        joint_velocity_ns<T, RPT, NSMAX, MODE_FWD_NOWE>(e.ns, p, q, d.y, d.z, bp);
    }
}

template <typename T, int RPT, int NSMAX, int MSEL>
void joint_pair(int g, int k, int sblocks, int vblocks, int by, cudaStream_t st)
{
    const dim3 blk(32, by, 1);
    k_joint_stress<T, RPT, NSMAX><<<sblocks, blk, 0, st>>>(g, k);
    k_joint_velocity<T, RPT, NSMAX, MSEL><<<vblocks, blk, 0, st>>>(g, k);
}

template <typename T, int RPT, int NSMAX>
void joint_pair_m(int g, int k, int sblocks, int vblocks, int by, int msel, cudaStream_t st)
{
    switch (msel) {
    case MODE_FWD: joint_pair<T, RPT, NSMAX, MODE_FWD>(g, k, sblocks, vblocks, by, st); break;
    case MODE_ADJ: joint_pair<T, RPT, NSMAX, MODE_ADJ>(g, k, sblocks, vblocks, by, st); break;
    default: joint_pair<T, RPT, NSMAX, MODE_FWD_NOWE>(g, k, sblocks, vblocks, by, st); break;
    }
}

// The mixed-mode kernel comes in the full-order instantiation only.
template <typename T, int RPT>
void joint_pair_r(int g, int k, int sblocks, int vblocks, int by, int nsmax, int msel, cudaStream_t st)
{
    if (msel == JOINT_MIXED) joint_pair<T, RPT, 4, JOINT_MIXED>(g, k, sblocks, vblocks, by, st);
    else if (nsmax <= 2) joint_pair_m<T, RPT, 2>(g, k, sblocks, vblocks, by, msel, st);
    else joint_pair_m<T, RPT, 4>(g, k, sblocks, vblocks, by, msel, st);
}

// One joint step k of segment g; msel: the pass's velocity mode or JOINT_MIXED.
template <typename T>
cudaError_t launch_joint_step(int g, int k, int sblocks, int vblocks, int rpt, int by, int nsmax,
                              int msel, cudaStream_t st)
{
    if constexpr (sizeof(T) == 8) {
        joint_pair_r<T, 1>(g, k, sblocks, vblocks, by, nsmax, msel, st);
    } else {
        if (rpt == 2) joint_pair_r<T, 2>(g, k, sblocks, vblocks, by, nsmax, msel, st);
        else joint_pair_r<T, 1>(g, k, sblocks, vblocks, by, nsmax, msel, st);
    }
    return cudaGetLastError();
}

// The entry and segment tables live in constant memory shared by every
// joint object of the process: one joint pass at a time.
std::mutex &joint_mutex()
{
    static std::mutex m;
    return m;
}

}  // namespace

}  // namespace psv

using psv::fail;

struct psv_joint {
    std::vector<psv_plan *> plans;
    int prec = 0, rpt = 1, by = 4;
    bool tune = false;                     // pick the tile shape on the first pass
    int nsmax = 1, maxk = 0, nseg = 0;
    int msel = 0;                          // the pass's one velocity mode, or JOINT_MIXED
    std::vector<int> seg_end;              // last joint step + 1 of each segment
    std::vector<psv::JointSeg> segs;
    std::vector<long long> sblocks, vblocks;  // launch extents per segment
    long long entry_bytes = 0;
    std::vector<unsigned char> entries;    // host copies of the entries
    std::vector<int> active;               // plans taking part in the current batch
    std::vector<std::vector<psv::JointOp>> ops;  // per active plan: the pass's operations
    std::vector<std::vector<int4>> copies; // per active plan: (joint step it precedes, slot, op, par)
    int4 *dops[3] = {nullptr, nullptr, nullptr};  // step descriptors per pass (device)
    size_t dcap[3] = {0, 0, 0};
    cudaStream_t st = nullptr;
    // one graph per pass (0 forward modelling, 1 gradient forward, 2 adjoint)
    // and shot batch, captured with the shape (rpt, by) it records
    struct Graph {
        cudaGraphExec_t x;
        int rpt, by;
        long long launches;
    };
    std::map<int, Graph> graphs;
    long long launches = 0;                // kernel launches of the last call
    ~psv_joint()
    {
        for (auto &g : graphs)
            if (g.second.x) cudaGraphExecDestroy(g.second.x);
        for (auto d : dops)
            if (d) cudaFree(d);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

template <typename T> psv::JointSurvey<T> *entry_of(psv_joint *J, int k)
{
    return reinterpret_cast<psv::JointSurvey<T> *>(J->entries.data() + k * J->entry_bytes);
}

// The plans taking part in shot batch `batch` (those with more batches).
void joint_activate(psv_joint *J, int batch)
{
    J->active.clear();
    for (int k = 0; k < (int)J->plans.size(); k++)
        if (J->plans[k]->impl->batches() > batch) J->active.push_back(k);
}

// Fills the entry and operations of every active plan: plan k's call
// fill(k, entry, ops) (joint_begin or a joint gradient phase), its error
// prefixed with the plan's index.
template <typename F> int joint_fill(psv_joint *J, F fill)
{
    const int n = (int)J->active.size();
    J->ops.resize(n);
    for (int j = 0; j < n; j++) {
        const int k = J->active[j];
        const int s = fill(k, J->entries.data() + j * J->entry_bytes, &J->ops[j]);
        if (s != PSV_OK) return fail(s, "plan " + std::to_string(k) + ": " + psv_last_error());
    }
    return PSV_OK;
}

// The same call for every plan (joint_end), outside the batches.
template <typename F> int joint_each(psv_joint *J, F call)
{
    for (int k = 0; k < (int)J->plans.size(); k++) {
        const int s = call(k);
        if (s != PSV_OK) return fail(s, "plan " + std::to_string(k) + ": " + psv_last_error());
    }
    return PSV_OK;
}

// From the filled entries and operations of pass `pass`: the step
// descriptors (uploaded), each plan's copies, the segment tables and launch
// extents; uploads the entries and the tables.
int joint_tables(psv_joint *J, int pass)
{
    const int n = (int)J->active.size();
    std::vector<int4> desc;
    std::vector<int> nops(n), first(n);
    int mode = -2;  // the one velocity mode of the pass, JOINT_MIXED when they differ
    std::vector<long long> nsb(n), nvb(n);
    J->copies.assign(n, {});
    J->nsmax = 1;
    for (int k = 0; k < n; k++) {
        first[k] = (int)desc.size();
        for (const psv::JointOp &o : J->ops[k]) {
            if (o.copy)
                J->copies[k].push_back(make_int4((int)desc.size() - first[k], o.ck_slot, o.ck_op, o.par));
            else {
                desc.push_back(make_int4(o.flags, o.it, o.slot, 0));
                const int m = o.flags >> 3;
                mode = mode == -2 || mode == m ? m : psv::JOINT_MIXED;
            }
        }
        nops[k] = (int)desc.size() - first[k];
        if (nops[k] < 1) return fail(PSV_ERR_ARG, "joint launch: a survey without time steps");
        int ns, nb, sx, sy, vx, vy;
        if (J->prec == 32) {
            const auto *x = entry_of<float>(J, k);
            ns = x->ns; nb = x->nb; sx = x->sx; sy = x->sy; vx = x->vx; vy = x->vy;
        } else {
            const auto *x = entry_of<double>(J, k);
            ns = x->ns; nb = x->nb; sx = x->sx; sy = x->sy; vx = x->vx; vy = x->vy;
        }
        J->nsmax = std::max(J->nsmax, ns);
        nsb[k] = (long long)nb * sx * sy;
        nvb[k] = (long long)nb * vx * vy;
    }
    J->msel = mode;
    if (desc.size() > J->dcap[pass]) {
        if (J->dops[pass]) cudaFree(J->dops[pass]);
        J->dops[pass] = nullptr;
        J->dcap[pass] = 0;
        PSV_CU(cudaMalloc(&J->dops[pass], desc.size() * sizeof(int4)));
        J->dcap[pass] = desc.size();
    }
    PSV_CU(cudaMemcpyAsync(J->dops[pass], desc.data(), desc.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           J->st));
    for (int k = 0; k < n; k++) {
        if (J->prec == 32) {
            entry_of<float>(J, k)->ops = J->dops[pass] + first[k];
            entry_of<float>(J, k)->nops = nops[k];
        } else {
            entry_of<double>(J, k)->ops = J->dops[pass] + first[k];
            entry_of<double>(J, k)->nops = nops[k];
        }
    }
    std::vector<int> ends(nops.begin(), nops.end());
    std::sort(ends.begin(), ends.end());
    ends.erase(std::unique(ends.begin(), ends.end()), ends.end());
    J->maxk = ends.back();
    J->seg_end = ends;
    J->nseg = (int)ends.size();
    J->segs.assign(J->nseg, psv::JointSeg{});
    J->sblocks.assign(J->nseg, 0);
    J->vblocks.assign(J->nseg, 0);
    for (int g = 0; g < J->nseg; g++) {
        const int lo = g ? ends[g - 1] : 0;  // surveys with more than lo steps run this segment
        psv::JointSeg &sg = J->segs[g];
        long long sb = 0, vb = 0;
        for (int k = 0; k < n; k++) {
            if (nops[k] <= lo) continue;
            sg.idx[sg.n] = k;
            sg.s0[sg.n] = (int)sb;
            sg.v0[sg.n] = (int)vb;
            sg.n++;
            sb += nsb[k];
            vb += nvb[k];
        }
        if (sb > 0x7fffffffLL || vb > 0x7fffffffLL)
            return fail(PSV_ERR_UNSUPPORTED, "joint launch: more than 2^31 blocks in one launch");
        J->sblocks[g] = sb;
        J->vblocks[g] = vb;
    }
    if (J->prec == 32) {
        PSV_CU(cudaMemcpyToSymbolAsync(psv::c_joint_f, J->entries.data(), (size_t)J->entry_bytes * n, 0,
                                       cudaMemcpyHostToDevice, J->st));
    } else {
        PSV_CU(cudaMemcpyToSymbolAsync(psv::c_joint_d, J->entries.data(), (size_t)J->entry_bytes * n, 0,
                                       cudaMemcpyHostToDevice, J->st));
    }
    PSV_CU(cudaMemcpyToSymbolAsync(psv::c_seg, J->segs.data(), sizeof(psv::JointSeg) * J->nseg, 0,
                                   cudaMemcpyHostToDevice, J->st));
    PSV_CU(cudaStreamSynchronize(J->st));  // the host descriptors go out of scope
    return PSV_OK;
}

// Forward-modelling entries and operations of the plans of shot batch
// `batch` with shape (rpt, by), then the tables of pass 0.
int joint_prepare(psv_joint *J, int rpt, int by, int batch)
{
    joint_activate(J, batch);
    PSV_TRY(joint_fill(J, [&](int k, void *e, std::vector<psv::JointOp> *ops) {
        return J->plans[k]->impl->joint_begin(rpt, by, batch, e, (size_t)J->entry_bytes, ops);
    }));
    return joint_tables(J, 0);
}

// The copies the active plans' operations put before joint step `step`, on
// the joint stream.
int joint_copies(psv_joint *J, int step)
{
    for (size_t j = 0; j < J->active.size(); j++)
        for (const int4 &c : J->copies[j])
            if (c.x == step) {
                const int k = J->active[j];
                const int s = J->plans[k]->impl->joint_ck_copy(c.y, c.z, c.w, (void *)J->st);
                if (s != PSV_OK) return fail(s, "plan " + std::to_string(k) + ": " + psv_last_error());
            }
    return PSV_OK;
}

// Captures joint steps [0, nsteps) of the current tables (and, for the whole
// pass, the copies after the last step) with shape (rpt, by) into *exec;
// counts its kernel launches.
int joint_capture(psv_joint *J, int rpt, int by, int nsteps, cudaGraphExec_t *exec, long long *nk)
{
    cudaGraph_t graph = nullptr;
    PSV_CU(cudaStreamBeginCapture(J->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    int s = PSV_OK;
    long long n = 0;
    int k = 0;
    for (int g = 0; g < J->nseg && e == cudaSuccess && s == PSV_OK; g++)
        for (; k < std::min(J->seg_end[g], nsteps) && e == cudaSuccess && s == PSV_OK; k++) {
            s = joint_copies(J, k);
            if (s != PSV_OK) break;
            e = J->prec == 32
                    ? psv::launch_joint_step<float>(g, k, (int)J->sblocks[g], (int)J->vblocks[g], rpt, by,
                                                    J->nsmax, J->msel, J->st)
                    : psv::launch_joint_step<double>(g, k, (int)J->sblocks[g], (int)J->vblocks[g], rpt,
                                                     by, J->nsmax, J->msel, J->st);
            n += 2;
        }
    if (s == PSV_OK && e == cudaSuccess && nsteps >= J->maxk) s = joint_copies(J, J->maxk);
    const cudaError_t ce = cudaStreamEndCapture(J->st, &graph);
    if (s != PSV_OK || e != cudaSuccess || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (s != PSV_OK) return s;
        return fail(PSV_ERR_CUDA, std::string("joint launch capture: ") +
                                      cudaGetErrorString(e != cudaSuccess ? e : ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        *exec = nullptr;
        return fail(PSV_ERR_CUDA, std::string("joint launch instantiate: ") + cudaGetErrorString(ie));
    }
    if (nk) *nk = n;
    return PSV_OK;
}

// Device milliseconds of one replay of `exec` on the joint stream.
int joint_replay(psv_joint *J, cudaGraphExec_t exec, float *ms)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t c = cudaEventCreate(&e0);
    if (c == cudaSuccess) c = cudaEventCreate(&e1);
    if (c == cudaSuccess) c = cudaEventRecord(e0, J->st);
    if (c == cudaSuccess) c = cudaGraphLaunch(exec, J->st);
    if (c == cudaSuccess) c = cudaEventRecord(e1, J->st);
    if (c == cudaSuccess) c = cudaStreamSynchronize(J->st);
    if (c == cudaSuccess) c = cudaEventElapsedTime(ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (c != cudaSuccess) return fail(PSV_ERR_CUDA, std::string("joint launch: ") + cudaGetErrorString(c));
    return PSV_OK;
}

// The whole pass `pass` of shot batch `batch` (the current tables), captured
// once per shape and replayed; adds its device time to *ms.
int joint_run(psv_joint *J, int pass, int batch, float *ms)
{
    const int key = batch * 4 + pass;
    auto it = J->graphs.find(key);
    if (it != J->graphs.end() && (it->second.rpt != J->rpt || it->second.by != J->by)) {
        cudaGraphExecDestroy(it->second.x);
        J->graphs.erase(it);
        it = J->graphs.end();
    }
    if (it == J->graphs.end()) {
        psv_joint::Graph g{nullptr, J->rpt, J->by, 0};
        PSV_TRY(joint_capture(J, J->rpt, J->by, J->maxk, &g.x, &g.launches));
        it = J->graphs.emplace(key, g).first;
    }
    J->launches += it->second.launches;
    float t = 0.f;
    PSV_TRY(joint_replay(J, it->second.x, &t));
    *ms += t;
    return PSV_OK;
}

// Tile shape of the joint launches: each candidate times the first steps of
// the forward-modelling pass (up to 24), replayed after a warm-up; the
// fastest is kept.  The plans' wavefields are zeroed again by the pass.
int joint_autotune(psv_joint *J)
{
    static const int f32[][2] = {{1, 4}, {1, 8}, {2, 4}, {2, 2}, {2, 8}, {1, 2}};
    static const int f64[][2] = {{1, 4}, {1, 8}, {1, 2}};
    const int nc = J->prec == 32 ? 6 : 3;
    float best = 0.f;
    int br = J->rpt, bb = J->by;
    for (int c = 0; c < nc; c++) {
        const int r = J->prec == 32 ? f32[c][0] : f64[c][0], b = J->prec == 32 ? f32[c][1] : f64[c][1];
        PSV_TRY(joint_prepare(J, r, b, 0));
        cudaGraphExec_t x = nullptr;
        PSV_TRY(joint_capture(J, r, b, std::min(24, J->seg_end[0]), &x, nullptr));
        float t0 = 0.f, t = 0.f;
        int s = joint_replay(J, x, &t0);
        if (s == PSV_OK) s = joint_replay(J, x, &t);
        cudaGraphExecDestroy(x);
        PSV_TRY(s);
        if (c == 0 || t < best) {
            best = t;
            br = r;
            bb = b;
        }
    }
    J->rpt = br;
    J->by = bb;
    J->tune = false;
    return PSV_OK;
}

}  // namespace

extern "C" {

int psv_joint_create(psv_plan *const *plans, int nplans, int rows_per_thread, int block_y,
                     psv_joint **out)
{
    if (!out) return fail(PSV_ERR_ARG, "null output handle");
    *out = nullptr;
    if (!plans || nplans < 1 || nplans > psv::JOINT_MAX)
        return fail(PSV_ERR_ARG, "joint launch: 1 to 8 plans");
    const bool tune = rows_per_thread == 0;
    if (!tune && (block_y < 1 || block_y > 8)) return fail(PSV_ERR_ARG, "joint launch: block_y in 1..8");
    for (int k = 0; k < nplans; k++) {
        if (!plans[k] || !plans[k]->impl) return fail(PSV_ERR_ARG, "joint launch: null plan");
        for (int j = 0; j < k; j++)
            if (plans[j] == plans[k]) return fail(PSV_ERR_ARG, "joint launch: a plan given twice");
    }
    const int prec = plans[0]->impl->precision();
    for (int k = 1; k < nplans; k++)
        if (plans[k]->impl->precision() != prec)
            return fail(PSV_ERR_ARG, "joint launch: every plan of one precision");
    if (!tune && prec == 64 && rows_per_thread != 1)
        return fail(PSV_ERR_ARG, "joint launch: FP64 plans take 1 row per thread");
    if (!tune && rows_per_thread != 1 && rows_per_thread != 2)
        return fail(PSV_ERR_ARG, "joint launch: rows_per_thread 0 (autotuned), 1 or 2");
    auto J = std::make_unique<psv_joint>();
    J->plans.assign(plans, plans + nplans);
    J->prec = prec;
    J->tune = tune;
    J->rpt = tune ? 1 : rows_per_thread;
    J->by = tune ? 4 : block_y;
    J->entry_bytes = prec == 32 ? (long long)sizeof(psv::JointSurvey<float>)
                                : (long long)sizeof(psv::JointSurvey<double>);
    J->entries.assign((size_t)J->entry_bytes * nplans, 0);
    PSV_CU(cudaStreamCreateWithFlags(&J->st, cudaStreamNonBlocking));
    *out = J.release();
    return PSV_OK;
}

int psv_joint_forward(psv_joint *J, double *const *rtf_uz, double *const *rtf_ux, double *ms)
{
    if (!J) return fail(PSV_ERR_ARG, "null joint handle");
    std::lock_guard<std::mutex> lk(psv::joint_mutex());
    if (J->tune) PSV_TRY(joint_autotune(J));
    J->launches = 0;
    int nb = 0;
    for (auto *p : J->plans) nb = std::max(nb, p->impl->batches());
    float t = 0.f;
    for (int b = 0; b < nb; b++) {  // batch b of every plan that has one, jointly
        PSV_TRY(joint_prepare(J, J->rpt, J->by, b));
        PSV_TRY(joint_run(J, 0, b, &t));
    }
    if (ms) *ms = t;
    return joint_each(J, [&](int k) {
        return J->plans[k]->impl->joint_end(rtf_uz ? rtf_uz[k] : nullptr, rtf_ux ? rtf_ux[k] : nullptr);
    });
}

int psv_joint_gradient(psv_joint *J, double *L2, double *ms)
{
    if (!J) return fail(PSV_ERR_ARG, "null joint handle");
    std::lock_guard<std::mutex> lk(psv::joint_mutex());
    if (J->tune) PSV_TRY(joint_autotune(J));
    J->launches = 0;
    const int r = J->rpt, by = J->by;
    const size_t eb = (size_t)J->entry_bytes;
    int nb = 0;
    for (auto *p : J->plans) nb = std::max(nb, p->impl->batches());
    float t = 0.f;
    for (int b = 0; b < nb; b++) {  // batch b of every plan that has one, jointly
        joint_activate(J, b);
        for (int phase = 0; phase < 2; phase++) {
            PSV_TRY(joint_fill(J, [&](int k, void *e, std::vector<psv::JointOp> *ops) {
                return J->plans[k]->impl->joint_gradient_phase(phase, r, by, b, e, eb, nullptr, ops);
            }));
            PSV_TRY(joint_tables(J, 1 + phase));
            PSV_TRY(joint_run(J, 1 + phase, b, &t));
        }
        PSV_TRY(joint_fill(J, [&](int k, void *e, std::vector<psv::JointOp> *ops) {
            return J->plans[k]->impl->joint_gradient_phase(2, r, by, b, e, eb, L2 ? L2 + k : nullptr, ops);
        }));
    }
    if (ms) *ms = t;
    return PSV_OK;
}

int psv_joint_shape(const psv_joint *J, int *rows_per_thread, int *block_y)
{
    if (!J) return fail(PSV_ERR_ARG, "null joint handle");
    if (rows_per_thread) *rows_per_thread = J->tune ? 0 : J->rpt;
    if (block_y) *block_y = J->tune ? 0 : J->by;
    return PSV_OK;
}

long long psv_joint_launches(const psv_joint *J) { return J ? J->launches : 0; }

int psv_joint_destroy(psv_joint *J)
{
    delete J;
    return PSV_OK;
}

}  // extern "C"
