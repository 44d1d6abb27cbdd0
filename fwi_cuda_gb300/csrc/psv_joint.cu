// psv_joint.cu -- forward modelling and FWI gradients of several surveys in
// one launch per half-step.
//
// A joint pass steps up to JOINT_MAX surveys (one plan each: any grid size,
// stencil order, step count and shot count) together: every time step is one
// stress launch and one velocity launch whose blocks cover every shot of
// every survey still running.  The survey entries (JointSurvey: the plans'
// own step and source / receiver parameters) sit in constant memory; a
// step's launch carries only its step index and the segment it belongs to.
// Block b of a launch belongs to the survey whose first block is the last one
// <= b (a block-uniform scan of at most JOINT_MAX entries), and runs the
// direct family's block body for that survey's stencil order
// (stress_block / velocity_block, psv_kernels_impl.cuh): each survey gets
// the operations of its own plan's direct launches.  The survey's parameters
// are read from constant memory instead of kernel arguments, and the
// compiler may contract multiply-adds differently in this context, so FP32
// traces agree with the plan's own to rounding (not bit for bit).
//
// Uneven step counts: the surveys sorted by step count split the time axis
// into segments; segment g holds the surveys with more than its first step
// (their order and first blocks in c_seg[g]).  A survey leaves the launches
// after its last step.  The whole loop (2 x the longest step count launches)
// is one CUDA graph per velocity mode, captured once per joint object and
// replayed per call.
//
// Gradient (psv_joint_gradient, full snapshot storage): the gradient forward
// pass (MODE_FWD, snapshots every sdt-th step) and the adjoint pass
// (MODE_ADJ, imaging) each run jointly; at joint step k a survey runs its own
// step k, or nt - 1 - k in the time-reversed adjoint pass, with its own
// snapshot slot.  Residuals, adjoint sources and preconditioning run per plan
// between and after the passes (PlanIface::joint_gradient_phase).
#include <algorithm>
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
__global__ void __launch_bounds__(256) k_joint_stress(const int g)
{
    const JointSeg &sg = c_seg[g];
    const int j = joint_slot(sg.s0, sg.n, (int)blockIdx.x);
    const JointSurvey<T> &e = joint_entry<T>(sg.idx[j]);
    const BlockPos bp = joint_pos((int)blockIdx.x - sg.s0[j], e.sx, e.sy);
    if constexpr (NSMAX >= 4) {
        if (e.ns == 4) return stress_block<T, 4, RPT, false>(e.p, bp);
        if (e.ns == 3) return stress_block<T, 3, RPT, false>(e.p, bp);
    }
    if (e.ns == 2) return stress_block<T, 2, RPT, false>(e.p, bp);
    stress_block<T, 1, RPT, false>(e.p, bp);
}

// Velocity step of mode MODE (MODE_FWD_NOWE: forward modelling; MODE_FWD:
// the gradient's forward pass with snapshots; MODE_ADJ: the adjoint pass
// with imaging) at joint step k: the survey's own step it (k, or nt - 1 - k
// in the time-reversed pass) and snapshot slot.
template <typename T, int RPT, int NSMAX, int MODE>
__global__ void __launch_bounds__(256) k_joint_velocity(const int g, const int k)
{
    const JointSeg &sg = c_seg[g];
    const int j = joint_slot(sg.v0, sg.n, (int)blockIdx.x);
    const JointSurvey<T> &e = joint_entry<T>(sg.idx[j]);
    const BlockPos bp = joint_pos((int)blockIdx.x - sg.v0[j], e.vx, e.vy);
    const int it = e.rev ? e.nt - 1 - k : k;
    const int slot = (e.sdt > 0 && !(it % e.sdt)) ? (it / e.sdt) % e.ring : -1;
    if constexpr (NSMAX >= 4) {
        if (e.ns == 4) return velocity_block<T, 4, MODE, RPT, false>(e.p, e.q, it, slot, bp);
        if (e.ns == 3) return velocity_block<T, 3, MODE, RPT, false>(e.p, e.q, it, slot, bp);
    }
    if (e.ns == 2) return velocity_block<T, 2, MODE, RPT, false>(e.p, e.q, it, slot, bp);
    velocity_block<T, 1, MODE, RPT, false>(e.p, e.q, it, slot, bp);
}

template <typename T, int RPT, int NSMAX>
void joint_pair(int g, int k, int sblocks, int vblocks, int by, int mode, cudaStream_t st)
{
    const dim3 blk(32, by, 1);
    k_joint_stress<T, RPT, NSMAX><<<sblocks, blk, 0, st>>>(g);
    if (mode == MODE_FWD) k_joint_velocity<T, RPT, NSMAX, MODE_FWD><<<vblocks, blk, 0, st>>>(g, k);
    else if (mode == MODE_ADJ) k_joint_velocity<T, RPT, NSMAX, MODE_ADJ><<<vblocks, blk, 0, st>>>(g, k);
    else k_joint_velocity<T, RPT, NSMAX, MODE_FWD_NOWE><<<vblocks, blk, 0, st>>>(g, k);
}

template <typename T, int RPT>
void joint_pair_r(int g, int k, int sblocks, int vblocks, int by, int nsmax, int mode, cudaStream_t st)
{
    if (nsmax <= 2) joint_pair<T, RPT, 2>(g, k, sblocks, vblocks, by, mode, st);
    else joint_pair<T, RPT, 4>(g, k, sblocks, vblocks, by, mode, st);
}

// One joint time step k of segment g (mode: MODE_FWD_NOWE, MODE_FWD or MODE_ADJ).
template <typename T>
cudaError_t launch_joint_step(int g, int k, int sblocks, int vblocks, int rpt, int by, int nsmax,
                              int mode, cudaStream_t st)
{
    if constexpr (sizeof(T) == 8) {
        joint_pair_r<T, 1>(g, k, sblocks, vblocks, by, nsmax, mode, st);
    } else {
        switch (rpt) {
        case 2: joint_pair_r<T, 2>(g, k, sblocks, vblocks, by, nsmax, mode, st); break;
        case 4: joint_pair_r<T, 4>(g, k, sblocks, vblocks, by, nsmax, mode, st); break;
        default: joint_pair_r<T, 1>(g, k, sblocks, vblocks, by, nsmax, mode, st); break;
        }
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
    int nsmax = 1, maxnt = 0, nseg = 0;
    std::vector<int> seg_end;              // last step + 1 of each segment
    std::vector<psv::JointSeg> segs;
    std::vector<long long> sblocks, vblocks;  // launch extents per segment
    long long entry_bytes = 0;
    std::vector<unsigned char> entries;    // host copies of the entries
    cudaStream_t st = nullptr;
    // whole time loops per velocity mode (forward modelling, gradient
    // forward, adjoint), each captured with the shape in g_shape
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    int g_shape[3][2] = {};
    ~psv_joint()
    {
        for (auto g : graph)
            if (g) cudaGraphExecDestroy(g);
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

int mode_slot(int mode) { return mode == psv::MODE_FWD ? 1 : mode == psv::MODE_ADJ ? 2 : 0; }

// Fills every plan's entry: plan k's call fill(k, entry) (joint_begin or a
// joint gradient phase), its error prefixed with the plan's index.
template <typename F> int joint_fill(psv_joint *J, F fill)
{
    const int n = (int)J->plans.size();
    for (int k = 0; k < n; k++) {
        const int s = fill(k, J->entries.data() + k * J->entry_bytes);
        if (s != PSV_OK) return fail(s, "plan " + std::to_string(k) + ": " + psv_last_error());
    }
    return PSV_OK;
}

// Segment tables and launch extents from the filled entries; uploads both.
int joint_tables(psv_joint *J)
{
    const int n = (int)J->plans.size();
    std::vector<int> nt(n);
    std::vector<long long> nsb(n), nvb(n);
    J->nsmax = 1;
    for (int k = 0; k < n; k++) {
        const unsigned char *e = J->entries.data() + k * J->entry_bytes;
        int ns, ntk, nb, sx, sy, vx, vy;
        if (J->prec == 32) {
            const auto *x = reinterpret_cast<const psv::JointSurvey<float> *>(e);
            ns = x->ns; ntk = x->nt; nb = x->nb; sx = x->sx; sy = x->sy; vx = x->vx; vy = x->vy;
        } else {
            const auto *x = reinterpret_cast<const psv::JointSurvey<double> *>(e);
            ns = x->ns; ntk = x->nt; nb = x->nb; sx = x->sx; sy = x->sy; vx = x->vx; vy = x->vy;
        }
        J->nsmax = std::max(J->nsmax, ns);
        nt[k] = ntk;
        nsb[k] = (long long)nb * sx * sy;
        nvb[k] = (long long)nb * vx * vy;
    }
    std::vector<int> ends(nt.begin(), nt.end());
    std::sort(ends.begin(), ends.end());
    ends.erase(std::unique(ends.begin(), ends.end()), ends.end());
    J->maxnt = ends.back();
    J->seg_end = ends;
    J->nseg = (int)ends.size();
    J->segs.assign(J->nseg, psv::JointSeg{});
    J->sblocks.assign(J->nseg, 0);
    J->vblocks.assign(J->nseg, 0);
    for (int g = 0; g < J->nseg; g++) {
        const int first = g ? ends[g - 1] : 0;  // surveys with nt > first run this segment
        psv::JointSeg &sg = J->segs[g];
        long long sb = 0, vb = 0;
        for (int k = 0; k < n; k++) {
            if (nt[k] <= first) continue;
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
    return PSV_OK;
}

// Forward-modelling entries of every plan with shape (rpt, by), then the tables.
int joint_prepare(psv_joint *J, int rpt, int by)
{
    PSV_TRY(joint_fill(J, [&](int k, void *e) {
        return J->plans[k]->impl->joint_begin(rpt, by, e, (size_t)J->entry_bytes);
    }));
    return joint_tables(J);
}

// Captures joint steps [0, nsteps) with shape (rpt, by) and velocity mode
// `mode` into *exec.
int joint_capture(psv_joint *J, int rpt, int by, int nsteps, int mode, cudaGraphExec_t *exec)
{
    cudaGraph_t graph = nullptr;
    PSV_CU(cudaStreamBeginCapture(J->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    int k = 0;
    for (int g = 0; g < J->nseg && e == cudaSuccess; g++)
        for (; k < std::min(J->seg_end[g], nsteps) && e == cudaSuccess; k++)
            e = J->prec == 32
                    ? psv::launch_joint_step<float>(g, k, (int)J->sblocks[g], (int)J->vblocks[g], rpt, by,
                                                    J->nsmax, mode, J->st)
                    : psv::launch_joint_step<double>(g, k, (int)J->sblocks[g], (int)J->vblocks[g], rpt,
                                                     by, J->nsmax, mode, J->st);
    const cudaError_t ce = cudaStreamEndCapture(J->st, &graph);
    if (e != cudaSuccess || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(PSV_ERR_CUDA, std::string("joint launch capture: ") +
                                      cudaGetErrorString(e != cudaSuccess ? e : ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        *exec = nullptr;
        return fail(PSV_ERR_CUDA, std::string("joint launch instantiate: ") + cudaGetErrorString(ie));
    }
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

// The whole joint time loop of velocity mode `mode` (tables uploaded),
// captured once per shape and replayed.
int joint_run(psv_joint *J, int mode, float *ms)
{
    const int m = mode_slot(mode);
    if (J->graph[m] && (J->g_shape[m][0] != J->rpt || J->g_shape[m][1] != J->by)) {
        cudaGraphExecDestroy(J->graph[m]);
        J->graph[m] = nullptr;
    }
    if (!J->graph[m]) {
        PSV_TRY(joint_capture(J, J->rpt, J->by, J->maxnt, mode, &J->graph[m]));
        J->g_shape[m][0] = J->rpt;
        J->g_shape[m][1] = J->by;
    }
    return joint_replay(J, J->graph[m], ms);
}

// Tile shape of the joint launches: each candidate times the first steps of
// the forward-modelling loop (up to 24), replayed after a warm-up; the
// fastest is kept.  The plans' wavefields are zeroed again by the pass.
int joint_autotune(psv_joint *J)
{
    static const int f32[][2] = {{1, 4}, {1, 8}, {2, 4}, {2, 2}, {4, 2}, {1, 2}};
    static const int f64[][2] = {{1, 4}, {1, 8}, {1, 2}};
    const int nc = J->prec == 32 ? 6 : 3;
    float best = 0.f;
    int br = J->rpt, bb = J->by;
    for (int c = 0; c < nc; c++) {
        const int r = J->prec == 32 ? f32[c][0] : f64[c][0], b = J->prec == 32 ? f32[c][1] : f64[c][1];
        PSV_TRY(joint_prepare(J, r, b));
        cudaGraphExec_t x = nullptr;
        PSV_TRY(joint_capture(J, r, b, std::min(24, J->seg_end[0]), psv::MODE_FWD_NOWE, &x));
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
    if (!tune && rows_per_thread != 1 && rows_per_thread != 2 && rows_per_thread != 4)
        return fail(PSV_ERR_ARG, "joint launch: rows_per_thread 0 (autotuned), 1, 2 or 4");
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
    PSV_TRY(joint_prepare(J, J->rpt, J->by));
    float t = 0.f;
    PSV_TRY(joint_run(J, psv::MODE_FWD_NOWE, &t));
    if (ms) *ms = t;
    return joint_fill(J, [&](int k, void *) {
        return J->plans[k]->impl->joint_end(rtf_uz ? rtf_uz[k] : nullptr, rtf_ux ? rtf_ux[k] : nullptr);
    });
}

int psv_joint_gradient(psv_joint *J, double *L2, double *ms)
{
    if (!J) return fail(PSV_ERR_ARG, "null joint handle");
    std::lock_guard<std::mutex> lk(psv::joint_mutex());
    if (J->tune) PSV_TRY(joint_autotune(J));
    const int r = J->rpt, b = J->by;
    const size_t eb = (size_t)J->entry_bytes;
    float tf = 0.f, ta = 0.f;
    PSV_TRY(joint_fill(J, [&](int k, void *e) {
        return J->plans[k]->impl->joint_gradient_phase(0, r, b, e, eb, nullptr);
    }));
    PSV_TRY(joint_tables(J));
    PSV_TRY(joint_run(J, psv::MODE_FWD, &tf));
    PSV_TRY(joint_fill(J, [&](int k, void *e) {
        return J->plans[k]->impl->joint_gradient_phase(1, r, b, e, eb, nullptr);
    }));
    PSV_TRY(joint_tables(J));
    PSV_TRY(joint_run(J, psv::MODE_ADJ, &ta));
    if (ms) *ms = tf + ta;
    return joint_fill(J, [&](int k, void *e) {
        return J->plans[k]->impl->joint_gradient_phase(2, r, b, e, eb, L2 ? L2 + k : nullptr);
    });
}

int psv_joint_shape(const psv_joint *J, int *rows_per_thread, int *block_y)
{
    if (!J) return fail(PSV_ERR_ARG, "null joint handle");
    if (rows_per_thread) *rows_per_thread = J->tune ? 0 : J->rpt;
    if (block_y) *block_y = J->tune ? 0 : J->by;
    return PSV_OK;
}

long long psv_joint_launches(const psv_joint *J) { return J ? 2LL * J->maxnt : 0; }

int psv_joint_destroy(psv_joint *J)
{
    delete J;
    return PSV_OK;
}

}  // extern "C"
