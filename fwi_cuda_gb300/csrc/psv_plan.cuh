// psv_plan.cuh -- the device-resident survey plan (host C++ side).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "fwi_psv.h"
#include "psv_fwi.cuh"
#include "psv_internal.h"
#include "psv_kernels.cuh"

namespace psv {

template <typename T>
cudaError_t launch_stress(const StepParams<T> &, int ns, int rpt, dim3, int, cudaStream_t);
template <typename T>
cudaError_t launch_velocity(const StepParams<T> &, const SrcRecParams<T> &, int ns, int mode,
                            int it, int slot, int rpt, dim3, int, cudaStream_t);
template <typename T>
cudaError_t launch_zero_planes(T *base, long long shot_stride, long long off, long long count,
                               int nbatch, cudaStream_t st);
cudaError_t launch_transpose(const double *in, double *out, int rows, int cols, int nbatch,
                             cudaStream_t st);

// TMA tile kernels (FP32, psv_tiled.cu): tiles of 64 columns x 4 rpt rows,
// rpt in {2, 4, 8}.  Maps of one field block: halo'd and own boxes of the
// field planes, own boxes of the 7 coefficient planes.
struct TileMaps {
    CUtensorMap halo;  // field planes, box 72 x (4 rpt + 2 ns)
    CUtensorMap own;   // field planes, box 64 x 4 rpt
    CUtensorMap coef;  // coefficient planes, box 64 x 4 rpt
};
// 3-D tensor map (column, row, plane) over nplanes planes of nz x nx floats
// (row pitch `pitch`, plane stride `plane` elements), box bx x by x 1, zero
// fill outside (psv_tiled.cu).
int encode3(CUtensorMap *map, const float *base, int nx, int nz, int pitch, long long plane,
            int nplanes, int bx, int by);
int encode_tile_maps(TileMaps *m, const float *fld, int nfplanes, const float *coef, int nx, int nz,
                     int pitch, long long plane, int ns, int rpt);
// Four-columns-per-thread kernels (FP32, psv_vec.cu): blocks of 32 x by
// threads over 128 columns x by * rpt rows, rpt in {1, 2, 4}.
cudaError_t launch_stress_v4(const StepParams<float> &p, int ns, int rpt, int by, int nbatch,
                             cudaStream_t st);
cudaError_t launch_velocity_v4(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                               int mode, int it, int slot, int rpt, int by, int nbatch,
                               cudaStream_t st);
// Fused time step (FP32, psv_fused.cu): one launch per step over tiles of
// 64 columns x tz rows (tz 16 or 32), reading field copy `par` and writing
// copy 1 - par.  fused_supported: the surfaces it handles (top only).
bool fused_supported(int ns, int tz, int st, int sb, int sl, int sr, int nz1);
cudaError_t launch_step_fused(const StepParams<float> &p, const SrcRecParams<float> &q, int ns,
                              int mode, int it, int slot, int par, int tz, int nbatch,
                              cudaStream_t st);
// Fused time step as a vertical march (FP32, psv_march.cu): one launch per
// step; a CTA of 256 threads owns 128 - 2 ns columns and `rows` rows (32, 64
// or 128) of one shot and walks down them `stage` rows (2 or 4) at a time,
// old v staged by TMA through the map of MarchMaps, reading copy `par` and
// writing copy 1 - par.  march_supported: no free surface or a top one on the
// first interior row.
struct MarchMaps {
    CUtensorMap fld;  // field planes, box (128 + 2 ns + 4) x stage
};
bool march_supported(int ns, int rows, int stage, int st, int sb, int sl, int sr, int nz1);
int march_tile_width(int ns, int stage);
int encode_march_maps(MarchMaps *m, const float *fld, int nfplanes, int nx, int nz, int pitch,
                      long long plane, int ns, int stage);
cudaError_t launch_step_march(const StepParams<float> &p, const SrcRecParams<float> &q,
                              const MarchMaps &mm, int ns, int mode, int it, int slot, int par,
                              int rows, int stage, int nbatch, cudaStream_t st);
// Exact discrete adjoint of the FP64 time loop (psv_exact.cu).  Work planes
// of one shot slot: v-bar (2), two copies of sigma-bar (3 each), e-bar (4),
// d-bar (4), and the derivatives of L2 with respect to dt (lam + 2 mu),
// dt lam, dt mu_zx, dt / rho_z, dt / rho_x and, in row 0 of the last plane,
// the top surface factor.
enum {
    EX_VBZ = 0, EX_VBX = 1, EX_SB0 = 2, EX_SB1 = 5, EX_EB = 8, EX_DB = 12,
    EX_GC2 = 16, EX_GCL, EX_GCM, EX_GRZ, EX_GRX, EX_GFS, EXACT_WORK_PLANES
};
struct ExactBufs {
    double *store;             // [nt][batch][8][plane]: d' (4), e' (4) of every step
    long long step_stride;     // batch * 8 * plane
    double *work;              // [batch][EXACT_WORK_PLANES][plane]
    double *qz, *qx;           // adjoint CPML memories, layout of StepParams::memz / memx
    const double *rsum_z, *rsum_x;  // receiver adjoint sources [shot][nt][nrec]
};
cudaError_t launch_exact_forward_step(const StepParams<double> &p, const SrcRecParams<double> &q,
                                      const ExactBufs &X, int ns, int n, int nbatch, int maxsrc,
                                      cudaStream_t st);
cudaError_t launch_exact_revsum(double *res_z, double *res_x, int nt, int nrec, long long stride,
                                double dt, double gain, int nbatch, cudaStream_t st);
cudaError_t launch_exact_adjoint_step(const StepParams<double> &p, const SrcRecParams<double> &q,
                                      const ExactBufs &X, int ns, int n, int sin, int sout,
                                      int nbatch, int maxsrc, cudaStream_t st);
cudaError_t launch_exact_chain(const StepParams<double> &p, const ExactBufs &X, const double *lam,
                               const double *mu, const double *rho, double *gl, double *gm,
                               double *gr, double dt, double sign, cudaStream_t st);
// Joint launches over several surveys (psv_joint.cu): one stress and one
// velocity launch per time step cover every shot of up to JOINT_MAX surveys
// of any grid size, stencil order and step count, the direct family's block
// bodies with one tile shape.  A survey's entry: its plan's step and forward
// source / receiver parameters, stencil terms, step count, and the blocks of
// its stress (interior) and velocity (whole plane) grids per shot.
constexpr int JOINT_MAX = 8;
template <typename T>
struct JointSurvey {
    StepParams<T> p, p2;   // the main state and the checkpoint recompute state
    SrcRecParams<T> q[3];  // sources / receivers: forward, recompute, adjoint
    const int4 *ops;       // the pass's step descriptors (device), one per joint step
    int nops;              // steps of the survey in the pass
    int ns, nb;            // stencil terms, shots
    int sx, sy;            // stress grid blocks along x and z
    int vx, vy;            // velocity grid blocks along x and z
};
// Step descriptor: x = state | source set << 1 | velocity mode << 3 (state 0
// main, 1 recompute; set 0 forward, 1 recompute, 2 adjoint), y = the
// survey's own time step, z = snapshot slot or -1.
__host__ __device__ constexpr int joint_flags(int state, int qsel, int mode)
{
    return state | qsel << 1 | mode << 3;
}
// One operation of a survey's joint pass: a time step (its descriptor), or a
// checkpoint copy (slot, operation, field copy) before the survey's next step.
struct JointOp {
    int copy;
    int flags, it, slot;
    int ck_slot, ck_op, par;
};
cudaError_t launch_stress_tma(const StepParams<float> &p, const TileMaps &m, int ns, int rpt,
                              int nbatch, cudaStream_t st);
cudaError_t launch_velocity_tma(const StepParams<float> &p, const SrcRecParams<float> &q,
                                const TileMaps &m, int ns, int mode, int it, int slot, int rpt,
                                int nbatch, cudaStream_t st);

#define PSV_CU(call)                                                                        \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return ::psv::fail(PSV_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define PSV_TRY(call)                  \
    do {                               \
        int s_ = (call);               \
        if (s_ != PSV_OK) return s_;   \
    } while (0)

// Validated host copy of a survey and the geometry derived from it.
struct Survey {
    psv_grid g{};
    psv_shots s{};
    std::vector<double> prof[12];  // a_z b_z K_z ah_z bh_z Kh_z a_x b_x K_x ah_x bh_x Kh_x
    std::vector<int> z_src, x_src, fire, z_rec, x_rec;
    std::vector<double> stf_z, stf_x;
    int ns = 1, fpad = 1, nz1 = 0, nz2 = 0, nx1 = 0, nx2 = 0;
    int pz0 = 0, pz1 = 0, px0 = 0, px1 = 0;  // identity (non-strip) ranges
    int snt = 1, snz = 1, snx = 1;
    int st = 0, sb = 0, sl = 0, sr = 0;
};

int make_survey(const psv_grid *g, const psv_shots *s, Survey &out);

// Owning device allocation.
struct DevMem {
    void *p = nullptr;
    size_t bytes = 0;
    DevMem() = default;
    DevMem(const DevMem &) = delete;
    DevMem &operator=(const DevMem &) = delete;
    ~DevMem() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    int alloc(size_t n, size_t &total)
    {
        total -= bytes;
        release();
        if (n == 0) return PSV_OK;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();
            return fail(e == cudaErrorMemoryAllocation ? PSV_ERR_OOM : PSV_ERR_CUDA,
                        std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
        }
        bytes = n;
        total += n;
        return PSV_OK;
    }
    template <typename U> U *as() const { return static_cast<U *>(p); }
};

// Interface of a plan, independent of the wavefield precision.
struct PlanIface {
    virtual ~PlanIface() = default;
    virtual long long device_bytes() const = 0;
    virtual int precision() const = 0;  // 32 or 64: the wavefields' floating-point width
    virtual int set_model(const double *lam, const double *mu, const double *rho) = 0;
    virtual int get_model(double *lam, double *mu, double *rho) = 0;
    virtual int set_observed(const double *uz, const double *ux) = 0;
    virtual int forward(double *uz, double *ux) = 0;
    virtual int gradient(double *L2) = 0;
    virtual int get_gradient(double *gl, double *gm, double *gr) = 0;
    virtual int set_gradient(const double *gl, const double *gm, const double *gr) = 0;
    virtual int reset_gradient() = 0;
    virtual int get_shot(int ishot, double *gl, double *gm, double *gr, double *We, double *WeA,
                         double *uz, double *ux, double *L2) = 0;
    virtual int fwi_iteration(double *step, double *L2, int *ntrials, double *tlog, int maxt) = 0;
    virtual int save_model() = 0;
    virtual int taper_gradient() = 0;
    virtual int pcg_gradient() = 0;
    virtual int update_model(double step) = 0;
    virtual int trial_misfit(double step, double *L2) = 0;
    virtual int timing(double *ms3) const = 0;
    virtual void *stream() const = 0;
    virtual long long launches() const = 0;
    virtual int profile(int nsteps, double *ms6) = 0;
    virtual int autotune(int nsteps, int *fam, int *rpt, int *by) = 0;
    virtual void shape(int *fam, int *rpt, int *by) const = 0;
    virtual void storage(int *kind, int *segment_steps, int *slots, long long *advances) const = 0;
    virtual int chain_count() const = 0;
    virtual int prepare() = 0;  // history buffers and the pending autotune, before concurrent use
    // Joint forward modelling (psv_joint.cu): switch to the direct family with
    // rpt rows per thread and 32 x by blocks, select shot batch `batch`, zero
    // the wavefields, fill the JointSurvey<T> at `entry` (`bytes` = its size:
    // the precisions agree) and the pass's operations; after the joint time
    // loops of every batch, fetch the traces.
    virtual int joint_begin(int rpt, int by, int batch, void *entry, size_t bytes,
                            std::vector<JointOp> *ops) = 0;
    virtual int joint_end(double *rtf_uz, double *rtf_ux) = 0;
    virtual int batches() const = 0;  // shot batches of the plan (max_batch, HBM budget)
    // Joint gradient, the plan's work around the two joint passes: phase 0
    // sets up the forward pass (as joint_begin; snapshots, or checkpoint
    // saves), phase 1 forms the residuals and adjoint sources and sets up the
    // adjoint pass (with checkpoints: the schedule's restores, recomputed
    // segments and adjoint steps), phase 2 preconditions the shot gradients
    // into the global ones and returns L2.
    virtual int joint_gradient_phase(int phase, int rpt, int by, int batch, void *entry,
                                     size_t bytes, double *L2, std::vector<JointOp> *ops) = 0;
    // A checkpoint copy of the plan's schedule, enqueued on `stream`.
    virtual int joint_ck_copy(int slot, int op, int par, void *stream) = 0;
    // kernel_PSV drop-in support
    virtual int kernel_call(const double *lam, const double *mu, const double *mu_zx,
                            const double *rho_zp, const double *rho_xp, int ishot, int grad,
                            int accu, double *const *accu_in_out, double *const *fields_out,
                            double *const *mem_out, double *rtf_uz, double *rtf_ux,
                            double *const *grad_out) = 0;
};

std::unique_ptr<PlanIface> make_plan_f32(const Survey &sv, const psv_options &opt, int &status);
std::unique_ptr<PlanIface> make_plan_f64(const Survey &sv, const psv_options &opt, int &status);

}  // namespace psv

struct psv_plan {
    std::unique_ptr<psv::PlanIface> impl;
};
