// The call a maintainer puts in the reference's commented-out GPU branch
// (src/h_simulate_PSV.cpp:198-213), with the reference's globals declared
// here under placeholder names and types: contiguous row-major blocks
// (allocate_array, include/cpu/n_contiguous_arrays.hpp:54-64), so LAM[0],
// RTF_Z_TRUE[0][0] etc. are the flat pointers the ABI takes.  Compiled and
// linked against the library by the C ABI test; not run.
#include <iostream>
#include <vector>

#include "fwi_psv.h"

int NT, NZ, NX, FDORDER, SURF, ISURF[4], PML_Z, PML_X, SNAP_Z1, SNAP_Z2, SNAP_X1, SNAP_X2;
int SNAP_DT, SNAP_DZ, SNAP_DX, TAPER_T1, TAPER_T2, TAPER_B1, TAPER_B2, TAPER_L1, TAPER_L2;
int TAPER_R1, TAPER_R2, NSHOT, NSRC, NREC, STF_TYPE, RTF_TYPE, GPU_CODE, FWINV;
double DT, DX, DZ, HC[7];
double *A_Z, *B_Z, *K_Z, *A_HALF_Z, *B_HALF_Z, *K_HALF_Z;
double *A_X, *B_X, *K_X, *A_HALF_X, *B_HALF_X, *K_HALF_X;
int *Z_SRC, *X_SRC, *SRC_SHOT_TO_FIRE, *Z_REC, *X_REC;
double **STF_Z, **STF_X, **LAM, **MU, **RHO, ***RTF_Z_TRUE, ***RTF_X_TRUE;

int gpu_branch()
{
    int st = PSV_OK;
    if (GPU_CODE) {
        psv_grid g = {};
        g.nt = NT; g.nz = NZ; g.nx = NX; g.dt = DT; g.dx = DX; g.dz = DZ;
        g.fdorder = FDORDER; g.stencil = PSV_STENCIL_REFERENCE; g.surf = SURF;
        for (int k = 0; k < 4; k++) g.isurf[k] = ISURF[k];
        for (int k = 0; k < 7; k++) g.hc[k] = HC[k];          // holbergcoeff output
        g.pml_z = PML_Z; g.pml_x = PML_X;
        g.a_z = A_Z; g.b_z = B_Z; g.K_z = K_Z; g.a_half_z = A_HALF_Z; g.b_half_z = B_HALF_Z; g.K_half_z = K_HALF_Z;
        g.a_x = A_X; g.b_x = B_X; g.K_x = K_X; g.a_half_x = A_HALF_X; g.b_half_x = B_HALF_X; g.K_half_x = K_HALF_X;
        g.snap_z1 = SNAP_Z1; g.snap_z2 = SNAP_Z2; g.snap_x1 = SNAP_X1; g.snap_x2 = SNAP_X2;
        g.snap_dt = SNAP_DT; g.snap_dz = SNAP_DZ; g.snap_dx = SNAP_DX;
        int taper[8] = {TAPER_T1, TAPER_T2, TAPER_B1, TAPER_B2, TAPER_L1, TAPER_L2, TAPER_R1, TAPER_R2};
        for (int k = 0; k < 8; k++) g.taper[k] = taper[k];
        g.imaging_sign = -1;                                 // CPU path sign; +1 = CUDA path sign

        psv_shots s = {NSHOT, NSRC, NREC, STF_TYPE, RTF_TYPE, Z_SRC, X_SRC, SRC_SHOT_TO_FIRE,
                       STF_Z[0], STF_X[0], Z_REC, X_REC};
        psv_options o; psv_options_default(&o);             // FP32, CUDA graphs, 180 GB budget
        psv_plan *plan = nullptr;
        st = psv_plan_create(&g, &s, &o, &plan);
        if (st == PSV_OK) st = psv_plan_set_model(plan, LAM[0], MU[0], RHO[0]);
        if (FWINV) {
            if (st == PSV_OK) st = psv_plan_set_observed(plan, RTF_Z_TRUE[0][0], RTF_X_TRUE[0][0]);
            double step = 0.01, L2 = 0; int ntrials = 0;
            for (int it = 0; st == PSV_OK && it < 1000; it++)
                st = psv_fwi_iteration(plan, &step, &L2, &ntrials, nullptr, 0);
            if (st == PSV_OK) st = psv_plan_get_model(plan, LAM[0], MU[0], RHO[0]);
        } else {
            std::vector<double> uz((size_t)NSHOT * NREC * NT), ux(uz.size());
            if (st == PSV_OK) st = psv_forward(plan, uz.data(), ux.data());  // [shot][rec][t]
        }
        if (st != PSV_OK) std::cerr << psv_error_string(st) << ": " << psv_last_error() << "\n";
        psv_plan_destroy(plan);
    }
    return st;
}

// Choosing a storage layout and reading back what the plan chose.
int binomial_plan(const psv_grid &g, const psv_shots &s)
{
    psv_plan *plan = nullptr;
    psv_options o; psv_options_default(&o);
    o.storage = PSV_STORE_BINOMIAL;   // e.g. a long record whose states do not fit
    o.checkpoint_slots = 40;          // state slots per shot (0: library choice)
    int st = psv_plan_create(&g, &s, &o, &plan);
    int kind, seg, slots; long long adv;
    if (st == PSV_OK) st = psv_plan_storage(plan, &kind, &seg, &slots, &adv);
    psv_plan_destroy(plan);
    return st;
}

int main() { return GPU_CODE ? gpu_branch() : 0; }
