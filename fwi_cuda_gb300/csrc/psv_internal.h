// psv_internal.h -- shared host-side declarations of the engine library.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fwi_psv.h"

namespace psv {

// Records the message of a failing call (thread-local) and returns status.
int fail(int status, const std::string &msg);

// Everything the reference's simulate_PSV reads from its binary inputs
// (src/h_simulate_PSV.cpp:99-148).
struct RefInputs {
    bool gpu_code = false, surf = false, pml_z = false, pml_x = false, accu_save = false;
    bool seismo_save = false, fwinv = false, rtf_meas_true = false;
    int nt = 0, nz = 0, nx = 0, snap_t1 = 0, snap_t2 = 0, snap_z1 = 0, snap_z2 = 0;
    int snap_x1 = 0, snap_x2 = 0, snap_dt = 1, snap_dz = 1, snap_dx = 1;
    int taper[8] = {0};
    int nsrc = 0, nrec = 0, nshot = 0, stf_type = 0, rtf_type = 0, fdorder = 2, fpad = 1;
    int mat_save_interval = 0, mat_grid = 0;
    int npml[4] = {0}, isurf[4] = {0};
    std::vector<int32_t> z_src, x_src, src_shot_to_fire, z_rec, x_rec;
    double dt = 0, dz = 0, dx = 0, npower = 0, damp_v_pml = 0, rcoef = 0, k_max_pml = 0;
    double freq_pml = 0, scalar_lam = 0, scalar_mu = 0, scalar_rho = 0;
    std::vector<double> lam, mu, rho, rtf_z_true, rtf_x_true;
};

int read_inputs(const std::string &dir, RefInputs &in);
int write_f64(const std::string &path, const double *data, size_t n);

}  // namespace psv
