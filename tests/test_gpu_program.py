"""psv_simulate_PSV -- the reference's whole program on the GPU -- fed the
reference's binary input files: forward outputs against the reference's own
program run (golden case program_fwd), FWI iterations against the oracle."""
import os
import tempfile

import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import engine
from fwi_cuda_gb300 import io as fio

pytestmark = pytest.mark.gpu
NAME = "program_fwd"


def _inputs(z):
    work = tempfile.mkdtemp()
    os.makedirs(os.path.join(work, "bin"))
    for f in ("metaint", "intarray", "metafloat", "mat"):
        z[f"{NAME}/{f}.bin"].tofile(os.path.join(work, "bin", f + ".bin"))
    return work


@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 1e-5)])
def test_program_forward_matches_reference_program(gpu, precision, tol):
    z = np.load(helpers.GOLDEN)
    sv = helpers.load_case(z, NAME)
    work = _inputs(z)
    engine.simulate_PSV(work, precision=precision)
    snt, snz, snx = sv.snap_dims()
    for s in range(sv.nshot):
        uz, ux = fio.read_seismo(work, s, sv.nrec, sv.nt)
        assert helpers.rel_l2(uz, z[f"{NAME}/shot{s}_rtf_uz"]) < tol
        assert helpers.rel_l2(ux, z[f"{NAME}/shot{s}_rtf_ux"]) < tol
        acc = fio.read_accu(work, s, (snt, snz, snx))
        for k in ("vz", "szx"):
            assert helpers.rel_l2(acc[k], z[f"{NAME}/shot{s}_{k}"]) < tol * 10, k


def test_program_fwi_matches_oracle(gpu, orc):
    sv, true, init = helpers.crosswell(nt=300, nz=51, nx=41, nshot=2, nrec=12, npml=8)
    uz, ux = orc.simulate_fwd(sv, *true)
    work = tempfile.mkdtemp()
    fio.write_inputs(work, sv, *init, fwinv=True, mat_save_interval=1)
    fio.write_observed(work, uz, ux)
    engine.simulate_PSV(work, max_iter=2, imaging_sign=1, precision=64)
    r = orc.simulate_fwi(sv, *init, uz, ux, niter=2)
    assert r["rc"] == 0
    m = fio.read_mat(work, 1, sv.nz, sv.nx)
    for k, a in zip(("lam", "mu", "rho"), m):
        assert helpers.rel_l2(a, r[k]) < 1e-9, k
