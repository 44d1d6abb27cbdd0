"""The reference's binary file formats (fwi_cuda_gb300/io.py) and the
program-level semantics of simulate_PSV, pinned to the reference's own
program run on those files (golden case program_fwd)."""
import os
import tempfile

import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import io as fio
from fwi_cuda_gb300 import survey as S

NAME = "program_fwd"


@pytest.fixture(scope="module")
def golden():
    return np.load(helpers.GOLDEN)


def test_writer_reproduces_reference_input_bytes(golden):
    sv = helpers.load_case(golden, NAME)
    work = tempfile.mkdtemp()
    fio.write_inputs(work, sv, *golden[f"{NAME}/model"], fwinv=False, accu_save=True,
                     seismo_save=True, gpu_code=False)
    for f in ("metaint", "intarray", "metafloat", "mat"):
        got = np.fromfile(os.path.join(work, "bin", f + ".bin"), np.uint8)
        assert np.array_equal(got, golden[f"{NAME}/{f}.bin"]), f


def test_oracle_reproduces_reference_program_outputs(orc, golden):
    # simulate_PSV derives its sources itself: Ricker at the PML frequency,
    # z amplitude 0, x amplitude 1 (src/h_simulate_PSV.cpp:182-185)
    sv = helpers.load_case(golden, NAME)
    w = S.ricker(sv.nt, sv.dt, sv.freq_pml)
    sv.stf_z = np.zeros((sv.nsrc, sv.nt))
    sv.stf_x = np.stack([w] * sv.nsrc)
    lam, mu, rho = golden[f"{NAME}/model"]
    mz, rz, rx, _ = orc.mat_av2(lam, mu, rho)
    for s in range(sv.nshot):
        o = orc.kernel_PSV(sv, s, lam, mu, mz, rz, rx, accu=True)
        assert np.array_equal(o["rtf_uz"], golden[f"{NAME}/shot{s}_rtf_uz"])
        assert np.array_equal(o["rtf_ux"], golden[f"{NAME}/shot{s}_rtf_ux"])
        assert np.array_equal(o["history"]["vz"], golden[f"{NAME}/shot{s}_vz"])
