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


def _program_status(work):
    from fwi_cuda_gb300 import _lib, engine
    try:
        engine.simulate_PSV(str(work))
    except _lib.PSVError as e:
        return e.status, str(e)
    return _lib.PSV_OK, ""


def test_program_input_errors(golden, tmp_path):
    # simulate_PSV reads bin/*.bin (and io/*.bin for FWI) before any device
    # work: a missing or short file is PSV_ERR_IO naming it, where the
    # reference's readers (src/h_io_PSV.cpp) read on regardless
    from fwi_cuda_gb300 import _lib
    sv = helpers.load_case(golden, NAME)
    model = golden[f"{NAME}/model"]
    b = tmp_path / "bin"

    def fresh(**kw):
        for f in tmp_path.rglob("*.bin"):
            f.unlink()
        fio.write_inputs(str(tmp_path), sv, *model, **kw)

    assert _program_status(tmp_path)[0] == _lib.PSV_ERR_IO  # nothing written yet
    fresh()
    (b / "metaint.bin").write_bytes((b / "metaint.bin").read_bytes()[:100])
    st, msg = _program_status(tmp_path)
    assert st == _lib.PSV_ERR_IO and "metaint.bin: short read" in msg
    fresh()
    meta = np.fromfile(b / "metaint.bin", np.int32)
    meta[9] = 0  # nz
    meta.tofile(b / "metaint.bin")
    st, msg = _program_status(tmp_path)
    assert st == _lib.PSV_ERR_IO and "invalid sizes" in msg
    for name in ("intarray", "metafloat", "mat"):
        fresh()
        data = (b / f"{name}.bin").read_bytes()
        (b / f"{name}.bin").write_bytes(data[:len(data) - 8])
        st, msg = _program_status(tmp_path)
        assert st == _lib.PSV_ERR_IO and f"{name}.bin" in msg, (name, msg)
        (b / f"{name}.bin").unlink()
        st, msg = _program_status(tmp_path)
        assert st == _lib.PSV_ERR_IO and f"cannot open bin/{name}.bin" in msg, (name, msg)
    fresh(fwinv=True, rtf_meas_true=False)
    assert _program_status(tmp_path)[0] == _lib.PSV_ERR_ARG
    fresh(fwinv=True)
    st, msg = _program_status(tmp_path)
    assert st == _lib.PSV_ERR_IO and "shot0_rtf_uz.bin" in msg
    if not _lib.device_available():
        fresh()  # complete inputs: the first device call fails, no CPU fallback
        assert _program_status(tmp_path)[0] == _lib.PSV_ERR_CUDA


def test_seis_fwi_program(golden, tmp_path):
    # the reference's program name on the engine: a missing input is an error
    # exit naming the file; complete inputs reach the device (on a machine
    # without one, the CUDA error, never a CPU fallback)
    import subprocess
    from fwi_cuda_gb300 import _lib
    from fwi_cuda_gb300 import build as B
    _lib.lib()
    assert os.path.exists(B.EXE)
    out = subprocess.run([B.EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "bin/metaint.bin" in out.stderr
    if not _lib.device_available():
        sv = helpers.load_case(golden, NAME)
        fio.write_inputs(str(tmp_path), sv, *golden[f"{NAME}/model"])
        out = subprocess.run([B.EXE, str(tmp_path)], capture_output=True, text=True, timeout=60)
        assert out.returncode == 1 and "CUDA error" in out.stderr
