"""psv_misfit_noalloc: the misfit entry point that allocates nothing.

Callers that cannot allocate device memory (code whose GPU memory belongs to
a framework allocator or a fixed pool, loops that must stay free of
allocation latency) hand it device buffers for the traces and results; the reduction's scratch is a fixed array inside the library.  This
test checks it through the C ABI against psv_misfit (the allocating entry
point) on two calls in a row, so the second call runs on scratch the first
one left behind.  The buffers here are allocated by the test with torch; the
entry point itself allocates nothing.

The file is named to be collected last: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from fwi_cuda_gb300 import _lib, engine

pytestmark = pytest.mark.gpu


def _traces(seed, nshot, nrec, nt):
    rng = np.random.default_rng(seed)
    mod = rng.standard_normal((nshot, nrec, nt)) * 1e-9
    obs = mod + rng.standard_normal(mod.shape) * 3e-11
    return mod, mod[:, ::-1].copy() * 0.7, obs, obs[:, ::-1].copy() * 0.7


def _noalloc(lib, arrays, dt, stream):
    import torch
    nshot, nrec, nt = arrays[0].shape
    d_in = [torch.from_numpy(a).cuda() for a in arrays]
    d_res = [torch.full_like(d_in[0], np.nan) for _ in range(2)]
    d_L2 = torch.full((nshot,), np.nan, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ptrs = [C.c_void_p(t.data_ptr()) for t in d_in + d_res]
    rc = lib.psv_misfit_noalloc(*ptrs, nshot, nrec, nt, dt, C.c_void_p(d_L2.data_ptr()),
                                C.c_void_p(stream))
    _lib.check(rc)
    torch.cuda.synchronize()
    return d_L2.cpu().numpy(), d_res[0].cpu().numpy(), d_res[1].cpu().numpy()


def test_misfit_noalloc_matches_allocating_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    lib = _lib.lib()
    dt = 5e-5
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row with different data and shot counts: the second
    # reuses the scratch the first one filled
    for seed, shape in ((1, (5, 23, 333)), (2, (3, 40, 127))):
        arrays = _traces(seed, *shape)
        L2_ref, rz_ref, rx_ref = engine.misfit(*arrays, dt)
        L2, rz, rx = _noalloc(lib, arrays, dt, stream)
        np.testing.assert_allclose(L2, L2_ref, rtol=1e-13, atol=0)
        assert np.array_equal(rz, rz_ref) and np.array_equal(rx, rx_ref)


def test_misfit_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    lib = _lib.lib()
    n = 1025  # PSV_MISFIT_NOALLOC_MAX_SHOTS + 1: rejected before any device access
    one = C.c_void_p(1)
    rc = lib.psv_misfit_noalloc(one, one, one, one, None, None, n, 1, 1, 1.0, one, None)
    assert rc == _lib.PSV_ERR_ARG
    assert b"PSV_MISFIT_NOALLOC_MAX_SHOTS" in lib.psv_last_error()
