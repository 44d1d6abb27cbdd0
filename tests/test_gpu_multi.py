"""Several surveys of uneven size, time-step count and stencil order run
concurrently (psv_multi_forward / psv_multi_gradient) give exactly what each
survey gives on its own."""
import numpy as np
import pytest

import helpers
from fwi_cuda_gb300 import _lib, engine

pytestmark = pytest.mark.gpu

CASES = [dict(fdorder=4, nz=61, nx=91, nt=300, nshot=2),
         dict(fdorder=8, nz=75, nx=121, nt=360, nshot=3),
         dict(fdorder=2, stencil="reference", nz=50, nx=70, nt=250, nshot=1)]
SHAPE = dict(precision=32, kernels="direct", rows_per_thread=1, block=(32, 4))


def _surveys(orc):
    out = []
    for kw in CASES:
        kw = dict(dict(stencil="holberg"), **kw)
        sv, true, init = helpers.case(**kw)
        uz, ux = orc.simulate_fwd(sv, *true)
        out.append((sv, true, init, uz, ux))
    return out


def test_multi_forward_and_gradient_equal_single(gpu, orc):
    surveys = _surveys(orc)
    single = []
    for sv, true, init, uz, ux in surveys:
        with engine.Plan(sv, **SHAPE) as p:
            p.set_model(*true)
            f = p.forward()
            p.set_model(*init)
            p.set_observed(uz, ux)
            L2, g = p.gradient()
            single.append((f, L2, g))
    plans = [engine.Plan(sv, **SHAPE) for sv, *_ in surveys]
    try:
        for p, (sv, true, init, uz, ux) in zip(plans, surveys):
            p.set_model(*true)
        fw = engine.multi_forward(plans)
        for p, (sv, true, init, uz, ux) in zip(plans, surveys):
            p.set_model(*init)
            p.set_observed(uz, ux)
        L2 = engine.multi_gradient(plans)
        for k, p in enumerate(plans):
            (uz, ux), L2s, gs = single[k]
            assert np.array_equal(fw[k][0], uz) and np.array_equal(fw[k][1], ux)
            assert L2[k] == L2s
            for a, b in zip(p.get_gradient(), gs):
                assert np.array_equal(a, b)
    finally:
        for p in plans:
            p.close()


def test_multi_rejects_a_plan_listed_twice(gpu, orc):
    sv, true, init, uz, ux = _surveys(orc)[0]
    with engine.Plan(sv, **SHAPE) as p:
        p.set_model(*init)
        p.set_observed(uz, ux)
        with pytest.raises(_lib.PSVError, match="twice"):
            engine.multi_gradient([p, p])
