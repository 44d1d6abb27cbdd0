"""Optional preconditioners on the CPU: the library's Gaussian filter weights
against the oracle's restatement of gauss_filter_kernel, and the oracle's
smoothing and Fletcher-Reeves semantics (src/cpu/n_kernel_lib_PSV.cpp:1012-1084,
src/cpu/n_PCG_PSV.cpp:13-44)."""
import numpy as np
import pytest

from fwi_cuda_gb300 import _lib, engine


@pytest.mark.parametrize("hfs", [2, 3, 4, 5, 8, -3])
def test_filter_weights_match_the_oracle(orc, hfs):
    a = engine.gauss_filter_kernel(hfs)
    assert np.array_equal(a, orc.gauss_filter_kernel(hfs))
    assert a.shape == (2 * abs(hfs) + 1,) * 2
    assert abs(a.sum() - 1.0) < 1e-14
    assert np.array_equal(a, a.T) and np.array_equal(a, a[::-1, ::-1])


@pytest.mark.parametrize("hfs", [0, 1])
def test_filter_without_width_is_rejected(hfs):
    # the reference's sigma = hfs / 2 is 0 there and its weights are NaN
    with pytest.raises(_lib.PSVError):
        engine.gauss_filter_kernel(hfs)


def test_smoothing_keeps_constants_and_the_border(orc):
    hfs = 3
    m = np.full((31, 40), 2.5)
    m[0, :] = 7.0  # border rows and columns are not filtered
    out = orc.apply_gauss_filter(m, hfs)
    assert np.array_equal(out[:hfs], m[:hfs]) and np.array_equal(out[-hfs - 1:], m[-hfs - 1:])
    assert np.array_equal(out[:, :hfs], m[:, :hfs]) and np.array_equal(out[:, -hfs - 1:], m[:, -hfs - 1:])
    inner = out[hfs + 3:-hfs - 1, hfs:-hfs - 1]
    assert np.allclose(inner, 2.5, rtol=1e-14)
    # the filtered gradient is not truncated to 0 (the reference's int sum would)
    g = np.random.default_rng(1).standard_normal((31, 40)) * 1e-20
    assert np.abs(orc.apply_gauss_filter(g, hfs)[hfs:-hfs - 1, hfs:-hfs - 1]).max() > 1e-22


def test_fletcher_reeves_steps(orc):
    rng = np.random.default_rng(2)
    g1, g2 = rng.standard_normal((2, 9, 13))
    d, old = np.zeros((9, 13)), np.zeros((9, 13))
    a = g1.copy()
    orc.PCG_PSV(d, old, a)  # first call: steepest descent
    assert np.array_equal(a, -g1) and np.array_equal(d, -g1) and np.array_equal(old, -g1)
    b = g2.copy()
    orc.PCG_PSV(d, old, b)
    beta = np.sum(g2 * g2) / np.sum(g1 * g1)
    assert np.allclose(b, -g2 + beta * -g1, rtol=1e-13, atol=0)
    assert np.array_equal(old, -g2) and np.array_equal(d, b)
