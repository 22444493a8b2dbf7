"""GETFOURIER and DOUBLE, the time loop's point-doubling policy (electric.f:181-219), on
the GPU.

GETFOURIER (electric.f:531-570) takes each drop's Fourier coefficients c = DCFFTF(z)/nd
and flags the drop for doubling when one of the ten modes below the Nyquist mode has
|c_i| + |c_{nd-i}| > 1e-11; DOUBLE (electric.f:721-757) resamples a flagged drop to
2 nd nodes with FINTERC (pv_integral.f:276-328). Checked against numpy's FFT (the same
exp(-i..) convention as DCFFTF) for the coefficients and flags, and against the oracle's
FINTERC for the resampling, 1e-13 relative; the even nodes of a doubled drop are its
original nodes.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def drops():
    """Three drops: smooth ones (no doubling) and one with content in its top modes."""
    z1 = configs.perturbed_circle(128, 1.0, 0.05, 2, 0j)
    z2 = configs.perturbed_circle(256, 0.8, 0.05, 2, 3 + 0j)
    t = 2 * np.pi * np.arange(128) / 128
    z3 = (-3 + 0.5j) + 0.9 * np.exp(1j * t) * (1 + 1e-8 * np.cos(60 * t))  # mode 60 of 64
    nd = np.array([128, 256, 128], np.int32)
    return nd, np.concatenate([z1, z2, z3])


def test_getfourier_flags_and_modes(gpu_ctx_factory):
    ctx = gpu_ctx_factory()
    nd, z = drops()
    idoub, fmode = ctx.getfourier(nd, z.view(np.float64))
    starts = np.r_[0, np.cumsum(nd)]
    for b, (a, n) in enumerate(zip(starts[:-1], nd)):
        c = np.fft.fft(z[a:a + n]) / n
        h = n // 2
        ref = np.abs(c[:h]) + np.r_[0.0, np.abs(c[n - 1:n - h:-1])]
        np.testing.assert_allclose(fmode[b], ref, rtol=1e-12, atol=1e-16)
        flag = int(any(ref[i] > 1e-11 for i in range(max(1, h - 10), h)))
        assert idoub[b] == flag
    assert list(idoub) == [0, 0, 1]


def test_double_matches_finterc(gpu_ctx_factory, oracle):
    ctx = gpu_ctx_factory()
    nd, z = drops()
    flags = np.array([1, 0, 1], np.int32)
    nd2, y2 = ctx.double(nd, z.view(np.float64), flags)
    assert list(nd2) == [256, 256, 256]
    z2 = y2.view(np.complex128)
    s_in, s_out = np.r_[0, np.cumsum(nd)], np.r_[0, np.cumsum(nd2)]
    for b in range(3):
        zin = z[s_in[b]:s_in[b + 1]]
        got = z2[s_out[b]:s_out[b + 1]]
        if flags[b]:
            ref = oracle.finterc(zin)
            assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-13
            assert np.abs(got[0::2] - zin).max() < 1e-12  # the original nodes
        else:
            np.testing.assert_array_equal(got, zin)
