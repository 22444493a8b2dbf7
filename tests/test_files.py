"""The reference's input deck and checkpoint files (host only, no GPU): `bubbin` as
READINI reads it, GEOINIT's initial curves, and `geometry.data` as DUMPDATA writes and
READDATA reads it. tests/golden/bubbin_deck3 is a three-drop deck in the reference's
layout followed by a second deck that READINI never reads."""
import os

import numpy as np
import pytest

from electricbubbles_gb300 import files

HERE = os.path.dirname(os.path.abspath(__file__))
DECK = os.path.join(HERE, "golden", "bubbin_deck3")


@pytest.fixture(scope="module")
def lib_built():
    from electricbubbles_gb300 import _lib
    if not os.path.exists(_lib.library_path()):
        pytest.skip("libeb_gb300.so not built")


def test_read_bubbin_first_deck(lib_built):
    d = files.read_bubbin(DECK)
    assert d["k"] == 3
    assert list(d["nd"]) == [64, 128, 256]
    assert (d["dt"], d["tfinal"], d["nplot"]) == (0.005, 0.25, 5)
    assert d["cap"] == 0.1 and d["zbond"] == 0j and d["E0"] == 0.75
    np.testing.assert_array_equal(d["ai"], [1.0, 1.2, 0.9])
    np.testing.assert_array_equal(d["bi"], [1.0, 0.8, 0.1])
    np.testing.assert_array_equal(d["thetax"], [0.0, 0.3, 0.0])
    np.testing.assert_array_equal(d["zk"], [-2.0 + 0.5j, 1.5 - 1.0j, 0.0 + 2.5j])
    np.testing.assert_array_equal(d["ncyc"], [0, 0, 5])


def test_geoinit_shapes(lib_built):
    d = files.read_bubbin(DECK)
    z, dsdth, kappa, area0 = files.geoinit(d)
    n0, n1, n2 = d["nd"]
    th0 = 2 * np.pi * np.arange(n0) / n0
    # circle of radius 1: unit curvature, |z - zk| = 1, dsdth = 1
    np.testing.assert_allclose(np.abs(z[:n0] - d["zk"][0]), 1.0, atol=1e-14)
    np.testing.assert_allclose(z[:n0], d["zk"][0] + np.exp(1j * th0), atol=1e-14)
    np.testing.assert_allclose(kappa[:n0], 1.0, atol=1e-13)
    np.testing.assert_allclose(dsdth[:n0], 1.0, atol=1e-14)
    # rotated ellipse: the point lies on the rotated ellipse at polar angle theta
    w = z[n0:n0 + n1] - d["zk"][1]
    u = w * np.exp(-1j * d["thetax"][1])
    np.testing.assert_allclose((u.real / 1.2) ** 2 + (u.imag / 0.8) ** 2, 1.0, atol=1e-13)
    th1 = 2 * np.pi * np.arange(n1) / n1
    np.testing.assert_allclose(np.angle(w), np.angle(np.exp(1j * th1)), atol=1e-13)
    # starfish a e^{i t} + eps e^{-i n t}
    th2 = 2 * np.pi * np.arange(n2) / n2
    np.testing.assert_allclose(z[n0 + n1:], d["zk"][2] + 0.9 * np.exp(1j * th2) + 0.1 * np.exp(-5j * th2),
                               atol=1e-14)
    np.testing.assert_allclose(area0, [np.pi, np.pi * 1.2 * 0.8, np.pi * (0.81 - 5 * 0.01)])
    # curvature of the ellipse against the spectral derivative of the samples
    zp = np.fft.ifft(1j * np.fft.fftfreq(n1, 1.0 / n1) * np.fft.fft(w))
    zpp = np.fft.ifft(-np.fft.fftfreq(n1, 1.0 / n1) ** 2 * np.fft.fft(w))
    kap = (zp.real * zpp.imag - zp.imag * zpp.real) / np.abs(zp) ** 3
    np.testing.assert_allclose(kappa[n0:n0 + n1], kap, atol=1e-9)


def test_geometry_data_round_trip(lib_built, tmp_path):
    rng = np.random.default_rng(3)
    nd = np.array([16, 32], np.int32)
    z = rng.standard_normal(48) * 10 + 1j * rng.standard_normal(48) * 10
    z[0] = 0.0
    z[1] = -1e-5 + 3e120j
    area0 = np.array([np.pi, -2.5])
    arcl0 = np.array([6.283185307179586, 1e-3])
    path = tmp_path / "geometry.data"
    files.dumpdata(path, nd, 1e-3, 0.125, area0, arcl0, z)
    lines = path.read_text().splitlines()
    assert lines[0] == "%12d%12d%12d" % (2, 48, 96)
    assert lines[1] == "%12d%12d" % (16, 32)
    assert lines[2] == "0.1000000000000000E-02  0.1250000000000000E+00"
    assert lines[3] == "0.3141592653589793E+01"
    assert lines[4] == "-.2500000000000000E+01"
    assert lines[7] == "0.0000000000000000E+00  0.0000000000000000E+00"
    assert lines[8] == "-.1000000000000000E-04  0.3000000000000000+121"
    assert len(lines) == 3 + 2 + 2 + 48
    assert all(len(x) == 22 for x in lines[3:7])
    nd2, dt, time, a2, l2, z2 = files.readdata(path)
    np.testing.assert_array_equal(nd2, nd)
    assert (dt, time) == (1e-3, 0.125)
    np.testing.assert_allclose(a2, area0, rtol=1e-15)
    np.testing.assert_allclose(l2, arcl0, rtol=1e-15)
    np.testing.assert_allclose(z2, z, rtol=1e-15, atol=0)


def test_bad_files_are_reported(lib_built, tmp_path):
    from electricbubbles_gb300 import EbError
    p = tmp_path / "bubbin"
    p.write_text("2\n64\n")
    with pytest.raises(EbError):
        files.read_bubbin(p)
    with pytest.raises(EbError):
        files.read_bubbin(tmp_path / "missing")
    q = tmp_path / "geometry.data"
    q.write_text("1 10 20\n12\n")
    with pytest.raises(EbError):
        files.readdata(q)
