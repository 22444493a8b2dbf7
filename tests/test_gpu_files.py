"""A run started the reference's way: the first deck of a `bubbin` file (READINI), its
GEOINIT curves, two RK2 steps on the GPU against the oracle (positions within 1e-10),
and the state written and read back as `geometry.data` (DUMPDATA / READDATA)."""
import os

import numpy as np
import pytest

from electricbubbles_gb300 import files

pytestmark = pytest.mark.gpu
DECK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bubbin_deck3")


def test_deck_to_rk2_to_dump(gpu_ctx_factory, oracle, tmp_path):
    ctx = gpu_ctx_factory()
    d = files.read_bubbin(DECK)
    z, dsdth, kappa, area0 = files.geoinit(d)
    y = np.ascontiguousarray(z).view(np.float64).copy()
    y_ref = y.copy()
    m = oracle.make_model(cap=d["cap"], e0=d["E0"])
    for _ in range(2):
        y_ref = oracle.rk2(m, d["nd"], d["dt"], y_ref)
        ctx.rk2(d["nd"], d["dt"], y, cap=d["cap"], e0=d["E0"])
    assert np.abs(y - y_ref).max() < 1e-10
    zs = y.view(np.complex128)
    geo = ctx.extractdat(d["nd"], y)
    arcl = np.array([np.sum(geo["dsda"][a:b]) * 2 * np.pi / n
                     for a, b, n in zip(np.r_[0, np.cumsum(d["nd"])[:-1]], np.cumsum(d["nd"]), d["nd"])])
    path = tmp_path / "geometry.data"
    files.dumpdata(path, d["nd"], d["dt"], 2 * d["dt"], geo["area"], arcl, zs)
    nd2, dt2, t2, a2, l2, z2 = files.readdata(path)
    np.testing.assert_array_equal(nd2, d["nd"])
    assert dt2 == d["dt"] and abs(t2 - 2 * d["dt"]) < 1e-18
    np.testing.assert_allclose(z2, zs, rtol=1e-15, atol=1e-300)
    np.testing.assert_allclose(a2, geo["area"], rtol=1e-15)
