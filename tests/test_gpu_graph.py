"""The GMRES solves run as CUDA graphs (device-side Arnoldi loop in a conditional WHILE
node, DHEQR/DHELS on the device) by default. They must take the same iterations and give
the same solutions as the host-driven loop (graphs = -1), which follows DPIGMR step by
step on the host. Tolerance on the solutions: 1e-13 relative in FP64 mode (same kernels;
only the host/device rounding of the Givens and back-substitution arithmetic differs);
1e-11 in refined mode, where such rounding differences reach the FP32 operator's input
and change its float rounding (both solutions still meet the 1e-10 residual)."""
import numpy as np
import pytest

from electricbubbles_gb300 import EbError, configs
from electricbubbles_gb300.api import Context

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def pair():
    g = Context(graphs=1, direct_max=-1)
    e = Context(graphs=-1, direct_max=-1)
    yield g, e
    g.close()
    e.close()


@pytest.mark.parametrize("case", ["single256", "drops16x256"])
@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_graph_solve_matches_host_loop(pair, case, mode):
    cfg = {"single256": lambda: configs.single_drop(256),
           "drops16x256": lambda: configs.many_drops(16, 256, seed=11, box=8.0)}[case]()
    g, e = pair
    tol = 1e-13 if mode == "fp64" else 1e-11
    ex = g.extractdat(cfg.nd, cfg.rku())
    e.extractdat(cfg.nd, cfg.rku())
    rhs = np.ascontiguousarray(-0.5 * ex["dz"] / ex["dsda"]).view(np.float64).copy()
    xg, ig = g.solvei(rhs, mode)
    xe, ie = e.solvei(rhs, mode)
    assert ig["graph"] == 1 and ie["graph"] == 0
    for key in ("iters", "outer", "matvecs64", "matvecs32", "ierr"):
        assert ig[key] == ie[key], key
    # the refined mode's error is the true residual, a cancellation-limited quantity
    assert ig["err"] <= 1e-10 and ie["err"] <= 1e-10
    assert abs(ig["err"] - ie["err"]) <= 0.05 * ie["err"] + 1e-14
    assert relmax(xg, xe) < tol
    rl = -2.0 * ex["z"].real.copy()
    lg, jg = g.solve_lapl(rl, mode)
    le, je = e.solve_lapl(rl, mode)
    assert jg["graph"] == 1 and jg["iters"] == je["iters"] and jg["ierr"] == 0
    assert relmax(lg, le) < tol


def test_graph_reuse_and_launch_count(pair):
    """A second solve on the same geometry reuses the captured graph; launch counts
    advance by the kernels the graph executed."""
    g, _ = pair
    cfg = configs.small_drops(3, 128)
    ex = g.extractdat(cfg.nd, cfg.rku())
    rhs = np.ascontiguousarray(-0.5 * ex["dz"] / ex["dsda"]).view(np.float64).copy()
    l0 = g.launch_count()
    x1, i1 = g.solvei(rhs, "fp32_refined")
    l1 = g.launch_count()
    x2, i2 = g.solvei(rhs, "fp32_refined")
    l2 = g.launch_count()
    assert np.array_equal(x1, x2)
    assert i1["iters"] == i2["iters"]
    assert l1 - l0 == l2 - l1 > 0


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_graph_zero_and_nonfinite_rhs(pair, mode):
    g, e = pair
    cfg = configs.single_drop(64)
    g.extractdat(cfg.nd, cfg.rku())
    x, info = g.solvei(np.zeros(2 * cfg.nbk), mode)
    assert info["ierr"] == 0 and not np.any(x)
    bad = np.ones(2 * cfg.nbk)
    bad[7] = np.nan
    with pytest.raises(EbError) as ex:
        g.solvei(bad, mode)
    assert ex.value.status == 6  # EB_ERR_NAN
    # the context stays usable
    x, info = g.solvei(np.ones(2 * cfg.nbk), mode)
    assert info["ierr"] == 0 and info["err"] <= 1e-10


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_graph_across_geometry_installs(mode):
    """Captured graphs are reused only while everything they take by value from the
    geometry is unchanged: re-installing the same geometry reproduces the first solve bit
    for bit, and a different geometry of the same sizes solves as in a fresh context."""
    a = configs.many_drops(8, 128, seed=21, box=5.0)
    b = configs.many_drops(8, 128, seed=22, box=5.0)
    g = Context(graphs=1, direct_max=-1)
    f = Context(graphs=1, direct_max=-1)
    try:
        def solve(ctx, cfg):
            ex = ctx.extractdat(cfg.nd, cfg.rku())
            rhs = np.ascontiguousarray(-0.5 * ex["dz"] / ex["dsda"]).view(np.float64).copy()
            return ctx.solvei(rhs, mode)
        xa1, ia1 = solve(g, a)
        xb, ib = solve(g, b)
        xa2, ia2 = solve(g, a)
        xf, jf = solve(f, b)
        assert ia1["graph"] == ib["graph"] == ia2["graph"] == 1
        assert np.array_equal(xa1, xa2) and ia1["iters"] == ia2["iters"]
        assert ib["iters"] == jf["iters"]
        assert np.array_equal(xb, xf)
    finally:
        g.close()
        f.close()
