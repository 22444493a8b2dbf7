"""The deflated Laplace solve (eb_opts.lap_deflate).

FASMVP_LAP (laplace.f:159-262) maps a constant density on drop k to -2 h_k s' times it
(the double layer of a constant vanishes off its curve and cancels the identity on it;
the -2 h u s' term, laplace.f:235-236, remains), so the k drop constants are
eigenvectors with small, distinct eigenvalues and unpreconditioned GMRES pays about one
iteration per drop. The option right-preconditions the same GMRES by the deflation of
those modes. CPU tests pin the premise and the algorithm on the oracle (exact direct
sums); GPU tests check the CUDA path against the oracle's deflated and plain solves and
against the GPU's own plain solve. Bars: 1e-10 relative for the eigen-relation (the
quadrature error at nearby drops), 1e-13 for M M^-1 = I, 1e-9 for
solutions at the default tolerance 1e-10, 1e-12 at 1e-14, 1e-10 for RK2 positions.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def geometry(oracle, cfg):
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    return ex, oracle.Geometry.from_extract(cfg.nd, ex)


def test_drop_constants_are_laplace_eigenvectors(oracle):
    cfg = configs.many_drops(8, 64, seed=11, box=7.0)
    ex, g = geometry(oracle, cfg)
    off = 0
    for n in cfg.nd:
        v = np.zeros(cfg.nbk)
        v[off:off + n] = 1.0
        av = oracle.fasmvp_lap(g, v)
        mu = -2.0 * (2.0 * np.pi / n) * ex["dsda"][off:off + n].mean()
        assert mu < 0
        # exact up to the trapezoidal rule's error for the double layer of a constant
        # at the nodes of a nearby drop (5e-12 here, with 64 nodes per drop)
        assert np.linalg.norm(av - mu * v) < 1e-10 * np.linalg.norm(av)
        off += n


def test_deflation_pair_is_inverse(oracle):
    cfg = configs.many_drops(4, 64, seed=3, box=5.0)
    ex, g = geometry(oracle, cfg)
    x = np.random.default_rng(0).standard_normal(cfg.nbk)
    y = oracle.deflate(cfg.nd, ex["dsda"], oracle.deflate(cfg.nd, ex["dsda"], x, True), False)
    assert relmax(y, x) < 1e-13


def test_deflated_gmres_same_solution_fewer_iterations(oracle):
    cfg = configs.many_drops(16, 64, seed=11, box=10.0)
    ex, g = geometry(oracle, cfg)
    b = -2.0 * g.z.real  # GETBCs (laplace.f:14-18)
    xp, ip = oracle.solve_lapl(g, b, tol=1e-13)
    xd, idf = oracle.solve_lapl_deflated(g, b, tol=1e-13)
    assert ip["ierr"] == 0 and idf["ierr"] == 0
    assert relmax(xd, xp) < 1e-11
    assert np.linalg.norm(b - oracle.fasmvp_lap(g, xd)) < 1e-12 * np.linalg.norm(b)
    assert idf["iters"] <= ip["iters"] // 2, (idf["iters"], ip["iters"])


# ---- the CUDA path -------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("graphs", [1, -1])
@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_gpu_deflated_solve_matches_oracle(gpu_ctx_factory, oracle, mode, graphs):
    cfg = configs.many_drops(16, 256, seed=11, box=8.0)
    ex, g = geometry(oracle, cfg)
    b = -2.0 * g.z.real
    xo, io = oracle.solve_lapl_deflated(g, b, tol=1e-14)
    ctx = gpu_ctx_factory(lap_deflate=1, graphs=graphs)
    ctx.extractdat(cfg.nd, cfg.rku())
    x, info = ctx.solve_lapl(b, mode)
    assert info["ierr"] == 0 and info["err"] <= 1e-10
    assert relmax(x, xo) < 1e-9
    if mode == "fp64":
        # the same Krylov iterates as the oracle's deflated GMRES (at 1e-10)
        _, io10 = oracle.solve_lapl_deflated(g, b, tol=1e-10)
        assert abs(info["iters"] - io10["iters"]) <= 1


@pytest.mark.gpu
def test_gpu_deflated_solve_tight_tolerance(gpu_ctx_factory, oracle):
    """At GMRES tolerance 1e-14 the deflated solve gives the unpreconditioned oracle
    solve's density within 1e-12: the same linear system."""
    cfg = configs.small_drops(3, 128)
    ex, g = geometry(oracle, cfg)
    b = -2.0 * g.z.real
    xo, _ = oracle.solve_lapl(g, b, tol=1e-14)
    ctx = gpu_ctx_factory(lap_deflate=1, gmres_tol=1e-14)
    ctx.extractdat(cfg.nd, cfg.rku())
    x, info = ctx.solve_lapl(b, "fp64")
    assert info["ierr"] == 0
    assert relmax(x, xo) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_gpu_deflation_iterations_and_solution_64x512(gpu_ctx_factory, mode):
    cfg = configs.many_drops()
    plain = gpu_ctx_factory()
    defl = gpu_ctx_factory(lap_deflate=1)
    ex = plain.extractdat(cfg.nd, cfg.rku())
    defl.extractdat(cfg.nd, cfg.rku())
    b = -2.0 * np.asarray(ex["z"]).real
    xp, ip = plain.solve_lapl(b, mode)
    xd, idf = defl.solve_lapl(b, mode)
    assert ip["ierr"] == 0 and idf["ierr"] == 0
    assert relmax(xd, xp) < 1e-9
    # true residual of the deflated solution through the plain FP64 operator
    r = b - plain.fasmvp_lap(xd, "fp64")
    assert np.abs(r).max() < 1e-9 * np.abs(b).max()
    assert idf["iters"] <= 0.4 * ip["iters"], (idf["iters"], ip["iters"])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_gpu_rk2_with_deflation(gpu_ctx_factory, mode):
    cfg = configs.many_drops(16, 256, seed=11, box=8.0)
    ya, yb = cfg.rku(), cfg.rku()
    plain = gpu_ctx_factory()
    defl = gpu_ctx_factory(lap_deflate=1)
    for _ in range(2):
        ia = plain.rk2(cfg.nd, 1e-3, ya, e0=0.5, mode=mode)
        ib = defl.rk2(cfg.nd, 1e-3, yb, e0=0.5, mode=mode)
        assert ia["lap_ierr"] == 0 and ib["lap_ierr"] == 0
        assert ib["lap_iters"] < ia["lap_iters"]
    assert np.abs(ya - yb).max() < 1e-10


@pytest.mark.gpu
def test_gpu_deflation_leaves_stokes_and_adjoint_alone(gpu_ctx_factory):
    cfg = configs.small_drops(3, 64)
    a = gpu_ctx_factory()
    b = gpu_ctx_factory(lap_deflate=1)
    a.extractdat(cfg.nd, cfg.rku())
    b.extractdat(cfg.nd, cfg.rku())
    rhs = np.random.default_rng(5).standard_normal(2 * cfg.nbk)
    xa, ia = a.solvei(rhs)
    xb, ib = b.solvei(rhs)
    assert ia["iters"] == ib["iters"] and np.array_equal(xa, xb)
    rl = rhs[:cfg.nbk]
    la, ja = a.solve_lapl_adjoint(rl)
    lb, jb = b.solve_lapl_adjoint(rl)
    assert ja["iters"] == jb["iters"] and np.array_equal(la, lb)


@pytest.mark.gpu
def test_gpu_deflation_in_wall_mode(gpu_ctx_factory):
    """The wall's images enter the Stokes sums only; the Laplace operator and its drop
    constants are unchanged, and the deflated solve gives the plain one's density."""
    cfg = configs.wall_drops()
    plain = gpu_ctx_factory()
    defl = gpu_ctx_factory(lap_deflate=1)
    for c in (plain, defl):
        c.set_wall(1)
    ex = plain.extractdat(cfg.nd, cfg.rku())
    defl.extractdat(cfg.nd, cfg.rku())
    b = -2.0 * np.asarray(ex["z"]).real
    xp, ip = plain.solve_lapl(b, "fp64")
    xd, idf = defl.solve_lapl(b, "fp64")
    assert ip["ierr"] == 0 and idf["ierr"] == 0
    assert relmax(xd, xp) < 1e-9
    assert idf["iters"] < ip["iters"]
