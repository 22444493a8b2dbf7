"""The transposed operators and adjoint solves on the GPU.

The reference has no adjoint; the transposes are checked against the dense transpose
of the oracle's FASMVP / FASMVP_LAP (built column by column on a small geometry), by the
dot-product identity <v, A u> = <A^T v, u> on the workloads, and through a gradient: for
J(E0) = <c, x(E0)> with A x = SETVELF(dphi, cap, E0), dJ/dE0 = <lambda, db/dE0> with
A^T lambda = c, against central differences of the GPU's forward solves and against the
oracle's dense solves. Bars: 1e-12 relative for the FP64-class transposes, 1e-6 for the
FP32 ones, 1e-9 for solves.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs
from electricbubbles_gb300.api import EbError

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def small(oracle):
    cfg = configs.small_drops(3, 32)
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, ex)
    n = cfg.nbk
    A = np.empty((2 * n, 2 * n))
    for c in range(2 * n):
        e = np.zeros(2 * n)
        e[c] = 1.0
        A[:, c] = oracle.fasmvp(g, e)
    AL = np.empty((n, n))
    for c in range(n):
        e = np.zeros(n)
        e[c] = 1.0
        AL[:, c] = oracle.fasmvp_lap(g, e)
    return cfg, ex, A, AL


@pytest.mark.parametrize("arith", ["native", "df", "fp32"])
def test_adjoint_matches_dense_transpose(gpu_ctx_factory, small, arith):
    cfg, ex, A, AL = small
    ctx = gpu_ctx_factory(df64=1 if arith == "df" else -1)
    ctx.extractdat(cfg.nd, cfg.rku())
    prec = "fp32" if arith == "fp32" else "fp64"
    bar = 1e-6 if arith == "fp32" else 1e-12
    rng = np.random.default_rng(60)
    for _ in range(2):
        v = rng.standard_normal(2 * cfg.nbk)
        assert relmax(ctx.fasmvp_adjoint(v, prec), A.T @ v) < bar
        vl = rng.standard_normal(cfg.nbk)
        assert relmax(ctx.fasmvp_lap_adjoint(vl, prec), AL.T @ vl) < bar


@pytest.mark.parametrize("case", ["drops16x256", "drops64x512"])
@pytest.mark.parametrize("arith", ["native", "df", "fp32"])
def test_adjoint_dot_product_identity(gpu_ctx_factory, case, arith):
    cfg = configs.many_drops(16, 256, seed=11, box=8.0) if case == "drops16x256" else configs.many_drops()
    ctx = gpu_ctx_factory(df64=1 if arith == "df" else -1)
    ctx.extractdat(cfg.nd, cfg.rku())
    prec = "fp32" if arith == "fp32" else "fp64"
    bar = 1e-6 if arith == "fp32" else 1e-13
    rng = np.random.default_rng(61)
    u, v = rng.standard_normal(2 * cfg.nbk), rng.standard_normal(2 * cfg.nbk)
    au, atv = ctx.fasmvp(u, prec), ctx.fasmvp_adjoint(v, prec)
    assert abs(v @ au - atv @ u) < bar * np.linalg.norm(v) * np.linalg.norm(au)
    ul, vl = rng.standard_normal(cfg.nbk), rng.standard_normal(cfg.nbk)
    au, atv = ctx.fasmvp_lap(ul, prec), ctx.fasmvp_lap_adjoint(vl, prec)
    assert abs(vl @ au - atv @ ul) < bar * np.linalg.norm(vl) * np.linalg.norm(au)


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_adjoint_solves_match_dense(gpu_ctx_factory, small, mode):
    cfg, ex, A, AL = small
    ctx = gpu_ctx_factory()
    ctx.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(62)
    b = rng.standard_normal(2 * cfg.nbk)
    lam, info = ctx.solvei_adjoint(b, mode)
    assert info["ierr"] == 0
    assert relmax(lam, np.linalg.solve(A.T, b)) < 1e-9
    bl = rng.standard_normal(cfg.nbk)
    lam, info = ctx.solve_lapl_adjoint(bl, mode)
    assert info["ierr"] == 0
    assert relmax(lam, np.linalg.solve(AL.T, bl)) < 1e-9


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_gradient_wrt_e0(gpu_ctx_factory, oracle, mode):
    """dJ/dE0 of J = <c, x>, A x = SETVELF(dphi, cap, E0), by one adjoint solve."""
    cfg = configs.many_drops(16, 256, seed=11, box=8.0)
    ctx = gpu_ctx_factory()
    ex = ctx.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(63)
    dphi = rng.standard_normal(cfg.nbk)
    c = rng.standard_normal(2 * cfg.nbk)
    e0, cap = 0.5, 0.1
    db = ctx.setvelf(dphi, cap, 1.0) - ctx.setvelf(dphi, cap, 0.0)  # the rhs is affine in E0
    lam, info = ctx.solvei_adjoint(c, mode)
    assert info["ierr"] == 0
    grad = lam @ db
    hstep = 1e-2

    def J(e):
        x, inf = ctx.solvei(ctx.setvelf(dphi, cap, e), "fp64")
        return c @ x
    fd = (J(e0 + hstep) - J(e0 - hstep)) / (2 * hstep)
    assert abs(grad - fd) < 1e-8 * abs(fd)
    # and against the oracle's own solve (exact direct sums)
    g = oracle.Geometry.from_extract(cfg.nd, oracle.extractdat(cfg.nd, cfg.rku()))
    xo, _ = oracle.solvei(g, db, tol=1e-13)
    assert abs(grad - c @ xo) < 1e-8 * abs(c @ xo)


def test_adjoint_solves_in_a_batch(gpu_ctx_factory):
    """A batch's transposed operator is block diagonal: per simulation, the same solve."""
    sims = configs.uneven_simulations(count=3, seed=13)
    nd = np.concatenate([s.nd for s in sims])
    y = np.concatenate([s.rku() for s in sims])
    b = gpu_ctx_factory()
    b.batch_define([s.k for s in sims])
    b.extractdat(nd, y)
    rng = np.random.default_rng(64)
    rhs = rng.standard_normal(2 * int(nd.sum()))
    lam, info = b.solvei_adjoint(rhs, "fp64")
    assert info["ierr"] == 0
    off = 0
    for s in sims:
        one = gpu_ctx_factory()
        one.extractdat(s.nd, s.rku())
        m = 2 * s.nbk
        ref, _ = one.solvei_adjoint(rhs[off:off + m], "fp64")
        assert relmax(lam[off:off + m], ref) < 1e-9
        off += m


def test_adjoint_refused_on_a_wall(gpu_ctx_factory):
    cfg = configs.wall_drops(k=4, n=64)
    ctx = gpu_ctx_factory()
    ctx.set_wall(1)
    ctx.extractdat(cfg.nd, cfg.rku())
    with pytest.raises(EbError):
        ctx.fasmvp_adjoint(np.ones(2 * cfg.nbk))
    with pytest.raises(EbError):
        ctx.solvei_adjoint(np.ones(2 * cfg.nbk))
