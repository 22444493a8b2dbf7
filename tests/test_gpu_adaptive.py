"""The adaptive tree on multi-scale geometries, against the oracle's direct sums.

A small dense drop (4,096 nodes on a circle of radius 0.1) sits among unit drops of 128
nodes: a uniform-depth tree would give it leaves of hundreds of points (quadratic near
field), while the adaptive tree (below its uniform floor, boxes split while they hold
more than the leaf cap, DAASSI, dapif1.f:1165-1255) refines only there. Leaves of different levels then meet,
so the U lists hold leaves of other levels (evaluated directly) and the W lists boxes
below the leaf's level (evaluated from their multipoles, M2P), which every sum here
exercises. Tolerances as in the other parity tests: FP64 1e-12, FP32 1e-5 relative to
the largest value (max norm).
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def multiscale(n_small=4096, r_small=0.1, k_big=8, n_big=128):
    """One small dense drop at the origin and k_big unit drops on a ring around it."""
    nds = [n_small] + [n_big] * k_big
    centres = [0j] + [3.2 * np.exp(2j * np.pi * (i + 0.3) / k_big) for i in range(k_big)]
    radii = [r_small] + [1.0] * k_big
    z = np.concatenate([configs.perturbed_circle(n, r, 0.05, 2, c) for n, r, c in zip(nds, radii, centres)])
    return configs.DropConfig("multiscale", nds, z, np.array(centres), np.array(radii),
                              np.full(len(nds), 0.05))


CASES = {
    "dense_among_unit": lambda: multiscale(),
    "two_scales_close": lambda: multiscale(n_small=2048, r_small=0.25, k_big=4, n_big=256),
}


@pytest.fixture(scope="module")
def ctxs(gpu_ctx_factory):
    return {"native": gpu_ctx_factory(df64=-1), "df": gpu_ctx_factory(df64=1)}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("sign", [-1, 1])
def test_stokes_sum_multiscale(ctxs, oracle, case, sign):
    cfg = CASES[case]()
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(50)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    ref = oracle.stokes_direct(ex["z"], ex["dz"], oracle.point_h(cfg.nd), dens, sign)
    for arith, ctx in ctxs.items():
        ctx.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
        assert relmax(ctx.stokes_sum(dens, sign, "fp64"), ref) < 1e-12, arith
    assert relmax(ctxs["native"].stokes_sum(dens, sign, "fp32"), ref) < 1e-5
    t = ctxs["native"].tree_info()
    assert t["w_pairs"] > 0  # the W lists are exercised
    # the dense drop's leaves lie deeper than the unit drops' ones and hold at most the
    # leaf cap (96) points, so its near field is far below the all-pairs count
    assert t["u_pairs"] < 0.25 * cfg.nbk * cfg.nd[0]


@pytest.mark.parametrize("case", list(CASES))
def test_cauchy_and_fasmvp_multiscale(ctxs, oracle, case):
    cfg = CASES[case]()
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, ex)
    rng = np.random.default_rng(51)
    q = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    refc = oracle.cauchy_direct(ex["z"], ex["z"], q, True)
    u = rng.standard_normal(2 * cfg.nbk)
    reff = oracle.fasmvp(g, u, 0)
    ul = rng.standard_normal(cfg.nbk)
    refl = oracle.fasmvp_lap(g, ul)
    for arith, ctx in ctxs.items():
        assert relmax(ctx.dapif2(ex["z"], q, "fp64"), refc) < 1e-12, arith
        ctx.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
        assert relmax(ctx.fasmvp(u, "fp64"), reff) < 1e-12, arith
        assert relmax(ctx.fasmvp_lap(ul, "fp64"), refl) < 1e-12, arith
    assert relmax(ctxs["native"].dapif2(ex["z"], q, "fp32"), refc) < 1e-5
    assert relmax(ctxs["native"].fasmvp(u, "fp32"), reff) < 1e-5


def test_solve_multiscale(ctxs, oracle):
    cfg = CASES["dense_among_unit"]()
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, ex)
    rhs = np.random.default_rng(52).standard_normal(2 * cfg.nbk)
    ref, rinfo = oracle.solvei(g, rhs)
    ctx = ctxs["native"]
    ctx.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    for mode in ("fp64", "fp32_refined"):
        got, info = ctx.solvei(rhs, mode)
        assert info["ierr"] == 0 and info["err"] <= 1e-10, mode
        assert relmax(got, ref) < 1e-9, mode


def test_autotune_picks_a_candidate_and_keeps_parity(gpu_ctx_factory, oracle):
    """eb_autotune times the FP32 operator for every leaf-size candidate on the installed
    geometry and keeps the fastest; the operators are as accurate afterwards."""
    cfg = configs.many_drops(16, 256, seed=11, box=8.0)
    ctx = gpu_ctx_factory()
    ctx.extractdat(cfg.nd, cfg.rku())
    t = ctx.autotune()
    cands = t["candidates"]
    assert len(cands) >= 4 and all(c["apply_us"] > 0 for c in cands)
    best = min(cands, key=lambda c: c["apply_us"])
    assert (t["leaf64"], t["leaf_cap"]) == (best["leaf64"], best["leaf_cap"])
    g = oracle.Geometry.from_extract(cfg.nd, oracle.extractdat(cfg.nd, cfg.rku()))
    u = np.random.default_rng(53).standard_normal(2 * cfg.nbk)
    ref = oracle.fasmvp(g, u, 0)
    assert relmax(ctx.fasmvp(u, "fp64"), ref) < 1e-12
    assert relmax(ctx.fasmvp(u, "fp32"), ref) < 1e-5
    got, info = ctx.solvei(u, "fp32_refined")
    assert info["ierr"] == 0 and info["err"] <= 1e-10
