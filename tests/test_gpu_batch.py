"""Independent simulations in one context (eb_batch_define) against each simulation run
alone.

The reference runs one simulation per process (electric.f:134-251); a batch must give
every simulation exactly what it would get alone: no layer sum may mix simulations (the
tree is a forest with one cell per simulation), every GMRES solve runs per simulation,
and FASMVP's far-field pressure, SETVELF's E0 and its stale `alpha` are per simulation.
Checks, per simulation of the batch:
* operators (FASMVP, FASMVP_LAP, the Stokes sum) against the oracle's direct sums on that
  simulation alone, 1e-12 (FP64) and 1e-5 (FP32) relative;
* solves against the oracle's GMRES on that simulation, 1e-9 relative, iteration counts
  within one of the simulation's own;
* two RK2 steps (electric.f:762-786) of the uneven simulations (one drop each, N from 128
  to 4,096, E0 per simulation) and of multi-drop simulations against the oracle, node
  positions within 1e-10, in both solver modes.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def uneven_sample(count=6):
    """Seeded uneven simulations covering the size classes 128 .. 4096."""
    sims, seen = [], set()
    for s in configs.uneven_simulations():
        if s.nbk not in seen:
            sims.append(s)
            seen.add(s.nbk)
        if len(sims) == count:
            break
    return sims


def multi_drop_sims():
    """Simulations of several drops each (the far-field pressure of each simulation's first
    drop and the alpha of its last one differ between simulations)."""
    return [configs.small_drops(2, 64, seed=3, box=3.0), configs.small_drops(3, 128, seed=7, box=3.0),
            configs.single_drop(256), configs.small_drops(2, 256, seed=9, box=3.5)]


def concat(sims):
    nd = np.concatenate([s.nd for s in sims])
    y = np.concatenate([s.rku() for s in sims])
    return nd, y


def split(v, sims, per_node):
    out, o = [], 0
    for s in sims:
        m = per_node * s.nbk
        out.append(v[o:o + m])
        o += m
    return out


@pytest.fixture(scope="module")
def bctx(gpu_ctx_factory):
    return gpu_ctx_factory()


@pytest.mark.parametrize("group", ["uneven", "multi"])
def test_batch_operators_match_each_simulation(bctx, oracle, group):
    sims = uneven_sample() if group == "uneven" else multi_drop_sims()
    nd, y = concat(sims)
    bctx.batch_define([s.k for s in sims])
    bctx.extractdat(nd, y)
    rng = np.random.default_rng(60)
    u = rng.standard_normal(2 * int(nd.sum()))
    ul = rng.standard_normal(int(nd.sum()))
    dens = u.view(np.complex128)
    got = {p: bctx.fasmvp(u, p) for p in ("fp64", "fp32")}
    gotl = bctx.fasmvp_lap(ul, "fp64")
    gots = bctx.stokes_sum(dens, 1, "fp64")
    for s, gu, gl, gs, g64, g32, gs1 in zip(sims, split(u, sims, 2), split(ul, sims, 1), split(dens, sims, 1),
                                             split(got["fp64"], sims, 2), split(got["fp32"], sims, 2),
                                             split(gots, sims, 1)):
        ex = oracle.extractdat(s.nd, s.rku())
        g = oracle.Geometry.from_extract(s.nd, ex)
        ref = oracle.fasmvp(g, gu, 0)
        assert relmax(g64, ref) < 1e-12, s.name
        assert relmax(g32, ref) < 1e-5, s.name
        assert relmax(split(gotl, sims, 1)[sims.index(s)], oracle.fasmvp_lap(g, gl)) < 1e-12, s.name
        refs = oracle.stokes_direct(ex["z"], ex["dz"], oracle.point_h(s.nd), gs, 1)
        assert relmax(gs1, refs) < 1e-12, s.name
    bctx.batch_define([])


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_batch_solves_match_each_simulation(bctx, oracle, mode):
    sims = uneven_sample()
    nd, y = concat(sims)
    bctx.batch_define([s.k for s in sims])
    bctx.extractdat(nd, y)
    rhs = np.random.default_rng(61).standard_normal(2 * int(nd.sum()))
    got, info = bctx.solvei(rhs, mode)
    assert info["ierr"] == 0 and info["err"] <= 1e-10
    rl = -2.0 * y[0::2]
    gotl, infol = bctx.solve_lapl(rl, mode)
    assert infol["ierr"] == 0 and infol["err"] <= 1e-10
    for s, b, x, bl, xl in zip(sims, split(rhs, sims, 2), split(got, sims, 2), split(rl, sims, 1),
                               split(gotl, sims, 1)):
        g = oracle.Geometry.from_extract(s.nd, oracle.extractdat(s.nd, s.rku()))
        ref, rinfo = oracle.solvei(g, b)
        assert relmax(x, ref) < 1e-9, s.name
        refl, _ = oracle.solve_lapl(g, bl)
        assert relmax(xl, refl) < 1e-9, s.name
    bctx.batch_define([])


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
@pytest.mark.parametrize("group", ["uneven", "multi"])
def test_batch_rk2_matches_each_simulation(bctx, oracle, mode, group):
    sims = uneven_sample() if group == "uneven" else multi_drop_sims()
    e0 = np.array([s.params.get("E0", 0.3 + 0.1 * i) for i, s in enumerate(sims)])
    nd, y = concat(sims)
    bctx.batch_define([s.k for s in sims], e0)
    for _ in range(2):
        info = bctx.rk2(nd, 1e-3, y, e0=0.0, mode=mode)
        assert info["lap_ierr"] == 0 and info["stokes_ierr"] == 0
    for s, e, ys in zip(sims, e0, split(y, sims, 2)):
        m = oracle.make_model(cap=0.0, e0=float(e))
        yr = s.rku()
        for _ in range(2):
            yr = oracle.rk2(m, s.nd, 1e-3, yr)
        assert np.abs(ys - yr).max() < 1e-10, (s.name, s.nbk)
    bctx.batch_define([])


def test_batch_define_errors(bctx):
    from electricbubbles_gb300 import EbError
    sims = multi_drop_sims()
    nd, y = concat(sims)
    bctx.batch_define([1, 1])  # 2 drops declared, more installed
    with pytest.raises(EbError) as e:
        bctx.extractdat(nd, y)
    assert e.value.status == 1  # EB_ERR_ARG
    bctx.batch_define([])
    bctx.extractdat(nd, y)  # back to one simulation


def test_autotuned_batch_step_matches(gpu_ctx_factory):
    """eb_autotune on a batch's forest picks leaf sizes; an RK2 step with them gives the
    positions of the untuned step (the same operators to FMM accuracy)."""
    sims = configs.uneven_simulations(count=8, seed=17)
    nd = np.concatenate([s.nd for s in sims])
    e0 = np.array([s.params["E0"] for s in sims])
    ys = []
    for tune in (False, True):
        b = gpu_ctx_factory()
        b.batch_define([s.k for s in sims], e0)
        y = np.concatenate([s.rku() for s in sims])
        b.extractdat(nd, y.copy())
        if tune:
            info = b.autotune()
            assert len(info["candidates"]) >= 2 and (info["leaf64"], info["leaf_cap"]) in \
                [(c["leaf64"], c["leaf_cap"]) for c in info["candidates"]]
        step = b.rk2(nd, 1e-3, y, mode="fp64")
        assert step["lap_ierr"] == 0 and step["stokes_ierr"] == 0
        ys.append(y)
    assert np.abs(ys[0] - ys[1]).max() < 1e-10
