"""The small-problem direct sums (eb_opts.direct_max, default 1,024 points).

A layer sum over at most direct_max points (one problem, no wall) is a direct O(N^2)
sum in one kernel, with the FMM's charges and post-processing. The oracle's sums are
direct too, so the GPU's FP64 sums match them to rounding (both sides round terms of up
to ~60x the result's size on these cases): 1e-12 relative for the sums and operators, 1e-5
for the FP32 operator, 1e-12 for solves at GMRES tolerance 1e-14,
iteration counts within one of the oracle's DGMRES at the default tolerance, and 1e-10
in node positions after RK2 steps. A wall or a batch keeps the FMM.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu

CASES = {
    "single256": lambda: configs.single_drop(256),
    "small3x128": lambda: configs.small_drops(3, 128),
    "small4x256": lambda: configs.small_drops(4, 256, seed=3, box=5.0),  # 1,024 points: the limit
}


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def direct_ctx(factory, **kw):
    return factory(direct_max=0, **kw)  # 0: the default limit of 1,024 points


@pytest.fixture(scope="module")
def setups(oracle):
    out = {}
    for name, mk in CASES.items():
        cfg = mk()
        ex = oracle.extractdat(cfg.nd, cfg.rku())
        g = oracle.Geometry.from_extract(cfg.nd, ex)
        rng = np.random.default_rng(70)
        dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
        h = oracle.point_h(cfg.nd)
        ref = {s: oracle.stokes_direct(ex["z"], ex["dz"], h, dens, s) for s in (-1, 1)}
        out[name] = (cfg, ex, g, dens, ref)
    return out


@pytest.mark.parametrize("case", list(CASES))
def test_direct_sums_and_operators_match_oracle(gpu_ctx_factory, setups, oracle, case):
    cfg, ex, g, dens, ref = setups[case]
    ctx = direct_ctx(gpu_ctx_factory)
    ctx.extractdat(cfg.nd, cfg.rku())
    for s in (-1, 1):
        l0 = ctx.launch_count()
        assert relmax(ctx.stokes_sum(dens, s, "fp64"), ref[s]) < 1e-12
        assert ctx.launch_count() - l0 == 2  # the charges and the direct sum
        assert relmax(ctx.stokes_sum(dens, s, "fp32"), ref[s]) < 1e-5
    u = dens.view(np.float64).copy()
    assert relmax(ctx.fasmvp(u, "fp64"), oracle.fasmvp(g, u)) < 1e-12
    assert relmax(ctx.fasmvp(u, "fp32"), oracle.fasmvp(g, u)) < 1e-5
    ul = np.random.default_rng(71).standard_normal(cfg.nbk)
    assert relmax(ctx.fasmvp_lap(ul, "fp64"), oracle.fasmvp_lap(g, ul)) < 1e-12
    assert relmax(ctx.fasmvp_lap(ul, "fp32"), oracle.fasmvp_lap(g, ul)) < 1e-5


@pytest.mark.parametrize("case", ["single256", "small3x128"])
def test_direct_and_fmm_agree(gpu_ctx_factory, setups, case):
    cfg, ex, g, dens, ref = setups[case]
    d = direct_ctx(gpu_ctx_factory)
    f = gpu_ctx_factory(direct_max=-1)
    d.extractdat(cfg.nd, cfg.rku())
    f.extractdat(cfg.nd, cfg.rku())
    u = dens.view(np.float64).copy()
    l0 = f.launch_count()
    assert relmax(d.fasmvp(u, "fp64"), f.fasmvp(u, "fp64")) < 1e-12
    assert f.launch_count() - l0 > 4  # the FMM's passes
    # the PV integral (2N fine points) and the DtN map
    ul = np.random.default_rng(72).standard_normal(cfg.nbk)
    for a, b in zip(d.dirich_neu_map(ul), f.dirich_neu_map(ul)):
        assert relmax(a, b) < 1e-11


def test_direct_cauchy_sum_on_points(gpu_ctx_factory, oracle):
    rng = np.random.default_rng(73)
    z = rng.uniform(-3, 3, 700) + 1j * rng.uniform(-3, 3, 700)
    q = rng.standard_normal(700) + 1j * rng.standard_normal(700)
    ctx = direct_ctx(gpu_ctx_factory)
    assert relmax(ctx.dapif2(z, q), oracle.cauchy_direct(z, z, q, True)) < 1e-12


@pytest.mark.parametrize("case", ["single256", "small3x128"])
def test_direct_solves_match_oracle(gpu_ctx_factory, setups, oracle, case):
    cfg, ex, g, dens, ref = setups[case]
    rng = np.random.default_rng(74)
    rhs = rng.standard_normal(2 * cfg.nbk)
    rl = -2.0 * g.z.real
    tight = direct_ctx(gpu_ctx_factory, gmres_tol=1e-14)
    tight.extractdat(cfg.nd, cfg.rku())
    xo, _ = oracle.solvei(g, rhs, tol=1e-14)
    x, info = tight.solvei(rhs, "fp64")
    assert info["ierr"] == 0 and relmax(x, xo) < 1e-12
    lo, _ = oracle.solve_lapl(g, rl, tol=1e-14)
    xl, info = tight.solve_lapl(rl, "fp64")
    assert info["ierr"] == 0 and relmax(xl, lo) < 1e-12
    ctx = direct_ctx(gpu_ctx_factory)
    ctx.extractdat(cfg.nd, cfg.rku())
    _, io = oracle.solvei(g, rhs)
    x, info = ctx.solvei(rhs, "fp64")
    assert abs(info["iters"] - io["iters"]) <= 1
    x, info = ctx.solvei(rhs, "fp32_refined")
    assert info["ierr"] == 0 and relmax(x, xo) < 1e-9


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_direct_rk2_single_drop(gpu_ctx_factory, oracle, mode):
    cfg = configs.single_drop(256)
    m = oracle.make_model(cap=0.0, e0=0.5)
    y_ref, y = cfg.rku(), cfg.rku()
    ctx = direct_ctx(gpu_ctx_factory)
    for _ in range(5):
        y_ref = oracle.rk2(m, cfg.nd, 1e-3, y_ref)
        info = ctx.rk2(cfg.nd, 1e-3, y, cap=0.0, e0=0.5, mode=mode)
        assert info["lap_ierr"] == 0 and info["stokes_ierr"] == 0
    assert np.abs(y - y_ref).max() < 1e-10


def test_wall_and_batch_keep_the_fmm(gpu_ctx_factory, oracle):
    """256 points above a wall: the images are in the sums (the FMM path)."""
    cfg = configs.wall_drops(k=4, n=64)
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    h = oracle.point_h(cfg.nd)
    dens = np.random.default_rng(75).standard_normal(cfg.nbk) * (1 + 0j)
    ref = oracle.stokes_direct(ex["z"], ex["dz"], h, dens, -1) + oracle.stokes_image_direct(ex["z"], ex["dz"], h,
                                                                                            dens, -1)
    ctx = direct_ctx(gpu_ctx_factory)
    ctx.set_wall(1)
    ctx.extractdat(cfg.nd, cfg.rku())
    assert relmax(ctx.stokes_sum(dens, -1, "fp64"), ref) < 1e-12
    # a batch of three small simulations: per simulation the same solve as alone
    sims = [configs.single_drop(128), configs.single_drop(256), configs.small_drops(2, 64)]
    b = direct_ctx(gpu_ctx_factory)
    b.batch_define([s.k for s in sims])
    b.extractdat(np.concatenate([s.nd for s in sims]), np.concatenate([s.rku() for s in sims]))
    rng = np.random.default_rng(76)
    rhs = rng.standard_normal(2 * sum(s.nbk for s in sims))
    xb, info = b.solvei(rhs, "fp64")
    assert info["ierr"] == 0
    off = 0
    for s in sims:
        one = direct_ctx(gpu_ctx_factory)
        one.extractdat(s.nd, s.rku())
        xs, _ = one.solvei(rhs[off:off + 2 * s.nbk], "fp64")
        assert relmax(xb[off:off + 2 * s.nbk], xs) < 1e-9
        off += 2 * s.nbk


def test_direct_install_checks_and_reports(gpu_ctx_factory, oracle):
    """A direct problem installs no tree: the install still rejects a non-finite node
    (EB_ERR_NAN) and the tree info reports one box whose pairs are all summed directly."""
    from electricbubbles_gb300.api import EbError
    cfg = configs.single_drop(64)
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    ctx = direct_ctx(gpu_ctx_factory)
    ctx.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    info = ctx.tree_info()
    assert info["npoints"] == 64 and info["nboxes"] == 1 and info["levels"] == 0
    assert info["u_pairs"] == 64 * 63 and info["v_pairs"] == 0
    z = ex["z"].copy()
    z[5] = np.nan
    with pytest.raises(EbError) as e:
        ctx.set_geometry(cfg.nd, z, ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    assert e.value.status == 6  # EB_ERR_NAN


@pytest.mark.parametrize("direct_max", [0, -1])
@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_rk2_nonfinite_state_is_an_error(gpu_ctx_factory, direct_max, mode):
    """A non-finite node in the RK state is EB_ERR_NAN, whether the install checks it at
    once (a tree build) or after the step (a direct-sum install inside the RK call), and
    the context stays usable."""
    from electricbubbles_gb300.api import EbError
    cfg = configs.single_drop(128)
    ctx = gpu_ctx_factory(direct_max=direct_max)
    y = cfg.rku()
    y[10] = np.nan
    with pytest.raises(EbError) as e:
        ctx.rk2(cfg.nd, 1e-3, y, e0=0.5, mode=mode)
    assert e.value.status == 6  # EB_ERR_NAN
    y = cfg.rku()
    info = ctx.rk2(cfg.nd, 1e-3, y, e0=0.5, mode=mode)
    assert info["lap_ierr"] == 0 and info["stokes_ierr"] == 0 and np.isfinite(y).all()
