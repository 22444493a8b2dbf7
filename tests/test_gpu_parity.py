"""Parity of the CUDA path (through the C ABI) with the CPU oracle on the same inputs.

FP64 tolerances: the GPU FMM approximates the exact sums the oracle computes directly;
its truncation is set for ~1e-14 relative, and the tests allow 1e-12 relative to the
largest entry (max-norm). FP32 operator: 1e-5 relative. Solves: the GPU and oracle
GMRES take the same number of iterations (+-1) and agree within 1e-9 relative; the
refined solver's true FP64 residual is at most the GMRES tolerance 1e-10.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def geometry(oracle, cfg):
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    return ex, oracle.Geometry.from_extract(cfg.nd, ex)


def install(ctx, cfg, ex):
    ctx.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])


CASES = {
    "single256": lambda: configs.single_drop(256),
    "small3x128": lambda: configs.small_drops(3, 128),
    "drops16x256": lambda: configs.many_drops(16, 256, seed=11, box=8.0),
}


@pytest.fixture(scope="module")
def ctx(gpu_ctx_factory):
    return gpu_ctx_factory()


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("sign", [-1, 1])
def test_stokes_sum_fp64(ctx, oracle, case, sign):
    cfg = CASES[case]()
    ex, g = geometry(oracle, cfg)
    install(ctx, cfg, ex)
    rng = np.random.default_rng(10)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    ref = oracle.stokes_direct(g.z, g.dz, oracle.point_h(cfg.nd), dens, sign)
    got = ctx.stokes_sum(dens, sign, "fp64")
    assert relmax(got, ref) < 1e-12


@pytest.mark.parametrize("case", list(CASES))
def test_stokes_sum_fp32(ctx, oracle, case):
    cfg = CASES[case]()
    ex, g = geometry(oracle, cfg)
    install(ctx, cfg, ex)
    rng = np.random.default_rng(11)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    ref = oracle.stokes_direct(g.z, g.dz, oracle.point_h(cfg.nd), dens, -1)
    got = ctx.stokes_sum(dens, -1, "fp32")
    assert relmax(got, ref) < 1e-5


@pytest.mark.parametrize("n", [5, 40, 1000, 20000])
def test_cauchy_sum_random_points(ctx, oracle, n):
    rng = np.random.default_rng(n)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    q = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = oracle.cauchy_direct(z, z, q, True)
    assert relmax(ctx.dapif2(z, q, "fp64"), ref) < 1e-12
    assert relmax(ctx.dapif2(z, q, "fp32"), ref) < 1e-5


@pytest.mark.parametrize("case", list(CASES))
def test_fasmvp_matches_oracle(ctx, oracle, case):
    cfg = CASES[case]()
    ex, g = geometry(oracle, cfg)
    install(ctx, cfg, ex)
    u = np.random.default_rng(12).standard_normal(2 * cfg.nbk)
    ref = oracle.fasmvp(g, u, 0)
    assert relmax(ctx.fasmvp(u, "fp64"), ref) < 1e-12
    assert relmax(ctx.fasmvp(u, "fp32"), ref) < 1e-5


@pytest.mark.parametrize("case", list(CASES))
def test_fasmvp_lap_matches_oracle(ctx, oracle, case):
    cfg = CASES[case]()
    ex, g = geometry(oracle, cfg)
    install(ctx, cfg, ex)
    u = np.random.default_rng(13).standard_normal(cfg.nbk)
    ref = oracle.fasmvp_lap(g, u)
    assert relmax(ctx.fasmvp_lap(u, "fp64"), ref) < 1e-12
    assert relmax(ctx.fasmvp_lap(u, "fp32"), ref) < 1e-5
    np.testing.assert_allclose(ctx.laplace_constraints(u),
                               [np.sum(2 * np.pi / n * d * x) for n, d, x in
                                zip(cfg.nd, np.split(g.dsda, np.cumsum(cfg.nd)[:-1]),
                                    np.split(u, np.cumsum(cfg.nd)[:-1]))], rtol=1e-13)


def test_extractdat_matches_oracle(ctx, oracle):
    cfg = configs.small_drops(3, 128)
    ref = oracle.extractdat(cfg.nd, cfg.rku())
    got = ctx.extractdat(cfg.nd, cfg.rku())
    for key in ("zk", "dz", "dsda", "kappa", "ckern", "tha", "area"):
        assert relmax(got[key], ref[key]) < 1e-12, key


def test_fdiff_matches_oracle(ctx, oracle):
    cfg = configs.small_drops(3, 128)
    ctx.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(14)
    f = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    ref = np.concatenate([oracle.fdifff(x) for x in np.split(f, np.cumsum(cfg.nd)[:-1])])
    assert relmax(ctx.fdifff(f), ref) < 1e-12


@pytest.mark.parametrize("case", ["inverse", "zzprime"])
def test_pvintev_circle_known_answer(ctx, oracle, case):
    n = 32
    z = configs.perturbed_circle(n, 1.0, 0.0)
    ctx.extractdat([n], z.view(np.float64))
    f = 1.0 / (z - (3 + 2j)) if case == "inverse" else z
    phi = ctx.pvintev(f * (1j * z))
    np.testing.assert_allclose(phi, f / 2, atol=1e-12)


def test_pvintev_and_dtn_match_oracle(ctx, oracle):
    cfg = configs.small_drops(3, 128)
    ex = ctx.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, oracle.extractdat(cfg.nd, cfg.rku()))
    rng = np.random.default_rng(15)
    uc = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    assert relmax(ctx.pvintev(uc), oracle.pvintev(cfg.nd, g.z, uc)) < 1e-11
    u = rng.standard_normal(cfg.nbk)
    got = ctx.dirich_neu_map(u)
    ref = oracle.dirich_neu_map(g, u)
    for a, b in zip(got, ref):
        assert relmax(a, b) < 1e-10


def test_interfacenew_matches_oracle(ctx, oracle):
    cfg = configs.small_drops(3, 128)
    ex = ctx.extractdat(cfg.nd, cfg.rku())
    oex = oracle.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, oex)
    rng = np.random.default_rng(16)
    u = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    zc = np.zeros(cfg.k, complex)
    un, flux = ctx.interfacenew(u, zc, cap=0.3)
    run, rflux = oracle.interfacenew(g, oex["ckern"], zc, 0.3, u)
    assert relmax(un, run) < 1e-12
    assert abs(flux - rflux) < 1e-10 * np.abs(run).max()
    zc2 = 0.01j * np.arange(1, cfg.k + 1)
    un2, _ = ctx.interfacenew(u, zc2, cap=0.0)
    run2, _ = oracle.interfacenew(g, oex["ckern"], zc2, 0.0, u)
    assert relmax(un2, run2) < 1e-12


@pytest.mark.parametrize("case", ["single256", "small3x128"])
def test_solves_match_oracle(ctx, oracle, case):
    cfg = CASES[case]()
    ex, g = geometry(oracle, cfg)
    install(ctx, cfg, ex)
    rng = np.random.default_rng(17)
    rhs = rng.standard_normal(2 * cfg.nbk)
    ref, rinfo = oracle.solvei(g, rhs)
    got, info = ctx.solvei(rhs, "fp64")
    assert info["ierr"] == 0 and info["err"] <= 1e-10
    assert abs(info["iters"] - rinfo["iters"]) <= 1
    assert relmax(got, ref) < 1e-9
    got32, info32 = ctx.solvei(rhs, "fp32_refined")
    assert info32["ierr"] == 0 and info32["err"] <= 1e-10
    assert relmax(got32, ref) < 1e-9
    rl = -2.0 * g.z.real
    refl, _ = oracle.solve_lapl(g, rl)
    gotl, infol = ctx.solve_lapl(rl, "fp64")
    assert infol["ierr"] == 0 and relmax(gotl, refl) < 1e-9
    gotl32, infol32 = ctx.solve_lapl(rl, "fp32_refined")
    assert infol32["ierr"] == 0 and relmax(gotl32, refl) < 1e-9


def test_operator_linearity_full_size(ctx, oracle):
    """Size-independent property on the 64 x 512 workload: A(a x + b y) = a A x + b A y."""
    cfg = configs.many_drops()
    ex = ctx.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(18)
    x, y = rng.standard_normal((2, 2 * cfg.nbk))
    lhs = ctx.fasmvp(0.7 * x - 1.3 * y)
    rhs = 0.7 * ctx.fasmvp(x) - 1.3 * ctx.fasmvp(y)
    assert relmax(lhs, rhs) < 1e-13


def test_full_size_sampled_targets_vs_direct(ctx, oracle):
    """64 x 512 workload: the GPU Stokes sum on 256 sampled targets against the FP64
    direct sum over all 32,768 sources."""
    cfg = configs.many_drops()
    ex = ctx.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(19)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    got = ctx.stokes_sum(dens, -1, "fp64")
    got32 = ctx.stokes_sum(dens, -1, "fp32")
    ref = oracle.stokes_direct(ex["z"], ex["dz"], oracle.point_h(cfg.nd), dens, -1)
    assert relmax(got, ref) < 1e-12
    assert relmax(got32, ref) < 1e-5


def test_errors_are_returned(ctx, oracle):
    from electricbubbles_gb300 import EbError
    cfg = configs.single_drop(64)
    ex, g = geometry(oracle, cfg)
    install(ctx, cfg, ex)
    assert ctx._lib.eb_stokes_matvec(ctx._h, 3, None, None, 0, 0) == 1  # EB_ERR_ARG
    z = ex["z"].copy()
    z[5] = np.nan
    with pytest.raises(EbError) as e:
        ctx.set_geometry(cfg.nd, z, ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    assert e.value.status == 6  # EB_ERR_NAN
    with pytest.raises(EbError) as e:
        ctx.fasmvp(np.zeros(2 * cfg.nbk))
    assert e.value.status == 3  # EB_ERR_NOGEOM
