"""Wall-bounded flow (zbond != 0, the IFLAG2 = 1 branch) on the GPU against the oracle.

With a wall at y = 0 the reference's Stokes sums (CADAPDR for FASMVP, CADAPMOD for
INTERFACENEW) add the images of all sources across the wall: reflected multipoles of
the first two rows of every level (MPREFLECT + MKINTR, cadapdrop2.f:159-197) and the
reflected near field of the first row (MKNBRRFL + SLDREFDR, cadapdrop2.f:690-721); SETVELF
and INTERFACENEW add REFSING's reflected log sources (reflect.f:28-86). The GPU sums are
checked against the oracle's exact direct-plus-image sums and its restatement of the
wall-bounded CADAPDR; SETVELF, INTERFACENEW, FASMVP, the solves and RK2 steps against the
oracle's wall branch. Bars as for free space: 1e-12 relative for the FP64-class sums
(native and double-float), 1e-5 for the FP32 operator, 1e-10 for positions after a step.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs
from electricbubbles_gb300.api import EbError

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def near_wall():
    """Six drops of 128 nodes moved down until the lowest node is 0.02 above the wall."""
    cfg = configs.wall_drops(k=6, n=128, seed=9, box=4.0, gap=0.05)
    cfg.z = cfg.z - 1j * (cfg.z.imag.min() - 0.02)
    return cfg


CASES = {
    "wall16x256": lambda: configs.wall_drops(),
    "near6x128": near_wall,
    "wall48x512": lambda: configs.wall_drops(k=48, n=512, seed=10, box=20.0),
}


@pytest.fixture(scope="module")
def setups(oracle):
    out = {}
    for name, mk in CASES.items():
        cfg = mk()
        ex = oracle.extractdat(cfg.nd, cfg.rku())
        rng = np.random.default_rng(40)
        dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
        h = oracle.point_h(cfg.nd)
        ref = {}
        for s in (-1, 1):
            ref[s] = oracle.stokes_direct(ex["z"], ex["dz"], h, dens, s) + \
                oracle.stokes_image_direct(ex["z"], ex["dz"], h, dens, s)
        out[name] = (cfg, ex, dens, ref)
    return out


def wall_ctx(factory, cfg, **kw):
    ctx = factory(**kw)
    ctx.set_wall(1)
    ctx.extractdat(cfg.nd, cfg.rku())
    return ctx


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("arith", ["native", "df", "fp32"])
def test_wall_stokes_sums_match_exact_images(gpu_ctx_factory, setups, case, arith):
    cfg, ex, dens, ref = setups[case]
    ctx = wall_ctx(gpu_ctx_factory, cfg, df64=1 if arith == "df" else -1)
    prec = "fp32" if arith == "fp32" else "fp64"
    bar = 1e-5 if arith == "fp32" else 1e-12
    for s in (-1, 1):
        got = ctx.stokes_sum(dens, s, prec)
        assert relmax(got, ref[s]) < bar, (case, arith, s, relmax(got, ref[s]))


def test_wall_sum_matches_restated_cadapdr(gpu_ctx_factory, setups, oracle):
    cfg, ex, dens, _ = setups["wall16x256"]
    ctx = wall_ctx(gpu_ctx_factory, cfg)
    iw, xl, sl = ctx.get_wall()
    oxl, osl = oracle.wallinfo(ex["z"])
    assert iw == 1 and abs(xl - oxl) < 1e-12 and abs(sl - osl) < 1e-12 * osl
    h = oracle.point_h(cfg.nd)
    for s in (-1, 1):
        ref = oracle.cadap_fmm_wall(ex["z"], ex["dz"], h, dens, s, oxl, osl)
        assert relmax(ctx.stokes_sum(dens, s, "fp64"), ref) < 1e-11


def test_wall_mode_switches_on_installed_geometry(gpu_ctx_factory, setups, oracle):
    """eb_set_wall on an installed geometry rebuilds its tree: free, wall, free again."""
    cfg, ex, dens, ref = setups["wall16x256"]
    ctx = gpu_ctx_factory()
    ctx.extractdat(cfg.nd, cfg.rku())
    h = oracle.point_h(cfg.nd)
    free = oracle.stokes_direct(ex["z"], ex["dz"], h, dens, -1)
    assert relmax(ctx.stokes_sum(dens, -1, "fp64"), free) < 1e-12
    ctx.set_wall(1)
    assert relmax(ctx.stokes_sum(dens, -1, "fp64"), ref[-1]) < 1e-12
    ctx.set_wall(0)
    assert relmax(ctx.stokes_sum(dens, -1, "fp64"), free) < 1e-12


def test_wall_fasmvp_setvelf_interfacenew(gpu_ctx_factory, setups, oracle):
    cfg, ex, dens, _ = setups["wall16x256"]
    g = oracle.Geometry.from_extract(cfg.nd, ex, wall=True)
    ctx = wall_ctx(gpu_ctx_factory, cfg)
    u = dens.view(np.float64).copy()
    assert relmax(ctx.fasmvp(u, "fp64"), oracle.fasmvp(g, u)) < 1e-12
    zbond = cfg.params["zbond"]
    zc = 1j * zbond * ex["area"] / (8 * np.pi)
    rng = np.random.default_rng(41)
    dphi = rng.standard_normal(cfg.nbk)
    for cap in (0.0, 0.3):
        ref = oracle.setvelf(g, zc, zbond, cap, 0.5, dphi)
        assert relmax(ctx.setvelf(dphi, cap=cap, e0=0.5, zbond=zbond, zc=zc), ref) < 1e-12
        un, flux = ctx.interfacenew(dens, zc, cap=cap)
        un_ref, flux_ref = oracle.interfacenew(g, ex["ckern"], zc, cap, dens)
        assert relmax(un, un_ref) < 1e-12
        assert abs(flux - flux_ref) < 1e-12 * np.abs(un_ref).max()


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_wall_solve(gpu_ctx_factory, setups, oracle, mode):
    cfg, ex, _, _ = setups["wall16x256"]
    g = oracle.Geometry.from_extract(cfg.nd, ex, wall=True)
    ctx = wall_ctx(gpu_ctx_factory, cfg)
    rng = np.random.default_rng(42)
    rhs = rng.standard_normal(2 * cfg.nbk)
    ref, rinfo = oracle.solvei(g, rhs, tol=1e-14)
    got, info = ctx.solvei(rhs, mode)
    assert info["ierr"] == 0
    assert relmax(got, ref) < 1e-9
    # the GPU solution's true residual against the exact wall-bounded operator
    assert relmax(oracle.fasmvp(g, got), rhs) < 1e-9


@pytest.fixture(scope="module")
def wall_rk_ref(oracle):
    cfg = configs.wall_drops()
    m = oracle.make_model(cap=0.0, e0=0.5, zbond=cfg.params["zbond"], mode=0)
    ys = [cfg.rku()]
    for _ in range(2):
        ys.append(oracle.rk2(m, cfg.nd, 1e-3, ys[-1]))
    return cfg, ys


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_wall_rk2_two_steps_vs_oracle(gpu_ctx_factory, wall_rk_ref, mode):
    cfg, ys = wall_rk_ref
    ctx = gpu_ctx_factory()
    y = cfg.rku()
    for s in range(2):
        info = ctx.rk2(cfg.nd, 1e-3, y, e0=0.5, zbond=cfg.params["zbond"], mode=mode)
        assert info["lap_ierr"] == 0 and info["stokes_ierr"] == 0
        assert np.abs(y - ys[s + 1]).max() < 1e-10, (mode, s)
    assert ctx.get_wall()[0] == 1
    # zbond = 0 returns the context to free space
    ctx.rk2(cfg.nd, 1e-3, y, e0=0.5, mode=mode)
    assert ctx.get_wall()[0] == 0


def test_wall_errors(gpu_ctx_factory):
    cfg = configs.wall_drops(k=4, n=64)
    ctx = gpu_ctx_factory()
    ctx.set_wall(1)
    z = cfg.z.copy()
    z -= 1j * (z.imag.min() + 0.1)  # the lowest node 0.1 below the wall
    with pytest.raises(EbError):
        ctx.extractdat(cfg.nd, z.view(np.float64).copy())
    with pytest.raises(EbError):
        ctx.batch_define([2, 2])
    ctx.set_wall(0)
    ctx.batch_define([2, 2])
    with pytest.raises(EbError):
        ctx.set_wall(1)
