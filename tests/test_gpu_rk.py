"""Parity of the GPU RK stage (SETVELF, F, RK2) with the CPU oracle.

The oracle evaluates the Stokes and Laplace operators by direct summation and solves
with SLATEC-semantics GMRES; the GPU solves stop at the same relative residual 1e-10
on FMM operators, so stage outputs agree to ~1e-9 relative and positions after a step
to ~dt * 1e-9. Tolerances: SETVELF 1e-12 relative (no solve inside); F 1e-8 relative
to the largest node velocity; positions after RK2 steps 1e-10 absolute (drops of
radius ~1).
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def ctx(gpu_ctx_factory):
    return gpu_ctx_factory()


CASES = {
    "single256": lambda: configs.single_drop(256),
    "small3x128": lambda: configs.small_drops(3, 128),
}


@pytest.mark.parametrize("case", list(CASES))
def test_setvelf_matches_oracle(ctx, oracle, case):
    cfg = CASES[case]()
    ctx.extractdat(cfg.nd, cfg.rku())
    oex = oracle.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, oex)
    rng = np.random.default_rng(30)
    dphi = rng.standard_normal(cfg.nbk)
    got = ctx.setvelf(dphi, cap=0.3, e0=0.64)
    ref = oracle.setvelf(g, np.zeros(cfg.k, complex), 0j, 0.3, 0.64, dphi)
    assert relmax(got, ref) < 1e-12


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_f_matches_oracle(ctx, oracle, case, mode):
    cfg = CASES[case]()
    m = oracle.make_model(cap=0.1, e0=0.5)
    ref = oracle.f_eval(m, cfg.nd, cfg.rku())
    got, info = ctx.f(cfg.nd, cfg.rku(), cap=0.1, e0=0.5, mode=mode)
    assert info["lap_ierr"] == 0 and info["stokes_ierr"] == 0
    assert info["lap_err"] <= 1e-10 and info["stokes_err"] <= 1e-10
    assert relmax(got, ref) < 1e-8
    assert abs(info["flux"] - m.flux) < 1e-8


def test_rk2_single_drop_100_steps(ctx, oracle):
    """The single-drop workload (N = 256, E0 = 0.5, cap = 0, dt = 1e-3) for its full
    100 RK2 steps: node positions against the oracle's."""
    cfg = configs.single_drop(256)
    m = oracle.make_model(cap=0.0, e0=0.5)
    y_ref = cfg.rku()
    y = cfg.rku()
    for _ in range(100):
        y_ref = oracle.rk2(m, cfg.nd, 1e-3, y_ref)
        ctx.rk2(cfg.nd, 1e-3, y, cap=0.0, e0=0.5, mode="fp64")
    assert np.abs(y - y_ref).max() < 1e-10
    a0 = oracle.extractdat(cfg.nd, cfg.rku())["area"].sum()
    a1 = oracle.extractdat(cfg.nd, y)["area"].sum()
    assert abs(a1 - a0) / a0 < 1e-8


def test_rk2_small_drops_refined(ctx, oracle):
    cfg = configs.small_drops(3, 128)
    m = oracle.make_model(cap=0.1, e0=0.64)
    y_ref = cfg.rku()
    y = cfg.rku()
    for _ in range(5):
        y_ref = oracle.rk2(m, cfg.nd, 1e-3, y_ref)
        ctx.rk2(cfg.nd, 1e-3, y, cap=0.1, e0=0.64, mode="fp32_refined")
    assert np.abs(y - y_ref).max() < 1e-10


def test_rk2_device_state_matches_host(ctx):
    """With the state in device memory (mem = EB_DEVICE) the step is the same
    computation as through host buffers."""
    import torch
    cfg = configs.small_drops(3, 128)
    yh = cfg.rku()
    yd = torch.from_numpy(cfg.rku()).cuda()
    for _ in range(2):
        ctx.rk2(cfg.nd, 1e-3, yh, cap=0.0, e0=0.5)
        ctx.rk2(cfg.nd, 1e-3, yd, cap=0.0, e0=0.5)
    torch.cuda.synchronize()
    np.testing.assert_allclose(yd.cpu().numpy(), yh, rtol=0, atol=1e-14)


def test_rk2_many_drops_modes_agree(ctx, oracle):
    """64 x 512 workload: one RK2 step with the FP32-refined solver equals the plain FP64
    one, conserves each drop's area, and keeps the interface flux at zero."""
    cfg = configs.many_drops()
    y64 = cfg.rku()
    y32 = cfg.rku()
    i64 = ctx.rk2(cfg.nd, 1e-3, y64, e0=0.5, mode="fp64")
    i32 = ctx.rk2(cfg.nd, 1e-3, y32, e0=0.5, mode="fp32_refined")
    assert np.abs(y64 - y32).max() < 1e-10
    assert abs(i64["flux"]) < 1e-8 and abs(i32["flux"]) < 1e-8
    a0 = oracle.extractdat(cfg.nd, cfg.rku())["area"]
    a1 = oracle.extractdat(cfg.nd, y64)["area"]
    assert np.abs(a1 - a0).max() / a0.max() < 1e-8


def test_rk_errors(ctx):
    from electricbubbles_gb300 import EbError
    cfg = configs.single_drop(64)
    with pytest.raises(EbError) as e:
        ctx.f(cfg.nd, cfg.rku(), zbond=0.1)
    assert e.value.status == 1  # EB_ERR_ARG: wall-bounded flow
    z = configs.single_drop(96)
    with pytest.raises(EbError) as e:
        ctx.f(z.nd, z.rku())
    assert e.value.status == 1  # EB_ERR_ARG: not a power of two
