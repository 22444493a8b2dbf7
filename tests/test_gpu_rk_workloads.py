"""RK2 parity over several steps on the workloads themselves.

* 64 drops x 512 nodes (N = 32,768): two RK2 steps (electric.f:762-786) in both solver
  modes against the oracle's, which evaluates the Stokes sums with the restated CADAPDR
  FMM (cadapdrop.f, TOL 1e-13) and the Cauchy sums directly; then the full 20 steps of
  the workload with native FP64 against the double-float FP64-class operators.
* Uneven independent simulations (one drop each, N from 128 to 4,096, each with its own
  E0): two RK2 steps per simulation against the oracle.
* The reference's own first `bubbin` deck (4 drops x 128 nodes, E0 = .64, dt = .01):
  two RK2 steps from its GEOINIT curves against the oracle.

Positions are compared as max |y_gpu - y_oracle| over all node coordinates (drops of
radius ~1). Each solve stops at the relative residual 1e-10, so positions after a step
of size dt agree to ~dt * 1e-9; the bar is 1e-10 (1e-9 for the 20-step comparison of
the two FP64 arithmetics, which accumulates 40 solves of each).
"""
import os

import numpy as np
import pytest

from electricbubbles_gb300 import configs, files

pytestmark = pytest.mark.gpu
DECK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bubbin_reference_deck1")


@pytest.fixture(scope="module")
def many_ref(oracle):
    cfg = configs.many_drops()
    m = oracle.make_model(cap=0.0, e0=0.5, mode=1)  # 1: the restated CADAPDR Stokes FMM
    ys = [cfg.rku()]
    for _ in range(2):
        ys.append(oracle.rk2(m, cfg.nd, 1e-3, ys[-1]))
    return cfg, ys


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_many_drops_two_steps_vs_oracle(gpu_ctx_factory, many_ref, mode):
    cfg, ys = many_ref
    ctx = gpu_ctx_factory()
    y = cfg.rku()
    for s in range(2):
        info = ctx.rk2(cfg.nd, 1e-3, y, e0=0.5, mode=mode)
        assert info["lap_ierr"] == 0 and info["stokes_ierr"] == 0
        assert np.abs(y - ys[s + 1]).max() < 1e-10, (mode, s)


def test_many_drops_twenty_steps_native_vs_double_float(gpu_ctx_factory, oracle):
    cfg = configs.many_drops()
    native = gpu_ctx_factory(df64=-1)
    dfl = gpu_ctx_factory(df64=1)
    yn, yd = cfg.rku(), cfg.rku()
    for _ in range(cfg.params["steps"]):
        native.rk2(cfg.nd, 1e-3, yn, e0=0.5, mode="fp64")
        dfl.rk2(cfg.nd, 1e-3, yd, e0=0.5, mode="fp64")
    assert np.abs(yn - yd).max() < 1e-9
    a0 = oracle.extractdat(cfg.nd, cfg.rku())["area"]
    a1 = oracle.extractdat(cfg.nd, yn)["area"]
    assert np.abs(a1 - a0).max() / a0.max() < 1e-7


def uneven_sample():
    """Four of the seeded uneven simulations, one of each size class 128, 512, 2048, 4096."""
    sims = configs.uneven_simulations()
    pick, seen = [], set()
    for s in sims:
        if s.nbk in (128, 512, 2048, 4096) and s.nbk not in seen:
            pick.append(s)
            seen.add(s.nbk)
    assert len(pick) == 4
    return pick


@pytest.mark.parametrize("mode", ["fp64", "fp32_refined"])
def test_uneven_simulations_two_steps_vs_oracle(gpu_ctx_factory, oracle, mode):
    ctx = gpu_ctx_factory()
    for sim in uneven_sample():
        e0 = sim.params["E0"]
        m = oracle.make_model(cap=0.0, e0=e0)
        y_ref, y = sim.rku(), sim.rku()
        for _ in range(2):
            y_ref = oracle.rk2(m, sim.nd, 1e-3, y_ref)
            ctx.rk2(sim.nd, 1e-3, y, e0=e0, mode=mode)
        assert np.abs(y - y_ref).max() < 1e-10, (sim.name, sim.nbk)


def test_reference_bubbin_deck_two_steps(gpu_ctx_factory, oracle):
    d = files.read_bubbin(DECK)
    assert list(d["nd"]) == [128] * 4 and d["E0"] == 0.64 and d["dt"] == 0.01
    z, _, _, _ = files.geoinit(d)
    y = np.ascontiguousarray(z).view(np.float64).copy()
    y_ref = y.copy()
    m = oracle.make_model(cap=d["cap"], e0=d["E0"])
    ctx = gpu_ctx_factory()
    for _ in range(2):
        y_ref = oracle.rk2(m, d["nd"], d["dt"], y_ref)
        ctx.rk2(d["nd"], d["dt"], y, cap=d["cap"], e0=d["E0"])
    assert np.abs(y - y_ref).max() < 1e-10
