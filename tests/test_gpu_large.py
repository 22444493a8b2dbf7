"""The 1,024-drop x 1,024-node workload (N = 1,048,576 nodes): the GPU Stokes sum on
4,096 sampled targets (seed 3) against the oracle's FP64 direct sum over every source,
and one full GMRES solve to 1e-10 in both solver modes (the refined one in two
refinement steps: the second step's inner tolerance is tightened so that it ends the
solve); repeated applies give identical bits (every sum is added in a fixed order).

Tolerances: FP64 FMM 1e-12 relative to the largest sampled value, FP32 FMM 1e-5; the
two solvers' solutions agree within 1e-9 relative (max-norm)."""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def large(gpu_ctx_factory):
    cfg = configs.large_drops()
    ctx = gpu_ctx_factory()
    ex = ctx.extractdat(cfg.nd, cfg.rku())
    return cfg, ctx, ex


@pytest.mark.parametrize("sign", [-1, 1])
def test_large_sampled_targets_vs_direct(large, oracle, sign):
    cfg, ctx, ex = large
    rng = np.random.default_rng(2)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    tidx = np.sort(np.random.default_rng(3).choice(cfg.nbk, 4096, replace=False)).astype(np.int32)
    ref = oracle.stokes_direct_at(ex["z"], ex["dz"], oracle.point_h(cfg.nd), dens, sign, tidx)
    got = ctx.stokes_sum(dens, sign, "fp64")
    assert relmax(got[tidx], ref) < 1e-12
    got32 = ctx.stokes_sum(dens, sign, "fp32")
    assert relmax(got32[tidx], ref) < 1e-5


def test_large_full_solve(large):
    cfg, ctx, ex = large
    rhs = np.ascontiguousarray(-0.5 * ex["dz"] / ex["dsda"]).view(np.float64).copy()
    x64, i64 = ctx.solvei(rhs, "fp64")
    x32, i32 = ctx.solvei(rhs, "fp32_refined")
    assert i64["ierr"] == 0 and i64["err"] <= 1e-10
    assert i32["ierr"] == 0 and i32["err"] <= 1e-10
    assert i32["outer"] == 2
    assert relmax(x32, x64) < 1e-9
    # the certified residual: recompute ||b - A x|| / ||b|| with the FP64 operator
    r = rhs - ctx.fasmvp(x32, "fp64")
    assert np.linalg.norm(r) / np.linalg.norm(rhs) <= 1.01e-10


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_large_apply_deterministic(large, prec):
    cfg, ctx, ex = large
    rng = np.random.default_rng(5)
    u = rng.standard_normal(2 * cfg.nbk)
    a = ctx.fasmvp(u, prec)
    b = ctx.fasmvp(u, prec)
    assert np.array_equal(a, b)
