"""The FP32 M2L on the tensor cores (eb_opts.m2l_tc, tcgen05 kind::tf32 with the 3xTF32
split) against the oracle's direct sums and against the CUDA-core M2L.

Both M2L kernels sum the same terms (SLSHIFT's binomial contraction, cadap2.f:1149-1215);
the tensor-core one forms the contraction with products of 11-bit operands recombined
to FP32 accuracy, so the FP32 operators keep their 1e-5 bar against the FP64 direct
sum and agree with the CUDA-core version to a few 1e-7.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


CASES = {
    "drops16x256": lambda: configs.many_drops(16, 256, seed=11, box=8.0),
    "drops64x512": lambda: configs.many_drops(),
}


@pytest.fixture(scope="module")
def pair(gpu_ctx_factory):
    return gpu_ctx_factory(m2l_tc=1), gpu_ctx_factory(m2l_tc=-1)


@pytest.mark.parametrize("case", list(CASES))
def test_tensor_m2l_stokes(pair, oracle, case):
    tc, cc = pair
    cfg = CASES[case]()
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(70)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    for c in pair:
        c.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    got = tc.stokes_sum(dens, -1, "fp32")
    ref32 = cc.stokes_sum(dens, -1, "fp32")
    if cfg.nbk <= 5000:
        ref = oracle.stokes_direct(ex["z"], ex["dz"], oracle.point_h(cfg.nd), dens, -1)
    else:
        idx = np.random.default_rng(71).choice(cfg.nbk, 512, replace=False)
        ref = oracle.stokes_direct_at(ex["z"], ex["dz"], oracle.point_h(cfg.nd), dens, -1, idx)
        got, ref32 = got[idx], ref32[idx]
    assert relmax(got, ref) < 1e-5
    assert relmax(got, ref32) < 2e-6
    assert np.isfinite(got).all()


def test_tensor_m2l_cauchy_and_solve(pair, oracle):
    tc, _ = pair
    cfg = configs.many_drops(16, 256, seed=11, box=8.0)
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    g = oracle.Geometry.from_extract(cfg.nd, ex)
    rng = np.random.default_rng(72)
    q = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    assert relmax(tc.dapif2(ex["z"], q, "fp32"), oracle.cauchy_direct(ex["z"], ex["z"], q, True)) < 1e-5
    tc.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    rhs = rng.standard_normal(2 * cfg.nbk)
    ref, _ = oracle.solvei(g, rhs)
    got, info = tc.solvei(rhs, "fp32_refined")
    assert info["ierr"] == 0 and info["err"] <= 1e-10
    assert relmax(got, ref) < 1e-9
