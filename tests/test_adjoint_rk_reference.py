"""The autograd reference of the GPU's adjoint (tests/torch_stage.py) against the oracle,
on the CPU: its F equals the oracle's F (eb_or_f, direct sums, GMRES to 1e-15) to 1e-12,
its interpolations equal the oracle's FINTERC / FINTER, and its Taylor deformation is
the one numpy computes."""
import numpy as np
import pytest

from electricbubbles_gb300 import configs

torch = pytest.importorskip("torch")
import torch_stage as T  # noqa: E402


@pytest.mark.parametrize("cfg", [configs.small_drops(2, 32), configs.small_drops(3, 64)],
                         ids=["2x32", "3x64"])
def test_torch_f_matches_oracle(oracle, cfg):
    y = cfg.rku()
    m = oracle.make_model(cap=0.3, e0=0.7, gmres_tol=1e-15)
    fo = oracle.f_eval(m, cfg.nd, y)
    ft = T.f_stage(cfg.nd, torch.tensor(y), 0.7, 0.3).numpy()
    assert np.abs(fo - ft).max() < 1e-12 * np.abs(fo).max()


def test_torch_interpolation_matches_oracle(oracle):
    z = configs.single_drop(64).z
    assert np.abs(T.finterc(torch.tensor(z)).numpy() - oracle.finterc(z)).max() < 1e-14
    assert np.abs(T.finter(torch.tensor(z.real)).numpy() - oracle.finter(z.real)).max() < 1e-14


def test_torch_deformation():
    cfg = configs.gradient_drops(4, 64)
    y = cfg.rku()
    z = y[0::2] + 1j * y[1::2]
    ref = 0.0
    for b in range(cfg.k):
        r = np.abs(z[64 * b:64 * (b + 1)] - z[64 * b:64 * (b + 1)].mean())
        ref += (r.max() - r.min()) / (r.max() + r.min())
    assert abs(float(T.deformation(cfg.nd, torch.tensor(y))) - ref) < 1e-14
