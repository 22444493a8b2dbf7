"""The FP64-class operators in double-float arithmetic (df64 = 1, which the refined
solver's residuals use) against the native FP64 kernels (df64 = -1, the default plain
path) and the oracle's FP64 direct sums. The two differ by the double-float rounding
(about 2^-48 per operation against 2^-53), so the results agree within 5e-13 relative to
the largest value, and both stay within 1e-12 of the direct sum."""
import numpy as np
import pytest

from electricbubbles_gb300 import configs
from electricbubbles_gb300.api import Context

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def pair():
    d = Context(df64=1, direct_max=-1)
    n = Context(df64=-1, direct_max=-1)
    yield d, n
    d.close()
    n.close()


CASES = {
    "single256": lambda: configs.single_drop(256),
    "small3x128": lambda: configs.small_drops(3, 128),
    "many64x512": lambda: configs.many_drops(),
}


@pytest.mark.parametrize("case", list(CASES))
def test_df64_stokes_and_cauchy(pair, oracle, case):
    cfg = CASES[case]()
    d, n = pair
    ex = d.extractdat(cfg.nd, cfg.rku())
    n.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(40)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    h = oracle.point_h(cfg.nd)
    for sign in (-1, 1):
        gd = d.stokes_sum(dens, sign, "fp64")
        gn = n.stokes_sum(dens, sign, "fp64")
        assert relmax(gd, gn) < 5e-13
        if cfg.nbk <= 4096:
            ref = oracle.stokes_direct(ex["z"], ex["dz"], h, dens, sign)
            assert relmax(gd, ref) < 1e-12
    q = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    fd = d.dapif2(ex["z"], q, "fp64")
    fn = n.dapif2(ex["z"], q, "fp64")
    assert relmax(fd, fn) < 5e-13


def test_df64_solve_matches_native(pair):
    cfg = configs.many_drops(16, 256, seed=11, box=8.0)
    d, n = pair
    ex = d.extractdat(cfg.nd, cfg.rku())
    n.extractdat(cfg.nd, cfg.rku())
    rhs = np.ascontiguousarray(-0.5 * ex["dz"] / ex["dsda"]).view(np.float64).copy()
    xd, idd = d.solvei(rhs, "fp64")
    xn, inn = n.solvei(rhs, "fp64")
    assert idd["iters"] == inn["iters"] and idd["ierr"] == 0
    assert relmax(xd, xn) < 1e-11
