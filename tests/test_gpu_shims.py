"""The DGMRES drop-in shims matvec_ / matvec_lapl_ driven by a compiled C caller.

tests/shim_gmres.c is built with gcc against include/eb_gb300.h and libeb_gb300.so. It
installs a geometry, registers it with eb_set_default_ctx and runs its own SLATEC-style
GMRES (x0 = b, MGS, Givens, no restart) whose every operator apply calls the shim with
by-reference N, X, Y, NELT, IA, JA, A, ISYM (dpigmr.f:316-318). Its solution must agree
with eb_stokes_solve / eb_laplace_solve on the same system (1e-9 relative, the solves'
own agreement bar) and with the oracle's GMRES on exact direct sums, in about the same
number of iterations.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from electricbubbles_gb300 import build, configs

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def harness(tmp_path_factory, eblib):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    out = str(tmp_path_factory.mktemp("shim") / "shim_gmres")
    libdir = os.path.dirname(build.LIB)
    cmd = ["gcc", "-O2", "-std=c99", "-o", out, os.path.join(HERE, "shim_gmres.c"),
           "-I", os.path.join(ROOT, "include"), "-L", libdir, "-leb_gb300",
           "-Wl,-rpath," + libdir, "-lm"]
    subprocess.run(cmd, check=True)
    return out


def run_harness(harness, tmp_path, cfg, rhs, which, tol=1e-10):
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        np.array([cfg.k], np.int32).tofile(f)
        np.asarray(cfg.nd, np.int32).tofile(f)
        cfg.rku().astype(np.float64).tofile(f)
        np.array([rhs.shape[0]], np.int32).tofile(f)
        rhs.astype(np.float64).tofile(f)
    r = subprocess.run([harness, fin, fout, str(which), repr(tol)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    with open(fout, "rb") as f:
        iters = int(np.fromfile(f, np.int32, 1)[0])
        err = float(np.fromfile(f, np.float64, 1)[0])
        x = np.fromfile(f, np.float64, rhs.shape[0])
    return x, iters, err


CASES = {"single256": lambda: configs.single_drop(256), "small3x128": lambda: configs.small_drops(3, 128)}


@pytest.mark.parametrize("case", list(CASES))
def test_stokes_shim_gmres(harness, tmp_path, gpu_ctx_factory, oracle, case):
    cfg = CASES[case]()
    rhs = np.random.default_rng(40).standard_normal(2 * cfg.nbk)
    x, iters, err = run_harness(harness, tmp_path, cfg, rhs, 0)
    assert err <= 1e-10
    ctx = gpu_ctx_factory()
    ctx.extractdat(cfg.nd, cfg.rku())
    xs, info = ctx.solvei(rhs, "fp64")
    assert abs(iters - info["iters"]) <= 1
    assert relmax(x, xs) < 1e-9
    g = oracle.Geometry.from_extract(cfg.nd, oracle.extractdat(cfg.nd, cfg.rku()))
    xr, rinfo = oracle.solvei(g, rhs)
    assert abs(iters - rinfo["iters"]) <= 1
    assert relmax(x, xr) < 1e-9


@pytest.mark.parametrize("case", list(CASES))
def test_laplace_shim_gmres(harness, tmp_path, gpu_ctx_factory, oracle, case):
    cfg = CASES[case]()
    z = cfg.z
    rhs = -2.0 * z.real  # GETBCs, laplace.f:14-18
    x, iters, err = run_harness(harness, tmp_path, cfg, rhs, 1)
    assert err <= 1e-10
    ctx = gpu_ctx_factory()
    ctx.extractdat(cfg.nd, cfg.rku())
    xs, info = ctx.solve_lapl(rhs, "fp64")
    assert abs(iters - info["iters"]) <= 1
    assert relmax(x, xs) < 1e-9
    g = oracle.Geometry.from_extract(cfg.nd, oracle.extractdat(cfg.nd, cfg.rku()))
    xr, rinfo = oracle.solve_lapl(g, rhs)
    assert abs(iters - rinfo["iters"]) <= 1
    assert relmax(x, xr) < 1e-9
