"""eb_stokes_sum_noalloc, the entry point for callers that cannot allocate GPU memory.

It is called through the C ABI with device buffers the test allocated beforehand, twice
in a row with different densities (the second call reuses the library's fixed scratch
array), and each result is checked against eb_stokes_sum on the same nodes, within the
FP64 tolerance of the other parity tests (1e-12 relative, max norm). This file is named to
be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_stokes_sum_twice(gpu_ctx_factory, oracle):
    import torch
    from electricbubbles_gb300 import configs

    cfg = configs.many_drops(8, 256, seed=21, box=6.0)  # 2,048 nodes
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    ctx = gpu_ctx_factory()
    ctx.set_geometry(cfg.nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"])
    lib = ctx._lib
    n = cfg.nbk
    dev = torch.device("cuda", 0)
    z = torch.from_numpy(ex["z"].view(np.float64).copy()).to(dev)
    dz = torch.from_numpy(ex["dz"].view(np.float64).copy()).to(dev)
    h = torch.from_numpy(oracle.point_h(cfg.nd)).to(dev)
    out = torch.empty(2 * n, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(22)
    for call, sign in enumerate((-1, +1)):
        dens_h = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        dens = torch.from_numpy(dens_h.view(np.float64).copy()).to(dev)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        st = lib.eb_stokes_sum_noalloc(n, _p(z), _p(dz), _p(h), _p(dens), sign, _p(out), None)
        assert st == 0, lib.eb_last_error()
        torch.cuda.synchronize()
        if call > 0:
            assert torch.cuda.mem_get_info(dev)[0] == free0
        got = out.cpu().numpy().view(np.complex128)
        ref = ctx.stokes_sum(dens_h, sign, "fp64")
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 1e-12, (call, err)


def test_noalloc_rejects_sizes_beyond_the_maximum(eblib):
    import torch
    dev = torch.device("cuda", 0)
    big = 16385
    buf = torch.zeros(2 * big, dtype=torch.float64, device=dev)
    h = torch.zeros(big, dtype=torch.float64, device=dev)
    st = eblib.eb_stokes_sum_noalloc(big, _p(buf), _p(buf), _p(h), _p(buf), -1, _p(buf), None)
    assert st == 4  # EB_ERR_WORKSPACE
    assert b"EB_NOALLOC_MAX_POINTS" in eblib.eb_last_error()
