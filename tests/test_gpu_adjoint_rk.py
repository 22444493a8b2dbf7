"""Reverse mode through the RK stage and the RK2 step (eb_rk_f_vjp, eb_rk2_step_vjp,
eb_deformation) on the GPU.

References: PyTorch autograd through a float64 restatement of F with direct sums and dense
solves (tests/torch_stage.py, itself checked against the oracle's F in
test_adjoint_rk_reference.py), and central differences (step 1e-6) of the GPU's own
forward RK2 steps on the 16 x 512 gradient workload. The solves run to a relative residual
of 1e-14, so the GPU's forward and adjoint solves differ from exact ones by about that.
Bars: 1e-9 of the largest gradient entry against autograd (1e-8 through three steps);
against central differences, as the 16 x 512 test states.
"""
import numpy as np
import pytest

from electricbubbles_gb300 import configs
from electricbubbles_gb300.api import EbError

torch = pytest.importorskip("torch")
import torch_stage as T  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = {
    "2x32": lambda: configs.small_drops(2, 32),
    "3x64": lambda: configs.small_drops(3, 64),
}


def relmax(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def untied(cfg, seed, amp=1e-3):
    """cfg's RK state with a smooth random perturbation of amplitude amp per drop (random
    complex coefficients of e^(+-i m theta), m = 2, 3, 4): the symmetric drop shapes tie
    their largest and smallest radii, where the deformation has no derivative."""
    y = cfg.rku()
    z = y[0::2] + 1j * y[1::2]
    rng = np.random.default_rng(seed)
    o = 0
    for n in cfg.nd:
        th = 2 * np.pi * np.arange(n) / n
        for m in (2, 3, 4):
            a, b = rng.standard_normal(2) + 1j * rng.standard_normal(2)
            z[o:o + n] += amp * (a * np.exp(1j * m * th) + b * np.exp(-1j * m * th))
        o += n
    return np.ascontiguousarray(np.stack([z.real, z.imag], 1).reshape(-1))


@pytest.mark.parametrize("pairs", ["df", "fp64"])
@pytest.mark.parametrize("sums", ["direct", "fmm"])
@pytest.mark.parametrize("case", list(CASES))
def test_f_vjp_matches_autograd(gpu_ctx_factory, case, sums, pairs):
    """pairs: the derivative sums in double-float (the default) or native FP64."""
    cfg = CASES[case]()
    ctx = gpu_ctx_factory(gmres_tol=1e-14, direct_max=0 if sums == "direct" else -1,
                          adj_df=1 if pairs == "df" else -1)
    y = cfg.rku()
    rng = np.random.default_rng(90)
    v = rng.standard_normal(2 * cfg.nbk)
    e0, cap = 0.7, 0.3
    f_ref, gy, ge, gc = T.f_vjp(cfg.nd, y, v, e0, cap)
    yb, pb, info = ctx.f_vjp(cfg.nd, y, v, cap=cap, e0=e0)
    assert info["ierr"] == 0 and info["stokes_adj_iters"] > 0 and info["lap_adj_iters"] > 0
    assert relmax(yb, gy) < 1e-9
    assert abs(pb["e0"] - ge) < 1e-9 * abs(ge)
    assert abs(pb["cap"] - gc) < 1e-9 * abs(gc)
    # the forward the call reran is F itself
    f, _ = ctx.f(cfg.nd, y, cap=cap, e0=e0)
    assert relmax(f, f_ref) < 1e-11


def low_modes(g, nd, kmax):
    """Each drop's Fourier modes |k| <= kmax of a node gradient (complex per node)."""
    z = g[0::2] + 1j * g[1::2]
    out, o = [], 0
    for n in nd:
        c = np.fft.fft(z[o:o + n])
        c[np.abs(np.fft.fftfreq(n, 1.0 / n)) > kmax] = 0
        out.append(c)
        o += n
    return np.concatenate(out)


def test_f_vjp_16x512_matches_autograd_on_the_gpu(gpu_ctx_factory):
    """The gradient workload's size (16 x 512, 8,192 nodes): the FP64 direct-sum reference
    gradient, PyTorch autograd through the dense restatement of F run on the GPU (dense
    16,384-unknown Stokes and 8,192-unknown Laplace solves, some 25 GB of autograd state),
    against eb_rk_f_vjp (FMM forward, transposed GMRES to 1e-14, direct pair derivatives).
    The two FP64 computations of F differ by rounding (2e-10 here: EXTRACTDAT's z'' = D^2 z
    amplifies the last bits of z by up to (n/2)^2), and the node gradient carries the
    transposed second derivative, which amplifies that difference at wavenumber k by k^2:
    the gradients agree to 1e-8 in each drop's modes |k| <= 32 (measured 3e-9) and to 2e-6 (max norm,
    measured 3.8e-7, from 1.6e-9 at 128 nodes per drop and 3.3e-8 at 256) in all of them."""
    if not torch.cuda.is_available():
        pytest.skip("autograd reference on the GPU needs torch CUDA")
    cfg = configs.gradient_drops()
    y = untied(cfg, 97)
    rng = np.random.default_rng(98)
    v = rng.standard_normal(2 * cfg.nbk)
    e0, cap = 0.5, 0.1
    f_ref, gy, ge, gc = T.f_vjp(cfg.nd, y, v, e0, cap, device="cuda")
    torch.cuda.empty_cache()
    ctx = gpu_ctx_factory(gmres_tol=1e-14)
    yb, pb, info = ctx.f_vjp(cfg.nd, y, v, cap=cap, e0=e0)
    assert info["ierr"] == 0
    lo, lo_ref = low_modes(yb, cfg.nd, 32), low_modes(gy, cfg.nd, 32)
    assert np.linalg.norm(lo - lo_ref) < 1e-8 * np.linalg.norm(lo_ref)
    assert relmax(yb, gy) < 2e-6
    assert abs(pb["e0"] - ge) < 1e-9 * abs(ge)
    assert abs(pb["cap"] - gc) < 1e-9 * abs(gc)
    f, _ = ctx.f(cfg.nd, y, cap=cap, e0=e0)
    assert relmax(f, f_ref) < 1e-9


def test_rk2_vjp_matches_autograd(gpu_ctx_factory):
    cfg = CASES["2x32"]()
    ctx = gpu_ctx_factory(gmres_tol=1e-14)
    y = cfg.rku()
    dt, e0, cap = 1e-2, 0.6, 0.2
    r = np.random.default_rng(91).standard_normal(2 * cfg.nbk)
    yt = torch.tensor(y, requires_grad=True)
    et = torch.tensor(e0, dtype=torch.float64, requires_grad=True)
    ct = torch.tensor(cap, dtype=torch.float64, requires_grad=True)
    k1 = T.f_stage(cfg.nd, yt, et, ct)
    k2 = T.f_stage(cfg.nd, yt + dt * k1, et, ct)
    yn = yt + 0.5 * dt * k1 + 0.5 * dt * k2
    gy, ge, gc = torch.autograd.grad(yn, (yt, et, ct), torch.tensor(r))
    rb = r.copy()
    pb, info = ctx.rk2_vjp(cfg.nd, dt, y, rb, cap=cap, e0=e0)
    assert info["ierr"] == 0
    assert relmax(rb, gy.numpy()) < 1e-10
    assert abs(pb["e0"] - float(ge)) < 1e-9 * abs(float(ge))
    assert abs(pb["cap"] - float(gc)) < 1e-9 * abs(float(gc))


def test_deformation_matches_autograd(gpu_ctx_factory):
    cfg = configs.gradient_drops(4, 64)
    ctx = gpu_ctx_factory()
    y = untied(cfg, 93)
    J, g = ctx.deformation(cfg.nd, y)
    yt = torch.tensor(y, requires_grad=True)
    Jt = T.deformation(cfg.nd, yt)
    (gt,) = torch.autograd.grad(Jt, (yt,))
    assert abs(J - float(Jt.detach())) < 1e-14 * cfg.k
    assert relmax(g, gt.numpy()) < 1e-12


def test_rk2_gradient_matches_autograd(gpu_ctx_factory):
    """dJ/dy0, dJ/dE0 and dJ/dcap of the deformation after three steps."""
    cfg = CASES["2x32"]()
    ctx = gpu_ctx_factory(gmres_tol=1e-14)
    y0 = untied(cfg, 94)
    dt, e0, cap, steps = 1e-2, 0.6, 0.2, 3
    J_ref, gy, ge, gc = T.rk2_gradient(cfg.nd, dt, y0, steps, e0, cap)
    g = ctx.rk2_gradient(cfg.nd, dt, y0, steps, cap=cap, e0=e0)
    assert g["info"]["ierr"] == 0
    assert abs(g["J"] - J_ref) < 1e-10 * abs(J_ref)
    assert relmax(g["y0"], gy) < 1e-8
    assert abs(g["e0"] - ge) < 1e-8 * abs(ge)
    assert abs(g["cap"] - gc) < 1e-8 * abs(gc)


def test_rk2_gradient_equals_its_steps(gpu_ctx_factory):
    """eb_rk2_gradient (stages replayed with the solutions kept from the forward pass, on
    device arrays) against the composition of eb_rk2_step, eb_deformation and
    eb_rk2_step_vjp (stages re-solved, host arrays), three steps."""
    cfg = CASES["3x64"]()
    ctx = gpu_ctx_factory(gmres_tol=1e-14)
    y0 = untied(cfg, 99)
    dt, e0, cap, steps = 1e-2, 0.6, 0.2, 3
    ys = [y0.copy()]
    for _ in range(steps):
        y = ys[-1].copy()
        ctx.rk2(cfg.nd, dt, y, cap=cap, e0=e0)
        ys.append(y)
    J, rbar = ctx.deformation(cfg.nd, ys[-1])
    pe = pc = 0.0
    for yc in reversed(ys[:-1]):
        p, _ = ctx.rk2_vjp(cfg.nd, dt, yc, rbar, cap=cap, e0=e0)
        pe += p["e0"]
        pc += p["cap"]
    g = ctx.rk2_gradient(cfg.nd, dt, torch.from_numpy(y0).cuda(), steps, cap=cap, e0=e0)
    assert abs(g["J"] - J) < 1e-13 * abs(J)
    assert relmax(g["y0"].cpu().numpy(), rbar) < 1e-9
    assert abs(g["e0"] - pe) < 1e-10 * abs(pe) and abs(g["cap"] - pc) < 1e-10 * abs(pc)


def smooth_direction(cfg, rng):
    """A unit node displacement made of each drop's Fourier modes 1 to 5."""
    z = np.zeros(cfg.nbk, complex)
    o = 0
    for n in cfg.nd:
        th = 2 * np.pi * np.arange(n) / n
        for m in range(1, 6):
            a, b = rng.standard_normal(2) + 1j * rng.standard_normal(2)
            z[o:o + n] += a * np.exp(1j * m * th) + b * np.exp(-1j * m * th)
        o += n
    d = np.stack([z.real, z.imag], 1).reshape(-1)
    return d / np.linalg.norm(d)


def test_gradient_vs_central_differences_16x512(gpu_ctx_factory):
    """The 16 x 512 gradient workload, two RK2 steps at dt = 1e-3: directional derivatives
    of J and dJ/dE0 against central differences of the GPU's forward steps. The differences
    carry the forward's rounding (J to about 1e-13 relative, GMRES at 1e-14) divided by
    the step, allowed as 2e-13 |J| / h on top of the relative bars: 1e-5 at the step 1e-6
    for smooth displacements and E0. A displacement
    of random nodes (every Fourier mode) also moves the curvature nonlinearly, by k^2 per
    mode k: its bar is 1e-4 at the step 1e-6. At the step 1e-4 the smooth directions and
    E0 agree to 1e-6 (measured 1e-8)."""
    cfg = configs.gradient_drops()
    ctx = gpu_ctx_factory(gmres_tol=1e-14)
    y0 = untied(cfg, 95)
    dt, e0, steps = 1e-3, 0.5, 2
    g = ctx.rk2_gradient(cfg.nd, dt, y0, steps, e0=e0)
    assert g["info"]["ierr"] == 0

    def J(y, e):
        y = y.copy()
        for _ in range(steps):
            ctx.rk2(cfg.nd, dt, y, e0=e)
        return ctx.deformation(cfg.nd, y, grad=False)[0]

    def fd(d, h):
        return (J(y0 + h * d, e0) - J(y0 - h * d, e0)) / (2 * h)

    def close(a, b, bar, h):
        return abs(a - b) < bar * abs(a) + 2e-13 * abs(g["J"]) / h

    rng = np.random.default_rng(92)
    for _ in range(2):
        d = smooth_direction(cfg, rng)
        ad = float(g["y0"] @ d)
        assert close(ad, fd(d, 1e-6), 1e-5, 1e-6)
        assert close(ad, fd(d, 1e-4), 1e-6, 1e-4)
    d = rng.standard_normal(2 * cfg.nbk)
    d /= np.linalg.norm(d)
    ad = float(g["y0"] @ d)
    assert close(ad, fd(d, 1e-6), 1e-4, 1e-6)
    for h, bar in ((1e-6, 1e-5), (1e-4, 1e-6)):
        fe = (J(y0, e0 + h) - J(y0, e0 - h)) / (2 * h)
        assert close(g["e0"], fe, bar, h)


def test_adjoint_rejects_wall_and_batch(gpu_ctx_factory):
    cfg = CASES["2x32"]()
    ctx = gpu_ctx_factory()
    y = cfg.rku()
    v = np.ones(2 * cfg.nbk)
    m = ctx._model(0.0, 0.5, -0.2, "fp64")
    out = np.empty_like(y)
    import ctypes
    from electricbubbles_gb300.api import _ptr
    nd = np.asarray(cfg.nd, dtype=np.int32)
    st = ctx._lib.eb_rk_f_vjp(ctx._h, 2, _ptr(nd), _ptr(y), _ptr(v), ctypes.byref(m), _ptr(out), None, None, 0)
    assert st == 1  # EB_ERR_ARG: zbond != 0
    b = gpu_ctx_factory()
    b.batch_define([1, 1])
    with pytest.raises(EbError) as e:
        b.f_vjp(cfg.nd, y, v, e0=0.5)
    assert e.value.status == 1
