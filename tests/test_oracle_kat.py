"""The CPU oracle against the analytic known answers the reference itself carries.

- PVINTEV's commented driver (pv_integral.f:1-49): unit circle, 32 nodes, densities
  1/(z - z0) with z0 = (3, 2) and z z', whose principal-value Cauchy integrals are f(z)/2.
- CHECK (laplace.f:30-73): after the Laplace solve on a circle, the exterior double-layer
  potential at z* = (3, 0.5) equals Re(z*)/|z*|^2.
- the restated CADAPDR/CADAPMOD FMM reproduces its exact direct sum.
"""
import numpy as np
import pytest


def circle(n):
    th = 2 * np.pi * np.arange(n) / n
    return np.exp(1j * th)


def test_fft_matches_definition(oracle):
    rng = np.random.default_rng(0)
    for n in (8, 64, 12):
        c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        np.testing.assert_allclose(oracle.fft(c, -1), np.fft.fft(c), rtol=0, atol=1e-12)
        np.testing.assert_allclose(oracle.fft(c, +1), np.fft.ifft(c) * n, rtol=0, atol=1e-12)


def test_fdifff_exact_on_trig_polynomial(oracle):
    n = 64
    a = 2 * np.pi * np.arange(n) / n
    f = np.exp(3j * a) + 0.5 * np.cos(5 * a)
    df = 3j * np.exp(3j * a) - 2.5 * np.sin(5 * a)
    np.testing.assert_allclose(oracle.fdifff(f), df, atol=1e-12)


def test_fdifff_zeroes_nyquist(oracle):
    n = 16
    a = 2 * np.pi * np.arange(n) / n
    f = np.cos(8 * a)  # pure Nyquist mode
    np.testing.assert_allclose(oracle.fdifff(f), 0, atol=1e-13)


def test_finterc_interpolates(oracle):
    n = 32
    a = 2 * np.pi * np.arange(n) / n
    f = np.exp(2j * a) + 0.3 * np.exp(-5j * a)
    a2 = np.pi * np.arange(2 * n) / n
    np.testing.assert_allclose(oracle.finterc(f), np.exp(2j * a2) + 0.3 * np.exp(-5j * a2), atol=1e-13)


@pytest.mark.parametrize("case", ["inverse", "zzprime"])
def test_pvintev_circle_known_answer(oracle, case):
    n = 32
    z = circle(n)
    zp = 1j * z  # z'(theta) of the counter-clockwise unit circle (xp = -y, yp = x)
    if case == "inverse":
        f = 1.0 / (z - (3 + 2j))
    else:
        f = z
    phi = oracle.pvintev([n], z, f * zp)
    np.testing.assert_allclose(phi, f / 2, atol=1e-12)


def _check_answer(g, u, n, zstar):
    h = 2 * np.pi / n
    delz = g.z - zstar
    zn = -1j * g.dz / g.dsda
    akern = (delz * np.conj(zn)).real / np.abs(delz) ** 2
    return -np.sum(0.5 * h * akern * u * g.dsda / np.pi)


def test_laplace_check_exterior_potential(oracle):
    """CHECK (laplace.f:30-73): exterior potential at z* = (3, 0.5) after the Laplace
    solve on the unit circle equals Re(z*)/|z*|^2.

    The double-layer part of FASMVP_LAP satisfies it to rounding. The full operator
    also subtracts 2 h s'_i u_i on the diagonal (laplace.f:235-236, where the older
    DIRECT_MATVEC subtracted the rank-one 2 sum_j h s'_j u_j / (2 pi)); that term is
    O(h), so with it the answer converges to the closed form at first order in 1/n."""
    from electricbubbles_gb300 import configs
    zstar = 3 + 0.5j
    exact = zstar.real / abs(zstar) ** 2
    errs = []
    for n in (128, 256):
        z = configs.perturbed_circle(n, 1.0, 0.0)
        ex = oracle.extractdat([n], z.view(np.float64))
        g = oracle.Geometry.from_extract([n], ex)
        h = 2 * np.pi / n
        rhs = -2.0 * g.z.real
        u2, _ = oracle.gmres(lambda v: oracle.fasmvp_lap(g, v) + 2 * h * v * g.dsda, rhs, rhs)
        assert abs(_check_answer(g, u2, n, zstar) - exact) < 1e-13
        u, info = oracle.solve_lapl(g, rhs)
        assert info["ierr"] == 0 and info["err"] <= 1e-10
        errs.append(_check_answer(g, u, n, zstar) - exact)
    assert 1.8 < errs[0] / errs[1] < 2.2


@pytest.mark.parametrize("sign", [-1, 1])
def test_cadap_restatement_matches_direct(oracle, sign):
    from electricbubbles_gb300 import configs
    cfg = configs.small_drops(3, 128)
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(3)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    h = oracle.point_h(cfg.nd)
    d = oracle.stokes_direct(ex["z"], ex["dz"], h, dens, sign)
    f = oracle.cadap_fmm(ex["z"], ex["dz"], h, dens, sign, levmax=5, tol=1e-13)
    assert np.abs(f - d).max() / np.abs(d).max() < 1e-12


def test_cauchy_direct_antisymmetry(oracle):
    """sum_i q_i F_i = 0 for the Hilbert matrix 1/(z_i - z_j) (antisymmetric)."""
    rng = np.random.default_rng(4)
    z = rng.standard_normal(200) + 1j * rng.standard_normal(200)
    q = rng.standard_normal(200) + 1j * rng.standard_normal(200)
    f = oracle.cauchy_direct(z, z, q, True)
    assert abs(np.sum(q * f)) < 1e-10 * np.sum(np.abs(q * f))


def test_gmres_dense_system(oracle):
    rng = np.random.default_rng(5)
    n = 60
    a = np.eye(n) + 0.3 * rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n)
    x, info = oracle.gmres(lambda v: a @ v, b, b, maxl=100, tol=1e-12)
    assert info["ierr"] == 0
    np.testing.assert_allclose(x, np.linalg.solve(a, b), rtol=0, atol=1e-9)


def test_extractdat_circle(oracle):
    n = 64
    z = 2.0 * circle(n) + (1 - 1j)
    ex = oracle.extractdat([n], z.view(np.float64))
    np.testing.assert_allclose(ex["zk"], [1 - 1j], atol=1e-14)
    np.testing.assert_allclose(ex["kappa"], -0.5, atol=1e-12)
    np.testing.assert_allclose(ex["dsda"], 2.0, atol=1e-12)
    np.testing.assert_allclose(ex["area"], [4 * np.pi], atol=1e-12)


def test_rk2_conserves_area(oracle):
    """Incompressibility: the total area stays constant (electric.f:246-250)."""
    from electricbubbles_gb300 import configs
    cfg = configs.single_drop(64)
    m = oracle.make_model(cap=0.0, e0=0.5)
    y = cfg.rku()
    a0 = oracle.extractdat(cfg.nd, y)["area"].sum()
    for _ in range(3):
        y = oracle.rk2(m, cfg.nd, 1e-3, y)
    a1 = oracle.extractdat(cfg.nd, y)["area"].sum()
    assert abs(a1 - a0) / a0 < 1e-8
    assert abs(m.flux) < 1e-8


@pytest.mark.parametrize("n", [40, 3000])
def test_dapif2_restatement_matches_direct_sum(oracle, n):
    """The restated DAPIF2 FMM (IFLAG7 = 3, dapif1.f:458-1077; NAPB 30, TOL 1e-11) against
    the exact Cauchy sum, on random points and on drop curves."""
    rng = np.random.default_rng(n)
    z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    q = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = oracle.cauchy_direct(z, z, q, True)
    got = oracle.dapif2(z, q)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-11
    from electricbubbles_gb300 import configs
    cfg = configs.small_drops(3, 256)
    g = oracle.Geometry.from_extract(cfg.nd, oracle.extractdat(cfg.nd, cfg.rku()))
    u = rng.standard_normal(cfg.nbk)
    a, b = oracle.fasmvp_lap(g, u), oracle.fasmvp_lap(g, u, mode=1)
    assert np.abs(a - b).max() / np.abs(a).max() < 1e-11


# ---- wall-bounded flow (IFLAG2 = 1) ------------------------------------------------
def _wall_case(oracle, k=6, n=128):
    from electricbubbles_gb300 import configs
    cfg = configs.wall_drops(k=k, n=n)
    ex = oracle.extractdat(cfg.nd, cfg.rku())
    rng = np.random.default_rng(2)
    dens = rng.standard_normal(cfg.nbk) + 1j * rng.standard_normal(cfg.nbk)
    return cfg, ex, oracle.point_h(cfg.nd), dens


def test_refsing_images_cancel_log_sources_on_the_wall(oracle):
    """REFSING's reflected system cancels the free field of the log sources
    (INTERFACENEW's zck, electric.f:861-866) on y = 0: the no-slip wall."""
    zk = np.array([0.3 + 1.2j, -1 + 0.7j, 2.0 + 0.4j])
    zc = np.array([0.2 - 0.5j, -0.1 + 0.3j, 0.05 + 0.02j])
    for x in (-2.0, 0.1, 1.5, 4.0):
        z = complex(x, 0.0)
        zck = sum(2 * c * np.log(abs(z - k)) + np.conj(c) * (z - k) / np.conj(z - k) for c, k in zip(zc, zk))
        phi, phip, psi = oracle.refsing(z, zk, zc)
        assert abs(zck + phi + z * np.conj(phip) + np.conj(psi)) < 1e-14


@pytest.mark.parametrize("sign", [-1, 1])
def test_wall_images_on_the_wall(oracle, sign):
    """The image sum of SLDREF / SLDREFDR on the wall itself: with the sign of CADAPMOD
    (the velocity of INTERFACENEW) the images cancel the direct sum (no slip); with the
    sign of CADAPDR they equal it. Probes at y = 1e-12 carry no density."""
    cfg, ex, h, dens = _wall_case(oracle)
    xp = np.linspace(-9.0, 9.0, 7) + 1e-12j
    z = np.concatenate([ex["z"], xp])
    dz = np.concatenate([ex["dz"], np.ones(xp.shape[0])])
    hh = np.concatenate([h, np.ones(xp.shape[0])])
    d = np.concatenate([dens, np.zeros(xp.shape[0])])
    free = oracle.stokes_direct(z, dz, hh, d, sign)[cfg.nbk:]
    img = oracle.stokes_image_direct(z, dz, hh, d, sign)[cfg.nbk:]
    scale = np.abs(free).max()
    if sign == 1:
        assert np.abs(free + img).max() < 1e-10 * scale
    else:
        assert np.abs(free - img).max() < 1e-10 * scale


@pytest.mark.parametrize("sign", [-1, 1])
def test_cadap_wall_restatement_matches_exact_images(oracle, sign):
    """The restated wall-bounded CADAPDR / CADAPMOD (MPREFLECT, MKINTR, MKNBRRFL and
    SLDREFDR / SLDREF) reproduces the exact direct plus image sum."""
    cfg, ex, h, dens = _wall_case(oracle)
    xl, sl = oracle.wallinfo(ex["z"])
    got = oracle.cadap_fmm_wall(ex["z"], ex["dz"], h, dens, sign, xl, sl)
    ref = oracle.stokes_direct(ex["z"], ex["dz"], h, dens, sign) + \
        oracle.stokes_image_direct(ex["z"], ex["dz"], h, dens, sign)
    assert np.abs(got - ref).max() < 1e-11 * np.abs(ref).max()
    assert np.abs(oracle.stokes_image_direct(ex["z"], ex["dz"], h, dens, sign)).max() > 1e-2 * np.abs(ref).max()
