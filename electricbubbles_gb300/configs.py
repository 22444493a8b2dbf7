"""Synthetic drop configurations (seeded) with the shapes and sizes of the workloads.

The reference reads its drops from the `bubbin` deck (READINI, electric.f:275-337) and
places nodes at equal arclength with CLUSTPARAM (electric.f:1192-1265) and GEOSHIFT
(electric.f:394-426). This module does the same for perturbed circles
    z(theta) = c + r (1 + a cos(m theta)) e^{i theta},
which have no INITPARAM branch in the reference, with seeded random drop layouts.
Host-side set-up code (run once per simulation), not part of the GPU hot path.
"""
import numpy as np


def _fourier_coeffs(f):
    return np.fft.fft(f) / f.shape[0]


def _foureval(c, theta):
    """FOUREVAL, electric.f:1336-1355: sum of the modes |k| < M/2 of coefficients c,
    evaluated at every entry of theta."""
    m = c.shape[0]
    h = m // 2
    k = np.arange(1, h)
    e = np.exp(1j * np.outer(np.atleast_1d(theta), k))
    return c[0] + e @ c[1:h] + np.conj(e) @ c[m - 1:m - h:-1]


def equiarclength_params(dsdth):
    """CLUSTPARAM: parameters beta_j with equal arclength spacing, found by Newton's
    method on s(beta) = j L / n with s from the Fourier series of ds/dtheta.
    `dsdth` holds M samples of ds/dtheta at theta = 2 pi i / M; `n` nodes follow.
    All nodes are iterated together (the reference iterates node by node from the
    previous node's root; both converge to the same roots)."""
    return _equiarc(dsdth, dsdth.shape[0])


def _equiarc(dsdth, n):
    m = dsdth.shape[0]
    csa = _fourier_coeffs(dsdth.astype(complex))
    csa[m // 2] = 0.0
    arcl = 2 * np.pi * csa[0].real
    csai = np.zeros(m, complex)
    h = m // 2
    k = np.arange(1, h)
    csai[1:h] = csa[1:h] / (1j * k)
    csai[m - 1:m - h:-1] = -csa[m - 1:m - h:-1] / (1j * k)
    csai[0] = -_foureval(csai, 0.0)[0].real
    target = np.arange(n) * arcl / n
    b = 2 * np.pi * np.arange(n) / n
    for _ in range(100):
        fk = _foureval(csai, b).real + csa[0].real * b - target
        fpk = _foureval(csa, b).real
        d = -fk / fpk
        b = b + d
        if np.max(np.abs(d)) < 1e-14:
            break
    else:
        raise RuntimeError("equi-arclength Newton iteration did not converge")
    return b, arcl


_BETA_CACHE = {}


def perturbed_circle(n, radius=1.0, amp=0.05, mode=2, center=0j):
    """Nodes of one drop at equal arclength, counter-clockwise from theta = 0.
    The parameters depend only on (n, amp, mode) and are cached."""
    key = (int(n), float(amp), int(mode))
    if key not in _BETA_CACHE:
        m = int(min(max(n, 64), 256))
        th = 2 * np.pi * np.arange(m) / m
        r = 1 + amp * np.cos(mode * th)
        rd = -amp * mode * np.sin(mode * th)
        beta, _ = _equiarc(np.sqrt(r ** 2 + rd ** 2), int(n))
        _BETA_CACHE[key] = beta
    beta = _BETA_CACHE[key]
    rb = radius * (1 + amp * np.cos(mode * beta))
    return center + rb * np.exp(1j * beta)


def _place(rng, nrad, radii_fn, box, gap, pad_factor):
    radii = radii_fn(rng, nrad)
    centres = []
    rr = []
    tries = 0
    for r in radii:
        while True:
            tries += 1
            if tries > 10_000_000:
                raise RuntimeError("could not place drops without overlap")
            c = rng.uniform(-box, box) + 1j * rng.uniform(-box, box)
            ok = all(abs(c - c2) > pad_factor * (r + r2) + gap for c2, r2 in zip(centres, rr))
            if ok:
                centres.append(c)
                rr.append(r)
                break
    return np.array(centres), np.array(rr)


class DropConfig:
    """k drops: nd[k] nodes, z (complex, concatenated), per-drop radius/centre/amplitude."""

    def __init__(self, name, nd, z, centres, radii, amps, params=None):
        self.name = name
        self.nd = np.asarray(nd, dtype=np.int32)
        self.z = np.ascontiguousarray(z, dtype=np.complex128)
        self.centres = centres
        self.radii = radii
        self.amps = amps
        self.params = params or {}

    @property
    def k(self):
        return int(self.nd.shape[0])

    @property
    def nbk(self):
        return int(self.nd.sum())

    def rku(self):
        """The RK state of the reference: interleaved x, y of all nodes (INITCOND)."""
        return self.z.view(np.float64).copy()


def _build(name, nds, centres, radii, amps, params):
    zs = [perturbed_circle(int(n), r, a, 2, c) for n, r, a, c in zip(nds, radii, amps, centres)]
    return DropConfig(name, nds, np.concatenate(zs), centres, radii, amps, params)


def single_drop(n=256, amp=0.05):
    """One drop r(theta) = 1 + 0.05 cos(2 theta), N = 256: the single-drop case."""
    return _build("single_drop_n%d" % n, [n], np.array([0j]), np.array([1.0]), np.array([amp]),
                  {"E0": 0.5, "cap": 0.0, "dt": 1e-3, "steps": 100})


def many_drops(k=64, n=512, seed=1, box=20.0, gap=0.2):
    """64 drops, radii U[0.5, 1.0], centres in [-20, 20]^2 with gaps > 0.2, 512 nodes each."""
    rng = np.random.default_rng(seed)
    c, r = _place(rng, k, lambda g, m: g.uniform(0.5, 1.0, m), box, gap, 1.05)
    return _build("many_drops_%dx%d" % (k, n), np.full(k, n), c, r, np.full(k, 0.05),
                  {"E0": 0.5, "cap": 0.0, "dt": 1e-3, "steps": 20, "seed": seed})


def large_drops(k=1024, n=1024, seed=2, box=100.0, gap=0.2):
    """1,024 drops, radii log-uniform in [0.2, 1.0], centres in [-100, 100]^2, 1,024 nodes each."""
    rng = np.random.default_rng(seed)
    c, r = _place(rng, k, lambda g, m: np.exp(g.uniform(np.log(0.2), np.log(1.0), m)), box, gap, 1.05)
    return _build("large_%dx%d" % (k, n), np.full(k, n), c, r, np.full(k, 0.05),
                  {"seed": seed})


def uneven_simulations(count=256, seed=4):
    """256 independent single-drop runs, N log-uniform in [128, 4096] rounded to powers of 2."""
    rng = np.random.default_rng(seed)
    sims = []
    for i in range(count):
        n = int(2 ** int(round(np.log2(np.exp(rng.uniform(np.log(128), np.log(4096)))))))
        e0 = rng.uniform(0.1, 1.0)
        rr = rng.uniform(0.5, 4.0)
        qq = rng.uniform(0.5, 4.0)
        amp = rng.uniform(0.01, 0.1)
        cfg = _build("sim%d" % i, [n], np.array([0j]), np.array([1.0]), np.array([amp]),
                     {"E0": e0, "R": rr, "Q": qq, "cap": 0.0})
        sims.append(cfg)
    return sims


def gradient_drops(k=16, n=512, seed=5, box=10.0, gap=0.2):
    """16 drops of 512 nodes, radii U[0.6, 1.0], centres in [-10, 10]^2."""
    rng = np.random.default_rng(seed)
    c, r = _place(rng, k, lambda g, m: g.uniform(0.6, 1.0, m), box, gap, 1.05)
    return _build("grad_%dx%d" % (k, n), np.full(k, n), c, r, np.full(k, 0.05),
                  {"seed": seed, "E0": 0.5, "dt": 1e-3, "steps": 50})


def small_drops(k=3, n=64, seed=7, box=3.0, gap=0.3):
    """A small multi-drop case for tests."""
    rng = np.random.default_rng(seed)
    c, r = _place(rng, k, lambda g, m: g.uniform(0.5, 1.0, m), box, gap, 1.05)
    return _build("small_%dx%d" % (k, n), np.full(k, n), c, r, np.full(k, 0.05), {"seed": seed})


def wall_drops(k=16, n=256, seed=8, box=8.0, gap=0.3, zbond=-0.2 + 0j):
    """16 drops of 256 nodes above the wall y = 0 (wall-bounded flow, zbond != 0): radii
    U[0.5, 1.0], centres x in [-8, 8], y in [gap + r, gap + r + box/2], at least `gap`
    from the wall and from each other."""
    rng = np.random.default_rng(seed)
    radii = rng.uniform(0.5, 1.0, k)
    centres, rr = [], []
    for r in radii:
        for _ in range(1_000_000):
            c = rng.uniform(-box, box) + 1j * (1.06 * r + gap + rng.uniform(0.0, 0.5 * box))
            if all(abs(c - c2) > 1.05 * (r + r2) + gap for c2, r2 in zip(centres, rr)):
                centres.append(c)
                rr.append(r)
                break
        else:
            raise RuntimeError("could not place drops without overlap")
    return _build("wall_%dx%d" % (k, n), np.full(k, n), np.array(centres), np.array(rr), np.full(k, 0.05),
                  {"seed": seed, "E0": 0.5, "cap": 0.0, "zbond": zbond, "dt": 1e-3})
