"""Test helper: the RK stage F (electric.f:968-1109, free space) restated in PyTorch
float64 on the CPU, with direct sums and dense solves, so that autograd gives the exact
gradient of the discrete F. It is the reference the GPU's hand-written adjoint of F is
checked against; it is never part of the library.

Every step follows the oracle's C restatement (oracle/eb_oracle.c): EXTRACTDAT
(electric.f:636-716), FASMVP_LAP (laplace.f:159-262), DIRICH_NEU_MAP / PVINTEV
(laplace.f:266-331, pv_integral.f:53-345), SETVELF (stokesbubb.f:4-135, zbond = 0),
FASMVP (stokesbubb.f:496-614), INTERFACENEW (electric.f:791-912), EQUIT
(electric.f:1270-1302) and FILTER (electric.f:1152-1187). The GMRES solves are replaced
by exact dense solves: the gradient is that of F with exact solves.
"""
import math

import numpy as np
import torch

PI = math.pi
DEV = "cpu"  # the device of the tensors the helpers create (set by f_vjp)


def _fft(x):
    return torch.fft.fft(x)


def _bfft(x):
    return torch.fft.ifft(x) * x.shape[-1]


def _wavenum(n):
    m = torch.arange(n, dtype=torch.float64, device=DEV)
    k = torch.where(m <= n // 2, m, m - n)
    k[n // 2] = 0.0
    return k


def fdifff(f):
    """FDIFFF (dcfft.f:1371-1428): spectral derivative, Nyquist mode zeroed."""
    n = f.shape[-1]
    return _bfft(_fft(f) / n * (1j * _wavenum(n)))


def fourint(c):
    """FOURINT (electric.f:1307-1331) on Fourier coefficients: c_k/(i k), mean and
    Nyquist dropped."""
    n = c.shape[-1]
    k = _wavenum(n)
    kk = torch.where(k == 0, torch.ones_like(k), k)
    return torch.where(k == 0, torch.zeros_like(c), c / (1j * kk))


def antideriv(g):
    """Samples of the periodic antiderivative of g: DCFFTB(FOURINT(DCFFTF(g)/n))."""
    n = g.shape[-1]
    return _bfft(fourint(_fft(g) / n))


def finterc(f):
    """FINTERC (pv_integral.f:276-328): complex samples n -> 2n, Nyquist dropped."""
    n = f.shape[-1]
    c = _fft(f)
    c = torch.cat([c[: n // 2], torch.zeros(1, dtype=c.dtype, device=DEV), c[n // 2 + 1:]])
    w = torch.cat([c[: n // 2 + 1], torch.zeros(n, dtype=c.dtype, device=DEV), c[n // 2 + 1:]])
    return _bfft(w / n)


def finter(x):
    """FINTER (pv_integral.f:206-260) of a real sample, with the reference's zeroing of
    the imaginary part of mode n/2-1 and the real part of mode n/2 (:235-236)."""
    n = x.shape[-1]
    c = _fft(x.to(torch.complex128))
    ny = n // 2
    c = torch.cat([c[: ny - 1], c[ny - 1: ny].real.to(torch.complex128),
                   1j * c[ny: ny + 1].imag, c[ny + 1:]])
    w = torch.cat([c[: ny + 1], torch.zeros(n, dtype=c.dtype, device=DEV), c[ny + 1:]])
    return _bfft(w / n).real


def filter_(c):
    """FILTER: exp(-10 (k/n)^25) (k/n in single precision), then parts below 1e-13
    zeroed. The zeroing is in the values only: its derivative is taken as the identity,
    as the GPU's adjoint takes it (it moves F by at most 1e-13 per coefficient)."""
    n = c.shape[-1]
    h = n // 2
    m = np.arange(n)
    i = np.where(m <= h, m, n - m)
    ratio = (i.astype(np.float32) / np.float32(h)).astype(np.float64)
    sig = torch.tensor(np.exp(-10.0 * ratio ** 25), device=DEV)
    v = c * sig
    re, im = v.real, v.imag
    re = re + (torch.where(re.abs() < 1e-13, torch.zeros_like(re), re) - re).detach()
    im = im + (torch.where(im.abs() < 1e-13, torch.zeros_like(im), im) - im).detach()
    out = torch.complex(re, im)
    out = torch.cat([out[:h], torch.zeros(1, dtype=out.dtype, device=DEV), out[h + 1:]])
    return out


def _drops(nd):
    st = np.concatenate([[0], np.cumsum(nd)]).astype(int)
    return [(int(st[b]), int(st[b + 1])) for b in range(len(nd))]


def extractdat(nd, z):
    zk, dz, s, kap, ck, tha = [], [], [], [], [], []
    for a, b in _drops(nd):
        zz = z[a:b]
        zk.append(zz.mean())
        za = fdifff(zz)
        zai = fdifff(za)
        ss = za.abs()
        m = (za.conj() * zai).imag
        kap.append(-m / ss ** 3)
        ck.append(-zai / za)
        tha.append(m / ss ** 2)
        dz.append(-za)
        s.append(ss)
    return (torch.stack(zk), torch.cat(dz), torch.cat(s), torch.cat(kap), torch.cat(ck), torch.cat(tha))


def point_h(nd):
    return torch.tensor(np.concatenate([np.full(n, 2.0 * PI / n) for n in nd]), device=DEV)


def drop_index(nd):
    return torch.tensor(np.concatenate([np.full(n, b) for b, n in enumerate(nd)]), device=DEV)


def _offdiag_inv(zt, zs):
    d = zt[:, None] - zs[None, :]
    eye = torch.eye(d.shape[0], dtype=torch.bool, device=DEV)
    d = torch.where(eye, torch.ones_like(d), d)
    return torch.where(eye, torch.zeros_like(d), 1.0 / d)


def laplace_matrix(nd, z, dz, s, kap):
    """FASMVP_LAP as a dense real matrix: w = u + 2 (h kappa s u/(4 pi) - Re(cf/(2 pi i)))
    - 2 h s u, cf_t = sum_{j != t} u_j dz_j h / (z_t - z_j)."""
    h = point_h(nd)
    K = _offdiag_inv(z, z)
    M = -(K * (dz * h)[None, :]).imag / PI
    return M + torch.diag(1.0 + h * kap * s / (2.0 * PI) - 2.0 * h * s)


def stokes_pq(z, dz, h, sign):
    """The Stokes sum gradw_t = sum_{j != t} qa/D + s (conj(qb/D) - D conj(qa/D^2)),
    D = z_j - z_t, qa = c0 dens dz, qb = c0 (-conj(dens) dz + dens conj(dz)),
    c0 = h / (2 pi i), as gradw = P dens + Q conj(dens)."""
    n = z.shape[0]
    D = z[None, :] - z[:, None]
    eye = torch.eye(n, dtype=torch.bool, device=DEV)
    Ds = torch.where(eye, torch.ones_like(D), D)
    c0 = (h / (2j * PI))[None, :]
    dzj = dz[None, :]
    P = c0 * dzj / Ds - sign * c0.conj() * dzj.conj() / Ds.conj()
    Q = sign * c0.conj() * dzj / Ds.conj() - sign * c0.conj() * dzj.conj() * Ds / Ds.conj() ** 2
    zero = torch.zeros_like(P)
    return torch.where(eye, zero, P), torch.where(eye, zero, Q)


def _real_matrix(P, Q):
    """The real 2n x 2n matrix (interleaved Re/Im) of dens -> P dens + Q conj(dens)."""
    A, B = P + Q, P - Q
    n = P.shape[0]
    R = torch.zeros(2 * n, 2 * n, dtype=torch.float64, device=DEV)
    R[0::2, 0::2] = A.real
    R[0::2, 1::2] = -B.imag
    R[1::2, 0::2] = A.imag
    R[1::2, 1::2] = B.real
    return R


def stokes_matrix(nd, z, dz, s, kap, zk):
    """FASMVP as a dense real matrix."""
    h = point_h(nd)
    drop = drop_index(nd)
    P, Q = stokes_pq(z, dz, h, -1.0)
    same = (drop[:, None] == drop[None, :])
    # za_b = h sum dens
    P = P + torch.where(same, h[None, :].to(torch.complex128), torch.zeros_like(P))
    # 0.5 i pk_b z_t, pk_b = sum_i (2h/pi) Re(dens_i e_i), e_i = dz_i/(z_i - zk_b)^2
    e = dz / (z - zk[drop]) ** 2
    coef = 0.5j * z[:, None] * (2.0 * h[None, :] / PI) * 0.5
    P = P + torch.where(same, coef * e[None, :], torch.zeros_like(P))
    Q = Q + torch.where(same, coef * e.conj()[None, :], torch.zeros_like(Q))
    # zself = dens h s kappa/(2 pi) + conj(dens) h kappa dz^2/(2 pi s), and the identity
    P = P + torch.diag(1.0 + h * s * kap / (2.0 * PI) + 0j)
    Q = Q + torch.diag(h * kap * dz ** 2 / (2.0 * PI * s))
    return _real_matrix(P, Q)


def f_stage(nd, y, e0, cap):
    """F(y): the node velocities (interleaved real 2N) of one RK stage."""
    nd = [int(n) for n in nd]
    z = torch.complex(y[0::2], y[1::2])
    zk, dz, s, kap, ck, tha = extractdat(nd, z)
    h = point_h(nd)
    # Laplace solve (GETBCs rhs -2 Re z)
    ul = torch.linalg.solve(laplace_matrix(nd, z, dz, s, kap), -2.0 * z.real)
    # DIRICH_NEU_MAP: PV integral on the 2x interpolated curve
    uc = ul * dz
    # (sources on the odd fine nodes, the field at the even ones: FINTER's positions)
    zsrc, ztgt, qs = [], [], []
    for a, b in _drops(nd):
        n = b - a
        u2 = finterc(uc[a:b])
        x2, y2 = finter(z[a:b].real), finter(z[a:b].imag)
        zsrc.append(torch.complex(x2[1::2], y2[1::2]))
        ztgt.append(torch.complex(x2[0::2], y2[0::2]))
        qs.append(u2[1::2] * (2.0 * PI / n))
    zsrc, ztgt, qs = torch.cat(zsrc), torch.cat(ztgt), torch.cat(qs)
    cfp = (qs[None, :] / (ztgt[:, None] - zsrc[None, :])).sum(1)
    psi = -cfp.real / (2.0 * PI) - z.imag
    dphi = torch.cat([-fdifff(psi[a:b].to(torch.complex128)).real for a, b in _drops(nd)]) / s
    # SETVELF (zbond = 0): -dz/(2 s) + i cap conj(z)/2 + (i E0/4)(alpha c0 + G_i - G_0)
    alpha_c = 2.0 * PI * (nd[-1] - 1) / nd[-1]
    rhs = -0.5 * dz / s + 0.5j * cap * z.conj()
    st = []
    for a, b in _drops(nd):
        g = dz[a:b] * dphi[a:b] ** 2
        G = antideriv(g)
        st.append(0.25j * e0 * (alpha_c * g.mean() + G - G[0]))
    rhs = rhs + torch.cat(st)
    rr = torch.stack([rhs.real, rhs.imag], 1).reshape(-1)
    sol = torch.linalg.solve(stokes_matrix(nd, z, dz, s, kap, zk), rr)
    u = torch.complex(sol[0::2], sol[1::2])
    # INTERFACENEW (zc = 0, no wall)
    udot = torch.cat([fdifff(u[a:b]) for a, b in _drops(nd)])
    P, Q = stokes_pq(z, dz, h, 1.0)
    gw = P @ u + Q @ u.conj()
    gw = gw - u.conj() * h * kap * dz ** 2 / (2.0 * PI * s)
    gw = gw + (h * ck.real * u - 2.0 * h * udot) / (2j * PI)
    gw = gw + 0.5j * cap * z.conj()
    un = (gw * dz.conj()).real / s
    # EQUIT, the node velocity, FILTER
    out = []
    for a, b in _drops(nd):
        n = b - a
        tt = -antideriv((-tha[a:b] * un[a:b]).to(torch.complex128)).real
        zf = -(un[a:b] * 1j * dz[a:b] + tt * dz[a:b]) / s[a:b]
        out.append(_bfft(filter_(_fft(zf) / n)))
    r = torch.cat(out)
    return torch.stack([r.real, r.imag], 1).reshape(-1)


def deformation(nd, y):
    """Sum over drops of (L - B)/(L + B), L and B the largest and smallest distance of a
    drop's nodes from its centroid (the mean of its nodes)."""
    z = torch.complex(y[0::2], y[1::2])
    tot = 0.0
    for a, b in _drops([int(n) for n in nd]):
        r = (z[a:b] - z[a:b].mean()).abs()
        L, B = r.max(), r.min()
        tot = tot + (L - B) / (L + B)
    return tot


def f_vjp(nd, y, v, e0, cap, device="cpu"):
    """(F(y), v^T dF/dy, v^T dF/dE0, v^T dF/dcap) by autograd, on `device`."""
    global DEV
    DEV = device
    try:
        yt = torch.tensor(np.asarray(y, dtype=np.float64), requires_grad=True, device=device)
        e0t = torch.tensor(float(e0), dtype=torch.float64, requires_grad=True, device=device)
        capt = torch.tensor(float(cap), dtype=torch.float64, requires_grad=True, device=device)
        f = f_stage(nd, yt, e0t, capt)
        gy, ge, gc = torch.autograd.grad(f, (yt, e0t, capt),
                                         torch.tensor(np.asarray(v, dtype=np.float64), device=device))
        return f.detach().cpu().numpy(), gy.cpu().numpy(), float(ge), float(gc)
    finally:
        DEV = "cpu"


def rk2_gradient(nd, dt, y0, steps, e0, cap):
    """J = deformation after `steps` RK2 (Heun) steps from y0, and dJ/dy0, dJ/dE0,
    dJ/dcap by autograd through every step."""
    yt = torch.tensor(np.asarray(y0, dtype=np.float64), requires_grad=True)
    e0t = torch.tensor(float(e0), dtype=torch.float64, requires_grad=True)
    capt = torch.tensor(float(cap), dtype=torch.float64, requires_grad=True)
    y = yt
    for _ in range(steps):
        k1 = f_stage(nd, y, e0t, capt)
        k2 = f_stage(nd, y + dt * k1, e0t, capt)
        y = y + 0.5 * dt * k1 + 0.5 * dt * k2
    J = deformation(nd, y)
    gy, ge, gc = torch.autograd.grad(J, (yt, e0t, capt))
    return float(J.detach()), gy.numpy(), float(ge), float(gc)
