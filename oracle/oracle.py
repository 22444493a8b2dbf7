"""numpy binding of the CPU oracle (oracle/eb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the checker
and by bench.py's CPU-baseline leg. The product never imports it.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


class C2(ctypes.Structure):
    """A C99 double _Complex passed by value (same register class as two doubles)."""
    _fields_ = [("re", _D), ("im", _D)]


class Geom(ctypes.Structure):
    _fields_ = [("k", _I), ("nd", _P), ("nbk", _I), ("z", _P), ("dz", _P), ("dsda", _P),
                ("kappa", _P), ("zk", _P), ("iwall", _I), ("xleft", _D), ("slength", _D)]


class Model(ctypes.Structure):
    _fields_ = [("cap", _D), ("e0", _D), ("zbond", _D * 2), ("mode", _I), ("nthreads", _I),
                ("maxl", _I), ("gmres_tol", _D), ("lap_iter", _I), ("stokes_iter", _I),
                ("lap_err", _D), ("stokes_err", _D), ("flux", _D)]


MATVEC_FN = ctypes.CFUNCTYPE(None, _I, ctypes.POINTER(_D), ctypes.POINTER(_D), _P)

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        sig = {
            "eb_or_fft": (None, [_I, _P, _I]),
            "eb_or_fdifff": (None, [_I, _P, _P]),
            "eb_or_fourint": (None, [_I, _P, _P]),
            "eb_or_filter": (None, [_I, _P]),
            "eb_or_finterc": (None, [_I, _P, _P]),
            "eb_or_finter": (None, [_I, _P, _P]),
            "eb_or_extractdat": (None, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "eb_or_stokes_direct": (None, [_I, _P, _P, _P, _P, _I, _P, _I]),
            "eb_or_stokes_direct_at": (None, [_I, _P, _P, _P, _P, _I, _I, _P, _P, _I]),
            "eb_or_cadap_fmm": (_I, [_I, _P, _P, _P, _P, _I, _I, _D, _P, _I]),
            "eb_or_cadap_fmm_w": (_I, [_I, _P, _P, _P, _P, _I, _I, _D, _I, _D, _D, _P, _I]),
            "eb_or_stokes_image_direct": (None, [_I, _P, _P, _P, _P, _I, _P, _I]),
            "eb_or_refsing": (None, [C2, _I, _P, _P, _P, _P, _P, _P]),
            "eb_or_wallinfo": (None, [_I, _P, _P, _P]),
            "eb_or_cauchy_direct": (None, [_I, _P, _I, _P, _P, _I, _P, _I]),
            "eb_or_fasmvp": (None, [ctypes.POINTER(Geom), _P, _P, _I, _I]),
            "eb_or_fasmvp_lap": (None, [ctypes.POINTER(Geom), _P, _P, _I]),
            "eb_or_fasmvp_lap2": (None, [ctypes.POINTER(Geom), _P, _P, _I, _I]),
            "eb_or_dapif2": (None, [_I, _P, _P, _D, _I, _P, _I]),
            "eb_or_pvintev": (None, [_I, _P, _P, _P, _P, _I]),
            "eb_or_dirich_neu_map": (None, [ctypes.POINTER(Geom), _P, _P, _P, _P, _I]),
            "eb_or_interfacenew": (None, [ctypes.POINTER(Geom), _P, _P, _D, _P, _P, _P, _I, _I]),
            "eb_or_setvelf": (None, [ctypes.POINTER(Geom), _P, C2, _D, _D, _P, _P]),
            "eb_or_equit": (None, [_I, _P, _P, _P]),
            "eb_or_gmres": (_I, [_I, _P, _P, MATVEC_FN, _P, _I, _D, ctypes.POINTER(_I),
                                 ctypes.POINTER(_D)]),
            "eb_or_f": (None, [ctypes.POINTER(Model), _I, _P, _P, _P]),
            "eb_or_rk2": (None, [ctypes.POINTER(Model), _I, _P, _D, _P]),
            "eb_or_max_threads": (_I, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _r(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def max_threads():
    return lib().eb_or_max_threads()


# ---- spectral -------------------------------------------------------------------
def fft(c, direction):
    c = _c(c).copy()
    lib().eb_or_fft(c.shape[0], _p(c), int(direction))
    return c


def fdifff(f):
    f = _c(f)
    d = np.empty_like(f)
    lib().eb_or_fdifff(f.shape[0], _p(f), _p(d))
    return d


def fourint(zf):
    zf = _c(zf)
    o = np.empty_like(zf)
    lib().eb_or_fourint(zf.shape[0], _p(zf), _p(o))
    return o


def filter_(cn):
    cn = _c(cn).copy()
    lib().eb_or_filter(cn.shape[0], _p(cn))
    return cn


def finterc(f):
    f = _c(f)
    o = np.empty(2 * f.shape[0], np.complex128)
    lib().eb_or_finterc(f.shape[0], _p(f), _p(o))
    return o


def finter(f):
    f = _r(f)
    o = np.empty(2 * f.shape[0])
    lib().eb_or_finter(f.shape[0], _p(f), _p(o))
    return o


def extractdat(nd, rku):
    nd = _i(nd)
    rku = _r(rku)
    k = nd.shape[0]
    nbk = int(nd.sum())
    out = {"z": np.empty(nbk, np.complex128), "zk": np.empty(k, np.complex128),
           "dz": np.empty(nbk, np.complex128), "tha": np.empty(nbk), "dsda": np.empty(nbk),
           "kappa": np.empty(nbk), "ckern": np.empty(nbk, np.complex128), "area": np.empty(k)}
    lib().eb_or_extractdat(k, _p(nd), _p(rku), _p(out["z"]), _p(out["zk"]), _p(out["dz"]),
                           _p(out["tha"]), _p(out["dsda"]), _p(out["kappa"]), _p(out["ckern"]),
                           _p(out["area"]))
    return out


# ---- sums -----------------------------------------------------------------------
def point_h(nd):
    return np.concatenate([np.full(int(n), 2 * np.pi / int(n)) for n in nd])


def stokes_direct(z, dz, hpt, dens, sign, nthreads=0):
    z, dz, dens = _c(z), _c(dz), _c(dens)
    hpt = _r(hpt)
    g = np.empty_like(z)
    lib().eb_or_stokes_direct(z.shape[0], _p(z), _p(dz), _p(hpt), _p(dens), int(sign), _p(g),
                              int(nthreads))
    return g


def stokes_direct_at(z, dz, hpt, dens, sign, tidx, nthreads=0):
    """The direct Stokes sum at the nodes tidx only (self excluded)."""
    z, dz, dens = _c(z), _c(dz), _c(dens)
    hpt = _r(hpt)
    tidx = _i(tidx)
    out = np.empty(tidx.shape[0], np.complex128)
    lib().eb_or_stokes_direct_at(z.shape[0], _p(z), _p(dz), _p(hpt), _p(dens), int(sign),
                                 tidx.shape[0], _p(tidx), _p(out), int(nthreads))
    return out


def cadap_fmm(z, dz, hpt, dens, sign, levmax=7, tol=1e-13, nthreads=0):
    z, dz, dens = _c(z), _c(dz), _c(dens)
    hpt = _r(hpt)
    g = np.empty_like(z)
    st = lib().eb_or_cadap_fmm(z.shape[0], _p(z), _p(dz), _p(hpt), _p(dens), int(sign),
                               int(levmax), float(tol), _p(g), int(nthreads))
    if st != 0:
        raise RuntimeError("cadap_fmm IER=%d" % st)
    return g


def cadap_fmm_wall(z, dz, hpt, dens, sign, xleft, slength, levmax=7, tol=1e-13, nthreads=0):
    """CADAPDR (sign -1) / CADAPMOD (sign +1) with IFLAG2 = 1: the wall y = 0."""
    z, dz, dens = _c(z), _c(dz), _c(dens)
    hpt = _r(hpt)
    g = np.empty_like(z)
    st = lib().eb_or_cadap_fmm_w(z.shape[0], _p(z), _p(dz), _p(hpt), _p(dens), int(sign),
                                 int(levmax), float(tol), 1, float(xleft), float(slength), _p(g),
                                 int(nthreads))
    if st != 0:
        raise RuntimeError("cadap_fmm IER=%d" % st)
    return g


def stokes_image_direct(z, dz, hpt, dens, sign, nthreads=0):
    """The exact reflected part of the wall-bounded Stokes sum (images across y = 0)."""
    z, dz, dens = _c(z), _c(dz), _c(dens)
    hpt = _r(hpt)
    g = np.empty_like(z)
    lib().eb_or_stokes_image_direct(z.shape[0], _p(z), _p(dz), _p(hpt), _p(dens), int(sign), _p(g),
                                    int(nthreads))
    return g


def refsing(zt, zk, zc, zb=None):
    """REFSING (reflect.f:28-86) from zero: (phi, phi', psi) of the reflected singularities."""
    zk, zc = _c(zk), _c(zc)
    zb = np.zeros_like(zk) if zb is None else _c(zb)
    out = np.zeros(3, np.complex128)
    zt = complex(zt)
    lib().eb_or_refsing(C2(zt.real, zt.imag), zk.shape[0], _p(zk), _p(zc), _p(zb),
                        _p(out[0:1]), _p(out[1:2]), _p(out[2:3]))
    return out[0], out[1], out[2]


def wallinfo(z):
    """EXTRACTDAT's xleft, slength (electric.f:657-711)."""
    z = _c(z)
    xl, sl = _D(), _D()
    lib().eb_or_wallinfo(z.shape[0], _p(z), ctypes.byref(xl), ctypes.byref(sl))
    return xl.value, sl.value


def cauchy_direct(zt, zs, q, self_exclude, nthreads=0):
    zt, zs, q = _c(zt), _c(zs), _c(q)
    f = np.empty_like(zt)
    lib().eb_or_cauchy_direct(zt.shape[0], _p(zt), zs.shape[0], _p(zs), _p(q),
                              1 if self_exclude else 0, _p(f), int(nthreads))
    return f


# ---- operators ------------------------------------------------------------------
class Geometry:
    """Geometry arrays kept alive together with the C struct that points at them."""

    def __init__(self, nd, z, dz, dsda, kappa, zk, wall=False):
        self.nd = _i(nd)
        self.z, self.dz, self.zk = _c(z), _c(dz), _c(zk)
        self.dsda, self.kappa = _r(dsda), _r(kappa)
        self.nbk = int(self.nd.sum())
        self.k = int(self.nd.shape[0])
        xl, sl = wallinfo(self.z) if wall else (0.0, 0.0)
        self.xleft, self.slength = xl, sl
        self.s = Geom(self.k, _p(self.nd), self.nbk, _p(self.z), _p(self.dz), _p(self.dsda),
                      _p(self.kappa), _p(self.zk), 1 if wall else 0, xl, sl)

    @classmethod
    def from_extract(cls, nd, ex, wall=False):
        return cls(nd, ex["z"], ex["dz"], ex["dsda"], ex["kappa"], ex["zk"], wall)


def fasmvp(g, u, mode=0, nthreads=0):
    u = _r(u)
    w = np.empty(2 * g.nbk)
    lib().eb_or_fasmvp(ctypes.byref(g.s), _p(u), _p(w), int(mode), int(nthreads))
    return w


def fasmvp_lap(g, u, nthreads=0, mode=0):
    """FASMVP_LAP; mode 1: the Cauchy sum by the restated DAPIF2 FMM (TOL 1e-11)."""
    u = _r(u)
    w = np.empty(g.nbk)
    lib().eb_or_fasmvp_lap2(ctypes.byref(g.s), _p(u), _p(w), int(mode), int(nthreads))
    return w


def dapif2(z, q, tol=1e-11, napb=30, nthreads=0):
    """DAPIF2 with IFLAG7 = 3: sum_{j != i} q_j / (z_i - z_j) by the adaptive FMM."""
    z, q = _c(z), _c(q)
    f = np.empty_like(z)
    lib().eb_or_dapif2(z.shape[0], _p(z), _p(q), float(tol), int(napb), _p(f), int(nthreads))
    return f


def pvintev(nd, z, ucmplx, nthreads=0):
    nd, z, u = _i(nd), _c(z), _c(ucmplx)
    phi = np.empty_like(u)
    lib().eb_or_pvintev(nd.shape[0], _p(nd), _p(z), _p(u), _p(phi), int(nthreads))
    return phi


def dirich_neu_map(g, u, nthreads=0):
    u = _r(u)
    phi, psi, dphi = np.empty(g.nbk), np.empty(g.nbk), np.empty(g.nbk)
    lib().eb_or_dirich_neu_map(ctypes.byref(g.s), _p(u), _p(phi), _p(psi), _p(dphi), int(nthreads))
    return phi, psi, dphi


def interfacenew(g, ckern, zc, cap, u, mode=0, nthreads=0):
    ckern, zc, u = _c(ckern), _c(zc), _c(u)
    un = np.empty(g.nbk)
    flux = np.zeros(1)
    lib().eb_or_interfacenew(ctypes.byref(g.s), _p(ckern), _p(zc), float(cap), _p(u), _p(un),
                             _p(flux), int(mode), int(nthreads))
    return un, float(flux[0])


def setvelf(g, zc, zbond, cap, e0, dphi_dn):
    zc = _c(zc)
    dphi = _r(dphi_dn)
    rhs = np.empty(2 * g.nbk)
    zb = C2(complex(zbond).real, complex(zbond).imag)
    lib().eb_or_setvelf(ctypes.byref(g.s), _p(zc), zb, float(cap), float(e0), _p(dphi), _p(rhs))
    return rhs


def equit(tha, un):
    tha, un = _r(tha), _r(un)
    t = np.empty_like(tha)
    lib().eb_or_equit(tha.shape[0], _p(tha), _p(un), _p(t))
    return t


def gmres(matvec, b, x0, maxl=100, tol=1e-10):
    """SLATEC-semantics GMRES with a Python callback matvec(x) -> y."""
    b = _r(b)
    x = _r(x0).copy()
    n = b.shape[0]

    def cb(nn, xp, yp, ud):
        xv = np.ctypeslib.as_array(xp, shape=(nn,))
        yv = np.ctypeslib.as_array(yp, shape=(nn,))
        yv[:] = matvec(xv.copy())

    f = MATVEC_FN(cb)
    it = _I()
    err = _D()
    ierr = lib().eb_or_gmres(n, _p(b), _p(x), f, None, int(maxl), float(tol), ctypes.byref(it),
                             ctypes.byref(err))
    return x, {"iters": it.value, "err": err.value, "ierr": ierr}


def deflate(nd, dsda, x, inverse):
    """The per-drop deflation of the Laplace solve's right preconditioner: with P_k the
    mean over drop k spread over its nodes and mu_k = -2 h_k mean_k(s') (FASMVP_LAP's
    eigenvalue on the drop's constant, from its -2 h u s' term, laplace.f:235-236),
    M^-1 x = x + sum_k (1/mu_k - 1) P_k x (inverse) or M x = x + sum_k (mu_k - 1) P_k x.
    No counterpart in the reference (DGMRES runs with JPRE = 0); this checks the CUDA
    path's eb_opts.lap_deflate."""
    x = _r(x)
    dsda = _r(dsda)
    y = x.copy()
    off = 0
    for n in np.asarray(nd, dtype=np.int64):
        s = slice(off, off + int(n))
        mu = -2.0 * (2.0 * np.pi / n) * dsda[s].mean()
        c = 1.0 / mu - 1.0 if inverse else mu - 1.0
        y[s] += c * x[s].mean()
        off += int(n)
    return y


def solve_lapl_deflated(g, rhs, nthreads=0, maxl=100, tol=1e-10, mode=0):
    """SOLVE_LAPL's GMRES on A M^-1 t = rhs from t0 = M rhs; returns x = M^-1 t."""
    t0 = deflate(g.nd, g.dsda, rhs, False)
    t, info = gmres(lambda t: fasmvp_lap(g, deflate(g.nd, g.dsda, t, True), nthreads, mode), rhs, t0, maxl,
                    tol)
    return deflate(g.nd, g.dsda, t, True), info


def solvei(g, rhs, mode=0, nthreads=0, maxl=100, tol=1e-10):
    return gmres(lambda x: fasmvp(g, x, mode, nthreads), rhs, rhs, maxl, tol)


def solve_lapl(g, rhs, nthreads=0, maxl=100, tol=1e-10, mode=0):
    return gmres(lambda x: fasmvp_lap(g, x, nthreads, mode), rhs, rhs, maxl, tol)


def make_model(cap=0.0, e0=0.5, zbond=0j, mode=0, nthreads=0, maxl=100, gmres_tol=1e-10):
    m = Model()
    m.cap, m.e0 = cap, e0
    m.zbond[0], m.zbond[1] = complex(zbond).real, complex(zbond).imag
    m.mode, m.nthreads, m.maxl, m.gmres_tol = mode, nthreads, maxl, gmres_tol
    return m


def f_eval(model, nd, rku):
    nd, rku = _i(nd), _r(rku)
    out = np.empty_like(rku)
    lib().eb_or_f(ctypes.byref(model), nd.shape[0], _p(nd), _p(rku), _p(out))
    return out


def rk2(model, nd, dt, ybar):
    nd = _i(nd)
    y = _r(ybar).copy()
    lib().eb_or_rk2(ctypes.byref(model), nd.shape[0], _p(nd), float(dt), _p(y))
    return y
