"""Python mirror of the reference's operator interface, backed by libeb_gb300.so.

The reference (Fortran 77) exposes its hot path as subroutines that share the geometry
through COMMON blocks. Here a `Context` holds that geometry on the GPU and offers the
same operations under the reference's names:

    fasmvp / matvec            Stokes operator          (stokesbubb.f:419-614)
    fasmvp_lap / matvec_lapl   Laplace operator         (laplace.f:159-262, 429-465)
    cadapdr / cadapmod         Stokes layer sums        (cadapdrop.f, cadapmod.f)
    dapif2                     Cauchy sum, IFLAG7 = 3   (dapif1.f:458-1077)
    solvei / solve_lapl        GMRES solves             (stokesbubb.f:294-415, laplace.f:335-425)
    fdifff                     spectral derivative      (dcfft.f:1371-1428)
    pvintev, dirich_neu_map    PV integral, DtN map     (pv_integral.f:53-204, laplace.f:266-331)
    interfacenew               interface velocity       (electric.f:791-912)
    extractdat                 geometry from the RK state (electric.f:636-716)
    setvelf                    Stokes right-hand side   (stokesbubb.f:4-135)
    f / rk2                    RK right-hand side and step (electric.f:968-1109, 762-786)

Arrays may be numpy arrays (host memory; copied in and out) or CUDA tensors exposing
`data_ptr()` and `is_cuda` (device memory; used in place). Errors raise `EbError`,
where the reference would print and STOP. There is no CPU fallback: without the built
library or a CUDA device, construction fails.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (EB_DEVICE, EB_FP32, EB_FP64, EB_HOST, EB_SOLVE_FP32_REFINED, EB_SOLVE_FP64,
                   AdjointInfo, EbError, Model, Opts, SolveInfo, StageInfo, TreeInfo, check)

PRECISION = {"fp64": EB_FP64, "fp32": EB_FP32}
SOLVE_MODE = {"fp64": EB_SOLVE_FP64, "fp32_refined": EB_SOLVE_FP32_REFINED}


def _is_device(a):
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):  # CUDA tensor, or a (pinned) host tensor
        return ctypes.c_void_p(a.data_ptr())
    if not (isinstance(a, np.ndarray) and a.flags["C_CONTIGUOUS"]):
        raise TypeError("expected a C-contiguous numpy array or a CUDA tensor")
    return ctypes.c_void_p(a.ctypes.data)


def _mem(*arrays):
    dev = [_is_device(a) for a in arrays if a is not None]
    if all(dev):
        return EB_DEVICE
    if not any(dev):
        return EB_HOST
    raise TypeError("mix of host and device arrays in one call")


def _host(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Context:
    """One GPU context: geometry, trees, expansion work space and a CUDA stream."""

    def __init__(self, p64=0, p32=0, leaf64=0, leaf_cap=0, tol64=0.0, tol32=0.0, maxl=0,
                 gmres_tol=0.0, inner_tol=0.0, max_outer=0, device=0, graphs=0, df64=0,
                 resid_df=0, m2l_tc=0, lap_deflate=0, direct_max=0, adj_df=0):
        self._lib = _lib.load()
        o = Opts()
        self._lib.eb_opts_default(ctypes.byref(o))
        for name, v in (("p64", p64), ("p32", p32), ("leaf64", leaf64), ("leaf_cap", leaf_cap),
                        ("tol64", tol64), ("tol32", tol32), ("maxl", maxl),
                        ("gmres_tol", gmres_tol), ("inner_tol", inner_tol),
                        ("max_outer", max_outer), ("graphs", graphs), ("df64", df64),
                        ("resid_df", resid_df), ("m2l_tc", m2l_tc),
                        ("lap_deflate", lap_deflate), ("direct_max", direct_max), ("adj_df", adj_df)):
            if v:
                setattr(o, name, v)
        o.device = device
        h = ctypes.c_void_p()
        check("eb_ctx_create", self._lib.eb_ctx_create(ctypes.byref(h), ctypes.byref(o)))
        self._h = h
        self.k = 0
        self.nbk = 0
        self.nd = None

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.eb_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- context -------------------------------------------------------------
    def set_stream(self, stream_handle):
        """Run on an existing CUDA stream (an integer cudaStream_t), or None."""
        check("eb_ctx_set_stream", self._lib.eb_ctx_set_stream(
            self._h, ctypes.c_void_p(stream_handle) if stream_handle else None))

    def sync(self):
        check("eb_ctx_sync", self._lib.eb_ctx_sync(self._h))

    def launch_count(self):
        return int(self._lib.eb_ctx_launch_count(self._h))

    def set_profiling(self, on=True):
        check("eb_ctx_set_profiling", self._lib.eb_ctx_set_profiling(self._h, 1 if on else 0))

    def kernel_time(self, cls):
        n = ctypes.c_longlong()
        ms = ctypes.c_double()
        check("eb_ctx_kernel_time", self._lib.eb_ctx_kernel_time(self._h, cls, ctypes.byref(n),
                                                                 ctypes.byref(ms)))
        return n.value, ms.value

    def measure_fp64_peak(self):
        v = ctypes.c_double()
        check("eb_measure_fp64_peak", self._lib.eb_measure_fp64_peak(self._h, ctypes.byref(v)))
        return v.value

    def measure_fp32_peak(self):
        v = ctypes.c_double()
        check("eb_measure_fp32_peak", self._lib.eb_measure_fp32_peak(self._h, ctypes.byref(v)))
        return v.value

    def tree_info(self):
        t = TreeInfo()
        check("eb_ctx_tree_info", self._lib.eb_ctx_tree_info(self._h, ctypes.byref(t)))
        return t.as_dict()

    def getfourier(self, nd, rku):
        """GETFOURIER per drop: (idoub flags, fmode per drop)."""
        nd = _host(nd, np.int32)
        rku = _host(rku, np.float64)
        k = int(nd.shape[0])
        idoub = np.zeros(k, np.int32)
        fmode = np.zeros(int(nd.sum()))
        check("eb_getfourier", self._lib.eb_getfourier(self._h, k, _ptr(nd), _ptr(rku), _ptr(idoub),
                                                      _ptr(fmode), EB_HOST))
        starts = np.r_[0, np.cumsum(nd)]
        return idoub, [fmode[a:a + n // 2] for a, n in zip(starts[:-1], nd)]

    def double(self, nd, rku, idoub):
        """DOUBLE: (new nd, new RK state) with the flagged drops resampled to 2 nd."""
        nd = _host(nd, np.int32)
        rku = _host(rku, np.float64)
        idoub = _host(idoub, np.int32)
        nd2 = np.where(idoub != 0, 2 * nd, nd).astype(np.int32)
        out = np.zeros(2 * int(nd2.sum()))
        check("eb_double", self._lib.eb_double(self._h, int(nd.shape[0]), _ptr(nd), _ptr(rku), _ptr(idoub),
                                              _ptr(out), EB_HOST))
        return nd2, out

    def autotune(self):
        """Pick the tree's leaf sizes for the installed geometry by timing the FP32
        operator; returns the chosen sizes and every candidate's time."""
        t = _lib.TuneInfo()
        check("eb_autotune", self._lib.eb_autotune(self._h, ctypes.byref(t)))
        return t.as_dict()

    def batch_define(self, sim_k, e0=None):
        """Make the context hold independent simulations: simulation s is the next
        sim_k[s] drops of every geometry installed from now on, with its own E0 (e0[s]).
        An empty sim_k returns to one simulation."""
        sim_k = _host(sim_k, np.int32)
        e = None if e0 is None else _host(e0, np.float64)
        check("eb_batch_define", self._lib.eb_batch_define(
            self._h, int(sim_k.shape[0]), _ptr(sim_k) if sim_k.shape[0] else None,
            _ptr(e) if e is not None else None))
        self._batch_keep = (sim_k, e)

    # ---- geometry ------------------------------------------------------------
    def set_geometry(self, nd, z, dz, dsda, kappa, zk):
        """Install the geometry (COMMON /inteqn/ and /problem/)."""
        nd = _host(nd, np.int32)
        arrs = [z, dz, dsda, kappa, zk]
        mem = _mem(*arrs)
        if mem == EB_HOST:
            z, dz, zk = (_host(a, np.complex128) for a in (z, dz, zk))
            dsda, kappa = (_host(a, np.float64) for a in (dsda, kappa))
        check("eb_set_geometry", self._lib.eb_set_geometry(
            self._h, int(nd.shape[0]), _ptr(nd), _ptr(z), _ptr(dz), _ptr(dsda), _ptr(kappa),
            _ptr(zk), mem))
        self.k = int(nd.shape[0])
        self.nbk = int(nd.sum())
        self.nd = nd
        self._keep = (z, dz, dsda, kappa, zk)

    def extractdat(self, nd, rku):
        """EXTRACTDAT on the GPU: install the geometry of the RK state `rku`
        (interleaved x, y) and return it as a dict of host arrays."""
        nd = _host(nd, np.int32)
        k = int(nd.shape[0])
        nbk = int(nd.sum())
        rku = _host(rku, np.float64)
        out = {"zk": np.zeros(k, np.complex128), "dz": np.zeros(nbk, np.complex128),
               "dsda": np.zeros(nbk), "kappa": np.zeros(nbk), "ckern": np.zeros(nbk, np.complex128),
               "tha": np.zeros(nbk), "area": np.zeros(k)}
        check("eb_extractdat", self._lib.eb_extractdat(
            self._h, k, _ptr(nd), _ptr(rku), _ptr(out["zk"]), _ptr(out["dz"]), _ptr(out["dsda"]),
            _ptr(out["kappa"]), _ptr(out["ckern"]), _ptr(out["tha"]), _ptr(out["area"]), EB_HOST))
        self.k = k
        self.nbk = nbk
        self.nd = nd
        out["z"] = rku.view(np.complex128).copy()
        return out

    def extractdat_device(self, nd, rku_dev):
        """EXTRACTDAT from a device RK state; nothing is copied back."""
        nd = _host(nd, np.int32)
        k = int(nd.shape[0])
        check("eb_extractdat", self._lib.eb_extractdat(
            self._h, k, _ptr(nd), _ptr(rku_dev), None, None, None, None, None, None, None,
            EB_DEVICE))
        self.k = k
        self.nbk = int(nd.sum())
        self.nd = nd

    # ---- operators -----------------------------------------------------------
    def _out(self, x, n, dtype):
        if _is_device(x):
            import torch
            tdt = {np.float64: torch.float64, np.complex128: torch.complex128}[dtype]
            return torch.empty(n, dtype=tdt, device=x.device)
        return np.empty(n, dtype)

    def fasmvp(self, x, precision="fp64", out=None):
        """Stokes operator FASMVP / MATVEC: x, y real of length 2 nbk."""
        if not _is_device(x):
            x = _host(x, np.float64)
        y = out if out is not None else self._out(x, 2 * self.nbk, np.float64)
        check("eb_stokes_matvec", self._lib.eb_stokes_matvec(
            self._h, 2 * self.nbk, _ptr(x), _ptr(y), PRECISION[precision], _mem(x, y)))
        return y

    matvec = fasmvp

    def fasmvp_lap(self, x, precision="fp64", out=None):
        """Laplace operator FASMVP_LAP / MATVEC_LAPL: x, y real of length nbk."""
        if not _is_device(x):
            x = _host(x, np.float64)
        y = out if out is not None else self._out(x, self.nbk, np.float64)
        check("eb_laplace_matvec", self._lib.eb_laplace_matvec(
            self._h, self.nbk, _ptr(x), _ptr(y), PRECISION[precision], _mem(x, y)))
        return y

    matvec_lapl = fasmvp_lap

    def laplace_constraints(self, x):
        x = _host(x, np.float64)
        s = np.empty(self.k)
        check("eb_laplace_constraints", self._lib.eb_laplace_constraints(
            self._h, self.nbk, _ptr(x), _ptr(s), EB_HOST))
        return s

    def stokes_sum(self, dens, sign, precision="fp64"):
        """GRADW of CADAPDR (sign -1) or CADAPMOD (sign +1) at the installed nodes."""
        if not _is_device(dens):
            dens = _host(dens, np.complex128)
        g = self._out(dens, self.nbk, np.complex128)
        check("eb_stokes_sum", self._lib.eb_stokes_sum(
            self._h, self.nbk, _ptr(dens), int(sign), _ptr(g), PRECISION[precision], _mem(dens, g)))
        return g

    def cadapdr(self, dens, precision="fp64"):
        return self.stokes_sum(dens, -1, precision)

    def cadapmod(self, dens, precision="fp64"):
        return self.stokes_sum(dens, +1, precision)

    def dapif2(self, z, q, precision="fp64"):
        """FIELD of DAPIF2 with IFLAG7 = 3: sum_{j != i} q_j / (z_i - z_j)."""
        if not _is_device(z):
            z = _host(z, np.complex128)
            q = _host(q, np.complex128)
        n = int(z.shape[0])
        f = self._out(z, n, np.complex128)
        check("eb_cauchy_sum", self._lib.eb_cauchy_sum(
            self._h, n, _ptr(z), _ptr(q), _ptr(f), PRECISION[precision], _mem(z, q, f)))
        return f

    def _solve(self, fn, n, rhs, mode, out):
        if not _is_device(rhs):
            rhs = _host(rhs, np.float64)
        x = out if out is not None else self._out(rhs, n, np.float64)
        info = SolveInfo()
        st = getattr(self._lib, fn)(self._h, n, _ptr(rhs), _ptr(x), SOLVE_MODE[mode],
                                    ctypes.byref(info), _mem(rhs, x))
        check(fn, st)
        return x, info.as_dict()

    def fasmvp_adjoint(self, x, precision="fp64", out=None):
        """The transpose of the Stokes operator: y = A^T x, x and y real of length 2 nbk."""
        if not _is_device(x):
            x = _host(x, np.float64)
        y = out if out is not None else self._out(x, 2 * self.nbk, np.float64)
        check("eb_stokes_matvec_adjoint", self._lib.eb_stokes_matvec_adjoint(
            self._h, 2 * self.nbk, _ptr(x), _ptr(y), PRECISION[precision], _mem(x, y)))
        return y

    def fasmvp_lap_adjoint(self, x, precision="fp64", out=None):
        """The transpose of the Laplace operator: y = A^T x, x and y real of length nbk."""
        if not _is_device(x):
            x = _host(x, np.float64)
        y = out if out is not None else self._out(x, self.nbk, np.float64)
        check("eb_laplace_matvec_adjoint", self._lib.eb_laplace_matvec_adjoint(
            self._h, self.nbk, _ptr(x), _ptr(y), PRECISION[precision], _mem(x, y)))
        return y

    def solvei_adjoint(self, rhs, mode="fp64", out=None):
        """GMRES on the transposed Stokes operator (A^T x = rhs). Returns (soln, info)."""
        return self._solve("eb_stokes_solve_adjoint", 2 * self.nbk, rhs, mode, out)

    def solve_lapl_adjoint(self, rhs, mode="fp64", out=None):
        """GMRES on the transposed Laplace operator. Returns (soln, info)."""
        return self._solve("eb_laplace_solve_adjoint", self.nbk, rhs, mode, out)

    def solvei(self, rhs, mode="fp64", out=None):
        """SOLVEI: GMRES on the Stokes operator, x0 = rhs. Returns (soln, info)."""
        return self._solve("eb_stokes_solve", 2 * self.nbk, rhs, mode, out)

    def solve_lapl(self, rhs, mode="fp64", out=None):
        """SOLVE_LAPL: GMRES on the Laplace operator, x0 = rhs. Returns (soln, info)."""
        return self._solve("eb_laplace_solve", self.nbk, rhs, mode, out)

    def fdifff(self, f):
        """FDIFFF per drop of the installed geometry (complex samples)."""
        f = _host(f, np.complex128)
        df = np.empty_like(f)
        check("eb_fdiff", self._lib.eb_fdiff(self._h, _ptr(f), _ptr(df), EB_HOST))
        return df

    def pvintev(self, ucmplx, precision="fp64"):
        u = _host(ucmplx, np.complex128)
        phi = np.empty_like(u)
        check("eb_pvintev", self._lib.eb_pvintev(self._h, _ptr(u), _ptr(phi),
                                                 PRECISION[precision], EB_HOST))
        return phi

    def dirich_neu_map(self, u, precision="fp64"):
        u = _host(u, np.float64)
        phi = np.empty(self.nbk)
        psi = np.empty(self.nbk)
        dphi = np.empty(self.nbk)
        check("eb_dirich_neu_map", self._lib.eb_dirich_neu_map(
            self._h, _ptr(u), _ptr(phi), _ptr(psi), _ptr(dphi), PRECISION[precision], EB_HOST))
        return phi, psi, dphi

    def interfacenew(self, u, zc, cap=0.0, precision="fp64"):
        """INTERFACENEW: (Un, FLUX) from the Stokes density u (complex)."""
        u = _host(u, np.complex128)
        zc = _host(zc, np.complex128)
        un = np.empty(self.nbk)
        flux = ctypes.c_double()
        check("eb_interface_velocity", self._lib.eb_interface_velocity(
            self._h, _ptr(u), _ptr(zc), float(cap), _ptr(un), ctypes.byref(flux),
            PRECISION[precision], EB_HOST))
        return un, flux.value

    def setvelf(self, dphi_dn, cap=0.0, e0=0.0, zbond=0.0, zc=None):
        """SETVELF: the Stokes right-hand side, 2 nbk reals. zbond != 0 needs the
        per-drop C_k zc; in wall mode (set_wall) the reflected log sources join in."""
        d = _host(dphi_dn, np.float64)
        rhs = np.empty(2 * self.nbk)
        if zbond == 0:
            check("eb_setvelf", self._lib.eb_setvelf(self._h, _ptr(d), float(cap), float(e0),
                                                     _ptr(rhs), EB_HOST))
            return rhs
        zb = np.array([np.real(zbond), np.imag(zbond)], np.float64)
        zc = _host(zc, np.complex128)
        check("eb_setvelf_bond", self._lib.eb_setvelf_bond(self._h, _ptr(d), float(cap), float(e0), _ptr(zb),
                                                           _ptr(zc), _ptr(rhs), EB_HOST))
        return rhs

    def set_wall(self, iwall=1):
        """Wall-bounded flow (the wall is y = 0): every Stokes sum adds the images."""
        check("eb_set_wall", self._lib.eb_set_wall(self._h, int(iwall)))

    def get_wall(self):
        """(iwall, xleft, slength) of the installed geometry."""
        w, xl, sl = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        check("eb_get_wall", self._lib.eb_get_wall(self._h, ctypes.byref(w), ctypes.byref(xl), ctypes.byref(sl)))
        return w.value, xl.value, sl.value

    # ---- RK stage ------------------------------------------------------------
    @staticmethod
    def _model(cap, e0, zbond, mode):
        m = Model()
        m.cap = float(cap)
        m.e0 = float(e0)
        m.zbond[0] = float(np.real(zbond))
        m.zbond[1] = float(np.imag(zbond))
        m.mode = SOLVE_MODE[mode]
        return m

    def _set_drops(self, nd):
        self.k = int(nd.shape[0])
        self.nbk = int(nd.sum())
        self.nd = nd

    def f(self, nd, rku, cap=0.0, e0=0.0, zbond=0.0, mode="fp64", out=None):
        """F: the node velocities rkup of the RK state rku (both interleaved x, y, length
        2 nbk). Returns (rkup, info); installs the geometry of rku."""
        nd = _host(nd, np.int32)
        if not _is_device(rku):
            rku = _host(rku, np.float64)
        rkup = out if out is not None else self._out(rku, 2 * int(nd.sum()), np.float64)
        info = StageInfo()
        m = self._model(cap, e0, zbond, mode)
        check("eb_rk_f", self._lib.eb_rk_f(self._h, int(nd.shape[0]), _ptr(nd), _ptr(rku),
                                           _ptr(rkup), ctypes.byref(m), ctypes.byref(info),
                                           _mem(rku, rkup)))
        self._set_drops(nd)
        return rkup, info.as_dict()

    def rk2(self, nd, dt, ybar, cap=0.0, e0=0.0, zbond=0.0, mode="fp64"):
        """RK2: one modified-Euler step of size dt; ybar (float64 numpy array or CUDA
        tensor, length 2 nbk) is updated in place. Returns the stage diagnostics."""
        nd = _host(nd, np.int32)
        if not _is_device(ybar):
            if not (isinstance(ybar, np.ndarray) and ybar.dtype == np.float64
                    and ybar.flags["C_CONTIGUOUS"]):
                raise TypeError("ybar must be a C-contiguous float64 array (updated in place)")
        info = StageInfo()
        m = self._model(cap, e0, zbond, mode)
        check("eb_rk2_step", self._lib.eb_rk2_step(self._h, int(nd.shape[0]), _ptr(nd),
                                                   float(dt), _ptr(ybar), ctypes.byref(m),
                                                   ctypes.byref(info), _mem(ybar)))
        self._set_drops(nd)
        return info.as_dict()

    # ---- reverse mode through the time stepper -------------------------------
    def f_vjp(self, nd, rku, v, cap=0.0, e0=0.0, mode="fp64"):
        """v^T dF/drku at the RK state rku (free space, one simulation): returns
        (rku_bar, {"e0": v^T dF/dE0, "cap": v^T dF/dcap}, info)."""
        nd = _host(nd, np.int32)
        if not _is_device(rku):
            rku = _host(rku, np.float64)
            v = _host(v, np.float64)
        out = self._out(rku, 2 * int(nd.sum()), np.float64)
        pb = np.zeros(2)
        info = AdjointInfo()
        m = self._model(cap, e0, 0.0, mode)
        check("eb_rk_f_vjp", self._lib.eb_rk_f_vjp(self._h, int(nd.shape[0]), _ptr(nd), _ptr(rku),
                                                   _ptr(v), ctypes.byref(m), _ptr(out), _ptr(pb),
                                                   ctypes.byref(info), _mem(rku, v, out)))
        self._set_drops(nd)
        return out, {"e0": float(pb[0]), "cap": float(pb[1])}, info.as_dict()

    def rk2_vjp(self, nd, dt, ybar, rbar, cap=0.0, e0=0.0, mode="fp64"):
        """The transpose of one RK2 step from the state ybar: rbar (dJ/dy after the step,
        float64, updated in place to dJ/dy before it). Returns ({"e0", "cap"} parts, info)."""
        nd = _host(nd, np.int32)
        if not _is_device(ybar):
            ybar = _host(ybar, np.float64)
            if not (isinstance(rbar, np.ndarray) and rbar.dtype == np.float64
                    and rbar.flags["C_CONTIGUOUS"]):
                raise TypeError("rbar must be a C-contiguous float64 array (updated in place)")
        pb = np.zeros(2)
        info = AdjointInfo()
        m = self._model(cap, e0, 0.0, mode)
        check("eb_rk2_step_vjp", self._lib.eb_rk2_step_vjp(self._h, int(nd.shape[0]), _ptr(nd), float(dt),
                                                           _ptr(ybar), _ptr(rbar), ctypes.byref(m),
                                                           _ptr(pb), ctypes.byref(info), _mem(ybar, rbar)))
        self._set_drops(nd)
        return {"e0": float(pb[0]), "cap": float(pb[1])}, info.as_dict()

    def deformation(self, nd, rku, grad=True):
        """The summed Taylor deformation (L - B)/(L + B) of the drops of rku, and its
        gradient with respect to rku (None when grad is False)."""
        nd = _host(nd, np.int32)
        if not _is_device(rku):
            rku = _host(rku, np.float64)
        g = self._out(rku, 2 * int(nd.sum()), np.float64) if grad else None
        val = ctypes.c_double(0.0)
        check("eb_deformation", self._lib.eb_deformation(self._h, int(nd.shape[0]), _ptr(nd), _ptr(rku),
                                                         ctypes.byref(val), _ptr(g) if grad else None,
                                                         _mem(rku)))
        return float(val.value), g

    def rk2_gradient(self, nd, dt, y0, steps, cap=0.0, e0=0.0, mode="fp64"):
        """J = the deformation after `steps` RK2 steps from y0, and dJ/dy0, dJ/dE0 and
        dJ/dcap by reverse mode (eb_rk2_gradient: one checkpoint, the state, per step on
        the device; the reverse pass recomputes each step's stages from its checkpoint)."""
        nd = _host(nd, np.int32)
        if not _is_device(y0):
            y0 = _host(y0, np.float64)
        g = self._out(y0, 2 * int(nd.sum()), np.float64)
        pb = np.zeros(2)
        val = ctypes.c_double(0.0)
        info = AdjointInfo()
        m = self._model(cap, e0, 0.0, mode)
        check("eb_rk2_gradient", self._lib.eb_rk2_gradient(self._h, int(nd.shape[0]), _ptr(nd), float(dt),
                                                           int(steps), _ptr(y0), ctypes.byref(m),
                                                           ctypes.byref(val), _ptr(g), _ptr(pb),
                                                           ctypes.byref(info), _mem(y0, g)))
        self._set_drops(nd)
        return {"J": float(val.value), "y0": g, "e0": float(pb[0]), "cap": float(pb[1]), "info": info.as_dict()}

def geometry_from_extract(ctx, cfg):
    """Install cfg's geometry by EXTRACTDAT on the GPU; returns the geometry dict."""
    return ctx.extractdat(cfg.nd, cfg.rku())


__all__ = ["Context", "EbError", "geometry_from_extract", "PRECISION", "SOLVE_MODE"]
