"""The reference's input deck (`bubbin`) and checkpoint (`geometry.data`) files, through
the host-side C ABI of libeb_gb300.so (no GPU needed):

    read_bubbin     READINI (electric.f:275-337): the first deck of the file
    geoinit         GEOINIT / INITPARAM (electric.f:340-496): initial curves
    dumpdata        DUMPDATA (electric.f:1360-1384): write geometry.data
    readdata        READDATA (electric.f:1389-1421): read geometry.data
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def read_bubbin(path, kmax=4096):
    """Returns a dict: k, nd, dt, tfinal, nplot, cap, zbond, E0 and per drop ai, bi,
    thetax, zk, ncyc."""
    lib = _lib.load()
    k = ctypes.c_int()
    nd = np.zeros(kmax, np.int32)
    params = np.zeros(7)
    drops = np.zeros(6 * kmax)
    check("eb_bubbin_read", lib.eb_bubbin_read(str(path).encode(), kmax, ctypes.byref(k), _p(nd),
                                               _p(params), _p(drops)))
    k = k.value
    d = drops[:6 * k].reshape(k, 6)
    return {"k": k, "nd": nd[:k].copy(), "dt": params[0], "tfinal": params[1],
            "nplot": int(round(params[2])), "cap": params[3], "zbond": complex(params[4], params[5]),
            "E0": params[6], "ai": d[:, 0].copy(), "bi": d[:, 1].copy(), "thetax": d[:, 2].copy(),
            "zk": d[:, 3] + 1j * d[:, 4], "ncyc": np.rint(d[:, 5]).astype(np.int32)}


def geoinit(deck):
    """Initial curves of the deck at equispaced theta: (z, dsdth, kappa, area0)."""
    lib = _lib.load()
    nd = np.ascontiguousarray(deck["nd"], np.int32)
    k = int(nd.shape[0])
    drops = np.ascontiguousarray(np.stack([deck["ai"], deck["bi"], deck["thetax"], np.real(deck["zk"]),
                                           np.imag(deck["zk"]), deck["ncyc"]], axis=1), np.float64)
    nbk = int(nd.sum())
    z = np.zeros(nbk, np.complex128)
    dsdth = np.zeros(nbk)
    kappa = np.zeros(nbk)
    area0 = np.zeros(k)
    check("eb_geoinit", lib.eb_geoinit(k, _p(nd), _p(drops), _p(z), _p(dsdth), _p(kappa), _p(area0)))
    return z, dsdth, kappa, area0


def dumpdata(path, nd, dt, time, area0, arcl0, z):
    lib = _lib.load()
    nd = np.ascontiguousarray(nd, np.int32)
    area0 = np.ascontiguousarray(area0, np.float64)
    arcl0 = np.ascontiguousarray(arcl0, np.float64)
    z = np.ascontiguousarray(z, np.complex128)
    check("eb_dumpdata", lib.eb_dumpdata(str(path).encode(), int(nd.shape[0]), _p(nd), float(dt),
                                         float(time), _p(area0), _p(arcl0), _p(z)))


def readdata(path, kmax=4096, nmax=1 << 24):
    """Returns (nd, dt, time, area0, arcl0, z)."""
    lib = _lib.load()
    k = ctypes.c_int()
    nd = np.zeros(kmax, np.int32)
    dt, time = ctypes.c_double(), ctypes.c_double()
    area0 = np.zeros(kmax)
    arcl0 = np.zeros(kmax)
    z = np.zeros(nmax, np.complex128)
    check("eb_readdata", lib.eb_readdata(str(path).encode(), kmax, nmax, ctypes.byref(k), _p(nd),
                                         ctypes.byref(dt), ctypes.byref(time), _p(area0), _p(arcl0),
                                         _p(z)))
    k = k.value
    nbk = int(nd[:k].sum())
    return nd[:k].copy(), dt.value, time.value, area0[:k].copy(), arcl0[:k].copy(), z[:nbk].copy()
