"""ctypes loader for the C++ oracle (oracle/cpml_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests, the smoke check and the CPU-baseline
leg of the benchmark as the checker / timed CPU implementation of the
reference programs. The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    if force or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "cpml_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.oracle_run.restype = ctypes.c_int
        L.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                 ctypes.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
                                 _dp, ctypes.c_int]
        L.oracle_profile.restype = ctypes.c_int
        L.oracle_profile.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, _dp]
        L.oracle_source_term.restype = ctypes.c_double
        L.oracle_source_term.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_session_create.restype = ctypes.c_void_p
        L.oracle_session_create.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int]
        L.oracle_session_run.restype = ctypes.c_int
        L.oracle_session_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.oracle_session_destroy.restype = None
        L.oracle_session_destroy.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _ptr(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


@dataclass
class Result:
    sisvx: np.ndarray
    sisvy: np.ndarray
    sisvz: np.ndarray | None
    ek: np.ndarray
    ep: np.ndarray
    vmax: np.ndarray | None = None
    fields: dict = field(default_factory=dict)


def run(p, nsteps=None, rec=(), lam=None, mu=None, rho=None, double=True,
        keep_fields=False, vmax=False, energy=True, nthreads=0) -> Result:
    """Run the C++ restatement. ``p`` is a ``CpmlParams``; rec holds 1-based
    (ix, iy[, iz]) tuples."""
    L = lib()
    nsteps = p.nstep if nsteps is None else nsteps
    nrec = len(rec)
    ix = np.array([r[0] for r in rec] or [0], np.int32)
    iy = np.array([r[1] for r in rec] or [0], np.int32)
    iz = np.array([(r[2] if len(r) > 2 else 1) for r in rec] or [0], np.int32)
    sx = np.zeros((max(nrec, 1), nsteps)); sy = np.zeros_like(sx); sz = np.zeros_like(sx)
    ek = np.zeros(nsteps) if energy else None
    ep = np.zeros(nsteps) if energy else None
    vm = np.zeros(nsteps) if vmax else None
    ncell = p.nx * p.ny * (p.nz if p.ndim == 3 else 1)
    nf = 9 if p.ndim == 3 else 5
    fo = np.zeros((nf, ncell)) if keep_fields else None
    cv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()
    lam, mu, rho = cv(lam), cv(mu), cv(rho)
    st = L.oracle_run(ctypes.byref(p), nsteps, 1 if double else 0, _ptr(lam), _ptr(mu), _ptr(rho),
                      nrec, _ptr(ix, _ip), _ptr(iy, _ip), _ptr(iz, _ip), _ptr(sx), _ptr(sy),
                      _ptr(sz) if p.ndim == 3 else None, _ptr(ek), _ptr(ep), _ptr(vm), _ptr(fo),
                      int(nthreads))
    if st != 0:
        raise RuntimeError(f"oracle_run failed: {st}")
    res = Result(sx[:nrec], sy[:nrec], sz[:nrec] if p.ndim == 3 else None, ek, ep, vm)
    if keep_fields:
        names = ["vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz"] if p.ndim == 3 \
            else ["vx", "vy", "sxx", "syy", "sxy"]
        shp = (p.nz, p.ny, p.nx) if p.ndim == 3 else (p.ny, p.nx)
        res.fields = {n: fo[q].reshape(shp) for q, n in enumerate(names)}
    return res


def profile(p, axis):
    """FP64 C-PML profile of one axis: dict like oracle_np.pml_profile."""
    n = [p.nx, p.ny, p.nz][axis]
    delta = [p.deltax, p.deltay, p.deltaz][axis]
    out = np.zeros((10, n))
    lib().oracle_profile(ctypes.byref(p), axis, n, delta, _ptr(out))
    keys = ["d", "K", "alpha", "a", "b", "d_half", "K_half", "alpha_half", "a_half", "b_half"]
    return {k: out[q] for q, k in enumerate(keys)}


def source_term(p, it):
    return lib().oracle_source_term(ctypes.byref(p), it)


def max_threads():
    return lib().oracle_max_threads()


class Session:
    """The restated time loop kept alive between calls, so its set-up
    (allocation and zeroing of every array) is outside a timed region."""

    def __init__(self, p, nthreads=0, lam=None, mu=None, rho=None):
        self.p = p.copy()
        cv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel()
        self._m = [cv(lam), cv(mu), cv(rho)]
        self.h = lib().oracle_session_create(ctypes.byref(self.p), *[_ptr(a) for a in self._m],
                                             int(nthreads))
        if not self.h:
            raise RuntimeError("oracle_session_create failed")

    def run(self, nsteps):
        return lib().oracle_session_run(self.h, int(nsteps))

    def close(self):
        if self.h:
            lib().oracle_session_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
