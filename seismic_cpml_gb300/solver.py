"""Python host mirror of the C ABI: one ``Solver`` per simulation handle.

Mirrors the flow of the reference programs (set-up 2D:283-544 /
3D:399-756, time loop 2D:550-735 / 3D:802-1245, outputs 2D:738-808):
  s = Solver(params, receivers, model=(lam, mu, rho))
  s.run()                      # NSTEP steps, blow-up check at display steps
  vx, vy, vz = s.seismograms() # [nrec, nstep] float64
  ek, ep = s.energy()
Every call goes through libcpml.so; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import lib as _L
from .params import CpmlParams, FIELDS

_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


class Solver:
    def __init__(self, params: CpmlParams, receivers=(), model=None, tuning=None):
        self.L = _L.load()
        self.p = params.copy()
        h = ctypes.c_void_p()
        _L.check(self.L.cpml_create(ctypes.byref(self.p), ctypes.byref(h)), "cpml_create")
        self.h = h
        self.shape = (self.p.nz, self.p.ny, self.p.nx) if self.p.ndim == 3 else (self.p.ny, self.p.nx)
        if tuning is not None:
            self.set_tuning(*tuning)
        if model is not None:
            self.set_model(*model)
        self.receivers = []
        if receivers:
            self.set_receivers(receivers)

    # -- set-up ----------------------------------------------------------
    def set_model(self, lam=None, mu=None, rho=None):
        arrs = [_f32(a) for a in (lam, mu, rho)]
        for a in arrs:
            if a is not None and a.size != int(np.prod(self.shape)):
                raise ValueError("model arrays must have nx*ny(*nz) values")
        ptr = [None if a is None else a.ctypes.data_as(_fp) for a in arrs]
        _L.check(self.L.cpml_set_model(self.h, *ptr), "cpml_set_model")

    def set_receivers(self, receivers):
        rec = [tuple(int(v) for v in r) for r in receivers]
        n = len(rec)
        ix = np.array([r[0] for r in rec], np.int32)
        iy = np.array([r[1] for r in rec], np.int32)
        iz = np.array([(r[2] if len(r) > 2 else self.p.ksource) for r in rec], np.int32)
        _L.check(self.L.cpml_set_receivers(self.h, n, ix.ctypes.data_as(_ip), iy.ctypes.data_as(_ip),
                                           iz.ctypes.data_as(_ip)), "cpml_set_receivers")
        self.receivers = rec

    def set_tuning(self, kernel: int = 0, tile_y: int = 8, zchunk: int = 24, lookahead: int = 2) -> None:
        """Step kernel (0 auto, 1 two-sweep, 2 fused 3D, 3 persistent 2D, 4 on-chip 2D
        cluster) and launch shape (lookahead: the fused kernel's TMA look-ahead, 2)."""
        _L.check(self.L.cpml_set_tuning(self.h, int(kernel), int(tile_y), int(zchunk), int(lookahead)),
                 "set_tuning")

    def launches_per_step(self):
        """(kernels per time step, kernels per chunk of steps)."""
        a, b = ctypes.c_int(), ctypes.c_int()
        _L.check(self.L.cpml_launches_per_step(self.h, ctypes.byref(a), ctypes.byref(b)), "cpml_launches_per_step")
        return a.value, b.value

    def tuning(self):
        k, t, z, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _L.check(self.L.cpml_get_tuning(self.h, ctypes.byref(k), ctypes.byref(t), ctypes.byref(z),
                                        ctypes.byref(d)))
        return k.value, t.value, z.value, d.value

    def autotune(self, trial_steps: int = 20, cache_path: str | None = None):
        """Time the candidate launch shapes and keep the fastest (cpml_autotune)."""
        k, t, z = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = ctypes.c_double()
        _L.check(self.L.cpml_autotune(self.h, int(trial_steps),
                                      cache_path.encode() if cache_path else None, ctypes.byref(k),
                                      ctypes.byref(t), ctypes.byref(z), ctypes.byref(ms)), "autotune")
        return {"kernel": k.value, "tile_y": t.value, "zchunk": z.value, "ms_per_step": ms.value}

    # -- time loop -------------------------------------------------------
    def run(self, nsteps: int | None = None) -> None:
        it, _ = self.status()
        n = self.p.nstep - it if nsteps is None else nsteps
        _L.check(self.L.cpml_run(self.h, int(n)), "cpml_run")

    def reset(self) -> None:
        _L.check(self.L.cpml_reset(self.h), "cpml_reset")

    def status(self):
        it = ctypes.c_int()
        vm = ctypes.c_double()
        _L.check(self.L.cpml_status(self.h, ctypes.byref(it), ctypes.byref(vm)))
        return it.value, vm.value

    def last_run_ms(self) -> float:
        v = ctypes.c_double()
        _L.check(self.L.cpml_last_run_ms(self.h, ctypes.byref(v)))
        return v.value

    def stream_ptr(self) -> int:
        """The handle's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = ctypes.c_void_p()
        _L.check(self.L.cpml_get_stream(self.h, ctypes.byref(p)))
        return int(p.value or 0)

    def algorithmic_bytes_per_step(self) -> float:
        return float(self.L.cpml_algorithmic_bytes_per_step(self.h))

    # -- results ---------------------------------------------------------
    def seismograms(self):
        n = max(len(self.receivers), 1)
        out = [np.zeros((n, self.p.nstep)) for _ in range(3)]
        vz = out[2].ctypes.data_as(_dp) if self.p.ndim == 3 else None
        _L.check(self.L.cpml_get_seismograms(self.h, out[0].ctypes.data_as(_dp),
                                             out[1].ctypes.data_as(_dp), vz))
        k = len(self.receivers)
        return out[0][:k], out[1][:k], (out[2][:k] if self.p.ndim == 3 else None)

    def energy(self):
        ek = np.zeros(self.p.nstep)
        ep = np.zeros(self.p.nstep)
        _L.check(self.L.cpml_get_energy(self.h, ek.ctypes.data_as(_dp), ep.ctypes.data_as(_dp)))
        return ek, ep

    def field(self, name: str) -> np.ndarray:
        out = np.zeros(self.shape, np.float32)
        _L.check(self.L.cpml_get_field(self.h, FIELDS[name], out.ctypes.data_as(_fp)), "get_field")
        return out

    def set_field(self, name: str, arr) -> None:
        a = _f32(arr).reshape(self.shape)
        _L.check(self.L.cpml_set_field(self.h, FIELDS[name], a.ctypes.data_as(_fp)), "set_field")

    # -- checkpoint / restart ---------------------------------------------
    def save_state(self) -> np.ndarray:
        """Snapshot of the time loop's state (cpml_save_state) as a uint8 array."""
        n = ctypes.c_size_t()
        _L.check(self.L.cpml_state_size(self.h, ctypes.byref(n)), "cpml_state_size")
        buf = np.zeros(n.value, np.uint8)
        _L.check(self.L.cpml_save_state(self.h, buf.ctypes.data_as(ctypes.c_void_p), n.value),
                 "cpml_save_state")
        return buf

    def load_state(self, buf) -> None:
        """Restore a snapshot made by save_state on a handle of the same
        parameters, model and receivers (cpml_load_state)."""
        b = np.ascontiguousarray(buf, dtype=np.uint8)
        _L.check(self.L.cpml_load_state(self.h, b.ctypes.data_as(ctypes.c_void_p), b.size),
                 "cpml_load_state")

    def plane(self, name: str, axis: int, index: int) -> np.ndarray:
        dims = list(self.shape) if self.p.ndim == 3 else [1] + list(self.shape)
        nz, ny, nx = dims
        shp = {2: (ny, nx), 1: (nz, nx), 0: (nz, ny)}[axis]
        out = np.zeros(shp, np.float32)
        _L.check(self.L.cpml_get_plane(self.h, FIELDS[name], axis, index, out.ctypes.data_as(_fp)),
                 "get_plane")
        return out

    # -- reference output files -------------------------------------------
    def write_outputs(self, directory: str = ".") -> None:
        os.makedirs(directory, exist_ok=True)
        vx, vy, vz = self.seismograms()
        it, _ = self.status()
        d = directory.encode()
        if len(self.receivers):
            vx = np.ascontiguousarray(vx[:, :it]); vy = np.ascontiguousarray(vy[:, :it])
            vzp = None
            if vz is not None:
                vz = np.ascontiguousarray(vz[:, :it]); vzp = vz.ctypes.data_as(_dp)
            _L.check(self.L.cpml_write_seismograms(d, vx.ctypes.data_as(_dp), vy.ctypes.data_as(_dp),
                                                   vzp, it, len(self.receivers), self.p.deltat))
        ek, ep = self.energy()
        ek = np.ascontiguousarray(ek[:it]); ep = np.ascontiguousarray(ep[:it])
        _L.check(self.L.cpml_write_energy(d, ek.ctypes.data_as(_dp), ep.ctypes.data_as(_dp), it,
                                          self.p.deltat, 4 if self.p.ndim == 2 else 2))

    def write_snapshot(self, directory: str = ".") -> None:
        """imageNNNNNN_Vx/Vy.pnm of the current step (2D:729-732; 3D on plane
        k = ksource, 3D:1236-1239)."""
        it, _ = self.status()
        ix = np.array([r[0] for r in self.receivers] or [0], np.int32)
        iy = np.array([r[1] for r in self.receivers] or [0], np.int32)
        use = np.array(list(self.p.use_pml)[:4], np.int32)
        for fn, name in ((1, "vx"), (2, "vy")):
            pl = self.plane(name, 2, self.p.ksource if self.p.ndim == 3 else 1)
            pl = np.ascontiguousarray(pl)
            _L.check(self.L.cpml_write_pnm(directory.encode(), pl.ctypes.data_as(_fp), self.p.nx,
                                           self.p.ny, it, self.p.isource, self.p.jsource,
                                           ix.ctypes.data_as(_ip), iy.ctypes.data_as(_ip),
                                           len(self.receivers), self.p.npoints_pml,
                                           use.ctypes.data_as(_ip), fn))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.cpml_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
