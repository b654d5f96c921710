"""Python mirror of the batched multi-shot 2D engine (cpml_batch_* in
include/cpml.h): many independent 2D shots in one persistent launch."""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib as _L
from .params import CpmlParams, FIELDS

_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Batch:
    def __init__(self, params, models=None, receivers=None):
        self.L = _L.load()
        self.params = [p.copy() for p in params]
        arr = (CpmlParams * len(self.params))(*self.params)
        h = ctypes.c_void_p()
        _L.check(self.L.cpml_batch_create(len(self.params), arr, ctypes.byref(h)), "cpml_batch_create")
        self.h = h
        self.receivers = [[] for _ in self.params]
        if models is not None:
            for s, m in enumerate(models):
                if m is not None:
                    self.set_model(s, *m)
        if receivers is not None:
            for s, r in enumerate(receivers):
                self.set_receivers(s, r)

    def set_model(self, shot, lam, mu, rho):
        a = [np.ascontiguousarray(x, dtype=np.float32) for x in (lam, mu, rho)]
        _L.check(self.L.cpml_batch_set_model(self.h, shot, *[x.ctypes.data_as(_fp) for x in a]),
                 "cpml_batch_set_model")

    def set_receivers(self, shot, rec):
        rec = [tuple(int(v) for v in r) for r in rec]
        ix = np.array([r[0] for r in rec] or [0], np.int32)
        iy = np.array([r[1] for r in rec] or [0], np.int32)
        _L.check(self.L.cpml_batch_set_receivers(self.h, shot, len(rec), ix.ctypes.data_as(_ip),
                                                 iy.ctypes.data_as(_ip)), "cpml_batch_set_receivers")
        self.receivers[shot] = rec

    def run(self) -> None:
        _L.check(self.L.cpml_batch_run(self.h), "cpml_batch_run")

    def set_wait_limit(self, cycles: int) -> None:
        """Bound of one grid-barrier wait in SM cycles (0 = default)."""
        _L.check(self.L.cpml_batch_set_wait_limit(self.h, int(cycles)), "cpml_batch_set_wait_limit")

    def set_tuning(self, depth: int = 1, tile_y: int = 8) -> None:
        """Time steps per shared-memory pass (temporal blocking) and tile rows
        (cpml_batch_set_tuning): (1, 8), (2, 8), (2, 16) or (3, 16)."""
        _L.check(self.L.cpml_batch_set_tuning(self.h, int(depth), int(tile_y)), "cpml_batch_set_tuning")

    def tuning(self):
        d, t = ctypes.c_int(), ctypes.c_int()
        _L.check(self.L.cpml_batch_get_tuning(self.h, ctypes.byref(d), ctypes.byref(t)))
        return d.value, t.value

    def autotune(self, trial_steps: int = 100):
        """Time every (depth, tile_y) on the first trial_steps steps and keep
        the fastest (cpml_batch_autotune)."""
        d, t, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _L.check(self.L.cpml_batch_autotune(self.h, int(trial_steps), ctypes.byref(d), ctypes.byref(t),
                                            ctypes.byref(ms)), "cpml_batch_autotune")
        return {"depth": d.value, "tile_y": t.value, "ms_per_step": ms.value}

    def last_run_ms(self) -> float:
        v = ctypes.c_double()
        _L.check(self.L.cpml_batch_last_run_ms(self.h, ctypes.byref(v)))
        return v.value

    def seismograms(self, shot):
        n = len(self.receivers[shot])
        ns = self.params[shot].nstep
        vx = np.zeros((max(n, 1), ns))
        vy = np.zeros((max(n, 1), ns))
        _L.check(self.L.cpml_batch_get_seismograms(self.h, shot, vx.ctypes.data_as(_dp),
                                                   vy.ctypes.data_as(_dp)))
        return vx[:n], vy[:n]

    def field(self, shot, name):
        p = self.params[shot]
        out = np.zeros((p.ny, p.nx), np.float32)
        _L.check(self.L.cpml_batch_get_field(self.h, shot, FIELDS[name], out.ctypes.data_as(_fp)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.cpml_batch_destroy(self.h)
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


def _main(argv=None):
    """Run a seeded batch (the batched workload's shot generator at a reduced
    size) a few times and print each run's device time and rate."""
    import argparse
    from .workloads import batch2d_shots
    ap = argparse.ArgumentParser(prog="python -m seismic_cpml_gb300.batch")
    ap.add_argument("--shots", type=int, default=32)
    ap.add_argument("--interior", type=int, nargs=2, default=(400, 600), help="interior cells per side, range")
    ap.add_argument("--record-s", type=float, default=0.1, help="simulated seconds per shot")
    ap.add_argument("--runs", type=int, default=2)
    ap.add_argument("--tuning", type=str, default=None, help="depth,tile_y (default: autotune)")
    a = ap.parse_args(argv)
    shots = batch2d_shots(nshots=a.shots, interior=tuple(a.interior), record_s=a.record_s)
    cells = sum(p.nx * p.ny * p.nstep for p, _, _ in shots)
    with Batch([p for p, _, _ in shots], models=[m for _, m, _ in shots], receivers=[r for _, _, r in shots]) as b:
        if a.tuning:
            b.set_tuning(*(int(x) for x in a.tuning.split(",")))
        else:
            print("autotune:", b.autotune())
        for r in range(a.runs):
            b.run()
            ms = b.last_run_ms()
            print(f"run {r}: {a.shots} shots, {cells:.3e} cell-updates, {ms:.2f} ms, "
                  f"{cells / ms / 1e6:.1f} Gcell-updates/s")


if __name__ == "__main__":
    _main()
