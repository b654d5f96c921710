"""Seeded heterogeneous models for the parity tests (float32 values, so the
GPU path and the FP64 oracle see identical inputs)."""
from seismic_cpml_gb300.earth import layered_model


def layered_2d(p, seed):
    (lam, mu, rho), cpmax = layered_model((p.ny, p.nx), 4, 2400.0, 3200.0, seed, anomalies=2,
                                          amp=0.05, radius=(3, 6))
    assert cpmax <= p.cp
    return lam, mu, rho


def layered_3d(p, seed):
    (lam, mu, rho), cpmax = layered_model((p.nz, p.ny, p.nx), 3, 2400.0, 3200.0, seed,
                                          anomalies=2, amp=0.05, radius=(2, 4))
    assert cpmax <= p.cp
    return lam, mu, rho
