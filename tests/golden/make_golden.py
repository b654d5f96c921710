"""Generate the golden fixtures of tests/golden/ with the FP64 C++ oracle.

These fixtures are outputs of the oracle restatement (oracle/cpml_oracle.cpp).
At generation time they are cross-checked against the independent numpy
restatement (oracle/oracle_np.py) on every case small enough to run it. They
pin the oracle against regressions and give the GPU tests FP64 answers at the
reference's own sizes. The reference ships no tests, golden vectors or
known-answer files. Its own outputs, from its Fortran statements translated
by oracle/ref_f90c.py, are the refpin_*.npz fixtures of
make_ref_vectors.py. tests/test_ref_pin.py checks that those equal the
fixtures made here (ref2d_*, config_3d_plain) bit for bit, in traces and
2D energies.

Run:  python tests/golden/make_golden.py [name ...]   (no name: every fixture)

config_3d_plain is the 3D plain workload at its full size (276^3, 2500 time
steps, 64 receivers): about 5 minutes on 8 cores. Its traces and energies
are what the GPU run of the benchmarked kernels is compared with.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle_c, oracle_np  # noqa: E402
from seismic_cpml_gb300 import params as P  # noqa: E402
from tests.models import layered_2d, layered_3d  # noqa: E402


def save(name, p, rec, res, model=None):
    d = dict(sisvx=res.sisvx, sisvy=res.sisvy, ek=res.ek, ep=res.ep,
             rec=np.array(rec, np.int32))
    if res.sisvz is not None:
        d["sisvz"] = res.sisvz
    if res.vmax is not None:
        d["vmax"] = res.vmax
    if model is not None:
        d["lam"], d["mu"], d["rho"] = [np.asarray(m, np.float32) for m in model]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print("wrote", name, {k: v.shape for k, v in d.items()})


def cross_check(p, rec, res, model=None):
    kw = {}
    if model is not None:
        kw = dict(lam=model[0], mu=model[1], rho=model[2])
    run = oracle_np.run2d if p.ndim == 2 else oracle_np.run3d
    if p.ndim == 2 and p.order == 4:
        run = oracle_np.run2d4
    if p.ndim == 2 and p.scheme == P.SCHEME_SPLIT:
        run = oracle_np.run_split
    rn = run(p, rec=rec, **kw)
    for a, b in ((res.sisvx, rn.sisvx), (res.sisvy, rn.sisvy)):
        assert np.array_equal(a, b), "C++ and numpy restatements disagree"
    e = np.abs((res.ek + res.ep) - (rn.ek + rn.ep)).max() / np.abs(rn.ek + rn.ep).max()
    assert e < 1e-12, e


def make_ref2d_default():
    # the 2D program exactly as shipped (2D:138-218)
    p = P.default_2d()
    rec = P.reference_receivers_2d(p)
    res = oracle_c.run(p, rec=rec, vmax=True)
    cross_check(p, rec, res)
    save("ref2d_default", p, rec, res)


def make_config_2d_plain():
    # 2D plain benchmark workload (Ricker at the centre, PML off on top)
    p, rec = P.config_2d_plain()
    res = oracle_c.run(p, rec=rec, vmax=True)
    save("config_2d_plain", p, rec, res)


def make_small2d_het():
    # small heterogeneous 2D (model stored in the fixture, float32 values)
    p, rec = P.small_2d()
    model = layered_2d(p, seed=7)
    res = oracle_c.run(p, rec=rec, lam=model[0], mu=model[1], rho=model[2], vmax=True)
    cross_check(p, rec, res, model)
    save("small2d_het", p, rec, res, model)


def make_small3d_hom():
    # 3D program at a reduced size (homogeneous, reference wavelet and angle)
    p, rec = P.small_3d()
    res = oracle_c.run(p, rec=rec, vmax=True)
    cross_check(p, rec, res)
    save("small3d_hom", p, rec, res)


def make_small3d_het():
    # small heterogeneous 3D, per-cell extension
    p, rec = P.small_3d()
    model = layered_3d(p, seed=11)
    res = oracle_c.run(p, rec=rec, lam=model[0], mu=model[1], rho=model[2], vmax=True)
    cross_check(p, rec, res, model)
    save("small3d_het", p, rec, res, model)


def make_config_3d_plain():
    # the 3D plain benchmark workload at full size: 276^3, 2500 steps, 64
    # receivers on the x line through the centre (too large for the numpy
    # restatement; the C++ oracle is cross-checked against it on the small cases)
    p, rec = P.config_3d_plain()
    res = oracle_c.run(p, rec=rec)
    save("config_3d_plain", p, rec, res)


def make_ref2d_fourth():
    # the fourth-order program as shipped (2D4:132-190): 101 x 641, 4000 steps of 1 ms
    p = P.default_2d_fourth()
    rec = P.reference_receivers_2d(p)
    res = oracle_c.run(p, rec=rec, vmax=True)
    cross_check(p, rec, res)
    save("ref2d_fourth", p, rec, res)


def make_ref2d_split():
    # the classical split-field PML program as shipped (PML:96-141)
    p = P.default_2d_split()
    rec = P.reference_receivers_2d(p)
    res = oracle_c.run(p, rec=rec, vmax=True)
    cross_check(p, rec, res)
    save("ref2d_split", p, rec, res)


MAKERS = {"ref2d_default": make_ref2d_default, "config_2d_plain": make_config_2d_plain,
          "small2d_het": make_small2d_het, "small3d_hom": make_small3d_hom,
          "small3d_het": make_small3d_het, "config_3d_plain": make_config_3d_plain,
          "ref2d_fourth": make_ref2d_fourth, "ref2d_split": make_ref2d_split}


def main(names):
    for n in names or MAKERS:
        MAKERS[n]()


if __name__ == "__main__":
    main(sys.argv[1:])
