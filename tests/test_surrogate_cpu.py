"""CPU checks of the surrogate's FP64 oracle (finite differences), of the
im2col/col2im adjoint pair, of the cosine basis, and of the seeded shot
generator. No GPU work."""
import math

import numpy as np
import pytest

from oracle import surrogate_np as S
from seismic_cpml_gb300.surrogate import NetConfig, ShotSpec, dct_basis, encode_input, make_shot, source_slot

TINY = NetConfig(h=16, w=24, cin=3, chans=(3, 4, 5, 4, 3), latent=6, nrec=3, nt=20, modes=5, head_weight=0.3)


def tiny_params(cfg, seed=0):
    rng = np.random.default_rng(seed)
    return {n: rng.standard_normal(s) * (0.5 if n.endswith("_w") else 0.1) for n, s in cfg.param_shapes()}


def tiny_batch(cfg, B=3, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, cfg.h, cfg.w, cfg.cin))
    t = rng.standard_normal((B, cfg.nrec * cfg.nt))
    slot = rng.integers(0, cfg.nrec, B)
    return x, slot, t


def test_im2col_col2im_are_adjoint():
    rng = np.random.default_rng(3)
    for shape in [(2, 8, 8, 3), (1, 7, 5, 2), (3, 2, 2, 1)]:
        x = rng.standard_normal(shape)
        col, _ = S.im2col(x)
        y = rng.standard_normal(col.shape)
        assert abs(np.sum(col * y) - np.sum(x * S.col2im(y, shape))) < 1e-10 * (1 + abs(np.sum(col * y)))


def test_im2col_layout():
    x = np.arange(2 * 4 * 4 * 3, dtype=np.float64).reshape(2, 4, 4, 3)
    col, (Ho, Wo) = S.im2col(x)
    assert (Ho, Wo) == (2, 2) and col.shape == (8, 27)
    b, y, xo, ky, kx, c = 1, 1, 0, 2, 1, 2          # row (b, y, x), column (ky*3 + kx)*C + c
    iy, ix = 2 * y + ky - 1, 2 * xo + kx - 1
    assert col[(b * Ho + y) * Wo + xo, (ky * 3 + kx) * 3 + c] == x[b, iy, ix, c]
    assert col[0, 0] == 0.0                          # top-left tap of the first patch is padding


def test_oracle_gradients_match_finite_differences():
    cfg = TINY
    params = tiny_params(cfg)
    x, slot, t = tiny_batch(cfg)
    basis = dct_basis(cfg.modes, cfg.nt)
    loss, head, g = S.loss_and_grads(params, x, slot, t, basis, cfg.nrec, cfg.modes, cfg.head_weight)
    rng = np.random.default_rng(5)
    h = 1e-6
    for name, shp in cfg.param_shapes():
        for _ in range(3):
            idx = tuple(int(rng.integers(0, s)) for s in shp)
            p2 = {k: v.copy() for k, v in params.items()}
            if name.startswith("head"):
                def obj(pp):
                    _, hd, _ = S.total_loss(pp, x, slot, t, basis, cfg.nrec, cfg.modes, cfg.head_weight)
                    return cfg.head_weight * np.mean((hd - np.log(loss)) ** 2)
            else:
                def obj(pp):
                    return S.total_loss(pp, x, slot, t, basis, cfg.nrec, cfg.modes, cfg.head_weight)[0]
            p2[name][idx] += h
            fp = obj(p2)
            p2[name][idx] -= 2 * h
            fm = obj(p2)
            fd = (fp - fm) / (2 * h)
            assert abs(fd - g[name][idx]) < 1e-5 * (1 + abs(fd)), (name, idx, fd, g[name][idx])


def test_dct_basis_is_orthogonal():
    B = dct_basis(40, 500)
    G = B @ B.T
    d = np.diag(G)
    assert abs(d[0] - 500) < 1e-9 and np.allclose(d[1:], 250)
    assert np.max(np.abs(G - np.diag(d))) < 1e-9


def test_default_network_size():
    cfg = NetConfig()
    assert cfg.flat() == 4 * 8 * 256
    assert [lv[:2] for lv in cfg.levels()] == [(128, 256), (64, 128), (32, 64), (16, 32), (8, 16)]
    assert cfg.noff() == 127
    assert 3.0e6 < cfg.n_params() < 6.0e6 and cfg.cin == 8


def test_shot_generator_is_seeded_and_stable():
    spec = ShotSpec()
    a = make_shot(spec, 5, 17)
    b = make_shot(spec, 5, 17)
    c = make_shot(spec, 5, 18)
    assert np.array_equal(a[1][0], b[1][0]) and a[4] == b[4]
    assert not np.array_equal(a[1][0], c[1][0])
    p = a[0]
    assert p.nx == p.ny == 296 and p.nstep == 2000 and p.npoints_pml == 20
    assert p.courant() < 1.0
    assert len(a[2]) == 64 and all(21 <= r[0] <= 276 for r in a[2])
    assert 21 <= p.isource <= 276
    x = encode_input(spec, a[3], a[4])
    assert x.shape == (128, 256, 8) and not x[..., 5:].any()
    assert np.all(np.abs(x[..., 3]) <= 1.0) and set(np.unique(x[..., 4])) <= {0.0, 1.0}
    o = 128 - a[4] // 2                       # model window starts here; source column lands on 128
    assert x[..., 1].sum() == 128 * 128 and np.all(x[:, o:o + 128, 1] == 1.0)
    small = a[3].reshape(128, 2, 128, 2).mean(axis=(1, 3))
    assert np.allclose(x[:, o + a[4] // 2, 0], (small[:, a[4] // 2] - 3000.0) / 1000.0)
    assert x[..., 2].sum() == 64 and np.all(x[127, :, 2][x[127, :, 2] > 0] == 1.0)
    s = source_slot(spec, a[4])
    assert abs(a[2][s][0] - p.isource) <= 2    # nearest receiver column within two cells
    assert np.all(np.abs(x[..., 0]) <= 2.0)
    assert 1500 * 0.85 <= a[3].min() and a[3].max() <= 4500 * 1.15


@pytest.mark.parametrize("seed", [5, 50005])
def test_courant_below_one_for_many_shots(seed):
    spec = ShotSpec()
    worst = max(make_shot(spec, seed, i)[0].courant() for i in range(40))
    assert worst < 1.0 / math.sqrt(1.0) and worst < 0.8
