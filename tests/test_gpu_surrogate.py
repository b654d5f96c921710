"""GPU checks of the surrogate kernels and network.

Kernels against torch FP32/FP64 references of the same op on the same BF16
inputs; the whole network's gradients against the FP64 numpy oracle
(oracle/surrogate_np.py) on identical FP32 master weights; and an ablation:
a trained network against the untrained one and against a mean-trace
predictor, with FD fallback on the shots it flags."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from seismic_cpml_gb300.build import build
    from seismic_cpml_gb300 import lib
    build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return lib.load()


def vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("fn", ["cpml_nn_gemm", "cpml_nn_gemm_tc"])
@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("M,N,K,splits", [(1, 1, 1, 1), (70, 33, 50, 1), (128, 192, 640, 1), (37, 65, 3000, 7),
                                          (200, 18, 4096, 64), (300, 136, 96, 1)])
def test_gemm_matches_fp64_reference(L, fn, ta, tb, M, N, K, splits):
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(K, N, generator=g).to(torch.bfloat16)
    bias = torch.randn(N, generator=g)
    C0 = torch.randn(M, N, generator=g)
    ref = A.double() @ B.double()
    dA = (A.t().contiguous() if ta else A).cuda()
    dB = (B.t().contiguous() if tb else B).cuda()
    lda = M if ta else K
    ldb = K if tb else N
    for relu, accum, use_bias, alpha in [(0, 0, False, 1.0), (1, 0, True, 0.5), (0, 1, True, 2.0)]:
        Cf = C0.clone().cuda()
        Cb = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
        work = torch.empty(splits * M * N + 1, device="cuda")
        b = bias.cuda() if use_bias else None
        assert getattr(L, fn)(M, N, K, vp(dA), lda, ta, vp(dB), ldb, tb, vp(Cf), vp(Cb), N, vp(b), relu, accum,
                              alpha, splits, vp(work), work.numel(), stream()) == 0
        torch.cuda.synchronize()
        err = ctypes.c_int(-1)
        assert L.cpml_nn_error(ctypes.byref(err)) == 0 and err.value == 0
        exp = alpha * ref
        if use_bias:
            exp = exp + bias.double()
        if relu:
            exp = exp.clamp_min(0)
        if accum:
            exp = exp + C0.double()
        err = (Cf.cpu().double() - exp).abs().max().item()
        scale = exp.abs().max().item() + 1.0
        assert err <= 2e-5 * scale * max(1.0, (K / 256) ** 0.5), (relu, accum, err, scale)
        assert torch.equal(Cb.cpu(), Cf.cpu().to(torch.bfloat16))


def test_gemm_rejects_bad_arguments(L):
    x = torch.zeros(4, dtype=torch.bfloat16, device="cuda")
    c = torch.zeros(4, device="cuda")
    assert L.cpml_nn_gemm(2, 2, 2, vp(x), 2, 0, vp(x), 2, 0, None, None, 2, None, 0, 0, 1.0, 1, None, 0,
                          stream()) != 0
    assert L.cpml_nn_gemm(2, 2, 64, vp(x), 2, 0, vp(x), 2, 0, vp(c), None, 2, None, 0, 0, 1.0, 2, None, 0,
                          stream()) != 0
    assert L.cpml_nn_gemm(2, 2, 2, vp(x), 2, 0, vp(x), 2, 0, None, vp(x), 2, None, 0, 1, 1.0, 1, None, 0,
                          stream()) != 0


def test_im2col_col2im_match_oracle(L):
    from oracle import surrogate_np as S
    rng = np.random.default_rng(2)
    for (B, H, W, C) in [(2, 16, 16, 3), (1, 9, 7, 5), (3, 4, 4, 32)]:
        x = rng.standard_normal((B, H, W, C)).astype(np.float32)
        xb = torch.from_numpy(x).to(torch.bfloat16)
        col_ref, (Ho, Wo) = S.im2col(xb.float().numpy().astype(np.float64))
        col = torch.empty(B * Ho * Wo * 9 * C, dtype=torch.bfloat16, device="cuda")
        assert L.cpml_nn_im2col(vp(xb.cuda()), vp(col), B, H, W, C, stream()) == 0
        assert np.array_equal(col.cpu().float().numpy().reshape(col_ref.shape), col_ref.astype(np.float32))
        d = rng.standard_normal(col_ref.shape).astype(np.float32)
        out = torch.empty(B * H * W * C, device="cuda")
        assert L.cpml_nn_col2im(vp(torch.from_numpy(d).cuda()), vp(out), B, H, W, C, stream()) == 0
        ref = S.col2im(d.astype(np.float64), (B, H, W, C))
        assert np.max(np.abs(out.cpu().numpy().reshape(ref.shape) - ref)) < 1e-5


def test_elementwise_kernels(L):
    rng = np.random.default_rng(4)
    n = 100003
    dy = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
    db = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    df = torch.empty(n, device="cuda")
    assert L.cpml_nn_relu_bwd(vp(dy), vp(y), vp(db), vp(df), n, stream()) == 0
    exp = torch.where(y > 0, dy, torch.zeros_like(dy))
    assert torch.equal(df, exp) and torch.equal(db, exp.to(torch.bfloat16))
    M, N = 1000, 77
    x = torch.from_numpy(rng.standard_normal((M, N)).astype(np.float32)).cuda()
    out = torch.full((N,), 3.0, device="cuda")
    work = torch.empty(8 * N, device="cuda")
    assert L.cpml_nn_colsum(vp(x), vp(out), M, N, 1, vp(work), work.numel(), stream()) == 0
    assert torch.allclose(out.double(), x.double().sum(0) + 3.0, atol=1e-4)
    B, Lr = 5, 777
    p = torch.from_numpy(rng.standard_normal((B, Lr)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((B, Lr)).astype(np.float32)).cuda()
    grad = torch.empty_like(p)
    loss = torch.empty(B, device="cuda")
    assert L.cpml_nn_rel_l2(vp(p), vp(t), vp(grad), vp(loss), B, Lr, stream()) == 0
    pd, td = p.double().cpu(), t.double().cpu()
    lref = ((pd - td) ** 2).sum(1) / (td ** 2).sum(1)
    assert torch.allclose(loss.cpu().double(), lref, rtol=1e-6)
    gref = 2 * (pd - td) / (td ** 2).sum(1, keepdim=True) / B
    assert torch.allclose(grad.cpu().double(), gref, rtol=1e-5, atol=1e-9)


def test_shift_rows_matches_gather(L):
    rng = np.random.default_rng(8)
    B, rs, rd, Lr = 4, 9, 5, 33
    src = rng.standard_normal((B, rs, Lr)).astype(np.float32)
    shift = np.array([-3, 0, 4, 7], np.int32)
    out = torch.empty(B * rd * Lr, device="cuda")
    outb = torch.empty(B * rd * Lr, dtype=torch.bfloat16, device="cuda")
    assert L.cpml_nn_shift_rows(vp(torch.from_numpy(src).cuda()), vp(torch.from_numpy(shift).cuda()), vp(out),
                                vp(outb), B, rs, rd, Lr, stream()) == 0
    ref = np.zeros((B, rd, Lr), np.float32)
    for b in range(B):
        for r in range(rd):
            q = r + shift[b]
            if 0 <= q < rs:
                ref[b, r] = src[b, q]
    assert np.array_equal(out.cpu().numpy().reshape(ref.shape), ref)
    assert torch.equal(outb, out.to(torch.bfloat16))


def test_adam_matches_formula(L):
    rng = np.random.default_rng(6)
    n = 4097
    w0 = rng.standard_normal(n).astype(np.float32)
    w = torch.from_numpy(w0.copy()).cuda()
    wb = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    m = torch.zeros(n, device="cuda")
    v = torch.zeros(n, device="cuda")
    mr, vr, wr = np.zeros(n), np.zeros(n), w0.astype(np.float64)
    for step in range(1, 4):
        g = rng.standard_normal(n).astype(np.float32)
        assert L.cpml_nn_adam(vp(w), vp(wb), vp(torch.from_numpy(g).cuda()), vp(m), vp(v), n, 1e-2, 0.9, 0.999,
                              1e-8, step, 1e-3, stream()) == 0
        gr = g + 1e-3 * wr
        mr = 0.9 * mr + 0.1 * gr
        vr = 0.999 * vr + 0.001 * gr * gr
        wr = wr - 1e-2 * (mr / (1 - 0.9 ** step)) / (np.sqrt(vr / (1 - 0.999 ** step)) + 1e-8)
    assert np.max(np.abs(w.cpu().numpy() - wr)) < 1e-5
    assert torch.equal(wb, w.to(torch.bfloat16))


SMALL = dict(h=32, w=48, cin=3, chans=(8, 16, 16, 32, 32), latent=48, nrec=8, nt=120, modes=24, head_weight=0.2)


@pytest.mark.parametrize("gemm", ["mma", "tcgen05"])
def test_network_gradients_match_fp64_oracle(L, gemm):
    from oracle import surrogate_np as S
    from seismic_cpml_gb300.surrogate import NetConfig, Surrogate, dct_basis
    cfg = NetConfig(**SMALL)
    net = Surrogate(cfg, seed=3, gemm=gemm)
    # generic weights (the product's near-zero output-layer init would make
    # the trunk gradients tiny), rounded to BF16 so the oracle sees the same
    # values the tensor cores multiply
    wr = np.random.default_rng(12)
    gen = {}
    for name, shp in cfg.param_shapes():
        scale = np.sqrt(2.0 / shp[1]) if name.endswith("_w") else 0.05
        gen[name] = wr.standard_normal(shp) * scale
    net.set_params(gen)
    net.w.copy_(net.w.to(torch.bfloat16).float())
    net.refresh_bf16()
    params = net.get_params()
    rng = np.random.default_rng(9)
    B = 16
    x = torch.from_numpy(rng.standard_normal((B, cfg.h, cfg.w, cfg.cin)).astype(np.float32)).to(torch.bfloat16)
    slot = rng.integers(0, cfg.nrec, B).astype(np.int32)
    basis = dct_basis(cfg.modes, cfg.nt)
    coef = rng.standard_normal((B * cfg.nrec, cfg.modes)) * np.exp(-np.arange(cfg.modes) / 6.0)
    t = (coef @ basis).reshape(B, -1).astype(np.float32)
    S_ = net.forward(x.cuda(), torch.from_numpy(slot).cuda(), B)
    net.backward(torch.from_numpy(t).cuda(), B)
    torch.cuda.synchronize()
    basis_b = torch.from_numpy(basis).to(torch.bfloat16).double().numpy()
    loss, head, g = S.loss_and_grads(params, x.double().numpy(), slot, t.astype(np.float64), basis_b, cfg.nrec,
                                     cfg.modes, cfg.head_weight)
    assert np.allclose(S_["loss"][:B].cpu().numpy(), loss, rtol=3e-2)
    assert np.allclose(S_["head"][:B].cpu().numpy(), head, rtol=3e-2, atol=3e-2)
    errs = {}
    for name, _ in cfg.param_shapes():
        got = net.G[name].cpu().double().numpy()
        ref = g[name]
        errs[name] = np.linalg.norm(got - ref) / (np.linalg.norm(ref) + 1e-30)
    assert max(errs.values()) < 5e-2, errs


def test_training_fits_a_small_problem(L):
    from seismic_cpml_gb300.surrogate import NetConfig, Surrogate, dct_basis
    cfg = NetConfig(**SMALL)
    net = Surrogate(cfg, seed=1)
    rng = np.random.default_rng(11)
    n = 256
    x = rng.standard_normal((n, cfg.h, cfg.w, cfg.cin)).astype(np.float32)
    basis = dct_basis(cfg.modes, cfg.nt)
    # a smooth function of the input: coefficients from channel means
    feats = x.reshape(n, -1, cfg.cin).mean(1)
    W = rng.standard_normal((cfg.cin, cfg.nrec * cfg.modes))
    coef = (np.tanh(feats @ W) + 1.5).reshape(n * cfg.nrec, cfg.modes) * np.exp(-np.arange(cfg.modes) / 5.0)
    t = (coef @ basis).reshape(n, -1).astype(np.float32)
    X = torch.from_numpy(x).to(torch.bfloat16).cuda()
    T = torch.from_numpy(t).cuda()
    sl = torch.full((n,), cfg.nrec - 1, dtype=torch.int32, device="cuda")
    P0, _ = net.predict(X, sl, batch=64)
    m0 = net.misfit(P0, T).median().item()
    hist = net.train(X, sl, T, epochs=40, batch=32, lr=2e-3, lr_min=1e-4)
    P1, head = net.predict(X, sl, batch=64)
    m1 = net.misfit(P1, T)
    assert m1.median().item() < 0.2 * m0, (m0, m1.median().item(), hist[-1])
    assert np.isfinite(head.cpu().numpy()).all()


def test_ablation_trained_network_with_fd_fallback(L):
    """What the trained network gains over the method without it: on held-out
    FD shots, the trained surrogate beats both the untrained network and a
    mean-trace predictor, and the fallback returns the FD traces bit for bit
    for every shot it flags."""
    from seismic_cpml_gb300.surrogate import NetConfig, ShotSpec, Surrogate, fd_seismograms, run_with_fallback
    spec = ShotSpec(interior=64, npml=10, nstep=600, decimate=2, nrec=16, hw=32)
    cfg = NetConfig(h=32, w=64, chans=(16, 32, 32, 64, 64), latent=128, nrec=16, nt=300, modes=24)
    Xtr, Str, Ytr = fd_seismograms(spec, 7, range(768))
    Xte, Ste, Yte = fd_seismograms(spec, 70007, range(64))
    scale = float(np.sqrt(np.mean(Ytr ** 2)))
    Xt = torch.from_numpy(Xtr).to(torch.bfloat16).cuda()
    St = torch.from_numpy(Str).cuda()
    Tt = torch.from_numpy(Ytr.reshape(len(Ytr), -1) / scale).cuda()
    Xv = torch.from_numpy(Xte).to(torch.bfloat16).cuda()
    Sv = torch.from_numpy(Ste).cuda()
    Tv = torch.from_numpy(Yte.reshape(len(Yte), -1) / scale).cuda()
    net = Surrogate(cfg, seed=2)
    untrained = net.misfit(net.predict(Xv, Sv)[0], Tv).sqrt().median().item()
    net.train(Xt, St, Tt, epochs=60, batch=32, lr=2e-3, lr_min=2e-5)
    P, head = net.predict(Xv, Sv)
    mis = net.misfit(P, Tv).sqrt()
    trained = mis.median().item()
    mean_trace = Tt.mean(0, keepdim=True).expand_as(Tv).contiguous()
    baseline = net.misfit(mean_trace, Tv).sqrt().median().item()
    assert trained < 0.5 * untrained and trained < 0.8 * baseline, (trained, untrained, baseline)
    # the misfit head ranks shots: predicted and true misfits correlate
    pred = (0.5 * head).exp().cpu().numpy()
    assert np.corrcoef(np.log(pred), np.log(mis.cpu().numpy()))[0, 1] > 0.2
    thr = float(np.median(pred))
    out, mask, t_nn, t_fd = run_with_fallback(net, spec, 70007, list(range(64)), Xv, Sv, threshold=thr,
                                              scale=scale)
    assert 0 < mask.sum() < 64
    ref = torch.from_numpy(Yte.reshape(64, -1) / scale).cuda()
    m = torch.from_numpy(mask).cuda()
    assert torch.equal(out[m], ref[m])
    final = net.misfit(out, Tv).sqrt().cpu().numpy()
    assert np.all(final[mask] == 0.0)
    assert np.median(final) <= trained
