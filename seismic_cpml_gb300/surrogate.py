"""Learned seismogram surrogate with FD fallback.

A small convolutional network maps a 2D velocity model and a source position
to the vertical-velocity seismograms of a line of surface receivers. It is
trained only on shots that the batched FD engine (cpml_batch_*) computes, and
at inference every shot whose predicted misfit is above a threshold is re-run
by that engine, which is both the fallback and the yardstick the misfit is
measured against. No counterpart in
the reference, which has no learned component.

The network works in the source's frame, so that what it learns does not
depend on where the source is:
  input [B, 128, 256, 8]: the 2 x 2 mean of the 256 x 256 interior cp map,
        (cp - 3000) / 1000, written into a window twice as wide whose centre
        column is the source column; a channel that is 1 inside the model;
        a channel marking the receivers (top row); the source's offset from
        its nearest receiver and its position inside its downsampled pixel
        (two constant planes); three zero channels, so that every pixel is
        16 bytes and the first layer's patches and weights take the 16-byte
        vector paths
  5 x { 3x3 stride-2 conv + bias + ReLU }: 8 -> 32 -> 64 -> 128 -> 256 -> 256
  dense 4 * 8 * 256 -> latent (ReLU); dense latent -> (2 nrec - 1) x modes
        coefficients, one trace per receiver offset -(nrec-1) .. nrec-1
  spectral synthesis: coefficients x truncated cosine (DCT-II) basis
        [modes, nt]; then each receiver takes the trace of its offset from
        the source's nearest receiver slot (cpml_nn_shift_rows)
  misfit head: dense latent -> 1, trained on the trunk's detached features
        to predict log(squared relative L2 misfit) of the shot
BF16 weights and activations, FP32 accumulation, FP32 Adam. Every layer runs
on the hand-written kernels behind cpml_nn_* (surrogate.cu); torch only owns
device memory and the stream.
"""
from __future__ import annotations

import ctypes
import math
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np
import torch

from . import lib as _L
from .batch import Batch
from .earth import gardner, lame_from_velocity
from .params import STF_RICKER, default_2d

IN_CHANNELS = 8   # cp, model mask, receivers, source offset, source sub-pixel + 3 zero channels


@dataclass(frozen=True)
class NetConfig:
    h: int = 128
    w: int = 256
    cin: int = 8
    chans: tuple = (32, 64, 128, 256, 256)
    latent: int = 256
    nrec: int = 64
    nt: int = 1000
    modes: int = 64
    head_weight: float = 0.05

    def levels(self):
        """(H, W, Cin, Cout) of every conv layer's input."""
        out, h, w, c = [], self.h, self.w, self.cin
        for co in self.chans:
            out.append((h, w, c, co))
            h, w, c = (h + 1) // 2, (w + 1) // 2, co
        return out

    def flat(self):
        h, w, _, co = self.levels()[-1]
        return ((h + 1) // 2) * ((w + 1) // 2) * co

    def noff(self):
        """Receiver offsets from the source slot: -(nrec-1) .. nrec-1."""
        return 2 * self.nrec - 1

    def param_shapes(self):
        shapes = []
        for l, (_, _, ci, co) in enumerate(self.levels()):
            shapes += [(f"conv{l}_w", (co, 9 * ci)), (f"conv{l}_b", (co,))]
        R = self.noff() * self.modes
        shapes += [("fc1_w", (self.latent, self.flat())), ("fc1_b", (self.latent,)),
                   ("fc2_w", (R, self.latent)), ("fc2_b", (R,)),
                   ("head_w", (1, self.latent)), ("head_b", (1,))]
        return shapes

    def n_params(self):
        return sum(int(np.prod(s)) for _, s in self.param_shapes())


def dct_basis(modes, nt):
    """[modes, nt] with row k = cos(pi k (n + 1/2) / nt): the first DCT-II
    modes, which represent a trace that does not end at zero without the
    wrap-around jump of a DFT basis."""
    n = np.arange(nt) + 0.5
    return np.cos(np.pi * np.arange(modes)[:, None] * n[None, :] / nt)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class Surrogate:
    """Weights, Adam state and per-batch-size work buffers on one GPU."""

    def __init__(self, cfg: NetConfig = NetConfig(), seed: int = 0, device: str = "cuda", gemm: str = "tcgen05"):
        if not torch.cuda.is_available():
            raise RuntimeError("the surrogate needs a CUDA device")
        if gemm not in ("mma", "tcgen05"):
            raise ValueError("gemm is 'mma' (mma.sync) or 'tcgen05'")
        self.L = _L.load()
        self.cfg = cfg
        self.gemm_entry = "cpml_nn_gemm_tc" if gemm == "tcgen05" else "cpml_nn_gemm"
        self.dev = torch.device(device)
        self.sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        self.launches = 0        # kernels this object has launched (launch accounting)
        self.shapes = cfg.param_shapes()
        self.off, o = {}, 0
        for name, shp in self.shapes:
            self.off[name] = o
            o += (int(np.prod(shp)) + 63) // 64 * 64
        self.n = o
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.w = torch.zeros(self.n, **f32)
        self.g = torch.zeros(self.n, **f32)
        self.m = torch.zeros(self.n, **f32)
        self.v = torch.zeros(self.n, **f32)
        self.wb = torch.zeros(self.n, dtype=torch.bfloat16, device=self.dev)
        self.P, self.Pb, self.G = {}, {}, {}
        for name, shp in self.shapes:
            k, o = int(np.prod(shp)), self.off[name]
            self.P[name] = self.w[o:o + k].view(shp)
            self.Pb[name] = self.wb[o:o + k].view(shp)
            self.G[name] = self.g[o:o + k].view(shp)
        self.init_weights(seed)
        self.basis = torch.tensor(dct_basis(cfg.modes, cfg.nt), dtype=torch.float32, device=self.dev)
        self.basis_b = self.basis.to(torch.bfloat16)
        self.basis_tb = self.basis_b.t().contiguous()   # [nt, modes]: k-contiguous B operand of the synthesis
        self.step_count = 0
        self._bufs = {}

    # ---- parameters -------------------------------------------------------
    def init_weights(self, seed):
        rng = np.random.default_rng(seed)
        host = np.zeros(self.n, np.float32)
        for name, shp in self.shapes:
            k, o = int(np.prod(shp)), self.off[name]
            if name.endswith("_w"):
                # He init for the ReLU layers; the coefficient and head layers
                # start near zero so that the first steps do not drive the
                # latent ReLUs to zero to shrink a large initial output
                fan_in = shp[1]
                gain = 2.0 if name.startswith(("conv", "fc1")) else 1.0
                std = math.sqrt(gain / fan_in) * (0.01 if name in ("fc2_w", "head_w") else 1.0)
                host[o:o + k] = rng.standard_normal(k) * std
        self.w.copy_(torch.from_numpy(host))
        self.refresh_bf16()

    def refresh_bf16(self):
        self._call("cpml_nn_cast", _ptr(self.w), _ptr(self.wb), self.n, self._stream())

    def get_params(self):
        return {name: self.P[name].detach().cpu().numpy().astype(np.float64) for name, _ in self.shapes}

    def set_params(self, params):
        for name, shp in self.shapes:
            self.P[name].copy_(torch.as_tensor(np.asarray(params[name], np.float32).reshape(shp)))
        self.refresh_bf16()

    def state_dict(self):
        return {"cfg": self.cfg.__dict__, "w": self.w.cpu(), "m": self.m.cpu(), "v": self.v.cpu(),
                "step": self.step_count}

    def load_state_dict(self, sd):
        self.w.copy_(sd["w"])
        self.m.copy_(sd["m"])
        self.v.copy_(sd["v"])
        self.step_count = int(sd["step"])
        self.refresh_bf16()

    # ---- kernel calls -----------------------------------------------------
    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _call(self, name, *args, kernels=1):
        """One library entry point; raises CpmlError on a non-zero status and
        counts the kernels it launches."""
        _L.check(getattr(self.L, name)(*args), name)
        self.launches += kernels

    def _gemm(self, M, N, K, A, lda, ta, B, ldb, tb, Cf=None, Cb=None, ldc=None, bias=None, relu=0,
              accum=0, alpha=1.0, work=None):
        tm = 128 if self.gemm_entry == "cpml_nn_gemm_tc" else 64
        tiles = -(-M // tm) * -(-N // tm)
        splits = max(1, min(K // 512, -(-2 * self.sms // tiles)))
        wk = work if splits > 1 else None
        if wk is not None and wk.numel() < splits * M * N:
            splits = max(1, wk.numel() // (M * N))
            wk = wk if splits > 1 else None
        self._call(self.gemm_entry, M, N, K, _ptr(A), lda, ta, _ptr(B), ldb, tb, _ptr(Cf), _ptr(Cb),
                   ldc if ldc is not None else N, _ptr(bias), relu, accum, alpha, splits,
                   _ptr(wk), wk.numel() if wk is not None else 0, self._stream(), kernels=2 if splits > 1 else 1)

    def _buffers(self, B):
        if B in self._bufs:
            return self._bufs[B]
        c = self.cfg
        f32 = dict(dtype=torch.float32, device=self.dev)
        b16 = dict(dtype=torch.bfloat16, device=self.dev)
        S = {"col": [], "y": [], "a": []}
        max_dy, max_dcol, max_da = 0, 0, B * c.flat()
        for (H, W, ci, co) in c.levels():
            Ho, Wo = (H + 1) // 2, (W + 1) // 2
            M = B * Ho * Wo
            S["col"].append(torch.empty(M * 9 * ci, **b16))
            S["y"].append(torch.empty(M * co, **f32))
            S["a"].append(torch.empty(M * co, **b16))
            max_dy = max(max_dy, M * co)
            max_dcol = max(max_dcol, M * 9 * ci)
            max_da = max(max_da, B * H * W * ci)
        R = c.noff() * c.modes
        S.update(
            h=torch.empty(B * c.latent, **f32), hb=torch.empty(B * c.latent, **b16),
            zb=torch.empty(B * R, **b16), head=torch.empty(B, **f32),
            poff=torch.empty(B * c.noff() * c.nt, **f32), dpoffb=torch.empty(B * c.noff() * c.nt, **b16),
            p=torch.empty(B * c.nrec * c.nt, **f32), loss=torch.empty(B, **f32),
            dp=torch.empty(B * c.nrec * c.nt, **f32),
            dz=torch.empty(B * R, **f32), dzb=torch.empty(B * R, **b16),
            dhead=torch.empty(B, **f32), dheadb=torch.empty(B, **b16),
            dh=torch.empty(B * c.latent, **f32), dh1f=torch.empty(B * c.latent, **f32),
            dh1b=torch.empty(B * c.latent, **b16),
            dyf=torch.empty(max_dy, **f32), dyb=torch.empty(max_dy, **b16),
            dcol=torch.empty(max_dcol, **f32), da=torch.empty(max_da, **f32),
            shift=torch.empty(B, dtype=torch.int32, device=self.dev),
            shift_neg=torch.empty(B, dtype=torch.int32, device=self.dev),
            work=torch.empty(max(1 << 21, 2 * self.sms * 64 * 64 * 4), **f32))
        self._bufs[B] = S
        return S

    # ---- forward / backward -------------------------------------------------
    def forward(self, xb, slot, B, keep=True):
        """xb: bf16 [B, h, w, cin] and slot: int32 [B] (each shot's source
        receiver slot), on the device. Leaves the traces in buffer 'p'
        ([B, nrec*nt] FP32) and the misfit head in 'head'. keep=False (pure
        inference) skips the FP32 copies of the activations that only the
        backward pass reads."""
        c, S, st = self.cfg, self._buffers(B), self._stream()
        a = xb
        for l, (H, W, ci, co) in enumerate(c.levels()):
            Ho, Wo = (H + 1) // 2, (W + 1) // 2
            M, K = B * Ho * Wo, 9 * ci
            self._call("cpml_nn_im2col", _ptr(a), _ptr(S["col"][l]), B, H, W, ci, st)
            self._gemm(M, co, K, S["col"][l], K, 0, self.Pb[f"conv{l}_w"], K, 1, Cf=S["y"][l] if keep else None,
                       Cb=S["a"][l], bias=self.P[f"conv{l}_b"], relu=1, work=S["work"])
            a = S["a"][l]
        F, lat, R, no = c.flat(), c.latent, c.noff() * c.modes, c.noff()
        self._gemm(B, lat, F, a, F, 0, self.Pb["fc1_w"], F, 1, Cf=S["h"], Cb=S["hb"], bias=self.P["fc1_b"],
                   relu=1, work=S["work"])
        self._gemm(B, R, lat, S["hb"], lat, 0, self.Pb["fc2_w"], lat, 1, Cb=S["zb"], bias=self.P["fc2_b"],
                   work=S["work"])
        self._gemm(B, 1, lat, S["hb"], lat, 0, self.Pb["head_w"], lat, 1, Cf=S["head"], bias=self.P["head_b"],
                   work=S["work"])
        self._gemm(B * no, c.nt, c.modes, S["zb"], c.modes, 0, self.basis_tb, c.modes, 1, Cf=S["poff"],
                   work=S["work"])
        # receiver r of shot b is offset r - slot_b: row r + (nrec - 1 - slot_b) of the offset traces
        torch.sub(slot[:B], c.nrec - 1, out=S["shift_neg"])
        torch.neg(S["shift_neg"], out=S["shift"])
        self._call("cpml_nn_shift_rows", _ptr(S["poff"]), _ptr(S["shift"]), _ptr(S["p"]), None, B, no, c.nrec,
                   c.nt, st)
        return S

    def backward(self, target, B):
        """target: FP32 [B, nrec*nt]. Writes every gradient into self.g and
        the per-shot squared relative misfits into buffer 'loss'."""
        c, S, st = self.cfg, self._buffers(B), self._stream()
        T = c.nrec * c.nt
        R, lat, F, no = c.noff() * c.modes, c.latent, c.flat(), c.noff()
        self._call("cpml_nn_rel_l2", _ptr(S["p"]), _ptr(target), _ptr(S["dp"]), _ptr(S["loss"]), B, T, st)
        self._call("cpml_nn_head_grad", _ptr(S["head"]), 1, _ptr(S["loss"]), _ptr(S["dhead"]), B, c.head_weight,
                   st)
        self._call("cpml_nn_cast", _ptr(S["dhead"]), _ptr(S["dheadb"]), B, st)
        # receiver traces back to the offset axis (offsets without a receiver get 0)
        self._call("cpml_nn_shift_rows", _ptr(S["dp"]), _ptr(S["shift_neg"]), None, _ptr(S["dpoffb"]), B, c.nrec,
                   no, c.nt, st)
        # spectral synthesis and the coefficient layer
        self._gemm(B * no, c.modes, c.nt, S["dpoffb"], c.nt, 0, self.basis_b, c.nt, 1, Cf=S["dz"], Cb=S["dzb"],
                   work=S["work"])
        self._gemm(R, lat, B, S["dzb"], R, 1, S["hb"], lat, 0, Cf=self.G["fc2_w"], work=S["work"])
        self._colsum(S["dz"], self.G["fc2_b"], B, R, S)
        # misfit head (no gradient into the trunk)
        self._gemm(1, lat, B, S["dheadb"], 1, 1, S["hb"], lat, 0, Cf=self.G["head_w"], work=S["work"])
        self._colsum(S["dhead"], self.G["head_b"], B, 1, S)
        # dense 1
        self._gemm(B, lat, R, S["dzb"], R, 0, self.Pb["fc2_w"], lat, 0, Cf=S["dh"], work=S["work"])
        self._call("cpml_nn_relu_bwd", _ptr(S["dh"]), _ptr(S["h"]), _ptr(S["dh1b"]), _ptr(S["dh1f"]), B * lat, st)
        a_last = S["a"][-1]
        self._gemm(lat, F, B, S["dh1b"], lat, 1, a_last, F, 0, Cf=self.G["fc1_w"], work=S["work"])
        self._colsum(S["dh1f"], self.G["fc1_b"], B, lat, S)
        self._gemm(B, F, lat, S["dh1b"], lat, 0, self.Pb["fc1_w"], F, 0, Cf=S["da"], work=S["work"])
        # conv layers, last to first
        for l in reversed(range(len(c.chans))):
            H, W, ci, co = c.levels()[l]
            Ho, Wo = (H + 1) // 2, (W + 1) // 2
            M, K = B * Ho * Wo, 9 * ci
            self._call("cpml_nn_relu_bwd", _ptr(S["da"]), _ptr(S["y"][l]), _ptr(S["dyb"]), _ptr(S["dyf"]), M * co, st)
            self._gemm(co, K, M, S["dyb"], co, 1, S["col"][l], K, 0, Cf=self.G[f"conv{l}_w"], work=S["work"])
            self._colsum(S["dyf"], self.G[f"conv{l}_b"], M, co, S)
            if l > 0:
                self._gemm(M, K, co, S["dyb"], co, 0, self.Pb[f"conv{l}_w"], K, 0, Cf=S["dcol"], work=S["work"])
                self._call("cpml_nn_col2im", _ptr(S["dcol"]), _ptr(S["da"]), B, H, W, ci, st)

    def _colsum(self, x, out, M, N, S):
        self._call("cpml_nn_colsum", _ptr(x), _ptr(out), M, N, 0, _ptr(S["work"]), S["work"].numel(),
                   self._stream(), kernels=2)

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
        self.step_count += 1
        self._call("cpml_nn_adam", _ptr(self.w), _ptr(self.wb), _ptr(self.g), _ptr(self.m), _ptr(self.v),
                   self.n, lr, b1, b2, eps, self.step_count, wd, self._stream())

    # ---- training and inference ---------------------------------------------
    def train(self, X, slot, T, epochs=1, batch=64, lr=1e-3, lr_min=1e-5, seed=0, time_budget_s=None, log=None):
        """X: bf16 [N, h, w, cin], slot: int32 [N], T: FP32 [N, nrec*nt], all
        on the device. Adam with a cosine learning-rate decay over all
        iterations. Returns a list of (epoch, mean training squared misfit)."""
        n = X.shape[0]
        iters = n // batch
        total = epochs * iters
        gen = torch.Generator().manual_seed(seed)
        xb = torch.empty((batch,) + tuple(X.shape[1:]), dtype=X.dtype, device=self.dev)
        sb = torch.empty(batch, dtype=slot.dtype, device=self.dev)
        tb = torch.empty((batch, T.shape[1]), dtype=T.dtype, device=self.dev)
        acc = torch.zeros((), dtype=torch.float64, device=self.dev)
        hist, k, t0 = [], 0, time.perf_counter()
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen).to(self.dev)
            acc.zero_()
            for i in range(iters):
                idx = perm[i * batch:(i + 1) * batch]
                torch.index_select(X, 0, idx, out=xb)
                torch.index_select(slot, 0, idx, out=sb)
                torch.index_select(T, 0, idx, out=tb)
                S = self.forward(xb, sb, batch)
                self.backward(tb, batch)
                f = k / max(total - 1, 1)
                self.adam(lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * f)))
                acc += S["loss"].sum(dtype=torch.float64)
                k += 1
            mean = float(acc) / (iters * batch)
            hist.append((ep, mean))
            if log:
                log(f"epoch {ep} train misfit^2 {mean:.5f} ({time.perf_counter() - t0:.1f} s)")
            if time_budget_s is not None and time.perf_counter() - t0 > time_budget_s:
                break
        return hist

    def predict(self, X, slot, batch=512, out=None):
        """Traces [N, nrec*nt] FP32 and predicted log squared misfit [N]."""
        n = X.shape[0]
        c = self.cfg
        P = out if out is not None else torch.empty((n, c.nrec * c.nt), dtype=torch.float32, device=self.dev)
        head = torch.empty(n, dtype=torch.float32, device=self.dev)
        for s in range(0, n, batch):
            b = min(batch, n - s)
            S = self.forward(X[s:s + b], slot[s:s + b], b, keep=False)
            P[s:s + b].copy_(S["p"][:b * c.nrec * c.nt].view(b, -1))
            head[s:s + b].copy_(S["head"][:b])
        return P, head

    def misfit(self, P, T):
        """Squared relative L2 misfit per shot, on the device (cpml_nn_rel_l2)."""
        n = P.shape[0]
        loss = torch.empty(n, dtype=torch.float32, device=self.dev)
        self._call("cpml_nn_rel_l2", _ptr(P), _ptr(T), None, _ptr(loss), n, P.shape[1], self._stream())
        return loss


# ---- shots and their FD seismograms ----------------------------------------

@dataclass
class ShotSpec:
    """A seeded surrogate shot: 256 x 256 interior + 20-point C-PML on every
    side, DELTAX = DELTAY = 10 m, DELTAT = 1 ms, 2000 steps, Ricker f0 = 4 Hz
    vertical force three cells below the top interior row, 64 receivers one
    row below the top interior row, 4-10 layers with cp ~ U[1500, 4500] and
    0-4 Gaussian anomalies, cs = cp / sqrt(3), Gardner density."""
    interior: int = 256
    npml: int = 20
    delta: float = 10.0
    deltat: float = 1.0e-3
    nstep: int = 2000
    decimate: int = 2
    f0: float = 4.0
    nrec: int = 64
    layers: tuple = (4, 10)
    cp_range: tuple = (1500.0, 4500.0)
    anomalies: tuple = (0, 4)
    hw: int = 128


def _layered_cp_2d(n, nlayers, cp_range, anomalies, rng):
    """cp [n, n] (y slowest): horizontal layers at sorted uniform depths with
    uniform velocities, times 1 +/- 0.1 Gaussian anomalies of radius 5-40
    cells (each a separable outer product)."""
    tops = np.sort(rng.uniform(0, n, nlayers - 1))
    vals = rng.uniform(cp_range[0], cp_range[1], nlayers)
    prof = vals[np.searchsorted(tops, np.arange(n))]
    cp = np.repeat(prof[:, None], n, axis=1)
    g = np.arange(n, dtype=np.float64)
    for _ in range(anomalies):
        cy, cx = rng.uniform(0, n), rng.uniform(0, n)
        r = rng.uniform(5.0, 40.0)
        s = rng.choice([-1.0, 1.0]) * 0.1
        cp *= 1.0 + s * np.outer(np.exp(-(g - cy) ** 2 / (2 * r * r)), np.exp(-(g - cx) ** 2 / (2 * r * r)))
    return cp


def make_shot(spec: ShotSpec, seed: int, index: int):
    """(params, (lam, mu, rho), receivers, cp_interior, source_column)."""
    rng = np.random.default_rng([seed, index])
    n = spec.interior + 2 * spec.npml
    nl = int(rng.integers(spec.layers[0], spec.layers[1] + 1))
    na = int(rng.integers(spec.anomalies[0], spec.anomalies[1] + 1))
    cp = _layered_cp_2d(n, nl, spec.cp_range, na, rng)
    lam, mu, rho = lame_from_velocity(cp, cp / np.sqrt(3.0), gardner(cp))
    p = default_2d()
    p.nx = p.ny = n
    p.deltax = p.deltay = spec.delta
    p.deltat = spec.deltat
    p.nstep = spec.nstep
    p.npoints_pml = spec.npml
    p.use_pml[:] = [1, 1, 1, 1, 0, 0]
    p.cp = float(cp.max())
    p.cs = p.cp / math.sqrt(3.0)
    p.rho = float(gardner(p.cp))
    p.f0 = spec.f0
    p.t0 = 1.2 / spec.f0
    p.stf = STF_RICKER
    p.angle_force = 0.0
    p.factor = 1.0e7
    p.it_display = 100
    col = int(rng.integers(0, spec.interior))
    p.isource = spec.npml + 1 + col
    p.jsource = n - spec.npml - 3
    jr = n - spec.npml - 1
    rec = [(spec.npml + 1 + int(round(r * (spec.interior - 1) / (spec.nrec - 1))), jr) for r in range(spec.nrec)]
    inner = cp[spec.npml:spec.npml + spec.interior, spec.npml:spec.npml + spec.interior]
    return p, (lam, mu, rho), rec, inner.astype(np.float32), col


def source_slot(spec: ShotSpec, col):
    """Index of the receiver nearest to interior source column `col`."""
    return int(round(col * (spec.nrec - 1) / (spec.interior - 1)))


def encode_input(spec: ShotSpec, cp_inner, col):
    """[hw, 2 hw, 8] float32 network input in the source's frame: the
    downsampled normalised cp map placed so that the source column lands on
    column hw, a mask of the model window, the receiver positions on the
    receivers' row, two constant planes that restore what the 2 x
    downsampling and the receiver slots lose about the source position (the
    source's offset from its nearest receiver in cells / 2, and the source
    column's position inside its downsampled pixel), and three zero channels
    (16-byte pixels)."""
    f = spec.interior // spec.hw
    small = cp_inner.reshape(spec.hw, f, spec.hw, f).mean(axis=(1, 3))
    x = np.zeros((spec.hw, 2 * spec.hw, IN_CHANNELS), np.float32)
    o = spec.hw - col // f
    x[:, o:o + spec.hw, 0] = (small - 3000.0) / 1000.0
    x[:, o:o + spec.hw, 1] = 1.0
    row = (spec.interior - 2) // f          # receivers one row below the top interior row
    rcol = [int(round(r * (spec.interior - 1) / (spec.nrec - 1))) for r in range(spec.nrec)]
    for c in rcol:
        x[row, o + c // f, 2] = 1.0
    x[:, o:o + spec.hw, 3] = (col - rcol[source_slot(spec, col)]) / 2.0
    x[:, o:o + spec.hw, 4] = (col % f) / max(f - 1, 1)
    return x


def make_inputs(spec: ShotSpec, seed: int, indices):
    """Network inputs [n, hw, 2 hw, 8] float32 and source slots [n] int32 for
    shots (seed, index)."""
    out = np.zeros((len(indices), spec.hw, 2 * spec.hw, IN_CHANNELS), np.float32)
    slots = np.zeros(len(indices), np.int32)
    for q, i in enumerate(indices):
        _, _, _, inner, col = make_shot(spec, seed, i)
        out[q] = encode_input(spec, inner, col)
        slots[q] = source_slot(spec, col)
    return out, slots


def fd_seismograms(spec: ShotSpec, seed: int, indices, chunk=1024, timing=None, threads=8):
    """Run shots (seed, index) through the batched FD engine and return
    (inputs [n, hw, 2 hw, 8], source slots [n], vertical-velocity traces
    [n, nrec, nstep/decimate]) as numpy arrays. Host threads build the next
    chunk's models while the engine runs the current one. `timing`, if a
    list, receives the engine's device milliseconds per chunk."""
    indices = list(indices)
    X = np.zeros((len(indices), spec.hw, 2 * spec.hw, IN_CHANNELS), np.float32)
    slots = np.zeros(len(indices), np.int32)
    nt = spec.nstep // spec.decimate
    Y = np.zeros((len(indices), spec.nrec, nt), np.float32)
    starts = list(range(0, len(indices), chunk))
    with ThreadPoolExecutor(max_workers=threads) as ex:
        def submit(s):
            return [ex.submit(make_shot, spec, seed, i) for i in indices[s:s + chunk]]
        pending = submit(starts[0]) if starts else []
        for n_, s in enumerate(starts):
            shots = [f.result() for f in pending]
            pending = submit(starts[n_ + 1]) if n_ + 1 < len(starts) else []
            for q, sh in enumerate(shots):
                X[s + q] = encode_input(spec, sh[3], sh[4])
                slots[s + q] = source_slot(spec, sh[4])
            with Batch([sh[0] for sh in shots], models=[sh[1] for sh in shots],
                       receivers=[sh[2] for sh in shots]) as b:
                b.run()
                if timing is not None:
                    timing.append(b.last_run_ms())
                for q in range(len(shots)):
                    _, vy = b.seismograms(q)
                    Y[s + q] = vy[:, spec.decimate - 1::spec.decimate]
    return X, slots, Y


def run_with_fallback(net: Surrogate, spec: ShotSpec, seed: int, indices, X, slot, threshold=0.05, scale=1.0,
                      batch=512):
    """Surrogate inference for shots (seed, index) with inputs X (bf16) and
    source slots (int32) on the device, then FD re-runs of every shot whose
    predicted relative misfit exceeds `threshold`. Returns (traces
    [n, nrec*nt] FP32 on the device, scaled by 1/scale; boolean mask of the
    FD-run shots; seconds in the surrogate; seconds in FD)."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    P, head = net.predict(X, slot, batch=batch)
    flagged = torch.exp(0.5 * head) > threshold
    mask = flagged.cpu().numpy()
    t1 = time.perf_counter()
    rows = np.nonzero(mask)[0]
    if len(rows):
        _, _, Y = fd_seismograms(spec, seed, [indices[q] for q in rows])
        P[torch.as_tensor(rows, device=P.device)] = torch.as_tensor(Y.reshape(len(rows), -1) / scale,
                                                                    device=P.device)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return P, mask, t1 - t0, t2 - t1


def _main(argv=None):
    """`python -m seismic_cpml_gb300.surrogate [--shots N] [--batch B] [--gemm tcgen05|mma] [--repeat R]`:
    time inference of an untrained default network on random inputs (the
    kernel mix of a prediction pass; the accuracy is not exercised)."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--shots", type=int, default=2048)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--gemm", choices=["tcgen05", "mma"], default="tcgen05")
    ap.add_argument("--repeat", type=int, default=5)
    a = ap.parse_args(argv)
    cfg = NetConfig()
    g = torch.Generator(device="cpu").manual_seed(0)
    X = torch.randn(a.shots, cfg.h, cfg.w, cfg.cin, generator=g).to(torch.bfloat16).cuda()
    S = torch.randint(0, cfg.nrec, (a.shots,), generator=g, dtype=torch.int32).cuda()
    net = Surrogate(cfg, seed=0, gemm=a.gemm)
    P, _ = net.predict(X, S, batch=a.batch)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(a.repeat):
        net.predict(X, S, batch=a.batch, out=P)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t) / a.repeat
    print(f"{a.gemm}: {a.shots / dt:.0f} shots/s ({a.shots} shots, batch {a.batch})")


if __name__ == "__main__":
    _main()
