"""Learned surrogate with exact-tracer fallback.

Task: from the straight-line (unbent-ray) path integrals of a density field,
predict what the full trace gives -- the deflection of each pixel-centre ray
and its phase -- and fall back to the exact FP32 tracer where the network's
own error estimate says the prediction would miss.

Per realisation (an S^3 field of side L, drawn like the batched ensemble):
  maps     tt_straight_line_maps: straight-line deflection (2 maps) and phase
           of the S x S pixel-centre rays -- the method without the network --
           and the deflection accumulated in each of nslab slabs along the
           path (2 maps per slab)
  inputs   the deflection maps (total and per slab) / s, s the rms of the
           total deflection, and a constant map log10(s (S - 1)) -- the
           straight-line drift across the box in cells, i.e. how far into the
           nonlinear regime the field is
  targets  (full-trace deflection - straight-line deflection) / (s^2 (S - 1))
           and (full-trace phase - straight-line phase) / (k0 L s^2): both
           corrections are second order in the field, so these are O(1)
           from weak to strong fields
  network  the FNO of fno.py (4 layers, width 32, 16 modes), trained by the
           library's own forward/backward kernels and Adam, one CUDA graph
           per step
Shadowgram intensity comes from tt_shadowgram (geometric optics, drift D set
per field from the straight-line map so the contrast is 20%); the error of a
prediction is ||I_pred - I_trace||_2 / ||I_trace||_2.  The error estimate is
kappa * ||I_net - I_straight|| / ||I_net|| (how far the network moved the
answer), kappa calibrated on held-out fields so that 90% of them are bounded.
"""
import math
import time

import numpy as np
import torch

from . import core, fno as fno_mod

C_LIGHT = 299792458.0


def draw_fields(n, seed=0, exponents=(-5.0 / 3.0, -3.0, -11.0 / 3.0), delta=(0.05, 0.3), ne0=(1e23, 1e25)):
    """Per-field parameters drawn like the batched ensemble (fixed grid size)."""
    rng = np.random.default_rng(seed)
    return [dict(alpha=float(rng.choice(exponents)), delta=float(rng.uniform(*delta)),
                 ne0=float(rng.uniform(*ne0)), seed=int(rng.integers(0, 2 ** 62))) for _ in range(n)]


class Workload:
    """Fields, straight-line maps, exact traces and shadowgrams at one grid size."""

    def __init__(self, S, L=2e-3, lwl=1064e-9, rtol=1e-7, contrast=0.2, nslab=4):
        self.dev = core.require_cuda()
        self.S, self.L, self.lwl, self.rtol, self.contrast = S, L, lwl, rtol, contrast
        self.nslab = nslab
        self.in_ch = in_channels(nslab)
        self.n_maps = 3 + 2 * nslab
        self.x = np.linspace(-L / 2, L / 2, S)
        self.ext = float(self.x.max())
        self.t_end = float(np.linspace(0.0, math.sqrt(8.0) * self.ext / C_LIGHT, 2)[-1])
        omega = 2 * math.pi * C_LIGHT / lwl
        self.k0 = omega / C_LIGHT
        self.pitch = L / S
        pc = -L / 2 + (np.arange(S) + 0.5) * (L / S)
        X, Y = np.meshgrid(pc, pc, indexing="ij")
        s0 = np.zeros((6, S * S))
        s0[0], s0[1], s0[2], s0[5] = X.ravel(), Y.ravel(), -L / 2, C_LIGHT
        self.s0 = torch.as_tensor(s0, device=self.dev)
        self.vol = None
        self.trace_out = None

    def field(self, p):
        return core.grf_field(self.S, self.L, p["alpha"], p["ne0"], p["delta"], p["seed"], dtype=torch.float32)

    def maps(self, ne, out=None):
        return core.straight_line_maps(ne, self.x, self.x, self.x, self.S, lwl=self.lwl, out=out, nslab=self.nslab)

    def trace(self, ne):
        """Exact FP32 trace of the pixel-centre rays: (theta (2,S,S) f32, phase (S,S) f64, steps tensor)."""
        if self.vol is None:
            self.vol = core.build_volume(ne, self.x, self.x, self.x, 2, lwl=self.lwl)
        else:
            self.vol = core.build_volume(ne, self.x, self.x, self.x, 2, lwl=self.lwl, nodes=self.vol.nodes)
        o = core.trace_f32(self.vol, self.s0, self.t_end, self.ext, rtol=self.rtol, phase=True,
                           ws=None if self.trace_out is None else self.trace_out["_ws"], out=self.trace_out)
        self.trace_out = o
        S = self.S
        theta = torch.stack([o["rf"][1].view(S, S), o["rf"][3].view(S, S)]).float()
        return theta, o["phase"].view(S, S), o["nsteps"].sum()

    def drift(self, straight):
        """Free drift D (m) giving the straight-line map the set shadowgram contrast."""
        _, div = core.shadowgram(straight[0:2].contiguous(), self.pitch, 0.0, want_intensity=False, want_div=True)
        return self.contrast / torch.sqrt((div.double() ** 2).mean())

    def shadow(self, theta, D):
        return core.shadowgram(theta.contiguous(), self.pitch, float(D))[0]


def in_channels(nslab):
    return 3 + 2 * nslab


def encode(maps, S):
    """Network input (3 + 2 nslab, S, S) and the scale s from straight-line maps
    (3 + 2 nslab, S, S): total and slab deflections / s, then log10 drift."""
    nin = maps.shape[0]
    s = torch.sqrt((maps[0:2].double() ** 2).mean()).float().clamp_min(1e-30)
    inp = torch.empty((nin, S, S), dtype=torch.float32, device=maps.device)
    inp[0:2] = maps[0:2] / s
    inp[2:nin - 1] = maps[3:nin] / s
    inp[nin - 1] = torch.log10(s * (S - 1))
    return inp, s


def targets(maps, theta, phase, s, k0, L):
    S = maps.shape[-1]
    t = torch.empty((3, S, S), dtype=torch.float32, device=maps.device)
    t[0:2] = (theta - maps[0:2]) / (s * s * (S - 1))
    t[2] = ((phase - maps[2].double()) / (k0 * L * s.double() ** 2)).float()
    return t


def decode(out, maps, s, k0, L):
    """Predicted deflection (2, S, S) and phase (S, S) from network output (3, S, S)."""
    S = maps.shape[-1]
    theta = maps[0:2] + (s * s * (S - 1)) * out[0:2]
    phase = maps[2].double() + (k0 * L) * s.double() ** 2 * out[2].double()
    return theta, phase


def rel_l2(a, b):
    return float(torch.linalg.norm((a - b).double()) / torch.linalg.norm(b.double()))


def build_dataset(W, params, keep_truth=False):
    """Inputs and targets (N, 3, S, S) on the device; optionally the straight-line
    maps, exact deflections and phases for evaluation."""
    N, S = len(params), W.S
    X = torch.empty((N, W.in_ch, S, S), dtype=torch.float32, device=W.dev)
    Y = torch.empty((N, 3, S, S), dtype=torch.float32, device=W.dev)
    scale = torch.empty(N, dtype=torch.float32, device=W.dev)
    truth = None
    if keep_truth:
        truth = {"maps": torch.empty((N, W.n_maps, S, S), dtype=torch.float32, device=W.dev), "theta": torch.empty((N, 2, S, S), dtype=torch.float32, device=W.dev),
                 "phase": torch.empty((N, S, S), dtype=torch.float64, device=W.dev)}
    steps = torch.zeros((), dtype=torch.int64, device=W.dev)
    for i, p in enumerate(params):
        ne = W.field(p)
        m = W.maps(ne)
        theta, phase, st = W.trace(ne)
        X[i], s = encode(m, S)
        scale[i] = s
        Y[i] = targets(m, theta, phase, s, W.k0, W.L)
        steps += st
        if keep_truth:
            truth["maps"][i] = m
            truth["theta"][i] = theta
            truth["phase"][i] = phase
    return X, Y, scale, truth, steps


class Trainer:
    """Adam training of an FNO on device-resident (X, Y), one CUDA graph per step."""

    def __init__(self, net, X, Y, batch=8, weights=(1.0, 1.0, 0.5), graph=True):
        self.net, self.X, self.Y, self.B, self.w = net, X, Y, batch, list(weights)
        dev = X.device
        self.a = torch.empty((batch,) + tuple(X.shape[1:]), dtype=torch.float32, device=dev)
        self.t = torch.empty((batch,) + tuple(Y.shape[1:]), dtype=torch.float32, device=dev)
        self.idx = torch.zeros(batch, dtype=torch.int64, device=dev)
        self.lr = torch.zeros(1, dtype=torch.float32, device=dev)
        self.step = torch.zeros(1, dtype=torch.int64, device=dev)
        self.graph = None
        self._body()  # allocates the workspaces; discard its gradient
        net.grads.zero_()
        net.loss.zero_()
        torch.cuda.synchronize()
        if graph:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g):
                    self._body()
                    net.adam_device(self.lr, self.step)
            torch.cuda.current_stream().wait_stream(s)
            self.graph = g

    def _body(self):
        torch.index_select(self.X, 0, self.idx, out=self.a)
        torch.index_select(self.Y, 0, self.idx, out=self.t)
        self.net.train_step(self.a, self.t, weights=self.w)

    def fit(self, epochs, lr=1e-3, lr_min=1e-5, warmup=50, seed=0):
        """Returns per-epoch mean losses and the samples/s of training."""
        N = self.X.shape[0]
        nb = N // self.B
        total = epochs * nb
        g = torch.Generator(device=self.X.device).manual_seed(seed)
        hist = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        k = 0
        for ep in range(epochs):
            perm = torch.randperm(N, generator=g, device=self.X.device)
            self.net.loss.zero_()
            for b in range(nb):
                frac = k / max(total - 1, 1)
                cur = lr * min(1.0, (k + 1) / warmup) * (lr_min / lr + (1 - lr_min / lr) * 0.5 * (1 + math.cos(math.pi * frac)))
                self.idx.copy_(perm[b * self.B:(b + 1) * self.B])
                self.lr.fill_(cur)
                if self.graph is not None:
                    self.graph.replay()
                else:
                    self._body()
                    self.net.adam_device(self.lr, self.step)
                k += 1
            hist.append(self.net.loss.item() / nb)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        return hist, total * self.B / dt


def predict(net, X, batch=8):
    out = torch.empty((X.shape[0], net.out_ch) + tuple(X.shape[2:]), dtype=torch.float32, device=X.device)
    for b in range(0, X.shape[0], batch):
        e = min(b + batch, X.shape[0])
        if e - b == batch:
            net.forward(X[b:e], out=out[b:e])
        else:
            out[b:e] = net.forward(X[b:e].contiguous())
    return out


def evaluate(W, net, X, scale, truth, batch=8):
    """Per-field shadowgram errors of the straight-line map, the network and the
    network's own correction size (the basis of its error estimate)."""
    out = predict(net, X, batch)
    res = []
    for i in range(X.shape[0]):
        m = truth["maps"][i]
        D = W.drift(m)
        th_net, ph_net = decode(out[i], m, scale[i], W.k0, W.L)
        I_t = W.shadow(truth["theta"][i], D)
        I_s = W.shadow(m[0:2], D)
        I_n = W.shadow(th_net, D)
        res.append({"err_straight": rel_l2(I_s, I_t), "err_net": rel_l2(I_n, I_t), "moved": rel_l2(I_n, I_s) *
                    float(torch.linalg.norm(I_s.double()) / torch.linalg.norm(I_n.double())),
                    "theta_err_straight": rel_l2(m[0:2], truth["theta"][i]),
                    "theta_err_net": rel_l2(th_net, truth["theta"][i]),
                    "phase_corr_err_net": float(torch.linalg.norm(ph_net - truth["phase"][i]) /
                                                torch.linalg.norm(truth["phase"][i] - m[2].double())),
                    "log_drift": float(X[i, -1, 0, 0])})
    return res


def calibrate(res, quantile=0.9):
    """kappa with err_net <= kappa * moved for the given fraction of fields."""
    r = np.array([e["err_net"] / max(e["moved"], 1e-12) for e in res])
    return float(np.quantile(r, quantile))


class Pipeline:
    """Surrogate with fallback: for each field, straight-line maps -> network ->
    shadowgram and error estimate; fields whose estimate exceeds tol are traced."""

    def __init__(self, W, net, kappa, tol=0.02, batch=8):
        self.W, self.net, self.kappa, self.tol, self.B = W, net, kappa, tol, batch
        S = W.S
        self.X = torch.empty((batch, W.in_ch, S, S), dtype=torch.float32, device=W.dev)
        self.out = torch.empty((batch, 3, S, S), dtype=torch.float32, device=W.dev)
        self.maps = torch.empty((batch, W.n_maps, S, S), dtype=torch.float32, device=W.dev)

    def run(self, fields):
        """fields: list of density tensors.  Returns (intensity list, fell_back list)."""
        W, S = self.W, self.W.S
        I_out, fell = [], []
        for b0 in range(0, len(fields), self.B):
            chunk = fields[b0:b0 + self.B]
            n = len(chunk)
            sc = []
            for i, ne in enumerate(chunk):
                W.maps(ne, out=self.maps[i])
                self.X[i], s = encode(self.maps[i], S)
                sc.append(s)
            self.net.forward(self.X, out=self.out)
            for i in range(n):
                m = self.maps[i]
                D = W.drift(m)
                th, _ = decode(self.out[i], m, sc[i], W.k0, W.L)
                I_n = W.shadow(th, D)
                I_s = W.shadow(m[0:2], D)
                est = self.kappa * rel_l2(I_n, I_s) * float(torch.linalg.norm(I_s.double()) /
                                                            torch.linalg.norm(I_n.double()))
                if est > self.tol:
                    theta, _, _ = W.trace(chunk[i])
                    I_n = W.shadow(theta, D)
                    fell.append(True)
                else:
                    fell.append(False)
                I_out.append(I_n)
        return I_out, fell

    def run_tracer(self, fields):
        """The exact method alone: trace every field."""
        out = []
        for ne in fields:
            m = self.W.maps(ne)
            D = self.W.drift(m)
            theta, _, _ = self.W.trace(ne)
            out.append(self.W.shadow(theta, D))
        return out
