"""2D Fourier neural operator: parameters, training and inference through the
tcgen05 tensor-core kernels of libturbotrace (tt_fno_* in include/turbotrace.h).

The network (width 32, 16 x 32 retained modes, GELU, BF16 activations with
FP32 accumulation) maps in_ch straight-line maps plus two coordinate channels
to out_ch outputs on an S x S grid, S in {128, 256}.  Parameters, gradients
and the Adam moments are FP32 device tensors in the flat layout of the C ABI.
Every pass runs on the current CUDA stream and allocates nothing after the
first call with a given batch size, so training steps can be captured in a
CUDA graph.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib, core


def param_layout(in_ch, out_ch, layers=4):
    """[(name, offset, shape)] of the flat parameter array and its length."""
    C, M, cin = _lib.FNO_WIDTH, 2 * _lib.FNO_MODES ** 2, in_ch + 2
    lay, off = [], 0
    for name, shape in ([("P", (C, cin)), ("pb", (C,))] +
                        [item for l in range(layers) for item in
                         (("W%d" % l, (C, C)), ("b%d" % l, (C,)), ("R%d" % l, (M, C, C, 2)))] +
                        [("Q", (out_ch, C)), ("qb", (out_ch,))]):
        lay.append((name, off, shape))
        off += int(np.prod(shape))
    return lay, off


def init_params(in_ch, out_ch, layers=4, seed=0):
    """Seeded initial parameters: uniform with fan-in scaling, zero biases."""
    rng = np.random.default_rng(seed)
    C, M = _lib.FNO_WIDTH, 2 * _lib.FNO_MODES ** 2
    lay, n = param_layout(in_ch, out_ch, layers)
    flat = np.zeros(n, dtype=np.float32)
    for name, off, shape in lay:
        k = int(np.prod(shape))
        if name == "P":
            v = rng.uniform(-1, 1, k) / math.sqrt(in_ch + 2)
        elif name[0] == "W":
            v = rng.uniform(-1, 1, k) / math.sqrt(C)
        elif name[0] == "R":
            v = rng.uniform(-1, 1, k) / (C * C)
        elif name == "Q":
            v = rng.uniform(-1, 1, k) / math.sqrt(C)
        else:
            v = np.zeros(k)
        flat[off:off + k] = v
    return flat


class FNO:
    def __init__(self, size, in_ch=2, out_ch=3, layers=4, params=None, seed=0):
        if size not in (128, 256):
            raise ValueError("size must be 128 or 256")
        self.dev = core.require_cuda()
        self.S, self.in_ch, self.out_ch, self.layers = size, in_ch, out_ch, layers
        self.layout, self.n = param_layout(in_ch, out_ch, layers)
        L = _lib.lib()
        d = self._dims(1)
        if L.tt_fno_param_count(ctypes.byref(d)) != self.n:
            raise RuntimeError("parameter layout disagrees with the library")
        p = init_params(in_ch, out_ch, layers, seed) if params is None else np.asarray(params, dtype=np.float32)
        if p.size != self.n:
            raise ValueError("params must hold %d values" % self.n)
        self.params = torch.as_tensor(p, device=self.dev).clone()
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self._ws = {}

    def _dims(self, batch):
        return _lib.TTFnoDims(batch, self.S, self.in_ch, self.out_ch, self.layers)

    def _workspace(self, batch, training):
        key = (batch, bool(training))
        ws = self._ws.get(key)
        if ws is None:
            d = self._dims(batch)
            nb = _lib.lib().tt_fno_workspace_bytes(ctypes.byref(d), int(bool(training)))
            ws = torch.zeros(nb, dtype=torch.uint8, device=self.dev)
            self._ws[key] = ws
        return ws

    def _check_in(self, a, ch):
        if not (isinstance(a, torch.Tensor) and a.is_cuda and a.dtype == torch.float32 and a.is_contiguous()):
            raise TypeError("expected a contiguous float32 CUDA tensor")
        if a.dim() != 4 or a.shape[1:] != (ch, self.S, self.S):
            raise ValueError("expected shape (B, %d, %d, %d), got %s" % (ch, self.S, self.S, tuple(a.shape)))

    def forward(self, a, out=None):
        """out (B, out_ch, S, S) = network(a), a (B, in_ch, S, S) float32 on the device."""
        self._check_in(a, self.in_ch)
        B = a.shape[0]
        if out is None:
            out = torch.empty((B, self.out_ch, self.S, self.S), dtype=torch.float32, device=self.dev)
        ws = self._workspace(B, False)
        d = self._dims(B)
        _lib.check(_lib.lib().tt_fno_forward(ctypes.byref(d), core._ptr(self.params), core._ptr(a), core._ptr(out),
                                             core._ptr(ws), ws.numel(), core._stream()), "tt_fno_forward")
        return out

    def train_step(self, a, target, weights=None, out=None):
        """Accumulate the loss into self.loss and the gradient into self.grads."""
        self._check_in(a, self.in_ch)
        self._check_in(target, self.out_ch)
        B = a.shape[0]
        ws = self._workspace(B, True)
        d = self._dims(B)
        w = (ctypes.c_float * self.out_ch)(*([1.0] * self.out_ch if weights is None else list(weights)))
        _lib.check(_lib.lib().tt_fno_train_step(ctypes.byref(d), core._ptr(self.params), core._ptr(self.grads),
                                                core._ptr(a), core._ptr(target), w, core._ptr(self.loss),
                                                core._ptr(out) if out is not None else None, core._ptr(ws),
                                                ws.numel(), core._stream()), "tt_fno_train_step")
        return self.loss

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, step=None):
        """One Adam update from the accumulated gradient (which it zeroes)."""
        self.step_count = self.step_count + 1 if step is None else int(step)
        _lib.check(_lib.lib().tt_fno_adam(self.n, core._ptr(self.params), core._ptr(self.grads), core._ptr(self.m),
                                          core._ptr(self.v), float(lr), float(beta1), float(beta2), float(eps),
                                          self.step_count, core._stream()), "tt_fno_adam")

    def adam_device(self, lr_dev, step_dev, beta1=0.9, beta2=0.999, eps=1e-8):
        """Adam with the learning rate and step counter in device tensors
        (float32 (1,), int64 (1,)); the step is incremented on the device."""
        _lib.check(_lib.lib().tt_fno_adam_device(self.n, core._ptr(self.params), core._ptr(self.grads),
                                                 core._ptr(self.m), core._ptr(self.v), core._ptr(lr_dev),
                                                 float(beta1), float(beta2), float(eps), core._ptr(step_dev),
                                                 core._stream()), "tt_fno_adam_device")

    def error_flag(self):
        """1 if any bounded tensor-core wait ran out in any workspace (synchronises)."""
        flag = 0
        for ws in self._ws.values():
            f = ctypes.c_int(0)
            _lib.check(_lib.lib().tt_fno_error_flag(core._ptr(ws), ctypes.byref(f)), "tt_fno_error_flag")
            flag |= f.value
        return flag

    def blocks(self):
        """Parameter blocks as host numpy arrays, keyed like the layout."""
        p = self.params.cpu().numpy()
        return {name: p[off:off + int(np.prod(sh))].reshape(sh) for name, off, sh in self.layout}


# ----------------------------------------------------------------------------- building blocks (tests)
def pack(mat):
    """bf16 canonical K-major tcgen05 layout of a float32 (rows, k) device matrix."""
    dev = core.require_cuda()
    m = mat.to(device=dev, dtype=torch.float32).contiguous()
    rows, k = m.shape
    out = torch.empty(rows * k * 2, dtype=torch.uint8, device=dev)
    _lib.check(_lib.lib().tt_fno_pack(rows, k, core._ptr(m), core._ptr(out), core._stream()), "tt_fno_pack")
    return out


def _flag_ws(dev):
    return torch.zeros(256, dtype=torch.uint8, device=dev)


def rowdft(S, x_bf16, mat_packed):
    dev = core.require_cuda()
    rows = x_bf16.numel() // S
    out = torch.empty((rows, 2 * _lib.FNO_MODES), dtype=torch.float32, device=dev)
    ws = _flag_ws(dev)
    _lib.check(_lib.lib().tt_fno_rowdft(S, rows, core._ptr(x_bf16), core._ptr(mat_packed), core._ptr(out),
                                        core._ptr(ws), core._stream()), "tt_fno_rowdft")
    return out, ws


def mix(S, B, mode, x_bf16, w_packed, a_packed, sp, bias=None, zprev=None, want_z=True):
    dev = core.require_cuda()
    shape = (B, _lib.FNO_WIDTH, S, S)
    out0 = torch.empty(shape, dtype=torch.bfloat16, device=dev) if (mode == 1 or want_z) else None
    out1 = torch.empty(shape, dtype=torch.bfloat16, device=dev) if mode == 0 else None
    ws = _flag_ws(dev)
    _lib.check(_lib.lib().tt_fno_mix(S, B, mode, core._ptr(x_bf16), core._ptr(w_packed), core._ptr(a_packed),
                                     core._ptr(sp), core._ptr(bias) if bias is not None else None,
                                     core._ptr(zprev) if zprev is not None else None,
                                     core._ptr(out0) if out0 is not None else None,
                                     core._ptr(out1) if out1 is not None else None, core._ptr(ws),
                                     core._stream()), "tt_fno_mix")
    return out0, out1, ws


def wgrad(S, B, dz_bf16, v_bf16):
    dev = core.require_cuda()
    dW = torch.zeros((_lib.FNO_WIDTH, _lib.FNO_WIDTH), dtype=torch.float32, device=dev)
    db = torch.zeros(_lib.FNO_WIDTH, dtype=torch.float32, device=dev)
    ws = _flag_ws(dev)
    _lib.check(_lib.lib().tt_fno_wgrad(S, B, core._ptr(dz_bf16), core._ptr(v_bf16), core._ptr(dW), core._ptr(db),
                                       core._ptr(ws), core._stream()), "tt_fno_wgrad")
    return dW, db, ws


def error_flag(ws):
    f = ctypes.c_int(0)
    _lib.check(_lib.lib().tt_fno_error_flag(core._ptr(ws), ctypes.byref(f)), "tt_fno_error_flag")
    return f.value
