"""CPU oracle of the 2D Fourier neural operator surrogate (TEST INFRASTRUCTURE ONLY).

The reference has no learned surrogate: this module is the specification of
the one built here, restated in numpy float64, and the checker of its CUDA
kernels (forward pass, loss, backward pass).  Parity against the reference is
unpinned because there is nothing in the reference to pin to; the oracle's own
backward pass is checked against central finite differences of its forward
pass (tests/test_oracle_fno.py).

Network (width C, retained modes m in each direction, grid S x S):
  v0     = P a + pb                                  (lift, per pixel)
  for each of the layers:
    T1[y, kx]  = sum_x v[y, x] exp(-2 pi i kx x / S),      kx in [0, m)
    T2[ky, kx] = sum_y T1[y, kx] exp(-2 pi i ky y / S),    ky in [0, m) u [S-m, S)
    U[o]       = sum_c R[o, c] T2[c]                       (per mode, complex)
    S1[y, kx]  = sum_ky U[ky, kx] exp(+2 pi i ky y / S)
    s[y, x]    = sum_kx c_kx Re(S1[y, kx] exp(+2 pi i kx x / S)) / S^2,  c_0 = 1, c_k = 2
    z          = W v + b + s ;   v = GELU(z)   (tanh form)
  out    = Q v + qb                                  (projection, per pixel)
  loss   = sum_k w_k sum (out_k - target_k)^2 / (B S^2)

Real/imaginary parts of kx are the columns j < m / j >= m of the row-DFT
arrays (T1, S1 and their gradients), as on the GPU.  With bf16=True the
oracle rounds exactly where the GPU stores bfloat16: the DFT matrices, the
1x1 weights, the activations v and pre-activations z, the spectral rows S1 and
dT1 fed to the tensor cores, and the backward activations dz.
"""
import math

import numpy as np

WIDTH = 32
MODES = 16


def bf16(x):
    """Round to bfloat16 (round to nearest even) and return as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


GELU_A = math.sqrt(2.0 / math.pi)
GELU_B = 0.044715


def gelu(z):
    """GELU in its tanh form (Hendrycks & Gimpel 2016):
    z/2 (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))."""
    return 0.5 * z * (1.0 + np.tanh(GELU_A * (z + GELU_B * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GELU_A * (z + GELU_B * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_A * (1.0 + 3.0 * GELU_B * z * z)


def ky_list(S, m=MODES):
    return np.concatenate([np.arange(m), np.arange(S - m, S)])


def dft_mats(S, m=MODES):
    """FxT[j, x] (forward row DFT, j < m: cos, j >= m: -sin) and G[j, x] (inverse
    row DFT with the c_kx / S^2 weights, j < m: c cos, j >= m: -c sin)."""
    x = np.arange(S)
    k = np.arange(m)
    th = 2.0 * np.pi * (np.outer(k, x) % S) / S
    ck = np.where(k == 0, 1.0, 2.0)[:, None] / (S * S)
    FxT = np.concatenate([np.cos(th), -np.sin(th)], axis=0)
    G = np.concatenate([ck * np.cos(th), -ck * np.sin(th)], axis=0)
    return FxT, G


def ydft_mat(S, m=MODES, sign=-1.0):
    ky = ky_list(S, m)
    return np.exp(sign * 2j * np.pi * np.outer(ky, np.arange(S)) / S)  # [2m, S]


# --------------------------------------------------------------------------- parameters
def param_layout(cin, cout, C=WIDTH, m=MODES, layers=4):
    """Offsets (in floats) of each parameter block in the flat FP32 array,
    in the packing order of the C ABI (include/turbotrace.h)."""
    M = 2 * m * m
    lay = []
    off = 0

    def add(name, shape):
        nonlocal off
        n = int(np.prod(shape))
        lay.append((name, off, shape))
        off += n

    add("P", (C, cin))
    add("pb", (C,))
    for l in range(layers):
        add("W%d" % l, (C, C))
        add("b%d" % l, (C,))
        add("R%d" % l, (M, C, C, 2))
    add("Q", (cout, C))
    add("qb", (cout,))
    return lay, off


def unpack(flat, cin, cout, C=WIDTH, m=MODES, layers=4):
    lay, n = param_layout(cin, cout, C, m, layers)
    assert flat.size == n
    return {name: flat[o:o + int(np.prod(sh))].reshape(sh).astype(np.float64) for name, o, sh in lay}


def pack(p, cin, cout, C=WIDTH, m=MODES, layers=4):
    lay, n = param_layout(cin, cout, C, m, layers)
    out = np.zeros(n, dtype=np.float64)
    for name, o, sh in lay:
        out[o:o + int(np.prod(sh))] = np.asarray(p[name], dtype=np.float64).ravel()
    return out


def init_params(cin, cout, seed=0, C=WIDTH, m=MODES, layers=4):
    """Seeded initial parameters (uniform fan-in scaling); FP32 values."""
    rng = np.random.default_rng(seed)
    M = 2 * m * m
    p = {"P": rng.uniform(-1, 1, (C, cin)) / math.sqrt(cin), "pb": np.zeros(C)}
    for l in range(layers):
        p["W%d" % l] = rng.uniform(-1, 1, (C, C)) / math.sqrt(C)
        p["b%d" % l] = np.zeros(C)
        p["R%d" % l] = rng.uniform(-1, 1, (M, C, C, 2)) / (C * C)
    p["Q"] = rng.uniform(-1, 1, (cout, C)) / math.sqrt(C)
    p["qb"] = np.zeros(cout)
    return {k: v.astype(np.float32).astype(np.float64) for k, v in p.items()}


# --------------------------------------------------------------------------- forward / backward
def _c(X, m):
    return X[..., :m] + 1j * X[..., m:]


def _r(Z):
    return np.concatenate([Z.real, Z.imag], axis=-1)


def forward(p, a, layers=4, m=MODES, bf16_mode=True):
    """a: (B, cin, S, S).  Returns (out, cache)."""
    rnd = bf16 if bf16_mode else (lambda x: np.asarray(x, dtype=np.float64))
    B, cin, S, _ = a.shape
    FxT, G = dft_mats(S, m)
    FxT_b, G_b = rnd(FxT), rnd(G)
    Ey = ydft_mat(S, m, -1.0)
    Ey_inv = ydft_mat(S, m, +1.0)
    v = rnd(np.einsum("ci,biyx->bcyx", p["P"], a) + p["pb"][None, :, None, None])
    cache = {"a": a, "v": [v], "z": [], "T2": [], "FxT_b": FxT_b, "G_b": G_b, "Ey": Ey, "Ey_inv": Ey_inv}
    for l in range(layers):
        R = p["R%d" % l][..., 0] + 1j * p["R%d" % l][..., 1]  # [M, o, c]
        T1 = np.einsum("bcyx,jx->bcyj", v, FxT_b)
        T2 = np.einsum("ky,bcyx->bckx", Ey, _c(T1, m))  # [B, C, 2m, m]
        T2 = T2.reshape(B, T2.shape[1], -1).transpose(0, 2, 1)  # [B, M, C], mode = kyi * m + kx
        U = np.einsum("moc,bmc->bmo", R, T2)
        Ug = U.transpose(0, 2, 1).reshape(B, -1, 2 * m, m)  # [B, o, 2m, m]
        S1 = _r(np.einsum("yk,bokx->boyx", Ey_inv.T, Ug))  # [B, o, S, 2m]
        acc = (np.einsum("oc,bcyx->boyx", rnd(p["W%d" % l]), v) +
               np.einsum("boyj,jx->boyx", rnd(S1), G_b))
        z = rnd(acc + p["b%d" % l][None, :, None, None])
        v = rnd(gelu(z))
        cache["z"].append(z)
        cache["T2"].append(T2)
        cache["v"].append(v)
    out = np.einsum("kc,bcyx->bkyx", p["Q"], v) + p["qb"][None, :, None, None]
    return out, cache


def loss_and_grad(p, a, target, weights, layers=4, m=MODES, bf16_mode=True):
    """Loss and the gradient of every parameter block (dict like p)."""
    rnd = bf16 if bf16_mode else (lambda x: np.asarray(x, dtype=np.float64))
    out, K = forward(p, a, layers, m, bf16_mode)
    B, cout, S, _ = out.shape
    w = np.asarray(weights, dtype=np.float64)[None, :, None, None]
    d = out - target
    loss = float((w * d * d).sum() / (B * S * S))
    dout = 2.0 * w * d / (B * S * S)
    g = {}
    v4 = K["v"][-1]
    g["Q"] = np.einsum("bkyx,bcyx->kc", dout, v4)
    g["qb"] = dout.sum(axis=(0, 2, 3))
    dv = np.einsum("kc,bkyx->bcyx", p["Q"], dout)
    dz = rnd(dv * gelu_grad(K["z"][-1]))
    FxT_b, G_b, Ey, Ey_inv = K["FxT_b"], K["G_b"], K["Ey"], K["Ey_inv"]
    for l in range(layers - 1, -1, -1):
        v = K["v"][l]
        R = p["R%d" % l][..., 0] + 1j * p["R%d" % l][..., 1]
        g["W%d" % l] = np.einsum("boyx,bcyx->oc", dz, v)
        g["b%d" % l] = dz.sum(axis=(0, 2, 3))
        dS1 = np.einsum("boyx,jx->boyj", dz, G_b)
        dU = np.einsum("ky,boyx->bokx", Ey, _c(dS1, m))
        dU = dU.reshape(B, dU.shape[1], -1).transpose(0, 2, 1)  # [B, M, o]
        T2 = K["T2"][l]
        dR = np.einsum("bmo,bmc->moc", dU, np.conj(T2))
        g["R%d" % l] = np.stack([dR.real, dR.imag], axis=-1)
        dT2 = np.einsum("moc,bmo->bmc", np.conj(R), dU)
        dT2g = dT2.transpose(0, 2, 1).reshape(B, -1, 2 * m, m)
        dT1 = _r(np.einsum("yk,bckx->bcyx", Ey_inv.T, dT2g))
        dvv = (np.einsum("oc,boyx->bcyx", rnd(p["W%d" % l]), dz) +
               np.einsum("bcyj,jx->bcyx", rnd(dT1), FxT_b))
        if l > 0:
            dz = rnd(dvv * gelu_grad(K["z"][l - 1]))
        else:
            g0 = rnd(dvv)
    g["P"] = np.einsum("bcyx,biyx->ci", g0, K["a"])
    g["pb"] = g0.sum(axis=(0, 2, 3))
    return loss, out, g


def with_coords(a):
    """Append the two coordinate channels the GPU lift adds: row and column
    index (i + 0.5) * 2 / S - 1."""
    B, cd, S, _ = a.shape
    r = (np.arange(S) + 0.5) * (2.0 / S) - 1.0
    ry = np.broadcast_to(r[:, None], (S, S))
    rx = np.broadcast_to(r[None, :], (S, S))
    co = np.broadcast_to(np.stack([ry, rx])[None], (B, 2, S, S))
    return np.concatenate([np.asarray(a, dtype=np.float64), co], axis=1)
