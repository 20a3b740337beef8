"""FNO surrogate kernels against the CPU oracle (oracle/fno.py).

Each tcgen05 building block is compared with the same contraction in float64
over identical bf16 operands; the full training step (forward, loss,
backward) is compared with the oracle's bf16-emulating restatement.
Tolerances: FP32-accumulated contractions of bf16 products agree to 1e-5
relative; outputs stored as bf16 may differ by one bf16 rounding (2^-8
relative) where FP32 summation order moves a value across a rounding
boundary, and those differences propagate through the layers, so network
outputs and gradients are checked in relative L2 norm.
"""
import numpy as np
import pytest
import torch

from oracle import fno as O

pytestmark = pytest.mark.gpu


def _bf(t):
    return t.to(torch.bfloat16)


def _f64(t):
    return t.detach().to(torch.float64).cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))


@pytest.mark.parametrize("S,rows", [(128, 384), (256, 384), (256, 128 * 700)])
def test_rowdft_matches_float64(cuda, S, rows):
    """Few tiles, and more 128-row tiles than the grid's blocks (each block
    then loads its next tile while it finishes the current one)."""
    from turbulence_tracing_gb300 import fno

    g = torch.Generator(device="cuda").manual_seed(S + rows)
    x = _bf(torch.randn((rows, S), device="cuda", generator=g))
    FxT, G = O.dft_mats(S)
    for M in (FxT, G * S * S):
        Mp = fno.pack(torch.as_tensor(M, dtype=torch.float32))
        out, ws = fno.rowdft(S, x, Mp)
        ref = _f64(x) @ O.bf16(M).T
        assert fno.error_flag(ws) == 0
        assert np.abs(_f64(out) - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("S", [128, 256])
def test_mix_forward_and_backward_match_float64(cuda, S):
    from turbulence_tracing_gb300 import fno

    g = torch.Generator(device="cuda").manual_seed(7)
    B = 2
    x = _bf(torch.randn((B, 32, S, S), device="cuda", generator=g))
    Wm = torch.randn((32, 32), device="cuda", generator=g) / 6
    A = torch.randn((S, 32), device="cuda", generator=g) / 6
    sp = torch.randn((B, 32, S, 32), device="cuda", generator=g)
    bias = torch.randn(32, device="cuda", generator=g) / 4
    acc = (np.einsum("oc,bcyx->boyx", O.bf16(_f64(Wm)), _f64(x)) +
           np.einsum("boyj,xj->boyx", O.bf16(_f64(sp)), O.bf16(_f64(A))))
    # forward: z = bf16(acc + b), v = bf16(gelu(z))
    z, v, ws = fno.mix(S, B, 0, x, fno.pack(Wm), fno.pack(A), sp, bias=bias)
    assert fno.error_flag(ws) == 0
    z_ref = O.bf16(acc + _f64(bias)[None, :, None, None])
    assert np.abs(_f64(z) - z_ref).max() <= 2 ** -7 * np.abs(z_ref).max()
    assert (np.abs(_f64(z) - z_ref) <= 2 ** -8 * np.abs(z_ref) + 1e-30).mean() > 0.999
    assert np.abs(_f64(v) - O.bf16(O.gelu(_f64(z)))).max() <= 2 ** -7 * np.abs(_f64(v)).max()
    # backward: out = bf16(acc * gelu'(zprev))
    zp = _bf(torch.randn((B, 32, S, S), device="cuda", generator=g))
    d, _, ws = fno.mix(S, B, 1, x, fno.pack(Wm), fno.pack(A), sp, zprev=zp)
    assert fno.error_flag(ws) == 0
    d_ref = O.bf16(acc * O.gelu_grad(_f64(zp)))
    assert np.abs(_f64(d) - d_ref).max() <= 2 ** -7 * np.abs(d_ref).max()


@pytest.mark.parametrize("S", [128, 256])
def test_wgrad_matches_float64(cuda, S):
    from turbulence_tracing_gb300 import fno

    g = torch.Generator(device="cuda").manual_seed(11)
    B = 3
    dz = _bf(torch.randn((B, 32, S, S), device="cuda", generator=g))
    v = _bf(torch.randn((B, 32, S, S), device="cuda", generator=g))
    dW, db, ws = fno.wgrad(S, B, dz, v)
    assert fno.error_flag(ws) == 0
    ref = np.einsum("boyx,bcyx->oc", _f64(dz), _f64(v))
    assert np.abs(_f64(dW) - ref).max() <= 1e-4 * np.abs(ref).max()
    assert np.abs(_f64(db) - _f64(dz).sum(axis=(0, 2, 3))).max() <= 1e-3 * np.abs(_f64(dz)).sum() / 32 / B / S


def _case(B=2, S=128, layers=4, seed=0):
    rng = np.random.default_rng(seed)
    p = O.init_params(4, 3, seed=seed, layers=layers)
    for k in p:  # move off the zero biases so every gradient block is exercised
        p[k] = (p[k] + 0.05 * rng.standard_normal(p[k].shape) * (np.abs(p[k]).max() + 0.1)).astype(np.float32)
    a = rng.standard_normal((B, 2, S, S)).astype(np.float32)
    t = (0.5 * rng.standard_normal((B, 3, S, S))).astype(np.float32)
    return p, a, t


def test_train_step_matches_oracle(cuda):
    from turbulence_tracing_gb300 import fno

    layers = 4
    p, a, t = _case(layers=layers)
    w = [1.0, 1.0, 0.5]
    flat = O.pack(p, 4, 3, layers=layers).astype(np.float32)
    net = fno.FNO(128, in_ch=2, out_ch=3, layers=layers, params=flat)
    at, tt_ = torch.as_tensor(a, device="cuda"), torch.as_tensor(t, device="cuda")
    out = torch.empty_like(tt_)
    net.train_step(at, tt_, weights=w, out=out)
    torch.cuda.synchronize()
    assert net.error_flag() == 0
    loss_ref, out_ref, g_ref = O.loss_and_grad(p, O.with_coords(a), t, w, layers=layers)
    assert abs(net.loss.item() - loss_ref) <= 1e-3 * loss_ref
    assert _rel(_f64(out), out_ref) <= 1e-2
    grads = net.grads.cpu().numpy()
    for name, off, sh in net.layout:
        got = grads[off:off + int(np.prod(sh))].reshape(sh)
        assert _rel(got, g_ref[name]) <= 3e-2, (name, _rel(got, g_ref[name]))
    # inference runs the same arithmetic as the training forward pass
    inf = net.forward(at)
    assert torch.equal(inf, out)


def test_adam_training_reduces_loss_and_graph_replay_matches(cuda):
    from turbulence_tracing_gb300 import fno

    p, a, _ = _case(B=4, layers=2, seed=4)
    # a learnable target: pointwise and smooth non-local functions of the input
    t = np.stack([a[:, 0], -a[:, 1], 0.5 * (np.roll(a[:, 0], 3, axis=-1) + a[:, 1])], axis=1).astype(np.float32)
    net = fno.FNO(128, in_ch=2, out_ch=3, layers=2, seed=1)
    at, tt_ = torch.as_tensor(a, device="cuda"), torch.as_tensor(t, device="cuda")
    losses = []
    for _ in range(40):
        net.loss.zero_()
        net.train_step(at, tt_)
        net.adam(3e-3)
        losses.append(net.loss.item())
    assert losses[-1] < 0.3 * losses[0], losses
    # one training step captured in a CUDA graph gives the same update as eager
    net2 = fno.FNO(128, in_ch=2, out_ch=3, layers=2, seed=1)
    net3 = fno.FNO(128, in_ch=2, out_ch=3, layers=2, seed=1)
    for n_ in (net2, net3):
        n_.loss.zero_()
        n_.train_step(at, tt_)  # allocate workspaces outside capture
        n_.grads.zero_()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph):
            net2.loss.zero_()
            net2.train_step(at, tt_)
            net2.adam(1e-3, step=1)
    graph.replay()
    net3.loss.zero_()
    net3.train_step(at, tt_)
    net3.adam(1e-3, step=1)
    torch.cuda.synchronize()
    # gradients are summed with atomics, so the two runs may differ in the last bits
    assert torch.allclose(net2.params, net3.params, rtol=0, atol=1e-6)
    assert not torch.equal(net2.params, torch.as_tensor(fno.init_params(2, 3, 2, 1), device="cuda"))
    assert net2.error_flag() == 0 and net3.error_flag() == 0
