"""Host logic of the surrogate on CPU tensors: tiling of large fields, the
target scaling and its inverse, and the fallback calibration; the input
encoding refuses to run without a GPU."""
import numpy as np
import torch

from turbulence_tracing_gb300 import surrogate as SG


def test_tiles_round_trip_and_pixel_indices():
    for N in (512, 768):
        m = torch.randn(5, N, N)
        t = SG.tile_maps(m)
        k = N // SG.TILE
        assert t.shape == (k * k, 5, SG.TILE, SG.TILE) and t.is_contiguous()
        assert torch.equal(SG.untile(t, N), m)
        for i in (0, k * k - 1, k + 1):
            idx = SG.tile_pixels(N, i)
            assert torch.equal(t[i, 2].reshape(-1), m[2].reshape(-1)[idx])


def test_encode_needs_the_gpu():
    """The input encoding, decoding and error estimate are CUDA kernels
    (tt_surrogate_encode/decode/estimate): without a GPU they raise rather
    than computing on the host."""
    import pytest

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    mm = torch.zeros((1, 5, 8, 8))
    with pytest.raises(RuntimeError, match="CUDA"):
        SG.encode_batch(mm, 8, torch.empty((1, SG.IN_CHANNELS, 8, 8)))
    from turbulence_tracing_gb300 import core

    with pytest.raises(RuntimeError, match="CUDA"):
        core.surrogate_decode(mm, torch.zeros((1, 3, 8, 8)), torch.zeros((1, 4)), torch.ones(3))
    with pytest.raises(RuntimeError, match="CUDA"):
        core.surrogate_estimate(torch.ones((1, 8, 8)), torch.ones((1, 8, 8)), 1.0)


def test_targets_decode_round_trip():
    g = torch.Generator().manual_seed(1)
    S, k0, L = 32, 5.9e6, 2e-3
    mm = torch.randn((5, S, S), generator=g) * 1e-3
    theta = mm[0:2] + 1e-6 * torch.randn((2, S, S), generator=g)
    phase = mm[2].double() + 1e-2 * torch.randn((S, S), generator=g, dtype=torch.float64)
    s = torch.tensor(1.3e-3)
    gain = torch.tensor([700.0, 650.0, 40.0])
    t = SG.targets(mm, theta, phase, s, k0, L) * gain[:, None, None]
    th, ph = SG.decode(t, mm, s, k0, L, gain)
    assert torch.allclose(th, theta, rtol=0, atol=1e-9)
    assert torch.allclose(ph, phase, rtol=0, atol=1e-6)


def test_calibrate_is_the_error_ratio_quantile():
    res = [{"err_net": e, "moved": m} for e, m in zip(np.linspace(0.001, 0.01, 10), np.full(10, 0.001))]
    k = SG.calibrate(res, quantile=0.9)
    ratios = np.array([r["err_net"] / r["moved"] for r in res])
    assert abs(k - np.quantile(ratios, 0.9)) < 1e-12
    assert np.mean(ratios <= k) >= 0.9
