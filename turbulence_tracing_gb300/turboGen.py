"""Drop-in for turboGen.gaussian3D_FFT (gaussian_fields/turboGen.py:488-537),
plus the seeded band-limited field used by the benchmark workloads.

gaussian3D_FFT(N, k_func) keeps the reference's signature and statistics:
(2N+1)^3 points, |k| in cycles/sample, complex Gaussian noise made Hermitian
(W(-k) = conj W(k), real and imaginary parts of variance 2 as the
reference's Wr + flip(Wr), Wi - flip(Wi)), times sqrt(k_func(|k|)), zero
mean, real part of the inverse FFT.  The noise comes from Philox4x32-10 on
the GPU; its key is drawn from numpy's global random state, so
np.random.seed() still fixes the result.  Passing the reference's own
(Wr, Wi) arrays reproduces the reference's output exactly.
"""
import numpy as np
import torch

from . import core


def _k_half(M, dev):
    k = torch.as_tensor(np.fft.fftfreq(M), dtype=torch.float64, device=dev)
    h = M // 2 + 1
    # meshgrid(k, k, k) ('xy'): KX varies along axis 1, KY along axis 0; sum in the reference's order
    k0 = k[:, None, None]
    k1 = k[None, :, None]
    k2 = k[None, None, :h]
    return torch.sqrt((k1 * k1 + k0 * k0) + k2 * k2)


def _sqrt_power(k_func, K):
    try:
        P = k_func(K)
        if not isinstance(P, torch.Tensor):
            raise TypeError
        P = P.to(torch.float64)
    except Exception:
        # k_func only understands numpy: evaluate once on the host grid
        with np.errstate(divide="ignore", invalid="ignore"):
            P = torch.as_tensor(np.asarray(k_func(K.cpu().numpy()), dtype=np.float64), device=K.device)
    return torch.sqrt(P)


def gaussian3D_FFT(N, k_func, *, seed=None, Wr=None, Wi=None, return_device=False):
    """A realisation of a 3D Gaussian process on (2N+1)^3 points with power spectrum k_func(|k|)."""
    dev = core.require_cuda()
    M = 2 * N + 1
    if seed is None and Wr is None:
        seed = int(np.random.randint(0, 2 ** 62))
    sp = _sqrt_power(k_func, _k_half(M, dev))
    out = core.grf_fft(N, sp, seed=seed or 0, Wr=Wr, Wi=Wi)
    return out if return_device else out.cpu().numpy()


def workload_field(n, L, alpha, delta, ne0, seed, dtype=torch.float32):
    """Density of the benchmark workloads on an n^3 grid of side L:
    ne = ne0 (1 + delta g), g a unit-variance Gaussian random field with power
    |k|^alpha for 2 pi / L <= |k| <= pi n / L, clipped at >= 0.
    Returns (device tensor, coordinate array linspace(-L/2, L/2, n))."""
    ne = core.grf_field(n, L, alpha, ne0, delta, seed, dtype=dtype)
    return ne, np.linspace(-L / 2, L / 2, n)
