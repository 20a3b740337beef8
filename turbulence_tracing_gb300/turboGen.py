"""Drop-in for turboGen's field generators (gaussian_fields/turboGen.py):
gaussian1Dcos / gaussian2Dcos / gaussian3Dcos (:40-385), gaussian1D_FFT /
gaussian2D_FFT / gaussian3D_FFT (:388-537), plus the seeded band-limited field
used by the benchmark workloads.

The cosine-sum generators draw their wavenumbers and phases exactly as the
reference does (numpy's global random state, same order, same arithmetic),
so a seeded np.random gives the reference's field; the O(n^d x modes)
summation runs on the GPU (tt_cos_field).

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


def _cos_modes(wnn, wn1, nmodes, especf, power):
    """Wavenumbers and amplitudes as the reference forms them."""
    dk = (wnn - wn1) / nmodes
    wn = wn1 + 0.5 * dk + np.arange(0, nmodes) * dk
    dkn = np.ones(nmodes) * dk
    espec = especf(wn)
    espec = espec.clip(0.0)
    return wn, np.sqrt(2.0 * espec * dkn ** power)


def gaussian1Dcos(lx, nx, nmodes, wn1, especf):
    """A 1-D Gaussian field with the given energy spectrum as a sum of nmodes
    random-phase cosines at nx cell centres (turboGen.py:40-121)."""
    dx = lx / nx
    wnn = np.pi / dx
    print("This function will generate data up to wavenumber: ", wnn)
    wn, A_m = _cos_modes(wnn, wn1, nmodes, especf, 1)
    phi = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
    psi = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)  # drawn, unused, as the reference
    del psi
    k = np.zeros((3, nmodes))
    k[0] = wn
    ph = np.zeros((4, nmodes))
    ph[0] = phi
    print("Generating 1-D turbulence...")
    r = core.cos_field(1, (nx,), (dx,), k, ph, A_m).cpu().numpy()
    print("Done! 1-D Turbulence has been generated!")
    return r


def gaussian2Dcos(lx, ly, nx, ny, nmodes, wn1, especf):
    """2-D counterpart (turboGen.py:130-245): (nx, ny) field indexed [i, j]."""
    dx, dy = lx / nx, ly / ny
    wnn = max(np.pi / dx, np.pi / dy)
    print("This function will generate data up to wavenumber: ", wnn)
    wn, A_m = _cos_modes(wnn, wn1, nmodes, especf, 2)
    phi = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
    psi = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
    theta = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
    k = np.zeros((3, nmodes))
    k[0] = np.cos(theta) * wn
    k[1] = np.sin(theta) * wn
    ph = np.zeros((4, nmodes))
    ph[0], ph[1] = phi, psi
    print("Generating 2-D turbulence...")
    r = core.cos_field(2, (nx, ny), (dx, dy), k, ph, A_m).cpu().numpy()
    print("Done! 2-D Turbulence has been generated!")
    return r


def gaussian3Dcos(lx, ly, lz, nx, ny, nz, nmodes, wn1, especf):
    """3-D counterpart (turboGen.py:254-385): (nx, ny, nz) field indexed [i, j, k]."""
    dx, dy, dz = lx / nx, ly / ny, lz / nz
    wnn = max(np.pi / dx, np.pi / dy, np.pi / dz)
    print("This function will generate data up to wavenumber: ", wnn)
    wn, A_m = _cos_modes(wnn, wn1, nmodes, especf, 3)
    psi = [2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes) for _ in range(4)]
    theta = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
    phi = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
    k = np.zeros((3, nmodes))
    k[0] = np.sin(theta) * np.cos(phi) * wn
    k[1] = np.sin(theta) * np.sin(phi) * wn
    k[2] = np.cos(theta) * wn
    print("Generating 3-D turbulence...")
    r = core.cos_field(3, (nx, ny, nz), (dx, dy, dz), k, np.stack(psi), A_m).cpu().numpy()
    print("Done! 3-D Turbulence has been generated!")
    return r


def _k_half_nd(dim, M, dev):
    """|k| on the half spectrum of an M^dim grid in the reference's summation order."""
    k = torch.as_tensor(np.fft.fftfreq(M), dtype=torch.float64, device=dev)
    h = M // 2 + 1
    if dim == 1:
        return torch.sqrt(k[:h] * k[:h])
    if dim == 2:
        # meshgrid(k, k) ('xy'): K[a][b] = sqrt(k[b]^2 + k[a]^2)
        return torch.sqrt(k[None, :h] * k[None, :h] + k[:, None] * k[:, None])
    return _k_half(M, dev)


def _gaussian_nd_fft(dim, N, k_func, seed, Wr, Wi, return_device):
    dev = core.require_cuda()
    M = 2 * N + 1
    if seed is None and Wr is None:
        seed = int(np.random.randint(0, 2 ** 62))
    sp = _sqrt_power(k_func, _k_half_nd(dim, M, dev))
    out = core.grf_fft_nd(dim, N, sp, seed=seed or 0, Wr=Wr, Wi=Wi)
    return out if return_device else out.cpu().numpy()


def gaussian1D_FFT(N, k_func, *, seed=None, Wr=None, Wi=None, return_device=False):
    """A realisation of a 1D Gaussian process on 2N+1 points (turboGen.py:388-434)."""
    return _gaussian_nd_fft(1, N, k_func, seed, Wr, Wi, return_device)


def gaussian2D_FFT(N, k_func, *, seed=None, Wr=None, Wi=None, return_device=False):
    """A realisation of a 2D Gaussian process on (2N+1)^2 points (turboGen.py:436-485)."""
    return _gaussian_nd_fft(2, N, k_func, seed, Wr, Wi, return_device)


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
