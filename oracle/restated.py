"""numpy restatements of the reference path (test infrastructure only).

Each function cites the reference code it restates.  Nothing here is used by
the product package.
"""
import numpy as np

C_LIGHT = 299792458.0  # scipy.constants.c, particle_tracker.py:118


# ---------------------------------------------------------------------------
# particle_tracker.py
# ---------------------------------------------------------------------------
def critical_density(lwl):
    """omega and n_c exactly as calc_dndr forms them (particle_tracker.py:227-228)."""
    omega = 2 * np.pi * (C_LIGHT / lwl)
    return omega, 3.14207787e-4 * omega ** 2


def init_beam(Np, beam_size, divergence, extent, probing_direction="z"):
    """ElectronCube.init_beam (particle_tracker.py:258-310), drawing from the
    global numpy random state in the same order, so that a seeded
    np.random gives the same s0 as the reference."""
    s0 = np.zeros((6, Np))
    t = 2 * np.pi * np.random.rand(Np)
    u = np.random.rand(Np) + np.random.rand(Np)
    u[u > 1] = 2 - u[u > 1]
    phi = np.pi * np.random.rand(Np)
    chi = divergence * np.random.randn(Np)
    if probing_direction == "x":
        s0[3] = C_LIGHT * np.cos(chi)
        s0[4] = C_LIGHT * np.sin(chi) * np.cos(phi)
        s0[5] = C_LIGHT * np.sin(chi) * np.sin(phi)
        s0[0] = extent
        s0[1] = beam_size * u * np.cos(t)
        s0[2] = beam_size * u * np.sin(t)
    elif probing_direction == "y":
        s0[4] = C_LIGHT * np.cos(chi)
        s0[3] = C_LIGHT * np.sin(chi) * np.cos(phi)
        s0[5] = C_LIGHT * np.sin(chi) * np.sin(phi)
        s0[0] = beam_size * u * np.cos(t)
        s0[1] = -extent
        s0[2] = beam_size * u * np.sin(t)
    elif probing_direction == "z":
        s0[3] = C_LIGHT * np.sin(chi) * np.cos(phi)
        s0[4] = C_LIGHT * np.sin(chi) * np.sin(phi)
        s0[5] = C_LIGHT * np.cos(chi)
        s0[0] = beam_size * u * np.cos(t)
        s0[1] = beam_size * u * np.sin(t)
        s0[2] = -extent
    return s0


def gaussian_beam(Np, sigma, divergence, extent, rng):
    """Beam of the benchmark workloads: x, y ~ N(0, sigma); small angles
    theta_x, theta_y ~ N(0, divergence); speed c along +z; start plane
    z = -extent.  (The reference's init_beam draws a uniform disk; the
    workloads ask for Gaussian positions and are supplied by assigning s0.)"""
    s0 = np.zeros((6, Np))
    s0[0] = rng.normal(0.0, sigma, Np)
    s0[1] = rng.normal(0.0, sigma, Np)
    s0[2] = -extent
    tx = np.tan(rng.normal(0.0, divergence, Np))
    ty = np.tan(rng.normal(0.0, divergence, Np))
    nrm = np.sqrt(1.0 + tx * tx + ty * ty)
    s0[3] = C_LIGHT * tx / nrm
    s0[4] = C_LIGHT * ty / nrm
    s0[5] = C_LIGHT / nrm
    return s0


def ray_at_exit(sf, extent, probing_direction="z"):
    """ElectronCube.ray_at_exit (particle_tracker.py:333-380): back-project to
    the exit plane, angles from arctan of the velocity ratios."""
    x, y, z, vx, vy, vz = sf
    rp = np.zeros((4, sf.shape[1]))
    with np.errstate(divide="ignore", invalid="ignore"):
        if probing_direction == "x":
            t_bp = (x - extent) / vx
            rp[0] = y - vy * t_bp
            rp[2] = z - vz * t_bp
            rp[1] = np.arctan(vy / vx)
            rp[3] = np.arctan(vz / vx)
        elif probing_direction == "y":
            t_bp = (y - extent) / vy
            rp[0] = x - vx * t_bp
            rp[2] = z - vz * t_bp
            rp[1] = np.arctan(vx / vy)
            rp[3] = np.arctan(vz / vy)
        else:
            t_bp = (z - extent) / vz
            rp[0] = x - vx * t_bp
            rp[2] = y - vy * t_bp
            rp[1] = np.arctan(vx / vz)
            rp[3] = np.arctan(vy / vz)
    return rp


def t_end(extent):
    """Integration end time of solve (particle_tracker.py:317)."""
    return np.linspace(0.0, np.sqrt(8.0) * extent / C_LIGHT, 2)[-1]


# ---------------------------------------------------------------------------
# ray_transfer_matrix.py
# ---------------------------------------------------------------------------
def m_to_mm(r):
    rr = np.array(r, dtype=np.float64, copy=True)
    rr[0::2, :] *= 1e3
    return rr


def lens(r, f1, f2):
    L = np.zeros((4, 4))
    L[:2, :2] = [[1, 0], [-1 / f1, 1]]
    L[2:, 2:] = [[1, 0], [-1 / f2, 1]]
    return np.matmul(L, r)


def sym_lens(r, f):
    return lens(r, f, f)


def distance(r, d):
    D = np.zeros((4, 4))
    D[:2, :2] = [[1, d], [0, 1]]
    D[2:, 2:] = [[1, d], [0, 1]]
    return np.matmul(D, r)


def circular_aperture(r, R):
    filt = r[0, :] ** 2 + r[2, :] ** 2 > R ** 2
    r[:, filt] = None
    return r


def circular_stop(r, R):
    filt = r[0, :] ** 2 + r[2, :] ** 2 < R ** 2
    r[:, filt] = None
    return r


def annular_stop(r, R1, R2):
    return (r[0, :] ** 2 + r[2, :] ** 2 > R1 ** 2) & (r[0, :] ** 2 + r[2, :] ** 2 < R2 ** 2)


def angular_filter(r, Rs):
    f = np.zeros((r.shape[1]), dtype=bool)
    for i in range(0, len(Rs) // 2):
        f += annular_stop(r, Rs[2 * i], Rs[2 * i + 1])
    r[:, f] = None
    return r


def rect_aperture(r, Lx, Ly):
    filt = (r[0, :] ** 2 > Lx ** 2) * (r[2, :] ** 2 > Ly ** 2)
    r[:, filt] = None
    return r


def knife_edge(r, offset, axis, direction):
    a = 2 if axis == "y" else 0
    if direction > 0:
        filt = r[a, :] > offset
    elif direction < 0:
        filt = r[a, :] < offset
    else:
        return r
    r[:, filt] = None
    return r


def shadowgraphy(r0_mm, L, R, focal_plane=0.0):
    """Shadowgraphy.solve, ray_transfer_matrix.py:214-227."""
    r = distance(r0_mm, L - focal_plane)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    r = distance(r, L * 2)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    return distance(r, L)


def schlieren_df(r0_mm, L, R, Rstop=1.0, focal_plane=0.0):
    """Schlieren_DF.solve, ray_transfer_matrix.py:236-250."""
    r = distance(r0_mm, L - focal_plane)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    r = distance(r, L)
    r = circular_stop(r, Rstop)
    r = distance(r, L)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    return distance(r, L)


def schlieren_lf(r0_mm, L, R, Rstop=1.0, focal_plane=0.0):
    """Schlieren_LF.solve, ray_transfer_matrix.py:259-273."""
    r = distance(r0_mm, L - focal_plane)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    r = distance(r, L)
    r = circular_aperture(r, Rstop)
    r = distance(r, L)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    return distance(r, L)


def schlieren_knife(r0_mm, L, R, offset=0.0, axis="x", direction=1, focal_plane=0.0):
    """Knife-edge schlieren composed from reference pieces: Schlieren_DF's relay
    (ray_transfer_matrix.py:236-250) with the stop replaced by knife_edge (:138-154)."""
    r = distance(r0_mm, L - focal_plane)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    r = distance(r, L)
    r = knife_edge(r, offset, axis, direction)
    r = distance(r, L)
    r = circular_aperture(r, R)
    r = sym_lens(r, L)
    return distance(r, L)


def afr(r0_mm, L, R, Rs, focal_plane=0.0):
    """AFR.solve, ray_transfer_matrix.py:285-299."""
    r = distance(r0_mm, L / 2 - focal_plane)
    r = circular_aperture(r, R)
    r = sym_lens(r, L / 2)
    r = distance(r, L / 4)
    r = angular_filter(r, Rs)
    r = distance(r, L / 4)
    r = circular_aperture(r, R)
    r = sym_lens(r, L / 2)
    return distance(r, L / 2)


def histogram(rf_mm, Lx, Ly, bin_scale=10, pix_x=3448, pix_y=2574, weights=None):
    """Rays.histogram (ray_transfer_matrix.py:173-195): NaN rays dropped,
    histogram2d over [-Lx/2, Lx/2] x [-Ly/2, Ly/2], then transposed."""
    x = rf_mm[0, :]
    y = rf_mm[2, :]
    keep = ~(np.isnan(x) | np.isnan(y))
    w = None if weights is None else np.asarray(weights)[keep]
    H, xe, ye = np.histogram2d(x[keep], y[keep], bins=[pix_x // bin_scale, pix_y // bin_scale],
                               range=[[-Lx / 2, Lx / 2], [-Ly / 2, Ly / 2]], weights=w)
    return H.T, xe, ye


# ---------------------------------------------------------------------------
# gaussian_fields
# ---------------------------------------------------------------------------
def gaussian3D_FFT(N, k_func, Wr=None, Wi=None):
    """turboGen.gaussian3D_FFT (gaussian_fields/turboGen.py:488-537).  Noise is
    drawn from the global numpy state in the reference's order unless given."""
    M = 2 * N + 1
    k = np.fft.fftfreq(M)
    KX, KY, KZ = np.meshgrid(k, k, k)
    K = np.fft.fftshift(np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2))
    if Wr is None:
        Wr = np.random.randn(M, M, M)
    if Wi is None:
        Wi = np.random.randn(M, M, M)
    Wr = Wr + np.flip(Wr)
    Wi = Wi - np.flip(Wi)
    W = Wr + 1j * Wi
    with np.errstate(divide="ignore", invalid="ignore"):
        F = W * np.sqrt(k_func(K))
    Fs = np.fft.ifftshift(F)
    Fs[0, 0, 0] = 0
    return np.fft.ifftn(Fs).real


def spectrum_3D_scalar(data, dx, k_bin_num=100):
    """calculate_spectrum_3d.spectrum_3D_scalar (gaussian_fields/calculate_spectrum_3d.py:3-59):
    shell-averaged |FFT|^2 in k_bin_num bins of width K.max()/k_bin_num;
    bin i-1 holds (i-1) w <= K < i w for i = 1..k_bin_num-1, the last bin
    stays zero.  Computed with one bincount instead of a mask per bin."""
    f = np.fft.fftn(data)
    fsqr = (f * np.conj(f)).real
    Mx, My, Mz = data.shape
    kx = np.fft.fftfreq(Mx, dx)
    ky = np.fft.fftfreq(My, dx)
    kz = np.fft.fftfreq(Mz, dx)
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
    K = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2).ravel()
    w = K.max() / k_bin_num
    kb = w * np.arange(0, k_bin_num + 1)
    kbw = (0.5 * (kb[:-1] ** 3 + kb[1:] ** 3)) ** (1 / 3)
    # reference: bin i-1 keeps K < i*w and K >= (i-1)*w
    idx = np.floor(K / w).astype(np.int64)
    # guard the floor against rounding at exact multiples of w
    lo = idx * w
    idx = np.where(K < lo, idx - 1, idx)
    idx = np.where(K >= (idx + 1) * w, idx + 1, idx)
    sel = idx < (k_bin_num - 1)
    s = np.bincount(idx[sel], weights=fsqr.ravel()[sel], minlength=k_bin_num)[:k_bin_num]
    c = np.bincount(idx[sel], minlength=k_bin_num)[:k_bin_num]
    spect = np.zeros(k_bin_num)
    with np.errstate(invalid="ignore", divide="ignore"):
        spect[: k_bin_num - 1] = s[: k_bin_num - 1] / c[: k_bin_num - 1]
    return kbw, spect


# ---------------------------------------------------------------------------
# Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and Box-Muller
# ---------------------------------------------------------------------------
_PH_M0 = np.uint64(0xD2511F53)
_PH_M1 = np.uint64(0xCD9E8D57)
_PH_W0 = np.uint32(0x9E3779B9)
_PH_W1 = np.uint32(0xBB67AE85)
_MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 block function; counters are uint32 arrays."""
    c0 = np.asarray(c0, np.uint32)
    c1 = np.asarray(c1, np.uint32)
    c2 = np.asarray(c2, np.uint32)
    c3 = np.asarray(c3, np.uint32)
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    c0, c1, c2, c3 = c0.copy(), c1.copy(), c2.copy(), c3.copy()
    for r in range(10):
        p0 = _PH_M0 * c0.astype(np.uint64)
        p1 = _PH_M1 * c2.astype(np.uint64)
        hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
        lo0 = (p0 & _MASK32).astype(np.uint32)
        hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
        lo1 = (p1 & _MASK32).astype(np.uint32)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        if r < 9:
            k0 = np.uint32((int(k0) + int(_PH_W0)) & 0xFFFFFFFF)
            k1 = np.uint32((int(k1) + int(_PH_W1)) & 0xFFFFFFFF)
    return c0, c1, c2, c3


def box_muller(u0, u1):
    """Two standard normals from two uint32 words: u = (x + 0.5) 2^-32 in (0, 1)."""
    a = (u0.astype(np.float64) + 0.5) * (1.0 / 4294967296.0)
    b = (u1.astype(np.float64) + 0.5) * (1.0 / 4294967296.0)
    r = np.sqrt(-2.0 * np.log(a))
    th = 2.0 * np.pi * b
    return r * np.cos(th), r * np.sin(th)


def _mode_noise(lin, seed):
    k0 = seed & 0xFFFFFFFF
    k1 = (seed >> 32) & 0xFFFFFFFF
    lin = np.asarray(lin, np.uint64)
    c0 = (lin & _MASK32).astype(np.uint32)
    c1 = (lin >> np.uint64(32)).astype(np.uint32)
    o0, o1, _, _ = philox4x32_10(c0, c1, np.uint32(0), np.uint32(0x47524631), k0, k1)
    return box_muller(o0, o1)


def grf_spectrum_half(n, L, alpha, seed, kmin=None, kmax=None):
    """Half spectrum (n, n, n//2+1) of the benchmark-workload field.

    Modes are indexed by signed integer frequencies m (numpy.fft.fftfreq
    order, k = 2 pi m / L).  Complex Gaussian noise a + ib comes from
    Philox4x32-10 keyed by seed with counter = the mode's linear index in the
    half spectrum; on the kz = 0 (and, for even n, kz = n/2) planes the mode
    with the larger (ix, iy) linear index takes the conjugate of its partner's
    noise and self-paired modes are real.  Amplitude (m.m)^(alpha/4), i.e.
    |k|^(alpha/2) up to a constant, for kmin <= |k| <= kmax (band test done
    on the integer m.m; defaults 2 pi / L and pi n / L), zero elsewhere and
    at m = 0.  Same algorithm as the GPU generator."""
    h = n // 2 + 1
    kmin = 2 * np.pi / L if kmin is None else kmin
    kmax = np.pi * n / L if kmax is None else kmax
    mlo2 = (kmin * L / (2 * np.pi)) ** 2
    mhi2 = (kmax * L / (2 * np.pi)) ** 2
    ix = np.arange(n)[:, None, None]
    iy = np.arange(n)[None, :, None]
    iz = np.arange(h)[None, None, :]
    edge = (iz == 0) | ((n % 2 == 0) & (iz == h - 1))
    px = (n - ix) % n
    py = (n - iy) % n
    lin_self = ix * n + iy
    lin_part = px * n + py
    use_part = edge & (lin_part < lin_self)
    self_conj = edge & (lin_part == lin_self)
    six = np.where(use_part, px, ix)
    siy = np.where(use_part, py, iy)
    lin = np.broadcast_to(((six * n + siy) * h + iz).astype(np.uint64), (n, n, h))
    a, b = _mode_noise(lin.ravel(), seed)
    a = a.reshape(n, n, h)
    b = b.reshape(n, n, h)
    b = np.where(use_part, -b, b)
    b = np.where(self_conj, 0.0, b)
    m = np.concatenate([np.arange(0, (n - 1) // 2 + 1), np.arange(-(n // 2), 0)])  # fftfreq order
    m2 = (m[:, None, None] ** 2 + m[None, :, None] ** 2 + m[None, None, :h] ** 2).astype(np.float64)
    band = (m2 >= mlo2) & (m2 <= mhi2) & (m2 > 0)
    with np.errstate(divide="ignore"):
        amp = np.where(band, np.power(m2, alpha / 4.0), 0.0)
    return (a + 1j * b) * amp


def grf_unit(n, L, alpha, seed):
    """Unit-variance band-limited Gaussian random field g (n, n, n)."""
    F = grf_spectrum_half(n, L, alpha, seed)
    f = np.fft.irfftn(F, s=(n, n, n), axes=(0, 1, 2))
    f = f - f.mean()
    return f / np.sqrt(np.mean(f * f))


def workload_density(n, L, alpha, delta, ne0, seed):
    """n_e = ne0 (1 + delta g), clipped at >= 0, with coordinates linspace(-L/2, L/2, n)."""
    g = grf_unit(n, L, alpha, seed)
    ne = ne0 * (1.0 + delta * g)
    np.maximum(ne, 0.0, out=ne)
    x = np.linspace(-L / 2, L / 2, n)
    return ne, x


# ---------------------------------------------------------------------------
# gaussian_fields/turboGen.py: cosine-sum generators (:40-385), vectorised
# ---------------------------------------------------------------------------
def gaussian_cos(dim, l, n, nmodes, wn1, especf):
    """gaussian1Dcos / gaussian2Dcos / gaussian3Dcos with the reference's draws
    from the global numpy state (same order), summed over modes at once."""
    d = [li / ni for li, ni in zip(l, n)]
    wnn = max(np.pi / di for di in d)
    dk = (wnn - wn1) / nmodes
    wn = wn1 + 0.5 * dk + np.arange(0, nmodes) * dk
    dkn = np.ones(nmodes) * dk
    espec = especf(wn).clip(0.0)
    A = np.sqrt(2.0 * espec * dkn ** dim)
    c = [di / 2.0 + np.arange(0, ni) * di for di, ni in zip(d, n)]
    if dim == 1:
        phi = 2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes)
        np.random.uniform(0.0, 1.0, nmodes)
        arg = wn[None, :] * c[0][:, None] + phi
        return (A * np.sqrt(2.0) * np.cos(arg)).sum(-1)
    if dim == 2:
        phi, psi, theta = (2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes) for _ in range(3))
        kx, ky = np.cos(theta) * wn, np.sin(theta) * wn
        ax = kx * c[0][:, None, None]
        ay = ky * c[1][None, :, None]
        return (A * np.sqrt(2.0) * (np.cos(ax + ay + phi) + np.cos(ax - ay + psi))).sum(-1)
    p1, p2, p3, p4, theta, phi = (2.0 * np.pi * np.random.uniform(0.0, 1.0, nmodes) for _ in range(6))
    kx = np.sin(theta) * np.cos(phi) * wn
    ky = np.sin(theta) * np.sin(phi) * wn
    kz = np.cos(theta) * wn
    ax = kx * c[0][:, None, None, None]
    ay = ky * c[1][None, :, None, None]
    az = kz * c[2][None, None, :, None]
    return (A * np.sqrt(2.0) * (np.cos(ax + ay + az + p1) + np.cos(ax + ay - az + p2) +
                                np.cos(ax - ay + az + p3) + np.cos(ax - ay - az + p4))).sum(-1)


def gaussian_fft_nd(dim, N, k_func, Wr, Wi):
    """gaussian1D_FFT / gaussian2D_FFT / gaussian3D_FFT (turboGen.py:388-537) for
    given noise arrays (as the reference draws them)."""
    M = 2 * N + 1
    k = np.fft.fftfreq(M)
    if dim == 1:
        K = np.sqrt(k ** 2)
    elif dim == 2:
        KX, KY = np.meshgrid(k, k)
        K = np.sqrt(KX ** 2 + KY ** 2)
    else:
        KX, KY, KZ = np.meshgrid(k, k, k)
        K = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    K = np.fft.fftshift(K)
    W = (Wr + np.flip(Wr)) + 1j * (Wi - np.flip(Wi))
    with np.errstate(divide="ignore", invalid="ignore"):
        F = W * np.sqrt(k_func(K))
    F = np.fft.ifftshift(F)
    F[(0,) * dim] = 0
    return np.fft.ifftn(F).real
