"""Generate golden fixtures by running the reference implementation itself.

Run in a checkout where the reference repository is available:
    python tests/golden/make_golden.py <reference checkout> [fixture names]
It imports particle_tracking/particle_tracker.py, ray_transfer_matrix.py
(with a stub matplotlib, which the reference imports only for plotting) and
gaussian_fields/turboGen.py + calculate_spectrum_3d.py, runs them on small
seeded inputs and writes tests/golden/*.npz.  The fixtures are committed; the
tests read only the .npz files.
"""
import os
import sys
import types

import numpy as np
from scipy.integrate import solve_ivp

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(root):
    mpl = types.ModuleType("matplotlib")
    mpl.patches = types.SimpleNamespace()
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    sys.path.insert(0, os.path.join(root, "particle_tracking"))
    sys.path.insert(0, os.path.join(root, "gaussian_fields"))
    import particle_tracker as pt  # noqa: E402
    import ray_transfer_matrix as rtm  # noqa: E402
    import turboGen  # noqa: E402
    import calculate_spectrum_3d as cs3  # noqa: E402
    return pt, rtm, turboGen, cs3


def small_field(n, L, seed, ne0=1e24, delta=0.2):
    """A smooth random density on an n^3 linspace grid (sum of a few random
    Fourier modes); only used as a fixture input."""
    rng = np.random.default_rng(seed)
    x = np.linspace(-L / 2, L / 2, n)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    g = np.zeros_like(X)
    for _ in range(6):
        k = rng.normal(0, 2 * np.pi / L * 2, 3)
        g += np.cos(k[0] * X + k[1] * Y + k[2] * Z + rng.uniform(0, 2 * np.pi))
    g /= g.std()
    return np.maximum(ne0 * (1 + delta * g), 0.0), x


def main(root, only=None):
    pt, rtm, turboGen, cs3 = _import_reference(root)
    out = {}

    # --- calc_dndr on uniform, non-uniform and clipped grids (particle_tracker.py:220-241)
    rng = np.random.default_rng(1)
    cases = {}
    x = np.linspace(-1e-3, 1e-3, 9)
    y = np.linspace(-2e-3, 2e-3, 7)
    z = np.linspace(-1.5e-3, 1.5e-3, 6)
    cases["uniform"] = (x, y, z, 1e24 * (1 + 0.2 * rng.standard_normal((9, 7, 6))), 1053e-9, 1.0)
    xn = np.sort(rng.uniform(-1e-3, 1e-3, 8))
    yn = np.cumsum(rng.uniform(0.5e-4, 2e-4, 5))
    zn = np.linspace(0, 1e-3, 4) ** 1.5
    cases["nonuniform"] = (xn, yn, zn, 1e25 * rng.uniform(0.5, 1.5, (8, 5, 4)), 1064e-9, 1.0)
    cases["clipped"] = (x, y, z, 1e27 * rng.uniform(0.0, 2.5, (9, 7, 6)), 1053e-9, 1.0)
    cases["clip_half"] = (x, y, z, 1e27 * rng.uniform(0.0, 2.5, (9, 7, 6)), 1053e-9, 0.5)
    ar = np.arange(-5e-3, 5e-3, 1e-3)
    cases["arange"] = (ar, ar[:6], ar[:7], 1e24 * rng.uniform(0.5, 1.5, (ar.size, 6, 7)), 1053e-9, 1.0)
    for name, (cx, cy, cz, ne, lwl, ne_max) in cases.items():
        cube = pt.ElectronCube(cx, cy, cz)
        cube.external_ne(ne.copy())
        cube.calc_dndr(lwl=lwl, ne_max=ne_max)
        pts = np.stack([rng.uniform(cx.min() - 1e-4, cx.max() + 1e-4, 64),
                        rng.uniform(cy.min() - 1e-4, cy.max() + 1e-4, 64),
                        rng.uniform(cz.min() - 1e-4, cz.max() + 1e-4, 64)])
        pts[0, :8] = cx[rng.integers(0, cx.size, 8)]
        pts[1, 8:16] = cy[-1]
        pts[2, 16:24] = cz[0]
        pts[:, 24] = [cx[-1], cy[-1], cz[-1]]
        pts[:, 25] = [cx[0], cy[0], cz[0]]
        out[f"dndr_{name}"] = dict(x=cx, y=cy, z=cz, ne=ne, lwl=lwl, ne_max=ne_max, omega=cube.omega,
                                   ne_nc=cube.ne_nc, dndx=cube.dndx, dndy=cube.dndy, dndz=cube.dndz,
                                   pts=pts, grad=cube.dndr(pts))

    # --- test densities (particle_tracker.py:147-210)
    xs = np.linspace(-5e-3, 5e-3, 11)
    for name, kw in [("test_null", {}), ("test_slab", dict(s=8, n_e0=1e25)),
                     ("test_linear_cos", dict(s1=0.1, s2=0.1, n_e0=2e23, Ly=1)),
                     ("test_exponential_cos", dict(n_e0=1e24, Ly=1e-3, s=2e-3)),
                     ("test_lens", dict(n_e0=5e25, LR=1e-3)), ("test_liner", dict(n_e0=2e27, LR=1e-3))]:
        cube = pt.ElectronCube(xs, xs * 0.8, xs * 1.2)
        getattr(cube, name)(**kw)
        out[f"dens_{name}"] = dict(ne=cube.ne)

    # --- init_beam with the global numpy state (particle_tracker.py:258-310)
    for d in "xyz":
        cube = pt.ElectronCube(xs, xs * 0.8, xs * 1.2, probing_direction=d)
        np.random.seed(7)
        cube.init_beam(Np=50, beam_size=2e-3, divergence=5e-3)
        out[f"beam_{d}"] = dict(s0=cube.s0, extent=cube.extent)

    # --- ray_at_exit for the three probing directions (:333-380)
    sf = np.vstack([rng.uniform(-1e-3, 1e-3, (3, 40)), 3e8 * rng.uniform(0.2, 1.0, (3, 40))])
    for d in "xyz":
        cube = pt.ElectronCube(xs, xs, xs, probing_direction=d)
        cube.extent = 4e-3
        cube.sf = sf
        out[f"exit_{d}"] = dict(sf=sf, extent=4e-3, rf=cube.ray_at_exit())

    # --- full trace through the reference's dsdt at rtol 1e-10 (:312-331, :398-419)
    for name, n, L, np_, seed in [("grf16", 16, 2e-3, 24, 3), ("grf12_strong", 12, 1e-3, 16, 4)]:
        ne, cx = small_field(n, L, seed, ne0=1e24 if name == "grf16" else 2e25)
        cube = pt.ElectronCube(cx, cx, cx)
        cube.external_ne(ne)
        cube.calc_dndr(lwl=1064e-9)
        np.random.seed(seed)
        cube.init_beam(Np=np_, beam_size=0.35 * L, divergence=2e-3)
        s0 = cube.s0.copy()
        tend = np.linspace(0.0, np.sqrt(8.0) * cube.extent / pt.c, 2)[-1]
        sol = solve_ivp(lambda t, y: pt.dsdt(t, y, cube), [0, tend], s0.flatten(),
                        t_eval=[0, tend], method="RK45", rtol=1e-10, atol=1e-12)
        cube.sf = sol.y[:, -1].reshape(6, np_)
        rf_tight = cube.ray_at_exit()
        sf_tight = cube.sf.copy()
        cube.s0 = s0.copy()
        rf_def = cube.solve()
        out[f"trace_{name}"] = dict(x=cx, ne=ne, s0=s0, t_end=tend, lwl=1064e-9,
                                    sf_tight=sf_tight, rf_tight=rf_tight,
                                    sf_default=cube.sf, rf_default=rf_def)

    # --- slab with a closed-form trajectory (notebook cells 6-9)
    xs = np.linspace(-5e-3, 5e-3, 21)
    cube = pt.ElectronCube(xs, xs, xs)
    cube.test_slab(s=8, n_e0=1e25)
    cube.calc_dndr()
    np.random.seed(11)
    cube.init_beam(Np=20, beam_size=2e-3, divergence=10e-3)
    s0 = cube.s0.copy()
    rf = cube.solve()
    out["slab_default"] = dict(x=xs, s0=s0, rf=rf, sf=cube.sf)

    # --- ray transfer matrices and histograms (ray_transfer_matrix.py:37-299)
    r = np.vstack([rng.normal(0, 2e-3, 4000), rng.normal(0, 4e-3, 4000),
                   rng.normal(0, 2e-3, 4000), rng.normal(0, 4e-3, 4000)])
    r[:, :5] = np.nan
    r[0, 5:10] = 0.0
    rtm_out = {"r0": r}
    for cls, kw, sv in [("Shadowgraphy", dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6), {}),
                        ("Schlieren_DF", dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6), dict(R=3)),
                        ("Schlieren_LF", dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6), dict(R=3)),
                        ("AFR", dict(focal_plane=5, L=100, R=25, Lx=15, Ly=10),
                         dict(Rs=np.arange(0, 6, 0.5)))]:
        obj = getattr(rtm, cls)(r0=r.copy(), **kw)
        obj.solve(**sv)
        obj.histogram(bin_scale=25)
        rtm_out[f"{cls}_rf"] = obj.rf
        rtm_out[f"{cls}_H"] = obj.H
        rtm_out[f"{cls}_xe"] = obj.xedges
        rtm_out[f"{cls}_ye"] = obj.yedges
        obj2 = getattr(rtm, cls)(r0=r.copy(), **kw)
        obj2.solve(**sv)
        obj2.histogram(bin_scale=10, pix_x=500, pix_y=300)
        rtm_out[f"{cls}_H2"] = obj2.H
    rr = r.copy() * 1e3
    rtm_out["knife_x_pos"] = rtm.knife_edge(rr.copy(), 0.5, "x", 1)
    rtm_out["knife_y_neg"] = rtm.knife_edge(rr.copy(), -0.5, "y", -1)
    rtm_out["rect"] = rtm.rect_aperture(rr.copy(), 2.0, 3.0)
    rtm_out["lens"] = rtm.lens(rr.copy(), 100.0, 50.0)
    rtm_out["dist"] = rtm.distance(rr.copy(), 123.0)
    out["rtm"] = rtm_out

    # --- gaussian3D_FFT with the global numpy state (turboGen.py:488-537)
    def k41(k):
        return k ** (-5 / 3)

    np.random.seed(1234)
    sig = turboGen.gaussian3D_FFT(6, k41)
    np.random.seed(1234)
    M = 13
    Wr = np.random.randn(M, M, M)
    Wi = np.random.randn(M, M, M)
    out["grf_fft"] = dict(N=6, signal=sig, Wr=Wr, Wi=Wi)

    # --- cosine-sum generators and the 1D / 2D FFT generators (turboGen.py:40-485)
    def k53(k):
        return k ** (-5 / 3)

    tg = {}
    np.random.seed(11)
    tg["cos1"] = turboGen.gaussian1Dcos(1.0, 64, 50, 2 * np.pi, k53)
    np.random.seed(12)
    tg["cos2"] = turboGen.gaussian2Dcos(1.0, 0.8, 32, 24, 40, 2 * np.pi, k53)
    np.random.seed(13)
    tg["cos3"] = turboGen.gaussian3Dcos(1.0, 0.9, 0.8, 16, 12, 10, 30, 2 * np.pi, k53)
    np.random.seed(14)
    tg["fft1"] = turboGen.gaussian1D_FFT(20, k41)
    np.random.seed(15)
    tg["fft2"] = turboGen.gaussian2D_FFT(8, k41)
    out["turbogen_more"] = tg

    # --- spectrum_3D_scalar (calculate_spectrum_3d.py:3-59)
    d = np.random.default_rng(5).standard_normal((11, 9, 13))
    kb, sp = cs3.spectrum_3D_scalar(d, 0.5, k_bin_num=20)
    out["spectrum"] = dict(data=d, dx=0.5, kb=kb, sp=sp)

    for name, arrs in out.items():
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                            **{k: np.asarray(v) for k, v in arrs.items()})
    print("wrote", len(out), "fixtures")


if __name__ == "__main__":
    # python make_golden.py [reference root] [fixture names to (re)write ...]
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout> [fixture names ...]")
    main(sys.argv[1], only=set(sys.argv[2:]) or None)
