"""The reference's CPU path, restated with its current API, for timing.

TEST INFRASTRUCTURE / CPU BASELINE ONLY.  bench.py times this as the
reference arm and as its cpu_baseline leg; nothing in the product uses it.

What runs is what particle_tracking/particle_tracker.py does:
  calc_dndr (:220-241)  numpy ne/nc clip + np.gradient x3 + RegularGridInterpolator x3
  solve     (:312-331)  one RK45 system over a whole ray bundle (one global step,
                        rtol 1e-3 / atol 1e-6 unless given), dsdt (:398-419)
                        and dndr (:243-256) as the right-hand side
  ray_at_exit (:333-380)
spread over host processes the way particle_tracking/example_multiprocess.py
does (Pool.map over ray bundles, :44-51), with the cube shared by fork
(the stale script pickles it per task; fork sharing is cheaper, not slower).
Accepted steps are counted by driving scipy's RK45 solver object directly
(the loop solve_ivp runs); ray-steps = accepted global steps x rays.

Run as a module to time a sample from a density file without touching CUDA:
  python -m oracle.ref_path --density ne.npy --L 5e-3 --rays 2000 --json out.json
"""
import argparse
import json
import multiprocessing as mp
import os
import time

import numpy as np
from scipy.integrate import RK45
from scipy.interpolate import RegularGridInterpolator

from . import restated as R

_CUBE = None


class RefCube:
    def __init__(self, ne, x, y, z, lwl=1064e-9, ne_max=1.0):
        self.x, self.y, self.z = x, y, z
        omega = 2 * np.pi * (R.C_LIGHT / lwl)
        nc = 3.14207787e-4 * omega ** 2
        ne_nc = np.asarray(ne, dtype=np.float64) / nc
        ne_nc[ne_nc > ne_max] = ne_max
        k = -0.5 * R.C_LIGHT ** 2
        self.dndx = k * np.gradient(ne_nc, x, axis=0)
        self.dndy = k * np.gradient(ne_nc, y, axis=1)
        self.dndz = k * np.gradient(ne_nc, z, axis=2)
        self.ix = RegularGridInterpolator((x, y, z), self.dndx, bounds_error=False, fill_value=0.0)
        self.iy = RegularGridInterpolator((x, y, z), self.dndy, bounds_error=False, fill_value=0.0)
        self.iz = RegularGridInterpolator((x, y, z), self.dndz, bounds_error=False, fill_value=0.0)

    def dndr(self, p):
        g = np.zeros_like(p)
        g[0, :] = self.ix(p.T)
        g[1, :] = self.iy(p.T)
        g[2, :] = self.iz(p.T)
        return g


def dsdt(t, s, cube):
    Np = s.size // 6
    s = s.reshape(6, Np)
    sp = np.zeros_like(s)
    sp[3:6, :] = cube.dndr(s[:3, :])
    sp[:3, :] = s[3:, :]
    return sp.flatten()


def solve_bundle(s0, t_end, rtol=1e-3, atol=1e-6, cube=None):
    """One solve() over a bundle: returns (sf, accepted_steps, nfev)."""
    cube = cube or _CUBE
    solver = RK45(lambda t, y: dsdt(t, y, cube), 0.0, s0.flatten(), t_end, rtol=rtol, atol=atol)
    steps = 0
    while solver.status == "running":
        solver.step()
        steps += 1
    return solver.y.reshape(6, -1), steps, solver.nfev


def _work(args):
    s0, t_end, rtol, atol = args
    t0 = time.perf_counter()
    sf, steps, nfev = solve_bundle(s0, t_end, rtol, atol)
    return sf, steps, nfev, time.perf_counter() - t0


def run_pool(cube, s0, t_end, nproc, bundle=None, rtol=1e-3, atol=1e-6):
    """Trace s0 in bundles over nproc forked workers.  Returns dict with rf,
    ray_steps (sum of accepted global steps x bundle size) and wall time."""
    global _CUBE
    _CUBE = cube
    Np = s0.shape[1]
    bundle = bundle or max(1, -(-Np // nproc))
    chunks = [(s0[:, i:i + bundle], t_end, rtol, atol) for i in range(0, Np, bundle)]
    ctx = mp.get_context("fork")
    t0 = time.perf_counter()
    with ctx.Pool(nproc) as pool:
        res = pool.map(_work, chunks)
    wall = time.perf_counter() - t0
    sf = np.concatenate([r[0] for r in res], axis=1)
    ray_steps = sum(r[1] * c[0].shape[1] for r, c in zip(res, chunks))
    return dict(sf=sf, rf=R.ray_at_exit(sf, cube.z.max()), ray_steps=int(ray_steps), wall=wall,
                nfev=sum(r[2] for r in res), steps=[r[1] for r in res])


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--density", required=True, help=".npy (n, n, n) density, m^-3")
    ap.add_argument("--L", type=float, required=True, help="box side (m); coords linspace(-L/2, L/2, n)")
    ap.add_argument("--rays", type=int, default=2000)
    ap.add_argument("--sigma", type=float, required=True)
    ap.add_argument("--div", type=float, required=True)
    ap.add_argument("--lwl", type=float, default=1064e-9)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--procs", type=int, default=0)
    ap.add_argument("--rtol", type=float, default=1e-3, help="solve_ivp rtol (the reference's default 1e-3)")
    ap.add_argument("--atol", type=float, default=1e-6, help="solve_ivp atol (the reference's default 1e-6)")
    ap.add_argument("--bundle", type=int, default=0, help="rays per solve_ivp call (0: rays / procs)")
    ap.add_argument("--json", required=True)
    a = ap.parse_args(argv)
    ne = np.load(a.density, mmap_mode="r")
    n = ne.shape[0]
    x = np.linspace(-a.L / 2, a.L / 2, n)
    t0 = time.perf_counter()
    cube = RefCube(ne, x, x, x, lwl=a.lwl)
    t_setup = time.perf_counter() - t0
    s0 = R.gaussian_beam(a.rays, a.sigma, a.div, x.max(), np.random.default_rng(a.seed))
    nproc = a.procs or host_cores()
    r = run_pool(cube, s0, R.t_end(x.max()), nproc, bundle=a.bundle or None, rtol=a.rtol, atol=a.atol)
    out = dict(ray_steps=r["ray_steps"], wall=r["wall"], rays=a.rays, procs=nproc, setup_s=t_setup,
               ray_steps_per_s=r["ray_steps"] / r["wall"], rays_per_s=a.rays / r["wall"], rtol=a.rtol, atol=a.atol,
               bundle=a.bundle or -(-a.rays // nproc))
    with open(a.json, "w") as f:
        json.dump(out, f)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
