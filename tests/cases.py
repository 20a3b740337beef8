"""Shared inputs for the parity tests: seeded fields and beams, and the oracle
runs they are compared with."""
import numpy as np

from oracle import restated as R
from oracle import tto

LWL = 1064e-9


def grf_case(n=32, L=2e-3, alpha=-11 / 3, delta=0.2, ne0=1e24, seed=1, nrays=256, sigma_frac=0.25,
             div=0.05e-3, ray_seed=0):
    """A config-1-shaped workload at small size: GRF density, Gaussian beam at -L/2."""
    ne, x = R.workload_density(n, L, alpha, delta, ne0, seed)
    rng = np.random.default_rng(ray_seed)
    s0 = R.gaussian_beam(nrays, sigma_frac * L, div, x.max(), rng)
    return ne, x, s0


def oracle_trace(ne, x, s0, rtol=1e-10, atol=1e-12, phase=True, lwl=LWL, y=None, z=None, direction="z"):
    y = x if y is None else y
    z = x if z is None else z
    om, q, gx, gy, gz = tto.calc_dndr(ne, x, y, z, lwl, 1.0)
    ext = {"x": x.max(), "y": y.max(), "z": z.max()}[direction]
    r = tto.trace(gx, gy, gz, x, y, z, s0, R.t_end(ext), rtol, atol,
                  ne_nc=q if phase else None, omega=om)
    r["rf"] = R.ray_at_exit(r["sf"], ext, direction)
    r["omega"] = om
    return r


def errors(rf, ref_rf, L, phase=None, ref_phase=None):
    e = dict(pos=np.nanmax(np.abs(rf[0::2] - ref_rf[0::2])) / L,
             ang=np.nanmax(np.abs(rf[1::2] - ref_rf[1::2])))
    if phase is not None:
        e["phase"] = np.nanmax(np.abs(phase - ref_phase))
    return e
