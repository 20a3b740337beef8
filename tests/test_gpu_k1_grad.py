"""K1 (calc_dndr, particle_tracker.py:220-241) on the GPU vs the reference's
own numpy arrays (golden fixtures) and vs the oracle; FP64 must be bit-exact."""
import glob
import os

import numpy as np
import pytest
import torch

from oracle import restated as R
from oracle import tto
from tests.cases import grf_case
from tests.conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "dndr_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_calc_dndr_bit_exact_vs_reference(cuda, path):
    from turbulence_tracing_gb300 import core

    d = np.load(path)
    f = core.calc_dndr(d["ne"], d["x"], d["y"], d["z"], float(d["lwl"]), float(d["ne_max"]))
    assert f["omega"] == float(d["omega"])
    for k in ("ne_nc", "dndx", "dndy", "dndz"):
        assert np.array_equal(f[k].cpu().numpy(), d[k]), k
    g = core.dndr([f["dndx"], f["dndy"], f["dndz"]], f["coords"], d["pts"]).cpu().numpy()
    assert np.array_equal(g, d["grad"])  # RegularGridInterpolator, operation by operation


def test_calc_dndr_bit_exact_vs_oracle_grf(cuda):
    from turbulence_tracing_gb300 import core

    ne, x, _ = grf_case(n=48, seed=5)
    y = np.linspace(-1e-3, 1.2e-3, 40)
    z = np.cumsum(np.linspace(1e-5, 3e-5, 36))
    ne = ne[:, :40, :36]
    f = core.calc_dndr(ne, x, y, z, 1064e-9, 1.0)
    om, q, gx, gy, gz = tto.calc_dndr(ne, x, y, z, 1064e-9, 1.0)
    for a, k in [(q, "ne_nc"), (gx, "dndx"), (gy, "dndy"), (gz, "dndz")]:
        assert np.array_equal(f[k].cpu().numpy(), a), k
    # float32 input: same as the oracle on the widened values
    f32 = core.calc_dndr(ne.astype(np.float32), x, y, z, 1064e-9, 1.0)
    om, q, gx, gy, gz = tto.calc_dndr(ne.astype(np.float32).astype(np.float64), x, y, z, 1064e-9, 1.0)
    assert np.array_equal(f32["dndz"].cpu().numpy(), gz)


def test_lookup_edges_nan_and_outside(cuda):
    from turbulence_tracing_gb300 import core

    d = golden("dndr_uniform")
    f = core.calc_dndr(d["ne"], d["x"], d["y"], d["z"], float(d["lwl"]), 1.0)
    x, y, z = d["x"], d["y"], d["z"]
    pts = np.array([[x[0], y[0], z[0]], [x[-1], y[-1], z[-1]], [np.nan, 0, 0], [x[-1] * 1.0000001, 0, 0],
                    [x[0], y[3], z[2]]]).T
    g = core.dndr([f["dndx"]], f["coords"], pts).cpu().numpy()[0]
    want = tto.interp(d["dndx"], x, y, z, pts)
    assert np.array_equal(g, want, equal_nan=True)
    assert np.isnan(g[2]) and g[3] == 0.0


def test_volume32_nodes(cuda):
    """FP32 brick volume: every stored node holds -0.5 d(ne_nc)/dx * spacing_c
    and ne_nc of its grid node, within FP32 rounding of the FP64 values."""
    from turbulence_tracing_gb300 import core

    ne, x, _ = grf_case(n=37, seed=2)
    y = np.linspace(-0.8e-3, 0.8e-3, 30)
    z = np.linspace(-1e-3, 1e-3, 21)
    ne = ne[:, :30, :21]
    for axis in (2, 0, 1):
        vol = core.build_volume(ne, x, y, z, probing_axis=axis, lwl=1064e-9)
        nodes = vol.nodes.cpu().numpy()
        om, q, gx, gy, gz = tto.calc_dndr(ne, x, y, z, 1064e-9, 1.0)
        c2 = R.C_LIGHT ** 2
        grads = [gx, gy, gz]
        desc = vol.desc
        axes = list(desc.axis)
        n = list(desc.n)
        dc = desc.spacing[2]
        tile_f4 = desc.bricks_c * 200
        st_b = desc.supertiles[1]

        def spread3(v):
            return (v & 1) | ((v & 2) << 1) | ((v & 4) << 2)

        rng = np.random.default_rng(axis)
        for _ in range(400):
            a, b, cc = (int(rng.integers(0, n[0])), int(rng.integers(0, n[1])), int(rng.integers(0, n[2])))
            ta, tb = min(a, n[0] - 2) >> 2, min(b, n[1] - 2) >> 2
            al, bl = a - 4 * ta, b - 4 * tb
            tile = ((ta >> 3) * st_b + (tb >> 3)) * 64 + (spread3(ta & 7) | (spread3(tb & 7) << 1))
            off = tile * tile_f4 + (cc >> 3) * 200 + (al * 5 + bl) * 8 + (cc & 7)
            phys = [0, 0, 0]
            for k, v in zip(axes, (a, b, cc)):
                phys[k] = v
            ix = tuple(phys)
            want = [grads[axes[k]][ix] / c2 * dc for k in range(3)] + [q[ix]]
            got = nodes[off]
            np.testing.assert_allclose(got, want, rtol=2e-5, atol=1e-6 * np.abs(want[:3]).max() + 1e-12)


def test_uniform_grid_required_for_fp32(cuda):
    from turbulence_tracing_gb300 import _lib, core

    x = np.cumsum(np.linspace(1, 2, 10))
    with pytest.raises(_lib.TTError):
        core.volume_plan((10, 10, 10), x, x, x, 2, 1064e-9)
