"""The benchmark's own workload (512^3 field, 1e7-ray beam) against the CPU
oracle: both GPU tracers on a sample of the very rays the benchmark traces.

Field: n_e = 5e24 (1 + 0.1 g) m^-3, g a unit-variance Gaussian random field
with |k|^-5/3 for 2 pi/L <= |k| <= pi 512/L, L = 5 mm, FP32 on the device
(seed 2, as bench.py).  Beam: the first rays of bench.py's 1e7-ray draw
(x, y ~ N(0, 1.5 mm), angles ~ N(0, 0.1 mrad), seed 2).  Oracle: the C
restatement of solve_ivp(RK45) per ray at rtol 1e-10 / atol 1e-12 with the
restated phase (tt_oracle.c), from the same FP32 density.

Bars (the benchmark spec): positions within 1e-6 of the box length, angles within
1 urad, phase within 1e-3 rad, on every ray."""
import numpy as np
import pytest
import torch

from oracle import restated as R
from oracle import tto
from tests.cases import errors

pytestmark = pytest.mark.gpu

N, L, ALPHA, DELTA, NE0, SEED = 512, 5e-3, -5.0 / 3.0, 0.1, 5e24, 2
SIGMA, DIV, LWL = 1.5e-3, 0.1e-3, 1064e-9
BEAM_RAYS = 10_000_000  # bench.py's draw; its first CHECK rays are checked
CHECK = 1500


@pytest.fixture(scope="module")
def workload(cuda):
    from turbulence_tracing_gb300 import turboGen

    ne, x = turboGen.workload_field(N, L, ALPHA, DELTA, NE0, seed=SEED, dtype=torch.float32)
    torch.cuda.synchronize()
    s0 = R.gaussian_beam(BEAM_RAYS, SIGMA, DIV, x.max(), np.random.default_rng(SEED))[:, :CHECK].copy()
    ne_h = ne.cpu().numpy()
    om, q, gx, gy, gz = tto.calc_dndr(ne_h, x, x, x, LWL, 1.0)
    ref = tto.trace(gx, gy, gz, x, x, x, s0, R.t_end(x.max()), 1e-10, 1e-12, ne_nc=q, omega=om)
    del q, gx, gy, gz
    assert (ref["status"] == 0).all()
    ref["rf"] = R.ray_at_exit(ref["sf"], x.max())
    return dict(ne=ne, x=x, s0=s0, ref=ref)


def test_fp32_tracer_meets_bars_on_benchmark_workload(workload):
    """The FP32 persistent tracer at the benchmark's tolerances (rtol 1e-7,
    atol 1e-5 cells, atol_phase 1e-5 rad, phase on)."""
    from turbulence_tracing_gb300 import core

    x, s0, ref = workload["x"], workload["s0"], workload["ref"]
    vol = core.build_volume(workload["ne"], x, x, x, probing_axis=2, lwl=LWL)
    out = core.trace_f32(vol, s0, R.t_end(x.max()), x.max(), rtol=1e-7, atol=1e-5, atol_phase=1e-5, phase=True)
    st = out["status"].cpu().numpy()
    assert (st == 0).all()
    e = errors(out["rf"].cpu().numpy(), ref["rf"], L, out["phase"].cpu().numpy(), ref["phase"])
    assert e["pos"] <= 1e-6 and e["ang"] <= 1e-6 and e["phase"] <= 1e-3, e
    # rays that meet the box take about one step per cell crossed
    n = out["nsteps"].cpu().numpy()
    assert np.median(n[n > 0]) <= 1.2 * N


def test_fp64_dropin_meets_bars_on_benchmark_workload(workload):
    """The plain FP64 drop-in at the tolerance the benchmark's equal-accuracy
    comparison uses (rtol 1e-10, atol 1e-13), against the oracle."""
    from turbulence_tracing_gb300 import core

    x, s0, ref = workload["x"], workload["s0"], workload["ref"]
    fields = core.calc_dndr(workload["ne"], x, x, x, lwl=LWL)
    out = core.trace_f64(fields, s0, R.t_end(x.max()), 2, x.max(), rtol=1e-10, atol=1e-13, phase=True)
    st = out["status"].cpu().numpy()
    assert (st == 0).all()
    e = errors(out["rf"].cpu().numpy(), ref["rf"], L, out["phase"].cpu().numpy(), ref["phase"])
    assert e["pos"] <= 1e-6 and e["ang"] <= 1e-6 and e["phase"] <= 1e-3, e
