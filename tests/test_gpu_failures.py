"""Failure paths, exercised without faulting the GPU.

- The per-ray step cap (tt_trace_opts.max_steps): both tracers stop a ray
  after that many attempted steps and report TT_RAY_MAX_STEPS, as the oracle
  does (it counts accepted + rejected steps the same way).
- solve_ivp's TOO_SMALL_STEP (particle_tracker.py:323 calls solve_ivp, which
  stops when the step falls below ten spacings of t): with the velocity
  tolerance at 1e-15 m/s (about 100 times below where it starts to bind), a ray that crosses the box's exit face, where the
  interpolated field jumps to the fill value 0, needs a step below that
  spacing; the FP64 drop-in reports TT_RAY_STEP_TOO_SMALL for exactly the rays
  the oracle does.
- The tensor-core kernels' bounded waits: a test entry point runs the row-DFT
  kernel with a short wait limit and without the copies of each block's first
  tile, so the tile barrier never completes.  Every block's wait runs out, the
  error flag is set, TMEM is freed and the kernel returns; the context stays
  usable and the next ordinary launch is correct.
"""
import numpy as np
import pytest
import torch

from oracle import restated as R
from oracle import tto
from tests.cases import LWL, grf_case

pytestmark = pytest.mark.gpu

RAY_OK, RAY_STEP_TOO_SMALL, RAY_MAX_STEPS = 0, 1, 2


def test_max_steps_both_tracers(cuda):
    from turbulence_tracing_gb300 import core

    ne, x, s0 = grf_case(n=24, nrays=64)
    s0[0, :4] = 5 * x.max()  # four rays miss the box
    t_end = R.t_end(x.max())
    om, q, gx, gy, gz = tto.calc_dndr(ne, x, x, x, LWL, 1.0)
    ref = tto.trace(gx, gy, gz, x, x, x, s0, t_end, 1e-10, 1e-12, max_steps=3)
    capped = ref["status"] == RAY_MAX_STEPS
    assert capped.mean() > 0.8 and not capped[:4].any()
    # FP64 drop-in: the oracle's algorithm, so the same rays run out of steps
    f = core.calc_dndr(ne, x, x, x, LWL, 1.0)
    o64 = core.trace_f64(f, s0, t_end, 2, x.max(), rtol=1e-10, atol=1e-12, max_steps=3)
    assert np.array_equal(o64["status"].cpu().numpy(), ref["status"])
    # FP32 tracer: a ray that crosses the box needs more than 3 steps; rays that
    # miss it are straight lines and take none
    vol = core.build_volume(ne, x, x, x, 2, lwl=LWL)
    o32 = core.trace_f32(vol, s0, t_end, x.max(), phase=True, max_steps=3)
    st = o32["status"].cpu().numpy()
    assert (st[:4] == RAY_OK).all() and (st[capped] == RAY_MAX_STEPS).all()
    assert set(np.unique(st)) <= {RAY_OK, RAY_MAX_STEPS}
    assert (o32["nsteps"].cpu().numpy() <= 3).all()
    # uncapped runs of the same rays finish
    assert (core.trace_f32(vol, s0, t_end, x.max())["status"] == RAY_OK).all()
    assert (core.trace_f64(f, s0, t_end, 2, x.max())["status"] == RAY_OK).all()


def test_step_too_small_fp64(cuda):
    from turbulence_tracing_gb300 import core

    ne, x, _ = grf_case(n=16, nrays=4)
    ext, dx, c = x.max(), x[1] - x[0], R.C_LIGHT
    s0 = np.zeros((6, 3))
    s0[:, 0] = [0.3 * ext, 0.1 * ext, ext - 1.5 * dx, 0.0, 0.0, c]          # 1.5 cells before the exit face
    s0[:, 1] = [-0.3 * ext, 0.2 * ext, -ext, 0.01 * c, 0.0, c * np.sqrt(1 - 1e-4)]  # through the whole box
    s0[:, 2] = [5 * ext, 0.0, -ext, 0.0, 0.0, c]                             # misses the box: no jump
    rtol, atol = 1e-30, 1e-15  # the crossing needs a step below 10 spacings of t from atol ~2e-13 down
    t_end = R.t_end(ext)
    f = core.calc_dndr(ne, x, x, x, LWL, 1.0)
    out = core.trace_f64(f, s0, t_end, 2, ext, rtol=rtol, atol=atol)
    om, q, gx, gy, gz = tto.calc_dndr(ne, x, x, x, LWL, 1.0)
    ref = tto.trace(gx, gy, gz, x, x, x, s0, t_end, rtol, atol)
    st = out["status"].cpu().numpy()
    assert list(ref["status"]) == [RAY_STEP_TOO_SMALL, RAY_STEP_TOO_SMALL, RAY_OK]
    assert list(st) == list(ref["status"])
    # the state is left where the step size ran out: at the exit face, inside the box
    sf = out["sf"].cpu().numpy()
    assert np.all(np.abs(sf[2, :2] - ext) < 1e-3 * dx)


def test_tensor_core_wait_timeout_sets_error_flag(cuda):
    from turbulence_tracing_gb300 import _lib, core, fno

    S, rows = 128, 128 * 40
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn((rows, S), device="cuda", generator=g).to(torch.bfloat16)
    Mf = torch.randn((32, S), device="cuda", generator=g)
    M = fno.pack(Mf)
    out = torch.zeros((rows, 32), dtype=torch.float32, device="cuda")
    ws = torch.zeros(256, dtype=torch.uint8, device="cuda")
    L = _lib.lib()
    _lib.check(L.tt_fno_rowdft_timeout_test(S, rows, core._ptr(x), core._ptr(M), core._ptr(out), core._ptr(ws),
                                            100_000, core._stream()), "tt_fno_rowdft_timeout_test")
    torch.cuda.synchronize()
    assert fno.error_flag(ws) == 1
    assert float(out.abs().max()) == 0.0  # the aborted blocks wrote nothing
    # bad limits are refused before any launch
    assert L.tt_fno_rowdft_timeout_test(S, rows, core._ptr(x), core._ptr(M), core._ptr(out), core._ptr(ws), 10,
                                        core._stream()) == 1
    # the context is still usable: the ordinary launch is correct with a fresh flag
    ref = x.double() @ Mf.to(torch.bfloat16).double().T
    got, ws2 = fno.rowdft(S, x, M)
    assert fno.error_flag(ws2) == 0
    assert float((got.double() - ref).abs().max()) <= 1e-5 * float(ref.abs().max())

