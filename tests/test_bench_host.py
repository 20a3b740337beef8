"""bench.py's host-side arithmetic, without a GPU: the trace roofline figures
derived from the committed counter capture, and the workload naming the
capture is keyed on."""
import argparse

import pytest

import bench


def _args(**kw):
    a = argparse.Namespace(n=512, rays=1e7, det=1024, L=5e-3, alpha=-5 / 3, delta=0.1, ne0=5e24, sigma=1.5e-3,
                           div=1e-4, lwl=1.064e-6, seed=2)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


def test_capture_is_keyed_on_the_default_workload():
    assert bench.workload_config(_args())["workload"] == bench.TRACE32_CAPTURE["workload"]
    assert bench.workload_config(_args(n=256, rays=1e6))["workload"] != bench.TRACE32_CAPTURE["workload"]


def test_trace_roofline_arithmetic():
    cap = bench.TRACE32_CAPTURE
    rs, sec, peak, sms, mhz = cap["ray_steps"], 0.17, 6800.0, 152, 2070.0
    r = bench.trace_roofline(cap["workload"], rs, sec, peak, "measured", sms, mhz)
    # the contract's figure: algorithmic bytes over the launch time, against the peak
    assert r["achieved"] == pytest.approx(rs * bench.ALG_BYTES_PHASE / sec / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    # DRAM bytes of the captured launch, unscaled for the captured workload
    assert r["traffic"] == cap["dram_read_bytes"] + cap["dram_write_bytes"]
    assert r["dram_frac"] == pytest.approx(r["traffic"] / sec / 1e9 / peak)
    # issue: warp instructions per ray-step x ray-steps/s over SMs x 4 schedulers x clock
    wipr = cap["warp_inst"] / cap["ray_steps"]
    assert r["issue_frac"] == pytest.approx(wipr * rs / sec / (sms * 4 * mhz * 1e6))
    assert 0.0 < r["issue_frac"] < 1.0
    # another workload: the captured bytes scale with its ray-steps, and it says so
    r2 = bench.trace_roofline("grf256_1e+06rays_phase_3det1024", rs // 20, sec / 20, peak, "measured", sms, mhz)
    assert r2["traffic"] == pytest.approx(r["traffic"] * (rs // 20) / rs)
    assert "scaled by ray-steps" in r2["traffic_source"]
