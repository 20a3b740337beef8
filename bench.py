"""Benchmark: ray-steps/s of the GB300 ray-integration path.

Workload (default): 512^3 Gaussian-random-field density (|k|^-5/3 for
2 pi/L <= |k| <= pi n/L, L = 5 mm, n_e = 5e24 (1 + 0.1 g), FP32), 1e7 rays at
1064 nm (x, y ~ N(0, 1.5 mm), angles ~ N(0, 0.1 mrad)), phase on, then
1024 x 1024 shadowgraphy, knife-edge schlieren (knife at x = 0) and
interferometry (phase-weighted) detectors.  Synthetic, seeded inputs.

One step = K1 FP32 volume build + K2b persistent FP32 trace of all rays +
K3 three detectors, inputs resident in HBM (density 0.5 GB, volume 3.4 GB,
rays 0.5 GB: all larger than the 129 MB L2, so no flush is needed).
value = accepted ray-steps (one ray-step = one accepted Dormand-Prince step of
one ray) per second over the timed steps.  e2e = the same through the public
API (ElectronCube.solve + ray_transfer_matrix diagnostics) from pinned host
rays to host results.  Beside it: the plain FP64 drop-in on a ray subset at
the accuracy bar, the FP32 error against FP64, the roofline of the trace
kernel, and the reference's CPU path timed on this host.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun each rank traces its own replica (weak scaling).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "ray-steps/s at 512^3, 1e7 rays (FP32 persistent tracer, phase on, <=1 urad vs FP64)"
UNIT = "ray-steps/s"
ALG_BYTES_PHASE = 768  # 6 stages x 8 corners x 4 components x 4 B per ray-step (phase needs ne_nc)
# Counters of one trace32_kernel launch on the default workload from a one-pass
# ncu capture of this build (command and figures in
# profiles/trace32_grf512_1e7rays_counters.md): warp instructions issued and
# DRAM bytes.  The bench line scales them by accepted ray-steps for other
# workloads and says so.
TRACE32_CAPTURE = {"workload": "grf512_1e+07rays_phase_3det1024", "ray_steps": 4225457556,
                   "warp_inst": 143832795789, "dram_read_bytes": 20968995072, "dram_write_bytes": 6026149376}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--rays", type=float, default=1e7)
    ap.add_argument("--L", type=float, default=5e-3)
    ap.add_argument("--alpha", type=float, default=-5.0 / 3.0)
    ap.add_argument("--delta", type=float, default=0.1)
    ap.add_argument("--ne0", type=float, default=5e24)
    ap.add_argument("--sigma", type=float, default=1.5e-3)
    ap.add_argument("--div", type=float, default=0.1e-3)
    ap.add_argument("--lwl", type=float, default=1064e-9)
    ap.add_argument("--det", type=int, default=1024)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--block", type=int, default=0, help="FP32 tracer threads per block (0 = the library's 256)")
    ap.add_argument("--brick-depth", type=int, default=0, help="node-volume brick depth, 4..32 (0 = the library's 8)")
    ap.add_argument("--refill", type=int, default=0, help="FP32 tracer refill_lanes, 1..32 (0 = the library's 2)")
    ap.add_argument("--fp64-rays", type=int, default=1000000)
    ap.add_argument("--check-rays", type=int, default=20000)
    ap.add_argument("--cpu-rays", type=int, default=8000)
    ap.add_argument("--cpu-bar-rays", type=int, default=128, help="CPU sample at the accuracy-bar tolerance")
    ap.add_argument("--ref-rays", type=int, default=8000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=64)
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--sur-size", type=int, default=256)
    ap.add_argument("--sur-train", type=int, default=2048)
    ap.add_argument("--sur-test", type=int, default=96)
    ap.add_argument("--sur-epochs", type=int, default=15)
    ap.add_argument("--sur-batch", type=int, default=16, help="fields per chunk in the surrogate pipeline")
    ap.add_argument("--sur-time", type=int, default=96, help="fresh fields for timing the pipeline")
    ap.add_argument("--sur-stride", type=int, default=1, help="node planes per march step (1 or 2)")
    ap.add_argument("--no-stress", action="store_true", help="skip the stress workload (1024^3, 1e8 rays)")
    ap.add_argument("--stress-n", type=int, default=1024)
    ap.add_argument("--stress-rays", type=float, default=1e8)
    ap.add_argument("--stress-chunk", type=float, default=1e7)
    ap.add_argument("--stress-check", type=int, default=2000, help="rays of the first chunk checked against FP64")
    ap.add_argument("--no-screen", action="store_true", help="skip the per-tile screening of the stress field")
    ap.add_argument("--screen-n", type=int, default=1024, help="stress-field grid for the tile screening leg")
    ap.add_argument("--screen-train", type=int, default=8, help="training fields (16 tiles each at 1024^3)")
    ap.add_argument("--fp64-only", action="store_true",
                    help="time only the plain FP64 drop-in on all --rays rays (--fp64-rtol/--fp64-atol)")
    ap.add_argument("--fp64-rtol", type=float, default=1e-10)
    ap.add_argument("--fp64-atol", type=float, default=1e-13)
    ap.add_argument("--json-out", default="")
    return ap.parse_args()


def workload_config(a):
    return {"workload": "grf%d_%grays_phase_3det%d" % (a.n, a.rays, a.det), "grid": [a.n] * 3, "L_m": a.L,
            "spectrum_exponent": a.alpha, "delta": a.delta, "ne0_m3": a.ne0, "rays": int(a.rays),
            "beam_sigma_m": a.sigma, "divergence_rad": a.div, "lwl_m": a.lwl,
            "detectors": ["shadowgraphy", "schlieren_knife_x0", "interferometry"], "detector_bins": [a.det, a.det],
            "detector_extent_mm": 8.0 * a.sigma * 1e3, "optics_f_mm": 100.0, "aperture_mm": 25.0,
            "fp32_tol": {"rtol": 1e-7, "atol_cells": 1e-5, "atol_phase": 1e-5}, "seed": a.seed,
            "l2": "inputs larger than L2 (density 0.5 GB, node volume 3.4 GB, rays 0.5 GB); no flush"}


# ---------------------------------------------------------------------------- helpers
def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        for line in self.f:
            p = [s.strip() for s in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def across_ranks(units, seconds, dist, dev):
    """Whole-job units and time over the replicas (one rank per GPU, each on
    its own inputs): units summed, seconds maximised over ranks.  Without a
    process group the local values are returned."""
    if not dist:
        return units, seconds
    import torch

    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item())


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------- our arm
def run_ours(a):
    import torch

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from turbulence_tracing_gb300 import core, turboGen
    from turbulence_tracing_gb300 import particle_tracker as pt
    from turbulence_tracing_gb300 import ray_transfer_matrix as rtm
    from turbulence_tracing_gb300 import _lib

    dev = torch.device("cuda", local)
    n, L = a.n, a.L
    Np = int(a.rays)
    ne, x = turboGen.workload_field(n, L, a.alpha, a.delta, a.ne0, seed=a.seed + rank, dtype=torch.float32)
    ext = float(x.max())
    t_end = float(np.linspace(0.0, np.sqrt(8.0) * ext / 299792458.0, 2)[-1])
    rng = np.random.default_rng(a.seed + 1000 * rank)
    s0_host = np.empty((6, Np))
    s0_host[0] = rng.normal(0.0, a.sigma, Np)
    s0_host[1] = rng.normal(0.0, a.sigma, Np)
    s0_host[2] = -ext
    tx = np.tan(rng.normal(0.0, a.div, Np))
    ty = np.tan(rng.normal(0.0, a.div, Np))
    nrm = np.sqrt(1.0 + tx * tx + ty * ty)
    s0_host[3] = 299792458.0 * tx / nrm
    s0_host[4] = 299792458.0 * ty / nrm
    s0_host[5] = 299792458.0 / nrm
    del tx, ty, nrm
    s0 = torch.as_tensor(s0_host, device=dev)

    det = a.det
    ext_mm = 4.0 * a.sigma * 1e3  # +-4 beam sigma (6 mm for the default 1.5 mm beam)
    f_mm, R_mm = 100.0, 25.0
    relay = lambda mid: ([(_lib.OPTIC_M_TO_MM, 0, 0, 0), (_lib.OPTIC_DISTANCE, f_mm, 0, 0),
                          (_lib.OPTIC_CIRC_APERTURE, R_mm, 0, 0), (_lib.OPTIC_LENS, f_mm, f_mm, 0),
                          (_lib.OPTIC_DISTANCE, f_mm, 0, 0)] + mid +
                         [(_lib.OPTIC_DISTANCE, f_mm, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R_mm, 0, 0),
                          (_lib.OPTIC_LENS, f_mm, f_mm, 0), (_lib.OPTIC_DISTANCE, f_mm, 0, 0)])
    chain_shadow = relay([])
    chain_knife = relay([(_lib.OPTIC_KNIFE_EDGE, 0.0, 0, 1.0)])
    H = [torch.empty((det, det), dtype=torch.float64, device=dev) for _ in range(3)]
    Hw = torch.empty((det, det), dtype=torch.float64, device=dev)
    rng_mm = (-ext_mm, ext_mm)

    # persistent buffers so the timed steps allocate nothing
    vol = core.build_volume(ne, x, x, x, probing_axis=2, lwl=a.lwl, brick_depth=a.brick_depth or 8)
    out = core._ray_outputs(Np, dev, want_sf=True)
    ws_bytes = _lib.lib().tt_trace_f32_workspace_bytes(__import__("ctypes").byref(vol.desc), Np)
    wsp = core.workspace(ws_bytes, dev)
    tr_ev = []

    def step(record=False):
        L_ = _lib.lib()
        import ctypes

        _lib.check(L_.tt_volume_build(ctypes.byref(vol.desc), ctypes.c_void_p(ne.data_ptr()), _lib.TT_F32,
                                      core._stream()), "tt_volume_build")
        e0 = e1 = None
        if record:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
        core.trace_f32(vol, s0, t_end, ext, rtol=1e-7, atol=1e-5, atol_phase=1e-5, phase=True, ws=wsp, out=out,
                       block_size=a.block, refill_lanes=a.refill)
        if record:
            e1.record()
            tr_ev.append((e0, e1))
        core.detect(out["rf"], chain_shadow, det, det, rng_mm, rng_mm, H=H[0])
        core.detect(out["rf"], chain_knife, det, det, rng_mm, rng_mm, H=H[1])
        core.detect(out["rf"], chain_shadow, det, det, rng_mm, rng_mm, weights=out["phase"], H=H[2], Hw=Hw)

    launches_per_step = 1 + 4 + 3  # volume build; bin count/scan/scatter + trace; three detector kernels
    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    ray_steps_step = int(out["nsteps"].sum().item())
    st = out["status"]
    n_bad = int((st != 0).sum().item())

    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(a.steps):
        step(record=True)
    ev1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms_total = ev0.elapsed_time(ev1)
    trace_ms = [e0.elapsed_time(e1) for e0, e1 in tr_ev]
    ms_step = ms_total / a.steps
    steps_all, sec_step = across_ranks(ray_steps_step, ms_step / 1e3, dist, dev)
    ms_step = sec_step * 1e3
    value = steps_all / sec_step
    rays_per_s = Np * ws / sec_step

    peak, peak_kind = peaks()
    trace_ms_avg = float(np.mean(trace_ms))
    roof = trace_roofline(workload_config(a)["workload"], ray_steps_step, trace_ms_avg / 1e3, peak, peak_kind,
                          torch.cuda.get_device_properties(dev).multi_processor_count,
                          (clocks or {}).get("sm_mhz") or 2070.0)
    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded GRF density and Gaussian beam)",
           "config": workload_config(a), "gpu_launches": launches_per_step * a.steps,
           "roofline": roof, "clocks": clocks,
           "detail": {"ray_steps_per_step": ray_steps_step, "rays_per_s": rays_per_s,
                      "steps_per_ray": ray_steps_step / Np, "trace_ms": trace_ms_avg,
                      "non_ok_rays": n_bad,
                      "tracer": {"block": a.block or 256, "brick_depth": a.brick_depth or 8,
                                 "refill_lanes": a.refill or 2}}}

    if not a.no_e2e:
        # right after the device-timed leg: the FP64 leg's buffers (other sizes)
        # left in the allocators' caches made every other e2e step allocate anew
        torch.cuda.empty_cache()
        res["e2e"] = e2e_run(a, pt, rtm, ne, x, s0_host, ext_mm, det, dev, ws, dist)
    if rank == 0 and not a.no_fp64:
        res["fp64_dropin"], res["accuracy"] = fp64_compare(a, core, ne, x, s0_host, t_end, ext, out, rays_per_s / ws)
    if rank == 0 and not a.no_batched:
        del out, wsp, vol
        torch.cuda.empty_cache()
        res["batched"] = batched_run(a)
    if rank == 0 and not a.no_surrogate:
        torch.cuda.empty_cache()
        res["surrogate"] = surrogate_run(a)
    if rank == 0 and not a.no_stress:
        torch.cuda.empty_cache()
        res["stress"] = stress_run(a)
    if rank == 0 and not a.no_screen:
        torch.cuda.empty_cache()
        res["screen"] = screen_run(a)
    if rank == 0 and not a.no_cpu_baseline:
        # the CPU path at equal accuracy: the tolerance the FP64 drop-in needed in this run
        at = (res.get("fp64_dropin") or {}).get("at_bar") or {}
        res["cpu_baseline"] = cpu_baseline(a, ne, x, at.get("rtol", 1e-10), at.get("atol", 1e-13))
    if dist:
        dist.destroy_process_group()
    return res if rank == 0 else None


def trace_roofline(workload, ray_steps, seconds, peak, peak_kind, sms, sm_mhz):
    """Rooflines of the trace launch.  HBM gathers (the contract's figure):
    768 algorithmic bytes per ray-step over the launch time, against the
    measured copy bandwidth; a face-aimed step reads one cell's 8 nodes once for
    all stages and rays bucketed by entry tile share them in L1/L2, so this
    exceeds 1 and DRAM carries a few bytes per ray-step.  Issue: the warp
    instructions per ray-step of the captured launch times the ray-steps per
    second, against SMs x 4 schedulers x the SM clock sampled during the run --
    the resource the kernel is bound by."""
    cap = TRACE32_CAPTURE
    same = workload == cap["workload"] and ray_steps == cap["ray_steps"]
    scale = 1.0 if same else ray_steps / cap["ray_steps"]
    traffic = (cap["dram_read_bytes"] + cap["dram_write_bytes"]) * scale
    wipr = cap["warp_inst"] / cap["ray_steps"]
    issue_slots = sms * 4 * sm_mhz * 1e6
    roof = {"kernel": "tt_trace_f32 (ray bucketing + persistent trace32_kernel)", "bound": "hbm",
            "achieved": ray_steps * ALG_BYTES_PHASE / seconds / 1e9, "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "traffic": traffic,
            "traffic_source": ("one-pass ncu capture of this workload (profiles/trace32_grf512_1e7rays_counters.md)"
                               if same else "ncu capture of %s scaled by ray-steps" % cap["workload"]),
            "dram_gbs": traffic / seconds / 1e9,
            "issue": {"warp_inst_per_ray_step": wipr, "issue_slots_per_s": issue_slots, "sms": sms,
                      "sm_mhz": sm_mhz, "achieved_warp_inst_per_s": wipr * ray_steps / seconds},
            "note": "algorithmic bytes = 768 B per ray-step (6 stages x 8 corners x 4 comps x 4 B), served from "
                    "L1/L2 (frac > 1 is cache reuse; DRAM is dram_gbs); the binding resource is instruction "
                    "issue: issue_frac = warp instructions per ray-step x ray-steps/s / (SMs x 4 x SM clock)"}
    roof["frac"] = roof["achieved"] / peak
    roof["dram_frac"] = roof["dram_gbs"] / peak
    roof["issue_frac"] = roof["issue"]["achieved_warp_inst_per_s"] / issue_slots
    return roof


def fp64_compare(a, core, ne, x, s0_host, t_end, ext, out32, rays_per_s32):
    """The plain FP64 drop-in against the FP32 tracer at equal accuracy.
    Reference for the accuracy bars: the FP64 drop-in at rtol 1e-11 / atol 1e-13
    on the first a.check_rays rays (the parity tests tie it to the CPU oracle).
    The loosest FP64 tolerance that meets the bars on those rays is found
    first (rtol 1e-8, 1e-9, 1e-10 in turn); the FP64 drop-in is then timed at
    that tolerance on the first a.fp64_rays rays of the workload (1e6 by
    default: every SM holds its full complement of warps for the whole
    launch), and the FP32 tracer's rays/s is compared with that."""
    import torch

    fields = core.calc_dndr(ne, x, x, x, lwl=a.lwl)
    c = min(a.check_rays, s0_host.shape[1])
    m = min(a.fp64_rays, s0_host.shape[1])
    sub = torch.as_tensor(np.ascontiguousarray(s0_host[:, :max(m, c)]), device="cuda")
    ref = core.trace_f64(fields, sub[:, :c], t_end, 2, ext, rtol=1e-11, atol=1e-13, phase=True)
    torch.cuda.synchronize()
    rf_ref = ref["rf"].cpu().numpy()
    ph_ref = ref["phase"].cpu().numpy()
    bars = {"pos_over_L": 1e-6, "angle_rad": 1e-6, "phase_rad": 1e-3}

    def err(rf, ph):
        return {"pos_over_L": float(np.abs(rf[0::2] - rf_ref[0::2]).max() / a.L),
                "angle_rad": float(np.abs(rf[1::2] - rf_ref[1::2]).max()),
                "phase_rad": float(np.abs(ph - ph_ref).max())}

    def meets(e):
        return all(e[k] <= bars[k] for k in bars)

    def timed(n, rtol, atol):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        o = core.trace_f64(fields, sub[:, :n], t_end, 2, ext, rtol=rtol, atol=atol, phase=True)
        e1.record()
        torch.cuda.synchronize()
        return o, e0.elapsed_time(e1) / 1e3

    acc = {"fp32": err(out32["rf"][:, :c].cpu().numpy(), out32["phase"][:c].cpu().numpy())}
    acc["fp32"]["meets_bars"] = meets(acc["fp32"])
    core.trace_f64(fields, sub[:, :256], t_end, 2, ext, rtol=1e-8, atol=1e-11, phase=True)  # warm-up
    checks = []
    for rtol, atol in ((1e-8, 1e-11), (1e-9, 1e-12), (1e-10, 1e-13)):
        o64, sec = timed(c, rtol, atol)
        e = err(o64["rf"].cpu().numpy(), o64["phase"].cpu().numpy())
        e["meets_bars"] = meets(e)
        checks.append({"rtol": rtol, "atol": atol, "rays": c, "seconds": sec, "error": e})
        if e["meets_bars"]:
            break
    bar = next((r for r in checks if r["error"]["meets_bars"]), checks[-1])
    o64, sec = timed(m, bar["rtol"], bar["atol"])
    steps = int(o64["nsteps"].sum().item())
    acc["reference"] = "FP64 drop-in at rtol 1e-11, atol 1e-13 on %d rays (the tests tie it to the CPU oracle)" % c
    acc["bars"] = bars
    del fields, o64
    torch.cuda.empty_cache()
    f64 = {"tolerance_search": checks,
           "at_bar": {"rtol": bar["rtol"], "atol": bar["atol"], "rays": m, "seconds": sec, "rays_per_s": m / sec,
                      "ray_steps_per_s": steps / sec, "steps_per_ray": steps / m,
                      "kernel": "trace64_kernel: persistent lanes, 3 blocks of 128 per SM (168 registers)"},
           "fp32_speedup_equal_accuracy_rays_per_s": rays_per_s32 / (m / sec)}
    return f64, acc


def batched_run(a):
    """The batched ensemble: a.batch_instances realisations drawn as the batched
    workload (grid 128/192/256/384^3, exponent -5/3/-3/-11/3, delta in
    [0.05, 0.3], background 1e23..1e25 m^-3, 1e5..4e6 rays log-uniform,
    sigma 0.25 L, 0.05 mrad, L = 2 mm, 512^2 shadowgram each).  Pipeline per
    step, one CUDA graph: volume builds, ray bucketing, the persistent trace
    launches, shadowgrams.  The ensemble's set-up times the launch forms on
    the ensemble itself (one mixed-shape launch for all instances, one
    batched launch per grid shape, or one launch per instance), each with
    the library's lane refill (a warp refills once two lanes are idle) and
    with a warp's 32 lanes refilled together, and keeps the fastest; the eager one-launch-per-instance form
    with the tracer's defaults is timed beside it.  The same is repeated for
    small instances (2e3..8e4 rays)."""
    import torch

    from turbulence_tracing_gb300 import ensemble

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def one(inst):
        E = ensemble.Ensemble(inst, L=2e-3, det=512, phase=False, tune=True).setup()
        E.capture()
        ms = timed(E.replay)
        steps = E.ray_steps()
        bad = int((E.out["status"] != 0).sum().item())
        chosen = E.mode
        trace_ms = {m: E.mode_ms[m] for m in E.mode_ms}
        best = {m: min(v for k, v in trace_ms.items() if k.startswith(m + "/"))
                for m in ("one_launch", "grouped", "per_instance")}
        ms_eager = timed(E.run_unbatched, 1)
        r = {"instances": len(inst), "rays": E.ntot, "ray_steps_per_step": steps, "mode": chosen,
             "refill_lanes": E.refill, "one_launch_over_per_instance": best["one_launch"] / best["per_instance"],
             "launches": len(E._launches()), "block_size": E.block, "graph_ms_per_step": ms,
             "ray_steps_per_s": steps / (ms / 1e3), "rays_per_s": E.ntot / (ms / 1e3), "non_ok_rays": bad,
             "trace_only_ms_by_mode_refill": trace_ms, "eager_one_launch_per_instance_ms_per_step": ms_eager,
             "speedup_vs_eager_per_instance": ms_eager / ms}
        sizes = {}
        for p in inst:
            sizes[p["n"]] = sizes.get(p["n"], 0) + 1
        r["grid_counts"] = {str(k): v for k, v in sorted(sizes.items())}
        r["autotuned_per_grid"] = {str(k): {"block": v["block"], "brick_depth": v["brick_depth"]}
                                   for k, v in E.tuned.items()}
        del E
        torch.cuda.empty_cache()
        return r

    out = one(ensemble.draw_instances(a.batch_instances, seed=a.seed))
    out["small_instances"] = one(ensemble.draw_instances(a.batch_instances, seed=a.seed, rays=(2e3, 8e4)))
    out["pipeline"] = "CUDA graph: volume builds + bucketing + persistent trace launches + shadowgrams"
    return out


def surrogate_run(a):
    """The learned surrogate (straight-line and marched maps -> full-trace
    deflection and phase) at a.sur_size^2 on fields drawn as the batched
    workload at that grid: data made by the tracer itself, FNO training by the
    library's kernels, held-out evaluation against the exact tracer, then the
    surrogate-with-fallback pipeline timed against tracing every field (one
    field per launch, and a chunk of fields per batched launch with either
    lane-refill rule, the faster of the two being the baseline)."""
    import time

    import torch

    from turbulence_tracing_gb300 import core, fno, surrogate as SG

    S = a.sur_size
    W = SG.Workload(S, plane_stride=a.sur_stride)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    X, Y, _, _, steps_tr = SG.build_dataset(W, SG.draw_fields(a.sur_train, seed=a.seed + 11))
    Xte, _, ste, truth, _ = SG.build_dataset(W, SG.draw_fields(a.sur_test, seed=a.seed + 12), keep_truth=True)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    target_rms = [float(1.0 / g) for g in W.gain.tolist()]  # rms of the unscaled targets
    net = fno.FNO(S, in_ch=W.in_ch, out_ch=3, layers=4, seed=a.seed)
    trainer = SG.Trainer(net, X, Y, batch=8)
    hist, sps = trainer.fit(a.sur_epochs, lr=1e-3)
    res = SG.evaluate(W, net, Xte, ste, truth)
    half = len(res) // 2
    kappa = SG.calibrate(res[:half])
    held = res[half:]

    def mean(k):
        return float(np.mean([r[k] for r in held]))

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e3 / reps

    # inference kernel throughput: forward passes of a batch of 8
    xb = Xte[:8].contiguous()
    ob = net.forward(xb)
    us_fwd = timed(lambda: net.forward(xb, out=ob), 10) / 8
    ne0 = W.field(SG.draw_fields(1, seed=a.seed + 13)[0])
    mo = torch.empty((W.n_maps, S, S), dtype=torch.float32, device=W.dev)
    so = torch.empty((3, S, S), dtype=torch.float32, device=W.dev)
    us_march = timed(lambda: W.march(ne0, out=mo), 20)
    f8 = [W.field(p_) for p_ in SG.draw_fields(8, seed=a.seed + 14)]
    mb = torch.empty((8, W.n_maps, S, S), dtype=torch.float32, device=W.dev)
    wsb = torch.empty(core.march_batched_workspace_bytes(8, f8[0].shape), dtype=torch.uint8, device=W.dev)
    us_march_b = timed(lambda: core.march_maps_batched(f8, W.x, W.x, W.x, S, lwl=W.lwl, out=mb, ws=wsb,
                                                       plane_stride=W.plane_stride), 10) / 8
    del f8, mb, wsb
    us_maps = timed(lambda: W.maps(ne0, out=so), 20)
    C = 32
    fwd_bytes = 4 * (6 * C * S * S * 1 + 16 * C * 32 * S) + (4 * W.in_ch + 2 * C) * S * S + (2 * C + 12) * S * S
    march_bytes = 4 * S ** 3 * 3 + 20 * S * S  # density read, plane-major q written and read once, 5 maps
    peak, peak_kind = peaks()
    # the pipeline against tracing every field, on fresh fields drawn the same way
    fields = [W.field(p) for p in SG.draw_fields(a.sur_time, seed=a.seed + 15)]
    # detector set-up: each field's drift for 20% straight-line contrast
    Ds = [float(W.drift(W.maps(f))) for f in fields]
    pipe = SG.Pipeline(W, net, kappa, batch=a.sur_batch)
    bts = {rl: SG.BatchedTracer(W, batch=a.sur_batch, refill_lanes=rl) for rl in (2, 32)}
    pipe.run(fields[:a.sur_batch], Ds[:a.sur_batch])
    pipe.run_tracer(fields[:2], Ds[:2])
    for bt in bts.values():
        bt.run(fields[:a.sur_batch], Ds[:a.sur_batch])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    I_p, fell = pipe.run(fields, Ds)
    torch.cuda.synchronize()
    t_pipe = time.perf_counter() - t0
    t0 = time.perf_counter()
    I_t = pipe.run_tracer(fields, Ds)
    torch.cuda.synchronize()
    t_tr = time.perf_counter() - t0
    # the batched exact tracer with both lane-refill rules; the faster is the baseline
    t_bts, I_b = {}, None
    for rl, bt in bts.items():
        t0 = time.perf_counter()
        I_b = bt.run(fields, Ds)
        torch.cuda.synchronize()
        t_bts[rl] = time.perf_counter() - t0
    t_bt = min(t_bts.values())
    errs = [SG.rel_l2(p_, t_) for p_, t_ in zip(I_p, I_t)]
    acc = [e for e, f in zip(errs, fell) if not f]
    bt_dev = max(SG.rel_l2(b_, t_) for b_, t_ in zip(I_b, I_t))
    return {"grid": S, "march_plane_stride": W.plane_stride, "train_fields": a.sur_train, "test_fields": a.sur_test,
            "timed_fields": len(fields),
            "epochs": a.sur_epochs,
            "data_s": t_data, "train_samples_per_s": sps, "loss_first_last": [hist[0], hist[-1]],
            "target_rms": target_rms,
            "heldout": {"shadow_err_straight": mean("err_straight"), "shadow_err_march": mean("err_march"),
                        "shadow_err_net": mean("err_net"),
                        "shadow_err_max": {k: max(r[k] for r in held) for k in ("err_straight", "err_march", "err_net")},
                        "theta_err_straight": mean("theta_err_straight"), "theta_err_march": mean("theta_err_march"),
                        "theta_err_net": mean("theta_err_net"),
                        "phase_corr_err_march": mean("phase_corr_err_march"),
                        "phase_corr_err_net": mean("phase_corr_err_net"), "fields": len(held)},
            "fno_forward_us_per_field": us_fwd,
            "fno_forward_roofline": {"bound": "hbm", "achieved": fwd_bytes / (us_fwd * 1e-6) / 1e9, "peak": peak,
                                     "unit": "GB/s", "frac": fwd_bytes / (us_fwd * 1e-6) / 1e9 / peak,
                                     "bytes_per_field": fwd_bytes, "peak_kind": peak_kind},
            "march_us_per_field": us_march, "march_batched8_us_per_field": us_march_b,
            "straight_maps_us_per_field": us_maps,
            "march_roofline": {"bound": "hbm", "achieved": march_bytes / (us_march_b * 1e-6) / 1e9, "peak": peak,
                               "unit": "GB/s", "frac": march_bytes / (us_march_b * 1e-6) / 1e9 / peak,
                               "launch": "8 fields per launch",
                               "bytes_per_field": march_bytes, "peak_kind": peak_kind},
            "pipeline": {"kappa": kappa, "tol": 0.02, "chunk": a.sur_batch, "fallback_fraction": float(np.mean(fell)),
                         "err_max": max(errs), "accepted_err_max": max(acc) if acc else None,
                         "accepted_err_mean": float(np.mean(acc)) if acc else None,
                         "pipeline_s": t_pipe, "tracer_per_field_s": t_tr, "tracer_batched_s": t_bt,
                         "tracer_batched_s_by_refill": {str(k): v for k, v in t_bts.items()},
                         "batched_vs_per_field_max_dev": bt_dev,
                         "speedup_vs_tracer_per_field": t_tr / t_pipe,
                         "speedup_vs_tracer_batched": t_bt / t_pipe},
            "error_flag": net.error_flag()}


def stress_run(a):
    """The stress workload: a 1024^3 FP32 field (L = 10 mm, |k|^-11/3,
    delta = 0.3, n_e = 1e25 m^-3; node volume 26.8 GB), 1e8 rays (x, y ~
    N(0, 3 mm), angles ~ N(0, 0.1 mrad)) drawn on the device and traced in
    device-resident chunks of 1e7 by the FP32 tracer with the phase summed in
    FP64, each chunk's rays accumulated into 2048^2 shadowgraphy, knife-edge
    schlieren and interferometry detectors.  Accuracy on the first
    a.stress_check rays of the first chunk against the FP64 drop-in at rtol
    1e-10 (and the FP64 drop-in's own spread between rtol 1e-10 and 1e-11, which
    marks the rays whose answer is not determined to the bars), plus the
    detectors those rays fill, FP32 against FP64, up to rays that cross a bin
    edge by less than the position bar."""
    import torch

    from oracle import restated as R
    from turbulence_tracing_gb300 import _lib, core, turboGen

    N = a.stress_n
    L = 10e-3 * N / 1024
    sigma, div, det = 3e-3 * N / 1024, 0.1e-3, 2048
    ne, x = turboGen.workload_field(N, L, -11.0 / 3.0, 0.3, 1e25, seed=a.seed + 900, dtype=torch.float32)
    ext = float(x.max())
    t_end = R.t_end(ext)
    dev = ne.device
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    vol = core.build_volume(ne, x, x, x, probing_axis=2, lwl=a.lwl)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    chunk, total = int(a.stress_chunk), int(a.stress_rays)
    nchunks = -(-total // chunk)
    gen = torch.Generator(device=dev).manual_seed(a.seed + 901)

    def draw(n, s0):
        s0[0].normal_(0.0, sigma, generator=gen)
        s0[1].normal_(0.0, sigma, generator=gen)
        s0[2].fill_(-ext)
        tx = torch.tan(torch.empty(n, dtype=torch.float64, device=dev).normal_(0.0, div, generator=gen))
        ty = torch.tan(torch.empty(n, dtype=torch.float64, device=dev).normal_(0.0, div, generator=gen))
        nrm = torch.sqrt(1.0 + tx * tx + ty * ty)
        s0[3] = 299792458.0 * tx / nrm
        s0[4] = 299792458.0 * ty / nrm
        s0[5] = 299792458.0 / nrm

    ext_mm = 4.0 * sigma * 1e3
    f_mm, R_mm = 100.0, 25.0
    relay = lambda mid: ([(_lib.OPTIC_M_TO_MM, 0, 0, 0), (_lib.OPTIC_DISTANCE, f_mm, 0, 0),
                          (_lib.OPTIC_CIRC_APERTURE, R_mm, 0, 0), (_lib.OPTIC_LENS, f_mm, f_mm, 0),
                          (_lib.OPTIC_DISTANCE, f_mm, 0, 0)] + mid +
                         [(_lib.OPTIC_DISTANCE, f_mm, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R_mm, 0, 0),
                          (_lib.OPTIC_LENS, f_mm, f_mm, 0), (_lib.OPTIC_DISTANCE, f_mm, 0, 0)])
    chains = [relay([]), relay([(_lib.OPTIC_KNIFE_EDGE, 0.0, 0, 1.0)])]
    rng_mm = (-ext_mm, ext_mm)
    H = [torch.zeros((det, det), dtype=torch.float64, device=dev) for _ in range(3)]
    Hw = torch.zeros((det, det), dtype=torch.float64, device=dev)
    s0 = torch.empty((6, chunk), dtype=torch.float64, device=dev)
    out = core._ray_outputs(chunk, dev, want_sf=False)
    ws = core.workspace(_lib.lib().tt_trace_f32_workspace_bytes(ctypes.byref(vol.desc), chunk), dev)
    first = None
    steps_total, bad = 0, 0
    # one warm-up chunk, not counted
    draw(chunk, s0)
    core.trace_f32(vol, s0, t_end, ext, rtol=1e-7, atol=1e-5, atol_phase=1e-5, phase=True, phase_f64=True,
                   ws=ws, out=out, want_sf=False)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for c in range(nchunks):
        n = min(chunk, total - c * chunk)
        sv = s0[:, :n]
        draw(n, sv)
        o = {k: (v[..., :n] if v is not None else None) for k, v in out.items()}
        core.trace_f32(vol, sv, t_end, ext, rtol=1e-7, atol=1e-5, atol_phase=1e-5, phase=True, phase_f64=True,
                       ws=ws, out=o, want_sf=False)
        for k, ch in enumerate(chains):
            core.detect(o["rf"], ch, det, det, rng_mm, rng_mm, H=H[k], accumulate=True)
        core.detect(o["rf"], chains[0], det, det, rng_mm, rng_mm, weights=o["phase"], H=H[2], Hw=Hw, accumulate=True)
        steps_total += o["nsteps"].sum()
        bad += (o["status"] != 0).sum()
        if c == 0:
            m = min(a.stress_check, n)
            first = (sv[:, :m].clone(), o["rf"][:, :m].clone(), o["phase"][:m].clone())
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    steps_total = int(steps_total.item())
    res = {"grid": N, "L_m": L, "rays": total, "chunk": chunk, "chunks": nchunks, "detectors": [det, det],
           "phase_accumulation": "fp64", "node_volume_gb": vol.nbytes / 1e9, "volume_build_s": t_build,
           "seconds": sec, "ray_steps": steps_total, "ray_steps_per_s": steps_total / sec, "rays_per_s": total / sec,
           "steps_per_ray": steps_total / total, "non_ok_rays": int(bad.item()),
           "timed": "all chunks: on-device ray draw, trace, 3 detectors (CUDA events)"}
    del out, ws, s0
    # accuracy on the first rays of chunk 0
    sub, rf32, ph32 = first
    del vol
    torch.cuda.empty_cache()
    fields = core.calc_dndr(ne, x, x, x, lwl=a.lwl)
    r10 = core.trace_f64(fields, sub, t_end, 2, ext, rtol=1e-10, atol=1e-13, phase=True)
    r11 = core.trace_f64(fields, sub, t_end, 2, ext, rtol=1e-11, atol=1e-14, phase=True)
    torch.cuda.synchronize()
    del fields
    torch.cuda.empty_cache()

    def per_ray(u, pu, v, pv):
        pos = (u[0::2] - v[0::2]).abs().amax(dim=0) / L
        ang = (u[1::2] - v[1::2]).abs().amax(dim=0)
        return pos, ang, (pu - pv).abs()

    p32, a32, f32 = per_ray(rf32, ph32, r10["rf"], r10["phase"])
    p64, a64, f64 = per_ray(r11["rf"], r11["phase"], r10["rf"], r10["phase"])
    ok32 = (p32 <= 1e-6) & (a32 <= 1e-6) & (f32 <= 1e-3)
    posed = (p64 <= 1e-7) & (a64 <= 1e-7) & (f64 <= 1e-4)
    acc = {"rays": int(sub.shape[1]), "reference": "FP64 drop-in, rtol 1e-10 / atol 1e-13",
           "fraction_within_bars": float(ok32.double().mean()),
           "fraction_well_conditioned": float(posed.double().mean()),
           "fraction_within_bars_well_conditioned": float(ok32[posed].double().mean()) if bool(posed.any()) else None,
           "fp32_max_on_well_conditioned": {"pos_over_L": float(p32[posed].max()), "angle_rad": float(a32[posed].max()),
                                            "phase_rad": float(f32[posed].max())} if bool(posed.any()) else None,
           "fp64_rtol1e-10_vs_1e-11_max": {"pos_over_L": float(p64.max()), "angle_rad": float(a64.max()),
                                           "phase_rad": float(f64.max())}}
    # the detectors those rays fill, FP32 against FP64: bin moves within the position bar
    Hs = []
    for rf_ in (rf32, r10["rf"]):
        _, _, ro = core.detect(rf_, chains[0], r_out=True, histogram=False)
        Hs.append(ro)
    step_mm = 2 * ext_mm / det

    def bins(ro):
        bx = torch.floor((ro[0] + ext_mm) / step_mm)
        by = torch.floor((ro[2] + ext_mm) / step_mm)
        inside = (bx >= 0) & (bx < det) & (by >= 0) & (by < det)
        return torch.where(inside, by * det + bx, torch.full_like(bx, -1.0))

    b32, b64 = bins(Hs[0]), bins(Hs[1])
    moved = b32 != b64
    dpos = ((Hs[0][0] - Hs[1][0]).abs().nan_to_num(0.0).maximum((Hs[0][2] - Hs[1][2]).abs().nan_to_num(0.0)))
    bar_mm = 1e-6 * L * 1e3  # the position bar, imaged 1:1 onto the detector
    mp = moved & posed
    acc["detector"] = {"bins": [det, det], "extent_mm": 2 * ext_mm, "bin_mm": step_mm,
                       "rays_in_other_bin": int(moved.sum()),
                       "rays_in_other_bin_well_conditioned": int(mp.sum()),
                       "max_detector_shift_of_moved_well_conditioned_mm": float(dpos[mp].max()) if bool(mp.any()) else 0.0,
                       "position_bar_mm": bar_mm,
                       "counts_match_up_to_bin_edge_moves": bool((not bool(mp.any())) or float(dpos[mp].max()) <= bar_mm)}
    res["accuracy"] = acc
    return res


def screen_run(a):
    """The stress field's surrogate screening (1024^3, L = 10 mm, -11/3,
    delta = 0.3, 1e25 m^-3): the network, trained on 256^2 tiles of other
    realisations of the same configuration, screens the field per tile and
    only flagged tiles are re-traced; timed against tracing all N^2 pixel-centre
    rays (volume build + trace), both followed by the field's shadowgram."""
    import time

    import torch

    from turbulence_tracing_gb300 import fno, surrogate as SG

    N = a.screen_n
    W = SG.Workload(N, L=10e-3 * N / 1024)

    def stress(seed):
        return dict(alpha=-11.0 / 3.0, delta=0.3, ne0=1e25, seed=seed)

    t0 = time.perf_counter()
    X, Y, _, _ = SG.build_tile_dataset(W, [stress(a.seed + 500 + i) for i in range(a.screen_train)])
    Xc, _, sc, tc = SG.build_tile_dataset(W, [stress(a.seed + 600), stress(a.seed + 601)], keep_truth=True)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = fno.FNO(SG.TILE, in_ch=W.in_ch, out_ch=3, layers=4, seed=a.seed)
    hist, _ = SG.Trainer(net, X, Y, batch=8).fit(8, lr=1e-3)
    fields = [W.field(stress(a.seed + 700 + i)) for i in range(2)]
    Ds = [float(W.drift(W.march(f)[3:5])) for f in fields]
    tiles = SG.tile_errors(W, net, Xc, sc, tc, Ds[0])
    kappa = SG.calibrate(tiles)
    scr = SG.TileScreen(W, net, kappa)
    scr.run(fields[0], Ds[0])
    W.trace(fields[0])
    out = []
    for f, D in zip(fields, Ds):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        I_s, _, flagged = scr.run(f, D)
        torch.cuda.synchronize()
        t_scr = time.perf_counter() - t0
        t0 = time.perf_counter()
        th, _, steps = W.trace(f)
        I_t = W.shadow(th, D)
        torch.cuda.synchronize()
        t_tr = time.perf_counter() - t0
        out.append({"screen_s": t_scr, "tracer_s": t_tr, "speedup": t_tr / t_scr, "flagged_tiles": len(flagged),
                    "tiles": scr.nt, "shadow_err": SG.rel_l2(I_s, I_t), "tracer_ray_steps": int(steps)})
    return {"grid": N, "tile": SG.TILE, "train_fields": a.screen_train, "train_tiles": int(X.shape[0]),
            "data_s": t_data, "loss_first_last": [hist[0], hist[-1]], "kappa": kappa,
            "calibration_tiles": {"err_march_mean": float(np.mean([r["err_march"] for r in tiles])),
                                  "err_net_mean": float(np.mean([r["err_net"] for r in tiles])),
                                  "err_straight_mean": float(np.mean([r["err_straight"] for r in tiles]))},
            "fields": out, "error_flag": net.error_flag()}


def e2e_run(a, pt, rtm, ne, x, s0_host, ext_mm, det, dev, ws, dist):
    """Public API, host buffers in and out, one new field per step: the
    density (pinned host FP32) given to ElectronCube.external_ne, calc_dndr,
    the pinned host rays as s0, solve(precision='fp32', phase=True) (the FP32
    node volume is built from the uploaded density inside the step), then
    three ray_transfer_matrix diagnostics on the returned numpy rays."""
    import torch

    ne_pinned = ne.cpu().pin_memory()
    pinned = torch.from_numpy(s0_host).pin_memory()
    cube = pt.ElectronCube(x, x, x)
    bins_scale = 1
    import builtins

    quiet = builtins.print

    parts = []

    def one():
        t0 = time.perf_counter()
        builtins.print = lambda *k, **kw: None
        try:
            cube.external_ne(ne_pinned)
            cube.calc_dndr(lwl=a.lwl)
            cube.s0 = pinned
            rf = cube.solve(precision="fp32", phase=True)  # returns after its stream is synchronised
        finally:
            builtins.print = quiet
        parts.append(time.perf_counter() - t0)
        sh = rtm.Shadowgraphy(rf, focal_plane=0, L=100.0, R=25.0, Lx=2 * ext_mm, Ly=2 * ext_mm)
        sh.solve()
        sh.histogram(bin_scale=bins_scale, pix_x=det, pix_y=det)
        ke = rtm.Schlieren_KE(rf, focal_plane=0, L=100.0, R=25.0, Lx=2 * ext_mm, Ly=2 * ext_mm)
        ke.solve(offset=0.0, axis="x", direction=1)
        ke.histogram(bin_scale=bins_scale, pix_x=det, pix_y=det)
        it = rtm.Shadowgraphy(rf, focal_plane=0, L=100.0, R=25.0, Lx=2 * ext_mm, Ly=2 * ext_mm)
        it.solve()
        it.histogram(bin_scale=bins_scale, pix_x=det, pix_y=det, weights=cube.phase)
        return int(cube.nsteps.sum()), sh.H.sum() + ke.H.sum() + it.Hw.sum()

    # warm-up: the first steps allocate the device buffers and the pinned host
    # staging buffers that later steps reuse (a solve's results alternate
    # between two of them while the previous results are still referenced;
    # after the device-timed leg this takes a few more steps to settle)
    for _ in range(6):
        one()
    torch.cuda.synchronize()
    # each step ends in host arrays, so steps are timed one by one; the median
    # of at least 7 steps is reported (now and then a step takes ~45 ms longer
    # in the host-side copies, which moves the median of fewer steps)
    k = max(7, min(a.steps, 15))
    if dist:
        dist.barrier()
    times, tot = [], 0
    del parts[:]
    for _ in range(k):
        t0 = time.perf_counter()
        rs, _chk = one()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        tot += rs
    sec = float(np.median(times))
    units, sec = across_ranks(tot / k, sec, dist, dev)
    Np = s0_host.shape[1]
    h2d = ne.numel() * ne.element_size() + Np * 6 * 8   # density, s0 (the diagnostics use the rays' device twins)
    d2h = Np * (4 + 1) * 8 + Np * 2 * 4 + 4 * det * det * 8  # rf, phase; status, steps; 3 H + 1 Hw (sf stays on the device until read)
    return {"value": units / sec, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "seconds_per_step": sec, "steps": k, "step_seconds": times, "timing": "median step",
            "solve_seconds": parts,  # density in, volume build, rays in, trace, results out (the rest: diagnostics)
            "path": "ElectronCube.external_ne(host density) + calc_dndr + solve(precision='fp32', phase=True) "
                    "+ Shadowgraphy, Schlieren_KE, phase-weighted Shadowgraphy histograms (host arrays in and out)"}


def _ref_path(a, dpath, td, rays, extra=()):
    jpath = os.path.join(td, "cpu_%d.json" % len(os.listdir(td)))
    cmd = [sys.executable, "-m", "oracle.ref_path", "--density", dpath, "--L", str(a.L), "--rays", str(rays),
           "--sigma", str(a.sigma), "--div", str(a.div), "--lwl", str(a.lwl), "--json", jpath] + list(extra)
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=1200)
    if r.returncode != 0:
        return {"error": r.stderr[-500:]}
    with open(jpath) as f:
        return json.load(f)


def cpu_baseline(a, ne, x, bar_rtol=1e-10, bar_atol=1e-13):
    """The reference's CPU path (restated: oracle/ref_path.py) on ray samples
    through the same density, on this host's cores, in subprocesses that never
    touch CUDA: at the reference's default tolerance (the reported value), and
    a smaller sample at bar_rtol / bar_atol, the tolerance at which the FP64
    drop-in met the accuracy bars in the same run (rays/s at equal accuracy)."""
    with tempfile.TemporaryDirectory() as td:
        dpath = os.path.join(td, "ne.npy")
        np.save(dpath, ne.cpu().numpy())
        d = _ref_path(a, dpath, td, a.cpu_rays)
        if "error" in d:
            return d
        bar = _ref_path(a, dpath, td, a.cpu_bar_rays,
                        ("--rtol", repr(float(bar_rtol)), "--atol", repr(float(bar_atol)), "--bundle", "8"))
    out = {"value": d["ray_steps_per_s"], "unit": UNIT, "cores": d["procs"], "kind": "port",
           "sample": "%d rays of the same workload (same density) traced by the reference's CPU path "
                     "(global-step solve_ivp RK45 at rtol 1e-3/atol 1e-6 with RegularGridInterpolator "
                     "lookups), in bundles over %d forked processes" % (d["rays"], d["procs"]),
           "rays_per_s": d["rays_per_s"], "wall_s": d["wall"], "setup_s": d["setup_s"]}
    if "error" not in bar:
        out["at_bar"] = {"rtol": bar["rtol"], "atol": bar["atol"], "rays": bar["rays"], "bundle": bar["bundle"],
                         "rays_per_s": bar["rays_per_s"], "ray_steps_per_s": bar["ray_steps_per_s"],
                         "wall_s": bar["wall"]}
    return out


# ---------------------------------------------------------------------------- reference arm
def run_reference(a):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return None
    from oracle import ref_path as RP
    from oracle import restated as R

    ne, x = R.workload_density(a.n, a.L, a.alpha, a.delta, a.ne0, a.seed)
    ne = ne.astype(np.float32)
    cube = RP.RefCube(ne, x, x, x, lwl=a.lwl)
    del ne
    nproc = host_cores()
    ext = float(x.max())
    t_end = R.t_end(ext)
    rng = np.random.default_rng(a.seed)
    times, steps_done, rays_done = [], 0, 0
    for i in range(a.warmup + a.steps):
        s0 = R.gaussian_beam(a.ref_rays, a.sigma, a.div, ext, rng)
        r = RP.run_pool(cube, s0, t_end, nproc)
        if i >= a.warmup:
            times.append(r["wall"])
            steps_done += r["ray_steps"]
            rays_done += a.ref_rays
    sec = float(np.sum(times))
    value = steps_done / sec
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * sec / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded GRF density and Gaussian beam)", "impl": "reference",
            "config": workload_config(a),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nproc, "kind": "port",
                             "sample": "%d rays per step through the full %d^3 field: the reference's CPU path "
                                       "(global-step solve_ivp RK45, rtol 1e-3, RegularGridInterpolator) "
                                       "restated, bundles over %d forked processes" % (a.ref_rays, a.n, nproc)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": {"rays_per_s": rays_done / sec}}


def run_fp64_only(a):
    """The plain FP64 drop-in (tt_trace_f64, per-ray RK45, phase on) alone on
    the workload's field and beam, every ray traced: one warm-up launch on a
    small slice, then one launch over all rays timed with CUDA events."""
    import torch

    from oracle import restated as R
    from turbulence_tracing_gb300 import core, turboGen

    ne, x = turboGen.workload_field(a.n, a.L, a.alpha, a.delta, a.ne0, seed=a.seed, dtype=torch.float32)
    ext = float(x.max())
    s0 = torch.as_tensor(R.gaussian_beam(int(a.rays), a.sigma, a.div, ext, np.random.default_rng(a.seed)),
                         device="cuda")
    f = core.calc_dndr(ne, x, x, x, lwl=a.lwl)
    t_end = R.t_end(ext)
    core.trace_f64(f, s0[:, :1024], t_end, 2, ext, rtol=a.fp64_rtol, atol=a.fp64_atol, phase=True)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    out = core.trace_f64(f, s0, t_end, 2, ext, rtol=a.fp64_rtol, atol=a.fp64_atol, phase=True)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    steps = int(out["nsteps"].sum().item())
    return {"leg": "fp64_only", "grid": a.n, "rays": int(a.rays), "rtol": a.fp64_rtol, "atol": a.fp64_atol,
            "seconds": sec, "rays_per_s": a.rays / sec, "ray_steps": steps, "ray_steps_per_s": steps / sec,
            "steps_per_ray": steps / a.rays, "non_ok_rays": int((out["status"] != 0).sum().item())}


def main():
    a = parse()
    if a.fp64_only:
        print(json.dumps(run_fp64_only(a)))
        return
    res = run_ours(a) if a.impl == "ours" else run_reference(a)
    if res is not None:
        line = json.dumps(res)
        print(line)
        if a.json_out:
            with open(a.json_out, "w") as f:
                f.write(line + "\n")


if __name__ == "__main__":
    main()
