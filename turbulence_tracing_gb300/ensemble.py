"""Batched ensemble: many field realisations of uneven grid size and ray count
traced by persistent batched launches from a CUDA-graph-captured pipeline,
with block size and brick depth chosen by the autotuner.

Instances are ordered by grid shape.  Launch modes:
  grouped       one persistent launch per grid shape (uniform-shape kernel:
                geometry in the constant bank, per-instance node buffer and
                ray block)
  one_launch    every instance in one launch of the mixed-shape kernel
                (per-lane geometry)
  per_instance  one launch per instance
With tune=True the set-up times grouped and per_instance on the ensemble
itself and keeps the faster: batching wins when instances are small (launch
tails and launch overhead dominate), separate launches when they are large
(each launch starts with all lanes on neighbouring rays, which keeps the
cache hit rate up).

Each instance gets a seeded band-limited Gaussian-random-field density
(n^3 grid of side L, |k|^alpha, n_e = ne0 (1 + delta g)), a Gaussian beam
(x, y ~ N(0, sigma_frac L), angles ~ N(0, divergence)) and a shadowgram.
The per-instance parameters are drawn from a seeded generator.

Pipeline per step (captured once, replayed): K1 volume build per instance ->
ray bucketing + one batched persistent trace over all instances -> one
shadowgraphy histogram per instance.  The fields themselves are generated
once at set-up (cuFFT plan creation is not part of the graph).
"""
import math

import numpy as np
import torch

from . import _lib, autotune, core, turboGen

C_LIGHT = 299792458.0
REFILLS = (2, 32)  # lane refill thresholds the set-up times (tt_trace_opts.refill_lanes; 2 is the library's default)


def draw_instances(n_inst=64, seed=0, sizes=(128, 192, 256, 384), exponents=(-5.0 / 3.0, -3.0, -11.0 / 3.0),
                   delta=(0.05, 0.3), ne0=(1e23, 1e25), rays=(1e5, 4e6), ray_scale=1.0):
    """Per-instance parameters: grid size, spectral exponent, amplitude,
    background density and log-uniform ray count."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_inst):
        nr = math.exp(rng.uniform(math.log(rays[0]), math.log(rays[1])))
        out.append(dict(n=int(rng.choice(sizes)), alpha=float(rng.choice(exponents)),
                        delta=float(rng.uniform(*delta)), ne0=float(rng.uniform(*ne0)),
                        nrays=max(1, int(round(nr * ray_scale))), seed=int(rng.integers(0, 2 ** 62))))
    return out


def gaussian_beam_into(dst, nrays, sigma, divergence, extent, rng):
    """Fill dst (6, nrays) with the workload beam (see oracle-free restatement in
    the tests): x, y ~ N(0, sigma), z = -extent, small Gaussian angles."""
    dst[0] = rng.normal(0.0, sigma, nrays)
    dst[1] = rng.normal(0.0, sigma, nrays)
    dst[2] = -extent
    tx = np.tan(rng.normal(0.0, divergence, nrays))
    ty = np.tan(rng.normal(0.0, divergence, nrays))
    nrm = np.sqrt(1.0 + tx * tx + ty * ty)
    dst[3] = C_LIGHT * tx / nrm
    dst[4] = C_LIGHT * ty / nrm
    dst[5] = C_LIGHT / nrm


class Ensemble:
    def __init__(self, instances, L=2e-3, sigma_frac=0.25, divergence=0.05e-3, lwl=1064e-9, det=512,
                 phase=False, rtol=1e-7, tune=True, tune_rays=200000, beam_seed=1, mode="grouped", refill_lanes=2):
        order = sorted(range(len(instances)), key=lambda i: instances[i]["n"])
        self.order = order  # instance k here is instances[order[k]]
        self.inst = [instances[i] for i in order]
        if mode not in ("grouped", "one_launch", "per_instance"):
            raise ValueError("mode must be grouped, one_launch or per_instance")
        self.mode = mode
        self.refill = int(refill_lanes)
        self.L, self.sigma, self.div, self.lwl, self.det = L, sigma_frac * L, divergence, lwl, det
        self.phase, self.rtol = phase, rtol
        self.tune, self.tune_rays, self.beam_seed = tune, tune_rays, beam_seed
        self.graph = None

    # ------------------------------------------------------------------ set-up
    def setup(self):
        dev = core.require_cuda()
        n = len(self.inst)
        self.offsets = np.zeros(n + 1, dtype=np.int64)
        for i, p in enumerate(self.inst):
            self.offsets[i + 1] = self.offsets[i] + p["nrays"]
        # contiguous instance ranges of one grid shape
        self.groups = []
        for i, p in enumerate(self.inst):
            if self.groups and self.inst[self.groups[-1][0]]["n"] == p["n"]:
                self.groups[-1][1] = i + 1
            else:
                self.groups.append([i, i + 1])
        ntot = int(self.offsets[-1])
        self.ntot = ntot
        host = torch.empty(6 * ntot, dtype=torch.float64).pin_memory()
        h = host.numpy()
        rng = np.random.default_rng(self.beam_seed)
        self.coords = []
        self.fields = []
        for i, p in enumerate(self.inst):
            ne, x = turboGen.workload_field(p["n"], self.L, p["alpha"], p["delta"], p["ne0"], seed=p["seed"],
                                            dtype=torch.float32)
            self.fields.append(ne)
            self.coords.append(x)
            b, e = self.offsets[i], self.offsets[i + 1]
            gaussian_beam_into(h[6 * b:6 * e].reshape(6, e - b), e - b, self.sigma, self.div, x.max(), rng)
        self.s0 = host.to(dev, non_blocking=True)
        self.extents = [float(x.max()) for x in self.coords]
        self.t_ends = [float(np.linspace(0.0, np.sqrt(8.0) * ex / C_LIGHT, 2)[-1]) for ex in self.extents]
        # autotune brick depth per grid size, and the block size of the batched launch
        self.tuned = {}
        if self.tune:
            for i, p in enumerate(self.inst):
                if p["n"] in self.tuned:
                    continue
                b, e = self.offsets[i], self.offsets[i + 1]
                m = min(self.tune_rays, e - b)
                sample = core.ray_block(self.s0, 6, self.offsets, i)[:, :m].contiguous()
                x = self.coords[i]
                self.tuned[p["n"]] = autotune.tune(self.fields[i], x, x, x, sample, self.t_ends[i], self.extents[i],
                                                   2, lwl=self.lwl, phase=self.phase)
        self.vols = []
        for i, p in enumerate(self.inst):
            bd = self.tuned[p["n"]]["brick_depth"] if self.tune else 8
            x = self.coords[i]
            self.vols.append(core.build_volume(self.fields[i], x, x, x, 2, lwl=self.lwl, brick_depth=bd))
        self.block = 128
        self.out = None
        self.ws = {}
        self.H = torch.zeros((n, self.det, self.det), dtype=torch.float64, device=dev)
        ext_mm = self.L * 1e3
        self.det_range = (-ext_mm, ext_mm)
        f, R = 100.0, 25.0
        self.chain = [(_lib.OPTIC_M_TO_MM, 0, 0, 0), (_lib.OPTIC_DISTANCE, f, 0, 0),
                      (_lib.OPTIC_CIRC_APERTURE, R, 0, 0), (_lib.OPTIC_LENS, f, f, 0),
                      (_lib.OPTIC_DISTANCE, 2 * f, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R, 0, 0),
                      (_lib.OPTIC_LENS, f, f, 0), (_lib.OPTIC_DISTANCE, f, 0, 0)]
        self.step()  # allocates outputs and workspace once
        torch.cuda.synchronize()
        if self.tune:
            # launch mode and lane refill (the library's default, or a warp's 32
            # lanes together), then the block size, timed on the ensemble itself
            self.mode_ms = {}
            for m in ("grouped", "per_instance", "one_launch"):
                for rl in REFILLS:
                    self.mode, self.refill = m, rl
                    self.mode_ms["%s/%d" % (m, rl)] = autotune._time(self._trace_only, 1)
            best = min(self.mode_ms, key=self.mode_ms.get)
            self.mode, self.refill = best.split("/")[0], int(best.split("/")[1])
            self.block_ms = {}
            for b in autotune.BLOCKS:
                self.block = b
                self.block_ms[b] = autotune._time(self._trace_only, 1)
            self.block = min(self.block_ms, key=self.block_ms.get)
        return self

    def _launches(self):
        """(instance range, ray range) of each batched launch."""
        if self.mode == "one_launch":
            ranges = [(0, len(self.inst))]
        elif self.mode == "per_instance":
            ranges = [(i, i + 1) for i in range(len(self.inst))]
        else:
            ranges = [tuple(g) for g in self.groups]
        return [((a, b), (int(self.offsets[a]), int(self.offsets[b]))) for a, b in ranges]

    def _trace_only(self):
        if self.out is None:
            ntot = int(self.offsets[-1])
            dev = self.s0.device
            self.out = dict(sf=torch.empty(6 * ntot, dtype=torch.float64, device=dev),
                            rf=torch.empty(4 * ntot, dtype=torch.float64, device=dev),
                            phase=torch.empty(ntot, dtype=torch.float64, device=dev),
                            status=torch.empty(ntot, dtype=torch.int32, device=dev),
                            nsteps=torch.empty(ntot, dtype=torch.int32, device=dev))
        for (a, b), (r0, r1) in self._launches():
            if r1 == r0:
                continue
            view = {k: v[{"sf": 6, "rf": 4}.get(k, 1) * r0:{"sf": 6, "rf": 4}.get(k, 1) * r1]
                    for k, v in self.out.items() if not k.startswith("_")}
            o = core.trace_f32_batched(self.vols[a:b], self.s0[6 * r0:6 * r1], self.offsets[a:b + 1] - r0,
                                       self.t_ends[a:b], self.extents[a:b], rtol=self.rtol, phase=self.phase,
                                       out=view, ws=self.ws.get((self.mode, a)), block_size=self.block,
                                       refill_lanes=self.refill)
            self.ws[(self.mode, a)] = o["_ws"]

    # ------------------------------------------------------------------ one pass
    def step(self):
        """Enqueue the whole pipeline on the current stream (allocation-free
        after the first call, so it can be captured)."""
        for v in self.vols:
            core.rebuild_volume(v)
        self._trace_only()
        for i in range(len(self.inst)):
            rf = core.ray_block(self.out["rf"], 4, self.offsets, i)
            core.detect(rf, self.chain, self.det, self.det, self.det_range, self.det_range, H=self.H[i])

    def capture(self):
        """Capture step() in a CUDA graph (torch.cuda.graph), after a warm pass."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.step()
        torch.cuda.synchronize()
        return self.graph

    def replay(self):
        self.graph.replay()

    # ------------------------------------------------------------------ reference form
    def run_unbatched(self):
        """The same work one instance at a time (one trace launch per instance,
        the tracer's default options), without a graph: the comparison point
        for batching."""
        outs = []
        for i, v in enumerate(self.vols):
            core.rebuild_volume(v)
            s0 = core.ray_block(self.s0, 6, self.offsets, i)
            o = core.trace_f32(v, s0, self.t_ends[i], self.extents[i], rtol=self.rtol, phase=self.phase,
                               block_size=self.block)
            core.detect(o["rf"], self.chain, self.det, self.det, self.det_range, self.det_range, H=self.H[i])
            outs.append(o)
        return outs

    def ray_steps(self):
        return int(self.out["nsteps"].sum().item())


def _main(argv=None):
    """Trace an ensemble once in each launch mode and print the timings:
    python -m turbulence_tracing_gb300.ensemble --instances 8 --grid 128 --rays 2e5"""
    import argparse
    import json

    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--instances", type=int, default=8)
    ap.add_argument("--grid", type=int, default=0, help="one grid size for all instances (0: drawn)")
    ap.add_argument("--rays", type=float, default=0, help="rays per instance (0: drawn)")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args(argv)
    inst = draw_instances(a.instances, seed=a.seed)
    for p in inst:
        if a.grid:
            p["n"] = a.grid
        if a.rays:
            p["nrays"] = int(a.rays)
    E = Ensemble(inst, tune=False).setup()
    res = {}
    for m in ("grouped", "one_launch", "per_instance"):
        for rl in REFILLS:
            E.mode, E.refill = m, rl
            res["%s/%d" % (m, rl)] = autotune._time(E._trace_only, a.reps)
    print(json.dumps({"instances": len(inst), "rays": E.ntot, "trace_ms_by_mode": res}))


if __name__ == "__main__":
    _main()
