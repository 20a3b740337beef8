"""Batched ensemble (one persistent launch over many realisations, CUDA-graph
pipeline, autotuned block and brick shapes) against the single-volume tracer,
which the other tests tie to the oracle.  A ray's arithmetic does not depend
on which launch, block size or brick depth carries it, so the comparisons
are exact."""
import numpy as np
import pytest
import torch

from oracle import restated as R
from tests.cases import LWL, errors, oracle_trace

pytestmark = pytest.mark.gpu


def _small_ensemble(phase=True, **kw):
    from turbulence_tracing_gb300 import ensemble

    inst = ensemble.draw_instances(n_inst=7, seed=3, sizes=(24, 32, 40), rays=(200, 3000))
    inst[2]["nrays"] = 0  # an instance with no rays
    return ensemble.Ensemble(inst, L=1e-3, det=64, phase=phase, **kw).setup()


@pytest.mark.parametrize("mode,phase", [("grouped", True), ("one_launch", True), ("grouped", False),
                                        ("one_launch", False)])
def test_batched_equals_single_launches(cuda, mode, phase):
    """grouped: one uniform-shape launch per grid size; one_launch: one mixed-shape launch;
    with the phase and without it (each a kernel of its own)."""
    from turbulence_tracing_gb300 import core

    E = _small_ensemble(phase=phase, tune=False, mode=mode)
    torch.cuda.synchronize()
    rf_b = E.out["rf"].clone()
    ph_b = E.out["phase"].clone()
    ns_b = E.out["nsteps"].clone()
    singles = E.run_unbatched()
    torch.cuda.synchronize()
    for i, o in enumerate(singles):
        b, e = E.offsets[i], E.offsets[i + 1]
        assert torch.equal(core.ray_block(rf_b, 4, E.offsets, i), o["rf"])
        if phase:
            assert torch.equal(ph_b[b:e], o["phase"][: e - b])
        assert torch.equal(ns_b[b:e], o["nsteps"][: e - b])
    assert (E.out["status"] == 0).all()


def test_batched_at_the_instance_limit(cuda):
    """TT_MAX_INSTANCES volumes of mixed shapes in one launch (the whole table
    a kernel parameter): every instance equals its own single launch."""
    from turbulence_tracing_gb300 import _lib, core

    n = _lib.MAX_INSTANCES
    rng = np.random.default_rng(7)
    vols, s0s, xs = [], [], []
    for i in range(n):
        m = int(rng.choice((10, 12, 14)))
        ne, x = R.workload_density(m, 1e-3, -11 / 3, 0.2, 1e24, i)
        vols.append(core.build_volume(ne, x, x, x, 2, lwl=LWL))
        s0s.append(R.gaussian_beam(int(rng.integers(1, 80)), 0.25e-3, 1e-4, x.max(), rng))
        xs.append(x)
    offs = np.concatenate([[0], np.cumsum([s.shape[1] for s in s0s])])
    flat = np.concatenate([s.reshape(-1) for s in s0s])
    t_ends = [R.t_end(x.max()) for x in xs]
    ext = [x.max() for x in xs]
    for rl in (0, 32):
        o = core.trace_f32_batched(vols, flat, offs, t_ends, ext, phase=True, refill_lanes=rl)
        for i in (0, 1, n // 2, n - 1):
            single = core.trace_f32(vols[i], s0s[i], t_ends[i], ext[i], phase=True)
            assert torch.equal(core.ray_block(o["rf"], 4, offs, i), single["rf"]), (rl, i)
            assert torch.equal(o["nsteps"][offs[i]:offs[i + 1]], single["nsteps"]), (rl, i)
        assert (o["status"] == 0).all()


def test_batched_instance_against_oracle(cuda):
    from turbulence_tracing_gb300 import core

    E = _small_ensemble(tune=False)
    i = int(np.argmax(np.diff(E.offsets)))
    x = E.coords[i]
    ne = E.fields[i].double().cpu().numpy()
    s0 = core.ray_block(E.s0, 6, E.offsets, i)[:, :300].cpu().numpy()
    ref = oracle_trace(ne, x, s0)
    rf = core.ray_block(E.out["rf"], 4, E.offsets, i)[:, :300].cpu().numpy()
    b = E.offsets[i]
    ph = E.out["phase"][b:b + 300].cpu().numpy()
    e = errors(rf, ref["rf"], 2 * x.max(), ph, ref["phase"])
    assert e["pos"] <= 1e-6 and e["ang"] <= 1e-6 and e["phase"] <= 1e-3, e


def test_brick_depth_and_block_size_do_not_change_results(cuda):
    from turbulence_tracing_gb300 import core

    ne, x = R.workload_density(36, 1e-3, -5 / 3, 0.2, 5e24, 4)
    s0 = R.gaussian_beam(2000, 0.25e-3, 1e-3, x.max(), np.random.default_rng(2))
    t_end = R.t_end(x.max())
    ref = None
    for bd in (4, 8, 16, 32):
        vol = core.build_volume(ne, x, x, x, 2, lwl=LWL, brick_depth=bd)
        for block in (64, 128, 256):
            o = core.trace_f32(vol, s0, t_end, x.max(), phase=True, block_size=block)
            got = (o["rf"].cpu(), o["phase"].cpu(), o["nsteps"].cpu())
            if ref is None:
                ref = got
            else:
                assert all(torch.equal(a, b) for a, b in zip(got, ref)), (bd, block)


def test_refill_lanes_do_not_change_results(cuda):
    """A warp refilled lane by lane (refill_lanes 1) or 32 lanes at a time
    carries each ray through the same arithmetic: single and batched launches
    agree bit for bit."""
    from turbulence_tracing_gb300 import core

    ne, x = R.workload_density(36, 1e-3, -5 / 3, 0.2, 5e24, 4)
    s0 = R.gaussian_beam(3000, 0.25e-3, 1e-3, x.max(), np.random.default_rng(5))
    t_end = R.t_end(x.max())
    vol = core.build_volume(ne, x, x, x, 2, lwl=LWL)
    ref = core.trace_f32(vol, s0, t_end, x.max(), phase=True)
    for rl in (8, 32):
        o = core.trace_f32(vol, s0, t_end, x.max(), phase=True, refill_lanes=rl)
        for k in ("rf", "sf", "phase", "nsteps", "status"):
            assert torch.equal(o[k], ref[k]), (rl, k)
    E1 = _small_ensemble(tune=False, mode="one_launch")
    torch.cuda.synchronize()
    out1 = {k: v.clone() for k, v in E1.out.items()}
    E1.refill = 32
    E1._trace_only()
    torch.cuda.synchronize()
    for k in ("rf", "phase", "nsteps", "status"):
        assert torch.equal(E1.out[k], out1[k]), k


def test_graph_replay_matches_eager(cuda):
    E = _small_ensemble(tune=False)
    torch.cuda.synchronize()
    H_eager = E.H.clone()
    rf_eager = E.out["rf"].clone()
    E.out["rf"].zero_()
    E.H.zero_()
    E.capture()
    E.replay()
    torch.cuda.synchronize()
    assert torch.equal(E.out["rf"], rf_eager)
    assert torch.equal(E.H, H_eager)
    assert E.H.sum().item() > 0
    E.replay()  # a second replay gives the same again
    torch.cuda.synchronize()
    assert torch.equal(E.H, H_eager)


def test_autotune_picks_a_candidate_and_caches(cuda, tmp_path):
    from turbulence_tracing_gb300 import autotune

    ne, x = R.workload_density(32, 1e-3, -11 / 3, 0.2, 1e24, 1)
    s0 = R.gaussian_beam(3000, 0.25e-3, 5e-5, x.max(), np.random.default_rng(0))
    cache = str(tmp_path / "tune.json")
    r1 = autotune.tune(ne, x, x, x, s0, R.t_end(x.max()), x.max(), lwl=LWL, blocks=(64, 128),
                       brick_depths=(8, 16), cache_file=cache, force=True)
    assert r1["block"] in (64, 128) and r1["brick_depth"] in (8, 16)
    assert len(r1["ms"]) == 4 and all(v > 0 for v in r1["ms"].values())
    r2 = autotune.tune(ne, x, x, x, s0, R.t_end(x.max()), x.max(), lwl=LWL, cache_file=cache)
    assert r2 == r1
