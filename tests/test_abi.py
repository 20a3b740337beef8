"""The C ABI without a GPU: the library loads, exports every entry point the
header declares, and the host-only paths (argument checks, volume planning)
behave."""
import ctypes
import re
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT


def _declared():
    src = open(ROOT + "/include/turbotrace.h").read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(tt_\w+)\s*\(", src, re.M)))


def test_header_symbols_exported():
    from turbulence_tracing_gb300 import _lib

    L = _lib.lib()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, n
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.library_path()], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert set(names) <= exported


def test_status_strings_and_version():
    from turbulence_tracing_gb300 import _lib

    L = _lib.lib()
    assert L.tt_abi_version() == 1
    for code in range(0, 7):
        assert L.tt_strerror(code)


def test_argument_checks_without_gpu():
    from turbulence_tracing_gb300 import _lib

    L = _lib.lib()
    assert L.tt_calc_dndr(None, 1, 1, 4, 4, None, None, None, 1e-6, 1.0, None, None, None, None, None,
                          None, 0, None) == 1
    assert b"at least 2 points" in L.tt_last_error_detail()
    opts = _lib.TTTraceOpts()
    opts.rtol = 0.0
    assert L.tt_trace_f64(None, None, None, None, 4, 4, 4, None, None, None, 1.0, None, 0, 1.0, 2, 1.0,
                          ctypes.byref(opts), None, None, None, None, None, None) == 1
    chain = (_lib.TTOptic * 1)()
    chain[0].kind = 99
    assert L.tt_detect(None, 0, chain, 1, 4, 4, -1.0, 1.0, -1.0, 1.0, None, ctypes.c_void_p(16), None, None, 0,
                       None) == 1
    chain[0].kind = _lib.OPTIC_KNIFE_EDGE
    chain[0].p[2] = 0.0
    assert L.tt_detect(None, 0, chain, 1, 4, 4, -1.0, 1.0, -1.0, 1.0, None, ctypes.c_void_p(16), None, None, 0,
                       None) == 1
    assert b"knife edge direction" in L.tt_last_error_detail()


def test_volume_plan_geometry():
    from turbulence_tracing_gb300 import _lib, core

    x = np.linspace(-2.5e-3, 2.5e-3, 512)
    v = core.volume_plan((512, 512, 512), x, x, x, 2, 1064e-9)
    assert list(v.n) == [512, 512, 512] and list(v.axis) == [0, 1, 2]
    assert list(v.tiles) == [128, 128] and list(v.supertiles) == [16, 16] and v.bricks_c == 64
    assert v.n_float4 == 16 * 16 * 64 * 64 * 200
    y = np.linspace(0, 1e-3, 30)
    z = np.linspace(0, 2e-3, 70)
    v = core.volume_plan((512, 30, 70), x, y, z, 0, 1064e-9)
    assert list(v.axis) == [1, 2, 0] and list(v.n) == [30, 70, 512]
    assert v.spacing[2] == pytest.approx(5e-3 / 511)
    with pytest.raises(_lib.TTError):
        core.volume_plan((10, 10, 10), np.cumsum(np.arange(1, 11.0)), x[:10], x[:10], 2, 1064e-9)


def test_trace_f32_options_checked_before_any_launch():
    """tt_trace_opts is validated before the FP32 tracer touches the device
    (with np = 0 the call returns right after the checks)."""
    from turbulence_tracing_gb300 import _lib, core

    L = _lib.lib()
    x = np.linspace(-1e-3, 1e-3, 40)
    v = core.volume_plan((40, 40, 40), x, x, x, 2, 1064e-9)
    v.nodes = ctypes.c_void_p(256)  # never dereferenced: no ray is traced
    for refill, want in ((0, 0), (1, 0), (32, 0), (33, 1), (-1, 1)):
        o = core._opts(1e-7, 1e-5, 1e-5, None, True, refill_lanes=refill)
        assert L.tt_trace_f32(ctypes.byref(v), None, 0, 1e-11, 1e-3, ctypes.byref(o), None, None, None, None, None,
                              None, 0, None) == want, refill
    assert b"refill_lanes" in L.tt_last_error_detail()
    o = core._opts(1e-7, 1e-5, 1e-5, None, True, block_size=96)
    assert L.tt_trace_f32(ctypes.byref(v), None, 0, 1e-11, 1e-3, ctypes.byref(o), None, None, None, None, None,
                          None, 0, None) == 1
    o = core._opts(1e-7, 1e-5, 1e-5, None, True, ray_chunk=48)
    assert L.tt_trace_f32(ctypes.byref(v), None, 0, 1e-11, 1e-3, ctypes.byref(o), None, None, None, None, None,
                          None, 0, None) == 1


def test_trace_f32_batched_arguments_checked_before_any_launch():
    """Instance count (1..TT_MAX_INSTANCES) and the ray offsets are checked
    before the batched tracer touches the device."""
    from turbulence_tracing_gb300 import _lib, core

    L = _lib.lib()
    x = np.linspace(-1e-3, 1e-3, 20)
    v = core.volume_plan((20, 20, 20), x, x, x, 2, 1064e-9)
    v.nodes = ctypes.c_void_p(256)  # never dereferenced: no ray is traced
    n = _lib.MAX_INSTANCES + 1
    descs = (_lib.TTVolume * n)(*([v] * n))
    o = core._opts(1e-7, 1e-5, 1e-5, None, False)
    dp = ctypes.POINTER(ctypes.c_double)

    def call(ninst, offs):
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        te = np.full(max(ninst, 1), 1e-11)
        return L.tt_trace_f32_batched(descs, ninst, offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                      te.ctypes.data_as(dp), te.ctypes.data_as(dp), None, ctypes.byref(o), None,
                                      None, None, None, None, None, 0, None)

    assert call(_lib.MAX_INSTANCES, np.zeros(_lib.MAX_INSTANCES + 1)) == 0  # all empty: nothing to trace
    assert call(n, np.zeros(n + 1)) == 1
    assert call(0, np.zeros(1)) == 1
    assert call(2, [1, 2, 3]) == 1       # offsets must start at 0
    assert call(2, [0, 5, 3]) == 1       # and not decrease


def test_no_gpu_means_loud_failure():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from turbulence_tracing_gb300 import core

    with pytest.raises(RuntimeError, match="CUDA"):
        core.calc_dndr(np.zeros((4, 4, 4)), np.arange(4.0), np.arange(4.0), np.arange(4.0))


def test_march_and_shadowgram_arguments_checked_before_any_launch():
    """Invalid calls are refused by the library's own checks (no CUDA call is
    made), with the status and a detail string."""
    import ctypes

    from turbulence_tracing_gb300 import _lib

    L = _lib.lib(build_if_missing=False)
    x = np.linspace(0.0, 1e-3, 8)
    dp = ctypes.POINTER(ctypes.c_double)
    xp = x.ctypes.data_as(dp)
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: every call below fails its checks first
    assert L.tt_march_maps_workspace_bytes(1, 8, 8) == 0
    need = L.tt_march_maps_workspace_bytes(8, 8, 8)
    assert need > 8 * 8 * 8 * 4
    assert L.tt_march_maps_batched_workspace_bytes(3, 8, 8, 8) >= 3 * need - 3 * 256
    cases = [
        (lambda: L.tt_march_maps(None, _lib.TT_F32, 8, 8, 8, xp, xp, xp, 1e-6, 1.0, 8, fake, fake, need, None),
         b"NULL"),

        (lambda: L.tt_march_maps(fake, _lib.TT_F32, 8, 8, 1, xp, xp, xp, 1e-6, 1.0, 8, fake, fake, need, None),
         b"bad sizes"),
        (lambda: L.tt_march_maps(fake, 7, 8, 8, 8, xp, xp, xp, 1e-6, 1.0, 8, fake, fake, need, None), b"ne_dtype"),
        (lambda: L.tt_march_maps(fake, _lib.TT_F32, 8, 8, 8, xp, xp, xp, 1e-6, 1.0, 8, fake,
                                 ctypes.c_void_p(0x1004), need, None), b"aligned"),
        (lambda: L.tt_march_maps_batched((ctypes.c_void_p * 1)(fake), 0, _lib.TT_F32, 8, 8, 8, xp, xp, xp, 1e-6, 1.0,
                                         8, fake, fake, need, None), b"fields"),
        (lambda: L.tt_march_maps_batched((ctypes.c_void_p * 33)(*([fake] * 33)), 33, _lib.TT_F32, 8, 8, 8, xp, xp, xp,
                                         1e-6, 1.0, 8, fake, fake, 33 * need, None), b"fields"),
        (lambda: L.tt_surrogate_encode(fake, 0, 8, fake, fake, None), b"bad arguments"),
        (lambda: L.tt_surrogate_encode(fake, 1, 8, fake, ctypes.c_void_p(0x1004), None), b"aligned"),
        (lambda: L.tt_surrogate_decode(fake, fake, fake, None, 1, 8, fake, None, None), b"bad arguments"),
        (lambda: L.tt_surrogate_estimate(fake, fake, 1, 8, -1.0, fake, None), b"bad arguments"),
        (lambda: L.tt_shadowgram_batched(fake, 0, 8, 1e-5, fake, fake, None), b"bad arguments"),
        (lambda: L.tt_shadowgram_batched(fake, 2, 1, 1e-5, fake, fake, None), b"bad arguments"),
        (lambda: L.tt_shadowgram_batched(fake, 2, 8, 0.0, fake, fake, None), b"bad arguments"),
    ]
    for call, detail in cases:
        assert call() == 1  # invalid argument
        assert detail in L.tt_last_error_detail(), L.tt_last_error_detail()
    assert L.tt_march_maps(fake, _lib.TT_F32, 8, 8, 8, xp, xp, xp, 1e-6, 1.0, 8, fake, fake, need - 4, None) == 2
    assert b"workspace needs" in L.tt_last_error_detail()
