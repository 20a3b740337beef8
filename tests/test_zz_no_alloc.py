"""tt_calc_dndr_noalloc: the allocation-free calc_dndr for callers that
cannot allocate device memory (a host application whose memory manager owns
every device buffer and allows no allocation behind its back).

Called through the C ABI and compared with tt_calc_dndr (which takes a caller
workspace) on two calls in a row with different grids, so a stale table from
the first call would show in the second.  Both are bit-exact ports of
numpy.gradient, so the comparison is exact.  This file sorts last so that a
failure here comes after every other test has run."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _run(L, fn, ne, x, y, z, lwl, ne_max, ws=None):
    dev = ne.device
    nx, ny, nz = ne.shape
    out = [torch.empty((nx, ny, nz), dtype=torch.float64, device=dev) for _ in range(4)]
    om = ctypes.c_double(0.0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    code = 0 if ne.dtype == torch.float32 else 1
    if fn == "noalloc":
        rc = L.tt_calc_dndr_noalloc(_p(ne), code, nx, ny, nz, _p(x), _p(y), _p(z), lwl, ne_max, _p(out[0]),
                                    _p(out[1]), _p(out[2]), _p(out[3]), ctypes.byref(om), stream)
    else:
        rc = L.tt_calc_dndr(_p(ne), code, nx, ny, nz, _p(x), _p(y), _p(z), lwl, ne_max, _p(out[0]), _p(out[1]),
                            _p(out[2]), _p(out[3]), ctypes.byref(om), _p(ws), ws.numel(), stream)
    torch.cuda.synchronize()
    return rc, om.value, [o.cpu().numpy() for o in out]


def test_calc_dndr_noalloc_matches_workspace_version(cuda):
    from turbulence_tracing_gb300 import _lib

    L = _lib.lib()
    rng = np.random.default_rng(0)
    cases = [
        # non-uniform x (coefficient tables with per-node values), float64 density
        ((40, 33, 28), np.sort(rng.uniform(-1e-3, 1e-3, 40)), np.float64),
        # a different, smaller uniform grid, float32 density: any stale table entry would show
        ((17, 21, 9), np.linspace(-5e-4, 5e-4, 17), np.float32),
    ]
    for (nx, ny, nz), x, dt in cases:
        y = np.linspace(-2e-3, 2e-3, ny)
        z = np.cumsum(rng.uniform(1e-5, 3e-5, nz))
        ne = (1e25 * rng.uniform(0.5, 1.5, (nx, ny, nz))).astype(dt)
        dev = cuda
        ne_t = torch.as_tensor(ne, device=dev)
        xs, ys, zs = (torch.as_tensor(a, dtype=torch.float64, device=dev) for a in (x, y, z))
        ws = torch.empty(L.tt_calc_dndr_workspace_bytes(nx, ny, nz), dtype=torch.uint8, device=dev)
        rc_a, om_a, want = _run(L, "workspace", ne_t, xs, ys, zs, 1064e-9, 1.0, ws)
        rc_b, om_b, got = _run(L, "noalloc", ne_t, xs, ys, zs, 1064e-9, 1.0)
        assert rc_a == 0 and rc_b == 0, (rc_a, rc_b, L.tt_last_error_detail())
        assert om_a == om_b
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_calc_dndr_noalloc_rejects_grids_above_its_limit(cuda):
    from turbulence_tracing_gb300 import _lib

    L = _lib.lib()
    nx = 8193  # one node above the fixed tables' per-axis capacity
    ne = torch.zeros((nx, 2, 2), dtype=torch.float64, device=cuda)
    xs = torch.linspace(0, 1, nx, dtype=torch.float64, device=cuda)
    ys = torch.linspace(0, 1, 2, dtype=torch.float64, device=cuda)
    rc, _, _ = _run(L, "noalloc", ne, xs, ys, ys, 1064e-9, 1.0)
    assert rc == 6  # TT_ERR_TOO_LARGE
    assert b"at most 8192 nodes per axis" in L.tt_last_error_detail()
