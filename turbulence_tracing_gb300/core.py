"""Device-level API: one function per libturbotrace entry point.

Inputs and outputs are torch CUDA tensors (torch owns every buffer: outputs
and scratch are allocated here and handed to the C ABI as raw pointers).
Work is enqueued on ``torch.cuda.current_stream()``; nothing here
synchronises the host except ``tt_volume_plan`` (pure host arithmetic) and
the FP64 calc_dndr omega (returned through a host scalar).

There is no CPU path: every function raises when CUDA or the library is
unavailable.
"""
import ctypes
import math
import weakref

import numpy as np
import torch

from . import _lib
from ._lib import check

C_LIGHT = 299792458.0


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("turbulence_tracing_gb300 needs a CUDA GPU (sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _f64_dev(a, dev):
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=torch.float64).contiguous()
    tw = device_twin(a)
    if tw is not None and tw.device == dev and tw.dtype == torch.float64:
        return tw
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)


def _dens_dev(ne, dev):
    """Density to the device, keeping float32 as float32 and everything else float64."""
    if isinstance(ne, torch.Tensor):
        t = ne.to(device=dev)
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float64)
        return t.contiguous()
    a = np.asarray(ne)
    if a.dtype == np.float32:
        return torch.as_tensor(np.ascontiguousarray(a), device=dev)
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)


def _dtype_code(t):
    return _lib.TT_F32 if t.dtype == torch.float32 else _lib.TT_F64


# Device twins: host arrays returned with twin=True remember the device tensor
# they were copied from, so handing the same array back to a library call
# (e.g. ElectronCube.rf to a ray_transfer_matrix diagnostic) uses the device
# copy instead of uploading it again.  Such arrays are returned read-only: an
# in-place write needs arr.setflags(write=True) first, which ends the twin
# (a writeable array is always uploaded afresh), so a twin never goes stale.
_twins = {}


def _forget(key):
    _twins.pop(key, None)


def to_host(t, twin=False):
    """Device tensor -> numpy array through a pinned staging buffer (torch's
    caching host allocator), so large results come back at the host link's
    speed rather than through pageable copies.  Each call returns fresh memory.
    twin=True: the array comes back read-only and keeps t as its device twin."""
    if t.numel() * t.element_size() < (1 << 20):
        a = t.cpu().numpy()
    else:
        h = torch.empty(tuple(t.shape), dtype=t.dtype, device="cpu", pin_memory=True)
        h.copy_(t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        a = h.numpy()
    if twin:
        a.flags.writeable = False
        key = id(a)
        _twins[key] = (weakref.ref(a, lambda _r, k=key: _forget(k)), t)
    return a


def device_twin(a):
    """The device tensor a read-only array returned by to_host(twin=True) was
    copied from, or None (not such an array, or made writeable since)."""
    if not isinstance(a, np.ndarray):
        return None
    e = _twins.get(id(a))
    if e is None or e[0]() is not a or a.flags.writeable:
        return None
    return e[1]


def release_twin(a):
    """Drop a's device twin and make a writeable again (for in-place writes)."""
    if isinstance(a, np.ndarray) and id(a) in _twins and _twins[id(a)][0]() is a:
        _forget(id(a))
        a.flags.writeable = True


def workspace(nbytes, dev):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=dev)


# ---------------------------------------------------------------------------
# K1
# ---------------------------------------------------------------------------
def calc_dndr(ne, x, y, z, lwl=1053e-9, ne_max=1.0):
    """FP64 calc_dndr on the GPU.  Returns dict(omega, ne_nc, dndx, dndy, dndz)
    of device tensors shaped like ne (bit-identical to numpy)."""
    dev = require_cuda()
    L = _lib.lib()
    ne_t = _dens_dev(ne, dev)
    if ne_t.dim() != 3:
        raise ValueError("ne must be a 3D array (nx, ny, nz)")
    nx, ny, nz = ne_t.shape
    xs, ys, zs = _f64_dev(x, dev), _f64_dev(y, dev), _f64_dev(z, dev)
    if (xs.numel(), ys.numel(), zs.numel()) != (nx, ny, nz):
        raise ValueError("coordinate lengths %s do not match ne.shape %s"
                         % ((xs.numel(), ys.numel(), zs.numel()), tuple(ne_t.shape)))
    out = {k: torch.empty((nx, ny, nz), dtype=torch.float64, device=dev) for k in ("ne_nc", "dndx", "dndy", "dndz")}
    ws = workspace(L.tt_calc_dndr_workspace_bytes(nx, ny, nz), dev)
    omega = ctypes.c_double(0.0)
    check(L.tt_calc_dndr(_ptr(ne_t), _dtype_code(ne_t), nx, ny, nz, _ptr(xs), _ptr(ys), _ptr(zs), float(lwl),
                         float(ne_max), _ptr(out["ne_nc"]), _ptr(out["dndx"]), _ptr(out["dndy"]),
                         _ptr(out["dndz"]), ctypes.byref(omega), _ptr(ws), ws.numel(), _stream()),
          "tt_calc_dndr")
    out["omega"] = omega.value
    out["coords"] = (xs, ys, zs)
    out["_ws"] = ws  # keep alive until the stream has consumed it
    return out


def dndr(vols, coords, pts):
    """Trilinear lookups (fill 0 outside) of up to 4 FP64 volumes at pts (3, N)."""
    dev = require_cuda()
    L = _lib.lib()
    pts_t = _f64_dev(pts, dev)
    if pts_t.dim() != 2 or pts_t.shape[0] != 3:
        raise ValueError("pts must be (3, N)")
    n = pts_t.shape[1]
    nx, ny, nz = vols[0].shape
    out = torch.empty((len(vols), n), dtype=torch.float64, device=dev)
    arr = (ctypes.c_void_p * len(vols))(*[v.data_ptr() for v in vols])
    xs, ys, zs = coords
    check(L.tt_dndr(arr, len(vols), nx, ny, nz, _ptr(xs), _ptr(ys), _ptr(zs), _ptr(pts_t), n, _ptr(out),
                    _stream()), "tt_dndr")
    return out


def volume_plan(shape, x, y, z, probing_axis, lwl, ne_max=1.0):
    L = _lib.lib()
    vol = _lib.TTVolume()
    xa, ya, za = (np.ascontiguousarray(np.asarray(c, dtype=np.float64)) for c in (x, y, z))
    dp = ctypes.POINTER(ctypes.c_double)
    check(L.tt_volume_plan(shape[0], shape[1], shape[2], xa.ctypes.data_as(dp), ya.ctypes.data_as(dp),
                           za.ctypes.data_as(dp), int(probing_axis), float(lwl), float(ne_max),
                           ctypes.byref(vol)), "tt_volume_plan")
    return vol


class Volume32:
    """FP32 brick volume: the tt_volume descriptor plus the torch tensor holding its nodes."""

    def __init__(self, desc, nodes):
        self.desc = desc
        self.nodes = nodes

    @property
    def nbytes(self):
        return self.nodes.numel() * self.nodes.element_size()


def build_volume(ne, x, y, z, probing_axis=2, lwl=1053e-9, ne_max=1.0, brick_depth=8, nodes=None):
    """K1 FP32: write the brick-tiled node volume from a density (numpy or tensor).
    brick_depth: nodes per brick along the probing axis (4, 8, 16 or 32)."""
    dev = require_cuda()
    L = _lib.lib()
    ne_t = _dens_dev(ne, dev)
    desc = volume_plan(tuple(ne_t.shape), x, y, z, probing_axis, lwl, ne_max)
    if brick_depth != desc.brick_depth:
        check(L.tt_volume_set_brick_depth(ctypes.byref(desc), int(brick_depth)), "tt_volume_set_brick_depth")
    if nodes is None or nodes.numel() < desc.n_float4 * 4:
        nodes = torch.empty((desc.n_float4, 4), dtype=torch.float32, device=dev)
    desc.nodes = nodes.data_ptr()
    check(L.tt_volume_build(ctypes.byref(desc), _ptr(ne_t), _dtype_code(ne_t), _stream()), "tt_volume_build")
    vol = Volume32(desc, nodes)
    vol.density = ne_t  # kept so rebuilding (rebuild_volume) needs no host round trip
    return vol


def rebuild_volume(vol):
    """Re-run K1 into the existing node buffer (enqueue only: graph-capturable)."""
    L = _lib.lib()
    check(L.tt_volume_build(ctypes.byref(vol.desc), _ptr(vol.density), _dtype_code(vol.density), _stream()),
          "tt_volume_build")


# ---------------------------------------------------------------------------
# K2
# ---------------------------------------------------------------------------
def _opts(rtol, atol, atol_phase, max_steps, with_phase, block_size=0, ray_chunk=0, phase_f64=False,
          refill_lanes=0):
    o = _lib.TTTraceOpts()
    o.phase_f64 = 1 if phase_f64 else 0
    o.refill_lanes = int(refill_lanes or 0)
    o.rtol = float(rtol)
    o.atol = float(atol)
    o.atol_phase = float(atol_phase)
    o.max_steps = int(max_steps or 0)
    o.with_phase = 1 if with_phase else 0
    o.block_size = int(block_size or 0)
    o.ray_chunk = int(ray_chunk or 0)
    return o


def _ray_outputs(np_, dev, want_sf=True):
    return dict(sf=torch.empty((6, np_), dtype=torch.float64, device=dev) if want_sf else None,
                rf=torch.empty((4, np_), dtype=torch.float64, device=dev),
                phase=torch.empty((np_,), dtype=torch.float64, device=dev),
                status=torch.empty((np_,), dtype=torch.int32, device=dev),
                nsteps=torch.empty((np_,), dtype=torch.int32, device=dev))


EXPLICIT_RK_METHODS = ("RK23", "RK45", "DOP853")


def rk_tableau(method):
    """tt_rk_tableau of an explicit Runge-Kutta method of scipy.integrate:
    'RK23', 'RK45', 'DOP853' or a RungeKutta subclass (as solve_ivp's `method`
    accepts).  The coefficients are the class attributes solve_ivp itself
    integrates with (A, B, C, E, or E5/E3 for DOP853; error_estimator_order)."""
    import scipy.integrate as si

    cls = getattr(si, method, None) if isinstance(method, str) else method
    if cls is None or not all(hasattr(cls, a) for a in ("A", "B", "C", "n_stages", "error_estimator_order")):
        raise NotImplementedError(
            "method %r: the GPU integrates solve_ivp's explicit Runge-Kutta methods (%s); the implicit "
            "stiff solvers (Radau, BDF, LSODA) are not provided -- the ray equation is not stiff"
            % (method, ", ".join(EXPLICIT_RK_METHODS)))
    ns = int(cls.n_stages)
    if ns not in (3, 6, 12):
        raise NotImplementedError("method %r: %d stages; the GPU kernels take 3, 6 or 12" % (method, ns))
    t = _lib.TTRKTableau()
    t.n_stages = ns
    t.error_order = int(cls.error_estimator_order)
    A = np.asarray(cls.A, dtype=np.float64)
    for i in range(ns):
        for j in range(min(i, A.shape[1])):
            t.A[i][j] = float(A[i, j])
    for i in range(ns):
        t.B[i] = float(np.asarray(cls.B, dtype=np.float64)[i])
        t.C[i] = float(np.asarray(cls.C, dtype=np.float64)[i])
    if hasattr(cls, "E5"):
        t.error_kind = 1
        for i in range(ns + 1):
            t.E[i] = float(cls.E5[i])
            t.E3[i] = float(cls.E3[i])
    else:
        t.error_kind = 0
        for i in range(ns + 1):
            t.E[i] = float(cls.E[i])
    return t


def trace_f64(fields, s0, t_end, probing_axis, extent, rtol=1e-3, atol=1e-6, phase=False, max_steps=None,
              method="RK45"):
    """Plain FP64 drop-in tracer.  fields: dict from calc_dndr.  s0: (6, Np).
    method: solve_ivp's explicit Runge-Kutta methods ('RK45' built in; 'RK23',
    'DOP853' or a scipy RungeKutta subclass through tt_trace_f64_rk)."""
    dev = require_cuda()
    L = _lib.lib()
    tab = None if (isinstance(method, str) and method == "RK45") else rk_tableau(method)
    s0_t = _f64_dev(s0, dev)
    if s0_t.dim() != 2 or s0_t.shape[0] != 6:
        raise ValueError("s0 must be (6, Np)")
    np_ = s0_t.shape[1]
    out = _ray_outputs(np_, dev)
    nx, ny, nz = fields["dndx"].shape
    xs, ys, zs = fields["coords"]
    o = _opts(rtol, atol, 0.0, max_steps, phase)
    args = (_ptr(fields["dndx"]), _ptr(fields["dndy"]), _ptr(fields["dndz"]), _ptr(fields["ne_nc"]),
            nx, ny, nz, _ptr(xs), _ptr(ys), _ptr(zs), float(fields["omega"]), _ptr(s0_t), np_,
            float(t_end), int(probing_axis), float(extent), ctypes.byref(o))
    outs = (_ptr(out["sf"]), _ptr(out["rf"]), _ptr(out["phase"]), _ptr(out["status"]), _ptr(out["nsteps"]),
            _stream())
    if tab is None:
        check(L.tt_trace_f64(*args, *outs), "tt_trace_f64")
    else:
        check(L.tt_trace_f64_rk(*args, ctypes.byref(tab), *outs), "tt_trace_f64_rk")
    return out


def trace_f32(vol, s0, t_end, extent, rtol=1e-7, atol=1e-5, atol_phase=1e-5, phase=False, max_steps=None,
              want_sf=True, ws=None, out=None, block_size=0, ray_chunk=0, phase_f64=False, refill_lanes=0):
    """Persistent FP32 tracer over a Volume32.  s0: (6, Np) float64.
    phase_f64: accumulate the phase in FP64 rather than a compensated FP32 pair.
    refill_lanes: a warp takes new rays once this many lanes are idle (0 = 2;
    32 keeps a warp on 32 neighbouring rays to the end; results are the same)."""
    dev = require_cuda()
    L = _lib.lib()
    s0_t = _f64_dev(s0, dev)
    if s0_t.dim() != 2 or s0_t.shape[0] != 6:
        raise ValueError("s0 must be (6, Np)")
    np_ = s0_t.shape[1]
    if out is None:
        out = _ray_outputs(np_, dev, want_sf)
    need = L.tt_trace_f32_workspace_bytes(ctypes.byref(vol.desc), np_)
    if ws is None or ws.numel() < need:
        ws = workspace(need, dev)
    o = _opts(rtol, atol, atol_phase, max_steps, phase, block_size, ray_chunk, phase_f64, refill_lanes)
    check(L.tt_trace_f32(ctypes.byref(vol.desc), _ptr(s0_t), np_, float(t_end), float(extent), ctypes.byref(o),
                         _ptr(out["sf"]), _ptr(out["rf"]), _ptr(out["phase"]) if phase else None,
                         _ptr(out["status"]), _ptr(out["nsteps"]), _ptr(ws), ws.numel(), _stream()),
          "tt_trace_f32")
    out["_ws"] = ws
    return out


def trace_f32_batched(vols, s0, ray_offsets, t_ends, extents, rtol=1e-7, atol=1e-5, atol_phase=1e-5,
                      phase=False, max_steps=None, want_sf=True, ws=None, out=None, block_size=0, ray_chunk=0,
                      refill_lanes=0):
    """All instances in one persistent launch.  s0 is the instance-blocked ray
    array: a flat float64 tensor holding instance i's (6, n_i) block at
    6 * ray_offsets[i].  Outputs are blocked the same way (see ray_block)."""
    dev = require_cuda()
    L = _lib.lib()
    n = len(vols)
    if not (1 <= n <= _lib.MAX_INSTANCES):
        raise ValueError("1..%d instances per launch" % _lib.MAX_INSTANCES)
    offs = np.ascontiguousarray(np.asarray(ray_offsets, dtype=np.int64))
    ntot = int(offs[-1])
    s0_t = s0 if isinstance(s0, torch.Tensor) and s0.is_cuda else torch.as_tensor(np.asarray(s0), device=dev)
    s0_t = s0_t.reshape(-1)
    if s0_t.dtype != torch.float64 or s0_t.numel() != 6 * ntot:
        raise ValueError("s0 must hold 6 * ray_offsets[-1] float64 values")
    descs = (_lib.TTVolume * n)(*[v.desc for v in vols])
    te = np.ascontiguousarray(np.asarray(t_ends, dtype=np.float64))
    ex = np.ascontiguousarray(np.asarray(extents, dtype=np.float64))
    if out is None:
        out = dict(sf=torch.empty(6 * ntot, dtype=torch.float64, device=dev) if want_sf else None,
                   rf=torch.empty(4 * ntot, dtype=torch.float64, device=dev),
                   phase=torch.empty(ntot, dtype=torch.float64, device=dev),
                   status=torch.empty(ntot, dtype=torch.int32, device=dev),
                   nsteps=torch.empty(ntot, dtype=torch.int32, device=dev))
    need = L.tt_trace_f32_batched_workspace_bytes(descs, n, ntot)
    if ws is None or ws.numel() < need:
        ws = workspace(need, dev)
    o = _opts(rtol, atol, atol_phase, max_steps, phase, block_size, ray_chunk, refill_lanes=refill_lanes)
    dp = ctypes.POINTER(ctypes.c_double)
    check(L.tt_trace_f32_batched(descs, n, offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), te.ctypes.data_as(dp),
                                 ex.ctypes.data_as(dp), _ptr(s0_t), ctypes.byref(o), _ptr(out["sf"]), _ptr(out["rf"]),
                                 _ptr(out["phase"]) if phase else None, _ptr(out["status"]), _ptr(out["nsteps"]),
                                 _ptr(ws), ws.numel(), _stream()), "tt_trace_f32_batched")
    out["_ws"] = ws
    out["_keep"] = (descs, offs, te, ex)
    return out


def ray_block(flat, rows, ray_offsets, i):
    """Instance i's (rows, n_i) view of an instance-blocked array."""
    b, e = int(ray_offsets[i]), int(ray_offsets[i + 1])
    return flat[rows * b:rows * e].view(rows, e - b)


# ---------------------------------------------------------------------------
# K3
# ---------------------------------------------------------------------------
def make_chain(ops):
    """ops: list of (kind, p0, p1, p2) tuples -> ctypes array of tt_optic."""
    if len(ops) > _lib.MAX_OPTICS:
        raise ValueError("at most %d optics per chain" % _lib.MAX_OPTICS)
    arr = (_lib.TTOptic * max(len(ops), 1))()
    for i, op in enumerate(ops):
        arr[i].kind = int(op[0])
        for k, v in enumerate(op[1:4]):
            arr[i].p[k] = float(v)
    return arr, len(ops)


def detect(rf, ops, nbx=1, nby=1, xr=(-1.0, 1.0), yr=(-1.0, 1.0), weights=None, H=None, Hw=None, r_out=False,
           accumulate=False, histogram=True):
    """Push rf (4, N) through the optic chain and (unless histogram=False)
    histogram it.  Returns (H, Hw, r_out) device tensors; H is (nby, nbx) like Rays.H."""
    dev = require_cuda()
    L = _lib.lib()
    rf_t = _f64_dev(rf, dev)
    if rf_t.dim() != 2 or rf_t.shape[0] != 4:
        raise ValueError("rf must be (4, N)")
    n = rf_t.shape[1]
    if histogram and H is None:
        H = torch.empty((nby, nbx), dtype=torch.float64, device=dev)
    w_t = _f64_dev(weights, dev) if weights is not None else None
    if not histogram:
        H, w_t = None, None
    if w_t is not None and Hw is None:
        Hw = torch.empty((nby, nbx), dtype=torch.float64, device=dev)
    ro = torch.empty((4, n), dtype=torch.float64, device=dev) if r_out else None
    chain, nops = make_chain(ops)
    check(L.tt_detect(_ptr(rf_t), n, chain, nops, int(nbx), int(nby), float(xr[0]), float(xr[1]),
                      float(yr[0]), float(yr[1]), _ptr(w_t), _ptr(H), _ptr(Hw) if w_t is not None else None,
                      _ptr(ro), 1 if accumulate else 0, _stream()), "tt_detect")
    return H, (Hw if w_t is not None else None), ro


# ---------------------------------------------------------------------------
# K4
# ---------------------------------------------------------------------------
def straight_line_maps(ne, x, y, z, P, lwl=1053e-9, ne_max=1.0, out=None, nslab=0):
    """(3 + 2 nslab, P, P) float32: straight-line deflection angles (x, y) and
    phase at the centres of a P x P pixel grid over the z = z0 face, then the
    deflection over each of nslab slabs along z (tt_straight_line_maps)."""
    dev = require_cuda()
    ne_t = _dens_dev(ne, dev)
    nx, ny, nz = ne_t.shape
    xa, ya, za = (np.ascontiguousarray(np.asarray(c, dtype=np.float64)) for c in (x, y, z))
    nout = 3 + 2 * int(nslab)
    if out is None:
        out = torch.empty((nout, P, P), dtype=torch.float32, device=dev)
    dp = ctypes.POINTER(ctypes.c_double)
    check(_lib.lib().tt_straight_line_maps(_ptr(ne_t), _dtype_code(ne_t), nx, ny, nz, xa.ctypes.data_as(dp),
                                           ya.ctypes.data_as(dp), za.ctypes.data_as(dp), float(lwl), float(ne_max),
                                           int(P), int(nslab), _ptr(out), _stream()), "tt_straight_line_maps")
    return out


def march_workspace_bytes(shape):
    nx, ny, nz = (int(v) for v in shape)
    return int(_lib.lib().tt_march_maps_workspace_bytes(nx, ny, nz))


def march_batched_workspace_bytes(nfields, shape):
    nx, ny, nz = (int(v) for v in shape)
    return int(_lib.lib().tt_march_maps_batched_workspace_bytes(int(nfields), nx, ny, nz))


def march_maps_batched(fields, x, y, z, P, lwl=1053e-9, ne_max=1.0, out=None, ws=None, plane_stride=1):
    """march_maps over a list of same-shape density tensors in one pass
    (tt_march_maps_batched_stride): (len(fields), 5, P, P) float32.
    plane_stride 2: one march step per two node planes (half the work)."""
    dev = require_cuda()
    nf = len(fields)
    if not (1 <= nf <= _lib.MAX_MARCH_FIELDS):
        raise ValueError("1..%d fields per call" % _lib.MAX_MARCH_FIELDS)
    ts = [_dens_dev(f, dev) for f in fields]
    shape, dt = tuple(ts[0].shape), ts[0].dtype
    if any(tuple(t.shape) != shape or t.dtype != dt for t in ts):
        raise ValueError("fields must share shape and dtype")
    nx, ny, nz = shape
    xa, ya, za = (np.ascontiguousarray(np.asarray(c, dtype=np.float64)) for c in (x, y, z))
    if out is None:
        out = torch.empty((nf, 5, P, P), dtype=torch.float32, device=dev)
    L = _lib.lib()
    need = int(L.tt_march_maps_batched_workspace_bytes(nf, nx, ny, nz))
    if ws is None or ws.numel() < need:
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
    ptrs = (ctypes.c_void_p * nf)(*[t.data_ptr() for t in ts])
    dp = ctypes.POINTER(ctypes.c_double)
    check(L.tt_march_maps_batched_stride(ptrs, nf, _dtype_code(ts[0]), nx, ny, nz, xa.ctypes.data_as(dp),
                                         ya.ctypes.data_as(dp), za.ctypes.data_as(dp), float(lwl), float(ne_max),
                                         int(P), int(plane_stride), _ptr(out), _ptr(ws), need, _stream()),
          "tt_march_maps_batched_stride")
    return out


def march_maps(ne, x, y, z, P, lwl=1053e-9, ne_max=1.0, out=None, ws=None, plane_stride=1):
    """(5, P, P) float32 from one pass over the density (tt_march_maps): exit
    angles (x, y) and phase of the pixel-centre rays marched one node plane per
    step through the ray equation -- the coarse solution the surrogate
    corrects -- then the straight-line deflection angles of the same rays (as
    straight_line_maps).  ws: optional uint8 device workspace of at least
    march_workspace_bytes(ne.shape) bytes, reused across calls."""
    dev = require_cuda()
    ne_t = _dens_dev(ne, dev)
    nx, ny, nz = ne_t.shape
    xa, ya, za = (np.ascontiguousarray(np.asarray(c, dtype=np.float64)) for c in (x, y, z))
    if out is None:
        out = torch.empty((5, P, P), dtype=torch.float32, device=dev)
    need = march_workspace_bytes((nx, ny, nz))
    if ws is None or ws.numel() < need:
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
    dp = ctypes.POINTER(ctypes.c_double)
    if plane_stride == 1:
        check(_lib.lib().tt_march_maps(_ptr(ne_t), _dtype_code(ne_t), nx, ny, nz, xa.ctypes.data_as(dp),
                                       ya.ctypes.data_as(dp), za.ctypes.data_as(dp), float(lwl), float(ne_max),
                                       int(P), _ptr(out), _ptr(ws), need, _stream()), "tt_march_maps")
    else:
        ptrs = (ctypes.c_void_p * 1)(ne_t.data_ptr())
        check(_lib.lib().tt_march_maps_batched_stride(ptrs, 1, _dtype_code(ne_t), nx, ny, nz, xa.ctypes.data_as(dp),
                                                      ya.ctypes.data_as(dp), za.ctypes.data_as(dp), float(lwl),
                                                      float(ne_max), int(P), int(plane_stride), _ptr(out), _ptr(ws),
                                                      need, _stream()), "tt_march_maps_batched_stride")
    return out


def shadowgram(theta, pitch, D, intensity=None, div=None, want_intensity=True, want_div=False):
    """Geometric-optics shadowgram of a (2, P, P) float32 deflection map (tt_shadowgram).
    Returns (intensity, div); either is None when not asked for."""
    dev = require_cuda()
    P = theta.shape[-1]
    if want_intensity and intensity is None:
        intensity = torch.empty((P, P), dtype=torch.float32, device=dev)
    if want_div and div is None:
        div = torch.empty((P, P), dtype=torch.float32, device=dev)
    check(_lib.lib().tt_shadowgram(_ptr(theta), P, float(pitch), float(D),
                                   _ptr(intensity) if want_intensity else None,
                                   _ptr(div) if want_div else None, _stream()), "tt_shadowgram")
    return (intensity if want_intensity else None), (div if want_div else None)


def shadowgram_batched(theta, pitch, D, intensity=None):
    """Intensities (n, P, P) of n deflection maps theta (n, 2, P, P) float32 with
    drifts D (n,) float64 on the device (tt_shadowgram_batched)."""
    dev = require_cuda()
    n, P = theta.shape[0], theta.shape[-1]
    if intensity is None:
        intensity = torch.empty((n, P, P), dtype=torch.float32, device=dev)
    check(_lib.lib().tt_shadowgram_batched(_ptr(theta), n, P, float(pitch), _ptr(D), _ptr(intensity), _stream()),
          "tt_shadowgram_batched")
    return intensity


def _f32_maps(t, nch, name):
    if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.dim() == 4 and t.shape[1] == nch
            and t.shape[2] == t.shape[3]):
        raise ValueError("%s must be a contiguous float32 CUDA tensor (n, %d, P, P)" % (name, nch))


def _f32_dev(t, shape, name):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
            and tuple(t.shape) == tuple(shape)):
        raise ValueError("%s must be a contiguous float32 CUDA tensor of shape %s" % (name, tuple(shape)))


def surrogate_encode(maps, X=None, stats=None):
    """Network input X (n, 6, P, P) and stats (n, 4) = (s, phase mean, phase
    sd, log10(s (P - 1))) from march outputs maps (n, 5, P, P)
    (tt_surrogate_encode)."""
    dev = require_cuda()
    _f32_maps(maps, 5, "maps")
    n, P = maps.shape[0], maps.shape[-1]
    if X is None:
        X = torch.empty((n, 6, P, P), dtype=torch.float32, device=dev)
    if stats is None:
        stats = torch.empty((n, 4), dtype=torch.float32, device=dev)
    _f32_maps(X, 6, "X")
    _f32_dev(stats, (n, 4), "stats")
    if X.shape[0] != n or X.shape[-1] != P:
        raise ValueError("X must be (%d, 6, %d, %d)" % (n, P, P))
    check(_lib.lib().tt_surrogate_encode(_ptr(maps), n, P, _ptr(X), _ptr(stats), _stream()), "tt_surrogate_encode")
    return X, stats


def surrogate_decode(maps, net_out, stats, gain, theta=None, theta_march=None):
    """theta (n, 2, P, P) = marched deflection + s / gain * network output, and
    optionally the marched deflection into theta_march (tt_surrogate_decode)."""
    dev = require_cuda()
    _f32_maps(maps, 5, "maps")
    _f32_maps(net_out, 3, "net_out")
    n, P = maps.shape[0], maps.shape[-1]
    if tuple(net_out.shape) != (n, 3, P, P):
        raise ValueError("net_out must be (%d, 3, %d, %d)" % (n, P, P))
    _f32_dev(stats, (n, 4), "stats")
    _f32_dev(gain, (3,), "gain")
    if theta is None:
        theta = torch.empty((n, 2, P, P), dtype=torch.float32, device=dev)
    _f32_dev(theta, (n, 2, P, P), "theta")
    if theta_march is not None:
        _f32_dev(theta_march, (n, 2, P, P), "theta_march")
    check(_lib.lib().tt_surrogate_decode(_ptr(maps), _ptr(net_out), _ptr(stats), _ptr(gain), n, P, _ptr(theta),
                                         _ptr(theta_march), _stream()), "tt_surrogate_decode")
    return theta


def surrogate_estimate(I_net, I_march, kappa, est=None):
    """est (n,) = kappa ||I_net - I_march|| / ||I_net|| per map (tt_surrogate_estimate)."""
    dev = require_cuda()
    n, P = I_net.shape[0], I_net.shape[-1]
    _f32_dev(I_net, (n, P, P), "I_net")
    _f32_dev(I_march, (n, P, P), "I_march")
    if est is None:
        est = torch.empty(n, dtype=torch.float32, device=dev)
    _f32_dev(est, (n,), "est")
    check(_lib.lib().tt_surrogate_estimate(_ptr(I_net), _ptr(I_march), n, P, float(kappa), _ptr(est), _stream()),
          "tt_surrogate_estimate")
    return est


def grf_field(n, L_box, alpha, ne0, delta, seed, dtype=torch.float32, kmin=None, kmax=None):
    """Band-limited unit-variance GRF density ne0 (1 + delta g) clipped >= 0, (n, n, n)."""
    dev = require_cuda()
    L = _lib.lib()
    kmin = 2 * math.pi / L_box if kmin is None else kmin
    kmax = math.pi * n / L_box if kmax is None else kmax
    out = torch.empty((n, n, n), dtype=dtype, device=dev)
    ws = workspace(L.tt_grf_field_workspace_bytes(n), dev)
    code = _lib.TT_F32 if dtype == torch.float32 else _lib.TT_F64
    check(L.tt_grf_field(int(seed) & 0xFFFFFFFFFFFFFFFF, n, float(L_box), float(alpha), float(kmin), float(kmax),
                         float(ne0), float(delta), code, _ptr(out), _ptr(ws), ws.numel(), _stream()),
          "tt_grf_field")
    del ws
    return out


def grf_fft(N, sqrt_p_half, seed=0, Wr=None, Wi=None):
    """gaussian3D_FFT core: sqrt_p_half (M, M, N+1) device float64."""
    dev = require_cuda()
    L = _lib.lib()
    M = 2 * N + 1
    sp = _f64_dev(sqrt_p_half, dev)
    if tuple(sp.shape) != (M, M, N + 1):
        raise ValueError("sqrt_p_half must be (M, M, N+1)")
    wr = _f64_dev(Wr, dev) if Wr is not None else None
    wi = _f64_dev(Wi, dev) if Wi is not None else None
    out = torch.empty((M, M, M), dtype=torch.float64, device=dev)
    ws = workspace(L.tt_grf_fft_workspace_bytes(N), dev)
    check(L.tt_grf_fft(int(seed) & 0xFFFFFFFFFFFFFFFF, N, _ptr(sp), _ptr(wr), _ptr(wi), _ptr(out), _ptr(ws),
                       ws.numel(), _stream()), "tt_grf_fft")
    return out


def grf_fft_nd(dim, N, sqrt_p_half, seed=0, Wr=None, Wi=None):
    """gaussian{1,2,3}D_FFT core: sqrt_p_half (M,)*(dim-1) + (N+1,) device float64."""
    dev = require_cuda()
    L = _lib.lib()
    M = 2 * N + 1
    sp = _f64_dev(sqrt_p_half, dev)
    if tuple(sp.shape) != (M,) * (dim - 1) + (N + 1,):
        raise ValueError("sqrt_p_half must be (M,)*(dim-1) + (N+1,)")
    wr = _f64_dev(Wr, dev) if Wr is not None else None
    wi = _f64_dev(Wi, dev) if Wi is not None else None
    out = torch.empty((M,) * dim, dtype=torch.float64, device=dev)
    ws = workspace(L.tt_grf_fft_nd_workspace_bytes(dim, N), dev)
    check(L.tt_grf_fft_nd(int(seed) & 0xFFFFFFFFFFFFFFFF, dim, N, _ptr(sp), _ptr(wr), _ptr(wi), _ptr(out), _ptr(ws),
                          ws.numel(), _stream()), "tt_grf_fft_nd")
    return out


def cos_field(dim, n, d, k, phase, amp):
    """Cosine-sum field at cell centres (tt_cos_field): n, d per axis (dim
    entries), k (3, nm), phase (4, nm), amp (nm) float64."""
    dev = require_cuda()
    nm = int(np.asarray(amp).shape[0])
    kt = _f64_dev(np.zeros((3, nm)) if nm == 0 else k, dev).contiguous()
    pt = _f64_dev(np.zeros((4, nm)) if nm == 0 else phase, dev).contiguous()
    at = _f64_dev(amp, dev).contiguous()
    nn = list(n) + [1] * (3 - dim)
    dd = list(d) + [1.0] * (3 - dim)
    out = torch.empty(tuple(nn[:dim]), dtype=torch.float64, device=dev)
    check(_lib.lib().tt_cos_field(dim, nn[0], nn[1], nn[2], float(dd[0]), float(dd[1]), float(dd[2]), nm, _ptr(kt),
                                  _ptr(pt), _ptr(at), _ptr(out), _stream()), "tt_cos_field")
    return out


def philox(seed, tag, count):
    dev = require_cuda()
    out = torch.empty((4, count), dtype=torch.int32, device=dev)
    check(_lib.lib().tt_philox(int(seed) & 0xFFFFFFFFFFFFFFFF, int(tag) & 0xFFFFFFFF, int(count), _ptr(out),
                               _stream()), "tt_philox")
    return out
