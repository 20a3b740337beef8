"""ctypes front end of the C oracle (tt_oracle.c).  Test infrastructure only.

Functions mirror the reference call sites they restate:
  calc_dndr  -- particle_tracking/particle_tracker.py:220-237
  interp     -- RegularGridInterpolator built at particle_tracker.py:239-241
  trace      -- solve (:312-331) with dsdt (:398-419) and dndr (:243-256),
                one ray per RK45 instance; optional phase as a 7th state
  histogram2d-- ray_transfer_matrix.py:182-191
"""
import ctypes
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import build_oracle

C_LIGHT = 299792458.0

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.tto_calc_dndr.restype = ctypes.c_double
        L.tto_calc_dndr.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                    _dp, _dp, _dp, _dp]
        L.tto_interp.restype = None
        L.tto_interp.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 _dp, _dp, _dp, _dp, ctypes.c_int64, _dp]
        L.tto_trace.restype = ctypes.c_int
        L.tto_trace.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                _dp, _dp, _dp, ctypes.c_double, _dp, ctypes.c_int64,
                                ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int64,
                                _dp, _dp, _i64p, _i64p, _i64p, _i32p]
        L.tto_trace_rk.restype = ctypes.c_int
        L.tto_trace_rk.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   _dp, _dp, _dp, ctypes.c_double, _dp, ctypes.c_int64,
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int64,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp,
                                   _dp, _dp, _i64p, _i64p, _i64p, _i32p]
        L.tto_histogram2d.restype = None
        L.tto_histogram2d.argtypes = [_dp, _dp, _dp, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a, t=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def calc_dndr(ne, x, y, z, lwl=1053e-9, ne_max=1.0):
    """Returns (omega, ne_nc, dndx, dndy, dndz) as ElectronCube.calc_dndr computes them."""
    ne = _f64(ne)
    x, y, z = _f64(x), _f64(y), _f64(z)
    nx, ny, nz = ne.shape
    ne_nc = np.empty_like(ne)
    dndx = np.empty_like(ne)
    dndy = np.empty_like(ne)
    dndz = np.empty_like(ne)
    omega = lib().tto_calc_dndr(_p(ne), nx, ny, nz, _p(x), _p(y), _p(z), float(lwl),
                                float(ne_max), _p(ne_nc), _p(dndx), _p(dndy), _p(dndz))
    return omega, ne_nc, dndx, dndy, dndz


def interp(vol, x, y, z, pts):
    """Trilinear lookup with fill 0 outside the grid; pts is (3, N) like dndr's x."""
    vol = _f64(vol)
    P = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).T)
    out = np.empty(P.shape[0])
    nx, ny, nz = vol.shape
    lib().tto_interp(_p(vol), nx, ny, nz, _p(_f64(x)), _p(_f64(y)), _p(_f64(z)),
                     _p(P), P.shape[0], _p(out))
    return out


def default_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def rk_pair(method):
    """(ns, kind, order, A, B, E, E3) of a scipy.integrate RungeKutta method
    ('RK23', 'RK45', 'DOP853' or a RungeKutta subclass): the class attributes
    solve_ivp itself integrates with."""
    import scipy.integrate as si

    cls = getattr(si, method) if isinstance(method, str) else method
    ns = int(cls.n_stages)
    a = np.asarray(cls.A, dtype=np.float64)
    A = np.zeros((ns, ns))
    A[:, :min(ns, a.shape[1])] = a[:ns, :ns]
    B = _f64(np.asarray(cls.B)[:ns])
    if hasattr(cls, "E5"):
        return ns, 1, int(cls.error_estimator_order), A, B, _f64(cls.E5), _f64(cls.E3)
    return ns, 0, int(cls.error_estimator_order), A, B, _f64(cls.E), _f64(np.zeros(ns + 1))


def trace(dndx, dndy, dndz, x, y, z, s0, t_end, rtol=1e-10, atol=1e-12,
          ne_nc=None, omega=None, max_steps=10_000_000, threads=None, method=None):
    """Integrate every ray of s0 (6, Np) with its own RK45 instance (or the
    scipy RungeKutta method `method`, e.g. 'RK23', 'DOP853').

    Returns dict(sf=(6,Np), phase=(Np,) or None, nacc, nrej, nfev, status).
    Phase is integrated (as a 7th state) when ne_nc and omega are given.
    """
    dndx, dndy, dndz = _f64(dndx), _f64(dndy), _f64(dndz)
    x, y, z = _f64(x), _f64(y), _f64(z)
    s0 = _f64(s0)
    Np = s0.shape[1]
    with_phase = ne_nc is not None
    ne_nc_a = _f64(ne_nc) if with_phase else None
    sf = np.empty_like(s0)
    phase = np.zeros(Np)
    nacc = np.zeros(Np, np.int64)
    nrej = np.zeros(Np, np.int64)
    nfev = np.zeros(Np, np.int64)
    status = np.zeros(Np, np.int32)
    nx, ny, nz = dndx.shape
    L = lib()
    threads = threads or default_threads()
    chunk = max(1, -(-Np // (threads * 4)))

    rk = rk_pair(method) if method not in (None, "RK45") else None

    def run(first):
        cnt = min(chunk, Np - first)
        if rk is None:
            L.tto_trace(_p(dndx), _p(dndy), _p(dndz), _p(ne_nc_a), nx, ny, nz,
                        _p(x), _p(y), _p(z), float(omega or 0.0), _p(s0), Np, first, cnt,
                        float(t_end), float(rtol), float(atol), int(with_phase), int(max_steps),
                        _p(sf), _p(phase), _p(nacc, _i64p), _p(nrej, _i64p), _p(nfev, _i64p),
                        _p(status, _i32p))
        else:
            ns, kind, order, A, B, E, E3 = rk
            L.tto_trace_rk(_p(dndx), _p(dndy), _p(dndz), _p(ne_nc_a), nx, ny, nz,
                           _p(x), _p(y), _p(z), float(omega or 0.0), _p(s0), Np, first, cnt,
                           float(t_end), float(rtol), float(atol), int(with_phase), int(max_steps),
                           ns, kind, order, _p(A), _p(B), _p(E), _p(E3),
                           _p(sf), _p(phase), _p(nacc, _i64p), _p(nrej, _i64p), _p(nfev, _i64p),
                           _p(status, _i32p))

    starts = list(range(0, Np, chunk))
    if threads == 1 or len(starts) == 1:
        for s in starts:
            run(s)
    else:
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(run, starts))
    return dict(sf=sf, phase=phase if with_phase else None, nacc=nacc, nrej=nrej,
                nfev=nfev, status=status)


def histogram2d(xs, ys, nbx, nby, xr, yr, weights=None):
    """H (nby, nbx) as Rays.histogram leaves it (transposed histogram2d)."""
    xs, ys = _f64(xs), _f64(ys)
    w = _f64(weights) if weights is not None else None
    xe = np.linspace(xr[0], xr[1], nbx + 1)
    ye = np.linspace(yr[0], yr[1], nby + 1)
    H = np.empty((nby, nbx))
    lib().tto_histogram2d(_p(xs), _p(ys), _p(w), xs.size, nbx, nby, float(xr[0]), float(xr[1]),
                          float(yr[0]), float(yr[1]), _p(xe), _p(ye), _p(H))
    return H, xe, ye
