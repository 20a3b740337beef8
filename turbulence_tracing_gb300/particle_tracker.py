"""Drop-in replacement for turbulence_tracing's ``particle_tracker`` module.

Same class, methods, keyword defaults and attribute layouts as
particle_tracking/particle_tracker.py (ElectronCube :121-395, dsdt :398-419);
the gradient, the lookups and the ray integration run in libturbotrace on the
GPU.  Ray arrays keep the reference's shapes: s0 and sf are (6, Np) float64
[x, y, z, vx, vy, vz] in m and m/s, rf is (4, Np) [x, theta, y, phi] in m and
rad on the exit plane.

Additions (keyword-only, defaults keep the reference behaviour):
  solve(method='RK45', rtol=None, atol=None, precision='fp64', phase=False, max_steps=None)
    precision='fp64'  plain drop-in: per-ray RK45 (or solve_ivp's RK23 / DOP853)
                      with scipy's controller, rtol/atol default to solve_ivp's
                      1e-3 / 1e-6;
    precision='fp32'  persistent FP32 tracer (uniform grids), rtol default 1e-7
                      on velocity/phase, atol default 1e-5 cells;
    phase=True        also integrates k0 * int (n - 1) ds into self.phase.
  set_up_interps()    (re)builds the FP64 device lookup state now (calc_dndr
                      defers it to first use).
  rf, phase, status and nsteps from a solve of host rays are read-only numpy
  arrays that keep their device copies (setflags(write=True) before writing
  into one in place).
  self.status, self.nsteps  per-ray outcome and accepted-step count.
"""
from datetime import datetime
from time import time

import numpy as np
import torch

from . import core

c = 299792458.0  # scipy.constants.c (particle_tracker.py:118)

_AXIS = {"x": 0, "y": 1, "z": 2}


class _DeviceInterp:
    """Stand-in for the RegularGridInterpolator objects calc_dndr stores
    (particle_tracker.py:239-241): called with (N, 3) points, returns (N,)."""

    def __init__(self, cube, which):
        self._cube = cube
        self._which = which

    def __call__(self, xi):
        xi = np.asarray(xi, dtype=np.float64)
        pts = np.atleast_2d(xi).reshape(-1, 3).T
        f = self._cube._fields()
        out = core.dndr([f[self._which]], f["coords"], pts)
        return out[0].cpu().numpy().reshape(xi.shape[:-1] if xi.ndim > 1 else (1,))


class ElectronCube:
    """A class to hold and generate electron density cubes (drop-in)."""

    def __init__(self, x, y, z, probing_direction="z"):
        self.z, self.y, self.x = z, y, x
        self.extent_x = x.max()
        self.extent_y = y.max()
        self.extent_z = z.max()
        self.probing_direction = probing_direction
        self._dev = None
        self._vol32 = None
        self._host_cache = {}
        self._dndr_args = None

    # --- densities (particle_tracker.py:147-218), host arrays as in the reference
    def test_null(self):
        self.XX, self.YY, self.ZZ = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        self.ne = np.zeros_like(self.XX)

    def test_slab(self, s=1, n_e0=2e23):
        self.XX, self.YY, self.ZZ = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        self.ne = n_e0 * (1.0 + s * self.XX / self.extent_x)

    def test_linear_cos(self, s1=0.1, s2=0.1, n_e0=2e23, Ly=1):
        self.XX, self.YY, self.ZZ = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        self.ne = n_e0 * (1.0 + s1 * self.XX / self.extent_x) * (1 + s2 * np.cos(2 * np.pi * self.YY / Ly))

    def test_exponential_cos(self, n_e0=1e24, Ly=1e-3, s=2e-3):
        self.XX, self.YY, self.ZZ = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        self.ne = n_e0 * 10 ** (self.XX / s) * (1 + np.cos(2 * np.pi * self.YY / Ly))

    def test_lens(self, n_e0=1e24, LR=1e-3):
        self.XX, self.YY, self.ZZ = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        RR = np.sqrt(self.XX ** 2 + self.YY ** 2)
        self.ne = n_e0 * np.exp(-RR ** 2 / LR ** 2)

    def test_liner(self, n_e0=1e24, LR=1e-3):
        self.XX, self.YY, self.ZZ = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        RR = np.sqrt(self.XX ** 2 + self.ZZ ** 2)
        self.ne = n_e0 * np.exp(-RR ** 2 / LR ** 2)

    def external_ne(self, ne):
        """Load an externally generated grid (numpy array or torch tensor, CPU or CUDA)."""
        self.ne = ne

    # --- gradient and lookups (particle_tracker.py:220-256)
    def calc_dndr(self, lwl=1053e-9, ne_max=1):
        """Gradient of n_e/n_c times -c^2/2 on the GPU; builds the lookups.
        The FP64 arrays are formed when first used (the FP64 solve, dndr, the
        ne_nc/dndx/dndy/dndz attributes); the FP32 tracer builds its own
        volume from ne, so a precision='fp32' solve never forms them."""
        self._dndr_args = (lwl, ne_max)
        self._dev = None
        self._vol32 = None
        self._host_cache = {}
        self.omega = 2 * np.pi * (c / lwl)  # particle_tracker.py:227
        self._interps()

    def set_up_interps(self):
        """(Re)build the device state now: FP64 ne_nc and gradients
        (bit-identical to numpy) and the trilinear lookups.  Idempotent."""
        if self._dndr_args is None:
            raise RuntimeError("call calc_dndr(lwl, ne_max) first")
        lwl, ne_max = self._dndr_args
        f = core.calc_dndr(self.ne, self.x, self.y, self.z, lwl=lwl, ne_max=ne_max)
        self._dev = f
        self._vol32 = None
        self._host_cache = {}
        self.omega = f["omega"]
        self._interps()

    def _interps(self):
        self.dndx_interp = _DeviceInterp(self, "dndx")
        self.dndy_interp = _DeviceInterp(self, "dndy")
        self.dndz_interp = _DeviceInterp(self, "dndz")

    def _fields(self):
        if self._dev is None:
            self.set_up_interps()
        return self._dev

    def _host(self, name):
        if name not in self._host_cache:
            self._host_cache[name] = self._fields()[name].cpu().numpy()
        return self._host_cache[name]

    ne_nc = property(lambda self: self._host("ne_nc"))
    dndx = property(lambda self: self._host("dndx"))
    dndy = property(lambda self: self._host("dndy"))
    dndz = property(lambda self: self._host("dndz"))

    # sf (6, Np), the final ray states: after a solve from host rays it stays on
    # the device until first read (the diagnostics use rf), then it is the same
    # numpy array the reference keeps.
    @property
    def sf(self):
        d = self.__dict__
        if d.get("_sf_dev") is not None:
            d["_sf"] = core.to_host(d["_sf_dev"])
            d["_sf_dev"] = None
        if "_sf" not in d:
            raise AttributeError("'ElectronCube' object has no attribute 'sf'")
        return d["_sf"]

    @sf.setter
    def sf(self, value):
        self.__dict__["_sf"] = value
        self.__dict__["_sf_dev"] = None

    def volume32(self):
        """The FP32 brick volume for the probing direction (built on first use)."""
        if self._vol32 is None:
            lwl, ne_max = self._dndr_args
            self._vol32 = core.build_volume(self.ne, self.x, self.y, self.z, _AXIS[self.probing_direction],
                                            lwl=lwl, ne_max=ne_max)
        return self._vol32

    def dndr(self, x):
        """Gradients at the (3, N) locations x, 0 outside the grid."""
        f = self._fields()
        out = core.dndr([f["dndx"], f["dndy"], f["dndz"]], f["coords"], np.asarray(x, dtype=np.float64))
        return out.cpu().numpy()

    # --- beam (particle_tracker.py:258-310): host numpy, same draws as the reference
    def init_beam(self, Np, beam_size, divergence):
        s0 = np.zeros((6, Np))
        t = 2 * np.pi * np.random.rand(Np)
        u = np.random.rand(Np) + np.random.rand(Np)
        u[u > 1] = 2 - u[u > 1]
        phi = np.pi * np.random.rand(Np)
        chi = divergence * np.random.randn(Np)
        if self.probing_direction == "x":
            self.extent = self.extent_x
            s0[3, :] = c * np.cos(chi)
            s0[4, :] = c * np.sin(chi) * np.cos(phi)
            s0[5, :] = c * np.sin(chi) * np.sin(phi)
            s0[0, :] = self.extent
            s0[1, :] = beam_size * u * np.cos(t)
            s0[2, :] = beam_size * u * np.sin(t)
        elif self.probing_direction == "y":
            self.extent = self.extent_y
            s0[4, :] = c * np.cos(chi)
            s0[3, :] = c * np.sin(chi) * np.cos(phi)
            s0[5, :] = c * np.sin(chi) * np.sin(phi)
            s0[0, :] = beam_size * u * np.cos(t)
            s0[1, :] = -self.extent
            s0[2, :] = beam_size * u * np.sin(t)
        elif self.probing_direction == "z":
            self.extent = self.extent_z
            s0[3, :] = c * np.sin(chi) * np.cos(phi)
            s0[4, :] = c * np.sin(chi) * np.sin(phi)
            s0[5, :] = c * np.cos(chi)
            s0[0, :] = beam_size * u * np.cos(t)
            s0[1, :] = beam_size * u * np.sin(t)
            s0[2, :] = -self.extent
        self.s0 = s0

    def _extent(self):
        if not hasattr(self, "extent"):
            self.extent = {"x": self.extent_x, "y": self.extent_y, "z": self.extent_z}[self.probing_direction]
        return self.extent

    # --- integration (particle_tracker.py:312-331)
    def solve(self, method="RK45", *, rtol=None, atol=None, precision="fp64", phase=False, max_steps=None):
        """Trace self.s0 to t_end (particle_tracker.py:312-331).  method is
        solve_ivp's: 'RK45' (default), 'RK23', 'DOP853' or an explicit
        RungeKutta subclass, integrated per ray in FP64 with scipy's step
        control; the implicit methods (Radau, BDF, LSODA) raise
        NotImplementedError.  precision='fp32' is the persistent FP32 tracer,
        which integrates RK45 only."""
        if precision == "fp32" and not (isinstance(method, str) and method == "RK45"):
            raise NotImplementedError("precision='fp32' integrates RK45 (Dormand-Prince 5(4)) only")
        if precision == "fp64" and not (isinstance(method, str) and method == "RK45"):
            core.rk_tableau(method)  # raises for methods the GPU does not integrate
        extent = self._extent()
        t = np.linspace(0.0, np.sqrt(8.0) * extent / c, 2)
        t_end = t[-1]
        on_device = isinstance(self.s0, torch.Tensor) and self.s0.is_cuda
        start = time()
        if precision == "fp64":
            out = core.trace_f64(self._fields(), self.s0, t_end, _AXIS[self.probing_direction], extent,
                                 rtol=1e-3 if rtol is None else rtol, atol=1e-6 if atol is None else atol,
                                 phase=phase, max_steps=max_steps, method=method)
        elif precision == "fp32":
            if self._dndr_args is None:
                raise RuntimeError("call calc_dndr(lwl, ne_max) first")
            out = core.trace_f32(self.volume32(), self.s0, t_end, extent,
                                 rtol=1e-7 if rtol is None else rtol, atol=1e-5 if atol is None else atol,
                                 phase=phase, max_steps=max_steps)
        else:
            raise ValueError("precision must be 'fp64' or 'fp32'")
        torch.cuda.current_stream().synchronize()
        finish = time()
        print("Ray trace completed in:\t", finish - start, "s")
        # host rays in -> host arrays out; rf and phase keep their device copies
        # as twins (read-only arrays), so diagnostics given them upload nothing
        conv = (lambda t_: t_) if on_device else (lambda t_: core.to_host(t_, twin=True))
        if on_device:
            self.sf = out["sf"]
        else:
            self.__dict__["_sf_dev"] = out["sf"]  # copied on first read of self.sf
        self.rf = conv(out["rf"])
        self.status = conv(out["status"])
        self.nsteps = conv(out["nsteps"])
        if phase:
            self.phase = conv(out["phase"])
        return self.rf

    def ray_at_exit(self):
        """Back-project self.sf to the exit plane (particle_tracker.py:333-380); runs on the GPU."""
        dev = core.require_cuda()
        lazy = self.__dict__.get("_sf_dev")
        host = lazy is not None or not isinstance(self.sf, torch.Tensor)
        if lazy is not None:
            sf = lazy
        else:
            sf = self.sf if isinstance(self.sf, torch.Tensor) else torch.as_tensor(np.asarray(self.sf), device=dev)
        sf = sf.to(device=dev, dtype=torch.float64)
        x, y, z, vx, vy, vz = sf
        extent = self._extent()
        rp = torch.zeros((4, sf.shape[1]), dtype=torch.float64, device=dev)
        if self.probing_direction == "x":
            t_bp = (x - extent) / vx
            rp[0], rp[2], rp[1], rp[3] = y - vy * t_bp, z - vz * t_bp, torch.atan(vy / vx), torch.atan(vz / vx)
        elif self.probing_direction == "y":
            t_bp = (y - extent) / vy
            rp[0], rp[2], rp[1], rp[3] = x - vx * t_bp, z - vz * t_bp, torch.atan(vx / vy), torch.atan(vz / vy)
        elif self.probing_direction == "z":
            t_bp = (z - extent) / vz
            rp[0], rp[2], rp[1], rp[3] = x - vx * t_bp, y - vy * t_bp, torch.atan(vx / vz), torch.atan(vy / vz)
        if not host:
            return rp
        return rp.cpu().numpy()

    def save_output_rays(self, fn=None):
        """np.save of rf to '<fn>.npy' or '<date>_<time> rays.npy' (particle_tracker.py:382-395)."""
        now = datetime.now()
        dt_string = now.strftime("%Y-%m-%d_%H-%M-%S")
        if fn is None:
            fn = "{} rays.npy".format(dt_string)
        else:
            fn = "{}.npy".format(fn)
        rf = self.rf.cpu().numpy() if isinstance(self.rf, torch.Tensor) else self.rf
        with open(fn, "wb") as f:
            np.save(f, rf)

    # --- pickling (the reference's multiprocess driver pickles bound methods)
    def __getstate__(self):
        if self.__dict__.get("_sf_dev") is not None:
            self.sf  # bring the final states to the host before pickling
        st = dict(self.__dict__)
        st["_dev"] = None
        st["_vol32"] = None
        st["_host_cache"] = {}
        for k in ("dndx_interp", "dndy_interp", "dndz_interp"):
            st.pop(k, None)
        return st

    def __setstate__(self, st):
        self.__dict__.update(st)
        if self._dndr_args is not None:
            self.dndx_interp = _DeviceInterp(self, "dndx")
            self.dndy_interp = _DeviceInterp(self, "dndy")
            self.dndz_interp = _DeviceInterp(self, "dndz")


def dsdt(t, s, ElectronCube):
    """Right-hand side for an ODE solver (particle_tracker.py:398-419): s is the
    flattened (6, Np) state; returns the flattened derivative."""
    Np = s.size // 6
    s = s.reshape(6, Np)
    sprime = np.zeros_like(s)
    sprime[3:6, :] = ElectronCube.dndr(s[:3, :])
    sprime[:3, :] = s[3:, :]
    return sprime.flatten()
