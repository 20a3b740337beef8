"""Drop-in replacement for turbulence_tracing's ``ray_transfer_matrix`` module.

Same functions and classes as particle_tracking/ray_transfer_matrix.py:37-299.
Rays are (4, N) arrays [x, theta, y, phi]; the module-level functions act on
numpy arrays or torch tensors (filters modify their argument in place and
return it, as the reference's ``r[:, filt] = None`` does).  The diagnostics
record their optic chain in solve(); the chain and the histogram run as one
fused GPU kernel (libturbotrace tt_detect) when histogram() is called, and
``rf`` is produced on first access.  Plotting (plot_afr, Rays.plot) is not
part of this library: no graphics stack is used.
"""
import numpy as np
import torch

from . import _lib
from . import core


def _is_t(r):
    return isinstance(r, torch.Tensor)


def _run_chain(r, ops, inplace):
    """Apply ops to r (4, N) on the GPU; writes back into r when inplace."""
    if r.ndim != 2 or r.shape[0] != 4:
        raise ValueError("rays must be a (4, N) array")
    _, _, out = core.detect(r, ops, r_out=True, histogram=False)
    if _is_t(r):
        if inplace:
            r.copy_(out.to(dtype=r.dtype, device=r.device))
            return r
        return out
    host = out.cpu().numpy()
    if inplace:
        core.release_twin(r)  # an in-place filter on a solve() result: writeable again, twin dropped
        r[...] = host
        return r
    return host


def m_to_mm(r):
    return _run_chain(r, [(_lib.OPTIC_M_TO_MM, 0, 0, 0)], inplace=False)


def lens(r, f1, f2):
    """4x4 thin-lens matrix applied to r (ray_transfer_matrix.py:42-54)."""
    return _run_chain(r, [(_lib.OPTIC_LENS, f1, f2, 0)], inplace=False)


def sym_lens(r, f):
    return lens(r, f, f)


def distance(r, d):
    """4x4 free-space matrix applied to r (ray_transfer_matrix.py:62-71)."""
    return _run_chain(r, [(_lib.OPTIC_DISTANCE, d, 0, 0)], inplace=False)


def circular_aperture(r, R):
    """Rejects (NaN) rays outside radius R, in place (ray_transfer_matrix.py:73-79)."""
    return _run_chain(r, [(_lib.OPTIC_CIRC_APERTURE, R, 0, 0)], inplace=True)


def circular_stop(r, R):
    """Rejects rays inside radius R, in place (ray_transfer_matrix.py:81-87)."""
    return _run_chain(r, [(_lib.OPTIC_CIRC_STOP, R, 0, 0)], inplace=True)


def annular_stop(r, R1, R2):
    """Boolean mask of rays with R1 < r < R2 (ray_transfer_matrix.py:89-97); r untouched."""
    t = r if _is_t(r) else torch.as_tensor(np.asarray(r, dtype=np.float64), device=core.require_cuda())
    q = t[0] ** 2 + t[2] ** 2
    m = (q > R1 ** 2) & (q < R2 ** 2)
    return m if _is_t(r) else m.cpu().numpy()


def _annuli(Rs):
    Rs = list(np.asarray(Rs, dtype=np.float64).ravel())
    return [(_lib.OPTIC_ANNULUS_STOP, Rs[2 * i], Rs[2 * i + 1], 0) for i in range(len(Rs) // 2)]


def angular_filter(r, Rs):
    """Rejects rays inside any annulus (Rs[2i], Rs[2i+1]), in place (ray_transfer_matrix.py:99-111)."""
    return _run_chain(r, _annuli(Rs), inplace=True)


def rect_aperture(r, Lx, Ly):
    """Rejects rays with x^2 > Lx^2 AND y^2 > Ly^2 -- the reference's test, kept
    as is (ray_transfer_matrix.py:128-136)."""
    return _run_chain(r, [(_lib.OPTIC_RECT_APERTURE, Lx, Ly, 0)], inplace=True)


def _knife(offset, axis, direction):
    if axis not in ("x", "y"):
        raise ValueError("knife_edge axis must be 'x' or 'y'")
    if direction == 0:
        raise ValueError("Direction must be <0 or >0")
    return (_lib.OPTIC_KNIFE_EDGE, offset, 2 if axis == "y" else 0, 1.0 if direction > 0 else -1.0)


def knife_edge(r, offset, axis, direction):
    """Rejects rays beyond a knife edge, in place (ray_transfer_matrix.py:138-154)."""
    return _run_chain(r, [_knife(offset, axis, direction)], inplace=True)


def plot_afr(Rs):
    raise NotImplementedError("plotting is not part of turbulence_tracing_gb300 (no graphics stack)")


class Rays:
    """Inheritable class for ray diagnostics (ray_transfer_matrix.py:156-206)."""

    def __init__(self, r0, focal_plane=0, L=400, R=25, Lx=18, Ly=13.5):
        self.focal_plane, self.L, self.R, self.Lx, self.Ly = focal_plane, L, R, Lx, Ly
        # rays as given (m); the m -> mm conversion is the first op of the fused chain
        self._src = r0
        self._src_in_m = True
        self._ops = None
        self._rf = None

    # r0 reads as the mm-converted copy that Rays.__init__ stores
    @property
    def r0(self):
        if self._src is None:
            return None
        return m_to_mm(self._src) if self._src_in_m else self._src

    @r0.setter
    def r0(self, v):
        # an assigned r0 is taken to be in mm already, as in the reference
        self._src = v
        self._src_in_m = False
        self._rf = None

    @property
    def _r0_m(self):
        return self._src

    def _chain(self):
        head = [(_lib.OPTIC_M_TO_MM, 0, 0, 0)] if self._src_in_m else []
        return head + list(self._ops)

    def _set_ops(self, ops):
        self._ops = ops
        self._rf = None

    @property
    def rf(self):
        if self._rf is None and self._ops is not None and self._r0_m is not None:
            _, _, out = core.detect(self._r0_m, self._chain(), r_out=True, histogram=False)
            self._rf = out if _is_t(self._r0_m) else core.to_host(out)
        return self._rf

    @rf.setter
    def rf(self, v):
        self._rf = v

    def histogram(self, bin_scale=10, pix_x=3448, pix_y=2574, clear_mem=False, weights=None):
        """Bin the detector-plane rays (ray_transfer_matrix.py:173-195).  H is
        (pix_y//bin_scale, pix_x//bin_scale) like the reference's H.T.  With
        weights (e.g. phase per ray) also fills self.Hw, the weighted sum per bin."""
        if self._ops is None:
            raise RuntimeError("call solve() before histogram()")
        nbx, nby = pix_x // bin_scale, pix_y // bin_scale
        xr = (-self.Lx / 2, self.Lx / 2)
        yr = (-self.Ly / 2, self.Ly / 2)
        # the detector-plane rays (self.rf) are computed when first read, not here
        H, Hw, _ = core.detect(self._r0_m, self._chain(), nbx, nby, xr, yr, weights=weights)
        on_dev = _is_t(self._r0_m)
        self.H = H if on_dev else core.to_host(H)
        if Hw is not None:
            self.Hw = Hw if on_dev else core.to_host(Hw)
        self.xedges = np.linspace(xr[0], xr[1], nbx + 1)
        self.yedges = np.linspace(yr[0], yr[1], nby + 1)
        if clear_mem:
            self.clear_rays()

    def plot(self, ax, clim=None, cmap=None):
        raise NotImplementedError("plotting is not part of turbulence_tracing_gb300 (no graphics stack)")

    def clear_rays(self):
        self._src = None
        self._rf = None


class Shadowgraphy(Rays):
    """Two-lens 1:1 relay with apertures (ray_transfer_matrix.py:208-227)."""

    def solve(self):
        L, R, fp = self.L, self.R, self.focal_plane
        self._set_ops([(_lib.OPTIC_DISTANCE, L - fp, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R, 0, 0),
                       (_lib.OPTIC_LENS, L, L, 0), (_lib.OPTIC_DISTANCE, L * 2, 0, 0),
                       (_lib.OPTIC_CIRC_APERTURE, R, 0, 0), (_lib.OPTIC_LENS, L, L, 0),
                       (_lib.OPTIC_DISTANCE, L, 0, 0)])


class _Schlieren(Rays):
    def _focal_chain(self, focal_op):
        L, R, fp = self.L, self.R, self.focal_plane
        return [(_lib.OPTIC_DISTANCE, L - fp, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R, 0, 0),
                (_lib.OPTIC_LENS, L, L, 0), (_lib.OPTIC_DISTANCE, L, 0, 0)] + focal_op + \
               [(_lib.OPTIC_DISTANCE, L, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R, 0, 0),
                (_lib.OPTIC_LENS, L, L, 0), (_lib.OPTIC_DISTANCE, L, 0, 0)]


class Schlieren_DF(_Schlieren):
    """Dark-field schlieren: circular stop at the focal plane (ray_transfer_matrix.py:229-250)."""

    def solve(self, R=1):
        self._set_ops(self._focal_chain([(_lib.OPTIC_CIRC_STOP, R, 0, 0)]))


class Schlieren_LF(_Schlieren):
    """Light-field schlieren: circular aperture at the focal plane (ray_transfer_matrix.py:252-273)."""

    def solve(self, R=1):
        self._set_ops(self._focal_chain([(_lib.OPTIC_CIRC_APERTURE, R, 0, 0)]))


class Schlieren_KE(_Schlieren):
    """Knife-edge schlieren: Schlieren_DF's relay with knife_edge
    (ray_transfer_matrix.py:138-154) at the focal plane in place of the stop."""

    def solve(self, offset=0.0, axis="x", direction=1):
        self._set_ops(self._focal_chain([_knife(offset, axis, direction)]))


class AFR(Rays):
    """Angular fringe refractometry: f = L/2 relay with annular stops (ray_transfer_matrix.py:275-299)."""

    def solve(self, Rs):
        L, R, fp = self.L, self.R, self.focal_plane
        self._set_ops([(_lib.OPTIC_DISTANCE, L / 2 - fp, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R, 0, 0),
                       (_lib.OPTIC_LENS, L / 2, L / 2, 0), (_lib.OPTIC_DISTANCE, L / 4, 0, 0)] + _annuli(Rs) +
                      [(_lib.OPTIC_DISTANCE, L / 4, 0, 0), (_lib.OPTIC_CIRC_APERTURE, R, 0, 0),
                       (_lib.OPTIC_LENS, L / 2, L / 2, 0), (_lib.OPTIC_DISTANCE, L / 2, 0, 0)])
