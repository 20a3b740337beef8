"""K3 (ray_transfer_matrix.py:37-299) on the GPU vs the reference's own
outputs (golden fixtures) and the numpy restatement.  Counts are exact."""
import numpy as np
import pytest
import torch

from oracle import restated as R
from tests.conftest import golden

pytestmark = pytest.mark.gpu


def _diag(cls, r0, kw, sv):
    from turbulence_tracing_gb300 import ray_transfer_matrix as rtm

    obj = getattr(rtm, cls)(r0=r0.copy(), **kw)
    obj.solve(**sv)
    return obj


CASES = [("Shadowgraphy", dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6), {}),
         ("Schlieren_DF", dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6), dict(R=3)),
         ("Schlieren_LF", dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6), dict(R=3)),
         ("AFR", dict(focal_plane=5, L=100, R=25, Lx=15, Ly=10), dict(Rs=np.arange(0, 6, 0.5)))]


def edge_ties(rf, xe, ye, tol=1e-9):
    """Rays whose detector coordinate sits within tol of a bin edge: their bin can
    move with the last bit of the matrix products (the reference's matmul may
    fuse multiply-adds), which the parity bar allows."""
    x, y = rf[0], rf[2]
    ok = ~(np.isnan(x) | np.isnan(y))
    dx = np.min(np.abs(x[ok][:, None] - xe[None, :]), axis=1)
    dy = np.min(np.abs(y[ok][:, None] - ye[None, :]), axis=1)
    return int(((dx < tol) | (dy < tol)).sum())


@pytest.mark.parametrize("cls,kw,sv", CASES, ids=[c[0] for c in CASES])
def test_diagnostics_vs_reference(cuda, cls, kw, sv):
    d = golden("rtm")
    obj = _diag(cls, d["r0"], kw, sv)
    obj.histogram(bin_scale=25)
    assert np.array_equal(obj.xedges, d[f"{cls}_xe"]) and np.array_equal(obj.yedges, d[f"{cls}_ye"])
    rf = obj.rf
    assert np.array_equal(np.isnan(rf), np.isnan(d[f"{cls}_rf"]))
    np.testing.assert_allclose(rf, d[f"{cls}_rf"], rtol=1e-13, atol=1e-12)
    for bs, px, py, key in ((25, 3448, 2574, "H"), (10, 500, 300, "H2")):
        obj.histogram(bin_scale=bs, pix_x=px, pix_y=py)
        # binning rule exact on our own rays
        assert np.array_equal(obj.H, R.histogram(rf, kw["Lx"], kw["Ly"], bin_scale=bs, pix_x=px, pix_y=py)[0])
        # against the reference: only edge ties may move, each between two bins
        moved = np.abs(obj.H - d[f"{cls}_{key}"]).sum()
        assert obj.H.sum() == d[f"{cls}_{key}"].sum()
        assert moved <= 2 * edge_ties(d[f"{cls}_rf"], obj.xedges, obj.yedges), (key, moved)


def test_light_plus_dark_field_is_shadowgraphy(cuda):
    rng = np.random.default_rng(3)
    r0 = np.vstack([rng.normal(0, 1.5e-3, 200000), rng.normal(0, 3e-3, 200000),
                    rng.normal(0, 1.5e-3, 200000), rng.normal(0, 3e-3, 200000)])
    kw = dict(focal_plane=0, L=400, R=25, Lx=6, Ly=6)
    sh = _diag("Shadowgraphy", r0, kw, {})
    df = _diag("Schlieren_DF", r0, kw, dict(R=1.2))
    lf = _diag("Schlieren_LF", r0, kw, dict(R=1.2))
    for o in (sh, df, lf):
        o.histogram(bin_scale=5)
    assert np.array_equal(df.H + lf.H, sh.H)
    assert sh.H.sum() > 0 and df.H.sum() > 0 and lf.H.sum() > 0


def test_large_detector_and_weights_vs_numpy(cuda):
    """2048^2 detector (global-atomic path) and a phase-weighted histogram."""
    from turbulence_tracing_gb300 import core, _lib

    rng = np.random.default_rng(5)
    n = 300000
    rf = np.vstack([rng.normal(0, 2e-3, n), rng.normal(0, 1e-3, n), rng.normal(0, 2e-3, n), rng.normal(0, 1e-3, n)])
    w = rng.normal(-70, 3, n)
    ops = [(_lib.OPTIC_M_TO_MM, 0, 0, 0), (_lib.OPTIC_DISTANCE, 100, 0, 0), (_lib.OPTIC_CIRC_APERTURE, 25, 0, 0),
           (_lib.OPTIC_LENS, 100, 100, 0), (_lib.OPTIC_DISTANCE, 100, 0, 0),
           (_lib.OPTIC_KNIFE_EDGE, 0.0, 0, 1.0), (_lib.OPTIC_DISTANCE, 100, 0, 0),
           (_lib.OPTIC_CIRC_APERTURE, 25, 0, 0), (_lib.OPTIC_LENS, 100, 100, 0), (_lib.OPTIC_DISTANCE, 100, 0, 0)]
    for nb in (64, 2048):
        H, Hw, ro = core.detect(rf, ops, nb, nb, (-8, 8), (-8, 8), weights=w, r_out=True)
        want_r = R.schlieren_knife(R.m_to_mm(rf), 100, 25, 0.0, "x", 1)
        np.testing.assert_allclose(ro.cpu().numpy(), want_r, rtol=1e-13, atol=1e-12)
        Hn, _, _ = R.histogram(want_r, 16, 16, bin_scale=1, pix_x=nb, pix_y=nb)
        Hwn, _, _ = R.histogram(want_r, 16, 16, bin_scale=1, pix_x=nb, pix_y=nb, weights=w)
        assert np.array_equal(H.cpu().numpy(), Hn)
        np.testing.assert_allclose(Hw.cpu().numpy(), Hwn, rtol=1e-12, atol=1e-9)


def test_module_functions_in_place(cuda):
    from turbulence_tracing_gb300 import ray_transfer_matrix as rtm

    d = golden("rtm")
    rr = d["r0"] * 1e3
    a = rr.copy()
    out = rtm.knife_edge(a, 0.5, "x", 1)
    assert out is a and np.array_equal(a, d["knife_x_pos"], equal_nan=True)
    a = rr.copy()
    rtm.knife_edge(a, -0.5, "y", -1)
    assert np.array_equal(a, d["knife_y_neg"], equal_nan=True)
    a = rr.copy()
    rtm.rect_aperture(a, 2.0, 3.0)
    assert np.array_equal(a, d["rect"], equal_nan=True)
    np.testing.assert_allclose(rtm.lens(rr.copy(), 100.0, 50.0), d["lens"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(rtm.distance(rr.copy(), 123.0), d["dist"], rtol=1e-13, atol=1e-13)
    m = rtm.annular_stop(rr, 1.0, 3.0)
    assert np.array_equal(m, R.annular_stop(rr, 1.0, 3.0))
    with pytest.raises(ValueError):
        rtm.knife_edge(rr.copy(), 0.0, "x", 0)
    t = torch.as_tensor(rr.copy(), device="cuda")
    rtm.circular_aperture(t, 2.0)
    assert np.array_equal(t.cpu().numpy(), R.circular_aperture(rr.copy(), 2.0), equal_nan=True)


def test_empty_and_all_rejected(cuda):
    from turbulence_tracing_gb300 import ray_transfer_matrix as rtm

    sh = rtm.Shadowgraphy(np.zeros((4, 0)), L=400, R=25, Lx=6, Ly=6)
    sh.solve()
    sh.histogram(bin_scale=25)
    assert sh.H.shape == (2574 // 25, 3448 // 25) and sh.H.sum() == 0
    r = np.full((4, 10), np.nan)
    sh = rtm.Shadowgraphy(r, L=400, R=25, Lx=6, Ly=6)
    sh.solve()
    sh.histogram(bin_scale=25)
    assert sh.H.sum() == 0
