"""The oracle's other Runge-Kutta methods (solve(method=...): the reference
hands `method` to solve_ivp, particle_tracker.py:312, 323) pinned to scipy's
own solve_ivp.

One ray at a time through scipy.integrate.solve_ivp with the reference's
right-hand side (dsdt, :398-419: x' = v, v' = the RegularGridInterpolator
lookups of the gradients built at :239-241), against the C oracle's generic
RungeKutta restatement with the tableau scipy's class holds.  The two sum the
stages in different orders (numpy's dot products against sequential sums), so
their step sequences part where a step's error lands near the acceptance
threshold at the interpolant's cell-face kinks: the accepted-step counts
agree within 10% (the three methods differ from one another by 30-70% at
these tolerances) and the final states within a few times the tolerance."""
import numpy as np
import pytest
from scipy.integrate import solve_ivp
from scipy.interpolate import RegularGridInterpolator

from oracle import restated as R
from oracle import tto
from tests.cases import LWL, grf_case


@pytest.mark.parametrize("method,rtol,atol", [("RK23", 1e-6, 1e-9), ("DOP853", 1e-9, 1e-12), ("RK45", 1e-7, 1e-10)])
def test_generic_rk_oracle_follows_solve_ivp(method, rtol, atol):
    ne, x, s0 = grf_case(n=12, nrays=3, ne0=5e24, ray_seed=5)
    om, q, gx, gy, gz = tto.calc_dndr(ne, x, x, x, LWL, 1.0)
    interps = [RegularGridInterpolator((x, x, x), g, bounds_error=False, fill_value=0.0) for g in (gx, gy, gz)]

    def dsdt(t, s):
        p = s[:3][None, :]
        return np.concatenate([s[3:], [f(p)[0] for f in interps]])

    t_end = R.t_end(x.max())
    got = tto.trace(gx, gy, gz, x, x, x, s0, t_end, rtol, atol, method=method, threads=1)
    assert (got["status"] == 0).all()
    for r in range(s0.shape[1]):
        sol = solve_ivp(dsdt, [0.0, t_end], s0[:, r], method=method, rtol=rtol, atol=atol)
        assert sol.status == 0
        want = sol.y[:, -1]
        n_scipy = len(sol.t) - 1
        assert abs(int(got["nacc"][r]) - n_scipy) <= 0.1 * n_scipy + 2, (r, got["nacc"][r], n_scipy)
        assert np.abs(got["sf"][:3, r] - want[:3]).max() <= 3 * rtol * 2 * x.max()
        assert np.abs(got["sf"][3:, r] - want[3:]).max() <= 3 * rtol * R.C_LIGHT


def test_rk_pair_reads_scipy_classes():
    import scipy.integrate as si

    for name, ns, kind, order in (("RK23", 3, 0, 2), ("RK45", 6, 0, 4), ("DOP853", 12, 1, 7)):
        n, k, o, A, B, E, E3 = tto.rk_pair(name)
        assert (n, k, o) == (ns, kind, order)
        assert A.shape == (ns, ns) and np.allclose(A.sum(axis=1), np.asarray(getattr(si, name).C)[:ns])
        assert abs(B.sum() - 1.0) < 1e-14 and abs(E.sum()) < 1e-14 and abs(E3.sum()) < 1e-14


def test_dropin_tableau_from_scipy_classes():
    """The drop-in's tt_rk_tableau is filled from the same scipy classes; the
    implicit methods are refused with NotImplementedError."""
    import scipy.integrate as si

    from turbulence_tracing_gb300 import core

    for name in ("RK23", "RK45", "DOP853"):
        t = core.rk_tableau(name)
        cls = getattr(si, name)
        ns = cls.n_stages
        assert t.n_stages == ns and t.error_order == cls.error_estimator_order
        A = np.array([[t.A[i][j] for j in range(ns)] for i in range(ns)])
        assert np.allclose(A.sum(axis=1), np.asarray(cls.C)[:ns], atol=1e-15)
        assert t.error_kind == (1 if name == "DOP853" else 0)
    assert core.rk_tableau(si.RK23).n_stages == 3
    for name in ("Radau", "BDF", "LSODA", "Euler"):
        with pytest.raises(NotImplementedError):
            core.rk_tableau(name)
