"""The oracle's restatement of FDM (src/heat.jl:1466-1616) against known
answers: an insulated body with one face held at T_a reaches T_a
everywhere; the theta-method with a small step agrees with the explicit
update; a non-positive capacity on a free DoF is rejected."""
import numpy as np
import pytest


def _heat_pair(llf, orc, lumped):
    m = llf.structured_box_mesh(lx=2.0, n=3, order=1)
    rule = llf._lib.builtin_rule(m.family, m.order)
    K = orc.assemble(orc.HEAT, 3, 3, 1, m.xyz, m.conn, rule, [45.0]).scipy()
    C = orc.assemble(orc.MASS, 3, 3, 1, m.xyz, m.conn, rule, [7.85e-9 * 4.2e8], lumped=lumped).scipy()
    fixed = np.zeros(m.non, dtype=bool)
    fixed[m.group("left").nodes - 1] = True
    return m, K, C, fixed


def test_insulated_body_reaches_the_held_temperature(llf, orc):
    m, K, C, fixed = _heat_pair(llf, orc, lumped=False)
    n = 60
    T = np.zeros((n, m.non))
    T[:, fixed] = 100.0
    T = orc.fdm(K, C, np.zeros(m.non), fixed, T, dt=50.0, theta=1.0)
    assert np.abs(T[-1] - 100.0).max() < 1e-6
    assert np.all(np.diff(T[:, ~fixed].mean(axis=1)) >= -1e-12)   # monotone heating


def test_theta_method_agrees_with_explicit_at_small_steps(llf, orc):
    m, K, C, fixed = _heat_pair(llf, orc, lumped=True)
    # explicit stability: dt below 2 / lambda_max(C^-1 K) on the free DoFs
    free = ~fixed
    d = 1.0 / np.sqrt(C.diagonal()[free])
    lam = np.linalg.eigvalsh(d[:, None] * K.toarray()[np.ix_(free, free)] * d[None, :]).max()
    n, dt = 400, 0.5 / lam
    T0 = np.zeros((n, m.non))
    T0[:, fixed] = 100.0
    Te = orc.fdm(K, C, np.zeros(m.non), fixed, T0.copy(), dt=dt, theta=0.0)
    Ti = orc.fdm(K, C, np.zeros(m.non), fixed, T0.copy(), dt=dt, theta=0.5)
    assert np.abs(Te[-1] - Ti[-1]).max() < 2e-2 * 100.0
    assert Te[-1][free].mean() > 1.0   # heat has entered the body


def test_non_positive_capacity_is_rejected(llf, orc):
    m, K, C, fixed = _heat_pair(llf, orc, lumped=True)
    with pytest.raises(ValueError):
        orc.fdm(K, -C, np.zeros(m.non), fixed, np.zeros((3, m.non)), dt=1.0, theta=0.5)
