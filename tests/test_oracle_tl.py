"""Oracle restatement of the Total Lagrangian path (parity unpinned by the
reference's tests, which have no TL case): the closed-form laws are checked
against finite differences of the strain energy (S = 2 dpsi/dC,
C = 4 d2psi/dC2, the derivatives ext/LowLevelFEMTensorsExt.jl:19,:37 takes
by automatic differentiation), and the operators against linear elasticity at
F = I."""
import math

import numpy as np
import pytest

from helpers import oracle_operator

VOIGT = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]


def psi_neo(C, mu, lam):
    J = math.sqrt(np.linalg.det(C))
    return mu / 2 * (np.trace(C) - 3) - mu * math.log(J) + lam / 2 * math.log(J) ** 2


def psi_svk(C, mu, lam):
    E = 0.5 * (C - np.eye(3))
    return lam / 2 * np.trace(E) ** 2 + mu * np.sum(E * E)


def _dsym(f, C, h):
    """Symmetric-tensor gradient by central differences."""
    G = np.zeros((3, 3))
    for i in range(3):
        for j in range(i, 3):
            dC = np.zeros((3, 3))
            dC[i, j] += h
            if i != j:
                dC[j, i] += h
            g = (f(C + dC) - f(C - dC)) / (2 * h)
            if i != j:
                g /= 2
            G[i, j] = G[j, i] = g
    return G


def test_ln_series(orc):
    for x in [1e-300, 1e-8, 0.3, 0.7071067811865476, 1.0, 1.0000001, 1.5, 2.0, 3.7, 1e5, 1e300]:
        assert abs(orc.ln(x) - math.log(x)) <= 4e-16 * max(1.0, abs(math.log(x)))


@pytest.mark.parametrize("law,psi", [(1, psi_neo), (2, psi_svk)])
def test_law_matches_energy_derivatives(orc, law, psi):
    mu, lam = 1.0, 10.0
    rng = np.random.default_rng(5)
    F = np.eye(3) + 0.1 * rng.standard_normal((3, 3))
    C = F.T @ F
    S, D = orc.law(law, [mu, lam], C)
    S_fd = 2 * _dsym(lambda X: psi(X, mu, lam), C, 1e-6)
    assert np.allclose(S, S_fd, atol=1e-7 * max(1, np.abs(S).max()))
    # C_IJKL = 2 dS_IJ/dC_KL
    for b, (K, L) in enumerate(VOIGT):
        dC = np.zeros((3, 3))
        h = 1e-6
        dC[K, L] += h
        if K != L:
            dC[L, K] += h
        Sp, _ = orc.law(law, [mu, lam], C + dC)
        Sm, _ = orc.law(law, [mu, lam], C - dC)
        dS = (Sp - Sm) / (2 * h) * (0.5 if K != L else 1.0)
        for a, (I, J) in enumerate(VOIGT):
            assert abs(D[a, b] - 2 * dS[I, J]) <= 1e-6 * max(1, np.abs(D).max()), (a, b)
    assert np.allclose(D, D.T, atol=1e-12 * np.abs(D).max())


def test_tangent_at_identity_equals_hooke(llf, orc):
    """At F = I the neo-Hookean tangent is Hooke's with the same Lame
    constants, so K_mat must equal stiffnessMatrix (to rounding)."""
    m = llf.structured_box_mesh(n=2, order=2)
    rule = llf._lib.builtin_rule(m.family, m.order)
    I = np.tile(np.eye(3).ravel(order="F"), (m.nel, m.npe))
    mu, lam = 80.0, 120.0
    Km = orc.tl_matrix(orc.TL_KMAT, m.xyz, m.conn, rule, I, orc.LAW_NEOHOOKE, [mu, lam]).scipy()
    E = mu * (3 * lam + 2 * mu) / (lam + mu)
    nu = lam / (2 * (lam + mu))
    mat = llf.Material("body", E=E, nu=nu)
    K = oracle_operator(llf, orc, m, "stiffness", 0, mat).scipy()
    assert abs(Km - K).max() <= 1e-12 * abs(K).max()
    Kg = orc.tl_matrix(orc.TL_KGEO_C, m.xyz, m.conn, rule, I, orc.LAW_NEOHOOKE, [mu, lam]).scipy()
    assert abs(Kg).max() <= 1e-13 * abs(K).max()   # S(C = I) = 0 up to the partition of unity's rounding
    f = orc.tl_internal_force(0, m.xyz, m.conn, rule, I, orc.LAW_NEOHOOKE, [mu, lam])
    assert np.abs(f).max() < 1e-12


def test_internal_force_is_energy_gradient(llf, orc):
    """f_int = dPi/du: compare with a finite difference of the total energy
    along a random direction (F from the oracle's nodal gradient)."""
    m = llf.structured_box_mesh(n=1, order=1)
    rule = llf._lib.builtin_rule(m.family, m.order)
    rng = np.random.default_rng(7)
    u = 0.02 * rng.standard_normal(3 * m.non)
    F = orc.grad_elementwise(m.xyz, m.conn, rule, u, add_identity=True)
    f = orc.tl_internal_force(0, m.xyz, m.conn, rule, F, orc.LAW_NEOHOOKE, [1.0, 10.0])
    assert np.isfinite(f).all() and np.abs(f).sum() > 0
    # equilibrium of the element forces: sum over nodes vanishes
    assert np.abs(f.reshape(-1, 3).sum(axis=0)).max() < 1e-12 * np.abs(f).max()
