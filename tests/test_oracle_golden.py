"""The CPU oracle pinned against the reference's own published numbers.

Golden values (all from the reference tree):
  * sum(abs, K) = 4.0073076923076982e9 and sum(u) = 0.07057241535937334 for
    the unit cube, structured_box_mesh(n=30) hex8, E=2e5, nu=0.3, left face
    clamped, unit traction x on "right"
    (examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/results.txt:7,
    lowlevelfem_elasticity_benchmark.jl:25-48);
  * 15,944,049 structural entries for hex8 n=40
    (examples/dev/DSL_vs_legacy_test.ipynb:170);
  * plane-stress patch u(1,1) = (1/E, -nu/E) (test/test_validation.jl);
  * unit-cube volume and traction resultants [1,1,1] (test/test_dsl.jl:60-85);
  * symmetry ||K-K'||/||K|| < 1e-10 (test/test_assembly.jl:13).
"""
import numpy as np
import pytest

from helpers import oracle_operator


def test_sum_abs_K_hex8_n30(llf, orc):
    m = llf.structured_box_mesh(n=30, order=1)
    mat = llf.Material("body")
    K = oracle_operator(llf, orc, m, "stiffness", 0, mat)
    s = np.abs(K.arrays()[2]).sum()
    assert abs(s - 4.0073076923076982e9) <= 1e-15 * 4.0073076923076982e9, repr(s)


def test_structural_nnz_hex8_n40(llf, orc):
    m = llf.structured_box_mesh(n=40, order=1)
    assert orc.pattern(m.non, m.conn, 3).nnz == 15944049


def test_sum_u_hex8_n30(llf, orc):
    m = llf.structured_box_mesh(n=30, order=1)
    mat = llf.Material("body")
    K = oracle_operator(llf, orc, m, "stiffness", 0, mat)
    g = m.group("right")
    rule_b = llf._lib.builtin_rule(g.family, g.order)
    f = orc.load_vector(3, 3, m.xyz, g.conn, rule_b, t=[1.0, 0.0, 0.0])
    fixed = np.zeros(3 * m.non, dtype=np.uint8)
    left = m.group("left").nodes
    for c in range(3):
        fixed[(left - 1) * 3 + c] = 1
    u, it, rr = K.cg(f, np.zeros(3 * m.non), fixed, precond=1, reltol=1e-14, maxiter=20000)
    assert rr <= 1e-14
    assert abs(u.sum() - 0.07057241535937334) <= 1e-12 * 0.0706, repr(u.sum())


def test_plane_stress_patch(llf, orc):
    m = llf.structured_rect_mesh()
    mat = llf.Material("body")
    K = oracle_operator(llf, orc, m, "stiffness", 1, mat)
    g = m.group("right")
    f = orc.load_vector(2, 2, m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), t=[1.0, 0.0])
    fixed = np.zeros(2 * m.non, dtype=np.uint8)
    fixed[(m.group("left").nodes - 1) * 2 + 0] = 1
    fixed[(m.group("bottom").nodes - 1) * 2 + 1] = 1
    u, it, rr = K.cg(f, np.zeros(2 * m.non), fixed, precond=1, reltol=1e-14, maxiter=10000)
    node = int(np.where((np.abs(m.xyz[:, 0] - 1) < 1e-12) & (np.abs(m.xyz[:, 1] - 1) < 1e-12))[0][0])
    assert abs(u[2 * node] - 1 / mat.E) < 1e-2 / mat.E
    assert abs(u[2 * node + 1] + mat.nu / mat.E) < 1e-2 * mat.nu / mat.E
    # the patch test is exact for bilinear elements
    assert abs(u[2 * node] - 1 / mat.E) < 1e-10 / mat.E


def test_resultants_unit_cube(llf, orc):
    m = llf.structured_box_mesh(n=2, order=1)
    g = m.group("right")
    f = orc.load_vector(3, 3, m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), t=[1.0, 1.0, 1.0])
    assert np.allclose(f.reshape(-1, 3).sum(axis=0), [1, 1, 1], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kind,n,order,simplex,ptype", [
    ("rect", 4, 1, False, 1), ("rect", 3, 2, False, 2), ("rect", 3, 2, True, 2),
    ("box", 2, 1, False, 0), ("box", 2, 2, False, 0), ("box", 2, 2, True, 0),
])
def test_symmetry_and_rigid_modes(llf, orc, kind, n, order, simplex, ptype):
    from helpers import make_mesh
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body")
    K = oracle_operator(llf, orc, m, "stiffness", ptype, mat).scipy()
    assert abs(K - K.T).max() == 0.0  # exactly symmetric by construction
    d = m.dim
    for c in range(d):
        t = np.zeros(K.shape[0]); t[c::d] = 1.0
        assert np.abs(K @ t).max() <= 1e-9 * abs(K).max()


def test_mass_totals(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2, lx=2.0)
    mat = llf.Material("body", rho=7.85e-9)
    M = oracle_operator(llf, orc, m, "mass", 0, mat).scipy()
    vol = 2.0
    assert abs(M.sum() / 3 - mat.rho * vol) < 1e-12 * mat.rho * vol
    L = oracle_operator(llf, orc, m, "mass", 0, mat, lumped=True).scipy()
    assert np.allclose(L.diagonal(), np.asarray(M.sum(axis=1)).ravel(), rtol=1e-14, atol=0)


def test_heat_constant_nullspace(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2)
    mat = llf.Material("body")
    K = oracle_operator(llf, orc, m, "heat", 3, mat).scipy()
    assert np.abs(K @ np.ones(K.shape[0])).max() <= 1e-12 * abs(K).max()


@pytest.mark.parametrize("simplex", [False, True])
def test_support_totals(llf, orc, simplex):
    """elasticSupportMatrix: symmetric, diagonal blocks only, and each
    component's entries sum to k_i times the supported area (2 x 3 face)."""
    m = llf.structured_box_mesh(lx=2.0, ly=1.0, lz=3.0, n=2, order=2, simplex=simplex)
    g = m.group("bottom")
    rule = llf._lib.builtin_rule(g.family, g.order)
    k = [3.0, 5.0, 11.0]
    C = orc.support_matrix(3, 3, m.xyz.shape[0], m.xyz, g.conn, rule, k).scipy().tocoo()
    assert np.all(C.row % 3 == C.col % 3)
    for i in range(3):
        s = C.data[C.row % 3 == i].sum()
        assert abs(s - k[i] * 6.0) < 1e-12 * k[i] * 6.0
    D = C.tocsc()
    assert abs(D - D.T).max() == 0.0
    m2 = llf.structured_rect_mesh(lx=2.0, n=4, order=3)
    g2 = m2.group("top")
    C2 = orc.support_matrix(2, 1, m2.xyz.shape[0], m2.xyz, g2.conn, llf._lib.builtin_rule(g2.family, g2.order),
                            [4.0], 0.5).scipy()
    assert abs(C2.sum() - 4.0 * 2.0 * 0.5) < 1e-13 * 4.0
