"""Boundary support matrices on the GPU: elasticSupportMatrix
(src/linear.jl:2859-3005) and heatConvectionMatrix / heatConvectionVector
(src/heat.jl:562-567, :667-673), bit-identical to the oracle, plus the
convection solve against the closed-form 1D answer."""
import numpy as np
import pytest

from helpers import assert_csc_identical, make_mesh

pytestmark = pytest.mark.gpu

# (mesh kind, n, order, simplex, problem type, thickness)
SUPPORT_CASES = [("box", 3, 2, False, "Solid", 1.0), ("box", 2, 1, True, "Solid", 1.0),
                 ("rect", 4, 3, True, "PlaneStress", 0.5), ("rect", 3, 2, False, "PlaneStrain", 1.0)]


def _ids(c):
    return f"{c[0]}-n{c[1]}-p{c[2]}{'-simplex' if c[3] else ''}-{c[4]}"


def _oracle(llf, orc, m, p, names, k, kn=None):
    """All groups' elements in one triplet list, as the reference's single
    sparse() call collects them."""
    conn = np.concatenate([m.group(nm).conn for nm in names], axis=0)
    g = m.group(names[0])
    rule = llf._lib.builtin_rule(g.family, g.order)
    b = p.thickness if m.dim == 2 else 1.0
    return orc.support_matrix(m.dim, p.pdim, m.xyz.shape[0], m.xyz, conn, rule, k, b, kn)


@pytest.mark.parametrize("case", SUPPORT_CASES, ids=_ids)
def test_elastic_support_bit_identical(llf, orc, case):
    kind, n, order, simplex, pt, t = case
    m = make_mesh(llf, kind, n, order, simplex)
    p = llf.Problem([llf.Material("body")], type=pt, thickness=t)
    ks = {"right": [1.5e3, 2.5e3, 4.0e3][: p.pdim], "top": [0.7e3, 3.1e3, 0.9e3][: p.pdim]}
    names = ["right", "top"]   # two groups sharing an edge (3D) or a corner node (2D)
    sup = [llf.elasticSupport(nm, **dict(zip(["kx", "ky", "kz"], ks[nm]))) for nm in names]
    C = llf.elasticSupportMatrix(p, sup)
    kel = np.concatenate([np.tile(ks[nm], (m.group(nm).conn.shape[0], 1)) for nm in names])
    ref = _oracle(llf, orc, m, p, names, kel)
    assert_csc_identical(C.csc(), ref.julia(), f"elasticSupportMatrix {_ids(case)}")


def test_elastic_support_one_component_and_area(llf, orc):
    """Only ky given: the x and z diagonals are absent (dropzeros!), and the
    entries of the y block sum to ky times the face area."""
    m = llf.structured_box_mesh(lx=2.0, ly=1.0, lz=3.0, n=3, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    C = llf.elasticSupportMatrix(p, [llf.elasticSupport("bottom", ky=7.0)])
    ref = _oracle(llf, orc, m, p, ["bottom"], [0.0, 7.0, 0.0])
    assert_csc_identical(C.csc(), ref.julia(), "ky only")
    A = C.A.tocoo()
    assert np.all(A.row % 3 == 1) and np.all(A.col % 3 == 1)
    assert abs(A.data.sum() - 7.0 * 2.0 * 3.0) < 1e-12 * 42.0


def test_elastic_support_function_stiffness(llf, orc):
    """ky(x, y, z) sampled at the group's nodes and interpolated at the points."""
    m = llf.structured_rect_mesh(n=5, order=2)
    p = llf.Problem([llf.Material("body")], type="PlaneStress", thickness=0.25)
    fy = lambda x, y, z: 1.0 + 3.0 * x * x
    C = llf.elasticSupportMatrix(p, [llf.elasticSupport("bottom", kx=2.0, ky=fy)])
    g = m.group("bottom")
    kn = np.zeros(2 * m.non)
    kn[(g.nodes - 1) * 2] = 2.0
    kn[(g.nodes - 1) * 2 + 1] = [fy(*m.xyz[v - 1]) for v in g.nodes]
    ref = _oracle(llf, orc, m, p, ["bottom"], [0.0, 0.0], kn)
    assert_csc_identical(C.csc(), ref.julia(), "function ky")


@pytest.mark.parametrize("case", [("box", 3, 2, False), ("box", 2, 3, True), ("rect", 4, 2, True)],
                         ids=["hex27", "tet20", "tri6"])
def test_heat_convection_matrix_bit_identical(llf, orc, case):
    kind, n, order, simplex = case
    m = make_mesh(llf, kind, n, order, simplex)
    pt = "HeatConduction" if m.dim == 3 else "PlaneHeatConduction"
    p = llf.Problem([llf.Material("body", k=45.0)], type=pt, thickness=0.3)
    C = llf.heatConvectionMatrix(p, [llf.heatConvection("left", h=12.5, Tinf=20.0)])
    ref = _oracle(llf, orc, m, p, ["left"], [12.5])
    assert_csc_identical(C.csc(), ref.julia(), f"heatConvectionMatrix {kind} p{order}")


def test_heat_convection_vector_is_the_h_tinf_load(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2)
    p = llf.Problem([llf.Material("body", k=45.0)], type="HeatConduction")
    q = llf.heatConvectionVector(p, [llf.heatConvection("right", h=12.5, Tinf=20.0)])
    g = m.group("right")
    ref = orc.load_vector(3, 1, m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), t=[12.5 * 20.0])
    assert np.array_equal(q.a[:, 0], ref)


def test_solve_temperature_with_convection_matches_1d(llf):
    """Bar 0 <= x <= L, T = 100 at x = 0, convection h to T∞ = 20 at x = L:
    T(L) = (k T0 / L + h T∞) / (k / L + h); the field is linear in x, which
    the elements represent exactly."""
    L, k, h, T0, Tinf = 2.0, 45.0, 30.0, 100.0, 20.0
    m = llf.structured_box_mesh(lx=L, ly=0.5, lz=0.5, n=4, order=1)
    p = llf.Problem([llf.Material("body", k=k)], type="HeatConduction")
    T = llf.solveTemperature(p, temperatureConstraint=[llf.temperatureConstraint("left", T=T0)],
                             heatConvection=[llf.heatConvection("right", h=h, Tinf=Tinf)])
    TL = (k * T0 / L + h * Tinf) / (k / L + h)
    x = m.xyz[:, 0]
    assert np.allclose(T.a[:, 0], T0 + (TL - T0) * x / L, rtol=0, atol=1e-8)


def test_solve_displacement_with_elastic_support(llf):
    """Bar on an axial spring: fixed in y, z, pulled by a load F at x = L and
    held by a support kx at x = 0 (no ux constraint): u(x) = F / kx + F x / E
    per unit cross-section area."""
    L, E, kx, F = 3.0, 2.0e5, 5.0e4, 1.0e3
    m = llf.structured_box_mesh(lx=L, ly=1.0, lz=1.0, n=3, order=1)
    p = llf.Problem([llf.Material("body", E=E, nu=0.0)], type="Solid")
    sup = [llf.displacementConstraint(nm, uy=0, uz=0) for nm in ("left", "right")]
    u = llf.solveDisplacement(p, load=[llf.load("right", fx=F)], support=sup,
                              elasticSupport=[llf.elasticSupport("left", kx=kx)])
    ux = u.a[0::3, 0]
    x = m.xyz[:, 0]
    expect = F / kx + F * x / E
    assert np.allclose(ux, expect, rtol=1e-9, atol=1e-9 * np.abs(expect).max())


def test_support_group_of_wrong_dimension_is_an_error(llf):
    llf.structured_box_mesh(n=2, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    with pytest.raises(NotImplementedError):
        llf.elasticSupportMatrix(p, [llf.elasticSupport("body", kx=1.0)])
