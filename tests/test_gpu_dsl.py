"""Weak-form DSL bilinear terms on the GPU (src/multifield.jl:4385-4931,
:5280-5346).  The reference's own check is DSL = legacy (test/test_dsl.jl:
30-31, to 1e-12); here the DSL forms run on the same kernels, so they are
bit-identical to the legacy operators, and the csc_matrix accumulation is
bit-identical to the oracle's in-place accumulation into a kept pattern."""
import numpy as np
import pytest

from helpers import assert_csc_identical

pytestmark = pytest.mark.gpu


def _lame(E, nu):
    return E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))


def _D(dim, lam, mu):
    n = 6 if dim == 3 else 3
    D = np.zeros((n, n))
    D[:dim, :dim] = lam
    D[np.arange(dim), np.arange(dim)] = lam + 2.0 * mu
    D[np.arange(dim, n), np.arange(dim, n)] = mu
    return D


@pytest.mark.parametrize("case", [("box", 3, 2, False, "Solid"), ("box", 2, 1, True, "Solid"),
                                  ("rect", 5, 2, False, "PlaneStrain"), ("rect", 4, 3, True, "PlaneStrain")],
                         ids=["hex27", "tet4", "quad9", "tri10"])
def test_symgrad_equals_stiffness(llf, orc, case):
    kind, n, order, simplex, pt = case
    m = (llf.structured_box_mesh if kind == "box" else llf.structured_rect_mesh)(n=n, order=order, simplex=simplex)
    E, nu = 2.1e5, 0.3
    p = llf.Problem([llf.Material("body", E=E, nu=nu)], type=pt)
    lam, mu = _lame(E, nu)
    K = llf.integrate(llf.SymGrad(p) @ _D(m.dim, lam, mu) @ llf.SymGrad(p))
    assert_csc_identical(K.csc(), llf.stiffnessMatrix(p).csc(), "DSL vs stiffnessMatrix")
    ref = orc.assemble(orc.ELASTIC, orc.PT_LAME, m.dim, m.dim, m.xyz, m.conn,
                       llf._lib.builtin_rule(m.family, m.order), [lam, mu])
    assert_csc_identical(K.csc(), ref.julia(), "DSL vs oracle")


def test_grad_and_id_equal_conduction_and_mass(llf):
    llf.structured_box_mesh(n=3, order=2)
    ph = llf.Problem([llf.Material("body", k=45.0)], type="HeatConduction")
    K = llf.integrate(llf.Grad(ph) @ 45.0 @ llf.Grad(ph))
    assert_csc_identical(K.csc(), llf.heatConductionMatrix(ph).csc(), "Grad⋅k⋅Grad")
    ps = llf.Problem([llf.Material("body", rho=7.85e-9)], type="Solid")
    M = llf.integrate(llf.Id(ps) @ 7.85e-9 @ llf.Id(ps))
    assert_csc_identical(M.csc(), llf.massMatrix(ps, lumped=False).csc(), "Id⋅ρ⋅Id")
    # a scalar chain collapses left to right
    M2 = llf.integrate(llf.Id(ps) @ 7.85 @ 1e-9 @ llf.Id(ps))
    assert M2.nnz() == M.nnz()


def test_csc_matrix_accumulates_and_keeps_pattern(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2, simplex=True)
    p = llf.Problem([llf.Material("body", k=3.0)], type="HeatConduction")
    Kp = llf.build_csc_pattern(p)
    colptr, rowval = p.pattern().copy()
    assert Kp.nnz() == len(rowval)
    out = llf.integrate(llf.Id(p) @ 2.5 @ llf.Id(p), csc_matrix=Kp)
    assert out is Kp and Kp.nnz() == len(rowval)
    rule = llf._lib.builtin_rule(m.family, m.order)
    zero = (colptr - 1, rowval - 1, np.zeros(len(rowval)))
    r1 = orc.assemble(orc.MASS, orc.PT_LAME, 3, 1, m.xyz, m.conn, rule, [2.5], init=zero)
    assert_csc_identical(Kp.csc(), r1.julia(), "Id⋅c⋅Id into a zero pattern")
    llf.integrate(llf.Grad(p) @ 3.0 @ llf.Grad(p), csc_matrix=Kp)
    r2 = orc.assemble(orc.HEAT, orc.PT_LAME, 3, 1, m.xyz, m.conn, rule, [3.0], init=r1.arrays())
    assert_csc_identical(Kp.csc(), r2.julia(), "Grad⋅k⋅Grad added in element order")
    # the accumulated matrix solves like any other
    assert Kp.nnz() == len(rowval)


def test_unsupported_forms_raise(llf):
    llf.structured_box_mesh(n=2, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    D = _D(3, 1.0, 1.0)
    D[0, 5] = D[5, 0] = 0.2
    with pytest.raises(NotImplementedError):
        llf.integrate(llf.SymGrad(p) @ D @ llf.SymGrad(p))
    with pytest.raises(NotImplementedError):
        llf.integrate(llf.Grad(p) @ llf.Grad(p))
    with pytest.raises(NotImplementedError):
        llf.integrate(llf.Id(p) @ 1.0 @ llf.Id(p), weight=2.0)
