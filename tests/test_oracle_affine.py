"""Oracle: the affine-element form against the quadrature form.

For an element whose nodes are an affine image of the reference nodes the
Jacobian is the same at every quadrature point, so the element matrix
factors through reference tables (J^-T R_ab J^-1 and det * Mref_ab).  The
two forms agree to rounding; an element that fails the affinity test takes
the quadrature form unchanged.
"""
import numpy as np
import pytest

from helpers import PT

CASES = [("box", 3, 1, False), ("box", 2, 2, False), ("box", 1, 3, False), ("box", 2, 2, True),
         ("rect", 4, 2, False), ("rect", 3, 3, True)]


def _ops(orc):
    return [(orc.ELASTIC, True), (orc.HEAT, False), (orc.MASS, True)]


def _assemble(llf, orc, m, kind, vector, affine):
    rule = llf._lib.builtin_rule(m.family, m.order)
    dim = m.dim
    ptype = PT["Solid"] if dim == 3 else PT["PlaneStrain"]
    params = {orc.ELASTIC: [2.1e5, 0.3], orc.HEAT: [45.0], orc.MASS: [7.85e-9]}[kind]
    pdim = dim if vector else 1
    return orc.assemble(kind, ptype, dim, pdim, m.xyz, m.conn, rule, params, affine=affine).scipy()


def _mesh(llf, kind, n, order, simplex):
    if kind == "box":
        return llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    return llf.structured_rect_mesh(n=n, order=order, simplex=simplex)


@pytest.mark.parametrize("case", CASES)
def test_affine_form_agrees_with_quadrature(llf, orc, case):
    m = _mesh(llf, *case)
    for kind, vector in _ops(orc):
        A = _assemble(llf, orc, m, kind, vector, True)
        Q = _assemble(llf, orc, m, kind, vector, False)
        d = abs(A - Q)
        assert d.max() <= 1e-12 * abs(Q).max(), (case, kind)


@pytest.mark.parametrize("case", [("box", 2, 2, False), ("rect", 3, 3, False), ("box", 1, 3, False)])
def test_distorted_elements_take_the_quadrature_form(llf, orc, case):
    """Moving a mid-side node of every element breaks affinity: both
    settings give the same matrix bit for bit."""
    m = _mesh(llf, *case)
    rng = np.random.default_rng(7)
    h = 1.0 / case[1]
    interior = np.all((m.xyz[:, :m.dim] > 1e-9) & (m.xyz[:, :m.dim] < 1 - 1e-9), axis=1)
    m.xyz[interior, :m.dim] += rng.uniform(-0.05, 0.05, (interior.sum(), m.dim)) * h
    conn = np.asarray(m.conn)
    moved = np.zeros(m.non, dtype=bool)
    moved[np.nonzero(interior)[0]] = True
    every = moved[conn - 1].any(axis=1)
    if not every.all():
        pytest.skip("not every element has an interior node")
    for kind, vector in _ops(orc):
        A = _assemble(llf, orc, m, kind, vector, True)
        Q = _assemble(llf, orc, m, kind, vector, False)
        assert (A != Q).nnz == 0, kind


def test_mixed_mesh_affine_and_distorted(llf, orc):
    """Half the elements distorted: the affine half differs from the
    quadrature form only by rounding, the distorted half not at all."""
    m = _mesh(llf, "box", 2, 2, False)
    rng = np.random.default_rng(11)
    sel = (m.xyz[:, 0] > 0.5 + 1e-9) & (m.xyz[:, 0] < 1 - 1e-9)
    m.xyz[sel, :] += rng.uniform(-0.02, 0.02, (sel.sum(), 3))
    A = _assemble(llf, orc, m, orc.ELASTIC, True, True)
    Q = _assemble(llf, orc, m, orc.ELASTIC, True, False)
    assert abs(A - Q).max() <= 1e-12 * abs(Q).max()
