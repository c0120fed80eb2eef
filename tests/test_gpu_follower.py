"""Follower loads on the GPU, bit-identical to the oracle:
loadVector(...; F) (src/linear.jl:3333-3372), externalTangentFollower
(src/nonlinear.jl:3053-3258) and elementsToNodes (src/general.jl:5519-5640)."""
import numpy as np
import pytest

from helpers import assert_csc_identical
from test_oracle_follower import nodal_F

pytestmark = pytest.mark.gpu

FACE_CASES = [(3, 2, False), (2, 1, False), (2, 2, True), (2, 1, True)]


def _ids(c):
    return f"n{c[0]}-p{c[1]}{'-simplex' if c[2] else ''}"


def _problem(llf, n, order, simplex):
    m = llf.structured_box_mesh(lx=1.5, n=n, order=order, simplex=simplex)
    return m, llf.Problem([llf.Material("body", E=2.0e5, nu=0.3)], type="Solid")


@pytest.mark.parametrize("case", FACE_CASES, ids=_ids)
def test_follower_load_vector_bit_identical(llf, orc, case):
    m, p = _problem(llf, *case)
    Fn = nodal_F(m.xyz)
    F = llf.TensorField(None, p, a=Fn.reshape(-1, 1))
    f = llf.loadVector(p, [llf.load("right", fx=1.0, fy=-2.0, fz=0.5), llf.load("top", fy=3.0)], F=F)
    rule = llf._lib.builtin_rule(m.group("right").family, m.group("right").order)
    ref, st = orc.load_vector_follower(m.xyz, m.group("right").conn, rule, Fn, t=[1.0, -2.0, 0.5])
    ref, st2 = orc.load_vector_follower(m.xyz, m.group("top").conn, rule, Fn, t=[0.0, 3.0, 0.0], f=ref)
    assert st == 0 and st2 == 0
    assert np.array_equal(f.a[:, 0], ref)


@pytest.mark.parametrize("case", FACE_CASES, ids=_ids)
def test_follower_tangent_bit_identical(llf, orc, case):
    m, p = _problem(llf, *case)
    Fn = nodal_F(m.xyz)
    F = llf.TensorField(None, p, a=Fn.reshape(-1, 1))
    loads = [llf.load("right", fx=1.0, fy=-2.0, fz=0.5), llf.load("top", fx=0.25, fy=3.0)]
    K = llf.externalTangentFollower(p, loads, F)
    conn = np.concatenate([m.group("right").conn, m.group("top").conn])
    te = np.concatenate([np.tile([1.0, -2.0, 0.5], (m.group("right").conn.shape[0], 1)),
                         np.tile([0.25, 3.0, 0.0], (m.group("top").conn.shape[0], 1))])
    rule = llf._lib.builtin_rule(m.group("right").family, m.group("right").order)
    ref, st = orc.follower_tangent(m.xyz, conn, rule, Fn, t=te)
    assert st == 0
    assert_csc_identical(K.csc(), ref.julia(), f"externalTangentFollower {_ids(case)}")


def test_follower_tangent_function_traction_and_elementwise_F(llf, orc):
    """A function traction (sampled at the nodes, interpolated) and F given
    elementwise (averaged to the nodes first, elementsToNodes)."""
    m, p = _problem(llf, 3, 2, False)
    rng = np.random.default_rng(20261203)
    u = llf.VectorField((0.02 * rng.standard_normal(3 * m.non)).reshape(-1, 1), p)
    Fe = llf.deformationGradient(u)
    fz = lambda x, y, z: 1.0 + y * z
    K = llf.externalTangentFollower(p, [llf.load("right", fx=2.0, fz=fz)], Fe)
    Fn = orc.elements_to_nodes(m.non, m.conn, Fe.A, 9)
    assert np.array_equal(llf.elementsToNodes(Fe).a[:, 0], Fn.reshape(-1))
    g = m.group("right")
    tn = np.zeros((m.non, 3))
    tn[g.nodes - 1, 0] = 2.0
    tn[g.nodes - 1, 2] = [fz(*m.xyz[v - 1]) for v in g.nodes]
    ref, st = orc.follower_tangent(m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), Fn, tn=tn)
    assert st == 0
    assert_csc_identical(K.csc(), ref.julia(), "function traction")


def test_follower_inverted_F_is_an_error(llf):
    m, p = _problem(llf, 2, 1, False)
    bad = np.tile(np.diag([1.0, 1.0, -1.0]).reshape(-1), (m.non, 1))
    F = llf.TensorField(None, p, a=bad.reshape(-1, 1))
    with pytest.raises(llf.LLFError):
        llf.loadVector(p, [llf.load("right", fx=1.0)], F=F)
    with pytest.raises(llf.LLFError):
        llf.externalTangentFollower(p, [llf.load("right", fx=1.0)], F)
    # the context stays usable
    K = llf.externalTangentFollower(p, [llf.load("right", fx=1.0)],
                                    llf.TensorField(None, p, a=np.tile(np.eye(3).reshape(-1), m.non)[:, None]))
    assert K.nnz() > 0
