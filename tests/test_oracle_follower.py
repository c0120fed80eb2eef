"""Follower loads in the oracle, against a literal numpy transcription of
the reference's loops (externalTangentFollower, src/nonlinear.jl:3053-3258;
loadVector(...; F), src/linear.jl:3333-3372) and against known answers.
The face Jacobian is completed with the unit normal as gmsh completes the
Jacobian of a surface element, so jacDet = |t1 x t2|."""
import numpy as np
import pytest


def nodal_F(xyz, scale=0.1):
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    F = np.zeros((xyz.shape[0], 3, 3))
    F[:, 0, 0] = 1 + scale * x
    F[:, 0, 1] = scale * y * z
    F[:, 1, 1] = 1 - 0.5 * scale * z
    F[:, 1, 2] = scale * x * y
    F[:, 2, 0] = -scale * y
    F[:, 2, 2] = 1 + scale * (x + z)
    F[:, 1, 0] = 0.3 * scale
    return F.transpose(0, 2, 1).reshape(-1, 9)     # column-major per node


def reference_follower(xyz, conn0, rule, Fn, t):
    """The reference's element loop, transcribed with numpy linear algebra."""
    n = 3 * xyz.shape[0]
    K = np.zeros((n, n))
    w, N, dN = rule["w"], rule["N"].reshape(len(rule["w"]), -1), rule["dN"].reshape(len(rule["w"]), -1, 3)
    npe = conn0.shape[1]
    Id = np.eye(3)
    for c in conn0:
        X = xyz[c]
        Ke = np.zeros((3 * npe, 3 * npe))
        for q in range(len(w)):
            t1, t2 = X.T @ dN[q, :, 0], X.T @ dN[q, :, 1]
            nv = np.cross(t1, t2)
            da = np.linalg.norm(nv)
            Jm = np.column_stack([t1, t2, nv / da])
            invJ = np.linalg.inv(Jm).T
            wq = da * w[q]
            Fgp = sum(N[q, a] * Fn[c[a]].reshape(3, 3, order="F") for a in range(npe))
            Finv = np.linalg.inv(Fgp)
            FinvT = Finv.T
            Jgp = np.linalg.det(Fgp)
            tgp = Fgp @ t
            tloc = Finv @ tgp
            for b in range(npe):
                g = invJ @ dN[q, b, :]
                for jb in range(3):
                    fcol = Finv[:, jb]
                    dt0 = Jgp * FinvT @ (fcol @ g * Id - np.outer(g, fcol)) @ tgp
                    dt0 = dt0 + Jgp * FinvT[:, jb] * (g @ tloc)
                    for a in range(npe):
                        Ke[3 * a:3 * a + 3, 3 * b + jb] += N[q, a] * dt0 * wq
        dofs = (3 * c[:, None] + np.arange(3)[None, :]).ravel()
        K[np.ix_(dofs, dofs)] += Ke
    return K


@pytest.mark.parametrize("case", [(2, 1, False), (2, 2, False), (2, 2, True)], ids=["quad4", "quad9", "tri6"])
def test_follower_tangent_matches_reference_loop(llf, orc, case):
    n, order, simplex = case
    m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    g = m.group("right")
    rule = llf._lib.builtin_rule(g.family, g.order)
    Fn = nodal_F(m.xyz)
    t = np.array([0.3, -1.2, 0.7])
    K, st = orc.follower_tangent(m.xyz, g.conn, rule, Fn, t=t)
    assert st == 0
    ref = reference_follower(m.xyz, g.conn - 1, rule, Fn, t)
    A = K.scipy().toarray()
    assert np.abs(A - ref).max() <= 1e-12 * np.abs(ref).max()
    # dropzeros!: no stored exact zeros
    assert np.all(K.scipy().data != 0.0)


def test_follower_tangent_identity_F(llf, orc):
    """At F = I the follower tangent is g_jb t - t_jb g + (g.t) e_jb per
    column, integrated: the columns of every node sum to zero for a
    constant traction when summed over b (sum_b g_b = 0)."""
    m = llf.structured_box_mesh(n=2, order=2)
    g = m.group("top")
    rule = llf._lib.builtin_rule(g.family, g.order)
    Fn = np.tile(np.eye(3).reshape(-1), (m.non, 1))
    K, st = orc.follower_tangent(m.xyz, g.conn, rule, Fn, t=[1.0, 2.0, 3.0])
    A = K.scipy().toarray()
    for j in range(3):
        col = np.zeros(3 * m.non)
        col[j::3] = 1.0
        assert np.abs(A @ col).max() <= 1e-13 * np.abs(A).max()


def test_follower_load_known_answers(llf, orc):
    m = llf.structured_box_mesh(lx=2.0, n=3, order=2)
    g = m.group("right")                       # 1 x 1 face
    rule = llf._lib.builtin_rule(g.family, g.order)
    t = np.array([1.0, -2.0, 0.5])
    dead = orc.load_vector(3, 3, m.xyz, g.conn, rule, t=t)
    ident = np.tile(np.eye(3).reshape(-1), (m.non, 1))
    f1, st = orc.load_vector_follower(m.xyz, g.conn, rule, ident, t=t)
    assert st == 0 and np.abs(f1 - dead).max() <= 1e-15 * np.abs(dead).max() * 10
    c, s = np.cos(0.4), np.sin(0.4)
    R = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    fR, st = orc.load_vector_follower(m.xyz, g.conn, rule, np.tile(R.reshape(-1, order="F"), (m.non, 1)), t=t)
    assert np.allclose(fR.reshape(-1, 3).sum(axis=0), R @ t, rtol=0, atol=1e-13)
    bad = np.tile(np.diag([1.0, 1.0, -1.0]).reshape(-1), (m.non, 1))
    _, st = orc.load_vector_follower(m.xyz, g.conn, rule, bad, t=t)
    assert st == -1


def test_elements_to_nodes_is_the_mean(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2)
    rng = np.random.default_rng(20261203)
    ev = rng.standard_normal((m.nel, 9 * m.npe))
    nv = orc.elements_to_nodes(m.non, m.conn, ev, 9)
    s = np.zeros((m.non, 9)); cnt = np.zeros(m.non)
    for e in range(m.nel):
        for a in range(m.npe):
            s[m.conn[e, a] - 1] += ev[e, 9 * a:9 * a + 9]
            cnt[m.conn[e, a] - 1] += 1
    assert np.allclose(nv, s / cnt[:, None], rtol=1e-14, atol=1e-15)
