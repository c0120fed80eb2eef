"""GPU Total Lagrangian operators vs the oracle (bit-identical CSC / vectors)
and the Newton-step properties of the hyperelastic configuration."""
import numpy as np
import pytest

from helpers import assert_csc_identical

pytestmark = pytest.mark.gpu

CASES = [("hex8", 2, 1, False), ("hex27", 2, 2, False), ("tet10", 1, 2, True), ("hex64", 1, 3, False)]


def _F(llf, m, p, scale, seed):
    rng = np.random.default_rng(seed)
    u = llf.VectorField(scale * rng.standard_normal((3 * m.non, 1)), p)
    return llf.grad(u, add_identity=True), u


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("law", ["NeoHookeCompressible", "StVenantKirchhoff"])
def test_material_tangent_bit_identical(llf, orc, case, law):
    _, n, order, simplex = case
    m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    p = llf.Problem([llf.Material("body")], type="Solid")
    F, _ = _F(llf, m, p, 0.03, 11)
    params = {"mu": 1.0, "lambda": 10.0}
    K = llf.materialTangentMatrix(p, F=F, energy=law, params=params)
    rule = llf._lib.builtin_rule(m.family, m.order)
    lid = orc.LAW_NEOHOOKE if law.startswith("Neo") else orc.LAW_SVK
    ref = orc.tl_matrix(orc.TL_KMAT, m.xyz, m.conn, rule, F.A, lid, [1.0, 10.0])
    assert_csc_identical(K.csc(), ref.julia(), f"Kmat {case[0]} {law}")


def test_material_tangent_constant_C(llf, orc):
    m = llf.structured_box_mesh(n=2, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    F, _ = _F(llf, m, p, 0.05, 3)
    Cv = np.diag([3.0, 3.0, 3.0, 1.0, 1.0, 1.0]) + 0.5
    K = llf.materialTangentMatrix(p, F=F, C=Cv)
    ref = orc.tl_matrix(orc.TL_KMAT, m.xyz, m.conn, llf._lib.builtin_rule(m.family, m.order), F.A, orc.LAW_CONST,
                        np.asarray(Cv).ravel(order="F"))
    assert_csc_identical(K.csc(), ref.julia(), "Kmat constant C")


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_initial_stress_bit_identical(llf, orc, case):
    _, n, order, simplex = case
    m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    p = llf.Problem([llf.Material("body")], type="Solid")
    F, _ = _F(llf, m, p, 0.03, 13)
    rule = llf._lib.builtin_rule(m.family, m.order)
    # C path (energy)
    FA = F.A.reshape(m.nel, m.npe, 3, 3)          # [e, a, j, i] column-major -> F[i][j] = FA[..., j, i]
    Fm = np.swapaxes(FA, -1, -2)
    Cm = np.einsum("eaki,eakj->eaij", Fm, Fm)
    Celem = np.swapaxes(Cm, -1, -2).reshape(m.nel, 9 * m.npe)
    Kg = llf.initialStressMatrix(p, energy="NeoHookeCompressible", params={"mu": 1.0, "lambda": 10.0},
                                 C=llf.TensorField(Celem, p))
    ref = orc.tl_matrix(orc.TL_KGEO_C, m.xyz, m.conn, rule, Celem, orc.LAW_NEOHOOKE, [1.0, 10.0])
    assert_csc_identical(Kg.csc(), ref.julia(), f"Kgeo(C) {case[0]}")
    # S path (given stress field)
    rng = np.random.default_rng(17)
    Sn = rng.standard_normal((m.nel, m.npe, 3, 3))
    Sn = Sn + np.swapaxes(Sn, -1, -2)
    Selem = Sn.reshape(m.nel, 9 * m.npe)
    Ks = llf.initialStressMatrix(p, S=llf.TensorField(Selem, p))
    refs = orc.tl_matrix(orc.TL_KGEO_S, m.xyz, m.conn, rule, Selem)
    assert_csc_identical(Ks.csc(), refs.julia(), f"Kgeo(S) {case[0]}")


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_internal_force_bit_identical(llf, orc, case):
    _, n, order, simplex = case
    m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    p = llf.Problem([llf.Material("body")], type="Solid")
    F, _ = _F(llf, m, p, 0.03, 19)
    rule = llf._lib.builtin_rule(m.family, m.order)
    f = llf.internalForceVector(p, F=F, energy="NeoHookeCompressible", params={"mu": 1.0, "lambda": 10.0})
    ref = orc.tl_internal_force(0, m.xyz, m.conn, rule, F.A, orc.LAW_NEOHOOKE, [1.0, 10.0])
    assert np.array_equal(f.a[:, 0], ref)
    P = llf.TensorField(np.random.default_rng(23).standard_normal((m.nel, 9 * m.npe)), p)
    fp = llf.internalForceVector(p, P=P)
    refp = orc.tl_internal_force(1, m.xyz, m.conn, rule, P.A)
    assert np.array_equal(fp.a[:, 0], refp)


def test_newton_step_consistency(llf):
    """The tangent K_mat + K_geo is the derivative of f_int: a directional
    finite difference of f_int matches K du (hex8, neo-Hookean)."""
    m = llf.structured_box_mesh(n=3, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    prm = {"mu": 1.0, "lambda": 10.0}
    rng = np.random.default_rng(29)
    # affine fields: their nodal gradients interpolate exactly to the Gauss points,
    # so f_int(u) and K_mat + K_geo describe the same discrete energy
    u = (m.xyz @ (0.05 * rng.standard_normal((3, 3))).T).ravel()
    du = (m.xyz @ rng.standard_normal((3, 3)).T).ravel()
    h = 1e-6

    def fint(v):
        F = llf.grad(llf.VectorField(v.reshape(-1, 1), p), add_identity=True)
        return llf.internalForceVector(p, F=F, energy="NeoHookeCompressible", params=prm).a[:, 0]

    F = llf.grad(llf.VectorField(u.reshape(-1, 1), p), add_identity=True)
    FA = np.swapaxes(F.A.reshape(m.nel, m.npe, 3, 3), -1, -2)
    Cm = np.einsum("eaki,eakj->eaij", FA, FA)
    C = llf.TensorField(np.swapaxes(Cm, -1, -2).reshape(m.nel, 9 * m.npe), p)
    K = llf.materialTangentMatrix(p, F=F, energy="NeoHookeCompressible", params=prm) + \
        llf.initialStressMatrix(p, energy="NeoHookeCompressible", params=prm, C=C)
    fd = (fint(u + h * du) - fint(u - h * du)) / (2 * h)
    Kdu = K * du
    assert np.linalg.norm(fd - Kdu) <= 1e-6 * np.linalg.norm(Kdu)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fused_tangent_bit_identical(llf, orc, case):
    _, n, order, simplex = case
    m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    p = llf.Problem([llf.Material("body")], type="Solid")
    F, _ = _F(llf, m, p, 0.03, 31)
    K = llf.tangentMatrix(p, F, energy="NeoHookeCompressible", params={"mu": 1.0, "lambda": 10.0})
    ref = orc.tl_matrix(3, m.xyz, m.conn, llf._lib.builtin_rule(m.family, m.order), F.A, orc.LAW_NEOHOOKE,
                        [1.0, 10.0])
    assert_csc_identical(K.csc(), ref.julia(), f"Kt {case[0]}")


def test_fused_tangent_is_derivative_of_internal_force(llf):
    m = llf.structured_box_mesh(n=2, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    prm = {"mu": 1.0, "lambda": 10.0}
    rng = np.random.default_rng(37)
    u = (m.xyz @ (0.05 * rng.standard_normal((3, 3))).T).ravel()
    du = (m.xyz @ rng.standard_normal((3, 3)).T).ravel()
    fint = lambda v: llf.internalForceVector(p, F=llf.grad(llf.VectorField(v.reshape(-1, 1), p), add_identity=True),
                                             energy="NeoHookeCompressible", params=prm).a[:, 0]
    K = llf.tangentMatrix(p, llf.grad(llf.VectorField(u.reshape(-1, 1), p), add_identity=True), params=prm)
    h = 1e-6
    fd = (fint(u + h * du) - fint(u - h * du)) / (2 * h)
    assert np.linalg.norm(fd - K * du) <= 1e-6 * np.linalg.norm(K * du)


def test_newton_stretch_converges(llf):
    """Hyperelastic TL configuration in miniature: compressible neo-Hookean
    (mu=1, lambda=10) unit cube, 30% axial stretch in 3 steps, full Newton
    with the consistent tangent reassembled every iteration."""
    m = llf.structured_box_mesh(n=3, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    sup = [llf.displacementConstraint("left", ux=0.0), llf.displacementConstraint("right", ux=0.3),
           llf.displacementConstraint("bottom", uy=0.0), llf.displacementConstraint("rear", uz=0.0)]
    u = llf.solveDeformation(p, support=sup, params={"mu": 1.0, "lambda": 10.0}, steps=3, tol=1e-10)
    ux = u.a[0::3, 0]
    assert abs(ux[np.abs(m.xyz[:, 0] - 1) < 1e-12] - 0.3).max() < 1e-14
    last = [h for h in u.history if h["step"] == 3]
    assert last[-1]["residual"] <= 1e-10 * max(1.0, last[0]["residual"]) or len(last) <= 25
    # quadratic convergence: the last reductions shrink fast
    res = [h["residual"] for h in last]
    assert res[-1] < 1e-9
    # homogeneous uniaxial stretch: lateral contraction is uniform
    uy = u.a[1::3, 0]
    top = np.abs(m.xyz[:, 1] - 1) < 1e-12
    assert np.ptp(uy[top]) < 1e-9


TC_CASES = [("hex27", 2, 2, False), ("hex64", 2, 3, False), ("hex125", 1, 4, False), ("tet20", 1, 3, True)]


def _smooth_F(llf, m, p):
    """F = I + grad u of a smooth, moderate deformation (stretch, shear and a
    bending mode): well-conditioned, as in a Newton step of a physical load."""
    x, y, z = m.xyz[:, 0], m.xyz[:, 1], m.xyz[:, 2]
    u = np.stack([0.10 * x + 0.03 * y * z, -0.02 * y + 0.05 * np.sin(np.pi * x), 0.04 * z * x], axis=1)
    return llf.grad(llf.VectorField(u.reshape(-1, 1), p), add_identity=True)


@pytest.mark.parametrize("case", TC_CASES, ids=[c[0] for c in TC_CASES])
def test_tensor_core_tangent_within_tf32x3_tolerance(llf, case):
    """Tensor-core form (tcgen05, split TF32 products, FP32 accumulation):
    every structural value within 5e-5 of the largest FP64 value for a
    well-conditioned deformation (tile operands formed in FP32, FP32 sums over
    15 rows x nip points in tensor memory)."""
    _, n, order, simplex = case
    m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
    p = llf.Problem([llf.Material("body")], type="Solid")
    F = _smooth_F(llf, m, p)
    prm = {"mu": 1.0, "lambda": 10.0}
    K64 = llf.tangentMatrix(p, F, energy="NeoHookeCompressible", params=prm)
    Ktc = llf.tangentMatrix(p, F, energy="NeoHookeCompressible", params=prm, precision="tf32x3")
    a, b = K64.dm.copy_structural(), Ktc.dm.copy_structural()
    scale = np.abs(a).max()
    err = np.abs(a - b).max() / scale
    assert err <= 5e-5, err
    assert err > 0.0  # the tensor-core path really ran (TF32 splits are not bit-exact)
    # mirrored entries are made equal, so the tangent is symmetric bit for bit
    A = Ktc.A
    assert abs(A - A.T).max() == 0.0


@pytest.mark.parametrize("order,n", [(3, 2), (4, 2)], ids=["hex64", "hex125"])
def test_newton_converges_with_tensor_core_tangent(llf, order, n):
    """The order-3/4 hexahedra of the hyperelastic configuration with the
    tangent assembled on the tensor cores (tf32x3): f_int and the update stay
    FP64, so Newton reaches the same FP64 residual tolerance as with the FP64
    tangent and the same displacement, at most a few iterations later."""
    llf.structured_box_mesh(n=n, order=order)
    p = llf.Problem([llf.Material("body")], type="Solid")
    sup = [llf.displacementConstraint("left", ux=0.0), llf.displacementConstraint("right", ux=0.3),
           llf.displacementConstraint("bottom", uy=0.0), llf.displacementConstraint("rear", uz=0.0)]
    prm = {"mu": 1.0, "lambda": 10.0}
    u64 = llf.solveDeformation(p, support=sup, params=prm, steps=3, tol=1e-8)
    utc = llf.solveDeformation(p, support=sup, params=prm, steps=3, tol=1e-8, tangent="tf32x3")
    for step in (1, 2, 3):
        # a step that converged ends with a residual record and no solve after it
        last = [h for h in utc.history if h["step"] == step][-1]
        assert "cg_iterations" not in last, (step, last)
    it64, ittc = len(u64.history), len(utc.history)
    assert ittc <= it64 + 6, (it64, ittc)
    d = np.linalg.norm(utc.a - u64.a) / np.linalg.norm(u64.a)
    assert d <= 1e-7, d
