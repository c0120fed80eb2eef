"""GPU assembly vs the CPU oracle, through the C-ABI.

The FP64 form follows the same arithmetic contract as the oracle, so the
stored CSC (colptr, rowval, nzval) must be identical bit for bit, including
the dropzeros! pattern.  Full-size configurations are checked through
size-independent properties.
"""
import numpy as np
import pytest

from helpers import PT, assert_csc_identical, make_mesh, oracle_operator

pytestmark = pytest.mark.gpu

SOLID_CASES = [
    # kind, n, order, simplex, ptype
    ("rect", 6, 1, False, "PlaneStress"),
    ("rect", 5, 2, False, "PlaneStrain"),
    ("rect", 3, 3, False, "PlaneStrain"),
    ("rect", 2, 4, False, "PlaneStress"),
    ("rect", 5, 1, True, "PlaneStrain"),
    ("rect", 3, 2, True, "PlaneStress"),
    ("rect", 2, 4, True, "PlaneStrain"),
    ("box", 3, 1, False, "Solid"),
    ("box", 3, 2, False, "Solid"),
    ("box", 2, 3, False, "Solid"),
    ("box", 1, 4, False, "Solid"),
    ("box", 2, 1, True, "Solid"),
    ("box", 2, 2, True, "Solid"),
    ("box", 1, 3, True, "Solid"),
    ("box", 1, 4, True, "Solid"),
]


def _ids(c):
    return f"{c[0]}-n{c[1]}-p{c[2]}{'-simplex' if c[3] else ''}-{c[4]}"


@pytest.mark.parametrize("case", SOLID_CASES, ids=_ids)
def test_stiffness_bit_identical(llf, orc, case):
    kind, n, order, simplex, ptype = case
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body", E=2.1e5, nu=0.3)
    p = llf.Problem([mat], type=ptype, thickness=0.7)
    K = llf.stiffnessMatrix(p)
    ref = oracle_operator(llf, orc, m, "stiffness", PT[ptype], mat, thickness=0.7)
    assert_csc_identical(K.csc(), ref.julia(), f"K {_ids(case)}")


@pytest.mark.parametrize("case", SOLID_CASES[::2], ids=_ids)
@pytest.mark.parametrize("lumped", [False, True])
def test_mass_bit_identical(llf, orc, case, lumped):
    kind, n, order, simplex, ptype = case
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body", rho=7.85e-9)
    p = llf.Problem([mat], type=ptype, thickness=0.7)
    M = llf.massMatrix(p, lumped=lumped)
    ref = oracle_operator(llf, orc, m, "mass", PT[ptype], mat, thickness=0.7, lumped=lumped)
    assert_csc_identical(M.csc(), ref.julia(), f"M lumped={lumped} {_ids(case)}")


HEAT_CASES = [("rect", 6, 1, False), ("rect", 3, 3, False), ("rect", 3, 2, True),
              ("box", 3, 1, False), ("box", 2, 2, False), ("box", 1, 4, False), ("box", 2, 2, True)]


@pytest.mark.parametrize("case", HEAT_CASES, ids=lambda c: f"{c[0]}-n{c[1]}-p{c[2]}{'-simplex' if c[3] else ''}")
def test_heat_bit_identical(llf, orc, case):
    kind, n, order, simplex = case
    m = make_mesh(llf, kind, n, order, simplex)
    ptype = "HeatConduction" if kind == "box" else "PlaneHeatConduction"
    mat = llf.Material("body", k=45.0)
    p = llf.Problem([mat], type=ptype, thickness=2.0)
    K = llf.heatConductionMatrix(p)
    ref = oracle_operator(llf, orc, m, "heat", PT[ptype], mat, thickness=2.0)
    assert_csc_identical(K.csc(), ref.julia(), f"KT {case}")


def test_two_materials_and_skipped_elements(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2)
    cx = m.xyz[m.conn - 1][:, :, 0].mean(axis=1)
    sel_a = np.where(cx < 0.5)[0]
    sel_b = np.where(cx >= 0.5)[0]
    for name, sel in (("a", sel_a), ("b", sel_b)):
        g = llf.Group(name, 3, np.unique(m.conn[sel]), m.family, m.order, m.conn[sel])
        g.elems = sel
        m.groups[name] = g
    ma = llf.Material("a", E=1e5, nu=0.25)
    mb = llf.Material("b", E=3e5, nu=0.35)
    p = llf.Problem([ma, mb], type="Solid")
    K = llf.stiffnessMatrix(p)
    emat = np.where(cx < 0.5, 0, 1).astype(np.int32)
    rule = llf._lib.builtin_rule(m.family, m.order)
    ref = orc.assemble(orc.ELASTIC, 0, 3, 3, m.xyz, m.conn, rule, [ma.E, ma.nu, mb.E, mb.nu], emat=emat)
    assert_csc_identical(K.csc(), ref.julia(), "two materials")
    # a single material on half of the body: the other elements contribute nothing
    p1 = llf.Problem([ma], type="Solid")
    K1 = llf.stiffnessMatrix(p1)
    em1 = np.where(cx < 0.5, 0, -1).astype(np.int32)
    ref1 = orc.assemble(orc.ELASTIC, 0, 3, 3, m.xyz, m.conn, rule, [ma.E, ma.nu], emat=em1)
    assert_csc_identical(K1.csc(), ref1.julia(), "half body")


def test_pattern_copy_matches_oracle(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    colptr, rowval = p.pattern().copy()
    rc, rr, _ = orc.pattern(m.non, m.conn, 3).julia()
    assert np.array_equal(colptr, rc) and np.array_equal(rowval, rr)


def test_axpby_same_pattern(llf, orc):
    llf.structured_box_mesh(n=2, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    K = llf.stiffnessMatrix(p)
    M = llf.massMatrix(p, lumped=False)
    S = K + M
    D = K - K
    assert D.nnz() == 0
    Ks = K.dm.copy_structural()
    Ms = M.dm.copy_structural()
    Ss = S.dm.copy_structural()
    assert np.array_equal(Ss, Ks + Ms)
    c, r, v = S.csc()
    assert np.array_equal(v, (Ks + Ms)[(Ks + Ms) != 0])


def test_spmv_matches_scipy(llf):
    llf.structured_box_mesh(n=4, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    K = llf.stiffnessMatrix(p)
    x = np.random.default_rng(0).standard_normal(K.shape[0])
    y = K * x
    yref = K.A @ x
    assert np.abs(y - yref).max() <= 1e-13 * np.abs(yref).max()


def test_grad_bit_identical(llf, orc):
    m = llf.structured_box_mesh(n=2, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    rng = np.random.default_rng(1)
    u = llf.VectorField(rng.standard_normal((3 * m.non, 1)) * 1e-2, p)
    F = llf.grad(u, add_identity=True)
    rule = llf._lib.builtin_rule(m.family, m.order)
    ref = orc.grad_elementwise(m.xyz, m.conn, rule, u.a[:, 0], add_identity=True)
    assert np.array_equal(F.A, ref)
    # a linear field has a constant gradient
    A = np.array([[0.1, 0.2, -0.3], [0.05, -0.1, 0.0], [0.3, 0.0, 0.2]])
    ul = (m.xyz @ A.T).ravel()
    T = llf.grad(llf.VectorField(ul.reshape(-1, 1), p)).A.reshape(m.nel, m.npe, 3, 3)
    assert np.abs(T - A.T[None, None]).max() < 1e-13   # column-major T[i,j] = A[i,j]


def test_load_vector_bit_identical(llf, orc):
    m = llf.structured_box_mesh(n=3, order=2)
    p = llf.Problem([llf.Material("body")], type="Solid")
    f = llf.loadVector(p, [llf.load("right", fx=1.0, fy=-2.0, fz=0.5)])
    g = m.group("right")
    ref = orc.load_vector(3, 3, m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), t=[1.0, -2.0, 0.5])
    assert np.array_equal(f.a[:, 0], ref)
    assert np.allclose(f.a[:, 0].reshape(-1, 3).sum(axis=0), [1.0, -2.0, 0.5], rtol=1e-13)
    m2 = llf.structured_rect_mesh(n=4, order=3)
    p2 = llf.Problem([llf.Material("body")], type="PlaneStress", thickness=0.5)
    f2 = llf.loadVector(p2, [llf.load("top", fy=-1.0)])
    g2 = m2.group("top")
    ref2 = orc.load_vector(2, 2, m2.xyz, g2.conn, llf._lib.builtin_rule(g2.family, g2.order), t=[0.0, -1.0],
                           thickness=0.5)
    assert np.array_equal(f2.a[:, 0], ref2)


PRECISION_CASES = [("rect", 5, 2, False, "PlaneStrain"), ("box", 3, 1, False, "Solid"),
                   ("box", 3, 2, False, "Solid"), ("box", 2, 2, True, "Solid")]


@pytest.mark.parametrize("case", PRECISION_CASES, ids=_ids)
def test_precision_form_within_fp32_tolerance(llf, case):
    """FP32 quadrature / FP64 accumulation: every structural value within
    1e-6 of the column's largest FP64 value (FP32 has 6e-8 unit roundoff)."""
    kind, n, order, simplex, ptype = case
    make_mesh(llf, kind, n, order, simplex)
    p = llf.Problem([llf.Material("body", E=2.1e5, nu=0.3)], type=ptype)
    for op in ("stiffness", "mass", "heat"):
        if op == "heat":
            p = llf.Problem([llf.Material("body")], type="HeatConduction" if kind == "box" else "PlaneHeatConduction")
            A64, A32 = llf.heatConductionMatrix(p), llf.heatConductionMatrix(p, precision="fp32")
        elif op == "mass":
            A64, A32 = llf.massMatrix(p, lumped=False), llf.massMatrix(p, lumped=False, precision="fp32")
        else:
            A64, A32 = llf.stiffnessMatrix(p), llf.stiffnessMatrix(p, precision="fp32")
        v64, v32 = A64.dm.copy_structural(), A32.dm.copy_structural()
        scale = np.abs(v64).max()
        assert np.abs(v32 - v64).max() <= 1e-6 * scale, op


DISTORTED_CASES = [("box", 2, 2, False, "Solid"), ("box", 3, 1, False, "Solid"),
                   ("rect", 3, 3, False, "PlaneStrain"), ("box", 2, 2, True, "Solid")]


@pytest.mark.parametrize("case", DISTORTED_CASES, ids=_ids)
@pytest.mark.parametrize("part", ["all", "half"])
def test_distorted_mesh_bit_identical(llf, orc, case, part):
    """Interior nodes moved (everywhere, or only for x > 0.5): distorted
    elements take the quadrature form, the others the affine form, on both
    sides."""
    kind, n, order, simplex, ptype = case
    m = make_mesh(llf, kind, n, order, simplex)
    d = m.dim
    sel = np.all((m.xyz[:, :d] > 1e-9) & (m.xyz[:, :d] < 1 - 1e-9), axis=1)
    if part == "half":
        sel &= m.xyz[:, 0] > 0.5 + 1e-9
    rng = np.random.default_rng(5)
    m.xyz[sel, :d] += rng.uniform(-0.04, 0.04, (sel.sum(), d)) / n
    mat = llf.Material("body", E=2.1e5, nu=0.3, rho=7.85e-9, k=45.0)
    p = llf.Problem([mat], type=ptype)
    assert_csc_identical(llf.stiffnessMatrix(p).csc(), oracle_operator(llf, orc, m, "stiffness", PT[ptype], mat).julia(),
                         f"K {_ids(case)} {part}")
    assert_csc_identical(llf.massMatrix(p, lumped=False).csc(),
                         oracle_operator(llf, orc, m, "mass", PT[ptype], mat).julia(), f"M {_ids(case)} {part}")
    hp = "HeatConduction" if d == 3 else "PlaneHeatConduction"
    ph = llf.Problem([mat], type=hp)
    assert_csc_identical(llf.heatConductionMatrix(ph).csc(), oracle_operator(llf, orc, m, "heat", PT[hp], mat).julia(),
                         f"H {_ids(case)} {part}")


def _turned(xyz, d, angle):
    """xyz turned by angle about (1, 2, 3) (3D) or the z axis (2D) through
    the centre of the unit cell."""
    if d == 3:
        ax = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
        K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        R = np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)
    else:
        c, s = np.cos(angle), np.sin(angle)
        R = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    out = (xyz - 0.5) @ R.T + 0.5
    if d == 2:
        out[:, 2] = xyz[:, 2]
    return out


AFFINE_CASES = [("box", 2, 2, False, "Solid"), ("box", 2, 1, True, "Solid"), ("rect", 3, 3, False, "PlaneStrain"),
                ("rect", 2, 2, True, "PlaneStress")]


@pytest.mark.parametrize("case", AFFINE_CASES, ids=_ids)
@pytest.mark.parametrize("geometry", ["turned", "turned-1e-9", "turned-1e-15", "stretched"])
def test_affine_geometry_forms_bit_identical(llf, orc, case, geometry):
    """Affine elements that are axis-aligned bricks (stretched, or turned by
    less than the rounding of their Jacobian) take the reduced node-pair
    form, the others the full one; both are the oracle's bit for bit."""
    kind, n, order, simplex, ptype = case
    m = make_mesh(llf, kind, n, order, simplex)
    d = m.dim
    if geometry == "stretched":
        m.xyz[:, :d] *= np.array([2.5, 0.75, 1.3])[:d]
    else:
        m.xyz[:] = _turned(m.xyz, d, {"turned": 0.3, "turned-1e-9": 1e-9, "turned-1e-15": 1e-15}[geometry])
    mat = llf.Material("body", E=2.1e5, nu=0.3, rho=7.85e-9, k=45.0)
    p = llf.Problem([mat], type=ptype, thickness=0.7)
    assert_csc_identical(llf.stiffnessMatrix(p).csc(),
                         oracle_operator(llf, orc, m, "stiffness", PT[ptype], mat, thickness=0.7).julia(),
                         f"K {_ids(case)} {geometry}")
    assert_csc_identical(llf.massMatrix(p, lumped=False).csc(),
                         oracle_operator(llf, orc, m, "mass", PT[ptype], mat, thickness=0.7).julia(),
                         f"M {_ids(case)} {geometry}")
    hp = "HeatConduction" if d == 3 else "PlaneHeatConduction"
    ph = llf.Problem([mat], type=hp, thickness=0.7)
    assert_csc_identical(llf.heatConductionMatrix(ph).csc(),
                         oracle_operator(llf, orc, m, "heat", PT[hp], mat, thickness=0.7).julia(),
                         f"H {_ids(case)} {geometry}")


# ---------------------------------------------------------------- error paths
def test_inverted_element_is_an_error(llf):
    m = llf.structured_box_mesh(n=2, order=1)
    m.conn[0] = m.conn[0][[1, 0, 3, 2, 5, 4, 7, 6]]  # mirror element 0
    p = llf.Problem([llf.Material("body")], type="Solid")
    with pytest.raises(llf.LLFError, match="Jacobian"):
        llf.stiffnessMatrix(p)


def test_bad_node_tag_is_an_error(llf):
    m = llf.structured_box_mesh(n=2, order=1)
    m.conn[3, 2] = m.non + 5
    p = llf.Problem([llf.Material("body")], type="Solid")
    with pytest.raises(llf.LLFError, match="node tag"):
        p.device_mesh()


def test_nan_coordinate_is_an_error(llf):
    m = llf.structured_box_mesh(n=2, order=1)
    m.xyz[4, 1] = np.nan
    p = llf.Problem([llf.Material("body")], type="Solid")
    with pytest.raises(llf.LLFError, match="NaN"):
        p.device_mesh()


# ---------------------------------------------------------------- full size
def test_c1_quad4_full_size_properties(llf, orc):
    m = llf.structured_rect_mesh(lx=10.0, ly=5.0, dx=0.05, dy=0.05)
    mat = llf.Material("body", E=2e5, nu=0.3)
    p = llf.Problem([mat], type="PlaneStrain")
    K = llf.stiffnessMatrix(p)
    ref = oracle_operator(llf, orc, m, "stiffness", PT["PlaneStrain"], mat)
    assert_csc_identical(K.csc(), ref.julia(), "C1 quad4 200x100")


def test_c2_hex27_full_size_bit_identical(llf, orc):
    """Config 2 at full size, the bench's headline workload: hex27 40^3
    (531,441 nodes, 64,000 elements, 297,685,449 structural entries), K and
    the consistent M against the oracle's serial restatement of the
    reference's COO assembly + sparse + dropzeros!, bit for bit.  This is the
    case with two degree-class gather launches, 64,000-element persistent
    grids and row positions up to degree 125."""
    m = llf.structured_box_mesh(n=40, order=2)
    mat = llf.Material("body", E=2.1e5, nu=0.3, rho=7.85e-9)
    p = llf.Problem([mat], type="Solid")
    assert p.pattern().nnz == 297685449
    K = llf.stiffnessMatrix(p)
    got = K.csc()
    K.dm = None
    ref = oracle_operator(llf, orc, m, "stiffness", 0, mat)
    assert_csc_identical(got, ref.julia(), "C2 K hex27 40^3")
    del got, ref
    M = llf.massMatrix(p, lumped=False)
    got = M.csc()
    M.dm = None
    ref = oracle_operator(llf, orc, m, "mass", 0, mat)
    assert_csc_identical(got, ref.julia(), "C2 consistent M hex27 40^3")
    assert len(got[2]) == 99228483   # same-component couplings only (the survey's count)


def test_connectivity_change_requires_new_pattern(llf, orc):
    """The pattern carries an element-to-column map: re-uploading the same
    connectivity keeps it valid; a changed connectivity makes assembly fail
    with LLF_ERR_STATE until a new pattern is built."""
    L = llf._lib
    m = llf.structured_box_mesh(n=2, order=2)
    ctx = L.Context(0)
    dm = L.DeviceMesh(ctx, m.dim, m.xyz, m.conn, m.family, m.order)
    pat = L.DevicePattern(dm, 3)
    E, nu = np.array([2.1e5]), np.array([0.3])

    def assemble(p):
        h = L.C.c_void_p()
        rc = L.lib().llf_assemble_stiffness(ctx.h, dm.h, p.h, 0, L.ptr(E, L.C.c_double), L.ptr(nu, L.C.c_double),
                                            1, 1.0, 0, L.C.byref(h))
        return rc, (L.DeviceMatrix(ctx, h, p) if rc == 0 else None)

    rc, K0 = assemble(pat)
    assert rc == 0
    dm.update(m.xyz, m.conn)                       # same connectivity: pattern still valid
    rc, K1 = assemble(pat)
    assert rc == 0
    assert all(np.array_equal(a, b) for a, b in zip(K0.copy_csc(), K1.copy_csc()))
    conn2 = np.asarray(m.conn).copy()
    conn2[[0, 1]] = conn2[[1, 0]]                  # same elements, another element order
    dm.update(m.xyz, conn2)
    rc, _ = assemble(pat)
    assert rc == -5 and "pattern" in L.lib().llf_last_error(ctx.h).decode()
    pat2 = L.DevicePattern(dm, 3)
    rc, K2 = assemble(pat2)
    assert rc == 0
    ref = orc.assemble(orc.ELASTIC, 0, 3, 3, m.xyz, conn2, L.builtin_rule(m.family, m.order), [2.1e5, 0.3])
    assert_csc_identical(K2.copy_csc(), ref.julia(), "K after connectivity change")


@pytest.mark.parametrize("case", [("box", 3, 2, False), ("rect", 4, 3, True), ("box", 2, 1, True)],
                         ids=["hex27", "tri10", "tet4"])
@pytest.mark.parametrize("lumped", [False, True])
def test_heat_capacity_bit_identical(llf, orc, case, lumped):
    """heatCapacityMatrix (src/heat.jl:257-376): c rho sum H^T H detJ w with b = 1."""
    kind, n, order, simplex = case
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body", rho=7.85e-9, c=4.2e8)
    pt = "HeatConduction" if m.dim == 3 else "PlaneHeatConduction"
    p = llf.Problem([mat], type=pt, thickness=0.7)
    C = llf.heatCapacityMatrix(p, lumped=lumped)
    rule = llf._lib.builtin_rule(m.family, m.order)
    ref = orc.assemble(orc.MASS, PT[pt], m.dim, 1, m.xyz, m.conn, rule, [mat.c * mat.rho], 0.7, lumped)
    assert_csc_identical(C.csc(), ref.julia(), f"C {kind} {order} lumped={lumped}")


@pytest.mark.parametrize("case", [("box", 17, 1, False), ("box", 9, 2, True), ("rect", 70, 2, False)],
                         ids=["hex8-4913", "tet10-4374", "quad9-4900"])
def test_larger_meshes_bit_identical(llf, orc, case):
    """Meshes of several thousand elements (many gather CTAs and grid-stride
    passes per kernel) against the oracle."""
    kind, n, order, simplex = case
    m = make_mesh(llf, kind, n, order, simplex)
    assert m.nel >= 4096
    pt = "Solid" if m.dim == 3 else "PlaneStrain"
    mat = llf.Material("body", E=2.1e5, nu=0.3, k=45.0)
    p = llf.Problem([mat], type=pt)
    K = llf.stiffnessMatrix(p)
    ref = oracle_operator(llf, orc, m, "stiffness", PT[pt], mat)
    assert_csc_identical(K.csc(), ref.julia(), f"stiffness {kind} n{n} p{order}")
    ph = llf.Problem([mat], type="HeatConduction" if m.dim == 3 else "PlaneHeatConduction")
    H = llf.heatConductionMatrix(ph)
    refh = oracle_operator(llf, orc, m, "heat", PT[ph.type], mat)
    assert_csc_identical(H.csc(), refh.julia(), f"conduction {kind} n{n} p{order}")


# ------------------------------------------------------- caller-supplied tables
def _permuted_rule(rule, scale=1.0):
    """The built-in rule with its points in reverse order and its weights
    scaled: what a caller passing gmsh's own getIntegrationPoints /
    getBasisFunctions output (src/linear.jl:235-243) may hand over, in
    another point order and normalisation."""
    q = np.arange(rule["nip"])[::-1]
    return {"nip": rule["nip"], "npe": rule["npe"], "w": rule["w"][q] * scale,
            "N": np.ascontiguousarray(rule["N"][q]), "dN": np.ascontiguousarray(rule["dN"][q]),
            "node_ref": None}


@pytest.mark.parametrize("case", [("box", 2, 2, False, "Solid"), ("box", 2, 2, True, "Solid"),
                                  ("rect", 3, 3, False, "PlaneStrain"), ("rect", 2, 2, True, "PlaneStress")],
                         ids=["hex27", "tet10", "quad16", "tri6"])
@pytest.mark.parametrize("scale", [1.0, 0.5])
def test_tables_upload_bit_identical(llf, orc, case, scale):
    """llf_tables_upload (the path the Julia shim takes with gmsh's tables):
    K, M and the conduction matrix from caller-supplied tables equal the
    oracle fed the same tables bit for bit, with the table layout
    N[q*npe+a], dN[(q*npe+a)*3+j]; scale 1 agrees with the built-in rule to
    rounding (only the point order differs)."""
    kind, n, order, simplex, ptype = case
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body", E=2.1e5, nu=0.3, rho=7.85e-9, k=45.0)
    rule = _permuted_rule(llf._lib.builtin_rule(m.family, m.order), scale)
    p = llf.Problem([mat], type=ptype, thickness=0.7)
    p.device_mesh().set_tables(rule["w"], rule["N"], rule["dN"])
    K = llf.stiffnessMatrix(p)
    ref = orc.assemble(orc.ELASTIC, PT[ptype], m.dim, m.dim, m.xyz, m.conn, rule, [mat.E, mat.nu], 0.7,
                       affine=False)
    assert_csc_identical(K.csc(), ref.julia(), f"K from uploaded tables {kind} p{order}")
    M = llf.massMatrix(p, lumped=False)
    refm = orc.assemble(orc.MASS, PT[ptype], m.dim, m.dim, m.xyz, m.conn, rule, [mat.rho], 0.7, affine=False)
    assert_csc_identical(M.csc(), refm.julia(), f"M from uploaded tables {kind} p{order}")
    pt = "HeatConduction" if m.dim == 3 else "PlaneHeatConduction"
    ph = llf.Problem([mat], type=pt, thickness=0.7)
    ph.device_mesh().set_tables(rule["w"], rule["N"], rule["dN"])
    H = llf.heatConductionMatrix(ph)
    refh = orc.assemble(orc.HEAT, PT[pt], m.dim, 1, m.xyz, m.conn, rule, [mat.k], 0.7, affine=False)
    assert_csc_identical(H.csc(), refh.julia(), f"conduction from uploaded tables {kind} p{order}")
    if scale == 1.0:
        Kb = oracle_operator(llf, orc, m, "stiffness", PT[ptype], mat, thickness=0.7).scipy()
        d = abs(K.A - Kb).max() / abs(Kb).max()
        assert d <= 1e-13, d
