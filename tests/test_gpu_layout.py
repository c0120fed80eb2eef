"""Stored-layout reuse.  An assembly whose pattern holds the stored layout of
an earlier assembly of the same operator and arithmetic form writes the
stored CSC straight from the gather into that layout and checks every
column's count; a column whose count differs sends the assembly through the
counting compaction, whose layout then replaces the kept one.  Either way
the stored CSC is the oracle's bit for bit."""
import os

import numpy as np
import pytest

from helpers import PT, assert_csc_identical, make_mesh, oracle_operator

pytestmark = pytest.mark.gpu


def _two_material_box(llf, n=3, order=2):
    m = llf.structured_box_mesh(n=n, order=order)
    cx = m.xyz[m.conn - 1][:, :, 0].mean(axis=1)
    for name, sel in (("a", np.where(cx < 0.5)[0]), ("b", np.where(cx >= 0.5)[0])):
        g = llf.Group(name, 3, np.unique(m.conn[sel]), m.family, m.order, m.conn[sel])
        g.elems = sel
        m.groups[name] = g
    return m, np.where(cx < 0.5, 0, 1).astype(np.int32)


def _assemble(llf, p, precision, ctx):
    ctx.profile_reset()
    ctx.profile(True)
    K = llf.stiffnessMatrix(p, precision=precision)
    ctx.sync()
    ctx.profile(False)
    return K, set(ctx.profile_report())


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_reuse_through_value_changes(llf, orc, precision):
    m, emat = _two_material_box(llf)
    ma = llf.Material("a", E=1e5, nu=0.25)
    mb = llf.Material("b", E=3e5, nu=0.35)
    p = llf.Problem([ma, mb], type="Solid")
    ctx = p._ctx
    rule = llf._lib.builtin_rule(m.family, m.order)
    # (E_b, nu_b, whether the kept layout fits, None: either): E_b = 0
    # empties the columns of the nodes inside part b, so the counts change
    # when it comes and when it goes
    seq = [(3e5, 0.35, False), (3e5, 0.35, True), (2e5, 0.3, None), (0.0, 0.3, False), (0.0, 0.3, True),
           (3e5, 0.35, False), (3e5, 0.35, True)]
    for k, (E_b, nu_b, reused) in enumerate(seq):
        mb.E, mb.nu = E_b, nu_b
        K, kernels = _assemble(llf, p, precision, ctx)
        if reused is not None:
            assert ("k_compact" not in kernels) == reused, (k, sorted(kernels))
        if precision == "fp64":
            ref = orc.assemble(orc.ELASTIC, 0, 3, 3, m.xyz, m.conn, rule, [ma.E, ma.nu, mb.E, mb.nu], emat=emat)
            assert_csc_identical(K.csc(), ref.julia(), f"step {k}: E_b = {E_b}")
        else:
            os.environ["LLF_STORED_LAYOUT"] = "0"
            try:
                fresh = llf.stiffnessMatrix(p, precision=precision).csc()
            finally:
                del os.environ["LLF_STORED_LAYOUT"]
            assert_csc_identical(K.csc(), fresh, f"step {k}: E_b = {E_b}")


def test_operators_keep_separate_layouts(llf, orc):
    """K and M on one pattern each keep their own layout; a lumped mass
    matrix uses none."""
    m = llf.structured_box_mesh(n=3, order=2)
    mat = llf.Material("body", E=2.1e5, nu=0.3, rho=7.85e-9)
    p = llf.Problem([mat], type="Solid")
    rule = llf._lib.builtin_rule(m.family, m.order)
    refK = orc.assemble(orc.ELASTIC, 0, 3, 3, m.xyz, m.conn, rule, [mat.E, mat.nu]).julia()
    refM = orc.assemble(orc.MASS, 0, 3, 3, m.xyz, m.conn, rule, [mat.rho]).julia()
    refL = orc.assemble(orc.MASS, 0, 3, 3, m.xyz, m.conn, rule, [mat.rho], lumped=True).julia()
    for _ in range(3):
        assert_csc_identical(llf.stiffnessMatrix(p).csc(), refK, "K")
        assert_csc_identical(llf.massMatrix(p, lumped=False).csc(), refM, "M")
        assert_csc_identical(llf.massMatrix(p, lumped=True).csc(), refL, "lumped M")


def test_reused_matrix_solves_like_a_fresh_one(llf):
    """A matrix assembled into a kept layout holds the stored CSC only; its
    structural values, expanded on first use, equal a fresh assembly's (the
    entries dropzeros! removed come back as +0.0, equal in value to the
    fresh assembly's zeros of either sign), and CG gives the same iterates."""
    m = llf.structured_box_mesh(n=4, order=2)
    mat = llf.Material("body", E=2.1e5, nu=0.3)
    p = llf.Problem([mat], type="Solid")
    K1 = llf.stiffnessMatrix(p)   # leaves the layout
    K2 = llf.stiffnessMatrix(p)   # writes into it
    assert_csc_identical(K1.csc(), K2.csc(), "stored CSC")
    a, b = K1.dm.copy_structural(), K2.dm.copy_structural()
    assert np.array_equal(a, b)
    nz = a != 0
    assert np.array_equal(a[nz].view(np.uint64), b[nz].view(np.uint64))
    n = K1.dm.n
    rng = np.random.default_rng(3)
    f = rng.standard_normal(n)
    fixed = np.zeros(n, dtype=np.uint8)
    fixed[:30] = 1
    x0 = np.zeros(n)
    u1, it1, _ = K1.dm.pcg(f, x0, fixed, precond=1, reltol=1e-10, maxiter=20 * n)
    u2, it2, _ = K2.dm.pcg(f, x0, fixed, precond=1, reltol=1e-10, maxiter=20 * n)
    assert it1 == it2 and np.array_equal(u1, u2)


def test_geometry_kept_until_the_mesh_changes(llf, orc):
    """The affine geometry is kept on the device mesh between assemblies and
    recomputed after a coordinate upload: turning the mesh and turning it
    back gives the oracle's matrices each time."""
    m = llf.structured_box_mesh(n=3, order=2)
    mat = llf.Material("body", E=2.1e5, nu=0.3)
    p = llf.Problem([mat], type="Solid")
    rule = llf._lib.builtin_rule(m.family, m.order)
    xyz0 = m.xyz.copy()
    c, s_ = np.cos(0.4), np.sin(0.4)
    turned = (xyz0 - 0.5) @ np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]]).T + 0.5
    dm = p.device_mesh()
    for xyz in (xyz0, turned, turned, xyz0, xyz0):
        dm.update(xyz, m.conn)
        K = llf.stiffnessMatrix(p)
        ref = orc.assemble(orc.ELASTIC, 0, 3, 3, xyz, m.conn, rule, [mat.E, mat.nu])
        assert_csc_identical(K.csc(), ref.julia(), "after a coordinate upload")


@pytest.mark.parametrize("case", [("rect", 6, 2, False), ("rect", 4, 1, True), ("box", 3, 2, True)],
                         ids=["quad9", "tri3", "tet10"])
def test_scalar_and_plane_operators_reuse(llf, orc, case):
    """Conduction and plane-strain stiffness assembled three times on one
    pattern (the second and third into the kept layout): the oracle's
    matrices each time."""
    kind, n, order, simplex = case
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body", E=2.1e5, nu=0.3, k=45.0)
    d = m.dim
    hp = "HeatConduction" if d == 3 else "PlaneHeatConduction"
    ph = llf.Problem([mat], type=hp, thickness=0.5)
    sp_ = "Solid" if d == 3 else "PlaneStrain"
    ps = llf.Problem([mat], type=sp_, thickness=0.5)
    refH = oracle_operator(llf, orc, m, "heat", PT[hp], mat, thickness=0.5).julia()
    refK = oracle_operator(llf, orc, m, "stiffness", PT[sp_], mat, thickness=0.5).julia()
    for _ in range(3):
        assert_csc_identical(llf.heatConductionMatrix(ph).csc(), refH, f"H {case}")
        assert_csc_identical(llf.stiffnessMatrix(ps).csc(), refK, f"K {case}")
