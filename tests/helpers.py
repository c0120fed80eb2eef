"""Shared helpers for the tests (mesh factories, CSC comparison)."""
import numpy as np

PT = {"Solid": 0, "PlaneStress": 1, "PlaneStrain": 2, "HeatConduction": 3, "PlaneHeatConduction": 4}


def make_mesh(llf, kind, n, order, simplex=False):
    if kind == "rect":
        return llf.structured_rect_mesh(n=n, order=order, simplex=simplex)
    return llf.structured_box_mesh(n=n, order=order, simplex=simplex)


def oracle_operator(llf, orc, mesh, op, ptype, mat, thickness=1.0, lumped=False):
    rule = llf._lib.builtin_rule(mesh.family, mesh.order)
    dim = mesh.dim
    if op == "stiffness":
        return orc.assemble(orc.ELASTIC, ptype, dim, dim, mesh.xyz, mesh.conn, rule, [mat.E, mat.nu], thickness)
    if op == "mass":
        return orc.assemble(orc.MASS, ptype, dim, dim, mesh.xyz, mesh.conn, rule, [mat.rho], thickness, lumped)
    if op == "heat":
        return orc.assemble(orc.HEAT, ptype, dim, 1, mesh.xyz, mesh.conn, rule, [mat.k], thickness)
    raise ValueError(op)


def assert_csc_identical(got, ref, what=""):
    gc, gr, gv = got
    rc, rr, rv = ref
    assert len(gc) == len(rc), f"{what}: n differs"
    assert np.array_equal(gc, rc), f"{what}: colptr differs"
    assert np.array_equal(gr, rr), f"{what}: rowval differs"
    if not np.array_equal(gv, rv):
        d = np.abs(gv - rv).max() / max(np.abs(rv).max(), 1e-300)
        raise AssertionError(f"{what}: nzval not bit-identical (max rel diff {d:.3e})")


def benchmark_msh_mesh(llf):
    """The reference's elasticity_benchmark.msh (unit cube, 30^3 hex8, MSH node
    numbering and element order), rebuilt bit for bit from the committed
    fixture tests/golden/elasticity_benchmark_msh.npz, and made current."""
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    if here not in sys.path:
        sys.path.insert(0, here)
    from make_msh_fixture import FACES, decode
    xyz, conn, faces = decode()
    groups = {}
    for name in FACES:
        c = faces[name]
        groups[name] = llf.Group(name, 2, np.unique(c), llf.QUAD, 1, c)
    groups["body"] = llf.Group("body", 3, np.arange(1, xyz.shape[0] + 1, dtype=np.int64), llf.HEX, 1, conn,
                               np.arange(conn.shape[0]))
    return llf.set_current(llf.Mesh(3, llf.HEX, 1, xyz, conn, groups, name="elasticity_benchmark.msh"))
