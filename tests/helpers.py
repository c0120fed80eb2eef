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
