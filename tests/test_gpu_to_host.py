"""llf_assemble_stiffness_csc: stiffness straight into host CSC arrays,
column slabs copied out while the next slab is gathered; the result must
be the one of llf_assemble_stiffness + llf_matrix_copy_csc, bit for bit."""
import numpy as np
import pytest

from helpers import make_mesh

pytestmark = pytest.mark.gpu


def _to_host(llf, p, form, capacity=None):
    L = llf._lib
    ctx, dm, pat = p._ctx, p.device_mesh(), p.pattern()
    E = np.array([m.E for m in p.material])
    nu = np.array([m.nu for m in p.material])
    cap = pat.nnz if capacity is None else capacity
    colptr = np.zeros(pat.ndof + 1, dtype=np.int64)
    rowval = np.zeros(cap, dtype=np.int64)
    nzval = np.zeros(cap)
    nnz = L.C.c_int64(0)
    rc = L.lib().llf_assemble_stiffness_csc(ctx.h, dm.h, pat.h, p.ptype, L.ptr(E, L.C.c_double),
                                            L.ptr(nu, L.C.c_double), len(E), p.thickness, form, cap,
                                            L.ptr(colptr, L.C.c_int64), L.ptr(rowval, L.C.c_int64),
                                            L.ptr(nzval, L.C.c_double), L.C.byref(nnz))
    return rc, colptr, rowval[:nnz.value], nzval[:nnz.value]


@pytest.mark.parametrize("case", [("box", 3, 2, False, "Solid"), ("box", 4, 2, True, "Solid"),
                                  ("rect", 20, 1, False, "PlaneStrain"), ("rect", 1, 1, False, "PlaneStress"),
                                  ("box", 6, 1, False, "Solid"), ("box", 17, 1, False, "Solid"),
                                  ("box", 9, 2, True, "Solid")],
                         ids=["hex27", "tet10", "quad4", "one-quad", "hex8", "hex8-4913", "tet10-4374"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_to_host_equals_assemble_then_copy(llf, case, precision):
    kind, n, order, simplex, pt = case
    make_mesh(llf, kind, n, order, simplex)
    p = llf.Problem([llf.Material("body", E=2.1e5, nu=0.3)], type=pt, thickness=0.5)
    form = llf._lib.FP64 if precision == "fp64" else llf._lib.FP32Q
    for _ in range(2):   # two calls in a row on the same context
        rc, c, r, v = _to_host(llf, p, form)
        assert rc == 0, p._ctx.last_error() if hasattr(p._ctx, "last_error") else rc
        gc, gr, gv = llf.stiffnessMatrix(p, precision=precision).csc()
        assert np.array_equal(c, gc) and np.array_equal(r, gr) and np.array_equal(v, gv)


def test_to_host_capacity_is_checked(llf):
    llf.structured_box_mesh(n=2, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    rc, *_ = _to_host(llf, p, llf._lib.FP64, capacity=p.pattern().nnz - 1)
    assert rc == -1   # LLF_ERR_ARG
    rc, c, r, v = _to_host(llf, p, llf._lib.FP64)
    assert rc == 0 and len(v) == llf.stiffnessMatrix(p).nnz()


def _values(llf, p, form):
    L = llf._lib
    ctx, dm, pat = p._ctx, p.device_mesh(), p.pattern()
    E = np.array([m.E for m in p.material])
    nu = np.array([m.nu for m in p.material])
    colptr = np.zeros(pat.ndof + 1, dtype=np.int64)
    nzval = np.zeros(pat.nnz)
    keep = np.zeros((pat.nnz + 31) // 32, dtype=np.uint32)
    nnz = L.C.c_int64(0)
    changed = L.C.c_int(-1)
    rc = L.lib().llf_assemble_stiffness_values(ctx.h, dm.h, pat.h, p.ptype, L.ptr(E, L.C.c_double),
                                               L.ptr(nu, L.C.c_double), len(E), p.thickness, form, pat.nnz,
                                               L.ptr(colptr, L.C.c_int64), L.ptr(nzval, L.C.c_double),
                                               L.ptr(keep, L.C.c_uint32), L.C.byref(nnz), L.C.byref(changed))
    return rc, colptr, nzval[:nnz.value], keep, changed.value


@pytest.mark.parametrize("case", [("box", 3, 2, False, "Solid"), ("box", 4, 2, True, "Solid"),
                                  ("rect", 20, 1, False, "PlaneStrain"), ("box", 17, 1, False, "Solid")],
                         ids=["hex27", "tet10", "quad4", "hex8-4913"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_values_and_keep_bits_give_the_csc(llf, case, precision):
    """llf_assemble_stiffness_values: colptr and nzval of the stored CSC plus
    one bit per structural entry; the structural rowval (llf_pattern_copy)
    filtered by the bits (llf_rowval_from_keep) is the stored rowval."""
    L = llf._lib
    kind, n, order, simplex, pt = case
    make_mesh(llf, kind, n, order, simplex)
    p = llf.Problem([llf.Material("body", E=2.1e5, nu=0.3)], type=pt, thickness=0.5)
    form = L.FP64 if precision == "fp64" else L.FP32Q
    sc, sr = p.pattern().copy()
    for call in range(2):
        rc, c, v, keep, changed = _values(llf, p, form)
        assert rc == 0
        assert changed == (1 if call == 0 else 0)   # the second call's bits equal the first's
        gc, gr, gv = llf.stiffnessMatrix(p, precision=precision).csc()
        assert np.array_equal(c, gc) and np.array_equal(v, gv)
        rows = np.zeros(len(sr), dtype=np.int64)
        got = L.lib().llf_rowval_from_keep(len(sr), L.ptr(sr, L.C.c_int64), L.ptr(keep, L.C.c_uint32),
                                           L.ptr(rows, L.C.c_int64))
        assert got == len(gv) and np.array_equal(rows[:got], gr)
        assert int(np.unpackbits(keep.view(np.uint8)).sum()) == len(gv)
