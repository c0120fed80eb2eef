"""Python access to the CPU oracle (llfem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.  The
product (lowlevelfem.jl_gb300) never imports it.

``build()`` compiles the restatement with OpenMP and without floating-point
contraction (-ffp-contract=off): the arithmetic contract it shares with the
CUDA kernels names every fused multiply-add explicitly.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "llfem_oracle.c")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libllfem_oracle.so")

ELASTIC, HEAT, MASS = 0, 1, 2

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
                           "-ffp-contract=off", "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
        Pd, Pi32, Pi64, Pu8 = (C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                               C.POINTER(C.c_uint8))
        L.orc_pattern.restype = vp
        L.orc_pattern.argtypes = [i64, i64, i32, Pi32, Pi32, i32]
        L.orc_assemble.restype = vp
        L.orc_assemble.argtypes = [i32, i32, i32, i32, i64, Pd, i64, i32, Pi32, Pi32, i32, Pd, Pd, Pd,
                                   Pd, i32, dbl, i32, Pd, C.POINTER(i32)]
        L.orc_assemble_csc_threaded.restype = dbl
        L.orc_assemble_csc_threaded.argtypes = [i32, i32, i32, i32, Pd, i64, i32, Pi32, i32, Pd, Pd,
                                                Pd, Pd, dbl, vp, i32, i32, Pd]
        L.orc_assemble_bdb_threaded.restype = dbl
        L.orc_assemble_bdb_threaded.argtypes = [i32, i32, Pd, i64, i32, Pi32, i32, Pd, Pd, dbl, dbl, dbl, vp,
                                                i32, i32]
        L.orc_free.argtypes = [vp]
        L.orc_n.restype = i64
        L.orc_n.argtypes = [vp]
        L.orc_nnz.restype = i64
        L.orc_nnz.argtypes = [vp]
        L.orc_export.argtypes = [vp, Pi64, Pi64, Pd]
        L.orc_element_matrix.restype = i32
        L.orc_element_matrix.argtypes = [i32, i32, i32, i32, i32, Pd, Pd, Pd, Pd, dbl, dbl, Pd]
        L.orc_cg.restype = i64
        L.orc_cg.argtypes = [vp, Pd, Pd, Pu8, i32, dbl, i64, Pd]
        L.orc_spmv.argtypes = [vp, Pd, Pd]
        L.orc_lame.argtypes = [i32, dbl, dbl, dbl, Pd, Pd]
        L.orc_load_vector.argtypes = [i32, i32, Pd, i64, i32, Pi32, i32, Pd, Pd, Pd, Pd, Pd, dbl, Pd]
        L.orc_num_threads.restype = i32
        L.orc_support_matrix.restype = vp
        L.orc_support_matrix.argtypes = [i32, i32, i64, Pd, i64, i32, Pi32, i32, Pd, Pd, Pd, Pd, Pd, dbl]
        L.orc_assemble_ex.restype = vp
        L.orc_assemble_ex.argtypes = [i32, i32, i32, i32, i64, Pd, i64, i32, Pi32, Pi32, i32, Pd, Pd, Pd, Pd, i32,
                                      dbl, i32, Pd, Pi64, Pi64, Pd, C.POINTER(C.c_int)]
        L.orc_load_vector_follower.restype = i32
        L.orc_load_vector_follower.argtypes = [Pd, i64, i32, Pi32, i32, Pd, Pd, Pd, Pd, Pd, Pd, Pd]
        L.orc_follower_tangent.restype = vp
        L.orc_follower_tangent.argtypes = [i64, Pd, i64, i32, Pi32, i32, Pd, Pd, Pd, Pd, Pd, Pd, C.POINTER(i32)]
        L.orc_elements_to_nodes.argtypes = [i64, i64, i32, Pi32, i32, Pd, Pd]
        L.orc_grad_elementwise.restype = i32
        L.orc_grad_elementwise.argtypes = [Pd, i64, i32, Pi32, Pd, Pd, i32, Pd]
        L.orc_tl_matrix.restype = vp
        L.orc_tl_matrix.argtypes = [i32, i64, Pd, i64, i32, Pi32, i32, Pd, Pd, Pd, Pd, i32, Pd, C.POINTER(i32)]
        L.orc_tl_internal_force.restype = i32
        L.orc_tl_internal_force.argtypes = [i32, i64, Pd, i64, i32, Pi32, i32, Pd, Pd, Pd, Pd, i32, Pd, Pd]
        L.orc_law.restype = i32
        L.orc_law.argtypes = [i32, Pd, Pd, Pd, Pd]
        L.orc_ln.restype = dbl
        L.orc_ln.argtypes = [dbl]
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class CSC:
    """Oracle CSC matrix (0-based arrays kept in C memory, exported lazily)."""

    def __init__(self, h):
        self.h = h

    @property
    def n(self):
        return lib().orc_n(self.h)

    @property
    def nnz(self):
        return lib().orc_nnz(self.h)

    def arrays(self):
        n, nnz = self.n, self.nnz
        colptr = np.zeros(n + 1, dtype=np.int64)
        rowval = np.zeros(nnz, dtype=np.int64)
        nzval = np.zeros(nnz)
        lib().orc_export(self.h, _p(colptr, C.c_int64), _p(rowval, C.c_int64), _p(nzval, C.c_double))
        return colptr, rowval, nzval

    def julia(self):
        """1-based SparseMatrixCSC arrays."""
        c, r, v = self.arrays()
        return c + 1, r + 1, v

    def scipy(self):
        import scipy.sparse as sp
        c, r, v = self.arrays()
        return sp.csc_matrix((v, r, c), shape=(self.n, self.n))

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        lib().orc_spmv(self.h, _p(x, C.c_double), _p(y, C.c_double))
        return y

    def cg(self, b, x0, fixed, precond=0, reltol=1.4901161193847656e-08, maxiter=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(x0, dtype=np.float64).copy()
        fx = np.ascontiguousarray(fixed, dtype=np.uint8)
        rr = C.c_double(0.0)
        it = lib().orc_cg(self.h, _p(b, C.c_double), _p(x, C.c_double), _p(fx, C.c_uint8), precond,
                          reltol, self.n if maxiter is None else int(maxiter), C.byref(rr))
        return x, it, rr.value

    def __del__(self):
        try:
            if self.h:
                lib().orc_free(self.h)
        except Exception:
            pass


def _conn0(conn):
    return np.ascontiguousarray(np.asarray(conn) - 1, dtype=np.int32)


def pattern(non, conn, pdim, emat=None):
    conn0 = _conn0(conn)
    em = None if emat is None else np.ascontiguousarray(emat, dtype=np.int32)
    h = lib().orc_pattern(non, conn0.shape[0], conn0.shape[1], _p(conn0, C.c_int32), _p(em, C.c_int32), pdim)
    return CSC(h)


PT_LAME = -1   # DSL forms: params are the coefficients themselves (lambda, mu / k / c), b = 1


def assemble(kind, ptype, dim, pdim, xyz, conn, rule, params, thickness=1.0, lumped=False, emat=None, affine=True,
             init=None):
    """Reference-order COO assembly + sparse + dropzeros! (see llfem_oracle.c).
    init: (colptr, rowval, nzval) 0-based arrays of a matrix with the full
    structural pattern, whose values the assembly adds into (no dropzeros!)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn0 = _conn0(conn)
    params = np.ascontiguousarray(params, dtype=np.float64).ravel()
    em = None if emat is None else np.ascontiguousarray(emat, dtype=np.int32)
    w = np.ascontiguousarray(rule["w"], dtype=np.float64)
    N = np.ascontiguousarray(rule["N"], dtype=np.float64)
    dN = np.ascontiguousarray(rule["dN"], dtype=np.float64)
    err = C.c_int(0)
    nmat = 1
    nref = None if rule.get("node_ref") is None or not affine else np.ascontiguousarray(rule["node_ref"], dtype=np.float64)
    icp = irv = inz = None
    if init is not None:
        icp, irv, inz = (np.ascontiguousarray(a, dtype=t) for a, t in zip(init, (np.int64, np.int64, np.float64)))
    h = lib().orc_assemble_ex(kind, ptype, dim, pdim, xyz.shape[0], _p(xyz, C.c_double), conn0.shape[0],
                              conn0.shape[1], _p(conn0, C.c_int32), _p(em, C.c_int32), len(w),
                              _p(w, C.c_double), _p(N, C.c_double), _p(dN, C.c_double),
                              _p(params, C.c_double), nmat, float(thickness), int(lumped), _p(nref, C.c_double),
                              _p(icp, C.c_int64), _p(irv, C.c_int64), _p(inz, C.c_double), C.byref(err))
    if not h:
        raise ValueError("oracle: non-positive Jacobian determinant")
    return CSC(h)


def assemble_threaded(kind, ptype, dim, pdim, xyz, conn, rule, params, pat: CSC, thickness=1.0,
                      nthreads=None, chunk=256, affine=True):
    """Timed CPU baseline: threaded direct-CSC assembly into `pat` (overwritten).
    Returns seconds."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn0 = _conn0(conn)
    params = np.ascontiguousarray(params, dtype=np.float64).ravel()
    w = np.ascontiguousarray(rule["w"], dtype=np.float64)
    N = np.ascontiguousarray(rule["N"], dtype=np.float64)
    dN = np.ascontiguousarray(rule["dN"], dtype=np.float64)
    T = nthreads or lib().orc_num_threads()
    return lib().orc_assemble_csc_threaded(kind, ptype, dim, pdim, _p(xyz, C.c_double), conn0.shape[0],
                                           conn0.shape[1], _p(conn0, C.c_int32), len(w), _p(w, C.c_double),
                                           _p(N, C.c_double), _p(dN, C.c_double), _p(params, C.c_double),
                                           float(thickness), pat.h, T, chunk,
                                           _p(np.ascontiguousarray(rule["node_ref"], dtype=np.float64), C.c_double)
                                           if affine else None)


def assemble_bdb_threaded(ptype, dim, xyz, conn, rule, E, nu, pat: CSC, thickness=1.0, nthreads=None,
                          chunk=64):
    """CPU baseline: the reference's per-point B^T D B element arithmetic
    (src/linear.jl:190-330) with the threaded direct-CSC scatter of
    src/multifield.jl:2394-2499, into `pat` (overwritten).  Returns seconds."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn0 = _conn0(conn)
    w = np.ascontiguousarray(rule["w"], dtype=np.float64)
    dN = np.ascontiguousarray(rule["dN"], dtype=np.float64)
    T = nthreads or lib().orc_num_threads()
    return lib().orc_assemble_bdb_threaded(ptype, dim, _p(xyz, C.c_double), conn0.shape[0], conn0.shape[1],
                                           _p(conn0, C.c_int32), len(w), _p(w, C.c_double), _p(dN, C.c_double),
                                           float(E), float(nu), float(thickness), pat.h, T, chunk)


def element_matrix(kind, dim, pdim, X, rule, c1, c2=0.0):
    X = np.ascontiguousarray(X, dtype=np.float64)
    npe = X.shape[0]
    nd = pdim * npe
    Ke = np.zeros((nd, nd))
    w = np.ascontiguousarray(rule["w"]); N = np.ascontiguousarray(rule["N"]); dN = np.ascontiguousarray(rule["dN"])
    rc = lib().orc_element_matrix(kind, dim, pdim, npe, len(w), _p(w, C.c_double), _p(N, C.c_double),
                                  _p(dN, C.c_double), _p(X, C.c_double), c1, c2, _p(Ke, C.c_double))
    if rc:
        raise ValueError("oracle: non-positive Jacobian determinant")
    return Ke


def lame(ptype, E, nu, thickness=1.0):
    a, b = C.c_double(), C.c_double()
    lib().orc_lame(ptype, E, nu, thickness, C.byref(a), C.byref(b))
    return a.value, b.value


def load_vector(problem_dim, pdim, xyz, connb, rule, t=None, tn=None, thickness=1.0, f=None):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    cb = _conn0(connb)
    ndof = pdim * xyz.shape[0]
    f = np.zeros(ndof) if f is None else np.ascontiguousarray(f, dtype=np.float64)
    t = None if t is None else np.ascontiguousarray(t, dtype=np.float64)
    tn = None if tn is None else np.ascontiguousarray(tn, dtype=np.float64)
    w = np.ascontiguousarray(rule["w"]); N = np.ascontiguousarray(rule["N"]); dN = np.ascontiguousarray(rule["dN"])
    lib().orc_load_vector(problem_dim, pdim, _p(xyz, C.c_double), cb.shape[0], cb.shape[1], _p(cb, C.c_int32),
                          len(w), _p(w, C.c_double), _p(N, C.c_double), _p(dN, C.c_double), _p(t, C.c_double),
                          _p(tn, C.c_double), float(thickness), _p(f, C.c_double))
    return f


def _face_traction(cb, t, tn):
    """(per-element constants, element-node values) of a face traction: t is
    3 constants or a (nel, 3) array; tn (replaces t) nodal values (non, 3)."""
    nel, npe = cb.shape
    if tn is not None:
        tn = np.asarray(tn, dtype=np.float64).reshape(-1, 3)
        return None, np.ascontiguousarray(tn[cb.astype(np.int64)].reshape(nel, npe, 3))
    t = np.asarray(t, dtype=np.float64)
    return np.ascontiguousarray(np.broadcast_to(t.reshape(-1, 3) if t.ndim == 2 else t[:3], (nel, 3))), None


def load_vector_follower(xyz, connb, rule, Fn, t=None, tn=None, f=None):
    """Follower traction F t on 3D boundary faces, F nodal (non, 9)
    column-major.  Returns (f, status)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    cb = _conn0(connb)
    f = np.zeros(3 * xyz.shape[0]) if f is None else np.ascontiguousarray(f, dtype=np.float64)
    Fn = np.ascontiguousarray(Fn, dtype=np.float64)
    te, ten = _face_traction(cb, t, tn)
    w = np.ascontiguousarray(rule["w"]); N = np.ascontiguousarray(rule["N"]); dN = np.ascontiguousarray(rule["dN"])
    rc = lib().orc_load_vector_follower(_p(xyz, C.c_double), cb.shape[0], cb.shape[1], _p(cb, C.c_int32), len(w),
                                        _p(w, C.c_double), _p(N, C.c_double), _p(dN, C.c_double),
                                        _p(Fn, C.c_double), _p(te, C.c_double), _p(ten, C.c_double),
                                        _p(f, C.c_double))
    return f, rc


def follower_tangent(xyz, connb, rule, Fn, t=None, tn=None):
    """externalTangentFollower over 3D boundary faces; returns (CSC, status)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    cb = _conn0(connb)
    Fn = np.ascontiguousarray(Fn, dtype=np.float64)
    te, ten = _face_traction(cb, t, tn)
    w = np.ascontiguousarray(rule["w"]); N = np.ascontiguousarray(rule["N"]); dN = np.ascontiguousarray(rule["dN"])
    st = C.c_int32(0)
    h = lib().orc_follower_tangent(xyz.shape[0], _p(xyz, C.c_double), cb.shape[0], cb.shape[1], _p(cb, C.c_int32),
                                   len(w), _p(w, C.c_double), _p(N, C.c_double), _p(dN, C.c_double),
                                   _p(Fn, C.c_double), _p(te, C.c_double), _p(ten, C.c_double), C.byref(st))
    return CSC(h), st.value


def elements_to_nodes(non, conn, ev, ncomp):
    """elementsToNodes: ev (nel, npe*ncomp) -> nodal (non, ncomp)."""
    c0 = _conn0(conn)
    ev = np.ascontiguousarray(ev, dtype=np.float64)
    out = np.zeros((non, ncomp))
    lib().orc_elements_to_nodes(non, c0.shape[0], c0.shape[1], _p(c0, C.c_int32), ncomp, _p(ev, C.c_double),
                                _p(out, C.c_double))
    return out


def grad_elementwise(xyz, conn, rule, u, add_identity=False):
    """Elementwise nodal gradient (nel, 9*npe) of a nodal 3-vector field."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn0 = _conn0(conn)
    dNn = np.ascontiguousarray(rule["dN_nodes"], dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros((conn0.shape[0], 9 * conn0.shape[1]))
    rc = lib().orc_grad_elementwise(_p(xyz, C.c_double), conn0.shape[0], conn0.shape[1], _p(conn0, C.c_int32),
                                    _p(dNn, C.c_double), _p(u, C.c_double), int(add_identity),
                                    _p(out, C.c_double))
    if rc:
        raise ValueError("oracle: non-positive Jacobian determinant")
    return out


LAW_CONST, LAW_NEOHOOKE, LAW_SVK = 0, 1, 2
TL_KMAT, TL_KGEO_S, TL_KGEO_C = 0, 1, 2


def _prm(params):
    p = np.zeros(36)
    v = np.asarray(params, dtype=np.float64).ravel()
    p[: len(v)] = v
    return p


def tl_matrix(mode, xyz, conn, rule, Telem, law=LAW_NEOHOOKE, params=(1.0, 10.0)):
    """Total Lagrangian material (mode 0) or initial-stress (1: nodal S, 2:
    nodal C with law) stiffness in the reference's triplet order."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn0 = _conn0(conn)
    T = np.ascontiguousarray(Telem, dtype=np.float64)
    prm = _prm(params)
    w = np.ascontiguousarray(rule["w"]); N = np.ascontiguousarray(rule["N"]); dN = np.ascontiguousarray(rule["dN"])
    err = C.c_int(0)
    h = lib().orc_tl_matrix(mode, xyz.shape[0], _p(xyz, C.c_double), conn0.shape[0], conn0.shape[1],
                            _p(conn0, C.c_int32), len(w), _p(w, C.c_double), _p(N, C.c_double), _p(dN, C.c_double),
                            _p(T, C.c_double), law, _p(prm, C.c_double), C.byref(err))
    if not h:
        raise ValueError(f"oracle TL: error {err.value}")
    return CSC(h)


def tl_internal_force(mode, xyz, conn, rule, Telem, law=LAW_NEOHOOKE, params=(1.0, 10.0)):
    """mode 0: Telem = F with law; mode 1: Telem = P."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn0 = _conn0(conn)
    T = np.ascontiguousarray(Telem, dtype=np.float64)
    prm = _prm(params)
    w = np.ascontiguousarray(rule["w"]); N = np.ascontiguousarray(rule["N"]); dN = np.ascontiguousarray(rule["dN"])
    f = np.zeros(3 * xyz.shape[0])
    rc = lib().orc_tl_internal_force(mode, xyz.shape[0], _p(xyz, C.c_double), conn0.shape[0], conn0.shape[1],
                                     _p(conn0, C.c_int32), len(w), _p(w, C.c_double), _p(N, C.c_double),
                                     _p(dN, C.c_double), _p(T, C.c_double), law, _p(prm, C.c_double),
                                     _p(f, C.c_double))
    if rc:
        raise ValueError(f"oracle TL force: error {rc}")
    return f


def law(law_id, params, Cmat):
    """(S, D) of a law at the right Cauchy-Green tensor Cmat."""
    Cm = np.ascontiguousarray(Cmat, dtype=np.float64)
    S = np.zeros((3, 3)); D = np.zeros((6, 6))
    prm = _prm(params)
    rc = lib().orc_law(law_id, _p(prm, C.c_double), _p(Cm, C.c_double), _p(S, C.c_double), _p(D, C.c_double))
    if rc:
        raise ValueError("det C <= 0")
    return S, D


def ln(x: float) -> float:
    return lib().orc_ln(float(x))


def num_threads() -> int:
    return lib().orc_num_threads()


def support_matrix(problem_dim, pdim, non, xyz, bconn, rule, k, thickness=1.0, kn=None):
    """elasticSupportMatrix / heatConvectionMatrix over the boundary elements
    bconn (1-based node tags of the volume mesh, all groups in group order).
    k: pdim constants for every element, or a (nel, pdim) array of
    per-element constants; kn (optional, replaces k): nodal values
    kn[non*pdim], taken at every element's nodes and interpolated."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    c0 = _conn0(bconn)
    nel, npe = c0.shape
    k = np.asarray(k, dtype=np.float64)
    ke = np.ascontiguousarray(np.broadcast_to(k.reshape(-1, pdim) if k.ndim == 2 else k[:pdim], (nel, pdim)))
    ken = None
    if kn is not None:
        kn = np.asarray(kn, dtype=np.float64).reshape(-1, pdim)
        ken = np.ascontiguousarray(kn[c0.astype(np.int64)].reshape(nel, npe, pdim))
    w = np.ascontiguousarray(rule["w"], dtype=np.float64)
    N = np.ascontiguousarray(rule["N"], dtype=np.float64)
    dN = np.ascontiguousarray(rule["dN"], dtype=np.float64)
    h = lib().orc_support_matrix(problem_dim, pdim, non, _p(xyz, C.c_double), nel, npe,
                                 _p(c0, C.c_int32), len(w), _p(w, C.c_double), _p(N, C.c_double),
                                 _p(dN, C.c_double), _p(ke, C.c_double), _p(ken, C.c_double), float(thickness))
    return CSC(h)


def fdm(K, C, q, fixed, T, dt, theta):
    """FDM (src/heat.jl:1466-1616) restated with scipy: K, C scipy sparse (C
    may be diagonal), q (ndof, 1 or n), fixed bool mask, T (n, ndof) with row
    0 the initial state and the fixed entries of every row prescribed; fills
    the free entries of rows 1.. .  Explicit branch when theta == 0 and
    C_ff is diagonal, else one LU of C_ff + theta dt K_ff."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = T.shape[0]
    free = np.flatnonzero(~fixed)
    fix = np.flatnonzero(fixed)
    K = sp.csc_matrix(K)
    C = sp.csc_matrix(C)
    Kff, Cff = K[free][:, free], C[free][:, free]
    Kfc, Cfc = K[free][:, fix], C[free][:, fix]
    q = np.asarray(q).reshape(K.shape[0], -1)
    qf = lambda i: q[free, 0 if q.shape[1] == 1 else i]
    d = Cff.diagonal()
    if not np.all(d > 0):
        raise ValueError("FDM: non-positive diagonal entry detected in Cff on free DOFs.")
    T0 = T[0, free].copy()
    if theta == 0 and (Cff - sp.diags(d)).count_nonzero() == 0:
        invd = 1.0 / d
        for i in range(1, n):
            Tc_n, Tc_np1 = T[i - 1, fix], T[i, fix]
            r = qf(i - 1) - Kff @ T0 - Kfc @ Tc_n
            T1 = T0 + invd * (dt * r - Cfc @ (Tc_np1 - Tc_n))
            T[i, free] = T1
            T0 = T1
        return T
    A = (Cff + theta * dt * Kff).tocsc()
    B = Cff - (1 - theta) * dt * Kff
    Afc = Cfc + theta * dt * Kfc
    Bfc = Cfc - (1 - theta) * dt * Kfc
    lu = spla.splu(A)
    for i in range(1, n):
        Tc_n, Tc_np1 = T[i - 1, fix], T[i, fix]
        qth = qf(0) if q.shape[1] == 1 else (1 - theta) * qf(i - 1) + theta * qf(i)
        rhs = B @ T0 + dt * qth - Afc @ Tc_np1 + Bfc @ Tc_n
        T1 = lu.solve(rhs)
        T[i, free] = T1
        T0 = T1
    return T
