"""ctypes binding of libllfem_gb300.so (the C-ABI of include/llfem_gb300.h).

The shared library is built in-tree by ``build.build_library()``.  Nothing in
this package computes on the host what the library computes on the GPU: when
the library or a CUDA device is missing, every compute call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libllfem_gb300.so")

LLF_OK = 0
ERRORS = {
    -1: "LLF_ERR_ARG", -2: "LLF_ERR_CUDA", -3: "LLF_ERR_MESH",
    -4: "LLF_ERR_NOT_CONVERGED", -5: "LLF_ERR_STATE", -6: "LLF_ERR_UNSUPPORTED",
    -7: "LLF_ERR_LIMIT", -8: "LLF_ERR_NUMERIC",
}

LINE, TRI, QUAD, TET, HEX = 1, 2, 3, 4, 5
SOLID, PLANE_STRESS, PLANE_STRAIN, HEAT_CONDUCTION, PLANE_HEAT_CONDUCTION = 0, 1, 2, 3, 4
FP64, FP32Q = 0, 1
FORM_SYMGRAD, FORM_GRAD, FORM_ID = 0, 1, 2
LAW_CONSTANT_C, LAW_NEOHOOKE_COMP, LAW_SVK = 0, 1, 2
PRECOND_NONE, PRECOND_JACOBI, PRECOND_BJACOBI, PRECOND_IC0 = 0, 1, 2, 3


class LLFError(RuntimeError):
    """Error raised for a negative status of the C-ABI (the Julia shim raises
    ``error(msg)`` with the same text)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


vp = C.c_void_p
i32, i64, dbl = C.c_int, C.c_int64, C.c_double
P_i64 = C.POINTER(C.c_int64)
P_i32 = C.POINTER(C.c_int32)
P_dbl = C.POINTER(C.c_double)
P_u8 = C.POINTER(C.c_uint8)
PP = C.POINTER(C.c_void_p)

SIGNATURES = {
    "llf_version": (C.c_char_p, []),
    "llf_ctx_create": (i32, [i32, PP]),
    "llf_ctx_destroy": (i32, [vp]),
    "llf_last_error": (C.c_char_p, [vp]),
    "llf_ctx_sync": (i32, [vp]),
    "llf_ctx_stream": (i32, [vp, PP]),
    "llf_builtin_rule": (i32, [i32, i32, C.POINTER(i32), C.POINTER(i32), P_dbl, P_dbl, P_dbl, P_dbl, P_dbl]),
    "llf_builtin_node_gradients": (i32, [i32, i32, P_dbl]),
    "llf_profile_enable": (i32, [vp, i32]),
    "llf_profile_reset": (i32, [vp]),
    "llf_profile_report": (i32, [vp, C.c_char_p, i64, P_i64]),
    "llf_launch_count": (i32, [vp, P_i64]),
    "llf_alloc_count": (i32, [vp, P_i64]),
    "llf_mesh_upload": (i32, [vp, i32, i64, P_dbl, i64, i32, P_i64, i32, i32, PP]),
    "llf_mesh_update": (i32, [vp, vp, P_dbl, P_i64]),
    "llf_mesh_set_materials": (i32, [vp, vp, P_i32]),
    "llf_tables_upload": (i32, [vp, vp, i32, P_dbl, P_dbl, P_dbl]),
    "llf_mesh_destroy": (i32, [vp, vp]),
    "llf_pattern_build": (i32, [vp, vp, i32, P_i64, PP]),
    "llf_pattern_copy": (i32, [vp, vp, P_i64, P_i64]),
    "llf_pattern_info": (i32, [vp, P_i64, P_i64, C.POINTER(i32)]),
    "llf_pattern_destroy": (i32, [vp, vp]),
    "llf_autotune_stiffness": (i32, [vp, vp, vp, i32, P_dbl, P_dbl, i32, dbl, i32, i32, C.c_char_p, i64, P_i64]),
    "llf_assemble_stiffness_values": (i32, [vp, vp, vp, i32, P_dbl, P_dbl, i32, dbl, i32, i64, P_i64, P_dbl,
                                            C.POINTER(C.c_uint32), P_i64, C.POINTER(i32)]),
    "llf_rowval_from_keep": (i64, [i64, P_i64, C.POINTER(C.c_uint32), P_i64]),
    "llf_assemble_stiffness": (i32, [vp, vp, vp, i32, P_dbl, P_dbl, i32, dbl, i32, PP]),
    "llf_assemble_mass": (i32, [vp, vp, vp, i32, P_dbl, i32, dbl, i32, i32, PP]),
    "llf_assemble_heat": (i32, [vp, vp, vp, i32, P_dbl, i32, dbl, i32, PP]),
    "llf_assemble_support": (i32, [vp, vp, vp, P_dbl, P_dbl, dbl, PP]),
    "llf_heat_fdm": (i32, [vp, vp, vp, P_dbl, i32, P_dbl, P_u8, i64, dbl, dbl, i32, dbl, i64, P_i64]),
    "llf_assemble_stiffness_csc": (i32, [vp, vp, vp, i32, P_dbl, P_dbl, i32, dbl, i32, i64, P_i64, P_i64, P_dbl,
                                         P_i64]),
    "llf_assemble_form": (i32, [vp, vp, vp, i32, P_dbl, P_dbl, i32, vp, i32, PP]),
    "llf_matrix_zero_pattern": (i32, [vp, vp, PP]),
    "llf_follower_tangent": (i32, [vp, vp, vp, P_dbl, P_dbl, P_dbl, PP]),
    "llf_load_vector_follower": (i32, [vp, vp, P_dbl, P_dbl, P_dbl, P_dbl, i64]),
    "llf_elements_to_nodes": (i32, [vp, vp, i32, P_dbl, P_dbl]),
    "llf_tl_material_tangent": (i32, [vp, vp, vp, P_dbl, i32, P_dbl, i32, PP]),
    "llf_tl_tangent": (i32, [vp, vp, vp, P_dbl, i32, P_dbl, i32, PP]),
    "llf_tl_tangent_form": (i32, [vp, vp, vp, P_dbl, i32, P_dbl, i32, i32, PP]),
    "llf_tl_initial_stress": (i32, [vp, vp, vp, P_dbl, P_dbl, i32, P_dbl, i32, PP]),
    "llf_tl_internal_force": (i32, [vp, vp, P_dbl, P_dbl, i32, P_dbl, i32, P_dbl]),
    "llf_grad_elementwise": (i32, [vp, vp, P_dbl, i32, P_dbl]),
    "llf_load_vector": (i32, [vp, vp, i32, i32, P_dbl, P_dbl, dbl, P_dbl, i64]),
    "llf_matrix_nnz": (i32, [vp, vp, P_i64]),
    "llf_matrix_copy_csc": (i32, [vp, vp, P_i64, P_i64, P_dbl]),
    "llf_matrix_copy_structural": (i32, [vp, vp, P_dbl]),
    "llf_matrix_prepare": (i32, [vp, vp]),
    "llf_matrix_axpby": (i32, [vp, dbl, vp, dbl, vp, PP]),
    "llf_matrix_from_structural": (i32, [vp, vp, P_dbl, PP]),
    "llf_matrix_spmv": (i32, [vp, vp, P_dbl, P_dbl]),
    "llf_matrix_destroy": (i32, [vp, vp]),
    "llf_pcg": (i32, [vp, vp, P_dbl, P_dbl, P_u8, i32, dbl, i64, P_i64, P_dbl]),
    "llf_pcg_batched": (i32, [vp, vp, P_dbl, P_dbl, P_u8, i32, P_i64, i32, dbl, i64, P_i64, P_dbl]),
    "llf_pcg_mixed": (i32, [vp, vp, P_dbl, P_dbl, P_u8, i32, P_i64, i32, dbl, i64, P_i64, P_dbl]),
    "llf_pcg_noalloc": (i32, [vp, vp, vp, vp, vp, i32, dbl, i64, P_i64, P_dbl]),
    "llf_server_create": (i32, [i32, i32, i64, PP]),
    "llf_server_create_batched": (i32, [i32, i32, i32, i64, PP]),
    "llf_server_timing": (i32, [vp, P_dbl, P_dbl, P_dbl, P_dbl, P_i64, P_dbl]),
    "llf_server_submit_heat": (i32, [vp, i32, i64, P_dbl, i64, i32, P_i64, i32, i32, dbl, dbl, P_dbl, P_dbl, P_u8,
                                     i32, dbl, i64, P_i64]),
    "llf_server_wait": (i32, [vp, i64, dbl, P_dbl, P_i64, P_dbl, P_dbl, P_dbl, C.c_char_p, i64]),
    "llf_server_stats": (i32, [vp, P_i64, P_i64, P_i64, P_i64]),
    "llf_server_destroy": (i32, [vp]),
}

_lib = None


def lib():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} is not built; run __graft_entry__.build()")
        L = C.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def i64a(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int64)


def builtin_rule(family: int, order: int) -> dict:
    """Built-in quadrature + Lagrange tables (host-only call)."""
    L = lib()
    nip, npe = C.c_int(0), C.c_int(0)
    rc = L.llf_builtin_rule(family, order, C.byref(nip), C.byref(npe), None, None, None, None, None)
    if rc != LLF_OK:
        raise LLFError(rc, f"no built-in rule for family {family} order {order}")
    q, n = nip.value, npe.value
    xi = np.zeros((q, 3)); w = np.zeros(q); N = np.zeros((q, n)); dN = np.zeros((q, n, 3))
    ref = np.zeros((n, 3))
    rc = L.llf_builtin_rule(family, order, None, None, ptr(xi, C.c_double), ptr(w, C.c_double),
                            ptr(N, C.c_double), ptr(dN, C.c_double), ptr(ref, C.c_double))
    if rc != LLF_OK:
        raise LLFError(rc, "llf_builtin_rule")
    dNn = np.zeros((n, n, 3))
    rc = L.llf_builtin_node_gradients(family, order, ptr(dNn, C.c_double))
    if rc != LLF_OK:
        raise LLFError(rc, "llf_builtin_node_gradients")
    return {"nip": q, "npe": n, "xi": xi, "w": w, "N": N, "dN": dN, "node_ref": ref, "dN_nodes": dNn}


class Context:
    """One CUDA device + stream of the library (llf_ctx)."""

    def __init__(self, device: int = 0):
        L = lib()
        h = C.c_void_p()
        rc = L.llf_ctx_create(device, C.byref(h))
        if rc != LLF_OK:
            raise LLFError(rc, f"llf_ctx_create(device={device}) failed: no usable CUDA device")
        self.h = h
        self.device = device

    def check(self, rc: int, what: str = ""):
        if rc != LLF_OK:
            msg = lib().llf_last_error(self.h).decode()
            raise LLFError(rc, msg or what)

    def sync(self):
        self.check(lib().llf_ctx_sync(self.h), "sync")

    def stream_handle(self) -> int:
        s = C.c_void_p()
        self.check(lib().llf_ctx_stream(self.h, C.byref(s)))
        return s.value or 0

    def profile(self, on: bool = True):
        self.check(lib().llf_profile_enable(self.h, int(on)))

    def profile_reset(self):
        self.check(lib().llf_profile_reset(self.h))

    def profile_report(self) -> dict:
        import json
        need = C.c_int64(0)
        self.check(lib().llf_profile_report(self.h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value + 1)
        self.check(lib().llf_profile_report(self.h, buf, need.value + 1, C.byref(need)))
        return json.loads(buf.value.decode())

    def launches(self) -> int:
        n = C.c_int64(0)
        self.check(lib().llf_launch_count(self.h, C.byref(n)))
        return n.value

    def allocs(self) -> int:
        """Device allocations the context has made so far."""
        n = C.c_int64(0)
        self.check(lib().llf_alloc_count(self.h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "h", None):
            lib().llf_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request server of the library (llf_server): worker threads with their
    own streams, admission by device-memory budget."""

    def __init__(self, device: int = 0, workers: int = 4, budget_bytes: int = 64 << 30, batched: bool = False,
                 max_systems: int = 256):
        """batched=True: continuous batching (llf_server_create_batched), with
        `workers` preparation threads and one engine iterating every prepared
        request in shared launches; otherwise a pool of `workers` solvers."""
        h = C.c_void_p()
        if batched:
            rc = lib().llf_server_create_batched(device, workers, int(max_systems), int(budget_bytes), C.byref(h))
        else:
            rc = lib().llf_server_create(device, workers, int(budget_bytes), C.byref(h))
        if rc != LLF_OK:
            raise LLFError(rc, "llf_server_create failed")
        self.h = h
        self._non = {}

    def submit_heat(self, dim, xyz, conn, family, order, k, x0, fixed, rhs=None, thickness=1.0,
                    precond=PRECOND_JACOBI, reltol=1e-10, maxiter=0) -> int:
        xyz, conn, x0 = f64(xyz), i64a(conn), f64(x0)
        fx = np.ascontiguousarray(fixed, dtype=np.uint8)
        rhs = None if rhs is None else f64(rhs)
        t = C.c_int64(0)
        rc = lib().llf_server_submit_heat(self.h, dim, xyz.shape[0], ptr(xyz, C.c_double), conn.shape[0],
                                          conn.shape[1], ptr(conn, C.c_int64), family, order, float(k),
                                          float(thickness), ptr(rhs, C.c_double), ptr(x0, C.c_double),
                                          ptr(fx, C.c_uint8), int(precond), float(reltol), int(maxiter), C.byref(t))
        if rc != LLF_OK:
            raise LLFError(rc, "llf_server_submit_heat: bad request")
        self._non[t.value] = xyz.shape[0]
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        n = self._non.pop(ticket)
        x = np.zeros(n)
        it, rr, lat, svc = C.c_int64(0), C.c_double(0), C.c_double(0), C.c_double(0)
        err = C.create_string_buffer(512)
        rc = lib().llf_server_wait(self.h, ticket, float(timeout), ptr(x, C.c_double), C.byref(it), C.byref(rr),
                                   C.byref(lat), C.byref(svc), err, 512)
        if rc != LLF_OK:
            raise LLFError(rc, err.value.decode() or "server request failed")
        return x, it.value, rr.value, lat.value, svc.value

    def stats(self) -> dict:
        q, s, b, p = C.c_int64(0), C.c_int64(0), C.c_int64(0), C.c_int64(0)
        lib().llf_server_stats(self.h, C.byref(q), C.byref(s), C.byref(b), C.byref(p))
        return {"queued": q.value, "served": s.value, "bytes_in_use": b.value, "peak_bytes": p.value}

    def timing(self) -> dict:
        v = [C.c_double(0) for _ in range(4)]
        n, a = C.c_int64(0), C.c_double(0)
        lib().llf_server_timing(self.h, *[C.byref(x) for x in v], C.byref(n), C.byref(a))
        return {"prep_s": v[0].value, "engine_step_s": v[1].value, "engine_collect_s": v[2].value,
                "engine_idle_s": v[3].value, "replays": n.value, "mean_admitted": a.value}

    def close(self):
        if getattr(self, "h", None):
            lib().llf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("LLF_DEVICE", "0")))
    return _default_ctx


class DeviceMesh:
    """llf_mesh handle (device-resident nodes, connectivity, tables)."""

    def __init__(self, ctx: Context, dim: int, xyz: np.ndarray, conn: np.ndarray, family: int, order: int):
        self.ctx = ctx
        xyz = f64(xyz)
        conn = i64a(conn)
        self.non, self.nel = xyz.shape[0], conn.shape[0]
        self.npe = conn.shape[1] if conn.ndim == 2 else 0
        h = C.c_void_p()
        ctx.check(lib().llf_mesh_upload(ctx.h, dim, self.non, ptr(xyz, C.c_double), self.nel, self.npe,
                                        ptr(conn, C.c_int64), family, order, C.byref(h)), "mesh upload")
        self.h = h

    def set_materials(self, elem_mat: np.ndarray | None):
        em = None if elem_mat is None else np.ascontiguousarray(elem_mat, dtype=np.int32)
        self.ctx.check(lib().llf_mesh_set_materials(self.ctx.h, self.h, ptr(em, C.c_int32)))

    def set_tables(self, w, N, dN):
        w, N, dN = f64(w), None if N is None else f64(N), f64(dN)
        self.ctx.check(lib().llf_tables_upload(self.ctx.h, self.h, len(w), ptr(w, C.c_double),
                                               ptr(N, C.c_double), ptr(dN, C.c_double)))

    def update(self, xyz, conn=None):
        xyz = f64(xyz)
        conn = None if conn is None else i64a(conn)
        self.ctx.check(lib().llf_mesh_update(self.ctx.h, self.h, ptr(xyz, C.c_double), ptr(conn, C.c_int64)))

    def __del__(self):
        try:
            if self.h:
                lib().llf_mesh_destroy(self.ctx.h, self.h)
        except Exception:
            pass


class DevicePattern:
    def __init__(self, mesh: DeviceMesh, pdim: int):
        self.mesh = mesh
        self.ctx = mesh.ctx
        nnz = C.c_int64(0)
        h = C.c_void_p()
        self.ctx.check(lib().llf_pattern_build(self.ctx.h, mesh.h, pdim, C.byref(nnz), C.byref(h)),
                       "pattern build")
        self.h = h
        self.nnz = nnz.value
        self.pdim = pdim
        self.ndof = pdim * mesh.non

    def copy(self):
        colptr = np.zeros(self.ndof + 1, dtype=np.int64)
        rowval = np.zeros(self.nnz, dtype=np.int64)
        self.ctx.check(lib().llf_pattern_copy(self.ctx.h, self.h, ptr(colptr, C.c_int64), ptr(rowval, C.c_int64)))
        return colptr, rowval

    def __del__(self):
        try:
            if self.h:
                lib().llf_pattern_destroy(self.ctx.h, self.h)
        except Exception:
            pass


class DeviceMatrix:
    """llf_matrix handle: device CSC values on a pattern."""

    def __init__(self, ctx: Context, h, pattern: DevicePattern):
        self.ctx, self.h, self.pattern = ctx, h, pattern

    @property
    def n(self) -> int:
        return self.pattern.ndof

    def nnz(self) -> int:
        v = C.c_int64(0)
        self.ctx.check(lib().llf_matrix_nnz(self.ctx.h, self.h, C.byref(v)))
        return v.value

    def copy_csc(self):
        nnz = self.nnz()
        colptr = np.zeros(self.n + 1, dtype=np.int64)
        rowval = np.zeros(nnz, dtype=np.int64)
        nzval = np.zeros(nnz)
        self.ctx.check(lib().llf_matrix_copy_csc(self.ctx.h, self.h, ptr(colptr, C.c_int64),
                                                 ptr(rowval, C.c_int64), ptr(nzval, C.c_double)))
        return colptr, rowval, nzval

    def prepare(self):
        """Make the structural values resident (llf_matrix_prepare)."""
        self.ctx.check(lib().llf_matrix_prepare(self.ctx.h, self.h))

    def copy_structural(self):
        nz = np.zeros(self.pattern.nnz)
        self.ctx.check(lib().llf_matrix_copy_structural(self.ctx.h, self.h, ptr(nz, C.c_double)))
        return nz

    def axpby(self, a: float, b: float, other: "DeviceMatrix") -> "DeviceMatrix":
        h = C.c_void_p()
        self.ctx.check(lib().llf_matrix_axpby(self.ctx.h, a, self.h, b, other.h, C.byref(h)))
        return DeviceMatrix(self.ctx, h, self.pattern)

    def spmv(self, x: np.ndarray) -> np.ndarray:
        x = f64(x)
        y = np.zeros(self.n)
        self.ctx.check(lib().llf_matrix_spmv(self.ctx.h, self.h, ptr(x, C.c_double), ptr(y, C.c_double)))
        return y

    def pcg(self, b, x0, fixed, precond=PRECOND_NONE, reltol=1.4901161193847656e-08, maxiter=None,
            raise_on_fail=True):
        b, x = f64(b), f64(x0).copy()
        fx = np.ascontiguousarray(fixed, dtype=np.uint8)
        it, rr = C.c_int64(0), C.c_double(0.0)
        maxiter = self.n if maxiter is None else int(maxiter)
        rc = lib().llf_pcg(self.ctx.h, self.h, ptr(b, C.c_double), ptr(x, C.c_double), ptr(fx, C.c_uint8),
                           int(precond), float(reltol), maxiter, C.byref(it), C.byref(rr))
        if rc != LLF_OK and (raise_on_fail or rc != -4):
            self.ctx.check(rc, "pcg")
        return x, it.value, rr.value

    def pcg_batched(self, b, x0, fixed, seg_off, precond=PRECOND_NONE, reltol=1.4901161193847656e-08,
                    maxiter=None, raise_on_fail=True, mixed=False):
        """Independent CG per block-diagonal segment [seg_off[g], seg_off[g+1]);
        mixed: FP32 iterations with FP64 reliable updates (llf_pcg_mixed)."""
        b, x = f64(b), f64(x0).copy()
        fx = np.ascontiguousarray(fixed, dtype=np.uint8)
        so = i64a(seg_off)
        nseg = len(so) - 1
        its = np.zeros(nseg, dtype=np.int64)
        rr = np.zeros(nseg)
        maxiter = self.n if maxiter is None else int(maxiter)
        fn = lib().llf_pcg_mixed if mixed else lib().llf_pcg_batched
        rc = fn(self.ctx.h, self.h, ptr(b, C.c_double), ptr(x, C.c_double), ptr(fx, C.c_uint8),
                nseg, ptr(so, C.c_int64), int(precond), float(reltol), maxiter,
                ptr(its, C.c_int64), ptr(rr, C.c_double))
        if rc != LLF_OK and (raise_on_fail or rc != -4):
            self.ctx.check(rc, "pcg_batched")
        return x, its, rr

    def __del__(self):
        try:
            if self.h:
                lib().llf_matrix_destroy(self.ctx.h, self.h)
        except Exception:
            pass
