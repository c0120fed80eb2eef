"""Weak-form DSL bilinear terms on the assembly kernels — the reference's
second public assembly surface (src/multifield.jl:4385-4931 for the
operators and the ⋅ chain, :5280-5346 for ∫).  Python has no ⋅ or ∫, so the
chain is written with @ and the integral is `integrate`:

    K = integrate(SymGrad(P) @ D @ SymGrad(P))           # ∫(SymGrad(P)⋅D⋅SymGrad(P))
    K = integrate(Grad(P) @ k @ Grad(P), csc_matrix=Kp)  # adds into Kp, keeps its pattern
    M = integrate(Id(P) @ rho @ Id(P))

Three forms run on the GPU: SymGrad⋅D⋅SymGrad with an isotropic D (the
elastic kernel with the Lamé constants read off D), Grad⋅k⋅Grad of a scalar
field (the conduction kernel) and Id⋅c⋅Id (the mass kernel), each with a
constant coefficient and b = 1.  Other operator pairs, field-valued
coefficients, sub-domains and weights raise NotImplementedError."""
from __future__ import annotations

from functools import reduce

import numpy as np

from . import _lib
from .api import Problem, SystemMatrix, _form


class OpApplied:
    """An operator applied to a field (OpApplied, src/multifield.jl:4385)."""

    def __init__(self, P: Problem, op: str):
        self.P, self.op = P, op

    def __matmul__(self, other):
        if isinstance(other, OpApplied):
            return BilinearTerm(self, 1.0, other)
        return MatrixChain(self, [other])

    def __repr__(self):
        return f"{self.op}({self.P.type})"


class MatrixChain:
    """Operator followed by coefficients (MatrixChain, src/multifield.jl:4814)."""

    def __init__(self, a: OpApplied, mats: list):
        self.a, self.mats = a, mats

    def __matmul__(self, other):
        if isinstance(other, OpApplied):
            return BilinearTerm(self.a, self.mats, other)
        return MatrixChain(self.a, self.mats + [other])


class BilinearTerm:
    """∫ a(v)ᵀ coef b(u) (BilinearTerm, src/multifield.jl:4672)."""

    def __init__(self, a: OpApplied, coef, b: OpApplied):
        self.a, self.coef, self.b = a, coef, b


def Grad(P: Problem) -> OpApplied:
    return OpApplied(P, "Grad")


def SymGrad(P: Problem) -> OpApplied:
    """Engineering-strain symmetric gradient: rows (xx, yy, zz, xy, xz, yz)
    in 3D, (xx, yy, xy) in 2D (src/multifield.jl:607-660)."""
    return OpApplied(P, "SymGrad")


def Id(P: Problem) -> OpApplied:
    return OpApplied(P, "Id")


def _coefficient(coef):
    """Collapse a coefficient chain (numbers and matrices, left to right)."""
    items = coef if isinstance(coef, list) else [coef]
    for c in items:
        if not (np.isscalar(c) or isinstance(c, np.ndarray) or isinstance(c, (list, tuple))):
            raise NotImplementedError(f"∫: coefficient of type {type(c).__name__} is not accelerated")
    items = [float(c) if np.isscalar(c) else np.asarray(c, dtype=np.float64) for c in items]
    return reduce(lambda x, y: x * y if np.isscalar(x) or np.isscalar(y) else x @ y, items)


def _isotropic(D: np.ndarray, dim: int):
    """(lambda, mu) of an isotropic Voigt matrix with engineering shear, or None."""
    n = 6 if dim == 3 else 3
    if D.shape != (n, n):
        return None
    lam, mu = D[0, 1], D[n - 1, n - 1]
    ref = np.zeros((n, n))
    ref[:dim, :dim] = lam
    ref[np.arange(dim), np.arange(dim)] = lam + 2.0 * mu
    ref[np.arange(dim, n), np.arange(dim, n)] = mu
    if np.abs(D - ref).max() > 1e-12 * max(np.abs(D).max(), 1e-300):
        return None
    return float(lam), float(mu)


def build_csc_pattern(P: Problem) -> SystemMatrix:
    """Structural zeros on the problem's pattern, keeping every entry
    (build_csc_pattern, src/multifield.jl:2083-2250): the csc_matrix of ∫."""
    ctx, pat = P._ctx, P.pattern()
    h = _lib.C.c_void_p()
    ctx.check(_lib.lib().llf_matrix_zero_pattern(ctx.h, pat.h, _lib.C.byref(h)), "build_csc_pattern")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), P)


def integrate(term: BilinearTerm, Omega=None, Gamma=None, weight=None, gauss="full", threads="auto",
              assembly="csc", csc_matrix: SystemMatrix | None = None, element_chunk_size="auto",
              precision="fp64") -> SystemMatrix:
    """∫(term; Ω, Γ, weight, gauss, threads, assembly, csc_matrix,
    element_chunk_size) (src/multifield.jl:5280-5346).  Without csc_matrix
    the result has dropzeros! applied; with it the values are added into
    csc_matrix in element order, its full pattern is kept, and csc_matrix
    (updated in place, as the reference updates K.nzval) is returned.
    `threads` and `element_chunk_size` are accepted for signature
    compatibility; the GPU path has no thread switch."""
    if assembly not in ("csc", "ijv"):
        raise ValueError(f"Unsupported matrix assembly mode {assembly}. Expected :csc or :ijv.")
    if assembly == "ijv" and csc_matrix is not None:
        raise ValueError("csc_matrix is only valid with assembly=:csc.")
    if not isinstance(term, BilinearTerm):
        raise NotImplementedError("∫: only bilinear terms are accelerated")
    P = term.a.P
    if term.b.P is not P:
        raise NotImplementedError("∫: multi-field (mixed) bilinear terms are not accelerated")
    if Gamma is not None or weight is not None or gauss != "full":
        raise NotImplementedError("∫: boundary domains, weights and reduced Gauss rules are not accelerated")
    if Omega is not None and Omega not in [m.phName for m in P.material]:
        raise NotImplementedError("∫: sub-domains other than the problem's material groups are not accelerated")
    C = _coefficient(term.coef)
    ops = (term.a.op, term.b.op)
    c2 = None
    if ops == ("SymGrad", "SymGrad"):
        lm = None if np.isscalar(C) else _isotropic(np.asarray(C), P.dim)
        if lm is None:
            raise NotImplementedError("∫(SymGrad⋅D⋅SymGrad): only isotropic D is accelerated")
        kind, c1, c2 = _lib.FORM_SYMGRAD, lm[0], lm[1]
    elif ops == ("Grad", "Grad") and P.pdim == 1 and np.isscalar(C):
        kind, c1 = _lib.FORM_GRAD, C
    elif ops == ("Id", "Id") and np.isscalar(C):
        kind, c1 = _lib.FORM_ID, C
    else:
        raise NotImplementedError(f"∫({ops[0]}⋅coef⋅{ops[1]}) with this coefficient is not accelerated")
    nmat = len(P.material)
    c1a = np.full(nmat, float(c1))
    c2a = None if c2 is None else np.full(nmat, float(c2))
    ctx, dm, pat = P._ctx, P.device_mesh(), P.pattern()
    acc = None
    if csc_matrix is not None:
        if not isinstance(csc_matrix, SystemMatrix) or csc_matrix.dm.pattern is not pat:
            raise ValueError("assemble_operator: csc_matrix must be a matrix on the problem's pattern")
        acc = csc_matrix.dm.h
    h = _lib.C.c_void_p()
    ctx.check(_lib.lib().llf_assemble_form(ctx.h, dm.h, pat.h, kind, _lib.ptr(c1a, _lib.C.c_double),
                                           _lib.ptr(c2a, _lib.C.c_double), nmat, acc, _form(precision),
                                           _lib.C.byref(h)), "∫")
    out = _lib.DeviceMatrix(ctx, h, pat)
    if csc_matrix is not None:
        csc_matrix.dm, csc_matrix._csc = out, None
        return csc_matrix
    return SystemMatrix(out, P)
