"""llf_pcg_noalloc: the allocation-free CG entry point.

It serves callers that cannot allocate device memory once running (a host
framework that already reserved the GPU's memory for its own pool, real-time
loops that forbid allocation after start-up).  They hand in device buffers
they own; the CG's work vectors come from a fixed array inside the library.
This file is collected last so that a failure here never hides the results of
the other tests.  It checks, through the C-ABI, that two calls in a row give
the same solutions as llf_pcg, and that oversized systems are refused.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(llf, n, order=2, scale=1.0):
    llf.structured_box_mesh(n=n, order=order)
    P = llf.Problem([llf.Material("body")], type="Solid")
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load("right", fx=scale, fz=-0.3 * scale)])
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    fixed = np.zeros(3 * P.non, dtype=np.uint8)
    fixed[llf.constrainedDoFs(P, sup) - 1] = 1
    return P, K, f.a[:, 0].copy(), fixed


def _noalloc(llf, K, b, x0, fixed, precond, reltol, maxiter):
    torch = pytest.importorskip("torch")
    db = torch.tensor(b, dtype=torch.float64, device="cuda")
    dx = torch.tensor(x0, dtype=torch.float64, device="cuda")
    dfx = torch.tensor(fixed, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    it, rr = C.c_int64(0), C.c_double(0.0)
    L = llf._lib.lib()
    allocs0 = K.dm.ctx.allocs()
    rc = L.llf_pcg_noalloc(K.dm.ctx.h, K.dm.h, C.c_void_p(db.data_ptr()), C.c_void_p(dx.data_ptr()),
                           C.c_void_p(dfx.data_ptr()), precond, reltol, maxiter, C.byref(it), C.byref(rr))
    K.dm.ctx.check(rc, "llf_pcg_noalloc")
    # the library's own allocation counter: the call made no device allocation
    assert K.dm.ctx.allocs() == allocs0, "llf_pcg_noalloc allocated device memory"
    torch.cuda.synchronize()
    return dx.cpu().numpy(), it.value, rr.value


@pytest.mark.parametrize("precond", [0, 1, 2])
def test_noalloc_matches_pcg_twice(llf, precond):
    _, K, f, fixed = _system(llf, 4)
    x0 = np.zeros_like(f)
    maxiter = 20 * len(f)
    for scale in (1.0, -2.5):   # two calls in a row, different right-hand sides
        b = scale * f
        ref, it_ref, rr_ref = K.dm.pcg(b, x0, fixed, precond=precond, reltol=1e-10, maxiter=maxiter)
        got, it, rr = _noalloc(llf, K, b, x0, fixed, precond, 1e-10, maxiter)
        assert it == it_ref
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
        assert rr <= 1e-10


def test_noalloc_prescribed_values_and_second_system(llf):
    """A different (smaller) system right after: stale scratch contents from
    the previous call must not leak into the result."""
    _, K, f, fixed = _system(llf, 3, order=2)
    x0 = np.zeros_like(f)
    x0[fixed == 1] = 1e-4      # non-zero prescribed displacement
    ref, _, _ = K.dm.pcg(f, x0, fixed, precond=1, reltol=1e-10, maxiter=20 * len(f))
    got, _, _ = _noalloc(llf, K, f, x0, fixed, 1, 1e-10, 20 * len(f))
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


def test_noalloc_rejects_oversized_system(llf):
    # 3 * 33^3 = 107,811 DoFs fits; 3 * 35^3 = 128,625 fits; 3 * 37^3 = 151,959 does not
    _, K, f, fixed = _system(llf, 18, order=2)
    assert len(f) > 131072
    with pytest.raises(llf.LLFError, match="at most 131072"):
        _noalloc(llf, K, f, np.zeros_like(f), fixed, 1, 1e-8, 10)


def test_noalloc_refuses_ic0(llf):
    """IC(0) needs a factor sized by the matrix, so this path refuses it with
    a message that says so (not as an unknown preconditioner)."""
    _, K, f, fixed = _system(llf, 2, order=1)
    with pytest.raises(llf.LLFError, match="IC\\(0\\) is not supported"):
        _noalloc(llf, K, f, np.zeros_like(f), fixed, 3, 1e-8, 10)


def test_noalloc_after_layout_reuse_needs_prepare(llf):
    """A matrix assembled into the stored layout its pattern kept holds the
    stored CSC only: llf_pcg_noalloc refuses it until llf_matrix_prepare has
    expanded its structural values; then it solves as llf_pcg does."""
    P, K1, f, fixed = _system(llf, 3, order=2)
    K = llf.stiffnessMatrix(P)   # second assembly on the pattern: the kept layout
    x0 = np.zeros_like(f)
    with pytest.raises(llf.LLFError, match="not expanded"):
        _noalloc(llf, K, f, x0, fixed, 1, 1e-10, 20 * len(f))
    K.dm.prepare()
    got, it, _ = _noalloc(llf, K, f, x0, fixed, 1, 1e-10, 20 * len(f))
    ref, it_ref, _ = K1.dm.pcg(f, x0, fixed, precond=1, reltol=1e-10, maxiter=20 * len(f))
    assert it == it_ref
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
