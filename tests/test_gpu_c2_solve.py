"""The unit-cube hex27 40^3 solid (1,594,323 DoFs, E = 2.1e5, nu = 0.3) end
to end through the public API: K and the consistent M, face x = 0 clamped,
face x = 1 under a uniform traction along x, IC(0)-preconditioned CG to a
relative residual of 1e-10 (solveDisplacement, src/linear.jl:3711-3870).

Checked with quantities that do not use the library's own product: the true
residual of the solution, computed by scipy on the stored CSC copied to the
host; the load resultant; the sum of M's entries (3 rho V); and agreement
with a block-Jacobi CG solution."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RHO = 7.85e-9


def test_clamped_traction_solve_full_size(llf):
    sp = pytest.importorskip("scipy.sparse")
    llf.structured_box_mesh(n=40, order=2)
    mat = llf.Material("body", E=2.1e5, nu=0.3, rho=RHO)
    P = llf.Problem([mat], type="Solid")
    K = llf.stiffnessMatrix(P)
    M = llf.massMatrix(P, lumped=False)
    f = llf.loadVector(P, [llf.load("right", fx=1.0)])
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    u = llf.solveDisplacement(K, f, support=sup, iterative=True, reltol=1e-10, preconditioner="ic0",
                              maxiter=20 * P.non)
    assert u.relres <= 1e-10
    n = 3 * P.non
    c, r, v = K.csc()
    A = sp.csc_matrix((v, r - 1, c - 1), shape=(n, n))
    fixed = np.zeros(n, dtype=bool)
    fixed[llf.constrainedDoFs(P, sup) - 1] = True
    fa, x = f.a[:, 0], u.a[:, 0]
    assert np.all(x[fixed] == 0.0)
    res = (fa - A @ x)[~fixed]
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(fa[~fixed])
    # a unit traction on the unit face: resultant 1 along x, nothing across
    assert abs(fa[0::3].sum() - 1.0) <= 1e-12 and abs(fa[1::3].sum()) <= 1e-15 and abs(fa[2::3].sum()) <= 1e-15
    # the pulled body moves along +x, most at the loaded face
    assert x[0::3].max() > 0 and x[0::3].min() >= -1e-3 * x[0::3].max()
    # the consistent mass matrix: its entries sum to 3 rho V (V = 1)
    assert abs(M.csc()[2].sum() - 3 * RHO) <= 1e-12 * 3 * RHO
    # another preconditioner, tighter tolerance: the same displacement
    u2 = llf.solveDisplacement(K, f, support=sup, iterative=True, reltol=1e-12, preconditioner="bjacobi",
                               maxiter=20 * P.non)
    assert np.linalg.norm(u2.a[:, 0] - x) <= 1e-6 * np.linalg.norm(x)
