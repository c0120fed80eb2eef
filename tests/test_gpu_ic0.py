"""IC(0) preconditioner (multicolour node-block incomplete Cholesky) in the
GPU PCG: same solution as the other preconditioners and the oracle's
solve, fewer iterations than Jacobi, batched systems identical to lone ones."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu


def _direct(K, f, fixed):
    A = K.A.tocsc()
    free = ~fixed
    u = np.zeros(A.shape[0])
    u[free] = spla.spsolve(A[free][:, free].tocsc(), f[free])
    return u


@pytest.mark.parametrize("case", [("box", 4, 1), ("box", 3, 2), ("rect", 8, 2), ("box", 2, 2, True)])
def test_ic0_elasticity_matches_direct_and_beats_jacobi(llf, case):
    kind, n, order = case[:3]
    simplex = len(case) > 3
    if kind == "box":
        m = llf.structured_box_mesh(n=n, order=order, simplex=simplex)
        P = llf.Problem([llf.Material("body", E=2.1e5, nu=0.3)], type="Solid")
        sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
        ld = [llf.load("right", fx=1.0, fy=0.5)]
    else:
        m = llf.structured_rect_mesh(n=n, order=order, simplex=simplex)
        P = llf.Problem([llf.Material("body", E=2.1e5, nu=0.3)], type="PlaneStrain")
        sup = [llf.displacementConstraint("left", ux=0, uy=0)]
        ld = [llf.load("right", fy=-1.0)]
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, ld)
    fixed = np.zeros(K.A.shape[0], dtype=bool)
    fixed[llf.constrainedDoFs(P, sup) - 1] = True
    ud = _direct(K, f.a[:, 0], fixed)
    uj = llf.solveDisplacement(K, f, support=sup, iterative=True, preconditioner="jacobi", reltol=1e-12)
    ui = llf.solveDisplacement(K, f, support=sup, iterative=True, preconditioner="ic0", reltol=1e-12)
    assert np.linalg.norm(ui.a[:, 0] - ud) <= 1e-9 * np.linalg.norm(ud)
    assert np.all(ui.a[fixed, 0] == 0.0)
    assert ui.iterations < uj.iterations, (ui.iterations, uj.iterations)


def test_ic0_heat_linear_field(llf):
    """Scalar problem (p = 1): the linear temperature between two prescribed
    faces lies in the P2 space, so IC(0)-PCG reproduces it to its tolerance."""
    llf.structured_box_mesh(n=6, order=2, simplex=True)
    P = llf.Problem([llf.Material("body", k=3.0)], type="HeatConduction")
    bc = [llf.temperatureConstraint("left", T=0.0), llf.temperatureConstraint("right", T=10.0)]
    Tj = llf.solveTemperature(P, temperatureConstraint=bc, iterative=True, preconditioner="jacobi", reltol=1e-13)
    Ti = llf.solveTemperature(P, temperatureConstraint=bc, iterative=True, preconditioner="ic0", reltol=1e-13)
    x = P.mesh.xyz[:, 0]
    assert np.abs(Ti.a[:, 0] - 10.0 * x).max() < 1e-9
    assert Ti.iterations < Tj.iterations


def test_ic0_batched_equals_alone(llf):
    ms = [llf.structured_box_mesh(n=n, order=2, simplex=True) for n in (2, 3)]
    batch, noff = llf.concat_meshes(ms)
    mats = [llf.Material(f"body#{i}", E=E, nu=0.3) for i, E in enumerate((1e5, 2e5))]
    P = llf.Problem(mats, type="Solid", mesh=batch)
    K = llf.stiffnessMatrix(P)
    sup = [llf.displacementConstraint(f"left#{i}", ux=0, uy=0, uz=0) for i in range(2)]
    f = llf.loadVector(P, [llf.load(f"right#{i}", fx=1.0) for i in range(2)])
    ub = llf.solveFieldBatched(K, f, support=sup, node_offsets=noff, preconditioner="ic0", reltol=1e-12)
    for i, mi in enumerate(ms):
        Pi = llf.Problem([llf.Material("body", E=(1e5, 2e5)[i], nu=0.3)], type="Solid", mesh=mi)
        Ki = llf.stiffnessMatrix(Pi)
        fi = llf.loadVector(Pi, [llf.load("right", fx=1.0)])
        ui = llf.solveField(Ki, fi, support=[llf.displacementConstraint("left", ux=0, uy=0, uz=0)],
                            iterative=True, preconditioner="ic0", reltol=1e-12)
        a, b = 3 * noff[i], 3 * noff[i + 1]
        assert np.array_equal(ub.a[a:b, 0], ui.a[:, 0]), i
        assert ub.iterations[i] == ui.iterations
