"""Mixed-precision PCG (llf_pcg_mixed): FP32 iterations with FP64 reliable
updates, replacing the same cg(K.A[free,free], ...) call
(src/linear.jl:3827-3828).  The stopping test is on the true FP64 residual,
so the solution must agree with the FP64 solve and with a direct solve of
the oracle's matrix to the accuracy the tolerance implies; a system's result
is the same alone and in a batch."""
import numpy as np
import pytest

from helpers import oracle_operator

pytestmark = pytest.mark.gpu


def _problem(llf, n=4, order=2, simplex=False, lx=1.0, E=2.1e5, nu=0.3, name="body"):
    m = llf.structured_box_mesh(n=n, lx=lx, order=order, simplex=simplex)
    P = llf.Problem([llf.Material(name, E=E, nu=nu)], type="Solid")
    return m, P


def _direct(llf, orc, m, P, f, sup):
    import scipy.sparse.linalg as spla
    mat = P.material[0]
    A = oracle_operator(llf, orc, m, "stiffness", 0, mat).scipy().tocsc()
    fixed = np.zeros(3 * m.non, bool)
    fixed[llf.constrainedDoFs(P, sup) - 1] = True
    fr = ~fixed
    ud = np.zeros(3 * m.non)
    ud[fr] = spla.spsolve(A[fr][:, fr].tocsc(), f[fr])
    return ud


@pytest.mark.parametrize("prec", ["jacobi", "bjacobi", "ic0"])
@pytest.mark.parametrize("simplex", [False, True], ids=["hex27", "tet10"])
def test_mixed_matches_direct(llf, orc, prec, simplex):
    m, P = _problem(llf, n=4, simplex=simplex)
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load("right", fx=1.0, fz=-0.3)])
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    u = llf.solveFieldBatched(K, f, support=sup, preconditioner=prec, reltol=1e-12, precision="mixed",
                              maxiter=20 * 3 * m.non)
    assert u.relres[0] <= 1e-12
    ud = _direct(llf, orc, m, P, f.a[:, 0], sup)
    err = np.linalg.norm(u.a[:, 0] - ud) / np.linalg.norm(ud)
    assert err <= 1e-10, err
    u64 = llf.solveFieldBatched(K, f, support=sup, preconditioner=prec, reltol=1e-12, maxiter=20 * 3 * m.non)
    # FP32 recurrences lose conjugacy faster: measured 1.1-1.7x the FP64
    # products on these stiffness systems (the residual replacements keep the
    # stopping test on the FP64 residual); more than 2x would mean the
    # replacements no longer keep the iteration on track
    assert u.iterations[0] <= 2.0 * u64.iterations[0] + 20, (u.iterations[0], u64.iterations[0])
    assert np.linalg.norm(u.a - u64.a) <= 1e-10 * np.linalg.norm(u64.a)


def test_mixed_batch_equals_alone(llf):
    rng = np.random.default_rng(5)
    specs = [(2, 1.0), (3, 0.5), (2, 1.7)]
    meshes = [llf.structured_box_mesh(n=n, lx=lx, order=2, simplex=True) for n, lx in specs]
    mats = [(float(rng.uniform(1e4, 3e5)), float(rng.uniform(0.2, 0.45))) for _ in specs]
    alone = []
    for mm, (E, nu) in zip(meshes, mats):
        llf.set_current(mm)
        Pi = llf.Problem([llf.Material("body", E=E, nu=nu)], type="Solid")
        Ki = llf.stiffnessMatrix(Pi)
        fi = llf.loadVector(Pi, [llf.load("right", fx=1.0)])
        si = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
        alone.append(llf.solveFieldBatched(Ki, fi, support=si, preconditioner="ic0", reltol=1e-11,
                                           precision="mixed"))
    batch, noff = llf.concat_meshes(meshes)
    P = llf.Problem([llf.Material(f"body#{i}", E=E, nu=nu) for i, (E, nu) in enumerate(mats)], type="Solid",
                    mesh=batch)
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load(f"right#{i}", fx=1.0) for i in range(len(meshes))])
    sup = [llf.displacementConstraint(f"left#{i}", ux=0, uy=0, uz=0) for i in range(len(meshes))]
    u = llf.solveFieldBatched(K, f, support=sup, node_offsets=noff, preconditioner="ic0", reltol=1e-11,
                              precision="mixed")
    for i, ui in enumerate(alone):
        a, b = 3 * noff[i], 3 * noff[i + 1]
        assert np.array_equal(u.a[a:b, 0], ui.a[:, 0]), i
        assert u.iterations[i] == ui.iterations[0]


def test_mixed_prescribed_displacement_and_heat(llf):
    """Non-zero prescribed values (f_kin path) and a scalar problem."""
    m = llf.structured_box_mesh(n=3, order=2)
    P = llf.Problem([llf.Material("body", E=2e5, nu=0.0)], type="Solid")
    supp = [llf.displacementConstraint("left", ux=0.0), llf.displacementConstraint("right", ux=1e-3),
            llf.displacementConstraint("bottom", uy=0.0), llf.displacementConstraint("rear", uz=0.0)]
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [])
    u = llf.solveFieldBatched(K, f, support=supp, preconditioner="jacobi", reltol=1e-13, precision="mixed")
    assert np.abs(u.a[0::3, 0] - 1e-3 * m.xyz[:, 0]).max() < 1e-14
    Ph = llf.Problem([llf.Material("body", k=45.0)], type="HeatConduction")
    H = llf.heatConductionMatrix(Ph)
    bc = [llf.temperatureConstraint("left", T=0.0), llf.temperatureConstraint("right", T=10.0)]
    T = llf.solveFieldBatched(H, np.zeros(m.non), support=bc, preconditioner="ic0", reltol=1e-13,
                              precision="mixed")
    assert np.abs(T.a[:, 0] - 10.0 * m.xyz[:, 0]).max() < 1e-10


def test_mixed_not_converged_reports(llf):
    m, P = _problem(llf, n=3, order=1)
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load("right", fx=1.0)])
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    u = llf.solveFieldBatched(K, f, support=sup, preconditioner="jacobi", reltol=1e-12, precision="mixed",
                              maxiter=3)
    assert u.iterations[0] == 3 and u.relres[0] > 1e-6
