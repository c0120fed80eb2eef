"""GPU solves (solveDisplacement / solveTemperature / solveField) against the
reference's known answers and the oracle's CG."""
import numpy as np
import pytest

from helpers import oracle_operator

pytestmark = pytest.mark.gpu


def test_plane_stress_validation(llf):
    """test/test_validation.jl: u(1,1) = (1/E, -nu/E)."""
    llf.structured_rect_mesh()
    mat = llf.Material("body")
    prob = llf.Problem([mat], type="PlaneStress")
    supp1 = llf.displacementConstraint("left", ux=0)
    supp2 = llf.displacementConstraint("bottom", uy=0)
    ld = llf.load("right", fx=1)
    u = llf.solveDisplacement(prob, load=[ld], support=[supp1, supp2])
    xyz = prob.mesh.xyz
    node = int(np.where((np.abs(xyz[:, 0] - 1) < 1e-12) & (np.abs(xyz[:, 1] - 1) < 1e-12))[0][0])
    ux, uy = u.a[2 * node, 0], u.a[2 * node + 1, 0]
    assert np.isclose(ux, 1 / mat.E, rtol=1e-2) and np.isclose(uy, -mat.nu / mat.E, rtol=1e-2)
    assert np.isclose(ux, 1 / mat.E, rtol=1e-10) and np.isclose(uy, -mat.nu / mat.E, rtol=1e-10)


def test_sum_u_golden_hex8_n30(llf):
    """results.txt:7 — sum(u) = 0.07057241535937334 (direct solve in the reference)."""
    llf.structured_box_mesh(n=30)
    mat = llf.Material("body")
    P = llf.Problem([mat], type="Solid")
    support = [llf.BoundaryCondition("left", ux=0.0, uy=0.0, uz=0.0)]
    K = llf.stiffnessMatrix(P)
    assert abs(np.abs(K.csc()[2]).sum() - 4.0073076923076982e9) <= 1e-15 * 4.0073076923076982e9
    f = llf.loadVector(P, [llf.load("right", fx=1.0, fy=0.0, fz=0.0)])
    u = llf.solveField(K, f, support=support)
    assert u.relres <= 1e-13
    assert abs(u.a.sum() - 0.07057241535937334) <= 1e-11 * 0.0706
    fixed = llf.constrainedDoFs(P, support) - 1
    assert np.all(u.a[fixed, 0] == 0.0)
    free = llf.freeDoFs(P, support) - 1
    res = K * u.a[:, 0] - f.a[:, 0]
    assert np.linalg.norm(res[free]) / np.linalg.norm(f.a[free, 0]) < 1e-10   # test/test_dsl.jl:106


def test_pcg_matches_oracle_cg(llf, orc):
    """IterativeSolvers.cg semantics: same recurrence and stopping rule as the
    oracle's restatement; the iteration counts agree up to rounding."""
    m = llf.structured_box_mesh(n=6, order=2)
    mat = llf.Material("body")
    P = llf.Problem([mat], type="Solid")
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load("top", fy=-1.0)])
    support = [llf.displacementConstraint("bottom", ux=0, uy=0, uz=0)]
    for pre, code in (("identity", 0), ("jacobi", 1)):
        u = llf.solveDisplacement(K, f, support=support, iterative=True, preconditioner=pre)
        Ko = oracle_operator(llf, orc, m, "stiffness", 0, mat)
        fixed = np.zeros(3 * m.non, dtype=np.uint8)
        fixed[llf.constrainedDoFs(P, support) - 1] = 1
        uo, ito, rro = Ko.cg(f.a[:, 0], np.zeros(3 * m.non), fixed, precond=code,
                             reltol=np.sqrt(np.finfo(float).eps), maxiter=m.non * 3)
        assert abs(u.iterations - ito) <= max(2, 0.02 * ito), (pre, u.iterations, ito)
        assert u.relres <= np.sqrt(np.finfo(float).eps)
        # run to convergence, both agree to the contract's 1e-12 relative
        u = llf.solveDisplacement(K, f, support=support, iterative=True, preconditioner=pre, reltol=1e-15,
                                  maxiter=20 * 3 * m.non)
        uo, ito, rro = Ko.cg(f.a[:, 0], np.zeros(3 * m.non), fixed, precond=code, reltol=1e-15,
                             maxiter=20 * 3 * m.non)
        assert u.relres <= 1e-15 and rro <= 1e-15
        assert np.linalg.norm(u.a[:, 0] - uo) <= 1e-12 * np.linalg.norm(uo), \
            np.linalg.norm(u.a[:, 0] - uo) / np.linalg.norm(uo)


def test_prescribed_nonzero_displacement(llf):
    """f_kin = K[:,fixed] u[fixed] path (src/linear.jl:3825): a prescribed
    uniform stretch gives a homogeneous field."""
    m = llf.structured_box_mesh(n=3, order=2)
    P = llf.Problem([llf.Material("body", E=2e5, nu=0.0)], type="Solid")
    supp = [llf.displacementConstraint("left", ux=0.0),
            llf.displacementConstraint("right", ux=1e-3),
            llf.displacementConstraint("bottom", uy=0.0),
            llf.displacementConstraint("rear", uz=0.0)]
    u = llf.solveDisplacement(P, support=supp)
    ux = u.a[0::3, 0]
    assert np.abs(ux - 1e-3 * m.xyz[:, 0]).max() < 1e-13


def test_heat_solve(llf, orc):
    """solveTemperature: linear temperature between two prescribed faces."""
    m = llf.structured_box_mesh(n=4, order=2)
    P = llf.Problem([llf.Material("body", k=45.0)], type="HeatConduction")
    bc = [llf.temperatureConstraint("left", T=0.0), llf.temperatureConstraint("right", T=10.0)]
    T = llf.solveTemperature(P, temperatureConstraint=bc)
    assert np.abs(T.a[:, 0] - 10.0 * m.xyz[:, 0]).max() < 1e-10


def test_not_converged_reports(llf):
    llf.structured_box_mesh(n=4, order=1)
    P = llf.Problem([llf.Material("body")], type="Solid")
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load("right", fx=1.0)])
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    u = llf.solveDisplacement(K, f, support=sup, iterative=True, maxiter=3)
    assert u.iterations == 3 and u.relres > 1e-3
    fixed = np.zeros(K.shape[0], np.uint8)
    fixed[llf.constrainedDoFs(P, sup) - 1] = 1
    with pytest.raises(llf.LLFError, match="not converged"):
        K.dm.pcg(f.a[:, 0], np.zeros(K.shape[0]), fixed, maxiter=3, reltol=1e-12, raise_on_fail=True)


def test_c1_cantilever_u_matches_oracle(llf, orc):
    """Config 1 end to end: plane-strain cantilever, 200 x 100 quad4 on the
    10 x 5 rectangle (40,602 DoFs), E = 2e5, nu = 0.3, left edge clamped,
    distributed fy = -1 on the right edge; solveDisplacement's CG
    (src/linear.jl:3827-3828) run to 1e-15 against the oracle's CG to the
    same tolerance: u within 1e-12 relative.  The direct solution (the
    reference's default) is itself off by about 1e-12 here (cond(K_ff) ~1e7
    times eps), so it is checked to 3e-12."""
    import scipy.sparse.linalg as spla
    m = llf.structured_rect_mesh(lx=10.0, ly=5.0, dx=0.05, dy=0.05)
    mat = llf.Material("body", E=2e5, nu=0.3)
    P = llf.Problem([mat], type="PlaneStrain")
    ld = [llf.load("right", fy=-1.0)]
    sup = [llf.displacementConstraint("left", ux=0.0, uy=0.0)]
    u = llf.solveDisplacement(P, load=ld, support=sup, iterative=True, preconditioner="jacobi", reltol=1e-15,
                              maxiter=200000)
    assert u.relres <= 1e-15
    Ko = oracle_operator(llf, orc, m, "stiffness", 2, mat)
    g = m.group("right")
    fo = orc.load_vector(2, 2, m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), t=[0.0, -1.0])
    fixed = np.zeros(2 * m.non, dtype=np.uint8)
    fixed[llf.constrainedDoFs(P, sup) - 1] = 1
    uo, ito, rro = Ko.cg(fo, np.zeros(2 * m.non), fixed, precond=1, reltol=1e-15, maxiter=200000)
    assert rro <= 1e-15
    d = np.linalg.norm(u.a[:, 0] - uo) / np.linalg.norm(uo)
    assert d <= 1e-12, d
    A = Ko.scipy().tocsc()
    fr = fixed == 0
    ud = np.zeros(2 * m.non)
    ud[fr] = spla.spsolve(A[fr][:, fr].tocsc(), fo[fr])
    assert np.linalg.norm(u.a[:, 0] - ud) <= 3e-12 * np.linalg.norm(ud)
