"""Transient heat on the GPU (FDM, src/heat.jl:1466-1616) against the
oracle's scipy restatement of the reference's loop, on the same K and C.
The implicit branch solves by PCG to 1e-13 where the reference
back-substitutes one LU, so the states agree to 1e-9 of their magnitude;
the explicit branch (ϑ = 0, lumped C) differs only in the SpMV's summation
order (1e-12)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(llf, simplex=False, order=1):
    m = llf.structured_box_mesh(lx=2.0, n=4, order=order, simplex=simplex)
    p = llf.Problem([llf.Material("body", k=45.0, rho=7.85e-9, c=4.2e8)], type="HeatConduction")
    return m, p


@pytest.mark.parametrize("case", [(0.5, False, 1, "bjacobi"), (1.0, False, 1, "ic0"), (0.5, True, 1, "jacobi"),
                                  (0.0, False, 1, "bjacobi"), (2 / 3, False, 8, "bjacobi")],
                         ids=["CN-consistent", "implicit-ic0", "CN-lumped", "theta0-consistent", "q-per-step"])
def test_fdm_matches_oracle(llf, orc, case):
    theta, lumped, nq, prec = case
    m, p = _setup(llf)
    K = llf.heatConductionMatrix(p)
    C = llf.heatCapacityMatrix(p, lumped=lumped)
    n, dt = 8, 20.0
    rng = np.random.default_rng(20261203)
    qa = rng.uniform(0.0, 5.0, (m.non, nq))
    q = llf.ScalarField(qa, p)
    T0 = llf.ScalarField(rng.uniform(10.0, 30.0, (m.non, 1)), p)
    bc = [llf.temperatureConstraint("left", T=100.0), llf.temperatureConstraint("right", T=0.0)]
    T = llf.FDM(K, C, q, bc, T0, n, dt, theta=theta, preconditioner=prec)
    fixed = np.zeros(m.non, dtype=bool)
    cd = llf.constrainedDoFs(p, bc)
    fixed[cd - 1] = True
    R = np.zeros((n, m.non))
    R[0] = T0.a[:, 0]
    R[:, m.group("left").nodes - 1] = 100.0
    R[:, m.group("right").nodes - 1] = 0.0
    Cm = C.A if not lumped else __import__("scipy.sparse", fromlist=["diags"]).diags(C.A.diagonal())
    R = orc.fdm(K.A, Cm, qa, fixed, R, dt, theta)
    assert T.a.shape == (m.non, n)
    assert np.abs(T.a.T - R).max() <= 1e-9 * np.abs(R).max()


def test_fdm_explicit_lumped_matches_oracle(llf, orc):
    m, p = _setup(llf, simplex=True, order=1)
    K = llf.heatConductionMatrix(p)
    C = llf.heatCapacityMatrix(p, lumped=True)
    n, dt = 20, 0.5
    q = llf.ScalarField(np.full((m.non, 1), 2.0), p)
    T0 = llf.ScalarField(np.full((m.non, 1), 20.0), p)
    bc = [llf.temperatureConstraint("bottom", T=80.0)]
    T = llf.FDM(K, C, q, bc, T0, n, dt, theta=0.0)
    fixed = np.zeros(m.non, dtype=bool)
    fixed[llf.constrainedDoFs(p, bc) - 1] = True
    R = np.zeros((n, m.non))
    R[0] = 20.0
    R[:, fixed] = 80.0
    import scipy.sparse as sp
    R = orc.fdm(K.A, sp.diags(C.A.diagonal()), np.full(m.non, 2.0), fixed, R, dt, 0.0)
    assert T.iterations == 0
    assert np.abs(T.a.T - R).max() <= 1e-12 * np.abs(R).max()


def test_fdm_rejects_non_positive_lumped_capacity(llf):
    """Row-sum lumping of quadratic tetrahedra leaves non-positive vertex
    capacities; the reference stops on them and so does the GPU path."""
    m, p = _setup(llf, simplex=True, order=2)
    K = llf.heatConductionMatrix(p)
    C = llf.heatCapacityMatrix(p, lumped=True)
    q = llf.ScalarField(np.zeros((m.non, 1)), p)
    with pytest.raises(llf.LLFError, match="non-positive diagonal"):
        llf.FDM(K, C, q, [], q, 3, 1.0, theta=0.0)


def test_fdm_rejects_bad_arguments(llf):
    m, p = _setup(llf)
    K = llf.heatConductionMatrix(p)
    C = llf.heatCapacityMatrix(p)
    q = llf.ScalarField(np.zeros((m.non, 1)), p)
    with pytest.raises(ValueError):
        llf.FDM(K, C, q, [], q, 1, 1.0)
    with pytest.raises(ValueError):
        llf.FDM(K, C, q, [], q, 3, -1.0)
    with pytest.raises(llf.LLFError):
        llf.FDM(K, -1.0 * C, q, [], q, 3, 1.0)
