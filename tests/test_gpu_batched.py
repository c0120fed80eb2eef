"""Batched assembly + batched CG: many independent meshes (different sizes,
materials, loads) assembled in one launch and solved by one segmented CG;
each instance's result must equal its solve alone, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instance(llf, n, lx, simplex=True, order=2):
    return llf.structured_box_mesh(n=n, lx=lx, order=order, simplex=simplex)


def _solve_alone(llf, m, E, nu):
    llf.set_current(m)
    P = llf.Problem([llf.Material("body", E=E, nu=nu)], type="Solid")
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load("right", fx=1.0, fz=-0.5)])
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    u = llf.solveDisplacement(K, f, support=sup, iterative=True, preconditioner="jacobi", reltol=1e-10)
    return K, u


def test_batch_equals_alone(llf):
    rng = np.random.default_rng(3)
    specs = [(2, 1.0), (3, 0.5), (1, 2.0), (2, 1.5)]
    meshes = [_instance(llf, n, lx) for n, lx in specs]
    mats = [(float(rng.uniform(1e4, 3e5)), float(rng.uniform(0.2, 0.45))) for _ in specs]
    alone = [_solve_alone(llf, m, E, nu) for m, (E, nu) in zip(meshes, mats)]
    batch, noff = llf.concat_meshes(meshes)
    P = llf.Problem([llf.Material(f"body#{i}", E=E, nu=nu) for i, (E, nu) in enumerate(mats)], type="Solid",
                    mesh=batch)
    K = llf.stiffnessMatrix(P)
    f = llf.loadVector(P, [llf.load(f"right#{i}", fx=1.0, fz=-0.5) for i in range(len(meshes))])
    sup = [llf.displacementConstraint(f"left#{i}", ux=0, uy=0, uz=0) for i in range(len(meshes))]
    u = llf.solveFieldBatched(K, f, support=sup, node_offsets=noff, preconditioner="jacobi", reltol=1e-10)
    Kb = K.A
    for i, (Ki, ui) in enumerate(alone):
        a, b = 3 * noff[i], 3 * noff[i + 1]
        # the instance's block of the batched matrix is its matrix alone
        assert abs(Kb[a:b, a:b] - Ki.A).max() == 0.0
        assert np.array_equal(u.a[a:b, 0], ui.a[:, 0]), i
        assert u.iterations[i] == ui.iterations
    # no coupling between instances
    assert Kb[: 3 * noff[1], 3 * noff[1]:].nnz == 0
