"""Built-in quadrature and shape tables (stand-ins for gmsh's
getIntegrationPoints("Gauss(2p+1)") / getBasisFunctions)."""
import itertools

import numpy as np
import pytest

FAMS = [(1, "line"), (2, "tri"), (3, "quad"), (4, "tet"), (5, "hex")]


def _dim(fam):
    return {1: 1, 2: 2, 3: 2, 4: 3, 5: 3}[fam]


def _exact_monomial(fam, powers):
    # exact integral of x^i y^j z^k over the reference element
    from math import factorial
    d = _dim(fam)
    if fam in (1, 3, 5):
        v = 1.0
        for p in powers[:d]:
            v *= 0.0 if p % 2 else 2.0 / (p + 1)
        return v
    num = 1
    for p in powers[:d]:
        num *= factorial(p)
    return num / factorial(sum(powers[:d]) + d)


@pytest.mark.parametrize("fam,name", FAMS)
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_rule_exactness(llf, fam, name, order):
    r = llf._lib.builtin_rule(fam, order)
    d = _dim(fam)
    deg = 2 * order + 1
    for powers in itertools.product(range(deg + 1), repeat=d):
        if fam in (2, 4) and sum(powers) > deg:
            continue
        if fam in (1, 3, 5) and max(powers) > deg:
            continue
        f = np.ones(r["nip"])
        for j, p in enumerate(powers):
            f = f * r["xi"][:, j] ** p
        got = float(f @ r["w"])
        want = _exact_monomial(fam, list(powers) + [0] * (3 - d))
        assert abs(got - want) < 1e-13, (name, order, powers, got, want)


@pytest.mark.parametrize("fam,name", FAMS)
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_partition_of_unity(llf, fam, name, order):
    r = llf._lib.builtin_rule(fam, order)
    assert np.abs(r["N"].sum(axis=1) - 1.0).max() < 1e-13
    assert np.abs(r["dN"].sum(axis=1)).max() < 1e-12
    # gradients reproduce linear functions: sum_a x_a dN_a/dxi_j = delta_ij
    ref = r["node_ref"]
    d = _dim(fam)
    for q in range(r["nip"]):
        J = ref[:, :d].T @ r["dN"][q, :, :d]
        assert np.abs(J - np.eye(d)).max() < 1e-12
        x = ref[:, :d].T @ r["N"][q]
        assert np.abs(x - r["xi"][q, :d]).max() < 1e-12


def test_gmsh_first_and_second_order_vertices(llf):
    # hex8 / quad4 vertex order of gmsh (MSH node ordering)
    h = llf._lib.builtin_rule(5, 1)["node_ref"]
    want = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
    assert np.array_equal(h, np.array(want, float))
    q9 = llf._lib.builtin_rule(3, 2)["node_ref"][:, :2]
    want9 = [(-1, -1), (1, -1), (1, 1), (-1, 1), (0, -1), (1, 0), (0, 1), (-1, 0), (0, 0)]
    assert np.array_equal(q9, np.array(want9, float))
    t10 = llf._lib.builtin_rule(4, 2)["node_ref"]
    assert np.array_equal(t10[:4], np.array([(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)], float))
