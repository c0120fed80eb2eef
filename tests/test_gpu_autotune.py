"""The assembly schedule autotuner (llf_autotune_stiffness): every schedule
it tries must give the same stored CSC bit for bit (it checks that itself),
and assemblies after tuning stay bit-identical to the oracle."""
import numpy as np
import pytest

from helpers import PT, assert_csc_identical, make_mesh, oracle_operator

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [("box", 4, 2, False, "Solid"), ("box", 5, 2, True, "Solid"),
                                  ("rect", 12, 3, False, "PlaneStrain")], ids=["hex27", "tet10", "quad16"])
@pytest.mark.parametrize("precision", ["fp64", "fp32q"])
def test_tuned_schedules_keep_the_bits(llf, orc, case, precision):
    kind, n, order, simplex, ptype = case
    m = make_mesh(llf, kind, n, order, simplex)
    mat = llf.Material("body", E=2.1e5, nu=0.3)
    p = llf.Problem([mat], type=ptype)
    K0 = llf.stiffnessMatrix(p, precision=precision).csc()
    rep = llf.autotune(p, precision=precision, trials=1)
    assert len(rep["trials"]) >= 10            # coordinate descent over three knobs
    chosen = rep["chosen"]
    assert chosen["gather_warps_per_cta"] in (2, 4, 8)
    K1 = llf.stiffnessMatrix(p, precision=precision).csc()
    assert_csc_identical(K1, K0, f"after autotune {chosen}")
    if precision == "fp64":
        ref = oracle_operator(llf, orc, m, "stiffness", PT[ptype], mat)
        assert_csc_identical(K1, ref.julia(), "tuned K vs oracle")


def test_tuned_schedule_is_reused_for_the_same_shape(llf, orc):
    """A second problem of the same shape picks up the tuned schedule and its
    matrix is still the oracle's."""
    llf.structured_box_mesh(n=3, order=2)
    p = llf.Problem([llf.Material("body", E=2e5, nu=0.25)], type="Solid")
    rep = llf.autotune(p, trials=1)
    m = llf.structured_box_mesh(n=3, order=2, lx=2.0)
    mat = llf.Material("body", E=1e5, nu=0.35)
    p2 = llf.Problem([mat], type="Solid")
    K = llf.stiffnessMatrix(p2).csc()
    ref = oracle_operator(llf, orc, m, "stiffness", 0, mat)
    assert_csc_identical(K, ref.julia(), "K after a tuned schedule of the same shape")
    assert rep["key"]
