"""The reference's own mesh fixture, elasticity_benchmark.msh, with its MSH
node numbering and element order (rebuilt exactly from
tests/golden/elasticity_benchmark_msh.npz), against the reference's published
checksums (examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/results.txt:7):
sum(abs, K) = 4.0073076923076982e9 and sum(u) = 0.07057241535937334 for
E = 2e5, nu = 0.3, "left" clamped, unit traction x on "right", direct solve
(lowlevelfem_elasticity_benchmark.jl:25-48).  The CPU tests pin the oracle;
the GPU tests pin the library through the C-ABI.

Tolerances.  On this mesh sum|K| comes out as 4.0073076923077044e9, 1.5e-15
relative (13 ulps of the sum) from the published value: the MSH coordinates
sit up to a few ulps off i/30 (the structured generator's exact lattice
reproduces all 17 printed digits, tests/test_oracle_golden.py), and a sum of
2.4 M magnitudes in another order moves its last digits.  The pin is
therefore 1e-14 relative, i.e. the 15 leading digits.  sum(u) is pinned to
1e-12 relative (the reference's value is a direct solve; Ferrite's
independent solve differs from it by 1.6e-14)."""
import numpy as np
import pytest

from helpers import assert_csc_identical, benchmark_msh_mesh

SUM_ABS_K = 4.0073076923076982e9
SUM_U = 0.07057241535937334


def _oracle_K(llf, orc, m):
    return orc.assemble(orc.ELASTIC, 0, 3, 3, m.xyz, m.conn, llf._lib.builtin_rule(m.family, m.order), [2e5, 0.3])


def test_fixture_is_the_reference_mesh(llf):
    m = benchmark_msh_mesh(llf)
    assert (m.non, m.nel) == (29791, 27000)
    for name in ("left", "right", "front", "rear", "bottom", "top"):
        assert len(m.group(name).nodes) == 961 and m.group(name).conn.shape == (900, 4)
    assert np.abs(m.xyz[m.group("left").nodes - 1, 0]).max() == 0.0
    assert np.abs(m.xyz[m.group("right").nodes - 1, 0] - 1.0).max() == 0.0


def test_oracle_sum_abs_K_on_reference_msh(llf, orc):
    m = benchmark_msh_mesh(llf)
    s = np.abs(_oracle_K(llf, orc, m).arrays()[2]).sum()
    assert abs(s - SUM_ABS_K) <= 1e-14 * SUM_ABS_K, repr(s)


def test_oracle_sum_u_on_reference_msh(llf, orc):
    m = benchmark_msh_mesh(llf)
    K = _oracle_K(llf, orc, m)
    g = m.group("right")
    f = orc.load_vector(3, 3, m.xyz, g.conn, llf._lib.builtin_rule(g.family, g.order), t=[1.0, 0.0, 0.0])
    fixed = np.zeros(3 * m.non, dtype=np.uint8)
    for c in range(3):
        fixed[(m.group("left").nodes - 1) * 3 + c] = 1
    u, it, rr = K.cg(f, np.zeros(3 * m.non), fixed, precond=1, reltol=1e-14, maxiter=20000)
    assert rr <= 1e-14
    assert abs(u.sum() - SUM_U) <= 1e-12 * SUM_U, repr(u.sum())


@pytest.mark.gpu
def test_gpu_K_and_u_on_reference_msh(llf, orc):
    """GPU K on the reference's mesh: bit-identical to the oracle and
    sum|K| equal to the published value to 15 digits; the GPU
    solve reproduces the published sum(u) to 1e-12."""
    m = benchmark_msh_mesh(llf)
    P = llf.Problem([llf.Material("body", E=2e5, nu=0.3)], type="Solid")
    K = llf.stiffnessMatrix(P)
    got = K.csc()
    assert_csc_identical(got, _oracle_K(llf, orc, m).julia(), "K on elasticity_benchmark.msh")
    s = np.abs(got[2]).sum()
    assert abs(s - SUM_ABS_K) <= 1e-14 * SUM_ABS_K, repr(s)
    support = [llf.displacementConstraint("left", ux=0.0, uy=0.0, uz=0.0)]
    u = llf.solveDisplacement(P, load=[llf.load("right", fx=1.0, fy=0.0, fz=0.0)], support=support)
    assert abs(u.a.sum() - SUM_U) <= 1e-12 * SUM_U, repr(u.a.sum())
