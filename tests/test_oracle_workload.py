"""The bench's oracle-side workload (oracle/workload.py, oracle/hex27_rule.npz)
is the library's: the committed tables equal llf_builtin_rule bit for bit
and the box equals structured_box_mesh array for array, so the CPU
reference arm times the same workload without loading the GPU library."""
import numpy as np


def test_rule_fixture_is_builtin_rule(llf):
    from oracle import workload
    r = workload.hex27_rule()
    b = llf._lib.builtin_rule(llf.HEX, 2)
    for k in ("w", "N", "dN", "node_ref", "xi"):
        assert np.array_equal(r[k].view(np.int64), np.ascontiguousarray(b[k]).view(np.int64)), k


def test_box_is_structured_box_mesh(llf):
    from oracle import workload
    for n, lz in ((3, 1.0), (4, 0.5), (40, 4 / 40)):
        xyz, conn = workload.box_hex27(n, lz)
        m = llf.structured_box_mesh(n=n, lz=lz, order=2)
        assert np.array_equal(xyz.view(np.int64), m.xyz.view(np.int64)) and np.array_equal(conn, m.conn)


def test_bdb_baseline_agrees_with_oracle(llf, orc):
    """The CPU baseline's reference arithmetic (per-point B^T D B) agrees
    with the oracle's contract form to rounding."""
    from oracle import workload
    xyz, conn = workload.box_hex27(2, 1.0)
    r = workload.hex27_rule()
    pat = orc.pattern(xyz.shape[0], conn, 3)
    orc.assemble_bdb_threaded(0, 3, xyz, conn, r, 2.1e5, 0.3, pat, nthreads=2)
    K = orc.assemble(orc.ELASTIC, 0, 3, 3, xyz, conn, r, [2.1e5, 0.3]).scipy()
    assert abs(pat.scipy() - K).max() <= 1e-13 * abs(K).max()
