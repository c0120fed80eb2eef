"""Writes oracle/hex27_rule.npz: the library's built-in hex27 tables
(3 x 3 x 3 Gauss-Legendre points and weights, Lagrange values and reference
gradients, node coordinates on [-1, 1]^3, from llf_builtin_rule), so that the
benchmark's CPU reference arm builds its workload and runs the oracle
without loading the GPU library.  tests/test_oracle_workload.py checks the
committed file against llf_builtin_rule bit for bit.

TEST INFRASTRUCTURE ONLY.  Usage: python oracle/make_rule_fixture.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "hex27_rule.npz")


def main():
    sys.path.insert(0, os.path.dirname(HERE))
    import __graft_entry__ as entry
    llf = entry.load_package()
    r = llf._lib.builtin_rule(llf.HEX, 2)
    np.savez_compressed(OUT, w=r["w"], N=r["N"], dN=r["dN"], node_ref=r["node_ref"], xi=r["xi"])
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
