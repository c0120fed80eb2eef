"""The benchmark's workload on the oracle side: the unit-cube hex27 box and
its quadrature tables, built without the GPU library so that the CPU
reference arm loads nothing but the oracle.

TEST INFRASTRUCTURE ONLY (the bench's reference arm and CPU baseline).

The mesh restates the library's structured generator (nodes on the lattice
i/(2n), x fastest; elements x fastest, each element's nodes at the lattice
offsets of the hex27 node order); tests/test_oracle_workload.py checks it
against the library's structured_box_mesh array for array.  The tables come
from the committed oracle/hex27_rule.npz (made by make_rule_fixture.py and
checked against llf_builtin_rule bit for bit by the same test file).
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def hex27_rule() -> dict:
    z = np.load(os.path.join(HERE, "hex27_rule.npz"))
    r = {k: z[k] for k in ("w", "N", "dN", "node_ref", "xi")}
    r["nip"], r["npe"] = len(r["w"]), r["N"].shape[1]
    return r


def box_hex27(n: int, lz: float = 1.0) -> tuple[np.ndarray, np.ndarray]:
    """(xyz (non, 3), conn (nel, 27) 1-based) of [0,1] x [0,1] x [0,lz] with
    n x n x ceil(lz*n) hex27 elements."""
    p = 2
    d = 1.0 / n
    nx = ny = n
    nz = int(np.ceil(lz / d))
    NX, NY, NZ = p * nx + 1, p * ny + 1, p * nz + 1
    xs = 1.0 * (np.arange(NX) / (NX - 1))
    ys = 1.0 * (np.arange(NY) / (NY - 1))
    zs = lz * (np.arange(NZ) / (NZ - 1))
    kk, jj, ii = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    xyz = np.stack([xs[ii.ravel()], ys[jj.ravel()], zs[kk.ravel()]], axis=1)
    lat = np.rint((hex27_rule()["node_ref"] + 1.0) * p / 2.0).astype(np.int64)
    ck, cj, ci = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    I = p * ci[:, None] + lat[None, :, 0]
    J = p * cj[:, None] + lat[None, :, 1]
    K = p * ck[:, None] + lat[None, :, 2]
    conn = (I + NX * (J + NY * K)).astype(np.int64) + 1
    return xyz, conn
