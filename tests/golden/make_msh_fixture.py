"""Writes tests/golden/elasticity_benchmark_msh.npz, a compact exact copy of
the reference's mesh fixture
examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/elasticity_benchmark.msh
(unit cube, 30 x 30 x 30 hex8, 29,791 nodes, 27,000 elements, six face
groups of 900 quad4 each; written by that directory's
lowlevelfem_elasticity_benchmark.jl:26-27).

The mesh is a lattice, so the fixture stores:
  * tag[i, j, k]: the MSH node tag of lattice point (i, j, k), 0 <= i,j,k <= 30;
  * ulp[t - 1, c]: coordinate c of node t as a step count from i/30 along the
    float64 line (np.nextafter), because gmsh's coordinates are not all the
    nearest doubles to i/30 (72 % differ by one or a few ulps);
  * local: the lattice corner (bit 0 = x, 1 = y, 2 = z) of each of the 8
    element nodes, the same for every element; elements are the cells in
    x-fastest order, as in the file;
  * faces: the quad4 connectivity of each face group, as in the file.
decode() rebuilds coordinates and connectivity bit for bit; this script
checks that against the file before writing.

Usage: python tests/golden/make_msh_fixture.py <reference checkout>
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "elasticity_benchmark_msh.npz")
REL = "examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/elasticity_benchmark.msh"
N = 30
FACES = ("left", "right", "front", "rear", "bottom", "top")


def _steps(base: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Signed number of nextafter steps from base to x (same sign, finite)."""
    bi = base.view(np.int64).astype(np.int64)
    xi = x.view(np.int64).astype(np.int64)
    return xi - bi


def decode(path: str = OUT):
    """(xyz (non, 3) float64, conn (nel, 8) int64 1-based, faces {name: (900, 4) int64})."""
    z = np.load(path)
    tag = z["tag"].astype(np.int64)
    non = int(tag.max())
    lat = np.zeros((non, 3), dtype=np.int64)
    ii, jj, kk = np.meshgrid(np.arange(N + 1), np.arange(N + 1), np.arange(N + 1), indexing="ij")
    lat[tag.ravel() - 1] = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1)
    base = lat.astype(np.float64) / float(N)
    bits = base.view(np.int64) + z["ulp"].astype(np.int64)
    xyz = bits.view(np.float64).reshape(non, 3)
    ci, cj, ck = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    cells = np.stack([ci.transpose(2, 1, 0).ravel(), cj.transpose(2, 1, 0).ravel(),
                      ck.transpose(2, 1, 0).ravel()], axis=1)   # x fastest
    loc = z["local"].astype(np.int64)
    off = np.stack([loc & 1, (loc >> 1) & 1, (loc >> 2) & 1], axis=1)
    corner = cells[:, None, :] + off[None, :, :]
    conn = tag[corner[..., 0], corner[..., 1], corner[..., 2]]
    faces = {name: z[f"face_{name}"].astype(np.int64) for name in FACES}
    return xyz, conn, faces


def main(ref_root: str):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import __graft_entry__ as entry
    llf = entry.load_package()
    m = llf.read_msh(os.path.join(ref_root, REL))
    assert (m.non, m.nel, m.npe) == ((N + 1) ** 3, N ** 3, 8)
    lat = np.rint(m.xyz * N).astype(np.int64)
    assert np.abs(lat / float(N) - m.xyz).max() < 1e-14
    tag = np.zeros((N + 1,) * 3, dtype=np.int32)
    tag[lat[:, 0], lat[:, 1], lat[:, 2]] = np.arange(1, m.non + 1, dtype=np.int32)
    assert len(np.unique(tag)) == m.non
    ulp = _steps(lat.astype(np.float64) / float(N), m.xyz)
    assert np.abs(ulp).max() < 127
    L = lat[m.conn - 1]
    loc = L - L.min(axis=1)[:, None, :]
    codes = loc[:, :, 0] + 2 * loc[:, :, 1] + 4 * loc[:, :, 2]
    assert (codes == codes[0]).all()
    arrays = {"tag": tag, "ulp": ulp.astype(np.int8), "local": codes[0].astype(np.int8)}
    for name in FACES:
        g = m.group(name)
        arrays[f"face_{name}"] = g.conn.astype(np.int32)
    np.savez_compressed(OUT, **arrays)
    xyz, conn, faces = decode(OUT)
    assert np.array_equal(xyz.view(np.int64), m.xyz.view(np.int64)), "coordinates differ"
    assert np.array_equal(conn, m.conn), "connectivity differs"
    for name in FACES:
        assert np.array_equal(faces[name], m.group(name).conn)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes); round trip exact")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LLF_REFERENCE_DIR")
    if not root:
        sys.exit("usage: make_msh_fixture.py <reference checkout>")
    main(root)
