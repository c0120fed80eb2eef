"""Meshes: structured generators, an MSH 4.1 reader and physical groups.

The reference builds meshes with gmsh and reads connectivity, coordinates and
physical groups back through gmsh queries.  This module produces the same
data as plain arrays:

* ``structured_rect_mesh`` / ``structured_box_mesh`` follow the reference
  helpers (src/general.jl:8802-8871, :8910-8996): uniform spacing
  ``d = min(dx, dy)`` (``dz`` is ignored, as at :8948), ``ceil(l/d)`` element
  layers per edge, quadrilaterals/hexahedra ("RecombineAll"), physical groups
  named as the reference names them ("left", "right", "bottom", "top",
  "front", "rear", "body" and, in 2D, the corner points).  ``simplex=True``
  splits each cell into triangles (2 per cell) or tetrahedra (6 per cell).
* ``read_msh`` reads gmsh's MSH 4.1 ASCII files (e.g. the reference's
  ``elasticity_benchmark.msh`` written by
  examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/lowlevelfem_elasticity_benchmark.jl:26-27).

Node tags are dense and 1-based (src/multifield.jl:1602-1611); DoFs are
interleaved ``(node-1)*pdim + comp``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib

LINE, TRI, QUAD, TET, HEX = 1, 2, 3, 4, 5

# gmsh element type number -> (family, order)
GMSH_TYPES = {
    1: (LINE, 1), 2: (TRI, 1), 3: (QUAD, 1), 4: (TET, 1), 5: (HEX, 1),
    8: (LINE, 2), 9: (TRI, 2), 10: (QUAD, 2), 11: (TET, 2), 12: (HEX, 2),
    15: (None, 0),
}

FAMILY_DIM = {LINE: 1, TRI: 2, QUAD: 2, TET: 3, HEX: 3}
TENSOR = {LINE, QUAD, HEX}


def node_lattice(family: int, order: int) -> np.ndarray:
    """Integer lattice coordinates of the element nodes, in element node order
    (tensor shapes: 0..p per direction; simplices: barycentric indices)."""
    rule = _lib.builtin_rule(family, order)
    ref = rule["node_ref"]
    if family in TENSOR:
        lat = np.rint((ref + 1.0) * order / 2.0)
    else:
        lat = np.rint(ref * order)
    lat = lat.astype(np.int64)
    d = FAMILY_DIM[family]
    lat[:, d:] = 0
    return lat


@dataclass
class Group:
    """A physical group: its dimension, node tags (1-based, sorted unique) and,
    for dim >= 1, its elements (1-based connectivity) of one family/order."""
    name: str
    dim: int
    nodes: np.ndarray
    family: int = 0
    order: int = 0
    conn: np.ndarray | None = None
    elems: np.ndarray | None = None   # volume groups: element indices into Mesh.conn


@dataclass
class Mesh:
    """Nodes, volume elements and physical groups of one model."""
    dim: int
    family: int
    order: int
    xyz: np.ndarray            # (non, 3) float64
    conn: np.ndarray           # (nel, npe) int64, 1-based node tags
    groups: dict = field(default_factory=dict)
    name: str = "model"

    @property
    def non(self) -> int:
        return int(self.xyz.shape[0])

    @property
    def nel(self) -> int:
        return int(self.conn.shape[0])

    @property
    def npe(self) -> int:
        return int(self.conn.shape[1])

    def group(self, name: str) -> Group:
        if name not in self.groups:
            raise KeyError(f"Physical group '{name}' not found.")
        return self.groups[name]


# The reference keeps the "current model" inside gmsh; the generators and the
# reader set this module-level current mesh, which Problem() picks up.
_current: Mesh | None = None


def current_mesh() -> Mesh:
    if _current is None:
        raise RuntimeError("no mesh: call structured_rect_mesh, structured_box_mesh or read_msh first")
    return _current


def set_current(mesh: Mesh) -> Mesh:
    global _current
    _current = mesh
    return mesh


# --------------------------------------------------------------------------
# structured generators
# --------------------------------------------------------------------------
def _layers(length: float, d: float) -> int:
    # setTransfiniteCurve(c, ceil(l/d) + 1) nodes -> ceil(l/d) element layers
    return int(math.ceil(length / d))


def structured_rect_mesh(x0=0.0, y0=0.0, lx=1.0, ly=1.0, n=10, dx=None, dy=None,
                         order=1, simplex=False) -> Mesh:
    """2D structured mesh of [x0,x0+lx] x [y0,y0+ly] (src/general.jl:8802-8871)."""
    dx = lx / n if dx is None else dx
    dy = ly / n if dy is None else dy
    d = min(dx, dy)
    nx, ny = _layers(lx, d), _layers(ly, d)
    p = int(order)
    NX, NY = p * nx + 1, p * ny + 1
    ii, jj = np.meshgrid(np.arange(NX), np.arange(NY), indexing="xy")
    xs = x0 + lx * (np.arange(NX) / (NX - 1))
    ys = y0 + ly * (np.arange(NY) / (NY - 1))
    xyz = np.zeros((NX * NY, 3))
    xyz[:, 0] = xs[ii.ravel()]
    xyz[:, 1] = ys[jj.ravel()]

    def nid(i, j):
        return i + NX * j

    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()
    if not simplex:
        fam = QUAD
        lat = node_lattice(QUAD, p)
        conn = nid(p * ci[:, None] + lat[None, :, 0], p * cj[:, None] + lat[None, :, 1])
    else:
        fam = TRI
        lat = node_lattice(TRI, p)
        tris = [((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1))]
        parts = []
        for v0, v1, v2 in tris:
            e1 = np.subtract(v1, v0)
            e2 = np.subtract(v2, v0)
            oi = p * v0[0] + lat[:, 0] * e1[0] + lat[:, 1] * e2[0]
            oj = p * v0[1] + lat[:, 0] * e1[1] + lat[:, 1] * e2[1]
            parts.append(nid(p * ci[:, None] + oi[None, :], p * cj[:, None] + oj[None, :]))
        conn = np.stack(parts, axis=1).reshape(-1, lat.shape[0])
    conn = conn.astype(np.int64) + 1

    groups = {}
    allnodes = np.arange(NX * NY, dtype=np.int64) + 1
    groups["body"] = Group("body", 2, allnodes, fam, p, conn)
    linelat = node_lattice(LINE, p)[:, 0]

    def edge(name, fixed_axis, fixed_idx, reverse=False):
        ncell = nx if fixed_axis == 1 else ny
        cells = np.arange(ncell)
        if reverse:
            cells = cells[::-1]
        if fixed_axis == 1:   # y fixed: edge along x
            i = p * cells[:, None] + (linelat[None, :] if not reverse else p - linelat[None, :])
            j = np.full_like(i, fixed_idx)
        else:
            j = p * cells[:, None] + (linelat[None, :] if not reverse else p - linelat[None, :])
            i = np.full_like(j, fixed_idx)
        c = (nid(i, j) + 1).astype(np.int64)
        nodes = np.unique(c)
        groups[name] = Group(name, 1, nodes, LINE, p, c)

    edge("bottom", 1, 0)
    edge("right", 0, NX - 1)
    edge("top", 1, NY - 1, reverse=True)
    edge("left", 0, 0, reverse=True)
    for name, (i, j) in {"leftbottom": (0, 0), "rightbottom": (NX - 1, 0),
                         "righttop": (NX - 1, NY - 1), "lefttop": (0, NY - 1)}.items():
        groups[name] = Group(name, 0, np.array([nid(i, j) + 1], dtype=np.int64))
    m = Mesh(2, fam, p, xyz, conn, groups, name="structured_rect")
    return set_current(m)


_KUHN = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def structured_box_mesh(x0=0.0, y0=0.0, z0=0.0, lx=1.0, ly=1.0, lz=1.0, n=10,
                        dx=None, dy=None, dz=None, order=1, simplex=False) -> Mesh:
    """3D structured mesh of a box (src/general.jl:8910-8996); the spacing is
    d = min(dx, dy) in all three directions, as in the reference."""
    dx = lx / n if dx is None else dx
    dy = ly / n if dy is None else dy
    d = min(dx, dy)
    nx, ny, nz = _layers(lx, d), _layers(ly, d), _layers(lz, d)
    p = int(order)
    NX, NY, NZ = p * nx + 1, p * ny + 1, p * nz + 1
    xs = x0 + lx * (np.arange(NX) / (NX - 1))
    ys = y0 + ly * (np.arange(NY) / (NY - 1))
    zs = z0 + lz * (np.arange(NZ) / (NZ - 1))
    kk, jj, ii = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    I, J, K = ii.ravel(), jj.ravel(), kk.ravel()
    xyz = np.stack([xs[I], ys[J], zs[K]], axis=1)

    def nid(i, j, k):
        return i + NX * (j + NY * k)

    ck, cj, ci = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    if not simplex:
        fam = HEX
        lat = node_lattice(HEX, p)
        conn = nid(p * ci[:, None] + lat[None, :, 0], p * cj[:, None] + lat[None, :, 1],
                   p * ck[:, None] + lat[None, :, 2])
    else:
        fam = TET
        lat = node_lattice(TET, p)
        parts = []
        for perm in _KUHN:
            v = [np.zeros(3, dtype=np.int64)]
            for ax in perm:
                nv = v[-1].copy()
                nv[ax] = 1
                v.append(nv)
            e1, e2, e3 = v[1] - v[0], v[2] - v[0], v[3] - v[0]
            if np.linalg.det(np.stack([e1, e2, e3]).astype(float)) < 0:
                v[1], v[2] = v[2], v[1]
                e1, e2 = v[1] - v[0], v[2] - v[0]
            off = lat[:, 0:1] * e1[None, :] + lat[:, 1:2] * e2[None, :] + lat[:, 2:3] * e3[None, :]
            off = off + p * v[0][None, :]
            parts.append(nid(p * ci[:, None] + off[None, :, 0], p * cj[:, None] + off[None, :, 1],
                             p * ck[:, None] + off[None, :, 2]))
        conn = np.stack(parts, axis=1).reshape(-1, lat.shape[0])
    conn = conn.astype(np.int64) + 1

    groups = {"body": Group("body", 3, np.arange(NX * NY * NZ, dtype=np.int64) + 1, fam, p, conn)}
    bfam = TRI if simplex else QUAD
    blat = node_lattice(bfam, p)

    def face(name, axis, idx):
        # in-plane axes (u, v) chosen so that u x v points along +axis
        u, v = {0: (1, 2), 1: (2, 0), 2: (0, 1)}[axis]
        nu = (nx, ny, nz)[u]
        nv = (nx, ny, nz)[v]
        cu, cv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="xy")
        cu, cv = cu.ravel(), cv.ravel()
        if not simplex:
            lu = p * cu[:, None] + blat[None, :, 0]
            lv = p * cv[:, None] + blat[None, :, 1]
            coords = [None, None, None]
            coords[u], coords[v] = lu, lv
            coords[axis] = np.full_like(lu, idx)
            c = nid(coords[0], coords[1], coords[2])
        else:
            parts = []
            for v0, v1, v2 in [((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1))]:
                e1 = np.subtract(v1, v0)
                e2 = np.subtract(v2, v0)
                ou = p * v0[0] + blat[:, 0] * e1[0] + blat[:, 1] * e2[0]
                ov = p * v0[1] + blat[:, 0] * e1[1] + blat[:, 1] * e2[1]
                lu = p * cu[:, None] + ou[None, :]
                lv = p * cv[:, None] + ov[None, :]
                coords = [None, None, None]
                coords[u], coords[v] = lu, lv
                coords[axis] = np.full_like(lu, idx)
                parts.append(nid(coords[0], coords[1], coords[2]))
            c = np.stack(parts, axis=1).reshape(-1, blat.shape[0])
        c = (c + 1).astype(np.int64)
        groups[name] = Group(name, 2, np.unique(c), bfam, p, c)

    face("left", 0, 0)
    face("right", 0, NX - 1)
    face("bottom", 1, 0)
    face("top", 1, NY - 1)
    face("rear", 2, 0)
    face("front", 2, NZ - 1)
    m = Mesh(3, fam, p, xyz, conn, groups, name="structured_box")
    return set_current(m)


def concat_meshes(meshes, sep="#") -> tuple[Mesh, np.ndarray]:
    """Several independent meshes of one family/order as one mesh (one
    assembly launch, one block-diagonal matrix).  Instance i keeps its node
    and element order; its groups are renamed "<name><sep><i>".  Returns the
    combined mesh and node offsets (length n+1), so instance i owns nodes
    offsets[i]..offsets[i+1]-1 (0-based)."""
    if not meshes:
        raise ValueError("concat_meshes: no meshes")
    m0 = meshes[0]
    for m in meshes:
        if (m.dim, m.family, m.order) != (m0.dim, m0.family, m0.order):
            raise ValueError("concat_meshes: all meshes must share dimension, family and order")
    noff = np.zeros(len(meshes) + 1, dtype=np.int64)
    eoff = np.zeros(len(meshes) + 1, dtype=np.int64)
    for i, m in enumerate(meshes):
        noff[i + 1] = noff[i] + m.non
        eoff[i + 1] = eoff[i] + m.nel
    xyz = np.concatenate([m.xyz for m in meshes], axis=0)
    conn = np.concatenate([m.conn + noff[i] for i, m in enumerate(meshes)], axis=0)
    groups = {}
    for i, m in enumerate(meshes):
        for name, g in m.groups.items():
            c = None if g.conn is None else g.conn + noff[i]
            ng = Group(f"{name}{sep}{i}", g.dim, g.nodes + noff[i], g.family, g.order, c)
            if g.dim == m.dim:
                ng.elems = np.arange(eoff[i], eoff[i + 1])
            groups[ng.name] = ng
    out = Mesh(m0.dim, m0.family, m0.order, xyz, conn, groups, name="batch")
    set_current(out)
    return out, noff


# --------------------------------------------------------------------------
# MSH 4.1 ASCII reader
# --------------------------------------------------------------------------
def read_msh(path: str) -> Mesh:
    """Read an MSH 4.1 ASCII file: nodes, elements of the highest dimension,
    and every physical group (with its boundary elements)."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    pos = 0

    def section(name):
        nonlocal pos
        while pos < len(lines) and lines[pos].strip() != f"${name}":
            pos += 1
        if pos >= len(lines):
            return False
        pos += 1
        return True

    if not section("MeshFormat"):
        raise ValueError("not an MSH file")
    ver = lines[pos].split()[0]
    if not ver.startswith("4"):
        raise ValueError(f"MSH version {ver} not supported (4.1 ASCII only)")
    phys_names = {}
    save = pos
    if section("PhysicalNames"):
        cnt = int(lines[pos]); pos += 1
        for _ in range(cnt):
            parts = lines[pos].split(None, 2); pos += 1
            phys_names[(int(parts[0]), int(parts[1]))] = parts[2].strip().strip('"')
    else:
        pos = save
    # entities -> physical tags
    ent_phys = {}
    pos = save
    section("Entities")
    npts, ncur, nsur, nvol = map(int, lines[pos].split()); pos += 1
    for dim, cnt in ((0, npts), (1, ncur), (2, nsur), (3, nvol)):
        for _ in range(cnt):
            v = lines[pos].split(); pos += 1
            tag = int(v[0])
            if dim == 0:
                nph = int(v[4]); ph = [int(x) for x in v[5:5 + nph]]
            else:
                nph = int(v[7]); ph = [int(x) for x in v[8:8 + nph]]
            ent_phys[(dim, tag)] = ph
    section("Nodes")
    nblocks, nnodes, mintag, maxtag = map(int, lines[pos].split()); pos += 1
    if mintag != 1 or maxtag != nnodes:
        raise ValueError("node tags must be dense 1..non (src/multifield.jl:1602-1611)")
    xyz = np.zeros((nnodes, 3))
    ent_nodes = {}
    for _ in range(nblocks):
        edim, etag, param, cnt = map(int, lines[pos].split()); pos += 1
        tags = np.array([int(lines[pos + i]) for i in range(cnt)], dtype=np.int64)
        pos += cnt
        if cnt:
            block = np.array([list(map(float, lines[pos + i].split()[:3])) for i in range(cnt)])
            xyz[tags - 1] = block
        pos += cnt
        ent_nodes[(edim, etag)] = tags
    section("Elements")
    nblocks, nelem, _, _ = map(int, lines[pos].split()); pos += 1
    blocks = []
    for _ in range(nblocks):
        edim, etag, etype, cnt = map(int, lines[pos].split()); pos += 1
        rows = np.array([list(map(int, lines[pos + i].split())) for i in range(cnt)], dtype=np.int64)
        pos += cnt
        blocks.append((edim, etag, etype, rows))
    dim = max(b[0] for b in blocks)
    vol = [b for b in blocks if b[0] == dim]
    types = {b[2] for b in vol}
    if len(types) != 1:
        raise ValueError("one volume element type per mesh is supported")
    etype = types.pop()
    fam, order = GMSH_TYPES.get(etype, (None, 0))
    if fam is None:
        raise ValueError(f"gmsh element type {etype} not supported")
    conn = np.concatenate([b[3][:, 1:] for b in vol], axis=0)
    groups = {}
    for (pdim_, ptag), name in phys_names.items():
        ents = [(d, t) for (d, t), ph in ent_phys.items() if d == pdim_ and ptag in ph]
        nodes, econn, bfam, border = [], [], 0, 0
        for (d, t) in ents:
            for b in blocks:
                if b[0] == d and b[1] == t:
                    f, o = GMSH_TYPES.get(b[2], (None, 0))
                    econn.append(b[3][:, 1:])
                    nodes.append(b[3][:, 1:].ravel())
                    bfam, border = f or 0, o
            if d == 0 and (d, t) in ent_nodes:
                nodes.append(ent_nodes[(d, t)])
        nodes = np.unique(np.concatenate(nodes)) if nodes else np.zeros(0, dtype=np.int64)
        c = np.concatenate(econn, axis=0) if econn and pdim_ > 0 else None
        groups[name] = Group(name, pdim_, nodes, bfam, border, c)
    m = Mesh(dim, fam, order, xyz, conn, groups, name=path)
    return set_current(m)
