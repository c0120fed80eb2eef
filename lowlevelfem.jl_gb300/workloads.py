"""Seeded synthetic workloads with the shapes, sizes and value distributions
of the accelerated path's configurations (the reference's meshes come from
gmsh; these generators stand in for them):

* ``batched_instance``: an independent 3D tet10 box — element count
  log-uniform in [1e3, 2e5], edge lengths uniform in [0.5, 2], E uniform in
  [1e4, 3e5], nu uniform in [0.2, 0.45]; clamped on "left", unit traction on
  "right".
* ``heat_request``: a steady heat-conduction request — DoFs log-uniform in
  [1e3, 1e6], Lagrange order uniform in 1..4, triangles (2D) or tetrahedra
  (3D) 50/50, conductivity log-normal(0, 1), random Dirichlet temperatures
  on two opposite faces.
"""
from __future__ import annotations

import math

import numpy as np

from . import mesh as _mesh

SEED = 20261203


def batched_instance(rng: np.random.Generator, ne_min=1e3, ne_max=2e5):
    ne = math.exp(rng.uniform(math.log(ne_min), math.log(ne_max)))
    lx, ly, lz = rng.uniform(0.5, 2.0, size=3)
    d = (lx * ly * lz * 6.0 / ne) ** (1.0 / 3.0)
    m = _mesh.structured_box_mesh(lx=lx, ly=ly, lz=lz, dx=d, dy=d, order=2, simplex=True)
    E = float(rng.uniform(1e4, 3e5))
    nu = float(rng.uniform(0.2, 0.45))
    return m, E, nu


def heat_request(rng: np.random.Generator, dofs_min=1e3, dofs_max=1e6, orders=(1, 2, 3, 4), cache=None):
    """One request (mesh, k, fixed, x0).  cache (a dict, optional) shares
    meshes between requests of the same shape (dimension, cells per edge,
    order); the random draws are the same with or without it."""
    dofs = math.exp(rng.uniform(math.log(dofs_min), math.log(dofs_max)))
    p = int(rng.choice(orders))
    three_d = bool(rng.integers(0, 2))
    if three_d:
        n = max(1, int(round((dofs ** (1.0 / 3.0) - 1.0) / p)))
    else:
        n = max(1, int(round((math.sqrt(dofs) - 1.0) / p)))
    key = (three_d, n, p)
    m = cache.get(key) if cache is not None else None
    if m is None:
        m = (_mesh.structured_box_mesh(n=n, order=p, simplex=True) if three_d
             else _mesh.structured_rect_mesh(n=n, order=p, simplex=True))
        if cache is not None:
            cache[key] = m
    faces = ("left", "right")
    k = float(math.exp(rng.normal(0.0, 1.0)))
    fixed = np.zeros(m.non, dtype=np.uint8)
    x0 = np.zeros(m.non)
    for f in faces:
        nodes = m.group(f).nodes - 1
        fixed[nodes] = 1
        x0[nodes] = rng.uniform(0.0, 100.0)
    return m, k, fixed, x0
