"""Host logic: structured meshes, MSH reader, DoF maps, material constants."""
import os

import numpy as np
import pytest

from conftest import REFERENCE

MSH = os.path.join(REFERENCE, "examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/elasticity_benchmark.msh") \
    if REFERENCE else ""


def test_config_sizes(llf):
    m = llf.structured_rect_mesh(lx=10.0, ly=5.0, dx=0.05, dy=0.05)
    assert (m.non, m.nel) == (20301, 20000)
    m = llf.structured_box_mesh(n=40, order=2)
    assert (m.non, m.nel, m.npe) == (531441, 64000, 27)


def test_d_is_min_dx_dy(llf):
    # n=200 on a 10x5 rectangle: d = min(0.05, 0.025) -> 400 x 200 cells
    m = llf.structured_rect_mesh(lx=10.0, ly=5.0, n=200)
    assert m.nel == 400 * 200


def test_generator_matches_reference_msh(llf):
    """The structured generator and the reference's elasticity_benchmark.msh
    (rebuilt from tests/golden/) hold the same node set and group sizes."""
    from helpers import benchmark_msh_mesh
    ref = benchmark_msh_mesh(llf)
    gen = llf.structured_box_mesh(n=30)
    assert ref.nel == gen.nel == 27000 and ref.non == gen.non == 29791
    a = np.round(np.sort(ref.xyz.view([("", float)] * 3), axis=0).view(float).reshape(-1, 3), 12)
    key = lambda x: np.lexsort(np.round(x, 12).T[::-1])
    assert np.allclose(ref.xyz[key(ref.xyz)], gen.xyz[key(gen.xyz)], atol=1e-12)
    for name in ("left", "right", "front", "rear", "bottom", "top"):
        assert len(ref.group(name).nodes) == len(gen.group(name).nodes) == 961


def test_groups_rect(llf):
    m = llf.structured_rect_mesh()
    assert set(m.groups) >= {"left", "right", "top", "bottom", "body", "leftbottom"}
    assert np.all(np.abs(m.xyz[m.group("left").nodes - 1, 0]) < 1e-14)
    assert np.all(np.abs(m.xyz[m.group("top").nodes - 1, 1] - 1) < 1e-14)


def test_elastic_constants(llf):
    ec = llf.elastic_constants()
    assert ec["E"] == 2e5 and ec["nu"] == 0.3
    assert abs(ec["mu"] - 2e5 / 2.6) < 1e-9
    ec2 = llf.elastic_constants(lam=ec["lam"], mu=ec["mu"])
    assert abs(ec2["E"] - 2e5) < 1e-6 and abs(ec2["nu"] - 0.3) < 1e-12
    with pytest.raises(ValueError):
        llf.elastic_constants(E=1.0, nu=0.3, mu=1.0)


def test_dof_maps(llf):
    llf.structured_rect_mesh(n=2)
    p = llf.Problem([llf.Material("body")], type="PlaneStress")
    bc = [llf.displacementConstraint("left", ux=0), llf.displacementConstraint("bottom", uy=0)]
    c = llf.constrainedDoFs(p, bc)
    left = p.mesh.group("left").nodes
    bottom = p.mesh.group("bottom").nodes
    assert set(c.tolist()) == set(((left - 1) * 2 + 1).tolist()) | set(((bottom - 1) * 2 + 2).tolist())
    f = llf.freeDoFs(p, bc)
    assert len(f) + len(c) == 2 * p.non and not set(f) & set(c)


def test_problem_type_errors(llf):
    llf.structured_rect_mesh(n=2)
    with pytest.raises(ValueError):
        llf.Problem(llf.Material("body"), type="PlaneStress")
    with pytest.raises(ValueError):
        llf.Problem([llf.Material("body")], type="Solid")  # 3D problem on a 2D mesh


@pytest.mark.skipif(not MSH or not os.path.exists(MSH), reason="set LLF_REFERENCE_DIR to a reference checkout")
def test_msh_reader_matches_fixture(llf):
    """read_msh on the reference's file gives the committed fixture bit for bit."""
    from helpers import benchmark_msh_mesh
    fx = benchmark_msh_mesh(llf)
    m = llf.read_msh(MSH)
    assert np.array_equal(m.xyz.view(np.int64), fx.xyz.view(np.int64)) and np.array_equal(m.conn, fx.conn)
