"""Embedded-boundary geometries (eb2.geom_type): the driver's host flags
(used for grid tagging) and the GPU flags kernel (mbg_geometry_flags, used to
define the levels) must agree bit for bit; the sphere also against the
oracle.  CPU tests check the host classification on analytic cases."""
import numpy as np
import pytest

import cases

BASE = """
geometry.prob_lo = 0.0 0.0 0.0
geometry.prob_hi = 32.0 24.0 16.0
geometry.is_periodic = 0 1 1
amr.n_cell = 32 24 16
amr.max_level = 0
amr.max_grid_size = 16
lbm.bc_lo = 2 0 0
lbm.bc_hi = 5 0 0
lbm.nu = 0.016
lbm.velocity_bc_type = "constant"
velocity_bc_constant.dir = 0
velocity_bc_constant.Mach_ref = 0.05
velocity_bc_constant.initial_temperature = 0.03
lbm.ic_type = "constant"
ic_constant.density = 1.0
ic_constant.mach_components = 0.05 0.0 0.0
ic_constant.initial_temperature = 0.03
"""

GEOMS = {
    "sphere": 'eb2.geom_type = "sphere"\neb2.sphere_radius = 4.5\neb2.sphere_center = 12.0 12.0 8.0\n'
              "eb2.sphere_has_fluid_inside = 0\n",
    "box": 'eb2.geom_type = "box"\neb2.box_lo = 10.0 8.5 4.0\neb2.box_hi = 16.0 15.5 12.0\n'
           "eb2.box_has_fluid_inside = 0\n",
    "cylinder": 'eb2.geom_type = "cylinder"\neb2.cylinder_radius = 3.5\neb2.cylinder_height = -1.0\n'
                "eb2.cylinder_direction = 2\neb2.cylinder_center = 12.0 12.0 8.0\n"
                "eb2.cylinder_has_fluid_inside = 0\n",
    "plane": 'eb2.geom_type = "plane"\neb2.plane_point = 0.0 20.5 0.0\neb2.plane_normal = 0.0 1.0 0.0\n',
    "rotated_box": 'eb2.geom_type = "rotated_box"\neb2.box_lo = 10.0 8.0 4.0\neb2.box_hi = 16.0 16.0 12.0\n'
                   "eb2.box_has_fluid_inside = 0\neb2.box_rotation = 30.0\neb2.box_rotation_axe = 2\n"
                   "eb2.box_rotation_center = 13.0 12.0 8.0\n",
    "rotated_cylinder": 'eb2.geom_type = "rotated_cylinder"\neb2.cylinder_radius = 3.0\n'
                        "eb2.cylinder_direction = 2\neb2.cylinder_center = 12.0 12.0 8.0\n"
                        "eb2.cylinder_has_fluid_inside = 0\neb2.cylinder_rotation = 20.0\n"
                        "eb2.cylinder_rotation_axe = 0\n",
    "extruded_triangles": 'eb2.geom_type = "extruded_triangles"\nextruded_triangles.num_tri = 2\n'
                          "extruded_triangles.tri_0_point_0 = 8.0 6.0 0.0\n"
                          "extruded_triangles.tri_0_point_1 = 16.0 6.0 0.0\n"
                          "extruded_triangles.tri_0_point_2 = 12.0 14.0 0.0\n"
                          "extruded_triangles.tri_1_point_0 = 18.0 10.0 0.0\n"
                          "extruded_triangles.tri_1_point_1 = 24.0 10.0 0.0\n"
                          "extruded_triangles.tri_1_point_2 = 21.0 18.0 0.0\n",
}


def _driver(name):
    import marbles_gb300 as M
    d = M.LBM(BASE + GEOMS[name])
    d.prepare()
    return d


def _valid_fluid(d, lev=0):
    """is_fluid of the valid cells, global (z, y, x) array of the level."""
    boxes, fl = d.boxes(lev), d.flags(lev)
    hi = boxes[:, 3:].max(axis=0) + 1
    out = -np.ones((hi[2], hi[1], hi[0]), dtype=np.int32)
    off = 0
    for b in boxes:
        nx, ny, nz = (int(v) for v in b[3:] - b[:3] + 1)
        g = fl[off:off + (nx + 6) * (ny + 6) * (nz + 6)].reshape(nz + 6, ny + 6, nx + 6)
        out[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = g[3:-3, 3:-3, 3:-3] & 1
        off += (nx + 6) * (ny + 6) * (nz + 6)
    return out


def _corner_covered(phi):
    z, y, x = np.meshgrid(np.arange(16), np.arange(24), np.arange(32), indexing="ij")
    cov = np.ones(x.shape, dtype=bool)
    for c in range(8):
        cov &= phi(x + (c & 1), y + ((c >> 1) & 1), z + ((c >> 2) & 1)) >= 0
    return cov


@pytest.mark.parametrize("name,phi", [
    ("box", lambda x, y, z: np.minimum.reduce([x - 10.0, 16.0 - x, y - 8.5, 15.5 - y, z - 4.0, 12.0 - z])),
    ("cylinder", lambda x, y, z: 3.5 ** 2 - ((x - 12.0) ** 2 + (y - 12.0) ** 2)),
    ("plane", lambda x, y, z: y - 20.5),
])
def test_host_classification_matches_implicit_function(name, phi):
    d = _driver(name)
    isf = _valid_fluid(d)
    assert (isf == np.where(_corner_covered(phi), 0, 1)).all()


def test_extruded_triangles_cover_their_interiors():
    d = _driver("extruded_triangles")
    isf = _valid_fluid(d)
    # cells well inside each triangle are covered in every z-plane, far cells fluid
    assert (isf[:, 8, 11] == 0).all() and (isf[:, 12, 20] == 0).all()
    assert (isf[:, 2, 2] == 1).all() and (isf[:, 20, 28] == 1).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GEOMS))
def test_gpu_flags_equal_host_flags(name):
    d = _driver(name)
    host = d.flags(0)
    d.init()               # init_data defines the levels with the GPU flags
    gpu = d.flags(0)
    assert np.array_equal(host, gpu)
    assert (gpu & 1).sum() < gpu.size        # the geometry covers something


@pytest.mark.gpu
def test_gpu_sphere_flags_match_oracle():
    import marbles_gb300 as M
    p, levels = cases.sphere_channel(32, 24, 16, radius=4.5, center=(12.0, 12.0, 8.0), mgs=16, t0=0.03)
    o = cases.run_oracle(p, levels, 0)
    d = M.LBM(BASE + GEOMS["sphere"])
    d.init()
    assert np.array_equal(d.flags(0), o.get_grown_flags(0))
