"""VTU output (written without meshio) and multi-layer stacking, on the CPU."""
import numpy as np

from jax_am_gb300.phase_field.utils import Field, cell_centroids, generate_new_mesh
from jax_am_gb300.phase_field.vtu import read_vtu, write_vtu


def test_vtu_round_trip_and_hexahedra(tmp_path):
    shape, h = (5, 4, 3), (1e-6, 2e-6, 0.5e-6)
    N = 60
    rng = np.random.default_rng(0)
    T = rng.random(N).astype(np.float32)
    ori = rng.integers(0, 7, N).astype(np.int32)
    vec = rng.random((N, 3))
    path = write_vtu(str(tmp_path / "u000.vtu"), shape, h, {"T": T, "ori_inds": ori, "v": vec})
    d = read_vtu(path)
    np.testing.assert_array_equal(d["T"], T)
    np.testing.assert_array_equal(d["ori_inds"], ori)
    np.testing.assert_array_equal(d["v"], vec)
    assert (d["types"] == 12).all() and d["offsets"][-1] == 8 * N
    pts = d["Points"].astype(np.float64)
    corners = pts[d["connectivity"].reshape(N, 8)]
    # every cell's corners average to its centre, in the cell order of the data
    np.testing.assert_allclose(corners.mean(axis=1), cell_centroids(shape, h), rtol=1e-6)
    # VTK hexahedron order: bottom face counter-clockwise, top face above it
    c0 = corners[0]
    np.testing.assert_allclose(c0[1] - c0[0], [h[0], 0, 0], atol=1e-12)
    np.testing.assert_allclose(c0[3] - c0[0], [0, h[1], 0], atol=1e-12)
    np.testing.assert_allclose(c0[4] - c0[0], [0, 0, h[2]], atol=1e-12)


def test_generate_new_mesh_stacks_layers():
    args = dict(Nx=6, Ny=5, Nz=4, h=1e-6, num_grains=7, num_oris=5)
    base = Field(dict(args), seed=2)
    two = generate_new_mesh(args, base.quaternions, base, 1)
    three = generate_new_mesh(args, base.quaternions, two, 2)
    assert two.shape_xyz == (6, 5, 8) and three.shape_xyz == (6, 5, 12)
    np.testing.assert_array_equal(two.cell_ori_inds[:120], base.cell_ori_inds)
    np.testing.assert_array_equal(three.cell_ori_inds[:240], two.cell_ori_inds)
    # the new layer's cells sit one domain height above the previous ones
    np.testing.assert_allclose(three.centroids[240:, 2] - three.centroids[:120, 2], 8e-6)
    np.testing.assert_allclose(two.unique_grain_directions, base.unique_grain_directions)
