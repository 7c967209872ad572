"""Polycrystal inputs: the drop-in for JAX-AM's ``Field``
(``jax_am/phase_field/utils.py:19-149``).

The reference reads a Neper Voronoi tessellation meshed to one hexahedron per
cell (``neper.py:16-19``, ``-regularization 0``), draws each grain's
orientation index with ``randint(num_oris)`` (``utils.py:39-40``) and turns
``num_oris`` random orientations into the three rotated cube axes that the
anisotropy term uses (``utils.py:104-109``).  Neper is not available, so
``Field`` builds the same model itself: ``num_grains`` seeds uniform in the
box, each cell assigned to its nearest seed (periodic distance on periodic
axes), orientations uniform on SO(3) (Shoemake's subgroup algorithm) stored
scalar-first as orix does.  IPF colouring and file output
(``utils.py:93-102,111-147``) are plotting only and are not reproduced.
"""
import numpy as np
from scipy.spatial import cKDTree
from scipy.spatial.transform import Rotation


def random_quaternions(n, rng):
    """``n`` unit quaternions uniform on SO(3), scalar-first (w, x, y, z)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    x, y = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    z, w = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    return np.stack((w, x, y, z), axis=1)


def grain_directions(quats):
    """(3, n, 3): the cube axes e_x, e_y, e_z rotated by each orientation
    (``utils.py:104-109``; the quaternion is converted to scipy's
    scalar-last order first, ``utils.py:107``)."""
    q = np.asarray(quats, dtype=np.float64)
    r = Rotation.from_quat(np.concatenate((q[:, 1:], q[:, :1]), axis=1))
    return np.stack((r.apply([1.0, 0.0, 0.0]), r.apply([0.0, 1.0, 0.0]), r.apply([0.0, 0.0, 1.0])))


def _bc_tuple(bc):
    if bc is None:
        return ("neumann",) * 3
    if isinstance(bc, str):
        return (bc,) * 3
    return tuple(bc)


def voronoi_grains(shape_xyz, h, num_grains, rng, periodic=(False, False, False),
                   chunk=1 << 21):
    """Nearest-seed grain index for every cell centre, cells in z-major order.

    Returns (cell_grain_inds (N,), seeds (num_grains, 3))."""
    Nx, Ny, Nz = shape_xyz
    box = np.array([Nx * h[0], Ny * h[1], Nz * h[2]])
    seeds = rng.random((num_grains, 3)) * box
    big = 1e30  # a box size that never wraps: non-periodic axis
    boxsize = np.where(np.array(periodic), box, big)
    tree = cKDTree(seeds, boxsize=boxsize)
    xs = (np.arange(Nx) + 0.5) * h[0]
    ys = (np.arange(Ny) + 0.5) * h[1]
    zs = (np.arange(Nz) + 0.5) * h[2]
    N = Nx * Ny * Nz
    inds = np.empty(N, dtype=np.int64)
    plane = Nx * Ny
    zz_per = max(1, chunk // plane)
    for z0 in range(0, Nz, zz_per):
        z1 = min(Nz, z0 + zz_per)
        Z, Y, X = np.meshgrid(zs[z0:z1], ys, xs, indexing="ij")
        pts = np.stack((X.ravel(), Y.ravel(), Z.ravel()), axis=1)
        _, idx = tree.query(pts, workers=-1)
        inds[z0 * plane:z1 * plane] = idx
    return inds, seeds


def cell_centroids(shape_xyz, h):
    """(N, 3) cell-centre coordinates, cells in z-major order (x fastest)."""
    Nx, Ny, Nz = shape_xyz
    xs = (np.arange(Nx) + 0.5) * h[0]
    ys = (np.arange(Ny) + 0.5) * h[1]
    zs = (np.arange(Nz) + 0.5) * h[2]
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack((X.ravel(), Y.ravel(), Z.ravel()), axis=1)


class Field:
    """Polycrystal and grain orientations for ``PFSolver``.

    ``pf_args`` needs ``num_grains``, ``num_oris`` and the grid: ``Nx, Ny,
    Nz`` together with ``domain_x/y/z`` (cell size = domain / N, as
    ``utils.py:55-57``), or ``Nx, Ny, Nz`` with ``h`` (one size or three).
    ``Nx, Ny, Nz`` are written back into ``pf_args`` as the reference does
    (``utils.py:47-49``).  ``ori2`` optionally gives the orientations as a
    (num_oris, 4) scalar-first quaternion array.  ``seed`` seeds every draw
    (the reference seeds NumPy's global generator with 1, ``utils.py:16``).
    """

    def __init__(self, pf_args, ori2=None, seed=1):
        self.pf_args = pf_args
        self.rng = np.random.default_rng(seed)
        Nx, Ny, Nz = int(pf_args["Nx"]), int(pf_args["Ny"]), int(pf_args["Nz"])
        if "h" in pf_args:
            h = pf_args["h"]
            h = (float(h),) * 3 if np.isscalar(h) else tuple(float(v) for v in h)
            pf_args.setdefault("domain_x", Nx * h[0])
            pf_args.setdefault("domain_y", Ny * h[1])
            pf_args.setdefault("domain_z", Nz * h[2])
        self.mesh_h_xyz = (pf_args["domain_x"] / Nx, pf_args["domain_y"] / Ny,
                           pf_args["domain_z"] / Nz)
        bc = _bc_tuple(pf_args.get("bc"))
        periodic = tuple(b == "periodic" for b in bc)
        grains, seeds = voronoi_grains((Nx, Ny, Nz), self.mesh_h_xyz,
                                       int(pf_args["num_grains"]), self.rng, periodic)
        self.shape_xyz = (Nx, Ny, Nz)
        self.cell_grain_inds = grains
        self.seeds = seeds
        self._centroids = None
        n = int(pf_args["num_oris"])
        grain_oris_inds = self.rng.integers(0, n, size=int(pf_args["num_grains"]))
        self.cell_ori_inds = np.take(grain_oris_inds, grains)
        if ori2 is None:
            self.quaternions = random_quaternions(n, self.rng)
        else:
            self.quaternions = np.asarray(getattr(ori2, "data", ori2), dtype=np.float64)
            assert self.quaternions.shape == (n, 4), "ori2 must hold num_oris quaternions"
        self.unique_grain_directions = grain_directions(self.quaternions)
        pf_args["Nx"], pf_args["Ny"], pf_args["Nz"] = Nx, Ny, Nz

    @property
    def centroids(self):
        """(N, 3) cell centres (``utils.py:53-54``), built on first use."""
        if self._centroids is None:
            self._centroids = cell_centroids(self.shape_xyz, self.mesh_h_xyz)
        return self._centroids


class StackedField:
    """Several layers of polycrystal stacked along z (what the reference's
    ``generate_new_mesh`` builds for multi-layer runs, ``utils.py:151-179``):
    cells of the lower layers first, the new layer's cells on top (z-major
    order, so concatenation is stacking); grain directions are those of the
    newest layer (every layer is built from the same ``ori2``)."""

    def __init__(self, lower, upper):
        Nx, Ny, Nz_l = lower.shape_xyz
        Ux, Uy, Nz_u = upper.shape_xyz
        if (Nx, Ny) != (Ux, Uy) or tuple(lower.mesh_h_xyz) != tuple(upper.mesh_h_xyz):
            raise ValueError("layers must share Nx, Ny and the cell size")
        self.shape_xyz = (Nx, Ny, Nz_l + Nz_u)
        self.mesh_h_xyz = tuple(lower.mesh_h_xyz)
        self.cell_ori_inds = np.concatenate((lower.cell_ori_inds, upper.cell_ori_inds))
        self.cell_grain_inds = np.concatenate((lower.cell_grain_inds, upper.cell_grain_inds))
        self.quaternions = upper.quaternions
        self.unique_grain_directions = upper.unique_grain_directions
        self._centroids = None

    @property
    def centroids(self):
        if self._centroids is None:
            self._centroids = cell_centroids(self.shape_xyz, self.mesh_h_xyz)
        return self._centroids


def generate_new_mesh(pf_args, ori2, polycrystal, layer, seed=None):
    """A new layer of ``pf_args``'s grid (its own Voronoi grains, the
    orientations ``ori2``) stacked on top of ``polycrystal``, as the
    reference's ``generate_new_mesh`` (``utils.py:151-179``) does: the new
    layer's cells sit ``layer`` domain heights up.  Run the stacked
    polycrystal with ``Nz`` = the total number of cell layers in ``pf_args``."""
    upper = Field(dict(pf_args), ori2, seed=1 + int(layer) if seed is None else seed)
    return StackedField(polycrystal, upper)
