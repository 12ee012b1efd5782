"""Element stiffness and seeded synthetic voxel domains.

The reference ships one model (armadillo_128) and no generator; the workloads
below are the seeded synthetic stand-ins for the benchmark configurations
(cantilever 32x16x16, 128^3 correlated porous field, 256^3 box with spherical
voids and lognormal modulus, 64^3 training fields, 384^3 porous field).

Conventions shared with the reference (``include/utils.hpp:85-86``,
``src/FEM.cpp:66-198``):
* voxel arrays are indexed ``[z, y, x]`` (x fastest in memory);
* a node is *used* when at least one filled voxel touches it, and used nodes are
  numbered 0.. in increasing linear order over the (nx+1)(ny+1)(nz+1) node grid;
* element-local node ``a = dx + 2 dy + 4 dz`` and local DOF ``3 a + c``.
"""
from dataclasses import dataclass, field
from typing import Optional

import numpy as np


def hex8_stiffness(E=1.0, nu=0.3):
    """24x24 stiffness of a unit trilinear hexahedron, 2x2x2 Gauss quadrature.

    Node order x fastest (a = dx + 2dy + 4dz), DOF 3a + c.  For E=1, nu=0.3 this
    is the reference's ``data/Ke0.dat`` up to the node permutation that the
    GMGS-3D exporter applies (``scripts/outputToC.m:13-14``); 1872*Ke is an
    integer matrix with entries of magnitude <= 440.
    """
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2 * mu
    D[3, 3] = D[4, 4] = D[5, 5] = mu
    g = np.array([-1.0, 1.0]) / np.sqrt(3.0)
    nodes = [(dx, dy, dz) for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)]
    Ke = np.zeros((24, 24))
    for gz in g:
        for gy in g:
            for gx in g:
                xi = ((gx + 1) / 2, (gy + 1) / 2, (gz + 1) / 2)
                B = np.zeros((6, 24))
                for a, (dx, dy, dz) in enumerate(nodes):
                    fx = xi[0] if dx else 1 - xi[0]
                    fy = xi[1] if dy else 1 - xi[1]
                    fz = xi[2] if dz else 1 - xi[2]
                    sx, sy, sz = (1 if dx else -1), (1 if dy else -1), (1 if dz else -1)
                    d = (sx * fy * fz, fx * sy * fz, fx * fy * sz)
                    B[0, 3 * a] = d[0]
                    B[1, 3 * a + 1] = d[1]
                    B[2, 3 * a + 2] = d[2]
                    B[3, 3 * a], B[3, 3 * a + 1] = d[1], d[0]
                    B[4, 3 * a + 1], B[4, 3 * a + 2] = d[2], d[1]
                    B[5, 3 * a], B[5, 3 * a + 2] = d[2], d[0]
                Ke += B.T @ D @ B / 8.0
    return 0.5 * (Ke + Ke.T)


# Node permutation between the reference's Ke0.dat local order and the x-fastest
# order: Ke0[3i+c, 3j+d] == hex8_stiffness()[3P[i]+c, 3P[j]+d].
KE0_NODE_PERM = (2, 0, 3, 1, 6, 4, 7, 5)


def used_nodes_mask(voxels):
    """Boolean [nz+1, ny+1, nx+1] mask of nodes touched by a filled voxel."""
    v = np.asarray(voxels, dtype=bool)
    sz, sy, sx = v.shape
    m = np.zeros((sz + 1, sy + 1, sx + 1), dtype=bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                m[dz:dz + sz, dy:dy + sy, dx:dx + sx] |= v
    return m


def node_numbering(voxels):
    """Compressed node ids on the node grid (-1 for unused), reference order."""
    m = used_nodes_mask(voxels)
    ids = np.full(m.shape, -1, dtype=np.int64)
    ids[m] = np.arange(int(m.sum()), dtype=np.int64)
    return ids


@dataclass
class Domain:
    """A voxel problem: occupancy, optional per-voxel modulus, fixed nodes, loads."""
    name: str
    voxels: np.ndarray                     # uint8 [z, y, x]
    fixed: np.ndarray                      # int64 compressed node ids
    load_nodes: np.ndarray                 # int64 compressed node ids
    load_values: np.ndarray                # float64 [n, 3]
    E: Optional[np.ndarray] = None         # float32 [z, y, x] or None (uniform 1)
    num_levels: int = 3
    seed: Optional[int] = None
    meta: dict = field(default_factory=dict)

    @property
    def shape(self):
        return self.voxels.shape

    @property
    def num_nodes(self):
        return int(used_nodes_mask(self.voxels).sum())

    @property
    def num_dofs(self):
        return 3 * self.num_nodes

    def load_vector(self):
        f = np.zeros(self.num_dofs, np.float64)
        f.reshape(-1, 3)[self.load_nodes] = self.load_values
        return f


def _face_bcs(voxels, load_total=-1.0):
    """Fix the used nodes of the z=0 face; spread ``load_total`` in z evenly over
    the used nodes of the highest node plane that has any."""
    ids = node_numbering(voxels)
    fixed = ids[0][ids[0] >= 0].reshape(-1)
    for zt in range(ids.shape[0] - 1, -1, -1):
        top = ids[zt][ids[zt] >= 0].reshape(-1)
        if top.size:
            break
    loads = np.zeros((top.size, 3))
    loads[:, 2] = load_total / top.size
    return np.sort(fixed), top, loads


def keep_grounded(voxels):
    """Keep the 6-connected components that touch the z=0 face."""
    from scipy import ndimage
    lab, n = ndimage.label(voxels.astype(bool), structure=ndimage.generate_binary_structure(3, 1))
    keep = np.unique(lab[0][lab[0] > 0])
    return np.isin(lab, keep).astype(np.uint8)


def cantilever(nx=32, ny=16, nz=16, levels=3):
    """Solid box; every node with x=0 fixed; unit total -z load spread over the
    nodes of the x=nx face (one share per node)."""
    vox = np.ones((nz, ny, nx), np.uint8)
    ids = node_numbering(vox)
    fixed = np.sort(ids[:, :, 0].reshape(-1))
    ln = np.sort(ids[:, :, nx].reshape(-1))
    lv = np.zeros((ln.size, 3))
    lv[:, 2] = -1.0 / ln.size
    return Domain("cantilever_%dx%dx%d" % (nx, ny, nz), vox, fixed, ln, lv, None, levels)


def porous(n=128, fill=0.40, sigma=6.0, seed=0, levels=4, lognormal_sigma=None):
    """Seeded Gaussian random field (white noise smoothed with a Gaussian of
    ``sigma`` voxels, periodic) thresholded so that ``fill`` of the voxels are
    solid, restricted to the components touching z=0; z=0 fixed, unit -z load on
    the top face."""
    from scipy import ndimage
    shape = (n, n, n) if np.isscalar(n) else tuple(n)
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape).astype(np.float32)
    field_ = ndimage.gaussian_filter(noise, sigma=sigma, mode="wrap")
    thr = np.quantile(field_, 1.0 - fill)
    vox = keep_grounded(field_ > thr)
    E = None
    if lognormal_sigma:
        E = rng.lognormal(0.0, lognormal_sigma, size=shape).astype(np.float32)
    fixed, ln, lv = _face_bcs(vox)
    return Domain("porous_%s_f%.2f_s%d" % ("x".join(map(str, shape)), fill, seed), vox, fixed, ln, lv,
                  E, levels, seed, {"fill_target": fill, "sigma": sigma})


def spheres(n=256, count=300, rmin=4.0, rmax=16.0, seed=0, levels=5, lognormal_sigma=0.5):
    """Box minus ``count`` seeded spherical voids (centres uniform, radii
    U[rmin, rmax]); per-voxel E ~ lognormal(0, sigma); grounded component only;
    z=0 fixed, unit -z load on the top face."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    vox = np.ones(shape, np.uint8)
    centres = rng.uniform(0, n, size=(count, 3))
    radii = rng.uniform(rmin, rmax, size=count)
    for (cz, cy, cx), r in zip(centres, radii):
        lo = np.maximum(np.floor([cz - r, cy - r, cx - r]).astype(int), 0)
        hi = np.minimum(np.ceil([cz + r, cy + r, cx + r]).astype(int) + 1, n)
        zz, yy, xx = np.ogrid[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        inside = ((zz + 0.5 - cz) ** 2 + (yy + 0.5 - cy) ** 2 + (xx + 0.5 - cx) ** 2) <= r * r
        vox[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]][inside] = 0
    vox = keep_grounded(vox)
    E = rng.lognormal(0.0, lognormal_sigma, size=shape).astype(np.float32) if lognormal_sigma else None
    fixed, ln, lv = _face_bcs(vox)
    return Domain("spheres_%d_c%d_s%d" % (n, count, seed), vox, fixed, ln, lv, E, levels, seed,
                  {"count": count, "rmin": rmin, "rmax": rmax})


def training_field(n=64, seed=0, levels=3):
    """A training domain: fill U[0.30, 0.60], a random axis-aligned load patch
    on the top face with total magnitude U[0.1, 1] in -z, z=0 fixed.  Raises
    ValueError when no filled voxel of the field is connected to z = 0."""
    from scipy import ndimage
    rng = np.random.default_rng(seed)
    fill = rng.uniform(0.30, 0.60)
    noise = rng.standard_normal((n, n, n)).astype(np.float32)
    field_ = ndimage.gaussian_filter(noise, sigma=rng.uniform(3.0, 8.0), mode="wrap")
    vox = keep_grounded(field_ > np.quantile(field_, 1.0 - fill))
    ids = node_numbering(vox)
    fixed = np.sort(ids[0][ids[0] >= 0].reshape(-1))
    mag = rng.uniform(0.1, 1.0)
    for zt in range(n, -1, -1):
        plane = ids[zt]
        if (plane >= 0).any():
            break
    for _ in range(64):
        w, h = rng.integers(n // 8, n // 2 + 1, size=2)
        x0, y0 = rng.integers(0, n + 1 - w), rng.integers(0, n + 1 - h)
        patch = plane[y0:y0 + h, x0:x0 + w]
        sel = patch[patch >= 0]
        if sel.size:
            break
    else:
        sel = plane[plane >= 0]
    ln = np.sort(sel.reshape(-1))
    if ln.size == 0:
        raise ValueError("training field %d (seed %d): no filled voxel is connected to z = 0" % (n, seed))
    lv = np.zeros((ln.size, 3))
    lv[:, 2] = -mag / ln.size
    return Domain("train_%d_s%d" % (n, seed), vox, fixed, ln, lv, None, levels, seed,
                  {"fill": fill, "load": mag})
