"""Patch test: analytic known answers for the operator and the solve.

On a solid box of unit trilinear hexahedra (E = 1, nu = 0.3, 2x2x2 Gauss
stiffness) with the z = 0 nodes fixed, a linear displacement field that
vanishes at z = 0 is represented exactly.  Its strain and stress are
constant, so K u is zero at every interior node.  At a boundary node it
equals the consistent nodal load of the traction t = sigma . n on each face
through the node: a quarter of t per adjacent unit face square.  Two fields
are used:

* uniaxial u = (0, 0, eps z): sigma_xx = sigma_yy = lam eps, sigma_zz = (lam + 2 mu) eps;
* shear u = (gam z, 0, 0): sigma_xz = mu gam.

The answers come from continuum mechanics, not from the reference's code, so
they pin the element stiffness, the assembly of the matrix-free product and
the fixed-row handling independently of the oracle.  Solving K u = f with
these loads must return the linear field.
"""
import numpy as np

from vulkanfem_gb300 import domains

E, NU = 1.0, 0.3
LAM = E * NU / ((1 + NU) * (1 - 2 * NU))
MU = E / (2 * (1 + NU))


def box(nx=8, ny=6, nz=5):
    """Solid box voxels [z, y, x], its fixed nodes (z = 0) and node coordinates."""
    vox = np.ones((nz, ny, nx), np.uint8)
    ids = domains.node_numbering(vox)
    fixed = np.sort(ids[0].reshape(-1))
    z, y, x = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([x.reshape(-1), y.reshape(-1), z.reshape(-1)], 1).astype(np.float64)
    return vox, fixed, coords


def _face_share(c, n):
    """Number of unit face squares touching coordinate c along an edge of n units, over 4."""
    return ((c > 0).astype(np.float64) + (c < n).astype(np.float64))


def fields(vox, coords, eps=1e-3, gam=2e-3):
    """[(name, u, K u)] for the two linear fields (compressed = full node order)."""
    nz, ny, nx = vox.shape
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    sx = _face_share(x, nx)  # squares along x touching the node (1 or 2)
    sy = _face_share(y, ny)
    sz = _face_share(z, nz)
    on = {"x0": x == 0, "x1": x == nx, "y0": y == 0, "y1": y == ny, "z1": z == nz}
    # area weight of the node on a face normal to axis a: product of the shares in the other two axes / 4
    wx, wy, wz = sy * sz / 4.0, sx * sz / 4.0, sx * sy / 4.0
    out = []
    # uniaxial
    u = np.zeros((coords.shape[0], 3))
    u[:, 2] = eps * z
    f = np.zeros_like(u)
    f[:, 0] += (on["x1"].astype(float) - on["x0"]) * LAM * eps * wx
    f[:, 1] += (on["y1"].astype(float) - on["y0"]) * LAM * eps * wy
    f[:, 2] += on["z1"] * (LAM + 2 * MU) * eps * wz
    out.append(("uniaxial", u.reshape(-1), f))
    # shear: sigma_xz = mu gam; x faces carry t_z = +-sigma_xz, the top face t_x = sigma_xz
    u = np.zeros((coords.shape[0], 3))
    u[:, 0] = gam * z
    f = np.zeros_like(u)
    f[:, 2] += (on["x1"].astype(float) - on["x0"]) * MU * gam * wx
    f[:, 0] += on["z1"] * MU * gam * wz
    out.append(("shear", u.reshape(-1), f))
    return out


def expected_product(f, fixed):
    """K u with the fixed rows zeroed (the reference's product, MatrixFreeSparse.hpp:211-213)."""
    g = f.copy()
    g[np.asarray(fixed)] = 0.0
    return g.reshape(-1)
