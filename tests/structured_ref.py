"""numpy restatement of the structured (dense-grid) formulation the CUDA kernels
use, for CPU tests that compare it with the oracle's element-list formulation.

Vectors here are dense [nz+1, ny+1, nx+1, 3] node arrays; ``to_dense`` /
``to_compressed`` map to and from the reference's compressed numbering.
"""
import numpy as np


def used_mask(elem):
    """elem: bool [ez, ey, ex] used elements -> bool [ez+1, ey+1, ex+1] used nodes."""
    ez, ey, ex = elem.shape
    m = np.zeros((ez + 1, ey + 1, ex + 1), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                m[dz:dz + ez, dy:dy + ey, dx:dx + ex] |= elem
    return m


def to_dense(v, mask):
    d = np.zeros(mask.shape + (3,))
    d[mask] = v.reshape(-1, 3)
    return d


def to_compressed(d, mask):
    return d[mask].reshape(-1)


def coarsen(elem, div=2):
    ez, ey, ex = elem.shape
    cz, cy, cx = -(-ez // div), -(-ey // div), -(-ex // div)
    pad = np.zeros((cz * div, cy * div, cx * div), bool)
    pad[:ez, :ey, :ex] = elem
    return pad.reshape(cz, div, cy, div, cx, div).any(axis=(1, 3, 5))


def _w1(d, div):
    return (div - abs(d)) / div


def restrict(fine, coarse_shape, div=2):
    """Full weighting: rc[C] = sum_{|d|<div} prod w(d_i) rf[div*C + d]."""
    cz, cy, cx = coarse_shape
    fz, fy, fx = fine.shape[:3]
    out = np.zeros((cz, cy, cx, 3))
    R = div - 1
    for dz in range(-R, R + 1):
        for dy in range(-R, R + 1):
            for dx in range(-R, R + 1):
                w = _w1(dz, div) * _w1(dy, div) * _w1(dx, div)
                Z = np.arange(cz) * div + dz
                Y = np.arange(cy) * div + dy
                X = np.arange(cx) * div + dx
                vz, vy, vx = (Z >= 0) & (Z < fz), (Y >= 0) & (Y < fy), (X >= 0) & (X < fx)
                sub = fine[np.ix_(Z[vz], Y[vy], X[vx])]
                out[np.ix_(vz, vy, vx)] += w * sub
    return out


def prolong(coarse, fine_mask, div=2):
    """Trilinear prolongation to the used fine nodes (0 elsewhere)."""
    fz, fy, fx = fine_mask.shape
    out = np.zeros((fz, fy, fx, 3))
    Z, Y, X = np.arange(fz), np.arange(fy), np.arange(fx)
    for iz in (0, 1):
        pz = Z // div + iz
        wz = np.where(iz, (Z % div) / div, (div - Z % div) / div)
        for iy in (0, 1):
            py = Y // div + iy
            wy = np.where(iy, (Y % div) / div, (div - Y % div) / div)
            for ix in (0, 1):
                px = X // div + ix
                wx = np.where(ix, (X % div) / div, (div - X % div) / div)
                w = wz[:, None, None] * wy[None, :, None] * wx[None, None, :]
                pzc = np.minimum(pz, coarse.shape[0] - 1)
                pyc = np.minimum(py, coarse.shape[1] - 1)
                pxc = np.minimum(px, coarse.shape[2] - 1)
                val = coarse[np.ix_(pzc, pyc, pxc)]
                out += (w * (w > 0))[..., None] * val
    out[~fine_mask] = 0
    return out


def matvec(elem_E, Ke, x, fixed_mask=None, scale=1.0):
    """Element-by-element y = sum_e E_e Ke x_e on the dense grid (local node
    a = dx + 2dy + 4dz), fixed rows zeroed."""
    ez, ey, ex = elem_E.shape
    y = np.zeros_like(x)
    corners = [(a >> 2, (a >> 1) & 1, a & 1) for a in range(8)]
    xe = np.concatenate([x[dz:dz + ez, dy:dy + ey, dx:dx + ex] for dz, dy, dx in corners], axis=-1)
    ye = np.einsum("rk,zyxk->zyxr", Ke, xe) * (scale * elem_E)[..., None]
    for a, (dz, dy, dx) in enumerate(corners):
        y[dz:dz + ez, dy:dy + ey, dx:dx + ex] += ye[..., 3 * a:3 * a + 3]
    if fixed_mask is not None:
        y[fixed_mask] = 0
    return y


def fixed_dilate(fine_fixed, coarse_shape, div=2):
    cz, cy, cx = coarse_shape
    fz, fy, fx = fine_fixed.shape
    out = np.zeros(coarse_shape, bool)
    R = div - 1
    for dz in range(-R, R + 1):
        for dy in range(-R, R + 1):
            for dx in range(-R, R + 1):
                Z, Y, X = np.arange(cz) * div + dz, np.arange(cy) * div + dy, np.arange(cx) * div + dx
                vz, vy, vx = (Z >= 0) & (Z < fz), (Y >= 0) & (Y < fy), (X >= 0) & (X < fx)
                out[np.ix_(vz, vy, vx)] |= fine_fixed[np.ix_(Z[vz], Y[vy], X[vx])]
    return out


class MultiplicativeMG:
    """numpy restatement of the library's multiplicative V-cycle
    (VFEM_MG_VCYCLE): rediscretised level operators 2^l sum_e E_e Ke (coarse
    elements carry the volume average of their children's modulus, empty
    children counting as 0), damped Jacobi on
    their diagonals, full weighting / trilinear prolongation, fixed DOFs masked
    on every level (fixed sets dilated from the finest), dense coarsest solve."""

    def __init__(self, voxels, Ke, fixed, levels, E=None, omega=0.6, pre=1, post=1):
        self.Ke, self.omega, self.pre, self.post = Ke, omega, pre, post
        E0 = voxels.astype(float) * (np.asarray(E, np.float32).astype(float) if E is not None else 1.0)
        self.Es, self.masks, self.fixeds, self.scales = [E0], [used_mask(E0 > 0)], [], [1.0]
        fm = np.zeros(self.masks[0].shape, bool)
        fm.reshape(-1)[np.flatnonzero(self.masks[0].reshape(-1))[np.asarray(fixed)]] = True
        self.fixeds.append(fm)
        for l in range(1, levels):
            Ef = self.Es[-1]
            ez, ey, ex = Ef.shape
            cz, cy, cx = -(-ez // 2), -(-ey // 2), -(-ex // 2)
            pad = np.zeros((cz * 2, cy * 2, cx * 2))
            pad[:ez, :ey, :ex] = Ef
            blk = pad.reshape(cz, 2, cy, 2, cx, 2)
            cnt = (blk > 0).sum(axis=(1, 3, 5))
            sm = blk.sum(axis=(1, 3, 5))
            Ec = np.where(cnt > 0, (sm / 8.0).astype(np.float32).astype(float), 0.0)
            self.Es.append(Ec)
            self.masks.append(used_mask(Ec > 0))
            self.fixeds.append(fixed_dilate(self.fixeds[-1], self.masks[-1].shape, 2))
            self.scales.append(2.0 ** l)
        self.L = levels
        self.act = [(m & ~f)[..., None] for m, f in zip(self.masks, self.fixeds)]
        self.D = [self._dinv(l) for l in range(levels)]
        lc = levels - 1
        self.cidx = np.flatnonzero(self.act[lc][..., 0].reshape(-1))
        n = 3 * self.cidx.size
        Kc = np.zeros((n, n))
        for j in range(n):
            e = np.zeros(self.masks[lc].shape + (3,))
            e.reshape(-1, 3)[self.cidx[j // 3], j % 3] = 1
            Kc[:, j] = self.A(lc, e).reshape(-1, 3)[self.cidx].reshape(-1)
        self.Kinv = np.linalg.inv(Kc)

    def A(self, l, x):
        return matvec(self.Es[l], self.Ke, x, self.fixeds[l], self.scales[l])

    def _dinv(self, l):
        diag = np.zeros(self.masks[l].shape + (3,))
        Ee = self.Es[l]
        ez, ey, ex = Ee.shape
        for a in range(8):
            dz, dy, dx = a >> 2, (a >> 1) & 1, a & 1
            diag[dz:dz + ez, dy:dy + ey, dx:dx + ex] += self.scales[l] * Ee[..., None] * np.diag(self.Ke)[3 * a:3 * a + 3]
        return np.where(self.masks[l][..., None], 1.0 / np.where(diag > 0, diag, 1.0), 0.0)

    def _coarse(self, r):
        z = np.zeros_like(r)
        z.reshape(-1, 3)[self.cidx] = (self.Kinv @ r.reshape(-1, 3)[self.cidx].reshape(-1)).reshape(-1, 3)
        return z

    def cycle(self, l, r):
        if l == self.L - 1:
            return self._coarse(r)
        act, D, w = self.act[l], self.D[l], self.omega
        z = act * w * D * r
        for _ in range(self.pre - 1):
            z = act * (z + w * D * (r - self.A(l, z)))
        t = act * (r - self.A(l, z))
        zc = self.cycle(l + 1, restrict(t, self.masks[l + 1].shape, 2))
        z = z + act * prolong(zc, self.masks[l], 2)
        for _ in range(self.post):
            z = act * (z + w * D * (r - self.A(l, z)))
        return z

    def apply(self, r_compressed):
        r = to_dense(r_compressed, self.masks[0])
        return to_compressed(self.cycle(0, r), self.masks[0])
