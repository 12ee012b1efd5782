"""Learned warm start for the MG-PCG solve (no counterpart in the reference).

A small BF16 3-D U-Net (``csrc/unet.cu``, C ABI in ``include/vfem_net.h``) maps
node-grid features (occupancy, modulus, fixed mask, load) to displacements.  It
is trained on solutions that this library's own solver produces, with the
library's own forward/backward kernels, and its prediction is passed to the
solver as the initial guess; every solve still runs to the same FP64 relative
residual, so the network can only change the iteration count, never the answer.

Features per node (channels-last, grid padded to a multiple of 8, 16 channels):
  0 used-node mask, 1 mean modulus of the adjacent filled voxels, 2 fixed mask,
  3..5 load / max|f|, 6..8 the multigrid preconditioner's response to the load
  z0 = M^-1 f (one V-cycle), divided by rms(z0), 9..15 zero.  The network thus
  learns to correct the V-cycle's approximation of the solution rather than to
  predict it from geometry alone.
Targets: u / rms(u) per sample (the displacement shape; magnitudes of porous
domains span orders of magnitude), counted on used, non-fixed nodes.  At solve
time the predicted shape y is zeroed on fixed nodes and scaled by the
energy-optimal factor gamma = f.y / y.Ky (one operator product).
"""
import ctypes
import os
import time

import numpy as np

from . import api, domains

NCH = 16


def _lib():
    lib = api.load_library()
    if not getattr(lib, "_net_bound", False):
        P = ctypes.c_void_p
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
        lib.vfem_net_create.argtypes = [ctypes.c_int32, ctypes.POINTER(P)]
        lib.vfem_net_destroy.argtypes = [P]
        lib.vfem_net_destroy.restype = None
        lib.vfem_net_num_params.argtypes = [P]
        lib.vfem_net_num_params.restype = ctypes.c_int64
        lib.vfem_net_set_params.argtypes = [P, f32p]
        lib.vfem_net_get_params.argtypes = [P, f32p]
        lib.vfem_net_forward.argtypes = [P, f32p, f32p]
        lib.vfem_net_train_batch.argtypes = [P, f32p, f32p, f32p, ctypes.c_int32, ctypes.c_float, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_float)]
        lib.vfem_net_last_error_message.restype = ctypes.c_char_p
        lib._net_bound = True
    return lib


def _check(s):
    if s != 0:
        raise api.VfemError(s, _lib().vfem_net_last_error_message().decode())


def padded(n_nodes):
    return -(-n_nodes // 8) * 8


def init_params(seed=0):
    """He-normal weights, zero biases, in the library's packed layout."""
    cin = (16, 16, 32, 64, 192, 96, 48, 16)
    cout = (16, 32, 64, 128, 64, 32, 16, 16)
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co in zip(cin, cout):
        parts.append((rng.standard_normal(27 * ci * co) * np.sqrt(2.0 / (27 * ci))).astype(np.float32))
        parts.append(np.zeros(co, np.float32))
    return np.concatenate(parts)


class UNet:
    """The network on an n^3 node grid (n a multiple of 8)."""

    def __init__(self, n, params=None):
        lib = _lib()
        h = ctypes.c_void_p()
        _check(lib.vfem_net_create(int(n), ctypes.byref(h)))
        self._h, self._lib, self.n = h, lib, int(n)
        self.num_params = int(lib.vfem_net_num_params(h))
        self.set_params(init_params() if params is None else params)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.vfem_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        _check(self._lib.vfem_net_set_params(self._h, p))

    def get_params(self):
        p = np.empty(self.num_params, np.float32)
        _check(self._lib.vfem_net_get_params(self._h, p))
        return p

    def forward(self, feats):
        x = np.ascontiguousarray(feats, np.float32).reshape(-1)
        y = np.empty(self.n ** 3 * 3, np.float32)
        _check(self._lib.vfem_net_forward(self._h, x, y))
        return y.reshape(self.n, self.n, self.n, 3)

    def train_batch(self, feats, targets, masks, lr, want_grads=False):
        b = feats.shape[0]
        x = np.ascontiguousarray(feats, np.float32).reshape(-1)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1)
        m = np.ascontiguousarray(masks, np.float32).reshape(-1)
        g = np.empty(self.num_params, np.float32) if want_grads else None
        loss = ctypes.c_float()
        _check(self._lib.vfem_net_train_batch(self._h, x, t, m, b, float(lr),
                                              g.ctypes.data_as(ctypes.c_void_p) if g is not None else None,
                                              ctypes.byref(loss)))
        return float(loss.value), g


def node_features(voxels, E, fixed, load_nodes, load_values, n_pad=None, z0=None):
    """Features [n,n,n,16] (float32), the used mask and the displacement scale
    (|f|_1 / n) of a domain; z0 (compressed numbering) fills channels 6..8."""
    vox = np.asarray(voxels, bool)
    mask = domains.used_nodes_mask(vox)
    nz, ny, nx = mask.shape
    n = n_pad or padded(max(mask.shape))
    f = np.zeros((n, n, n, NCH), np.float32)
    f[:nz, :ny, :nx, 0] = mask
    Ev = vox * (np.asarray(E, np.float32) if E is not None else 1.0)
    esum = np.zeros(mask.shape, np.float32)
    ecnt = np.zeros(mask.shape, np.float32)
    sz, sy, sx = vox.shape
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                esum[dz:dz + sz, dy:dy + sy, dx:dx + sx] += Ev
                ecnt[dz:dz + sz, dy:dy + sy, dx:dx + sx] += vox
    f[:nz, :ny, :nx, 1] = np.where(ecnt > 0, esum / np.maximum(ecnt, 1), 0)
    ids = np.flatnonzero(mask.reshape(-1))
    fm = np.zeros(mask.size, np.float32)
    fm[ids[np.asarray(fixed, np.int64)]] = 1
    f[:nz, :ny, :nx, 2] = fm.reshape(mask.shape)
    lv = np.asarray(load_values, np.float64).reshape(-1, 3)
    fmax = float(np.abs(lv).max()) if lv.size else 0.0
    ld = np.zeros((mask.size, 3), np.float32)
    if fmax > 0:
        ld[ids[np.asarray(load_nodes, np.int64)]] = lv / fmax
    f[:nz, :ny, :nx, 3:6] = ld.reshape(mask.shape + (3,))
    if z0 is not None:
        z = np.asarray(z0, np.float64).reshape(-1, 3)
        rms = float(np.sqrt(np.mean(z * z))) if z.size else 0.0
        zg = np.zeros((mask.size, 3), np.float32)
        zg[ids] = z / (rms if rms > 0 else 1.0)
        f[:nz, :ny, :nx, 6:9] = zg.reshape(mask.shape + (3,))
    total = float(np.abs(lv).sum())
    scale = 8.0 * total / max(vox.shape) if total > 0 else 1.0
    return f, mask, scale


def domain_features(d, n_pad=None, A=None, f=None):
    """Features of domain d; with the operator A, channels 6..8 carry M^-1 f."""
    z0 = None
    if A is not None:
        z0 = api.MultigridPreconditioner(A).solve(d.load_vector() if f is None else f)
    return node_features(d.voxels, d.E, d.fixed, d.load_nodes, d.load_values, n_pad, z0)


def target_grid(u, mask, scale, n):
    """Displacement shape u / rms(u) on the padded grid (scale is unused; kept
    for the feature tuple's signature)."""
    t = np.zeros((n, n, n, 3), np.float32)
    nz, ny, nx = mask.shape
    rms = float(np.sqrt(np.mean(u * u))) if u.size else 1.0
    t[:nz, :ny, :nx][mask] = (u.reshape(-1, 3) / (rms if rms > 0 else 1.0)).astype(np.float32)
    return t


def loss_mask(mask, fixed, n):
    m = np.zeros((n, n, n), np.float32)
    nz, ny, nx = mask.shape
    mm = mask.astype(np.float32).reshape(-1)
    ids = np.flatnonzero(mask.reshape(-1))
    mm[ids[np.asarray(fixed, np.int64)]] = 0
    m[:nz, :ny, :nx] = mm.reshape(mask.shape)
    return m


def predict_shape(net, d, A=None, f=None):
    """Predicted displacement shape (compressed numbering), zero on fixed nodes."""
    feats, mask, _ = domain_features(d, net.n, A, f)
    y = net.forward(feats)
    nz, ny, nx = mask.shape
    s = y[:nz, :ny, :nx][mask].astype(np.float64)
    s[np.asarray(d.fixed, np.int64)] = 0.0
    return s.reshape(-1)


def warm_start(net, d, A, f=None):
    """Initial guess gamma * y with the energy-optimal gamma = f.y / y.Ky."""
    f = d.load_vector() if f is None else f
    y = predict_shape(net, d, A, f)
    Ky = A @ y
    yKy = float(y @ Ky)
    gamma = float(f @ y) / yKy if yKy > 0 else 0.0
    return gamma * y


def coarse_correction(net, d, A, f=None):
    """The learned coarse correction: the network's predicted displacement shape
    v becomes the deflation coarse space of A's later solves
    (vfem_problem_set_coarse_space): PCG starts from x0 + v (v^T K v)^-1 v^T r0
    (the warm start's energy-optimal scaling of v) and keeps every search
    direction K-orthogonal to v.  Returns v."""
    f = d.load_vector() if f is None else f
    v = predict_shape(net, d, A, f)
    A.set_coarse_space(v)
    return v


def predict(net, d, A=None):
    """Initial guess (compressed numbering) for domain d (needs the operator A)."""
    if A is None:
        raise ValueError("the warm start is scaled with one product of the operator A")
    return warm_start(net, d, A)


def generate(count, n=64, seed0=0, levels=4, log=None):
    """Training pairs from the library's own solver (mixed precision, rtol 1e-6)."""
    ke = domains.hex8_stiffness()
    npad = padded(n + 1)
    X = np.zeros((count, npad, npad, npad, NCH), np.float32)
    T = np.zeros((count, npad, npad, npad, 3), np.float32)
    M = np.zeros((count, npad, npad, npad), np.float32)
    t0 = time.time()
    for i in range(count):
        d = domains.training_field(n, seed=seed0 + i, levels=levels)
        A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, levels)
        f = d.load_vector()
        u, _ = A.solve(f, precision="mixed")
        X[i], mask, scale = domain_features(d, npad, A, f)
        A.close()
        T[i] = target_grid(u, mask, scale, npad)
        M[i] = loss_mask(mask, d.fixed, npad)
        if log and (i + 1) % 50 == 0:
            log("generated %d/%d (%.1f s)" % (i + 1, count, time.time() - t0))
    return X, T, M


def train(net, X, T, M, epochs=10, batch=4, lr=1e-3, seed=0, log=None):
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(X.shape[0])
        losses = []
        lr_ep = lr * (0.5 ** (ep // max(1, epochs // 3)))
        for s in range(0, len(order) - batch + 1, batch):
            idx = order[s:s + batch]
            loss, _ = net.train_batch(X[idx], T[idx], M[idx], lr_ep)
            losses.append(loss)
        hist.append(float(np.mean(losses)))
        if log:
            log("epoch %d loss %.5f" % (ep, hist[-1]))
    return hist


def save(path, params, meta=None):
    np.savez_compressed(path, params_bf16=_to_bf16_bits(params), **(meta or {}))


def load(path):
    z = np.load(path)
    return _from_bf16_bits(z["params_bf16"])


def _to_bf16_bits(p):
    u = np.asarray(p, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def _from_bf16_bits(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


CHECKPOINT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "checkpoints", "unet_warmstart.npz")
