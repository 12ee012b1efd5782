"""CPU oracle for the MG-PCG path (test infrastructure only).

``vfem_oracle.cpp`` restates the reference's CPU solve path (assembly, matrix-free
product, additive multigrid preconditioner, Eigen-semantics PCG).  This module
compiles it with ``g++`` into ``oracle/_build/liboracle.so`` and wraps it with
ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import it; the product library never does.

PARITY UNPINNED: the reference has no golden outputs and cannot be built here,
so the oracle is pinned only by the derived known-answer tests in ``tests/``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "vfem_oracle.cpp")

_lib = None


def build(force=False):
    """Compile the oracle (g++, OpenMP).  Returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
        lib.oracle_create.restype = P
        lib.oracle_create.argtypes = [i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, f64p,
                                      i64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        lib.oracle_create_e.restype = P
        lib.oracle_create_e.argtypes = [i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, f64p, ctypes.c_void_p,
                                        i64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        lib.oracle_destroy.argtypes = [P]
        lib.oracle_set_threads.argtypes = [P, ctypes.c_int]
        lib.oracle_set_float_coeffs.argtypes = [P, ctypes.c_int]
        lib.oracle_num_levels.argtypes = [P]
        lib.oracle_num_levels.restype = ctypes.c_int
        for name in ("oracle_num_dofs", "oracle_num_elements", "oracle_num_fixed"):
            getattr(lib, name).argtypes = [P, ctypes.c_int]
            getattr(lib, name).restype = ctypes.c_int64
        lib.oracle_num_coarse_free.argtypes = [P]
        lib.oracle_num_coarse_free.restype = ctypes.c_int64
        lib.oracle_level_dims.argtypes = [P, ctypes.c_int, i32p]
        lib.oracle_nodes.argtypes = [P, ctypes.c_int, i64p]
        lib.oracle_fixed.argtypes = [P, ctypes.c_int, i64p]
        lib.oracle_inv_diag.argtypes = [P, ctypes.c_int, f64p]
        lib.oracle_restriction_coeffs.argtypes = [P, ctypes.c_int, f64p]
        lib.oracle_element_to_node.argtypes = [P, ctypes.c_int, i32p]
        lib.oracle_matvec.argtypes = [P, f64p, f64p]
        lib.oracle_precond.argtypes = [P, f64p, f64p]
        lib.oracle_restrict.argtypes = [P, ctypes.c_int, f64p, f64p]
        lib.oracle_interpolate.argtypes = [P, ctypes.c_int, f64p, f64p]
        lib.oracle_coarse_solve.argtypes = [P, f64p, f64p]
        lib.oracle_apply_loads.argtypes = [P, i64p, f64p, ctypes.c_int64, f64p]
        lib.oracle_pcg.argtypes = [P, f64p, f64p, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
        lib.oracle_pcg.restype = ctypes.c_int64
        _lib = lib
    return _lib


class Oracle:
    """One assembled problem (the reference's ``assembleSystemMatrix`` result)."""

    def __init__(self, voxels, Ke, fixed, num_levels=3, skip_levels=0, threads=1, E=None):
        lib = _load()
        vox = np.ascontiguousarray(voxels, dtype=np.int32)
        assert vox.ndim == 3, "voxels are indexed [z, y, x]"
        sz, sy, sx = vox.shape
        ke = np.ascontiguousarray(Ke, dtype=np.float64).reshape(24, 24)
        fx = np.ascontiguousarray(fixed, dtype=np.int64).reshape(-1)
        self._E = None
        eptr = None
        if E is not None:  # per-voxel modulus (extension; the reference has a uniform E)
            self._E = np.ascontiguousarray(E, dtype=np.float32)
            assert self._E.shape == vox.shape
            eptr = self._E.ctypes.data_as(ctypes.c_void_p)
        self._p = lib.oracle_create_e(vox.reshape(-1), sx, sy, sz, ke.reshape(-1), eptr, fx, fx.size,
                                      int(num_levels), int(skip_levels))
        if not self._p:
            raise ValueError("oracle_create failed")
        self._lib = lib
        lib.oracle_set_threads(self._p, int(threads))

    def __del__(self):
        if getattr(self, "_p", None):
            self._lib.oracle_destroy(self._p)
            self._p = None

    def set_threads(self, t):
        self._lib.oracle_set_threads(self._p, int(t))

    def set_float_coeffs(self, on):
        self._lib.oracle_set_float_coeffs(self._p, int(bool(on)))

    @property
    def num_levels(self):
        return self._lib.oracle_num_levels(self._p)

    def num_dofs(self, level=0):
        return self._lib.oracle_num_dofs(self._p, level)

    def num_elements(self, level=0):
        return self._lib.oracle_num_elements(self._p, level)

    def num_coarse_free(self):
        return self._lib.oracle_num_coarse_free(self._p)

    def level_dims(self, level):
        out = np.zeros(3, np.int32)
        self._lib.oracle_level_dims(self._p, level, out)
        return tuple(int(v) for v in out)

    def nodes(self, level=0):
        out = np.zeros(self.num_dofs(level) // 3, np.int64)
        self._lib.oracle_nodes(self._p, level, out)
        return out

    def fixed(self, level=0):
        out = np.zeros(self._lib.oracle_num_fixed(self._p, level), np.int64)
        self._lib.oracle_fixed(self._p, level, out)
        return out

    def inv_diag(self, level=0):
        out = np.zeros(self.num_dofs(level), np.float64)
        self._lib.oracle_inv_diag(self._p, level, out)
        return out

    def restriction_coeffs(self, level=0):
        out = np.zeros(self.num_dofs(level), np.float64)
        self._lib.oracle_restriction_coeffs(self._p, level, out)
        return out

    def element_to_node(self, level=0):
        out = np.zeros((self.num_elements(level), 4), np.int32)
        self._lib.oracle_element_to_node(self._p, level, out.reshape(-1))
        return out

    def matvec(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty_like(x)
        self._lib.oracle_matvec(self._p, x, y)
        return y

    def precond(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty_like(r)
        self._lib.oracle_precond(self._p, r, z)
        return z

    def restrict(self, level, v):
        v = np.ascontiguousarray(v, np.float64)
        out = np.empty(self.num_dofs(level + 1), np.float64)
        self._lib.oracle_restrict(self._p, level, v, out)
        return out

    def interpolate(self, level, v):
        v = np.ascontiguousarray(v, np.float64)
        out = np.empty(self.num_dofs(level), np.float64)
        self._lib.oracle_interpolate(self._p, level, v, out)
        return out

    def coarse_solve(self, rhs):
        rhs = np.ascontiguousarray(rhs, np.float64)
        out = np.empty_like(rhs)
        self._lib.oracle_coarse_solve(self._p, rhs, out)
        return out

    def load_vector(self, nodes, loads):
        f = np.zeros(self.num_dofs(0), np.float64)
        nd = np.ascontiguousarray(nodes, np.int64)
        ld = np.ascontiguousarray(loads, np.float64).reshape(-1)
        self._lib.oracle_apply_loads(self._p, nd, ld, nd.size, f)
        return f

    def pcg(self, b, tol=1e-6, max_iter=0, use_mg=True, iter_cap=0):
        """Eigen-semantics PCG.  Returns (x, iterations, recursive relative error)."""
        b = np.ascontiguousarray(b, np.float64)
        x = np.empty_like(b)
        err = ctypes.c_double(0.0)
        it = self._lib.oracle_pcg(self._p, b, x, float(tol), int(max_iter), int(bool(use_mg)),
                                  ctypes.byref(err), int(iter_cap))
        return x, int(it), float(err.value)
