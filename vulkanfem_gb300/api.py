"""Host-side mirror of the reference's solve-path interface over libvfem's C ABI.

Names follow the reference (include/FEM.hpp, include/FEMGPU.hpp,
include/MatrixFreeSparse.hpp, include/MultigridPreconditioner.hpp):

====================================  =========================================
reference                             here
====================================  =========================================
assembleSystemMatrix<double>(...)     assembleSystemMatrix / assemble_system_matrix
applyBoundaryConditions(f, loads, ..) applyBoundaryConditions
solveWithKompute(A, f, u)             solveWithKompute (GPU MG-PCG, FP64)
MatrixFreeSparse<double> * x          MatrixFreeSparse.__matmul__ / .dot
MultigridPreconditioner::solve(b)     MultigridPreconditioner.solve
====================================  =========================================

Unlike the reference (void returns, Eigen asserts), every failure raises
``VfemError`` carrying the library's status code.  The library must be built
(``vulkanfem_gb300.build.build()``); there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

OK = 0
STATUS_NAMES = {
    0: "VFEM_OK", 1: "VFEM_ERR_INVALID_ARGUMENT", 2: "VFEM_ERR_CUDA", 3: "VFEM_ERR_OUT_OF_MEMORY",
    4: "VFEM_ERR_NOT_CONVERGED", 5: "VFEM_ERR_BREAKDOWN", 6: "VFEM_ERR_SINGULAR", 7: "VFEM_ERR_EMPTY",
    8: "VFEM_ERR_COARSE_TOO_LARGE", 9: "VFEM_ERR_NO_DEVICE", 10: "VFEM_ERR_TIMEOUT",
}
MG_MODES = {"reference": 0, "vcycle": 1, "none": 2}
PRECISIONS = {"fp64": 0, "mixed": 1}

# Every symbol declared in include/vfem.h.
EXPORTED = (
    "vfem_options_default", "vfem_status_string", "vfem_hex8_stiffness", "vfem_problem_create",
    "vfem_problem_destroy", "vfem_problem_info", "vfem_problem_set_loads", "vfem_problem_set_rhs",
    "vfem_solve", "vfem_solve_device", "vfem_apply_operator", "vfem_apply_preconditioner",
    "vfem_apply_preconditioner_mixed",
    "vfem_restrict", "vfem_interpolate", "vfem_inverse_diagonal", "vfem_fixed_nodes",
    "vfem_kernel_launch_count", "vfem_last_error_message", "vfem_profile_kernels",
    "vfem_apply_operator_device_noalloc", "vfem_apply_operator_mixed", "vfem_problem_uses_tensor_cores",
    "vfem_problem_uses_tma", "vfem_problem_set_coarse_space",
    # learned warm start (include/vfem_net.h)
    "vfem_net_create", "vfem_net_destroy", "vfem_net_num_params", "vfem_net_set_params", "vfem_net_get_params",
    "vfem_net_forward", "vfem_net_train_batch", "vfem_net_last_error_message",
)

KERNEL_CLASSES = ("matvec_fp64", "matvec_fp32", "restrict_fp64", "restrict_fp32", "prolong_fp64", "prolong_fp32",
                  "update_xr_fp64", "update_xr_mixed", "update_p_fp64", "update_p_fp32", "coarse_fp64",
                  "coarse_fp32", "true_residual_df", "update_restrict_mixed", "matvec_fp32_simt",
                  "matvec_fp32_px")


class VfemError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = int(status)
        name = STATUS_NAMES.get(self.status, str(status))
        super().__init__("%s%s" % (name, (": " + message) if message else ""))


class Options(ctypes.Structure):
    _fields_ = [
        ("rtol", ctypes.c_double), ("max_iter", ctypes.c_int64), ("mg_mode", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("omega", ctypes.c_double), ("pre_sweeps", ctypes.c_int32),
        ("post_sweeps", ctypes.c_int32), ("replace_every", ctypes.c_int32), ("flexible", ctypes.c_int32),
        ("check_every", ctypes.c_int32), ("compute_true_residual", ctypes.c_int32),
        ("replace_delta", ctypes.c_double), ("fallback_fp64", ctypes.c_int32), ("debug_break_at", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 4),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int64), ("matvecs", ctypes.c_int64), ("residual_replacements", ctypes.c_int64),
        ("rel_residual", ctypes.c_double), ("recursive_rel_residual", ctypes.c_double),
        ("solve_ms", ctypes.c_double), ("h2d_ms", ctypes.c_double), ("d2h_ms", ctypes.c_double),
        ("kernel_launches", ctypes.c_int64), ("status", ctypes.c_int32), ("fallback", ctypes.c_int32),
        ("fallback_iterations", ctypes.c_int64), ("reserved", ctypes.c_int32 * 4),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


def library_path():
    return _build.LIB


def load_library(build_if_missing=True):
    """Load libvfem.so (building it in-tree first if needed).  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libvfem.so not built: run vulkanfem_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
    i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
    u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")
    i32 = ctypes.c_int32
    lib.vfem_options_default.argtypes = [ctypes.POINTER(Options)]
    lib.vfem_options_default.restype = None
    lib.vfem_status_string.argtypes = [ctypes.c_int]
    lib.vfem_status_string.restype = ctypes.c_char_p
    lib.vfem_last_error_message.restype = ctypes.c_char_p
    lib.vfem_kernel_launch_count.restype = ctypes.c_int64
    lib.vfem_hex8_stiffness.argtypes = [ctypes.c_double, ctypes.c_double, f64p]
    lib.vfem_problem_create.argtypes = [u8p, i32, i32, i32, f64p, ctypes.c_void_p, i64p, ctypes.c_int64, i32, i32,
                                        ctypes.POINTER(P)]
    lib.vfem_problem_destroy.argtypes = [P]
    lib.vfem_problem_destroy.restype = None
    lib.vfem_problem_info.argtypes = [P, i32, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)]
    lib.vfem_problem_set_loads.argtypes = [P, i64p, f64p, ctypes.c_int64]
    lib.vfem_problem_set_rhs.argtypes = [P, f64p]
    lib.vfem_solve.argtypes = [P, ctypes.POINTER(Options), ctypes.c_void_p, f64p, ctypes.POINTER(Stats)]
    lib.vfem_solve_device.argtypes = [P, ctypes.POINTER(Options), ctypes.c_void_p, ctypes.POINTER(Stats)]
    lib.vfem_apply_operator.argtypes = [P, f64p, f64p]
    lib.vfem_apply_preconditioner.argtypes = [P, i32, f64p, f64p]
    lib.vfem_apply_preconditioner_mixed.argtypes = [P, i32, f64p, f64p]
    lib.vfem_restrict.argtypes = [P, i32, f64p, f64p]
    lib.vfem_interpolate.argtypes = [P, i32, f64p, f64p]
    lib.vfem_inverse_diagonal.argtypes = [P, i32, f64p]
    lib.vfem_fixed_nodes.argtypes = [P, i32, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    lib.vfem_profile_kernels.argtypes = [P, i32, f64p]
    lib.vfem_apply_operator_device_noalloc.argtypes = [P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                       ctypes.c_void_p]
    lib.vfem_apply_operator_mixed.argtypes = [P, f64p, f64p, ctypes.c_void_p]
    lib.vfem_problem_uses_tensor_cores.argtypes = [P]
    lib.vfem_problem_uses_tensor_cores.restype = ctypes.c_int32
    lib.vfem_problem_set_coarse_space.argtypes = [P, ctypes.c_void_p, i32]
    lib.vfem_problem_uses_tma.argtypes = [P]
    lib.vfem_problem_uses_tma.restype = ctypes.c_int32
    for name in EXPORTED:
        fn = getattr(lib, name)
        if fn.restype is ctypes.c_int and name not in ("vfem_status_string",):
            fn.restype = ctypes.c_int
    _lib = lib
    return lib


def _check(status):
    if status != OK:
        msg = _lib.vfem_last_error_message().decode() if _lib is not None else ""
        raise VfemError(status, msg)


def kernel_launch_count():
    return int(load_library().vfem_kernel_launch_count())


def profile_kernels(A, reps=20):
    """Average CUDA-event time (ms) of each kernel class on A's finest level."""
    out = np.zeros(len(KERNEL_CLASSES), np.float64)
    _check(load_library().vfem_profile_kernels(A._h, int(reps), out))
    return dict(zip(KERNEL_CLASSES, out.tolist()))


def hex8_stiffness(E=1.0, nu=0.3):
    lib = load_library()
    ke = np.zeros(576, np.float64)
    _check(lib.vfem_hex8_stiffness(float(E), float(nu), ke))
    return ke.reshape(24, 24)


def make_options(rtol=1e-6, max_iter=0, mg_mode="reference", precision="fp64", omega=0.6, pre_sweeps=1,
                 post_sweeps=1, replace_every=0, flexible=False, check_every=8, compute_true_residual=True,
                 replace_delta=0.05, fallback_fp64=True, debug_break_at=0):
    lib = load_library()
    o = Options()
    lib.vfem_options_default(ctypes.byref(o))
    o.rtol = rtol
    o.max_iter = int(max_iter)
    o.mg_mode = MG_MODES[mg_mode] if isinstance(mg_mode, str) else int(mg_mode)
    o.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.omega = omega
    o.pre_sweeps = pre_sweeps
    o.post_sweeps = post_sweeps
    o.replace_every = replace_every
    o.flexible = int(bool(flexible))
    o.check_every = check_every
    o.compute_true_residual = int(bool(compute_true_residual))
    o.replace_delta = replace_delta
    o.fallback_fp64 = int(bool(fallback_fp64))
    o.debug_break_at = int(debug_break_at)
    return o


class MatrixFreeSparse:
    """The assembled operator + multigrid hierarchy on the GPU
    (``MatrixFreeSparse<double>`` after ``PrepareMultigrid``,
    include/MatrixFreeSparse.hpp:31-94)."""

    def __init__(self, voxels, Ke, fixed, num_levels=3, skip_levels=0, E=None):
        lib = load_library()
        vox = np.ascontiguousarray(voxels, dtype=np.uint8)
        if vox.ndim != 3:
            raise VfemError(1, "voxels must be a 3-D array indexed [z, y, x]")
        nz, ny, nx = vox.shape
        ke = np.ascontiguousarray(Ke, dtype=np.float64).reshape(-1)
        if ke.size != 576:
            raise VfemError(1, "Ke must be 24x24")
        fx = np.ascontiguousarray(fixed, dtype=np.int64).reshape(-1)
        self._E = None
        eptr = None
        if E is not None:
            self._E = np.ascontiguousarray(E, dtype=np.float32)
            if self._E.shape != vox.shape:
                raise VfemError(1, "E must have the voxel shape")
            eptr = self._E.ctypes.data_as(ctypes.c_void_p)
        h = ctypes.c_void_p()
        _check(lib.vfem_problem_create(vox.reshape(-1), nx, ny, nz, ke, eptr, fx, fx.size, int(num_levels),
                                       int(skip_levels), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.shape = vox.shape
        self._info = {}
        n, ne, nl, nc = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64()
        _check(lib.vfem_problem_info(h, 0, ctypes.byref(n), ctypes.byref(ne), ctypes.byref(nl), ctypes.byref(nc)))
        self.num_levels = int(nl.value)
        self.coarse_free_dofs = int(nc.value)
        self._nodes = []
        self._elems = []
        for lv in range(self.num_levels):
            _check(lib.vfem_problem_info(h, lv, ctypes.byref(n), ctypes.byref(ne), None, None))
            self._nodes.append(int(n.value))
            self._elems.append(int(ne.value))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.vfem_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference surface
    def rows(self):
        return 3 * self._nodes[0]

    def cols(self):
        return self.rows()

    def num_dofs(self, level=0):
        return 3 * self._nodes[level]

    def num_elements(self, level=0):
        return self._elems[level]

    def dot(self, x):
        x = np.ascontiguousarray(x, np.float64)
        if x.size != self.rows():
            raise VfemError(1, "vector size mismatch")
        y = np.empty_like(x)
        _check(self._lib.vfem_apply_operator(self._h, x, y))
        return y

    __matmul__ = dot

    def set_coarse_space(self, V=None):
        """Deflation coarse space for every later solve and preconditioner
        application (V: [rows] or [rows, k], k <= 4; entries at fixed DOFs are
        taken as 0; None removes it).  The preconditioner becomes
        M^-1 r + V G^-1 (V^T r - (KV)^T M^-1 r), G = V^T K V, and PCG starts
        from x0 + V G^-1 V^T r0."""
        if V is None:
            _check(self._lib.vfem_problem_set_coarse_space(self._h, None, 0))
            return
        V = np.asarray(V, np.float64)
        if V.ndim == 1:
            V = V[:, None]
        if V.shape[0] != self.rows() or not 1 <= V.shape[1] <= 4:
            raise VfemError(1, "coarse space must be [rows, k] with k <= 4")
        cols = np.ascontiguousarray(V.T)
        _check(self._lib.vfem_problem_set_coarse_space(self._h, cols.ctypes.data_as(ctypes.c_void_p), V.shape[1]))

    def dot_mixed(self, x):
        """The mixed-precision solver's product: FP32 (tensor cores when
        ``uses_tensor_cores``).  Returns (K x, x.(Kx))."""
        x = np.ascontiguousarray(x, np.float64)
        if x.size != self.rows():
            raise VfemError(1, "vector size mismatch")
        y = np.empty_like(x)
        d = ctypes.c_double()
        _check(self._lib.vfem_apply_operator_mixed(self._h, x, y, ctypes.cast(ctypes.pointer(d), ctypes.c_void_p)))
        return y, d.value

    @property
    def uses_tensor_cores(self):
        return bool(self._lib.vfem_problem_uses_tensor_cores(self._h))

    @property
    def uses_tma(self):
        return bool(self._lib.vfem_problem_uses_tma(self._h))

    def restrict(self, level, v):
        v = np.ascontiguousarray(v, np.float64)
        out = np.empty(self.num_dofs(level + 1), np.float64)
        _check(self._lib.vfem_restrict(self._h, int(level), v, out))
        return out

    def interpolate(self, level, v):
        v = np.ascontiguousarray(v, np.float64)
        out = np.empty(self.num_dofs(level), np.float64)
        _check(self._lib.vfem_interpolate(self._h, int(level), v, out))
        return out

    def inverse_diagonal(self, level=0):
        out = np.empty(self.num_dofs(level), np.float64)
        _check(self._lib.vfem_inverse_diagonal(self._h, int(level), out))
        return out

    def fixed_nodes(self, level=0):
        cnt = ctypes.c_int64()
        _check(self._lib.vfem_fixed_nodes(self._h, int(level), None, 0, ctypes.byref(cnt)))
        out = np.zeros(cnt.value, np.int64)
        _check(self._lib.vfem_fixed_nodes(self._h, int(level), out.ctypes.data_as(ctypes.c_void_p), cnt.value,
                                          ctypes.byref(cnt)))
        return out

    def set_loads(self, nodes, loads):
        nd = np.ascontiguousarray(nodes, np.int64).reshape(-1)
        ld = np.ascontiguousarray(loads, np.float64).reshape(-1)
        if ld.size != 3 * nd.size:
            raise VfemError(1, "loads must be [n, 3]")
        _check(self._lib.vfem_problem_set_loads(self._h, nd, ld, nd.size))

    def set_rhs(self, f):
        f = np.ascontiguousarray(f, np.float64)
        if f.size != self.rows():
            raise VfemError(1, "vector size mismatch")
        _check(self._lib.vfem_problem_set_rhs(self._h, f))

    def solve(self, f=None, u0=None, allow_not_converged=False, out=None, **opts):
        """Solve K u = f (f defaults to the loads already set).  Returns (u, stats);
        u is ``out`` when given (a C-contiguous float64 array of ``rows()``)."""
        if f is not None:
            self.set_rhs(f)
        o = make_options(**opts)
        if out is None:
            u = np.empty(self.rows(), np.float64)
        else:
            u = out
            if u.dtype != np.float64 or u.size != self.rows() or not u.flags.c_contiguous:
                raise VfemError(1, "out must be a C-contiguous float64 array of rows() values")
        st = Stats()
        u0p = None
        if u0 is not None:
            u0a = np.ascontiguousarray(u0, np.float64)
            u0p = u0a.ctypes.data_as(ctypes.c_void_p)
        s = self._lib.vfem_solve(self._h, ctypes.byref(o), u0p, u, ctypes.byref(st))
        if s != OK and not (allow_not_converged and s == 4):
            _check(s)
        return u, st.as_dict()

    def solve_device(self, want_solution=False, allow_not_converged=False, **opts):
        """Solve with the right-hand side already on the device; the solution stays there
        unless ``want_solution``."""
        o = make_options(**opts)
        st = Stats()
        u = np.empty(self.rows(), np.float64) if want_solution else None
        s = self._lib.vfem_solve_device(self._h, ctypes.byref(o),
                                        u.ctypes.data_as(ctypes.c_void_p) if u is not None else None,
                                        ctypes.byref(st))
        if s != OK and not (allow_not_converged and s == 4):
            _check(s)
        return u, st.as_dict()


class MultigridPreconditioner:
    """``Eigen::MultigridPreconditioner`` (include/MultigridPreconditioner.hpp:12-214):
    ``compute(A)`` then ``solve(b)`` applies one V-cycle in FP64."""

    def __init__(self, A=None, mode="reference", precision="fp64"):
        """precision "mixed": the V-cycle as the mixed-precision solver applies it."""
        self.mode = MG_MODES[mode]
        if precision not in ("fp64", "mixed"):
            raise VfemError(1, "precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self.A = None
        if A is not None:
            self.compute(A)

    def compute(self, A):
        self.A = A
        return self

    analyzePattern = compute
    factorize = compute

    def info(self):
        return 0 if self.A is not None else 1

    def solve(self, b):
        if self.A is None:
            raise VfemError(1, "MultigridPreconditioner is not initialized")
        b = np.ascontiguousarray(b, np.float64)
        if b.size != self.A.rows():
            raise VfemError(1, "invalid number of rows of the right hand side")
        z = np.empty_like(b)
        fn = (self.A._lib.vfem_apply_preconditioner_mixed if self.precision == "mixed"
              else self.A._lib.vfem_apply_preconditioner)
        _check(fn(self.A._h, self.mode, b, z))
        return z


def assembleSystemMatrix(voxelModel, Ke, fixedNodes, numLevels=3, skipLevels=0, E=None):
    """``assembleSystemMatrix<double>`` (src/FEM.cpp:157-554)."""
    return MatrixFreeSparse(voxelModel, Ke, fixedNodes, numLevels, skipLevels, E)


assemble_system_matrix = assembleSystemMatrix


def applyBoundaryConditions(f, loadedNodes, fixedNodes=None):
    """``applyBoundaryConditions`` (src/FEM.cpp:568-584), matrix-free branch:
    f[3*node + c] = load.  ``loadedNodes`` maps node id -> (x, y, z)."""
    fv = f.reshape(-1, 3)
    for node, val in loadedNodes.items():
        fv[int(node)] = val
    return f


def solveWithKompute(systemMatrix, f, u=None, **opts):
    """``solveWithKompute(A, f, u)`` (src/FEMGPU.cpp:32-554): GPU MG-PCG.  Writes the
    solution into ``u`` when given and returns (u, stats)."""
    sol, st = systemMatrix.solve(f, **opts)
    if u is not None:
        u[...] = sol
        return u, st
    return sol, st


solve = solveWithKompute
