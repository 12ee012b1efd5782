/*
 * vfem.h -- C ABI of libvfem, the GB300 (sm_103a) matrix-free voxel elasticity
 * MG-PCG solver.
 *
 * The entry points replace the reference's solve path of VulkanFEM (paths below
 * are relative to that project's root):
 *   assembleSystemMatrix<double>(...)      include/FEM.hpp:33-34, src/FEM.cpp:157-554
 *   applyBoundaryConditions(f, loads, ...) include/FEM.hpp:63-64, src/FEM.cpp:568-584
 *   solveWithKompute(A, f, u)              include/FEMGPU.hpp:11-12, src/FEMGPU.cpp:32-554
 *   solveWithEigen(A, f, u)                include/FEM.hpp:72-73,   src/FEM.cpp:589-637
 *   MatrixFreeSparse<double> * x           include/MatrixFreeSparse.hpp:31-94,191-215
 *   MultigridPreconditioner::solve(b)      include/MultigridPreconditioner.hpp:24-203
 *   MultigridPreconditioner::restrict / interpolate
 *                                          include/MultigridPreconditioner.hpp:67-155
 *
 * Conventions (the reference's, src/FEM.cpp:66-198):
 *   - voxels: uint8 occupancy, 1 = filled, x fastest, then y, then z;
 *   - a node is used when a filled voxel touches it; used nodes are numbered
 *     0..n-1 in increasing linear order (x fastest) over the node grid;
 *   - vectors are in that compressed numbering, DOF = 3*node + component;
 *   - Ke is 24x24 row-major; only its upper triangle is read and the matrix is
 *     symmetrised from it (src/FEM.cpp:200-210); element-local node
 *     a = dx + 2*dy + 4*dz, local DOF 3*a + c.
 * All pointers are host pointers unless a name ends in _device.  Every call
 * returns a vfem_status; nothing aborts.  A problem is not thread-safe: calls on
 * one problem must be serialised.  Work runs on the problem's own CUDA stream.
 */
#ifndef VFEM_H
#define VFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum vfem_status {
    VFEM_OK = 0,
    VFEM_ERR_INVALID_ARGUMENT = 1,  /* bad size, null pointer, out-of-range id */
    VFEM_ERR_CUDA = 2,              /* a CUDA runtime/library call failed */
    VFEM_ERR_OUT_OF_MEMORY = 3,
    VFEM_ERR_NOT_CONVERGED = 4,     /* max iterations reached above tolerance */
    VFEM_ERR_BREAKDOWN = 5,         /* p^T A p <= 0 or a non-finite scalar */
    VFEM_ERR_SINGULAR = 6,          /* coarsest system not positive definite */
    VFEM_ERR_EMPTY = 7,             /* no filled voxel */
    VFEM_ERR_COARSE_TOO_LARGE = 8,  /* coarsest free DOFs above the dense limit */
    VFEM_ERR_NO_DEVICE = 9,
    VFEM_ERR_TIMEOUT = 10
} vfem_status;

typedef struct vfem_problem vfem_problem;

/* Multigrid flavour. */
typedef enum vfem_mg_mode {
    VFEM_MG_REFERENCE = 0,  /* the reference's additive V-cycle: z_l = 2 D^-1 r_l + W o P^T z_(l+1)
                               (MultigridPreconditioner.hpp:158-193) */
    VFEM_MG_VCYCLE = 1,     /* multiplicative V-cycle, damped Jacobi (omega, pre/post sweeps) */
    VFEM_MG_NONE = 2        /* identity preconditioner (plain CG) */
} vfem_mg_mode;

typedef enum vfem_precision {
    VFEM_PREC_FP64 = 0,     /* plain FP64 MG-PCG */
    VFEM_PREC_MIXED = 1     /* FP32 CG + FP32 V-cycle, FP64 reductions, FP64 solution accumulation,
                               true residual f - K x in double-float arithmetic substituted for the
                               recursive one (reliable updates, `replace_delta`, `replace_every`)
                               and checked at exit */
} vfem_precision;

typedef struct vfem_options {
    double rtol;             /* relative residual tolerance (TOLERANCE, FEMDefines.hpp:7); default 1e-6 */
    int64_t max_iter;        /* <= 0: Eigen's default 2 * ndof (FEM.cpp:617-619) */
    int32_t mg_mode;         /* vfem_mg_mode */
    int32_t precision;       /* vfem_precision */
    double omega;            /* damped-Jacobi weight for VFEM_MG_VCYCLE; default 0.6 */
    int32_t pre_sweeps;      /* VFEM_MG_VCYCLE only; default 1 */
    int32_t post_sweeps;     /* VFEM_MG_VCYCLE only; default 1 */
    int32_t replace_every;   /* mixed precision: also replace the residual every this many iterations;
                                default 0 = off (replacements follow replace_delta) */
    int32_t flexible;        /* 1: flexible CG (Polak-Ribiere beta); default 0 (Fletcher-Reeves, as Eigen) */
    int32_t check_every;     /* iterations per device-side chunk between host polls; default 8 */
    int32_t compute_true_residual; /* 1: report the true FP64 residual at exit (one extra FP64 product
                                      outside the timed solve for VFEM_PREC_FP64); default 1 */
    double replace_delta;    /* mixed precision: replace the residual once |r| has dropped by this
                                factor since the last replacement (reliable updates); default 0.05,
                                0 = off.  A recursive residual that claims convergence is always
                                replaced and re-checked. */
    int32_t fallback_fp64;   /* mixed precision: when the mixed solve ends in VFEM_ERR_BREAKDOWN, or
                                stops short of rtol (stagnating true residual, or max_iter), plain
                                FP64 MG-PCG continues from its iterate (from 0 if that iterate is not
                                finite) with the iterations left of max_iter; default 1 */
    int32_t debug_break_at;  /* testing: the solve's p^T A p at this iteration (1-based) is taken
                                as -1, a forced VFEM_ERR_BREAKDOWN (a fallback phase does not
                                inherit it); default 0 = off */
    int32_t reserved[4];
} vfem_options;

typedef struct vfem_stats {
    int64_t iterations;      /* PCG iterations, counted as Eigen counts them */
    int64_t matvecs;         /* fine-level operator applications of the outer loop */
    int64_t residual_replacements;
    double rel_residual;     /* true FP64 ||f - K u|| / ||f|| at exit */
    double recursive_rel_residual; /* sqrt(r.r / f.f) of the recursive residual (Eigen's error()) */
    double solve_ms;         /* device time of the solve (CUDA events) */
    double h2d_ms, d2h_ms;   /* copies inside vfem_solve */
    int64_t kernel_launches; /* kernels launched by this call */
    int32_t status;          /* vfem_status of the solve */
    int32_t fallback;        /* 1: the mixed solve failed and plain FP64 MG-PCG continued (fallback_fp64) */
    int64_t fallback_iterations; /* iterations of that FP64 phase (included in `iterations`) */
    int32_t reserved[4];
} vfem_stats;

/* Fill `opt` with the defaults listed above. */
void vfem_options_default(vfem_options* opt);

/* Human-readable name of a status code. */
const char* vfem_status_string(vfem_status s);

/* 24x24 stiffness of a unit trilinear hexahedron with 2x2x2 Gauss quadrature,
 * node order x fastest (host-only helper, no GPU needed). */
vfem_status vfem_hex8_stiffness(double E, double nu, double* Ke_out);

/* assembleSystemMatrix<double>(voxels, dims, Ke, fixedNodes, numLevels, skipLevels)
 * (include/FEM.hpp:33-34).  E_or_null: per-voxel Young's modulus multiplier
 * (same layout as voxels) or NULL for a uniform 1.  fixed_nodes: compressed node
 * ids (0-based); at least one is required (VFEM_ERR_INVALID_ARGUMENT otherwise:
 * without fixed nodes the stiffness is singular through its rigid-body modes,
 * which the reference does not check).  Every connected component of the
 * voxels must contain a fixed node for the same reason; that is not checked.
 * num_levels >= 1; skip_levels in {0, 1} (4x first coarsening,
 * FEM.cpp:266-272).  The hierarchy stops early when a dimension reaches <= 2
 * elements (FEM.cpp:465-470). */
vfem_status vfem_problem_create(const uint8_t* voxels, int32_t nx, int32_t ny, int32_t nz,
                                const double* Ke, const float* E_or_null,
                                const int64_t* fixed_nodes, int64_t nfixed,
                                int32_t num_levels, int32_t skip_levels,
                                vfem_problem** out);

void vfem_problem_destroy(vfem_problem* p);

/* Sizes: number of used nodes at `level` (3x for DOFs), levels actually built,
 * coarsest free DOFs. */
vfem_status vfem_problem_info(const vfem_problem* p, int32_t level, int64_t* num_nodes,
                              int64_t* num_elements, int32_t* num_levels, int64_t* coarse_free_dofs);

/* applyBoundaryConditions (FEM.cpp:568-584): f[3*node + c] = loads[3*k + c].
 * Replaces any previous loads. */
vfem_status vfem_problem_set_loads(vfem_problem* p, const int64_t* nodes, const double* loads_xyz,
                                   int64_t n);

/* Set the right-hand side directly: f has 3 * num_nodes entries. */
vfem_status vfem_problem_set_rhs(vfem_problem* p, const double* f);

/* solveWithKompute / solveWithEigen: solve K u = f to opt->rtol.  u0_or_null:
 * initial guess (compressed numbering) or NULL for 0.  u_out: 3 * num_nodes. */
vfem_status vfem_solve(vfem_problem* p, const vfem_options* opt, const double* u0_or_null,
                       double* u_out, vfem_stats* st);

/* The same solve with the right-hand side already on the device (set by
 * vfem_problem_set_loads / set_rhs) and the solution left on the device; used to
 * time the device-resident path.  u_out_or_null receives the solution if given. */
vfem_status vfem_solve_device(vfem_problem* p, const vfem_options* opt, double* u_out_or_null,
                              vfem_stats* st);

/* MatrixFreeSparse product (MatrixFreeSparse.hpp:197-214): y = K x with the
 * fixed rows zeroed. */
vfem_status vfem_apply_operator(vfem_problem* p, const double* x, double* y);

/* Deflation coarse space (no counterpart in the reference; deflated PCG after
 * Saad, Yeung, Erhel and Guyomarc'h, SIAM J. Sci. Comput. 21 (2000), in the
 * A-DEF2 form of Tang, Nabben, Vuik and Erlangga, J. Sci. Comput. 39 (2009)).
 * V holds k <= 4 columns (compressed numbering, column j at V + j * 3 *
 * num_nodes); entries at fixed DOFs are taken as 0.  Every later solve starts
 * from x0 + V G^-1 V^T r0 (G = V^T K V, K V computed once here with the FP64
 * product) and every later preconditioner application, in solves and in
 * vfem_apply_preconditioner(_mixed), returns
 *   z = M^-1 r + V G^-1 (V^T r - (KV)^T M^-1 r),
 * with M^-1 the multigrid cycle (the identity for VFEM_MG_NONE).  For the
 * residuals of such a solve (orthogonal to V) this keeps every search direction
 * K-orthogonal to V, which cannot raise CG's effective condition number.  The
 * learned coarse correction passes the network's predicted displacement here
 * (vulkanfem_gb300/learned.py).  k = 0 removes it.  Storage: 2 k FP64 and 2 k
 * FP32 dense level-0 vectors.  VFEM_ERR_INVALID_ARGUMENT if V has a non-finite
 * entry or V^T K V is singular. */
vfem_status vfem_problem_set_coarse_space(vfem_problem* p, const double* V, int32_t k);

/* The same product as the mixed-precision solver applies it (no counterpart in
 * the reference): x rounded to FP32, y = K x with the fixed rows zeroed computed
 * in FP32 (on the tensor cores when vfem_problem_uses_tensor_cores is 1, else on
 * the CUDA cores), returned in FP64; xKx_or_null receives x.(Kx) summed in FP64. */
vfem_status vfem_apply_operator_mixed(vfem_problem* p, const double* x, double* y, double* xKx_or_null);

/* 1 when the mixed-precision solver's CG product runs on the tensor cores.  It
 * does when the environment variable VFEM_TENSOR_CORE_PRODUCT was set to a
 * non-zero value when the problem was created and Ke times some integer
 * q <= 65536 is integer-valued and exact in BF16 (q = 1872 for the 2x2x2-Gauss
 * hex at nu = 0.3).  Off by default: on GB300 the CUDA-core product is faster. */
int32_t vfem_problem_uses_tensor_cores(const vfem_problem* p);

/* Which staged transfer kernels the problem's mixed-precision V-cycle uses, as
 * bits: 1 = the FP32 2x restrictions stage their fine rows with TMA tensor
 * loads, 2 = the 2x up-leg stages its ranges with bulk copies.  Set from the
 * environment variable VFEM_TMA_MASK when the problem is created; default 0:
 * on GB300 both measured slower than the kernels that load directly. */
int32_t vfem_problem_uses_tma(const vfem_problem* p);

/* No counterpart in the reference.  The operator product of vfem_apply_operator
 * for callers that cannot allocate GPU memory at the point of the call: hosts
 * that hand every byte of device memory to their own pool up front (a solver
 * framework or plugin that owns the device), and loops that must not stall on
 * cudaMalloc's implicit device synchronisation.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.  The caller passes device arrays:
 * x_device and y_device hold 3 doubles per node of the full node grid,
 * (nx+1)*(ny+1)*(nz+1) nodes, x fastest (the grid index replaces the compressed
 * node id).  Values of x at unused nodes are ignored, even non-finite ones; y is
 * written at every grid node, 0 at unused nodes and fixed rows; xKx_device
 * receives x.(Kx) in FP64, summed over the used, free nodes.  Work is enqueued on
 * `stream` (a cudaStream_t; NULL = the default stream); the call returns without
 * synchronising.
 * Scratch: a fixed 1,049,600-byte device array inside the library (reduction
 * partials for up to 65,536 product blocks of 31 x 7 x 32 nodes, i.e. node grids
 * up to about 760^3 for a cube); larger grids are rejected with
 * VFEM_ERR_INVALID_ARGUMENT.  Every GPU that loads the library holds the array
 * until the process exits.  All calls share it and it keeps the last call's
 * contents; each call clears what must start at zero, but calls that overlap on
 * the GPU race.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current: make that first call before
 * any stream capture. */
vfem_status vfem_apply_operator_device_noalloc(vfem_problem* p, const double* x_device, double* y_device,
                                               double* xKx_device, void* stream);

/* MultigridPreconditioner::solve (MultigridPreconditioner.hpp:158-193): one
 * V-cycle of `mg_mode` (VFEM_MG_REFERENCE or VFEM_MG_VCYCLE) in FP64. */
vfem_status vfem_apply_preconditioner(vfem_problem* p, int32_t mg_mode, const double* r, double* z);

/* The same V-cycle as the mixed-precision solver applies it (no counterpart in
 * the reference): FP32 vectors, FP16 coarsest inverse tiles and, in the
 * reference cycle, an FP16 inverse diagonal; r and z in FP64. */
vfem_status vfem_apply_preconditioner_mixed(vfem_problem* p, int32_t mg_mode, const double* r, double* z);

/* MultigridPreconditioner::restrict / interpolate (MultigridPreconditioner.hpp:67-155)
 * between `level` (fine) and `level + 1` (coarse), compressed numbering of each
 * level. */
vfem_status vfem_restrict(vfem_problem* p, int32_t level, const double* fine, double* coarse);
vfem_status vfem_interpolate(vfem_problem* p, int32_t level, const double* coarse, double* fine);

/* Inverse diagonal used by the smoother on `level` (invDiagKOnLevels,
 * FEM.cpp:105-151,463), compressed numbering. */
vfem_status vfem_inverse_diagonal(vfem_problem* p, int32_t level, double* out);

/* Fixed nodes of `level` (fixedNodesInLevels, FEM.cpp:402-460): writes up to
 * `cap` compressed ids and the total count. */
vfem_status vfem_fixed_nodes(vfem_problem* p, int32_t level, int64_t* out, int64_t cap, int64_t* count);

/* Kernel classes timed by vfem_profile_kernels. */
typedef enum vfem_kernel_class {
    VFEM_K_MATVEC_FP64 = 0,
    VFEM_K_MATVEC_FP32 = 1,
    VFEM_K_RESTRICT_FP64 = 2,
    VFEM_K_RESTRICT_FP32 = 3,
    VFEM_K_PROLONG_FP64 = 4,
    VFEM_K_PROLONG_FP32 = 5,
    VFEM_K_UPDATE_XR_FP64 = 6,
    VFEM_K_UPDATE_XR_MIXED = 7,   /* mixed: r -= alpha Ap and r.r (x += alpha p is deferred to the p update) */
    VFEM_K_UPDATE_P_FP64 = 8,
    VFEM_K_UPDATE_P_FP32 = 9,     /* mixed: p = z + beta p with the deferred x += alpha p */
    VFEM_K_COARSE_FP64 = 10,
    VFEM_K_COARSE_FP32 = 11,
    VFEM_K_TRUE_RESIDUAL_DF = 12, /* f - K x on FP64 vectors in double-float arithmetic */
    VFEM_K_UPDATE_RESTRICT_MIXED = 13, /* mixed: r -= alpha Ap, r.r and the first restriction in one pass */
    VFEM_K_MATVEC_FP32_SIMT = 14, /* the FP32 CG product on the CUDA cores, whichever product the problem uses */
    VFEM_K_MATVEC_FP32_PX = 15,   /* the mixed solve's FP32 CG product with the direction update (p = z + beta p,
                                     x += alpha p) fused into it; 0 ms when the problem does not use it */
    VFEM_K_COUNT = 16
} vfem_kernel_class;

/* Measurement helper (no counterpart in the reference): average device time in
 * milliseconds of `reps` back-to-back launches of each kernel class on the finest
 * level (transfers between levels 0 and 1; coarse = the coarsest dense solve),
 * timed with CUDA events on the problem's stream.  ms_out has VFEM_K_COUNT
 * entries.  Overwrites the problem's work vectors. */
vfem_status vfem_profile_kernels(vfem_problem* p, int32_t reps, double* ms_out);

/* Number of kernels this library has launched in this process (all problems). */
int64_t vfem_kernel_launch_count(void);

/* Message of the last failing call on this thread ("" if none). */
const char* vfem_last_error_message(void);

#ifdef __cplusplus
}
#endif

#endif /* VFEM_H */
