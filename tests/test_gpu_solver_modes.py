"""GPU tests of the solver forms beside the default one, and of the failure paths.

* Plain CG (``mg_mode="none"``): the reference's matrix-free CG without the
  multigrid preconditioner (``Eigen::IdentityPreconditioner``, src/FEM.cpp:608-611;
  the non-MULTIGRID branch of src/FEMGPU.cpp:152-165), FP64 and mixed precision,
  against the oracle's identity-preconditioned CG.
* The porous FP32-vs-FP64 configuration at a reduced size (the 128^3 Gaussian
  random field at 40% fill, here 48^3 with the same generator).
* Failure paths, all made on the host or by a flag in the device scalars (no
  GPU fault): a forced non-convergence (max_iter), a forced breakdown
  (``debug_break_at``: the solve takes p^T A p as -1 at that iteration) with the
  mixed solve's FP64 fallback, and injected device-allocation failures during
  set-up (``VFEM_FAULT_ALLOC_AT``), after each of which the library stays usable.
* The 64-bit coarsest factorisation path (normally above 32,768 free DOFs),
  forced on a small problem with ``VFEM_COARSE_64BIT_MIN``.

Tolerances: iteration counts within +-1 (multigrid) of the oracle; displacement
within 1e-5 relative L2 of the oracle's answer at the same rtol (the bar of the
reference's CPU path); true relative residual < 1e-6.
"""
import os

import numpy as np
import pytest

import oracle
from vulkanfem_gb300 import api, domains

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _random_box(shape, fill, seed):
    rng = np.random.default_rng(seed)
    vox = (rng.random(shape) < fill).astype(np.uint8)
    vox[0] = 1
    vox = domains.keep_grounded(vox)
    ids = domains.node_numbering(vox)
    fixed = np.sort(ids[0][ids[0] >= 0])
    top = np.sort(ids[-1][ids[-1] >= 0])
    lv = np.zeros((top.size, 3))
    lv[:, 2] = -1.0 / max(top.size, 1)
    return vox, fixed, top, lv


@pytest.fixture(scope="module")
def small():
    vox, fixed, ln, lv = _random_box((12, 14, 16), 0.75, 11)
    ke = domains.hex8_stiffness()
    o = oracle.Oracle(vox, ke, fixed, 3, 0)
    A = api.assembleSystemMatrix(vox, ke, fixed, 3, 0)
    f = np.zeros(o.num_dofs())
    f.reshape(-1, 3)[ln] = lv
    x_o, it_o, _ = o.pcg(f, tol=1e-6)
    return {"vox": vox, "fixed": fixed, "ke": ke, "o": o, "A": A, "f": f, "x_o": x_o, "it_o": it_o}


def test_plain_cg_matches_oracle(small):
    o, A, f = small["o"], small["A"], small["f"]
    x_cg, it_cg, _ = o.pcg(f, tol=1e-6, use_mg=False)
    u, st = A.solve(f, mg_mode="none")
    # unpreconditioned CG is sensitive to the summation order: a few iterations either way
    assert abs(st["iterations"] - it_cg) <= max(3, it_cg // 50), (st["iterations"], it_cg)
    assert st["rel_residual"] < 1e-6
    assert rel(u, x_cg) < 1e-5
    assert rel(u, small["x_o"]) < 1e-5
    um, stm = A.solve(f, mg_mode="none", precision="mixed")
    assert stm["rel_residual"] < 1e-6 and stm["fallback"] == 0
    assert rel(um, x_cg) < 1e-5
    print("plain CG: oracle %d, fp64 %d, mixed %d iterations (MG-PCG: %d)"
          % (it_cg, st["iterations"], stm["iterations"], small["it_o"]))


def test_porous_fp32_vs_fp64_reduced():
    """The porous configuration (seeded Gaussian random field, sigma 6 voxels,
    40% fill, grounded component, z = 0 fixed, unit -z top load) at 48^3 with 3
    levels: FP64 and mixed precision against the oracle."""
    d = domains.porous(48, 0.40, 6.0, seed=0, levels=3)
    ke = domains.hex8_stiffness()
    o = oracle.Oracle(d.voxels, ke, d.fixed, 3, 0, threads=os.cpu_count() or 1)
    A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3, 0)
    f = o.load_vector(d.load_nodes, d.load_values)
    x_o, it_o, _ = o.pcg(f, tol=1e-6)
    u64, s64 = A.solve(f)
    um, sm = A.solve(f, precision="mixed")
    assert abs(s64["iterations"] - it_o) <= 1
    assert s64["rel_residual"] < 1e-6 and sm["rel_residual"] < 1e-6
    assert rel(u64, x_o) < 1e-5
    assert rel(um, x_o) < 1e-5
    assert sm["iterations"] <= 1.05 * it_o + 2
    print("porous48: oracle %d, fp64 %d, mixed %d iterations; mixed vs oracle %.2e, vs fp64 %.2e"
          % (it_o, s64["iterations"], sm["iterations"], rel(um, x_o), rel(um, u64)))


def test_forced_nonconvergence_status(small):
    A, f = small["A"], small["f"]
    for prec in ("fp64", "mixed"):
        u, st = A.solve(f, precision=prec, max_iter=3, allow_not_converged=True)
        assert st["status"] == 4 and st["iterations"] == 3, (prec, st)
        assert st["fallback"] == 0                        # the whole budget is spent
        with pytest.raises(api.VfemError) as ei:
            A.solve(f, precision=prec, max_iter=3)
        assert ei.value.status == 4
    u, st = A.solve(f)                                    # still usable
    assert st["status"] == 0 and st["iterations"] == small["it_o"]


def test_forced_breakdown_and_fp64_fallback(small):
    A, f = small["A"], small["f"]
    u_ref, st_ref = A.solve(f)
    with pytest.raises(api.VfemError) as ei:
        A.solve(f, debug_break_at=5)
    assert ei.value.status == 5                           # VFEM_ERR_BREAKDOWN
    with pytest.raises(api.VfemError) as ei:
        A.solve(f, precision="mixed", debug_break_at=5, fallback_fp64=False)
    assert ei.value.status == 5
    u, st = A.solve(f, precision="mixed", debug_break_at=5)
    assert st["status"] == 0 and st["fallback"] == 1
    assert st["fallback_iterations"] > 0 and st["iterations"] == 4 + st["fallback_iterations"]
    assert st["rel_residual"] < 1e-6
    assert rel(u, small["x_o"]) < 1e-5
    u2, st2 = A.solve(f)                                  # the problem is unchanged
    assert np.array_equal(u2, u_ref) and st2["iterations"] == st_ref["iterations"]


def test_injected_allocation_failures_leave_library_usable(small):
    torch = pytest.importorskip("torch")
    vox, fixed, ke = small["vox"], small["fixed"], small["ke"]
    api.assembleSystemMatrix(vox, ke, fixed, 3, 0).close()  # warm-up: kernels loaded
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failed = 0
    try:
        for k in (1, 2, 3, 5, 8, 13, 21, 34, 55, 89):
            os.environ["VFEM_FAULT_ALLOC_AT"] = str(k)
            try:
                api.assembleSystemMatrix(vox, ke, fixed, 3, 0).close()
            except api.VfemError as e:
                assert e.status == 3, e                   # VFEM_ERR_OUT_OF_MEMORY
                failed += 1
    finally:
        os.environ.pop("VFEM_FAULT_ALLOC_AT", None)
    assert failed >= 8
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) <= 16 << 20   # nothing leaked
    A = api.assembleSystemMatrix(vox, ke, fixed, 3, 0)
    u, st = A.solve(small["f"])
    assert st["iterations"] == small["it_o"] and rel(u, small["x_o"]) < 1e-5


def test_forced_64bit_coarse_factorisation(small):
    """The path for coarsest systems above 32,768 free DOFs (64-bit Cholesky,
    triangular inverse, syrk), forced on a small problem: the same FP64
    preconditioner as the 32-bit path to 1e-10, and the same mixed solve."""
    vox, fixed, ke, A = small["vox"], small["fixed"], small["ke"], small["A"]
    os.environ["VFEM_COARSE_64BIT_MIN"] = "16"
    try:
        B = api.assembleSystemMatrix(vox, ke, fixed, 3, 0)
    finally:
        os.environ.pop("VFEM_COARSE_64BIT_MIN", None)
    assert B.coarse_free_dofs > 16
    r = np.random.default_rng(5).standard_normal(A.rows())
    assert rel(api.MultigridPreconditioner(B).solve(r), api.MultigridPreconditioner(A).solve(r)) < 1e-10
    zb = api.MultigridPreconditioner(B, precision="mixed").solve(r)
    za = api.MultigridPreconditioner(A, precision="mixed").solve(r)
    assert rel(zb, za) < 1e-3
    u, st = B.solve(small["f"], precision="mixed")
    assert st["rel_residual"] < 1e-6 and rel(u, small["x_o"]) < 1e-5


def test_fused_direction_update_is_bit_identical():
    """The mixed solve's direction update fused into the CG product
    (p = z + beta p_old and the deferred x += alpha p_old in the product's input
    stage, alternating p buffers) against the separate update pass
    (VFEM_FUSED_DIRECTION=0): the same arithmetic on the same values, so the
    same iteration counts and bit-identical displacements, for the reference
    and multiplicative cycles, plain and flexible CG, periodic residual
    replacement, and the FP64 fallback after a forced breakdown.  The 40^3
    field spans several product blocks in x, y and z."""
    ke = domains.hex8_stiffness()
    d = domains.training_field(40, seed=7, levels=3)
    os.environ["VFEM_FUSED_DIRECTION"] = "0"
    try:
        B = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3)
    finally:
        os.environ.pop("VFEM_FUSED_DIRECTION", None)
    A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3)
    ms = api.profile_kernels(A, 1)
    assert ms["matvec_fp32_px"] > 0 and api.profile_kernels(B, 1)["matvec_fp32_px"] == 0
    f = d.load_vector()
    cases = [dict(), dict(mg_mode="vcycle"), dict(mg_mode="none"), dict(flexible=True),
             dict(replace_every=7), dict(debug_break_at=9)]
    for opts in cases:
        ua, sa = A.solve(f, precision="mixed", **opts)
        ub, sb = B.solve(f, precision="mixed", **opts)
        assert sa["iterations"] == sb["iterations"], (opts, sa["iterations"], sb["iterations"])
        assert sa["fallback"] == sb["fallback"]
        assert np.array_equal(ua, ub), (opts, rel(ua, ub))
        assert sa["rel_residual"] < 1e-6
    A.close()
    B.close()
