"""GPU parity of the staged FP32 transfers (transfer_tma.cu: the restriction
with TMA-staged fine rows and the mixed up-leg with bulk-staged ranges) against
the default kernels (kRestrict2, kProlongFlat).  The staged kernels are opt-in
(VFEM_TMA_MASK=3 when the problem is created): on GB300 they measured slower.

Both pairs compute the reference's transfers
(include/MultigridPreconditioner.hpp:67-155) with the same FP32 expressions per
node; only the grouping of the dot-product partial sums over threads and
blocks differs.  So the mixed V-cycle agrees to 1e-6 relative (FP32 rounding
of the r.r and r.z reductions only), and the
mixed solve takes the same iteration count (+-1) to the same answer (1e-6).
Cases cover several CTAs in every direction, odd fine sizes, coarse layer
counts that are not a multiple of the CTA's 4 and the 4x skipped level (which
keeps its own kernels).
"""
import os

import numpy as np
import pytest

from vulkanfem_gb300 import api, domains

pytestmark = pytest.mark.gpu


def _box(shape, fill, seed):
    rng = np.random.default_rng(seed)
    vox = (rng.random(shape) < fill).astype(np.uint8)
    vox[0] = 1
    vox = domains.keep_grounded(vox)
    ids = domains.node_numbering(vox)
    fixed = np.sort(ids[0][ids[0] >= 0])
    top = np.sort(ids[-1][ids[-1] >= 0])
    f_nodes, f_vals = top, np.tile([0.0, 0.0, -1.0 / max(top.size, 1)], (top.size, 1))
    return vox, fixed, f_nodes, f_vals


CASES = {
    "odd_7x5x3": lambda: _box((3, 5, 7), 0.8, 5) + (2, 0),
    "box_70x45x40": lambda: _box((40, 45, 70), 0.7, 8) + (4, 0),
    "box_33x66x27": lambda: _box((27, 66, 33), 0.75, 3) + (3, 0),
    "skip_34x36x40": lambda: _box((40, 36, 34), 0.75, 2) + (3, 1),
}


def _make(vox, fixed, levels, skip, tma):
    if tma:
        os.environ["VFEM_TMA_MASK"] = "3"
    try:
        return api.assembleSystemMatrix(vox, domains.hex8_stiffness(), fixed, levels, skip)
    finally:
        os.environ.pop("VFEM_TMA_MASK", None)


@pytest.mark.parametrize("name", sorted(CASES))
def test_staged_transfers_match(name):
    vox, fixed, ln, lv, levels, skip = CASES[name]()
    A = _make(vox, fixed, levels, skip, True)
    B = _make(vox, fixed, levels, skip, False)
    assert A._lib.vfem_problem_uses_tma(A._h) == 3 and not B.uses_tma
    r = np.random.default_rng(11).standard_normal(A.rows())
    za = api.MultigridPreconditioner(A, precision="mixed").solve(r)
    zb = api.MultigridPreconditioner(B, precision="mixed").solve(r)
    assert np.linalg.norm(za - zb) <= 1e-6 * np.linalg.norm(zb)
    f = np.zeros(A.rows())
    f.reshape(-1, 3)[ln] = lv
    ua, sa = A.solve(f, precision="mixed")
    ub, sb = B.solve(f, precision="mixed")
    assert abs(sa["iterations"] - sb["iterations"]) <= 1 and sa["fallback"] == 0
    assert np.linalg.norm(ua - ub) <= 1e-6 * np.linalg.norm(ub)
    assert sa["rel_residual"] < 1e-6
