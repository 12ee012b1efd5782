"""GPU parity of the tensor-core FP32 CG product (matvec_tc.cu, opt-in with
VFEM_TENSOR_CORE_PRODUCT=1) against the FP64 product, which itself matches the
oracle to 1e-11 (test_gpu_parity.py).

The mixed-precision solver's product y = K x (fixed rows zeroed, the reference's
MatrixFreeSparse product, include/MatrixFreeSparse.hpp:197-214) takes x rounded
to FP32 and accumulates in FP32: relative L2 error below 1e-6 of the FP64
product, for the tensor-core kernel and for the CUDA-core kernel (the default),
on grids that cover several CTA tiles in every direction, odd sizes, a skipped
level, per-voxel moduli and several 32-layer z chunks.  Fixed rows are exactly
zero; x.(Kx) agrees to 1e-6 relative; repeated products are bit-identical.
"""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT
from vulkanfem_gb300 import api, domains

pytestmark = pytest.mark.gpu

TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _box(shape, fill, seed):
    rng = np.random.default_rng(seed)
    vox = (rng.random(shape) < fill).astype(np.uint8)
    vox[0] = 1
    vox = domains.keep_grounded(vox)
    ids = domains.node_numbering(vox)
    fixed = np.sort(ids[0][ids[0] >= 0])
    return vox, fixed


CASES = {
    "cantilever": lambda: (lambda d: (d.voxels, d.fixed, None, 3, 0))(domains.cantilever()),
    "odd_7x5x3": lambda: _box((3, 5, 7), 0.8, 5) + (None, 2, 0),
    "tiles_70x45x40": lambda: _box((70, 45, 40), 0.7, 8) + (None, 3, 0),
    "skip_33x40x36": lambda: _box((33, 40, 36), 0.75, 2) + (None, 3, 1),
    "spheres48_lognormal": lambda: (lambda d: (d.voxels, d.fixed, d.E, 3, 0))(
        domains.spheres(48, 6, 2, 6, seed=4, levels=3, lognormal_sigma=0.5)),
}


def _make(name, tensor_cores):
    vox, fixed, E, levels, skip = CASES[name]()
    if tensor_cores:
        os.environ["VFEM_TENSOR_CORE_PRODUCT"] = "1"
    try:
        return api.assembleSystemMatrix(vox, domains.hex8_stiffness(), fixed, levels, skip, E=E), fixed
    finally:
        os.environ.pop("VFEM_TENSOR_CORE_PRODUCT", None)


@pytest.mark.parametrize("name", sorted(CASES))
def test_tensor_core_product_matches_fp64(name):
    A, fixed = _make(name, True)
    S, _ = _make(name, False)
    assert A.uses_tensor_cores and not S.uses_tensor_cores
    rng = np.random.default_rng(17)
    for trial in range(2):
        x = rng.standard_normal(A.rows())
        y64 = A @ x
        y_tc, d_tc = A.dot_mixed(x)
        y_ct, d_ct = S.dot_mixed(x)
        e_tc, e_ct = rel(y_tc, y64), rel(y_ct, y64)
        print("%s: tensor-core product %.2e, CUDA-core product %.2e (relative L2 vs FP64)" % (name, e_tc, e_ct))
        assert e_tc < TOL and e_ct < TOL
        assert np.all(y_tc.reshape(-1, 3)[np.asarray(fixed, np.int64)] == 0.0)
        ref_dot = float(x @ y64)
        assert abs(d_tc - ref_dot) <= TOL * abs(ref_dot)
        assert abs(d_ct - ref_dot) <= TOL * abs(ref_dot)
        y2, d2 = A.dot_mixed(x)  # fixed summation order: bit-identical
        assert np.array_equal(y2, y_tc) and d2 == d_tc
    A.close()
    S.close()


def test_tensor_core_and_cuda_core_solves_agree():
    """The mixed solve with either product converges to the same answer in about
    the same number of iterations, without the FP64 fallback."""
    A, _ = _make("spheres48_lognormal", True)
    S, _ = _make("spheres48_lognormal", False)
    d = domains.spheres(48, 6, 2, 6, seed=4, levels=3, lognormal_sigma=0.5)
    f = d.load_vector()
    u_tc, st_tc = A.solve(f, precision="mixed")
    u_ct, st_ct = S.solve(f, precision="mixed")
    u64, st64 = A.solve(f)
    assert st_tc["fallback"] == 0 and st_tc["rel_residual"] < 1e-6
    assert abs(st_tc["iterations"] - st_ct["iterations"]) <= 2
    assert rel(u_tc, u64) < 1e-5 and rel(u_ct, u64) < 1e-5
    print("iterations: tensor-core %d, CUDA-core %d, FP64 %d"
          % (st_tc["iterations"], st_ct["iterations"], st64["iterations"]))


def test_mma_rate_measurement(tmp_path):
    """Builds and runs tests/tcgen05_rate.cu, the measurement behind keeping the
    tensor-core product off by default: a single thread issues BF16
    tcgen05.mma (M = 128, K = 16) back to back for N = 32 .. 256 and the
    program prints ns per MMA.  Checks that every batch completed and that
    N = 32 costs at least as much time per MMA as N = 256 costs per N = 32 of
    its work (small-N MMAs do not run at the tensor pipe's rate)."""
    exe = tmp_path / "tcgen05_rate"
    src = os.path.join(ROOT, "tests", "tcgen05_rate.cu")
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", str(exe), src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    per = {}
    for line in out.stdout.splitlines():
        parts = line.split()
        if line.startswith("N=") and "reps=2400" in line.replace(" ", ""):
            per[int(line[2:5])] = float(line.split("(")[2].split()[0])
    assert set(per) == {32, 64, 128, 256}, out.stdout
    assert per[32] >= per[256] / 8.0
