"""GPU tests of the learned part (BF16 U-Net kernels in csrc/unet.cu).

Forward outputs and parameter gradients of the CUDA kernels are checked against
the numpy restatement (tests/unet_ref.py, same BF16 rounding points, float64
sums): relative L2 error <= 2e-2 for the output and for every layer's weight
and bias gradient (BF16 storage, FP32 tensor-core accumulation); repeated
gradients are bit-identical.
"""
import numpy as np
import pytest

from tests import unet_ref as U
from vulkanfem_gb300 import domains, learned

pytestmark = pytest.mark.gpu

TOL = 2e-2


def _rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, n, n, 16), np.float32)
    x[..., :6] = rng.standard_normal((n, n, n, 6)) * 0.5
    t = (rng.standard_normal((n, n, n, 3)) * 0.1).astype(np.float32)
    m = (rng.random((n, n, n)) < 0.8).astype(np.float32)
    return x, t, m


def test_unet_forward_and_gradients_match_numpy():
    U.ROUND = True
    n = 16
    p = U.init_params(3)
    net = learned.UNet(n, p)
    x, t, m = _problem(n, 0)
    y_gpu = net.forward(x)
    loss_ref, g_ref, y_ref = U.loss_and_grads(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64),
                                              m.astype(np.float64))
    assert _rel(y_gpu, y_ref[..., :3]) < TOL
    loss, g = net.train_batch(x[None], t[None], m[None], 0.0, want_grads=True)
    assert loss == pytest.approx(loss_ref, rel=TOL)
    lay, _ = U.param_layout()
    for l, ((w0, w1), (b0, b1)) in enumerate(lay):
        assert _rel(g[w0:w1], g_ref[w0:w1]) < TOL, ("weights", l, _rel(g[w0:w1], g_ref[w0:w1]))
        assert _rel(g[b0:b1], g_ref[b0:b1]) < TOL, ("bias", l, _rel(g[b0:b1], g_ref[b0:b1]))
    # batch of two identical samples: same mean gradient
    _, g2 = net.train_batch(np.stack([x, x]), np.stack([t, t]), np.stack([m, m]), 0.0, want_grads=True)
    assert _rel(g2, g) < 1e-5
    # the weight gradient sums its voxel chunks in a fixed order: bit-reproducible
    _, g3 = net.train_batch(x[None], t[None], m[None], 0.0, want_grads=True)
    assert np.array_equal(g3, g)


@pytest.fixture(scope="module")
def trained():
    """A net trained with the library's own kernels on 12 solver outputs (24^3)."""
    X, T, M = learned.generate(12, n=24, seed0=100, levels=3)
    net = learned.UNet(X.shape[1])
    l0 = net.train_batch(X[:4], T[:4], M[:4], 0.0)[0]
    hist = learned.train(net, X, T, M, epochs=10, batch=4, lr=1e-3)
    l1 = net.train_batch(X[:4], T[:4], M[:4], 0.0)[0]
    yield net, l0, l1, hist
    net.close()


def test_unet_training_reduces_loss(trained):
    _, l0, l1, hist = trained
    assert l1 < 0.8 * l0, (l0, l1, hist)


def test_warm_start_reaches_the_same_answer(trained):
    """A warm start only changes the starting point: the solve still stops on the
    same FP64 relative residual and returns the cold solve's answer to the
    tolerance.  (Measured on 64^3 fields the learned start saves no iterations;
    the iteration count may move by a few either way.)"""
    from vulkanfem_gb300 import api
    net = trained[0]
    ke = domains.hex8_stiffness()
    for seed in (50001, 50002):
        d = domains.training_field(24, seed=seed, levels=3)
        A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3)
        f = d.load_vector()
        u0 = learned.warm_start(net, d, A, f)
        assert np.all(u0.reshape(-1, 3)[d.fixed] == 0)
        uc, cold = A.solve(f, precision="mixed")
        uw, warm = A.solve(f, u0=u0, precision="mixed")
        A.close()
        assert warm["rel_residual"] < 1e-6 and cold["rel_residual"] < 1e-6
        assert _rel(uw, uc) < 1e-5
        assert warm["iterations"] <= 1.2 * cold["iterations"] + 5, (cold["iterations"], warm["iterations"])


def test_coarse_space_deflation_mechanism():
    """The deflation coarse space inside PCG (no counterpart in the reference):
    the preconditioner becomes z = M^-1 r + V G^-1 (V^T r - (KV)^T M^-1 r),
    G = V^T K V (checked against that formula to 1e-10 in FP64), and the solve
    starts from x0 + V G^-1 V^T r0.  With the exact solution as V the start is
    the answer (at most one iteration); with a smooth approximation of it (the
    solution restricted one level and interpolated back) or two columns the
    solve reaches the same answer at the same relative residual in no more
    iterations than without (deflation cannot raise the effective condition
    number), in FP64 and in mixed precision; removing the space restores the
    plain iteration count."""
    from vulkanfem_gb300 import api
    ke = domains.hex8_stiffness()
    d = domains.training_field(32, seed=50003, levels=3)
    A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3)
    f = d.load_vector()
    u_tight, _ = A.solve(f, rtol=1e-12)
    u_smooth = A.interpolate(0, A.restrict(0, u_tight))
    u0, st0 = A.solve(f)
    for prec in ("fp64", "mixed"):
        A.set_coarse_space(None)
        _, base = A.solve(f, precision=prec)
        A.set_coarse_space(u_tight)
        u1, st1 = A.solve(f, precision=prec)
        assert st1["iterations"] <= 1 and st1["rel_residual"] < 1e-6 and st1["fallback"] == 0
        assert _rel(u1, u0) < 1e-5
        A.set_coarse_space(u_smooth)
        u2, st2 = A.solve(f, precision=prec)
        assert st2["rel_residual"] < 1e-6 and st2["fallback"] == 0
        assert _rel(u2, u0) < 1e-5
        assert st2["iterations"] <= base["iterations"] + 1, (prec, base["iterations"], st2["iterations"])
        print("%s: %d iterations, %d with the smoothed solution as coarse space" % (prec, base["iterations"],
                                                                                 st2["iterations"]))
    # two columns (smoothed solution, load direction), also in flexible CG
    # (Polak-Ribiere beta, which tolerates the A-DEF2 operator's rounding
    # asymmetry), and removal
    A.set_coarse_space(np.stack([u_smooth, f], 1))
    u3, st3 = A.solve(f)
    assert st3["rel_residual"] < 1e-6 and _rel(u3, u0) < 1e-5
    assert st3["iterations"] <= st0["iterations"] + 1
    for prec in ("fp64", "mixed"):
        u5, st5 = A.solve(f, precision=prec, flexible=True)
        assert st5["rel_residual"] < 1e-6 and st5["fallback"] == 0 and _rel(u5, u0) < 1e-5
        assert st5["iterations"] <= st0["iterations"] + 2, (prec, st0["iterations"], st5["iterations"])
    A.set_coarse_space(None)
    _, st4 = A.solve(f)
    assert st4["iterations"] == st0["iterations"]
    # the deflated preconditioner against its formula (fixed entries of V are zeroed by the library)
    fx = np.asarray(d.fixed, np.int64)
    V = np.stack([u_smooth, f + 0.1 * u_tight], 1)
    V.reshape(-1, 3, 2)[fx] = 0.0
    r = np.random.default_rng(1).standard_normal(A.rows())
    r.reshape(-1, 3)[fx] = 0.0
    z_plain = api.MultigridPreconditioner(A).solve(r)
    KV = np.stack([A @ V[:, 0], A @ V[:, 1]], 1)
    z_ref = z_plain + V @ np.linalg.solve(V.T @ KV, V.T @ r - KV.T @ z_plain)
    A.set_coarse_space(V)
    z = api.MultigridPreconditioner(A).solve(r)
    assert _rel(z, z_ref) < 1e-10, _rel(z, z_ref)
    A.close()


def test_learned_coarse_correction_reaches_the_same_answer(trained):
    """The learned coarse correction (the trained network's predicted
    displacement as the deflation coarse space, learned.coarse_correction): same
    answer and residual as the solve without it, in at most 10% more iterations.
    Deflation cannot raise the effective condition number in exact arithmetic
    (FP64: unchanged counts), but in FP32 CG a rough coarse vector injects
    rounding along high-energy directions: a numpy restatement over the oracle
    with FP32 vectors takes 299 instead of 286 iterations on field 50002 with a
    random vector as the coarse space.  Prints the iteration counts."""
    from vulkanfem_gb300 import api
    net = trained[0]
    ke = domains.hex8_stiffness()
    for seed in (50001, 50002):
        d = domains.training_field(24, seed=seed, levels=3)
        A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, 3)
        f = d.load_vector()
        uc, cold = A.solve(f, precision="mixed")
        learned.coarse_correction(net, d, A, f)
        ul, lc = A.solve(f, precision="mixed")
        uf, lf = A.solve(f, precision="mixed", flexible=True)  # inside flexible PCG
        A.close()
        assert lc["rel_residual"] < 1e-6 and lc["fallback"] == 0
        assert lf["rel_residual"] < 1e-6 and lf["fallback"] == 0
        assert _rel(ul, uc) < 1e-5 and _rel(uf, uc) < 1e-5
        assert lc["iterations"] <= 1.10 * cold["iterations"] + 2, (cold["iterations"], lc["iterations"])
        assert lf["iterations"] <= 1.10 * cold["iterations"] + 2, (cold["iterations"], lf["iterations"])
        print("field %d: %d iterations plain, %d with the learned coarse correction (%d in flexible PCG)"
              % (seed, cold["iterations"], lc["iterations"], lf["iterations"]))
