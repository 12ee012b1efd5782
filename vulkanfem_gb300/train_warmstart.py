"""Train the warm-start U-Net on solutions of the library's own solver and
evaluate what it saves on unseen domains.

    python -m vulkanfem_gb300.train_warmstart --samples 2000 --epochs 10 \
        --out vulkanfem_gb300/checkpoints/unet_warmstart.npz --eval 8 --eval-n 128

Evaluation also measures the learned coarse correction (the predicted shape
as the deflation coarse space of PCG, learned.coarse_correction; it includes
the warm start's energy-optimal start) and, for scale, the same deflation with
a smooth approximation of the exact solution (restricted one level and
interpolated back: what a very good coarse-scale prediction would give).

Training domains: 64^3 seeded random fields at 30-60% fill, a random load patch
of total magnitude U[0.1, 1] in -z on the top face, z=0 fixed
(``domains.training_field``); targets are the mixed-precision MG-PCG solutions
(rtol 1e-6).  Evaluation: unseen seeds, cold start vs network warm start, both
solved to the same FP64 relative residual; prints one JSON line.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import api, domains, learned

NF = 9  # feature channels in use (see learned.py)
# Iteration caps: a field whose solve does not converge within them (floppy
# parts barely attached to the fixed face) is replaced by the next seed.
DATA_MAX_ITER = 5000
EVAL_MAX_ITER = 10000

def build_dataset(count, n, seed0, levels, log):
    ke = domains.hex8_stiffness()
    npad = learned.padded(n + 1)
    F = np.zeros((count, npad, npad, npad, NF), np.float16)
    T = np.zeros((count, npad, npad, npad, 3), np.float16)
    M = np.zeros((count, npad, npad, npad), np.uint8)
    t0 = time.time()
    its = []
    seed, skipped = seed0, 0
    for i in range(count):
        while True:
            # a field whose grounded part is tiny gets Eigen's small default cap
            # (2 x DOFs) and may not converge within it: take the next seed
            try:
                d = domains.training_field(n, seed=seed, levels=levels)
            except ValueError:  # nothing connected to the fixed face
                seed += 1
                skipped += 1
                continue
            seed += 1
            A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, levels)
            f = d.load_vector()
            u, st = A.solve(f, precision="mixed", max_iter=DATA_MAX_ITER, allow_not_converged=True)
            if st["status"] == 0:
                break
            A.close()
            skipped += 1
        its.append(st["iterations"])
        feats, mask, scale = learned.domain_features(d, npad, A, f)
        A.close()
        F[i] = feats[..., :NF]
        T[i] = learned.target_grid(u, mask, scale, npad)
        M[i] = learned.loss_mask(mask, d.fixed, npad) > 0
        if (i + 1) % 100 == 0:
            log("data %d/%d  %.0f s  mean iterations %.1f  (%d fields skipped: empty or not converged)"
                % (i + 1, count, time.time() - t0, np.mean(its), skipped))
    return F, T, M


def expand(F, T, M, idx):
    b = len(idx)
    x = np.zeros((b,) + F.shape[1:4] + (learned.NCH,), np.float32)
    x[..., :NF] = F[idx]
    return x, T[idx].astype(np.float32), M[idx].astype(np.float32)


def evaluate(params, count, n, seed0, levels, log):
    ke = domains.hex8_stiffness()
    net = learned.UNet(learned.padded(n + 1), params)
    rows = []
    seed = seed0
    while len(rows) < count:
        try:
            d = domains.training_field(n, seed=seed, levels=levels)
        except ValueError:  # nothing connected to the fixed face
            seed += 1
            continue
        seed += 1
        A = api.assembleSystemMatrix(d.voxels, ke, d.fixed, levels)
        f = d.load_vector()
        _, st = A.solve(f, precision="mixed", max_iter=EVAL_MAX_ITER,
                        allow_not_converged=True)  # graph capture outside the timing
        if st["status"] != 0:  # not converged within the default cap: next field
            A.close()
            continue
        i = len(rows)
        _, cold = A.solve(f, precision="mixed", max_iter=EVAL_MAX_ITER)
        t = time.perf_counter()
        u0 = learned.warm_start(net, d, A, f)
        t_pred = time.perf_counter() - t
        _, warm = A.solve(f, u0=u0, precision="mixed", max_iter=EVAL_MAX_ITER, allow_not_converged=True)
        # learned coarse correction: the predicted shape as the preconditioner's coarse space
        t = time.perf_counter()
        learned.coarse_correction(net, d, A, f)
        t_cc = time.perf_counter() - t
        A.solve(f, precision="mixed", max_iter=EVAL_MAX_ITER, allow_not_converged=True)  # graph capture
        _, cc = A.solve(f, precision="mixed", max_iter=EVAL_MAX_ITER, allow_not_converged=True)
        # for scale: a smooth approximation of the exact solution as the coarse space
        A.set_coarse_space(None)
        u_tight, _ = A.solve(f, precision="mixed", rtol=1e-10, max_iter=4 * EVAL_MAX_ITER, allow_not_converged=True)
        A.set_coarse_space(A.interpolate(0, A.restrict(0, u_tight)))
        A.solve(f, precision="mixed", max_iter=EVAL_MAX_ITER, allow_not_converged=True)  # graph capture
        _, smooth = A.solve(f, precision="mixed", max_iter=EVAL_MAX_ITER, allow_not_converged=True)
        A.set_coarse_space(None)
        feats = learned.domain_features(d, net.n, A, f)[0]
        net.forward(feats)
        t = time.perf_counter()
        net.forward(feats)
        t_fwd = time.perf_counter() - t
        rows.append({"forward_ms": 1e3 * t_fwd, "cold_it": cold["iterations"], "warm_it": warm["iterations"],
                     "cold_ms": cold["solve_ms"], "warm_ms": warm["solve_ms"], "predict_ms": 1e3 * t_pred,
                     "coarse_it": cc["iterations"], "coarse_ms": cc["solve_ms"], "coarse_setup_ms": 1e3 * t_cc,
                     "smooth_coarse_it": smooth["iterations"], "smooth_coarse_ms": smooth["solve_ms"],
                     "cold_relres": cold["rel_residual"], "warm_relres": warm["rel_residual"],
                     "coarse_relres": cc["rel_residual"], "smooth_coarse_relres": smooth["rel_residual"]})
        A.close()
        log("eval %d: cold %d it %.1f ms, warm %d it %.1f ms (+%.1f ms predict), learned coarse %d it %.1f ms, "
            "smoothed-solution coarse space %d it %.1f ms" % (
                i, cold["iterations"], cold["solve_ms"], warm["iterations"], warm["solve_ms"], 1e3 * t_pred,
                cc["iterations"], cc["solve_ms"], smooth["iterations"], smooth["solve_ms"]))
    net.close()
    return rows


def summarize(rows):
    """Means over the evaluated fields (iterations, times including the
    prediction or the coarse-space set-up, largest relative residuals)."""
    mean = lambda key: float(np.mean([r[key] for r in rows]))
    return {
        "eval_count": len(rows),
        "mean_cold_iterations": mean("cold_it"),
        "mean_warm_iterations": mean("warm_it"),
        "mean_coarse_iterations": mean("coarse_it"),
        "mean_smooth_coarse_iterations": mean("smooth_coarse_it"),
        "mean_cold_ms": mean("cold_ms"),
        "mean_warm_ms": mean("warm_ms"),
        "mean_predict_ms": mean("predict_ms"),
        "mean_coarse_ms": mean("coarse_ms"),
        "mean_coarse_setup_ms": mean("coarse_setup_ms"),
        "mean_smooth_coarse_ms": mean("smooth_coarse_ms"),
        "mean_forward_ms": mean("forward_ms"),
        "max_warm_relres": float(max(r["warm_relres"] for r in rows)),
        "max_coarse_relres": float(max(max(r["coarse_relres"], r["smooth_coarse_relres"]) for r in rows)),
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=2000)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=learned.CHECKPOINT)
    ap.add_argument("--eval", type=int, default=8)
    ap.add_argument("--eval-n", type=int, default=128)
    ap.add_argument("--eval-levels", type=int, default=5)
    ap.add_argument("--eval-only", default=None, metavar="CHECKPOINT",
                    help="evaluate a saved checkpoint instead of training")
    args = ap.parse_args(argv)
    log = lambda s: print(s, file=sys.stderr, flush=True)
    if args.eval_only:
        rows = evaluate(learned.load(args.eval_only), args.eval, args.eval_n, 1_000_000, args.eval_levels, log)
        print(json.dumps(dict(summarize(rows), checkpoint=args.eval_only, rows=rows)), flush=True)
        return
    t0 = time.time()
    F, T, M = build_dataset(args.samples, args.n, 0, args.levels, log)
    t_data = time.time() - t0
    net = learned.UNet(F.shape[1])
    rng = np.random.default_rng(0)
    hist = []
    t1 = time.time()
    for ep in range(args.epochs):
        lr = args.lr * (0.5 ** (ep // max(1, args.epochs // 3)))
        order = rng.permutation(args.samples)
        losses = []
        for s in range(0, args.samples - args.batch + 1, args.batch):
            x, t, m = expand(F, T, M, order[s:s + args.batch])
            losses.append(net.train_batch(x, t, m, lr)[0])
        hist.append(float(np.mean(losses)))
        log("epoch %d lr %.2e loss %.5f (%.0f s)" % (ep, lr, hist[-1], time.time() - t1))
    t_train = time.time() - t1
    params = net.get_params()
    net.close()
    if os.path.dirname(args.out):
        os.makedirs(os.path.dirname(args.out), exist_ok=True)
    learned.save(args.out, params, {"samples": args.samples, "epochs": args.epochs, "n": args.n,
                                     "loss_history": np.asarray(hist)})
    rows = evaluate(learned.load(args.out), args.eval, args.eval_n, 1_000_000, args.eval_levels, log)
    summary = dict({"samples": args.samples, "n": args.n, "epochs": args.epochs, "data_s": t_data,
                    "train_s": t_train, "loss_history": hist}, **summarize(rows))
    summary["rows"] = rows
    print(json.dumps(summary), flush=True)


if __name__ == "__main__":
    main()
