"""Benchmark of the voxel-elasticity MG-PCG solve (one JSON line on stdout).

A step is one complete solve of K u = f to rtol 1e-6 on the benchmark workload
(default: 256^3 box with 300 seeded spherical voids, per-voxel lognormal E,
5 multigrid levels).  Metric: MDOF/s = DOF x PCG iterations / solve time.

Arms:
  (default)          this library on the GPU.  `value`: device-resident solve
                     (right-hand side already in HBM; CUDA-event time of the
                     solve); `e2e`: the same solve through the C ABI with host
                     buffers (H2D of f and D2H of u inside the timed region).
  --impl reference   the CPU restatement of the reference's solve path
                     (additive MG-PCG, Eigen semantics) on all host cores,
                     timed on a bounded sample of PCG iterations.

N GPUs (torchrun): independent replicas, one per GPU (the solve has no
exchange step); value = all ranks' DOF x iterations / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (builder, description)
    "spheres256": (lambda: __import__("vulkanfem_gb300.domains", fromlist=["x"]).spheres(256, 300, 4, 16, seed=0,
                                                                                          levels=5,
                                                                                          lognormal_sigma=0.5),
                   "256^3 box minus 300 seeded spherical voids (r ~ U[4,16]), E ~ lognormal(0,0.5) per voxel, "
                   "nu=0.3, z=0 fixed, unit -z load on the top face, 5 MG levels"),
    "spheres224": (lambda: __import__("vulkanfem_gb300.domains", fromlist=["x"]).spheres(224, 200, 4, 14, seed=0,
                                                                                          levels=5,
                                                                                          lognormal_sigma=0.5),
                   "224^3 box minus 200 seeded spherical voids (r ~ U[4,14]), E ~ lognormal(0,0.5), 5 MG levels "
                   "(smaller profiling case: FP32 vectors still exceed L2)"),
    "porous128": (lambda: __import__("vulkanfem_gb300.domains", fromlist=["x"]).porous(128, 0.40, 6.0, seed=0,
                                                                                        levels=4),
                  "128^3 seeded Gaussian random field (sigma 6 voxels) at 40% fill, grounded component, "
                  "z=0 fixed, unit -z top load, 4 MG levels"),
    "porous384": (lambda: __import__("vulkanfem_gb300.domains", fromlist=["x"]).porous(384, 0.45, 6.0, seed=0,
                                                                                        levels=5,
                                                                                        lognormal_sigma=0.5),
                  "384^3 seeded Gaussian random field (sigma 6 voxels) at 45% fill, grounded component, "
                  "E ~ lognormal(0,0.5), z=0 fixed, unit -z top load, 5 MG levels (coarsest 24^3 elements, "
                  "45,006 free DOFs)"),
    "cantilever": (lambda: __import__("vulkanfem_gb300.domains", fromlist=["x"]).cantilever(32, 16, 16, 3),
                   "32x16x16 solid cantilever, x=0 fixed, unit -z load on x=32, 3 MG levels"),
}

SOLVERS = {
    "fp64": dict(precision="fp64", mg_mode="reference"),
    "mixed": dict(precision="mixed", mg_mode="reference"),
    "mixed_vcycle": dict(precision="mixed", mg_mode="vcycle", flexible=True),
    "fp64_vcycle": dict(precision="fp64", mg_mode="vcycle"),
}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """gloo process group for the barrier and the max/sum over ranks (replicas only)."""

    def __init__(self, ws):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def reduce(self, values, op):
        if not self.dist:
            return values
        import torch
        t = torch.tensor(values, dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return t.tolist()

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def replica_throughput(dist, seconds, dof_iterations):
    """Whole-job MDOF/s of independent replicas: all ranks' DOF x iterations over
    the slowest rank's time.  Returns (MDOF/s, max seconds)."""
    tmax, = dist.reduce([float(seconds)], "max")
    work, = dist.reduce([float(dof_iterations)], "sum")
    return work / tmax / 1e6, tmax


def algorithmic_bytes(kind, g0, g1, s):
    """Algorithmic bytes per launch on the finest level.  N = grid nodes, Ne = voxels
    (dense-grid model): matvec 6sN + Ne/8 + 4Ne + N/8 (x in, y out, occupancy bits,
    modulus, fixed bits); restrict 3sN_f + 3sN_c; prolong+smooth 3sN_c + 9sN_f (z_c,
    r, D^-1 in; z out) + N_f/8, 7.5sN_f in the mixed solve (D^-1 in FP16); x/r update 18sN (x, r, p, Ap in; x, r out); p
    update 9sN.  The mixed solve defers x += alpha p (its FP32 x correction) to
    the p update: r update 9sN, p update 15sN (z, p, x in; p, x out).  With the
    p update fused into the product (matvec_px): p_old, z, x in and p, x, Kp out
    plus the modulus and bits, 18sN + Ne/8 + 4Ne + N/8."""
    N, Ne = g0["nodes"], g0["voxels"]
    Nc = g1["nodes"]
    if kind == "matvec":
        return 6 * s * N + Ne / 8 + 4 * Ne + N / 8
    if kind == "matvec_px":
        return 18 * s * N + Ne / 8 + 4 * Ne + N / 8
    if kind == "update_restrict":  # r, Ap in and the new r out on the fine level; the coarse r out
        return 9 * s * N + 3 * s * Nc
    if kind == "coarse":  # the coarsest dense inverse: FP16 lower block triangle (mixed) or FP64 full
        n = g1["coarse_free"]
        return n * n if s == 4 else 8 * n * n
    if kind == "restrict":
        return 3 * s * N + 3 * s * Nc
    if kind == "prolong":  # the mixed up-leg reads D^-1 in FP16 (6 instead of 12 bytes per node)
        return 3 * s * Nc + (7.5 if s == 4 else 9) * s * N + N / 8
    if kind == "update_xr":
        return (9 if s == 4 else 18) * s * N
    if kind == "update_p":
        return (15 if s == 4 else 9) * s * N
    raise KeyError(kind)


def run_reference_arm(args, dom, ws, rank):
    """CPU restatement of the reference path, all host threads, bounded samples."""
    if rank != 0:
        return None
    import oracle
    from vulkanfem_gb300 import domains
    threads = os.cpu_count() or 1
    ke = domains.hex8_stiffness()
    t0 = time.perf_counter()
    o = oracle.Oracle(dom.voxels, ke, dom.fixed, dom.num_levels, 0, threads=threads, E=dom.E)
    setup_s = time.perf_counter() - t0
    f = o.load_vector(dom.load_nodes, dom.load_values)
    dof = o.num_dofs(0)
    cap = args.cpu_iters
    times, iters = [], []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        _, it, _ = o.pcg(f, tol=1e-6, iter_cap=cap)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            times.append(dt)
            iters.append(it)
    v = dof * sum(iters) / sum(times) / 1e6
    sample = ("%d PCG iterations (incl. the initial preconditioner application) per step on the full "
              "workload, %d threads" % (cap, threads))
    return {
        "metric": "MDOF/s (DOF x PCG iterations / solve time, rtol 1e-6 MG-PCG)",
        "value": v, "unit": "MDOF/s", "impl": "reference", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload][1], "dofs": dof,
                   "solver": "reference additive MG-PCG (CPU restatement)"},
        "cpu_baseline": {"value": v, "unit": "MDOF/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "MDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": setup_s,
    }


def cpu_baseline(args, dom, threads=None, iters=None):
    """The CPU restatement of the reference path on the host cores (all of them by
    default; threads=1 is the reference's serial Eigen product), timed over a
    bounded number of PCG iterations of the same workload."""
    import oracle
    from vulkanfem_gb300 import domains
    threads = threads or os.cpu_count() or 1
    iters = iters or args.cpu_iters
    o = oracle.Oracle(dom.voxels, domains.hex8_stiffness(), dom.fixed, dom.num_levels, 0, threads=threads, E=dom.E)
    f = o.load_vector(dom.load_nodes, dom.load_values)
    t = time.perf_counter()
    _, it, _ = o.pcg(f, tol=1e-6, iter_cap=iters)
    dt = time.perf_counter() - t
    return {"value": o.num_dofs(0) * it / dt / 1e6, "unit": "MDOF/s", "cores": threads, "kind": "port",
            "sample": "%d PCG iterations of the CPU restatement on the same workload, %d thread(s) (%.1f s)"
                      % (it, threads, dt)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spheres256", choices=sorted(WORKLOADS))
    ap.add_argument("--solver", default="mixed", choices=sorted(SOLVERS))
    ap.add_argument("--compare", default="fp64", help="second solver timed for the comparison ('' = none)")
    ap.add_argument("--compare-steps", type=int, default=2)
    ap.add_argument("--cpu-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-reps", type=int, default=20)
    ap.add_argument("--no-extra-configs", action="store_true",
                    help="skip the 128^3 porous FP32-vs-FP64 pair added to the line")
    ap.add_argument("--kernels-only", action="store_true",
                    help="profiling case for ncu: set-up, a 4-iteration solve and one launch of each kernel class; "
                         "prints the kernel-class times and no bench line")
    args = ap.parse_args()

    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dom = WORKLOADS[args.workload][0]()

    if args.impl == "reference":
        line = run_reference_arm(args, dom, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return

    from vulkanfem_gb300 import api, domains
    if args.kernels_only:
        A = api.assembleSystemMatrix(dom.voxels, domains.hex8_stiffness(), dom.fixed, dom.num_levels, 0, E=dom.E)
        A.set_loads(dom.load_nodes, dom.load_values)
        _, st = A.solve_device(allow_not_converged=True, max_iter=4, **SOLVERS[args.solver])
        print(json.dumps({"kernels_only": args.workload, "iterations": st["iterations"],
                          "kernel_ms": api.profile_kernels(A, 1)}), flush=True)
        return
    dist = Dist(ws)
    ke = domains.hex8_stiffness()
    t0 = time.perf_counter()
    A = api.assembleSystemMatrix(dom.voxels, ke, dom.fixed, dom.num_levels, 0, E=dom.E)
    setup_s = time.perf_counter() - t0
    A.set_loads(dom.load_nodes, dom.load_values)
    dof = A.rows()
    sopts = SOLVERS[args.solver]

    # ---- device-resident solves (value)
    for _ in range(args.warmup):
        A.solve_device(**sopts)
    dist.barrier()
    k0 = api.kernel_launch_count()
    stats = []
    with ClockSampler(local if ws == 1 else 0) as clk:
        w0 = time.perf_counter()
        for _ in range(args.steps):
            _, st = A.solve_device(**sopts)
            stats.append(st)
        wall = time.perf_counter() - w0
    launches = api.kernel_launch_count() - k0
    dist.barrier()
    dev_s = sum(st["solve_ms"] for st in stats) / 1e3
    iters = sum(st["iterations"] for st in stats)
    value, tmax = replica_throughput(dist, dev_s, dof * iters)

    # ---- end to end through the C ABI with host buffers (e2e)
    f = dom.load_vector()
    u = np.empty(dof)
    A.solve(f, out=u, **sopts)  # (the caller's output array is reused, as a C caller's would be)
    dist.barrier()
    e_it = 0
    e0 = time.perf_counter()
    for _ in range(args.steps):
        u, st = A.solve(f, out=u, **sopts)
        e_it += st["iterations"]
    e_s = time.perf_counter() - e0
    e2e, _ = replica_throughput(dist, e_s, dof * e_it)

    # ---- comparison solver (plain FP64 MG-PCG on the same GPU)
    comp = None
    if args.compare and args.compare not in ("none", args.solver):
        copts = SOLVERS[args.compare]
        A.solve_device(**copts)
        cst = [A.solve_device(**copts)[1] for _ in range(max(1, args.compare_steps))]
        cs = sum(s["solve_ms"] for s in cst) / 1e3 / len(cst)
        ci = sum(s["iterations"] for s in cst) / len(cst)
        # the answers themselves (untimed solves that read the solution back)
        u_main, _ = A.solve_device(want_solution=True, **sopts)
        u_comp, _ = A.solve_device(want_solution=True, **copts)
        comp = {"solver": args.compare, "time_to_rtol_s": cs, "iterations": ci,
                "mdof_s": dof * ci / cs / 1e6, "rel_residual": cst[-1]["rel_residual"],
                "speedup_time_to_rtol": cs / (dev_s / len(stats)),
                "rel_l2_vs_%s" % args.compare: float(np.linalg.norm(u_main - u_comp) / np.linalg.norm(u_comp))}

    # ---- roofline of the dominant kernel (CUDA events on the library stream)
    ms = api.profile_kernels(A, args.profile_reps)
    g0 = {"nodes": int(np.prod([n + 1 for n in dom.voxels.shape])), "voxels": int(dom.voxels.size)}
    sh1 = [-(-n // 2) + 1 for n in dom.voxels.shape]
    g1 = {"nodes": int(np.prod(sh1)), "coarse_free": int(A.coarse_free_dofs)}
    mixed = sopts["precision"] == "mixed"
    s = 4 if mixed else 8
    per_iter = {  # finest-level kernel class the solve runs once per iteration -> (ms, launches)
        "matvec": (ms["matvec_fp32" if mixed else "matvec_fp64"], 1),
        "update_xr": (ms["update_xr_mixed" if mixed else "update_xr_fp64"], 1),
        "prolong": (ms["prolong_fp32" if mixed else "prolong_fp64"], 1),
        "restrict": (ms["restrict_fp32" if mixed else "restrict_fp64"], 1),
        "update_p": (ms["update_p_fp32" if mixed else "update_p_fp64"], 1),
        "coarse": (ms["coarse_fp32" if mixed else "coarse_fp64"], 1),
    }
    if mixed and ms.get("update_restrict_mixed", 0) > 0:  # residual update fused with the first restriction
        per_iter["update_restrict"] = (ms["update_restrict_mixed"], 1)
        del per_iter["update_xr"], per_iter["restrict"]
    if mixed and ms.get("matvec_fp32_px", 0) > 0:  # the solve runs the fused product instead
        per_iter["matvec_px"] = (ms["matvec_fp32_px"], 1)
        del per_iter["matvec"], per_iter["update_p"]
    dom_k = max(per_iter, key=lambda k: per_iter[k][0])
    kms = per_iter[dom_k][0]
    abytes = algorithmic_bytes(dom_k, g0, g1, s)
    peak, peak_src = measured_peaks()
    achieved = abytes / (kms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tt = json.load(fh)
        key = "%s/%s_%s" % (args.workload, dom_k, "fp32" if mixed else "fp64")
        traffic = tt.get(key)
    per_kernel = {}
    for k, (kt, _) in per_iter.items():
        b = algorithmic_bytes(k, g0, g1, s)
        per_kernel["%s_%s" % (k, "fp32" if mixed else "fp64")] = {
            "ms_per_launch": kt, "algorithmic_bytes": b, "achieved_gbs": b / (kt * 1e-3) / 1e9 if kt > 0 else None,
            "frac": b / (kt * 1e-3) / 1e9 / peak if kt > 0 else None}
    roof = {"kernel": "%s_%s" % (dom_k, "fp32" if mixed else "fp64"), "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "algorithmic_bytes": abytes, "ms_per_launch": kms, "peak_source": peak_src,
            "per_kernel": per_kernel, "kernel_ms": ms}

    o_full = api.make_options(**sopts)
    solver_options = {k: getattr(o_full, k) for k, _ in api.Options._fields_ if k != "reserved"}
    line = {
        "metric": "MDOF/s (DOF x PCG iterations / solve time, rtol 1e-6 MG-PCG)",
        "value": value, "unit": "MDOF/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tmax / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64", "data": "synthetic",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload][1], "dofs": dof,
                   "solver": args.solver, "solver_options": solver_options,
                   "residual_replacement": "reliable updates (replace when |r| fell 20x since the last "
                                           "replacement, and on a convergence claim) instead of every 50 "
                                           "iterations: same iterations, fewer FP64-accurate products",
                   "parallelism": "replicas%d" % ws,
                   "l2": "inputs larger than L2 (vectors %.0f MB each)" % (g0["nodes"] * 3 * s / 1e6)},
        "e2e": {"value": e2e, "unit": "MDOF/s", "h2d_bytes_per_step": 8 * dof, "d2h_bytes_per_step": 8 * dof},
        "gpu_launches": launches,
        "time_to_rtol_s": dev_s / len(stats),
        "iterations": iters / len(stats),
        "rel_residual": stats[-1]["rel_residual"],
        "residual_replacements": stats[-1]["residual_replacements"],
        "wall_s": wall,
        "setup_s": setup_s,
        "compare": comp,
        "roofline": roof,
        "clocks": clk.summary(),
    }
    if rank == 0 and ws == 1 and not args.no_extra_configs:
        A.close()
        line["configs"] = {"porous128": precision_pair("porous128", args.steps)}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, dom)
        line["cpu_baseline_serial"] = cpu_baseline(args, dom, threads=1, iters=1)
    elif rank == 0:
        line["cpu_baseline"] = None
    if rank == 0:
        print(json.dumps(line), flush=True)
    A.close()
    dist.close()


def precision_pair(workload, steps):
    """The FP32-vs-FP64 configuration on a second workload: both solvers timed
    device-resident to rtol 1e-6 on the same problem, with the relative L2
    difference of their answers."""
    from vulkanfem_gb300 import api, domains
    dom = WORKLOADS[workload][0]()
    A = api.assembleSystemMatrix(dom.voxels, domains.hex8_stiffness(), dom.fixed, dom.num_levels, 0, E=dom.E)
    A.set_loads(dom.load_nodes, dom.load_values)
    dof = A.rows()
    out = {"description": WORKLOADS[workload][1], "dofs": dof}
    u = {}
    for name in ("mixed", "fp64"):
        A.solve_device(**SOLVERS[name])
        sts = [A.solve_device(**SOLVERS[name])[1] for _ in range(max(1, min(steps, 3)))]
        t = sum(st["solve_ms"] for st in sts) / len(sts) / 1e3
        it = sum(st["iterations"] for st in sts) / len(sts)
        u[name], _ = A.solve_device(want_solution=True, **SOLVERS[name])
        out[name] = {"time_to_rtol_s": t, "iterations": it, "mdof_s": dof * it / t / 1e6,
                     "rel_residual": sts[-1]["rel_residual"]}
    out["speedup_time_to_rtol"] = out["fp64"]["time_to_rtol_s"] / out["mixed"]["time_to_rtol_s"]
    out["rel_l2_mixed_vs_fp64"] = float(np.linalg.norm(u["mixed"] - u["fp64"]) / np.linalg.norm(u["fp64"]))
    A.close()
    return out


if __name__ == "__main__":
    main()
