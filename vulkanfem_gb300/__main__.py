"""Command-line driver with the reference's arguments and outputs
(src/main.cpp:28-127):

    python -m vulkanfem_gb300 <model>.dat [-n L] [--skip S] [--precision fp64|mixed]
                              [--rtol T] [--digits D]

Reads ``<model>.dat``, ``<model>_fixed.dat``, ``<model>_loading.dat`` and
``<model>_Ke0.dat`` (else ``data/Ke0.dat``) relative to the working directory,
assembles the matrix-free operator with an L-level hierarchy (S skipped levels),
solves on the GPU to rtol (1e-6 by default, as the reference's TOLERANCE,
include/FEMDefines.hpp), prints the compliance f.u and writes the solution to
``<model>_out.csv``.  ``--digits -1`` writes the reference's 6-decimal form;
the default 17 significant digits is loss-free.  Exit status 1 on a usage or
input error, 2 when the solver did not converge.
"""
import argparse
import sys
import time

import numpy as np

from . import api, inout


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m vulkanfem_gb300")
    ap.add_argument("model", help="<model>.dat")
    ap.add_argument("-n", dest="levels", type=int, default=3, help="multigrid levels (default 3)")
    ap.add_argument("--skip", type=int, default=0, help="levels skipped by the first coarsening")
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="mixed")
    ap.add_argument("--rtol", type=float, default=1e-6)
    ap.add_argument("--digits", type=int, default=17, help="significant digits in the output; -1: %%f")
    args = ap.parse_args(argv)

    name = inout.model_name_of(args.model)
    t0 = time.time()
    try:
        model, (sx, sy, sz) = inout.loadVoxel(name)
        print("Number of levels for Multigrid: %d%s" % (
            args.levels, " (+ %d jump(s))" % args.skip if args.skip else ""))
        ke = inout.getKe(name)
        fixed, loads = inout.getBoundaryConditions(name)
    except (OSError, ValueError) as e:
        print("error: %s" % e, file=sys.stderr)
        return 1
    A = api.assembleSystemMatrix(inout.occupancy(model), ke, fixed, args.levels, args.skip)
    n = A.rows()
    print("System statistics:")
    print("\tVoxel model resolution: %d x %d x %d" % (sx, sy, sz))
    print("\tElements: %d" % A.num_elements())
    print("\tDegrees of freedom: %d" % n)
    f = np.zeros(n, np.float64)
    api.applyBoundaryConditions(f, loads, fixed)
    print("Preparation took:    %g s" % (time.time() - t0))
    u, st = A.solve(f, allow_not_converged=True, rtol=args.rtol, precision=args.precision)
    print("Iterations: %d, relative residual %.3e, solve %.1f ms" % (
        st["iterations"], st["rel_residual"], st["solve_ms"]))
    print("Compliance:      %.17g" % float(f @ u))
    print("Saving the solution")
    inout.saveVector(u, name, digits=args.digits)
    A.close()
    return 0 if st["rel_residual"] <= args.rtol else 2


if __name__ == "__main__":
    sys.exit(main())
