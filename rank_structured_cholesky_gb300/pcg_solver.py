"""The reference's file-driven solver on the GPU (drop-in for src/pcg_solver.cpp).

    python -m rank_structured_cholesky_gb300.pcg_solver <prefix> [--eps 1e-6] [--maxit 10000]
                                                        [--precision fp64|mixed] [--out x.vector]

Reads ``<prefix>_system.bcsm.gz``, ``<prefix>_rhs.vector`` and, when present,
``<prefix>_meshPositions.dat`` (src/pcg_solver.cpp:67-96), factors with
maxDenseBlock 200 and maxDiagonalBlock 400, reordering the separators only
when positions were found (src/pcg_solver.cpp:100-111), runs PCG to a 1e-6
relative residual in at most 10000 iterations (src/pcg_solver.cpp:114-117)
and prints the solve time.  Unlike the reference (which aborts on an
indefinite factor), a failure exits with status 1 and a message; ``--out``
writes the solution in the .vector format.
"""
import argparse
import os
import sys
import time

import numpy as np

from . import fileio


def solve_files(prefix, eps=1e-6, maxit=10000, precision="fp64", out=None, device=0, log=sys.stdout):
    import rank_structured_cholesky_gb300 as rs

    n, colptr, rowind, vals = fileio.read_bcsm(prefix + "_system.bcsm.gz")
    rhs = fileio.read_vector(prefix + "_rhs.vector")
    if len(rhs) != n:
        raise fileio.FormatError("rhs has %d entries for a %d x %d system" % (len(rhs), n, n))
    pos_path = prefix + "_meshPositions.dat"
    xyz = None
    if os.path.exists(pos_path):
        xyz = fileio.read_positions(pos_path)
        if len(xyz) != n:
            raise fileio.FormatError("%d positions for %d unknowns" % (len(xyz), n))
    else:
        print("Warning: no system degree of freedom positions found - using default separator ordering",
              file=sys.stderr)
    t0 = time.perf_counter()
    ctx = rs.Context(max_dense_block=200, max_diag_block=400, reorder_separators=1 if xyz is not None else 0,
                     precision=rs.MIXED if precision == "mixed" else rs.FP64, device=device)
    G = rs.GpuFactor(ctx, colptr, rowind, vals, xyz)
    x, info = G.pcg(rhs, eps=eps, maxit=maxit)
    dt = time.perf_counter() - t0
    print(" total iterations: %d\n residual: %g" % (info["iterations"], info["true_residual"]), file=log)
    print("\nPCG solution took %f seconds" % dt, file=log)
    if out:
        fileio.write_vector(out, x)
    G.close()
    ctx.close()
    return x, info, dt


def main(argv=None):
    ap = argparse.ArgumentParser(prog="pcg_solver", description=__doc__.split("\n")[0])
    ap.add_argument("prefix", help="<prefix>_system.bcsm.gz, <prefix>_rhs.vector[, <prefix>_meshPositions.dat]")
    ap.add_argument("--eps", type=float, default=1e-6)
    ap.add_argument("--maxit", type=int, default=10000)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--out", default=None, help="write the solution (.vector)")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    try:
        solve_files(args.prefix, args.eps, args.maxit, args.precision, args.out, args.device)
    except (OSError, fileio.FormatError) as e:
        print("pcg_solver: %s" % e, file=sys.stderr)
        return 1
    except RuntimeError as e:   # RscholError and a missing library
        print("pcg_solver: %s" % e, file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
