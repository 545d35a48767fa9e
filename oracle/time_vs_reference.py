"""Test infrastructure only: anchors the oracle port's CPU times to the
reference's own.  Times, on the same sphere-masked system, the reference's
y |= A(x), (x, y) and z |= p1 x + p2 y (oracle/_ref/ref_driver, task timing:
the reference's classes compiled from its sources) against the port's
apply / dot / lincomb (oracle/liboracle.so) on one thread and on all threads,
and one TSLAE::SolveByConjugateGradients against the port's restatement of it
(cg_reference) from the same start.  Prints one JSON object.

    make -C oracle && make -C oracle ref REF=$XFLOW_REF
    python oracle/time_vs_reference.py [--n 128] [--reps 5] [--cg-n 48]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle.bagio import read_bag, write_bag  # noqa: E402
from xflow_gb300 import workloads as wl  # noqa: E402

DRIVER = os.path.join(HERE, "_ref", "ref_driver")


def system(n, seed=20261203):
    codes, nrm, nodes, sep, _ = wl.spheres_grid(n, 64, 0.02, 0.06, seed)
    b = wl.divergence_rhs(codes, (sep, sep, sep), seed + 1)
    return codes, nrm, nodes, sep, b


def reference(rec, threads):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_bag(fin, rec)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        p = subprocess.run([DRIVER, "timing", fin, fout], capture_output=True, text=True, timeout=3600, env=env)
        if p.returncode != 0:
            raise RuntimeError(p.stderr.strip()[-400:])
        return read_bag(fout)


def port(codes, nrm, sep, x, reps, threads):
    O.set_threads(threads)
    g = O.Grid(codes, nrm, sep, sep, sep)
    sm = g.smask
    y = O.apply(O.LAPLACE, g, x)
    out = {}
    t0 = time.perf_counter()
    for _ in range(reps):
        y = O.apply(O.LAPLACE, g, x)
    out["matvec_s"] = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        O.dot(x, y, sm)
    out["dot_s"] = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        O.lincomb(0.75, x, -1.25, y, sm, x)
    out["lincomb_s"] = (time.perf_counter() - t0) / reps
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128, help="interior cells per axis of the timed operator calls")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--cg-n", type=int, default=48, help="interior cells per axis of the timed CG solve")
    args = ap.parse_args()
    threads = os.cpu_count() or 1

    codes, nrm, nodes, sep, b = system(args.n)
    x = np.random.Generator(np.random.PCG64(7)).standard_normal(codes.shape)
    rec = {"dims": np.array(codes.shape, np.int32), "x_nodes": nodes, "y_nodes": nodes, "z_nodes": nodes,
           "codes": codes.astype(np.int32).ravel(), "normals": nrm.reshape(-1), "x": x.ravel(),
           "reps": np.array([args.reps], np.int32)}
    ref1 = reference(rec, 1)
    res = {"n": args.n, "cells": int(codes.size), "reps": args.reps, "host_threads": threads,
           "reference_1_thread": {k: float(ref1[k][0]) for k in ("matvec_s", "dot_s", "lincomb_s")},
           "port_1_thread": port(codes, nrm, sep, x, args.reps, 1),
           "port_all_threads": port(codes, nrm, sep, x, args.reps, threads)}
    res["port_speedup_1_thread"] = {k: res["reference_1_thread"][k] / res["port_1_thread"][k]
                                    for k in ("matvec_s", "dot_s", "lincomb_s")}

    # one full CG solve: the reference's own TSLAE against the port's restatement
    codes, nrm, nodes, sep, b = system(args.cg_n)
    x0 = np.zeros(codes.shape)
    rec = {"dims": np.array(codes.shape, np.int32), "x_nodes": nodes, "y_nodes": nodes, "z_nodes": nodes,
           "codes": codes.astype(np.int32).ravel(), "normals": nrm.reshape(-1), "x": x0.ravel(),
           "reps": np.array([1], np.int32), "cg": np.array([1], np.int32), "x0": x0.ravel(), "b": b.ravel()}
    refcg = reference(rec, 1)
    O.set_threads(1)
    g = O.Grid(codes, nrm, sep, sep, sep)
    t0 = time.perf_counter()
    _, st = O.cg_reference(O.LAPLACE, g, x0, b)
    tcg = time.perf_counter() - t0
    res["cg"] = {"n": args.cg_n, "reference_s": float(refcg["cg_s"][0]),
                 "reference_resid_l2": float(refcg["cg_resid_l2"][0]), "port_s": tcg,
                 "port_iterations": int(st.iterations), "port_1_thread_speedup": float(refcg["cg_s"][0]) / tcg}
    print(json.dumps(res))


if __name__ == "__main__":
    main()
