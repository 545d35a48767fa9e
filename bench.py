"""Benchmark: ms per pressure solve to 1e-8 relative residual at 256^3.

Workload (synthetic, seeded): unit cube, 256^3 cells plus a ghost layer
(box 258^3), Fictive ghost layer (homogeneous Neumann walls), 64
non-overlapping spheres with radii U[0.02, 0.06] masked Fictive; right-hand
side = -div of an i.i.d. N(0,1) staggered velocity, projected to zero mean.
One "step" is one solve from x = 0 to ||b - A x||_2 <= 1e-8 ||b||_2 (true
FP64 residual).

The timed solver is the learned two-level preconditioner under
mixed-precision flexible CG: FP32 vectors and stencils, FP64 dots, the FP32
recursion refreshed from the true FP64 residual every 50 iterations or after
a 10^3 drop of its residual norm; preconditioner
z = omega y + s p(A)(r - omega A y) with y = P U-Net(P^T r) on the coarse
grid of 4^3 blocks (BF16 tcgen05 convolutions) and p the degree-4 Chebyshev
polynomial over [lmax/6, lmax] as two FP32 two-level stencil passes.  The
network is trained on the GPU before the timed region, on a 64^3 system of
the same sphere family (another geometry).  After the timed region: the same
solver to 1e-10, plain FP64 CG (the metric's comparator), the
unpreconditioned mixed CG and the Chebyshev-preconditioned mixed CG without
the network on the same system, and the CPU baseline: one full FP64 CG solve
on all host cores (`cpu_baseline`, measured), whose solution the timed
result is compared with.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl xflow|reference]
    python bench.py --rows       # the other rows of the path at their sizes
    python bench.py --learned    # the U-Net as a full-resolution preconditioner
    python bench.py --size 64 --maxit 10 --steps 1 --warmup 1   # bounded run for launch lists

`--impl reference`: every step is one full FP64 CG solve of the same system
on the host cores (the CPU restatement of the reference's operator rows).

Multi-GPU: the path is one solve per GPU ("replicas only"); N ranks each solve
their own copy and `value` is the aggregate ms per solve (max-over-ranks time
divided by all ranks' solves).  `--gpus N` outside torchrun starts the N
ranks itself.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per pressure solve to 1e-8 rel resid @256³: learned+FP32 vs plain FP64 CG"
N_CELLS = 256
N_SPHERES = 64
SEED = 20261203
RTOL = 1e-8
CHEB_DEGREE = 8     # degree of the comparison mixed CG's polynomial preconditioner
CHEB_RATIO = 250    # its lambda_max / lambda_min
# the timed solver: learned two-level preconditioner under mixed-precision FCG
TL_BLOCK = 4     # coarse cells are 4^3 blocks of the fine interior
TL_DEGREE = 4    # smoothing polynomial degree (TL_DEGREE / 2 passes)
TL_RATIO = 6     # its lambda_max / lambda_min: the smoother damps the upper spectrum, the network the rest
TL_WINDOW = 1    # FCG window


def workload(n=N_CELLS):
    from xflow_gb300 import workloads as wl

    codes, nrm, nodes, sep, spheres = wl.spheres_grid(n, N_SPHERES, 0.02, 0.06, SEED)
    b = wl.divergence_rhs(codes, (sep, sep, sep), SEED + 1)
    return codes, sep, b


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
class Clocks:
    """Samples nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def workload_name(size):
    return (f"{size}^3 unit cube + ghost layer (box {size + 2}^3), {N_SPHERES} spheres r~U[0.02,0.06], "
            f"zero-mean -div(u) RHS, u~N(0,1), seed {SEED}")


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(dist, per_step_ms, world):
    """Aggregate ms per solve of N independent replicas: the slowest rank's
    total time over all ranks' solves (each rank ran len(per_step_ms))."""
    return max_over_ranks(dist, float(np.sum(per_step_ms))) / (len(per_step_ms) * world)


# ---------------------------------------------------------------------------
def cpu_fp64_solve(codes, sep, b, threads):
    """One plain FP64 CG solve of the system on the host cores, from x = 0 to
    the bench's relative tolerance: the oracle's restatement of the
    reference's operator rows (T3dLaplaceOperator, XOperator.cpp:938-1129) in
    a Hestenes-Stiefel CG, OpenMP over `threads` host threads.  Returns
    (solution, ms, iterations, relative residual)."""
    from oracle import oracle as O

    O.set_threads(threads)
    g = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
    t0 = time.perf_counter()
    x, st = O.cg_plain(O.LAPLACE, g, np.zeros(codes.shape), b, RTOL)
    ms = (time.perf_counter() - t0) * 1e3
    O.set_threads(1)
    return x, ms, st.iterations, st.resid


def cpu_one_thread_iteration_ms(codes, sep, b, iters=3):
    """Per-iteration cost of the same CPU CG on one host thread: a bounded
    sample (`iters` iterations after the set-up, which is timed apart)."""
    from oracle import oracle as O

    O.set_threads(1)
    g = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
    t0 = time.perf_counter()
    O.cg_plain(O.LAPLACE, g, np.zeros(codes.shape), b, 1e-30, maxit=1)
    t1 = time.perf_counter()
    O.cg_plain(O.LAPLACE, g, np.zeros(codes.shape), b, 1e-30, maxit=1 + iters)
    t2 = time.perf_counter()
    return ((t2 - t1) - (t1 - t0)) * 1e3 / iters


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_arm(args):
    """The reference's CPU path on this machine's host cores: every step is one
    full FP64 CG solve of the bench's system to the bench's tolerance (the
    oracle restatement of the reference's operator rows, all host threads);
    warm-up steps are the same solve, untimed."""
    world, rank, local, dist = dist_init()
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    codes, sep, b = workload(args.size)
    threads = host_threads()
    vals, its, res = [], [], []
    for k in range(args.warmup + args.steps):
        _, ms, it, rel = cpu_fp64_solve(codes, sep, b, threads)
        if k >= args.warmup:
            vals.append(ms)
            its.append(it)
            res.append(rel)
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": bench_config(args.size),
            "impl": "reference",
            "solver": f"plain FP64 CG on the host cores (oracle restatement of the reference's operator rows, "
                      f"OpenMP, {threads} threads), from x = 0 to the true relative residual {RTOL:g}",
            "iterations": its[-1], "rel_resid": res[-1], "ranks_with_work": 1,
            "cpu_baseline": {"value": v, "unit": "ms", "cores": threads, "kind": "port",
                             "sample": f"measured: {args.steps} full solves at {args.size}^3 "
                                       f"({its[-1]} iterations each), mean ms per solve; nproc {os.cpu_count()}"},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def bench_config(size):
    """The workload description both arms print (identical dicts)."""
    return {"workload": workload_name(size), "rtol": RTOL,
            "l2": "working set > 129 MB L2 (no flush needed)"}


def relaunch(args, argv):
    """`--gpus N` (N > 1) outside torchrun: start N ranks of this script with
    torch.distributed.run on 127.0.0.1 and return their exit status (rank 0
    prints the line)."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + list(argv)
    return subprocess.run(cmd).returncode


# ---------------------------------------------------------------------------
def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xflow", choices=["xflow", "reference"])
    ap.add_argument("--size", type=int, default=N_CELLS, help="interior cells per axis (a multiple of 16)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline solve")
    ap.add_argument("--maxit", type=int, default=0,
                    help="cap the timed solver's iterations, untrained network (a bounded command for launch lists "
                         "and ncu captures; no bench line)")
    ap.add_argument("--learned", action="store_true",
                    help="train the U-Net preconditioner and time it and its flexible CG at full size")
    ap.add_argument("--rows", action="store_true",
                    help="time the other rows of the path (time-step passes, IB, Thomas, packed SpMV, VTK)")
    ap.add_argument("--rows-no-cpu", action="store_true", help="with --rows: skip the CPU writer beside the VTK row")
    ap.add_argument("--timeloop", action="store_true",
                    help="time the GPU time loop: the lid-driven cavity (64^3, 10 steps), the channel with the "
                         "immersed icosphere (256x64x64, 100 steps) and the full loop (512x128x128 with the sphere "
                         "and a passive scalar, learned pressure solve against a plain FP64 run)")
    ap.add_argument("--loop-steps", type=int, default=20,
                    help="with --timeloop: steps of the 512x128x128 loop (each run)")
    ap.add_argument("--loop-only", action="store_true", help="with --timeloop: the 512x128x128 loop alone")
    ap.add_argument("--loop-solver", default="compare", choices=["compare", "learned", "mixed", "fp64"],
                    help="with --timeloop: the 512x128x128 loop's pressure solver; compare (default) runs the learned "
                         "solver and plain FP64 CG and reports the drift between them, the others one run (mixed and "
                         "fp64 without training: a bounded command for launch lists)")
    argv = sys.argv[1:] if argv is None else argv
    args = ap.parse_args(argv)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return relaunch(args, argv)
    if args.impl == "reference":
        return reference_arm(args)
    if args.rows:
        return rows(args)
    if args.timeloop:
        return timeloop(args)
    if args.learned:
        return learned(args)

    import xflow_gb300 as xf

    world, rank, local, dist = dist_init()
    codes, sep, b = workload(args.size)
    ctx = xf.Context(local)
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    bv = g.vec(b)
    x = g.vec(np.zeros(g.shape))
    ncell = int(np.prod(g.shape))

    from xflow_gb300 import capi
    from xflow_gb300 import workloads as wl

    # The timed solver: the learned two-level preconditioner under mixed-precision
    # FCG.  The U-Net is trained first (outside the timed region: once per
    # geometry family) on a 64^3 system of the sphere family, then runs on the
    # coarse grid of 4^3 blocks of this system.
    cc, s1, s2, s3 = wl.coarse_grid(codes, sep, TL_BLOCK)
    gc = xf.Grid(ctx, cc, s1, s2, s3, None)
    if args.maxit > 0:   # the bounded run launches the same kernels with untrained weights
        net, train = xf.UNet(gc, seed=1), None
    else:
        params, train = train_unet(ctx)
        net = xf.UNet(gc, params)

    def learned_solve(zero=True, rtol=RTOL, maxit=0):
        if zero:
            x.fill(0.0)
        return xf.solve_fcg(A, x, bv, unet=net, precond=capi.XF_PRECOND_UNET2, rtol=rtol, window=TL_WINDOW,
                            degree=TL_DEGREE, ratio=TL_RATIO, precision=xf.XF_PREC_MIXED, maxit=maxit)

    if args.maxit > 0:   # bounded command for launch lists and ncu captures
        for _ in range(args.warmup + args.steps):
            st = learned_solve(maxit=args.maxit)
        # the timed solve runs inside one CUDA graph with conditional nodes, whose
        # kernel nodes ncu does not profile; the same kernels once more outside
        # any graph: one coarse network application and one launch of each
        # stencil kernel of the solvers
        net.apply(gc.vec(np.zeros(gc.shape)), gc.vec(None))
        xf.profile_cg_kernels(A, reps=1)
        ctx.synchronize()
        print(json.dumps({"mode": "bounded timed-solver run", "workload": workload_name(args.size),
                          "maxit": args.maxit, "iterations": st.iterations, "launches_per_solve": int(st.reserved[0]),
                          "status": int(st.status)}))
        return 0

    for _ in range(args.warmup):
        learned_solve()
    clocks = Clocks(local)
    ctx.synchronize()
    barrier(dist)
    clocks.start()
    t0 = time.perf_counter()
    dev_ms, launches, sts = [], 0, []
    for _ in range(args.steps):
        st = learned_solve()
        assert st.status == 0, st.status
        dev_ms.append(st.ms)
        launches += int(st.reserved[0])
        sts.append(st)
    ctx.synchronize()
    wall = (time.perf_counter() - t0) * 1e3
    clk = clocks.stop()
    barrier(dist)
    value = replica_value(dist, dev_ms, world)
    xm = x.download()
    st_last = sts[-1]

    # End to end through the C ABI from host buffers: H2D of b and x0 from
    # pinned host memory, the learned solve, D2H of x into pinned memory, every
    # step.
    import torch

    hb = torch.empty(g.shape, dtype=torch.float64, pin_memory=True)
    hx = torch.empty(g.shape, dtype=torch.float64, pin_memory=True)
    hb.numpy()[...] = b
    e2e = []
    for k in range(args.warmup + args.steps):
        hx.numpy()[...] = 0.0
        ctx.synchronize()
        t1 = time.perf_counter()
        bv.upload(hb.numpy())
        x.upload(hx.numpy())
        s2 = learned_solve(zero=False)
        x.download(out=hx.numpy())
        t2 = time.perf_counter()
        if k >= args.warmup:
            e2e.append((t2 - t1) * 1e3)
        assert s2.status == 0
    e2e_ms = replica_value(dist, e2e, world)

    # The same solver to the config's outer-refinement tolerance, 1e-10 (once, after the timed region)
    st10 = learned_solve(rtol=1e-10)
    x10 = x.download()

    # Comparison solvers on the same system (after the timed region): plain
    # FP64 CG (the metric's comparator), unpreconditioned mixed CG, and the
    # Chebyshev-preconditioned mixed CG without the network.
    cheb = {"precond": capi.XF_PRECOND_CHEB, "cheb_degree": CHEB_DEGREE}

    def one(precision, **kw):
        x.fill(0.0)
        return xf.solve(A, x, bv, method=xf.XF_CG, precision=precision, rtol=RTOL, **kw)

    one(xf.XF_PREC_FP64)
    st64 = one(xf.XF_PREC_FP64)
    x64 = x.download()
    one(xf.XF_PREC_MIXED)
    st_plain = one(xf.XF_PREC_MIXED)
    one(xf.XF_PREC_MIXED, **cheb)
    cheb_sts = [one(xf.XF_PREC_MIXED, **cheb) for _ in range(3)]
    # Jacobi-preconditioned FP64 CG (flexible CG with the Laplace diagonal, FCG(1)), the other comparator
    jac = family_solvers(A, x, bv, None, ("jacobi_cg_fp64",))["jacobi_cg_fp64"]
    # the learned solver with the same parameters on a fresh 128^3 geometry of the family, beside
    # plain FP64 CG and Jacobi CG there
    family128 = family_check(ctx, params, 128, SEED + 11)

    # one coarse network application, CUDA events on the context stream
    stream = torch.cuda.ExternalStream(capi_stream(ctx))
    rc, zc = gc.vec(np.zeros(gc.shape)), gc.vec(None)
    net.apply(rc, zc)
    ctx.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(10):
        net.apply(rc, zc)
    ev1.record(stream)
    ev1.synchronize()
    unet_ms = ev0.elapsed_time(ev1) / 10
    unet_ex, _ = unet_flops(gc.shape)

    # Roofline: each stencil kernel timed alone (CUDA events on its launching
    # stream, the solver's own launch configuration), with its compulsory
    # bytes per box cell; the one with the largest share of the timed
    # iteration is the headline.
    kms = xf.profile_cg_kernels(A, reps=20)
    # compulsory bytes per box cell: pq_fused_f32 reads z (or r), p, kind and
    # writes p', q (17 B); poly2_f32 reads r, kind and writes z (9 B);
    # polyr_f32 reads r, q, e, p', kind and writes r', e, z (29 B); the others
    # as in their kernels' comments
    bpc = {"stencil_f32": 9, "xr_update_f32": 24, "p_update_f32": 12, "residual_f64": 29, "stencil_f64": 25,
           "pq_fused_f32": 17, "pq_march_f32": 17, "poly2_f32": 9, "polyr_f32": 29,
           "cheb_first_fused_f32": 29, "cheb_last_f32": 13, "cheb_middle_f32": 9,
           # the two-level passes: kind + y, A y; r, A y, kind + w; w, y, r, q_w, kind, mask + z, slot
           "tl_prolong_ay_f32": 9, "tl_first_f32": 13, "tl_last_f32": 26}
    # the learned two-level iteration's fine-grid passes: y = P zc with A y,
    # the smoother's first and last factor passes (TL_DEGREE / 2 - 2 middle
    # passes between them), and the FP32 stencil with a dot for A p
    per_iter = {"tl_prolong_ay_f32": 1, "tl_first_f32": 1, "tl_last_f32": 1, "cheb_middle_f32": TL_DEGREE // 2 - 2,
                "stencil_f32": 1}
    peak, peak_kind = peaks()
    kernels = {k: {"ms": kms[k], "bytes_per_cell": bpc[k], "GB_s": ncell * bpc[k] / (kms[k] * 1e-3) / 1e9,
                   "frac": ncell * bpc[k] / (kms[k] * 1e-3) / 1e9 / peak} for k in kms}
    share = {k: kms[k] * w for k, w in per_iter.items() if k in kms}
    dom = max(share, key=share.get)
    alg_bytes = ncell * bpc[dom]
    mv_ms = kms[dom]
    achieved = alg_bytes / (mv_ms * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(prof):
        traffic = json.load(open(prof)).get(dom)

    # FP64 error of the timed result: against the FP64 GPU CG solution and the
    # FP64 CPU solve, both as the max-norm of the zero-mean difference over the
    # solution's zero-mean range (the all-Neumann system fixes x up to a
    # constant); its true residual recomputed by the CPU oracle in FP64.
    act = np.isin(codes, (1, 4, 5, 6, 8))

    def rel_err(xa, xb):
        d = (xa - xa[act].mean()) - (xb - xb[act].mean())
        return float(np.abs(d[act]).max() / np.abs(xb[act] - xb[act].mean()).max())

    err_vs_fp64 = rel_err(xm, x64)
    oracle_resid = oracle_resid10 = None
    cpu = None
    cpu_extra = {}
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O

        threads = host_threads()
        O.set_threads(threads)
        og = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
        r = O.apply(O.LAPLACE, og, xm, b, -1)
        oracle_resid = float(np.linalg.norm(r[act]) / np.linalg.norm(b[act]))
        r = O.apply(O.LAPLACE, og, x10, b, -1)
        oracle_resid10 = float(np.linalg.norm(r[act]) / np.linalg.norm(b[act]))
        O.set_threads(1)
        xc, cms, cit, crel = cpu_fp64_solve(codes, sep, b, threads)
        one_ms = cpu_one_thread_iteration_ms(codes, sep, b)
        cpu = {"value": cms, "unit": "ms", "cores": threads, "kind": "port",
               "sample": f"measured: one full FP64 CG solve at {args.size}^3 from x = 0 to {RTOL:g} "
                         f"({cit} iterations, true relative residual {crel:.3g}; oracle restatement of the "
                         f"reference's operator rows, OpenMP, {threads} threads; nproc {os.cpu_count()})"}
        cpu_extra = {"cpu_fp64_one_thread_ms_per_iteration": one_ms,
                     "cpu_fp64_one_thread_note": "per-iteration cost on 1 host thread, 3 iterations (bounded sample)",
                     "err_vs_cpu_fp64": rel_err(xm, xc), "err_1e10_vs_cpu_fp64": rel_err(x10, xc)}

    line = {
        "metric": METRIC, "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 vectors and stencils, bf16 network (fp32 accumulate), f64 dots/scalars/residual refresh",
        "data": "synthetic",
        "config": bench_config(args.size),
        "solver": (f"mixed-precision flexible CG, FCG({TL_WINDOW}) (FP32 vectors and stencils, FP64 dots, "
                   "true FP64 residual refresh every 50 iterations or after a 10^3 drop of the residual norm)"),
        "preconditioner": (f"learned two-level: 3-level U-Net (16/32/64 channels, BF16 tcgen05 "
                           f"convolutions) on the coarse grid of {TL_BLOCK}^3 blocks as the coarse solver, "
                           f"degree-{TL_DEGREE} Chebyshev smoothing over [lmax/{TL_RATIO}, lmax] as "
                           f"{TL_DEGREE // 2} FP32 two-level stencil passes"),
        "training": (f"on the GPU before the timed region: {train['steps']} Adam steps on "
                     f"{train['pairs']} (residual, error) pairs from plain CG on a {train['grid']} system; "
                     f"the checkpoint kept is the one the timed solver needs fewest iterations with on a "
                     f"held-out {train['selection']['held_out']} system"),
        "parallelism": f"replicas x{world}",
        "iterations": st_last.iterations, "replacements": st_last.replacements, "rel_resid": st_last.rel_resid,
        "fallbacks": st_last.fallbacks,
        "oracle_rel_resid": oracle_resid, "err_vs_fp64_cg": err_vs_fp64,
        "refine_1e10": {"ms": st10.ms, "iterations": st10.iterations, "rel_resid": st10.rel_resid,
                        "oracle_rel_resid": oracle_resid10, "status": int(st10.status)},
        "fp64_cg_ms": st64.ms, "fp64_cg_iterations": st64.iterations, "fp64_cg_rel_resid": st64.rel_resid,
        "mixed_cg_unpreconditioned": {"ms": st_plain.ms, "iterations": st_plain.iterations,
                                      "rel_resid": st_plain.rel_resid},
        "mixed_cg_chebyshev": {"ms": float(np.mean([c.ms for c in cheb_sts])), "iterations": cheb_sts[-1].iterations,
                               "rel_resid": cheb_sts[-1].rel_resid,
                               "preconditioner": f"degree-{CHEB_DEGREE} Chebyshev, ratio {CHEB_RATIO}, no network"},
        "jacobi_cg_fp64": jac,
        "family_128": family128,
        "train": train,
        "coarse_unet": {"grid": f"{gc.shape[0] - 2}^3 (+ ghost layer)", "ms_per_apply": unet_ms,
                        "tflops_executed": unet_ex / (unet_ms * 1e-3) / 1e12},
        "speedup_vs_fp64_cg": st64.ms / value if value > 0 else None,
        "wall_ms_per_step": wall / args.steps,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 2 * ncell * 8, "d2h_bytes_per_step": ncell * 8},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": dom, "algorithmic_bytes_per_launch": alg_bytes,
                     "avg_launch_ms": mv_ms, "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
                     "kernels": kernels},
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
        line.update(cpu_extra)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def rows(args):
    """Time the other rows of the path at their configurations' sizes, each
    call end to end on the device (CUDA events on the context stream around
    `reps` calls; the calls that check the reference's throw conditions read a
    few bytes back inside the timed region):
      channel 256x64x64 (the immersed-body config): pressure RHS, velocity
        correction (u), control balance, momentum RHS (u), IB interpolate /
        forces / spread with an icosphere of 2562 markers, Thomas lines along
        x, the VTK volume (with the oracle's fprintf writer timed beside it);
      512x128x128 (the full time loop config): pressure RHS, velocity
        correction, control balance, momentum RHS;
      256^3 spheres Poisson system: packed-operator build and its SpMV.
    Prints one JSON line per row with ms per call and algorithmic GB/s."""
    import torch

    import xflow_gb300 as xf
    from xflow_gb300 import workloads as wl_step

    ctx = xf.Context(0)
    stream = torch.cuda.ExternalStream(capi_stream(ctx))
    peak, _ = peaks()

    def timed(fn, reps=20):
        for _ in range(3):
            fn()
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    out = []

    def report(row, config, ms, nbytes=None, **extra):
        d = {"row": row, "config": config, "ms": ms}
        if nbytes:
            d.update({"alg_bytes": nbytes, "GB_s": nbytes / (ms * 1e-3) / 1e9, "frac_of_measured_hbm":
                      nbytes / (ms * 1e-3) / 1e9 / peak})
        d.update(extra)
        out.append(d)
        print(json.dumps(d), flush=True)

    # --- time-step passes at the two channel sizes ---------------------------
    for (n1, n2, n3), name in (((257, 65, 65), "channel 256x64x64"), ((513, 129, 129), "channel 512x128x128")):
        cs = wl_step.staggered_channel(n1, n2, n3, seed=7)
        gp = xf.Grid(ctx, cs["pc"], *cs["hP"])
        gu, gv, gw = (xf.Grid(ctx, cs[c], *cs[h]) for c, h in (("uc", "hU"), ("vc", "hV"), ("wc", "hW")))
        u, v, w = gu.vec(cs["u"]), gv.vec(cs["v"]), gw.vec(cs["w"])
        rho, pb, rhs = gp.vec(cs["density"]), gp.vec(cs["p_border"]), gp.vec(None)
        p = gp.vec(cs["p"])
        ub, un = gu.vec(cs["u_border"]), gu.vec(None)
        npc, nuc = int(np.prod(gp.shape)), int(np.prod(gu.shape))
        ms = timed(lambda: xf.pressure_rhs(gp, u, v, w, cs["tau"], rhs, density=rho, border=pb))
        report("a20 pressure RHS (XProblem.cpp:5474-5512)", name, ms, npc * (1 + 8 + 8 + 8 + 8 + 8 + 8))
        ms = timed(lambda: xf.velocity_correct(1, u, p, cs["tau"], un, density=rho, border=ub))
        report("velocity correction u (XProblem.cpp:5598-5777)", name, ms, nuc * (1 + 8 + 8 + 8 + 8 + 8))
        ms = timed(lambda: xf.divergence_max(gp, u, v, w))
        report("control balance (XProblem.cpp:5782-5829)", name, ms, npc * (1 + 8 + 8 + 8))
        vis = gp.vec(np.full(gp.shape, 0.01))
        mom = tuple(gu.vec(None) for _ in range(5))
        ms = timed(lambda: xf.momentum_rhs(1, gu, u, v, w, vis=vis, border=ub, out=mom))
        # compulsory: code, u, v, w, vis, border in; uTr, vTr, wTr, visTr, rp out
        report("momentum RHS u: staggered interpolation + viscous terms (XProblem.cpp:5088-5419)", name, ms,
               nuc * (1 + 8 * 5 + 8 * 5))
        if n1 == 257:
            # Thomas lines along x of the u box: (n2 * n3) lines of n1-2 unknowns
            M, nl1, nl2, ls1, ls2, ms_ = xf.box_lines(gu.shape, 1)
            rng = np.random.Generator(np.random.PCG64(3))
            a = gu.vec(rng.uniform(-1, 0, gu.shape))
            c = gu.vec(rng.uniform(-1, 0, gu.shape))
            bb = gu.vec(2.5 + rng.uniform(0, 1, gu.shape))
            f = gu.vec(rng.standard_normal(gu.shape))
            uu = gu.vec(rng.standard_normal(gu.shape))
            ms = timed(lambda: xf.thomas_lines(ctx, M, uu, a, bb, c, f, nl1, nl2, ls1, ls2, ms_))
            report("a5 Thomas lines along x (XSLAE.cpp:416-445)", name + f", {nl1 * nl2} lines of {M + 1}", ms,
                   nuc * 8 * 6 + nuc * 8 * 2)
            # IB: icosphere r = 0.15 at (1, .5, .5), subdivision 4 (2562 vertices)
            from xflow_gb300 import workloads as wl

            verts = wl.icosphere(4) * 0.15 + np.array([1.0, 0.5, 0.5])
            nn = len(verts)
            nxt = np.roll(np.arange(nn), -1).astype(np.int32)
            prv = np.roll(np.arange(nn), 1).astype(np.int32)
            mk = xf.Markers(ctx, verts, verts, np.full(nn, xf.capi.XF_IB_TARGET, np.int32), nxt, prv,
                            np.zeros(nn), np.zeros((nn, 3)), np.ones(nn), np.array([1.0, 1.0, 1.0, 1e-4]))
            h0 = np.array([1 / 64] * 3)
            ms = timed(lambda: mk.interpolate(u, h0, 1))
            report("a17 IB interpolate (XProblem.cpp:8620-8791)", name + f", {nn} markers", ms)
            ms = timed(lambda: mk.compute_forces(1))
            report("a18 IB forces (XProblem.cpp:8436-8547)", name + f", {nn} markers", ms)
            ms = timed(lambda: mk.spread(un, h0, 1))
            report("a19 IB spread (XProblem.cpp:8550-8617)", name + f", {nn} markers", ms)
            # the same icosphere as a closed surface voxelised into the pressure box, its points spread
            # over the channel [0, 4] x [0, 1] x [0, 1]
            vs, fs = wl.icosphere_mesh(4)
            vs = vs * 0.15 + np.array([1.0, 0.5, 0.5])
            pts = [np.linspace(0.0, L, n_) for L, n_ in ((4.0, n1), (1.0, n2), (1.0, n3))]
            ms = timed(lambda: xf.voxelize_mesh(ctx, cs["pc"], *pts, vs, fs, 0), reps=5)
            report("voxelise a closed surface (planned boundary; host box in and out)",
                   name + f", {len(fs)} triangles", ms)
        if n1 == 257:
            # VTK volume of the step (node box one smaller than the pressure box)
            node_codes = np.ascontiguousarray(cs["pc"][:-1, :-1, :-1])
            xyz = [np.concatenate([[0.0], np.cumsum(h[:n - 2])]) for h, n in zip(cs["hP"], (n1, n2, n3))]
            gn = xf.Grid(ctx, node_codes, *(np.diff(a) for a in xyz))
            path = os.path.join(tempfile.gettempdir(), "xf_rows.vtk")
            nbytes = [0]

            def vtk():
                nbytes[0] = xf.write_vtk(path, gn, *xyz, u, v, w, p, rho, rho, vis)

            ms = timed(vtk, reps=3)
            extra = {"file_bytes": nbytes[0], "text_MB_s": nbytes[0] / (ms * 1e-3) / 1e6}
            if not args.rows_no_cpu:
                from oracle import oracle as O   # the reference's writer loops through the C library's fprintf

                t0 = time.perf_counter()
                O.vtk_write(path + ".cpu", node_codes, *xyz, cs["u"], cs["v"], cs["w"], cs["pc"], cs["p"], cs["pc"],
                            cs["density"], cs["pc"], cs["density"], np.full(gp.shape, 0.01))
                extra["cpu_baseline_ms"] = (time.perf_counter() - t0) * 1e3
                extra["cpu_baseline"] = "oracle restatement of the reference's VTK loops (fprintf), 1 thread"
                extra["identical_to_cpu"] = open(path, "rb").read() == open(path + ".cpu", "rb").read()
                os.remove(path + ".cpu")
            report("VTK legacy ASCII volume (XProblem.cpp:6132-6345)", name + f", {int(np.prod(gn.shape))} nodes",
                   ms, **extra)
            os.remove(path)
            gn.close()
        vis.close()
        for o in mom:
            o.close()
        for o in (u, v, w, rho, pb, rhs, p, ub, un):
            o.close()
        for gg in (gp, gu, gv, gw):
            gg.close()

    # --- packed operator at 256^3 ----------------------------------------------
    codes, sep, b = workload(args.size)
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    t0 = time.perf_counter()
    P = xf.PackedOperator(A)
    ctx.synchronize()
    build_ms = (time.perf_counter() - t0) * 1e3
    rows_, nnz, _ = P.size()
    x, y = g.vec(b), g.vec(None)
    ms = timed(lambda: P.apply(x, y))
    ncell = int(np.prod(g.shape))
    report("a9 packed operator SpMV (XOperator.cpp:1550-1571)", f"256^3 spheres, {rows_} rows, {nnz} nonzeros", ms,
           ncell * 1 + rows_ * (4 + 8 + 1) + nnz * (8 + 4) + rows_ * 8 * 2, build_ms=build_ms)
    return 0


# 72 (residual, error) pairs (8 right-hand sides x 9 CG iterates) of a 64^3 system of the sphere family,
# 3000 Adam steps with the learning rate halved every 1000 steps
def timeloop(args):
    """The time step of TVPProblem::SolveBySplitting on the GPU
    (xflow_gb300.timeloop), configs 1 and 2 all in FP64: momentum by the
    implicit transfer operator under Jacobi BiCGStab, pressure by plain FP64
    CG (both statements are all-Neumann: the cavity's walls, the channel's
    Defined inflow and convective, flux-balanced outflow), correction and
    control balance.  One JSON line per statement: per-step ms (wall,
    synchronised; the first step, which builds the solver graphs, apart),
    iterations and the control balance of the last step.  Then the full loop
    (config 5, full_loop)."""
    import xflow_gb300 as xf
    from xflow_gb300 import timeloop as tl

    ctx = xf.Context(0)
    cases = (("lid-driven cavity", tl.cavity(64, re=100.0, tau=1e-3), None, 10),
             ("channel with an immersed sphere",
              tl.channel(256, 64, 64, re=200.0, tau=2e-3, outflow="convective", walls="no_slip"),
              tl.sphere_markers((1.0, 0.5, 0.5), 0.15, 4), 100))
    for label, st, mk, steps in (() if args.loop_only else cases):
        loop = tl.SplittingLoop(ctx, st, markers=mk, pressure_solver="fp64")
        recs = [loop.step() for _ in range(steps)]
        line = {"mode": "time loop", "statement": st["name"], "steps": steps, "pressure": "FP64 CG",
                "markers": None if mk is None else int(len(mk["pos"])),
                "first_step_ms": recs[0]["ms"], "ms_per_step": float(np.mean([r["ms"] for r in recs[1:]])),
                "momentum_iterations_mean": float(np.mean([r["momentum_iterations"] for r in recs])),
                "pressure_iterations_mean": float(np.mean([r["pressure_iterations"] for r in recs])),
                "last": recs[-1]}
        print(json.dumps(line), flush=True)
        del loop
    full_loop(ctx, args.loop_steps, args.loop_solver)
    return 0


def full_loop(ctx, steps, solver_choice="compare"):
    """The full loop: the 512x128x128 channel on [0,4]x[0,1]^2 (8,388,608
    cells, h = 1/128), inflow u = 1, convective flux-balanced outflow,
    no-slip walls (free-slip ones let the momentum right-hand side's
    near-wall viscosity-gradient term, the reference's, accelerate the flow
    without bound: no wall friction balances it), Re = 200,
    dt = 2e-3, the icosphere of radius 0.15 at (1, 0.5, 0.5) as 2,562 target
    markers, and a passive scalar (Schmidt 1) entering as a Gaussian blob of
    sigma 0.05 on the inlet, transported by the upwind operator under
    BiCGStab.  Two runs from the same state: the pressure by the learned
    two-level mixed-precision FCG (the network trained as for the headline),
    and by plain FP64 CG, both warm-started from the previous step.  One JSON
    line: per-step ms of both (wall, synchronised, first step apart),
    iterations, and the drift of the velocity and the scalar between them."""
    import xflow_gb300 as xf
    from xflow_gb300 import timeloop as tl

    solvers = ("learned", "fp64") if solver_choice == "compare" else (solver_choice,)
    # the network trained as for the headline, on the sphere family: trained on the channel family instead (its
    # pressure box at 128x32x32, the coarse grid's own shape), it needed 300 iterations a step here against 61
    params, train = train_unet(ctx) if "learned" in solvers else (None, None)
    base = tl.channel(512, 128, 128, re=200.0, tau=2e-3, outflow="convective", walls="no_slip")
    mk = tl.sphere_markers((1.0, 0.5, 0.5), 0.15, 4)
    runs = {}
    for solver in solvers:
        st = tl.with_scalar(base, tl.gaussian_inlet(base["p"][0].shape, base["h"], sigma=0.05))
        loop = tl.SplittingLoop(ctx, st, markers=mk, pressure_solver=solver,
                                net_params=params if solver == "learned" else None)
        recs = []
        for _ in range(steps):
            try:
                recs.append(loop.step())
            except xf.XFError as e:   # report how far the run got, then fail
                print(json.dumps({"mode": "full loop", "pressure": solver, "failed_at_step": len(recs) + 1,
                                  "error": str(e), "last": recs[-1] if recs else None}), flush=True)
                raise
            r = recs[-1]
            print(f"[{solver}] step {r['step']}: {r['ms']:.1f} ms, pressure {r['pressure_iterations']} it, "
                  f"|u|max {max(r['velocity_max']):.4g}, div {r['divergence_max']:.3g}", file=sys.stderr, flush=True)
        runs[solver] = (recs, loop.fields())
        del loop

    def summary(recs):
        return {"first_step_ms": recs[0]["ms"], "ms_per_step": float(np.mean([r["ms"] for r in recs[1:]])),
                "pressure_iterations_mean": float(np.mean([r["pressure_iterations"] for r in recs])),
                "momentum_iterations_mean": float(np.mean([r["momentum_iterations"] for r in recs])),
                "scalar_iterations_mean": float(np.mean([r["scalar_iterations"] for r in recs])),
                "pressure_fallbacks": int(sum(r["pressure_fallbacks"] for r in recs)),
                "phase_ms_mean": {k: float(np.mean([r["phase_ms"][k] for r in recs[1:]])) for k in recs[0]["phase_ms"]},
                "last": recs[-1]}

    if solver_choice != "compare":
        print(json.dumps({"mode": "full loop", "statement": st["name"], "steps": steps, "pressure": solver_choice,
                          solver_choice: summary(runs[solver_choice][0])}), flush=True)
        return
    (lr, lf), (fr, ff) = runs["learned"], runs["fp64"]
    vel_scale = max(np.abs(f).max() for f in ff[:3])
    drift_u = max(np.abs(a - b).max() for a, b in zip(lf[:3], ff[:3])) / vel_scale
    act = base["p"][0] == 1
    pl, pf = lf[3][act], ff[3][act]
    drift_p = np.abs((pl - pl.mean()) - (pf - pf.mean())).max() / np.abs(pf - pf.mean()).max()
    cl, cf = lf[4], ff[4]
    drift_c = float(np.abs(cl - cf).max())

    line = {"mode": "full loop", "statement": st["name"] + ", Gaussian inlet sigma=0.05",
            "cells": int(act.sum()), "steps": steps, "markers": int(len(mk["pos"])),
            "learned": summary(lr), "fp64": summary(fr),
            "drift_vs_fp64": {"velocity_rel": float(drift_u), "pressure_rel": float(drift_p), "scalar_abs": drift_c,
                              "scalar_max": float(cf[base["p"][0] == 1].max())},
            "network": train}
    print(json.dumps(line), flush=True)


UNET_TRAIN = dict(n=64, spheres=16, seed=5, rhs_seeds=tuple(range(200, 208)),
                  iters=(2, 5, 10, 20, 40, 80, 120, 160, 240), steps=3000, lr=1e-3, halvings=3,
                  # checkpoint selection: the parameters after every `check_every` steps from
                  # `check_from` on are scored by the timed solver's iterations on a held-out
                  # system of the bench's family (another geometry and right-hand side)
                  check_from=1000, check_every=250, val_seed=7)


def family_solvers(A, x, bv, net, which):
    """Each solver of `which` once untimed, once timed, from x = 0 to RTOL on A x = b: "learned" (the
    timed solver, with `net` on the coarse grid), "fp64_cg", "jacobi_cg_fp64"."""
    import xflow_gb300 as xf
    from xflow_gb300 import capi

    calls = {
        "learned": lambda: xf.solve_fcg(A, x, bv, unet=net, precond=capi.XF_PRECOND_UNET2, rtol=RTOL,
                                        window=TL_WINDOW, degree=TL_DEGREE, ratio=TL_RATIO,
                                        precision=xf.XF_PREC_MIXED),
        "fp64_cg": lambda: xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_FP64, rtol=RTOL),
        "jacobi_cg_fp64": lambda: xf.solve_fcg(A, x, bv, precond=capi.XF_PRECOND_JACOBI, rtol=RTOL, window=1),
    }
    out = {}
    for k in which:
        for _ in range(2):
            x.fill(0.0)
            st = calls[k]()
        out[k] = {"ms": st.ms, "iterations": st.iterations, "rel_resid": st.rel_resid, "status": int(st.status)}
        if k == "learned":
            out[k]["fallbacks"] = st.fallbacks
    return out


def family_check(ctx, params, n, seed):
    """The trained network on another system of the sphere family (n^3, a fresh geometry and right-hand
    side): the learned solver beside plain FP64 CG and Jacobi CG."""
    import xflow_gb300 as xf
    from xflow_gb300 import workloads as wl

    codes, _, _, sep, _ = wl.spheres_grid(n, N_SPHERES, 0.02, 0.06, seed)
    b = wl.divergence_rhs(codes, (sep, sep, sep), seed + 1)
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    cc, c1, c2, c3 = wl.coarse_grid(codes, sep, TL_BLOCK)
    net = xf.UNet(xf.Grid(ctx, cc, c1, c2, c3, None), params)
    res = family_solvers(A, g.vec(np.zeros(g.shape)), g.vec(b), net, ("learned", "fp64_cg", "jacobi_cg_fp64"))
    res["system"] = f"{n}^3, {N_SPHERES} spheres, seed {seed}"
    return res


def unet_flops(shape):
    """Tensor-core FLOPs of one U-Net application on a box: executed (padded
    channels) and useful (1 input and 1 output channel in the end layers)."""
    import xflow_gb300 as xf

    cells, dims = [], list(shape)
    for _ in range(3):
        cells.append(int(np.prod(dims)))
        dims = [(d - 2) // 2 + 2 for d in dims]
    lev = {"enc0a": 0, "enc0b": 0, "enc1a": 1, "enc1b": 1, "mid_a": 2, "mid_b": 2, "dec1a": 1, "dec1b": 1,
           "dec0a": 0, "dec0b": 0, "out": 0}
    ex = us = 0
    for name, ci, co in xf.UNET_LAYERS:
        n = cells[lev[name]]
        ex += 2 * 27 * ci * co * n
        us += 2 * 27 * (1 if name == "enc0a" else ci) * (1 if name == "out" else co) * n
    return ex, us


def channel_codes(nx, ny, nz):
    """Point codes and separations (hx, hy, hz) of the channel's all-Neumann pressure box (the
    convective-outflow statement of the time loop: Actual interior, Fictive walls, inflow and outlet)."""
    from xflow_gb300 import timeloop as tl

    st = tl.channel(nx, ny, nz, outflow="convective", walls="no_slip")
    return st["p"][0], tuple(st["p"][3])


def train_unet(ctx, family="spheres"):
    """Trains the U-Net on the GPU (this library's forward/backward kernels,
    Adam, the A-norm loss) on (residual, error) pairs harvested from plain
    CG's own iterates on a small system of a family: "spheres" (the bench's,
    a 64^3 cube with 16 spheres, another seed) or "channel" (the time loop's
    channel pressure box at 128x32x32, divergence right-hand sides).  The
    training loss is a poor predictor of the two-level solver's iterations,
    so checkpoints are scored by the solver itself on a held-out larger
    system of the family (spheres: 256^3, another geometry and right-hand
    side, never the timed one; channel: 256x64x64) and the best is kept.
    Returns the parameters and a description."""
    import xflow_gb300 as xf
    from xflow_gb300 import capi
    from xflow_gb300 import workloads as wl

    T = UNET_TRAIN
    # the held-out system and its coarse grid
    if family == "channel":
        vcodes, vseps = channel_codes(256, 64, 64)
        held_out = "channel 256x64x64 pressure box, divergence right-hand side"
    else:
        vcodes, _, _, vsep, _ = wl.spheres_grid(N_CELLS, N_SPHERES, 0.02, 0.06, SEED + T["val_seed"])
        vseps = (vsep, vsep, vsep)
        held_out = f"{N_CELLS}^3, {N_SPHERES} spheres, seed {SEED + T['val_seed']}"
    vb = wl.divergence_rhs(vcodes, vseps, SEED + T["val_seed"] + 1)
    vg = xf.Grid(ctx, vcodes, *vseps, None)
    vA = xf.Operator(vg, xf.XF_OP_LAPLACE)
    vbv, vx = vg.vec(vb), vg.vec(np.zeros(vg.shape))
    vcc, v1, v2, v3 = wl.coarse_grid(vcodes, vseps[0], TL_BLOCK)
    vnet = xf.UNet(xf.Grid(ctx, vcc, v1, v2, v3, None), seed=1)

    def val_iters(params):
        vnet.set_params(params)
        vx.fill(0.0)
        st = xf.solve_fcg(vA, vx, vbv, unet=vnet, precond=capi.XF_PRECOND_UNET2, rtol=RTOL, window=TL_WINDOW,
                          degree=TL_DEGREE, ratio=TL_RATIO, precision=xf.XF_PREC_MIXED, maxit=2000)
        return st.iterations if st.status == capi.XF_OK and st.fallbacks == 0 else 10 ** 6

    if family == "channel":
        codes, seps = channel_codes(128, 32, 32)
        nrm = None
        grid_name = "channel 128x32x32 pressure box"
    else:
        codes, nrm, _, sep, _ = wl.spheres_grid(T["n"], T["spheres"], 0.02, 0.06, T["seed"])
        seps = (sep, sep, sep)
        grid_name = f"{T['n']}^3, {T['spheres']} spheres, seed {T['seed']}"
    g = xf.Grid(ctx, codes, *seps, nrm)
    A = xf.Operator(g)
    net = xf.UNet(g, seed=1)
    t0 = time.perf_counter()
    rs, es = [], []
    for s in T["rhs_seeds"]:
        b = wl.divergence_rhs(codes, seps, s)
        r_, e_ = xf.harvest_pairs(A, g.vec(b), iters=T["iters"])
        rs += r_
        es += e_
    first = float(np.mean([net.train_step(r, e, update=False, op=A) for r, e in zip(rs, es)]))
    t1 = time.perf_counter()
    checks, best = [], None
    for step in range(T["steps"]):
        q = step % len(rs)
        net.train_step(rs[q], es[q], lr=T["lr"] * 0.5 ** (T["halvings"] * step / T["steps"]), op=A)
        done = step + 1
        if done >= T["check_from"] and (done % T["check_every"] == 0 or done == T["steps"]):
            p = net.params()
            it = val_iters(p)
            checks.append([done, it])
            if best is None or it < best[1]:
                best = (done, it, p)
    ctx.synchronize()
    t2 = time.perf_counter()
    net.set_params(best[2])
    last = float(np.mean([net.train_step(r, e, update=False, op=A) for r, e in zip(rs, es)]))
    return best[2], {"grid": grid_name, "pairs": len(rs),
                     "steps": T["steps"], "lr": T["lr"], "lr_halvings": T["halvings"], "s": t2 - t1,
                     "harvest_s": t1 - t0, "anorm_loss_before": first, "anorm_loss_after": last,
                     "selection": {"held_out": held_out, "checkpoints": checks, "chosen_step": best[0],
                                   "held_out_iterations": best[1]}}


def learned(args):
    """The learned preconditioner at the bench's 256^3 system: a U-Net trained
    on the GPU (this library's forward/backward kernels, Adam, the A-norm
    loss) on (residual, error) pairs harvested from plain CG's own iterates on
    a 64^3 system of the same sphere family, then applied by flexible CG
    FCG(8) at full size.  Prints one JSON line: training time and loss, the
    U-Net application time and tensor FLOP rate, and the learned FCG solve
    (iterations, ms, true residual) beside plain FP64 CG on the same system.
    --learned-max-its caps the learned solve (0: to the tolerance)."""
    import torch

    import xflow_gb300 as xf
    from xflow_gb300 import workloads as wl

    ctx = xf.Context(0)
    stream = torch.cuda.ExternalStream(capi_stream(ctx))
    params, train = train_unet(ctx)
    codes2, sep2, b2 = workload(args.size)
    g2 = xf.Grid(ctx, codes2, sep2, sep2, sep2, None)
    A2 = xf.Operator(g2)
    net2 = xf.UNet(g2, params)
    bv = g2.vec(b2)
    z = g2.vec(None)
    for _ in range(2):
        net2.apply(bv, z)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record(stream)
    for _ in range(reps):
        net2.apply(bv, z)
    e1.record(stream)
    e1.synchronize()
    apply_ms = e0.elapsed_time(e1) / reps
    ex, us = unet_flops(g2.shape)
    line = {"mode": "learned preconditioner", "workload": f"{args.size}^3 spheres system (the bench's)",
            "train": train,
            "unet_apply_ms": apply_ms, "tensor_tflops_executed": ex / (apply_ms * 1e-3) / 1e12,
            "tensor_tflops_useful": us / (apply_ms * 1e-3) / 1e12, "tflop_per_apply": ex / 1e12}
    if not args.learned_applies_only:
        maxit = args.learned_max_its if args.learned_max_its > 0 else 100000
        x = g2.vec(np.zeros(g2.shape))
        st = xf.solve_fcg(A2, x, bv, unet=net2, rtol=RTOL, maxit=maxit)
        line["learned_fcg"] = {"iterations": st.iterations, "ms": st.ms, "rel_resid": st.rel_resid,
                               "status": int(st.status), "fallbacks": st.fallbacks, "window": 8}
        x = g2.vec(np.zeros(g2.shape))
        st = xf.solve(A2, x, bv, method=xf.XF_CG, rtol=RTOL)
        line["plain_fp64_cg"] = {"iterations": st.iterations, "ms": st.ms, "rel_resid": st.rel_resid}
        x = g2.vec(np.zeros(g2.shape))
        st = xf.solve(A2, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=RTOL)
        line["mixed_fp32_cg"] = {"iterations": st.iterations, "ms": st.ms, "rel_resid": st.rel_resid}
    print(json.dumps(line))
    return 0


def capi_stream(ctx):
    from xflow_gb300 import capi

    return capi.lib().xf_stream(ctx.h)


if __name__ == "__main__":
    sys.exit(main())
