"""Benchmark: ms per pressure solve to 1e-8 relative residual at 256^3.

Workload (synthetic, seeded): unit cube, 256^3 cells plus a ghost layer
(box 258^3), Fictive ghost layer (homogeneous Neumann walls), 64
non-overlapping spheres with radii U[0.02, 0.06] masked Fictive; right-hand
side = -div of an i.i.d. N(0,1) staggered velocity, projected to zero mean.
One "step" is one solve from x = 0 to ||b - A x||_2 <= 1e-8 ||b||_2 (true
FP64 residual).  The timed solver is the learned two-level preconditioner
under mixed-precision flexible CG: FP32 vectors and stencils, FP64 dots, the
FP32 recursion refreshed from the true FP64 residual every 50 iterations or
after a 10^3 drop; preconditioner z = omega y + s p(A)(r - omega A y) with
y = P U-Net(P^T r) on the coarse grid of 4^3 blocks (BF16 tcgen05
convolutions) and p the degree-6 Chebyshev polynomial over
[lmax/20, lmax] as three FP32 two-level stencil passes.  The network is
trained on the GPU before the timed region, on a 64^3 system of the same
sphere family (another geometry).  Plain FP64 CG, the unpreconditioned mixed
CG and the Chebyshev-preconditioned mixed CG without the network (degree
XF_BENCH_CHEB_DEGREE, default 8) are timed beside it on the same system.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl xflow|reference]

Multi-GPU: the path is one solve per GPU ("replicas only"); N ranks each solve
their own copy and `value` is the aggregate ms per solve (max-over-ranks time
divided by all ranks' solves).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per pressure solve to 1e-8 rel resid @256³: learned+FP32 vs plain FP64 CG"
N_CELLS = 256
N_SPHERES = 64
SEED = 20261203
RTOL = 1e-8
CHEB_DEGREE = int(os.environ.get("XF_BENCH_CHEB_DEGREE", "8"))   # degree of the polynomial preconditioner
CHEB_RATIO = {2: 30, 4: 120}.get(CHEB_DEGREE, 250)                # its default lambda_max / lambda_min
CALIB = os.path.join(ROOT, "profiles", "bench_calibration.json")
# the timed solver: learned two-level preconditioner under mixed-precision FCG
TL_BLOCK = 4     # coarse cells are 4^3 blocks of the fine interior
TL_DEGREE = int(os.environ.get("XF_BENCH_TL_DEGREE", "6"))  # smoothing polynomial degree (TL_DEGREE / 2 passes)
TL_RATIO = int(os.environ.get("XF_BENCH_TL_RATIO", "20"))   # its lambda_max / lambda_min
TL_WINDOW = int(os.environ.get("XF_BENCH_TL_WINDOW", "1"))  # FCG window


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
def cpu_baseline(codes, sep, b, fp64_iters, sample_iters=10):
    """The oracle port's plain FP64 CG on this machine's host cores: a bounded
    sample of `sample_iters` iterations at full size, extrapolated to the
    iteration count plain FP64 CG needs on this system."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    g = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
    t0 = time.perf_counter()
    _, st = O.cg_plain(O.LAPLACE, g, np.zeros(codes.shape), b, 1e-30, maxit=sample_iters)
    dt = time.perf_counter() - t0
    O.set_threads(1)
    per_it = dt * 1e3 / max(1, st.iterations)
    return {"value": per_it * fp64_iters, "unit": "ms", "cores": threads, "kind": "port",
            "sample": f"{st.iterations} FP64 CG iterations at 256^3 (incl. setup of the first residual), "
                      f"{per_it:.1f} ms/iteration x {fp64_iters} iterations (extrapolated)"}


def reference_arm(args):
    world, rank, local, dist = dist_init()
    if rank != 0:
        return 0
    codes, sep, b = workload()
    iters = None
    if os.path.exists(CALIB):
        iters = json.load(open(CALIB)).get("fp64_cg_iterations")
    if iters is None:
        iters = 1000
        note = " (iteration count not calibrated: 1000 assumed)"
    else:
        note = ""
    vals = []
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(codes, sep, b, iters, sample_iters=4)
        if k >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    cb["sample"] += note
    line = {"metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(N_CELLS),
                       "solver": "plain FP64 CG, oracle CPU port, all host cores"},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xflow", choices=["xflow", "reference"])
    ap.add_argument("--size", type=int, default=N_CELLS)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--learned", action="store_true",
                    help="train the U-Net preconditioner and time it and its flexible CG at full size")
    ap.add_argument("--learned-applies-only", action="store_true", help="with --learned: no solves")
    ap.add_argument("--learned-max-its", type=int, default=0, help="with --learned: cap of the learned solve")
    ap.add_argument("--two-level", action="store_true",
                    help="time the learned two-level preconditioner (U-Net coarse solver + Chebyshev smoothing)")
    ap.add_argument("--two-level-profile", action="store_true",
                    help="with --two-level: one 10-iteration solve with untrained weights (for a launch list)")
    ap.add_argument("--two-level-sweep",
                    default="8:60:2:32,8:60:2:64,8:60:1:32,8:250:2:32,8:30:2:32,4:60:2:32,4:30:2:32,12:60:2:32",
                    help="with --two-level: smoothing degree:ratio:FCG window:vector bits (32 mixed, 64) entries")
    ap.add_argument("--rows", action="store_true",
                    help="time the other rows of the path (time-step passes, IB, Thomas, packed SpMV, VTK)")
    ap.add_argument("--rows-no-cpu", action="store_true", help="with --rows: skip the CPU writer beside the VTK row")
    ap.add_argument("--unet-applies", type=int, default=0,
                    help="apply a random-initialised U-Net this many times to the bench's right-hand side (a bounded "
                         "command for per-layer launch lists)")
    ap.add_argument("--probes", action="store_true",
                    help="tcgen05.mma issue rate versus N and the FP64 / FP32 FMA rates (one JSON line each)")
    ap.add_argument("--degrees", default="",
                    help="degree:ratio pairs (e.g. 4:120,8:250): one JSON line per preconditioner, best of 3 solves")
    ap.add_argument("--kernels-only", action="store_true",
                    help="a few launches of each hot kernel on the full grid (for ncu captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.kernels_only:
        return kernels_only(args)
    if args.degrees:
        return degrees(args)
    if args.unet_applies > 0:
        return unet_applies(args)
    if args.probes:
        return probes(args)
    if args.two_level:
        return two_level(args)
    if args.rows:
        return rows(args)
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

    cheb = {"precond": capi.XF_PRECOND_CHEB, "cheb_degree": CHEB_DEGREE}   # the comparison mixed CG's polynomial

    def one(precision, **kw):
        x.fill(0.0)
        return xf.solve(A, x, bv, method=xf.XF_CG, precision=precision, rtol=RTOL, **kw)

    # FP64 plain CG: the comparison point of the metric
    one(xf.XF_PREC_FP64)
    st64 = one(xf.XF_PREC_FP64)
    x64 = x.download()
    fp64_ms = st64.ms
    fp64_iters = st64.iterations

    # unpreconditioned mixed CG, beside it
    one(xf.XF_PREC_MIXED)
    st_plain = one(xf.XF_PREC_MIXED)

    # the Chebyshev-preconditioned mixed CG (the same smoother, no network), beside it
    one(xf.XF_PREC_MIXED, **cheb)
    cheb_sts = [one(xf.XF_PREC_MIXED, **cheb) for _ in range(args.steps)]

    # The timed solver: the learned two-level preconditioner under mixed-precision
    # FCG.  The U-Net is trained first (outside the timed region: once per
    # geometry family) on a 64^3 system of the sphere family, then runs on the
    # coarse grid of 4^3 blocks of this system.
    from xflow_gb300 import workloads as wl

    params, train = train_unet(ctx)
    cc, s1, s2, s3 = wl.coarse_grid(codes, sep, TL_BLOCK)
    gc = xf.Grid(ctx, cc, s1, s2, s3, None)
    net = xf.UNet(gc, params)

    def learned_solve(zero=True):
        if zero:
            x.fill(0.0)
        return xf.solve_fcg(A, x, bv, unet=net, precond=capi.XF_PRECOND_UNET2, rtol=RTOL, window=TL_WINDOW,
                            degree=TL_DEGREE, ratio=TL_RATIO, precision=xf.XF_PREC_MIXED)

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

    # Roofline: each kernel of the mixed CG iteration timed alone (CUDA events
    # on its launching stream, the solver's own launch configuration), with
    # its compulsory bytes per box cell; the dominant one by share of the
    # iteration is the headline.
    kms = xf.profile_cg_kernels(A, reps=20)
    # compulsory bytes per box cell: pq_fused_f32 reads z (or r), p, kind and
    # writes p', q (17 B); poly2_f32 reads r, kind and writes z (9 B);
    # polyr_f32 reads r, q, e, p', kind and writes r', e, z (29 B); the others
    # as in their kernels' comments
    bpc = {"stencil_f32": 9, "xr_update_f32": 24, "p_update_f32": 12, "residual_f64": 29, "stencil_f64": 25,
           "pq_fused_f32": 17, "pq_march_f32": 17, "poly2_f32": 9, "polyr_f32": 29,
           "cheb_first_fused_f32": 29, "cheb_last_f32": 13, "cheb_middle_f32": 9}
    if "cheb_middle_f32" in kms and "stencil_f32" in kms:
        # the learned two-level iteration: the smoother's TL_DEGREE / 2 factor
        # passes (each the middle-pass kernel, w' = p_k(A) w), and two FP32
        # stencils with a dot (A y of the coarse correction, A p)
        per_iter = {"cheb_middle_f32": TL_DEGREE // 2, "stencil_f32": 2.0}
    elif "cheb_first_fused_f32" in kms and "pq_fused_f32" in kms and CHEB_DEGREE >= 4:
        # per chunk of 50: the passes of the m = degree / 2 factors once (the
        # first without the update: timed as a middle pass, the same work),
        # then K1, the first pass with the update, m - 2 middle passes and
        # the last pass 49 times, and K1 + the update + the FP64 replacement
        # once
        m = CHEB_DEGREE // 2
        per_iter = {"cheb_first_fused_f32": 49 / 50, "cheb_middle_f32": (m - 2) + 1 / 50,
                    "cheb_last_f32": 1.0, "pq_fused_f32": 1.0, "xr_update_f32": 1 / 50, "residual_f64": 1 / 50}
    elif "polyr_f32" in kms and "pq_fused_f32" in kms:
        # the degree-2 polynomial path, per chunk of 50: K0 once, K1 and the fused
        # update + K0 49 times, K1 + the update + the FP64 replacement once
        per_iter = {"polyr_f32": 49 / 50, "pq_fused_f32": 1.0, "poly2_f32": 1 / 50, "xr_update_f32": 1 / 50,
                    "residual_f64": 1 / 50}
    elif "pq_fused_f32" in kms:
        per_iter = {"pq_fused_f32": 1.0, "xr_update_f32": 1.0, "residual_f64": 1.0 / 50}
    else:
        per_iter = {"stencil_f32": 1.0, "xr_update_f32": 1.0, "p_update_f32": 1.0, "residual_f64": 1.0 / 50}
    peak, peak_kind = peaks()
    kernels = {k: {"ms": kms[k], "bytes_per_cell": bpc[k], "GB_s": ncell * bpc[k] / (kms[k] * 1e-3) / 1e9,
                   "frac": ncell * bpc[k] / (kms[k] * 1e-3) / 1e9 / peak} for k in kms}
    share = {k: kms[k] * w for k, w in per_iter.items()}
    dom = max(share, key=share.get)
    alg_bytes = ncell * bpc[dom]
    mv_ms = kms[dom]
    achieved = alg_bytes / (mv_ms * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(prof):
        traffic = json.load(open(prof)).get(dom)

    # FP64 error of the timed result: against the FP64 CG solution, and its
    # true residual recomputed by the CPU oracle in FP64.
    sm = codes != 0
    act = np.isin(codes, (1, 4, 5, 6, 8))
    d = (xm - xm[act].mean()) - (x64 - x64[act].mean())
    err_vs_fp64 = float(np.abs(d[act]).max() / np.abs(x64[act] - x64[act].mean()).max())
    oracle_resid = None
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O

        O.set_threads(os.cpu_count() or 1)
        og = O.Grid(codes, np.zeros(codes.shape + (3,)), sep, sep, sep)
        r = O.apply(O.LAPLACE, og, xm, b, -1)
        oracle_resid = float(np.linalg.norm(r[act]) / np.linalg.norm(b[act]))
        O.set_threads(1)
        cpu = cpu_baseline(codes, sep, b, fp64_iters)
        os.makedirs(os.path.dirname(CALIB), exist_ok=True)
        try:
            json.dump({"workload": "256^3 spheres, seed %d" % SEED, "fp64_cg_iterations": fp64_iters,
                       "timed_solver_iterations": st_last.iterations}, open(CALIB, "w"))
        except OSError:
            pass

    line = {
        "metric": METRIC, "value": value, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 vectors and stencils, bf16 network (fp32 accumulate), f64 dots/scalars/residual refresh",
        "data": "synthetic",
        "config": {"workload": workload_name(args.size),
                   "solver": (f"mixed-precision flexible CG, FCG({TL_WINDOW}) (FP32 vectors and stencils, FP64 dots, "
                              "true FP64 residual refresh every 50 iterations or after a 10^3 drop)"),
                   "preconditioner": (f"learned two-level: 3-level U-Net (16/32/64 channels, BF16 tcgen05 "
                                      f"convolutions) on the coarse grid of {TL_BLOCK}^3 blocks as the coarse solver, "
                                      f"degree-{TL_DEGREE} Chebyshev smoothing over [lmax/{TL_RATIO}, lmax] as "
                                      f"{TL_DEGREE // 2} FP32 two-level stencil passes"),
                   "training": (f"on the GPU before the timed region: {train['steps']} Adam steps on "
                                f"{train['pairs']} (residual, error) pairs from plain CG on a {train['grid']} system"),
                   "rtol": RTOL,
                   "l2": "working set ~0.6 GB > 129 MB L2 (no flush needed)",
                   "parallelism": f"replicas x{world}"},
        "iterations": st_last.iterations, "replacements": st_last.replacements, "rel_resid": st_last.rel_resid,
        "oracle_rel_resid": oracle_resid, "err_vs_fp64_cg": err_vs_fp64,
        "fp64_cg_ms": fp64_ms, "fp64_cg_iterations": fp64_iters, "fp64_cg_rel_resid": st64.rel_resid,
        "mixed_cg_unpreconditioned": {"ms": st_plain.ms, "iterations": st_plain.iterations,
                                      "rel_resid": st_plain.rel_resid},
        "mixed_cg_chebyshev": {"ms": float(np.mean([c.ms for c in cheb_sts])), "iterations": cheb_sts[-1].iterations,
                               "rel_resid": cheb_sts[-1].rel_resid,
                               "preconditioner": f"degree-{CHEB_DEGREE} Chebyshev, ratio {CHEB_RATIO}, no network"},
        "train": train,
        "coarse_unet": {"grid": f"{gc.shape[0] - 2}^3 (+ ghost layer)", "ms_per_apply": unet_ms,
                        "tflops_executed": unet_ex / (unet_ms * 1e-3) / 1e12},
        "speedup_vs_fp64_cg": fp64_ms / value if value > 0 else None,
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
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def probes(args):
    """The measurements behind two design decisions: cycles per tcgen05.mma
    versus N (1, 2, 4 CTAs per SM; both operand layouts) and the FP64 / FP32
    FMA rates."""
    import torch

    import xflow_gb300 as xf

    ctx = xf.Context(0)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for layout in (0, 1):
        for n in (16, 32, 64, 128, 256):
            for cps in (1, 2, 4):
                if (32 if n <= 32 else n) * cps > 512:
                    continue
                cyc = xf.probe_mma_rate(ctx, n, cps, layout)
                flop_clk = 2.0 * 128 * n * 16 / cyc
                print(json.dumps({"probe": "tcgen05.mma kind::f16 M=128 K=16", "layout": layout, "n": n,
                                  "ctas_per_sm": cps, "cycles_per_mma": cyc, "flop_per_clock_per_sm": flop_clk,
                                  "tflops_at_2070mhz": flop_clk * 2.07e9 * sms / 1e12}), flush=True)
    for fp64 in (1, 0):
        print(json.dumps({"probe": "FMA chains", "dtype": "f64" if fp64 else "f32",
                          "tflops": xf.probe_fma_rate(ctx, fp64)}), flush=True)
    return 0


def unet_applies(args):
    """K applications of a random-initialised U-Net (the learned
    preconditioner's network; weights do not change its time) to the bench's
    right-hand side: device ms per application."""
    import torch

    import xflow_gb300 as xf

    codes, sep, b = workload(args.size)
    ctx = xf.Context(0)
    stream = torch.cuda.ExternalStream(capi_stream(ctx))
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    net = xf.UNet(g, seed=1)
    bv, z = g.vec(b), g.vec(None)
    net.apply(bv, z)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.unet_applies):
        net.apply(bv, z)
    e1.record(stream)
    e1.synchronize()
    print(json.dumps({"mode": "U-Net applications", "workload": workload_name(args.size),
                      "applications": args.unet_applies, "ms_per_application": e0.elapsed_time(e1) / args.unet_applies}))
    return 0


def degrees(args):
    """The timed solve with other degrees and intervals of the Chebyshev
    preconditioner: iterations, true residual and device ms (best of 3)."""
    import xflow_gb300 as xf
    from xflow_gb300 import capi

    codes, sep, b = workload(args.size)
    ctx = xf.Context(0)
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    bv, x = g.vec(b), g.vec(np.zeros(g.shape))
    for pair in args.degrees.split(","):
        deg, ratio = (int(v) for v in pair.split(":"))
        ms = []
        for _ in range(3):
            x.fill(0.0)
            st = xf.solve(A, x, bv, method=xf.XF_CG, precision=xf.XF_PREC_MIXED, rtol=RTOL,
                          precond=capi.XF_PRECOND_CHEB, cheb_degree=deg, cheb_ratio=ratio)
            assert st.status == 0, st.status
            ms.append(st.ms)
        print(json.dumps({"degree": deg, "ratio": ratio, "iterations": st.iterations, "rel_resid": st.rel_resid,
                          "ms": min(ms)}), flush=True)
    return 0


def kernels_only(args):
    """Three launches of the FP32 and FP64 stencils and 32 iterations of the
    preconditioned mixed, plain mixed and FP64 CG on the full workload: a
    bounded command for ncu."""
    import xflow_gb300 as xf

    codes, sep, b = workload(args.size)
    ctx = xf.Context(0)
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    A = xf.Operator(g, xf.XF_OP_LAPLACE)
    rng = np.random.Generator(np.random.PCG64(1))
    xh = rng.standard_normal(g.shape)
    for dt in (xf.XF_F32, xf.XF_F64):
        p, q = g.vec(xh, dt), g.vec(None, dt)
        for _ in range(3):
            A.apply(p, q, flags=xf.XF_ZERO_INACTIVE)
    bv = g.vec(b)
    from xflow_gb300 import capi

    for prec, pre in ((xf.XF_PREC_MIXED, capi.XF_PRECOND_CHEB), (xf.XF_PREC_MIXED, None), (xf.XF_PREC_FP64, None)):
        x = g.vec(np.zeros(g.shape))
        st = xf.solve(A, x, bv, method=xf.XF_CG, precision=prec, rtol=RTOL, maxit=32, precond=pre)
        print(f"precision {prec} preconditioner {pre}: {st.iterations} iterations, {st.ms:.2f} ms, status {st.status}")
    ctx.synchronize()
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


UNET_TRAIN = dict(n=64, spheres=16, seed=5, rhs_seeds=(200, 201, 202), iters=(2, 5, 10, 20, 40, 80, 120, 160, 240),
                  steps=600, lr=2e-3)


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


def train_unet(ctx):
    """Trains the U-Net on the GPU (this library's forward/backward kernels,
    Adam, the A-norm loss) on (residual, error) pairs harvested from plain
    CG's own iterates on a 64^3 system of the bench's sphere family (16
    spheres, another seed).  Returns the parameters and a description."""
    import xflow_gb300 as xf
    from xflow_gb300 import workloads as wl

    T = UNET_TRAIN
    codes, nrm, _, sep, _ = wl.spheres_grid(T["n"], T["spheres"], 0.02, 0.06, T["seed"])
    g = xf.Grid(ctx, codes, sep, sep, sep, nrm)
    A = xf.Operator(g)
    net = xf.UNet(g, seed=1)
    t0 = time.perf_counter()
    rs, es = [], []
    for s in T["rhs_seeds"]:
        b = wl.divergence_rhs(codes, (sep,) * 3, s)
        r_, e_ = xf.harvest_pairs(A, g.vec(b), iters=T["iters"])
        rs += r_
        es += e_
    first = float(np.mean([net.train_step(r, e, update=False, op=A) for r, e in zip(rs, es)]))
    t1 = time.perf_counter()
    for step in range(T["steps"]):
        q = step % len(rs)
        net.train_step(rs[q], es[q], lr=T["lr"], op=A)
    ctx.synchronize()
    t2 = time.perf_counter()
    last = float(np.mean([net.train_step(r, e, update=False, op=A) for r, e in zip(rs, es)]))
    return net.params(), {"grid": f"{T['n']}^3, {T['spheres']} spheres, seed {T['seed']}", "pairs": len(rs),
                          "steps": T["steps"], "lr": T["lr"], "s": t2 - t1, "harvest_s": t1 - t0,
                          "anorm_loss_before": first, "anorm_loss_after": last}


def two_level(args):
    """The learned two-level preconditioner at the bench's 256^3 system: the
    U-Net trained as for --learned (64^3 sphere family, another geometry) runs
    on the coarse grid of 4^3 blocks (64^3) as the coarse solver, the FP32
    Chebyshev passes smooth, and FCG(window) drives both.  Prints one JSON
    line: training, the coarse application time, and per window the
    iterations and ms of the solve to a true 1e-8 relative residual, beside
    the untrained network and plain FP64 CG."""
    import torch

    import xflow_gb300 as xf
    from xflow_gb300 import capi
    from xflow_gb300 import workloads as wl

    ctx = xf.Context(0)
    stream = torch.cuda.ExternalStream(capi_stream(ctx))
    if args.two_level_profile:   # launch list of a short solve: untrained weights (the same kernels), 10 iterations
        codes, sep, b = workload(args.size)
        g = xf.Grid(ctx, codes, sep, sep, sep, None)
        cc, s1, s2, s3 = wl.coarse_grid(codes, sep, TL_BLOCK)
        gc = xf.Grid(ctx, cc, s1, s2, s3, None)
        net = xf.UNet(gc, seed=1)
        A = xf.Operator(g)
        for maxit in (2, 10):
            x = g.vec(np.zeros(g.shape))
            st = xf.solve_fcg(A, x, g.vec(b), unet=net, precond=capi.XF_PRECOND_UNET2, rtol=RTOL, maxit=maxit,
                              window=TL_WINDOW, degree=TL_DEGREE, ratio=TL_RATIO, precision=xf.XF_PREC_MIXED)
            print(json.dumps({"mode": "two-level profile", "maxit": maxit, "iterations": st.iterations,
                              "ms": st.ms, "launches": int(st.reserved[0]), "status": int(st.status)}))
        return 0
    params, train = train_unet(ctx)
    codes, sep, b = workload(args.size)
    g = xf.Grid(ctx, codes, sep, sep, sep, None)
    A = xf.Operator(g)
    cc, s1, s2, s3 = wl.coarse_grid(codes, sep, 4)
    gc = xf.Grid(ctx, cc, s1, s2, s3, None)
    net = xf.UNet(gc, params)
    bv = g.vec(b)
    rc, zc = gc.vec(np.zeros(gc.shape)), gc.vec(None)
    for _ in range(3):
        net.apply(rc, zc)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(10):
        net.apply(rc, zc)
    e1.record(stream)
    e1.synchronize()
    line = {"mode": "learned two-level preconditioner", "workload": f"{args.size}^3 spheres system (the bench's)",
            "coarse_grid": f"{gc.shape[0] - 2}^3 blocks of 4^3", "train": train,
            "coarse_unet_apply_ms": e0.elapsed_time(e1) / 10, "solves": {}}
    sweep = [tuple(int(v) for v in c.split(":")) for c in args.two_level_sweep.split(",")]
    fresh = xf.UNet(gc, seed=1)
    for label, nn in (("trained", net), ("untrained", fresh)):
        for deg, ratio, w, bits in sweep if nn is net else sweep[:1]:
            prec = xf.XF_PREC_MIXED if bits == 32 else xf.XF_PREC_FP64
            best = None
            for _ in range(2):
                x = g.vec(np.zeros(g.shape))
                st = xf.solve_fcg(A, x, bv, unet=nn, precond=capi.XF_PRECOND_UNET2, rtol=RTOL, window=w,
                                  degree=deg, ratio=ratio, precision=prec)
                if best is None or st.ms < best["ms"]:
                    best = {"iterations": st.iterations, "ms": st.ms, "rel_resid": st.rel_resid,
                            "status": int(st.status), "fallbacks": st.fallbacks, "refreshes": st.replacements}
            line["solves"][f"{label} degree {deg} ratio {ratio} window {w} fp{bits}"] = best
    x = g.vec(np.zeros(g.shape))
    st = xf.solve(A, x, bv, method=xf.XF_CG, rtol=RTOL)
    line["plain_fp64_cg"] = {"iterations": st.iterations, "ms": st.ms, "rel_resid": st.rel_resid}
    print(json.dumps(line))
    return 0


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
