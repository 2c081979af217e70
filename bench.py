"""Benchmark: H-matrix product throughput on one GB300 (and N replicas).

Workload (default): N = 1 000 000 points uniform on the unit sphere
(seeded), Laplace single-layer kernel 1/(4 pi r) with a zero diagonal, eta =
10, epsilon = 1e-6, partialACA, minclustersize 10; one N(0,1) right-hand side
per product.  The H-matrix is assembled on the GPU (device generator +
batched device partialACA, timed as `aca_seconds`); a "step" is one product
y = H x (mvprod_global_to_global), permutations included.

The headline `value` is the plain FP64 product (FP64 storage; each element
on the FP64 pipe or in double-float arithmetic on the FP32 pipe, as the
autotuner splits them), the arithmetic of the reference's CPU product it is
compared with.  The mixed-precision product (low-rank factors in FP32 / BF16
per column with per-column scaling, dense leaves FP64, FP32/FP64
accumulation) is measured in the same run (`mixed`), with its error against
the FP64 product and its speed-up over it.  Both read more than L2 holds per
product (tens of GB of factors), so no flush is needed.

Parity at full size: the CPU oracle builds the same H-matrix (bit-identical
leaves) and applies it to the same input; `rel_err_vs_reference` compares
the GPU products with that product.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--n N]
    python bench.py --workload batched [--steps K] [--warmup W]

The batched workload: 256 independent Laplace H-matrices on ellipsoids
(N_i log-uniform in [2 000, 50 000], axes uniform in [0.5, 2], 1 to 8
right-hand sides each, seed 4), all products captured as one CUDA graph and
replayed by one launch per step; `value` = right-hand sides applied per
second over the whole batch.

Prints one JSON line.  `value` is the device-resident throughput (x and y in
HBM); `e2e` is the same product through the C ABI from pinned host memory,
host<->device copies inside the timed region.  `--impl reference` times the
CPU restatement of htool's product (oracle/) on all host cores instead; that
arm does not load this package's library.
"""
import argparse
import importlib.util
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H-matvec/s and % HBM roofline at rel err ≤1e-6, mixed vs plain FP64; ACA secs"
UNIT = "H-matvec/s"
# the same `config` in both arms
WORKLOAD = dict(workload="laplace_sphere", n=1000000, kernel="1/(4 pi r), 0 on the diagonal", eta=10.0, epsilon=1e-6, minclustersize=10, compressor="partialACA", mu=1,
                l2="inputs larger than L2: the stored H-matrix read by every product is tens of GB")
DTYPE = "f64 (FP64 storage; DFMA and double-float FP32-pipe evaluation)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--n", type=int, default=WORKLOAD["n"])
    p.add_argument("--mu", type=int, default=WORKLOAD["mu"], help="sphere workload: right-hand sides per product")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-predictor", action="store_true", help="skip the rank-predictor rebuild")
    p.add_argument("--no-batched", action="store_true", help="skip the batched workload (the `batched` key)")
    p.add_argument("--workload", default="sphere", choices=["sphere", "batched", "helmholtz"],
                   help="sphere: the one-H-matrix product; batched: 256 H-matrices in one graph launch; helmholtz: the complex cube with 64 right-hand sides")
    p.add_argument("--count", type=int, default=256, help="batched: number of H-matrices")
    # fixed configuration instead of the autotuner (e.g. to replay a tuned run under a profiler)
    p.add_argument("--fp64-split", default=None, help="phase-1,phase-2 DFMA per mille, e.g. 0,650")
    p.add_argument("--phase1-mode", type=int, default=None, help="0 tile kernels, 1 streamed")
    p.add_argument("--mixed-split", type=int, default=None, help="mixed precision: DFMA per mille of the dense blocks")
    p.add_argument("--mixed-phase1-mode", type=int, default=None, help="mixed precision: 0 tile kernels, 1 streamed")
    p.add_argument("--phase2-mode", type=int, default=None, help="FP64: 0 per-warp streams, 1 producer-fed")
    p.add_argument("--mixed-phase2-mode", type=int, default=None, help="mixed precision: 0 per-warp streams, 1 producer-fed")
    p.add_argument("--mixed-dense-split", type=int, default=None, help="mixed precision, 4+ right-hand sides: 1 dense chunks first in the double-float kernel")
    p.add_argument("--tau", type=float, default=1.0, help="mixed precision: BF16 columns from the first whose storage bound is below tau * epsilon")
    p.add_argument("--digit-planes", type=int, default=None, help="8+ right-hand sides: 1 phase 1 on the BF16 tensor cores by exact digit slicing, 0 not")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def geometry():
    """htool_gb300/geometry.py loaded on its own: the point generators,
    without the package (whose import maps the GPU library)"""
    spec = importlib.util.spec_from_file_location("htool_gb300_geometry", os.path.join(ROOT, "htool_gb300", "geometry.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [c.strip() for c in r]
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference(n, reps, single_thread_reps=1, x=None, warmup=1, mu=1):
    """The CPU restatement of htool's product (oracle/htool_oracle.c, pinned
    to upstream htool) on the same workload: its assembly (HMatrix::build
    with partialACA, timed), then `reps` products on all host cores (median
    after one warm-up) and `single_thread_reps` on one core.  Returns the
    figures and the product of the seeded right-hand side."""
    G = geometry()
    from oracle.oracle import Oracle, build_port

    build_port()
    O = Oracle("port")
    threads = host_cores()
    O.set_num_threads(threads)
    pts = G.sphere(n, seed=1)
    t = O.cluster(pts)
    t0 = time.perf_counter()
    H = O.hmatrix(t, t, pts, pts, 1, WORKLOAD["epsilon"], WORKLOAD["eta"])
    build_s = time.perf_counter() - t0
    if x is None:
        x = G.rhs(n, mu, seed=2)
    for _ in range(max(0, warmup - 1)):  # time_mvprod warms up once more itself
        H.mvprod(x, mu)
    sec = H.time_mvprod(x, mu, reps)
    y = H.mvprod(x, mu)
    out = {"value": mu / sec, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": "%d products (median, after %d warm-up) of the N=%d Laplace-sphere H-matrix on %d threads; its assembly (%.2f s) not in the figure" % (reps, max(1, warmup), n, threads, build_s),
           "build_seconds": build_s, "threads": threads}
    if single_thread_reps:
        O.set_num_threads(1)
        t1 = time.perf_counter()
        for _ in range(single_thread_reps):
            H.mvprod(x, mu)
        st = (time.perf_counter() - t1) / single_thread_reps
        O.set_num_threads(threads)
        out["single_thread"] = {"value": mu / st, "unit": UNIT, "cores": 1, "sample": "%d product(s), one thread" % single_thread_reps}
    lr, dn = H.leaves()
    return out, y, (lr, dn)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cb, _, _ = cpu_reference(args.n, reps=max(args.steps, 3), single_thread_reps=0, warmup=args.warmup, mu=args.mu)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / cb["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded points on the unit sphere, N(0,1) right-hand side)", "config": dict(WORKLOAD, n=args.n, mu=args.mu),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}, "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "aca_seconds": cb["build_seconds"]}
    print(json.dumps(line), flush=True)


def sampled_dense_rows(pts, x, nrows=1000, seed=3):
    """rows (seeded sample) and (A x)[rows] of the dense Laplace matrix, in
    FP64 on the device (torch), 50 rows at a time"""
    import torch

    rows = np.random.default_rng(seed).choice(pts.shape[0], nrows, replace=False)
    P = torch.from_numpy(pts).cuda()
    X = torch.from_numpy(x).cuda()
    ref = torch.empty(nrows, dtype=torch.float64, device="cuda")
    for a in range(0, nrows, 50):
        r = torch.from_numpy(rows[a:a + 50]).cuda()
        d = torch.sqrt(((P[r][:, None, :] - P[None, :, :]) ** 2).sum(-1))
        k = torch.where(d == 0, torch.zeros_like(d), 1.0 / (4 * np.pi * d))
        ref[a:a + 50] = k @ X
        del d, k
    return rows, ref.cpu().numpy()


def run_gpu(args):
    import torch

    import htool_gb300 as H
    from htool_gb300 import geometry as G

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(v):
        if world > 1:
            tt = torch.tensor([v], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            return float(tt.item())
        return v

    n = args.n
    pts = G.sphere(n, seed=1)
    t = H.Cluster().build(n, pts)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hm = H.HMatrix(t, t, WORKLOAD["epsilon"], WORKLOAD["eta"], device=local).build(H.LAPLACE, pts)
    aca_seconds = time.perf_counter() - t0
    info = hm.get_infos()

    mu = args.mu
    x = G.rhs(n, mu, seed=2)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(n * mu, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    peak, peak_kind = measured_peaks()

    def timed_products():
        for _ in range(args.warmup):
            hm.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), mu, 0, sp)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            hm.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), mu, 0, sp)
        e1.record(stream)
        barrier()
        return max_over_ranks(e0.elapsed_time(e1)), hm.last_launches()

    def timed_e2e():
        """the product through the C ABI with host buffers: pinned x copied
        in, y copied out, inside the timed region, every step"""
        xh = torch.from_numpy(x).pin_memory()
        yh = torch.empty(n * mu, dtype=torch.float64).pin_memory()
        for _ in range(max(2, args.warmup)):
            hm.mvprod_ptr(xh.data_ptr(), yh.data_ptr(), mu, H.HOST_PTRS, None)
        barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            hm.mvprod_ptr(xh.data_ptr(), yh.data_ptr(), mu, H.HOST_PTRS, None)
        e2e_s = max_over_ranks(time.perf_counter() - w0)
        return {"value": world * args.steps * mu / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * n * mu, "d2h_bytes_per_step": 8 * n * mu}

    def profiled_traffic(kernel, precision, algorithmic):
        """DRAM bytes per launch of `kernel` from the committed ncu summaries
        (lines "traffic: kernel=K precision=P n=N [mu=M] bytes_per_launch=B
        algorithmic=A", mu 1 when absent; the same kernel, storage and
        right-hand sides): the captured launch's DRAM bytes scaled to this
        launch by its algorithmic bytes (traffic grows with the bytes
        streamed); None when no capture covers the kernel"""
        pdir = os.path.join(ROOT, "profiles")
        if not os.path.isdir(pdir):
            return None, None
        for name in sorted(os.listdir(pdir)):
            if not name.endswith(".md"):
                continue
            for line in open(os.path.join(pdir, name)):
                if line.startswith("traffic:"):
                    kv = dict(t.split("=", 1) for t in line.split()[1:] if "=" in t)
                    if kv.get("kernel") == kernel and kv.get("precision") == precision and kv.get("mu", "1") == str(mu) and "algorithmic" in kv:
                        ratio = int(kv["bytes_per_launch"]) / int(kv["algorithmic"])
                        return int(round(ratio * algorithmic)), "profiles/%s (n=%s capture, DRAM/algorithmic %.3f, scaled to this launch)" % (name, kv.get("n"), ratio)
        return None, None

    def describe(ms_total, precision):
        """per-step numbers, phase breakdown and the dominant kernel's roofline"""
        ms_step = ms_total / args.steps
        ph = hm.profile(mu, max(3, args.steps // 3))  # gather, phase 1, phase 2, sums, total
        pb = hm.phase_bytes(mu)
        mode1 = hm.get_phase1_mode()
        run = hm.get_rhs_bucket(mu) if mu <= 8 else mu
        if run <= 2:
            p1 = "phase 1 (tile kernels)" if mode1 == 0 else "phase1_cta_kernel"
        elif run >= 8 and hm.get_digit_planes()[0]:
            p1 = "phase1_oz_kernel"
        elif precision != "fp64":
            p1 = "phase1_mixed_kernel" if mode1 == 0 else ("phase1_tc_kernel" if mode1 == 2 and run >= 8 else "phase1_stack_kernel")
        else:
            p1 = "phase1_df_mrhs_kernel" if run >= 8 else "phase 1 (tile kernels)"
        if precision == "fp64" and run >= 8:
            p2 = "phase2_oz_kernel" if hm.get_digit_planes()[0] else "phase2_df_mrhs_kernel"
        else:
            p2 = "phase2_warp_kernel" if hm.get_phase2_mode() == 0 else "phase2_ws_kernel"
        names = ["gather_split_kernel", p1, p2, "zsum_kernel"]
        k = max(range(4), key=lambda i: ph[i])
        achieved = pb[k] / (ph[k] / 1e3) / 1e9
        total_bytes = sum(pb)
        traffic, traffic_src = profiled_traffic(names[k], precision, pb[k])
        return ms_step, {
            "phase_ms": {"gather": ph[0], "phase1": ph[1], "phase2": ph[2], "sums": ph[3], "total": ph[4]},
            "phase_bytes": {"gather": pb[0], "phase1": pb[1], "phase2": pb[2], "sums": pb[3]},
            "whole_product": {"bytes": total_bytes, "GB_per_s": total_bytes / (ms_step / 1e3) / 1e9, "frac_of_hbm_peak": total_bytes / (ms_step / 1e3) / 1e9 / peak},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src, "kernel": names[k], "kernel_ms": ph[k], "algorithmic_bytes": pb[k],
                         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind},
        }

    fixed = any(v is not None for v in (args.fp64_split, args.phase1_mode, args.mixed_split, args.mixed_phase1_mode, args.phase2_mode, args.mixed_phase2_mode, args.mixed_dense_split, args.digit_planes))
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.5)  # let the sampler start before the timed regions
    # plain FP64 (autotuned DFMA / FP32-pipe split): the headline
    hm.set_precision("fp64")
    if fixed:
        if args.fp64_split is not None:
            hm.set_fp64_split(*[int(v) for v in args.fp64_split.split(",")])
        if args.phase1_mode is not None:
            hm.set_phase1_mode(args.phase1_mode)
        if args.phase2_mode is not None:
            hm.set_phase2_mode(args.phase2_mode)
        if args.digit_planes is not None:
            hm.set_digit_planes(bool(args.digit_planes))
        tune64 = None
    else:
        tune64 = hm.autotune(mu, 5)
    split = hm.get_fp64_split()
    p1mode64, p2mode64 = hm.get_phase1_mode(), hm.get_phase2_mode()
    planes64 = hm.get_digit_planes()[0]
    ms64, launches64 = timed_products()
    y64 = yd.cpu().numpy().copy()
    step64, d64 = describe(ms64, "fp64")
    e2e64 = timed_e2e()
    # mixed precision
    tau = args.tau
    hm.set_precision("mixed", tau)
    if fixed:
        if args.mixed_split is not None:
            hm.set_fp64_split(split[0], args.mixed_split)
        if args.mixed_phase1_mode is not None:
            hm.set_phase1_mode(args.mixed_phase1_mode)
        if args.mixed_phase2_mode is not None:
            hm.set_phase2_mode(args.mixed_phase2_mode)
        if args.mixed_dense_split is not None:
            hm.set_phase2_dense_split(bool(args.mixed_dense_split))
        if args.digit_planes is not None:
            hm.set_digit_planes(bool(args.digit_planes))
        tunem = None
    else:
        tunem = hm.autotune(mu, 5)
    splitm = hm.get_fp64_split()[1]
    msm, launchesm = timed_products()
    ym = yd.cpu().numpy().copy()
    stepm, dm = describe(msm, "mixed")
    e2em = timed_e2e()
    pinfo = hm.precision_info()
    clk = clocks.stop()
    value64 = world * args.steps * mu / (ms64 / 1e3)
    valuem = world * args.steps * mu / (msm / 1e3)
    status = hm.device_status()
    hm.set_precision("fp64")
    rows, dense_ref = sampled_dense_rows(pts, x[:n])  # the first right-hand side

    # learned rank predictor: trained on the (geometry, crosses) pairs this
    # build's partialACA produced, then the same mesh re-assembled with it
    predictor = None
    if not args.no_predictor:
        X, yr = hm.aca_samples()
        mlp = H.RankPredictor(device=local, seed=1)
        t1 = time.perf_counter()
        loss = mlp.train(X, np.minimum(yr, 64), epochs=30, batch=2048, lr=3e-3, seed=2)
        train_s = time.perf_counter() - t1
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        hl = H.HMatrix(t, t, WORKLOAD["epsilon"], WORKLOAD["eta"], device=local).set_rank_predictor(mlp).build(H.LAPLACE, pts)
        aca_learned = time.perf_counter() - t1
        il = hl.get_infos()
        same = bool(np.array_equal(hl.get_leaves()[0], hm.get_leaves()[0]) and np.array_equal(hl.get_leaves()[1], hm.get_leaves()[1]))
        predictor = {"train_samples": int(yr.size), "train_seconds": train_s, "epochs": 30, "final_mse": float(loss[-1]),
                     "aca_seconds": {"fixed_first_attempt": aca_seconds, "predicted_first_attempt": aca_learned},
                     "scratch_bytes": {"fixed_first_attempt": int(info["GPU_aca_scratch_bytes"]), "predicted_first_attempt": int(il["GPU_aca_scratch_bytes"])},
                     "rerun_rate": int(il["GPU_aca_overflow_reruns"]) / max(1, int(il["GPU_aca_predicted_blocks"])), "same_leaves": same}
        # what pre-sizing buys when memory is short: both builds under the
        # same ACA scratch budget (1.1 x what the predicted first attempts
        # take), where the fixed first attempts need more slices
        budget = int(1.1 * int(il["GPU_aca_scratch_bytes"]))
        del hl
        under = {"budget_bytes": budget, "aca_seconds": {}, "aca_slices": {}, "same_leaves": True}
        for name, use in (("fixed_first_attempt", False), ("predicted_first_attempt", True)):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            hb = H.HMatrix(t, t, WORKLOAD["epsilon"], WORKLOAD["eta"], device=local).set_aca_budget(budget)
            if use:
                hb.set_rank_predictor(mlp)
            hb.build(H.LAPLACE, pts)
            under["aca_seconds"][name] = time.perf_counter() - t1
            under["aca_slices"][name] = int(float(hb.get_infos()["GPU_aca_rounds"]))
            under["same_leaves"] = under["same_leaves"] and bool(np.array_equal(hb.get_leaves()[0], hm.get_leaves()[0]))
            del hb
        predictor["under_scratch_budget"] = under

    gpu_leaves = hm.get_leaves()
    # the batched workload (256 H-matrices, one graph launch per step),
    # measured in the same run
    batched = None
    if not args.no_batched:
        hm.set_precision("fp64")
        batched = batched_workload(local, args.steps, args.warmup, args.count, world)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    err_mixed_vs_fp64 = float(np.linalg.norm(ym - y64) / np.linalg.norm(y64))
    dense_err = {k: float(np.linalg.norm(v[:n][rows] - dense_ref) / np.linalg.norm(dense_ref)) for k, v in (("fp64", y64), ("mixed", ym))}
    line = {
        "metric": METRIC, "value": value64, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step64, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
        "data": "synthetic (seeded points on the unit sphere, N(0,1) right-hand side)",
        "config": dict(WORKLOAD, n=n, mu=mu),
        "run": {"precision": "fp64", "parallelism": "replicas" if world > 1 else "single", "stored_gb": {"fp64": d64["whole_product"]["bytes"] / 1e9, "mixed": dm["whole_product"]["bytes"] / 1e9}},
        "roofline": d64["roofline"], "whole_product": d64["whole_product"], "phase_ms": d64["phase_ms"], "phase_bytes": d64["phase_bytes"],
        "fp64_split": {"phase1_dfma_permille": split[0], "phase2_dfma_permille": split[1], "autotune_ms": tune64, "phase1_mode": p1mode64, "phase2_mode": p2mode64, "digit_planes": planes64},
        "e2e": e2e64,
        "mixed": {"value": valuem, "unit": UNIT, "ms_per_step": stepm, "speedup_vs_fp64": valuem / value64, "rel_err_vs_fp64": err_mixed_vs_fp64, "tau": tau,
                  "dtype": "fp32/bf16 factors (per-column scaled), fp64 dense, fp32+fp64 accumulation", "e2e": e2em,
                  "roofline": dm["roofline"], "whole_product": dm["whole_product"], "phase_ms": dm["phase_ms"], "phase_bytes": dm["phase_bytes"],
                  "precision": {"fp32_columns": pinfo["fp32_columns"], "bf16_columns": pinfo["bf16_columns"], "stored_bytes": pinfo["stored_bytes"], "autotune_ms": tunem, "phase1_mode": hm.get_phase1_mode(), "phase2_mode": hm.get_phase2_mode(), "dense_dfma_permille": splitm, "digit_planes": hm.get_digit_planes()[0]},
                  "gpu_launches": launchesm * args.steps},
        "gpu_launches": launches64 * args.steps, "clocks": clk, "device_status": status,
        "rel_err_vs_dense_1000_rows": dense_err,
        "aca_seconds": aca_seconds,
        "assembly_breakdown_s": {"block_tree": float(info["GPU_block_tree_seconds"]), "aca_rounds": float(info["GPU_aca_seconds"]),
                                 "layout_and_uploads": float(info["GPU_build_seconds"]) - float(info["GPU_aca_seconds"]) - float(info["GPU_block_tree_seconds"]),
                                 "layout_host_lists": float(info.get("GPU_layout_host_seconds", 0)), "layout_device_copies": float(info.get("GPU_layout_device_seconds", 0)),
                                 "layout_launch_lists": float(info.get("GPU_layout_lists_seconds", 0)),
                                 "aca_blocks": int(info["GPU_aca_blocks"]), "aca_rounds_launched": int(float(info["GPU_aca_rounds"]))},
        "rank_predictor": predictor,
        "hmatrix": {k: info[k] for k in ("Number_of_lrmat", "Number_of_dmat", "Number_of_false_positive", "Rank_max", "Rank_mean", "Compression_ratio")},
        "batched": batched,
    }
    if not args.no_cpu_baseline:
        cb, y_ref, ref_leaves = cpu_reference(n, reps=5, single_thread_reps=1, x=x, mu=mu)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "single_thread")}
        line["cpu_aca_seconds"] = cb["build_seconds"]
        line["rel_err_vs_reference"] = {
            "fp64": float(np.linalg.norm(y64 - y_ref) / np.linalg.norm(y_ref)), "mixed": float(np.linalg.norm(ym - y_ref) / np.linalg.norm(y_ref)),
            "same_leaves": bool(np.array_equal(gpu_leaves[0], ref_leaves[0]) and np.array_equal(gpu_leaves[1], ref_leaves[1])),
            "reference": "the CPU oracle's product (oracle/htool_oracle.c, pinned to upstream htool) of its own build of this H-matrix on the same input"}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def batched_items(count, seed=4):
    """(n, axes, mu) of the batched workload's H-matrices"""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(2000), np.log(50000)))))
        axes = rng.uniform(0.5, 2.0, 3)
        mu = int(rng.integers(1, 9))
        out.append((n, axes, mu))
    return out


def batched_workload(local, steps, warmup, count=256, world=1, sample_parity=True):
    """The batched workload: every H-matrix of `batched_items(count)` is a
    member of one forest per right-hand-side count (a block-diagonal
    H-matrix built by one device assembly and applied by one product), and
    the forests' products are captured as one CUDA graph: one launch per
    step.  FP64 then mixed precision, each forest autotuned (kernel modes,
    FP64 split, right-hand-side bucket).  Returns the measurements."""
    import torch

    import htool_gb300 as H
    from htool_gb300 import geometry as G

    eps, eta = WORKLOAD["epsilon"], WORKLOAD["eta"]
    items = batched_items(count)
    buckets = {}
    for k, (_, _, mu) in enumerate(items):
        buckets.setdefault(mu, []).append(k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    forests = []
    for mu in sorted(buckets):
        ks = buckets[mu]
        trees, pts, ns = [], [], []
        for k in ks:
            n, axes, _ = items[k]
            p = G.ellipsoid(n, axes, seed=100 + k)
            trees.append(H.Cluster().build(n, p))
            pts.append(p)
            ns.append(n)
        F = H.Cluster.forest(trees)
        hm = H.HMatrix(F, F, eps, eta, device=local).build(H.LAPLACE, np.concatenate(pts))
        xs = [G.rhs(n, mu, seed=10 + k) for n, k in zip(ns, ks)]
        cat = np.concatenate([np.concatenate([x[c * n:(c + 1) * n] for x, n in zip(xs, ns)]) for c in range(mu)])
        N = int(sum(ns))
        forests.append(dict(mu=mu, ks=ks, ns=ns, N=N, hm=hm, pts=pts, x=torch.from_numpy(cat).cuda(), y=torch.zeros(N * mu, dtype=torch.float64, device="cuda")))
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    total_mu = sum(mu for _, _, mu in items)
    stream = torch.cuda.current_stream()

    def members(f, y):
        cols = y.reshape(f["mu"], f["N"])
        out, off = [], 0
        for n in f["ns"]:
            out.append(np.ascontiguousarray(cols[:, off:off + n]).reshape(-1))
            off += n
        return out

    def timed(policy):
        tune = {}
        for f in forests:
            if policy == "fp64":
                f["hm"].set_precision("fp64")
            else:
                f["hm"].set_precision(policy, 1.0)
            tune[f["mu"]] = f["hm"].autotune(f["mu"], 3)
        batch = H.HBatch(local)
        for f in forests:
            batch.add(f["hm"], f["x"].data_ptr(), f["y"].data_ptr(), f["mu"], keep=(f["x"], f["y"]))
        nodes = batch.capture(nstreams=len(forests))
        for _ in range(max(warmup, 3)):
            batch.launch(stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            batch.launch(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        nbytes = sum(sum(f["hm"].phase_bytes(f["mu"])) for f in forests)
        ys = [f["y"].cpu().numpy().copy() for f in forests]
        info = {"bucket_run": {str(f["mu"]): f["hm"].get_rhs_bucket(f["mu"]) for f in forests}, "autotune_ms": {str(k): v for k, v in tune.items()}, "graph_nodes": nodes}
        del batch
        return ms, nbytes, ys, info

    clocks = Clocks(local)
    clocks.start()
    ms64, bytes64, ys64, info64 = timed("fp64")
    msm, bytesm, ysm, infom = timed("mixed")
    ck = clocks.stop()
    err = 0.0
    for f, a, b in zip(forests, ysm, ys64):
        for ym, y6 in zip(members(f, a), members(f, b)):
            err = max(err, float(np.linalg.norm(ym - y6) / np.linalg.norm(y6)))
    parity = None
    if sample_parity:
        # the oracle's own build and product of one member per forest (its
        # smallest), against that member's rows of both products
        from oracle.oracle import Oracle, build_port

        build_port()
        O = Oracle("port")
        O.set_num_threads(host_cores())
        worst = {"fp64": 0.0, "mixed": 0.0}
        for f, a, b in zip(forests, ysm, ys64):
            q = int(np.argmin(f["ns"]))
            p = f["pts"][q]
            ot = O.cluster(p)
            oh = O.hmatrix(ot, ot, p, p, 1, eps, eta)
            yo = oh.mvprod(G.rhs(f["ns"][q], f["mu"], seed=10 + f["ks"][q]), f["mu"])
            for key, y in (("fp64", b), ("mixed", a)):
                worst[key] = max(worst[key], float(np.linalg.norm(members(f, y)[q] - yo) / np.linalg.norm(yo)))
        parity = {"max_rel_err": worst, "members_checked": len(forests), "reference": "the CPU oracle's build and product of the smallest member of every forest (oracle/htool_oracle.c, pinned to upstream htool)"}
    peak, peak_src = measured_peaks()
    free_b, total_b = torch.cuda.mem_get_info()
    out = {
        "value": world * total_mu / (msm * 1e-3), "ms_per_step": msm, "fp64_value": world * total_mu / (ms64 * 1e-3), "fp64_ms_per_step": ms64, "mixed_speedup_vs_fp64": ms64 / msm,
        "max_rel_err_mixed_vs_fp64": err, "rel_err_vs_reference": parity,
        "whole_batch": {"mixed": {"bytes": bytesm, "GB_per_s": bytesm / (msm * 1e-3) / 1e9, "frac_of_hbm_peak": bytesm / (msm * 1e-3) / 1e9 / peak},
                        "fp64": {"bytes": bytes64, "GB_per_s": bytes64 / (ms64 * 1e-3) / 1e9, "frac_of_hbm_peak": bytes64 / (ms64 * 1e-3) / 1e9 / peak}, "peak_source": peak_src},
        "forests": {str(f["mu"]): {"members": len(f["ks"]), "points": f["N"]} for f in forests}, "tuning": {"fp64": info64, "mixed": infom},
        "count": len(items), "n_total": int(sum(i[0] for i in items)), "rhs_total": total_mu, "build_seconds": build_s, "device_gb_in_use": (total_b - free_b) / 1e9, "clocks": ck,
    }
    for f in forests:
        del f["hm"]
    return out


def run_batched(args):
    """256 H-matrices in one forest per right-hand-side count, one graph
    launch per step (replicas under torchrun)"""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    b = batched_workload(local, args.steps, args.warmup, args.count, world)
    line = {
        "metric": "H-matvec/s over a batch of %d H-matrices (one graph launch per step), mixed vs plain FP64" % b["count"],
        "value": b["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/bf16 factors, f64 dense", "data": "synthetic (seeded ellipsoids)",
        "config": {"workload": "batched_laplace_ellipsoids", "count": b["count"], "n_total": b["n_total"], "rhs_total": b["rhs_total"], "epsilon": WORKLOAD["epsilon"], "eta": WORKLOAD["eta"], "tau": 1.0,
                   "l2": "inputs larger than L2 (%.1f GB per step)" % (b["whole_batch"]["mixed"]["bytes"] / 1e9)},
        "batched": b, "clocks": b["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_helmholtz(args):
    """Complex Helmholtz exp(ikr)/(4 pi r), k = 20, on N = 200 000 points of
    the unit-cube surface (seeded), eta = 3, epsilon = 1e-5: products with 64
    complex N(0,1) + i N(0,1) right-hand sides, FP64 (double-float kernels)
    and mixed precision (both low-rank contractions on the tensor cores,
    tcgen05 and the warp-level mma.sync kernels), errors against FP64."""
    import torch

    import htool_gb300 as H
    from htool_gb300 import geometry as G

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    n = args.n if args.n != WORKLOAD["n"] else 200000
    mu = 64
    pts = G.cube_surface(n, seed=1)
    t = H.Cluster().build(n, pts)
    t0 = time.perf_counter()
    hm = H.HMatrix(t, t, 1e-5, 3.0, device=local, dtype=np.complex128).build(H.HELMHOLTZ, pts, kernel_param=20.0)
    build_s = time.perf_counter() - t0
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n * mu) + 1j * rng.standard_normal(n * mu)
    xd = torch.from_numpy(x.view(np.float64).copy()).cuda()
    yd = torch.empty_like(xd)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def timed(steps):
        for _ in range(max(args.warmup, 3)):
            hm.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), mu, 0, stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            hm.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), mu, 0, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, yd.cpu().numpy().copy()

    steps = max(1, min(args.steps, 20))
    clocks = Clocks(local)
    clocks.start()
    ms64, y64 = timed(steps)
    ph64 = hm.profile(mu, 3)
    hm.set_precision("mixed", 1.0)
    hm.set_tensor_core_mode("tcgen05")
    ms_tc, y_tc = timed(steps)
    ph_tc = hm.profile(mu, 3)
    hm.set_tensor_core_mode("tcgen05_both")
    ms_both, y_both = timed(steps)
    ph_both = hm.profile(mu, 3)
    hm.set_tensor_core_mode("mma.sync")
    ms_mma, y_mma = timed(steps)
    ph_mma = hm.profile(mu, 3)
    hm.set_tensor_core_mode("tcgen05")
    # the tcgen05 phase 1 from the factors' pre-laid-out copy
    hm.set_tensor_core_arena(True)
    arena_bytes = hm.get_tensor_core_arena()[1]
    ms_arena, y_arena = timed(steps)
    ph_arena = hm.profile(mu, 3)
    hm.set_tensor_core_arena(False)
    # phase 1 on the BF16 tensor cores by exact digit slicing (4 planes)
    hm.set_digit_planes(True)
    ms_dpm, y_dpm = timed(steps)
    ph_dpm = hm.profile(mu, 3)
    # FP64 with 8 planes in both phases
    hm.set_precision("fp64")
    planes64 = hm.get_digit_planes()[1]
    ms_dp64, y_dp64 = timed(steps)
    ph_dp64 = hm.profile(mu, 3)
    hm.set_digit_planes(False)
    # the native complex layout (entries at 16 bytes instead of the real
    # form's 32) against the real form, FP64 and autotuned: one right-hand
    # side (bandwidth-bound) and 64 (the double-float kernels; the digit
    # planes serve the real form only)
    def timed_on(h, m, k):
        for _ in range(max(args.warmup, 3)):
            h.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), m, 0, stream.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            h.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), m, 0, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k, yd[: 2 * n * m].cpu().numpy().copy()

    peak, peak_kind = measured_peaks()
    t0 = time.perf_counter()
    hz = H.HMatrix(t, t, 1e-5, 3.0, device=local, dtype=np.complex128, complex_layout="native").build(H.HELMHOLTZ, pts, kernel_param=20.0)
    build_native_s = time.perf_counter() - t0
    single, y1 = {}, {}
    rel_to = lambda y, ref: float(np.linalg.norm(y - ref) / np.linalg.norm(ref))
    for prec in ("fp64", "mixed"):
        for name, h in (("real_form", hm), ("native", hz)):
            h.set_precision(prec, 1.0)
            h.autotune(1, 5)
            ms1, y = timed_on(h, 1, max(steps, 10))
            ph1 = h.profile(1, 5)
            b = h.precision_info()["stored_bytes"]
            key = name if prec == "fp64" else name + "_mixed"
            y1[key] = y
            single[key] = {"ms": ms1, "stored_bytes": b, "GB_per_s_stored": b / (ms1 * 1e-3) / 1e9, "frac_of_hbm_peak": b / (ms1 * 1e-3) / 1e9 / peak, "peak": peak_kind,
                           "phase_ms": {"gather": ph1[0], "phase1": ph1[1], "phase2": ph1[2], "sums": ph1[3], "total": ph1[4]}}
    for key in ("native", "real_form_mixed", "native_mixed"):
        single[key]["rel_err_vs_real_form_fp64"] = rel_to(y1[key], y1["real_form"])
    hm.set_precision("fp64")
    # 64 right-hand sides in the native layout: reduced precision (tensor
    # cores: phase 1 tcgen05, phase 2 mma.sync), then FP64 (double-float)
    ms64nm, y64nm = timed_on(hz, mu, min(steps, 3))
    hz.set_precision("fp64")
    ms64n, y64n = timed_on(hz, mu, min(steps, 3))
    native = {"build_seconds": build_native_s, "one_rhs": single, "speedup_one_rhs": single["real_form"]["ms"] / single["native"]["ms"],
              "speedup_one_rhs_mixed": single["real_form_mixed"]["ms"] / single["native_mixed"]["ms"],
              "fp64_64rhs": {"ms": ms64n, "rel_err_vs_fp64": rel_to(y64n, y64)},
              "mixed_64rhs": {"ms": ms64nm, "rel_err_vs_fp64": rel_to(y64nm, y64), "kernels": "phase 1 tcgen05, phase 2 mma.sync"},
              "status": hz.device_status()}
    del hz
    ck = clocks.stop()
    status = hm.device_status()
    info = hm.get_infos()
    err = lambda y: float(np.linalg.norm(y - y64) / np.linalg.norm(y64))
    # the headline: the fastest reduced-precision variant within epsilon of FP64
    variants = {"mixed_tcgen05": (ms_tc, y_tc), "mixed_tcgen05_arena": (ms_arena, y_arena), "mixed_digit_planes": (ms_dpm, y_dpm), "mixed_mma_sync": (ms_mma, y_mma), "mixed_tcgen05_both": (ms_both, y_both)}
    best_name = min((k for k in variants if err(variants[k][1]) <= 1e-5), key=lambda k: variants[k][0])
    ms_best = variants[best_name][0]
    phases = lambda ph: {"gather": ph[0], "phase1": ph[1], "phase2": ph[2], "sums": ph[3], "total": ph[4]}
    line = {
        "metric": "complex H-matmat with 64 right-hand sides per second (H-matvec/s = 64 / time)", "value": world * mu / (ms_best * 1e-3), "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_best, "headline_variant": best_name, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32/bf16 factors (per-column scaled), fp64 dense; tensor-core contractions (TF32x3 with FP32 accumulation, or exact BF16 digit planes: headline_variant)", "data": "synthetic (seeded points on the unit-cube surface)",
        "config": {"workload": "helmholtz_cube", "n": n, "wavenumber": 20.0, "eta": 3.0, "epsilon": 1e-5, "mu": mu, "l2": "inputs larger than L2 (the stored H-matrix, tens of GB)"},
        "mixed_tcgen05": {"ms": ms_tc, "rel_err_vs_fp64": err(y_tc), "phase_ms": phases(ph_tc), "kernels": "phase 1 tcgen05, phase 2 mma.sync (the default)"},
        "mixed_tcgen05_both": {"ms": ms_both, "rel_err_vs_fp64": err(y_both), "phase_ms": phases(ph_both)},
        "mixed_mma_sync": {"ms": ms_mma, "rel_err_vs_fp64": err(y_mma), "phase_ms": phases(ph_mma)},
        "mixed_tcgen05_arena": {"ms": ms_arena, "phase_ms": phases(ph_arena), "arena_bytes": arena_bytes, "bitwise_equal_to_tcgen05": bool(np.array_equal(y_arena, y_tc))},
        "mixed_digit_planes": {"ms": ms_dpm, "rel_err_vs_fp64": err(y_dpm), "phase_ms": phases(ph_dpm), "kernels": "phase 1 on 4 BF16 digit planes (exact sums), phase 2 mma.sync"},
        "fp64_digit_planes": {"ms": ms_dp64, "rel_err_vs_fp64": err(y_dp64), "phase_ms": phases(ph_dp64), "plane_bytes": planes64, "kernels": "both phases on 8 BF16 digit planes (exact sums)"},
        "fp64": {"ms": ms64, "phase_ms": phases(ph64)},
        "fp64_native_complex_layout": native,
        "build_seconds": build_s, "clocks": ck, "device_status": status,
        "hmatrix": {k: info[k] for k in ("Number_of_lrmat", "Number_of_dmat", "Rank_max", "Rank_mean", "Compression_ratio")},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "batched":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched workload has no reference arm in this script; the sphere workload carries it"}), flush=True)
            return
        run_batched(args)
    elif args.workload == "helmholtz":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the complex workload has no reference arm in this script; the sphere workload carries it"}), flush=True)
            return
        run_helmholtz(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
