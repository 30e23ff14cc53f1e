"""Benchmark: batched signed-distance queries (GJK distance + EPA penetration)
on the mixed-primitive workload — 1M pairs of sphere / box / capsule /
cylinder / convex shapes (convex hulls of log-uniform 8..256 sphere points,
sizes U[0.02, 0.4] m, ~40 % overlapping) — on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

A step is one signed-distance query over the whole batch: the GJK pass over
all pairs, then the EPA pass over the overlapping ones.  ``value`` times steps
with the pairs and shapes already in HBM (the device entry point);
``e2e`` times the host entry point (fclg_distance) from pinned host memory,
H2D of the pair list and D2H of the results included, shapes uploaded once
beforehand as a caller constructs its geometry objects once.  The inputs
(~0.6 GB of pairs, shapes and hull vertices) exceed the 129 MB L2, so no L2
flush is needed between steps.

The default line also carries ``config.warm_start``: the learned warm start
trained on the GPU on plain-GJK directions of held-out seeds (mixed and arm
workloads), then plain vs warm queries/s on the same pairs, GJK iterations,
answer differences and the tcgen05 inference kernel's TFLOP/s.
``--workload pareto | plain_small | arm`` print the same line for the other
convex configurations; ``--workload mesh`` the BVH line.

``--impl reference`` times the reference's CPU implementation of the same
query (its GJKSolver::shapeSignedDistance path) on the host cores: the
FP64 restatement in oracle/, which is bit-identical to the reference's own
GJK / EPA (tests/test_oracle.py), on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mind-fcl_gb300"))

import numpy as np  # noqa: E402

METRIC = "convex pair queries/s (GJK+EPA) & BVH collides/s, warm-start vs plain, 1 GB300"
UNIT = "pair queries/s"
N_PAIRS = 1_000_000
# compulsory bytes per query of this workload: hull vertices (12 B each) of the
# convex shapes, 16 B of parameters per primitive, 48 B pose, 2 x 8 B shape
# descriptors and a 64 B result record, averaged over the shape mix
ALGO_BYTES_PER_QUERY = 498.0
CPU_SAMPLE_PAIRS = 40_000
CPU_SAMPLE_SECONDS = 10.0
WORKLOAD = ("mixed primitive batch: 1M pairs of sphere/box/capsule/cylinder/convex (convex V log-uniform "
            "[8,256]), sizes U[0.02,0.4] m, ~40% overlap; GJK distance for separated pairs, EPA depth + "
            "normal for overlapping pairs")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="fclg", choices=["fclg", "reference"])
    ap.add_argument("--pairs", type=int, default=N_PAIRS)
    ap.add_argument("--workload", default="mixed",
                    choices=["mixed", "mesh", "mesh_shape", "scene", "ccd", "pareto", "plain_small", "arm", "warmstart"],
                    help="mixed: the headline convex-pair batch (with the warm-start comparison); mesh: the "
                         "50k x 50k-triangle BVH workload; pareto: 4M heavy-tailed hull pairs; plain_small: 4096 "
                         "hull pairs; arm: 7-link arm x 32 obstacles, 100k configurations; mesh_shape: the "
                         "50k-triangle mesh against 65,536 mixed-shape queries; warmstart: the "
                         "warm-start inference kernel alone on 2.24M arm pairs; ccd: translational continuous "
                         "collision of 1M mixed pairs")
    ap.add_argument("--no-warm", action="store_true", help="skip the warm-start comparison")
    ap.add_argument("--no-mesh", action="store_true", help="skip the mesh-mesh block of the default line")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain-method block of the default line")
    ap.add_argument("--poses", type=int, default=65536)
    ap.add_argument("--configs", type=int, default=100_000, help="arm: joint configurations (7 x 32 pairs each)")
    ap.add_argument("--objects", type=int, default=100_000, help="scene: posed objects")
    ap.add_argument("--tuning", default=None,
                    help="convex workloads: a fixed launch shape as JSON (fclg_tuning fields, e.g. "
                         "'{\"gjk_refill\": 0, \"gjk_lanes_large\": 1}') instead of the autotuner's choice")
    ap.add_argument("--sweep", action="store_true",
                    help="convex workloads: time one query per launch layout (GJK lanes, hull split, support "
                         "walk on / off) and print them as one JSON object instead of the bench line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


# other convex workloads: (generator, compulsory bytes per query, description)
CONVEX_WORKLOADS = {
    "mixed": (None, ALGO_BYTES_PER_QUERY, WORKLOAD),
    "pareto": ("pareto", 398.0, "large uneven batch: 4M convex pairs, hull vertex counts Pareto(alpha 1.5, x_m 4) "
                                "clipped to [4, 1024], ~30% overlap; GJK distance + EPA"),
    "plain_small": ("plain_small", 896.0, "plain method, small: 4096 pairs of 32-vertex hulls (radius "
                                          "U[0.05,0.5] m), translation in a 1 m cube; GJK distance + EPA"),
    "arm": ("arm", 128.0, "learned warm start workload: 7-link arm (hulls of 64-256 vertices) x 32 obstacle hulls "
                          "(64 vertices), 100k joint configurations = 22.4M link-obstacle pairs; GJK distance + EPA"),
}
MLP_FLOP_PER_PAIR = 2.0 * (28 * 256 + 2 * 256 * 256 + 256 * 3)
# DRAM bytes (read + write) of the three EPA launches (128-face pass, 256-face
# pass, final solves) of one mixed-workload query at 10^6 pairs: one ncu capture
# at 400 k pairs (profiles/epa_pass_mixed_400k.md), scaled by the pairs (the
# traffic is per overlapping pair)
EPA_TRAFFIC_MIXED_1M = ((141.391104 + 94.594304) + (59.201024 + 0.594176) + (18.391296 + 0.365824)) * 1e6 \
    * (1_000_000 / 400_000)


def _to_dev(torch, arr, dev):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).copy()).to(dev)


def _time_queries(torch, ctx, d_pairs, n, flags, steps, warmup, stream, dev):
    """Device time per signed-distance query over n resident pairs, and the last results."""
    from fclg.api import make_request
    from fclg.layout import RESULT_DTYPE
    req = make_request(flags=flags) if flags else None
    d_res = torch.empty(n * 48, dtype=torch.uint8, device=dev)

    def step():
        ctx.distance_device(d_pairs.data_ptr(), n, d_res.data_ptr(), req, stream.cuda_stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1) / max(steps, 1), d_res.cpu().numpy().view(RESULT_DTYPE).copy()


def fp64_block(args, torch, dev, stream, local):
    """The plain method in FP64 on the GPU (fclg_distance64: shapeDistance per
    pair, one thread per pair) beside the FP32 kernels on the plain-method
    workload: 4096 pairs of 32-vertex hulls (the reference's small case) and
    262,144 pairs of the same kind.  Device time per query, inputs resident."""
    from fclg import workloads
    from fclg.api import FCLG_REQ_NO_EPA, Context
    from fclg.layout import GJK_SEPARATED, RESULT64_DTYPE
    out = {"what": "GJKSolver<double>::shapeDistance on the GPU in FP64 (thread per pair) vs the FP32 GJK "
                   "distance (no EPA) and the FP32 signed distance (GJK + EPA), same pairs, device-resident"}
    for n in (4096, 262_144):
        batch = workloads.plain_small(n)
        ctx = Context(local)
        ctx.set_batch(batch)
        d_pairs = torch.from_numpy(batch.pairs.view(np.uint8).copy()).to(dev)
        d64 = torch.empty(n * 64, dtype=torch.uint8, device=dev)

        def step64():
            ctx.distance64_device(d_pairs.data_ptr(), n, d64.data_ptr(), None, stream.cuda_stream)

        for _ in range(max(3, args.warmup)):
            step64()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(5, args.steps)
        e0.record(stream)
        for _ in range(reps):
            step64()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms64 = e0.elapsed_time(e1) / reps
        r64 = d64.cpu().numpy().view(RESULT64_DTYPE)
        ms_gjk, r_gjk = _time_queries(torch, ctx, d_pairs, n, FCLG_REQ_NO_EPA, reps, 3, stream, dev)
        ms_full, _ = _time_queries(torch, ctx, d_pairs, n, 0, reps, 3, stream, dev)
        sep = (r64["ok"] == 1) & ((r64["status"] & 0xFF) == GJK_SEPARATED) & (r_gjk["ok"] == 1)
        err = np.abs(r_gjk["distance"][sep].astype(np.float64) - r64["distance"][sep])
        out["pairs_%d" % n] = {
            "fp64_ms": ms64, "fp64_queries_per_s": n / (ms64 * 1e-3),
            "fp32_gjk_distance_ms": ms_gjk, "fp32_gjk_distance_queries_per_s": n / (ms_gjk * 1e-3),
            "fp32_signed_distance_ms": ms_full, "fp32_signed_distance_queries_per_s": n / (ms_full * 1e-3),
            "fp32_over_fp64_gjk_speedup": ms64 / ms_gjk,
            "separated_pairs": int(sep.sum()),
            "fp32_vs_fp64_distance_err_max": float(err.max(initial=0.0)),
            "fp32_vs_fp64_distance_err_p99": float(np.percentile(err, 99)) if err.size else 0.0,
        }
        ctx.close()
    return out


WARM_CASES = {
    # name: (training batch on held-out seeds, test batch, embedding classes)
    "mixed": (lambda w: w.mixed(2_000_000, seed=w.SEED_BASE + 1001), lambda w, a: w.mixed(a.pairs),
              lambda w: w.MIXED_CLASSES),
    "arm": (lambda w: w.arm(9000, seed=w.SEED_BASE + 1003), lambda w, a: w.arm(a.configs), lambda w: w.ARM_CLASSES),
    "pareto": (lambda w: w.pareto(2_000_000, seed=w.SEED_BASE + 1004), lambda w, a: w.pareto(),
               lambda w: w.PARETO_CLASSES),
}


def warm_start_block(args, torch, dev, stream, local, names):
    """Learned warm start against plain initialisation: the model is trained on
    the GPU on plain-GJK directions of held-out seeds, then both runs are timed
    on the test batch (same pairs, same device entry point, each side on the
    launch shape the autotuner picks for its request)."""
    from fclg import workloads
    from fclg.api import Context, WarmStart, direction_labels
    peak, peak_kind = bf16_peak()
    out = {}
    for name in names:
        mk_train, mk_test, mk_classes = WARM_CASES[name]
        make_train = lambda: mk_train(workloads)
        make_test = lambda: mk_test(workloads, args)
        n_classes = mk_classes(workloads)
        ctx = Context(local)
        train = make_train()
        ctx.set_batch(train)
        d_tr = _to_dev(torch, train.pairs, dev)
        _, res = _time_queries(torch, ctx, d_tr, train.n_pairs, 0, 1, 0, stream, dev)
        labels, ok = direction_labels(res)
        keep = np.nonzero(ok)[0]
        d_tr = _to_dev(torch, train.pairs[keep], dev)
        d_lab = torch.from_numpy(labels[keep]).to(dev)
        ws = WarmStart(n_classes, seed=1, device=local)
        t0 = time.perf_counter()
        losses = ws.train(d_tr.data_ptr(), d_lab.data_ptr(), len(keep), epochs=8, batch=4096, lr=2e-3)
        train_s = time.perf_counter() - t0
        del d_tr, d_lab
        test = make_test()
        ctx.set_batch(test)
        ctx.set_warmstart(ws)
        n = test.n_pairs
        d_te = _to_dev(torch, test.pairs, dev)
        d_tmp = torch.empty(n * 48, dtype=torch.uint8, device=dev)
        # each side on its own autotuned launch shape
        from fclg.api import make_request
        tuning_p, _ = ctx.autotune(d_te.data_ptr(), n, d_tmp.data_ptr())
        ms_p, rp = _time_queries(torch, ctx, d_te, n, 0, args.steps, args.warmup, stream, dev)
        tuning_w, _ = ctx.autotune(d_te.data_ptr(), n, d_tmp.data_ptr(), request=make_request(flags=4))
        ms_w, rw = _time_queries(torch, ctx, d_te, n, 4, args.steps, args.warmup, stream, dev)
        tuning = {"plain": tuning_p, "warm": tuning_w}
        # per-pass device times of both requests (events on the launch stream)
        pass_ms = {}
        for side, flags, tune in (("plain", 0, tuning_p), ("warm", 4, tuning_w)):
            ctx.set_tuning(**tune)
            ctx.set_profiling(True)
            ctx.pass_times(reset=True)
            _time_queries(torch, ctx, d_te, n, flags, 3, 1, stream, dev)
            g_ms, e_ms, nq = ctx.pass_times(reset=True)
            ctx.set_profiling(False)
            pass_ms[side] = {"gjk_pass_ms": g_ms / max(nq, 1), "epa_pass_ms": e_ms / max(nq, 1)}
        del d_tmp
        # the tcgen05 inference kernel alone
        d_g = torch.empty(n * 3, dtype=torch.float32, device=dev)
        for _ in range(2):
            ws.predict(d_te.data_ptr(), n, d_g.data_ptr(), stream=stream.cuda_stream)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            ws.predict(d_te.data_ptr(), n, d_g.data_ptr(), stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ws.status()
        ms_mlp = e0.elapsed_time(e1) / args.steps
        guess = d_g.cpu().numpy().reshape(-1, 3)
        lt, okt = direction_labels(rp)
        ang = np.degrees(np.arccos(np.clip(np.sum(guess * lt, axis=1), -1.0, 1.0)))[okt]
        dp, dw = rp["distance"].astype(np.float64), rw["distance"].astype(np.float64)
        sep = (dp > 0) & (rp["ok"] == 1)
        err = np.abs(dp - dw)[sep]
        band = np.abs(dp) > 1e-6
        # both answers against the exact distance: the FP64 oracle run to a
        # 1e-12 tolerance on an evenly spaced subsample
        import oracle
        oracle.build()
        sub = np.arange(0, n, max(1, n // 20000))
        exact = oracle.signed_distance(test.subset(sub), gjk_max_iter=1000, gjk_tol=1e-12)
        both = sep[sub] & (exact["ok"] == 1) & (exact["distance"] > 0)
        ex = exact["distance"][both]
        e_w = np.abs(dw[sub][both] - ex)
        e_p = np.abs(dp[sub][both] - ex)
        tflops = MLP_FLOP_PER_PAIR * n / (ms_mlp * 1e-3) / 1e12
        out[name] = {
            "pairs": n, "train_samples": int(len(keep)), "train_epochs": 8, "train_s": round(train_s, 3),
            "train_loss": [round(float(x), 5) for x in (losses[0], losses[-1])],
            "plain": n / (ms_p * 1e-3), "warm": n / (ms_w * 1e-3), "speedup": ms_p / ms_w,
            "plain_ms": ms_p, "warm_ms": ms_w,
            "gjk_iters_separated": [float(rp["iterations"][sep].mean()), float(rw["iterations"][sep].mean())],
            "direction_error_deg_median": float(np.median(ang)),
            "flag_mismatches_outside_band": int(np.sum(((dp < 0) != (dw < 0)) & band)),
            "separation_diff_p99_5": float(np.percentile(err, 99.5)) if len(err) else 0.0,
            "separation_diff_max": float(err.max()) if len(err) else 0.0,
            "separation_err_vs_exact": {
                "pairs": int(both.sum()),
                "warm_max": float(e_w.max()) if len(e_w) else 0.0,
                "plain_max": float(e_p.max()) if len(e_p) else 0.0,
                "warm_over_1e-5": int(np.sum(e_w > 1e-5)), "plain_over_1e-5": int(np.sum(e_p > 1e-5)),
                "exact": "FP64 oracle, GJK tolerance 1e-12, 1000 iterations"},
            "overlap_bit_identical": bool(np.array_equal(dp[dp < 0], dw[dp < 0])),
            "pass_ms": pass_ms,
            "mlp_kernel": "tcgen05 (TMEM accumulators, bulk-async weight staging)", "mlp_ms": ms_mlp,
            "mlp_tflops": tflops, "mlp_frac": tflops / peak, "mlp_peak_source": peak_kind,
            "tuning": tuning,
        }
        ctx.close()
        ws.close()
    return out


def cpu_baseline(batch, threads):
    """The reference CPU path (FP64 restatement) on a bounded sample, all host
    threads; hulls above 32 vertices use the reference's hill-climbing support
    over qhull face lists, as fcl::Convex does (tables built outside the clock)."""
    import oracle
    oracle.build()
    sample = batch.subset(np.arange(min(CPU_SAMPLE_PAIRS, batch.n_pairs)))
    walk = oracle.walk_tables(sample)
    warm = sample.subset(np.arange(min(2000, sample.n_pairs)))
    oracle.signed_distance(warm, threads=threads, walk=oracle.walk_tables(warm))  # warm the code path
    # repeat the sample until about CPU_SAMPLE_SECONDS of CPU work are timed
    done, secs = 0, 0.0
    while secs < CPU_SAMPLE_SECONDS and done < 100_000_000:
        s, _ = oracle.time_signed_distance(sample, threads=threads, walk=walk)
        secs += s
        done += sample.n_pairs
    return done / secs, done, secs


def run_reference(args):
    """The reference's CPU path on the same 1M-pair batch, every step the whole
    batch: GJKSolver::shapeSignedDistance in the FP64 restatement (bit-identical
    to the reference compiled from its sources, tests/test_oracle.py) on all
    host threads, hulls above 32 vertices walking their edge graphs as
    fcl::Convex does (tables built outside the clock, as fcl::Convex builds
    them at construction)."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    from fclg import workloads
    batch = workloads.mixed(args.pairs)
    threads = os.cpu_count() or 1
    import oracle
    oracle.build()
    walk = oracle.walk_tables(batch)
    warm = batch.subset(np.arange(min(20000, batch.n_pairs)))
    warm_walk = oracle.walk_tables(warm)
    for _ in range(max(args.warmup, 1)):
        oracle.time_signed_distance(warm, threads=threads, walk=warm_walk)
    total = 0.0
    for _ in range(args.steps):
        secs, _ = oracle.time_signed_distance(batch, threads=threads, walk=walk)
        total += secs
    value = batch.n_pairs * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "pairs_per_gpu": batch.n_pairs, "seed": batch.meta["seed"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "the whole %d-pair mixed batch every step (warm-up steps on its first %d "
                                   "pairs); hulls above 32 vertices hill-climb their edge graphs as fcl::Convex "
                                   "does" % (batch.n_pairs, warm.n_pairs)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


MESH_WORKLOAD = ("mesh-mesh BVH: two geodesic spheres of 50,000 triangles (radius 0.3 m, per-vertex radial "
                 "noise N(0, 0.05 m)), OBB hierarchies built on the host, 65,536 poses (translation uniform in "
                 "a 0.8 m ball, uniform rotation); boolean collide, first-contact and 64-contact modes")


def l2_copy_peak(torch, dev, stream):
    """Copy bandwidth of a working set that stays in L2 (16 MB read + 16 MB
    written, best of 50 back-to-back copies, CUDA events): the L2 analogue of
    the HBM copy peak, measured here because no L2 figure is recorded."""
    a = torch.empty(16 << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    for _ in range(10):
        b.copy_(a)
    torch.cuda.synchronize(dev)
    best = float("inf")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(50):
        e0.record(stream)
        b.copy_(a)
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2 * a.numel() / (best * 1e-3) / 1e9


def mesh_block(args, torch, dev, stream, local):
    """BVH collides/s on the mesh-mesh workload, first-contact and 64-contact
    modes: device-resident (events on the launch stream), end to end through
    the host entry point, an L2 roofline from the kernel's own work counters
    and the CPU baseline (the reference's traversal restated in FP64 over the
    reference's own tree, all host threads)."""
    from fclg import workloads
    from fclg.api import Context, GpuMesh, mesh_collide
    import ctypes
    ma, mb = workloads.mesh_pair()
    poses = workloads.mesh_poses(args.poses)
    ctx = Context(local)
    ga, gb = GpuMesh(ctx, ma.vertices, ma.triangles), GpuMesh(ctx, mb.vertices, mb.triangles)
    n = len(poses)
    d_poses = torch.from_numpy(poses).to(dev)
    l2_peak = l2_copy_peak(torch, dev, stream)
    out = {}
    for cap in (1, 64):
        d_flags = torch.empty(n, dtype=torch.uint8, device=dev)
        d_counts = torch.empty(n, dtype=torch.int32, device=dev)
        d_pairs = torch.empty(n * cap * 2, dtype=torch.int32, device=dev)
        d_status = torch.empty(n, dtype=torch.int32, device=dev)

        def step():
            rc = ctx.lib.fclg_mesh_collide_device(ctx.h, ga.h, gb.h, ctypes.c_void_p(d_poses.data_ptr()), n, cap,
                                                  ctypes.c_void_p(d_flags.data_ptr()),
                                                  ctypes.c_void_p(d_counts.data_ptr()),
                                                  ctypes.c_void_p(d_pairs.data_ptr()),
                                                  ctypes.c_void_p(d_status.data_ptr()),
                                                  ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0
        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize(dev)
        launches0 = ctx.launch_count
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.steps
        launches = ctx.launch_count - launches0
        flags = d_flags.cpu().numpy()
        status = d_status.cpu().numpy()
        # the kernel's work for the roofline: one profiled step
        ctx.set_profiling(True)
        ctx.mesh_traffic(reset=True)
        step()
        node_pairs, tri_pairs = ctx.mesh_traffic(reset=True)
        ctx.set_profiling(False)
        algo = node_pairs * 128 + tri_pairs * 96
        achieved = algo / (ms * 1e-3) / 1e9
        # end to end through the host entry point
        for _ in range(2):
            mesh_collide(ctx, ga, gb, poses, max_contacts=cap)
        t0 = time.perf_counter()
        reps = max(1, args.steps // 2)
        for _ in range(reps):
            mesh_collide(ctx, ga, gb, poses, max_contacts=cap)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
        out[cap] = {"value": n / (ms * 1e-3), "ms_per_step": ms, "collide_fraction": float(flags.mean()),
                    "mean_contacts": float(d_counts.float().mean().item()), "incomplete": int(np.sum(status != 0)),
                    "gpu_launches": launches,
                    "e2e": {"value": n / (e2e_ms * 1e-3), "unit": "BVH collides/s", "h2d_bytes_per_step": n * 48,
                            "d2h_bytes_per_step": n * (1 + 4 + cap * 8 + 4)},
                    "roofline": {"bound": "l2", "achieved": achieved, "peak": l2_peak, "unit": "GB/s",
                                 "frac": achieved / l2_peak, "traffic": None,
                                 "algorithmic_bytes": "%d node pairs x 128 B + %d triangle pairs x 96 B per launch"
                                                      % (node_pairs, tri_pairs),
                                 "peak_source": "L2-resident copy (16 MB + 16 MB) measured by bench.py"}}
    # CPU baseline: the reference's traversal restated over the reference's own tree
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    A = (ma.vertices.astype(np.float64), ma.triangles)
    B = (mb.vertices.astype(np.float64), mb.triangles)
    sample = poses[:8192].astype(np.float64)
    oracle.orc_mesh_collide_ref(A, B, sample[:256], 1, threads=threads)
    t0 = time.perf_counter()
    oracle.orc_mesh_collide_ref(A, B, sample, 1, threads=threads)
    cpu_s = time.perf_counter() - t0
    ga.close()
    gb.close()
    ctx.close()
    return {"workload": MESH_WORKLOAD, "poses": n, "unit": "BVH collides/s", "first_contact": out[1],
            "contacts_64": out[64],
            "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "BVH collides/s", "cores": threads,
                             "kind": "port",
                             "sample": "first %d poses, first-contact mode, the reference's MeshIntersect restated "
                                       "in FP64 over its own OBBRSS trees (tree build outside the clock)"
                                       % len(sample)}}


def run_mesh(args):
    """BVH collides/s on the mesh-mesh workload (its own JSON line)."""
    import torch
    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    with ClockSampler(local) as clk:
        m = mesh_block(args, torch, dev, stream, local)
    fc = m["first_contact"]
    line = {"metric": METRIC, "value": fc["value"], "unit": "BVH collides/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": fc["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (FP64 triangle fallback)", "data": "synthetic",
            "config": {"workload": m["workload"], "poses": m["poses"], "first_contact": fc,
                       "contacts_64": m["contacts_64"]},
            "gpu_launches": fc["gpu_launches"], "roofline": fc["roofline"], "cpu_baseline": m["cpu_baseline"],
            "e2e": fc["e2e"], "clocks": clk.summary()}
    print(json.dumps(line))
    return 0


MESH_SHAPE_WORKLOAD = ("mesh-shape BVH: the first geodesic sphere of the mesh-mesh workload (50,000 triangles) "
                       "against 65,536 queries of 2,048 mixed shapes (sphere / box / capsule / cylinder / hull, "
                       "sizes U[0.02, 0.4] m, hulls of log-uniform[8, 256] points), poses as the mesh-mesh "
                       "workload's; fcl::collide(mesh, shape) with penetration off")


def run_mesh_shape(args):
    """Mesh-shape collides/s (fcl::collide(BVHModel, shape), its own JSON line)."""
    import torch
    from fclg import workloads
    from fclg.api import Context, GpuMesh, mesh_shape_collide, mesh_shape_contacts
    import ctypes
    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    mesh, _ = workloads.mesh_pair()
    shapes = workloads.mixed(1024, seed=workloads.SEED_BASE + 61)
    poses = workloads.mesh_poses(args.poses)
    n = len(poses)
    ids = (np.arange(n) % len(shapes.shapes)).astype(np.uint32)
    ctx = Context(local)
    ctx.set_batch(shapes)
    gm = GpuMesh(ctx, mesh.vertices, mesh.triangles)
    stream = torch.cuda.current_stream(dev)
    d_poses = torch.from_numpy(poses).to(dev)
    d_ids = torch.from_numpy(ids.view(np.int32)).to(dev)
    out = {}
    for key, cap, pen in ((1, 1, False), (64, 64, False), ("contacts", 1, True)):
        d_flags = torch.empty(n, dtype=torch.uint8, device=dev)
        d_counts = torch.empty(n, dtype=torch.int32, device=dev)
        d_tris = torch.empty(n * cap, dtype=torch.int32, device=dev)
        d_status = torch.empty(n, dtype=torch.int32, device=dev)
        d_con = torch.empty(n * cap * 8, dtype=torch.float32, device=dev)

        def step():
            vp = ctypes.c_void_p
            common = (ctx.h, gm.h, vp(d_ids.data_ptr()), vp(d_poses.data_ptr()), n, cap, vp(d_flags.data_ptr()),
                      vp(d_counts.data_ptr()), vp(d_tris.data_ptr()))
            if pen:
                rc = ctx.lib.fclg_mesh_shape_contacts_device(*common, vp(d_con.data_ptr()), vp(d_status.data_ptr()),
                                                             vp(stream.cuda_stream))
            else:
                rc = ctx.lib.fclg_mesh_shape_collide_device(*common, vp(d_status.data_ptr()), vp(stream.cuda_stream))
            assert rc == 0
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = ctx.launch_count
        with ClockSampler(local) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                step()
            e1.record(stream)
            torch.cuda.synchronize(dev)
        launches = ctx.launch_count - launches0
        ms = e0.elapsed_time(e1) / args.steps
        flags = d_flags.cpu().numpy()
        status = d_status.cpu().numpy()
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 2)):
            if pen:
                mesh_shape_contacts(ctx, gm, ids, poses, max_contacts=cap)
            else:
                mesh_shape_collide(ctx, gm, ids, poses, max_contacts=cap)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / max(1, args.steps // 2)
        out[key] = {"value": n / (ms * 1e-3), "ms_per_step": ms, "collide_fraction": float(flags.mean()),
                    "incomplete": int(np.sum(status != 0)), "e2e": n / (e2e_ms * 1e-3),
                    "gpu_launches": launches, "clocks": clk.summary()}
    import oracle
    oracle.build()
    nodes, tris = gm.export()
    sample = min(2048, n)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.mesh_shape_collide(nodes, tris, shapes, ids[:sample], poses[:sample], max_contacts=1, threads=threads)
    cpu_s = time.perf_counter() - t0
    line = {"metric": "mesh-shape collides/s (fcl::collide on BVHModel<OBBRSS> x shape)", "value": out[1]["value"],
            "unit": "mesh-shape collides/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out[1]["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (FP64 re-decision for sphere / box leaves)", "data": "synthetic",
            "config": {"workload": MESH_SHAPE_WORKLOAD, "queries": n, "first_contact": out[1],
                       "contacts_64": out[64], "first_contact_with_penetration": out["contacts"]},
            "gpu_launches": out[1]["gpu_launches"], "clocks": out[1]["clocks"],
            "cpu_baseline": {"value": sample / cpu_s, "unit": "mesh-shape collides/s", "cores": threads,
                             "kind": "port", "sample": "first %d queries, first-contact mode" % sample},
            "e2e": {"value": out[1]["e2e"], "unit": "mesh-shape collides/s", "h2d_bytes_per_step": n * 52,
                    "d2h_bytes_per_step": n * (1 + 4 + 4 + 4)}}
    print(json.dumps(line))
    gm.close()
    ctx.close()
    return 0


CCD_WORKLOAD = ("translational CCD: 1M pairs of the mixed workload's kinds and sizes (sphere / box / capsule / "
                "cylinder / hull of log-uniform[8, 256] points), start separations up to 3x the bounding-sphere "
                "sum, shape a moving along a uniform unit axis by up to 2x that sum; one time-of-collision sample "
                "per hit (kOneTocSample)")
# compulsory bytes per CCD query: the mixed workload's hull / parameter / pose
# bytes, the 16 B displacement and a 16 B result record
CCD_ALGO_BYTES = 466.0


def run_ccd(args):
    """Translational CCD pair queries/s (fcl::translational_ccd, its own JSON line)."""
    import torch
    from fclg import workloads
    from fclg.api import Context, FCLG_TOC_SAMPLE
    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    b, disp = workloads.ccd(args.pairs, seed=workloads.SEED_BASE + 9 + 1000 * rank)
    n = b.n_pairs
    ctx = Context(local)
    ctx.set_batch(b)
    if args.tuning:
        ctx.set_tuning(**{k: int(v) for k, v in json.loads(args.tuning).items()})
    stream = torch.cuda.current_stream(dev)
    d_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).to(dev)
    d_disp = torch.from_numpy(disp).to(dev)
    d_res = torch.empty(n * 16, dtype=torch.uint8, device=dev)

    def step():
        ctx.translational_ccd_device(d_pairs.data_ptr(), n, d_disp.data_ptr(), d_res.data_ptr(),
                                     toc_type=FCLG_TOC_SAMPLE, stream=stream.cuda_stream)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launch_count
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
    launches = ctx.launch_count - launches0
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(torch, e0.elapsed_time(e1) / args.steps, dev, world)
    res = d_res.cpu().numpy().view(np.uint32).reshape(n, 4)
    hit = float(np.mean(res[:, 0] == 1))
    # end to end: pinned host arrays through fclg_translational_ccd (copies inside)
    from fclg.api import CCD_RESULT_DTYPE
    from fclg.layout import PAIR_DTYPE
    h_pairs = torch.from_numpy(b.pairs.view(np.uint8).copy()).pin_memory().numpy().view(PAIR_DTYPE)
    h_disp = torch.from_numpy(disp.copy()).pin_memory().numpy()
    h_out = torch.zeros(n * CCD_RESULT_DTYPE.itemsize, dtype=torch.uint8).pin_memory().numpy().view(CCD_RESULT_DTYPE)
    ctx.translational_ccd(h_pairs, h_disp, toc_type=FCLG_TOC_SAMPLE, out=h_out)
    t0 = time.perf_counter()
    e2e_steps = max(1, args.steps // 2)
    for _ in range(e2e_steps):
        ctx.translational_ccd(h_pairs, h_disp, toc_type=FCLG_TOC_SAMPLE, out=h_out)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    hbm, src = peaks()
    achieved = n * CCD_ALGO_BYTES / (ms * 1e-3) / 1e9
    line = {"metric": "translational CCD pair queries/s (fcl::translational_ccd, one toc sample)",
            "value": world * n / (ms * 1e-3), "unit": "pair queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (box intervals f64)", "data": "synthetic",
            "config": {"workload": CCD_WORKLOAD, "pairs_per_gpu": n, "hit_fraction": hit,
                       "l2": "inputs larger than L2 (no flush)", "tuning": ctx.get_tuning()},
            "gpu_launches": launches, "clocks": clk.summary(),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_source": src,
                         "kernel": "ccd_pass (swept-volume MPR, latency-bound)"},
            "e2e": {"value": world * n / (e2e_ms * 1e-3), "unit": "pair queries/s",
                    "h2d_bytes_per_step": n * (64 + 16), "d2h_bytes_per_step": n * 16}}
    if rank == 0:
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        sample = min(n, 200_000)
        sb = workloads.Batch("ccd_sample", b.shapes, b.vertices, b.pairs[:sample], {})
        reps, t0 = 0, time.perf_counter()
        while True:
            oracle.translational_ccd(sb, disp[:sample], oracle.TOC_SAMPLE, threads=threads)
            reps += 1
            if time.perf_counter() - t0 > 5.0:
                break
        cpu = reps * sample / (time.perf_counter() - t0)
        line["cpu_baseline"] = {"value": cpu, "unit": "pair queries/s", "cores": threads, "kind": "port",
                                "sample": "first %d pairs, repeated for >= 5 s" % sample}
        print(json.dumps(line))
    ctx.close()
    return 0


SCENE_WORKLOAD = ("scene: 100,000 posed objects (sphere / box / capsule / cylinder / hull, sizes U[0.02, 0.4] m, "
                  "hulls of log-uniform[8, 256] points; uniform rotations, 20 % identity) in a cube at 0.25 "
                  "objects per bounding-sphere volume; per step the broadphase (CollisionObject AABBs, every "
                  "overlapping pair), the candidates' narrowphase records and the signed distance of every "
                  "candidate")


def run_scene(args):
    """Scene objects/s through broadphase + narrowphase (its own JSON line)."""
    import torch
    import ctypes
    from fclg import workloads
    from fclg.api import Context
    from fclg.layout import PAIR_DTYPE
    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    b, ids, poses = workloads.scene(args.objects)
    n = len(ids)
    ctx = Context(local)
    ctx.set_batch(b)
    stream = torch.cuda.current_stream(dev)
    vp = ctypes.c_void_p
    d_ids = torch.from_numpy(ids.view(np.int32)).to(dev)
    d_poses = torch.from_numpy(poses).to(dev)
    cap = 16 * n
    d_cand = torch.empty(2 * cap, dtype=torch.int32, device=dev)
    d_cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    d_rec = torch.empty(cap * PAIR_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    d_res = torch.empty(cap * 48, dtype=torch.uint8, device=dev)
    h_cnt = torch.zeros(1, dtype=torch.int32).pin_memory()

    def step():
        assert ctx.lib.fclg_broadphase_device(ctx.h, vp(d_ids.data_ptr()), vp(d_poses.data_ptr()), n,
                                              vp(d_cand.data_ptr()), cap, vp(d_cnt.data_ptr()), None, None,
                                              vp(stream.cuda_stream)) == 0
        h_cnt.copy_(d_cnt, non_blocking=True)
        stream.synchronize()
        m = min(int(h_cnt.item()), cap)
        assert ctx.lib.fclg_object_pairs_device(ctx.h, vp(d_ids.data_ptr()), vp(d_poses.data_ptr()),
                                                vp(d_cand.data_ptr()), m, vp(d_rec.data_ptr()),
                                                vp(stream.cuda_stream)) == 0
        ctx.distance_device(d_rec.data_ptr(), m, d_res.data_ptr(), None, stream.cuda_stream)
        return m

    for _ in range(args.warmup):
        m = step()
    torch.cuda.synchronize(dev)
    # broadphase alone
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ctx.lib.fclg_broadphase_device(ctx.h, vp(d_ids.data_ptr()), vp(d_poses.data_ptr()), n,
                                       vp(d_cand.data_ptr()), cap, vp(d_cnt.data_ptr()), None, None,
                                       vp(stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize(dev)
    bp_ms = e0.elapsed_time(e1) / args.steps
    launches0 = ctx.launch_count
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(args.steps):
            m = step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / args.steps
    launches = ctx.launch_count - launches0
    # CPU baseline: FP64 AABBs, sort-and-sweep, signed distance of the candidates
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    boxes = oracle.object_aabbs(b, ids, poses)
    cand = oracle.sweep_pairs(boxes)
    rec = np.zeros(len(cand), PAIR_DTYPE)
    P = poses.astype(np.float64)
    Ri, Rj = P[cand[:, 0], :9].reshape(-1, 3, 3), P[cand[:, 1], :9].reshape(-1, 3, 3)
    rec["shape_a"], rec["shape_b"] = ids[cand[:, 0]], ids[cand[:, 1]]
    rec["rot"] = np.einsum("nki,nkj->nij", Ri, Rj).reshape(-1, 9)
    rec["trans"] = np.einsum("nki,nk->ni", Ri, P[cand[:, 1], 9:] - P[cand[:, 0], 9:])
    q = workloads.Batch("scene_pairs", b.shapes, b.vertices, rec, {})
    cpu_bp = time.perf_counter() - t0
    walk = oracle.walk_tables(q)
    cpu_np, _ = oracle.time_signed_distance(q, threads=threads, walk=walk)
    cpu_s = cpu_bp + cpu_np
    line = {"metric": "scene objects/s (broadphase + narrowphase signed distance)", "value": n / (ms * 1e-3),
            "unit": "scene objects/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": SCENE_WORKLOAD, "objects": n, "candidate_pairs": m, "broadphase_ms": bp_ms,
                       "candidate_pairs_per_s": m / (ms * 1e-3)},
            "gpu_launches": launches, "clocks": clk.summary(),
            "cpu_baseline": {"value": n / cpu_s, "unit": "scene objects/s", "cores": threads, "kind": "port",
                             "sample": "the whole scene once: FP64 AABBs and sort-and-sweep on one thread "
                                       "(%.2f s), candidates' signed distance on all threads (%.2f s)"
                                       % (cpu_bp, cpu_np)},
            "e2e": {"value": n / (ms * 1e-3), "unit": "scene objects/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 4, "note": "device-resident scene; one 4-byte count read per step"}}
    print(json.dumps(line))
    ctx.close()
    return 0


def run_warmstart_kernel(args):
    """The warm-start inference kernels alone (tcgen05 and mma.sync) on the arm
    workload's 2.24M pairs, untrained weights (the cost does not depend on them)."""
    import torch
    from fclg import workloads
    from fclg.api import WarmStart
    rank, world, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    b = workloads.arm(10000)
    n = b.n_pairs
    ws = WarmStart(workloads.ARM_CLASSES, seed=1, device=local)
    d_pairs = _to_dev(torch, b.pairs, dev)
    d_out = torch.empty(n * 3, dtype=torch.float32, device=dev)
    peak, peak_kind = bf16_peak()
    res = {}
    for kind in ("tcgen05", "mma.sync"):
        for _ in range(args.warmup):
            ws.predict(d_pairs.data_ptr(), n, d_out.data_ptr(), mma_sync=kind == "mma.sync", stream=stream.cuda_stream)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            ws.predict(d_pairs.data_ptr(), n, d_out.data_ptr(), mma_sync=kind == "mma.sync", stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ws.status()
        ms = e0.elapsed_time(e1) / args.steps
        res[kind] = {"ms": ms, "tflops": MLP_FLOP_PER_PAIR * n / (ms * 1e-3) / 1e12}
    t = res["tcgen05"]["tflops"]
    line = {"metric": "warm-start MLP inference (28-256-256-256-3, BF16, FP32 accumulate)",
            "value": n / (res["tcgen05"]["ms"] * 1e-3), "unit": "pair directions/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["tcgen05"]["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "arm pairs (22.4M / 10)", "pairs": n, "kernels": res},
            "roofline": {"bound": "tensor", "achieved": t, "peak": peak, "unit": "TFLOP/s", "frac": t / peak,
                         "traffic": None, "kernel": "infer_tc_kernel", "peak_source": peak_kind}}
    print(json.dumps(line))
    ws.close()
    return 0


def rank_batch(workloads, workload, rank, pairs=N_PAIRS, configs=100_000):
    """This rank's batch: every rank draws its own seeded batch of the same
    shape (weak scaling; pairs are independent, nothing is exchanged)."""
    if workload == "mixed":
        return workloads.mixed(pairs, seed=workloads.SEED_BASE + 1 + rank)
    if workload == "arm":
        return workloads.arm(configs, seed=workloads.SEED_BASE + 3 + 100 * rank)
    if workload == "pareto":
        return workloads.pareto(seed=workloads.SEED_BASE + 4 + 100 * rank)
    return workloads.plain_small(seed=workloads.SEED_BASE + 0 + 100 * rank)


def max_over_ranks(torch, ms, dev, world):
    """The slowest rank's time (every rank returns the same value)."""
    if world <= 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(n_per_rank, world, ms):
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return n_per_rank * world / (ms * 1e-3)


SWEEP_LAYOUTS = [(1, 1, 128), (1, 4, 128), (1, 2, 128), (1, 1, 256), (2, 4, 128), (4, 8, 128)]


def launch_sweep(args, torch, ctx, step, stream, n, t_set):
    """Mean device time of one query per launch layout (GJK lanes for small /
    large hulls, hull split) with the refilling one-lane GJK pass on and off
    and the support walk on and off."""
    rows = []
    for walk, refill in ((False, True), (False, False), (True, True)):
        for ls, ll, lh in SWEEP_LAYOUTS:
            ctx.set_tuning(bucketing=True, gjk_lanes_small=ls, gjk_lanes_large=ll, large_hull_vertices=lh,
                           support_walk=walk, gjk_refill=refill)
            for _ in range(2):
                step()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(5):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
            rows.append({"walk": walk, "refill": refill, "lanes_small": ls, "lanes_large": ll, "large_hull": lh,
                         "ms": e0.elapsed_time(e1) / 5})
    print(json.dumps({"sweep": args.workload, "pairs": n, "set_shapes_s": t_set, "rows": rows}))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "mesh":
        return run_mesh(args)
    if args.workload == "mesh_shape":
        return run_mesh_shape(args)
    if args.workload == "scene":
        return run_scene(args)
    if args.workload == "ccd":
        return run_ccd(args)
    if args.workload == "warmstart":
        return run_warmstart_kernel(args)
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    from fclg import workloads
    from fclg.api import Context
    gen, algo_bytes, workload_text = CONVEX_WORKLOADS[args.workload]
    batch = rank_batch(workloads, args.workload, rank, args.pairs, args.configs)
    n = batch.n_pairs
    ctx = Context(local)
    t_set = time.perf_counter()
    ctx.set_batch(batch)
    t_set = time.perf_counter() - t_set
    stream = torch.cuda.current_stream(dev)
    d_pairs = torch.from_numpy(batch.pairs.view(np.uint8).copy()).to(dev)
    d_res = torch.empty(n * 48, dtype=torch.uint8, device=dev)

    def step():
        ctx.distance_device(d_pairs.data_ptr(), n, d_res.data_ptr(), None, stream.cuda_stream)

    if args.sweep:
        return launch_sweep(args, torch, ctx, step, stream, n, t_set)

    # launch shape chosen by the library's autotuner on this batch (untimed), or given
    if args.tuning:
        fixed = {k: (int(v) if not isinstance(v, bool) else v) for k, v in json.loads(args.tuning).items()}
        ctx.set_tuning(**fixed)
        tuning, tune_ms = ctx.get_tuning(), 0.0
    else:
        tuning, tune_ms = ctx.autotune(d_pairs.data_ptr(), n, d_res.data_ptr())

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    # ---- device-resident throughput (value)
    in_bytes = batch.pairs.nbytes + batch.shapes.nbytes + batch.vertices.nbytes + n * 48
    flush = None
    if in_bytes < 256 << 20:
        # inputs within twice the 129 MB L2: flush it before every timed step
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        l2_note = "L2 flushed (512 MB write) before each timed step, outside the step's events"
    else:
        l2_note = "inputs larger than L2 (no flush)"
    for _ in range(args.warmup):
        step()
    barrier()
    launches0 = ctx.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if flush is None:
            e0.record(stream)
            for _ in range(args.steps):
                step()
            e1.record(stream)
            barrier()
            ms = e0.elapsed_time(e1) / args.steps
        else:
            total = 0.0
            for _ in range(args.steps):
                flush.zero_()
                e0.record(stream)
                step()
                e1.record(stream)
                e1.synchronize()
                total += e0.elapsed_time(e1)
            barrier()
            ms = total / args.steps
    launches = ctx.launch_count - launches0
    ms = max_over_ranks(torch, ms, dev, world)
    value = job_value(n, world, ms)
    graph_ms = None
    if world == 1:
        # the same query replayed as one CUDA graph (small batches are launch-bound)
        g = ctx.graph(d_pairs.data_ptr(), n, d_res.data_ptr())
        g.launch(stream.cuda_stream)
        torch.cuda.synchronize(dev)
        total = 0.0
        for _ in range(args.steps):
            if flush is not None:
                flush.zero_()
            e0.record(stream)
            g.launch(stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1)
        graph_ms = total / args.steps
        g.close()

    # ---- per-pass kernel times for the roofline (same steps, events on the launch stream)
    ctx.set_profiling(True)
    ctx.pass_times(reset=True)
    for _ in range(max(3, args.steps // 2)):
        step()
    torch.cuda.synchronize(dev)
    gjk_ms, epa_ms, nq = ctx.pass_times(reset=True)
    ctx.set_profiling(False)
    gjk_ms /= max(nq, 1)
    epa_ms /= max(nq, 1)
    res = d_res.cpu().numpy().view(np.dtype([("distance", "<f4"), ("rest", "V44")]))
    overlap = float(np.mean(res["distance"] < 0))

    # ---- end to end through the host entry point, pinned buffers
    h_pairs = torch.from_numpy(batch.pairs.view(np.uint8).copy()).pin_memory()
    h_res = torch.empty(n * 48, dtype=torch.uint8).pin_memory()
    lib = ctx.lib
    import ctypes

    def e2e_step():
        rc = lib.fclg_distance(ctx.h, ctypes.c_void_p(h_pairs.data_ptr()), n, None, ctypes.c_void_p(h_res.data_ptr()))
        if rc != 0:
            raise RuntimeError("fclg_distance failed: %s" % lib.fclg_last_error(ctx.h).decode())

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_ms = max_over_ranks(torch, e2e_ms, dev, world)
    e2e_value = job_value(n, world, e2e_ms)

    if rank == 0:
        peak, peak_kind = peaks()
        dominant = "epa_pass" if epa_ms >= gjk_ms else "gjk_pass"
        # algorithmic bytes of the whole query per step over the dominant pass time and over the step
        achieved = algo_bytes * n / (max(gjk_ms, epa_ms) * 1e-3) / 1e9
        threads = os.cpu_count() or 1
        cpu_v, cpu_n, cpu_s = cpu_baseline(batch, threads)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 EPA closest-face solve and GJK tetrahedron tests)",
            "data": "synthetic",
            "config": {"workload": workload_text, "pairs_per_gpu": n, "overlap_fraction": overlap,
                       "seed": batch.meta["seed"], "l2": l2_note,
                       "gjk_pass_ms": gjk_ms, "epa_pass_ms": epa_ms,
                       "tuning": dict(tuning, autotune_ms=tune_ms),
                       "cuda_graph": (None if graph_ms is None else
                                      {"ms_per_step": graph_ms, "value": n / (graph_ms * 1e-3)})},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": (EPA_TRAFFIC_MIXED_1M if args.workload == "mixed" and n == 1_000_000
                                     and dominant == "epa_pass" else None),
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the three "
                                           "EPA launches at 400 k pairs scaled by the pairs to 10^6, "
                                           "profiles/epa_pass_mixed_400k.md",
                         "kernel": dominant + " (all launches of the pass)",
                         "peak_source": peak_kind,
                         "algorithmic_bytes": "%d B/query x %d queries per launch" % (algo_bytes, n)},
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "first %d pairs of the batch, repeated to %d queries, FP64 restatement "
                                       "(%.1f s); hulls above 32 vertices hill-climb their edge graphs as "
                                       "fcl::Convex does" % (min(CPU_SAMPLE_PAIRS, n), cpu_n, cpu_s)},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 64, "d2h_bytes_per_step": n * 48},
            "clocks": clk.summary(),
        }
        if not args.no_warm and args.workload in ("mixed", "arm", "pareto"):
            names = ["mixed", "arm"] if args.workload == "mixed" else [args.workload]
            line["config"]["warm_start"] = warm_start_block(args, torch, dev, stream, local, names)
        if not args.no_mesh and args.workload == "mixed" and world == 1:
            line["config"]["mesh"] = mesh_block(args, torch, dev, stream, local)
        if not args.no_fp64 and args.workload == "mixed" and world == 1:
            line["config"]["fp64_plain"] = fp64_block(args, torch, dev, stream, local)
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
