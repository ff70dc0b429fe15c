#!/usr/bin/env python
"""bench.py — batched ratio_match over a 240-view zone on one GB300.

Workload (the headline configuration): 3 cameras x 80 positions = 240 views,
n_v ~ U[300, 2000] SIFT-like descriptors per view, candidate_pairs(views, 5, 4,
16) = 3663 image pairs, overlapping pairs sharing 30-60 % of descriptors
(noisy copies, sigma 0.05). Seeded synthetic data (no dataset exists for it).

A step is one pass of the hot path over the zone: ratio_match(fa, fb, 0.8,
true) for every pair (crates/core/src/pipeline.rs:485-493, matching half) as
one planned batch replayed from a CUDA graph.

  value  image pairs/s with the descriptor store resident in HBM; device time
         of each step by CUDA events on the library stream; L2 flushed between
         steps outside the events.
  e2e    the same through the C ABI with host buffers: every step re-uploads
         all views from pinned host memory (slm_store_add_views), runs the
         batch and reads the match lists back (slm_plan_results); three
         contexts take the steps in turn, so one step's copies overlap the
         kernels of the two steps before it.
The match lists of the main arm are checked against the oracle (bit-exact) on
a sample of pairs before timing. `--impl reference` times the CPU restatement
of the reference (oracle/, all host threads) on a bounded sample.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "skylens-stream-rs_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

METRIC = "image pairs/s, batched ratio_match: BF16 shortlist vs FP32 GPU, bit-exact"
WORKLOAD = "zone240"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="slm", choices=["slm", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp32", "bf16", "fp8"])
    ap.add_argument("--positions", type=int, default=80)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--verify-pairs", type=int, default=400, help="pairs checked against the oracle (0: none, -1: all)")
    ap.add_argument("--fp32-steps", type=int, default=3, help="timed steps of the plain FP32 arm")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--scalar", action="store_true", help="FP32 kernel with all-scalar arithmetic")
    ap.add_argument("--json-out", default=None)
    ap.add_argument("--serve", action="store_true", help="serving workload (Poisson view arrivals)")
    ap.add_argument("--rates", default="10,50,200,burst",
                    help="serving arrival rates, views/s ('burst': every view at once, the saturated server)")
    ap.add_argument("--pairs", action="store_true", help="single-pair configurations (800, 8192, 32768 FP8)")
    ap.add_argument("--ransac", action="store_true", help="RANSAC hypothesis scoring (Sampson residuals)")
    ap.add_argument("--features", action="store_true", help="descriptor producer (detect_and_describe, 960 x 540)")
    ap.add_argument("--features-reps", type=int, default=5, help="timed calls per arm of --features")
    ap.add_argument("--no-scheduled", action="store_true",
                    help="skip the scheduled_pairs(PairSchedule::default()) batch with the < 20 filter")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations' sub-records (single pairs 800 / 8192 / 32768, serving)")
    ap.add_argument("--config-rates", default="50,burst", help="serving arrival rates in the default run's sub-record")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "25"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait for its first sample so the
        # samples cover the timed region
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0:
            self.f.flush()
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        loaded = [s for s in sm if mx and s >= 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def reduce_over_ranks(ms: float, units: int, dist, device=None):
    """Whole-job rate over replicas: every rank timed its own zone; the job time
    is the slowest rank's (MAX) and the work is the sum over ranks (SUM).
    Returns (max ms, total units, units per second)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return ms, units, units / (ms / 1e3)
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), int(u.item()), float(u.item()) / (float(t.item()) / 1e3)


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, \
        "fallback"


L2_NOTE = ("zone store 141 MB (raw f32) > 129 MB L2; the GPU arm also flushes L2 (512 MiB write) between steps, "
           "outside the timed events")
ORACLE_FLAGS = "gcc -O3 -std=c11 -ffp-contract=off -fno-fast-math -fPIC (portable: no -march/-mcpu=native)"


def workload_config(z, seed: int, ws: int = 1) -> dict:
    """The workload as both arms report it (the GPU arm's precision and tuned
    settings are top-level keys of its line)."""
    return {"workload": WORKLOAD, "views": len(z.counts), "pairs": int(len(z.pairs)), "distances": int(z.distances),
            "descriptors": int(z.counts.sum()), "ratio": 0.8, "mutual": True, "seed": seed, "l2": L2_NOTE,
            "parallelism": f"replicas{ws}"}


def cpu_baseline(z, budget_s: float, threads: int):
    """The oracle's blocked ratio_match (64-row blocks over `threads` host threads,
    pairs serial as in benches/pipeline.rs:247-253) on pairs in a fixed order until
    the time budget is used."""
    import oracle as O
    order = np.random.Generator(np.random.PCG64(123)).permutation(len(z.pairs))
    done, dist = 0, 0
    t0 = time.perf_counter()
    while done < len(order) and time.perf_counter() - t0 < budget_s:
        k = int(order[done])
        u, v = int(z.pairs[k, 0]), int(z.pairs[k, 1])
        O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=threads)
        dist += int(z.counts[u]) * int(z.counts[v])
        done += 1
    dt = time.perf_counter() - t0
    return done / dt, dist / dt, done, dt


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from skylens_match import synth
    z = synth.zone(positions=args.positions, seed=args.seed)
    threads = os.cpu_count() or 1
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_baseline(z, min(per_step, 1.0), threads)
    rates, drates, npairs = [], [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, dr, n, _dt = cpu_baseline(z, per_step, threads)
        rates.append(r)
        drates.append(dr)
        npairs.append(n)
    wall = time.perf_counter() - t0
    value = float(np.mean(rates))
    sample = {"pairs_per_step": int(np.mean(npairs)), "of_pairs": int(len(z.pairs)),
              "seconds_per_step": per_step,
              "order": "a fixed random permutation of the zone's pairs (PCG64 seed 123); each step starts at its "
                       "first pair and runs until the step's time budget is used"}
    line = {"metric": METRIC, "value": value, "unit": "image pairs/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": workload_config(z, args.seed, ws),
            "distances_per_s": float(np.mean(drates)),
            "cpu_baseline": {"value": value, "unit": "image pairs/s", "cores": threads, "kind": "port",
                             "sample": f"{int(np.mean(npairs))} of {len(z.pairs)} zone pairs per step",
                             "sample_detail": sample, "compiler": ORACLE_FLAGS},
            "e2e": {"value": value, "unit": "image pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def serve_configs(seed: int, rates: str, threads: int, prec_list=("bf16", "fp32")) -> dict:
    """Serving: zones of 48 positions x 3 cameras, n ~ log-uniform[500, 4000],
    views arriving as a Poisson process (or all at once: 'burst'); each view is
    matched against its candidate_pairs partners already on the device.
    Latency = submit -> match lists on the host; every 9th request's lists are
    checked against the oracle."""
    import oracle as O
    from skylens_match import serve
    z = serve.serving_zone(48, seed=seed + 2)
    reqs = serve.zone_requests(z)
    out = {"metric": "serving: image pairs/s and p50/p99 request latency (view arrival -> match lists on host)",
           "config": {"workload": "serve_zone144", "views": len(z.counts), "pairs": int(len(z.pairs)),
                      "n": "log-uniform [500, 4000]", "arrivals": "Poisson", "slots": 3,
                      "submission": "slm_server_submit_ptr: each view's rows read where they lie on admission"},
           "runs": []}
    # every run back to back (the GPU stays busy between them), then the
    # oracle's check of every 9th request of each run
    npairs = sum(len(p) for _, p in reqs)
    done = []
    for prec in prec_list:
        for rate in [None if r == "burst" else float(r) for r in rates.split(",")]:
            # a burst lasts milliseconds: on one server, a first zone (cold: the
            # server's first batches) and then three more zones of the same
            # views (ids after the earlier zones'), whose median is reported
            # (with each run and the cold one)
            runs = []
            zones = 1 if rate else 4
            srv = serve.Server(int(z.counts.sum()) * zones, len(z.counts) * zones, prec, slots=3)
            for k in range(zones):
                # the client's garbage collector stays out of the measured latencies
                gc.collect()
                gc.disable()
                try:
                    res, lats, wall = serve.stream_zone(srv, z, rate, seed=int(rate or 0),
                                                        view_offset=k * len(z.counts))
                finally:
                    gc.enable()
                runs.append((wall, res, lats))
            st = dict(srv.stats())
            srv.close()
            warm = runs[1:] if len(runs) > 1 else runs
            walls = [x[0] for x in warm]
            wall, res, lats = warm[int(np.argsort(walls)[len(walls) // 2])]
            st["zones"] = zones
            if len(runs) > 1:
                st["pairs_per_s_each"] = [npairs / x for x in walls]
                st["pairs_per_s_cold"] = npairs / runs[0][0]
            done.append((prec, rate, res, lats, wall, st))
    check = {}
    for prec, rate, res, lats, wall, st in done:
        mism = 0
        for k in range(0, len(reqs), 9):
            v, pairs = reqs[k]
            for (u, _), got in zip(pairs, res[k]):
                key = (u, v)
                if key not in check:
                    check[key] = O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=threads)
                mism += not np.array_equal(got, check[key])
        out["runs"].append({"precision": prec, "rate_views_per_s": rate if rate else "burst",
                            "p50_ms": float(np.percentile(lats, 50)),
                            "p99_ms": float(np.percentile(lats, 99)), "mean_ms": float(lats.mean()),
                            "pairs_per_s": npairs / wall, "wall_s": wall, "zones_served": st["zones"],
                            "batches": st["batches"],
                            "max_batch_requests": st["max_batch_requests"], "max_inflight": st["max_inflight"],
                            "bit_exact_sample_mismatches": int(mism)})
        if "pairs_per_s_each" in st and rate is None:
            out["runs"][-1]["pairs_per_s_each_run"] = st["pairs_per_s_each"]
            out["runs"][-1]["pairs_per_s_cold"] = st["pairs_per_s_cold"]
            out["runs"][-1]["runs"] = ("median of 3 bursts on a server that has served a zone before (each "
                                       "a zone of new views); pairs_per_s_cold: the server's first zone")
        print(json.dumps(out["runs"][-1]), file=sys.stderr, flush=True)
    return out


def run_serve(args):
    out = serve_configs(args.seed, args.rates, os.cpu_count() or 1)
    print(json.dumps(out), flush=True)
    if args.json_out:
        open(args.json_out, "w").write(json.dumps(out) + "\n")
    return 0


def pair_configs(m, steps: int, threads: int) -> list:
    """Single-pair configurations: 800 x 800, 8192 x 8192 (BF16 vs FP32), and
    32768 x 32768 (FP8 E4M3 shortlist), each in every precision through a
    one-pair plan: device time by CUDA events (median of `steps` launches),
    bit-exactness of the whole list against the oracle, distance-estimate
    error against FP64 on a 1024 x 1024 block, and the rows settled exactly."""
    import torch

    import oracle as O
    from skylens_match import synth
    ext = torch.cuda.ExternalStream(m.stream)
    pk, _ = peaks()
    cases = [("pair800", lambda: synth.pair_800(0)), ("pair8192", lambda: synth.pair_large(8192, 0.5, 0.05, seed=2)),
             ("pair32768", lambda: synth.pair_fp8(32768, seed=4))]
    out = []
    for name, make in cases:
        a, b = make()
        ref = O.ratio_match_np(a, b, 0.8, True, threads=threads)
        st = m.store(len(a) + len(b), 2)
        st.add_view(a)
        st.add_view(b)
        row = {"config": name, "na": len(a), "nb": len(b), "distances": len(a) * len(b), "precisions": {}}
        for prec in ("fp32", "bf16", "fp8"):
            plan = st.plan([(0, 1)], 0.8, True, prec)
            plan.launch()
            got, _ = plan.results()
            times = []
            for _ in range(max(1, steps)):
                with torch.cuda.stream(ext):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                plan.launch()
                with torch.cuda.stream(ext):
                    e1.record()
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            plan.results()
            s = plan.stats
            ms = float(np.median(times))
            # small pairs: bytes the pair must move (both operand images and
            # the match list) against the measured HBM copy rate
            nbytes = (len(a) + len(b)) * 128 * {"fp32": 4, "bf16": 2, "fp8": 1}[prec] + len(got) * 8
            hbm = nbytes / (ms / 1e3) / 1e9
            row["precisions"][prec] = {"ms": ms, "distances_per_s": len(a) * len(b) / (ms / 1e3),
                                       "hbm": {"bytes": nbytes, "achieved_gbs": hbm, "peak_gbs": pk["hbm_gbs"],
                                               "frac": hbm / pk["hbm_gbs"]},
                                       "bit_exact": bool(np.array_equal(got, ref)), "matches": int(len(got)),
                                       "rows_rescored_frac": s["rows_rescored"] / len(a),
                                       "rows_recomputed_frac": s["rows_recomputed"] / len(a),
                                       "cols_recomputed": s["cols_recomputed"],
                                       "pairs_routed": s["pairs_routed"],
                                       "pairs_rescued": s["pairs_rescued"],
                                       "settled_frac": settled_frac(s, len(a), prec),
                                       "pass_ms": [float(x) for x in s["pass_ms"]],
                                       "max_err_rescored_vs_f32": s["max_abs_err"]}
            plan.close()
        # distance-estimate error against FP64 on a block of up to 1024 x 1024
        nsub = min(1024, len(a), len(b))
        sub_a, sub_b = a[:nsub], b[:nsub]
        d64 = O.dist_matrix_f64(sub_a, sub_b)
        st2 = m.store(2 * nsub, 2)
        st2.add_view(sub_a)
        st2.add_view(sub_b)
        for prec in ("bf16", "fp8"):
            p = st2.plan([(0, 1)], 0.8, True, prec, variant=2)
            p.launch()
            p.results()
            dt = p.debug_dump(nsub, nsub)
            row["precisions"][prec]["max_abs_err_vs_fp64"] = float(np.abs(dt - d64).max())
            row["precisions"][prec]["err_block"] = f"{nsub}x{nsub}"
            p.close()
        st2.close()
        st.close()
        print(json.dumps(row), file=sys.stderr, flush=True)
        out.append(row)
    return out


def ransac_configs(m, threads: int, pairs: int = 100, hyps: int = 2000, reps: int = 3) -> dict:
    """The RANSAC stage's hypothesis scoring (two_view.rs:804-823) for a block
    of iterations of `pairs` kept pairs: matches per pair ~ U[200, 550] (the
    240-view zone keeps 373 matches per pair on average), `hyps` hypotheses each
    (500 iterations of up to 10 5-point solutions per pair in the reference).
    GPU: slm_sampson_score from host arrays (copies in the timed call); CPU:
    the oracle's restatement on all host threads. Counts must be equal."""
    import oracle as O
    from skylens_match import synth
    rng = np.random.default_rng(5)
    pts, off, th, hs, hp = [], [0], [], [], []
    for p in range(pairs):
        n = int(rng.integers(200, 551))
        n1, n2, e = synth.two_view(rng, n, inlier_frac=rng.uniform(0.3, 0.9))
        pts.append(np.concatenate([n1, n2], 1))
        off.append(off[-1] + n)
        th.append(1.5 / 800.0)
        hs.append(synth.essential_hypotheses(rng, e, hyps))
        hp += [p] * hyps
    pts = np.concatenate(pts)
    off = np.asarray(off, np.uint64)
    th = np.asarray(th)
    hs = np.concatenate(hs)
    hp = np.asarray(hp, np.uint32)
    residuals = int(sum(int(off[p + 1] - off[p]) for p in hp))
    got, _ = m.sampson_score(pts, off, th, hs, hp)  # warm-up
    gpu = []
    for _ in range(reps):
        t0 = time.perf_counter()
        got, _ = m.sampson_score(pts, off, th, hs, hp)
        gpu.append(time.perf_counter() - t0)
    cpu = []
    for _ in range(reps):
        t0 = time.perf_counter()
        want, _ = O.sampson_score(pts, off, th, hs, hp, threads=threads)
        cpu.append(time.perf_counter() - t0)
    g, c = float(np.median(gpu)), float(np.median(cpu))
    return {"metric": "RANSAC hypothesis scoring: Sampson residuals/s (count_at_least / inliers_of)",
            "config": {"pairs": pairs, "hypotheses": len(hs), "matches": int(off[-1]), "residuals": residuals,
                       "dtype": "f64, the reference's operation order"},
            "gpu": {"ms": g * 1e3, "residuals_per_s": residuals / g,
                    "timed": "slm_sampson_score from host arrays (uploads and read-back included)"},
            "cpu": {"ms": c * 1e3, "residuals_per_s": residuals / c, "threads": threads, "kind": "port"},
            "equal_counts": bool(np.array_equal(got, want))}


def features_configs(m, threads: int, n: int = 24, reps: int = 5, cpu_images: int = 32) -> dict:
    """The descriptor producer (features.rs:594 detect_and_describe, default
    DetectorConfig) on `n` RGB8 views of 960 x 540, the size of the
    pipeline's synthetic frames, of one seeded textured scene (a camera
    moving along a facade; the reference's rendered scenes stand in). GPU:
    slm_detect_and_describe_rgb8 on images already in HBM with descriptors
    left in HBM (`value`), and from pinned host images to host keypoints and
    descriptors (`e2e`). CPU: the oracle's restatement (the platform's float
    functions, as the reference) over `cpu_images` images on all host threads,
    one image per thread as the pipeline's par_iter does. Checks: two images
    bit-exact against the oracle with correctly rounded functions (the GPU's
    arithmetic), and the largest descriptor difference against the platform's."""
    import ctypes
    from concurrent.futures import ThreadPoolExecutor

    import torch

    import oracle as O
    from skylens_match import synth
    from skylens_match import features as F
    w, h = 960, 540
    views = synth.scene_views(n, w, h, seed=11)
    cfg = F.detector_config()
    cap = n * int(cfg.max_features)
    L = m._L
    off = np.zeros(n + 1, np.uint64)

    def call(img_ptr, kps_ptr, desc_ptr):
        st = L.slm_detect_and_describe_rgb8(m.handle, ctypes.c_void_p(img_ptr), n, w, h, ctypes.byref(cfg),
                                            ctypes.c_void_p(kps_ptr), ctypes.c_void_p(desc_ptr), cap,
                                            off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        if st:
            raise RuntimeError(f"slm_detect_and_describe_rgb8: status {st}")

    d_img = torch.from_numpy(views).cuda()
    d_desc = torch.empty((cap, 128), dtype=torch.float32, device="cuda")
    p_img = torch.from_numpy(views).pin_memory()
    p_kps = torch.empty((cap, 5), dtype=torch.float32).pin_memory()
    p_desc = torch.empty((cap, 128), dtype=torch.float32).pin_memory()
    call(d_img.data_ptr(), p_kps.data_ptr(), d_desc.data_ptr())  # warm-up
    dev, e2e = [], []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        call(d_img.data_ptr(), p_kps.data_ptr(), d_desc.data_ptr())
        dev.append(time.perf_counter() - t0)
    for _ in range(reps):
        t0 = time.perf_counter()
        call(p_img.data_ptr(), p_kps.data_ptr(), p_desc.data_ptr())
        e2e.append(time.perf_counter() - t0)
    nfeat = int(off[-1])
    kps = p_kps.numpy()[:nfeat].copy()
    desc = p_desc.numpy()[:nfeat].copy()
    exact, maxdiff = True, 0.0
    for k in range(2):
        g = O.gray_from_rgb8(views[k])
        a, b = int(off[k]), int(off[k + 1])
        k1, d1 = O.detect_and_describe(g, cr=True)
        exact &= bool(np.array_equal(k1, kps[a:b]) and np.array_equal(d1, desc[a:b]))
        k0, d0 = O.detect_and_describe(g, cr=False)
        if len(k0) == b - a:
            maxdiff = max(maxdiff, float(np.abs(d0 - desc[a:b]).max()))
        else:
            maxdiff = float("nan")
    cpu_views = synth.scene_views(cpu_images, w, h, seed=11) if cpu_images else []
    grays = [O.gray_from_rgb8(v) for v in cpu_views]
    cpu = []
    for _ in range(2 if cpu_images else 0):
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda g: O.detect_and_describe(g, cr=False), grays))
        cpu.append(time.perf_counter() - t0)
    cpu = cpu or [float("nan")]
    gd, ge, c = float(np.median(dev)), float(np.median(e2e)), float(np.median(cpu))
    return {"metric": "descriptor producer: images/s (detect_and_describe, 960 x 540 RGB8, default DetectorConfig)",
            "config": {"workload": "scene960", "images": n, "width": w, "height": h, "features": nfeat,
                       "features_per_image": nfeat / n},
            "value": n / gd, "unit": "images/s", "ms": gd * 1e3, "features_per_s": nfeat / gd,
            "timed": "slm_detect_and_describe_rgb8, images in HBM, descriptors left in HBM, keypoints to pinned host",
            "e2e": {"value": n / ge, "unit": "images/s", "ms": ge * 1e3, "h2d_bytes": int(views.nbytes),
                    "d2h_bytes": nfeat * (128 + 5) * 4},
            "bit_exact_vs_oracle_cr": exact, "max_desc_diff_vs_platform_functions": maxdiff,
            "cpu_baseline": {"value": cpu_images / c if cpu_images else None, "unit": "images/s", "threads": threads, "kind": "port",
                             "sample": f"{cpu_images} images of the same scene, one per thread, median of 2"}}


def tracks_configs(m, z, res, off, reps: int = 3) -> dict:
    """build_tracks with ConflictPolicy::Drop (tracks.rs:190) over the zone's
    match lists (every pair's BF16 list as its verified matches; the
    reference feeds RANSAC inliers). GPU: slm_build_tracks_drop from host
    arrays (upload, edge set, components on the device, grouping and the cap
    on the host); CPU: the oracle's restatement (one thread, as the
    reference's union-find). Tracks and counts must be equal."""
    import ctypes

    import oracle as O
    from skylens_match import tracks as T
    pairs = [(int(u), int(v), res[int(off[k]):int(off[k + 1])]) for k, (u, v) in enumerate(z.pairs.tolist())]
    nf = np.ascontiguousarray(z.counts, dtype=np.uint32)
    arr, flat = T.pack(pairs)
    oarr, oflat = O.pack_pairs(pairs)
    n_match = len(flat)
    P = ctypes.POINTER
    cap_t, cap_o = max(n_match, 1), max(2 * n_match, 1)
    toff = np.zeros(cap_t + 1, np.uint64)
    obs = np.zeros((cap_o, 2), np.uint32)
    nt, no = ctypes.c_uint64(), ctypes.c_uint64()
    gst = T.SlmTrackStats()

    def gpu():
        st = m._L.slm_build_tracks_drop(m.handle, nf.ctypes.data_as(P(ctypes.c_uint32)), len(nf), arr, len(pairs),
                                        flat.ctypes.data_as(P(T.SlmPair)), 3, 100000,
                                        toff.ctypes.data_as(P(ctypes.c_uint64)), cap_t, obs.ctypes.data_as(P(T.SlmPair)),
                                        cap_o, ctypes.byref(nt), ctypes.byref(no), ctypes.byref(gst))
        if st:
            raise RuntimeError(f"slm_build_tracks_drop: status {st}")

    otoff = np.zeros(cap_t + 1, np.uint64)
    onodes = np.zeros(cap_o, np.uint64)
    ost = O.TrackStats()

    def cpu():
        return O.lib().orc_build_tracks_drop(nf.ctypes.data_as(P(ctypes.c_uint32)), len(nf),
                                             ctypes.cast(oarr, ctypes.c_void_p), len(pairs),
                                             oflat.ctypes.data_as(P(ctypes.c_uint32)), 3, 100000,
                                             otoff.ctypes.data_as(P(ctypes.c_uint64)), cap_t,
                                             onodes.ctypes.data_as(P(ctypes.c_uint64)), cap_o, ctypes.byref(ost))

    gpu()
    g = []
    for _ in range(reps):
        t0 = time.perf_counter()
        gpu()
        g.append(time.perf_counter() - t0)
    c = []
    for _ in range(reps):
        t0 = time.perf_counter()
        ont = cpu()
        c.append(time.perf_counter() - t0)
    # equal: the same track boundaries and nodes ((image, feature) from nodes)
    noff = np.concatenate([[0], np.cumsum(z.counts, dtype=np.uint64)])
    nobs = int(no.value)
    nodes_g = noff[obs[:nobs, 0].astype(np.int64)] + obs[:nobs, 1].astype(np.uint64)
    equal = (int(nt.value) == int(ont) and np.array_equal(toff[:int(nt.value) + 1], otoff[:int(ont) + 1])
             and np.array_equal(nodes_g, onodes[:nobs]) and gst.as_dict() == ost.as_dict())
    gm, cm = float(np.median(g)), float(np.median(c))
    return {"metric": "tracks (ConflictPolicy::Drop): verified matches/s into tracks",
            "config": {"workload": "zone240 match lists", "pairs": len(pairs), "matches": n_match,
                       "nodes": int(nf.sum()), "min_length": 3, "max_tracks": 100000},
            "stats": gst.as_dict(),
            "gpu": {"ms": gm * 1e3, "matches_per_s": n_match / gm,
                    "timed": "slm_build_tracks_drop from host arrays (upload and read-back included)"},
            "cpu": {"ms": cm * 1e3, "matches_per_s": n_match / cm, "threads": 1, "kind": "port"},
            "equal": bool(equal)}


def settled_frac(s, na, prec):
    """Fractions of a single pair's rows settled by each tier: by the FP8 bound,
    by the BF16 bound (BF16 pairs, and FP8 pairs rescued by the BF16 passes),
    or with exact FP32 arithmetic (rescored, scanned, or routed whole)."""
    if prec == "fp32" or na == 0:
        return {"fp8_bound": 0.0, "bf16_bound": 0.0, "exact": 1.0}
    exact = min(1.0, (s["rows_rescored"] + s["rows_recomputed"]) / na)
    bf16 = prec == "bf16" or s["pairs_rescued"] > 0
    return {"fp8_bound": 0.0 if bf16 else 1.0 - exact, "bf16_bound": 1.0 - exact if bf16 else 0.0, "exact": exact}


def run_pairs(args):
    import skylens_match as sm
    m = sm.Matcher()
    out = pair_configs(m, args.steps, os.cpu_count() or 1)
    for r in out:
        print(json.dumps(r), flush=True)
    if args.json_out:
        open(args.json_out, "w").write("\n".join(json.dumps(r) for r in out) + "\n")
    m.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.serve:
        return run_serve(args)
    if args.pairs:
        return run_pairs(args)
    if args.ransac:
        import skylens_match as sm
        m = sm.Matcher()
        print(json.dumps(ransac_configs(m, os.cpu_count() or 1)), flush=True)
        m.close()
        return 0
    if args.features:
        import skylens_match as sm
        m = sm.Matcher()
        print(json.dumps(features_configs(m, os.cpu_count() or 1, reps=args.features_reps,
                                          cpu_images=0 if args.no_cpu_baseline else 32)), flush=True)
        m.close()
        return 0
    import torch

    import oracle as O
    import skylens_match as sm
    from skylens_match import synth

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist = None
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    built = getattr(sm, "BUILT_PRECISIONS", ("fp32",))
    prec = args.precision if args.precision != "auto" else ("bf16" if "bf16" in built else "fp32")

    # ---- workload (each rank its own zone: replicas, weak scaling)
    z = synth.zone(positions=args.positions, seed=args.seed + rank)
    n_rows = int(z.counts.sum())
    pinned = torch.from_numpy(z.desc).pin_memory()
    m = sm.Matcher(device=dev)
    ext = torch.cuda.ExternalStream(m.stream)
    store = m.store(n_rows, len(z.counts))
    store.add_views_ptr(pinned.data_ptr(), z.offsets, z.counts)
    # Both arms use settings chosen by the library's autotuner on this batch.
    tuned = {}
    for pr in ([prec] if prec == "fp32" else [prec, "fp32"]):
        tuned[pr] = store.autotune(z.pairs, 0.8, True, pr)[0]
    if args.scalar:
        plan = store.plan(z.pairs, 0.8, True, prec, variant=1)
    else:
        plan = store.plan(z.pairs, 0.8, True, prec, autotune=True)
    plan_fp32 = plan if prec == "fp32" else store.plan(z.pairs, 0.8, True, "fp32", autotune=True)

    # ---- correctness against the oracle on a sample of pairs
    plan.launch()
    got, off = plan.results()
    nverify = len(z.pairs) if args.verify_pairs < 0 else min(args.verify_pairs, len(z.pairs))
    sel = np.random.Generator(np.random.PCG64(7)).permutation(len(z.pairs))[:nverify]
    mism = 0
    for k in sel:
        u, v = int(z.pairs[k, 0]), int(z.pairs[k, 1])
        ref = O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=os.cpu_count() or 1)
        mism += not np.array_equal(got[int(off[k]):int(off[k + 1])], ref)
    bit_exact = mism == 0
    stats_main = dict(plan.stats)

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(p, steps, warm):
        for _ in range(warm):
            with torch.cuda.stream(ext):
                flush.zero_()
            p.launch()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        evs = []
        kern = []
        for _ in range(steps):
            with torch.cuda.stream(ext):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
            p.launch()
            with torch.cuda.stream(ext):
                e1.record()
            e1.synchronize()
            p.results()  # reads main-kernel times; not part of the device-timed region
            kern.append((p.stats["kernel_ms"], p.stats["pass_ms"][0], p.stats["pass_ms"][1]))
            evs.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return evs, kern

    clocks = Clocks(dev)
    clocks.start()
    t_wall0 = time.perf_counter()
    step_ms, kern_ms = timed(plan, args.steps, args.warmup)
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    ms = float(np.mean(step_ms))
    rdev = "cuda" if dist else None
    ms_local = ms
    ms, _, value = reduce_over_ranks(ms, len(z.pairs), dist, device=rdev)
    # distances over all ranks (each rank's zone has its own seed) per job time
    _, _, dist_rate = reduce_over_ranks(ms_local, z.distances, dist, device=rdev)

    fp32 = None
    if plan_fp32 is not plan:
        f_ms, f_kern = timed(plan_fp32, max(1, args.fp32_steps), 1)
        fms, _, fval = reduce_over_ranks(float(np.mean(f_ms)), len(z.pairs), dist, device=rdev)
        fp32 = {"value": fval, "unit": "image pairs/s", "ms_per_step": fms,
                "kernel_ms": float(np.mean([k[0] for k in f_kern]))}

    # ---- the run pipeline's own pair set (pipeline.rs:485-496): scheduled_pairs with
    # PairSchedule::default() and the filter that drops pairs with < 20 matches
    sched = None
    if not args.no_scheduled:
        spairs = sm.scheduled_pairs(z.views)
        store.autotune(spairs, 0.8, True, prec)
        splan = store.plan(spairs, 0.8, True, prec, autotune=True)
        splan.set_min_matches(20)
        s_ms, _ = timed(splan, max(3, args.steps // 2), 2)
        sgot, soff = splan.results()
        cnt = np.diff(soff.astype(np.int64))
        smism = 0
        ssel = np.random.Generator(np.random.PCG64(8)).permutation(len(spairs))[:min(100, len(spairs))]
        for k in ssel:
            u, v = spairs[int(k)]
            ref = O.ratio_match_np(z.view(u), z.view(v), 0.8, True, threads=os.cpu_count() or 1)
            ref = ref if len(ref) >= 20 else ref[:0]
            smism += not np.array_equal(sgot[int(soff[k]):int(soff[k + 1])], ref)
        sms = float(np.mean(s_ms))
        sdist = int(sum(int(z.counts[u]) * int(z.counts[v]) for u, v in spairs))
        sched = {"schedule": "PairSchedule::default()", "min_matches": 20, "pairs": len(spairs),
                 "pairs_kept": int((cnt > 0).sum()), "matches_kept": int(soff[-1]), "distances": sdist,
                 "ms_per_step": sms, "value": len(spairs) / (sms / 1e3), "unit": "image pairs/s",
                 "bit_exact": {"ok": smism == 0, "pairs_checked": int(len(ssel)), "mismatched_pairs": int(smism)}}
        splan.close()

    # ---- e2e through the C ABI with host buffers
    e2e = None
    out_bytes = 0
    if not args.no_e2e:
        # Three contexts (three library streams), each with its own store and
        # plan, take the batches in turn: batch k's upload and launch are issued
        # before batch k-2's match lists are read back, so the copies of one
        # batch overlap the kernels of the two before it. Every step still
        # uploads all views from pinned host memory (one copy per view, copy
        # engines only) and reads its match lists back into pinned host buffers
        # (slm_plan_results).
        NL = 3
        tp = tuned[prec]
        extra = []
        lanes = []
        for q in range(NL):
            if q == 0:
                st_, pl_ = store, plan
            else:
                mq = sm.Matcher(device=dev)
                st_ = mq.store(n_rows, len(z.counts))
                st_.add_views_ptr(pinned.data_ptr(), z.offsets, z.counts)
                pl_ = st_.plan(z.pairs, 0.8, True, prec, items_per_sm=tp["items_per_sm"],
                               shortlist_k=tp["shortlist_k"], use_graph=1, variant=tp["variant"],
                               row_tiles=tp["row_tiles"])
                extra.append((mq, st_, pl_))
            lanes.append((st_, pl_,
                          torch.empty((max(pl_.total_rows, 1), 2), dtype=torch.int32).pin_memory().numpy().view(np.uint32),
                          torch.empty(len(z.pairs) + 1, dtype=torch.int64).pin_memory().numpy().view(np.uint64)))

        def issue(k):
            st_, pl_ = lanes[k % NL][:2]
            st_.clear()
            st_.add_views_ptr(pinned.data_ptr(), z.offsets, z.counts)
            pl_.launch()

        def read(k):
            _, pl_, o_, f_ = lanes[k % NL]
            return pl_.results_into(o_, f_)

        def run(first, n):
            """Steps first .. first+n-1, at most NL-1 in flight; returns the last total."""
            tot = 0
            for k in range(first, first + n):
                issue(k)
                if k - first >= NL - 1:
                    tot = read(k - NL + 1)
            for k in range(max(first, first + n - NL + 1), first + n):
                tot = read(k)
            return tot

        run(0, 2 * NL)  # warm-up: every lane, graphs captured
        ref_pr, ref_of = plan.results()
        for _, _, o_, f_ in lanes:
            assert int(f_[-1]) == int(ref_of[-1]) and np.array_equal(o_[:int(f_[-1])], ref_pr)
        t0 = time.perf_counter()
        total = run(0, args.steps)
        e2e_s = (time.perf_counter() - t0) / args.steps
        # job time = the slowest rank's, work = every rank's pairs
        e2e_ms, _, e2e_value = reduce_over_ranks(1e3 * e2e_s, len(z.pairs), dist, device=rdev)
        out_bytes = total * 8 + lanes[0][3].nbytes
        for mq, st_, pl_ in extra:
            pl_.close()
            st_.close()
            mq.close()
        e2e = {"value": e2e_value, "unit": "image pairs/s", "ms_per_step": e2e_ms,
               "h2d_bytes_per_step": int(z.desc.nbytes), "d2h_bytes_per_step": int(out_bytes),
               "pipeline": f"{NL} contexts: a batch's upload overlaps the kernels of the {NL - 1} before it"}

    # ---- roofline of the dominant kernel
    pk, pk_kind = peaks()
    kms = float(np.mean([k[0] for k in kern_ms]))
    p1ms = float(np.mean([k[1] for k in kern_ms]))
    p2ms = float(np.mean([k[2] for k in kern_ms]))
    dist_n = z.distances
    if prec in ("bf16", "fp8"):
        # Each tensor-core pass contracts every (row, column) once: 2*128 flops per
        # distance. The dominant kernel is the slower pass, timed alone by events.
        flops = 2.0 * 128 * dist_n
        dom_ms, dom = (p2ms, "sl_pass_kernel<2> (pass 2)") if p2ms >= p1ms else (p1ms, "sl_pass_kernel<1> (pass 1)")
        achieved = flops / (dom_ms / 1e3) / 1e12
        peak = pk["bf16_tflops"] * (2 if prec == "fp8" else 1)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "kernel": dom, "kernel_ms": dom_ms, "pass1_ms": p1ms, "pass2_ms": p2ms,
                "pipeline_ms": kms, "algorithmic": "256 flops per distance x %d distances" % dist_n,
                "peak_source": f"{pk_kind} bf16_tflops (burst) of MEASURED_PEAKS.json"}
    else:
        # 384 FP32 instructions per distance (sub, mul, add per component, matching.rs:146-155)
        sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        mhz = clk.get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
        peak = sm_count * 128 * mhz * 1e6 / 1e12  # FP32 lane-instructions/s (T/s)
        achieved = 384.0 * dist_n / (kms / 1e3) / 1e12
        roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "T FP32 instr/s",
                "frac": achieved / peak, "traffic": None, "kernel": "exact_kernel",
                "peak_source": f"{sm_count} SMs x 128 lanes x {mhz:.0f} MHz (sampled)"}
    # DRAM bytes per launch of the dominant kernel from an ncu capture of this workload
    prof = os.path.join(REPO, "profiles", "sl_pass_kernel_zone240_dram.json")
    if os.path.exists(prof) and WORKLOAD == "zone240" and args.positions == 80:
        try:
            roof["traffic"] = json.load(open(prof)).get(roof["kernel"])
        except Exception:
            pass

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # three repeats on all host threads (value = their median) and three on
        # one thread, each repeat over the same pairs in the same order
        cores = os.cpu_count() or 1
        runs = [cpu_baseline(z, args.cpu_seconds / 3, cores) for _ in range(3)]
        one = [cpu_baseline(z, args.cpu_seconds / 6, 1) for _ in range(3)]
        med = float(np.median([x[0] for x in runs]))
        cpu = {"value": med, "unit": "image pairs/s", "cores": cores, "kind": "port",
               "sample": f"{int(np.median([x[2] for x in runs]))} of {len(z.pairs)} zone pairs in a fixed random "
                         f"order per repeat (~{args.cpu_seconds / 3:.0f} s), 3 repeats",
               "median": med, "min": float(min(x[0] for x in runs)), "compiler": ORACLE_FLAGS,
               "distances_per_s": float(np.median([x[1] for x in runs])),
               "one_thread": {"median": float(np.median([x[0] for x in one])), "min": float(min(x[0] for x in one)),
                              "unit": "image pairs/s",
                              "sample": f"{int(np.median([x[2] for x in one]))} pairs per repeat "
                                        f"(~{args.cpu_seconds / 6:.0f} s), 3 repeats"}}

    line = {"metric": METRIC, "value": value, "unit": "image pairs/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"fp32": "f32", "bf16": "bf16", "fp8": "e4m3"}[prec],
            "data": "synthetic",
            "config": workload_config(z, args.seed + rank, ws), "precision": prec, "tuned": tuned,
            "distances_per_s": dist_rate,
            "bit_exact": {"ok": bit_exact, "pairs_checked": int(nverify), "mismatched_pairs": int(mism)},
            "fp32_plain": fp32, "scheduled": sched,
            "kernel_ms": kms, "stats": stats_main,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(stats_main.get("kernel_launches", 0)) * args.steps,
            "clocks": clk, "wall_s_timed": t_wall}
    if rank == 0 and ws == 1 and not args.no_configs:
        # the other configurations, bounded (about half a minute): single pairs
        # in every precision and the serving workload at one rate and in a burst
        t_c = time.perf_counter()
        pairs_rec = pair_configs(m, 3, os.cpu_count() or 1)
        sclk = Clocks(dev)
        sclk.start()
        serve_rec = serve_configs(args.seed, args.config_rates, os.cpu_count() or 1)
        serve_rec["clocks"] = sclk.stop()
        line["configs"] = {"pairs": pairs_rec,
                           "serve": serve_rec,
                           "ransac_scoring": ransac_configs(m, os.cpu_count() or 1),
                           "descriptor_producer": features_configs(m, os.cpu_count() or 1)}
        if prec in ("bf16", "fp8", "fp32") and args.positions == 80:
            pr_, of_ = plan.results()
            line["configs"]["tracks"] = tracks_configs(m, z, pr_, of_)
        line["configs"]["wall_s"] = time.perf_counter() - t_c
    if rank == 0:
        s = json.dumps(line)
        print(s, flush=True)
        if args.json_out:
            open(args.json_out, "w").write(s + "\n")
    plan.close()
    if plan_fp32 is not plan:
        plan_fp32.close()
    store.close()
    m.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
