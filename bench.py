"""Benchmark of the RILS-ROLS fitness path on GB300.

Metric: candidate fitness evaluations per second (tune_constants + fitness of
rils_rols_cpp.cpp:445-541 per candidate) at n = 1M rows, in the certified
mixed-precision form: every fitness within 1e-6 relative of the FP64 path.

Workload (one step): the eight local-search rounds of a search on the 1M-row,
5-feature regression problem (X ~ U(-3, 3), y = 2.5 x1 x2 - sin(x3)/(1+x4^2) +
0.7 exp(0.3 x5) + 0.5% noise), submitted the way the search submits them:
one rrg_round_submit / rrg_round_wait per round, in order.  Round r holds the
local-search candidates (all_candidates, rils_rols_cpp.cpp:348-443) of the
r-th model of synth.REGRESSION_1M_TRAJECTORY, 264 to 1469 tuned candidates,
7083 in all (tests/golden/ls_rounds_regression_1m.txt.gz, made by the
reference's own generator).  Synthetic, seeded data; nothing is downloaded.

  value  device-resident: dataset in HBM, each step = the eight rounds (batch
         upload, kernels and results back per round), timed with CUDA events
         on the library's stream, L2 flushed (256 MB write) before every step;
  e2e    through the C ABI from host buffers: per step X and y are uploaded
         from pinned host memory (rrg_dataset_create) and every round's trees
         are flattened, scored and their results read back.

Reported beside it: the eight rounds concatenated into one batch, the
uncertified mixed form, the plain FP64 path batched and unbatched, the
fitness of a seeded sample of the candidates against the oracle (plain FP64
bit for bit, certified within 1e-6), a capped regression fit at n = 1M
through the drop-in module, the standalone batched-fitness configuration,
the classifier fits and the serving stream, the roofline of the dominant
kernel, the CPU oracle timed on the host cores, clocks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--serve-jobs J] [--serve-only] [--quick]

Measurement cases for profiling (one JSON line each, no bench contract):
  --round-only R        round R of the headline workload (R = 8: the eight
                        concatenated into one call), certified, once (with
                        RRG_TUNE_CACHE set, no launch-shape trials): its
                        phase times, algorithmic bytes and launches;
  --case NAME --fac-stage S
                        the double-float factor evaluator with X and y read
                        from global memory (S = 1) or staged in shared memory
                        by tensor copies (S = 2): local_search_d5 (the eight
                        rounds), random_d10 / random_d20 (1500 random trees,
                        n rows, d = 10 / 20); per step its time and the round's.
"""
from __future__ import annotations

import argparse
import gc
import gzip
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "rils-rols_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "candidate fitness evals/s at n=1M (certified mixed precision, local-search rounds)"
UNIT = "evals/s"
N_ROWS = 1_000_000
N_FEAT = 5
SEED = 12345
ROUNDS_FILE = ROOT / "tests" / "golden" / "ls_rounds_regression_1m.txt.gz"


def load_rounds() -> list[list[str]]:
    """The eight local-search rounds (prefix trees), in order."""
    rounds: dict[int, list[str]] = {}
    for line in gzip.open(ROUNDS_FILE, "rt").read().splitlines():
        r, tree = line.split("\t")
        rounds.setdefault(int(r), []).append(tree)
    return [rounds[k] for k in sorted(rounds)]


def regression_data(n=N_ROWS, seed=SEED):
    from rils_rols_gb300 import synth  # numpy only: the product library is not loaded
    return synth.regression_1m(n=n, seed=seed)


def config(n, rounds):
    sizes = [len(r) for r in rounds]
    return {"workload": f"the 8 local-search rounds of the 1M-row regression search, one call per round "
                        f"({min(sizes)}..{max(sizes)} tuned candidates, {sum(sizes)} in all) x n={n} rows, "
                        f"d={N_FEAT}",
            "n_rows": n, "n_features": N_FEAT, "rounds": len(rounds), "round_sizes": sizes,
            "candidates": "all_candidates(model, local_search) of the 8 models on the way to the generating formula",
            "precision": "RRG_MIXED_CERTIFIED: double-float factor table, FP64 Cholesky / SSE, every result within "
                         "1e-6 of the FP64 path (rank-ambiguous and non-finite candidates re-scored in FP64)",
            "l2": "flushed (256 MB write on the round's stream) before every timed step"}


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline --
def sample_index(total: int, sample: int, seed: int = 5) -> np.ndarray:
    return np.sort(np.random.default_rng(seed).choice(total, min(sample, total), replace=False))


def cpu_baseline(X, y, trees, idx, threads=None):
    """The oracle (oracle/rrg_oracle.c, FP64; trees flattened by the oracle's
    own encoder, oracle/tree_encode.py) on the candidates `idx` of `trees`
    with `threads` host threads.  Returns the baseline record and the
    oracle's results (kept for the accuracy comparison)."""
    from oracle import pyoracle, tree_encode
    threads = threads or os.cpu_count() or 1
    ods = pyoracle.OracleDataset(X, y)
    b = tree_encode.encode([trees[i] for i in idx], tuned=True)
    t = time.perf_counter()
    out = ods.evaluate(b, threads=threads)
    dt = time.perf_counter() - t
    rec = {"value": len(idx) / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{len(idx)} seeded random candidates of the {len(trees)} at n={len(y)} "
                     f"(oracle/rrg_oracle.c via oracle/tree_encode.py, FP64, {threads} threads, {dt:.1f} s)"}
    return rec, out


def fv(r):
    return (1 + r["loss"]) * (1 + r["rmse"]) * (1 + r["size"] * 1e-3)


def accuracy(test, ref):
    """Per-candidate fitness of `test` against `ref` (dicts of arrays)."""
    ok = (ref["loss"] != 1000) & np.isfinite(fv(ref))
    with np.errstate(all="ignore"):
        err = np.abs(fv(test)[ok] - fv(ref)[ok]) / fv(ref)[ok]
    err = np.where(np.isfinite(err), err, np.inf)
    best = lambda r: int(np.argmin(np.where(ok, fv(r), np.inf)))  # noqa: E731
    top = lambda r: set(np.argsort(np.where(ok, fv(r), np.inf))[:100].tolist())  # noqa: E731
    same = ((test["loss"] == ref["loss"]) & (test["rmse"] == ref["rmse"]) & (test["size"] == ref["size"]))
    return {"candidates_compared": int(len(ok)), "finite": int(ok.sum()),
            "bit_identical": int(same.sum()),
            "sentinel_agreement": float(np.mean((test["loss"] == 1000) == (ref["loss"] == 1000))),
            "size_agreement": float(np.mean(test["size"] == ref["size"])),
            "fitness_rel_err_median": float(np.median(err)) if len(err) else 0.0,
            "fitness_rel_err_p99": float(np.quantile(err, 0.99)) if len(err) else 0.0,
            "fitness_rel_err_max": float(err.max()) if len(err) else 0.0,
            "frac_within_1e-6": float(np.mean(err <= 1e-6)) if len(err) else 1.0,
            "argbest_same": best(test) == best(ref), "top100_overlap": len(top(test) & top(ref)) / 100.0}


def subset(out: dict, idx) -> dict:
    return {k: v[idx] for k, v in out.items() if k != "coefs"}


# ----------------------------------------------------------- multi-rank --
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = os.environ.get("BENCH_DIST_BACKEND", "nccl")
        if backend == "nccl":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    """Largest value of x over all ranks (the job's time is its slowest rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(units_per_rank: float, seconds: float, world: int) -> tuple[float, float]:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    t = max_over_ranks(seconds, world)
    return units_per_rank * world / t, t


# ------------------------------------------------------------------- ours --
def timed_rounds(ctx, ds, batches, prec, stream, flush):
    """One step: the rounds in order, each through the C ABI
    (rrg_round_submit + rrg_round_wait: host staging, every launch, results
    back in host memory), the whole step bracketed by CUDA events on the
    library's stream after an L2 flush; results are turned into Python
    objects after the timed region.  A step is one search's rounds: the
    column cache starts empty (cleared inside the timed region), so only the
    step's later rounds read columns its earlier rounds evaluated."""
    import torch

    from rils_rols_gb300.fitness import decode_results, result_dtype
    bufs = [(np.zeros(len(b), dtype=result_dtype()), np.zeros(max(1, b.n_coefs), dtype=np.float64)) for b in batches]
    gc.collect()
    gc.disable()  # no collector pause of the harness inside the timed region
    with torch.cuda.stream(stream):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
    ctx.clear_column_cache()
    for b, (res, coefs) in zip(batches, bufs):
        ds.submit(b, prec, res, coefs)
        ds.wait()
    with torch.cuda.stream(stream):
        e1.record(stream)
    e1.synchronize()
    gc.enable()
    return e0.elapsed_time(e1) / 1e3, [decode_results(r, c, b) for b, (r, c) in zip(batches, bufs)]


def concat_results(outs: list[dict]) -> dict:
    return {k: np.concatenate([o[k] for o in outs]) for k in ("loss", "rmse", "size", "rank", "flags")}


def run_ours(args):
    import torch

    from rils_rols_gb300.fitness import CERTIFIED, MIXED, PLAIN, Context, encode, tune_report

    rank, world = dist_setup()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    X, y = regression_data(args.n)
    rounds = load_rounds()
    trees = [t for r in rounds for t in r]
    B = len(trees)
    ctx = Context(local)
    ds = ctx.dataset(X, y)
    batches = [encode(r, tuned=True) for r in rounds]
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=torch.device("cuda", local))

    def phases_of_step(prec, bs=batches):
        """Per-phase device time, bytes, launches and statistics of one step,
        round by round (a separate, untimed pass with per-launch events)."""
        ctx.set_timing(True)
        ctx.clear_column_cache()
        pm, pb, launches, stats = {}, {}, 0, []
        for b in bs:
            ds.evaluate(b, prec)
            launches += ctx.last_round_launches()
            for k, (ms, cnt) in ctx.last_round_timing().items():
                pm[k] = pm.get(k, 0.0) + ms
            for k, v in ctx.last_round_bytes().items():
                pb[k] = pb.get(k, 0.0) + v
            stats.append(ctx.last_round_stats())
        ctx.set_timing(False)
        return pm, pb, launches, stats

    for _ in range(args.warmup):
        ctx.clear_column_cache()
        for b in batches:
            ds.evaluate(b, CERTIFIED)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        times = []
        cert_rounds = None
        for _ in range(args.steps):
            dt, cert_rounds = timed_rounds(ctx, ds, batches, CERTIFIED, stream, flush)
            times.append(dt)
    torch.cuda.synchronize()
    barrier(world)
    value, t_max = aggregate(B * args.steps, sum(times), world)
    cert = concat_results(cert_rounds)

    # e2e: trees in, fitness out, through the C ABI from host buffers
    Xp = torch.from_numpy(np.ascontiguousarray(X)).pin_memory().numpy()
    yp = torch.from_numpy(np.ascontiguousarray(y)).pin_memory().numpy()
    e2e_times = []
    for step in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        gc.collect()
        t = time.perf_counter()
        d2 = ctx.dataset(Xp, yp)
        for r in rounds:
            d2.evaluate(encode(r, tuned=True), CERTIFIED)
        d2.close()
        torch.cuda.synchronize()
        if step >= args.warmup:
            e2e_times.append(time.perf_counter() - t)
    e2e_value, _ = aggregate(B * args.steps, sum(e2e_times), world)
    h2d = X.nbytes + y.nbytes + sum(b.cands.nbytes + b.factors.nbytes + b.code.nbytes + b.consts.nbytes
                                    for b in batches)
    d2h = B * 32 + sum(b.n_coefs for b in batches) * 8

    # phases, launches and statistics of one step (untimed pass, per-launch events)
    phase_ms, phase_b, launches, stats = phases_of_step(CERTIFIED)
    if rank != 0:
        return
    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "df32/f64", "data": "synthetic (seeded)",
           "config": config(args.n, rounds),
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
           "gpu_launches": int(launches * args.steps), "gpu_launches_per_step": int(launches),
           "round_ms": [1e3 * t for t in times],
           "round_stats": {"fp64_rescored": sum(st["fp64_rescored"] for st in stats),
                           "plain_routed": sum(st["plain_routed"] for st in stats),
                           "residual_pass": sum(st["residual_pass"] for st in stats),
                           "qr_skipped_sentinel": sum(st["qr_skipped_sentinel"] for st in stats),
                           "rescore_reasons": {k: sum(st["rescore_reasons"].get(k, 0) for st in stats)
                                               for k in ctx.REASONS if any(k in st["rescore_reasons"] for st in stats)}}}
    res["phase_ms_per_step"] = {k: v for k, v in phase_ms.items() if v > 0}
    res["phase_bytes_per_step"] = {k: v for k, v in phase_b.items() if v > 0}
    res["roofline"] = roofline(res["phase_ms_per_step"], res["phase_bytes_per_step"])
    # secondary throughput: rows x tree nodes per second (nodes of each
    # candidate tree as submitted, every row)
    nodes = sum(len(t.split()) for t in trees)
    res["rows_nodes_per_s"] = nodes * float(args.n) * args.steps * world / t_max
    res["clocks"] = clk.summary()
    res["autotune"] = tune_report()
    res["column_cache"] = {
        "mode": "on (the library default), emptied at the start of every step: rounds 2-8 of a step read the "
                "factor columns that its earlier rounds evaluated, as the rounds of one search do",
        "double_float_columns_read": sum(st["cache_hits"] for st in stats),
        "double_float_columns_evaluated": sum(st["cache_evals"] for st in stats),
        "fp64_columns_read": sum(st["cache64_hits"] for st in stats),
        "fp64_columns_evaluated": sum(st["cache64_evals"] for st in stats),
        "pair_sums_read": sum(st["pair_hits"] for st in stats),
        "pair_sums_formed": sum(st["pair_evals"] for st in stats),
        "context_device_bytes": ctx.memory()}
    if args.quick:
        print(json.dumps(res))
        return
    # the same steps with the cache off: every round evaluates all its factors
    ctx.set_column_cache(False)
    ntimes = [timed_rounds(ctx, ds, batches, CERTIFIED, stream, flush)[0] for _ in range(max(2, args.steps // 2))]
    ctx.set_column_cache(True)
    res["column_cache"]["off_evals_per_s"] = B * len(ntimes) / sum(ntimes)
    # the eight rounds concatenated into one batch (one call)
    allb = encode(trees, tuned=True)
    ctimes = [timed_rounds(ctx, ds, [allb], CERTIFIED, stream, flush)[0] for _ in range(max(2, args.steps // 2))]
    res["concatenated_round_evals_per_s"] = B * len(ctimes) / sum(ctimes)
    # uncertified mixed form: the same rounds without the FP64 re-scoring of
    # rank-ambiguous candidates (does not meet the 1e-6 bar: reported only)
    mtimes = []
    for _ in range(max(2, args.steps // 2)):
        dt, mixed_rounds = timed_rounds(ctx, ds, batches, MIXED, stream, flush)
        mtimes.append(dt)
    mixed = concat_results(mixed_rounds)
    res["mixed_uncertified"] = {"evals_per_s": B * len(mtimes) / sum(mtimes),
                                "note": "no FP64 re-scoring: fitness errors above 1e-6 occur, see accuracy_vs_fp64"}
    # plain FP64: unbatched launches (one candidate per round, no column
    # cache: each candidate evaluated on its own) and the rounds
    singles = [encode([t], tuned=True) for t in trees[:args.unbatched_sample]]
    ctx.set_column_cache(False)
    ds.evaluate(singles[0], PLAIN)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for s1 in singles:
        ds.evaluate(s1, PLAIN)
    torch.cuda.synchronize()
    unbatched = len(singles) / (time.perf_counter() - t)
    ctx.set_column_cache(True)
    ptimes = []
    for _ in range(2):
        dt, plain_rounds = timed_rounds(ctx, ds, batches, PLAIN, stream, flush)
        ptimes.append(dt)
    plain = concat_results(plain_rounds)
    res["plain_fp64_unbatched_evals_per_s"] = unbatched
    res["plain_fp64_rounds_evals_per_s"] = B * len(ptimes) / sum(ptimes)
    res["certified_over_plain_unbatched"] = value / world / unbatched
    res["accuracy_vs_fp64"] = {"certified": accuracy(cert, plain), "mixed_uncertified": accuracy(mixed, plain),
                               "fitness": "(1 + (1 - R2)) (1 + RMSE) (1 + 0.001 size)"}
    # the CPU oracle on a seeded sample of the same candidates: its time is
    # the CPU baseline, its results the accuracy reference
    idx = sample_index(B, args.cpu_sample)
    res["cpu_baseline"], ora = cpu_baseline(X, y, trees, idx)
    res["accuracy_vs_oracle"] = {
        "sample": f"{len(idx)} seeded random candidates of the {B} (the CPU baseline's)",
        "plain_fp64": accuracy(subset(plain, idx), ora),
        "certified": accuracy(subset(cert, idx), ora),
        "mixed_uncertified": accuracy(subset(mixed, idx), ora)}
    res["certified_over_cpu_baseline"] = value / world / res["cpu_baseline"]["value"]
    # the reference runs single-threaded: the same oracle on one core
    one, _ = cpu_baseline(X, y, trees, sample_index(B, max(1, args.cpu_sample // 48), seed=6), threads=1)
    res["cpu_baseline_1core"] = one
    res["certified_over_cpu_1core"] = value / world / one["value"]
    res["target_500x_cpu"] = {"all_cores": res["certified_over_cpu_baseline"] >= 500,
                              "one_core": res["certified_over_cpu_1core"] >= 500}
    if args.fit_calls_1m > 0:
        res["regression_fit_1m"] = regression_fit_leg(X, y, args.fit_calls_1m)
    # standalone batched fitness: 8192 random trees (sizes 3..50 over + - * / sin
    # cos ln exp sqrt, leaves x_j or U(-5, 5)) on n = 100k rows, d = 10, X ~ N(0,1),
    # y = a random 15-node tree + 1% noise; certified and uncertified mixed
    # against the FP64 path and, on a sample, the oracle
    from rils_rols_gb300 import synth
    X2, y2, rtrees, _ = synth.batched_fitness(n=100_000, d=10, n_trees=8192, seed=SEED)
    ds2 = ctx.dataset(X2, y2)
    rb = encode(rtrees, tuned=True)
    ds2.evaluate(rb, CERTIFIED)
    rt = {}
    ctx.set_timing(True)
    for name, prec in (("certified", CERTIFIED), ("mixed_uncertified", MIXED), ("plain_fp64", PLAIN)):
        ts, out = [], None
        for _ in range(3):
            dt_, outs = timed_rounds(ctx, ds2, [rb], prec, stream, flush)
            ts.append(dt_)
            out = outs[0]
        rt[name] = {"evals_per_s": len(rtrees) / min(ts), "out": out, "round_stats": ctx.last_round_stats(),
                    "phase_ms": {k: v[0] for k, v in ctx.last_round_timing().items() if v[0] > 0}}
    ctx.set_timing(False)
    idx2 = sample_index(len(rtrees), args.cpu_sample // 2, seed=9)
    _, ora2 = cpu_baseline(X2, y2, rtrees, idx2)
    res["batched_fitness_8192_random_trees"] = {
        "config": "n=100000, d=10, 8192 random trees, sizes 3..50, tuned (best of 3 rounds)",
        **{k: {kk: v[kk] for kk in ("evals_per_s", "round_stats", "phase_ms")} for k, v in rt.items()},
        "accuracy_vs_fp64": {"certified": accuracy(rt["certified"]["out"], rt["plain_fp64"]["out"]),
                             "mixed_uncertified": accuracy(rt["mixed_uncertified"]["out"], rt["plain_fp64"]["out"])},
        "accuracy_vs_oracle": {"sample": f"{len(idx2)} seeded random trees of the 8192",
                               "plain_fp64": accuracy(subset(rt["plain_fp64"]["out"], idx2), ora2),
                               "certified": accuracy(subset(rt["certified"]["out"], idx2), ora2)}}
    ds2.close()
    # the serving and classifier legs make contexts of their own: this one's
    # tables and column caches go first
    ds.close()
    ctx.close()
    torch.cuda.synchronize()
    if args.serve_jobs > 0:
        res["serving"] = serving_leg(args, local)
    if args.cls_fit_calls > 0:
        res["classifier"] = classifier_leg(args)
    print(json.dumps(res))


def regression_fit_leg(X, y, calls, precision="mixed"):
    """A regression fit on the 1M-row data through the drop-in module
    (rils_rols_cpp.rils_rols, certified mixed precision unless `precision`
    is "plain"), max_fit_calls = `calls`: the search submits its own rounds,
    so evals/s here is what a fit sees (host search included in the wall
    time)."""
    import rils_rols_cpp
    n, d = X.shape
    m = rils_rols_cpp.rils_rols(False, calls, 1 << 30, 0.001, 50, 1.0, False, SEED % 100000)
    m.set_precision(precision)
    t = time.perf_counter()
    m.fit(X.reshape(-1), y, n, d)
    wall = time.perf_counter() - t
    cnt = m.counters()
    pred = m.predict(X.reshape(-1), n, d)
    r2 = 1 - float(np.sum((y - pred) ** 2) / np.sum((y - y.mean()) ** 2))
    return {"max_fit_calls": calls, "n_rows": n, "fit_s": wall, "fit_calls": m.get_fit_calls(),
            "rounds": cnt["device_rounds"], "candidates_scored": cnt["candidates_scored"],
            "backend_s": cnt["backend_ns"] / 1e9,
            "evals_per_s_backend": cnt["candidates_scored"] / max(1e-9, cnt["backend_ns"] / 1e9),
            "evals_per_s_wall": cnt["candidates_scored"] / wall, "model": m.get_model_string(), "train_r2": r2}


# ------------------------------------------------------------- serving ----
def serving_leg(args, device=0):
    """The serving stream (Poisson arrivals, mean 5/s; n log-uniform in
    [200, 1M], d in [1, 20], y a random 5-25-node tree + 1% noise,
    max_fit_calls 1e5): the first `serve_jobs` requests submitted at their
    arrival times to the serving loop in the certified mixed form (jobs in
    flight share the GPU).  On a prefix of `serve_serial` of those requests,
    the plain FP64 form both concurrently (its models must equal the same
    jobs run one after another) and one job after another (the serial
    baseline)."""
    from rils_rols_gb300 import synth
    from rils_rols_gb300._lib import RRG_MIXED_CERTIFIED, RRG_PLAIN_FP64
    from rils_rols_gb300.serve import Server
    jobs = synth.serving_stream(n_jobs=args.serve_jobs)
    data = [synth.serving_job_data(j) for j in jobs]
    params = dict(max_fit_calls=args.serve_fit_calls, max_seconds=1 << 30, complexity_penalty=0.001,
                  max_complexity=50, sample_size=1.0)

    def run(precision, max_active, paced, count):
        with Server(device=device, max_active=max_active) as srv:
            t0 = time.perf_counter()
            ids = []
            for j, (X, y) in list(zip(jobs, data))[:count]:
                if paced:
                    delay = j["arrival"] - (time.perf_counter() - t0)
                    if delay > 0:
                        time.sleep(delay)
                ids.append(srv.submit(X, y, random_state=j["seed"] % 100000, precision=precision, **params))
            out = [srv.result(i) for i in ids]
            wall = time.perf_counter() - t0
            st = srv.stats()
        return out, wall, st

    n_all = len(jobs)
    n_pre = min(args.serve_serial, n_all)
    conc, wall_c, st_c = run(RRG_MIXED_CERTIFIED, args.serve_active, True, n_all)
    concp, wall_cp, st_cp = run(RRG_PLAIN_FP64, args.serve_active, True, n_pre)
    ser, wall_s, st_s = run(RRG_PLAIN_FP64, 1, False, n_pre)
    ttm = sorted(i["time_to_model_s"] for _, i in conc)
    run_s = [i["run_s"] for _, i in ser]
    return {
        "requests": n_all, "arrivals": "Poisson, mean 5/s (the first requests of the 1000-request stream)",
        "max_fit_calls": args.serve_fit_calls, "n_rows_max": max(j["n"] for j in jobs),
        "n_features_max": max(j["d"] for j in jobs),
        "concurrent_certified": {"requests": n_all, "max_active": args.serve_active,
                                 "p50_time_to_model_s": st_c["p50_time_to_model_s"],
                                 "p99_time_to_model_s": st_c["p99_time_to_model_s"],
                                 "mean_time_to_model_s": st_c["mean_time_to_model_s"], "wall_s": wall_c,
                                 "fits_per_hour": 3600.0 * n_all / wall_c, "evals_per_s": st_c["candidates"] / wall_c,
                                 "peak_running": st_c["peak_running"], "done": st_c["done"],
                                 "failed": st_c["failed"], "time_to_model_s": ttm},
        "prefix_requests": n_pre,
        "concurrent_plain_fp64_prefix": {"max_active": args.serve_active, "p50_time_to_model_s":
                                         st_cp["p50_time_to_model_s"],
                                         "p99_time_to_model_s": st_cp["p99_time_to_model_s"], "wall_s": wall_cp,
                                         "fits_per_hour": 3600.0 * n_pre / wall_cp,
                                         "evals_per_s": st_cp["candidates"] / wall_cp},
        "serial_plain_fp64_prefix": {"wall_s": wall_s, "sum_run_s": sum(run_s),
                                     "fits_per_hour": 3600.0 * n_pre / wall_s,
                                     "evals_per_s": st_s["candidates"] / wall_s},
        # a job's model is the same alone and in the mix (plain FP64: bit-identical search)
        "plain_models_same_alone_and_in_mix": f"{sum(a[0] == b[0] for a, b in zip(concp, ser))}/{n_pre}",
        "certified_models_equal_plain": f"{sum(a[0] == b[0] for a, b in zip(conc, ser))}/{n_pre}",
    }


# ----------------------------------------------------------- classifier ----
def classifier_leg(args):
    """Binary classifier fits (d = 30 correlated lognormal features, labels =
    a random 10-node tree > 0 with 5% flipped; max_complexity 20,
    sample_size 1): n = 569 on the device in FP64 and certified form and on
    the host with the oracle as fitness backend (the reference's CPU path);
    n = 200k on the device, FP64 against certified."""
    import rils_rols_cpp
    from rils_rols_gb300 import synth
    out = {}
    for n, calls in ((569, 100000), (200_000, args.cls_fit_calls)):
        X, lab, _ = synth.classifier(n=n, d=30, seed=SEED)
        row = {"max_fit_calls": calls}
        # the device FP64 fit with its rounds as CUDA graphs beside the
        # directly launched one (same search, same model)
        arms = [("plain_fp64", "plain", None, False), ("plain_fp64_graph", "plain", None, True),
                ("certified", "mixed", None, False)]
        if n <= 5000:
            from oracle import pyoracle
            arms.append(("cpu_oracle", "plain", pyoracle.backend_struct(), False))
        # an untimed fit first: context, tuner trials and module loading are
        # paid there, not by whichever arm happens to run first
        w = rils_rols_cpp.rils_rols(True, min(calls, 5000), 1 << 30, 0.001, 20, 1.0, False, SEED % 100000)
        w.fit(X.reshape(-1), lab, n, X.shape[1])
        for name, prec, backend, graph in arms:
            m = rils_rols_cpp.rils_rols(True, calls, 1 << 30, 0.001, 20, 1.0, False, SEED % 100000)
            m.set_precision(prec)
            if graph:
                m.set_graph(True)
            if backend is not None:
                m.set_backend(backend)
            t = time.perf_counter()
            m.fit(X.reshape(-1), lab, n, X.shape[1])
            dt = time.perf_counter() - t
            cnt = m.counters()
            pred = m.predict(X.reshape(-1), n, X.shape[1])
            row[name] = {"fit_s": dt, "fit_calls": m.get_fit_calls(), "model": m.get_model_string(),
                         "train_accuracy": float(np.mean(pred == lab)),
                         # wall time inside the fitness backend; the rest is the host search
                         "backend_s": cnt["backend_ns"] / 1e9, "rounds": cnt["device_rounds"],
                         "candidates": cnt["candidates_scored"]}
        if "cpu_oracle" in row:
            row["device_fp64_equals_cpu"] = row["plain_fp64"]["model"] == row["cpu_oracle"]["model"]
        row["certified_equals_fp64"] = row["certified"]["model"] == row["plain_fp64"]["model"]
        row["graph_equals_fp64"] = row["plain_fp64_graph"]["model"] == row["plain_fp64"]["model"]
        out[f"n={n}"] = row
    return out


# kernels behind the timed phases (the roofline candidates)
PHASE_KERNELS = {
    "factor_eval": "fac_eval_kernel (double-float factor table)",
    "pair_sums": "pair_sum_kernel",
    "fp64_eval": "plain_eval_kernel (FP64 table)",
    "fp64_qr": "qr_passA_kernel + qr_sums_kernel (column-pivoted QR, FP64, chunked passes over the GPU)",
}


def roofline(phase_ms, phase_bytes):
    """Roofline of the phase with the largest device time in one round.  A
    "launch" here is that phase's kernels of one round; its bytes are the
    algorithmic ones the library counts (rrg_last_round_bytes), its time the
    CUDA-event phase time on the library's stream.  `traffic` scales them by
    the DRAM/algorithmic ratio of the committed ncu capture of the same
    kernels (profiles/<phase>_1m.txt); these kernels are FP64- or
    FP32-pipe-bound (the `pipe` figure of that capture), so their HBM
    fraction is small by construction."""
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    cand = {k: v for k, v in phase_ms.items() if k in PHASE_KERNELS}
    if not cand:
        return None
    top = max(cand, key=cand.get)
    ms = cand[top]
    algo = phase_bytes.get(top)
    achieved = algo / (ms / 1e3) / 1e9 if algo else None
    prof = read_profile(top) or {}
    ratio = prof.get("dram_over_algorithmic")
    return {"kernel": PHASE_KERNELS[top], "phase": top, "bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
            "traffic": ratio * algo if (ratio and algo) else None, "algorithmic_bytes": algo, "ms_per_launch": ms,
            "peak_source": "measured" if peaks else "fallback", "pipe": prof.get("pipe")}


def read_profile(phase):
    """`key=value` lines of the committed ncu summary of the phase's kernels."""
    p = ROOT / "profiles" / f"{phase}_1m.txt"
    if not p.exists():
        return None
    out = {}
    for line in p.read_text().splitlines():
        if "=" in line and not line.startswith(" ") and line.split("=")[0] in ("dram_over_algorithmic", "pipe"):
            k, v = line.split("=", 1)
            v = v.strip()
            try:
                out[k] = float(v.split()[0])
            except ValueError:
                out[k] = v
    return out


# -------------------------------------------------------------- reference --
REF_LIB = ROOT / "oracle" / "_ref" / "librr_ref.so"


def reference_scorer(X, y, threads):
    """A function scoring a list of prefix trees on the CPU with `threads`
    host threads and a description of what it runs: the reference's own
    tune_constants + fitness (oracle/_ref/librr_ref.so, compiled from the
    reference's sources, where this host built it), else the oracle port
    (oracle/rrg_oracle.c with the oracle's own encoder).  Neither loads the
    product library."""
    import ctypes as C
    from concurrent.futures import ThreadPoolExecutor
    n, d = X.shape
    lib = None
    if REF_LIB.exists():
        try:
            lib = C.CDLL(str(REF_LIB))
        except OSError:
            lib = None
    if lib is not None:
        Xc = np.ascontiguousarray(X.T)
        yc = np.ascontiguousarray(y)
        dp = C.POINTER(C.c_double)

        def one(tree):
            out3 = (C.c_double * 3)()
            buf = C.create_string_buffer(1 << 16)
            # ctypes releases the GIL for the call: the threads run in parallel
            lib.ref_tune_fitness(Xc.ctypes.data_as(dp), yc.ctypes.data_as(dp), n, d, tree.encode(), 1, 0, out3,
                                 buf, len(buf))
            return out3[0]

        pool = ThreadPoolExecutor(threads)

        def score(trees):
            list(pool.map(one, trees))
        return score, "reference", "the reference's own tune_constants + fitness (oracle/_ref/librr_ref.so)"
    from oracle import pyoracle, tree_encode
    ods = pyoracle.OracleDataset(X, y)

    def score(trees):
        ods.evaluate(tree_encode.encode(trees, tuned=True), threads=threads)
    return score, "port", "the oracle (oracle/rrg_oracle.c, trees flattened by oracle/tree_encode.py)"


def run_reference(args):
    """The reference's CPU path on this workload, all host threads, a bounded
    seeded sample of the rounds' candidates per step (no product code is
    loaded in this process)."""
    rank, world = dist_setup()
    if rank != 0:
        return
    X, y = regression_data(args.n)
    rounds = load_rounds()
    trees = [t for r in rounds for t in r]
    threads = os.cpu_count() or 1
    score, kind, what = reference_scorer(X, y, threads)
    sample = min(args.ref_sample, len(trees))
    rng = np.random.default_rng(7)
    times = []
    for step in range(args.warmup + args.steps):
        pick = [trees[i] for i in rng.choice(len(trees), sample, replace=False)]
        t = time.perf_counter()
        score(pick)
        dt = time.perf_counter() - t
        if step >= args.warmup:
            times.append(dt)
    value = sample * len(times) / sum(times)
    desc = (f"{sample} seeded random candidates of the {len(trees)} per step at n={args.n}, FP64, {threads} threads; "
            f"{what}")
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic (seeded)", "config": config(args.n, rounds),
                      "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": desc},
                      "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def round_only(args):
    """One headline round, certified, on a fresh context: phase times (CUDA
    events), the library's algorithmic bytes and the kernels launched."""
    import torch
    from rils_rols_gb300.fitness import CERTIFIED, Context, encode
    X, y = regression_data(args.n)
    rounds = load_rounds()
    ctx = Context(0)
    ds = ctx.dataset(X, y)
    trees = [t for r in rounds for t in r] if args.round_only == len(rounds) else rounds[args.round_only]
    b = encode(trees, tuned=True)
    torch.cuda.synchronize()
    ctx.set_timing(True)
    ds.evaluate(b, CERTIFIED)
    ctx.set_timing(False)
    out = {"round": args.round_only if args.round_only < len(rounds) else "all eight concatenated",
           "candidates": len(trees), "n": args.n,
           "phase_ms": {k: v[0] for k, v in ctx.last_round_timing().items() if v[0] > 0},
           "phase_bytes": {k: v for k, v in ctx.last_round_bytes().items() if v > 0},
           "launches": ctx.last_round_launches(), "stats": ctx.last_round_stats()}
    ds.close()
    ctx.close()
    print(json.dumps(out))


def eval_case(args):
    """The double-float factor evaluator on a named case with the tensor-copy
    staging knob pinned (1: X and y from global memory, 2: staged)."""
    from rils_rols_gb300 import synth
    from rils_rols_gb300.fitness import CERTIFIED, FAC_STAGE, Context, encode, tune_pin
    if args.case == "local_search_d5":
        X, y = regression_data(args.n)
        batches = [encode(r, tuned=True) for r in load_rounds()]
    else:
        d = 10 if args.case == "random_d10" else 20
        rng = np.random.default_rng(SEED)
        X = rng.standard_normal((args.n, d))
        _, y = synth.finite_target(rng, X, 15)
        y = y + rng.normal(0, 0.01 * np.std(y), args.n)
        batches = [encode([synth.random_tree(rng, int(rng.integers(3, 30)), d) for _ in range(1500)], tuned=True)]
    d = X.shape[1]
    if args.fac_stage:
        tune_pin(FAC_STAGE, min(d, 64), args.fac_stage)
    ctx = Context(0)
    ctx.set_mixed_min_rows(0)
    ctx.set_column_cache(False)  # every step evaluates every factor: the evaluator is what is timed
    ds = ctx.dataset(X, y)
    for b in batches:
        ds.evaluate(b, CERTIFIED)
    steps = []
    for _ in range(max(1, args.steps)):
        ctx.set_timing(True)
        fe, tot = 0.0, 0.0
        for b in batches:
            t = time.perf_counter()
            ds.evaluate(b, CERTIFIED)
            tot += time.perf_counter() - t
            fe += ctx.last_round_timing()["factor_eval"][0]
        ctx.set_timing(False)
        steps.append({"factor_eval_ms": fe, "rounds_ms": 1e3 * tot})
    ds.close()
    ctx.close()
    print(json.dumps({"case": args.case, "n": args.n, "d": d, "fac_stage": args.fac_stage, "steps": steps}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_ROWS)
    ap.add_argument("--cpu-sample", type=int, default=2400, help="oracle sample of the CPU baseline")
    ap.add_argument("--ref-sample", type=int, default=384, help="candidates per step of the reference arm")
    ap.add_argument("--fit-calls-1m", type=int, default=100000,
                    help="max_fit_calls of the regression fit at n = 1M (0: no fit leg)")
    ap.add_argument("--unbatched-sample", type=int, default=64)
    ap.add_argument("--quick", action="store_true", help="skip the FP64 comparison and the CPU baseline")
    ap.add_argument("--serve-jobs", type=int, default=200, help="requests of the serving stream (0: no serving leg)")
    ap.add_argument("--serve-serial", type=int, default=8,
                    help="prefix of the requests also run in plain FP64, concurrently and one after another")
    ap.add_argument("--serve-fit-calls", type=int, default=100000)
    ap.add_argument("--serve-active", type=int, default=16)
    ap.add_argument("--serve-only", action="store_true", help="only the serving leg")
    ap.add_argument("--fit-only", action="store_true",
                    help="only the 1M-row regression fit, certified mixed and plain FP64 (the drop-in default)")
    ap.add_argument("--cls-fit-calls", type=int, default=20000,
                    help="max_fit_calls of the 200k-row classifier fits (0: no classifier leg)")
    ap.add_argument("--cls-only", action="store_true", help="only the classifier leg")
    ap.add_argument("--round-only", type=int, default=-1, help="one headline round alone (profiling)")
    ap.add_argument("--case", choices=["local_search_d5", "random_d10", "random_d20"],
                    help="the factor evaluator on a named case (profiling)")
    ap.add_argument("--fac-stage", type=int, default=0, choices=[0, 1, 2],
                    help="with --case: 1 reads X and y from global memory, 2 stages them by tensor copies")
    args = ap.parse_args()
    if args.round_only >= 0:
        round_only(args)
        return
    if args.case:
        eval_case(args)
        return
    if args.serve_only:
        print(json.dumps(serving_leg(args)))
        return
    if args.fit_only:
        X, y = regression_data(args.n)
        print(json.dumps({p: regression_fit_leg(X, y, args.fit_calls_1m, p) for p in ("mixed", "plain")}))
        return
    if args.cls_only:
        print(json.dumps(classifier_leg(args)))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
