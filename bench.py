"""Benchmark of the batch-Hogwild SGD path (one JSON line on rank 0).

Workload (the c2 shape): planted-model matrix 480,189 x 17,770 with 99,072,112 train
ratings, k = 128, fp16 factors, 20 epochs, synthetic (seeded) in place of Netflix.
  value  updates/s = nnz * epochs / time, epochs run on device-resident data (one epoch =
         one step = one kernel launch), CUDA events on the launching stream;
  e2e    the same metric through the C ABI (cumf_train: pinned host ratings in, fp32 model
         out, 20 epochs including H2D, prep, export and D2H);
  roofline   algorithmic bytes of the update kernel (12 + 4k bytes per sample) / launch time
             against the measured HBM copy bandwidth;
  cpu_baseline  the oracle's threaded CPU port of the same algorithm (fp32) on the host cores;
  time_to_target  the second half of the metric: c2-shape growth scenario, cold fp16 SGD
             against the learned warm start with bf16 stochastic rounding (see
             run_warmstart_suite), time to reach the FP64 oracle's test RMSE + 0.002.
`--impl reference` times that CPU port alone as the reference arm (the reference's own
binaries are x86 builds of this container and do not exist on the GPU host).
Multi-GPU (torchrun): independent replicas, one per GPU (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

K = 128
BYTES_PER_SAMPLE = {"fp16": 12 + 4 * K * 2, "bf16": 12 + 4 * K * 2, "bf16sr": 12 + 4 * K * 2,
                    "fp16sr": 12 + 4 * K * 2, "fp32": 12 + 4 * K * 4}
WORKLOAD = "c2 planted 480189x17770, 99072112 train ratings, k=128"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world: int) -> None:
    """One process per GPU under torchrun: NCCL with CUDA, gloo without (CPU tests)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, world: int) -> float:
    """The largest value over all ranks (the slowest replica's time), returned on every rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def l2_copy_gbs(bytes_each: int = 16 << 20, passes: int = 400) -> float:
    """L2-resident copy bandwidth (bytes read + written): `passes` copies of a 16 MB buffer
    into another inside one launch (cumf_probe_copy_bandwidth).  Measured on GB300: 12.3-13.9
    TB/s for 8-48 MB buffers, 9.4 TB/s at 64 MB (spilling), 6.5-6.6 TB/s at 1-4 GB (HBM)."""
    import ctypes as C
    from cumf_sgd_gb300 import _lib
    out = C.c_double(0)
    _lib.check(_lib.load().cumf_probe_copy_bandwidth(bytes_each, passes, C.byref(out), None))
    return out.value


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# Copies of the most-rated rows (cumf_params.hot_rows): off in the library by default (the
# reference's update), on in these measurements at 0.5 expected workers per copy, the setting
# measured for the skewed item popularity of the c2 shape (same or lower test RMSE there, which
# every line reports beside the throughput); --hot-rows 0 measures without them.
BENCH_HOT_ROWS = 0.5


def hot_rows_of(args) -> float:
    v = getattr(args, "hot_rows", None)
    return BENCH_HOT_ROWS if v is None else float(v)


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the update kernel
# at the c2 shape in the default configuration (one fp16 epoch, 97,280 workers, 99.61M samples,
# row copies, no L2 prefetch), from one ncu capture of this kernel.  A constant: ncu cannot run
# inside the timed bench, and the capture is redone whenever the kernel or the defaults change;
# other configurations report no traffic.
UPDATE_KERNEL_DRAM_BYTES_C2 = 18.341e9
UPDATE_KERNEL_DRAM_BYTES_SOURCE = ("ncu capture of one c2 fp16 launch of sgd_hogwild_kernel<128,fp16,16>, "
                                   "97,280 workers, row copies, prefetch 0: 9.057 GB read + 9.284 GB written")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join("/tmp", f"cumf_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_port_baseline(train: np.ndarray, m: int, n: int, seconds_budget: float = 12.0):
    """Threaded CPU port (oracle) of the batch-Hogwild update on a bounded sample of the
    workload: fp32 factors of the full c2 shape; each pass gives every worker one batch of
    128 consecutive ratings from a rotating window of the c2 train set; passes repeat until
    about `seconds_budget` seconds of work are done."""
    from oracle import oracle
    oracle.build_oracle()
    threads = os.cpu_count() or 1
    lr = oracle.lr_table(0.08, 0.3, 0.0, 8)
    P = oracle.init_factors(m, K, "fp32", 1, 1)
    Q = oracle.init_factors(n, K, "fp32", 1, 2)
    nnz = len(train)
    workers = max(1, min(threads * 64, nnz // 128))
    win = workers * 128
    samples = passes = 0
    t0 = time.perf_counter()
    while True:
        start = (passes * 7919 * 128) % max(1, nnz - win + 1)
        oracle.hogwild_threads(train[start:start + win], P, Q, workers, lr, 0, 1, 0.05, 0.05, 1 + passes,
                               threads)
        samples += win
        passes += 1
        el = time.perf_counter() - t0
        if el >= seconds_budget:
            break
    return {"value": samples / el, "unit": "updates/s", "cores": threads, "kind": "port",
            "sample": f"{samples} Hogwild updates ({passes} passes x {workers} workers x 128) over "
                      f"windows of the c2 train set, fp32 factors 480189x128 / 17770x128, {el:.1f} s"}


def _reference_tools():
    """oracle/ref_tools with the reference trainers built (on the GPU host from the sources
    that oracle/ref_build.sh staged), or None."""
    from oracle import oracle, ref_tools
    try:
        oracle.build_reference()
    except Exception as e:  # reported by the caller as "not available"
        print(json.dumps({"note": "reference tools not built", "why": repr(e)[:300]}), file=sys.stderr)
    return ref_tools if ref_tools.available("mf-train", "mf-predict") else None


def libmf_baseline(ref_tools, train, iters: int, threads: int, tmpdir: str, warm_iters: int = 0,
                   test=None) -> dict:
    """LIBMF mf-train (test/mf-train.cpp; the reference's CPU trainer) on the host cores:
    `threads` threads, 2*threads+1 blocks, k=128, l2 0.05, `iters` iterations over `train`.
    With warm_iters > 0 a first run of warm_iters iterations is subtracted, so the rate is
    that of iterations warm_iters+1 .. iters (its "computation time" excludes file reading).
    Returns updates/s and, with `test`, the RMSE printed by mf-predict -e 0."""
    tr_path = os.path.join(tmpdir, "libmf_train.bin")
    mp = os.path.join(tmpdir, "libmf.model")
    ref_tools.write_records(train, tr_path)
    t_warm = 0.0
    if warm_iters > 0:
        w = ref_tools.run_libmf(tr_path, mp, warm_iters, threads)
        if w["rc"] != 0 or w["computation_s"] is None:
            raise RuntimeError("mf-train failed: " + w["tail"])
        t_warm = w["computation_s"]
    r = ref_tools.run_libmf(tr_path, mp, iters, threads)
    if r["rc"] != 0 or r["computation_s"] is None:
        raise RuntimeError("mf-train failed: " + r["tail"])
    timed = iters - warm_iters
    secs = r["computation_s"] - t_warm
    out = {"value": len(train) * timed / secs, "unit": "updates/s", "cores": threads, "kind": "reference",
           "perf_line": r["perf"], "computation_s": r["computation_s"], "timed_iterations": timed,
           "timed_s": secs, "build": ref_tools.build_info()}
    if test is not None:
        te_path = os.path.join(tmpdir, "libmf_test.bin")
        ref_tools.write_records(test, te_path)
        out["test_rmse_mf_predict"] = ref_tools.libmf_rmse(te_path, mp)
        out["model_path"] = mp
    return out


def run_reference_arm(args):
    """The reference's own CPU trainer, LIBMF mf-train, on the host cores (rank 0 only):
    W warm-up iterations, then K timed iterations over the c2 train set (for K > 30 a uniform
    sample of 30/K of the ratings, so the arm stays within a few minutes).  Falls back to the
    oracle's threaded port of the batch-Hogwild update when mf-train could not be built."""
    import tempfile
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from cumf_sgd_gb300 import synth
    t0 = time.time()
    train, test = synth.generate(synth.C2, seed=0, device="cuda" if _has_cuda() else "cpu")
    gen_s = time.time() - t0
    threads = os.cpu_count() or 1
    ref_tools = _reference_tools()
    line = {"impl": "reference", "metric": "sgd_updates_per_sec", "unit": "updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "gen_seconds": gen_s}
    if ref_tools is not None:
        frac = min(1.0, 30.0 / max(1, args.steps))
        sample = train
        if frac < 1.0:
            keep = np.random.default_rng(0).random(len(train)) < frac
            sample = train[keep]
        with tempfile.TemporaryDirectory() as tmp:
            base = libmf_baseline(ref_tools, sample, args.warmup + args.steps, threads, tmp,
                                  warm_iters=args.warmup, test=test if frac == 1.0 else None)
        v = base["value"]
        line.update({"value": v, "ms_per_step": len(sample) / v * 1e3,
                     "config": {"workload": WORKLOAD, "trainer": "LIBMF mf-train (test/mf-train.cpp)", "k": K,
                                "threads": threads, "blocks": 2 * threads + 1, "l2": 0.05,
                                "step": "one LIBMF iteration over the train set" +
                                        ("" if frac == 1.0 else f" (uniform {frac:.3f} sample)")},
                     "test_rmse": base.get("test_rmse_mf_predict"),
                     "cpu_baseline": {**{k2: base[k2] for k2 in ("value", "unit", "cores", "kind", "build")},
                                      "sample": f"{len(sample)} ratings x {args.steps} timed iterations "
                                                f"(after {args.warmup} warm-up iterations), {threads} threads"}})
    else:
        per_step = []
        budget = max(2.0, 60.0 / (args.warmup + args.steps))  # whole arm: about a minute of CPU work
        for i in range(args.warmup + args.steps):
            b = cpu_port_baseline(train, synth.C2.m, synth.C2.n, seconds_budget=budget)
            if i >= args.warmup:
                per_step.append(b)
        v = statistics.mean(b["value"] for b in per_step)
        line.update({"value": v, "config": {"workload": WORKLOAD, "storage": "fp32 (CPU port)", "k": K},
                     "cpu_baseline": dict(per_step[-1], value=v),
                     "note": "LIBMF mf-train not built on this host (no reference sources): oracle port timed"})
    line["e2e"] = {"value": line["value"], "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)


def run_precision_suite(args):
    """Precision sweep (the c3 shape): planted matrix 1,000,990 x 624,961, 252.8M
    train / 4.0M test ratings on 0..100, k=128, 20 epochs, for fp32 / fp16 / bf16 / bf16
    with stochastic rounding / fp16 with stochastic rounding storage (fp32 arithmetic).
    Full size: throughput and test RMSE per storage type.  Gap to the serial FP64 oracle:
    on a 1% user subsample (users whose relabelled id is a multiple of 100), every GPU
    variant and the FP64 oracle train the same sub-problem with the same worker count and
    report test RMSE.  Prints one JSON line per measurement."""
    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth, build
    from oracle import oracle
    build.build()
    oracle.build_oracle()
    spec = synth.C3 if args.scale >= 1.0 else synth.scaled(synth.C3, args.scale)
    t0 = time.time()
    train, test = synth.generate(spec, seed=0, device="cuda")
    print(json.dumps({"suite": "precision", "event": "generated", "nnz": len(train), "secs": time.time() - t0}),
          flush=True)
    sm, _, _ = cm.device_info(0)
    precs = ["fp32", "fp16", "bf16", "bf16sr", "fp16sr"]
    epochs = args.e2e_epochs
    if not args.no_e2e:
        prob = cm.MFProblem.from_arrays(train["u"], train["v"], train["r"], m=spec.m, n=spec.n, pinned=True)
        tprob = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"])
        W = cm.auto_workers(len(train), sm, K, "fp32")  # one worker count for every storage type
        for prec in precs:
            par = cm.Parameter(k=K, num_workers=W, num_iters=epochs, alpha=0.08, beta=0.3, seed=1, gpu=0,
                               precision=prec)
            model, st = cm.sgd_train(prob, None, par, with_stats=True)
            print(json.dumps({"suite": "precision", "config": "c3 full", "precision": prec, "workers": W,
                              "epochs": epochs, "train_ms": st.train_ms,
                              "updates_per_sec": len(train) * epochs / (st.train_ms * 1e-3),
                              "test_rmse": cm.calc_rmse(tprob, model)}), flush=True)
            del model
        del prob
    # 1% user subsample: compact user ids, keep item ids.
    keep_tr = train["u"] % 100 == 0
    keep_te = test["u"] % 100 == 0
    sub_tr, sub_te = train[keep_tr].copy(), test[keep_te].copy()
    sub_tr["u"] //= 100
    sub_te["u"] //= 100
    m_sub = (spec.m + 99) // 100
    W = cm.auto_workers(len(sub_tr), sm, K, "fp16")
    t0 = time.time()
    P, Q, b = oracle.train_f64(sub_tr, m_sub, spec.n, k=K, num_workers=W, num_iters=epochs, alpha=0.08,
                               beta=0.3, seed=1)
    ref = oracle.calc_rmse_f64(sub_te, P, Q, b)
    print(json.dumps({"suite": "precision", "config": "c3 1% users", "precision": "fp64 oracle (CPU, serial)",
                      "nnz": len(sub_tr), "workers": W, "test_rmse": ref, "secs": time.time() - t0}), flush=True)
    prob = cm.MFProblem.from_arrays(sub_tr["u"], sub_tr["v"], sub_tr["r"], m=m_sub, n=spec.n)
    tprob = cm.MFProblem.from_arrays(sub_te["u"], sub_te["v"], sub_te["r"])
    for prec in precs:
        par = cm.Parameter(k=K, num_workers=W, num_iters=epochs, alpha=0.08, beta=0.3, seed=1, gpu=0,
                           precision=prec)
        r = cm.calc_rmse(tprob, cm.sgd_train(prob, None, par))
        print(json.dumps({"suite": "precision", "config": "c3 1% users", "precision": prec, "workers": W,
                          "test_rmse": r, "gap_to_fp64": r - ref}), flush=True)


def run_warmstart_suite(args, quiet=False):
    """Learned warm start (the c1-family scenario; with --scale 2 the c2-shape headline).

    Scenario: a deployed model exists for a base matrix (c1 or c2 shape); 50,000 new users
    arrive with ratings amounting to 5% of the base train count (one planted model for all).
      1. MLP training data: 8 plain-SGD solves (fp16, 20 epochs) of planted matrices of the
         same family with other seeds; per user, features from (ratings, solved Q), target the
         solved P row.  The MLP trains on the tensor cores (cumf_mlp_train).
      2. Base model: plain fp16 SGD on the base matrix (not timed: the deployed model, kept
         in device memory).
      3. Target: the FP64 oracle trained from scratch on the grown matrix for 20 epochs (serial
         at c1 shape; at c2 shape its batches run on all host cores) + 0.002.
      4. Cold start: plain fp16 SGD from random init on the grown matrix (up to 40 epochs).
         Warm start: base P for old users, MLP(features) for new users, base Q, refined with the
         given storage and initial learning rate, the first epochs over the new users' ratings
         only (the tail of the rating array); its time includes feature extraction and MLP
         inference on device-resident data.  Ablation: random rows for new users (no MLP).
    Time-to-target = cumulative CUDA-event training time up to the first epoch whose test
    RMSE <= target (evaluation excluded) + the warm start's preparation time."""
    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth, build
    from oracle import oracle
    build.build()
    oracle.build_oracle()
    dev = torch.device("cuda", 0)
    sm, _, _ = cm.device_info(0)
    big = args.scale >= 2.0
    base_spec = synth.C2 if big else synth.C1
    new_users = 50_000
    results = []

    def out(d):
        results.append(d)
        if not quiet:
            print(json.dumps({"suite": "warmstart", "shape": "c2" if big else "c1", **d}), flush=True)

    def solve(tr, m, n, seed, precision="fp16", iters=20, init=None, te=None, alpha=0.08, tail_epochs=0,
              tail_start=0, beta=0.3):
        prob = cm.MFProblem.from_arrays(tr["u"], tr["v"], tr["r"], m=m, n=n)
        tprob = cm.MFProblem.from_arrays(te["u"], te["v"], te["r"]) if te is not None else None
        W = cm.auto_workers(len(tr), sm, K, precision)
        par = cm.Parameter(k=K, num_workers=W, num_iters=iters, alpha=alpha, beta=beta, seed=seed, gpu=0,
                           precision=precision, tail_epochs=tail_epochs, tail_start=tail_start,
                           hot_rows=hot_rows_of(args))
        return cm.sgd_train_ex(prob, tprob, par, init)

    def features(dR, nnz, m, n, dQ):
        dX = torch.empty(m, K + 3, device=dev)
        cm.user_features(dR.data_ptr(), nnz, dQ.data_ptr(), n, K, m, dX.data_ptr())
        return dX

    # 1. MLP training data from 8 solves of the same family
    t0 = time.time()
    Xs, Ts = [], []
    for s in range(8):
        tr, _ = synth.generate(base_spec, seed=10 + s, device="cuda")
        model, _, _, _ = solve(tr, base_spec.m, base_spec.n, seed=10 + s)
        dR = torch.from_numpy(tr.view(np.uint8).copy()).to(dev)
        X = features(dR, len(tr), base_spec.m, base_spec.n, torch.from_numpy(np.ascontiguousarray(model.Q)).to(dev))
        keep = torch.from_numpy(np.nonzero(np.bincount(tr["u"], minlength=base_spec.m) > 0)[0]).to(dev)
        Xs.append(X[keep])
        Ts.append(torch.from_numpy(np.ascontiguousarray(model.P)).to(dev)[keep])
    X = torch.cat(Xs).contiguous()
    T = torch.cat(Ts).contiguous()
    mlp = cm.MLP(K + 3, 512, K, seed=7)
    probe = min(len(X), 65536)
    loss0 = mlp.loss_grad(X.data_ptr(), T.data_ptr(), probe)
    torch.cuda.synchronize()
    t1 = time.time()
    loss = mlp.train(X.data_ptr(), T.data_ptr(), len(X), epochs=args.mlp_epochs, batch=4096 if big else 1024,
                     lr=1e-3, seed=3)
    torch.cuda.synchronize()
    out({"event": "mlp_trained", "rows": len(X), "loss_before": loss0, "loss_after": loss,
         "train_s": time.time() - t1, "data_s": t1 - t0})
    # One untimed inference over a full 65,536-row chunk sizes the network's forward workspace
    # (a one-time allocation of the deployed model, like the warm-up steps of the other legs).
    probe_rows = min(len(X), 65536)
    probe_out = torch.empty(probe_rows, K, device=dev)
    mlp.forward(X.data_ptr(), probe_rows, probe_out.data_ptr())
    torch.cuda.synchronize()
    del X, T, Xs, Ts, probe_out

    # 2. base + growth from one planted model; the deployed base model lives on the device
    b_tr, b_te, n_tr, n_te = synth.generate_growth(base_spec, new_users, 0.05, seed=100, device="cuda")
    m_all, n = base_spec.m + new_users, base_spec.n
    base_model, _, _, _ = solve(b_tr, base_spec.m, n, seed=1)
    base_P = torch.from_numpy(np.ascontiguousarray(base_model.P)).to(dev)
    base_Q = torch.from_numpy(np.ascontiguousarray(base_model.Q)).to(dev)
    g_tr = np.concatenate([b_tr, n_tr])
    g_te = np.concatenate([b_te, n_te])
    d_gtr = torch.from_numpy(g_tr.view(np.uint8).copy()).to(dev)
    out({"event": "data", "base_train": len(b_tr), "new_train": len(n_tr), "test": len(g_te),
         "new_test": len(n_te), "users": m_all, "items": n})

    # 3. FP64 target
    t0 = time.time()
    W = cm.auto_workers(len(g_tr), sm, K, "fp16")
    threads = 1 if not big else (os.cpu_count() or 1)
    P64, Q64, b64 = oracle.train_f64(g_tr, m_all, n, k=K, num_workers=W, num_iters=20, seed=5, threads=threads)
    oracle_rmse = oracle.calc_rmse_f64(g_te, P64, Q64, b64)
    target = oracle_rmse + 0.002
    out({"event": "oracle", "fp64_test_rmse": oracle_rmse, "target": target, "host_threads": threads,
         "secs": time.time() - t0})
    del P64, Q64

    def time_to_target(rm, ms):
        for e in range(len(rm)):
            if rm[e] <= target:
                return float(ms[e]), e + 1
        return None, None

    # 4. cold start
    _, _, crm, cms = solve(g_tr, m_all, n, seed=5, precision="fp16", iters=args.warm_max_epochs, te=g_te)
    cold_ms, cold_ep = time_to_target(crm, cms)
    out({"arm": "cold fp16", "epoch_rmse": [round(x, 5) for x in crm], "epoch_ms": [round(x, 3) for x in cms],
         "time_to_target_ms": cold_ms, "epochs_to_target": cold_ep})

    def warm(init_kind, precision, alpha, beta, tail_epochs):
        """init_kind: "mlp" (the learned encoder), or a non-learned start on the same deployed
        base model: "mean" (the mean of the rated items' factors, scaled so that its product
        with that mean is the user's mean rating), "qmean" (the encoder's own input, the
        rating-centred mean of the rated items' factors), "zero" (rows of zeros; the model
        has no bias term, so every first prediction is 0) or "random" (the plain SGD
        initialisation)."""
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        P0 = torch.empty(m_all, K, device=dev)
        P0[: base_spec.m] = base_P
        if init_kind in ("mlp", "qmean"):  # features of the new users (the tail of the array)
            tail = d_gtr[len(b_tr) * 12:].view(torch.int32).view(-1, 3).clone()
            tail[:, 0] -= base_spec.m  # the new users' own ids 0..new_users-1
            Xn = features(tail, len(n_tr), new_users, n, base_Q)
            if init_kind == "mlp":
                mlp.forward(Xn.data_ptr(), new_users, P0[base_spec.m:].data_ptr())
            else:
                P0[base_spec.m:] = Xn[:, :K]
        elif init_kind == "mean":  # p = mean_u * qbar_u / |qbar_u|^2, so p . qbar_u = the user's mean rating
            tail = d_gtr[len(b_tr) * 12:].view(torch.int32).view(-1, 3)
            uu = (tail[:, 0] - base_spec.m).long()
            vv = tail[:, 1].long()
            rr = tail[:, 2].view(torch.float32)
            deg = torch.zeros(new_users, device=dev).index_add_(0, uu, torch.ones_like(rr)).clamp_(min=1)
            mu = torch.zeros(new_users, device=dev).index_add_(0, uu, rr) / deg
            avg = torch.sparse_coo_tensor(torch.stack([uu, vv]), 1.0 / deg[uu], (new_users, n))
            qbar = torch.sparse.mm(avg, base_Q)  # mean of each new user's rated item rows
            P0[base_spec.m:] = qbar * (mu / (qbar * qbar).sum(1).clamp_(min=1e-12))[:, None]
        elif init_kind == "zero":
            P0[base_spec.m:] = 0
        else:
            P0[base_spec.m:] = torch.from_numpy(oracle.init_factors(new_users, K, "fp32", 9, 1)).to(dev)
        torch.cuda.synchronize()
        prep_ms = (time.perf_counter() - t0) * 1e3
        init = cm.DeviceModel(P0.data_ptr(), m_all, base_Q.data_ptr(), n, K)
        _, _, wrm, wms = solve(g_tr, m_all, n, seed=5, precision=precision, iters=args.warm_max_epochs, init=init,
                               te=g_te, alpha=alpha, beta=beta, tail_epochs=tail_epochs, tail_start=len(b_tr))
        Pn = P0[base_spec.m:].contiguous()
        d_nte = torch.from_numpy((n_te.copy()).view(np.uint8)).to(dev)
        d_nte_view = d_nte.view(torch.int32).view(-1, 3)
        d_nte_view[:, 0] -= base_spec.m
        init_rmse_new = cm.dev_rmse(d_nte.data_ptr(), len(n_te), Pn.data_ptr(), new_users, base_Q.data_ptr(), n, K,
                                    float(base_model.b))
        return prep_ms, wrm, wms, init_rmse_new

    configs = [c.split(":") for c in args.warm_configs.split(",")]
    labels = {"mlp": "", "mean": " (no MLP: item-factor mean scaled to the user's mean rating)",
              "qmean": " (no MLP: centred item-factor mean)", "zero": " (no MLP: zero rows)",
              "random": " (no MLP: random rows)"}
    for init_kind in ("mlp", "mean", "qmean", "zero", "random"):
        for precision, alpha, beta, tail in (configs if init_kind == "mlp" else configs[:1]):
            prep_ms, wrm, wms, init_new = warm(init_kind, precision, float(alpha), float(beta), int(tail))
            w_ms, w_ep = time_to_target(wrm, wms)
            total = None if w_ms is None else w_ms + prep_ms
            out({"arm": f"warm {precision} alpha={alpha} beta={beta} new-user epochs={tail}" + labels[init_kind],
                 "init": init_kind, "mlp": init_kind == "mlp",
                 "prep_ms": prep_ms, "new_user_test_rmse_at_init": init_new,
                 "epoch_rmse": [round(x, 5) for x in wrm], "epoch_ms": [round(x, 3) for x in wms],
                 "time_to_target_ms": total, "epochs_to_target": w_ep,
                 "speedup_vs_cold": (cold_ms / total) if (cold_ms and total) else None})
    return {"target_rmse": target, "fp64_oracle_rmse": oracle_rmse, "cold_fp16_ms": cold_ms,
            "cold_epochs": cold_ep, "arms": [r for r in results if "arm" in r and r["arm"] != "cold fp16"]}


def warm_summary(args, scale=2.0):
    """Time-to-target line for bench.py's default run (scale 2: the c2 shape; scale 1: the c1
    shape): cold fp16 against the MLP warm start with bf16 stochastic rounding (one schedule),
    and the same deployed base model and schedule without the MLP (centred item-factor mean,
    zero rows, random rows), every arm capped at 40 epochs."""
    a = argparse.Namespace(**vars(args))
    a.scale, a.e2e_epochs, a.warm_max_epochs = scale, 20, 40
    a.mlp_epochs = 10 if scale >= 2.0 else 30
    a.warm_configs = "bf16sr:0.04:0.3:4"
    r = run_warmstart_suite(a, quiet=True)
    warm = next(x for x in r["arms"] if x.get("init") == "mlp")
    heur = {x["init"]: x for x in r["arms"] if x.get("init") != "mlp"}
    reached = [x["time_to_target_ms"] for x in heur.values() if x["time_to_target_ms"]]
    best_heur = min(reached) if reached else None
    big = scale >= 2.0
    return {"shape": ("c2 base 480189x17770 (99.07M ratings)" if big else "c1 base 10000x2000 (0.9M ratings)") +
                     " + 50000 new users (+5% ratings), k=128",
            "target_rmse": r["target_rmse"], "target": "FP64 oracle (host threads) test RMSE + 0.002",
            "fp64_oracle_rmse": r["fp64_oracle_rmse"],
            "cold_fp16_ms": r["cold_fp16_ms"], "cold_fp16_epochs": r["cold_epochs"],
            "warm_bf16sr_ms": warm["time_to_target_ms"], "warm_bf16sr_epochs": warm["epochs_to_target"],
            "warm_prep_ms": warm["prep_ms"], "warm_schedule": warm["arm"],
            "warm_new_user_rmse_at_init": warm["new_user_test_rmse_at_init"],
            "speedup": warm["speedup_vs_cold"],
            "no_mlp_arms": {k: {"time_to_target_ms": v["time_to_target_ms"], "epochs": v["epochs_to_target"],
                                "new_user_rmse_at_init": v["new_user_test_rmse_at_init"]} for k, v in heur.items()},
            "no_mlp_ablation_ms": best_heur,
            "speedup_vs_heuristic": (best_heur / warm["time_to_target_ms"])
            if (best_heur and warm["time_to_target_ms"]) else None,
            "max_epochs": 40}


def batched_summary(args):
    """Compact batched line for the default run: the 64-problem c4 set, 20 epochs, one
    graph-captured persistent launch (autotuned) against 64 sequential plain launches per epoch."""
    a = argparse.Namespace(**vars(args))
    a.scale, a.e2e_epochs = 1.0, 20
    return run_batched_suite(a, quiet=True)


def precision_gap_summary(args):
    """Every storage type's test-RMSE gap to the serial FP64 oracle on the sub-problem the
    c3 sweep measures it on: 1% of the c3 users with all 624,961 items (10,009 users, 2.53M
    train / 40k test ratings on 0..100, the c3 family's Zipf exponents, rank 48 + N(0, 20)
    noise), k=128, 20 epochs, generated directly at that size; every GPU variant and the
    oracle use the same worker count."""
    import dataclasses
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth
    from oracle import oracle
    oracle.build_oracle()
    c3 = synth.C3
    total = c3.nnz_train + c3.nnz_test
    spec = dataclasses.replace(c3, m=c3.m // 100, nnz_train=c3.nnz_train // 100, nnz_test=c3.nnz_test // 100,
                               user_s=c3.user_s if c3.user_s >= 0 else synth.fit_zipf_exponent(c3.m, total, c3.top_user),
                               item_s=c3.item_s if c3.item_s >= 0 else synth.fit_zipf_exponent(c3.n, total, c3.top_item))
    train, test = synth.generate(spec, seed=3, device="cuda")
    sm, _, _ = cm.device_info(0)
    W = cm.auto_workers(len(train), sm, K, "fp16")
    t0 = time.time()
    P, Q, b = oracle.train_f64(train, spec.m, spec.n, k=K, num_workers=W, num_iters=20, alpha=0.08, beta=0.3,
                               seed=1)
    ref = oracle.calc_rmse_f64(test, P, Q, b)
    del P, Q
    out = {"shape": f"1% of c3's users: {spec.m}x{spec.n}, {len(train)} train / {len(test)} test ratings, k=128",
           "workers": W, "epochs": 20, "fp64_oracle_rmse": ref, "fp64_oracle_secs": time.time() - t0, "gap": {}}
    prob = cm.MFProblem.from_arrays(train["u"], train["v"], train["r"], m=spec.m, n=spec.n)
    tprob = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"])
    for prec in ("fp32", "fp16", "bf16", "bf16sr", "fp16sr"):
        par = cm.Parameter(k=K, num_workers=W, num_iters=20, alpha=0.08, beta=0.3, seed=1, gpu=0, precision=prec)
        out["gap"][prec] = cm.calc_rmse(tprob, cm.sgd_train(prob, None, par)) - ref
    return out


def run_batched_suite(args, quiet=False):
    """Batched factorizations: 64 planted problems, users log-uniform in
    [1k, 200k], items in [500, 20k], ratings in [50k, 10M], k in {32, 64, 128}, planted rank
    in [8, 32], integer ratings 1..5, fp16 factors, 20 epochs.
      sequential: per epoch, one plain update launch per problem (64 launches per epoch);
      batched:    autotuned schedule, all 20 epochs of all 64 problems in one persistent
                  launch captured in a CUDA graph.
    Reports wall time (CUDA events) of each arm and the per-problem test RMSE of both."""
    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth, build
    build.build()
    dev = torch.device("cuda", 0)
    sm, _, _ = cm.device_info(0)
    rng = np.random.default_rng(4)
    nprob, epochs = 64, args.e2e_epochs
    conc = hot_rows_of(args)
    logu = lambda a, b: float(np.exp(rng.uniform(np.log(a), np.log(b))))
    probs = []
    t0 = time.time()
    for i in range(nprob):
        m, n = int(logu(1_000, 200_000)), int(logu(500, 20_000))
        nnz = int(logu(50_000, 10_000_000) * args.scale)
        k = int(rng.choice([32, 64, 128]))
        spec = synth.PlantedSpec(m=m, n=n, nnz_train=nnz, nnz_test=max(1000, nnz // 9), rank=int(rng.integers(8, 33)),
                                 user_s=0.5, item_s=0.5, factor_var=0.25, noise_std=0.5, offset=3.5, gain=1.0,
                                 lo=1, hi=5, integer=True)
        tr, te = synth.generate(spec, seed=1000 + i, device="cuda")
        d_raw = torch.from_numpy(tr.view(np.uint8)).to(dev)
        mean, std = cm.dev_rating_stats(d_raw.data_ptr(), nnz)
        scale = max(np.float32(1e-4), np.float32(std))
        pm = torch.from_numpy(cm.random_map(i, m)).to(dev)
        qm = torch.from_numpy(cm.random_map(i, n)).to(dev)
        d_R = torch.empty_like(d_raw)
        cm.dev_shuffle_scale(d_raw.data_ptr(), d_R.data_ptr(), nnz, pm.data_ptr(), m, qm.data_ptr(), n,
                             float(np.float32(1.0 / float(scale))))
        # Copies of the most-rated rows, planned as cumf_train plans them for this problem alone.
        w = cm.auto_workers(nnz, sm, k, "fp16")
        per_copy = cm.HotRows.per_copy(nnz, w, k, "fp16", 0, conc)
        hot = cm.HotRows(d_R.data_ptr(), nnz, m, n, per_copy) if per_copy > 0 else None
        if hot is not None and hot.hot_users + hot.hot_items == 0:
            hot.close()
            hot = None
        if hot is not None:
            hot.assign(d_R.data_ptr(), nnz)
        mr, nr = (hot.m_rows, hot.n_rows) if hot else (m, n)
        P = torch.empty(mr * k * 2, dtype=torch.uint8, device=dev)
        Q = torch.empty(nr * k * 2, dtype=torch.uint8, device=dev)
        lr = torch.from_numpy(cm.lr_schedule(0.08, 0.3, 0.0, epochs + 4)).to(dev)
        probs.append(dict(m=m, n=n, nnz=nnz, k=k, d_R=d_R, P=P, Q=Q, pm=pm, qm=qm, lr=lr, scale=scale,
                          b=float(np.float32(mean) / np.float32(std)), lam=float(np.float32(0.05) / scale),
                          te=torch.from_numpy(te.view(np.uint8)).to(dev), nte=len(te), seed=i, hot=hot,
                          m_rows=mr, n_rows=nr, workers=w))
    results = []

    def emit(d):
        results.append(d)
        if not quiet:
            print(json.dumps({"suite": "batched", **d}), flush=True)

    emit({"event": "generated", "problems": nprob, "total_nnz": sum(p["nnz"] for p in probs),
          "secs": time.time() - t0})

    def init_all():
        for p in probs:
            cm.dev_init_factors(p["P"].data_ptr(), p["m"], p["k"], "fp16", p["seed"], 1)
            cm.dev_init_factors(p["Q"].data_ptr(), p["n"], p["k"], "fp16", p["seed"], 2)
            if p["hot"] is not None:
                p["hot"].spread(p["P"].data_ptr(), p["Q"].data_ptr(), p["k"], "fp16")
        torch.cuda.synchronize()

    def rmses():
        out = []
        for p in probs:
            f = float(np.float32(np.sqrt(p["scale"])))
            Pf = torch.empty(p["m"], p["k"], device=dev)
            Qf = torch.empty(p["n"], p["k"], device=dev)
            cm.dev_export_factors(p["P"].data_ptr(), "fp16", p["pm"].data_ptr(), p["m"], p["k"], f, Pf.data_ptr())
            cm.dev_export_factors(p["Q"].data_ptr(), "fp16", p["qm"].data_ptr(), p["n"], p["k"], f, Qf.data_ptr())
            out.append(cm.dev_rmse(p["te"].data_ptr(), p["nte"], Pf.data_ptr(), p["m"], Qf.data_ptr(), p["n"],
                                   p["k"], p["b"]))
        return np.array(out)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # sequential plain launches (each followed by the merge of that problem's row copies)
    init_all()
    e0.record()
    for e in range(epochs):
        for p in probs:
            cm.sgd_update(p["d_R"].data_ptr(), p["nnz"], p["P"].data_ptr(), p["m_rows"], p["Q"].data_ptr(),
                          p["n_rows"], p["k"], "fp16", p["workers"], 0, p["lr"].data_ptr(), e, 1, p["lam"], p["lam"],
                          p["seed"], rows_copied=int(p["hot"] is not None))
            if p["hot"] is not None:
                p["hot"].merge(p["P"].data_ptr(), p["Q"].data_ptr(), p["k"], "fp16")
    e1.record()
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1)
    seq_rmse = rmses()
    total = sum(p["nnz"] for p in probs)
    with_copies = sum(p["hot"] is not None for p in probs)
    emit({"arm": "64 sequential plain launches per epoch", "epochs": epochs, "ms": seq_ms,
          "updates_per_sec": total * epochs / (seq_ms * 1e-3), "launches": epochs * (nprob + with_copies),
          "problems_with_row_copies": with_copies})
    # batched persistent launch
    init_all()
    batch = cm.Batch([dict(d_R=p["d_R"].data_ptr(), nnz=p["nnz"], d_P=p["P"].data_ptr(), m=p["m"], n=p["n"],
                           d_Q=p["Q"].data_ptr(), k=p["k"], lambda_p=p["lam"], lambda_q=p["lam"], seed=p["seed"],
                           d_lr=p["lr"].data_ptr(), lr_len=epochs + 4, hot=p["hot"]) for p in probs])
    t0 = time.time()
    best = batch.autotune()
    tune_s = time.time() - t0
    batch.run(0, epochs, use_graph=True)  # capture + first replay happen here ...
    torch.cuda.synchronize()
    init_all()  # ... so start again from the same init for the timed replay
    e0.record()
    batch.run(0, epochs, use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    bat_ms = e0.elapsed_time(e1)
    assert batch.status() == 0
    bat_rmse = rmses()
    info = batch.info()
    emit({"arm": "one graph (one persistent launch per epoch with the merges when a problem has row copies)",
          "epochs": epochs, "ms": bat_ms,
          "updates_per_sec": total * epochs / (bat_ms * 1e-3), "graph_launches": 1, "tuning": best,
          "autotune_s": tune_s, "samples_per_epoch": info["samples_per_epoch"],
          "speedup_vs_sequential": seq_ms / bat_ms})
    emit({"event": "rmse", "sequential_mean": float(seq_rmse.mean()), "batched_mean": float(bat_rmse.mean()),
          "max_abs_diff": float(np.abs(seq_rmse - bat_rmse).max()),
          "per_problem": [[round(a, 4), round(b, 4)] for a, b in zip(seq_rmse, bat_rmse)]})
    return {"problems": nprob, "total_nnz": total, "epochs": epochs, "problems_with_row_copies": with_copies,
            "sequential_ms": seq_ms,
            "batched_graph_ms": bat_ms, "speedup_vs_sequential": seq_ms / bat_ms,
            "batched_updates_per_sec": total * epochs / (bat_ms * 1e-3), "tuning": best, "autotune_s": tune_s,
            "mean_test_rmse_sequential": float(seq_rmse.mean()), "mean_test_rmse_batched": float(bat_rmse.mean()),
            "max_abs_rmse_diff": float(np.abs(seq_rmse - bat_rmse).max())}



def run_gemm_suite(args):
    """tcgen05 BF16 GEMM (the MLP's products) on its training shapes: TFLOP/s from CUDA-event
    time over repeated launches, against the measured dense bf16 peak (MEASURED_PEAKS.json)."""
    import torch
    from cumf_sgd_gb300 import build, _lib
    build.build()
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    peak = 1955.0
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        peak = float(json.load(open(path))["bf16_tflops"])
    rows = int(65536 * args.scale)
    shapes = [("fwd layer 1", rows, 512, 192), ("fwd layer 2", rows, 512, 512), ("fwd layer 3", rows, 128, 512),
              ("dX layer 2", rows, 512, 512), ("dW layer 2", 512, 512, rows), ("dW layer 1", 512, 192, rows)]
    for name, M, N, K in shapes:
        A = (torch.randn(M, K, device=dev) * 0.5).to(torch.bfloat16)
        B = (torch.randn(N, K, device=dev) * 0.5).to(torch.bfloat16)
        out = torch.empty(M, N, device=dev)
        for _ in range(3):
            assert lib.cumf_tc_gemm(A.data_ptr(), B.data_ptr(), M, N, K, None, 0, out.data_ptr(), 1, N, None, None,
                                    None) == 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = args.steps
        e0.record()
        for _ in range(reps):
            lib.cumf_tc_gemm(A.data_ptr(), B.data_ptr(), M, N, K, None, 0, out.data_ptr(), 1, N, None, None, None)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        tf = 2.0 * M * N * K / (ms * 1e-3) / 1e12
        err = (out - A.float() @ B.float().T).abs().max().item()
        print(json.dumps({"suite": "gemm", "shape": name, "M": M, "N": N, "K": K, "ms": ms, "tflops": tf,
                          "peak_tflops": peak, "frac": tf / peak, "max_abs_err_vs_fp32": err}), flush=True)


def run_mlp_suite(args):
    """Warm-start MLP training (131 -> 512 -> 512 -> 128, batch 4096, Adam) on c2-sized
    (features, factor row) pairs: time per epoch and per step (CUDA events) and the tensor-core
    rate of the step's matrix products."""
    import torch
    import cumf_sgd_gb300 as cm
    dev = torch.device("cuda", 0)
    rows = int(3841512 * args.scale)
    d_in, h, d_out, batch = 131, 512, 128, 4096
    g = torch.Generator(device=dev).manual_seed(5)
    X = torch.randn(rows, d_in, device=dev, generator=g)
    A = torch.randn(d_in, d_out, device=dev, generator=g) / d_in ** 0.5
    T = torch.tanh(X @ A).contiguous()
    mlp = cm.MLP(d_in, h, d_out, seed=7)
    mlp.train(X.data_ptr(), T.data_ptr(), min(rows, 8 * batch), epochs=1, batch=batch, seed=1)  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    loss = mlp.train(X.data_ptr(), T.data_ptr(), rows, epochs=args.mlp_epochs, batch=batch, seed=3)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    steps = args.mlp_epochs * ((rows + batch - 1) // batch)
    dp = 192  # d_in padded to the 64-column tiles
    flops_step = 3 * 2.0 * batch * (dp * h + h * h + h * d_out)  # forward + two backward products
    print(json.dumps({"suite": "mlp", "rows": rows, "epochs": args.mlp_epochs, "batch": batch, "steps": steps,
                      "train_s": ms / 1e3, "ms_per_step": ms / steps, "rows_per_s": rows * args.mlp_epochs / (ms / 1e3),
                      "gemm_tflops_per_step": flops_step / (ms / steps * 1e-3) / 1e12, "final_loss": loss}), flush=True)


def ratings_text_gpu(train, header: bytes):
    """The records as rating text ("u v r" lines, integer ratings), built on the GPU: digits in
    fixed-width rows, then the padding bytes dropped with one masked select."""
    import torch
    dev = torch.device("cuda", 0)
    u = torch.from_numpy(train["u"].astype(np.int64)).to(dev)
    v = torch.from_numpy(train["v"].astype(np.int64)).to(dev)
    r = torch.from_numpy(np.rint(train["r"]).astype(np.int64)).to(dev)

    def digits(x, width):
        pw = 10 ** torch.arange(width - 1, -1, -1, device=dev)
        d = (x[:, None] // pw) % 10
        nd = torch.clamp((x[:, None] >= pw).sum(1), min=1)
        keep = torch.arange(width, device=dev)[None, :] >= (width - nd)[:, None]
        return (d + 48).to(torch.uint8), keep

    du, ku = digits(u, 10)
    dv, kv = digits(v, 10)
    dr, kr = digits(r, 2)
    n = len(train)
    sp = torch.full((n, 1), 32, dtype=torch.uint8, device=dev)
    nl = torch.full((n, 1), 10, dtype=torch.uint8, device=dev)
    one = torch.ones((n, 1), dtype=torch.bool, device=dev)
    rows = torch.cat([du, sp, dv, sp, dr, nl], 1)
    keep = torch.cat([ku, one, kv, one, kr, one], 1)
    body = rows[keep]
    head = torch.frombuffer(bytearray(header), dtype=torch.uint8).to(dev)
    return torch.cat([head, body, torch.zeros(16, dtype=torch.uint8, device=dev)])


def run_text_suite(args):
    """Rating text -> records (data/netflix/transform.cpp) for the c2 ratings as text: device
    parse (text resident in HBM) and end to end from pinned host text to pinned host records,
    against the oracle's strtol/strtof parse of a bounded sample on one host core."""
    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth, build
    from oracle import oracle
    build.build()
    spec = synth.C2 if args.scale >= 1.0 else synth.scaled(synth.C2, args.scale)
    train, _ = synth.generate(spec, seed=0, device="cuda")
    header = b"%%%%MatrixMarket matrix coordinate real general\n%% c2 synthetic\n%d %d %d\n" % (
        spec.m, spec.n, len(train))
    d_text = ratings_text_gpu(train, header)
    length = d_text.numel() - 16
    n = len(train)
    start = len(header)
    d_out = torch.empty(n * 12, dtype=torch.uint8, device=d_text.device)
    h_text = d_text.cpu().pin_memory()
    h_out = torch.empty(n * 12, dtype=torch.uint8).pin_memory()
    stream = torch.cuda.current_stream()

    def device_parse():
        assert cm.dev_parse_text(d_text.data_ptr(), length, start, d_out.data_ptr(), n) == n

    def end_to_end():
        d_text[:length].copy_(h_text[:length], non_blocking=True)
        device_parse()
        h_out.copy_(d_out, non_blocking=True)
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        end_to_end()
    got = h_out.numpy().view(synth.NODE_DTYPE)
    ok = bool(np.array_equal(got["u"], train["u"]) and np.array_equal(got["v"], train["v"]) and
              np.array_equal(got["r"], np.rint(train["r"]).astype(np.float32)))
    res = {}
    import ctypes as C
    from cumf_sgd_gb300 import _lib
    n_out = C.c_int64(0)

    def end_to_end_pipelined():
        _lib.check(_lib.load().cumf_parse_text_host(h_text.data_ptr(), length, 3, h_out.data_ptr(), n, C.byref(n_out)))

    for name, fn in (("device", device_parse), ("e2e", end_to_end), ("e2e_pipelined", end_to_end_pipelined)):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) / args.steps
        res[name] = {"ms": e0.elapsed_time(e1) / args.steps, "wall_ms": wall * 1e3}
    got = h_out.numpy().view(synth.NODE_DTYPE)
    ok_pipe = bool(n_out.value == n and np.array_equal(got["u"], train["u"]) and np.array_equal(got["v"], train["v"]))
    # Oracle (strtol/strtof, one core) on a bounded prefix of the same text.
    sample_lines = min(n, 4_000_000)
    cut = int(np.searchsorted(np.cumsum(h_text[start:length].numpy() == 10), sample_lines)) + start + 1
    sample = h_text[:cut].numpy().tobytes()
    t0 = time.perf_counter()
    recs = oracle.parse_text(sample)
    cpu_s = time.perf_counter() - t0
    print(json.dumps({"suite": "text", "records": n, "text_bytes": length, "parse_matches_records": ok,
                      "pipelined_matches_records": ok_pipe,
                      "device_ms": res["device"]["ms"], "device_GBps": length / res["device"]["ms"] / 1e6,
                      "device_records_per_s": n / res["device"]["ms"] * 1e3,
                      "e2e_ms": res["e2e"]["ms"], "e2e_records_per_s": n / res["e2e"]["ms"] * 1e3,
                      "e2e_pipelined_ms": res["e2e_pipelined"]["wall_ms"],
                      "e2e_pipelined_records_per_s": n / res["e2e_pipelined"]["wall_ms"] * 1e3,
                      "e2e_h2d_bytes": length, "e2e_d2h_bytes": n * 12,
                      "cpu_oracle": {"records": len(recs), "seconds": cpu_s, "records_per_s": len(recs) / cpu_s,
                                     "cores": 1, "kind": "port (strtol/strtof)"}}), flush=True)


def run_streamed_suite(args):
    """Modes A, B and C of sgd_update_k128 (sgd_kernel.cu:125-720) on the c2 ratings held in
    pinned host memory: updates/s over the training phase (wall clock: the host<->device
    copies of rating blocks and factor segments are inside it for modes B and C), total wall
    time and test RMSE after the same number of epochs."""
    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth, build
    build.build()
    spec = synth.C2 if args.scale >= 1.0 else synth.scaled(synth.C2, args.scale)
    train, test = synth.generate(spec, seed=0, device="cuda")
    m, n, nnz = spec.m, spec.n, len(train)
    prob = cm.MFProblem.from_arrays(train["u"], train["v"], train["r"], m=m, n=n, pinned=True)
    tprob = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"], m=m, n=n)
    sm, _, _ = cm.device_info(0)
    epochs = max(1, min(args.steps, 20))
    for grid in [(1, 1, 1, 1), "deterministic", (2, 2, 1, 1), (4, 1, 1, 1), (2, 1, 2, 2), (2, 2, 2, 2)]:
        det = grid == "deterministic"
        u, v, x, y = (1, 1, 1, 1) if det else grid
        blocks = u * v * x * y
        workers = cm.auto_workers(max(1, nnz // blocks), sm, K, "fp16", 0)
        par = cm.Parameter(k=K, num_workers=workers, num_iters=epochs, lambda_p=0.05, lambda_q=0.05, alpha=0.08,
                           beta=0.3, seed=0, gpu=0, precision="fp16", u_grid=u, v_grid=v, x_grid=x, y_grid=y, quiet=1,
                           deterministic=int(det))
        cm.sgd_train(prob, None, cm.Parameter(**{**par.__dict__, "num_iters": 1}))  # warm-up
        t0 = time.perf_counter()
        model, st = cm.sgd_train(prob, None, par, with_stats=True)
        wall = time.perf_counter() - t0
        rmse = cm.calc_rmse(tprob, model)
        mode = "A, deterministic" if det else "ABC"[st.mode]
        print(json.dumps({"suite": "streamed", "mode": mode, "u_v_x_y": (u, v, x, y), "workers_per_block": st.num_workers,
                          "epochs": epochs, "train_ms": st.train_ms, "updates_per_sec": nnz * epochs / (st.train_ms * 1e-3),
                          "wall_s": wall, "prep_ms": st.prep_ms, "export_ms": st.export_ms,
                          "test_rmse": rmse}), flush=True)
        del model


def _has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp16")
    ap.add_argument("--workers", type=int, default=0)
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--prefetch", type=int, default=-1, help="L2 prefetch distance in records (-1: default)")
    ap.add_argument("--l2-hints", type=int, default=-1, help="L2 eviction hints 0/1 (-1: default)")
    ap.add_argument("--ring", type=int, default=-1, help="shared-memory row ring 0/1 (-1: default)")
    ap.add_argument("--e2e-epochs", type=int, default=20)
    ap.add_argument("--hot-rows", type=float, default=None,
                    help="expected workers per copy of a most-rated row (default 0.5 here; 0 = no copies, "
                         "the library's default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-warm", action="store_true", help="skip the time-to-target measurement")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 oracle run (no RMSE gaps)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the c1 time-to-target, batched and precision-gap keys")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the workload size (tests only)")
    ap.add_argument("--mlp-epochs", type=int, default=30)
    ap.add_argument("--warm-max-epochs", type=int, default=40, help="epoch cap of every warm-start arm")
    ap.add_argument("--warm-configs",
                    default="bf16sr:0.04:0.3:4,bf16sr:0.02:0.05:8,bf16sr:0.04:0.3:2,fp16:0.04:0.3:4,bf16sr:0.02:0.3:0",
                    help="warm-start refinements as storage:alpha:beta:new_user_epochs, comma separated")
    ap.add_argument("--suite", default="", choices=["", "precision", "warmstart", "batched", "gemm", "text", "mlp",
                                                    "streamed"],
                    help="extra measurement suites (JSON lines, not the contract line)")
    args = ap.parse_args()
    if args.suite == "precision":
        run_precision_suite(args)
        return
    if args.suite == "warmstart":
        run_warmstart_suite(args)
        return
    if args.suite == "batched":
        run_batched_suite(args)
        return
    if args.suite == "gemm":
        run_gemm_suite(args)
        return
    if args.suite == "mlp":
        run_mlp_suite(args)
        return
    if args.suite == "text":
        run_text_suite(args)
        return
    if args.suite == "streamed":
        run_streamed_suite(args)
        return
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth, build

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    init_dist(world)
    build.build()
    spec = synth.C2 if args.scale >= 1.0 else synth.scaled(synth.C2, args.scale)
    train, test = synth.generate(spec, seed=rank, device="cuda")
    m, n, nnz = spec.m, spec.n, len(train)
    sm, _, _ = cm.device_info(local)
    workers = args.workers or cm.auto_workers(nnz, sm, K, args.precision, args.lanes)
    prec = args.precision
    eb = 4 if prec == "fp32" else 2
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    # Device-resident problem, prepared exactly as cumf_train does.
    d_raw = torch.from_numpy(train.view(np.uint8)).to(dev)
    mean, std = cm.dev_rating_stats(d_raw.data_ptr(), nnz, sp)
    std32 = np.float32(std)
    scale = max(np.float32(1e-4), std32)
    pm = torch.from_numpy(cm.random_map(rank, m)).to(dev)
    qm = torch.from_numpy(cm.random_map(rank, n)).to(dev)
    d_R = torch.empty_like(d_raw)
    cm.dev_shuffle_scale(d_raw.data_ptr(), d_R.data_ptr(), nnz, pm.data_ptr(), m, qm.data_ptr(), n,
                         float(np.float32(1.0 / float(scale))), 0, sp)
    del d_raw
    # Copies of the most-rated rows, laid out and assigned as cumf_train does by default.
    conc = hot_rows_of(args)
    per_copy = cm.HotRows.per_copy(nnz, workers, K, prec, args.lanes, conc)
    hot = cm.HotRows(d_R.data_ptr(), nnz, m, n, per_copy, stream=sp) if per_copy > 0 else None
    m_rows, n_rows = (hot.m_rows, hot.n_rows) if hot else (m, n)
    # The ratings as the reference's kernel sees them (every rating names its own row), kept
    # for the comparison run without copies after the timed region.
    d_R_plain = d_R.clone() if (hot and rank == 0 and world == 1 and not args.no_extras) else None
    if hot:
        hot.assign(d_R.data_ptr(), nnz, sp)
    P = torch.empty(m_rows * K * eb, dtype=torch.uint8, device=dev)
    Q = torch.empty(n_rows * K * eb, dtype=torch.uint8, device=dev)
    cm.dev_init_factors(P.data_ptr(), m, K, prec, rank, 1, sp)
    cm.dev_init_factors(Q.data_ptr(), n, K, prec, rank, 2, sp)
    merges = hot is not None and hot.hot_users + hot.hot_items > 0
    if merges:
        hot.spread(P.data_ptr(), Q.data_ptr(), K, prec, sp)
    # Step s runs epoch s mod 20 of the 20-epoch job's learning-rate schedule.
    job_epochs = 20
    epochs_total = args.warmup + args.steps
    lr = torch.from_numpy(cm.lr_schedule(0.08, 0.3, 0.0, job_epochs + 4)).to(dev)
    lp = float(np.float32(0.05) / scale)
    status = torch.zeros(1, dtype=torch.int32, device=dev)

    def epoch(e):
        cm.sgd_update(d_R.data_ptr(), nnz, P.data_ptr(), m_rows, Q.data_ptr(), n_rows, K, prec, workers, args.lanes,
                      lr.data_ptr(), e % job_epochs, 1, lp, lp, rank, status.data_ptr(), sp,
                      prefetch=args.prefetch, l2_hints=args.l2_hints, ring=args.ring, rows_copied=int(merges))
        if merges:
            hot.merge(P.data_ptr(), Q.data_ptr(), K, prec, sp)

    for e in range(args.warmup):
        epoch(e)
    torch.cuda.synchronize()
    barrier(world)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for e in range(args.warmup, epochs_total):
            epoch(e)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clocks = clk.summary()
    assert int(status.item()) == 0, "update kernel flagged an out-of-range index"
    ms = max_over_ranks(ms, world)
    barrier(world)
    secs = ms / 1e3
    updates_per_sec = nnz * args.steps * world / secs
    batches = cm.batches_per_worker(nnz, workers)
    samples_per_launch = workers * batches * 128
    launch_s = secs / args.steps
    achieved = samples_per_launch * BYTES_PER_SAMPLE[prec] / launch_s / 1e9
    peak, peak_kind = measured_peaks()
    l2_gbs = l2_copy_gbs()

    # The same epochs without row copies (each rating updates its own rows, as the reference's
    # kernel does), default prefetch: untimed by the driver's contract, reported beside value.
    plain = None
    if d_R_plain is not None:
        cm.dev_init_factors(P.data_ptr(), m, K, prec, rank, 1, sp)
        cm.dev_init_factors(Q.data_ptr(), n, K, prec, rank, 2, sp)
        def plain_epoch(e):
            cm.sgd_update(d_R_plain.data_ptr(), nnz, P.data_ptr(), m, Q.data_ptr(), n, K, prec, workers, args.lanes,
                          lr.data_ptr(), e % job_epochs, 1, lp, lp, rank, status.data_ptr(), sp,
                          l2_hints=args.l2_hints, ring=args.ring)
        for e in range(3):
            plain_epoch(e)
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        p0.record(stream)
        for e in range(3, 13):
            plain_epoch(e)
        p1.record(stream)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        pms = p0.elapsed_time(p1) / 10
        plain_gbs = samples_per_launch * BYTES_PER_SAMPLE[prec] / (pms * 1e-3) / 1e9
        plain = {"updates_per_sec": nnz / (pms * 1e-3), "ms_per_epoch": pms, "workers": workers, "epochs_timed": 10,
                 "achieved_gbs": plain_gbs, "l2_frac": plain_gbs / l2_gbs, "hbm_frac": plain_gbs / peak,
                 "what": "the same device-resident epochs without row copies (the library's default, the "
                         "reference's update), default L2 prefetch"}
        del d_R_plain

    hot_info = {"concurrency": conc, "per_copy": per_copy, "hot_users": hot.hot_users if hot else 0,
                "hot_items": hot.hot_items if hot else 0,
                "extra_rows": (m_rows - m) + (n_rows - n)}
    del P, Q, d_R, hot
    torch.cuda.empty_cache()

    # End to end through the C ABI: pinned host ratings -> cumf_train (20 epochs) -> fp32 model.
    e2e = None
    if not args.no_e2e:
        prob = cm.MFProblem.from_arrays(train["u"], train["v"], train["r"], m=m, n=n, pinned=True)
        tprob = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"])
        par = cm.Parameter(k=K, num_workers=workers, num_iters=args.e2e_epochs, lambda_p=0.05, lambda_q=0.05,
                           alpha=0.08, beta=0.3, seed=rank, gpu=local, precision=prec, lanes=args.lanes,
                           hot_rows=conc)
        cm.sgd_train(prob, None, cm.Parameter(**{**par.__dict__, "num_iters": 1}))  # warm-up call
        barrier(world)
        t0 = time.perf_counter()
        model, st = cm.sgd_train(prob, None, par, with_stats=True)
        wall = max_over_ranks(time.perf_counter() - t0, world)  # the slowest replica
        test_rmse = cm.calc_rmse(tprob, model)
        e2e = {"value": nnz * args.e2e_epochs * world / wall, "unit": "updates/s",
               "h2d_bytes_per_step": nnz * 12 + 4 * (m + n), "d2h_bytes_per_step": 4 * K * (m + n),
               "epochs_per_step": args.e2e_epochs, "wall_s": wall,
               "prep_ms": st.prep_ms, "train_ms": st.train_ms, "export_ms": st.export_ms,
               "model_pinned": int(model._c.pinned), "test_rmse": test_rmse,
               "hot_rows": {"hot_users": st.hot_users, "hot_items": st.hot_items, "extra_rows": st.extra_rows}}
        del model

    # The benchmark shape at the reference's recommended worker count (52 per SM,
    # README.md:61) through the same C ABI: throughput and test RMSE beside the default's.
    w52 = None
    if not args.no_e2e and rank == 0 and world == 1:
        W52 = 52 * sm
        par52 = cm.Parameter(**{**par.__dict__, "num_workers": W52})
        model52, st52 = cm.sgd_train(prob, None, par52, with_stats=True)
        w52 = {"workers": W52, "updates_per_sec": st52.updates_per_sec, "train_ms": st52.train_ms,
               "epochs": args.e2e_epochs, "test_rmse": cm.calc_rmse(tprob, model52),
               "timing": "CUDA events around the epochs inside cumf_train"}
        del model52

    import tempfile
    tmpdir = tempfile.mkdtemp(prefix="cumf_bench_")
    ref_tools = _reference_tools() if (rank == 0 and world == 1 and not args.no_cpu_baseline) else None

    # The reference's own GPU trainer (singleGPU/ built for sm_103a) at the same worker count:
    # its printed update_per_sec (host clock() around its one persistent launch) and the test
    # RMSE of the model it writes, scored by the same evaluator.
    refk = None
    if ref_tools is not None and w52 is not None and ref_tools.available("cumf_sgd_ref"):
        try:
            tr_path = os.path.join(tmpdir, "c2_train.bin")
            ref_tools.write_records(train, tr_path)
            mp = os.path.join(tmpdir, "ref_gpu.model")
            out = ref_tools.run_reference_gpu(tr_path, mp, w52["workers"], args.e2e_epochs, gpu=local)
            refk = {"binary": "singleGPU cumf_sgd, built unmodified for sm_103a (two-function __shfl shim)",
                    "kernel": "sgd_k128_kernel_hogwild_warp32_lrate", "workers": w52["workers"],
                    "epochs": args.e2e_epochs, "update_per_sec": out["update_per_sec"], "process_wall_s": out["wall_s"],
                    "timing": "the binary's own update_per_sec: host clock() around its launch and sync"}
            if out["rc"] == 0:
                refk["test_rmse"] = cm.calc_rmse(tprob, cm.load_model(mp))
                w52["rmse_minus_reference_kernel"] = w52["test_rmse"] - refk["test_rmse"]
                w52["speedup_vs_reference_kernel"] = (w52["updates_per_sec"] / refk["update_per_sec"]
                                                      if refk["update_per_sec"] else None)
            else:
                refk["error"] = out["tail"][-300:]
            os.unlink(tr_path)
        except Exception as e:  # reported, never fatal to the throughput line
            refk = {"error": repr(e)[:300]}

    # FP64 oracle (the same statistics, id maps and sample schedule; its batches on the host
    # threads) for the RMSE gaps.
    fp64 = None
    if not args.no_e2e and rank == 0 and world == 1 and not args.no_fp64:
        from oracle import oracle
        oracle.build_oracle()
        t0 = time.time()
        P64, Q64, b64 = oracle.train_f64(train, m, n, k=K, num_workers=workers, num_iters=args.e2e_epochs,
                                         seed=rank, threads=os.cpu_count() or 1)
        fp64 = {"test_rmse": oracle.calc_rmse_f64(test, P64, Q64, b64), "host_threads": os.cpu_count() or 1,
                "workers": workers, "secs": time.time() - t0}
        del P64, Q64
        e2e["rmse_gap_to_fp64"] = e2e["test_rmse"] - fp64["test_rmse"]
        if w52 is not None:
            w52["rmse_gap_to_fp64"] = w52["test_rmse"] - fp64["test_rmse"]
        if refk is not None and "test_rmse" in refk:
            refk["rmse_gap_to_fp64"] = refk["test_rmse"] - fp64["test_rmse"]

    # CPU baseline: LIBMF mf-train (the reference's CPU trainer) on the host cores, a bounded
    # sample of 8 iterations over the full train set; the oracle's threaded port beside it.
    cpu = cpu_port = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_port = cpu_port_baseline(train, m, n, seconds_budget=args.ref_seconds)
        if ref_tools is not None:
            try:
                threads = os.cpu_count() or 1
                cpu = libmf_baseline(ref_tools, train, 8, threads, tmpdir)
                cpu["sample"] = (f"LIBMF mf-train (test/mf-train.cpp), 8 iterations over the {nnz} c2 train "
                                 f"ratings, k=128, {threads} threads, {2 * threads + 1} blocks "
                                 f"({cpu.get('build', '')})")
                cpu["gpu_e2e_ratio"] = e2e["value"] / cpu["value"] if e2e else None
            except Exception as e:
                cpu = dict(cpu_port, note="LIBMF failed: " + repr(e)[:200])
        else:
            cpu = dict(cpu_port, note="LIBMF mf-train not built on this host: oracle port timed")
    import shutil
    shutil.rmtree(tmpdir, ignore_errors=True)

    ttt = ttt_c1 = batched = precision_gap = None
    if rank == 0 and world == 1 and not args.no_warm:
        del train, test
        try:
            ttt = warm_summary(args)
        except Exception as e:  # reported, never fatal to the throughput line
            ttt = {"error": repr(e)[:300]}
    if rank == 0 and world == 1 and not args.no_extras:
        torch.cuda.empty_cache()
        for key, fn in (("c1", lambda: warm_summary(args, scale=1.0)), ("batched", lambda: batched_summary(args)),
                        ("precision", lambda: precision_gap_summary(args))):
            try:
                res = fn()
            except Exception as e:  # reported, never fatal to the throughput line
                res = {"error": repr(e)[:300]}
            if key == "c1":
                ttt_c1 = res
            elif key == "batched":
                batched = res
            else:
                precision_gap = res
            torch.cuda.empty_cache()

    if rank == 0:
        line = {"metric": "sgd_updates_per_sec", "value": updates_per_sec, "unit": "updates/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": prec, "data": "synthetic",
                "config": {"workload": WORKLOAD, "m": m, "n": n, "nnz": nnz, "k": K, "storage": prec,
                           "workers": workers, "lanes": args.lanes or "auto",
                           "step": ("one epoch (update launch + merge of the row copies)" if merges
                                    else "one epoch (one launch)"),
                           "hot_rows": hot_info,
                           "samples_per_epoch": samples_per_launch,
                           "l2": "inputs larger than L2 (ratings 1.19 GB)", "parallelism": f"replicas{world}"},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind,
                             "traffic": (UPDATE_KERNEL_DRAM_BYTES_C2
                                         if (prec == "fp16" and args.scale >= 1.0 and not args.workers and merges
                                             and args.hot_rows in (None, 0.5) and args.prefetch < 0
                                             and args.lanes == 0) else None),
                             "traffic_source": UPDATE_KERNEL_DRAM_BYTES_SOURCE,
                             "bytes_per_sample": BYTES_PER_SAMPLE[prec]},
                "l2_roofline": {"achieved": achieved, "peak": l2_gbs, "unit": "GB/s", "frac": achieved / l2_gbs,
                                "peak_kind": "L2-resident copy (2 x 16 MB, 400 passes in one launch), measured in this run"},
                "clocks": clocks, "e2e": e2e, "gpu_launches": args.steps * (2 if merges else 1), "cpu_baseline": cpu,
                "cpu_port": cpu_port, "fp64_oracle": fp64, "value_w52": w52, "value_without_copies": plain,
                "reference_kernel": refk,
                "time_to_target": ttt, "time_to_target_c1": ttt_c1, "batched": batched,
                "precision_gap": precision_gap}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
