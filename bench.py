#!/usr/bin/env python
"""Benchmark: HMM read x peptide forwards per second on one GB300.

Workload (the batched persistent-HMM configuration): 3 channels, 16
timesteps (1 mock + 15 Edman cycles), 1,000 dye-seqs of length 8-30 with at
most 5 dyes per channel and at least one dye, 100,000 simulated reads, HMM
pruning cutoff 5 sigma; error model p_edman_failure 0.06, p_detach 0.05,
p_bleach 0.05, p_dud 0.07, intensity ~ N(n, sqrt(0.00667^2 + n 0.16^2)).
Inputs come from the package's seeded simulator (synthetic data).

A step is one `classify hmm` pass over the batch: 100,000 x 1,000 =
1e8 (read, peptide) forwards, argmax and count-weighted totals per read.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload classify|fit|hybrid|learned|tracks]

`--workload fit` measures the Baum-Welch E-step instead (reads/s): one
dye-seq of 20 positions with 4/3/3 dyes on 3 channels (positions seeded),
200,000 reads simulated from the error model above, 16 timesteps, no
pruning; a step is one E-step over all reads (the per-iteration work of
HMMFitter::fit); the line adds one full fit to a 1e-6 step from a seeded
+-50% perturbation of the generating model.

`--workload hybrid` measures the hybrid classifier (reads/s): 20,000
dye-seqs as above, a dye-track training set of 100 simulated reads per
dye-seq (about 945,000 unique tracks), kNN with k = 10,000 hits and sigma
0.5, the top 1,000 candidates rescored by the HMM (pruning 5 sigma), 100,000
query reads per step (--reads to change).

`--workload tracks` measures `simulate dt` (dye-tracks/s): the hybrid
workload's training set, 100 dye-tracks for each of the 20,000 dye-seqs
(2,000,000 instances), generated and deduplicated on the device; the CPU
baseline is the oracle's single-threaded generate + dedup on a sample.

`--workload learned` trains the proposal network (--epochs of 10,000,000
reads simulated on the GPU) and measures the hybrid with its top-200
proposals in place of the kNN stage on the hybrid workload's reads, next to
the kNN hybrid's accuracy and speed on the same reads.

Prints one JSON line (rank 0).  `value` is measured with the reads already in
device memory (CUDA events on the library's stream, L2 flushed between
steps); `e2e` is the same metric through the public C ABI call with host
buffers (pinned), host->device copy and result read-back inside the timed
region; `roofline` reports the forward kernel's algorithmic FP32 work (the
reference's pruned visited-state op count) per unit time against the
device's measured FP32 FMA throughput; `cpu_baseline` times the CPU oracle
(a restatement of the reference's algorithm) on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "HMM read x peptide forwards/s (classify hmm, -p 5)"
UNIT = "fwd/s"
T, C, P, READS, CUTOFF = 16, 3, 1000, 100_000, 5.0
WORKLOAD = ("classify hmm: 3 channels x 16 timesteps, 1000 dye-seqs (8-30 positions, <=5 dyes "
            "per channel, >=1 dye), 100000 reads float64 [100000,16,3], pruning 5 sigma")


HY_METRIC = "hybrid classify reads/s (kNN k=10000 hits, sigma 0.5, H=1000 -> HMM -p 5)"
HY_UNIT = "reads/s"
HY_P, HY_PER, HY_K, HY_SIG, HY_H, HY_READS = 20_000, 100, 10_000, 0.5, 1000, 100_000
HY_WORKLOAD = ("hybrid: 3 channels x 16 timesteps, 20000 dye-seqs (8-30 positions, <=5 dyes per channel), "
               "dye-track training set of 100 simulated reads per dye-seq deduplicated, kNN k=10000 hits, "
               "sigma 0.5, H=1000 candidates to the HMM with pruning 5 sigma")


def make_hybrid_data(seed: int, reads: int):
    from whatprot_gb300.simulate import (paper_model, random_dye_seqs, simulate_dye_track_set,
                                         simulate_radiometries)
    sm = paper_model(C)
    ds = random_dye_seqs(HY_P, C, 8, 30, max_per_channel=5, min_total=1, seed=1234)
    dts = simulate_dye_track_set(sm, ds, T, HY_PER, seed=4321)
    rads, ids = simulate_radiometries(sm, ds, T, int(reads * 1.05) + 64, seed=seed)
    return sm, ds, dts, rads[:reads].copy(), ids[:reads].copy()


def run_hybrid(args):
    import torch
    from whatprot_gb300 import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    reads = args.reads if args.reads != READS else HY_READS
    t0 = time.perf_counter()
    sm, ds, dts, rads, true_ids = make_hybrid_data(seed=5050 + rank, reads=reads)
    gen_s = time.perf_counter() - t0
    R = rads.shape[0]
    ctx = capi.Context(local)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    ctx.upload_tracks(dts)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    d_rads = torch.from_numpy(rads).to(f"cuda:{local}")
    d_id = torch.empty(R, dtype=torch.int32, device=f"cuda:{local}")
    d_sc = torch.empty(R, dtype=torch.float64, device=f"cuda:{local}")
    d_tot = torch.empty(R, dtype=torch.float64, device=f"cuda:{local}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def step():
        ctx.hybrid_classify_device(d_rads.data_ptr(), R, HY_K, HY_SIG, HY_H, CUTOFF, d_id.data_ptr(),
                                   d_sc.data_ptr(), d_tot.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ctx.timing_enable(True)
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    total_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        step()
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
    barrier()
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    kd_ms, kd_n = ctx.timing_read(ctx.KIND_KNN_DIST)
    ks_ms, _ = ctx.timing_read(ctx.KIND_KNN_SELECT)
    fw_ms, _ = ctx.timing_read(ctx.KIND_FORWARD)
    pr_ms, _ = ctx.timing_read(ctx.KIND_PREP)
    ctx.timing_enable(False)
    t_step = total_ms / args.steps
    if dist:
        t = torch.tensor([t_step], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    value = R * world / (t_step * 1e-3)
    acc = float((d_id.cpu().numpy() == true_ids).mean())
    # end to end through the host API (pinned reads)
    h_rads = torch.from_numpy(rads).pin_memory().numpy()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        last_gpu = ctx.hybrid_classify(h_rads, HY_K, HY_SIG, HY_H, CUTOFF)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e = {"value": R * world / e2e_s, "unit": HY_UNIT, "h2d_bytes_per_step": int(rads.nbytes),
           "d2h_bytes_per_step": int(R * (4 + 8 + 8))}
    # the kNN distance stage: algorithmic work = one (query, track) squared
    # distance per pair, 3 FP32 operations per dimension (sub, multiply-add)
    N = len(dts)
    algo = 3.0 * R * N * T * C
    peak = ctx.fp32_peak_tflops()
    kd_step = kd_ms / args.steps
    achieved = algo / (kd_step * 1e-3) / 1e12 if kd_step > 0 else None
    line = {"metric": HY_METRIC, "value": value, "unit": HY_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded simulator)",
            "config": {"workload": HY_WORKLOAD, "reads": R, "peptides": len(ds), "dye_tracks": N,
                       "track_sources": int(dts.src_off[-1]), "k": HY_K, "sigma": HY_SIG, "h": HY_H,
                       "dist_cutoff": CUTOFF, "l2": "flushed between steps (512 MB write)",
                       "data_generation_s": gen_s},
            "top1_vs_truth": acc,
            "roofline": {"bound": "fp32", "kernel": "wp_nn_hist_kernel + wp_nn_collect_kernel",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if (achieved and peak) else None, "traffic": None,
                         "peak_source": "FP32 FMA loop measured live (wp_probe_fp32_peak)",
                         "algorithmic_flops_per_step": algo,
                         "knn_distance_ms_per_step": kd_step, "knn_select_ms_per_step": ks_ms / args.steps,
                         "hmm_forward_ms_per_step": fw_ms / args.steps, "hmm_prep_ms_per_step": pr_ms / args.steps},
            "e2e": e2e, "gpu_launches": launches, "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"], o_out = cpu_baseline_hybrid(sm, ds, dts, rads)
        line["parity_vs_oracle"] = sample_parity(last_gpu, o_out)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


SUB_READS = 20_000  # query reads per step of the hybrid / learned sub-records


def _timed_steps(stream, flush, step, steps):
    """Mean CUDA-event time (ms) of `step` on `stream`, L2 flushed before each."""
    import torch
    total = 0.0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    return total / max(steps, 1)


def hybrid_learned_subrecords(local, steps=2, warmup=1, epochs=3, reads=SUB_READS, oracle_reads=64):
    """The second half of the headline metric on one GB300: the hybrid
    classifier's reads/s with the kNN stage (k = 10,000 hits, sigma 0.5,
    H = 1,000) in both k-hit selections -- the reference's kd-tree search
    (exact, the default) and the shortest-prefix fast mode -- and with the
    learned proposal (MLP 48-1024-1024-20000, H = 200) in its place, on the
    same 20,000 dye-seqs and the same query reads; top-1 against the truth,
    recall@H of the true peptide, the plain HMM over all peptides as the
    accuracy ceiling on a sample, and the kd-tree hybrid against the oracle
    on a sample.  Dye-track set and reads are simulated on the device."""
    import torch
    from whatprot_gb300 import capi
    from whatprot_gb300.simulate import paper_model, random_dye_seqs
    dev = f"cuda:{local}"
    sm = paper_model(C)
    ds = random_dye_seqs(HY_P, C, 8, 30, max_per_channel=5, min_total=1, seed=1234)
    ctx = capi.Context(local)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    t0 = time.perf_counter()
    dts = ctx.simulate_dye_track_set(HY_PER, seed=4321, to_nn=True)
    r_all, pep, _ = ctx.simulate_reads(int(reads * 1.1) + 64, seed=6060)
    keep = np.nonzero(pep >= 0)[0][:reads]
    rads = np.ascontiguousarray(r_all[keep])
    true_pep = pep[keep]
    true_ids = ds.ids[true_pep]
    R = rads.shape[0]
    gen_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    d_rads = torch.from_numpy(rads).to(dev)
    d_id = torch.empty(R, dtype=torch.int32, device=dev)
    d_sc = torch.empty(R, dtype=torch.float64, device=dev)
    d_tot = torch.empty(R, dtype=torch.float64, device=dev)
    h_rads = torch.from_numpy(rads).pin_memory().numpy()
    out = {"config": {"peptides": len(ds), "dye_tracks": len(dts), "track_sources": int(dts.src_off[-1]),
                      "reads_per_step": R, "k": HY_K, "sigma": HY_SIG, "h_knn": HY_H, "h_learned": LP_H,
                      "dist_cutoff": CUTOFF, "steps": steps, "warmup": warmup,
                      "l2": "flushed between steps (512 MB write)",
                      "data": "dye-track set (100 per dye-seq) and reads simulated on the device, seeded",
                      "data_generation_s": gen_s}}
    rows = {}
    for sel in ("kdtree", "prefix"):
        ctx.set_nn_selection(sel)

        def step():
            ctx.hybrid_classify_device(d_rads.data_ptr(), R, HY_K, HY_SIG, HY_H, CUTOFF, d_id.data_ptr(),
                                       d_sc.data_ptr(), d_tot.data_ptr())
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        ctx.timing_enable(True)
        ms = _timed_steps(stream, flush, step, steps)
        kt, _ = ctx.timing_read(ctx.KIND_KNN_TREE)
        kd, _ = ctx.timing_read(ctx.KIND_KNN_DIST)
        ks, _ = ctx.timing_read(ctx.KIND_KNN_SELECT)
        fw, _ = ctx.timing_read(ctx.KIND_FORWARD)
        ctx.timing_enable(False)
        gid = d_id.cpu().numpy()
        t0 = time.perf_counter()
        hid, hsc, htot = ctx.hybrid_classify(h_rads, HY_K, HY_SIG, HY_H, CUTOFF)
        e2e_s = time.perf_counter() - t0
        nc, cid, _, _ = ctx.nn_classify(rads, HY_K, HY_SIG, HY_H)
        recall = float(np.mean([true_ids[r] in set(cid[r, :nc[r]].tolist()) for r in range(R)]))
        rows[sel] = {"reads_per_s": R / (ms * 1e-3), "ms_per_step": ms,
                     "e2e": {"value": R / e2e_s, "unit": HY_UNIT, "h2d_bytes_per_step": int(rads.nbytes),
                             "d2h_bytes_per_step": int(R * 20)},
                     "top1_vs_truth": float(np.mean(gid == true_ids)), "recall_at_h": recall,
                     "ms_per_step_split": {"kd_tree_replay": kt / steps, "knn_distances": kd / steps,
                                           "knn_select": ks / steps, "hmm_forward": fw / steps},
                     "host_result": (hid, hsc, htot)}
    ctx.set_nn_selection("kdtree")
    # the learned proposal on the same reads
    net = capi.ProposalNet(ctx, hidden=LP_HIDDEN, seed=11)
    t0 = time.perf_counter()
    losses = [net.train(LP_EPOCH_READS, batch=LP_BATCH, lr=1e-3 if ep < epochs - 1 else 3e-4, seed=1000 + ep)
              for ep in range(epochs)]
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0

    def lstep():
        net.hybrid_classify_device(d_rads.data_ptr(), R, LP_H, CUTOFF, d_id.data_ptr(), d_sc.data_ptr(),
                                   d_tot.data_ptr())
    for _ in range(warmup):
        lstep()
    torch.cuda.synchronize()
    lms = _timed_steps(stream, flush, lstep, steps)
    lid = d_id.cpu().numpy()
    t0 = time.perf_counter()
    net.hybrid_classify(h_rads, LP_H, CUTOFF)
    le2e_s = time.perf_counter() - t0
    idx, _, _ = net.propose(rads, LP_H)
    lrecall = float(np.mean(np.any(idx == true_pep[:, None], axis=1)))
    net.close()
    learned = {"reads_per_s": R / (lms * 1e-3), "ms_per_step": lms,
               "e2e": {"value": R / le2e_s, "unit": HY_UNIT, "h2d_bytes_per_step": int(rads.nbytes),
                       "d2h_bytes_per_step": int(R * 20)},
               "top1_vs_truth": float(np.mean(lid == true_ids)), "recall_at_h": lrecall,
               "train_seconds": train_s, "train_epochs": epochs, "epoch_reads": LP_EPOCH_READS,
               "train_loss_per_epoch": losses}
    # accuracy ceiling: the plain HMM over all 20,000 peptides on a sample
    ns = min(R, 2000)
    fid, _, _, _ = ctx.classify(rads[:ns], CUTOFF)
    ceiling = {"reads": ns, "full_hmm_top1": float(np.mean(fid == true_ids[:ns])),
               "kdtree_hybrid_top1": float(np.mean(rows["kdtree"]["host_result"][0][:ns] == true_ids[:ns])),
               "prefix_hybrid_top1": float(np.mean(rows["prefix"]["host_result"][0][:ns] == true_ids[:ns])),
               "learned_hybrid_top1": float(np.mean(lid[:ns] == true_ids[:ns]))}
    # the kd-tree hybrid against the oracle's restatement of the reference
    parity = None
    try:
        sys.path.insert(0, os.path.join(REPO, "tests"))
        from oracle_lib import Oracle
        o = Oracle()
        n = min(R, oracle_reads)
        t0 = time.perf_counter()
        oid, osc, otot = o.hybrid_classify(sm, T, dts, ds, rads[:n], HY_K, HY_SIG, HY_H, CUTOFF,
                                           threads=os.cpu_count() or 1)
        o_s = time.perf_counter() - t0
        hid, hsc, htot = rows["kdtree"]["host_result"]
        same = hid[:n] == oid
        ga, oa = hsc[:n] / htot[:n], osc / otot
        rel = np.abs(ga - oa) / np.maximum(np.abs(oa), 1e-300)
        ll = None
        if not np.all(same):  # a different top-1 must be an HMM tie (equal probabilities to 1e-5)
            ll = ctx.loglik_all(rads[:n][~same], CUTOFF)
        tied = 0
        if ll is not None:
            index = {int(i): k for k, i in enumerate(ds.ids)}
            for j, r in enumerate(np.nonzero(~same)[0]):
                a, b = index[int(hid[r])], index[int(oid[r])]
                tied += int(abs(ll[j, a] - ll[j, b]) <= 1e-5)
        parity = {"reads": int(n), "top1_identical": float(np.mean(same)),
                  "top1_identical_or_tied": float((np.sum(same) + tied) / n),
                  "max_rel_err_adjusted_score": float(np.max(rel)), "tolerance": 1e-5,
                  "oracle": "oracle/wp_oracle.c kd-tree KBest restatement + FP64 HMM", "oracle_seconds": o_s}
    except Exception as e:  # the oracle is the checker: report, do not fail the bench
        parity = {"error": str(e)}
    for sel in rows:
        rows[sel].pop("host_result")
    ctx.close()
    res = {"config": out["config"], "knn_kdtree": rows["kdtree"], "knn_prefix": rows["prefix"],
           "learned": learned, "accuracy_ceiling": ceiling, "parity_kdtree_vs_oracle": parity,
           "learned_vs_knn_kdtree": learned["reads_per_s"] / rows["kdtree"]["reads_per_s"],
           "learned_vs_knn_prefix": learned["reads_per_s"] / rows["prefix"]["reads_per_s"],
           "learned_minus_knn_kdtree_top1_pts": 100 * (learned["top1_vs_truth"] - rows["kdtree"]["top1_vs_truth"]),
           "learned_minus_knn_prefix_top1_pts": 100 * (learned["top1_vs_truth"] - rows["prefix"]["top1_vs_truth"])}
    return res


def cpu_baseline_hybrid(sm, ds, dts, rads, seconds_target=15.0):
    """The CPU oracle's hybrid classifier (brute-force FP64 kNN, then the HMM
    over the candidates) on a bounded sample of the reads, all host threads."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_lib import Oracle
    threads = os.cpu_count() or 1
    o = Oracle()
    n = threads
    t0 = time.perf_counter()
    o.hybrid_classify(sm, T, dts, ds, rads[:n], HY_K, HY_SIG, HY_H, CUTOFF, threads=threads)
    dt = time.perf_counter() - t0
    n2 = int(min(len(rads), max(n, n * seconds_target / max(dt, 1e-3))))
    t0 = time.perf_counter()
    out = o.hybrid_classify(sm, T, dts, ds, rads[:n2], HY_K, HY_SIG, HY_H, CUTOFF, threads=threads)
    dt = time.perf_counter() - t0
    info = {"value": n2 / dt, "unit": HY_UNIT, "cores": threads, "kind": "port",
            "sample": f"{n2} reads of the same workload, {dt:.1f} s, oracle/wp_oracle.c "
                      f"wpo_hybrid_classify_batch (the reference's kd-tree KBest search, FP64) with "
                      f"{threads} threads"}
    return info, out[:3]


def run_reference_hybrid(args):
    """The reference's HybridClassifier (its own sources, oracle/_ref) on a
    bounded sample of the hybrid workload, all host threads; the oracle port
    where oracle/_ref is absent."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    sm, ds, dts, rads, _ = make_hybrid_data(seed=99, reads=4096)
    threads = os.cpu_count() or 1
    kind = "port"
    if oracle_lib.Reference.available():
        ref = oracle_lib.Reference()
        kind = "reference"

        def runner(x):
            return ref.hybrid_classify(sm, T, dts, ds, x, HY_K, HY_SIG, HY_H, CUTOFF, threads=threads)[3]
    else:
        o = oracle_lib.Oracle()

        def runner(x):
            t0 = time.perf_counter()
            o.hybrid_classify(sm, T, dts, ds, x, HY_K, HY_SIG, HY_H, CUTOFF, threads=threads)
            return time.perf_counter() - t0
    n = threads
    dt = runner(rads[:n])
    n = int(min(len(rads), max(n, n * 8.0 / max(dt, 1e-3))))
    for _ in range(args.warmup):
        runner(rads[:n])
    tot = 0.0
    for _ in range(args.steps):
        tot += runner(rads[:n])
    dt = tot / max(args.steps, 1)
    value = n / dt
    line = {"metric": HY_METRIC, "value": value, "unit": HY_UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded simulator)",
            "config": {"workload": HY_WORKLOAD, "sample_reads_per_step": n, "dye_tracks": len(dts),
                       "timed": "classify call only (classifier construction excluded)"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": HY_UNIT, "cores": threads, "kind": kind,
                             "sample": f"{n} reads per step"},
            "e2e": {"value": value, "unit": HY_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


DT_METRIC = "dye-tracks generated and deduplicated per second (simulate dt)"
DT_UNIT = "tracks/s"
DT_WORKLOAD = ("simulate dt: the hybrid workload's kNN training set -- 20000 dye-seqs (8-30 positions, <=5 dyes per "
               "channel, >=1 dye), 3 channels x 16 timesteps, 100 dye-tracks per dye-seq (2,000,000 instances) "
               "generated from the error model and deduplicated into unique tracks with (id, count, hits) sources")


def make_tracks_data(num=HY_P):
    from whatprot_gb300.simulate import paper_model, random_dye_seqs
    return paper_model(C), random_dye_seqs(num, C, 8, 30, max_per_channel=5, min_total=1, seed=1234)


def cpu_baseline_tracks(sm, ds, seconds_target=15.0):
    """The oracle's single-threaded generate_dye_tracks + dedup (C, as the
    reference runs them) on a bounded sample of the dye-seqs."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_lib import Oracle
    from whatprot_gb300.model import DyeSeqSet
    o = Oracle()

    def sample(m):
        return DyeSeqSet(ds.num_channels, ds.seqs[:m], ds.ids[:m], ds.counts[:m])

    m = 500
    t0 = time.perf_counter()
    o.simulate_dt(sm, T, sample(m), HY_PER, 11)
    dt = time.perf_counter() - t0
    m = int(min(len(ds), max(m, m * seconds_target / max(dt, 1e-3))))
    t0 = time.perf_counter()
    _, kept = o.simulate_dt(sm, T, sample(m), HY_PER, 12)
    dt = time.perf_counter() - t0
    n = m * HY_PER
    return {"value": n / dt, "unit": DT_UNIT, "cores": 1, "kind": "port",
            "sample": f"{m} dye-seqs x {HY_PER} tracks ({n} instances, {kept} detectable), {dt:.1f} s, "
                      f"oracle/wp_oracle.c wpo_simulate_dt (generate + sort-based dedup, one thread)"}


def run_tracks(args):
    import torch
    from whatprot_gb300 import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    sm, ds = make_tracks_data(args.dye_seqs)
    n = HY_PER * int(ds.counts.sum())
    ctx = capi.Context(local)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    seed = 100 + 1000003 * rank

    def step(i):
        ctx.simulate_dye_track_set(HY_PER, seed=seed + i, download=False)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    ctx.timing_enable(True)
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    total_ms = 0.0
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        step(args.warmup + i)
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
    barrier()
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    sim_ms, _ = ctx.timing_read(ctx.KIND_SIM)
    dd_ms, _ = ctx.timing_read(ctx.KIND_DEDUP)
    ctx.timing_enable(False)
    t_step = total_ms / args.steps
    if dist:
        t = torch.tensor([t_step], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    value = n * world / (t_step * 1e-3)
    # end to end through the public call: generate, dedup and download the
    # set into reusable page-locked host buffers
    bufs = capi.DyeTrackBuffers(n, n, T, C)
    ctx.simulate_dye_track_set(HY_PER, seed=seed, into=bufs)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        dts = ctx.simulate_dye_track_set(HY_PER, seed=seed + 7 * i, into=bufs)
    e2e_s = (time.perf_counter() - t0) / args.steps
    U, S = len(dts), int(dts.src_off[-1])
    TC = T * C
    e2e = {"value": n * world / e2e_s, "unit": DT_UNIT, "h2d_bytes_per_step": 0,
           "d2h_bytes_per_step": int(U * TC * 2 + (U + 1) * 4 + 3 * S * 4 + 8),
           "host_buffers": "page-locked, reused (capi.DyeTrackBuffers)"}
    # rooflines (HBM): the simulator's algorithmic traffic is its output,
    # n x (T*C track bytes + 4-byte peptide index); the dedup's is one read of
    # the instances (T*C bytes + 4-byte peptide index) and one write of the
    # set (int16 tracks, CSR offsets, 3 ints per source) -- what any dedup
    # must move; the sort passes in between are the dedup's own overhead
    peak = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f).get("hbm_gbs")
    except OSError:
        pass
    sim_step, dd_step = sim_ms / args.steps, dd_ms / args.steps
    sim_bytes = n * (TC + 4)
    dd_bytes = n * (TC + 4) + U * TC * 2 + (U + 1) * 4 + 3 * S * 4
    phases = {"simulator": {"kernel": "wp_sim_reads_kernel", "ms_per_step": sim_step,
                            "algorithmic_bytes": sim_bytes,
                            "achieved_gbs": sim_bytes / (sim_step * 1e-3) / 1e9 if sim_step > 0 else None},
              "dedup": {"kernel": "dd_* kernels + CUB radix sorts and scans", "ms_per_step": dd_step,
                        "algorithmic_bytes": dd_bytes,
                        "achieved_gbs": dd_bytes / (dd_step * 1e-3) / 1e9 if dd_step > 0 else None}}
    dom = "simulator" if sim_step >= dd_step else "dedup"
    ach = phases[dom]["achieved_gbs"]
    line = {"metric": DT_METRIC, "value": value, "unit": DT_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/int16 counts, fp64 draws", "data": "synthetic (seeded simulator)",
            "config": {"workload": DT_WORKLOAD if len(ds) == HY_P else f"{DT_WORKLOAD} (here {len(ds)} dye-seqs)",
                       "peptides": len(ds), "per_peptide": HY_PER, "instances": n,
                       "unique_tracks": U, "sources": S, "l2": "flushed between steps (512 MB write)"},
            "roofline": {"bound": "hbm", "kernel": phases[dom]["kernel"], "achieved": ach, "peak": peak,
                         "unit": "GB/s", "frac": ach / peak if (ach and peak) else None, "traffic": None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)", "phases": phases},
            "e2e": e2e, "gpu_launches": launches, "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_tracks(sm, ds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_reference_tracks(args):
    """The reference's generate_dye_tracks + dedup_dye_tracks (its own
    sources and MapReduce-MPI, oracle/_ref) on a bounded sample of the
    dye-seqs, one thread as it runs; the oracle port where oracle/_ref is
    absent."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    from whatprot_gb300.model import DyeSeqSet
    sm, ds = make_tracks_data()
    kind = "port"
    if oracle_lib.Reference.available():
        ref = oracle_lib.Reference()
        kind = "reference"

        def runner(sub, s):
            return ref.simulate_dt(sm, T, sub, HY_PER, s)[0]
    else:
        o = oracle_lib.Oracle()

        def runner(sub, s):
            t0 = time.perf_counter()
            o.simulate_dt(sm, T, sub, HY_PER, s)
            return time.perf_counter() - t0

    def sample(m):
        return DyeSeqSet(ds.num_channels, ds.seqs[:m], ds.ids[:m], ds.counts[:m])

    m = 500
    dt = runner(sample(m), 1)
    m = int(min(len(ds), max(m, m * 8.0 / max(dt, 1e-3))))
    for i in range(args.warmup):
        runner(sample(m), 2 + i)
    tot = 0.0
    for i in range(args.steps):
        tot += runner(sample(m), 100 + i)
    dt = tot / max(args.steps, 1)
    n = m * HY_PER
    value = n / dt
    line = {"metric": DT_METRIC, "value": value, "unit": DT_UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int16 counts, fp64 draws", "data": "synthetic (seeded simulator)",
            "config": {"workload": DT_WORKLOAD, "sample_peptides_per_step": m, "sample_instances_per_step": n},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": DT_UNIT, "cores": 1, "kind": kind,
                             "sample": f"{m} dye-seqs x {HY_PER} tracks per step"},
            "e2e": {"value": value, "unit": DT_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


LP_METRIC = "learned-proposal hybrid reads/s (MLP 48-1024-1024-20000 BF16, H=200 -> HMM -p 5)"
LP_H, LP_HIDDEN, LP_EPOCH_READS, LP_BATCH = 200, 1024, 10_000_000, 4096
LP_WORKLOAD = ("learned proposal: the hybrid workload's 20000 dye-seqs and query reads; MLP 48 -> 1024 -> 1024 -> "
               "20000 logits (GELU), BF16 weights and activations, FP32 accumulation on the tensor cores, trained "
               "with cross-entropy and Adam on 10,000,000 reads per epoch simulated on the GPU; top 200 proposals "
               "rescored by the HMM (-p 5)")


def run_learned(args):
    import torch
    from whatprot_gb300 import capi

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    reads = args.reads if args.reads != READS else HY_READS
    sm, ds, dts, rads, true_ids = make_hybrid_data(seed=5050 + rank, reads=reads)
    R = rads.shape[0]
    ctx = capi.Context(local)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    net = capi.ProposalNet(ctx, hidden=LP_HIDDEN, seed=11)
    t0 = time.perf_counter()
    losses = []
    for ep in range(args.epochs):
        losses.append(net.train(LP_EPOCH_READS, batch=LP_BATCH, lr=1e-3 if ep < args.epochs - 1 else 3e-4,
                                seed=1000 + ep))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    d_rads = torch.from_numpy(rads).to(f"cuda:{local}")
    d_id = torch.empty(R, dtype=torch.int32, device=f"cuda:{local}")
    d_sc = torch.empty(R, dtype=torch.float64, device=f"cuda:{local}")
    d_tot = torch.empty(R, dtype=torch.float64, device=f"cuda:{local}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def step():
        net.hybrid_classify_device(d_rads.data_ptr(), R, LP_H, CUTOFF, d_id.data_ptr(), d_sc.data_ptr(),
                                   d_tot.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ctx.timing_enable(True)
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        step()
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    fw_ms, _ = ctx.timing_read(4)
    tk_ms, _ = ctx.timing_read(5)
    hmm_ms, _ = ctx.timing_read(ctx.KIND_FORWARD)
    ctx.timing_enable(False)
    t_step = total_ms / args.steps
    value = R / (t_step * 1e-3)
    ids = d_id.cpu().numpy()
    acc = float((ids == true_ids).mean())
    idx, prob, mass = net.propose(rads, LP_H)
    index = {int(i): n for n, i in enumerate(ds.ids)}
    tidx = np.array([index[int(i)] for i in true_ids])
    recall = float(np.mean(np.any(idx == tidx[:, None], axis=1)))
    # the plain kNN hybrid on the same reads, for the comparison at matched accuracy
    ctx.upload_tracks(dts)
    t0 = time.perf_counter()
    kid, _, _ = ctx.hybrid_classify(rads, HY_K, HY_SIG, HY_H, CUTOFF)
    knn_s = time.perf_counter() - t0
    knn_acc = float((kid == true_ids).mean())
    h_rads = torch.from_numpy(rads).pin_memory().numpy()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        net.hybrid_classify(h_rads, LP_H, CUTOFF)
    e2e_s = (time.perf_counter() - t0) / args.steps
    fwd_flops = 2.0 * R * (64 * LP_HIDDEN + LP_HIDDEN * LP_HIDDEN + LP_HIDDEN * ((len(ds) + 63) // 64 * 64))
    fw_step = fw_ms / args.steps
    peak = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f).get("bf16_tflops")
    except OSError:
        pass
    achieved = fwd_flops / (fw_step * 1e-3) / 1e12 if fw_step > 0 else None
    line = {"metric": LP_METRIC, "value": value, "unit": HY_UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (network) / fp32 (HMM)", "data": "synthetic (seeded simulator)",
            "config": {"workload": LP_WORKLOAD, "reads": R, "peptides": len(ds), "h": LP_H, "epochs": args.epochs,
                       "epoch_reads": LP_EPOCH_READS, "batch": LP_BATCH, "l2": "flushed between steps (512 MB write)"},
            "top1_vs_truth": acc, "recall_at_h": recall, "train_seconds": train_s, "train_loss_per_epoch": losses,
            "knn_hybrid": {"reads_per_s_e2e": R / knn_s, "top1_vs_truth": knn_acc, "k": HY_K, "h": HY_H},
            "roofline": {"bound": "tensor", "kernel": "wp_gemm_tn_kernel (forward layers)", "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if (achieved and peak) else None,
                         "traffic": None, "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)",
                         "algorithmic_flops_per_step": fwd_flops, "forward_ms_per_step": fw_step,
                         "topk_ms_per_step": tk_ms / args.steps, "hmm_forward_ms_per_step": hmm_ms / args.steps},
            "e2e": {"value": R / e2e_s, "unit": HY_UNIT, "h2d_bytes_per_step": int(rads.nbytes),
                    "d2h_bytes_per_step": int(R * 20)},
            "gpu_launches": launches, "clocks": clk}
    print(json.dumps(line), flush=True)
    net.close()
    ctx.close()


def run_gemm(args):
    """The tensor-core GEMM alone on the proposal network's largest product
    (logits of 8192 reads: M 8192, N 20032, K 1024), BF16 in, FP32 out."""
    import torch
    from whatprot_gb300 import capi
    torch.cuda.set_device(0)
    M, N, K = 8192, 20032, 1024
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    for _ in range(args.warmup):
        capi.gemm_bf16(A, B)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        capi.gemm_bf16(A, B)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = sorted(ms)[len(ms) // 2]
    flops = 2.0 * M * N * K
    peak = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f).get("bf16_tflops")
    except OSError:
        pass
    tf = flops / (t * 1e-3) / 1e12
    print(json.dumps({"metric": "tcgen05 BF16 GEMM TFLOP/s (M 8192, N 20032, K 1024, FP32 out)", "value": tf,
                      "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t,
                      "higher_is_better": True, "dtype": "bf16", "data": "synthetic",
                      "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s",
                                   "frac": tf / peak if peak else None, "traffic": None,
                                   "kernel": "wp_gemm_tn_kernel"}}), flush=True)


FIT_METRIC = "Baum-Welch E-step reads/s (fit, 1 dye-seq 4/3/3 dyes, no pruning)"
FIT_UNIT = "reads/s"
FIT_READS, FIT_LEN = 200_000, 20
FIT_ORACLE_READS = 4000  # the subset fitted by both the GPU and the FP64 oracle
FIT_WORKLOAD = ("fit: 3 channels x 16 timesteps, 1 dye-seq of 20 positions with 4/3/3 dyes "
                "(positions seeded), 200000 reads float64 [200000,16,3], unpruned")


def make_fit_data(seed: int, reads: int):
    from whatprot_gb300.model import DyeSeqSet
    from whatprot_gb300.simulate import paper_model, simulate_radiometries
    sm = paper_model(C)
    rng = np.random.default_rng(4)
    seq = np.full(FIT_LEN, -1, np.int16)
    pos = rng.permutation(FIT_LEN)[:10]
    seq[pos[:4]] = 0
    seq[pos[4:7]] = 1
    seq[pos[7:]] = 2
    ds = DyeSeqSet(C, [seq], np.array([0], np.int32), np.array([1], np.int32))
    rads, _ = simulate_radiometries(sm, ds, T, int(reads * 1.1) + 64, seed=seed)
    return sm, seq, rads[:reads].copy()


def perturbed(sm, seed):
    import copy
    rng = np.random.default_rng(seed)
    out = copy.deepcopy(sm)
    out.p_edman_failure *= rng.uniform(0.5, 1.5)
    out.p_detach *= rng.uniform(0.5, 1.5)
    for cm in out.channel_models:
        cm.p_bleach *= rng.uniform(0.5, 1.5)
        cm.p_dud *= rng.uniform(0.5, 1.5)
    return out


def make_data(seed: int, reads: int):
    from whatprot_gb300.simulate import paper_model, random_dye_seqs, simulate_radiometries
    sm = paper_model(C)
    ds = random_dye_seqs(P, C, 8, 30, max_per_channel=5, min_total=1, seed=1234)
    rads, ids = simulate_radiometries(sm, ds, T, int(reads * 1.15) + 64, seed=seed)
    return sm, ds, rads[:reads].copy(), ids[:reads].copy()


class GpmDram:
    """DRAM traffic over an interval from NVML's GPU performance monitoring
    (GPM) counters, read through the driver's libnvidia-ml with ctypes: the
    DRAM bandwidth utilisation between two samples (percent of the
    theoretical bandwidth, bus width x memory clock x 2) times that
    bandwidth and the interval.  `measure(fn)` returns (bytes, seconds,
    percent) or raises; the GPU is only read, nothing is set."""

    METRIC_DRAM_BW_UTIL = 10
    METRIC_MAX = 210

    def __init__(self, device: int):
        import ctypes
        import torch
        self.ct = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        self.lib = lib
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        props = torch.cuda.get_device_properties(device)
        self.handle = ctypes.c_void_p()
        uuid = ("GPU-" + str(props.uuid)).encode()
        if lib.nvmlDeviceGetHandleByUUID(ctypes.c_char_p(uuid), ctypes.byref(self.handle)) != 0:
            raise RuntimeError("no NVML handle for the device")

        class Support(ctypes.Structure):
            _fields_ = [("version", ctypes.c_uint), ("isSupportedDevice", ctypes.c_uint)]

        sup = Support(1, 0)
        if lib.nvmlGpmQueryDeviceSupport(self.handle, ctypes.byref(sup)) != 0 or not sup.isSupportedDevice:
            raise RuntimeError("GPM not supported on this device")

        class Info(ctypes.Structure):
            _fields_ = [("shortName", ctypes.c_char_p), ("longName", ctypes.c_char_p), ("unit", ctypes.c_char_p)]

        class Metric(ctypes.Structure):
            _fields_ = [("metricId", ctypes.c_uint), ("nvmlReturn", ctypes.c_int), ("value", ctypes.c_double),
                        ("metricInfo", Info)]

        class MetricsGet(ctypes.Structure):
            _fields_ = [("version", ctypes.c_uint), ("numMetrics", ctypes.c_uint), ("sample1", ctypes.c_void_p),
                        ("sample2", ctypes.c_void_p), ("metrics", Metric * GpmDram.METRIC_MAX)]

        self.MetricsGet = MetricsGet
        # the theoretical bandwidth the percentage refers to: bus width x
        # maximum memory clock x 2 (double data rate)
        mhz, bits = ctypes.c_uint(0), ctypes.c_uint(0)
        if (lib.nvmlDeviceGetMaxClockInfo(self.handle, 2, ctypes.byref(mhz)) != 0 or
                lib.nvmlDeviceGetMemoryBusWidth(self.handle, ctypes.byref(bits)) != 0 or not mhz.value or
                not bits.value):
            raise RuntimeError("memory clock or bus width unavailable")
        self.peak_bytes_s = 2.0 * mhz.value * 1e6 * bits.value / 8.0

    def measure(self, fn):
        ct, lib = self.ct, self.lib
        s1, s2 = ct.c_void_p(), ct.c_void_p()
        if lib.nvmlGpmSampleAlloc(ct.byref(s1)) != 0 or lib.nvmlGpmSampleAlloc(ct.byref(s2)) != 0:
            raise RuntimeError("GPM sample allocation failed")
        try:
            if lib.nvmlGpmSampleGet(self.handle, s1) != 0:
                raise RuntimeError("GPM sample failed")
            t0 = time.perf_counter()
            fn()
            t1 = time.perf_counter()
            if lib.nvmlGpmSampleGet(self.handle, s2) != 0:
                raise RuntimeError("GPM sample failed")
            mg = self.MetricsGet()
            mg.version = 1
            mg.numMetrics = 1
            mg.sample1 = s1
            mg.sample2 = s2
            mg.metrics[0].metricId = self.METRIC_DRAM_BW_UTIL
            if lib.nvmlGpmMetricsGet(ct.byref(mg)) != 0 or mg.metrics[0].nvmlReturn != 0:
                raise RuntimeError("GPM metrics unavailable")
            pct = mg.metrics[0].value
            return pct / 100.0 * self.peak_bytes_s * (t1 - t0), t1 - t0, pct
        finally:
            lib.nvmlGpmSampleFree(s1)
            lib.nvmlGpmSampleFree(s2)


def engine_traffic_live(ctx, device: int, steps_equiv_ms: float):
    """DRAM bytes of one replay of the engine passes (all passes and the
    dense kernel of the last classify batch), measured on this run: NVML GPM
    over enough replays to span a few hundred ms (GPM samples refresh every
    100 ms).  Returns (bytes per replay, source note) or (None, reason)."""
    import torch
    try:
        g = GpmDram(device)
    except Exception as e:  # noqa: BLE001 - any NVML absence is reported, not fatal
        return None, f"NVML GPM unavailable: {e}"
    reps = max(8, int(400.0 / max(steps_equiv_ms, 0.1)))
    ctx.engine_replay(2)  # warm
    try:
        nbytes, secs, pct = g.measure(lambda: (ctx.engine_replay(reps), torch.cuda.synchronize()))
    except Exception as e:  # noqa: BLE001
        return None, f"NVML GPM failed: {e}"
    return nbytes / reps, (f"NVML GPM DRAM bandwidth utilisation {pct:.2f} % of the theoretical "
                           f"{g.peak_bytes_s / 1e9:.0f} GB/s over {reps} replays of the engine passes "
                           f"({secs * 1e3:.0f} ms), per replay")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_baseline(sm, ds, rads, seconds_target=15.0):
    """Time the CPU oracle (a restatement of the reference's algorithm,
    pthreads over reads) on a bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_lib import Oracle
    threads = os.cpu_count() or 1
    o = Oracle()
    n = max(threads, 16)
    t0 = time.perf_counter()
    o.classify(sm, T, ds, rads[:n], CUTOFF, threads=threads)
    dt = time.perf_counter() - t0
    # grow the sample to about seconds_target of work
    n2 = int(min(len(rads), max(n, n * seconds_target / max(dt, 1e-3))))
    t0 = time.perf_counter()
    oid, osc, otot = o.classify(sm, T, ds, rads[:n2], CUTOFF, threads=threads)
    dt = time.perf_counter() - t0
    info = {"value": n2 * len(ds) / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n2} reads x {len(ds)} dye-seqs of the same workload, "
                      f"{dt:.1f} s, oracle/wp_oracle.c with {threads} threads"}
    # the same on one host thread, a smaller sample (about 5 s)
    m = max(4, int(n2 * 5.0 / max(dt * threads, 1e-3)))
    t0 = time.perf_counter()
    o.classify(sm, T, ds, rads[:m], CUTOFF, threads=1)
    dt1 = time.perf_counter() - t0
    info["one_thread"] = {"value": m * len(ds) / dt1, "unit": UNIT, "cores": 1,
                          "sample": f"{m} reads x {len(ds)} dye-seqs, {dt1:.1f} s"}
    return info, (oid, osc, otot)


def unpruned_forward_flops(seqs, T, C):
    """The unpruned forward's op count per read summed over the dye-seqs
    (the context figure of the visited-state count): per dye-seq with D_c
    dyes per channel, S = prod_c (D_c + 1) states per Edman slice and
    B = sum_c (D_c + 2), the duds S * B at t = 0 and (t + 1) * S * (3 + [t > 0]
    * (8 + B)) at every timestep (emission and rescale 3; detach 2, Edman 6
    and the binomial steps about B per state)."""
    total = 0.0
    for seq in seqs:
        D = [int(np.sum(np.asarray(seq) == c)) for c in range(C)]
        S = float(np.prod([d + 1 for d in D]))
        B = float(sum(d + 2 for d in D))
        f = S * B
        for t in range(T):
            f += (t + 1) * S * (3.0 + ((8.0 + B) if t > 0 else 0.0))
        total += f
    return total


def loglik_parity(ctx, sm, ds, rads, n=500):
    """Per-pair log P of the GPU engine (FP32 with exact power-of-two
    rescaling) against the oracle's FP64 log P on the first n reads of the
    workload, all peptides: the largest and median |delta log P| over every
    pair both find possible, and over each read's best pair; pairs one side
    finds impossible (P = 0) and the other not are counted."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_lib import Oracle
    n = min(n, len(rads))
    g = ctx.loglik_all(rads[:n], CUTOFF)
    o = Oracle().loglik_all(sm, T, ds, rads[:n], CUTOFF, threads=os.cpu_count() or 1)
    fin = np.isfinite(g) & np.isfinite(o)
    d = np.abs(g[fin] - o[fin])
    best = np.argmax(np.where(np.isfinite(o), o, -np.inf), axis=1)
    db = np.abs(g[np.arange(n), best] - o[np.arange(n), best])
    db = db[np.isfinite(db)]
    return {"reads": int(n), "pairs": int(n * len(ds)), "finite_pairs": int(fin.sum()),
            "zero_mismatches": int(np.sum(np.isfinite(g) != np.isfinite(o))),
            "all_pairs_max_abs": float(d.max()) if d.size else None,
            "all_pairs_median_abs": float(np.median(d)) if d.size else None,
            "best_pair_max_abs": float(db.max()) if db.size else None,
            "best_pair_median_abs": float(np.median(db)) if db.size else None,
            "tolerance_abs": 1e-5}


def sample_parity(gpu, oracle_out):
    """The GPU's classify results against the oracle's FP64 results on the
    baseline's sample: top-1 agreement, and the largest relative difference
    of the adjusted score (P_best / total) where the ids agree."""
    gid, gsc, gtot = gpu
    oid, osc, otot = oracle_out
    n = len(oid)
    gid, gsc, gtot = gid[:n], gsc[:n], gtot[:n]
    same = gid == oid
    ga = np.where(gtot > 0, gsc / np.where(gtot > 0, gtot, 1), 0.0)
    oa = np.where(otot > 0, osc / np.where(otot > 0, otot, 1), 0.0)
    rel = np.abs(ga - oa) / np.maximum(np.abs(oa), 1e-300)
    # a different id whose probability equals the oracle's best within the
    # tolerance is a tie of the reference's own scores (first index wins
    # there; FP32 rounding may pick the other)
    tie = ~same & (np.abs(gsc - osc) <= 1e-5 * np.maximum(np.abs(osc), 1e-300))
    return {"reads": int(n), "top1_identical": float(np.mean(same)),
            "top1_identical_or_tied": float(np.mean(same | tie)),
            "max_rel_err_adjusted_score": float(np.max(rel[same])) if np.any(same) else None,
            "tolerance": 1e-5}


def run_reference(args):
    """The reference's CPU implementation of the path, timed on the host:
    oracle/_ref (the reference's own sources) when it was built for this
    machine, else the oracle port; all host threads; each step classifies a
    bounded sample of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    sm, ds, rads, _ = make_data(seed=99, reads=4096)
    threads = os.cpu_count() or 1
    kind = "port"
    runner = None
    if oracle_lib.Reference.available():
        try:
            ref = oracle_lib.Reference()
            kind = "reference"

            def runner(x):
                ref.classify(sm, T, ds, x, CUTOFF, threads=threads)
        except OSError:
            runner = None
    if runner is None:
        o = oracle_lib.Oracle()

        def runner(x):
            o.classify(sm, T, ds, x, CUTOFF, threads=threads)
    # size a step to about 8 s of CPU work
    n = max(threads * 2, 32)
    t0 = time.perf_counter()
    runner(rads[:n])
    dt = time.perf_counter() - t0
    n = int(min(len(rads), max(n, n * 8.0 / max(dt, 1e-3))))
    for _ in range(args.warmup):
        runner(rads[:n])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        runner(rads[:n])
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = n * len(ds) / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded simulator)",
            "config": {"workload": WORKLOAD, "sample_reads_per_step": n, "peptides": len(ds)},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{n} reads x {len(ds)} dye-seqs per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_fit(args):
    """The reference's E-step (PeptideHMM::improve_fit from its own sources,
    oracle/_ref) over a bounded sample of the fit workload's reads, split
    across all host threads; the oracle port where oracle/_ref is absent."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    from whatprot_gb300.model import dye_seq_string
    sm, seq, rads = make_fit_data(seed=99, reads=20000)
    threads = os.cpu_count() or 1
    kind = "port"
    runner = None
    if oracle_lib.Reference.available():
        try:
            ref = oracle_lib.Reference()
            kind = "reference"
            s = dye_seq_string(seq)

            def runner(x):
                ref.improve_fit_batch(sm, T, s, x, threads=threads)
        except OSError:
            runner = None
    if runner is None:
        o = oracle_lib.Oracle()

        def runner(x):
            o.improve_fit_batch(sm, T, seq, x, threads=threads)
    n = max(threads * 2, 32)
    t0 = time.perf_counter()
    runner(rads[:n])
    dt = time.perf_counter() - t0
    n = int(min(len(rads), max(n, n * 8.0 / max(dt, 1e-3))))
    for _ in range(args.warmup):
        runner(rads[:n])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        runner(rads[:n])
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = n / dt
    line = {"metric": FIT_METRIC, "value": value, "unit": FIT_UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded simulator)",
            "config": {"workload": FIT_WORKLOAD, "sample_reads_per_step": n}, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": FIT_UNIT, "cores": threads, "kind": kind,
                             "sample": f"{n} reads per step"},
            "e2e": {"value": value, "unit": FIT_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_fit(sm, seq, rads, seconds_target=15.0):
    """The CPU oracle's E-step on a bounded sample, all host threads."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    from oracle_lib import Oracle
    threads = os.cpu_count() or 1
    o = Oracle()
    n = max(threads * 2, 32)
    t0 = time.perf_counter()
    o.improve_fit_batch(sm, T, seq, rads[:n], threads=threads)
    dt = time.perf_counter() - t0
    n2 = int(min(len(rads), max(n, n * seconds_target / max(dt, 1e-3))))
    t0 = time.perf_counter()
    o.improve_fit_batch(sm, T, seq, rads[:n2], threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n2 / dt, "unit": FIT_UNIT, "cores": threads, "kind": "port",
            "sample": f"{n2} reads of the same workload, {dt:.1f} s, oracle/wp_oracle.c "
                      f"wpo_improve_fit_batch with {threads} threads"}


def run_fit(args):
    import torch
    from whatprot_gb300 import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    reads = args.reads if args.reads != READS else FIT_READS
    sm, seq, rads = make_fit_data(seed=3030 + rank, reads=reads)
    R = rads.shape[0]
    ctx = capi.Context(local)
    start = perturbed(sm, 77)
    ctx.upload_model(start, T)
    h_rads = torch.from_numpy(rads).pin_memory()
    h_np = h_rads.numpy()
    ctx.fit_begin(seq, h_np)  # reads resident on the device from here
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    for _ in range(args.warmup):
        ctx.fit_estep()
    torch.cuda.synchronize()
    ctx.timing_enable(True)
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    total_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        ctx.fit_estep()
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
    barrier()
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    k_ms, k_n = ctx.timing_read(ctx.KIND_FORWARD)
    prep_ms, _ = ctx.timing_read(ctx.KIND_PREP)
    ctx.timing_enable(False)
    t_step = total_ms / args.steps
    if dist:
        t = torch.tensor([t_step], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    value = R * world / (t_step * 1e-3)
    # end to end: stage the host reads and run the E-step, every step
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.fit_begin(seq, h_np)
        ctx.fit_estep()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e = {"value": R * world / e2e_s, "unit": FIT_UNIT, "h2d_bytes_per_step": int(rads.nbytes),
           "d2h_bytes_per_step": int(R * 8 + 8 * (6 + 2 * (T - 1) + 4 * C))}
    # one full fit from the perturbed start (stops on a 1e-6 step)
    t0 = time.perf_counter()
    fitted, step, log_l, iters = ctx.hmm_fit(start, T, seq, h_np, 1e-6, 600.0)
    fit_s = time.perf_counter() - t0
    # the detach rate enters as the curve base + initial * exp(-decay * t)
    # (base and initial trade off when decay is 0), so compare the curve
    curve = lambda m: [m.p_detach_at(t) for t in range(T - 1)]
    err = max([abs(fitted.p_edman_failure - sm.p_edman_failure)]
              + [abs(a - b) for a, b in zip(curve(fitted), curve(sm))]
              + [abs(a.p_bleach - b.p_bleach) for a, b in zip(fitted.channel_models, sm.channel_models)]
              + [abs(a.p_dud - b.p_dud) for a, b in zip(fitted.channel_models, sm.channel_models)])
    # every parameter, mu / sig / bg_sig included (fit_emission; the reference
    # fits the rates only), from a start with each of them perturbed too
    rng = np.random.default_rng(78)
    start_e = perturbed(sm, 77)
    for cm in start_e.channel_models:
        cm.mu *= float(rng.uniform(0.5, 1.5))
        cm.sig *= float(rng.uniform(0.5, 1.5))
        cm.bg_sig *= float(rng.uniform(0.5, 1.5))
    ctx.upload_model(start_e, T)
    ctx.fit_begin(seq, h_np)
    ctx.fit_set_emission(True)
    ctx.fit_estep()  # warm
    t0 = time.perf_counter()
    ctx.fit_estep()
    est_e_s = time.perf_counter() - t0
    ctx.fit_set_emission(False)
    t0 = time.perf_counter()
    fitted_e, step_e, log_l_e, iters_e = ctx.hmm_fit(start_e, T, seq, h_np, 1e-6, 600.0, fit_emission=True)
    fit_e_s = time.perf_counter() - t0
    rel = lambda a, b: abs(a - b) / abs(b)
    err_e = {"rates_max_abs": max([abs(fitted_e.p_edman_failure - sm.p_edman_failure)]
                                  + [abs(a - b) for a, b in zip(curve(fitted_e), curve(sm))]
                                  + [abs(a.p_bleach - b.p_bleach) for a, b in zip(fitted_e.channel_models,
                                                                                   sm.channel_models)]
                                  + [abs(a.p_dud - b.p_dud) for a, b in zip(fitted_e.channel_models,
                                                                             sm.channel_models)]),
             "mu_max_rel": max(rel(a.mu, b.mu) for a, b in zip(fitted_e.channel_models, sm.channel_models)),
             "sig_max_rel": max(rel(a.sig, b.sig) for a, b in zip(fitted_e.channel_models, sm.channel_models)),
             "bg_sig_max_rel": max(rel(a.bg_sig, b.bg_sig)
                                   for a, b in zip(fitted_e.channel_models, sm.channel_models))}
    # the FP32 E-step's effect on the fitted parameters: the same fit on a
    # bounded subset of the reads, on the GPU and with the oracle's FP64
    # E-step (same start, same host M-step)
    fit_oracle = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "tests"))
        from oracle_lib import oracle_em
        sub = np.ascontiguousarray(h_np[:FIT_ORACLE_READS])
        ctx.upload_model(start, T)
        g_fit, g_step, _, g_it = ctx.hmm_fit(start, T, seq, sub, 1e-6, 600.0)
        t0 = time.perf_counter()
        o_fit, o_step, o_it = oracle_em(start, T, seq, sub, 1e-6, threads=os.cpu_count() or 1)
        o_s = time.perf_counter() - t0
        per = {"p_edman_failure": abs(g_fit.p_edman_failure - o_fit.p_edman_failure),
               "p_detach_curve_max": max(abs(a - b) for a, b in zip(curve(g_fit), curve(o_fit))),
               "p_bleach": [abs(a.p_bleach - b.p_bleach) for a, b in zip(g_fit.channel_models, o_fit.channel_models)],
               "p_dud": [abs(a.p_dud - b.p_dud) for a, b in zip(g_fit.channel_models, o_fit.channel_models)]}
        worst = max([per["p_edman_failure"], per["p_detach_curve_max"]] + per["p_bleach"] + per["p_dud"])
        fit_oracle = {"reads": int(sub.shape[0]), "threshold": 1e-6, "gpu_iterations": g_it,
                      "oracle_iterations": o_it, "oracle_seconds": o_s,
                      "abs_diff_gpu_vs_fp64_oracle": per, "max_abs_diff": worst, "tolerance_abs": 1e-5,
                      "oracle": "oracle/wp_oracle.c FP64 E-step (wpo_improve_fit_batch) + the library's host "
                                "M-step (wp_fit_mstep)",
                      "gpu_max_abs_error_vs_generating_model": max(
                          [abs(g_fit.p_edman_failure - sm.p_edman_failure)]
                          + [abs(a - b) for a, b in zip(curve(g_fit), curve(sm))]
                          + [abs(a.p_bleach - b.p_bleach) for a, b in zip(g_fit.channel_models, sm.channel_models)]
                          + [abs(a.p_dud - b.p_dud) for a, b in zip(g_fit.channel_models, sm.channel_models)])}
    k_avg = k_ms / max(k_n, 1)
    fit_flops = 3.0 * R * unpruned_forward_flops([seq], T, C)
    fit_peak = ctx.fp32_peak_tflops()
    fit_achieved = fit_flops / (k_avg * 1e-3) / 1e12 if k_avg > 0 else None
    line = {"metric": FIT_METRIC, "value": value, "unit": FIT_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded simulator)",
            "config": {"workload": FIT_WORKLOAD, "reads": R, "timesteps": T, "channels": C,
                       "dye_seq": "".join("." if d < 0 else str(int(d)) for d in seq),
                       "l2": "flushed between steps (512 MB write)"},
            "roofline": {"bound": "fp32", "kernel": "wp_fit_cta_kernel", "achieved": fit_achieved,
                         "peak": fit_peak, "unit": "TFLOP/s",
                         "frac": (fit_achieved / fit_peak) if (fit_achieved and fit_peak) else None,
                         "traffic": None, "algorithmic_flops_per_step": fit_flops,
                         "flop_model": "3 x the unpruned forward op count of the dye-seq per read "
                                       "(forward, backward from the checkpoints, expected counts)",
                         "estep_kernel_ms": k_avg, "prep_ms_per_step": prep_ms / args.steps},
            "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "fit": {"iterations": iters, "seconds": fit_s, "final_step": step, "log_l": log_l,
                    "max_abs_error_vs_generating_model": err,
                    "fitted": {"p_edman_failure": fitted.p_edman_failure, "p_detach": fitted.p_detach,
                               "p_initial_detach": fitted.p_initial_detach,
                               "p_initial_detach_decay": fitted.p_initial_detach_decay,
                               "p_bleach": [c.p_bleach for c in fitted.channel_models],
                               "p_dud": [c.p_dud for c in fitted.channel_models]}},
            "fit_all_params": {"iterations": iters_e, "seconds": fit_e_s, "final_step": step_e, "log_l": log_l_e,
                               "estep_with_emission_statistics_s": est_e_s, "error_vs_generating_model": err_e,
                               "fitted_mu": [c.mu for c in fitted_e.channel_models],
                               "fitted_sig": [c.sig for c in fitted_e.channel_models],
                               "fitted_bg_sig": [c.bg_sig for c in fitted_e.channel_models]},
            "fit_vs_fp64_oracle": fit_oracle}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_fit(sm, seq, rads)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--reads", type=int, default=READS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-subrecords", action="store_true",
                    help="classify: leave out the hybrid / learned sub-records")
    ap.add_argument("--workload", default="classify",
                    choices=["classify", "fit", "hybrid", "learned", "gemm", "tracks"])
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--dye-seqs", type=int, default=HY_P,
                    help="tracks: number of dye-seqs (a smaller case for profiling)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="classify: skip the engine autotuner and use the default launch shapes")
    ap.add_argument("--engine-shape", default=None,
                    help="classify: fixed engine launch shapes t1,s1,t2,s2 instead of the autotuner's")
    args = ap.parse_args()
    if args.workload == "gemm":
        return run_gemm(args)
    if args.workload == "learned":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned proposal"}))
            return
        return run_learned(args)
    if args.workload == "hybrid":
        return run_reference_hybrid(args) if args.impl == "reference" else run_hybrid(args)
    if args.workload == "tracks":
        return run_reference_tracks(args) if args.impl == "reference" else run_tracks(args)
    if args.workload == "fit":
        return run_reference_fit(args) if args.impl == "reference" else run_fit(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    from whatprot_gb300 import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    sm, ds, rads, _ = make_data(seed=2024 + rank, reads=args.reads)
    R = rads.shape[0]
    ctx = capi.Context(local)
    ctx.upload_model(sm, T)
    ctx.upload_peptides(ds)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    d_rads = torch.from_numpy(rads).to(f"cuda:{local}")
    d_id = torch.empty(R, dtype=torch.int32, device=f"cuda:{local}")
    d_sc = torch.empty(R, dtype=torch.float64, device=f"cuda:{local}")
    d_tot = torch.empty(R, dtype=torch.float64, device=f"cuda:{local}")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def step_device():
        ctx.classify_device(d_rads.data_ptr(), R, CUTOFF, d_id.data_ptr(), d_sc.data_ptr(),
                            d_tot.data_ptr(), async_=True)

    # the project's autotuner picks the engine launch shapes on a sample
    if args.engine_shape:  # fixed shapes (profiling runs repeat a bench run's choice)
        tuned_cfg, tuned_ms = tuple(int(x) for x in args.engine_shape.split(",")), None
        ctx.set_engine_config(tuned_cfg)
    elif args.no_autotune:  # default shapes (used for short profiling runs)
        tuned_cfg, tuned_ms = (256, 2, 256, 1), None
    else:
        tuned_cfg, tuned_ms = ctx.autotune(rads[:min(R, 50000)], CUTOFF)
    for _ in range(args.warmup):  # the second call captures the CUDA graph
        step_device()
    torch.cuda.synchronize()
    stream.synchronize()

    algo_flops = ctx.count_flops(rads, CUTOFF)  # per step, outside the timed region
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    total_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)  # evict L2 (129 MB) between steps, outside the events
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        step_device()
        ev1.record(stream)
        ev1.synchronize()
        total_ms += ev0.elapsed_time(ev1)
    barrier()
    clk = clocks.stop()
    launches = ctx.launch_count() - launches0
    # per-kernel split from two more steps with event timing on (direct
    # launches: graphs are not used while per-kernel timing is on)
    ctx.timing_enable(True)
    split_steps = 2
    for _ in range(split_steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        step_device()
    stream.synchronize()
    work = ctx.last_batch_stats()
    fwd_ms, fwd_n = ctx.timing_read(ctx.KIND_FORWARD)
    prep_ms, _ = ctx.timing_read(ctx.KIND_PREP)
    ctx.timing_enable(False)
    t_step = total_ms / args.steps
    if dist:
        t = torch.tensor([t_step], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    pairs = float(R) * len(ds)
    value = pairs * world / (t_step * 1e-3)

    # End to end through the public API with host (pinned) buffers: the
    # reads in and the per-read outputs back, the caller's buffers reused
    # from batch to batch as a whatprot host loop would.
    h_rads = torch.from_numpy(rads).pin_memory()
    h_np = h_rads.numpy()
    h_out = (torch.zeros(R, dtype=torch.int32).pin_memory().numpy(),
             *(torch.zeros(R, dtype=torch.float64).pin_memory().numpy() for _ in range(3)))
    for _ in range(1):
        ctx.classify(h_np, CUTOFF, out=h_out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        last_gpu = ctx.classify(h_np, CUTOFF, out=h_out)[:3]
    e2e_s = (time.perf_counter() - t0) / args.steps
    if dist:
        t = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": pairs * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(rads.nbytes),
           "d2h_bytes_per_step": int(R * (4 + 8 + 8 + 8))}

    # DRAM traffic of the engine passes, measured now (replays of the last
    # batch's passes under NVML GPM); the ncu figure below is the fallback
    live_bytes, live_src = engine_traffic_live(ctx, local, fwd_ms / split_steps if split_steps else 20.0)
    peak = ctx.fp32_peak_tflops()
    fwd_avg_ms = fwd_ms / max(fwd_n, 1)
    flops_per_launch = algo_flops * split_steps / max(fwd_n, 1)
    achieved = flops_per_launch / (fwd_avg_ms * 1e-3) / 1e12 if fwd_n else None
    # DRAM traffic of the engine passes from one ncu capture of a 5,000-read
    # batch of this workload (38.1 + 3.85 + 2.69 + 0.62 + 0.10 MB over its
    # five passes), scaled by the reads (the traffic is per pair) and spread
    # over this step's forward launches
    launches_per_step = fwd_n / split_steps if fwd_n else 0.0
    traffic_ncu = (45.4e6 * R / 5000.0) / launches_per_step if launches_per_step else None
    ncu_src = ("ncu dram__bytes_read+write of the engine passes at 5,000 reads, scaled to this batch by reads, "
               "per forward launch")
    if live_bytes is not None and launches_per_step:
        traffic, traffic_src = live_bytes / launches_per_step, live_src + ", per forward launch"
    else:
        traffic, traffic_src = traffic_ncu, ncu_src + (f" ({live_src})" if live_src else "")
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if (achieved and peak) else None, "traffic": traffic,
                "traffic_source": traffic_src, "traffic_ncu": traffic_ncu, "traffic_ncu_source": ncu_src,
                "kernel": "wp_engine_kernel (passes 1-5) + wp_dense_kernel",
                "peak_source": "FP32 FMA loop measured live (wp_probe_fp32_peak); MEASURED_PEAKS.json has no FP32 figure",
                "algorithmic_flops_per_step": algo_flops,
                "unpruned_flops_per_step": float(R) * unpruned_forward_flops(ds.seqs, T, C),
                "forward_ms_per_step": fwd_ms / split_steps, "prep_ms_per_step": prep_ms / split_steps,
                "forward_launches_per_step": fwd_n / split_steps, "work": work}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded simulator)",
            "config": {"workload": WORKLOAD, "reads": R, "peptides": len(ds), "timesteps": T,
                       "channels": C, "dist_cutoff": CUTOFF, "pairs_per_step": pairs,
                       "l2": "flushed between steps (512 MB write)",
                       "engine_shapes": ({"fixed": list(tuned_cfg)} if args.engine_shape else
                                         {"default": list(tuned_cfg)} if args.no_autotune else
                                         {"autotuned": list(tuned_cfg), "sample_ms": tuned_ms}),
                       "cuda_graph": "launch sequence captured and replayed in the timed steps"},
            "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"], o_out = cpu_baseline(sm, ds, rads)
        line["parity_vs_oracle"] = sample_parity(last_gpu, o_out)
        line["parity_vs_oracle"]["log_p"] = loglik_parity(ctx, sm, ds, rads)
    ctx.close()
    if rank == 0 and not args.no_subrecords:
        line["hybrid_and_learned"] = hybrid_learned_subrecords(local, epochs=args.epochs)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
