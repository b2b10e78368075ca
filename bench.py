#!/usr/bin/env python3
"""Benchmark of the ABC simulation hot path on GB300.

Workload (one step): the five-model ABC batch -- all 5 gene models mixed in
one persistent FP32 SSA launch (FP64 clock), PER_MODEL particles per model x
2,000 synthetic cells (1,200 pulse, 800 chase, Beta(4,16) capture), the
reference time grid (cycle 20 h, 5 age groups, 11 labelling conditions),
followed by binomial capture and the 53 summary statistics per particle.
Metric: fired SSA events per second.  A fresh random stream (seed) per step.

  value       device-timed (CUDA events on the library's stream), inputs
              resident in HBM; the per-cell count buffer (> 129 MB L2) is
              rewritten every step, so no L2 flush is needed.
  e2e         the same step through the public host API (abc_simulate_batch
              with host theta / host statistics, copies inside the timed region).
  roofline    SSA kernel against the instruction-issue roofline (algorithmic
              ops per event x events / SSA kernel time vs 152 SMs x 128 lanes x
              max SM clock); capture+statistics kernel against HBM bandwidth.
  cpu_baseline  the FP64 CPU SSA (oracle port, OpenMP over host cores) on a
              bounded sample of the same particles.

--impl reference: the CPU implementation alone (rank 0), same metric/config.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS = 2000
# algorithmic operations per fired event: half a Philox4x32-10 block (10 rounds x
# 6 integer operations / 2), two uniforms, one log, one divide, ~9 propensity and
# channel-selection operations, the clock add and compare, the state update
OPS_PER_EVENT = 60
LANES_PER_SM = 128
SMS = 152
PER_MODEL_DEFAULT = 4000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--per-model", type=int, default=PER_MODEL_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-distance", action="store_true", help="skip the P x G distance section")
    ap.add_argument("--no-abc", action="store_true", help="skip the plain vs screened ABC section")
    ap.add_argument("--no-moment", action="store_true", help="skip the moment-ODE section")
    ap.add_argument("--no-graph", action="store_true", help="skip the CUDA-graph timing of the step")
    ap.add_argument("--dist-particles", type=int, default=5_000_000)
    ap.add_argument("--genes", type=int, default=2000)
    ap.add_argument("--section", default="all", choices=["all", "distance", "moment"],
                    help="'distance' / 'moment' run only that section and print its object")
    return ap.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return pk, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def workload(per_model: int, seed0: int, offset: int):
    """theta of the five-model batch (prior draws on the GPU), padded to 9 columns."""
    import numpy as np
    from abc_inference_transcription_gb300 import FP32, factor_prior, make_config, synthetic_cells
    from abc_inference_transcription_gb300.host import Context
    cfg = make_config("hour", precision=FP32)
    cells = synthetic_cells(seed=1)
    ctx = Context(cfg, cells)
    pr = factor_prior()
    thetas, models = [], []
    for m in range(1, 6):
        th = ctx.sample_prior(m, per_model, seed0 + m, pr, offset=offset + (m - 1) * per_model)
        pad = np.zeros((per_model, 9))
        pad[:, :th.shape[1]] = th
        thetas.append(pad)
        models.append(np.full(per_model, m, np.int32))
    return cfg, cells, ctx, np.vstack(thetas), np.concatenate(models)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_ssa_rate(cfg, cells, theta, models, seconds: float, threads: int):
    """FP64 CPU SSA (the oracle port) on a growing sample of the same particles,
    interleaved over the five models, until one run takes >= seconds/3."""
    import numpy as np
    from abc_inference_transcription_gb300 import FP64
    from oracle import oracle as orc
    orc.build()
    import copy
    cfg64 = copy.copy(cfg)
    cfg64.precision = FP64
    P = theta.shape[0]
    per_model = P // 5
    order = np.concatenate([[m * per_model + i for m in range(5)] for i in range(per_model)])
    # increments of 10 particles (2 per model) until the time budget is spent
    n, ev, dt = 0, 0, 0.0
    while n < P and dt < seconds:
        sel = order[n:n + 10]
        t0 = time.perf_counter()
        for m in range(1, 6):
            rows = sel[models[sel] == m]
            if rows.size == 0:
                continue
            npar = 5 if m <= 2 else 9
            out = orc.simulate(cfg64, cells, m, theta[rows, :npar], seed=77, n_threads=threads, want_cells=True)
            ev += int(out["events"].sum())
        dt += time.perf_counter() - t0
        n += sel.shape[0]
    return ev / dt, n, dt, ev


def distance_bench(P: int, G: int, K: int, q: float, seed: int, cpu_seconds: float):
    """Rejection error matrix + top-q acceptance at P x K x G with FP32
    candidate passes and FP64 rechecks; statistics stand-ins are log-normal
    perturbations of 256 base vectors (a K = 72 width has no reference
    derivation), genes are base vectors plus 5 % noise, se log-normal
    (sigma 0.5) around 10 % of the statistic."""
    import numpy as np
    import torch
    from abc_inference_transcription_gb300 import make_config
    from abc_inference_transcription_gb300.host import Context
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    NB = 256
    base = torch.exp(torch.randn((NB, K), device="cuda", dtype=torch.float64, generator=g) * 1.5)
    pick = torch.randint(0, NB, (P,), device="cuda", generator=g)
    stats = (base[pick] * torch.exp(0.25 * torch.randn((P, K), device="cuda", dtype=torch.float64,
                                                        generator=g))).contiguous()
    rng = np.random.default_rng(seed)
    b = base.cpu().numpy()
    data = b[rng.integers(0, NB, G)] * (1.0 + 0.05 * rng.normal(size=(G, K)))
    se = 0.1 * np.abs(data) * rng.lognormal(0.0, 0.5, (G, K))
    k = int(np.ceil(q * P))
    ctx = Context(make_config("hour"), None)
    try:
        ctx.profile(True)
        ctx.select_device(data, se, stats.data_ptr(), min(P, 200000), 1, q)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # the accepted index lists come back to the host (as the reference's
        # acceptance writes them); the FP64 errors stay on the device
        off, idx, _ = ctx.select_device(data, se, stats.data_ptr(), P, 1, q, errors=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        fast_ms, passes = ctx.select_profile()
        cands, rechecked = ctx.select_counters()
        mode_used = ctx.distance_mode()[1]
        # downstream of the acceptance: posterior summaries of the 10^7 accepted
        # pairs (theta on the device) and model probabilities for the genes
        theta = torch.randn((P, 9), device="cuda", dtype=torch.float64, generator=g)
        ctx.posterior_summary(theta.data_ptr(), npar=9, on_device=True, ld=9)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.posterior_summary(theta.data_ptr(), npar=9, on_device=True, ld=9)
        t_post = time.perf_counter() - t0
        mp_counts = np.stack([np.diff(off), np.random.default_rng(seed).integers(0, 3 * k, G)], 1)
        ctx.model_probs(mp_counts)
        t0 = time.perf_counter()
        ctx.model_probs(mp_counts)
        t_mp = time.perf_counter() - t0
        # data side: statistics + 100 bootstrap SEs of G genes' observed counts
        from abc_inference_transcription_gb300 import synthetic_cells
        cells_d = synthetic_cells(seed=1)
        rng_d = np.random.default_rng(seed)
        lam = rng_d.gamma(2.0, 3.0, (G, 1)) * cells_d.beta[None, :] * 5
        u_d = rng_d.poisson(lam, (G, cells_d.cond.shape[0])).astype(np.int32)
        l_d = rng_d.poisson(0.4 * lam, (G, cells_d.cond.shape[0])).astype(np.int32)
        with Context(make_config("hour"), cells_d) as dctx:
            dctx.data_stats(u_d[:8], l_d[:8], n_boot=100)
            t0 = time.perf_counter()
            dctx.data_stats(u_d, l_d, n_boot=100)
            t_ds = time.perf_counter() - t0
        down = {"posterior_summary_s": t_post, "model_probs_s": t_mp, "data_stats_s": t_ds,
                "workload": f"posterior MAP/mean/95 % bounds of 9 parameters over {int(off[-1])} accepted pairs "
                            f"in {G} genes; model probabilities of {G} genes x 2 groups, 100 bootstraps; data "
                            f"statistics + 100-resample SEs of {G} genes x 2,000 cells"}
        if cpu_seconds > 0:
            from oracle import oracle as orc
            orc.build()
            gs = min(G, 100)
            th_h = theta.cpu().numpy()
            t0 = time.perf_counter()
            orc.posterior_summary(th_h, off[:gs + 1], idx[:off[gs]], 0.95)
            down["cpu_posterior_summary_s_scaled"] = (time.perf_counter() - t0) * G / gs
            t0 = time.perf_counter()
            orc.model_probs(mp_counts)
            down["cpu_model_probs_s"] = time.perf_counter() - t0
            t0 = time.perf_counter()
            orc.data_stats(make_config("hour"), cells_d, u_d[:20], l_d[:20], n_boot=100)
            down["cpu_data_stats_s_scaled"] = (time.perf_counter() - t0) * G / 20
            down["cpu_sample"] = (f"posterior summary of the first {gs} genes and data statistics of the first 20 "
                                  f"genes, scaled to {G}, one core (oracle)")
            del th_h
        del theta
    finally:
        ctx.close()
        sh_keep = stats[:64].cpu().numpy()
        del stats, base, pick
        torch.cuda.empty_cache()
    out = {"workload": f"P={P} particles x K={K} statistics x G={G} genes, top {q:g} per gene",
           "pairs_per_s": P * G / dt, "seconds": dt, "accepted": int(off[-1]), "accepted_expected": k * G,
           "candidates": cands, "fp64_rechecked": rechecked, "candidate_passes": passes,
           "distance_mode": mode_used, "downstream": down}
    if mode_used in (1, 2):
        # tcgen05 TF32 MMAs issued per pass: 128 x 256 tiles, depth KA per term, 1 or 3 terms
        ka = -(-2 * K // 32) * 32
        tiles = -(-P // 128) * -(-G // 256)
        terms = 3 if mode_used == 2 else 1
        flops = 2.0 * 128 * 256 * ka * terms * tiles * passes
        pk, src = load_peaks()
        peak = float(pk.get("bf16_tflops", 1900.0)) / 2.0 * 1e12
        out["roofline"] = {"bound": "tensor", "achieved": flops / (fast_ms / 1e3) / 1e12, "peak": peak / 1e12,
                           "unit": "TFLOP/s", "frac": flops / (fast_ms / 1e3) / peak, "traffic": None,
                           "basis": f"TF32 MMA flops issued ({terms} term(s), 128 x 256 tiles, depth {ka}); "
                                    f"peak = half the {src} dense BF16 GEMM rate (TF32 runs at half the BF16 rate)",
                           "kernel_ms_per_pass": fast_ms / max(passes, 1),
                           "useful_fp32_tflops": 4.0 * P * G * K * passes / (fast_ms / 1e3) / 1e12}
    else:
        flops = 4.0 * P * G * K * passes
        peak = SMS * 128 * 2 * 2070.0e6
        out["roofline"] = {"bound": "fp32", "achieved": flops / (fast_ms / 1e3) / 1e12, "peak": peak / 1e12,
                           "unit": "TFLOP/s", "frac": flops / (fast_ms / 1e3) / peak, "traffic": None,
                           "basis": "2 FMA per (p, g, k) in the candidate pass; peak = nominal FP32 (152 SMs x "
                                    "128 lanes x 2 flop x 2,070 MHz), no measured FP32 peak available",
                           "kernel_ms_per_pass": fast_ms / max(passes, 1)}
    if cpu_seconds > 0:
        try:
            from oracle import oracle as orc
            orc.build()
            n = 64
            sh = sh_keep
            t0 = time.perf_counter()
            orc.errors(data, se, sh, None, n_threads=os.cpu_count() or 1)
            dtc = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": n * G / dtc, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
                                   "sample": f"{n} particles x {G} genes x K={K}, FP64 oracle errors"}
        except Exception as exc:
            out["cpu_baseline"] = {"value": None, "sample": repr(exc)}
    return out


def moment_bench(P: int, cpu_seconds: float):
    """The reference's deterministic simulation (moment ODE, all 53 statistics)
    for P particles of the five models (factor prior, reference time grid):
    FP32 production mode (substep cycle / 80) and the oracle-exact FP64 mode,
    beside the FP64 C oracle on all host cores at both grids."""
    import numpy as np
    from abc_inference_transcription_gb300 import FP32, FP64, factor_prior, make_config, synthetic_cells
    from abc_inference_transcription_gb300.config import beta_moments
    from abc_inference_transcription_gb300.host import Context
    cells = synthetic_cells(seed=1)
    bm = beta_moments(cells, 5)
    iv = np.zeros(9)
    iv[1] = 0.5
    out = {"workload": f"moment ODE statistics of {P} particles per model x 5 models, reference time grid (h), "
                       "factor prior, 2,000-cell capture moments", "unit": "particles/s"}
    thetas = {}
    for prec, name, n in ((FP32, "fp32_production", P), (FP64, "fp64_exact", max(P // 50, 200))):
        with Context(make_config("hour", precision=prec), cells) as ctx:
            tot, dt = 0, 0.0
            for m in range(1, 6):
                th = ctx.sample_prior(m, n, 100 + m, factor_prior())
                thetas[m] = th
                ctx.moment_simulate(m, th[:64], iv, bm, cells.age_dist)   # warm-up
                t0 = time.perf_counter()
                ctx.moment_simulate(m, th, iv, bm, cells.age_dist)
                dt += time.perf_counter() - t0
                tot += n
            out[name] = {"value": tot / dt, "particles": tot, "seconds": dt}
    if cpu_seconds > 0:
        from oracle import oracle as orc
        orc.build()
        cfg = make_config("hour", precision=FP64)
        for h_max, name in ((20.0 / 400, "cpu_h_cycle_over_400"), (20.0 / 80, "cpu_h_cycle_over_80")):
            n = 64
            t0 = time.perf_counter()
            for m in range(1, 6):
                orc.moment_batch(cfg, m, thetas[m][:n], iv, bm, cells.age_dist, n_threads=os.cpu_count() or 1,
                                 h_max=h_max)
            out[name] = {"value": 5 * n / (time.perf_counter() - t0), "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{n} particles per model, FP64 oracle"}
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from abc_inference_transcription_gb300 import FP64, factor_prior, make_config, synthetic_cells
    from oracle import oracle as orc
    orc.build()
    cfg = make_config("hour", precision=FP64)
    cells = synthetic_cells(seed=1)
    per_model = args.per_model
    thetas, models = [], []
    for m in range(1, 6):
        th = orc.sample_prior(cfg, m, per_model, 11 + m, factor_prior(), offset=(m - 1) * per_model)
        pad = np.zeros((per_model, 9))
        pad[:, :th.shape[1]] = th
        thetas.append(pad)
        models.append(np.full(per_model, m, np.int32))
    theta, mods = np.vstack(thetas), np.concatenate(models)
    threads = os.cpu_count() or 1
    rates = []
    n_sample = None
    for k in range(args.warmup + args.steps):
        budget = max(2.0, min(args.cpu_seconds, 150.0 / max(1, args.warmup + args.steps)))
        rate, n, dt, ev = cpu_ssa_rate(cfg, cells, theta, mods, budget, threads)
        n_sample = n
        if k >= args.warmup:
            rates.append(rate)
    value = statistics.median(rates)
    sample = f"first {n_sample} particles of the five-model batch (interleaved models) x {N_CELLS} cells per step"
    line = {
        "impl": "reference", "metric": "SSA events/s", "value": value, "unit": "events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded prior draws, synthetic cells)",
        "config": {"workload": f"five-model SSA batch, {args.per_model} particles/model x {N_CELLS} cells, "
                               "reference time grid (h)", "cells": N_CELLS},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Julia (not installed); this is the FP64 C restatement of its simulation, "
                "the exact SSA of the same reaction network",
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.section in ("distance", "moment"):
        if rank == 0:
            import __graft_entry__
            __graft_entry__.build()
            if args.section == "distance":
                print(json.dumps(distance_bench(args.dist_particles, args.genes, 72, 0.001, 5, args.cpu_seconds)))
            else:
                print(json.dumps(moment_bench(40000, args.cpu_seconds)))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if rank == 0:
        import __graft_entry__
        __graft_entry__.build()
    if dist:
        dist.barrier()

    P_rank = 5 * args.per_model
    cfg, cells, ctx, theta, models = workload(args.per_model, 11, rank * P_rank)
    ld = theta.shape[1]
    K = ctx.K
    d_theta = torch.from_numpy(theta).cuda()
    d_models = torch.from_numpy(models).cuda()
    d_stats = torch.empty((P_rank, K), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    # autotuner: kernel variant timed on a sample of the batch (model 1 rows)
    n_tune = min(args.per_model, 2000)
    variant, tune_ms = ctx.autotune(1, theta[:n_tune, :5], seed=7)
    ctx.profile(True)

    def step(seed):
        ctx.simulate_batch_device(d_models.data_ptr(), d_theta.data_ptr(), ld, P_rank, seed, d_stats.data_ptr(),
                                  offset=rank * P_rank)
        ctx.synchronize()
        ev, rej = ctx.last_counters()
        return ev, rej, ctx.phase_ms()

    for w in range(args.warmup):
        step(500 + w)
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    tot_ev = tot_rej = 0
    phase = np.zeros(3)
    for k in range(args.steps):
        ev, rej, ph = step(1000 + k)
        tot_ev += ev
        tot_rej += rej
        phase += np.array(ph)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    t_ms = e0.elapsed_time(e1)
    if dist:
        t = torch.tensor([t_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
        e = torch.tensor([tot_ev], device="cuda", dtype=torch.float64)
        dist.all_reduce(e, op=dist.ReduceOp.SUM)
        tot_ev_all = float(e.item())
    else:
        tot_ev_all = float(tot_ev)
    value = tot_ev_all / (t_ms / 1e3)

    # the same steps with the chain (setup -> work order -> SSA -> capture +
    # statistics) as one CUDA graph, updated in place per seed
    graph = None
    if not args.no_graph:
        ctx.profile(False)
        ctx.set_graph(True)
        step(700)
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        g0.record(stream)
        ng = min(args.steps, 3)
        for k in range(ng):
            step(1000 + k)
        g1.record(stream)
        torch.cuda.synchronize()
        gi, gu = ctx.graph_counters()
        graph = {"ms_per_step": g0.elapsed_time(g1) / ng, "plain_ms_per_step": t_ms / args.steps,
                 "instantiations": gi, "in_place_updates": gu, "steps": ng}
        ctx.set_graph(False)
        ctx.profile(True)

    # e2e through the host API
    e2e = None
    if not args.no_e2e:
        st_host = np.zeros((P_rank, K))
        ctx.simulate_batch(models, theta, 900, offset=rank * P_rank)  # warm host path
        t0 = time.perf_counter()
        ev_e2e = 0
        for k in range(args.steps):
            st_host = ctx.simulate_batch(models, theta, 1000 + k, offset=rank * P_rank)
            ev_e2e += ctx.last_counters()[0]
        dt = time.perf_counter() - t0
        if dist:
            t = torch.tensor([dt], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
            e = torch.tensor([ev_e2e], device="cuda", dtype=torch.float64)
            dist.all_reduce(e, op=dist.ReduceOp.SUM)
            ev_e2e = float(e.item())
        e2e = {"value": ev_e2e / dt, "unit": "events/s", "h2d_bytes_per_step": int(theta.nbytes + models.nbytes),
               "d2h_bytes_per_step": int(st_host.nbytes)}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, peak_src = load_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    ssa_s = phase[1] / 1e3
    achieved_ev = tot_ev / ssa_s
    peak_ev = SMS * LANES_PER_SM * sm_max * 1e6 / OPS_PER_EVENT
    stats_bytes = args.steps * (P_rank * N_CELLS * 8 + P_rank * K * 8)
    stats_gbs = stats_bytes / (phase[2] / 1e3) / 1e9
    cpu = None
    try:
        if args.cpu_seconds <= 0:
            raise RuntimeError("CPU baseline skipped (--cpu-seconds 0)")
        rate, n, dt, ev = cpu_ssa_rate(cfg, cells, theta, models, args.cpu_seconds, os.cpu_count() or 1)
        cpu = {"value": rate, "unit": "events/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"first {n} particles of the same batch (interleaved models) x {N_CELLS} cells, "
                         f"{ev} events in {dt:.1f} s, FP64 oracle SSA"}
    except Exception as exc:  # the oracle is a reported baseline only
        cpu = {"value": None, "unit": "events/s", "cores": os.cpu_count(), "kind": "port", "sample": repr(exc)}
    line = {
        "metric": "SSA events/s", "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 clock)", "data": "synthetic (seeded prior draws, synthetic cells)",
        "config": {"workload": f"five-model SSA batch: 5 x {args.per_model} particles x {N_CELLS} cells, "
                               "reference time grid (h), factor prior, capture + 53 statistics",
                   "particles_per_step": P_rank * world, "cells": N_CELLS, "parallelism": f"particle shards x{world}",
                   "l2": "per-cell count buffer (P x C x 8 B) exceeds L2 and is rewritten every step"},
        "events_per_step": tot_ev_all / args.steps, "thinning_rejections": tot_rej,
        "particles_per_s": P_rank * world * args.steps / (t_ms / 1e3),
        "phase_ms_per_step": {"setup": phase[0] / args.steps, "ssa": phase[1] / args.steps,
                              "capture_stats": phase[2] / args.steps},
        "roofline": {"bound": "issue", "achieved": achieved_ev / 1e9, "peak": peak_ev / 1e9, "unit": "Gevents/s",
                     "frac": achieved_ev / peak_ev, "traffic": None,
                     "basis": f"{OPS_PER_EVENT} algorithmic ops/event, {SMS} SMs x {LANES_PER_SM} lanes x "
                              f"{sm_max:.0f} MHz ({peak_src} sm_max)"},
        "roofline_stats": {"bound": "hbm", "achieved": stats_gbs, "peak": float(peaks.get("hbm_gbs", 6800.0)),
                           "unit": "GB/s", "frac": stats_gbs / float(peaks.get("hbm_gbs", 6800.0)),
                           "traffic": None, "peak_source": peak_src},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": 5 * args.steps,  # setup, 2 work-order kernels, SSA, capture+statistics
        "autotune": {"chosen_variant": variant, "ssa_ms_per_variant": tune_ms, "sample": f"{n_tune} particles"},
        "cuda_graph": graph,
        "clocks": clocks,
    }
    if not args.no_distance:
        try:
            line["distance"] = distance_bench(args.dist_particles, args.genes, 72, 0.001, 5, args.cpu_seconds)
        except Exception as exc:
            line["distance"] = {"error": repr(exc)}
    if not args.no_moment:
        try:
            line["moment_ode"] = moment_bench(40000, args.cpu_seconds)
        except Exception as exc:
            line["moment_ode"] = {"error": repr(exc)}
    if not args.no_abc:
        try:
            from abc_inference_transcription_gb300 import pipeline
            # accepted pairs per second, plain vs surrogate-screened, top 1 % per gene,
            # for 8, 50 and the full gene set (the screen's gain falls with the
            # number of genes a draw must be far from)
            line["abc_screened"] = pipeline.run(genes=(8, 50, args.genes), per_model_train=20000,
                                                per_model_plain=2000, screen_factor=10, q=0.01, seed=1, epochs=40)
            # a few genes at a small quantile: the regime where the screen can
            # drop most draws (top 0.2 % of 10^5 plain draws; four independent
            # sets of 4 genes, one surrogate)
            line["abc_screened_small_q"] = pipeline.run(genes=(4, 4, 4, 4), per_model_train=40000,
                                                        per_model_plain=20000, screen_factor=10, q=0.002, seed=2,
                                                        epochs=40)
        except Exception as exc:
            line["abc_screened"] = {"error": repr(exc)}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
