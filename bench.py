#!/usr/bin/env python3
"""Benchmark of the ABC simulation hot path on GB300.

Workload (one step): the five-model ABC batch of 10^6 particles (2 x 10^5 per
model: constant, constant non-scaling, and k_on / alpha / gamma varying over
the 5 age groups) x 2,000 synthetic cells (1,200 pulse, 800 chase, Beta(4,16)
capture), the reference time grid (cycle 20 h, 5 age groups, 11 labelling
conditions), in one persistent FP32 SSA launch, then binomial capture and the
53 summary statistics per particle.  Metric: fired SSA events per second.
Each step is one call of the public host API (abc_simulate_batch: host theta
in, host statistics out) with a fresh random stream (seed).

  value       events / device time of the step's kernels (setup, work order,
              SSA, capture + statistics; CUDA events on the library's stream),
              inputs resident in HBM; the per-cell count buffer (16 GB, > L2)
              is rewritten every step, so no L2 flush is needed.
  e2e         the same steps' events / their wall time, host<->device copies
              of theta and statistics included.
  roofline    SSA kernel against the instruction-issue roofline (algorithmic
              ops per event x events / SSA kernel time vs 152 SMs x 128 lanes x
              max SM clock).
  cpu_baseline  the FP64 CPU SSA (oracle port, OpenMP over host cores) on a
              bounded sample of the same particles.

Sections after the headline (flags turn them off / on): the P x G distance
and top-q acceptance at 5 x 10^6 x 2,000 with an FP64-oracle equality check,
the moment ODE, and surrogate-screened vs plain ABC.

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
PER_MODEL_DEFAULT = 200_000  # 10^6 particles over the five models
# DRAM bytes per (particle, cell) trajectory of the production SSA kernel,
# measured with ncu (dram__bytes_read.sum + dram__bytes_write.sum, one pass) on
# the 5 x 4,000-particle x 2,000-cell launch, whose 320 MB count buffer exceeds
# L2: 326.0 MB read + 269.4 MB write over 4 x 10^7 trajectories (the initial
# (u, G) pair in, the final counts out: 16 B algorithmic, part of the writes
# still in L2 when the kernel ends)
SSA_DRAM_BYTES_PER_TRAJECTORY = (326002688 + 269423104) / 4.0e7


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--per-model", type=int, default=PER_MODEL_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-distance", action="store_true", help="skip the P x G distance section")
    ap.add_argument("--no-abc", action="store_true", help="skip the plain vs screened ABC section (few genes)")
    ap.add_argument("--abc-wide", action="store_true",
                    help="also run screened vs plain ABC at 8, 50 and 2,000 genes (top 1 %%)")
    ap.add_argument("--no-moment", action="store_true", help="skip the moment-ODE section")
    ap.add_argument("--config5", action="store_true",
                    help="also run screened ABC at full scale: 2 x 10^6 training draws, 5 x 10^6 plain draws, "
                         "5 x 10^7 screened draws per gene set (about 10 minutes)")
    ap.add_argument("--no-graph", action="store_true", help="skip the CUDA-graph check of the chain")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (variant 0, chunk 1)")
    ap.add_argument("--dist-particles", type=int, default=5_000_000)
    ap.add_argument("--genes", type=int, default=2000)
    ap.add_argument("--oracle-genes", type=int, default=64,
                    help="genes of the distance section whose accepted lists are checked against the FP64 oracle")
    ap.add_argument("--section", default="all", choices=["all", "distance", "moment", "abc", "config5"],
                    help="'distance' / 'moment' / 'abc' run only that section and print its object")
    return ap.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return pk, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def workload_name(per_model: int) -> str:
    return (f"five-model ABC batch: 5 x {per_model} particles x {N_CELLS} cells, reference time grid (h), "
            "factor prior, SSA + capture + 53 statistics")


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
    order = (np.arange(5)[None, :] * per_model + np.arange(per_model)[:, None]).ravel()
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


def distance_bench(P: int, G: int, K: int, q: float, seed: int, cpu_seconds: float, oracle_genes: int = 0):
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
        # the tensor-core candidate passes on the same selection (indices only):
        # one term (TF32 hi, gene rows resident in shared memory), three terms
        # with TF32 hi/lo splits, three terms with BF16 hi/lo splits
        per_mode = {}
        default_mode = ctx.distance_mode()[0]
        for dm_try in (1, 2, 3):
            ctx.set_distance_mode(dm_try)
            ctx.select_device(data, se, stats.data_ptr(), min(P, 200000), 1, q)  # warm-up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            o_m, i_m, _ = ctx.select_device(data, se, stats.data_ptr(), P, 1, q, errors=False)
            torch.cuda.synchronize()
            dt_m = time.perf_counter() - t0
            f_ms, f_pass = ctx.select_profile()
            c_m, r_m = ctx.select_counters()
            per_mode[dm_try] = {"seconds": dt_m, "pairs_per_s": P * G / dt_m, "candidate_pass_ms": f_ms / max(f_pass, 1),
                                "candidate_passes": f_pass, "candidates": c_m, "fp64_rechecked": r_m,
                                "algorithmic_tflops": 2.0 * P * G * 2 * K / (f_ms / max(f_pass, 1) / 1e3) / 1e12,
                                "_lists": (o_m, i_m)}
        same_lists = all(np.array_equal(per_mode[1]["_lists"][0], per_mode[m]["_lists"][0]) and
                         np.array_equal(per_mode[1]["_lists"][1], per_mode[m]["_lists"][1]) for m in (2, 3))
        for v in per_mode.values():
            del v["_lists"]
        ctx.set_distance_mode(default_mode)
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
        # the same selection keeping the FP64 error of every accepted pair
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        off_e, idx_e, err_e = ctx.select_device(data, se, stats.data_ptr(), P, 1, q, errors=True)
        torch.cuda.synchronize()
        dt_e = time.perf_counter() - t0
        # accepted lists of the first genes against the FP64 oracle (errors of
        # all P particles, compute_errors.jl:30-43, then accepted_particles.jl:20-29)
        oracle_chk = None
        if oracle_genes > 0:
            from oracle import oracle as orc
            orc.build()
            ng = min(oracle_genes, G)
            st_h = stats.cpu().numpy()
            t0 = time.perf_counter()
            e_orc = orc.errors(data[:ng], se[:ng], st_h, n_threads=os.cpu_count() or 1)
            o_off, o_idx = orc.accept(e_orc, 1, q)
            t_orc = time.perf_counter() - t0
            n_o = int(o_off[ng])
            gene = np.repeat(np.arange(ng), np.diff(o_off))
            same_i = bool(np.array_equal(off[:ng + 1], o_off) and np.array_equal(idx[:off[ng]], o_idx))
            same_e = bool(np.array_equal(off_e[:ng + 1], o_off) and np.array_equal(idx_e[:off_e[ng]], o_idx))
            same_err = bool(same_e and np.array_equal(err_e[:n_o], e_orc[o_idx - 1, gene]))
            oracle_chk = {"genes": ng, "particles": P, "accepted_pairs": n_o,
                          "identical_indices_only_path": same_i, "identical_fp64_error_path": same_e,
                          "fp64_errors_bit_identical": same_err, "oracle_seconds": t_orc,
                          "oracle_cores": os.cpu_count()}
            del st_h, e_orc
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
           "distance_mode": mode_used, "downstream": down,
           "fp64_error_path": {"seconds": dt_e, "pairs_per_s": P * G / dt_e, "accepted": int(off_e[-1])},
           "candidate_pass_modes": {"one_term_tf32_resident_genes": per_mode[1], "three_term_tf32": per_mode[2],
                                    "three_term_bf16_resident_genes": per_mode[3],
                                    "identical_accepted_lists": same_lists},
           "oracle_check": oracle_chk}
    kernel_ms = fast_ms / max(passes, 1)
    pk, src = load_peaks()
    algo = 2.0 * P * G * (2 * K)  # one multiply-add per (particle, gene, operand column) of [s | s^2]
    if mode_used in (1, 2, 3):
        # tcgen05 MMAs issued per pass: 128 x 256 tiles, 1 or 3 terms, each of depth 2K rounded up to
        # the K-step (8 TF32 values for modes 1-2, 16 BF16 values for mode 3; steps of zero padding are skipped)
        step = 16 if mode_used == 3 else 8
        ka = -(-2 * K // step) * step
        tiles = -(-P // 128) * -(-G // 256)
        terms = 1 if mode_used == 1 else 3
        issued = 2.0 * 128 * 256 * ka * terms * tiles
        mma_kind, rate = ("BF16", "which run at") if mode_used == 3 else ("TF32", "which run at half")
        peak = float(pk.get("bf16_tflops", 1900.0)) * 1e12
        out["roofline"] = {"bound": "tensor", "achieved": algo / (kernel_ms / 1e3) / 1e12, "peak": peak / 1e12,
                           "unit": "TFLOP/s", "frac": algo / (kernel_ms / 1e3) / peak, "traffic": None,
                           "basis": f"algorithmic flops 2 P G (2K) per candidate pass over its kernel time, against "
                                    f"the {src} dense BF16 GEMM rate; the pass issues {mma_kind} MMAs ({terms} term(s), "
                                    f"128 x 256 tiles, depth {ka}), {rate} that rate",
                           "kernel_ms_per_pass": kernel_ms,
                           "issued_mma_tflops": issued / (kernel_ms / 1e3) / 1e12}
    else:
        peak = SMS * 128 * 2 * 2070.0e6
        out["roofline"] = {"bound": "fp32", "achieved": algo / (kernel_ms / 1e3) / 1e12, "peak": peak / 1e12,
                           "unit": "TFLOP/s", "frac": algo / (kernel_ms / 1e3) / peak, "traffic": None,
                           "basis": "2 FMA per (p, g, k) in the candidate pass; peak = nominal FP32 (152 SMs x "
                                    "128 lanes x 2 flop x 2,070 MHz), no measured FP32 peak available",
                           "kernel_ms_per_pass": kernel_ms}
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
        "config": {"workload": workload_name(args.per_model), "particles_per_step": 5 * per_model,
                   "cells": N_CELLS},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Julia (not installed); this is the FP64 C restatement of its simulation, "
                "the exact SSA of the same reaction network",
    }
    print(json.dumps(line))


def screened_sections(args):
    """Surrogate-screened vs plain ABC (the learned pre-screen of prior draws)."""
    from abc_inference_transcription_gb300 import pipeline
    out = {}
    # a few genes at a small quantile: the regime where the screen can drop
    # most draws (top 0.2 % of 10^5 plain draws; four independent sets of 4
    # genes, one surrogate)
    out["abc_screened_small_q"] = pipeline.run(genes=(4, 4, 4, 4), per_model_train=40000, per_model_plain=20000,
                                               screen_factor=10, q=0.002, seed=2, epochs=40)
    if args.abc_wide:
        # accepted pairs per second, plain vs screened, top 1 % per gene, for 8,
        # 50 and the full gene set (the screen's gain falls with the number of
        # genes a draw must be far from)
        out["abc_screened"] = pipeline.run(genes=(8, 50, args.genes), per_model_train=20000, per_model_plain=2000,
                                           screen_factor=10, q=0.01, seed=1, epochs=40)
    return out


def config5_section():
    """Surrogate-screened vs plain ABC at the workload's full scale: the
    surrogate trained on 2 x 10^6 exact draws (held-out error and calibration
    on 10^5 of the plain draws), 5 x 10^6 plain draws, and 5 x 10^7 screened
    draws for each of two sets of 4 genes at top 0.2 %; for 2,000 genes only
    the plain run's bound on any screen's gain."""
    from abc_inference_transcription_gb300 import pipeline
    return pipeline.run(genes=(4, 4), per_model_train=400_000, per_model_plain=1_000_000, screen_factor=10,
                        q=0.002, seed=3, epochs=40, bound_genes=(2000,))


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
    if args.section != "all":
        if rank == 0:
            import __graft_entry__
            __graft_entry__.build()
            if args.section == "distance":
                print(json.dumps(distance_bench(args.dist_particles, args.genes, 72, 0.001, 5, args.cpu_seconds,
                                                args.oracle_genes)))
            elif args.section == "moment":
                print(json.dumps(moment_bench(40000, args.cpu_seconds)))
            elif args.section == "abc":
                print(json.dumps(screened_sections(args)))
            else:
                print(json.dumps(config5_section()))
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
    K = ctx.K
    # autotuner: (register variant x work chunk) on an evenly spaced sample of the batch
    tune = None
    if not args.no_tune:
        n_tune = min(P_rank, 2000)
        rows = np.linspace(0, P_rank - 1, n_tune).astype(np.int64)
        variant, chunk, tune_ms = ctx.autotune_batch(models[rows], theta[rows], seed=7)
        tune = {"chosen_variant": variant, "chosen_chunk": chunk, "variants": [0, 1], "chunks": [1, 4, 16],
                "ssa_ms": tune_ms, "sample": f"{n_tune} particles spaced evenly over the batch"}
    ctx.profile(True)

    def step(seed):
        """One call of the public host API: host theta in, host statistics out."""
        t0 = time.perf_counter()
        st = ctx.simulate_batch(models, theta, seed, offset=rank * P_rank)
        wall = time.perf_counter() - t0
        ev, rej = ctx.last_counters()
        return ev, rej, np.array(ctx.phase_ms()), wall, st

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
    wall = 0.0
    st_host = None
    for k in range(args.steps):
        ev, rej, ph, w_s, st_host = step(1000 + k)
        tot_ev += ev
        tot_rej += rej
        phase += ph
        wall += w_s
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    t_ms = e0.elapsed_time(e1)
    compute_s = phase.sum() / 1e3
    if dist:
        t = torch.tensor([t_ms, compute_s, wall], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms, compute_s, wall = (float(x) for x in t.tolist())
        e = torch.tensor([tot_ev], device="cuda", dtype=torch.float64)
        dist.all_reduce(e, op=dist.ReduceOp.SUM)
        tot_ev_all = float(e.item())
    else:
        tot_ev_all = float(tot_ev)
    value = tot_ev_all / compute_s
    e2e = {"value": tot_ev_all / wall, "unit": "events/s", "h2d_bytes_per_step": int(theta.nbytes + models.nbytes),
           "d2h_bytes_per_step": int(st_host.nbytes), "seconds": wall,
           "path": "abc_simulate_batch (C ABI) with host theta and host statistics, the timed steps themselves"}

    # the chain (setup -> work order -> SSA -> capture + statistics) as one CUDA
    # graph, against plain launches, on a sub-batch of the same particles
    graph = None
    if not args.no_graph:
        sub = np.linspace(0, P_rank - 1, min(P_rank, 20000)).astype(np.int64)
        ctx.profile(False)
        res = {}
        for mode in (False, True):
            ctx.set_graph(mode)
            ctx.simulate_batch(models[sub], theta[sub], 700, offset=rank * P_rank)
            t0 = time.perf_counter()
            res[mode] = ctx.simulate_batch(models[sub], theta[sub], 701, offset=rank * P_rank)
            res[(mode, "s")] = time.perf_counter() - t0
        gi, gu = ctx.graph_counters()
        ctx.set_graph(False)
        ctx.profile(True)
        graph = {"particles": int(sub.shape[0]), "graph_seconds": res[(True, "s")],
                 "plain_seconds": res[(False, "s")], "identical_statistics": bool(
                     np.array_equal(res[True], res[False], equal_nan=True)),
                 "instantiations": gi, "in_place_updates": gu}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, peak_src = load_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    ssa_s = phase[1] / 1e3
    achieved_ev = tot_ev / ssa_s
    peak_ev = SMS * LANES_PER_SM * sm_max * 1e6 / OPS_PER_EVENT
    trajectories = P_rank * N_CELLS
    traffic = None if SSA_DRAM_BYTES_PER_TRAJECTORY is None else SSA_DRAM_BYTES_PER_TRAJECTORY * trajectories
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
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded prior draws, synthetic cells)",
        "config": {"workload": workload_name(args.per_model),
                   "particles_per_step": P_rank * world, "cells": N_CELLS, "parallelism": f"particle shards x{world}",
                   "l2": "per-cell count buffer (P x C x 8 B = 16 GB at 10^6 particles) exceeds L2 and is "
                         "rewritten every step"},
        "events_per_step": tot_ev_all / args.steps, "thinning_rejections": tot_rej,
        "particles_per_s": P_rank * world * args.steps / compute_s,
        "phase_ms_per_step": {"setup_work_order_initial_states": phase[0] / args.steps, "ssa": phase[1] / args.steps,
                              "capture_stats": phase[2] / args.steps},
        "roofline": {"bound": "issue", "achieved": achieved_ev / 1e9, "peak": peak_ev / 1e9, "unit": "Gevents/s",
                     "frac": achieved_ev / peak_ev, "traffic": traffic,
                     "basis": f"{OPS_PER_EVENT} algorithmic ops/event, {SMS} SMs x {LANES_PER_SM} lanes x "
                              f"{sm_max:.0f} MHz ({peak_src} sm_max); traffic = DRAM bytes per launch, "
                              "per-trajectory figure from ncu x trajectories"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": 6 * args.steps,  # per step: setup, 2 work-order kernels, initial states, SSA, capture+statistics
        "autotune": tune,
        "cuda_graph": graph,
        "clocks": clocks,
    }
    if not args.no_distance:
        try:
            line["distance"] = distance_bench(args.dist_particles, args.genes, 72, 0.001, 5, args.cpu_seconds,
                                              args.oracle_genes)
        except Exception as exc:
            line["distance"] = {"error": repr(exc)}
    if not args.no_moment:
        try:
            line["moment_ode"] = moment_bench(40000, args.cpu_seconds)
        except Exception as exc:
            line["moment_ode"] = {"error": repr(exc)}
    if not args.no_abc:
        try:
            line.update(screened_sections(args))
        except Exception as exc:
            line["abc_screened_small_q"] = {"error": repr(exc)}
    if args.config5:
        try:
            line["config5"] = config5_section()
        except Exception as exc:
            line["config5"] = {"error": repr(exc)}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
