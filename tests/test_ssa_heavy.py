"""SSA parity in the heavy regime and the FP32 production statistics at the
3-Monte-Carlo-standard-error bar.  Every call goes through the C ABI.

FP64 oracle mode, bit for bit against the FP64 CPU oracle: unclamped draws
from the reference prior (scripts/abc_simulation.jl:3-11: k_on, k_off, alpha
up to 10^3 per hour) for all five models on the full 2,000-cell table, with
one particle per model built at alpha >= 10^2.5 / h and gamma <= 10^-2 / h
(slow decay, counts accumulate over the cycles), and a per-minute
configuration whose counts reach several 10^5 (binomial capture then runs
BTRD at n p ~ 10^5).  Counts, captured counts, event counts, event-sequence
hashes and the 53 statistics must be identical.

FP32 production mode against the reference's own model, the moment ODE
(scripts/model.jl:67-239) started at its periodic solution: R replicate particles of one theta (distinct
random streams) on a table with N cells in every (condition, age) group and
one capture efficiency.  Per statistic of scripts/abc_simulation.jl:23-46,
the replicate mean must lie within 3 Monte Carlo standard errors of the
moment-ODE statistic, and per group the pooled mean, variance and covariance
of the captured counts within 3 standard errors of their exact values.  With
several hundred comparisons per theta a few |z| > 3 are expected by chance
(0.27 % each): the test allows the count that independent comparisons exceed
with probability 10^-3 (5 of 328) and none beyond 4.5; the seeds are fixed,
so the outcome is reproducible.
"""
import json
import math
import os

import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.config import (CellTable, age_distribution, make_config, reference_prior,
                                                       synthetic_cells)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Ctx(built):
    from abc_inference_transcription_gb300.host import Context
    return Context


def heavy_theta(model: int) -> np.ndarray:
    """log10 rates per hour: k_on, k_off moderate, alpha = 10^2.7, gamma = 10^-2.2,
    with the varying rate of models 3-5 spread over the age steps."""
    kon, koff, alpha, gamma, lam = [-0.2], [-0.3], [2.7], [-2.2], [-0.1]
    if model == 3:
        kon = [-0.6, -0.3, 0.0, 0.2, -0.1]
    if model == 4:
        alpha = [2.5, 2.6, 2.9, 2.7, 2.8]
    if model == 5:
        gamma = [-2.4, -2.1, -2.6, -2.2, -2.0]
    return np.array(kon + koff + alpha + gamma + lam, np.float64)[None, :]


def _compare_bitwise(got, ref):
    for key in ("counts", "captured", "events", "hash"):
        assert np.array_equal(got[key], ref[key]), key
    assert np.array_equal(got["stats"], ref["stats"], equal_nan=True)


@pytest.mark.parametrize("model", [1, 2, 3, 4, 5])
def test_ssa_fp64_bit_exact_heavy_reference_prior(Ctx, orc, model):
    cfg = make_config("hour", precision=abi.FP64)
    cells = synthetic_cells(seed=10 + model)  # the 2,000-cell table
    theta = orc.sample_prior(cfg, model, 3, 200 + model, reference_prior())
    theta = np.vstack([theta, heavy_theta(model)])
    with Ctx(cfg, cells) as ctx:
        got = ctx.simulate_cells(model, theta, seed=17)
        ev, rej = ctx.last_counters()
    ref = orc.simulate(cfg, cells, model, theta, seed=17)
    assert ref["status"] == 0
    info = (f"model {model}: max events per trajectory {int(ref['events'].max())}, total events "
            f"{int(ref['events'].sum())}, max count {int(ref['counts'].max())}, "
            f"max captured {int(ref['captured'].max())}")
    _compare_bitwise(got, ref)
    assert ev == int(ref["events"].sum()) and rej == ref["rejections"], info
    # the regime the test is for: long trajectories and large counts
    assert ref["events"].max() > 10_000 and ref["counts"].max() > 5_000, info


def test_ssa_fp64_bit_exact_counts_near_a_million(Ctx, orc):
    """Per-minute rates near the top of the benchmark prior: alpha = 10^2.8 / min,
    gamma = 10^-3 / min (counts of several 10^5 at the observation, ~4 x 10^6
    events per trajectory); two cells per (condition, age) group."""
    cfg = make_config("min", precision=abi.FP64)
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=5)
    th = np.array([[-0.5, -1.0, 2.8, -3.0, -0.1]])
    with Ctx(cfg, cells) as ctx:
        got = ctx.simulate_cells(1, th, seed=23)
    ref = orc.simulate(cfg, cells, 1, th, seed=23)
    assert ref["status"] == 0
    info = f"max count {int(ref['counts'].max())}, max events {int(ref['events'].max())}"
    _compare_bitwise(got, ref)
    assert ref["counts"].max() > 300_000 and ref["captured"].max() > 30_000, info


# --------------------------------------------------------------------------
# FP32 production mode: statistics within 3 Monte Carlo standard errors
# --------------------------------------------------------------------------
def group_cells(n_per_group: int, beta: float, A: int = 5, J: int = 11) -> CellTable:
    cond = np.repeat(np.arange(J, dtype=np.int32), A * n_per_group)
    age = np.tile(np.repeat(np.arange(A, dtype=np.int32), n_per_group), J)
    return CellTable(cond=cond, age=age, beta=np.full(cond.shape[0], beta),
                     age_dist=age_distribution(cond, age, A, J))


def captured_moments(raw: np.ndarray, b: float) -> np.ndarray:
    """Exact moments of per-cell Bin(n, b) captures of (u, l) with raw moments
    [E u, E l, Var u, Cov ul, Var l] (one capture efficiency for every cell)."""
    m = np.empty_like(raw)
    mu, ml, vu, cv, vl = (raw[..., i] for i in range(5))
    m[..., 0] = b * mu
    m[..., 1] = b * ml
    m[..., 2] = b * (1 - b) * mu + b * b * vu
    m[..., 3] = b * b * cv
    m[..., 4] = b * (1 - b) * ml + b * b * vl
    return m


def family_deviation(mean: np.ndarray, ode: np.ndarray) -> dict:
    """Largest relative deviation |mean - ode| / |ode| per statistic family."""
    names = ["pulse_mean", "pulse_ff", "chase_mean", "chase_ff", "ratio", "mean_corr", "corr_mean"]
    sizes = [5, 5, 5, 5, 11, 11, 11]
    out, k = {}, 0
    for nm, n in zip(names, sizes):
        d = np.abs(mean[k:k + n] - ode[k:k + n]) / np.maximum(np.abs(ode[k:k + n]), 1e-12)
        out[nm] = float(np.nanmax(d))
        k += n
    return out


def family_z(z: np.ndarray) -> dict:
    """Largest |z| (replicate mean vs moment ODE, in Monte Carlo standard errors) per statistic family."""
    names = ["pulse_mean", "pulse_ff", "chase_mean", "chase_ff", "ratio", "mean_corr", "corr_mean"]
    sizes = [5, 5, 5, 5, 11, 11, 11]
    out, k = {}, 0
    for nm, n in zip(names, sizes):
        out[nm] = float(np.nanmax(np.abs(z[k:k + n])))
        k += n
    return out


def allowed_beyond_3(n: int, alpha: float = 1e-3) -> int:
    """Smallest k with P(X > k) < alpha for X ~ Bin(n, 0.0027), the number of
    |z| > 3 among n independent standard normal z under exact agreement."""
    p, k, cdf = 0.0026997960632601866, 0, 0.0
    while True:
        cdf += math.comb(n, k) * p ** k * (1.0 - p) ** (n - k)
        if 1.0 - cdf < alpha:
            return k
        k += 1


def periodic_iv(orc, cfg, model: int, th: np.ndarray) -> np.ndarray:
    """Start of the moment ODE at its periodic solution, in the order of
    model.jl:74-86 (E G, E u, E l, Var G, Cov(G,u), Cov(G,l), Var u, Cov(u,l),
    Var l), from the fixed point the SSA also starts from.  The reference's
    transient_phase (model.jl:114-142) approaches the same point but stops at
    a 1 % change per cycle, which for slow decay (gamma = 10^-2 / h) leaves its
    means 3-5 x 10^-4 below it: about one Monte Carlo standard error at 1,024
    replicates, a bias of the stopping rule, not of the simulation."""
    S = cfg.n_steps
    rec = orc.setup(cfg, model, th)
    g0, u0, _, c0, v0 = rec[4 * S + 4:4 * S + 9]
    return np.array([g0, u0, 0.0, g0 * (1.0 - g0), c0, 0.0, v0, 0.0, 0.0])


FP32_THETAS = [
    (1, [0.5, 1.0, 20.0, 0.1, 0.7]),                          # scripts/model_realisation.jl:294-315
    (3, [0.1, 0.1, 30.0, 0.1, 0.1, 1.0, 15.0, 0.1, 0.7]),
    (5, [2.0, 1.0, 85.0, 2.0, 3.0, 1.0, 1.0, 1.5, 0.7]),
    (4, [0.5, 0.5, 400.0, 630.0, 320.0, 800.0, 500.0, 1.0, 0.6]),  # heavy: alpha ~ 10^2.5-10^2.9 / h
    (3, [0.1, 1.0, 3.0, 10.0, 0.3, 2.0, 630.0, 0.5, 0.8]),         # heavy, switching varies 100-fold
    # slow decay (gamma = 10^-2 / h): the initial state's variance relaxes least over the three cycles
    (1, [0.5, 1.0, 20.0, 0.01, 0.7]),
    (1, [0.05, 0.02, 300.0, 0.01, 0.5]),
]


@pytest.mark.parametrize("model,rates", FP32_THETAS)
def test_ssa_fp32_statistics_within_3_mc_se(Ctx, orc, model, rates):
    R, N, b = 256, 400, 0.3
    th = np.log10(np.array(rates))
    cells = group_cells(N, b)
    cfg = make_config("hour", precision=abi.FP32)
    with Ctx(cfg, cells) as ctx:
        out = ctx.simulate_cells(model, np.repeat(th[None, :], R, axis=0), seed=41)
    st = out["stats"]
    cap = out["captured"].astype(np.float64)  # R x C x 2
    raw = orc.moment_model(make_config("hour"), model, th, periodic_iv(orc, make_config("hour"), model, th))["moments"]
    mom = captured_moments(raw, b)
    ode = orc.stats_from_moments(make_config("hour"), mom, cells.age_dist)
    # statistics: replicate means vs the moment ODE
    mean, sd = st.mean(axis=0), st.std(axis=0, ddof=1)
    z_stat = (mean - ode) / (sd / math.sqrt(R))
    # per group: pooled moments of the captured counts vs their exact values
    z_mom = []
    for j in range(11):
        for a in range(5):
            sel = (cells.cond == j) & (cells.age == a)
            x, y = cap[:, sel, 0].ravel(), cap[:, sel, 1].ravel()
            n = x.shape[0]
            dx, dy = x - x.mean(), y - y.mean()
            e = mom[j, a]
            for val, exact, var in ((x.mean(), e[0], dx.var()), (y.mean(), e[1], dy.var()),
                                    (dx.var(ddof=1), e[2], ((dx * dx) - dx.var()).var()),
                                    ((dx * dy).sum() / (n - 1), e[3], ((dx * dy) - (dx * dy).mean()).var()),
                                    (dy.var(ddof=1), e[4], ((dy * dy) - dy.var()).var())):
                if var > 0:
                    z_mom.append((val - exact) / math.sqrt(var / n))
                else:
                    # every draw equal (e.g. no labelled molecule in a short pulse):
                    # consistent when the exact value predicts a handful of nonzero draws at most
                    assert n * abs(val - exact) < 5.0, (j, a, val, exact)
    z = np.concatenate([z_stat[np.isfinite(z_stat)], np.array(z_mom)])
    report = {"model": model, "theta": rates, "replicates": R, "cells_per_group": N,
              "max_abs_z_statistics": float(np.nanmax(np.abs(z_stat))),
              "max_abs_z_group_moments": float(np.max(np.abs(z_mom))),
              "frac_abs_z_above_3": float((np.abs(z) > 3).mean()), "comparisons": int(z.shape[0]),
              "rel_dev_by_family": family_deviation(mean, ode), "max_abs_z_by_family": family_z(z_stat)}
    if os.environ.get("ABC_REPORT_DIR"):
        with open(os.path.join(os.environ["ABC_REPORT_DIR"], f"fp32_stats_{model}_{int(rates[2])}_{rates[-2]:g}.json"), "w") as f:
            json.dump(report, f)
    assert np.isfinite(z_stat).sum() >= 50, report
    assert (np.abs(z) > 3).sum() <= allowed_beyond_3(z.shape[0]) and np.abs(z).max() <= 4.5, report


@pytest.mark.parametrize("precision", [abi.FP32, abi.FP64])
def test_capture_unbiased_given_counts(Ctx, precision):
    """The binomial capture alone (model.jl:221-239, realised per cell), given
    the simulated counts n and one capture efficiency b per cell: per (condition,
    age) group and species, the sum of c - b n against its binomial standard
    error, and the sum of (c - b n)^2 - b (1 - b) n against the standard error
    of that sum (Var (X - np)^2 = npq + (2 n^2 - 6 n) p^2 q^2).  Counts from 0
    to several 10^4 exercise both samplers (inversion below n b = 10, BTRD
    above, in FP32 arithmetic in the production mode)."""
    cfg = make_config("hour", precision=precision)
    zs = []
    for model, rates, b in ((1, [0.5, 1.0, 20.0, 0.1, 0.7], 0.3), (1, [0.05, 0.02, 300.0, 0.01, 0.5], 0.15),
                            (4, [0.5, 0.5, 400.0, 630.0, 320.0, 800.0, 500.0, 1.0, 0.6], 0.7)):
        cells = group_cells(200, b)
        th = np.repeat(np.log10(np.array(rates))[None, :], 64, axis=0)
        with Ctx(cfg, cells) as ctx:
            out = ctx.simulate_cells(model, th, seed=77)
        n = out["counts"].astype(np.float64)
        c = out["captured"].astype(np.float64)
        q = 1.0 - b
        for j in range(11):
            for a in range(5):
                sel = (cells.cond == j) & (cells.age == a)
                for sp in (0, 1):
                    nn, cc = n[:, sel, sp].ravel(), c[:, sel, sp].ravel()
                    var1 = (b * q * nn).sum()
                    if var1 <= 0:
                        assert (cc == 0).all()
                        continue
                    d = cc - b * nn
                    zs.append(d.sum() / np.sqrt(var1))
                    var2 = (nn * b * q + (2 * nn * nn - 6 * nn) * (b * q) ** 2).sum()
                    zs.append(((d * d) - b * q * nn).sum() / np.sqrt(var2))
    zs = np.array(zs)
    assert zs.shape[0] > 400
    # about 600 comparisons: by chance a couple beyond 3, none beyond 4.5
    assert (np.abs(zs) > 3).mean() <= 0.01 and np.abs(zs).max() <= 4.5, (np.abs(zs).max(), (np.abs(zs) > 3).sum())
    assert abs(zs.mean()) < 4.0 / np.sqrt(zs.shape[0]), zs.mean()
