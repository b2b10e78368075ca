"""ctypes wrapper of the FP64 CPU oracle (oracle/abc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's CPU-baseline / reference arm.  The product never
imports this module.

Pinning: the moment ODE against the reference's data/recovered_statistics
(tests/golden/), Philox against the Random123 known-answer vectors, the FP64
SSA statistically against the moment ODE; errors() and accept(): parity
unpinned (no reference error matrix or accepted list exists), checked against
an independent numpy restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from abc_inference_transcription_gb300.abi import AbcConfig, AbcPrior, nstats, num_params, ptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libabcoracle.so")

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "abc_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        i32p = C.POINTER(C.c_int32)
        i64p = C.POINTER(C.c_int64)
        u64p = C.POINTER(C.c_uint64)
        u32p = C.POINTER(C.c_uint32)
        cfgp = C.POINTER(AbcConfig)
        L.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.orc_xlog.argtypes = [C.c_double]
        L.orc_xlog.restype = C.c_double
        L.orc_xexp.argtypes = [C.c_double]
        L.orc_xexp.restype = C.c_double
        L.orc_binomial.argtypes = [C.c_int64, C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                   C.c_int64, i64p]
        L.orc_binomial.restype = C.c_int64
        L.orc_poisson.argtypes = [C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int64, i64p]
        L.orc_poisson.restype = C.c_int64
        L.orc_num_params.argtypes = [cfgp, C.c_int]
        L.orc_sample_prior.argtypes = [cfgp, C.c_int, C.c_int64, C.c_uint64, C.c_int64, C.POINTER(AbcPrior), dp]
        L.orc_setup.argtypes = [cfgp, C.c_int, dp, dp]
        L.orc_initial_states.argtypes = [cfgp, C.c_int, dp, C.c_uint64, C.c_uint32, C.c_int64, i32p, i64p]
        L.orc_simulate.argtypes = [cfgp, C.c_int64, i32p, i32p, dp, dp, C.c_int, dp, C.c_int64, C.c_uint64,
                                   C.c_int64, C.c_int, i32p, i32p, i64p, u64p, i64p, dp]
        L.orc_stats_from_moments.argtypes = [cfgp, dp, dp, dp]
        L.orc_moment_model.argtypes = [cfgp, C.c_int, dp, dp, C.c_double, dp, C.POINTER(C.c_int), dp, C.c_int,
                                       dp, C.c_int, dp]
        L.orc_moment_batch.argtypes = [cfgp, C.c_int, dp, C.c_int64, dp, C.c_double, dp, C.c_int, dp, C.c_int, dp]
        L.orc_errors.argtypes = [dp, dp, C.c_int64, C.c_int, C.c_int, i32p, dp, C.c_int64, C.c_int, dp]
        L.orc_accept.argtypes = [dp, C.c_int64, C.c_int64, C.c_int, C.c_double, i64p, i64p, C.c_int64]
        L.orc_accept.restype = C.c_int64
        L.orc_data_stats.argtypes = [C.POINTER(AbcConfig), C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp,
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int64, C.c_int, C.c_uint64,
                                     dp, dp]
        L.orc_data_stats.restype = C.c_int
        L.orc_model_probs.argtypes = [i64p, C.c_int64, C.c_int, C.c_int, C.c_double, C.c_uint64, dp, dp, dp]
        L.orc_model_probs.restype = C.c_int
        L.orc_posterior_summary.argtypes = [dp, C.c_int64, C.c_int, i64p, i64p, C.c_int64, C.c_double, dp, dp,
                                            dp, dp, i64p]
        L.orc_posterior_summary.restype = C.c_int
        _lib = L
    return _lib


def _check(st: int, what: str) -> None:
    if st != 0:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    u32p = C.POINTER(C.c_uint32)
    lib().orc_philox4x32_10(ptr(c, C.c_uint32), ptr(k, C.c_uint32), ptr(out, C.c_uint32))
    return out


def xlog(x: float) -> float:
    return lib().orc_xlog(float(x))


def xexp(x: float) -> float:
    return lib().orc_xexp(float(x))


def binomial(n: int, p: float, n_draws: int, seed: int = 1, stream: int = 1, cell: int = 0,
             particle: int = 0) -> np.ndarray:
    out = np.zeros(n_draws, np.int64)
    lib().orc_binomial(n, p, seed, stream, cell, particle, n_draws, ptr(out, C.c_int64))
    return out


def poisson(lam: float, n_draws: int, seed: int = 1, stream: int = 3, cell: int = 0, particle: int = 0) -> np.ndarray:
    out = np.zeros(n_draws, np.int64)
    lib().orc_poisson(lam, seed, stream, cell, particle, n_draws, ptr(out, C.c_int64))
    return out


def sample_prior(cfg: AbcConfig, model: int, P: int, seed: int, prior: AbcPrior, offset: int = 0) -> np.ndarray:
    th = np.zeros((P, num_params(cfg, model)))
    _check(lib().orc_sample_prior(C.byref(cfg), model, P, seed, offset, C.byref(prior), ptr(th)), "sample_prior")
    return th


def initial_states(cfg: AbcConfig, model: int, theta: np.ndarray, n: int, seed: int = 1, particle: int = 0):
    """(G, u) at the start of n trajectories of one particle, as the SSA draws them."""
    th = np.ascontiguousarray(theta, np.float64)
    G = np.zeros(n, np.int32)
    u = np.zeros(n, np.int64)
    _check(lib().orc_initial_states(C.byref(cfg), model, ptr(th), seed, particle, n, ptr(G, C.c_int32),
                                    ptr(u, C.c_int64)), "initial_states")
    return G, u


def setup(cfg: AbcConfig, model: int, theta: np.ndarray) -> np.ndarray:
    S = cfg.n_steps
    rec = np.zeros(4 * S + 9)  # kon, alpha, gamma, amax per step; koff, lam, beta, scal, g0, u0, s0, c0, v0
    th = np.ascontiguousarray(theta, np.float64)
    _check(lib().orc_setup(C.byref(cfg), model, ptr(th), ptr(rec)), "setup")
    return rec


def simulate(cfg: AbcConfig, cells, model: int, theta: np.ndarray, seed: int, offset: int = 0,
             n_threads: int = 0, want_cells: bool = True) -> dict:
    th = np.ascontiguousarray(theta, np.float64)
    P = th.shape[0]
    Cn = cells.n
    K = nstats(cfg.n_ages, cfg.n_conds)
    out = {"stats": np.zeros((P, K))}
    if want_cells:
        out["counts"] = np.zeros((P, Cn, 2), np.int32)
        out["captured"] = np.zeros((P, Cn, 2), np.int32)
        out["events"] = np.zeros((P, Cn), np.int64)
        out["hash"] = np.zeros((P, Cn), np.uint64)
    rej = C.c_int64(0)
    ad = np.ascontiguousarray(cells.age_dist, np.float64)
    st = lib().orc_simulate(
        C.byref(cfg), Cn, ptr(cells.cond, C.c_int32), ptr(cells.age, C.c_int32), ptr(cells.beta), ptr(ad),
        model, ptr(th), P, seed, offset, n_threads,
        ptr(out.get("counts"), C.c_int32), ptr(out.get("captured"), C.c_int32),
        ptr(out.get("events"), C.c_int64), ptr(out.get("hash"), C.c_uint64), C.byref(rej), ptr(out["stats"]))
    out["status"] = st
    out["rejections"] = rej.value
    return out


def stats_from_moments(cfg: AbcConfig, moments: np.ndarray, age_dist: np.ndarray) -> np.ndarray:
    m = np.ascontiguousarray(moments, np.float64)
    ad = np.ascontiguousarray(age_dist, np.float64)
    st = np.zeros(nstats(cfg.n_ages, cfg.n_conds))
    _check(lib().orc_stats_from_moments(C.byref(cfg), ptr(m), ptr(ad), ptr(st)), "stats_from_moments")
    return st


def moment_model(cfg: AbcConfig, model: int, theta: np.ndarray, iv: np.ndarray, h_max: float = 0.0,
                 beta_mom: np.ndarray | None = None, age_dist: np.ndarray | None = None,
                 exact_capture: bool = False, n_pulse_conds: int = 6) -> dict:
    th = np.ascontiguousarray(theta, np.float64)
    ivv = np.ascontiguousarray(iv, np.float64)
    mom = np.zeros((cfg.n_conds, cfg.n_ages, 5))
    it = C.c_int(0)
    stats = None
    bm = ad = None
    if beta_mom is not None:
        stats = np.zeros(nstats(cfg.n_ages, cfg.n_conds))
        bm = np.ascontiguousarray(beta_mom, np.float64)
        ad = np.ascontiguousarray(age_dist, np.float64)
    _check(lib().orc_moment_model(C.byref(cfg), model, ptr(th), ptr(ivv), h_max, ptr(mom), C.byref(it),
                                  ptr(bm), n_pulse_conds, ptr(ad), int(exact_capture), ptr(stats)),
           "moment_model")
    return {"moments": mom, "transient_iters": it.value, "stats": stats}


def moment_batch(cfg: AbcConfig, model: int, theta: np.ndarray, iv: np.ndarray, beta_mom: np.ndarray,
                 age_dist: np.ndarray, n_threads: int = 0, h_max: float = 0.0, n_pulse_conds: int = 6) -> np.ndarray:
    th = np.ascontiguousarray(theta, np.float64)
    P = th.shape[0]
    out = np.zeros((P, nstats(cfg.n_ages, cfg.n_conds)))
    _check(lib().orc_moment_batch(C.byref(cfg), model, ptr(th), P, ptr(np.ascontiguousarray(iv, np.float64)),
                                  h_max, ptr(np.ascontiguousarray(beta_mom, np.float64)), n_pulse_conds,
                                  ptr(np.ascontiguousarray(age_dist, np.float64)), n_threads, ptr(out)),
           "moment_batch")
    return out


def errors(data: np.ndarray, se: np.ndarray, stats: np.ndarray, families=None, n_threads: int = 0) -> np.ndarray:
    d = np.ascontiguousarray(data, np.float64)
    e = np.ascontiguousarray(se, np.float64)
    s = np.ascontiguousarray(stats, np.float64)
    G, K = d.shape
    P = s.shape[0]
    fam = None if families is None else np.ascontiguousarray(families, np.int32)
    out = np.zeros((P, G))
    _check(lib().orc_errors(ptr(d), ptr(e), G, K, 0 if fam is None else len(fam), ptr(fam, C.c_int32),
                            ptr(s), P, n_threads, ptr(out)), "errors")
    return out


def accept(err: np.ndarray, mode: int, eps_or_q: float):
    e = np.ascontiguousarray(err, np.float64)
    P, G = e.shape
    offsets = np.zeros(G + 1, np.int64)
    n = lib().orc_accept(ptr(e), P, G, mode, eps_or_q, ptr(offsets, C.c_int64), None, 0)
    idx = np.zeros(max(n, 1), np.int64)
    lib().orc_accept(ptr(e), P, G, mode, eps_or_q, ptr(offsets, C.c_int64), ptr(idx, C.c_int64), n)
    return offsets, idx[:n]


def model_probs(counts: np.ndarray, n_boot: int = 100, alpha: float = 0.95, seed: int = 1):
    """model_probs.jl:1-28 with the per-gene cases of :41-48 (bootstrap from Philox)."""
    cnt = np.ascontiguousarray(counts, np.int64)
    G, M = cnt.shape
    out = [np.zeros((G, M)) for _ in range(3)]
    _check(lib().orc_model_probs(ptr(cnt, C.c_int64), G, M, n_boot, alpha, seed, *[ptr(o) for o in out]),
           "orc_model_probs")
    return tuple(out)


def posterior_summary(theta: np.ndarray, offsets: np.ndarray, idx: np.ndarray, q: float = 0.95) -> dict:
    """posterior_kinetics.jl:1-33: MAP, mean, quantile bounds and counts per gene."""
    th = np.ascontiguousarray(theta, np.float64)
    off = np.ascontiguousarray(offsets, np.int64)
    ix = np.ascontiguousarray(idx if len(idx) else np.zeros(1, np.int64), np.int64)
    G = off.shape[0] - 1
    npar = th.shape[1]
    outs = [np.zeros((G, npar)) for _ in range(4)]
    n = np.zeros(G, np.int64)
    _check(lib().orc_posterior_summary(ptr(th), npar, npar, ptr(off, C.c_int64), ptr(ix, C.c_int64), G, q,
                                       *[ptr(o) for o in outs], ptr(n, C.c_int64)), "orc_posterior_summary")
    return {"map": outs[0], "mean": outs[1], "lower": outs[2], "upper": outs[3], "n_particles": n}


def data_stats(cfg: AbcConfig, cells, u: np.ndarray, l: np.ndarray, n_boot: int = 100, seed: int = 1):
    """data_summary_statistics.jl: statistics [G, K] of observed counts u, l [G, C]
    and bootstrap standard errors (None for n_boot < 2)."""
    uu = np.ascontiguousarray(u, np.int32)
    ll = np.ascontiguousarray(l, np.int32)
    G, Cn = uu.shape
    K = nstats(cfg.n_ages, cfg.n_conds)
    st = np.zeros((G, K))
    se = np.zeros((G, K)) if n_boot >= 2 else None
    _check(lib().orc_data_stats(C.byref(cfg), Cn, ptr(np.ascontiguousarray(cells.cond, np.int32), C.c_int32),
                                ptr(np.ascontiguousarray(cells.age, np.int32), C.c_int32),
                                ptr(np.ascontiguousarray(cells.age_dist, np.float64)), ptr(uu, C.c_int32),
                                ptr(ll, C.c_int32), G, n_boot, seed, ptr(st), ptr(se)), "orc_data_stats")
    return st, se
