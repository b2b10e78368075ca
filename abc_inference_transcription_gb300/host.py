"""Host-side mirror of the reference's hot-path interface over libabcgpu.so.

Reference functions and the calls that replace them (paths inside
pthomaslab/abc_inference_transcription):

  fix_params(vary_map, N)           scripts/abc_simulation.jl:3-11   -> fix_params / Context.sample_prior
  abc_sim(theta, ...)               scripts/abc_simulation.jl:13-62  -> abc_sim / Context.simulate
  the particle loop                 scripts/abc_simulation.jl:88-97  -> Context.simulate over a theta batch
  compute_trunc_errors(...)         scripts/compute_errors.jl:45-70  -> compute_trunc_errors / Context.errors
  acceptance loop                   scripts/accepted_particles.jl:12-32 -> accepted_particles / Context.select

Every call goes to the CUDA library; there is no CPU fallback (a missing
library raises ImportError, a failing call raises AbcError).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import AbcConfig, AbcError, AbcPrior, nstats, num_params, ptr
from .config import CellTable, REF_FAMILIES


class Context:
    """One CUDA stream and its device buffers (abc_create / abc_destroy)."""

    def __init__(self, cfg: AbcConfig, cells: CellTable | None = None):
        self.lib = abi.load_library()
        self.cfg = cfg
        h = C.c_void_p()
        st = self.lib.abc_create(C.byref(h), C.byref(cfg))
        if st != 0:
            raise AbcError(st, "abc_create failed (is a CUDA device visible?)")
        self.h = h
        self.K = nstats(cfg.n_ages, cfg.n_conds)
        self.cells = None
        if cells is not None:
            self.set_cells(cells)

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.abc_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        if st != 0:
            msg = self.lib.abc_last_error(self.h)
            raise AbcError(st, msg.decode() if msg else "")

    @property
    def stream(self) -> int:
        return int(self.lib.abc_stream(self.h) or 0)

    def num_params(self, model: int) -> int:
        return num_params(self.cfg, model)

    # -- cells -------------------------------------------------------------
    def set_cells(self, cells: CellTable) -> None:
        cond = np.ascontiguousarray(cells.cond, np.int32)
        age = np.ascontiguousarray(cells.age, np.int32)
        beta = np.ascontiguousarray(cells.beta, np.float64)
        w = np.ascontiguousarray(cells.age_dist, np.float64)
        if w.shape != (self.cfg.n_ages, self.cfg.n_conds):
            raise ValueError(f"age_dist must be {self.cfg.n_ages} x {self.cfg.n_conds}")
        self._check(self.lib.abc_set_cells(self.h, cond.shape[0], ptr(cond, C.c_int32), ptr(age, C.c_int32),
                                           ptr(beta), ptr(w)))
        self.cells = cells

    # -- prior ---------------------------------------------------------------
    def sample_prior(self, model: int, n: int, seed: int, prior: AbcPrior, offset: int = 0) -> np.ndarray:
        th = np.zeros((n, self.num_params(model)))
        self._check(self.lib.abc_sample_prior(self.h, model, n, seed, offset, C.byref(prior), ptr(th)))
        return th

    def sample_prior_device(self, model: int, n: int, seed: int, prior: AbcPrior, d_out: int, offset: int = 0) -> None:
        """Prior draw into device memory (n x npar doubles at d_out), on self.stream."""
        self._check(self.lib.abc_sample_prior_device(self.h, model, n, seed, offset, C.byref(prior),
                                                     C.c_void_p(d_out)))

    # -- simulation -------------------------------------------------------
    def simulate(self, model: int, theta: np.ndarray, seed: int, offset: int = 0) -> np.ndarray:
        th = np.ascontiguousarray(theta, np.float64)
        if th.ndim != 2 or th.shape[1] != self.num_params(model):
            raise ValueError(f"theta must be P x {self.num_params(model)}")
        out = np.zeros((th.shape[0], self.K))
        self._check(self.lib.abc_simulate(self.h, model, ptr(th), th.shape[0], seed, offset, ptr(out)))
        return out

    def simulate_device(self, model: int, d_theta: int, n: int, seed: int, d_stats: int, offset: int = 0) -> None:
        """Device pointers (e.g. torch tensors' data_ptr()); stream-ordered on self.stream."""
        self._check(self.lib.abc_simulate_device(self.h, model, C.c_void_p(d_theta), n, seed, offset,
                                                 C.c_void_p(d_stats)))

    def simulate_batch(self, models: np.ndarray, theta: np.ndarray, seed: int, offset: int = 0) -> np.ndarray:
        """Mixed-model batch: theta rows padded to the largest npar."""
        m = np.ascontiguousarray(models, np.int32)
        th = np.ascontiguousarray(theta, np.float64)
        out = np.zeros((th.shape[0], self.K))
        self._check(self.lib.abc_simulate_batch(self.h, ptr(m, C.c_int32), ptr(th), th.shape[1], th.shape[0], seed,
                                                offset, ptr(out)))
        return out

    def simulate_batch_device(self, d_models: int, d_theta: int, ld: int, n: int, seed: int, d_stats: int,
                              offset: int = 0) -> None:
        self._check(self.lib.abc_simulate_batch_device(self.h, C.c_void_p(d_models), C.c_void_p(d_theta), ld, n,
                                                       seed, offset, C.c_void_p(d_stats)))

    def synchronize(self) -> None:
        self._check(self.lib.abc_synchronize(self.h))

    def simulate_cells(self, model: int, theta: np.ndarray, seed: int, offset: int = 0) -> dict:
        th = np.ascontiguousarray(theta, np.float64)
        P, Cn = th.shape[0], self.cells.n
        out = {"counts": np.zeros((P, Cn, 2), np.int32), "captured": np.zeros((P, Cn, 2), np.int32),
               "events": np.zeros((P, Cn), np.int64), "hash": np.zeros((P, Cn), np.uint64),
               "stats": np.zeros((P, self.K))}
        self._check(self.lib.abc_simulate_cells(
            self.h, model, ptr(th), P, seed, offset, ptr(out["counts"], C.c_int32), ptr(out["captured"], C.c_int32),
            ptr(out["events"], C.c_int64), ptr(out["hash"], C.c_uint64), ptr(out["stats"])))
        return out

    def autotune(self, model: int, theta: np.ndarray, seed: int = 1) -> tuple[int, list[float]]:
        """Time the production kernel variants on `theta` and keep the fastest."""
        th = np.ascontiguousarray(theta, np.float64)
        ms = np.zeros(2)
        chosen = C.c_int()
        self._check(self.lib.abc_autotune(self.h, model, ptr(th), th.shape[0], seed, ptr(ms), C.byref(chosen)))
        return chosen.value, ms.tolist()

    def autotune_batch(self, models: np.ndarray, theta: np.ndarray, seed: int = 1) -> tuple[int, int, list[float]]:
        """Time (register variant x work chunk) on a mixed-model sample and keep the
        fastest pair: returns (variant, chunk, ms[variant * 3 + chunk index])."""
        m = np.ascontiguousarray(models, np.int32)
        th = np.ascontiguousarray(theta, np.float64)
        ms = np.zeros(6)
        v, ch = C.c_int(), C.c_int()
        self._check(self.lib.abc_autotune_batch(self.h, ptr(m, C.c_int32), ptr(th), th.shape[1], th.shape[0], seed,
                                                ptr(ms), C.byref(v), C.byref(ch)))
        return v.value, ch.value, ms.tolist()

    def set_variant(self, variant: int) -> None:
        self._check(self.lib.abc_set_variant(self.h, variant))

    def set_work_chunk(self, chunk: int) -> None:
        self._check(self.lib.abc_set_work_chunk(self.h, chunk))

    def profile(self, enable: bool = True) -> None:
        self._check(self.lib.abc_profile(self.h, int(enable)))

    def phase_ms(self) -> tuple[float, float, float]:
        """[setup, SSA, capture+statistics] kernel milliseconds of the last synchronized call."""
        out = np.zeros(3)
        self._check(self.lib.abc_profile_read(self.h, ptr(out)))
        return float(out[0]), float(out[1]), float(out[2])

    def last_counters(self) -> tuple[int, int]:
        ev, rej = C.c_int64(), C.c_int64()
        self._check(self.lib.abc_last_counters(self.h, C.byref(ev), C.byref(rej)))
        return ev.value, rej.value

    # -- distance + acceptance --------------------------------------------
    @staticmethod
    def _fam(families, K):
        if families is None:
            return 0, None
        f = np.ascontiguousarray(families, np.int32)
        if int(f.sum()) != K:
            raise ValueError("family sizes must sum to K")
        return f.shape[0], f

    def errors(self, data: np.ndarray, se: np.ndarray, stats: np.ndarray, families=None) -> np.ndarray:
        d = np.ascontiguousarray(data, np.float64)
        e = np.ascontiguousarray(se, np.float64)
        s = np.ascontiguousarray(stats, np.float64)
        G, K = d.shape
        nf, f = self._fam(families, K)
        out = np.zeros((s.shape[0], G))
        self._check(self.lib.abc_errors(self.h, ptr(d), ptr(e), G, K, nf, ptr(f, C.c_int32), ptr(s), s.shape[0],
                                        ptr(out)))
        return out

    def errors_candidate(self, data: np.ndarray, se: np.ndarray, stats: np.ndarray, families=None):
        """FP32 errors of the candidate pass for every pair [P, G], the bound
        terms (b0[G], b1) with |err32 - err| <= b0[g] + b1 err, and the mode used."""
        d = np.ascontiguousarray(data, np.float64)
        e = np.ascontiguousarray(se, np.float64)
        s = np.ascontiguousarray(stats, np.float64)
        G, K = d.shape
        nf, f = self._fam(families, K)
        out = np.zeros((s.shape[0], G), np.float32)
        b0 = np.zeros(G)
        b1, used = C.c_double(), C.c_int()
        self._check(self.lib.abc_errors_candidate(self.h, ptr(d), ptr(e), G, K, nf, ptr(f, C.c_int32), ptr(s),
                                                  s.shape[0], ptr(out, C.c_float), ptr(b0), C.byref(b1),
                                                  C.byref(used)))
        return out, b0, b1.value, used.value

    def select(self, data: np.ndarray, se: np.ndarray, stats: np.ndarray, mode: int, eps_or_q: float,
               families=None, errors: bool = True) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Accepted particles per gene: (offsets[G+1], 1-based indices, errors);
        errors=False returns None for them and lets the selection order the
        pairs from certified FP32 errors, computing FP64 only where those
        cannot decide (the reference's acceptance writes only the sorted
        indices); the accepted sets and their order are the same."""
        d = np.ascontiguousarray(data, np.float64)
        e = np.ascontiguousarray(se, np.float64)
        s = np.ascontiguousarray(stats, np.float64)
        G, K = d.shape
        nf, f = self._fam(families, K)
        tot = C.c_int64()
        self._check(self.lib.abc_set_select_errors(self.h, int(errors)))
        self._check(self.lib.abc_errors_select(self.h, ptr(d), ptr(e), G, K, nf, ptr(f, C.c_int32), ptr(s),
                                               s.shape[0], mode, float(eps_or_q), C.byref(tot)))
        return self._fetch(G, tot.value, errors)

    def _fetch(self, G: int, total: int, errors: bool = True):
        self._last_total = total
        self._sel_G = G
        off = np.zeros(G + 1, np.int64)
        idx = np.empty(max(total, 1), np.int64)
        err = np.empty(max(total, 1)) if errors else None
        self._check(self.lib.abc_accept_fetch(self.h, ptr(off, C.c_int64), ptr(idx, C.c_int64), ptr(err)))
        return off, idx[:total], (err[:total] if errors else None)

    def select_thr(self, data: np.ndarray, se: np.ndarray, stats: np.ndarray, thr: np.ndarray, families=None,
                   errors: bool = True):
        """Acceptance with one threshold per gene (errors: as in select)."""
        d = np.ascontiguousarray(data, np.float64)
        e = np.ascontiguousarray(se, np.float64)
        s = np.ascontiguousarray(stats, np.float64)
        t = np.ascontiguousarray(thr, np.float64)
        G, K = d.shape
        nf, f = self._fam(families, K)
        tot = C.c_int64()
        self._check(self.lib.abc_set_select_errors(self.h, int(errors)))
        self._check(self.lib.abc_errors_select_thr(self.h, ptr(d), ptr(e), G, K, nf, ptr(f, C.c_int32), ptr(s),
                                                   s.shape[0], ptr(t), C.byref(tot)))
        return self._fetch(G, tot.value, errors)

    def select_device(self, data: np.ndarray, se: np.ndarray, d_stats: int, n: int, mode: int, eps_or_q: float = 0.0,
                      thr: np.ndarray | None = None, families=None, errors: bool = True):
        """Acceptance with the statistics already in device memory (errors: as in select)."""
        d = np.ascontiguousarray(data, np.float64)
        e = np.ascontiguousarray(se, np.float64)
        t = None if thr is None else np.ascontiguousarray(thr, np.float64)
        G, K = d.shape
        nf, f = self._fam(families, K)
        tot = C.c_int64()
        self._check(self.lib.abc_set_select_errors(self.h, int(errors)))
        self._check(self.lib.abc_errors_select_device(self.h, ptr(d), ptr(e), G, K, nf, ptr(f, C.c_int32),
                                                      C.c_void_p(d_stats), n, mode, float(eps_or_q), ptr(t),
                                                      C.byref(tot)))
        return self._fetch(G, tot.value, errors)

    def accept_errors(self) -> np.ndarray:
        """FP64 errors of the last selection's accepted pairs (computed for them
        alone when the selection returned indices only)."""
        total = int(getattr(self, "_last_total", 0))
        out = np.zeros(total)
        if total:
            self._check(self.lib.abc_accept_errors(self.h, ptr(out)))
        return out

    def select_profile(self) -> tuple[float, int]:
        """(candidate-pass kernel ms, passes) of the last selection (needs profile(True))."""
        ms, n = C.c_double(), C.c_int()
        self._check(self.lib.abc_select_profile_read(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def select_counters(self) -> tuple[int, int]:
        """(pairs emitted by the FP32 candidate pass, pairs rechecked in FP64) of the last selection."""
        a, b = C.c_int64(), C.c_int64()
        self._check(self.lib.abc_select_counters(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def moment_simulate(self, model: int, theta: np.ndarray, iv, beta_mom: np.ndarray, age_dist: np.ndarray,
                        n_pulse_conds: int = 6, h_max: float = 0.0, moments: bool = False) -> dict:
        """Deterministic statistics of every particle from the moment ODE
        (the reference's abc_sim); {"stats", "moments" (optional), "transient_iters"}."""
        th = np.ascontiguousarray(theta, np.float64)
        P = th.shape[0]
        A, J = self.cfg.n_ages, self.cfg.n_conds
        st = np.zeros((P, nstats(A, J)))
        mo = np.zeros((P, J, A, 5)) if moments else None
        it = np.zeros(P, np.int32)
        self._check(self.lib.abc_moment_simulate(self.h, model, ptr(th), P, ptr(np.ascontiguousarray(iv, np.float64)),
                                                 float(h_max), ptr(np.ascontiguousarray(beta_mom, np.float64)),
                                                 n_pulse_conds, ptr(np.ascontiguousarray(age_dist, np.float64)),
                                                 ptr(st), ptr(mo), ptr(it, C.c_int32)))
        out = {"stats": st, "transient_iters": it}
        if moments:
            out["moments"] = mo
        return out

    def data_stats(self, u: np.ndarray, l: np.ndarray, n_boot: int = 100, seed: int = 1):
        """(statistics [G, K], bootstrap standard errors [G, K] or None) of the
        observed counts u, l [G, C] (data_summary_statistics.jl)."""
        uu = np.ascontiguousarray(u, np.int32)
        ll = np.ascontiguousarray(l, np.int32)
        G = uu.shape[0]
        K = nstats(self.cfg.n_ages, self.cfg.n_conds)
        st = np.zeros((G, K))
        se = np.zeros((G, K)) if n_boot >= 2 else None
        self._check(self.lib.abc_data_stats(self.h, ptr(uu, C.c_int32), ptr(ll, C.c_int32), G, int(n_boot),
                                            C.c_uint64(seed), ptr(st), ptr(se)))
        return st, se

    def model_probs(self, counts: np.ndarray, n_boot: int = 100, alpha: float = 0.95, seed: int = 1):
        """(prob, lower, upper) [G, M] from accepted counts [G, M] (scripts/model_probs.jl)."""
        cnt = np.ascontiguousarray(counts, np.int64)
        G, M = cnt.shape
        out = [np.zeros((G, M)) for _ in range(3)]
        self._check(self.lib.abc_model_probs(self.h, ptr(cnt, C.c_int64), G, M, int(n_boot), float(alpha),
                                             C.c_uint64(seed), *[ptr(o) for o in out]))
        return tuple(out)

    def posterior_summary(self, theta, npar: int | None = None, q: float = 0.95, on_device: bool = False,
                          ld: int | None = None) -> dict:
        """MAP, mean, quantile bounds [G, npar] and particle counts [G] of the last
        selection (scripts/posterior_kinetics.jl:1-33).  theta: host array [P, ld]
        or, with on_device, a device pointer (then pass npar and ld)."""
        if on_device:
            tp, ld_ = C.c_void_p(theta), int(ld)
        else:
            th = np.ascontiguousarray(theta, np.float64)
            tp, ld_ = ptr(th), th.shape[1]
            npar = npar or ld_
        G = int(self._sel_G)
        outs = [np.zeros((G, npar)) for _ in range(4)]
        n = np.zeros(G, np.int64)
        self._check(self.lib.abc_posterior_summary(self.h, C.cast(tp, C.POINTER(C.c_double)), ld_, npar,
                                                   1 if on_device else 0, float(q), *[ptr(o) for o in outs],
                                                   ptr(n, C.c_int64)))
        return {"map": outs[0], "mean": outs[1], "lower": outs[2], "upper": outs[3], "n_particles": n}

    def set_graph(self, enable: bool = True) -> None:
        """Run the simulation chain as one CUDA graph (captured, updated in place, launched)."""
        self._check(self.lib.abc_set_graph(self.h, 1 if enable else 0))

    def graph_counters(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        self._check(self.lib.abc_graph_counters(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_distance_mode(self, mode: int) -> None:
        """Candidate pass: 0 FP32 CUDA cores, 1 TF32 tensor cores (one term),
        2 TF32 tensor cores with hi/lo splits, 3 BF16 tensor cores with hi/lo
        splits (three terms; default; K > 96 runs mode 2)."""
        self._check(self.lib.abc_set_distance_mode(self.h, int(mode)))

    def distance_mode(self) -> tuple[int, int]:
        """(requested mode, mode used by the last selection; -1 before any)."""
        a, b = C.c_int(), C.c_int()
        self._check(self.lib.abc_get_distance_mode(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value


# ---------------------------------------------------------------------------
# Downstream of the acceptance, with the reference's names
# (scripts/model_probs.jl, scripts/posterior_kinetics.jl).
# ---------------------------------------------------------------------------
def get_model_probs(ctx: Context, counts: np.ndarray, alpha: float = 0.95, n_bootstraps: int = 100,
                    seed: int = 1):
    """Model probabilities with bootstrap bounds per gene (model_probs.jl:1-28
    and the per-gene cases :41-48).  counts[g, m]: accepted particles of model
    group m (the reference groups constant + constant-non-scaling against the
    three varying models)."""
    return ctx.model_probs(counts, n_boot=n_bootstraps, alpha=alpha, seed=seed)


def get_n_particles(offsets: np.ndarray) -> np.ndarray:
    """Accepted particles per gene (posterior_kinetics.jl:1-8; an empty list is 0)."""
    return np.diff(np.asarray(offsets, np.int64))


def get_burst_kinetics(sets: np.ndarray, model: int, n_steps: int = 5) -> np.ndarray:
    """log10 [burst frequency, burst size, synthesis rate, decay rate]
    (posterior_kinetics.jl:50-55): columns kon, alpha - koff, alpha, gamma with
    the varying rate's columns kept (vary map of model.jl:30-43)."""
    sets = np.asarray(sets, np.float64)
    nv = n_steps if model >= 3 else 1
    w = {1: 0, 2: 0, 3: 1, 4: 3, 5: 4}[model]   # index of the varying rate among kon, koff, alpha, gamma (+1)
    cols, c = [], 0
    for r in range(4):                            # kon, koff, alpha, gamma
        n = nv if (w and r == w - 1) else 1
        cols.append(list(range(c, c + n)))
        c += n
    kon, koff, alpha, gamma = (sets[:, cc] for cc in cols)
    return np.hstack([kon, alpha - koff, alpha, gamma])


# ---------------------------------------------------------------------------
# Several GPUs: particles are independent (scripts/abc_simulation.jl:88-97), so
# a run shards them by index with no data exchange; each shard keeps its
# random streams through particle_offset.  Acceptance needs one host-side
# merge per gene.
# ---------------------------------------------------------------------------
def shard_range(n_particles: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the particles simulated by `rank` of `world`."""
    base, rem = divmod(n_particles, world)
    start = rank * base + min(rank, rem)
    return start, start + base + (1 if rank < rem else 0)


def merge_accept_lists(parts, mode: int, eps_or_q: float, n_particles: int):
    """Merge per-shard acceptance results into the single-run result.

    parts: per shard (offsets[G+1], global 1-based indices, errors), each gene's
    list sorted by (err, index) -- what Context.select returns with the shard's
    start added to the indices.  mode 0 (err <= eps): concatenate and re-sort.
    mode 1 (top ceil(q P)): every member of the global top k is in its shard's
    top k, so each shard selects with the global k (q_local = k / P_shard) and
    the merge keeps the k smallest (err, index) pairs."""
    G = parts[0][0].shape[0] - 1
    k = int(np.ceil(eps_or_q * n_particles)) if mode == 1 else None
    offs = [0]
    idx_out, err_out = [], []
    for g in range(G):
        e = np.concatenate([p[2][p[0][g]:p[0][g + 1]] for p in parts])
        i = np.concatenate([p[1][p[0][g]:p[0][g + 1]] for p in parts])
        order = np.lexsort((i, e))
        if k is not None:
            order = order[:k]
        idx_out.append(i[order])
        err_out.append(e[order])
        offs.append(offs[-1] + order.shape[0])
    return (np.asarray(offs, np.int64), np.concatenate(idx_out) if idx_out else np.zeros(0, np.int64),
            np.concatenate(err_out) if err_out else np.zeros(0))


def shard_select(ctx: Context, data: np.ndarray, se: np.ndarray, d_stats: int, n_shard: int, start: int, mode: int,
                 eps_or_q: float, n_particles: int, families=None):
    """One shard's part of a sharded acceptance: the fast indices-only
    selection over the shard's particles (statistics in device memory), its
    accepted lists (top-q with the global k), the FP64 errors of those pairs
    only, and global 1-based indices -- an entry of merge_accept_lists' parts."""
    q = local_select_q(eps_or_q, n_particles, n_shard) if mode == 1 else eps_or_q
    off, idx, _ = ctx.select_device(data, se, d_stats, n_shard, mode, q, families=families, errors=False)
    err = ctx.accept_errors()
    return off, idx + start, err


def local_select_q(q: float, n_particles: int, n_shard: int) -> float:
    """q for a shard's local top-q so that it keeps the global k = ceil(q P)."""
    k = int(np.ceil(q * n_particles))
    return min(1.0, k / max(n_shard, 1))


# ---------------------------------------------------------------------------
# Reference-named entry points (same argument meaning; batched over particles)
# ---------------------------------------------------------------------------
def fix_params(ctx: Context, model: int, n: int, seed: int, prior: AbcPrior, offset: int = 0) -> np.ndarray:
    """Prior draw of n particles, column order hcat(kon, koff, alpha, gamma, lambda)
    with the varying rate expanded (scripts/abc_simulation.jl:3-11)."""
    return ctx.sample_prior(model, n, seed, prior, offset)


def abc_sim(ctx: Context, model: int, theta: np.ndarray, seed: int, offset: int = 0) -> dict:
    """Statistics of each particle in the reference's five outputs
    (scripts/abc_simulation.jl:47-61): s_pulse and s_chase (2 x A each: mean
    row then Fano-factor row), s_ratios, s_mean_corr, s_corr_mean (J each)."""
    st = ctx.simulate(model, theta, seed, offset)
    return split_stats(st, ctx.cfg.n_ages, ctx.cfg.n_conds)


def split_stats(st: np.ndarray, A: int, J: int) -> dict:
    return {
        "s_pulse": np.stack([st[:, 0:A], st[:, A:2 * A]], axis=1),
        "s_chase": np.stack([st[:, 2 * A:3 * A], st[:, 3 * A:4 * A]], axis=1),
        "s_ratios": st[:, 4 * A:4 * A + J],
        "s_mean_corr": st[:, 4 * A + J:4 * A + 2 * J],
        "s_corr_mean": st[:, 4 * A + 2 * J:4 * A + 3 * J],
    }


def compute_trunc_errors(ctx: Context, data: np.ndarray, se: np.ndarray, stats: np.ndarray,
                         families=tuple(REF_FAMILIES)) -> np.ndarray:
    """P x G clipped normalised errors (scripts/compute_errors.jl:45-70)."""
    return ctx.errors(data, se, stats, families)


def accepted_particles(ctx: Context, data: np.ndarray, se: np.ndarray, stats: np.ndarray, eps: float = 4.8,
                       families=tuple(REF_FAMILIES)) -> list[list[int]]:
    """Per gene: 1-based particle indices with err <= eps sorted by error, or [0]
    when none (scripts/accepted_particles.jl:20-29)."""
    off, idx, _ = ctx.select(data, se, stats, 0, eps, families)
    out = []
    for g in range(off.shape[0] - 1):
        lst = idx[off[g]:off[g + 1]].tolist()
        out.append(lst if lst else [0])
    return out
