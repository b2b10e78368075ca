"""Workload definitions: the reference's time grid and prior, the synthetic
benchmark grid, and synthetic cell tables.

Reference constants (paths inside pthomaslab/abc_inference_transcription):
  condition_id / cycle / t0 / agevec   scripts/abc_simulation.jl:64-76
  tau_ = (2k+1)/(2*5)                  scripts/load_process_data.jl:50-57
  prior ranges                         scripts/abc_simulation.jl:3-11
  age_id_distribution normalisation    scripts/load_process_data.jl:68-81
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .abi import AbcConfig, AbcPrior, FP32, FP64, nstats

# reference labelling conditions (hours): pulse, chase (abc_simulation.jl:65)
REF_PULSE_H = [0.25, 0.5, 0.75, 1.0, 2.0, 3.0, 22.0, 22.0, 22.0, 22.0, 22.0]
REF_CHASE_H = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 2.0, 4.0, 6.0]
N_PULSE_CONDS = 6
TAU = [(2 * k + 1) / (2 * 5) for k in range(5)]  # load_process_data.jl:52
# reference statistic families (compute_errors.jl:55-57): sizes for A=5, J=11
REF_FAMILIES = [5, 5, 5, 5, 11, 11, 11]


def make_config(unit: str = "hour", precision: int = FP32, splicing: bool = False,
                scaling_column: bool = False, event_cap: int = 0) -> AbcConfig:
    """Time grid of the reference (unit='hour', cycle 20 h) or the same grid in
    minutes (unit='min', cycle 1200 min: pulses 15..180 min, chases 0..360 min
    after a 22 h pulse)."""
    scale = {"hour": 1.0, "min": 60.0}[unit]
    cfg = AbcConfig()
    cfg.cycle = 20.0 * scale
    cfg.n_burn_cycles = 3
    cfg.n_steps = 5
    cfg.n_ages = 5
    cfg.n_conds = 11
    for a, t in enumerate(TAU):
        cfg.ages[a] = t * cfg.cycle
    for j in range(11):
        cfg.pulse[j] = REF_PULSE_H[j] * scale
        cfg.chase[j] = REF_CHASE_H[j] * scale
    cfg.pulse_stat_cond = 5   # abc_simulation.jl:29 (j == 6)
    cfg.chase_stat_cond = 6   # abc_simulation.jl:41 (j == 7)
    cfg.splicing = int(splicing)
    cfg.scaling_column = int(scaling_column)
    cfg.precision = int(precision)
    cfg.event_cap = int(event_cap)
    return cfg


def config_families(cfg: AbcConfig) -> list[int]:
    A, J = cfg.n_ages, cfg.n_conds
    return [A, A, A, A, J, J, J]


def reference_prior() -> AbcPrior:
    """log10 ranges per hour, scripts/abc_simulation.jl:4-9."""
    p = AbcPrior()
    p.kon[:] = (-3.0, 3.0)
    p.koff[:] = (-3.0, 3.0)
    p.alpha[:] = (-3.0, 3.0)
    p.gamma[:] = (-3.0, 2.0)
    p.lambda_[:] = (-0.7, 0.0)
    p.beta[:] = (-3.0, 1.0)
    p.scaling[:] = (0.5, 2.0)
    p.vary_mode = 0
    p.factor[:] = (0.2, 5.0)
    return p


def factor_prior() -> AbcPrior:
    """Reference ranges; a varying rate is a base draw times a per-step factor
    log-uniform in [0.2, 5] (the batched five-model workload)."""
    p = reference_prior()
    p.vary_mode = 1
    return p


def minute_prior() -> AbcPrior:
    """Per-minute ranges of the constant-scaling synthetic workload: k_on, k_off
    in [1e-3, 1e1], alpha in [1e-1, 1e3], beta, gamma in [1e-3, 1e1], scaling in
    [0.5, 2], lambda as in the reference."""
    p = AbcPrior()
    p.kon[:] = (-3.0, 1.0)
    p.koff[:] = (-3.0, 1.0)
    p.alpha[:] = (-1.0, 3.0)
    p.gamma[:] = (-3.0, 1.0)
    p.lambda_[:] = (-0.7, 0.0)
    p.beta[:] = (-3.0, 1.0)
    p.scaling[:] = (0.5, 2.0)
    p.vary_mode = 1
    p.factor[:] = (0.2, 5.0)
    return p


@dataclass
class CellTable:
    cond: np.ndarray      # int32 [C], 0-based labelling condition
    age: np.ndarray       # int32 [C], 0-based age group
    beta: np.ndarray      # float64 [C], capture efficiency
    age_dist: np.ndarray  # float64 [A, J], row-major weights

    @property
    def n(self) -> int:
        return int(self.cond.shape[0])


def age_distribution(cond: np.ndarray, age: np.ndarray, n_ages: int, n_conds: int) -> np.ndarray:
    """Fraction of all cells in each (age, condition) group, normalised by the
    total over all conditions as age_id_distribution is (load_process_data.jl:80-81)."""
    w = np.zeros((n_ages, n_conds), dtype=np.float64)
    np.add.at(w, (age, cond), 1.0)
    return w / float(cond.shape[0])


def synthetic_cells(n_per_pulse: int = 200, n_per_chase: int = 160, n_ages: int = 5,
                    seed: int = 1, beta: tuple[float, float] = (4.0, 16.0),
                    betas: np.ndarray | None = None) -> CellTable:
    """Synthetic cells: n_per_pulse per pulse condition, n_per_chase per chase
    condition (2,000 cells with the defaults), uniform age group, capture
    efficiency Beta(4,16) -- or taken in order from `betas` (e.g. the
    reference's capture_efficiencies.txt)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cond = np.concatenate([np.full(n_per_pulse, j, np.int32) for j in range(N_PULSE_CONDS)] +
                          [np.full(n_per_chase, j, np.int32) for j in range(N_PULSE_CONDS, 11)])
    C = cond.shape[0]
    for _ in range(20):
        age = rng.integers(0, n_ages, size=C).astype(np.int32)
        counts = np.zeros((11, n_ages), np.int64)
        np.add.at(counts, (cond, age), 1)
        if counts.min() >= 2:
            break
    else:
        # small tables: round-robin ages within each condition, then shuffled
        if min(n_per_pulse, n_per_chase) < 2 * n_ages:
            raise ValueError("need at least 2 cells per (condition, age) group")
        age = np.zeros(C, np.int32)
        for j in range(11):
            idx = np.nonzero(cond == j)[0]
            age[idx] = rng.permutation(np.arange(idx.shape[0]) % n_ages).astype(np.int32)
    if betas is None:
        b = rng.beta(beta[0], beta[1], size=C)
    else:
        b = np.resize(np.asarray(betas, np.float64), C)
    return CellTable(cond=cond, age=age, beta=np.ascontiguousarray(b, np.float64),
                     age_dist=age_distribution(cond, age, n_ages, 11))


def beta_moments(cells: CellTable, n_ages: int) -> np.ndarray:
    """Per (pulse/chase set, age group): mean, mean of squares, sample variance
    of the capture efficiencies (scripts/model.jl:229-234)."""
    out = np.zeros((2, n_ages, 3))
    for s in range(2):
        sel = (cells.cond < N_PULSE_CONDS) if s == 0 else (cells.cond >= N_PULSE_CONDS)
        for a in range(n_ages):
            b = cells.beta[sel & (cells.age == a)]
            out[s, a] = (b.mean(), (b * b).mean(), b.var(ddof=1))
    return out


__all__ = ["make_config", "reference_prior", "factor_prior", "minute_prior", "synthetic_cells",
           "CellTable", "age_distribution", "beta_moments", "config_families", "REF_FAMILIES",
           "N_PULSE_CONDS", "nstats", "FP32", "FP64"]
