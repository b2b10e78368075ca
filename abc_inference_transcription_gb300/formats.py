"""The reference's on-disk text files (tab-delimited, DelimitedFiles.writedlm
layout), written and read through the library's native formatter
(`abc_write_matrix`, `abc_write_particles`, `abc_read_particles`).

Files and the reference code that writes or reads them:
  sets_<model>_<n>.txt          theta rows                 scripts/abc_simulation.jl:93-94
  s_pulse / s_chase_<model>_<n> two rows per particle:      scripts/abc_simulation.jl:47-52,
                                means, Fano factors           read by compute_errors.jl:1-29
  s_ratios / s_mean_corr /      one row of J per particle   scripts/abc_simulation.jl:53-60
  s_corr_mean_<model>_<n>
  error_<model>.txt             one row of G errors per      scripts/compute_errors.jl:66-67
                                particle
  particles_<model>.txt         per gene: accepted 1-based   scripts/accepted_particles.jl:21-29,
                                indices by error, or 0        read by posterior_kinetics.jl:56-60
  model_prob / l_bound /        one row per gene             scripts/model_probs.jl:54-61
  u_bound.txt
  map_sets / post_mean_sets /   genes x parameters           scripts/posterior_kinetics.jl:72-75
  ci_lbs / ci_ubs_<model>.txt
The JDF column files of scripts/process_error_files.jl are Julia's binary
serialisation and are not produced (their content is error_<model>.txt).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import ERR_IO, STATUS_NAMES, load_library


def _lib():
    return load_library()


def _check(st: int, what: str) -> None:
    if st != 0:
        raise OSError(f"{what}: {STATUS_NAMES.get(st, st)}")


def _path(p) -> bytes:
    return os.fsencode(p)


def write_matrix(path, m: np.ndarray, append: bool = False) -> None:
    a = np.ascontiguousarray(np.atleast_2d(np.asarray(m, np.float64)))
    _check(_lib().abc_write_matrix(_path(path), int(append), a.shape[0], a.shape[1],
                                   a.ctypes.data_as(C.POINTER(C.c_double)), a.shape[1]), f"write {path}")


def format_double(x: float) -> str:
    buf = C.create_string_buffer(64)
    n = _lib().abc_format_double(float(x), buf, 64)
    if n < 0:
        raise ValueError(STATUS_NAMES.get(n, n))
    return buf.value.decode()


def write_particles(path, gene_offsets: np.ndarray, particle_idx: np.ndarray, append: bool = False) -> None:
    """particles_<model>.txt from the acceptance lists (offsets G + 1, 1-based indices)."""
    off = np.ascontiguousarray(gene_offsets, np.int64)
    idx = np.ascontiguousarray(particle_idx, np.int64)
    if idx.size == 0:
        idx = np.zeros(1, np.int64)
    _check(_lib().abc_write_particles(_path(path), int(append), off.shape[0] - 1,
                                      off.ctypes.data_as(C.POINTER(C.c_int64)),
                                      idx.ctypes.data_as(C.POINTER(C.c_int64))), f"write {path}")


def read_particles(path) -> tuple[np.ndarray, np.ndarray]:
    """(gene offsets, 1-based indices) of a particles_<model>.txt file."""
    lib = _lib()
    g, t = C.c_int64(), C.c_int64()
    _check(lib.abc_read_particles(_path(path), C.byref(g), C.byref(t), None, None), f"read {path}")
    off = np.zeros(g.value + 1, np.int64)
    idx = np.zeros(max(t.value, 1), np.int64)
    _check(lib.abc_read_particles(_path(path), C.byref(g), C.byref(t), off.ctypes.data_as(C.POINTER(C.c_int64)),
                                  idx.ctypes.data_as(C.POINTER(C.c_int64))), f"read {path}")
    return off, idx[:t.value]


def read_matrix(path) -> np.ndarray:
    """A tab-delimited numeric file (the reference's readdlm), as float64."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if line:
                rows.append([float(x) for x in line.split("\t")])
    return np.array(rows, np.float64)


def stats_blocks(stats: np.ndarray, n_ages: int, n_conds: int) -> dict:
    """Split P x K statistics ([pulse mean (A), pulse FF (A), chase mean (A),
    chase FF (A), ratio (J), mean_corr (J), corr_mean (J)]) into the five
    files' matrices: s_pulse and s_chase interleave a means row and an FF row
    per particle."""
    s = np.asarray(stats, np.float64)
    A, J = n_ages, n_conds
    P = s.shape[0]
    pulse = np.empty((2 * P, A))
    pulse[0::2] = s[:, 0:A]
    pulse[1::2] = s[:, A:2 * A]
    chase = np.empty((2 * P, A))
    chase[0::2] = s[:, 2 * A:3 * A]
    chase[1::2] = s[:, 3 * A:4 * A]
    return {"s_pulse": pulse, "s_chase": chase, "s_ratios": s[:, 4 * A:4 * A + J],
            "s_mean_corr": s[:, 4 * A + J:4 * A + 2 * J], "s_corr_mean": s[:, 4 * A + 2 * J:4 * A + 3 * J]}


def write_simulation(directory, model_name: str, n: int, theta: np.ndarray, stats: np.ndarray, n_ages: int,
                     n_conds: int, append: bool = True) -> list[str]:
    """sets_<model>_<n>.txt and the five statistics files of one simulation
    shard under directory/<model>/, as abc_simulation.jl writes them."""
    d = os.path.join(directory, model_name)
    os.makedirs(d, exist_ok=True)
    paths = [os.path.join(d, f"sets_{model_name}_{n}.txt")]
    write_matrix(paths[0], theta, append)
    for name, m in stats_blocks(stats, n_ages, n_conds).items():
        paths.append(os.path.join(d, f"{name}_{model_name}_{n}.txt"))
        write_matrix(paths[-1], m, append)
    return paths


def read_simulation_stats(directory, model_name: str, n: int, n_ages: int, n_conds: int) -> np.ndarray:
    """The P x K statistics back from the five files (compute_errors.jl:17-29)."""
    d = os.path.join(directory, model_name)
    rd = lambda name: read_matrix(os.path.join(d, f"{name}_{model_name}_{n}.txt"))
    pulse, chase = rd("s_pulse"), rd("s_chase")
    return np.hstack([pulse[0::2], pulse[1::2], chase[0::2], chase[1::2], rd("s_ratios"), rd("s_mean_corr"),
                      rd("s_corr_mean")])


def write_model_probs(directory, prob: np.ndarray, lb: np.ndarray, ub: np.ndarray, append: bool = True) -> None:
    """model_prob.txt, l_bound.txt, u_bound.txt: one row per gene."""
    os.makedirs(directory, exist_ok=True)
    for name, m in (("model_prob", prob), ("l_bound", lb), ("u_bound", ub)):
        write_matrix(os.path.join(directory, f"{name}.txt"), m, append)


def write_posterior_estimates(directory, model_name: str, summary: dict) -> None:
    """map_sets, post_mean_sets, ci_lbs, ci_ubs_<model>.txt (genes x parameters)."""
    os.makedirs(directory, exist_ok=True)
    for name, key in (("map_sets", "map"), ("post_mean_sets", "mean"), ("ci_lbs", "lower"), ("ci_ubs", "upper")):
        write_matrix(os.path.join(directory, f"{name}_{model_name}.txt"), summary[key], append=False)


__all__ = ["write_matrix", "format_double", "write_particles", "read_particles", "read_matrix", "stats_blocks",
           "write_simulation", "read_simulation_stats", "write_model_probs", "write_posterior_estimates", "ERR_IO"]
