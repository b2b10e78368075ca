"""Generate the golden fixtures from the reference's shipped data.

Run with the reference project's checkout as the argument,
  python tests/golden/make_golden.py <path to the reference project>
the outputs are committed so that tests never read the reference at run time:

  recovered_statistics.npz  theta_MAP rows (data/posterior_estimates/map_sets_<model>.txt)
                            and the moments the reference computed for them without
                            capture noise (data/recovered_statistics/<model>/<cond>/*.txt,
                            written by scripts/recover_statistics.jl:49-68)
  summary_stats.npz         data-side statistics and standard errors of the first
                            N_GENES genes (data/summary_stats/*.txt, 53 per gene in the
                            family order of scripts/compute_errors.jl:55-57)
  capture_efficiencies.npy  the 5,422 per-cell capture efficiencies (data/capture_efficiencies.txt)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MODELS = ["const", "const_const", "kon", "alpha", "gamma"]
COND_IDS = ["pulse_15", "pulse_30", "pulse_45", "pulse_60", "pulse_120", "pulse_180",
            "chase_0", "chase_60", "chase_120", "chase_240", "chase_360"]
MOMENTS = ["mean_u", "mean_l", "var_u", "cov_ul", "var_l"]
ROWS_PER_MODEL = 12
N_GENES = 256


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the reference project>")
    data = os.path.join(sys.argv[1], "data")
    if not os.path.isdir(data):
        sys.exit(f"reference data not found under {data}")
    out = {}
    for name in MODELS:
        maps = np.loadtxt(os.path.join(data, "posterior_estimates", f"map_sets_{name}.txt"), ndmin=2)
        n = min(ROWS_PER_MODEL, maps.shape[0])
        # rows spread over the file so that the fixture is not only its head
        rows = np.unique(np.linspace(0, maps.shape[0] - 1, n).astype(int))
        mom = np.zeros((len(rows), len(COND_IDS), 5, 5))  # row, condition, age, moment
        for qi, q in enumerate(MOMENTS):
            for j, cid in enumerate(COND_IDS):
                m = np.loadtxt(os.path.join(data, "recovered_statistics", name, cid, f"{q}.txt"), ndmin=2)
                mom[:, j, :, qi] = m[rows]
        out[f"{name}_rows"] = rows
        out[f"{name}_theta"] = maps[rows]
        out[f"{name}_moments"] = mom
    np.savez_compressed(os.path.join(HERE, "recovered_statistics.npz"), **out)

    ss = os.path.join(data, "summary_stats")
    fam = ["pulse_mean", "pulse_ff", "chase_mean", "chase_ff", "ratio", "mean_corr", "corr_mean"]
    dfile = {"ratio": "ratio_data", "mean_corr": "mean_corr_data", "corr_mean": "corr_mean_data"}
    sfile = {"ratio": "ratio_se", "mean_corr": "mean_corr_se", "corr_mean": "corr_mean_se"}
    d = np.concatenate([np.loadtxt(os.path.join(ss, dfile.get(f, f) + ".txt"))[:N_GENES] for f in fam], axis=1)
    s = np.concatenate([np.loadtxt(os.path.join(ss, sfile.get(f, f + "_se") + ".txt"))[:N_GENES] for f in fam],
                       axis=1)
    np.savez_compressed(os.path.join(HERE, "summary_stats.npz"), data=d, se=s)

    betas = np.loadtxt(os.path.join(data, "capture_efficiencies.txt"))
    np.save(os.path.join(HERE, "capture_efficiencies.npy"), betas)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
