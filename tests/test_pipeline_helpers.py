"""Host-side helpers of the screened ABC pipeline (no GPU): thresholds from
acceptance lists with the clip at 10, screen thresholds for genes without a
threshold, the shared log-rates of the five models' parameter layouts, and the
posterior-mean agreement statistic."""
import numpy as np

from abc_inference_transcription_gb300 import pipeline as pl


def test_thresholds_ignore_clipped_errors():
    # gene 0: clean list; gene 1: its k-th error is the clip; gene 2: only clipped; gene 3: empty
    off = np.array([0, 3, 6, 8, 8])
    err = np.array([0.1, 0.5, 0.9, 0.2, 4.0, 10.0, 10.0, 10.0])
    thr = pl.thresholds_from_lists(off, err)
    assert thr.tolist() == [0.9, 4.0, -1.0, -1.0]


def test_screen_thresholds_exclude_genes_without_threshold():
    thr = np.array([1.0, -1.0, 0.0])
    x = pl._screen_x(thr, 0.5)
    assert x[0] == 0.5 and x[2] == 0.0 and x[1] < -1e29
    x = pl._screen_x(thr, -0.2)        # a negative factor (error-distribution statistic)
    assert x[0] == -0.2 and x[1] < -1e29


def test_shared_rates_of_each_model_layout():
    th = np.zeros((5, 9))
    th[0, :5] = [1, 2, 3, 4, 5]                               # model 1: kon koff alpha gamma lambda
    th[1, :5] = [1, 2, 3, 4, 5]                               # model 2
    th[2] = [0, 1, 2, 3, 4, 7, 8, 9, 10]                      # model 3: kon over 5 steps
    th[3] = [1, 2, 0, 1, 2, 3, 4, 7, 8]                       # model 4: alpha over 5 steps
    th[4] = [1, 2, 3, 0, 1, 2, 3, 4, 8]                       # model 5: gamma over 5 steps
    r = pl.shared_rates(th, np.arange(1, 6))
    assert r[0].tolist() == [1, 2, 3, 4, 5] and r[1].tolist() == [1, 2, 3, 4, 5]
    assert r[2].tolist() == [2, 7, 8, 9, 10]
    assert r[3].tolist() == [1, 2, 2, 7, 8]
    assert r[4].tolist() == [1, 2, 3, 2, 8]


def test_posterior_agreement_z_statistics():
    rng = np.random.default_rng(3)
    same = [rng.normal(size=(400, 5)) for _ in range(20)]
    other = [rng.normal(size=(4000, 5)) for _ in range(20)]
    a = pl.posterior_agreement(same, other)
    assert a["genes_compared"] == 20
    assert 0.4 < a["abs_z_median"] < 1.0 and a["fraction_abs_z_above_3"] < 0.02
    shifted = [x + 0.5 for x in other]
    b = pl.posterior_agreement(same, shifted)
    assert b["abs_z_median"] > 5.0
    # genes with too few accepted particles in either run are skipped
    c = pl.posterior_agreement([np.zeros((5, 5))], [np.zeros((100, 5))])
    assert c == {"genes_compared": 0}


def test_binomial_ci_clopper_pearson():
    from abc_inference_transcription_gb300.pipeline import binomial_ci
    lo, hi = binomial_ci(0, 100)
    assert lo == 0.0 and abs(hi - (1 - 0.025 ** (1 / 100))) < 1e-12
    lo, hi = binomial_ci(100, 100)
    assert hi == 1.0 and abs(lo - 0.025 ** (1 / 100)) < 1e-12
    lo, hi = binomial_ci(9, 300)
    assert lo < 9 / 300 < hi and 0.01 < lo < 0.02 and 0.05 < hi < 0.06
