"""Downstream of the acceptance: model probabilities with bootstrap bounds
(scripts/model_probs.jl) and posterior summaries (scripts/posterior_kinetics.jl).

CPU tests pin the oracle against numpy restatements and the binomial
distribution of the bootstrap; GPU tests require bit-identical results from
the device kernels."""
import numpy as np
import pytest

from abc_inference_transcription_gb300.config import make_config


def test_model_probs_cases_and_bootstrap_distribution(orc):
    counts = np.array([[0, 0], [4, 0], [0, 9], [5, 7], [100, 300], [2000, 2000]], np.int64)
    p, lb, ub = orc.model_probs(counts, n_boot=100, alpha=0.95, seed=3)
    assert (p[0] == 0).all() and (lb[0] == 0).all() and (ub[0] == 0).all()         # no acceptance
    assert p[1].tolist() == [1, 0] and lb[1].tolist() == [1, 0] and ub[1].tolist() == [1, 0]  # one group
    assert p[2].tolist() == [0, 1] and ub[2].tolist() == [0, 1]
    assert np.array_equal(p[3:], counts[3:] / counts[3:].sum(1, keepdims=True))
    assert (lb[3:] <= p[3:]).all() and (p[3:] <= ub[3:]).all()
    # two groups: the bounds of one group mirror the other's
    assert np.allclose(lb[3:, 0] + ub[3:, 1], 1.0, atol=1e-12)
    # 5 %-95 % bootstrap quantiles of a binomial proportion: n p (1 - p) large -> normal, +-1.645 sd
    for row in (4, 5):
        n = counts[row].sum()
        q = counts[row, 0] / n
        sd = np.sqrt(q * (1 - q) / n)
        assert abs((ub[row, 0] - lb[row, 0]) / (2 * 1.645 * sd) - 1.0) < 0.25, (row, lb[row], ub[row])


def test_model_probs_multinomial_marginals(orc):
    """Five groups: each group's resampled proportion is Binomial(n, l_m / n) / n;
    over many genes with the same counts the bounds scatter around its quantiles."""
    l = np.array([50, 0, 150, 200, 100], np.int64)
    counts = np.tile(l, (400, 1))
    p, lb, ub = orc.model_probs(counts, n_boot=100, alpha=0.95, seed=11)
    n = l.sum()
    for m in (0, 2, 3, 4):
        q = l[m] / n
        sd = np.sqrt(q * (1 - q) / n)
        assert abs(lb[:, m].mean() - (q - 1.645 * sd)) < 0.15 * sd
        assert abs(ub[:, m].mean() - (q + 1.645 * sd)) < 0.15 * sd
    assert (lb[:, 1] == 0).all() and (ub[:, 1] == 0).all()


def test_quantile_is_julias_default(orc):
    """Julia's quantile (alpha = beta = 1) is numpy's linear method: checked
    through the posterior bounds of single-gene, single-column cases."""
    rng = np.random.default_rng(2)
    for n in (1, 2, 3, 10, 101, 1000):
        theta = rng.normal(size=(n, 1))
        off = np.array([0, n])
        idx = np.arange(1, n + 1)
        for q in (0.95, 0.9, 0.5):
            r = orc.posterior_summary(theta, off, idx, q)
            assert np.isclose(r["lower"][0, 0], np.quantile(theta[:, 0], 1 - q), rtol=0, atol=1e-12)
            assert np.isclose(r["upper"][0, 0], np.quantile(theta[:, 0], q), rtol=0, atol=1e-12)


def test_posterior_summary_matches_numpy(orc):
    rng = np.random.default_rng(5)
    P, npar, G = 500, 9, 6
    theta = rng.normal(size=(P, npar))
    lists = [rng.choice(P, size=k, replace=False) + 1 for k in (1, 0, 7, 50, 200, 3)]
    off = np.concatenate([[0], np.cumsum([len(x) for x in lists])])
    idx = np.concatenate(lists)
    r = orc.posterior_summary(theta, off, idx, 0.95)
    assert r["n_particles"].tolist() == [len(x) for x in lists]
    for g, lst in enumerate(lists):
        if len(lst) == 0:
            assert np.isnan(r["map"][g]).all() and np.isnan(r["mean"][g]).all()
            continue
        sub = theta[lst - 1]
        assert np.array_equal(r["map"][g], theta[lst[0] - 1])          # first = lowest error = MAP
        assert np.allclose(r["mean"][g], sub.mean(0), rtol=1e-13, atol=1e-15)
        assert np.allclose(r["lower"][g], np.quantile(sub, 1 - 0.95, axis=0), atol=1e-12)
        assert np.allclose(r["upper"][g], np.quantile(sub, 0.95, axis=0), atol=1e-12)


def test_burst_kinetics_columns():
    from abc_inference_transcription_gb300.host import get_burst_kinetics
    rng = np.random.default_rng(1)
    s5 = rng.normal(size=(4, 5))
    bk = get_burst_kinetics(s5, 1)          # kon, koff, alpha, gamma, lambda
    assert np.array_equal(bk, np.stack([s5[:, 0], s5[:, 2] - s5[:, 1], s5[:, 2], s5[:, 3]], 1))
    s9 = rng.normal(size=(4, 9))
    bk = get_burst_kinetics(s9, 4)          # kon, koff, alpha x5, gamma, lambda
    assert bk.shape == (4, 1 + 5 + 5 + 1)
    assert np.array_equal(bk[:, 1:6], s9[:, 2:7] - s9[:, [1]])
    bk = get_burst_kinetics(s9, 3)          # kon x5, koff, alpha, gamma, lambda
    assert np.array_equal(bk[:, :5], s9[:, :5]) and np.array_equal(bk[:, 5], s9[:, 6] - s9[:, 5])


@pytest.mark.gpu
def test_model_probs_gpu_bit_exact(built, orc):
    from abc_inference_transcription_gb300.host import Context
    rng = np.random.default_rng(9)
    for M in (2, 5):
        counts = rng.integers(0, 400, size=(2000, M))
        counts[rng.random(counts.shape) < 0.3] = 0
        counts[:5] = 0
        counts[5:10, 1:] = 0
        with Context(make_config("hour"), None) as ctx:
            got = ctx.model_probs(counts, n_boot=100, alpha=0.95, seed=7)
        want = orc.model_probs(counts, n_boot=100, alpha=0.95, seed=7)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_posterior_summary_gpu_bit_exact(built, orc):
    from abc_inference_transcription_gb300.host import Context
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    K, G, P = 24, 40, 30000
    base = np.abs(rng.normal(5.0, 3.0, (200, K))) + 0.1
    stats = base[rng.integers(0, 200, P)] * rng.lognormal(0, 0.2, (P, K))
    data = base[rng.integers(0, 200, G)] * rng.lognormal(0, 0.05, (G, K))
    se = 0.1 * np.abs(data) * rng.lognormal(0, 0.5, (G, K))
    theta = rng.normal(size=(P, 9))
    tied = np.round(theta * 2.0) / 2.0                   # heavy ties, negative values and zeros
    with Context(make_config("hour"), None) as ctx:
        # 9,000 per gene (columns keyed in place), small lists, one entry per gene
        for mode, x in ((1, 0.3), (1, 0.002), (0, 0.5), (1, 1.0 / P)):
            off, idx, _ = ctx.select(data, se, stats, mode, x, None)
            for th in (theta, tied):
                got = ctx.posterior_summary(th, q=0.95)
                want = orc.posterior_summary(th, off, idx, 0.95)
                for k in ("map", "mean", "lower", "upper", "n_particles"):
                    assert np.array_equal(got[k], want[k], equal_nan=True), (mode, x, k)
        off, idx, _ = ctx.select(data, se, stats, 1, 0.002, None)
        d_theta = torch.from_numpy(theta).cuda()
        got = ctx.posterior_summary(d_theta.data_ptr(), npar=5, on_device=True, ld=9, q=0.9)
        want = orc.posterior_summary(np.ascontiguousarray(theta[:, :5]), off, idx, 0.9)
        for k in ("map", "mean", "lower", "upper"):
            assert np.array_equal(got[k], want[k], equal_nan=True), k
