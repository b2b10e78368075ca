"""Data-side statistics and bootstrap standard errors
(scripts/data_summary_statistics.jl).  The reference's raw per-cell counts are
not shipped (only their statistics in data/summary_stats), so the oracle is
pinned against an independent numpy restatement of the reference's estimators
and against the sampling distribution of the bootstrap; the GPU must equal the
oracle bit for bit."""
import numpy as np
import pytest

from abc_inference_transcription_gb300.config import make_config, synthetic_cells


def _counts(cells, G, seed):
    rng = np.random.default_rng(seed)
    C = cells.cond.shape[0]
    lam_u = rng.gamma(2.0, 3.0, (G, 1)) * (1.0 + 0.1 * cells.age[None, :])
    lam_l = rng.gamma(1.5, 1.0, (G, 1)) * (1.0 + 0.3 * cells.cond[None, :] / 10.0)
    u = rng.poisson(lam_u * cells.beta[None, :] * 5, (G, C)).astype(np.int32)
    l = rng.poisson(lam_l * cells.beta[None, :] * 5, (G, C)).astype(np.int32)
    u[0] = 0                      # a gene with no unlabelled counts
    return u, l


def _numpy_stats(cfg, cells, u, l):
    """data_summary_statistics.jl:1-181 restated with numpy (ddof=1 moments)."""
    A, J = cfg.n_ages, cfg.n_conds
    st = np.zeros(4 * A + 3 * J)
    for f, cond in ((0, cfg.pulse_stat_cond), (1, cfg.chase_stat_cond)):
        x = (u + l)[cells.cond == cond].astype(np.float64)
        ag = cells.age[cells.cond == cond]
        off = 0 if f == 0 else 2 * A
        for a in range(A):
            xa = x[ag == a]
            m = xa.mean()
            st[off + a] = m
            st[off + A + a] = xa.var(ddof=1) / (m + (1e-4 if m == 0 else 0.0))
    for j in range(J):
        sel = cells.cond == j
        uj, lj, aj = u[sel].astype(float), l[sel].astype(float), cells.age[sel]
        st[4 * A + j] = lj.mean() / (uj.mean() + lj.mean()) if uj.mean() + lj.mean() > 0 else 0.0
        m1 = np.array([uj[aj == a].mean() for a in range(A)])
        m2 = np.array([lj[aj == a].mean() for a in range(A)])
        v1 = np.array([uj[aj == a].var(ddof=1) for a in range(A)])
        v2 = np.array([lj[aj == a].var(ddof=1) for a in range(A)])
        c12 = np.array([np.cov(uj[aj == a], lj[aj == a])[0, 1] for a in range(A)])
        w = cells.age_dist[:, j]
        wc = lambda x, y: np.sum(w * ((x - np.sum(w * x)) * (y - np.sum(w * y))))
        tv1 = np.sum(w * v1) + wc(m1, m1)
        tv2 = np.sum(w * v2) + wc(m2, m2)
        ok = tv1 != 0 and tv2 != 0
        st[4 * A + J + j] = np.sum(w * c12) / np.sqrt(abs(tv1 * tv2)) if ok and np.any(c12 != 0) else 0.0
        st[4 * A + 2 * J + j] = wc(m1, m2) / np.sqrt(abs(tv1 * tv2)) if ok else 0.0
    return st


def test_data_stats_oracle_matches_numpy(orc):
    cfg = make_config("hour")
    cells = synthetic_cells(seed=3)
    u, l = _counts(cells, 6, 1)
    st, se = orc.data_stats(cfg, cells, u, l, n_boot=0)
    assert se is None
    for g in range(6):
        want = _numpy_stats(cfg, cells, u[g], l[g])
        assert np.allclose(st[g], want, rtol=1e-12, atol=1e-14), g
    # unlabelled species silent: ratio of means 1, correlations fall back to 0 (zero total variance)
    assert (st[0, 20:31] == 1).all() and (st[0, 31:] == 0).all()


def test_data_stats_bootstrap_se(orc):
    """Bootstrap SE of a cluster mean is close to sd / sqrt(n) (100 resamples:
    relative sampling error ~7 %); the SEs are deterministic given the seed."""
    cfg = make_config("hour")
    cells = synthetic_cells(n_per_pulse=400, n_per_chase=300, seed=4)
    u, l = _counts(cells, 8, 2)
    st, se = orc.data_stats(cfg, cells, u, l, n_boot=100, seed=7)
    st2, se2 = orc.data_stats(cfg, cells, u, l, n_boot=100, seed=7)
    assert np.array_equal(se, se2)
    A = cfg.n_ages
    ratios = []
    for g in range(1, 8):
        sel = cells.cond == cfg.pulse_stat_cond
        x = (u[g] + l[g])[sel].astype(float)
        ag = cells.age[sel]
        for a in range(A):
            xa = x[ag == a]
            ratios.append(se[g, a] / (xa.std(ddof=1) / np.sqrt(xa.size)))
    ratios = np.array(ratios)
    assert abs(np.median(ratios) - 1.0) < 0.1 and ratios.min() > 0.6 and ratios.max() < 1.5, ratios


@pytest.mark.gpu
def test_data_stats_gpu_bit_exact(built, orc):
    from abc_inference_transcription_gb300.host import Context
    cfg = make_config("hour")
    cells = synthetic_cells(seed=3)
    u, l = _counts(cells, 40, 5)
    with Context(cfg, cells) as ctx:
        st, se = ctx.data_stats(u, l, n_boot=100, seed=11)
        st0, se0 = ctx.data_stats(u, l, n_boot=0)
    want_st, want_se = orc.data_stats(cfg, cells, u, l, n_boot=100, seed=11)
    assert np.array_equal(st, want_st, equal_nan=True)
    assert np.array_equal(se, want_se, equal_nan=True)
    assert np.array_equal(st0, want_st, equal_nan=True) and se0 is None
