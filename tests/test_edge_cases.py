"""Edge cases of the distance/acceptance step (every candidate-pass mode), the
moment ODE and the data-side statistics against the oracle: single particles
and genes, K = 1, all-NaN statistics, q = 1, eps = 0, eps at and above the
clip, tile boundaries, no candidates, extreme rates, silent genes."""
import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.config import (beta_moments, make_config, reference_prior,
                                                      synthetic_cells)

pytestmark = pytest.mark.gpu
MODES = (0, 1, 2, 3)


@pytest.fixture(scope="module")
def Ctx(built):
    from abc_inference_transcription_gb300.host import Context
    return Context


def _problem(P, G, K, seed):
    rng = np.random.default_rng(seed)
    base = np.abs(rng.normal(5.0, 3.0, (50, K))) + 0.1
    stats = base[rng.integers(0, 50, P)] * rng.lognormal(0, 0.2, (P, K))
    data = base[rng.integers(0, 50, G)] * rng.lognormal(0, 0.05, (G, K))
    se = 0.1 * np.abs(data) * rng.lognormal(0, 0.5, (G, K))
    return data, se, stats


def _check(ctx, orc, data, se, stats, sel, x, errors=True):
    off, idx, err = ctx.select(data, se, stats, sel, x, None, errors=errors)
    roff, ridx = orc.accept(orc.errors(data, se, stats, None), sel, x)
    assert np.array_equal(off, roff), (sel, x)
    assert np.array_equal(idx, ridx), (sel, x)
    return off


@pytest.mark.parametrize("errors", (True, False))
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("P,G,K", [(1, 1, 72), (1, 5, 53), (7, 1, 1), (129, 257, 72), (300, 3, 2)])
def test_selection_shapes(Ctx, orc, mode, P, G, K, errors):
    data, se, stats = _problem(P, G, K, P * 1000 + G + K)
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        for sel, x in ((0, 4.8), (0, 0.0), (0, 10.0), (0, 25.0), (1, 1.0), (1, 0.3), (1, 1e-9)):
            _check(ctx, orc, data, se, stats, sel, x, errors)


@pytest.mark.parametrize("errors", (True, False))
@pytest.mark.parametrize("mode", MODES)
def test_selection_nan_and_no_candidates(Ctx, orc, mode, errors):
    data, se, stats = _problem(400, 40, 24, 3)
    stats[::3] = np.nan                     # a third of the particles all-NaN
    stats[1, 7] = np.nan                    # a particle with one NaN statistic
    data[5] = np.nan                        # a gene with NaN data
    data[9, 2] = np.nan                     # a gene with one NaN statistic
    se[12, 4] = np.nan                      # a gene with one NaN standard error
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        off = _check(ctx, orc, data, se, stats, 0, 1e-12, errors)   # almost nothing accepted
        _check(ctx, orc, data, se, stats, 1, 0.05, errors)
        _check(ctx, orc, data, se, stats, 1, 1.0, errors)           # every non-NaN particle, NaN last
        all_nan = np.full_like(stats, np.nan)
        off = _check(ctx, orc, data, se, all_nan, 1, 0.1, errors)
        assert off[-1] == 0


@pytest.mark.parametrize("errors", (True, False))
@pytest.mark.parametrize("mode", MODES)
def test_selection_per_gene_extreme_thresholds(Ctx, orc, mode, errors):
    data, se, stats = _problem(500, 6, 16, 8)
    thr = np.array([-1.0, 0.0, 1e-300, 10.0, 50.0, 2.0])
    err = orc.errors(data, se, stats, None)
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        off, idx, _ = ctx.select_thr(data, se, stats, thr, None, errors=errors)
    want_off, want_idx = [0], []
    for g in range(6):
        _, i = orc.accept(err[:, g:g + 1], 0, thr[g])
        want_idx.append(i)
        want_off.append(want_off[-1] + i.shape[0])
    assert np.array_equal(off, want_off) and np.array_equal(idx, np.concatenate(want_idx))
    assert off[1] == 0                      # thr < 0 accepts nothing
    assert off[5] - off[4] == 500           # thr >= 10 accepts every finite particle


def test_moment_single_particle_and_stiff_rates(Ctx, orc):
    cfg = make_config("hour", precision=abi.FP64)
    cells = synthetic_cells(seed=2)
    bm = beta_moments(cells, 5)
    iv = np.zeros(9)
    iv[1] = 0.5
    th = np.array([[3.0, -3.0, 3.0, 2.0, 0.0],      # fast switching, fast transcription, fast decay
                   [-3.0, 3.0, -3.0, -3.0, -0.7],   # almost silent
                   [0.0, 0.0, 2.5, -2.9, -0.3]])    # slow decay
    with Ctx(cfg, cells) as ctx:
        for r in range(th.shape[0]):
            got = ctx.moment_simulate(1, th[r:r + 1], iv, bm, cells.age_dist, moments=True)
            want = orc.moment_model(cfg, 1, th[r], iv, beta_mom=bm, age_dist=cells.age_dist)
            assert np.array_equal(got["moments"][0], want["moments"])
            assert np.array_equal(got["stats"][0], want["stats"], equal_nan=True)
            assert got["transient_iters"][0] == want["transient_iters"]


def test_data_stats_silent_and_minimal_cells(Ctx, orc):
    cfg = make_config("hour")
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=6)   # 2 cells per (condition, age) group
    rng = np.random.default_rng(1)
    C = cells.cond.shape[0]
    u = rng.poisson(3.0, (4, C)).astype(np.int32)
    l = rng.poisson(1.0, (4, C)).astype(np.int32)
    u[1] = 0
    l[1] = 0                                # a silent gene: FF with eps, ratios 0, correlations 0
    l[2] = 0                                # labelled species silent
    with Ctx(cfg, cells) as ctx:
        st, se = ctx.data_stats(u, l, n_boot=50, seed=4)
    want_st, want_se = orc.data_stats(cfg, cells, u, l, n_boot=50, seed=4)
    assert np.array_equal(st, want_st, equal_nan=True)
    assert np.array_equal(se, want_se, equal_nan=True)
    assert (st[1][:20] == 0).all() and (st[1][20:] == 0).all()


@pytest.mark.parametrize("errors", (True, False))
@pytest.mark.parametrize("mode", (0, 2, 3))
def test_selection_sort_paths_and_ties(Ctx, orc, mode, errors):
    """Per-gene lists of every sort size class (one entry per thread up to
    1,024 entries, 2, 4 and 8 per thread, and the global-memory network above
    8,192) with exact error ties (duplicated particles), ordered by (err, index)."""
    data, se, stats = _problem(30000, 3, 8, 21)
    stats[1::3] = stats[0::3][: stats[1::3].shape[0]]      # every third particle repeated
    stats[7::50] = np.nan
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        for q in (0.0005, 0.01, 0.05, 0.1, 0.2, 0.4, 1.0):
            _check(ctx, orc, data, se, stats, 1, q, errors)
        for eps in (0.5, 2.0):
            _check(ctx, orc, data, se, stats, 0, eps, errors)


def test_indices_only_selection_refuses_error_fetch(Ctx):
    data, se, stats = _problem(200, 4, 16, 9)
    with Ctx(make_config("hour"), None) as ctx:
        off, idx, err = ctx.select(data, se, stats, 1, 0.1, None, errors=False)
        assert err is None and off[-1] == 4 * 20
        with pytest.raises(RuntimeError, match="ABC_ERR_STATE"):
            ctx._fetch(4, int(off[-1]), True)


@pytest.mark.parametrize("errors", (True, False))
def test_selection_extreme_magnitudes(Ctx, orc, errors):
    """Statistics and data far outside the certified FP32 path's range
    (|x| > 2^60 or < 2^-60, a denominator below 2^-120) take its FP64
    fallback; sets and order still equal the oracle's."""
    data, se, stats = _problem(600, 8, 12, 17)
    scale = np.array([1e20, 1e-20, 1.0, 3e18, 1e-19, 1.0, 1.0, 1e15])      # per gene
    data = data * scale[:, None]
    se = se * scale[:, None]
    se[5] = 0.0
    data[5, :6] = 0.0                                                        # eps = 1e-4 denominators
    stats = np.concatenate([stats * s for s in (1e20, 1e-20, 1.0)])[::3]    # particles at three scales
    stats[::7, 3] = 1e-200
    with Ctx(make_config("hour"), None) as ctx:
        for mode in (0, 2):
            ctx.set_distance_mode(mode)
            for sel, x in ((0, 4.8), (1, 0.05), (1, 0.5)):
                _check(ctx, orc, data, se, stats, sel, x, errors)
