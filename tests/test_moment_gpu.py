"""GPU moment-ODE integrator (the reference's deterministic simulation,
scripts/model.jl:67-239 and scripts/abc_simulation.jl:13-62) against the FP64
oracle: statistics, pre-capture moments and transient cycle counts are
bit-identical, for every model, on prior draws and on the reference's own
MAP parameter sets of data/recovered_statistics (whose golden moments the
oracle reproduces to ~1e-2, the reference's CVODE tolerance)."""
import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.config import (beta_moments, make_config, minute_prior, reference_prior,
                                                      synthetic_cells)

pytestmark = pytest.mark.gpu

GOLDEN = __file__.rsplit("/", 1)[0] + "/golden"
MODELS = ["const", "const_const", "kon", "alpha", "gamma"]


@pytest.fixture(scope="module")
def Ctx(built):
    from abc_inference_transcription_gb300.host import Context
    return Context


def _oracle_batch(orc, cfg, model, theta, iv, bm, ad):
    st, mo, it = [], [], []
    for r in range(theta.shape[0]):
        o = orc.moment_model(cfg, model, theta[r], iv, beta_mom=bm, age_dist=ad)
        st.append(o["stats"])
        mo.append(o["moments"])
        it.append(o["transient_iters"])
    return np.array(st), np.array(mo), np.array(it)


@pytest.mark.parametrize("model", [1, 2, 3, 4, 5])
def test_moment_gpu_bit_exact_prior_draws(Ctx, orc, model):
    cfg = make_config("hour", precision=abi.FP64)
    cells = synthetic_cells(seed=2)
    bm = beta_moments(cells, 5)
    iv = np.zeros(9)
    iv[1] = 0.5      # abc_simulation.jl:70-71
    with Ctx(cfg, cells) as ctx:
        theta = ctx.sample_prior(model, 24, 31, reference_prior())
        got = ctx.moment_simulate(model, theta, iv, bm, cells.age_dist, moments=True)
    st, mo, it = _oracle_batch(orc, cfg, model, theta, iv, bm, cells.age_dist)
    assert np.array_equal(got["transient_iters"], it)
    assert np.array_equal(got["moments"], mo)
    assert np.array_equal(got["stats"], st, equal_nan=True)


@pytest.mark.parametrize("mi", range(5))
def test_moment_gpu_reference_map_sets(Ctx, orc, mi):
    """The reference's MAP parameter sets (golden producer iv[1] = 1/2 in
    Julia's 1-based numbering: E G = 1/2): bit-identical to the oracle, and
    within the oracle's pin of the golden recovered moments."""
    z = np.load(f"{GOLDEN}/recovered_statistics.npz")
    theta, gold = z[f"{MODELS[mi]}_theta"], z[f"{MODELS[mi]}_moments"]
    cfg = make_config("hour", precision=abi.FP64)
    cells = synthetic_cells(seed=2)
    bm = beta_moments(cells, 5)
    iv = np.zeros(9)
    iv[0] = 0.5
    with Ctx(cfg, cells) as ctx:
        got = ctx.moment_simulate(mi + 1, theta, iv, bm, cells.age_dist, moments=True)
    st, mo, it = _oracle_batch(orc, cfg, mi + 1, theta, iv, bm, cells.age_dist)
    assert np.array_equal(got["moments"], mo)
    assert np.array_equal(got["stats"], st, equal_nan=True)
    err = np.max(np.abs(got["moments"] - gold) / (np.abs(gold) + 0.01), axis=(1, 2, 3))
    assert np.median(err) < 2.0e-2 and err.max() < 5.0e-2


def test_moment_gpu_minutes_and_errors(Ctx, orc):
    cfg = make_config("min", precision=abi.FP64)
    cells = synthetic_cells(seed=5)
    bm = beta_moments(cells, 5)
    iv = np.zeros(9)
    iv[1] = 0.5
    with Ctx(cfg, cells) as ctx:
        theta = ctx.sample_prior(1, 6, 3, minute_prior())
        got = ctx.moment_simulate(1, theta, iv, bm, cells.age_dist)
        st, _, _ = _oracle_batch(orc, cfg, 1, theta, iv, bm, cells.age_dist)
        assert np.array_equal(got["stats"], st, equal_nan=True)
        bad = theta.copy()
        bad[2, 0] = np.nan
        from abc_inference_transcription_gb300.abi import AbcError
        with pytest.raises(AbcError):
            ctx.moment_simulate(1, bad, iv, bm, cells.age_dist)
    with Ctx(make_config("hour", splicing=True), cells) as ctx:
        with pytest.raises(Exception):
            ctx.moment_simulate(1, np.zeros((2, 6)), iv, bm, cells.age_dist)


@pytest.mark.parametrize("model", [1, 2, 3, 4, 5])
def test_moment_fp32_production_mode_accuracy(Ctx, model):
    """FP32 production mode against the exact FP64 mode on prior draws: the
    statistics agree to a median relative deviation of ~2e-5 and at most 1e-2,
    the size of the reference's own solver error (CVODE at its default
    tolerances, reltol 1e-3 and abstol 1e-6, with the 1 % steady-state rule,
    reproduces through the oracle to ~1e-2).
    Compared on particles whose pre-capture means and variances are all above
    the reference's abstol; below it the reference's own solution carries no
    digits, and FP32 underflow can turn a 1e-50-sized moment into 0 (a NaN
    correlation, never accepted).  The exact FP64 mode covers those particles."""
    cells = synthetic_cells(seed=2)
    bm = beta_moments(cells, 5)
    iv = np.zeros(9)
    iv[1] = 0.5
    with Ctx(make_config("hour", precision=abi.FP64), cells) as ctx:
        theta = ctx.sample_prior(model, 200, 41, reference_prior())
        exact = ctx.moment_simulate(model, theta, iv, bm, cells.age_dist, moments=True)
    with Ctx(make_config("hour", precision=abi.FP32), cells) as ctx:   # the FP64 mode's grid, cycle / 400
        fast = ctx.moment_simulate(model, theta, iv, bm, cells.age_dist, moments=True, h_max=20.0 / 400)
    same_it = fast["transient_iters"] == exact["transient_iters"]
    mv = exact["moments"][..., [0, 1, 2, 4]].reshape(theta.shape[0], -1)
    resolved = (np.abs(mv) >= 1e-6).all(axis=1)
    keep = same_it & resolved
    ok = keep[:, None] & np.isfinite(exact["stats"])
    dev = np.abs(fast["stats"] - exact["stats"]) / (np.abs(exact["stats"]) + 1e-6)
    mdev = np.abs(fast["moments"] - exact["moments"]) / (np.abs(exact["moments"]) + 1e-6)
    print(f"model {model}: resolved particles {resolved.mean():.3f}, same transient cycles {same_it.mean():.3f}; "
          f"statistics median / max deviation {np.median(dev[ok]):.2e} / {dev[ok].max():.2e}, "
          f"moments {np.median(mdev[keep]):.2e} / {mdev[keep].max():.2e}")
    assert same_it.mean() > 0.9 and keep.sum() >= 20
    assert np.isfinite(fast["stats"][keep]).all() or not np.isfinite(exact["stats"][keep]).all()
    assert np.median(dev[ok]) < 5e-5 and dev[ok].max() < 1e-2


@pytest.mark.parametrize("mi", range(5))
def test_moment_fp32_default_grid_reference_map_sets(Ctx, mi):
    """Production mode as used (FP32, default substep cycle / 80) on the
    reference's MAP parameter sets: as close to the golden recovered moments
    as the exact oracle is."""
    z = np.load(f"{GOLDEN}/recovered_statistics.npz")
    theta, gold = z[f"{MODELS[mi]}_theta"], z[f"{MODELS[mi]}_moments"]
    cells = synthetic_cells(seed=2)
    iv = np.zeros(9)
    iv[0] = 0.5
    with Ctx(make_config("hour", precision=abi.FP32), cells) as ctx:
        got = ctx.moment_simulate(mi + 1, theta, iv, beta_moments(cells, 5), cells.age_dist, moments=True)
    err = np.max(np.abs(got["moments"] - gold) / (np.abs(gold) + 0.01), axis=(1, 2, 3))
    print(f"{MODELS[mi]}: production mode vs golden median {np.median(err):.2e} max {err.max():.2e}")
    assert np.median(err) < 2.0e-2 and err.max() < 5.0e-2
