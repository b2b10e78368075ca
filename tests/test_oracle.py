"""CPU tests of the FP64 oracle: pinned against the known-answer vectors and
the reference's golden outputs before it is trusted as the GPU checker."""
import math

import numpy as np
import pytest

from abc_inference_transcription_gb300.config import (N_PULSE_CONDS, REF_FAMILIES, beta_moments, make_config,
                                                       reference_prior, minute_prior, synthetic_cells)
from conftest import GOLDEN

MODELS = ["const", "const_const", "kon", "alpha", "gamma"]


# --- Philox4x32-10 known-answer vectors (Random123 kat_vectors, philox4x32 10 rounds)
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_kat(orc, ctr, key, want):
    assert [int(x) for x in orc.philox(ctr, key)] == want


def test_xlog_xexp_accuracy(orc):
    rng = np.random.default_rng(0)
    xs = np.exp(rng.uniform(-700, 700, 4000))
    rel = max(abs(orc.xlog(x) - math.log(x)) / abs(math.log(x)) for x in xs if abs(math.log(x)) > 1e-3)
    assert rel < 4.5e-16
    us = rng.uniform(2.0 ** -33, 1.0, 4000)
    assert max(abs(orc.xlog(u) - math.log(u)) for u in us) < 2e-15
    ys = rng.uniform(-700, 700, 4000)
    assert max(abs(orc.xexp(y) - math.exp(y)) / math.exp(y) for y in ys) < 4.5e-16
    assert orc.xexp(-800.0) == 0.0 and math.isinf(orc.xexp(800.0))
    assert orc.xexp(0.0) == 1.0 and orc.xlog(1.0) == 0.0


@pytest.mark.parametrize("n,p", [(7, 0.3), (40, 0.1), (1000, 0.004), (60, 0.5), (5000, 0.14), (123456, 0.2),
                                 (200, 0.93), (10 ** 6, 0.5)])
def test_binomial_moments(orc, n, p):
    draws = orc.binomial(n, p, 20000, seed=3, stream=1)
    assert draws.min() >= 0 and draws.max() <= n
    mean, var = n * p, n * p * (1 - p)
    se_mean = math.sqrt(var / draws.size)
    assert abs(draws.mean() - mean) < 5 * se_mean
    # variance within 5 standard errors (kurtosis of a binomial ~ 3)
    assert abs(draws.var() - var) < 5 * var * math.sqrt(2.0 / draws.size) + 1e-9


def test_binomial_small_exact_distribution(orc):
    n, p = 12, 0.35
    draws = orc.binomial(n, p, 60000, seed=9, stream=1)
    obs = np.bincount(draws, minlength=n + 1)
    expect = np.array([math.comb(n, k) * p ** k * (1 - p) ** (n - k) for k in range(n + 1)]) * draws.size
    mask = expect > 5
    chi2 = (((obs - expect) ** 2) / expect)[mask].sum()
    assert chi2 < 45  # ~ chi2 with <= 12 dof, p ~ 1e-5


def test_prior_ranges(orc):
    cfg = make_config("hour")
    pr = reference_prior()
    for model in range(1, 6):
        th = orc.sample_prior(cfg, model, 2000, 5, pr)
        npar = 5 if model <= 2 else 9
        assert th.shape == (2000, npar)
        lo = {1: -3, 2: -3, 3: -3, 4: -3, 5: -3}
        assert th.min() >= -3.0 and th.max() <= 3.0
        assert th[:, -1].min() >= -0.7 and th[:, -1].max() <= 0.0
    cfgm = make_config("min", splicing=True, scaling_column=True)
    th = orc.sample_prior(cfgm, 1, 3000, 6, minute_prior())
    assert th.shape == (3000, 7)
    assert 0.5 <= th[:, -1].min() and th[:, -1].max() <= 2.0


def _load_golden():
    z = np.load(f"{GOLDEN}/recovered_statistics.npz")
    return z


@pytest.mark.parametrize("mi", range(5))
def test_moment_ode_matches_reference_golden(orc, mi):
    """The moment-ODE restatement reproduces data/recovered_statistics (written
    by scripts/recover_statistics.jl with iv[1] = 1/2, no capture).  The golden
    values come from CVODE_BDF at default tolerances with the 1 % steady-state
    stopping rule (scripts/model.jl:114-142), so agreement is ~1e-2."""
    z = _load_golden()
    name = MODELS[mi]
    theta, gold = z[f"{name}_theta"], z[f"{name}_moments"]
    cfg = make_config("hour")
    iv = np.zeros(9)
    iv[0] = 0.5
    errs = []
    for r in range(theta.shape[0]):
        mom = orc.moment_model(cfg, mi + 1, theta[r], iv)["moments"]
        errs.append(np.max(np.abs(mom - gold[r]) / (np.abs(gold[r]) + 0.01)))
    errs = np.array(errs)
    assert np.median(errs) < 2.0e-2, errs
    assert errs.max() < 5.0e-2, errs


def test_stats_formulas_against_numpy(orc):
    """Aggregation of abc_simulation.jl:23-46 restated independently in numpy."""
    cfg = make_config("hour")
    rng = np.random.default_rng(4)
    m = np.abs(rng.normal(3, 1, (11, 5, 5)))
    w = rng.uniform(0.0, 0.05, (5, 11))
    got = orc.stats_from_moments(cfg, m, w)
    A, J = 5, 11
    want = np.zeros(53)
    for j in range(J):
        ww = w[:, j]
        mu, ml, vu, cv, vl = (m[j, :, q] for q in range(5))
        wc = lambda x, y: np.sum(ww * ((x - np.sum(ww * x)) * (y - np.sum(ww * y))))
        want[4 * A + j] = np.sum(ww * ml) / (np.sum(ww * mu) + np.sum(ww * ml))
        stds = math.sqrt(abs((np.sum(ww * vu) + wc(mu, mu)) * (np.sum(ww * vl) + wc(ml, ml))))
        want[4 * A + J + j] = np.sum(ww * cv) / stds
        want[4 * A + 2 * J + j] = wc(mu, ml) / stds
        if j in (5, 6):
            off = 0 if j == 5 else 2 * A
            want[off:off + A] = mu + ml
            want[off + A:off + 2 * A] = (vu + 2 * cv + vl) / (mu + ml)
    assert np.allclose(got, want, rtol=1e-13, atol=1e-15)


def test_ssa_oracle_bridge_to_moment_ode(orc):
    """SSA oracle raw counts vs the moment-ODE expectations: per (condition,
    age) mean of u and l within a few Monte Carlo standard errors."""
    cfg = make_config("hour", precision=0)
    cells = synthetic_cells(n_per_pulse=600, n_per_chase=600, seed=3)
    theta = np.log10([0.5, 1.0, 20.0, 0.1, 0.7])
    out = orc.simulate(cfg, cells, 1, theta[None, :], seed=7, n_threads=0)
    assert out["status"] == 0
    ode = orc.moment_model(cfg, 1, theta, np.array([0, 0.5, 0, 0, 0, 0, 0, 0, 0.0]))["moments"]
    z = []
    for j in range(11):
        for a in range(5):
            sel = (cells.cond == j) & (cells.age == a)
            n = sel.sum()
            for q, col in ((0, 0), (1, 1)):
                x = out["counts"][0, sel, col].astype(float)
                z.append((x.mean() - ode[j, a, q]) / math.sqrt(max(ode[j, a, 2 + 2 * q], 1e-9) / n))
    z = np.array(z)
    assert abs(z.mean()) < 0.5 and z.std() < 1.4 and np.abs(z).max() < 4.5, z


def test_ssa_oracle_deterministic_and_offset(orc):
    cfg = make_config("hour", precision=0)
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=2)
    th = orc.sample_prior(cfg, 3, 6, 1, reference_prior())
    th[:, :5] = np.minimum(th[:, :5], 1.0)
    th[:, 6] = np.minimum(th[:, 6], 1.5)
    a = orc.simulate(cfg, cells, 3, th, seed=4)
    b = orc.simulate(cfg, cells, 3, th, seed=4, n_threads=2)
    assert np.array_equal(a["hash"], b["hash"]) and np.array_equal(a["counts"], b["counts"])
    # particles keep their streams when split with particle_offset
    c = orc.simulate(cfg, cells, 3, th[3:], seed=4, offset=3)
    assert np.array_equal(c["counts"], a["counts"][3:]) and np.array_equal(c["hash"], a["hash"][3:])


def test_event_cap_reports_status(orc):
    cfg = make_config("hour", precision=0, event_cap=10)
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=2)
    th = np.log10([[5.0, 1.0, 50.0, 1.0, 0.7]])
    out = orc.simulate(cfg, cells, 1, th, seed=1)
    assert out["status"] == -4


def _numpy_errors(data, se, stats, fam):
    """compute_errors.jl:30-70 restated with numpy broadcasting."""
    eps = np.where(se + data != 0.0, 0.0, 0.0001)
    den = se ** 2 + 0.01 * data ** 2 + eps
    t = (data[None, :, :] - stats[:, None, :]) ** 2 / den[None, :, :]
    K = data.shape[1]
    out = np.zeros(t.shape[:2])
    k = 0
    for f in fam:
        out = out + t[:, :, k:k + f].sum(axis=2) / K
        k += f
    return np.minimum(out, 10.0, where=~np.isnan(out), out=out.copy())


def test_errors_oracle_matches_numpy_on_reference_data(orc):
    z = np.load(f"{GOLDEN}/summary_stats.npz")
    data, se = z["data"][:64], z["se"][:64]
    rng = np.random.default_rng(1)
    stats = data[rng.integers(0, 64, 40)] * rng.lognormal(0, 0.3, (40, 53))
    got = orc.errors(data, se, stats, REF_FAMILIES)
    want = _numpy_errors(data, se, stats, REF_FAMILIES)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-14)
    assert got.max() <= 10.0


def test_accept_oracle_semantics(orc):
    err = np.array([[1.0, 5.0], [0.5, np.nan], [1.0, 4.8], [9.9, 10.0]])
    off, idx = orc.accept(err, 0, 4.8)
    assert off.tolist() == [0, 3, 4]
    assert idx.tolist() == [2, 1, 3, 3]   # ties by index; 1-based; NaN never accepted
    off, idx = orc.accept(err, 1, 0.5)   # top ceil(0.5*4) = 2 per gene
    assert off.tolist() == [0, 2, 4]
    assert idx.tolist() == [2, 1, 3, 1]


def test_capture_moment_transform_quirk(orc):
    """downsample (model.jl:221-239) uses the sample variance of beta next to
    the population second moment; the exact expectation of the empirical
    moments differs from it by Var_pop(beta)/(n-1) * sigma^2."""
    cfg = make_config("hour")
    cells = synthetic_cells(seed=1)
    bm = beta_moments(cells, 5)
    th = np.log10([0.5, 1.0, 20.0, 0.1, 0.7])
    iv = np.array([0, 0.5, 0, 0, 0, 0, 0, 0, 0.0])
    a = orc.moment_model(cfg, 1, th, iv, beta_mom=bm, age_dist=cells.age_dist)["stats"]
    b = orc.moment_model(cfg, 1, th, iv, beta_mom=bm, age_dist=cells.age_dist, exact_capture=True)["stats"]
    assert np.allclose(a[:5], b[:5], rtol=1e-14)  # means agree exactly
    assert np.max(np.abs(a - b) / np.abs(b)) < 2e-2


def test_mlp_reference_gradients_finite_differences():
    """The FP64 reference network (without BF16 rounding) against central
    finite differences on random coordinates of every parameter block."""
    from oracle import mlp_ref
    rng = np.random.default_rng(2)
    in_dim, K, N = 4, 7, 12
    d = mlp_ref.dims(in_dim, K)
    p = rng.normal(0, 0.08, d["n"])
    th = rng.normal(0, 1, (N, in_dim))
    st = rng.normal(0, 1, (N, K))
    args = (np.zeros(in_dim), np.ones(in_dim), np.zeros(K), np.ones(K))
    loss, g = mlp_ref.loss_and_grads(p, d, th, st, *args, rounding=False)
    for name in ("w1", "b1", "w2", "b2", "w3", "b3", "w4", "b4"):
        a, b = d[name]
        if name == "w1":
            idx = rng.integers(0, in_dim, 4) * 256 + rng.integers(0, 256, 4) + a
        elif name == "w4" or name == "b4":
            cols = rng.integers(0, 2 * K, 4)
            idx = (rng.integers(0, 256, 4) * d["out_pad"] + cols + a) if name == "w4" else cols + a
        else:
            idx = rng.integers(a, b, 4)
        for i in idx:
            h = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            fd = (mlp_ref.loss_and_grads(pp, d, th, st, *args, rounding=False)[0] -
                  mlp_ref.loss_and_grads(pm, d, th, st, *args, rounding=False)[0]) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (name, i, fd, g[i])


def test_accept_oracle_matches_numpy_restatement(orc):
    """Random error matrices with ties and NaN: eps mode is findall(err <= eps)
    followed by a stable sortperm (scripts/accepted_particles.jl:20-26), top-q
    the ceil(q P) smallest finite errors ordered by (err, index); 1-based."""
    rng = np.random.default_rng(4)
    for trial in range(30):
        P, G = int(rng.integers(1, 300)), int(rng.integers(1, 6))
        err = np.round(rng.uniform(0, 10, (P, G)), int(rng.integers(0, 3)))   # many ties
        err[rng.random((P, G)) < 0.1] = np.nan
        for mode, x in ((0, float(rng.uniform(0, 10))), (1, float(rng.uniform(0.01, 1.0)))):
            off, idx = orc.accept(err, mode, x)
            want_off, want_idx = [0], []
            for g in range(G):
                e = err[:, g]
                if mode == 0:
                    v = np.flatnonzero(e <= x)
                    sel = v[np.argsort(e[v], kind="stable")]
                else:
                    k = int(np.ceil(x * P))
                    fin = np.flatnonzero(~np.isnan(e))
                    sel = fin[np.argsort(e[fin], kind="stable")][:k]
                want_idx.extend((sel + 1).tolist())
                want_off.append(len(want_idx))
            assert off.tolist() == want_off, (trial, mode)
            assert idx.tolist() == want_idx, (trial, mode)


# --------------------------------------------------------------------------
# SSA initial state: periodic moments and the moment-matched draw
# --------------------------------------------------------------------------
@pytest.mark.parametrize("lam", [0.3, 3.0, 9.99, 10.0, 37.5, 1000.0, 3e5])
def test_poisson_sampler_exact_distribution(orc, lam):
    """Inversion (lam < 10) and PTRS (lam >= 10) against the Poisson pmf: chi-square
    over the bins with at least 20 expected draws, plus mean and variance."""
    from scipy import stats
    n = 200_000
    x = orc.poisson(lam, n, seed=11)
    assert abs(x.mean() - lam) < 5 * math.sqrt(lam / n)
    assert abs(x.var() / lam - 1.0) < 5 * math.sqrt(2.0 / n) + 5.0 / (n * lam) ** 0.5
    lo, hi = int(stats.poisson.ppf(1e-4, lam)), int(stats.poisson.ppf(1 - 1e-4, lam))
    edges = np.unique(np.linspace(lo, hi + 1, min(hi - lo + 2, 60)).astype(np.int64))
    obs = np.histogram(x, bins=np.concatenate([[-1], edges[1:-1], [np.iinfo(np.int64).max]]))[0]
    cdf = stats.poisson.cdf(np.concatenate([edges[1:-1] - 1, [np.inf]]), lam)
    exp = np.diff(np.concatenate([[0.0], cdf])) * n
    keep = exp >= 20
    chi2 = (((obs - exp) ** 2) / exp)[keep].sum()
    assert stats.chi2.sf(chi2, keep.sum() - 1) > 1e-4, (chi2, keep.sum())


def _periodic_moments_scipy(kon, koff, alpha, gamma, scal, T=20.0, S=5):
    """Periodic (E G, E u, Cov(G,u), Var u) after division, by iterating the
    cycle map integrated with LSODA at tight tolerance."""
    from scipy.integrate import solve_ivp

    def rhs(k):
        def f(t, y):
            g, m, c, v = y
            a = alpha[k] * (1 + t / T) ** scal
            return [kon[k] - (kon[k] + koff) * g, a * g - gamma[k] * m,
                    a * g * (1 - g) - (kon[k] + koff + gamma[k]) * c,
                    a * g + gamma[k] * m + 2 * a * c - 2 * gamma[k] * v]
        return f
    y = np.zeros(4)
    for _ in range(400):
        z = y.copy()
        for k in range(S):
            z = solve_ivp(rhs(k), (k * T / S, (k + 1) * T / S), z, method="LSODA", rtol=1e-11, atol=1e-10).y[:, -1]
        z = np.array([z[0], z[1] / 2, z[2] / 2, z[3] / 4 + z[1] / 4])
        if np.max(np.abs(z - y) / (np.abs(z) + 1e-9)) < 1e-11:
            break
        y = z
    return z


@pytest.mark.parametrize("model,rates", [(1, [0.5, 1.0, 20.0, 0.01, 0.7]), (2, [0.5, 1.0, 20.0, 0.01, 0.7]),
                                         (1, [100.0, 300.0, 630.0, 3.0, 0.5]),
                                         (5, [0.2, 0.05, 50.0, 0.01, 0.02, 0.1, 0.005, 0.03, 0.8]),
                                         (3, [0.001, 0.01, 0.1, 1.0, 0.05, 0.5, 300.0, 0.002, 0.5])])
def test_initial_moments_are_the_periodic_solution(orc, model, rates):
    """The SSA's initial moments (periodic solution of the unlabelled moment
    equations, model.jl:67-111, with the exponential sub-step integrator)
    against LSODA at tight tolerance: within 5e-3 relative (second order in
    the sub-step)."""
    cfg = make_config("hour", precision=0)
    r = rates
    if model == 3:
        kon, koff, al, ga = r[:5], r[5], [r[6]] * 5, [r[7]] * 5
    elif model == 5:
        kon, koff, al, ga = [r[0]] * 5, r[1], [r[2]] * 5, r[3:8]
    else:
        kon, koff, al, ga = [r[0]] * 5, r[1], [r[2]] * 5, [r[3]] * 5
    rec = orc.setup(cfg, model, np.log10(rates))
    got = rec[[-5, -4, -2, -1]]  # g0, u0, c0, v0
    want = _periodic_moments_scipy(kon, koff, al, ga, 0.0 if model == 2 else 1.0)
    assert np.all(np.abs(got - want) <= 5e-3 * np.abs(want) + 1e-9), (got, want)


@pytest.mark.parametrize("rates", [[0.5, 1.0, 20.0, 0.01, 0.7], [100.0, 300.0, 630.0, 3.0, 0.5],
                                   [0.02, 0.01, 300.0, 0.01, 0.5]])
def test_initial_draw_matches_periodic_moments(orc, rates):
    """The initial (G, u) the SSA draws reproduce E G, E u, Cov(G, u) and Var u of
    the periodic solution (zero-inflated Poisson given G), within 4 standard errors."""
    cfg = make_config("hour", precision=0)
    th = np.log10(rates)
    g0, u0, _, c0, v0 = orc.setup(cfg, 1, th)[-5:]
    n = 400_000
    G, u = orc.initial_states(cfg, 1, th, n, seed=3)
    G = G.astype(float)
    u = u.astype(float)
    du = u - u.mean()
    dg = G - G.mean()
    checks = [(G.mean(), g0, G.var()), (u.mean(), u0, u.var()),
              ((dg * du).mean(), c0, (dg * du).var()), (u.var(), v0, (du * du).var())]
    for val, want, var in checks:
        assert abs(val - want) <= 4 * math.sqrt(var / n) + 1e-9 * abs(want), (val, want, math.sqrt(var / n))
