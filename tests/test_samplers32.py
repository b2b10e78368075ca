"""The production mode's FP32 samplers (csrc/sampler32.cuh) against the exact
distributions: binomial draws for the capture (model.jl:221-239: inversion
below n p = 10, BTRD above, both sides of p = 1/2) and Poisson draws for the
initial states (inversion below 10, PTRS above), 2^21 draws per case, by a
chi-square goodness-of-fit test on bins pooled to >= 20 expected draws and
by the mean and variance.  The FP64 samplers of the oracle mode run through
the same checks."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_DRAWS = 1 << 21
BINOMIAL = [(5, 0.3), (30, 0.2), (2000, 0.004), (60, 0.3), (1000, 0.2), (100000, 0.3), (5000000, 0.7),
            (4194304, 0.5)]
POISSON = [0.5, 3.0, 9.9, 10.5, 50.0, 1000.0, 100000.0]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = tmp_path_factory.mktemp("samplers") / "libsamplers.so"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", os.path.join(root, "tests", "gpu_helpers", "samplers32.cu"), "-o",
                    str(so)], check=True)
    return C.CDLL(str(so))


def _draw(lib, kind, n=0, p=0.0, lam=0.0, seed=11):
    out = np.zeros(N_DRAWS, np.int64)
    st = lib.sampler_draw(C.c_int(kind), C.c_longlong(n), C.c_double(p), C.c_float(lam), C.c_longlong(N_DRAWS),
                          C.c_ulonglong(seed), out.ctypes.data_as(C.POINTER(C.c_longlong)))
    assert st == 0
    return out


def _gof(x, pmf_fn, lo, hi):
    """Chi-square p-value of the draws against pmf on [lo, hi], tails pooled."""
    from scipy import stats
    ks = np.arange(lo, hi + 1)
    pm = pmf_fn(ks)
    exp = pm * x.shape[0]
    obs = np.bincount(np.clip(x - lo, 0, hi - lo), minlength=hi - lo + 1).astype(np.float64)  # tails clipped in
    exp[0] += pmf_fn(np.arange(0, lo)).sum() * x.shape[0] if lo > 0 else 0.0
    exp[-1] += (1.0 - pm.sum() - (pmf_fn(np.arange(0, lo)).sum() if lo > 0 else 0.0)) * x.shape[0]
    # pool adjacent bins until each expects >= 20 draws
    o2, e2, so, se = [], [], 0.0, 0.0
    for o, e in zip(obs, exp):
        so += o
        se += e
        if se >= 20.0:
            o2.append(so)
            e2.append(se)
            so = se = 0.0
    if se > 0.0:
        o2[-1] += so
        e2[-1] += se
    o2, e2 = np.array(o2), np.array(e2)
    chi2 = ((o2 - e2) ** 2 / e2).sum()
    return stats.chi2.sf(chi2, max(len(o2) - 1, 1)), len(o2)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("n,p", BINOMIAL)
def test_binomial_sampler(lib, kind, n, p):
    from scipy import stats
    x = _draw(lib, kind, n=n, p=p, seed=101 + n)
    if kind == 0:
        p = float(np.float32(p))  # the FP32 sampler takes the capture efficiency in FP32
    assert x.min() >= 0 and x.max() <= n
    mu, var = n * p, n * p * (1 - p)
    sd = np.sqrt(var)
    z_mean = (x.mean() - mu) / np.sqrt(var / x.shape[0])
    # Var of the sample variance ~ (mu4 - var^2) / N with mu4 = var (1 + 3 (n - 2) p q)
    mu4 = var * (1 + 3 * (n - 2) * p * (1 - p))
    z_var = (x.var() - var) / np.sqrt(max(mu4 - var * var, 1e-300) / x.shape[0])
    lo, hi = max(0, int(mu - 8 * sd) - 1), min(n, int(mu + 8 * sd) + 1)
    pval, bins = _gof(x, lambda k: stats.binom.pmf(k, n, p), lo, hi)
    info = dict(z_mean=z_mean, z_var=z_var, p_value=pval, bins=bins)
    assert abs(z_mean) < 5 and abs(z_var) < 5 and pval > 1e-5, info


@pytest.mark.parametrize("kind", [2, 3])
@pytest.mark.parametrize("lam", POISSON)
def test_poisson_sampler(lib, kind, lam):
    from scipy import stats
    x = _draw(lib, kind, lam=lam, seed=7 + int(lam))
    assert x.min() >= 0
    z_mean = (x.mean() - lam) / np.sqrt(lam / x.shape[0])
    z_var = (x.var() - lam) / np.sqrt((lam + 2 * lam * lam) / x.shape[0])
    sd = np.sqrt(lam)
    lo, hi = max(0, int(lam - 8 * sd) - 1), int(lam + 8 * sd) + 2
    pval, bins = _gof(x, lambda k: stats.poisson.pmf(k, lam), lo, hi)
    info = dict(z_mean=z_mean, z_var=z_var, p_value=pval, bins=bins)
    assert abs(z_mean) < 5 and abs(z_var) < 5 and pval > 1e-5, info
