"""The FP32 samplers' exact tests (csrc/sampler32.cuh) rewrite the log-density
comparisons of PTRS (Poisson) and BTRD (binomial) so that every term is of
order |k - mode| instead of order n log n.  This restates both rewrites in
float32 numpy and checks them against the log-densities from lgamma in FP64,
over +-5 standard deviations around the mode up to the production mode's
count limit.  (The kernels themselves are checked by their draws on the GPU,
tests/test_samplers32.py.)"""
import numpy as np
import pytest

scipy_special = pytest.importorskip("scipy.special")

F = np.float32
FC_TABLE = [0.08106146679532726, 0.0413406959554093, 0.02767792568499834, 0.020790672103765093,
            0.016644691189821193, 0.013876128823070748, 0.01189670994589177, 0.010411265261972096,
            0.009255462182712733, 0.00833056343336287]


def fc32(k):
    """Stirling remainder log k! - [(k + 1/2) log(k + 1) - (k + 1) + log(2 pi)/2], as stirling_fc32."""
    k = F(k)
    if k < 10:
        return F(FC_TABLE[int(k)])
    kp = F(k + F(1))
    r2 = F(1) / (kp * kp)
    return (F(0.08333333333333333) - (F(0.002777777777777778) - F(0.0007936507936507937) * r2) * r2) / kp


def log1p32(x):
    return np.log1p(F(x), dtype=np.float32)


@pytest.mark.parametrize("lam", [10.5, 50.0, 1000.0, 1e5, 1e6, 4e6])
def test_ptrs_exact_test_rewrite(lam):
    lam32 = F(lam)
    sd = np.sqrt(lam)
    worst = 0.0
    for k in np.unique(np.clip(np.round(np.linspace(lam - 5 * sd, lam + 5 * sd, 61)), 0, None)):
        k32 = F(k)
        d = (k32 + F(1)) - lam32
        rhs = ((d - k32 * log1p32(d / lam32)) - F(0.5) * np.log(k32 + F(1), dtype=np.float32)) \
            - F(0.91893853320467274) - fc32(k32)
        exact = k * np.log(float(lam32)) - float(lam32) - scipy_special.gammaln(k + 1)
        worst = max(worst, abs(float(rhs) - exact))
    # error of order 1e-7 |k - lam| (about 1e-3 at lam = 4e6); the comparison it feeds
    # decides only draws between PTRS's squeezes
    assert worst < 2e-7 * (5 * sd + 10) + 1e-5, worst


@pytest.mark.parametrize("n,p", [(60, 0.3), (1000, 0.2), (100000, 0.3), (5000000, 0.3), (4194304, 0.5),
                                 (8000000, 0.05)])
def test_btrd_exact_test_rewrite(n, p):
    p32 = F(p)
    q32 = F(1) - p32
    nd = F(n)
    m = np.floor((nd + F(1)) * p32)
    sd = np.sqrt(n * p * (1 - p))
    P = float(p32)

    def logpmf(k):
        return (scipy_special.gammaln(n + 1) - scipy_special.gammaln(k + 1) - scipy_special.gammaln(n - k + 1)
                + k * np.log(P) + (n - k) * np.log1p(-P))

    worst = 0.0
    for k in np.unique(np.clip(np.round(np.linspace(float(m) - 5 * sd, float(m) + 5 * sd, 61)), 0, n)):
        kd = F(k)
        nk = (nd - kd) + F(1)
        # fmaf(n + 2, p, -(j + 1)): the product-sum rounded once
        em = F((float(nd) + 2.0) * P - (float(m) + 1.0)) / ((m + F(1)) * q32)
        ek = F((float(nd) + 2.0) * P - (float(kd) + 1.0)) / ((kd + F(1)) * q32)
        h = ((m + F(0.5)) * -log1p32(em) + fc32(m)) + fc32(nd - m)
        bound = (((h + (nd + F(1)) * log1p32((kd - m) / nk)) + (kd + F(0.5)) * log1p32(ek))
                 - fc32(kd)) - fc32(nd - kd)
        exact = logpmf(k) - logpmf(float(m))
        worst = max(worst, abs(float(bound) - exact))
    assert worst < 2e-7 * (5 * sd / (1 - p) + 10) + 1e-5, worst
