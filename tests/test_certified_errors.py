"""Certified FP32 errors of the indices-only selection
(`approx_grouped_kernel`): an exact float32 restatement of the kernel's
arithmetic (truncation split of the statistics, round-to-nearest float
operations, Kahan summation) stays within the stated bound
B(e) = (1e-6 + 1e-12) e + 1e-12 of the FP64 oracle's error on
adversarial inputs: statistics equal or within an ulp of the data, zeros,
magnitudes from 1e-15 to 1e15, tiny standard errors."""
import numpy as np
import pytest

F32 = np.float32


def split_trunc(x):
    """x (float64 array) -> (h, l, ok) as the kernel's split_trunc."""
    b = x.view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    zero = (b << np.uint64(1)) == 0
    ok = zero | ((e >= 1023 - 60) & (e <= 1023 + 60))
    sign = (b >> np.uint64(63)).astype(np.uint32) << np.uint32(31)
    eh = np.clip(e - 1023 + 127, 1, 254).astype(np.uint32)
    hb = sign | (eh << np.uint32(23)) | ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.uint32)
    h = np.where(zero, 0, hb).astype(np.uint32).view(F32)
    r = (b & np.uint64(0x1FFFFFFF)).astype(F32)                       # round to nearest, as __uint2float_rn
    scale = (np.clip(e - 1075 + 127, 1, 254).astype(np.uint32) << np.uint32(23)).view(F32)
    l = ((r * scale).view(np.uint32) | sign).view(F32)
    l = np.where(zero, F32(0), l)
    h = np.where(zero, F32(0), h)
    return h, l, ok


def certified(data, se, stats):
    """P x G certified errors (NaN where the kernel would use FP64)."""
    K = data.shape[1]
    den = (se * se + 0.01 * (data * data)) + np.where(se + data != 0, 0.0, 1e-4)
    ad = np.abs(data)
    gok = ((data == 0) | ((ad >= 2.0 ** -60) & (ad <= 2.0 ** 60))) & (den >= 2.0 ** -120) & (den <= 2.0 ** 120)
    dh = data.astype(F32)
    dl = (data - dh.astype(np.float64)).astype(F32)
    rr = np.where(gok, (1.0 / den).astype(F32), F32(np.nan))
    sh, sl, sok = split_trunc(np.ascontiguousarray(stats))
    P, G = stats.shape[0], data.shape[0]
    acc = np.zeros((P, G), F32)
    comp = np.zeros((P, G), F32)
    with np.errstate(all="ignore"):
        for k in range(K):
            x = dh[None, :, k] - sh[:, None, k]
            y = dl[None, :, k] - sl[:, None, k]
            dd = x + y
            term = dd * (dd * rr[None, :, k])
            yk = term - comp
            t = acc + yk
            comp = (t - acc) - yk
            acc = t
        e = acc * F32(1.0 / K)
    ok = sok.all(axis=1)[:, None] & np.isfinite(e)
    return np.where(ok, e.astype(np.float64), np.nan)


def bound(v):
    """the selection's bound: the linear majorant of 1e-6 v + 1.5e-12 sqrt(v + 1e-12)"""
    return 1.000001e-6 * v + 1e-12


@pytest.mark.parametrize("case", ["generic", "cancellation", "magnitudes", "zeros_and_tiny_se"])
def test_certified_error_within_bound(orc, case):
    rng = np.random.default_rng(hash(case) % 2 ** 32)
    K, G, P = 72, 6, 400
    data = np.exp(rng.normal(0, 1.5, (G, K)))
    se = 0.1 * data * rng.lognormal(0, 0.5, (G, K))
    stats = data[rng.integers(0, G, P)] * np.exp(0.25 * rng.normal(size=(P, K)))
    if case == "cancellation":                  # statistics equal to the data or one ulp away
        src = rng.integers(0, G, P)
        stats = data[src].copy()
        m = rng.random((P, K)) < 0.5
        stats[m] = np.nextafter(stats[m], np.where(rng.random(m.sum()) < 0.5, np.inf, -np.inf))
        stats *= np.where(rng.random((P, K)) < 0.1, 1.0 + 1e-9 * rng.normal(size=(P, K)), 1.0)
    elif case == "magnitudes":
        scale = 10.0 ** rng.uniform(-15, 15, (1, K))
        data = data * scale
        se = se * scale
        stats = stats * scale
    elif case == "zeros_and_tiny_se":
        data[:, ::7] = 0.0
        stats[:, ::7] = np.where(rng.random((P, len(range(0, K, 7)))) < 0.5, 0.0, 1e-3)
        se[:, 1::5] = 1e-12 * data[:, 1::5]
    err = orc.errors(data, se, stats, None)
    got = certified(data, se, stats)
    ok = np.isfinite(got) & np.isfinite(err)
    assert ok.mean() > 0.9, ok.mean()
    e = np.minimum(err[ok], 10.0)
    g = np.minimum(got[ok], 10.0)      # the kernel stores 10 only when certainly clipped; compare clipped
    dev = np.abs(g - e)
    assert np.all(dev <= bound(np.minimum(got[ok], 1e300))), (case, np.max(dev / bound(got[ok])))
    if case == "generic":
        # the bound is not loose by orders of magnitude (else the selection would recheck too much)
        assert np.max(dev / bound(got[ok])) > 1e-2, np.max(dev / bound(got[ok]))


def _certified_order(v, x, thr, clip=10.0):
    """The selection's decision logic restated: sort by certified values v
    (ties by index), flag positions whose interval [v - B, v + B] touches a
    neighbour's, the clip or the threshold, give flagged positions their exact
    value x, and sort each run of consecutive flagged positions in place."""
    n = v.shape[0]
    order = np.lexsort((np.arange(n), v))
    vs, idx = v[order].copy(), order.copy()
    B = bound(vs)
    flag = np.zeros(n, bool)
    touch = vs[:-1] + B[:-1] >= vs[1:] - B[1:]
    flag[:-1] |= touch
    flag[1:] |= touch
    flag |= np.abs(vs - clip) <= B
    flag |= np.abs(vs - thr) <= B
    vs[flag] = x[idx[flag]]
    i = 0
    while i < n:
        if not flag[i]:
            i += 1
            continue
        j = i
        while j < n and flag[j]:
            j += 1
        run = np.lexsort((idx[i:j], vs[i:j]))
        vs[i:j], idx[i:j] = vs[i:j][run], idx[i:j][run]
        i = j
    return idx, vs


def test_certified_order_logic_equals_exact_order():
    """Adversarial certified values (at the edges of their bounds), exact ties,
    dense clusters, values at the clip and at the threshold: the decision
    logic gives the exact (err, index) order, and the set below the threshold
    is exact."""
    rng = np.random.default_rng(11)
    for trial in range(200):
        n = int(rng.integers(2, 400))
        x = np.round(rng.uniform(0, 12, n), int(rng.integers(2, 8)))        # exact errors, many ties
        x = np.minimum(x, 10.0)                                              # the clip
        x[rng.random(n) < 0.1] = 10.0
        if trial % 3 == 0:                                                   # a dense cluster
            x[: n // 2] = 3.0 + rng.uniform(-1e-6, 1e-6, n // 2)
        # certified values anywhere within the bound, often at its edges:
        # |v - x| <= B(x) (1 - 2e-6) <= B(v), the kernel's guarantee
        B = bound(x) * (1.0 - 2e-6)
        edge = rng.choice([-1.0, 1.0, 0.0], n) if trial % 2 else rng.uniform(-1, 1, n)
        v = x + edge * B
        thr = float(rng.choice([3.0, 5.0, 10.0, x[rng.integers(0, n)]]))
        idx, vs = _certified_order(v, x, thr)
        want = np.lexsort((np.arange(n), x))
        assert np.array_equal(idx, want), trial
        assert set(np.flatnonzero(x <= thr)) == set(idx[: int((x <= thr).sum())]), trial
