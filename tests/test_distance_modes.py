"""Candidate passes of the distance step: FP32 on the CUDA cores (mode 0) and
the tensor-core GEMM expansion (TF32 modes 1 and 2, BF16 hi/lo mode 3;
scripts/compute_errors.jl:30-43 expanded as K err = c_g + [s | s^2] . [-2 w d | w]).

Every candidate error lies within the stated bound of the exact FP64 error,
and the accepted sets after the FP64 recheck are identical to the oracle's in
every mode (eps, top-q and per-gene thresholds)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from abc_inference_transcription_gb300.config import REF_FAMILIES, make_config

pytestmark = pytest.mark.gpu

GOLDEN = __file__.rsplit("/", 1)[0] + "/golden"
MODES = (0, 1, 2, 3)


@pytest.fixture(scope="module")
def Ctx(built):
    from abc_inference_transcription_gb300.host import Context
    return Context


def _ref_data():
    z = np.load(f"{GOLDEN}/summary_stats.npz")
    return z["data"], z["se"]


def _synthetic(P, G, K, seed):
    rng = np.random.default_rng(seed)
    base = np.abs(rng.normal(5.0, 3.0, (300, K))) + 0.1
    stats = base[rng.integers(0, 300, P)] * rng.lognormal(0, 0.2, (P, K))
    data = base[rng.integers(0, 300, G)] * rng.lognormal(0, 0.05, (G, K))
    se = 0.1 * np.abs(data) * rng.lognormal(0, 0.5, (G, K))
    return data, se, stats


def _exact_unclipped(data, se, stats):
    """sum_k w (d - s)^2 / K in FP64 (numpy order; differs from the reference order by rounding only)"""
    w = 1.0 / ((se * se + 0.01 * data * data) + np.where(se + data != 0.0, 0.0, 1e-4))
    K = data.shape[1]
    out = np.empty((stats.shape[0], data.shape[0]))
    for i in range(0, stats.shape[0], 512):
        s = stats[i:i + 512]
        out[i:i + 512] = (((data[None] - s[:, None]) ** 2) * w[None]).sum(-1) / K
    return out


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("K", [72, 53])
def test_candidate_errors_within_bound(Ctx, mode, K):
    data, se, stats = _synthetic(3000, 300, K, 40 + K)
    stats[7] = np.nan            # a NaN row stays NaN
    stats[8] = 0.0
    data[5, 3], se[5, 3] = 0.0, 0.0   # eps = 1e-4 branch
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        e32, b0, b1, used = ctx.errors_candidate(data, se, stats)
    assert used == mode
    E = np.minimum(_exact_unclipped(data, se, stats), 10.0)
    assert np.isnan(e32[7]).all() and np.isfinite(np.delete(e32, 7, axis=0)).all()
    ok = np.isfinite(E)
    dev = np.abs(e32.astype(np.float64) - E)[ok]
    bound = (b0[None, :] + b1 * E)[ok]
    ratio = dev / bound
    # the measured deviation against FP64, stated per mode
    print(f"mode {mode} K {K}: max |e32 - e| = {dev.max():.3e}, max deviation / bound = {ratio.max():.3e}")
    assert ratio.max() <= 1.0


@pytest.mark.parametrize("mode", MODES)
def test_selection_identical_across_modes(Ctx, orc, mode):
    data, se = _ref_data()
    rng = np.random.default_rng(21)
    src = data[rng.integers(0, data.shape[0], 6000)]
    stats = src * rng.lognormal(0.0, 0.3, src.shape)
    stats[17] = np.nan
    stats[40:45] = stats[39]      # exact ties, broken by index
    err = orc.errors(data, se, stats, REF_FAMILIES)
    thr = np.nanquantile(err, 0.02, axis=0)
    thr[3] = -1.0
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        for sel, x in ((0, 4.8), (1, 0.005), (1, 0.05)):
            off, idx, e = ctx.select(data, se, stats, sel, x, REF_FAMILIES)
            roff, ridx = orc.accept(err, sel, x)
            assert np.array_equal(off, roff) and np.array_equal(idx, ridx), (sel, x)
            assert ctx.distance_mode() == (mode, mode)
        off, idx, _ = ctx.select_thr(data, se, stats, thr, REF_FAMILIES)
    want_off, want_idx = [0], []
    for g in range(data.shape[0]):
        _, i = orc.accept(err[:, g:g + 1], 0, thr[g])
        want_idx.append(i)
        want_off.append(want_off[-1] + i.shape[0])
    assert np.array_equal(off, want_off) and np.array_equal(idx, np.concatenate(want_idx))


def test_infinite_statistic_falls_back_to_fp32_pass(Ctx, orc):
    data, se, stats = _synthetic(4000, 64, 72, 5)
    stats[11, 2] = np.inf
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(2)
        off, idx, _ = ctx.select(data, se, stats, 1, 0.01, None)
        assert ctx.distance_mode() == (2, 0)
    roff, ridx = orc.accept(orc.errors(data, se, stats, None), 1, 0.01)
    assert np.array_equal(off, roff) and np.array_equal(idx, ridx)


def test_mode3_falls_back_to_mode2_for_long_rows(Ctx, orc):
    """Mode 3 keeps a 256-gene tile of BF16 rows (4K values, rounded up) in
    shared memory; beyond K = 96 it does not fit and the pass runs in mode 2."""
    data, se, stats = _synthetic(3000, 40, 120, 8)
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(3)
        off, idx, _ = ctx.select(data, se, stats, 1, 0.01, None)
        assert ctx.distance_mode() == (3, 2)
        e32, b0, b1, used = ctx.errors_candidate(data, se, stats)
        assert used == 2
    roff, ridx = orc.accept(orc.errors(data, se, stats, None), 1, 0.01)
    assert np.array_equal(off, roff) and np.array_equal(idx, ridx)
    E = np.minimum(_exact_unclipped(data, se, stats), 10.0)
    assert (np.abs(e32 - E) <= b0[None, :] + b1 * E).all()


@pytest.mark.parametrize("mode", (1, 2, 3))
def test_many_tiles_topq_and_segment_growth(Ctx, orc, mode):
    """391 particle tiles x 3 gene tiles: persistent CTAs loop over several
    tiles (both tensor-memory accumulators wrap), and the dense candidate
    query overflows the default per-CTA segment, which is then grown."""
    data, se, stats = _synthetic(50000, 600, 72, 77)
    err = orc.errors(data, se, stats, None)
    with Ctx(make_config("hour"), None) as ctx:
        ctx.set_distance_mode(mode)
        off, idx, _ = ctx.select(data, se, stats, 1, 0.002, None)
        roff, ridx = orc.accept(err, 1, 0.002)
        assert np.array_equal(off, roff) and np.array_equal(idx, ridx)
        cands, rechecked = ctx.select_counters()
        assert rechecked <= cands and rechecked >= int(off[-1])
        e32, b0, b1, _ = ctx.errors_candidate(data[:300], se[:300], stats[:40000])
    E = np.minimum(_exact_unclipped(data[:300], se[:300], stats[:40000]), 10.0)
    assert (np.abs(e32 - E) <= b0[None, :] + b1 * E).all()


@pytest.mark.gpu
def test_rn32_bits_matches_conversion(tmp_path):
    """The operand preparation of the tensor-core pass rounds FP64 to FP32 on
    the bit fields (rn32_bits); it must equal the conversion instruction bit
    for bit, here on 2 x 2^31 patterns including every exponent of the float
    range and its edges, ties and near-ties at the rounding position."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = tmp_path / "librn32.so"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-shared", "-Xcompiler", "-fPIC", os.path.join(root, "tests", "gpu_helpers", "rn32.cu"),
                    "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    for seed in (3, 0x5EED):
        bad, first = C.c_ulonglong(0), C.c_ulonglong(0)
        assert lib.rn32_check(C.c_ulonglong(1 << 31), C.c_ulonglong(seed), C.byref(bad), C.byref(first)) == 0
        assert bad.value == 0, hex(first.value)


def test_markstein_division_matches_ieee(tmp_path):
    """The FP64 recheck divides through div_rn (three operations from RN(1/b));
    it must equal the IEEE quotient bit for bit, here on 2^30 operand pairs
    including all-ones significands, powers of two, squares, exact quotients
    and the fallback range."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = tmp_path / "libdivrn.so"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
                    "-shared", "-Xcompiler", "-fPIC", os.path.join(root, "tests", "gpu_helpers", "div_rn.cu"),
                    "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    for seed in (1, 0xABCDEF):
        bad = C.c_ulonglong(0)
        first = (C.c_double * 4)()
        assert lib.div_rn_check(C.c_ulonglong(1 << 30), C.c_ulonglong(seed), C.byref(bad), first) == 0
        assert bad.value == 0, list(first)
