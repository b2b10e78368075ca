"""GPU parity tests: every call goes through the C ABI (libabcgpu.so) and is
compared with the FP64 CPU oracle on the same seeded inputs.

Tolerances: integer outputs (molecule counts, captured counts, event counts,
event-sequence hashes, accepted particle sets) are compared bit for bit; the
FP64-mode statistics and FP64 errors are compared bit for bit as well (same
integer moment sums, same operation order, no FMA contraction on either
side).  The FP32 production mode is compared statistically (Monte Carlo
standard errors and two-sample KS tests)."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.config import (REF_FAMILIES, factor_prior, make_config, minute_prior,
                                                       reference_prior, synthetic_cells)
from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Ctx(built):
    from abc_inference_transcription_gb300.host import Context
    return Context


def moderate(theta, model, S=5):
    """Clamp a reference-prior draw to rates that keep trajectories short."""
    th = theta.copy()
    ncol = th.shape[1]
    th[:, :ncol - 1] = np.minimum(th[:, :ncol - 1], 1.3)
    return th


# --------------------------------------------------------------------------
# random numbers
# --------------------------------------------------------------------------
def test_philox_matches_curand(orc, tmp_path):
    so = tmp_path / "libcurandkat.so"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler", "-fPIC",
                    os.path.join(ROOT, "tests", "gpu_helpers", "curand_philox.cu"), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    for seed, sub in [(0, 0), (0x123456789ABCDEF0, 7), (42, 2 ** 40 + 3)]:
        out = np.zeros((8, 4), np.uint32)
        assert lib.curand_philox_words(C.c_ulonglong(seed), C.c_ulonglong(sub), 8,
                                       out.ctypes.data_as(C.POINTER(C.c_uint32))) == 0
        for i in range(8):
            ctr = [i, 0, sub & 0xFFFFFFFF, sub >> 32]
            key = [seed & 0xFFFFFFFF, seed >> 32]
            assert [int(x) for x in orc.philox(ctr, key)] == [int(x) for x in out[i]]


@pytest.mark.parametrize("unit,splicing,scol,prior", [("hour", False, False, "ref"), ("hour", False, False, "factor"),
                                                     ("min", True, True, "min")])
def test_prior_bit_exact(Ctx, orc, unit, splicing, scol, prior):
    cfg = make_config(unit, precision=abi.FP64, splicing=splicing, scaling_column=scol)
    pr = {"ref": reference_prior, "factor": factor_prior, "min": minute_prior}[prior]()
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=1)
    with Ctx(cfg, cells) as ctx:
        for model in range(1, 6):
            got = ctx.sample_prior(model, 1000, 77, pr, offset=12345)
            want = orc.sample_prior(cfg, model, 1000, 77, pr, offset=12345)
            assert np.array_equal(got, want)


# --------------------------------------------------------------------------
# SSA, FP64 oracle mode: bit-exact
# --------------------------------------------------------------------------
@pytest.mark.parametrize("model", [1, 2, 3, 4, 5])
def test_ssa_fp64_bit_exact(Ctx, orc, model):
    cfg = make_config("hour", precision=abi.FP64)
    cells = synthetic_cells(n_per_pulse=12, n_per_chase=10, seed=model)
    theta = moderate(orc.sample_prior(cfg, model, 8, 100 + model, reference_prior()), model)
    with Ctx(cfg, cells) as ctx:
        got = ctx.simulate_cells(model, theta, seed=9)
        ev, rej = ctx.last_counters()
    ref = orc.simulate(cfg, cells, model, theta, seed=9)
    assert ref["status"] == 0
    for key in ("counts", "captured", "events", "hash"):
        assert np.array_equal(got[key], ref[key]), key
    assert np.array_equal(got["stats"], ref["stats"], equal_nan=True)
    assert ev == int(ref["events"].sum()) and rej == ref["rejections"]


def test_ssa_fp64_bit_exact_splicing_scaling_minutes(Ctx, orc):
    cfg = make_config("min", precision=abi.FP64, splicing=True, scaling_column=True)
    cells = synthetic_cells(n_per_pulse=12, n_per_chase=10, seed=3)
    theta = orc.sample_prior(cfg, 4, 6, 5, minute_prior())
    theta[:, :9] = np.minimum(theta[:, :9], -0.3)  # per-minute rates below 0.5
    with Ctx(cfg, cells) as ctx:
        got = ctx.simulate_cells(4, theta, seed=21)
    ref = orc.simulate(cfg, cells, 4, theta, seed=21)
    assert ref["status"] == 0
    for key in ("counts", "captured", "events", "hash"):
        assert np.array_equal(got[key], ref[key]), key
    assert np.array_equal(got["stats"], ref["stats"], equal_nan=True)


def test_ssa_particle_offset_sharding(Ctx, orc):
    """Shards of a particle batch (particle_offset) reproduce the single run:
    the host-side sharding used for several GPUs needs no data exchange."""
    cfg = make_config("hour", precision=abi.FP64)
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=4)
    theta = moderate(orc.sample_prior(cfg, 1, 10, 3, reference_prior()), 1)
    with Ctx(cfg, cells) as ctx:
        full = ctx.simulate(1, theta, seed=5)
        a = ctx.simulate(1, theta[:4], seed=5, offset=0)
        b = ctx.simulate(1, theta[4:], seed=5, offset=4)
    assert np.array_equal(np.vstack([a, b]), full, equal_nan=True)


def test_event_cap_is_a_status_not_a_fault(Ctx):
    cfg = make_config("hour", precision=abi.FP64, event_cap=10)
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=2)
    th = np.log10([[5.0, 1.0, 50.0, 1.0, 0.7]])
    with Ctx(cfg, cells) as ctx:
        with pytest.raises(abi.AbcError) as ei:
            ctx.simulate(1, th, seed=1)
        assert ei.value.status == abi.ERR_EVENT_CAP
        # the context stays usable
        cfg_ok = make_config("hour", precision=abi.FP64)
    with Ctx(cfg_ok, cells) as ctx:
        assert np.isfinite(ctx.simulate(1, np.log10([[0.5, 1.0, 5.0, 0.5, 0.7]]), seed=1)[:, :20]).all()


def test_invalid_arguments_are_errors(Ctx):
    cells = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=2)
    with Ctx(make_config("hour"), None) as ctx:
        with pytest.raises(abi.AbcError) as ei:
            ctx.simulate(1, np.zeros((1, 5)), seed=1)
        assert ei.value.status == abi.ERR_STATE
        bad = synthetic_cells(n_per_pulse=10, n_per_chase=10, seed=2)
        bad.beta = bad.beta.copy()
        bad.beta[0] = 1.5
        with pytest.raises(abi.AbcError):
            ctx.set_cells(bad)
        ctx.set_cells(cells)
        with pytest.raises(abi.AbcError) as ei:
            ctx.simulate(1, np.full((1, 5), 400.0), seed=1)  # 10^400 overflows
        assert ei.value.status == abi.ERR_NONFINITE


# --------------------------------------------------------------------------
# SSA, FP32 production mode: statistical agreement
# --------------------------------------------------------------------------
def _ks_2samp_p(a, b):
    from scipy.stats import ks_2samp
    return ks_2samp(a, b).pvalue


@pytest.mark.parametrize("model,theta", [(1, [0.5, 1.0, 20.0, 0.1, 0.7]),
                                         (3, [0.1, 0.1, 30.0, 0.1, 0.1, 1.0, 15.0, 0.1, 0.7]),
                                         (5, [2.0, 1.0, 85.0, 2.0, 3.0, 1.0, 1.0, 1.5, 0.7])])
def test_ssa_fp32_matches_moment_ode_and_fp64(Ctx, orc, model, theta):
    """FP32 production counts vs the moment ODE (expected values, within 4
    Monte Carlo standard errors per group) and vs the FP64 mode (two-sample
    KS per group, Bonferroni over 55 groups).  Example genes of
    scripts/model_realisation.jl:294-315."""
    th = np.log10(np.array([theta]))
    cells = synthetic_cells(n_per_pulse=1500, n_per_chase=1500, seed=11)
    out = {}
    for prec in (abi.FP32, abi.FP64):
        with Ctx(make_config("hour", precision=prec), cells) as ctx:
            out[prec] = ctx.simulate_cells(model, th, seed=31 + prec)["counts"][0]
    ode = orc.moment_model(make_config("hour"), model, th[0], np.array([0, 0.5, 0, 0, 0, 0, 0, 0, 0.0]))["moments"]
    zs, ps = [], []
    for j in range(11):
        for a in range(5):
            sel = (cells.cond == j) & (cells.age == a)
            n = sel.sum()
            for col, (mi, vi) in enumerate(((0, 2), (1, 4))):
                x = out[abi.FP32][sel, col].astype(float)
                zs.append((x.mean() - ode[j, a, mi]) / math.sqrt(max(ode[j, a, vi], 1e-9) / n))
                ps.append(_ks_2samp_p(x, out[abi.FP64][sel, col].astype(float)))
    zs = np.array(zs)
    assert np.abs(zs).max() < 4.5 and abs(zs.mean()) < 0.6, zs
    assert min(ps) > 1e-3 / len(ps) or min(ps) == 1.0, min(ps)


# --------------------------------------------------------------------------
# distance + acceptance
# --------------------------------------------------------------------------
def _ref_data():
    z = np.load(f"{GOLDEN}/summary_stats.npz")
    return z["data"], z["se"]


def _stats_near(data, P, rng, spread=0.25):
    src = data[rng.integers(0, data.shape[0], P)]
    return src * rng.lognormal(0.0, spread, src.shape)


def test_errors_bit_exact_reference_data(Ctx, orc):
    data, se = _ref_data()
    data, se = data[:128], se[:128]
    rng = np.random.default_rng(3)
    stats = _stats_near(data, 300, rng)
    stats[5, 7] = np.nan          # NaN statistic stays NaN
    stats[6, :] = 0.0
    d2, s2 = data.copy(), se.copy()
    d2[3, 4] = 0.0
    s2[3, 4] = 0.0                # eps = 1e-4 branch
    with Ctx(make_config("hour"), None) as ctx:
        got = ctx.errors(d2, s2, stats, REF_FAMILIES)
    want = orc.errors(d2, s2, stats, REF_FAMILIES)
    assert np.array_equal(got, want, equal_nan=True)
    assert np.isnan(got[5]).all()


@pytest.mark.parametrize("eps", [4.8, 0.6, 0.0, 11.0])
def test_select_eps_identical_to_oracle(Ctx, orc, eps):
    data, se = _ref_data()
    rng = np.random.default_rng(7)
    stats = _stats_near(data, 4000, rng, spread=0.3)
    stats[17] = np.nan
    with Ctx(make_config("hour"), None) as ctx:
        off, idx, err = ctx.select(data, se, stats, 0, eps, REF_FAMILIES)
    roff, ridx = orc.accept(orc.errors(data, se, stats, REF_FAMILIES), 0, eps)
    assert np.array_equal(off, roff)
    assert np.array_equal(idx, ridx)


@pytest.mark.parametrize("q,K", [(0.01, 72), (0.001, 53), (0.2, 16)])
def test_select_topq_identical_to_oracle(Ctx, orc, q, K):
    rng = np.random.default_rng(int(q * 1000) + K)
    G, P = 40, 20000
    base = np.abs(rng.normal(5.0, 3.0, (300, K))) + 0.1
    stats = base[rng.integers(0, 300, P)] * rng.lognormal(0, 0.2, (P, K))
    data = base[rng.integers(0, 300, G)] * rng.lognormal(0, 0.05, (G, K))
    se = 0.1 * np.abs(data) * rng.lognormal(0, 0.5, (G, K))
    stats[100:110] = stats[99]    # exact ties, broken by index
    stats[200, 3] = np.nan
    with Ctx(make_config("hour"), None) as ctx:
        off, idx, err = ctx.select(data, se, stats, 1, q, None)
    roff, ridx = orc.accept(orc.errors(data, se, stats, None), 1, q)
    assert np.array_equal(off, roff)
    assert np.array_equal(idx, ridx)


def test_accepted_particles_reference_format(Ctx, orc):
    from abc_inference_transcription_gb300.host import accepted_particles
    data, se = _ref_data()
    data, se = data[:32], se[:32]
    rng = np.random.default_rng(9)
    stats = _stats_near(data, 500, rng, spread=0.6)
    with Ctx(make_config("hour"), None) as ctx:
        lists = accepted_particles(ctx, data, se, stats, 4.8)
    roff, ridx = orc.accept(orc.errors(data, se, stats, REF_FAMILIES), 0, 4.8)
    for g in range(32):
        want = ridx[roff[g]:roff[g + 1]].tolist() or [0]
        assert lists[g] == want


def test_select_per_gene_thresholds_and_device_stats(Ctx, orc):
    """Per-gene thresholds (the screened pipeline's acceptance) and device-resident
    statistics give the oracle's accepted sets."""
    torch = pytest.importorskip("torch")
    data, se = _ref_data()
    data, se = data[:48], se[:48]
    rng = np.random.default_rng(12)
    stats = _stats_near(data, 3000, rng, spread=0.3)
    err = orc.errors(data, se, stats, REF_FAMILIES)
    thr = np.quantile(err, 0.03, axis=0)
    thr[5] = -1.0  # a gene with no acceptance
    want_off, want_idx = [0], []
    for g in range(48):
        o, i = orc.accept(err[:, g:g + 1], 0, thr[g])
        want_idx.append(i)
        want_off.append(want_off[-1] + i.shape[0])
    want_idx = np.concatenate(want_idx)
    with Ctx(make_config("hour"), None) as ctx:
        off, idx, e = ctx.select_thr(data, se, stats, thr, REF_FAMILIES)
        assert np.array_equal(off, want_off) and np.array_equal(idx, want_idx)
        d_stats = torch.from_numpy(np.ascontiguousarray(stats)).cuda()
        off2, idx2, _ = ctx.select_device(data, se, d_stats.data_ptr(), stats.shape[0], 2, thr=thr,
                                          families=REF_FAMILIES)
        assert np.array_equal(off2, want_off) and np.array_equal(idx2, want_idx)
        off3, idx3, _ = ctx.select_device(data, se, d_stats.data_ptr(), stats.shape[0], 1, 0.01,
                                          families=REF_FAMILIES)
        roff, ridx = orc.accept(err, 1, 0.01)
        assert np.array_equal(off3, roff) and np.array_equal(idx3, ridx)
