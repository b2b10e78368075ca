"""The reference's on-disk text files (scripts/accepted_particles.jl,
abc_simulation.jl, compute_errors.jl, model_probs.jl, posterior_kinetics.jl):
tab-delimited rows, particle lists with a "0" line for genes without
particles, floats that read back exactly.  Host code only."""
import numpy as np
import pytest

from abc_inference_transcription_gb300.config import make_config


@pytest.fixture(scope="module")
def F(built):
    from abc_inference_transcription_gb300 import formats
    return formats


def test_float_spelling_and_round_trip(F):
    assert [F.format_double(x) for x in (1.0, 0.1, 1e-5, 123456.0, 1e16, -0.0, np.nan, np.inf, -np.inf)] == \
        ["1.0", "0.1", "1.0e-5", "123456.0", "1.0e16", "-0.0", "NaN", "Inf", "-Inf"]
    # Julia switches to exponent notation outside 1e-4 <= |x| < 1e6
    assert [F.format_double(x) for x in (1e5, 1e-4, 2.5e-4, 999999.0, 1e6, 1234567.0, -0.00012, 123456.7, 0.5e-4,
                                         3.0e-300, 12.5)] == \
        ["100000.0", "0.0001", "0.00025", "999999.0", "1.0e6", "1.234567e6", "-0.00012", "123456.7", "5.0e-5",
         "3.0e-300", "12.5"]
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.normal(size=2000) * 10.0 ** rng.integers(-300, 300, 2000),
                         rng.integers(-10 ** 6, 10 ** 6, 500).astype(float), [5e-324, 1.7976931348623157e308]])
    for x in xs:
        assert float(F.format_double(x)) == x


def test_particles_file_layout_and_read_back(F, tmp_path):
    off = np.array([0, 3, 3, 4, 4, 6], np.int64)          # genes 2 and 4 without particles
    idx = np.array([17, 3, 250000, 1, 42, 9], np.int64)
    p = tmp_path / "particles_const.txt"
    F.write_particles(p, off, idx)
    assert p.read_text() == "17\t3\t250000\n0\n1\n0\n42\t9\n"
    # scripts/posterior_kinetics.jl:56-60 reads each line as parse.(Int64, split(line, "\t"))
    lines = [list(map(int, ln.split("\t"))) for ln in p.read_text().splitlines()]
    assert lines == [[17, 3, 250000], [0], [1], [0], [42, 9]]
    o2, i2 = F.read_particles(p)
    assert np.array_equal(o2, off) and np.array_equal(i2, idx)
    # appending, as the reference opens the file with "a" per gene
    F.write_particles(p, np.array([0, 1], np.int64), np.array([7], np.int64), append=True)
    o3, i3 = F.read_particles(p)
    assert o3.shape[0] == 7 and i3[-1] == 7
    F.write_particles(tmp_path / "empty.txt", np.zeros(3, np.int64), np.zeros(0, np.int64))
    assert (tmp_path / "empty.txt").read_text() == "0\n0\n"


def test_simulation_files_round_trip(F, tmp_path):
    cfg = make_config("hour")
    A, J = cfg.n_ages, cfg.n_conds
    rng = np.random.default_rng(2)
    P = 7
    theta = rng.uniform(-3, 3, (P, 5))
    stats = rng.lognormal(0, 2, (P, 4 * A + 3 * J))
    stats[2, 4 * A + J] = np.nan                              # a correlation of a silent particle
    paths = F.write_simulation(tmp_path, "const", 3, theta, stats, A, J, append=False)
    assert [p.split("/")[-1] for p in paths] == ["sets_const_3.txt", "s_pulse_const_3.txt", "s_chase_const_3.txt",
                                                 "s_ratios_const_3.txt", "s_mean_corr_const_3.txt",
                                                 "s_corr_mean_const_3.txt"]
    back = F.read_simulation_stats(tmp_path, "const", 3, A, J)
    assert np.array_equal(back, stats, equal_nan=True)
    assert np.array_equal(F.read_matrix(paths[0]), theta)
    # s_pulse: two rows per particle (compute_errors.jl:1-15 takes odd rows as means, even rows as FF)
    pulse = F.read_matrix(paths[1])
    assert pulse.shape == (2 * P, A)
    assert np.array_equal(pulse[0], stats[0, :A]) and np.array_equal(pulse[1], stats[0, A:2 * A])
    # appending a second shard extends every file
    F.write_simulation(tmp_path, "const", 3, theta, stats, A, J, append=True)
    assert F.read_simulation_stats(tmp_path, "const", 3, A, J).shape[0] == 2 * P


def test_error_and_estimate_files(F, tmp_path):
    rng = np.random.default_rng(3)
    err = np.minimum(rng.exponential(3.0, (5, 9)), 10.0)
    F.write_matrix(tmp_path / "error_kon.txt", err[:2])
    F.write_matrix(tmp_path / "error_kon.txt", err[2:], append=True)
    assert np.array_equal(F.read_matrix(tmp_path / "error_kon.txt"), err)
    p, lb, ub = rng.random((4, 3)), rng.random((4, 3)), rng.random((4, 3))
    F.write_model_probs(tmp_path / "ms", p, lb, ub, append=False)
    assert np.array_equal(F.read_matrix(tmp_path / "ms" / "l_bound.txt"), lb)
    summ = {k: rng.normal(size=(6, 5)) for k in ("map", "mean", "lower", "upper")}
    F.write_posterior_estimates(tmp_path / "pe", "alpha", summ)
    assert np.array_equal(F.read_matrix(tmp_path / "pe" / "ci_ubs_alpha.txt"), summ["upper"])


def test_bad_path_is_an_io_error(F, tmp_path):
    with pytest.raises(OSError, match="ABC_ERR_IO"):
        F.write_matrix(tmp_path / "no_such_dir" / "x.txt", np.zeros((1, 1)))
    with pytest.raises(OSError, match="ABC_ERR_IO"):
        F.read_particles(tmp_path / "missing.txt")


@pytest.mark.gpu
def test_selection_lists_to_particles_file(F, orc, tmp_path):
    """An acceptance on the GPU written as particles_<model>.txt reads back as
    the oracle's lists."""
    from abc_inference_transcription_gb300.host import Context
    rng = np.random.default_rng(5)
    base = np.abs(rng.normal(5.0, 3.0, (50, 16))) + 0.1
    stats = base[rng.integers(0, 50, 3000)] * rng.lognormal(0, 0.2, (3000, 16))
    data = base[rng.integers(0, 50, 12)] * rng.lognormal(0, 0.05, (12, 16))
    se = 0.1 * np.abs(data) * rng.lognormal(0, 0.5, data.shape)
    with Context(make_config("hour"), None) as ctx:
        off, idx, _ = ctx.select(data, se, stats, 0, 0.02, None)
    roff, ridx = orc.accept(orc.errors(data, se, stats, None), 0, 0.02)
    F.write_particles(tmp_path / "particles_const.txt", off, idx)
    o2, i2 = F.read_particles(tmp_path / "particles_const.txt")
    assert np.array_equal(o2, roff) and np.array_equal(i2, ridx)

