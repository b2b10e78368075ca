"""abc_simulate_noalloc: the simulation chain for callers that may not call
cudaMalloc while they run -- a runtime that reserved all device memory up
front in its own pool, or a latency-critical loop that must avoid the implicit
synchronisation of cudaMalloc/cudaFree -- and so cannot create a context.
The entry point keeps its scratch in a fixed device array inside the library.

Its statistics must equal those of the allocating entry point (abc_simulate)
on the same inputs: bit for bit, the tolerance of the other parity tests,
for two calls in a row (the shared array keeps the previous call's contents,
so the second call checks that everything that must start at zero is
cleared).  Collected last so that a stop-at-first-failure run has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.abi import ptr
from abc_inference_transcription_gb300.config import make_config, reference_prior, synthetic_cells

pytestmark = pytest.mark.gpu


def _noalloc(lib, cfg, model, cells, d_theta, P, seed, offset, d_stats, stream):
    return lib.abc_simulate_noalloc(
        C.byref(cfg), model, cells.n, ptr(cells.cond, C.c_int32), ptr(cells.age, C.c_int32), ptr(cells.beta),
        ptr(np.ascontiguousarray(cells.age_dist)), C.c_void_p(d_theta), P, seed, offset, C.c_void_p(d_stats),
        C.c_void_p(stream))


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
def test_noalloc_matches_allocating_entry_point(built, orc, precision):
    torch = pytest.importorskip("torch")
    from abc_inference_transcription_gb300.host import Context
    lib = abi.load_library()
    cfg = make_config("hour", precision=precision)
    cells = synthetic_cells(n_per_pulse=40, n_per_chase=30, seed=6)
    model = 3
    theta = orc.sample_prior(cfg, model, 24, 8, reference_prior())
    theta[:, :8] = np.minimum(theta[:, :8], 1.2)
    K = abi.nstats(cfg.n_ages, cfg.n_conds)
    stream = torch.cuda.current_stream().cuda_stream
    with Context(cfg, cells) as ctx:
        for call, (seed, offset, rows) in enumerate([(31, 0, slice(0, 24)), (32, 100, slice(4, 20))]):
            th = np.ascontiguousarray(theta[rows])
            want = ctx.simulate(model, th, seed=seed, offset=offset)
            d_theta = torch.from_numpy(th).cuda()
            d_stats = torch.full((th.shape[0], K), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            st = _noalloc(lib, cfg, model, cells, d_theta.data_ptr(), th.shape[0], seed, offset,
                          d_stats.data_ptr(), stream)
            assert st == 0, f"call {call}: status {st}"
            got = d_stats.cpu().numpy()
            assert np.array_equal(got, want, equal_nan=True), f"call {call} differs"


def test_noalloc_rejects_sizes_beyond_its_scratch(built):
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    cfg = make_config("hour")
    cells = synthetic_cells(seed=1)           # 2,000 cells
    P = 5000                                   # 5000 x 2000 x 8 B > 64 MiB
    d_theta = torch.zeros((P, 5), dtype=torch.float64, device="cuda")
    d_stats = torch.zeros((P, 53), dtype=torch.float64, device="cuda")
    st = _noalloc(lib, cfg, 1, cells, d_theta.data_ptr(), P, 1, 0, d_stats.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
    assert st == abi.ERR_INVALID
