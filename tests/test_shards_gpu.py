"""Particle shards through the library: each shard runs the fast
indices-only selection on its own particles, fetches FP64 errors for its
accepted pairs only (abc_accept_errors), and the host merge
(merge_accept_lists) reproduces the single-run selection -- indices, order and
FP64 errors bit for bit.  The shards run one after another on one GPU: they
exchange nothing, so this is the multi-GPU data path without the processes."""
import numpy as np
import pytest

from abc_inference_transcription_gb300.config import make_config
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H(built):
    from abc_inference_transcription_gb300 import host
    return host


@pytest.mark.parametrize("mode,eps_or_q", [(1, 0.01), (1, 0.003), (0, 4.8)])  # 4.8: accepted_particles.jl:10
def test_sharded_selection_merges_to_single_run(H, mode, eps_or_q):
    import torch
    z = np.load(f"{GOLDEN}/summary_stats.npz")
    data, se = z["data"][:48], z["se"][:48]
    rng = np.random.default_rng(5)
    P = 6000
    src = data[rng.integers(0, data.shape[0], P)]
    stats = src * rng.lognormal(0.0, 0.3, src.shape)
    d_stats = torch.from_numpy(stats).cuda()
    bounds = [0, 1700, 3900, P]  # uneven shards
    with H.Context(make_config("hour"), None) as ctx:
        off1, idx1, err1 = ctx.select_device(data, se, d_stats.data_ptr(), P, mode, eps_or_q, errors=True)
        parts = []
        for a, b in zip(bounds[:-1], bounds[1:]):
            parts.append(H.shard_select(ctx, data, se, d_stats[a:b].data_ptr(), b - a, a, mode, eps_or_q, P))
    off2, idx2, err2 = H.merge_accept_lists(parts, mode, eps_or_q, P)
    assert off1[-1] > 0
    assert np.array_equal(off1, off2) and np.array_equal(idx1, idx2)
    assert np.array_equal(err1, err2)
