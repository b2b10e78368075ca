"""CUDA graph mode of the simulation chain: identical statistics to plain
launches, graph updated in place across seeds, re-instantiated when the
batch shape changes."""
import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.config import factor_prior, make_config, synthetic_cells

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [abi.FP32, abi.FP64])
def test_graph_mode_identical_to_plain(built, prec):
    torch = pytest.importorskip("torch")
    from abc_inference_transcription_gb300.host import Context
    cells = synthetic_cells(n_per_pulse=20, n_per_chase=20, seed=3)
    with Context(make_config("hour", precision=prec), cells) as ctx:
        thetas, models = [], []
        for m in range(1, 6):
            th = np.zeros((60, 9))
            t = ctx.sample_prior(m, 60, 40 + m, factor_prior())
            t[:, 2] = np.minimum(t[:, 2], 1.0)     # moderate transcription: short trajectories
            th[:, :t.shape[1]] = t
            thetas.append(th)
            models.append(np.full(60, m, np.int32))
        theta = torch.from_numpy(np.concatenate(thetas)).cuda()
        mods = torch.from_numpy(np.concatenate(models)).cuda()
        K = ctx.K

        def run(P, seed):
            out = torch.empty((P, K), dtype=torch.float64, device="cuda")
            ctx.simulate_batch_device(mods.data_ptr(), theta.data_ptr(), 9, P, seed, out.data_ptr())
            ctx.synchronize()
            return out.cpu().numpy(), ctx.last_counters()

        plain = {(P, s): run(P, s) for P, s in ((300, 1), (300, 2), (120, 3))}
        ctx.set_graph(True)
        for (P, s), (want, cnt) in plain.items():
            got, gcnt = run(P, s)
            assert np.array_equal(got, want, equal_nan=True), (P, s)
            assert gcnt == cnt
        inst, upd = ctx.graph_counters()
        assert inst >= 1 and upd >= 1 and inst + upd == 3, (inst, upd)
