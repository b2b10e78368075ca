"""Plain and surrogate-screened ABC runs on one GPU.

Plain ABC (the reference's workflow, scripts/abc_simulation.jl:88-97 then
scripts/compute_errors.jl and scripts/accepted_particles.jl): draw particles of
the five models from the prior, simulate every draw exactly, accept per gene.

Screened ABC: a surrogate ensemble trained on the pipeline's own exact
simulations predicts each draw's statistics; only draws whose predicted
expected error is within a calibrated factor of a gene's threshold (or whose
ensemble disagrees) are simulated exactly and go through the exact,
FP64-checked acceptance.  Draws, statistics and flags stay in device memory;
torch tensors serve only as device buffers and for row gathers.
"""
from __future__ import annotations

import time

import numpy as np

from .config import factor_prior, make_config, synthetic_cells
from .host import Context
from .surrogate import Surrogate, calibrate_factor

LD = 9         # theta row stride of the five-model batch (largest npar)
IN_DIM = 14    # surrogate input: padded theta (9) + one-hot model (5)


def _torch():
    import torch
    return torch


def draw(ctx: Context, per_model: int, seed: int, prior, offset: int = 0):
    """Prior draws of the five models on the device: theta [5 per_model, 9] and model ids."""
    torch = _torch()
    P = 5 * per_model
    theta = torch.zeros((P, LD), dtype=torch.float64, device="cuda")
    models = torch.empty(P, dtype=torch.int32, device="cuda")
    for m in range(1, 6):
        npar = ctx.num_params(m)
        tmp = torch.empty((per_model, npar), dtype=torch.float64, device="cuda")
        ctx.sample_prior_device(m, per_model, seed + m, prior, tmp.data_ptr(), offset=offset + (m - 1) * per_model)
        torch.cuda.synchronize()
        theta[(m - 1) * per_model:m * per_model, :npar] = tmp
        models[(m - 1) * per_model:m * per_model] = m
    return theta, models


def surrogate_input(theta, models):
    torch = _torch()
    onehot = torch.nn.functional.one_hot((models - 1).long(), 5).to(torch.float64)
    return torch.cat([theta, onehot], dim=1).contiguous()


def simulate(ctx: Context, theta, models, seed: int, offset: int = 0):
    torch = _torch()
    P = theta.shape[0]
    stats = torch.empty((P, ctx.K), dtype=torch.float64, device="cuda")
    if P:
        ctx.simulate_batch_device(models.data_ptr(), theta.data_ptr(), LD, P, seed, stats.data_ptr(), offset=offset)
        ctx.synchronize()
    return stats


def make_genes(stats: np.ndarray, G: int, rng: np.random.Generator):
    """Synthetic genes: statistics of simulated particles plus 5 % Gaussian noise;
    standard errors log-normal (sigma 0.5) around 10 % of the statistic."""
    ok = np.flatnonzero(np.isfinite(stats).all(axis=1))
    src = stats[rng.choice(ok, size=G, replace=ok.shape[0] < G)]
    data = src + rng.normal(0.0, 1.0, src.shape) * 0.05 * np.abs(src)
    se = 0.1 * np.abs(data) * rng.lognormal(0.0, 0.5, data.shape)
    return data, se


CLIP = 10.0  # errors are clipped at 10 (scripts/compute_errors.jl:62-64)


def thresholds_from_lists(off: np.ndarray, err: np.ndarray) -> np.ndarray:
    """Per-gene threshold = largest accepted error of a top-k selection that is
    below the clip value.  A clipped error (10) says only "far away": when the
    k-th error of a gene is the clip, its top-k would be an arbitrary set of
    tied particles, so such a gene accepts only its unclipped particles (and
    none when it has none; threshold -1)."""
    G = off.shape[0] - 1
    thr = np.full(G, -1.0)
    for g in range(G):
        e = err[off[g]:off[g + 1]]
        e = e[e < CLIP]
        if e.shape[0]:
            thr[g] = e[-1]
    return thr


def _screen_x(thr: np.ndarray, factor: float) -> np.ndarray:
    """Screen thresholds f thr_g; genes without a threshold (thr < 0) keep no draw."""
    return np.where(thr >= 0, thr * factor, -1e30)


def _screened(ctx, sg, data, se, thr, factor, dmax, per_model_s, prior, seed, offset, z=2.0, mode=0,
              chunk_per_model=2_000_000):
    """Screened ABC: draw, screen, compact, simulate the survivors, accept with
    the per-gene thresholds.  Draws are made and screened in chunks of
    chunk_per_model per model (device memory stays bounded at any draw
    count); the survivors of all chunks are simulated together.  Returns
    (accepted pairs, simulated draws, draws, times, accepted lists)."""
    torch = _torch()
    t0 = time.perf_counter()
    kept_th, kept_m = [], []
    n_draw = 0
    for c0 in range(0, per_model_s, chunk_per_model):
        pm = min(chunk_per_model, per_model_s - c0)
        th_s, m_s = draw(ctx, pm, seed + 1000 * (c0 // chunk_per_model), prior, offset=offset + 5 * c0)
        x_s = surrogate_input(th_s, m_s)
        keep = torch.empty(th_s.shape[0], dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()  # the screen runs on the surrogate's own stream
        n_keep = sg.screen_device(x_s.data_ptr(), IN_DIM, th_s.shape[0], data, se, _screen_x(thr, factor), 0.0,
                                  dmax, keep.data_ptr(), z=z, mode=mode)
        sidx = torch.empty(max(n_keep, 1), dtype=torch.int64, device="cuda")
        sg.compact_device(keep.data_ptr(), 0, LD, th_s.shape[0], 0, sidx.data_ptr())
        sel = sidx[:n_keep]
        kept_th.append(th_s[sel].contiguous())
        kept_m.append(m_s[sel].contiguous())
        n_draw += int(th_s.shape[0])
        del th_s, m_s, x_s, keep, sidx
    th_k = torch.cat(kept_th).contiguous()
    m_k = torch.cat(kept_m).contiguous()
    n_keep = int(th_k.shape[0])
    torch.cuda.synchronize()
    t_screen = time.perf_counter() - t0
    st_k = simulate(ctx, th_k, m_k, seed + 7, offset=offset)
    t_sim = time.perf_counter() - t0 - t_screen
    acc = 0
    off_k = idx_k = None
    if n_keep:
        off_k, idx_k, _ = ctx.select_device(data, se, st_k.data_ptr(), n_keep, 2, thr=thr)
        acc = int(off_k[-1])
    torch.cuda.synchronize()
    t_all = time.perf_counter() - t0
    lists = None
    if n_keep:
        lists = (off_k, idx_k, th_k.cpu().numpy(), m_k.cpu().numpy())
    return acc, n_keep, n_draw, t_all, t_screen, t_sim, lists


def binomial_ci(k: int, n: int, level: float = 0.95) -> tuple[float, float]:
    """Clopper-Pearson interval of a proportion k / n."""
    from scipy.stats import beta
    if n <= 0:
        return 0.0, 1.0
    a = (1.0 - level) / 2.0
    lo = 0.0 if k == 0 else float(beta.ppf(a, k, n - k + 1))
    hi = 1.0 if k == n else float(beta.ppf(1.0 - a, k + 1, n - k))
    return lo, hi


def prediction_quality(sg, x: np.ndarray, y: np.ndarray) -> dict:
    """Held-out accuracy and calibration of the surrogate's predictive
    distribution: per statistic, the RMSE of the predicted mean relative to the
    statistic's spread, and the fraction of draws whose exact value lies within
    1 and 1.96 predictive standard deviations (68 % and 95 % when calibrated)."""
    mean, var, _ = sg.predict(x)
    ok = np.isfinite(y) & np.isfinite(mean) & (var > 0)
    z = np.where(ok, (y - mean) / np.sqrt(np.where(var > 0, var, 1.0)), np.nan)
    rel = []
    for k in range(y.shape[1]):
        o = ok[:, k]
        if o.sum() > 10 and np.std(y[o, k]) > 0:
            rel.append(np.sqrt(np.mean((y[o, k] - mean[o, k]) ** 2)) / np.std(y[o, k]))
    az = np.abs(z[ok])
    return {"draws": int(x.shape[0]), "rmse_over_sd_median": float(np.median(rel)) if rel else None,
            "rmse_over_sd_max": float(np.max(rel)) if rel else None,
            "coverage_1sd": float((az <= 1.0).mean()), "coverage_1.96sd": float((az <= 1.96).mean())}


def shared_rates(theta: np.ndarray, models: np.ndarray) -> np.ndarray:
    """log10 (k_on, k_off, alpha, gamma, lambda) of draws of any of the five
    models; a rate that varies over the age steps (k_on for model 3, alpha for
    4, gamma for 5) is represented by the mean of its per-step log values."""
    out = np.empty((theta.shape[0], 5))
    for m in range(1, 6):
        r = models == m
        t = theta[r]
        if m <= 2:
            out[r] = t[:, :5]
        elif m == 3:
            out[r] = np.column_stack([t[:, 0:5].mean(1), t[:, 5], t[:, 6], t[:, 7], t[:, 8]])
        elif m == 4:
            out[r] = np.column_stack([t[:, 0], t[:, 1], t[:, 2:7].mean(1), t[:, 7], t[:, 8]])
        else:
            out[r] = np.column_stack([t[:, 0], t[:, 1], t[:, 2], t[:, 3:8].mean(1), t[:, 8]])
    return out


def posterior_agreement(plain: list, screened: list, min_n: int = 10) -> dict:
    """Per gene and shared rate, z = (mean_screened - mean_plain) /
    sqrt(var_plain / n_plain + var_screened / n_screened) over the accepted
    particles of the two runs (genes with at least min_n accepted in both)."""
    zs = []
    for a, b in zip(plain, screened):
        if a.shape[0] < min_n or b.shape[0] < min_n:
            continue
        se = np.sqrt(a.var(0, ddof=1) / a.shape[0] + b.var(0, ddof=1) / b.shape[0])
        zs.append((b.mean(0) - a.mean(0)) / np.where(se > 0, se, np.inf))
    if not zs:
        return {"genes_compared": 0}
    z = np.abs(np.concatenate(zs))
    return {"genes_compared": len(zs), "abs_z_median": float(np.median(z)), "abs_z_max": float(z.max()),
            "fraction_abs_z_above_3": float((z > 3).mean())}


def run(genes=(2000,), per_model_train: int = 20000, per_model_plain: int = 2000, screen_factor: int = 10,
        q: float = 0.001, seed: int = 1, epochs: int = 40, ensemble: int = 4, cells=None, z: float = 2.0,
        screens=((0, 1.0), (0, 2.0)), recall: float = 0.995,
        disagree_q: float = 0.99, amortise_draws: float = 5e7, held_out_draws: int = 100_000,
        bound_genes=()) -> dict:
    """Plain vs screened ABC on the five-model batch for each gene-set size in
    `genes` (one surrogate, trained once on the pipeline's own simulations).
    `screens`: candidate screen statistics (mode, z), chosen per gene set on a
    calibration half of the plain draws; `recall`: fraction of the calibration
    half's accepted pairs the screen must keep; draws whose ensemble
    disagreement exceeds its `disagree_q` quantile are always simulated.

    Costs: the screened path needs its training data (exact SSA), the training
    and a plain run (thresholds and calibration) once; its accepted pairs per
    second are reported for the timed screened run alone, with those one-time
    costs added, and with them amortised over `amortise_draws` screened draws
    (the screened run's per-draw cost scaled to that count).  For every set
    size in `genes` and `bound_genes` the plain run also gives the fraction of
    draws accepted by at least one gene: no screen that keeps every accepted
    pair can simulate fewer draws, so its inverse bounds the gain (only this
    bound is computed for `bound_genes`)."""
    torch = _torch()
    cfg = make_config("hour")
    cells = cells if cells is not None else synthetic_cells(seed=1)
    prior = factor_prior()
    rng = np.random.default_rng(seed)
    out = {"q": q, "screen_factor": screen_factor, "recall_target": recall, "disagree_quantile": disagree_q,
           "runs": []}
    with Context(cfg, cells) as ctx:
        ctx.autotune(1, ctx.sample_prior(1, 500, seed + 99, prior)[:, :5], seed=3)
        # ---- training data: exact simulations the pipeline generates itself
        t0 = time.perf_counter()
        th_tr, m_tr = draw(ctx, per_model_train, seed * 1000 + 10, prior, offset=0)
        st_tr = simulate(ctx, th_tr, m_tr, seed + 1, offset=0)
        t_gen = time.perf_counter() - t0
        t0 = time.perf_counter()
        sg = Surrogate(IN_DIM, ctx.K, ensemble=ensemble, seed=seed + 5)
        loss = sg.train(surrogate_input(th_tr, m_tr).cpu().numpy(), st_tr.cpu().numpy(), epochs=epochs,
                        batch=2048, lr=2e-3)
        t_train = time.perf_counter() - t0
        out["surrogate"] = {"train_draws": int(th_tr.shape[0]), "epochs": epochs, "final_nll": float(loss[-1]),
                            "train_seconds": t_train, "data_generation_seconds": t_gen}
        # ---- plain ABC draws (simulated once, shared by the gene sets)
        off_plain = 5 * per_model_train
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        th_p, m_p = draw(ctx, per_model_plain, seed * 1000 + 20, prior, offset=off_plain)
        st_p = simulate(ctx, th_p, m_p, seed + 2, offset=off_plain)
        t_sim_plain = time.perf_counter() - t0
        st_host = st_p.cpu().numpy()
        th_host, m_host = th_p.cpu().numpy(), m_p.cpu().numpy()
        Pp = th_p.shape[0]
        x_p = surrogate_input(th_p, m_p)
        # the plain draws are held out from training: prediction error and calibration
        nh = min(Pp, held_out_draws)
        out["surrogate"]["held_out"] = prediction_quality(sg, x_p[:nh].cpu().numpy(), st_host[:nh])
        one_time = t_gen + t_train + t_sim_plain
        rows = rng.permutation(Pp)
        cal, hold = np.sort(rows[:Pp // 2]), np.sort(rows[Pp // 2:])
        x_cal = x_p[torch.from_numpy(cal).cuda()].contiguous()
        x_hold = x_p[torch.from_numpy(hold).cuda()].contiguous()
        _, _, dis = sg.predict(x_cal.cpu().numpy())
        dmax = float(np.quantile(dis, disagree_q))
        for gi, G in enumerate(genes):
            res = {"genes": G}
            data, se = make_genes(st_host, G, rng)
            t0 = time.perf_counter()
            off, idx, err = ctx.select_device(data, se, st_p.data_ptr(), Pp, 1, q)
            torch.cuda.synchronize()
            t_plain = t_sim_plain + (time.perf_counter() - t0)
            thr = thresholds_from_lists(off, err)
            below = err < CLIP
            gene_of = np.repeat(np.arange(G), np.diff(off))[below]
            p_of = idx[below] - 1
            acc_plain = int(below.sum())
            res["informative_genes"] = int((thr >= 0).sum())
            res["plain"] = {"draws": int(Pp), "accepted_pairs": acc_plain, "seconds": t_plain,
                            "accepted_per_s": acc_plain / t_plain}
            res["plain"]["fraction_draws_accepted_by_any_gene"] = np.unique(p_of).shape[0] / Pp
            res["gain_bound"] = Pp / max(np.unique(p_of).shape[0], 1)
            # calibration half: for each screen statistic (mode, z) the factor f
            # such that a fraction `recall` of the truly accepted pairs pass
            # (bound <= f thr), and the fraction of calibration draws it keeps;
            # the statistic keeping the fewest draws is used, and the held-out
            # half measures the false-rejection rate
            pos = np.full(Pp, -1, np.int64)
            pos[cal] = np.arange(cal.shape[0])
            in_cal = pos[p_of] >= 0
            informative = thr >= 0
            keep_cal = torch.zeros(cal.shape[0], dtype=torch.uint8, device="cuda")
            dis_keep = dis > dmax
            best = None
            tried = []
            for mode, zz in screens:
                pred = np.zeros((cal.shape[0], G))
                sg.screen_device(x_cal.data_ptr(), IN_DIM, cal.shape[0], data, se, thr, 0.0, 1e30,
                                 keep_cal.data_ptr(), err_out=pred, z=zz, mode=mode)
                ratios = pred[pos[p_of[in_cal]], gene_of[in_cal]] / np.maximum(thr[gene_of[in_cal]], 1e-12)
                ratios = np.where(np.isfinite(ratios), ratios, np.inf)
                if not ratios.size:
                    continue
                f = float(np.quantile(ratios, recall))
                if mode == 0:
                    f = max(0.05, f)
                kept_c = ((pred <= _screen_x(thr, f)[None, :]).any(axis=1) | dis_keep).mean()
                tried.append({"mode": mode, "z": zz, "factor": f, "kept_fraction": float(kept_c)})
                if best is None or kept_c < best[0]:
                    best = (float(kept_c), mode, zz, f)
            if best is None:
                best = (1.0, 0, z, 1.0)
            _, mode, zz, factor = best
            keep_h = torch.zeros(hold.shape[0], dtype=torch.uint8, device="cuda")
            sg.screen_device(x_hold.data_ptr(), IN_DIM, hold.shape[0], data, se, _screen_x(thr, factor), 0.0, dmax,
                             keep_h.data_ptr(), z=zz, mode=mode)
            kept = np.zeros(Pp, bool)
            kept[hold] = keep_h.cpu().numpy().astype(bool)
            n_hold = int((~in_cal).sum())
            frr = float((~kept[p_of[~in_cal]]).sum() / max(n_hold, 1))
            lost_h = int((~kept[p_of[~in_cal]]).sum())
            res["calibration"] = {"screen_mode": mode, "z": zz, "factor": factor,
                                  "calibration_kept_fraction": best[0], "recall_target": recall,
                                  "candidates": tried,
                                  "disagree_max": dmax, "calibration_pairs": int(in_cal.sum()),
                                  "held_out_pairs": n_hold, "false_rejection_rate": frr,
                                  "false_rejection_ci95": binomial_ci(lost_h, n_hold)}
            # warm-up of the whole screened path, then the timed run
            _screened(ctx, sg, data, se, thr, factor, dmax, 64, prior, seed * 1000 + 40 + gi, 10 ** 8, zz, mode)
            acc, n_sim, n_draw, t_all, t_scr, t_sim, lists = _screened(
                ctx, sg, data, se, thr, factor, dmax, per_model_plain * screen_factor, prior,
                seed * 1000 + 30 + gi, off_plain + Pp + gi * 5 * per_model_plain * screen_factor, zz, mode)
            res["screened"] = {"draws": n_draw, "simulated": n_sim, "simulated_fraction": n_sim / n_draw,
                               "accepted_pairs": acc, "seconds": t_all, "screen_seconds": t_scr,
                               "ssa_seconds": t_sim, "accepted_per_s": acc / t_all}
            scale = amortise_draws / max(n_draw, 1)
            res["screened"]["one_time_seconds"] = {"training_data_ssa": t_gen, "training": t_train,
                                                   "plain_calibration_run": t_sim_plain}
            res["screened"]["accepted_per_s_incl_training"] = acc / (t_all + one_time)
            res["screened"]["amortised"] = {"draws": amortise_draws,
                                            "accepted_per_s": acc * scale / (one_time + t_all * scale)}
            plain_rate = max(res["plain"]["accepted_per_s"], 1e-30)
            res["gain_accepted_per_s"] = res["screened"]["accepted_per_s"] / plain_rate
            res["gain_incl_training"] = res["screened"]["accepted_per_s_incl_training"] / plain_rate
            res["gain_amortised"] = res["screened"]["amortised"]["accepted_per_s"] / plain_rate
            # posterior means of the shared rates per gene, plain vs screened
            rates_p = shared_rates(th_host, m_host)
            post_p = [rates_p[p_of[gene_of == g]] for g in range(G)]
            post_s = [np.zeros((0, 5))] * G
            if lists is not None:
                off_k, idx_k, th_k, m_k = lists
                rates_k = shared_rates(th_k, m_k)
                post_s = [rates_k[idx_k[off_k[g]:off_k[g + 1]] - 1] for g in range(G)]
            res["posterior_agreement"] = posterior_agreement(post_p, post_s)
            res["_lost_held"] = (int((~kept[p_of[~in_cal]]).sum()), n_hold)
            out["runs"].append(res)
        out["bound_only"] = []
        for G in bound_genes:
            data, se = make_genes(st_host, G, rng)
            # genes in batches: a gene whose top-q threshold is the clip ties
            # every clipped draw, which bounds the candidates a batch may hold
            hit = np.zeros(Pp, bool)
            n_pairs = 0
            for g0 in range(0, G, 50):
                off, idx, err = ctx.select_device(data[g0:g0 + 50], se[g0:g0 + 50], st_p.data_ptr(), Pp, 1, q)
                below = err < CLIP
                hit[idx[below] - 1] = True
                n_pairs += int(below.sum())
            n_any = int(hit.sum())
            out["bound_only"].append({"genes": G, "plain_draws": int(Pp), "accepted_pairs": n_pairs,
                                      "fraction_draws_accepted_by_any_gene": n_any / Pp,
                                      "gain_bound": Pp / max(n_any, 1)})
        sg.close()
    # over the gene sets: median gain, false rejections pooled over held-out pairs
    lost = sum(r["_lost_held"][0] for r in out["runs"])
    held = sum(r["_lost_held"][1] for r in out["runs"])
    for r in out["runs"]:
        del r["_lost_held"]
    out["summary"] = {"gene_sets": len(out["runs"]),
                      "median_gain_accepted_per_s": float(np.median([r["gain_accepted_per_s"] for r in out["runs"]])),
                      "median_gain_incl_training": float(np.median([r["gain_incl_training"] for r in out["runs"]])),
                      "median_gain_amortised": float(np.median([r["gain_amortised"] for r in out["runs"]])),
                      "amortised_at_draws": amortise_draws,
                      "pooled_false_rejection_rate": lost / max(held, 1), "pooled_held_out_pairs": held,
                      "pooled_false_rejection_ci95": binomial_ci(lost, held),
                      "per_set_false_rejection": [(r["calibration"]["false_rejection_rate"],
                                                   r["calibration"]["false_rejection_ci95"]) for r in out["runs"]]}
    return out
