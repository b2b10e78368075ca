"""Learned pre-screen over libabcgpu.so (abc_surrogate_* entry points).

An ensemble of MLPs maps log-parameters to the means and log-variances of the
summary statistics.  It is trained on SSA output the pipeline itself
generates; screening keeps a prior draw for exact simulation when its
predicted expected error is within a gene's threshold plus a calibrated
margin for some gene, or when the ensemble members disagree.  The exact SSA
and the FP64-checked acceptance decide acceptance: the screen only decides which
draws are simulated.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import AbcError, ptr


class Surrogate:
    def __init__(self, in_dim: int, n_stats: int, ensemble: int = 4, seed: int = 1):
        self.lib = abi.load_library()
        h = C.c_void_p()
        st = self.lib.abc_surrogate_create(C.byref(h), in_dim, n_stats, ensemble, seed)
        if st != 0:
            raise AbcError(st, "abc_surrogate_create failed")
        self.h = h
        self.in_dim, self.K, self.members = in_dim, n_stats, ensemble
        self.n_params = self.lib.abc_surrogate_num_params(h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.abc_surrogate_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            msg = self.lib.abc_surrogate_last_error(self.h)
            raise AbcError(st, msg.decode() if msg else "")

    # -- training ------------------------------------------------------------
    def train(self, theta: np.ndarray, stats: np.ndarray, epochs: int = 20, batch: int = 4096,
              lr: float = 1e-3) -> np.ndarray:
        th = np.ascontiguousarray(theta, np.float64)
        st = np.ascontiguousarray(stats, np.float64)
        loss = np.zeros(epochs)
        self._check(self.lib.abc_surrogate_train(self.h, ptr(th), ptr(st), th.shape[0], epochs, batch, lr,
                                                 ptr(loss)))
        return loss

    def gradients(self, theta: np.ndarray, stats: np.ndarray):
        th = np.ascontiguousarray(theta, np.float64)
        st = np.ascontiguousarray(stats, np.float64)
        loss = np.zeros(self.members)
        g = np.zeros(self.members * self.n_params, np.float32)
        self._check(self.lib.abc_surrogate_gradients(self.h, ptr(th), ptr(st), th.shape[0], ptr(loss),
                                                     ptr(g, C.c_float)))
        return loss, g.reshape(self.members, self.n_params)

    def params(self) -> np.ndarray:
        p = np.zeros(self.members * self.n_params, np.float32)
        self._check(self.lib.abc_surrogate_get_params(self.h, ptr(p, C.c_float)))
        return p.reshape(self.members, self.n_params)

    def set_params(self, p: np.ndarray) -> None:
        q = np.ascontiguousarray(p, np.float32).reshape(-1)
        self._check(self.lib.abc_surrogate_set_params(self.h, ptr(q, C.c_float)))

    def norm(self):
        xm, xs = np.zeros(self.in_dim), np.zeros(self.in_dim)
        ym, ys = np.zeros(self.K), np.zeros(self.K)
        self._check(self.lib.abc_surrogate_get_norm(self.h, ptr(xm), ptr(xs), ptr(ym), ptr(ys)))
        return xm, xs, ym, ys

    def set_norm(self, xm, xs, ym, ys) -> None:
        a = [np.ascontiguousarray(v, np.float64) for v in (xm, xs, ym, ys)]
        self._check(self.lib.abc_surrogate_set_norm(self.h, *[ptr(v) for v in a]))

    # -- inference -------------------------------------------------------------
    def predict(self, theta: np.ndarray):
        th = np.ascontiguousarray(theta, np.float64)
        n = th.shape[0]
        mean, var, dis = np.zeros((n, self.K)), np.zeros((n, self.K)), np.zeros(n)
        self._check(self.lib.abc_surrogate_predict(self.h, ptr(th), n, ptr(mean), ptr(var), ptr(dis)))
        return mean, var, dis

    def screen_device(self, d_theta: int, ld: int, n: int, data, se, thr, margin: float, disagree_max: float,
                      d_keep: int, err_out: np.ndarray | None = None, z: float = 2.0, mode: int = 0) -> int:
        """mode 0: per-statistic lower bound; mode 1: lower z-quantile (normal
        approximation) of the error's predictive distribution."""
        self._check(self.lib.abc_surrogate_set_screen_mode(self.h, int(mode)))
        d = np.ascontiguousarray(data, np.float64)
        e = np.ascontiguousarray(se, np.float64)
        t = np.ascontiguousarray(thr, np.float64)
        nk = C.c_int64()
        self._check(self.lib.abc_surrogate_screen_device(self.h, C.c_void_p(d_theta), ld, n, ptr(d), ptr(e),
                                                         d.shape[0], ptr(t), float(margin), float(z),
                                                         float(disagree_max),
                                                         C.c_void_p(d_keep), C.byref(nk), ptr(err_out)))
        return nk.value


    def compact_device(self, d_keep: int, d_theta: int, ld: int, n: int, d_theta_out: int, d_idx_out: int = 0) -> int:
        nk = C.c_int64()
        self._check(self.lib.abc_surrogate_compact_device(self.h, C.c_void_p(d_keep), C.c_void_p(d_theta), ld, n,
                                                          C.c_void_p(d_theta_out or None),
                                                          C.c_void_p(d_idx_out or None), C.byref(nk)))
        return nk.value


def calibrate_margin(pred_err: np.ndarray, exact_err: np.ndarray, thr: np.ndarray, quantile: float = 0.99) -> float:
    """Additive margin m such that a fraction `quantile` of the truly accepted
    (p, g) pairs of a calibration set (exact_err <= thr) have pred_err <= thr + m."""
    acc = exact_err <= thr[None, :]
    if not acc.any():
        return 0.0
    short = (pred_err - thr[None, :])[acc]
    return float(max(0.0, np.quantile(short, quantile)))


def calibrate_factor(pred_err: np.ndarray, exact_err: np.ndarray, thr: np.ndarray, quantile: float = 0.99) -> float:
    """Multiplicative margin f (screen keeps pred_err <= f thr) such that a
    fraction `quantile` of the truly accepted pairs of a calibration set pass
    (f < 1 when the screen statistic is conservative).  Predicted errors are
    heavy-tailed, so a ratio calibrates better than a difference."""
    acc = exact_err <= thr[None, :]
    if not acc.any():
        return 1.0
    ratio = (pred_err / np.maximum(thr[None, :], 1e-12))[acc]
    ratio = np.where(np.isfinite(ratio), ratio, np.inf)
    return float(max(0.05, np.quantile(ratio, quantile)))


def false_rejection_rate(keep: np.ndarray, exact_err: np.ndarray, thr: np.ndarray) -> tuple[float, int]:
    """Fraction of truly accepted (p, g) pairs whose particle the screen dropped."""
    acc = exact_err <= thr[None, :]
    n = int(acc.sum())
    if n == 0:
        return 0.0, 0
    lost = int((acc & ~keep.astype(bool)[:, None]).sum())
    return lost / n, n
