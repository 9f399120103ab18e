"""Ensemble comparison of long runs (test infrastructure).

Long DPM runs are chaotic: trajectories that differ only by float rounding
drift apart, so a GPU run and the oracle's run of the same seed are compared
through statistics over seeds, not state by state.  For each observable the
runs are paired by seed, d_i = gpu_i - oracle_i, and the check is

    |mean(d)| <= 4 * sd(d) / sqrt(n) + 1e-3 * |mean(oracle)|

Four standard errors of the paired mean: with n = 16 seeds the t-statistic
has 15 degrees of freedom and |t| > 4 has two-sided probability about 0.001
when both sides sample the same dynamics.  The relative floor of 1e-3 covers
runs that stay close (a standard error near zero) but differ by the FP32
evaluation of the reference's double sub-expressions.  The unpaired interval
(4 standard errors of the difference of two independent means) is reported
beside it.
"""
from __future__ import annotations

import numpy as np

Z = 4.0
REL_FLOOR = 1e-3


def compare_ensembles(gpu: dict, oracle: dict) -> dict:
    out = {"ok": True}
    for k in oracle:
        x = np.asarray(gpu[k], np.float64)
        y = np.asarray(oracle[k], np.float64)
        assert x.shape == y.shape and x.size >= 2
        n = x.size
        d = x - y
        se_pair = float(np.std(d, ddof=1) / np.sqrt(n))
        se_unpaired = float(np.sqrt(np.var(x, ddof=1) / n + np.var(y, ddof=1) / n))
        tol = Z * se_pair + REL_FLOOR * abs(float(np.mean(y)))
        ok = abs(float(np.mean(d))) <= tol
        out[k] = {"gpu_mean": float(np.mean(x)), "oracle_mean": float(np.mean(y)),
                  "mean_diff": float(np.mean(d)), "tol": tol, "se_paired": se_pair,
                  "unpaired_ci": Z * se_unpaired, "ok": ok}
        out["ok"] &= ok
    return out
