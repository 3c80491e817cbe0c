"""R idioms the reference's tests rely on, restated in numpy.

These rebuild the inputs of tests/testthat/test-ci.R (reference project):
logistic_map (R/logistic_map.R:12-31), tslag / tsdiff (test-ci.R:1-21), R's
mean()/sd() and data.frame row subsetting with NA.
"""
import json
import math
from pathlib import Path

import numpy as np

NA = float("nan")
GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "test_ci.json").read_text())


def golden(line):
    """Numeric literals of test-ci.R at that 1-based line (NA -> nan)."""
    return [NA if v is None else v for v in GOLDEN["lines"][str(line)]["values"]]


def vector(name):
    return np.array(GOLDEN["vectors"][name], dtype=np.float64)


def logistic_map(obs):
    """R/logistic_map.R:12-31 (same double arithmetic, same operation order)."""
    r_x, r_y, beta_xy, beta_yx = 3.625, 3.77, 0.05, 0.4
    x = [NA] * obs
    y = [NA] * obs
    x[0], y[0] = 0.2, 0.4
    for i in range(1, obs):
        x[i] = x[i - 1] * (r_x * (1 - x[i - 1]) - beta_xy * y[i - 1])
        y[i] = y[i - 1] * (r_y * (1 - y[i - 1]) - beta_yx * x[i - 1])
    return np.array(x), np.array(y)


def tslag(t, x, lag=1, dt=1):
    """test-ci.R:1-10: value at time t - lag*dt (first match), else NA."""
    t = np.asarray(t, dtype=float)
    x = np.asarray(x, dtype=float)
    out = np.full(len(t), NA)
    for i in range(len(t)):
        lt = t[i] - lag * dt
        if not math.isnan(lt):
            hits = np.nonzero(t == lt)[0]
            if len(hits):
                out[i] = x[hits[0]]
    return out


def tsdiff(t, x, lag=1, dt=1):
    """test-ci.R:12-21."""
    t = np.asarray(t, dtype=float)
    x = np.asarray(x, dtype=float)
    out = np.full(len(t), NA)
    for i in range(len(t)):
        lt = t[i] - lag * dt
        if not math.isnan(x[i]) and not math.isnan(lt):
            hits = np.nonzero(t == lt)[0]
            if len(hits):
                out[i] = x[i] - x[hits[0]]
    return out


def r_mean(x):
    """R's mean(): long-double sum with one correction pass."""
    x = np.asarray(x, dtype=np.longdouble)
    s = x.sum() / len(x)
    s = s + (x - s).sum() / len(x)
    return float(s)


def r_sd(x):
    x = np.asarray(x, dtype=float)
    m = r_mean(x)
    return math.sqrt(float(((x - m) ** 2).sum()) / (len(x) - 1))


def seq(a, b, by):
    """R's seq(from, to, by): from + (0:n) * by."""
    n = int(math.floor((b - a) / by + 1e-10))
    return [a + i * by for i in range(n + 1)]


def max_abs_err_ok(x, y, tol=1e-4):
    """expect_approx_equal (test-ci.R:23-33)."""
    x = np.atleast_1d(np.asarray(x, dtype=float))
    y = np.atleast_1d(np.asarray(y, dtype=float))
    if len(x) != len(y) or not np.all(np.isfinite(x)) or not np.all(np.isfinite(y)):
        return False
    return float(np.max(np.abs(x - y))) < tol


def aggregate_mean_rho(stats):
    """aggregate(rho ~ E + library + theta, na.omit(stats), mean)$x with R's
    group order (first factor fastest)."""
    E, L, T, R, M = (np.asarray(stats[k], dtype=float) for k in ("E", "library", "theta", "rho", "mae"))
    keep = ~(np.isnan(R) | np.isnan(M) | np.isnan(E) | np.isnan(L) | np.isnan(T))
    groups = {}
    for e, l, t, r in zip(E[keep], L[keep], T[keep], R[keep]):
        groups.setdefault((t, l, e), []).append(r)
    return np.array([np.mean(groups[key]) for key in sorted(groups)])
