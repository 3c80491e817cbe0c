"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset is involved; every series is generated here from a seed:
  logistic   coupled logistic map x[t+1]=x[t](3.8-3.8x[t]-0.02y[t]),
             y[t+1]=y[t](3.5-3.5y[t]-0.1x[t]), x0,y0 ~ U(0.1,0.9), 100-step
             burn-in dropped (simplex / S-map / CCM workloads)
  panels     512 coupled logistic maps with per-panel growth rates, uneven
             log-uniform lengths, 5% NaN, irregular integer time gaps
  lorenz     Lorenz-63 by RK4 (dt=0.01), 1000-step burn-in, noisy x
"""
import math

import numpy as np


def coupled_logistic(T, seed=1, noise=0.0, burn=100):
    rng = np.random.default_rng(seed)
    x, y = rng.uniform(0.1, 0.9, size=2)
    xs = np.empty(T)
    ys = np.empty(T)
    for i in range(burn + T):
        if i >= burn:
            xs[i - burn], ys[i - burn] = x, y
        x, y = x * (3.8 - 3.8 * x - 0.02 * y), y * (3.5 - 3.5 * y - 0.1 * x)
    if noise:
        xs = xs + rng.normal(0, noise, T)
        ys = ys + rng.normal(0, noise, T)
    t = np.arange(1, T + 1, dtype=float)
    return t, xs, ys


def ccm_library_sizes(n=20, lo=100, hi=40000):
    """n log-spaced library sizes from lo to hi (rounded)."""
    return [int(round(v)) for v in np.logspace(math.log10(lo), math.log10(hi), n)]


def simplex_config(seed=1):
    """250-point library, 250-point prediction set, E = 1..10 (config 1)."""
    t, x, y = coupled_logistic(500, seed)
    lib = np.zeros(500, bool)
    lib[:250] = True
    return dict(t=t, x=x, y=y, library_rows=lib, prediction_rows=~lib, Es=list(range(1, 11)))


def smap_config(seed=2, T=20000):
    """S-map theta sweep on a noisy map: library first half, prediction second (config 2)."""
    t, x, y = coupled_logistic(T, seed, noise=0.01)
    lib = np.zeros(T, bool)
    lib[: T // 2] = True
    thetas = [round(0.1 * i, 10) for i in range(81)]
    return dict(t=t, x=x, y=y, library_rows=lib, prediction_rows=~lib, E=5, thetas=thetas)


def ccm_config(seed=3, T=50000, n_libs=20, reps=200, lo=100, hi=40000):
    """Batched convergent cross mapping (config 3)."""
    t, x, y = coupled_logistic(T, seed)
    return dict(t=t, x=x, y=y, E=4, libraries=ccm_library_sizes(n_libs, lo, hi), numReps=reps, seed=seed)


def panel_config(seed=4, n_panels=512, lo=50, hi=2000):
    """Uneven multispatial panels with missing data and irregular times (config 4)."""
    rng = np.random.default_rng(seed)
    ts, xs, ys, ps = [], [], [], []
    for pid in range(n_panels):
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        rx, ry, c = rng.uniform(3.6, 3.9), rng.uniform(3.4, 3.7), rng.uniform(0, 0.15)
        x, y = rng.uniform(0.1, 0.9, size=2)
        px, py = np.empty(n), np.empty(n)
        for i in range(100 + n):
            if i >= 100:
                px[i - 100], py[i - 100] = x, y
            x, y = x * (rx - rx * x - c * y), y * (ry - ry * y - c * x)
        gaps = rng.choice([1, 2, 3], size=n, p=[0.8, 0.15, 0.05])
        t = np.cumsum(gaps).astype(float)
        miss = rng.uniform(size=n) < 0.05
        px[miss] = np.nan
        ts.append(t)
        xs.append(px)
        ys.append(py)
        ps.append(np.full(n, pid, dtype=float))
    return dict(t=np.concatenate(ts), x=np.concatenate(xs), y=np.concatenate(ys), panel=np.concatenate(ps))


def lorenz_config(seed=5, T=100000, dt=0.01, burn=1000, noise=0.05):
    """Lorenz-63 x observed with noise (config 5)."""
    rng = np.random.default_rng(seed)
    s = np.array([1.0, 1.0, 1.0]) + rng.normal(0, 0.01, 3)
    sig, rho, beta = 10.0, 28.0, 8.0 / 3.0

    def f(v):
        return np.array([sig * (v[1] - v[0]), v[0] * (rho - v[2]) - v[1], v[0] * v[1] - beta * v[2]])

    out = np.empty(T)
    for i in range(burn + T):
        k1 = f(s)
        k2 = f(s + 0.5 * dt * k1)
        k3 = f(s + 0.5 * dt * k2)
        k4 = f(s + dt * k3)
        s = s + dt / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)
        if i >= burn:
            out[i - burn] = s[0]
    x = out + rng.normal(0, noise, T)
    return dict(t=np.arange(1, T + 1, dtype=float), x=x)
