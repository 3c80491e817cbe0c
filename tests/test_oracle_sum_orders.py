"""How far the reference's own builds spread: summation orders left to Eigen.

The reference takes mean(d), X^T X and X^T y of every S-map forecast from
Eigen (src/edm.cpp:745,781-782), whose vectorised reductions sum in an order
set by the SIMD width (packets of 2 doubles on SSE2 and NEON, 4 on AVX), and
its compiler may contract a*b+c into FMA (GCC does by default on aarch64).
The oracle -- and the GPU library, which matches it bit for bit -- uses the
plain sequential unfused order.  This test runs the oracle in each of the
other orders (oracle_set_sum_mode) and bounds the spread of forecasts and
rho against the sequential order:

  * S-map with k = E + 2 neighbours (CCM): the normal equations of 5
    unknowns from 6 rows are ill-conditioned, so the orders move forecasts by
    percents and rho by ~1e-3 (the same holds for a 1-ulp change of exp);
  * S-map with every library row (k = all): ~1e-11 relative;
  * simplex: no Eigen reduction, ~1e-16 (FMA contraction only).

FEDM_SPREAD_FULL=1 runs the full-size shapes (T = 50 000 CCM over library
sizes 100..40 000, every 25th prediction row; the 10 000 x 10 000, 81-theta
sweep, every 97th row) and prints the spreads.
"""
import os

import numpy as np
import pytest

import edm_oracle
from fedm_loader import fedm, workloads

ORDERS = {"sse2": 1, "avx": 2, "neon_fma": 1 | 4, "aarch64_gcc": 1 | 4 | 8, "avx2_fma": 2 | 4 | 8}
FULL = os.environ.get("FEDM_SPREAD_FULL") == "1"


def _strided(mask, stride, offset=0):
    rows = np.nonzero(mask)[0]
    sub = np.zeros_like(mask)
    sub[rows[np.arange(offset % stride, len(rows), stride)]] = True
    return sub


def _task(a_kw, t, x, y, lib, pred, E, k, order=0, exp_mode=0):
    edm_oracle.set_sum_mode(order)
    edm_oracle.set_exp_mode(exp_mode)
    try:
        return edm_oracle.oracle_task(edm_oracle.normalise(t, x, y, numThreads=8, **a_kw), lib, pred, E, k)
    finally:
        edm_oracle.set_sum_mode(0)
        edm_oracle.set_exp_mode(0)


def _spread(o0, o1):
    p0, p1 = o0["predictions"], o1["predictions"]
    m = (p0 != 1e100) & (p1 != 1e100)
    assert np.array_equal(p0 != 1e100, p1 != 1e100)
    rel = float(np.max(np.abs(p0[m] - p1[m]) / np.abs(p0[m]))) if m.any() else 0.0
    drho = float(np.nanmax(np.abs(o0["stats_rho"] - o1["stats_rho"])))
    same_nn = np.array_equal(o0["nn_idx"], o1["nn_idx"])
    return rel, drho, same_nn


def test_sequential_order_is_the_default():
    t, x, y = workloads.coupled_logistic(800, seed=2)
    lib = np.zeros(800, bool)
    lib[10:400] = True
    pred = np.zeros(800, bool)
    pred[400:] = True
    kw = dict(E=3, theta=[0.5, 2.0], algorithm="smap")
    a = _task(kw, t, x, None, lib, pred, 3, 5)
    b = _task(kw, t, x, None, lib, pred, 3, 5, order=0)
    assert np.array_equal(a["predictions"], b["predictions"])


@pytest.mark.parametrize("algorithm", ["smap", "simplex"])
def test_ccm_spread_across_orders(algorithm):
    w = workloads.ccm_config(reps=1) if FULL else workloads.ccm_config(T=6000, reps=1, n_libs=4, hi=5000)
    theta = 2.0 if algorithm == "smap" else 1.0
    kw = dict(E=4, library=w["libraries"], numReps=1, shuffle=True, seed=w["seed"], algorithm=algorithm,
              theta=theta)
    plan = fedm.host_plan(fedm.normalise(w["t"], w["x"], w["y"], **kw))
    tasks = (0, 6, 12, 19) if FULL else range(len(plan["E"]))
    worst = {}
    for f in tasks:
        sub = _strided(plan["pred"][f], 25 if FULL else 10, f)
        args = (kw, w["t"], w["x"], w["y"], plan["lib"][f], sub, 4, int(plan["k"][f]))
        base = _task(*args)
        for name, order in list(ORDERS.items()) + [("exp_1ulp", 0)]:
            o = _task(*args, order=order, exp_mode=1 if name == "exp_1ulp" else 0)
            rel, drho, same_nn = _spread(base, o)
            # summation orders and FMA never change which rows are neighbours here
            assert same_nn, (name, f)
            r0, d0 = worst.get(name, (0.0, 0.0))
            worst[name] = (max(r0, rel), max(d0, drho))
    print({k: f"max |dy|/|y| {v[0]:.2e}, max |drho| {v[1]:.2e}" for k, v in worst.items()})
    if algorithm == "smap":
        assert all(r <= 0.2 and d <= 1e-2 for r, d in worst.values()), worst
        assert max(r for r, _ in worst.values()) > 1e-9  # ill-conditioned: the orders matter
    else:
        assert all(r <= 1e-14 and d <= 1e-14 for r, d in worst.values()), worst


def test_all_neighbour_smap_spread_across_orders():
    w = workloads.smap_config() if FULL else workloads.smap_config(T=2000)
    thetas = w["thetas"] if FULL else w["thetas"][::8]
    kw = dict(E=5, theta=thetas, algorithm="smap")
    a = fedm.normalise(w["t"], w["x"], **kw)
    usable = fedm.host_usable(a, 5)
    lib, pred = w["library_rows"] & usable, w["prediction_rows"] & usable
    sub = _strided(pred, 97 if FULL else 20)
    args = (kw, w["t"], w["x"], None, lib, sub, 5, -1)
    base = _task(*args)
    worst = {}
    for name, order in list(ORDERS.items()) + [("exp_1ulp", 0)]:
        o = _task(*args, order=order, exp_mode=1 if name == "exp_1ulp" else 0)
        worst[name] = _spread(base, o)[:2]
    print({k: f"max |dy|/|y| {v[0]:.2e}, max |drho| {v[1]:.2e}" for k, v in worst.items()})
    assert all(r <= 1e-9 and d <= 1e-11 for r, d in worst.values()), worst
