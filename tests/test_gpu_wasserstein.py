"""Wasserstein distance on the GPU (src/distances.cpp:270-527, chosen at
src/edm.cpp:578-582) through fedm_run_task, against the oracle.

The cost matrix follows the reference step by step; the transport cost comes
from the device's successive-shortest-path solver, the oracle's from its
Hungarian restatement, pinned to the reference's own EMD_wrap
(tests/test_oracle_wasserstein.py).  Both are exact solvers of the same
problem, but the optimal plan is often not unique (costs that are sums of
absolute differences of one-dimensional values tie across many
permutations), and each solver sums the plan it found in EMD_wrap's arc
order: the distances agree to a few ulps (1e-14 relative), not bit for bit.
The bars: neighbour lists identical, distances within 1e-14, simplex
forecasts within 1e-12, S-map forecasts over every library row (well
conditioned) within 1e-9.  Columns left out for missing values (missing
distance 0) give unequal masses; the same bars hold.
"""
import numpy as np
import pytest

import edm_oracle
from fedm_loader import fedm, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device_exp():
    edm_oracle.set_exp_mode(1)
    yield
    edm_oracle.set_exp_mode(0)


@pytest.fixture(scope="module")
def ctx():
    c = fedm.Context(0)
    yield c
    c.close()


def _masks(n, split):
    lib = np.zeros(n, bool)
    lib[:split] = True
    return lib, ~lib


def _compare(g, o, pred_rtol):
    assert g["task_rc"] == o["task_rc"]
    assert np.array_equal(g["kused"], o["kused"])
    assert np.array_equal(g["rc"], o["rc"])
    assert np.array_equal(g["nn_offsets"], o["nn_offsets"])
    assert np.array_equal(g["nn_idx"], o["nn_idx"])
    assert np.allclose(g["nn_dist"], o["nn_dist"], rtol=1e-14, atol=0)
    m = o["predictions"] != 1e100
    assert np.array_equal(g["predictions"] != 1e100, m)
    assert np.allclose(g["predictions"][m], o["predictions"][m], rtol=pred_rtol, atol=1e-13)


def _both(ctx, a, lib, pred, E, k, pred_rtol=1e-12, aspect_ratio=0.0):
    g = ctx.run_task(a, lib, pred, E, k, distance=2, aspect_ratio=aspect_ratio)
    o = edm_oracle.oracle_task(edm_oracle.normalise(**a["_kw"]), lib, pred, E, k, distance=2,
                               aspect_ratio=aspect_ratio)
    assert g["n_pred"] == o["n_pred"] and g["n_lib"] == o["n_lib"]
    _compare(g, o, pred_rtol)
    return g


def _args(**kw):
    a = fedm.normalise(**kw)
    a["_kw"] = kw
    return a


@pytest.mark.parametrize("E", [1, 2, 4, 7])
def test_wasserstein_neighbours_and_forecasts(ctx, E):
    t, x, _ = workloads.coupled_logistic(260, seed=40 + E)
    lib, pred = _masks(260, 130)
    a = _args(t=t, x=x, E=E, theta=[0.0, 1.0, 3.0])
    for k in (E + 1, E + 2, -1):
        _both(ctx, a, lib, pred, E, k)
    a = _args(t=t, x=x, E=E, theta=[0.0, 1.0, 3.0], algorithm="smap")
    _both(ctx, a, lib, pred, E, -1, pred_rtol=1e-9)


def test_wasserstein_dt_aspect_ratio(ctx):
    """dt columns form the time row of the reference's point matrix, scaled
    by the aspect ratio of the library point's curve (src/distances.cpp:340-362,
    403-406)."""
    t, x, _ = workloads.coupled_logistic(240, seed=3)
    t = t.astype(float).copy()
    t[::7] += 0.5
    for ar in (1.5, 0.0):
        a = _args(t=t, x=x, E=3, theta=[1.0], dt=True)
        lib, pred = _masks(240, 120)
        _both(ctx, a, lib, pred, 3, 4, aspect_ratio=ar)


def test_wasserstein_missing_columns(ctx):
    """Missing values: with a missing distance a missing column costs it
    (equal masses, bit-exact); without one (missing distance 0) the column is
    left out and the masses are 1/len_i, 1/len_j (src/distances.cpp:325-337)."""
    t, x, _ = workloads.coupled_logistic(160, seed=9)
    x = x.copy()
    x[5::11] = np.nan
    lib, pred = _masks(160, 80)
    a = _args(t=t, x=x, E=4, theta=[1.0], allowMissing=True, missingDistance=0.7)
    _both(ctx, a, lib, pred, 4, 5)
    a = _args(t=t, x=x, E=4, theta=[1.0])
    _both(ctx, a, lib, pred, 4, 5)


@pytest.mark.parametrize("panel_weight", [0.25, float("inf")])
def test_wasserstein_panels_and_extras(ctx, panel_weight):
    """Panels (a penalty added to every cost, or other panels skipped) and an
    unlagged extra variable (its distance added to every cost)."""
    t, x, y = workloads.coupled_logistic(240, seed=12)
    panel = np.repeat(np.arange(4), 60)
    extra = np.sin(np.arange(240) * 0.3)
    a = _args(t=t, x=x, E=3, theta=[1.0], panel=panel, panelWeight=panel_weight, extras=[extra])
    lib = (np.arange(240) % 60) < 40
    _both(ctx, a, lib, ~lib, 3, 4)
    a = _args(t=t, x=x, E=3, theta=[0.5, 2.0], panel=panel, panelWeight=panel_weight, extras=[extra],
              algorithm="smap")
    _both(ctx, a, lib, ~lib, 3, -1, pred_rtol=1e-9)


def test_wasserstein_wider_embeddings_rejected_cleanly(ctx):
    t, x, _ = workloads.coupled_logistic(100, seed=2)
    a = _args(t=t, x=x, E=17, theta=[1.0])
    lib, pred = _masks(100, 50)
    with pytest.raises(RuntimeError):
        ctx.run_task(a, lib, pred, 17, 18, distance=2)


@pytest.mark.parametrize("algorithm,k", [("simplex", 6), ("smap", 7)])
def test_wasserstein_full_size(ctx, algorithm, k):
    """The benchmark's shape: T = 4 000, E = 5, library the first 2 000 rows,
    every 10th of the last 2 000 rows predicted, against the oracle (200
    points x 2 000 library rows of 5 x 5 transport problems).  Neighbour
    lists identical, distances within 1e-14.  Where a point's neighbour
    distances are the same bits, its forecasts are the same bits too (the
    forecast stage is the exact path's); elsewhere simplex forecasts are
    within 1e-12, and S-map forecasts from 7 neighbours (their normal
    equations are ill-conditioned) are only counted."""
    t, x, _ = workloads.coupled_logistic(4000, seed=61)
    lib = np.zeros(4000, bool)
    lib[:2000] = True
    pred = np.zeros(4000, bool)
    pred[2000::10] = True
    a = _args(t=t, x=x, E=5, theta=[1.0], algorithm=algorithm)
    g = ctx.run_task(a, lib, pred, 5, k, distance=2)
    o = edm_oracle.oracle_task(edm_oracle.normalise(**a["_kw"]), lib, pred, 5, k, distance=2)
    assert g["n_pred"] == o["n_pred"] == 200 and g["n_lib"] == o["n_lib"]
    assert g["task_rc"] == o["task_rc"]
    assert np.array_equal(g["kused"], o["kused"])
    assert np.array_equal(g["nn_offsets"], o["nn_offsets"])
    assert np.array_equal(g["nn_idx"], o["nn_idx"])
    assert np.allclose(g["nn_dist"], o["nn_dist"], rtol=1e-14, atol=0)
    same = np.array([np.array_equal(g["nn_dist"][s:e].view(np.int64), o["nn_dist"][s:e].view(np.int64))
                     for s, e in zip(o["nn_offsets"][:-1], o["nn_offsets"][1:])])
    assert same.sum() > 0
    gp, op = g["predictions"][0], o["predictions"][0]
    assert np.array_equal(gp[same].view(np.int64), op[same].view(np.int64))
    if algorithm == "simplex":
        assert np.allclose(gp, op, rtol=1e-12, atol=1e-13)
