"""CPU parity of the library's host layer against the oracle: the
splitter's MT19937-64 stream, usable-row masks, manifold rows (bit-exact) and
configure_tasks' task list with its library / prediction membership."""
import numpy as np
import pytest

import ci_cases
import edm_oracle
from fedm_loader import build, fedm, workloads


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    edm_oracle.load()


@pytest.mark.parametrize("seed", [0, 1, 12345678, 2**31 - 1, 4242])
def test_mt64_stream(seed):
    assert np.array_equal(fedm.host_mt_real2(seed, 2000), edm_oracle.mt_real2(seed, 2000))


def datasets():
    t, x, y = ci_cases.simple_data()
    yield "simple", dict(t=t, x=x, y=y), {}
    t, x, y, u = ci_cases.missing_data()
    yield "missing", dict(t=t, x=x, y=y), dict(extras=[u])
    t, x, y, u, u1 = ci_cases.bigger_missing_data()
    yield "bigger", dict(t=t, x=x, y=y), dict(copredict=u1)
    t, x, y, panel = ci_cases.panel_data()
    keep = np.fmod(t, 7) != 0
    yield "panel", dict(t=t[keep], x=x[keep], y=y[keep]), dict(panel=panel[keep])


OPTION_SETS = [
    {}, dict(dt=True), dict(allowMissing=True), dict(dt=True, allowMissing=True), dict(reldt=True),
    dict(p=-1), dict(p=3, tau=2),
]


@pytest.mark.parametrize("opts", OPTION_SETS, ids=lambda o: ",".join(f"{k}={v}" for k, v in o.items()) or "plain")
@pytest.mark.parametrize("ds", list(datasets()), ids=lambda d: d[0])
def test_usable_and_manifolds(ds, opts):
    name, data, extra = ds
    kw = dict(extra)
    kw.update(opts)
    for xmap in (False, True):
        a = edm_oracle.normalise(data["t"], data["x"], data["y"] if xmap else None, E=3, **kw)
        for maxE in (1, 3, 6):
            for co in ((False, True) if a["co_x"] is not None else (False,)):
                assert np.array_equal(fedm.host_usable(a, maxE, co), edm_oracle.usable(a, maxE, co))
        for E in (1, 2, 5):
            F = fedm.host_manifold(a, E)
            n = a["n"]
            o = edm_oracle.oracle_task(a, np.ones(n, bool), np.ones(n, bool), E, 1)
            rows = o["pred_point_rows"]
            assert F.shape[1] == o["e_actual"]
            assert np.array_equal(F[rows].view(np.int64), o["pred_manifold"].view(np.int64)), (name, E)


PLAN_CASES = [
    dict(E=[2, 3, 5]),
    dict(E=[2, 4], shuffle=True, seed=7),
    dict(E=3, crossfold=4),
    dict(E=[2, 3], crossfold=3, shuffle=True, seed=3),
    dict(E=2, full=True),
    dict(E=3, numReps=5, seed=11),
    dict(E=[2, 3], xmap=True, library=[10, 25, 60], numReps=4, seed=5),
    dict(E=2, xmap=True, library=[8, 16]),
    dict(E=2, xmap=True, library=[5, 10, 20], numReps=3, copredict=True),
    dict(E=[2, 3], theta=[0, 1], copredict=True, numReps=2),
]


@pytest.mark.parametrize("case", PLAN_CASES, ids=lambda c: ",".join(f"{k}={v}" for k, v in c.items()))
def test_task_plan_membership(case):
    t, x, y, u, u1 = ci_cases.bigger_missing_data()
    kw = dict(case)
    xmap = kw.pop("xmap", False)
    if kw.pop("copredict", False):
        kw["copredict"] = u1
    a = edm_oracle.normalise(t, x, y if xmap else None, allowMissing=True, **kw)
    g, o = fedm.host_plan(a), edm_oracle.plan(a)
    for key in ("E", "k", "library", "copredict", "lib", "pred"):
        assert np.array_equal(g[key], o[key]), key


def test_ccm_replicate_membership_large():
    """The CCM benchmark's replicate libraries (seeded MT19937-64 splits)."""
    w = workloads.ccm_config(T=6000, reps=6, n_libs=5, hi=4000)
    a = edm_oracle.normalise(w["t"], w["x"], w["y"], E=4, library=w["libraries"], numReps=6, seed=w["seed"])
    g, o = fedm.host_plan(a), edm_oracle.plan(a)
    assert np.array_equal(g["lib"], o["lib"]) and np.array_equal(g["pred"], o["pred"])
    assert list(g["lib"].sum(axis=1)[:5]) == w["libraries"]
