"""GPU parity: the GB300 library through its C ABI against the CPU oracle.

* every test block of the reference's test-ci.R, run through the GPU, must
  meet the reference's golden values (1e-4) and agree with the oracle call
  by call: identical return codes, k ranges and NA patterns; rho, MAE and
  forecasts within 1e-9 relative (FP64 exact path) -- the oracle computes the
  same FP64 operations in the same order, differences come from exp() and
  reduction order only;
* on explicit masks, neighbour indices and distances are bit-identical.
"""
import numpy as np
import pytest

import ci_cases
import edm_oracle
from fedm_loader import fedm, workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-9
ATOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _device_exp():
    # the oracle evaluates the same IEEE-only exp formula as the device
    edm_oracle.set_exp_mode(1)
    yield
    edm_oracle.set_exp_mode(0)


@pytest.fixture(scope="module", params=[fedm.PRECISION_FP64, fedm.PRECISION_MIXED], ids=["fp64", "mixed"])
def ctx(request):
    c = fedm.Context(0, precision=request.param)
    c.precision = request.param
    yield c
    c.close()


def _close(a, b, what, rtol=RTOL, atol=ATOL):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    assert np.array_equal(np.isnan(a), np.isnan(b)), (what, "NA pattern differs")
    m = ~np.isnan(a)
    assert np.allclose(a[m], b[m], rtol=rtol, atol=atol), (what, np.max(np.abs(a[m] - b[m])) if m.any() else 0)


def compare(g, o):
    assert g["rc"] == o["rc"], (g["rc"], o["rc"], g.get("error"))
    for key in ("stats", "copredStats"):
        assert (key in g) == (key in o), key
        if key in o:
            for f in ("E", "library", "theta"):
                assert np.array_equal(g[key][f], o[key][f]), (key, f)
            _close(g[key]["rho"], o[key]["rho"], key + ".rho")
            _close(g[key]["mae"], o[key]["mae"], key + ".mae")
    assert g.get("kMin") == o.get("kMin") and g.get("kMax") == o.get("kMax")
    for key in ("predictions", "copredictions", "coeffs"):
        assert (key in g) == (key in o), key
        if key in o:
            _close(g[key], o[key], key, rtol=1e-8, atol=1e-10)
    for key in ("missingdistance", "dtWeight"):
        assert (key in g) == (key in o)
        if key in o:
            assert g[key] == o[key], key


@pytest.mark.parametrize("case", ci_cases.CASES, ids=lambda c: c.__name__)
def test_reference_goldens_on_gpu(ctx, case):
    def both(t, x, y=None, **kw):
        g = fedm.edm(t, x, y, ctx=ctx, **kw)
        o = edm_oracle.oracle_edm(t, x, y, **kw)
        compare(g, o)
        return g

    case(both)


def _task_pair(ctx, a, lib, pred, E, k, **kw):
    g = ctx.run_task(a, lib, pred, E, k, **kw)
    o = edm_oracle.oracle_task(a, lib, pred, E, k, **kw)
    assert g["n_pred"] == o["n_pred"] and g["n_lib"] == o["n_lib"] and g["e_actual"] == o["e_actual"]
    assert np.array_equal(g["kused"], o["kused"])
    assert np.array_equal(g["nn_offsets"], o["nn_offsets"])
    assert np.array_equal(g["nn_idx"], o["nn_idx"]), "neighbour indices differ"
    assert np.array_equal(g["nn_dist"].view(np.int64), o["nn_dist"].view(np.int64)), "neighbour distances differ"
    assert np.array_equal(g["rc"], o["rc"])
    # both forms: the same neighbours (bit-exact), then the same FP64
    # operations in the same order as the oracle: identical bits
    assert np.array_equal(g["predictions"], o["predictions"]), "forecasts differ"
    assert np.array_equal(g["coeffs"], o["coeffs"]), "coefficients differ"
    _close(g["stats_rho"], o["stats_rho"], "rho")
    _close(g["stats_mae"], o["stats_mae"], "mae")
    return g, o


@pytest.mark.parametrize("masks", ["explicit", "usable"])
def test_simplex_config_neighbours_bit_exact(ctx, masks):
    """250/250 split of the coupled logistic map, E = 1..10, k = E+1.  The
    explicit masks include the first rows, whose lags are missing, so every
    task runs the exact kernels; with usable-row masks the mixed context runs
    the one-point scan for k <= 6, the 16-slot form for k = 7..9 and the wide
    form for E = 9, 10."""
    w = workloads.simplex_config()
    a = edm_oracle.normalise(w["t"], w["x"], E=1)
    for E in w["Es"]:
        lib, pred = w["library_rows"], w["prediction_rows"]
        if masks == "usable":
            usable = fedm.host_usable(edm_oracle.normalise(w["t"], w["x"], E=E), E)
            lib, pred = lib & usable, pred & usable
        _task_pair(ctx, a, lib, pred, E, E + 1)
        if masks == "usable" and ctx.precision == fedm.PRECISION_MIXED:
            assert ctx.timing()["mixed_form"] >= 0, E


@pytest.mark.parametrize("masks", ["raw", "usable"])
@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
@pytest.mark.parametrize("k", [0, 1, 3, 7, 40, -1, 500])
def test_random_task_edges(ctx, algorithm, k, masks):
    """Ties (duplicated values), self matches, k beyond the library, k = all.
    'raw' masks include the first rows, whose lags are missing (the exact
    kernels serve any task whose library holds such a row); 'usable' masks
    keep complete rows only, so the mixed context runs 1 <= k <= 16 through
    the FP32 scan, its certification and the bounded re-scan."""
    rng = np.random.default_rng(11)
    n = 300
    x = np.round(rng.normal(size=n), 1)  # many exact ties
    x[x == 0] = 0.1
    t = np.arange(1, n + 1, dtype=float)
    a = edm_oracle.normalise(t, x, E=3, theta=[0.0, 1.0, 3.0], algorithm=algorithm)
    lib = rng.uniform(size=n) < 0.5
    pred = np.ones(n, bool)
    if masks == "usable":
        usable = fedm.host_usable(a, 3)
        lib, pred = lib & usable, pred & usable
    _task_pair(ctx, a, lib, pred, 3, k)
    if masks == "usable" and ctx.precision == fedm.PRECISION_MIXED and 1 <= k <= 16:
        assert ctx.timing()["fp64_ops"] > 0  # the mixed kernels ran


def test_empty_library(ctx):
    t = np.arange(1, 51, dtype=float)
    x = np.sin(t)
    a = edm_oracle.normalise(t, x, E=2)
    lib = np.zeros(50, bool)
    g, o = _task_pair(ctx, a, lib, np.ones(50, bool), 2, 3)
    assert np.all(g["kused"] == -(2**31))


@pytest.mark.parametrize("series", ["all_missing", "one_value", "constant", "shorter_than_E"])
@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_degenerate_series(ctx, series, algorithm):
    """edm() on series that leave nothing or almost nothing to predict: no
    observed value, a single one, a constant series (every distance is zero
    and excluded), four points for E = 3.  Return codes, k ranges, NA
    patterns and statistics as the oracle's run_command gives them."""
    t = np.arange(1, 41, dtype=float)
    x = {
        "all_missing": np.full(40, np.nan),
        "one_value": np.where(t == 7, 0.3, np.nan),
        "constant": np.full(40, 0.5),
        "shorter_than_E": None,
    }[series]
    if x is None:
        t, x = np.arange(1, 5, dtype=float), np.array([0.1, 0.4, 0.2, 0.9])
    kw = dict(E=3, algorithm=algorithm, savePredictions=True)
    compare(fedm.edm(t, x, ctx=ctx, **kw), edm_oracle.oracle_edm(t, x, **kw))


@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_degenerate_tasks(ctx, algorithm):
    """Single tasks on degenerate masks, bit-exact: an empty prediction set;
    a constant series on raw masks, where the only valid neighbour is the
    first library row with its lag missing (a coordinate of 1e100); the same
    series on usable rows, where every distance is zero and no forecast is
    made."""
    t = np.arange(1, 41, dtype=float)
    a = edm_oracle.normalise(t, np.sin(t), E=2, algorithm=algorithm)
    g, o = _task_pair(ctx, a, np.ones(40, bool), np.zeros(40, bool), 2, 3)
    assert g["n_pred"] == 0
    a = edm_oracle.normalise(t, np.full(40, 0.5), E=2, theta=[0.0, 1.0], algorithm=algorithm)
    first = np.arange(40) < 20
    g, o = _task_pair(ctx, a, first, ~first, 2, 3)
    assert np.all(g["kused"] == 1)
    usable = fedm.host_usable(a, 2)
    g, o = _task_pair(ctx, a, first & usable, ~first & usable, 2, 3)
    assert np.all(np.isnan(g["predictions"]) | (g["predictions"] == 1e100))


@pytest.mark.parametrize("distance", [0, 1])
def test_missing_panels_l1(ctx, distance):
    rng = np.random.default_rng(5)
    n = 240
    t = np.arange(1, n + 1, dtype=float)
    x = rng.normal(size=n)
    x[rng.uniform(size=n) < 0.1] = np.nan
    panel = (t > 120) * 1.0
    a = edm_oracle.normalise(t, x, panel=panel, E=3, allowMissing=True, panelWeight=0.5)
    lib = rng.uniform(size=n) < 0.6
    _task_pair(ctx, a, lib, np.ones(n, bool), 3, 5, distance=distance)


def test_force_compute_off(ctx):
    t = np.arange(1, 81, dtype=float)
    x = np.cos(0.3 * t)
    a = edm_oracle.normalise(t, x, E=2, theta=[1.0, 2.0])
    lib = np.zeros(80, bool)
    lib[:4] = True
    _task_pair(ctx, a, lib, np.ones(80, bool), 2, 6, force_compute=False)
