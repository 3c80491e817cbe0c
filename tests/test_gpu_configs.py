"""GPU parity on the benchmark configurations' shapes (seeded synthetic data).

* S-map theta sweep with k = all (config 2 shape), at an oracle-tractable
  size: through the task seam (bit-exact) and through run_command.
* Uneven multispatial panels with missing values and dt (config 4 shape),
  reduced to 48 panels: run_command with pooled, penalised and independent
  panels; penalties outside the FP32 range stay on the FP64 kernels.
* Config 2 at full size (10 000 / 10 000): with theta = 0 every weight is 1,
  so S-map is ordinary least squares on the library; the forecasts must match
  numpy's lstsq (a check that needs no oracle).
* Batched CCM (config 3 shape) on a reduced grid: every replicate's rho
  against the oracle, for both precisions.
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


@pytest.fixture(scope="module", params=[fedm.PRECISION_FP64, fedm.PRECISION_MIXED], ids=["fp64", "mixed"])
def ctx(request):
    c = fedm.Context(0, precision=request.param)
    yield c
    c.close()


def _stats_close(g, o, key="stats", rtol=1e-9):
    assert g["rc"] == o["rc"]
    for f in ("E", "library", "theta"):
        assert np.array_equal(g[key][f], o[key][f])
    for f in ("rho", "mae"):
        a, b = np.asarray(g[key][f]), np.asarray(o[key][f])
        assert np.array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(a)
        assert np.allclose(a[m], b[m], rtol=rtol, atol=1e-12), (f, np.max(np.abs(a[m] - b[m])))


def test_smap_theta_sweep_all_neighbours_task(ctx):
    w = workloads.smap_config(T=1200)
    a = edm_oracle.normalise(w["t"], w["x"], E=5, theta=w["thetas"][::4], algorithm="smap", numThreads=16)
    g = ctx.run_task(a, w["library_rows"], w["prediction_rows"], 5, -1)
    o = edm_oracle.oracle_task(a, w["library_rows"], w["prediction_rows"], 5, -1)
    assert np.array_equal(g["nn_idx"], o["nn_idx"])
    assert np.array_equal(g["predictions"], o["predictions"])
    assert np.array_equal(g["coeffs"], o["coeffs"])


def test_smap_theta_sweep_all_neighbours_command(ctx):
    w = workloads.smap_config(T=1600)
    kw = dict(E=5, k=float("inf"), theta=w["thetas"][::8], algorithm="smap", savePredictions=True,
              saveSMAPCoeffs=True)
    g = fedm.edm(w["t"], w["x"], ctx=ctx, **kw)
    o = edm_oracle.oracle_edm(w["t"], w["x"], numThreads=16, **kw)
    _stats_close(g, o)
    assert np.array_equal(g["predictions"], o["predictions"], equal_nan=True)
    assert np.array_equal(g["coeffs"], o["coeffs"], equal_nan=True)


@pytest.mark.parametrize("panel_weight", [0.0, 0.02, 0.3, float("inf")],
                         ids=["mixed_panels", "penalty_0.02", "penalty_0.3", "independent_panels"])
@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_uneven_panels_missing_dt(ctx, panel_weight, algorithm):
    """48 uneven panels, E = 3..8 with dt: panels pooled (panelWeight = 0),
    pooled with a penalty for a library row of another panel (small enough
    that other panels' rows are often neighbours), and independent."""
    w = workloads.panel_config(n_panels=48, lo=40, hi=300)
    theta = [0.0, 1.0, 2.0, 4.0] if algorithm == "smap" else [1.0]
    kw = dict(panel=w["panel"], E=[3, 4, 5, 6, 7, 8], dt=True, algorithm=algorithm, theta=theta,
              panelWeight=panel_weight)
    g = fedm.edm(w["t"], w["x"], ctx=ctx, **kw)
    if ctx.precision == fedm.PRECISION_MIXED:
        assert ctx.timing()["mixed_form"] >= 0  # mixed or per-panel sub-tasks on the mixed kernels
    o = edm_oracle.oracle_edm(w["t"], w["x"], numThreads=16, **kw)
    _stats_close(g, o)
    assert g["kMin"] == o["kMin"] and g["kMax"] == o["kMax"] and g["dtWeight"] == o["dtWeight"]


@pytest.mark.parametrize("panel_weight", [1e-35, 1e35])
def test_panel_penalty_outside_fp32_range_stays_exact(panel_weight):
    """A penalty below 1e-30 or above 1e30 is no normal FP32 number the scan
    could add with a bounded error: such calls run on the FP64 kernels."""
    w = workloads.panel_config(n_panels=12, lo=40, hi=200)
    kw = dict(panel=w["panel"], E=[3, 5], dt=True, algorithm="simplex", theta=[1.0], panelWeight=panel_weight)
    c = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        g = fedm.edm(w["t"], w["x"], ctx=c, **kw)
        assert c.timing()["mixed_form"] < 0
    finally:
        c.close()
    o = edm_oracle.oracle_edm(w["t"], w["x"], numThreads=16, **kw)
    _stats_close(g, o)


def test_ccm_replicates_reduced(ctx):
    w = workloads.ccm_config(T=4000, reps=4, n_libs=6, hi=3000)
    for algorithm, theta in (("simplex", 1.0), ("smap", 2.0)):
        kw = dict(E=4, library=w["libraries"], numReps=4, seed=w["seed"], algorithm=algorithm, theta=theta)
        g = fedm.edm(w["t"], w["x"], w["y"], ctx=ctx, **kw)
        o = edm_oracle.oracle_edm(w["t"], w["x"], w["y"], numThreads=16, **kw)
        _stats_close(g, o)


def test_smap_theta0_is_least_squares_full_size(ctx):
    """Config 2 size: 10 000 library rows, 10 000 forecasts, k = all."""
    w = workloads.smap_config(T=20000)
    a = fedm.normalise(w["t"], w["x"], E=5, theta=[0.0], algorithm="smap", k=float("inf"), savePredictions=True)
    lib, pred = w["library_rows"].copy(), w["prediction_rows"]
    lib[:4] = False  # rows without a full lag window are not usable (src/manifold.cpp:314-360)
    g = ctx.run_task(a, lib, pred, 5, -1)
    F = fedm.host_manifold(a, 5)
    x = w["x"]
    lib_rows = np.nonzero(lib)[0]
    pred_rows = np.nonzero(pred)[0]
    A = np.column_stack([np.ones(len(lib_rows)), F[lib_rows]])
    coef, *_ = np.linalg.lstsq(A, x[lib_rows + 1], rcond=None)
    want = coef[0] + F[pred_rows] @ coef[1:]
    got = g["predictions"][0]
    # every prediction row gets a forecast, also the last one whose target
    # is not observed (prediction sets keep such rows, src/manifold.h:186-189)
    assert np.all(got != 1e100) and g["n_lib"] == len(lib_rows)
    assert np.allclose(got, want, rtol=1e-7, atol=1e-9)


@pytest.mark.parametrize("T", [1600, 20000], ids=["reduced", "full_size"])
def test_fast_precision_smap_all_neighbours(T):
    """FEDM_PRECISION_FAST (config 2 shape: E = 5, k = all, a theta sweep
    with theta = 0..8): FP32 weights and double-float normal equations, then
    the FP64 solve.  Against the bit-exact FP64 path the forecasts agree to
    the FP32 weights' rounding and rho to 1e-6; theta = 0 (every weight 1) is
    exact up to the double-float sums."""
    w = workloads.smap_config(T=T)
    thetas = [0.0, 0.5, 1.0, 2.0, 4.0, 8.0]
    kw = dict(E=5, k=float("inf"), theta=thetas, algorithm="smap", savePredictions=True)
    fast = fedm.Context(0, precision=fedm.PRECISION_FAST)
    exact = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        f = fedm.edm(w["t"], w["x"], ctx=fast, **kw)
        tf = fast.timing()
        e = fedm.edm(w["t"], w["x"], ctx=exact, **kw)
        te = exact.timing()
    finally:
        fast.close()
        exact.close()
    assert f["rc"] == e["rc"] == 0
    pf, pe = np.asarray(f["predictions"], float), np.asarray(e["predictions"], float)
    assert np.array_equal(np.isnan(pf), np.isnan(pe))
    m = ~np.isnan(pe)
    scale = np.max(np.abs(pe[m]))
    err = np.max(np.abs(pf[m] - pe[m])) / scale
    assert err < 1e-5, err
    assert np.max(np.abs(np.asarray(f["stats"]["rho"]) - np.asarray(e["stats"]["rho"]))) <= 1e-6
    print(f"T={T}: max |forecast difference| / max |forecast| = {err:.2e}; device ms fast {tf['device_ms']:.1f}, "
          f"exact {te['device_ms']:.1f}")


@pytest.mark.parametrize("T", [1600, 20000], ids=["reduced", "full_size"])
def test_fast_precision_tensor_core_normal_equations(T, monkeypatch):
    """FEDM_PRECISION_FAST's k = all S-map at E_a <= 5 forms its normal
    equations on the tensor cores (tcgen05, exact bf16 slices of the weights
    and of the library-side products, FP32 accumulation exact per 64-row
    block, int64 across blocks).  Against the bit-exact path the forecasts
    agree within the FAST bar, as the double-float SIMT kernel
    (FEDM_GRAM_TC=0) does, and rho within 1e-6."""
    w = workloads.smap_config(T=T)
    thetas = [0.0, 0.5, 1.0, 2.0, 4.0, 8.0]
    kw = dict(E=5, k=float("inf"), theta=thetas, algorithm="smap", savePredictions=True)
    out = {}
    for name, prec, env in (("tc", fedm.PRECISION_FAST, "1"), ("simt", fedm.PRECISION_FAST, "0"),
                            ("exact", fedm.PRECISION_MIXED, "1")):
        monkeypatch.setenv("FEDM_GRAM_TC", env)
        c = fedm.Context(0, precision=prec)
        try:
            out[name] = (fedm.edm(w["t"], w["x"], ctx=c, **kw), c.timing())
        finally:
            c.close()
    (tc, ttc), (simt, tsimt), (exact, _) = out["tc"], out["simt"], out["exact"]
    assert ttc["tensor_core_tiles"] > 0 and tsimt["tensor_core_tiles"] == 0
    assert tc["rc"] == simt["rc"] == exact["rc"] == 0
    pe = np.asarray(exact["predictions"], float)
    m = ~np.isnan(pe)
    scale = np.max(np.abs(pe[m]))
    err = {k: np.max(np.abs(np.asarray(v[0]["predictions"], float)[m] - pe[m])) / scale
           for k, v in (("tc", out["tc"]), ("simt", out["simt"]))}
    drho = np.max(np.abs(np.asarray(tc["stats"]["rho"]) - np.asarray(exact["stats"]["rho"])))
    print(f"T={T}: max |forecast - exact| / max |forecast|: tensor cores {err['tc']:.2e}, "
          f"double-float SIMT {err['simt']:.2e}; |drho| {drho:.2e}; forecast kernels "
          f"{ttc['forecast_kernel_ms']:.1f} ms vs {tsimt['forecast_kernel_ms']:.1f} ms")
    assert err["tc"] < 1e-5 and drho <= 1e-6


@pytest.mark.parametrize("case", ["missing", "simplex_k_all", "wide_dt", "finite_k"])
def test_fast_precision_elsewhere_is_mixed(case):
    """FEDM_PRECISION_FAST changes only the S-map with every library row as a
    neighbour, E_actual <= 8, no missing values.  Elsewhere (missing values,
    simplex, dt embeddings wider than 8, a finite k) it gives MIXED's bits."""
    t, x, _ = workloads.coupled_logistic(1500, seed=8)
    x = x.copy()
    kw = dict(E=3, k=float("inf"), theta=[0.0, 2.0], algorithm="smap", savePredictions=True)
    if case == "missing":
        x[::41] = np.nan
        kw.update(allowMissing=True)
    elif case == "simplex_k_all":
        kw.update(algorithm="simplex")
    elif case == "wide_dt":
        t = t.astype(float).copy()
        t[7::60] += 0.5
        kw.update(E=5, dt=True)
    else:
        kw.update(k=12)
    fast = fedm.Context(0, precision=fedm.PRECISION_FAST)
    mixed = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        f = fedm.edm(t, x, ctx=fast, **kw)
        m = fedm.edm(t, x, ctx=mixed, **kw)
    finally:
        fast.close()
        mixed.close()
    assert f["rc"] == m["rc"] == 0
    assert np.array_equal(f["stats"]["rho"], m["stats"]["rho"], equal_nan=True)
    assert np.array_equal(f["predictions"], m["predictions"], equal_nan=True)


def test_mixed_fp64_operation_count(ctx):
    """The mixed kernel counts the FP64 arithmetic of its re-rank and forecast
    stage (the roofline's numerator); the exact FP64 path reports none."""
    w = workloads.ccm_config(T=3000, reps=2, n_libs=4, hi=2000)
    per = {}
    for algorithm, theta in (("simplex", 1.0), ("smap", 2.0)):
        g = fedm.edm(w["t"], w["x"], w["y"], ctx=ctx, E=4, library=w["libraries"], numReps=2, seed=w["seed"],
                     algorithm=algorithm, theta=theta)
        assert g["rc"] == 0
        tm = ctx.timing()
        per[algorithm] = tm["fp64_ops"] / tm["predictions"]
    if ctx.precision == fedm.PRECISION_FP64:
        assert per["simplex"] == 0 and per["smap"] == 0
    else:
        # simplex E=4, k=5: >= 5 rescored distances (13 ops) + 5 * 38 ops
        assert 250 <= per["simplex"] <= 1000, per
        # S-map E=4, k=6: ~25 Jacobi rotations of ~170 ops plus the normal equations
        assert 2000 <= per["smap"] <= 20000, per


@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
@pytest.mark.parametrize("form", ["one6", "fused2", "ws4", "ws8", "split"])
def test_mixed_kernel_forms_agree(form, algorithm, monkeypatch):
    """The mixed path runs in one of five kernel forms: every warp scans then
    finishes its points, with one point per thread at six CTAs per SM or two
    points per thread at two; or (S-map) 8 scan warps hand candidate lists to
    4 or 8 FP64 solver warps through shared memory; or (S-map, E_a <= 4) the
    scan writes neighbour lists that a register-resident solver kernel turns
    into forecasts on a second stream.  All give the FP64 path's bits."""
    monkeypatch.setenv("FEDM_MIXED_KERNEL", form)
    w = workloads.ccm_config(T=6000, reps=3, n_libs=5, hi=5000)
    kw = dict(E=4, library=w["libraries"], numReps=3, seed=w["seed"], algorithm=algorithm,
              theta=2.0 if algorithm == "smap" else 1.0, savePredictions=True, saveSMAPCoeffs=algorithm == "smap")
    cm = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    c64 = fedm.Context(0, precision=fedm.PRECISION_FP64)
    try:
        g = fedm.edm(w["t"], w["x"], w["y"], ctx=cm, **kw)
        tm = cm.timing()
        f = fedm.edm(w["t"], w["x"], w["y"], ctx=c64, **kw)
    finally:
        cm.close()
        c64.close()
    assert g["rc"] == f["rc"] == 0
    assert np.array_equal(g["stats"]["rho"], f["stats"]["rho"], equal_nan=True)
    assert np.array_equal(g["predictions"], f["predictions"], equal_nan=True)
    if algorithm == "smap":
        assert np.array_equal(g["coeffs"], f["coeffs"], equal_nan=True)
    if form == "split":
        assert tm["mixed_form"] == (6 if algorithm == "smap" else 1)


@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
@pytest.mark.parametrize("point_order,item_order", [("list", "lpt"), ("morton3", "interleave"),
                                                    ("morton", "lpt"), ("morton", "interleave")])
def test_lane_and_item_orders_keep_bits(point_order, item_order, algorithm, monkeypatch):
    """The one-point kernels put a work item's points on lanes in list order
    or in Morton order of three or four manifold coordinates, and take work
    items largest first or large and small alternately: scheduling only, so
    every order gives the FP64 path's bits (E = 4 and E = 2 tasks)."""
    monkeypatch.setenv("FEDM_POINT_ORDER", point_order)
    monkeypatch.setenv("FEDM_ITEM_ORDER", item_order)
    w = workloads.ccm_config(T=5000, reps=2, n_libs=4, hi=4000)
    cm = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    c64 = fedm.Context(0, precision=fedm.PRECISION_FP64)
    try:
        for E in (4, 2):
            kw = dict(E=E, library=w["libraries"], numReps=2, seed=w["seed"], algorithm=algorithm,
                      theta=2.0 if algorithm == "smap" else 1.0, savePredictions=True)
            g = fedm.edm(w["t"], w["x"], w["y"], ctx=cm, **kw)
            assert cm.timing()["mixed_form"] >= 0
            f = fedm.edm(w["t"], w["x"], w["y"], ctx=c64, **kw)
            assert g["rc"] == f["rc"] == 0
            assert np.array_equal(g["stats"]["rho"], f["stats"]["rho"], equal_nan=True), E
            assert np.array_equal(g["predictions"], f["predictions"], equal_nan=True), E
    finally:
        cm.close()
        c64.close()


@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
@pytest.mark.parametrize("k", [5, 10])
def test_spatial_scan_keeps_bits(algorithm, k, monkeypatch):
    """Libraries of 2 048 rows and more are scanned in a Morton order of
    their rows, skipping tiles no point of a work item can use.  The kept
    candidates, and so every forecast and neighbour list, are those of the
    scan in list order (FEDM_PRUNE=0); fewer pairs are scored."""
    w = workloads.ccm_config(T=24000, reps=2, n_libs=4, hi=20000)
    kw = dict(E=4, k=k, library=w["libraries"], numReps=2, seed=w["seed"], algorithm=algorithm,
              theta=2.0 if algorithm == "smap" else 1.0, savePredictions=True,
              saveSMAPCoeffs=algorithm == "smap")
    monkeypatch.setenv("FEDM_PRUNE", "0")
    plain = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    monkeypatch.delenv("FEDM_PRUNE")
    pruned = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        f = fedm.edm(w["t"], w["x"], w["y"], ctx=plain, **kw)
        tf = plain.timing()
        g = fedm.edm(w["t"], w["x"], w["y"], ctx=pruned, **kw)
        tg = pruned.timing()
        assert g["rc"] == f["rc"] == 0 and tg["mixed_form"] >= 0
        assert np.array_equal(g["stats"]["rho"], f["stats"]["rho"], equal_nan=True)
        assert np.array_equal(g["predictions"], f["predictions"], equal_nan=True)
        if algorithm == "smap":
            assert np.array_equal(g["coeffs"], f["coeffs"], equal_nan=True)
        assert tf["scanned_pairs"] == tf["distance_pairs"]
        assert 0 < tg["scanned_pairs"] < tf["scanned_pairs"]
        # coprediction: the points come from the co_x manifold, the tile
        # boxes from the library's
        co = np.roll(w["x"], 11)
        gc = fedm.edm(w["t"], w["x"], w["y"], ctx=pruned, copredict=co, saveCoPredictions=True, **kw)
        fc = fedm.edm(w["t"], w["x"], w["y"], ctx=plain, copredict=co, saveCoPredictions=True, **kw)
        assert np.array_equal(gc["copredStats"]["rho"], fc["copredStats"]["rho"], equal_nan=True)
        assert np.array_equal(gc["copredictions"], fc["copredictions"], equal_nan=True)
        # heavy ties: a series quantised to 40 levels repeats rows exactly,
        # so zero distances and equal FP32 values at the C-th slot abound
        xq = np.round(w["x"] * 40) / 40
        yq = np.round(w["y"] * 40) / 40
        gq = fedm.edm(w["t"], xq, yq, ctx=pruned, **kw)
        fq = fedm.edm(w["t"], xq, yq, ctx=plain, **kw)
        assert gq["rc"] == fq["rc"]
        assert np.array_equal(gq["stats"]["rho"], fq["stats"]["rho"], equal_nan=True)
        assert np.array_equal(gq["predictions"], fq["predictions"], equal_nan=True)
        # neighbour lists of one large task through the task seam
        a = fedm.normalise(w["t"], w["x"], w["y"], E=4, theta=1.0, algorithm=algorithm)
        lib = np.zeros(len(w["t"]), bool)
        lib[np.random.default_rng(3).choice(len(w["t"]) - 10, 15000, replace=False) + 5] = True
        pred = np.ones(len(w["t"]), bool)
        rg = pruned.run_task(a, lib, pred, 4, k)
        rf = plain.run_task(a, lib, pred, 4, k)
        for key in ("nn_idx", "kused", "predictions"):
            assert np.array_equal(rg[key], rf[key], equal_nan=True), key
        assert np.array_equal(rg["nn_dist"].view(np.int64), rf["nn_dist"].view(np.int64))
    finally:
        plain.close()
        pruned.close()


@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
@pytest.mark.parametrize("form", ["one16", "fused2"])
def test_k_up_to_16_forms_agree(form, algorithm, monkeypatch):
    """For 7 <= k <= 14 the mixed path has two forms: one point per thread
    with 16 candidate slots at four CTAs per SM, or two points per thread.
    Both give the FP64 path's bits (k = 10 and k = 14, CCM replicates)."""
    monkeypatch.setenv("FEDM_MIXED_KERNEL", form)
    w = workloads.ccm_config(T=6000, reps=3, n_libs=5, hi=5000)
    cm = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    c64 = fedm.Context(0, precision=fedm.PRECISION_FP64)
    try:
        for k in (10, 14):
            kw = dict(E=4, k=k, library=w["libraries"], numReps=3, seed=w["seed"], algorithm=algorithm,
                      theta=2.0 if algorithm == "smap" else 1.0, savePredictions=True,
                      saveSMAPCoeffs=algorithm == "smap")
            g = fedm.edm(w["t"], w["x"], w["y"], ctx=cm, **kw)
            assert cm.timing()["mixed_form"] == (5 if form == "one16" else 0)
            f = fedm.edm(w["t"], w["x"], w["y"], ctx=c64, **kw)
            assert g["rc"] == f["rc"] == 0
            assert np.array_equal(g["stats"]["rho"], f["stats"]["rho"], equal_nan=True)
            assert np.array_equal(g["predictions"], f["predictions"], equal_nan=True)
            if algorithm == "smap":
                assert np.array_equal(g["coeffs"], f["coeffs"], equal_nan=True)
    finally:
        cm.close()
        c64.close()


@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_autotuner_keeps_bits_and_its_choice(algorithm, monkeypatch):
    """With autotuning on (the default), the first batch of an (algorithm,
    E_a, k) large enough to measure times each candidate form on the same
    leading tasks (simplex: two forms, S-map: three; two rounds) and the
    context keeps the fastest; a second call reuses it without probing.  Every form gives
    the same bits, so rho, forecasts and coefficients equal a context fixed
    to one form."""
    monkeypatch.delenv("FEDM_AUTOTUNE", raising=False)
    monkeypatch.delenv("FEDM_MIXED_KERNEL", raising=False)
    w = workloads.ccm_config(T=20000, reps=8, n_libs=4, hi=15000)
    kw = dict(E=4, library=w["libraries"], numReps=8, seed=w["seed"], algorithm=algorithm,
              theta=2.0 if algorithm == "smap" else 1.0, savePredictions=True, saveSMAPCoeffs=algorithm == "smap")
    tuned = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    monkeypatch.setenv("FEDM_MIXED_KERNEL", "one6")
    fixed = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        g = fedm.edm(w["t"], w["x"], w["y"], ctx=tuned, **kw)
        t1 = tuned.timing()
        g2 = fedm.edm(w["t"], w["x"], w["y"], ctx=tuned, **kw)
        t2 = tuned.timing()
        f = fedm.edm(w["t"], w["x"], w["y"], ctx=fixed, **kw)
        tf = fixed.timing()
    finally:
        tuned.close()
        fixed.close()
    assert t1["autotune_probes"] == 2 * (3 if algorithm == "smap" else 2)  # two timed rounds
    assert t1["mixed_form"] in ((0, 1, 3) if algorithm == "smap" else (0, 1))
    assert t2["autotune_probes"] == 0 and t2["mixed_form"] == t1["mixed_form"]
    assert tf["autotune_probes"] == 0 and tf["mixed_form"] == 1
    for r in (g, g2):
        assert r["rc"] == f["rc"] == 0
        assert np.array_equal(r["stats"]["rho"], f["stats"]["rho"], equal_nan=True)
        assert np.array_equal(r["predictions"], f["predictions"], equal_nan=True)
        if algorithm == "smap":
            assert np.array_equal(r["coeffs"], f["coeffs"], equal_nan=True)
    # k = 10: the 7 <= k <= 14 candidates (two points per thread, or one with
    # 16 slots), tuned separately
    monkeypatch.delenv("FEDM_MIXED_KERNEL", raising=False)
    tuned = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        fedm.edm(w["t"], w["x"], w["y"], ctx=tuned, **dict(kw, k=10))
        t3 = tuned.timing()
    finally:
        tuned.close()
    assert t3["autotune_probes"] == 4 and t3["mixed_form"] in (0, 5)


@pytest.mark.parametrize("E", [5, 8])
@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_wide_embedding_task_bit_exact(ctx, E, algorithm):
    """Panels with dt double the embedding (E_a = 2E = 10, 16): the mixed
    path's wide kernel (one point per thread, 32 candidate slots) must give
    the oracle's neighbour lists, distances and forecasts bit for bit."""
    w = workloads.panel_config(n_panels=24, lo=80, hi=400)
    n = len(w["t"])
    rng = np.random.default_rng(E)
    kw = dict(panel=w["panel"], E=E, dt=True, algorithm=algorithm, theta=[0.5, 2.0])
    a = fedm.normalise(w["t"], w["x"], **kw)
    # rows with a complete manifold only, as run_command's usable mask: a
    # missing coordinate in the library sends the task to the exact kernels
    usable = fedm.host_usable(a, E)
    lib = (rng.uniform(size=n) < 0.5) & usable
    pred = ~lib & usable
    Ea = fedm.host_manifold(a, E).shape[1]
    assert Ea == 2 * E
    k = Ea + 1 + (algorithm == "smap")
    g = ctx.run_task(a, lib, pred, E, k)
    if ctx.precision == fedm.PRECISION_MIXED:
        assert ctx.timing()["fp64_ops"] > 0  # the mixed kernels ran
    o = edm_oracle.oracle_task(edm_oracle.normalise(w["t"], w["x"], **kw), lib, pred, E, k)
    assert g["n_pred"] > 1000
    assert np.array_equal(g["nn_idx"], o["nn_idx"])
    assert np.array_equal(g["nn_dist"].view(np.int64), o["nn_dist"].view(np.int64))
    assert np.array_equal(g["predictions"], o["predictions"], equal_nan=True)


@pytest.mark.parametrize("case", ["explore_dt_missing", "ccm_copredict"])
def test_save_manifolds(ctx, case):
    """saveManifolds (src/edm.cpp:473-475, src/r.cpp:406-409, 440-443): per
    task in task order, the library manifold (the task's library rows whose
    target is observed) and the prediction manifold (co_x lags for a
    coprediction task), missing values as NA.  easy_edm() reads
    nrow(res$Ms[[1]]) as its largest library (R/easy_edm.R:297-312).  Each
    must be the oracle's manifold for the task's masks from the task plan."""
    if case == "explore_dt_missing":
        t, x, _ = workloads.coupled_logistic(400, seed=3)
        x = x.copy()
        x[::37] = np.nan
        t = t.astype(float).copy()
        t[5::50] += 0.5  # uneven times: dt columns
        kw = dict(E=[2, 3], dt=True, allowMissing=True, saveManifolds=True, full=True)
        y = co = None
    else:
        t, x, y = workloads.coupled_logistic(600, seed=4)
        co = np.roll(x, 7)
        kw = dict(E=3, library=[50, 200], numReps=2, seed=9, copredict=co, saveManifolds=True)
    g = fedm.edm(t, x, y, ctx=ctx, **kw)
    assert g["rc"] == 0
    a = edm_oracle.normalise(t, x, y, **kw)
    plan = fedm.host_plan(a)
    assert len(g["Ms"]) == len(g["Mps"]) == len(plan["E"]) > 1
    for f in range(len(plan["E"])):
        o = edm_oracle.oracle_task(a, plan["lib"][f], plan["pred"][f], int(plan["E"][f]), int(plan["k"][f]),
                                   copredict=bool(plan["copredict"][f]))
        for got, want in ((g["Ms"][f], o["lib_manifold"]), (g["Mps"][f], o["pred_manifold"])):
            want = np.where(want == 1e100, np.nan, want)
            assert got.shape == want.shape, (f, got.shape, want.shape)
            assert np.array_equal(got, want, equal_nan=True), f
    if case == "ccm_copredict":
        assert any(plan["copredict"]) and not all(plan["copredict"])


@pytest.mark.parametrize("case", ["panels_dt_missing_extras", "reldt_p2_tau3", "xmap_copredict_p_minus1"])
def test_device_manifold_is_host_manifold(case, monkeypatch):
    """The manifolds are built on the device (manifold_kernel: lag search
    with panel boundaries and missing observations, dt columns, extras);
    FEDM_HOST_MANIFOLD=1 builds them on host threads.  The saved manifolds
    and the forecasts of the two must be the same bits."""
    rng = np.random.default_rng(11)
    if case == "panels_dt_missing_extras":
        w = workloads.panel_config(n_panels=12, lo=40, hi=200)
        t, x, y = w["t"], w["x"].copy(), None
        x[rng.uniform(size=len(x)) < 0.03] = np.nan
        kw = dict(panel=w["panel"], E=[2, 4], tau=2, dt=True, allowMissing=True, missingDistance=0.5,
                  extras=[rng.normal(size=len(t)), rng.normal(size=len(t))], algorithm="smap", theta=[0.5, 2.0])
    elif case == "reldt_p2_tau3":
        t, x, _ = workloads.coupled_logistic(900, seed=6)
        t = t.astype(float).copy()
        t[7::40] += 0.5
        y = None
        kw = dict(E=3, tau=3, p=2, reldt=True, extras=[rng.normal(size=len(t))])
    else:
        t, x, y = workloads.coupled_logistic(900, seed=7)
        kw = dict(E=3, p=-1, library=[100, 400], numReps=2, seed=3, copredict=np.roll(x, 5), savePredictions=True,
                  saveCoPredictions=True)
    kw["saveManifolds"] = True
    out = {}
    for mode in ("device", "host"):
        if mode == "host":
            monkeypatch.setenv("FEDM_HOST_MANIFOLD", "1")
        else:
            monkeypatch.delenv("FEDM_HOST_MANIFOLD", raising=False)
        c = fedm.Context(0, precision=fedm.PRECISION_MIXED)
        try:
            out[mode] = fedm.edm(t, x, y, ctx=c, **kw)
        finally:
            c.close()
    d, h = out["device"], out["host"]
    assert d["rc"] == h["rc"] == 0 and len(d["Ms"]) == len(h["Ms"]) > 0
    for f in range(len(d["Ms"])):
        for a, b in ((d["Ms"][f], h["Ms"][f]), (d["Mps"][f], h["Mps"][f])):
            assert a.shape == b.shape and np.array_equal(a, b, equal_nan=True), (case, f)
    assert np.array_equal(np.asarray(d["stats"]["rho"]), np.asarray(h["stats"]["rho"]), equal_nan=True)
    for key in ("predictions", "copredictions"):
        if d.get(key) is not None:
            assert np.array_equal(np.asarray(d[key], float), np.asarray(h[key], float), equal_nan=True)


def test_easy_edm_call_sequence(ctx):
    """The edm() calls easy_edm() makes (R/easy_edm.R:160-410), in order, on a
    coupled logistic pair: explore E = 3..10; an S-map theta sweep with
    k = Inf; S-map k = 20 with replicates; saveManifolds with full for the
    largest library; CCM over 25 library sizes with k = Inf and shuffle; a
    replicate distribution at a small library and the final library.  Replicate
    counts are reduced from easy_edm's (1000) to keep the oracle quick.  Every
    call's statistics must be the oracle's."""
    t, x, y = workloads.coupled_logistic(500, seed=21)

    def both(first, second=None, **kw):
        g = fedm.edm(t, first, second, ctx=ctx, **kw)
        o = edm_oracle.oracle_edm(t, first, second, numThreads=16, **kw)
        _stats_close(g, o)
        return g

    r = both(x, E=list(range(3, 11)))
    E_best = int(r["stats"]["E"][int(np.nanargmax(r["stats"]["rho"]))])
    thetas = list(np.linspace(0, 8, 9))
    r = both(x, E=E_best, theta=thetas, algorithm="smap", k=float("inf"))
    opt_theta = float(r["stats"]["theta"][int(np.nanargmax(r["stats"]["rho"]))])
    both(x, E=E_best, theta=0.0, numReps=8, k=20, algorithm="smap")
    both(x, E=E_best, theta=opt_theta, numReps=8, k=20, algorithm="smap")
    m = fedm.edm(t, y, ctx=ctx, E=E_best, algorithm="simplex", full=True, saveManifolds=True)
    lib_max = m["Ms"][0].shape[0]
    assert m["rc"] == 0 and lib_max > 400 and m["Ms"][0].shape[1] == E_best
    libraries = [int(v) for v in np.ceil(np.linspace(10, lib_max, 25))]
    both(y, x, E=E_best, library=libraries, algorithm="simplex", k=float("inf"), shuffle=True)
    small = max(E_best + 2, lib_max // 10)
    both(y, x, E=E_best, library=small, numReps=20, theta=opt_theta, algorithm="simplex", k=float("inf"),
         shuffle=True)
    both(y, x, E=E_best, library=lib_max, theta=opt_theta, algorithm="simplex", k=float("inf"), shuffle=True)


def test_series_kept_on_the_device_across_calls(ctx):
    """A call on the series whose manifolds a context already holds takes
    them instead of uploading and building again (the easy_edm() pattern: many
    edm() calls on one series).  Its results are the bits of the same call on a
    fresh context; a call on another series, or on the same values with other
    times, builds its own; saved manifolds from the kept buffers are the
    oracle's."""
    t, x, y = workloads.coupled_logistic(1500, seed=33)
    fresh_ctx = fedm.Context(0, precision=ctx.precision)

    def run(c, series, times=t, **kw):
        r = fedm.edm(times, series, ctx=c, **kw)
        assert r["rc"] == 0
        return r, c.timing()

    r, tm = run(ctx, x, E=[2, 3, 4, 5])
    assert tm["manifold_builds"] + tm["manifolds_reused"] == 4
    r, tm = run(ctx, x, E=3, theta=[0.5, 2.0], algorithm="smap", k=12)
    assert (tm["manifold_builds"], tm["manifolds_reused"]) == (0, 1)
    f, tf = run(fresh_ctx, x, E=3, theta=[0.5, 2.0], algorithm="smap", k=12)
    assert tf["manifold_builds"] == 1
    for key in ("rho", "mae"):
        assert np.array_equal(np.asarray(r["stats"][key]), np.asarray(f["stats"][key]), equal_nan=True)
    # another series replaces the record; going back builds again
    r, tm = run(ctx, y, E=3)
    assert (tm["manifold_builds"], tm["manifolds_reused"]) == (1, 0)
    r, tm = run(ctx, y, E=3, saveManifolds=True, full=True)
    assert (tm["manifold_builds"], tm["manifolds_reused"]) == (0, 1)
    a = edm_oracle.normalise(t, y, E=3, saveManifolds=True, full=True)
    plan = fedm.host_plan(a)
    o = edm_oracle.oracle_task(a, plan["lib"][0], plan["pred"][0], 3, int(plan["k"][0]))
    for got, want in ((r["Ms"][0], o["lib_manifold"]), (r["Mps"][0], o["pred_manifold"])):
        assert np.array_equal(got, np.where(want == 1e100, np.nan, want), equal_nan=True)
    r, tm = run(ctx, x, E=3)
    assert tm["manifold_builds"] == 1
    # the same values at other times: a gap of three steps leaves the rows
    # after it without some lags
    t1 = np.asarray(t, dtype=float).copy()
    t1[700:] += 3.0
    r, tm = run(ctx, x, times=t1, E=3)
    assert tm["manifold_builds"] == 1
    _stats_close(r, edm_oracle.oracle_edm(t1, x, E=3))
    # dt columns are a setting of their own (with regular times dt switches
    # itself off: a zero default dt weight, src/manifold.h:53-67)
    r, tm = run(ctx, x, times=t1, E=3, dt=True)
    assert tm["manifold_builds"] == 1
    _stats_close(r, edm_oracle.oracle_edm(t1, x, E=3, dt=True))
    fresh_ctx.close()


def test_task_seam_outputs_pass_reuses_only_its_own_sizes_pass():
    """fedm_run_task's sizes pass keeps its task's outputs for the outputs
    pass that follows on the same inputs (one run of the task instead of
    two).  An outputs pass on other inputs runs its own task: here the sizes
    pass is for k = 4 and the outputs pass for k = 6, whose results must be
    those of a plain k = 6 call."""
    import ctypes as C

    t, x, _ = workloads.coupled_logistic(900, seed=71)
    ctx = fedm.Context(0)
    try:
        a = fedm.normalise(t, x, E=3, theta=[0.5, 2.0])
        lib = np.zeros(900, bool)
        lib[:450] = True
        pred = ~lib
        want = ctx.run_task(a, lib, pred, 3, 6)
        keep = []
        s = fedm.make_args(a, keep)
        lr = np.ascontiguousarray(lib.astype(np.uint8))
        pr = np.ascontiguousarray(pred.astype(np.uint8))

        def io_for(k):
            io = fedm.TaskIO()
            io.library_rows, io.prediction_rows = lr.ctypes.data, pr.ctypes.data
            io.E, io.k, io.copredict, io.distance, io.force_compute = 3, k, 0, 1, 1
            return io

        lib_so = ctx.lib
        assert lib_so.fedm_run_task(ctx.h, C.byref(s), C.byref(io_for(4))) == 0
        io6 = io_for(6)
        assert lib_so.fedm_run_task(ctx.h, C.byref(s), C.byref(io6)) == 0  # sizes of k = 6 (a new task)
        np_, tot = io6.n_pred, io6.total_nn
        out = dict(predictions=np.zeros(2 * np_), coeffs=np.zeros(np_ * 4), rc=np.zeros(2 * np_, np.int32),
                   kused=np.zeros(np_, np.int32), nn_offsets=np.zeros(np_ + 1, np.int32),
                   nn_idx=np.zeros(tot, np.int32), nn_dist=np.zeros(tot), stats_rho=np.zeros(2), stats_mae=np.zeros(2))
        for key, arr in out.items():
            setattr(io6, key, arr.ctypes.data)
        # a sizes pass of another task in between: the outputs pass below must
        # not take its outputs
        assert lib_so.fedm_run_task(ctx.h, C.byref(s), C.byref(io_for(4))) == 0
        lib_so.fedm_run_task(ctx.h, C.byref(s), C.byref(io6))
        assert np.array_equal(out["predictions"].reshape(2, np_), want["predictions"])
        assert np.array_equal(out["nn_idx"], want["nn_idx"])
        assert np.array_equal(out["kused"], want["kused"])
        assert np.array_equal(out["stats_rho"], want["stats_rho"])
    finally:
        ctx.close()


def test_concurrent_contexts_share_the_gpu():
    """Two contexts driven from two host threads at once -- a simplex and an
    S-map CCM call, their mixed kernels capped at 1 and 5 resident CTAs per
    SM (fedm_set_ctas_per_sm) -- give the bits of the same calls made one
    after the other on an uncapped context."""
    import threading
    w = workloads.ccm_config(T=8000, reps=6, n_libs=5, hi=6000)
    kw = {alg: dict(E=4, library=w["libraries"], numReps=6, seed=w["seed"], algorithm=alg,
                    theta=2.0 if alg == "smap" else 1.0, savePredictions=True) for alg in ("simplex", "smap")}
    ref = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    ctxs = {alg: fedm.Context(0, precision=fedm.PRECISION_MIXED) for alg in kw}
    ctxs["simplex"].set_ctas_per_sm(1)
    ctxs["smap"].set_ctas_per_sm(5)
    try:
        want = {alg: fedm.edm(w["t"], w["x"], w["y"], ctx=ref, **kw[alg]) for alg in kw}
        got = {}

        def run(alg):
            got[alg] = fedm.edm(w["t"], w["x"], w["y"], ctx=ctxs[alg], **kw[alg])

        threads = [threading.Thread(target=run, args=(alg,)) for alg in kw]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
    finally:
        ref.close()
        for c in ctxs.values():
            c.close()
    for alg in kw:
        assert got[alg]["rc"] == want[alg]["rc"] == 0
        assert np.array_equal(got[alg]["stats"]["rho"], want[alg]["stats"]["rho"], equal_nan=True)
        assert np.array_equal(got[alg]["predictions"], want[alg]["predictions"], equal_nan=True)


def test_keep_going_stops_between_batches():
    """keep_going() (src/edm.cpp:572-591) is polled before every task batch:
    returning false stops the run with rc 1 (BREAK_HIT).  The context (its
    stream, pool and the background splitter) is usable again afterwards."""
    c = fedm.Context(0, precision=fedm.PRECISION_MIXED)
    try:
        w = workloads.ccm_config(T=6000, reps=40, n_libs=5, hi=5000)
        kw = dict(E=4, library=w["libraries"], numReps=40, seed=w["seed"], algorithm="simplex")
        polls = []

        def keep_going():
            polls.append(1)
            return len(polls) < 2  # let the first batch run, stop before the second

        c.set_keep_going(keep_going)
        r = fedm.edm(w["t"], w["x"], w["y"], ctx=c, **kw)
        assert r["rc"] == 1 and len(polls) == 2
        c.set_keep_going(None)
        r2 = fedm.edm(w["t"], w["x"], w["y"], ctx=c, **kw)
        assert r2["rc"] == 0 and len(r2["stats"]["rho"]) == 40 * 5
        o = edm_oracle.oracle_edm(w["t"], w["x"], w["y"], numThreads=16, **kw)
        _stats_close(r2, o)
    finally:
        c.close()


@pytest.mark.parametrize("levels", [6, 40])
@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_ties_and_duplicate_rows_bit_exact(ctx, levels, algorithm):
    """A series quantised to a few levels has many identical manifold rows:
    exact-zero distances (excluded, src/distances.cpp:218), more zeros than
    the mixed kernel keeps slots for (those points fall back to the exact
    kernels), and many equal distances ordered by library index
    (src/edm.cpp:652-681).  Neighbours, distances and forecasts must be the
    oracle's bits."""
    t, x, _ = workloads.coupled_logistic(3000, seed=11)
    xq = np.round(x * levels) / levels
    kw = dict(E=3, theta=[0.0, 1.5], algorithm=algorithm)
    a = fedm.normalise(t, xq, **kw)
    usable = fedm.host_usable(a, 3)
    lib = np.zeros(3000, bool)
    lib[:1800] = True
    lib, pred = lib & usable, ~lib & usable
    k = 4 + (algorithm == "smap")
    g = ctx.run_task(a, lib, pred, 3, k)
    o = edm_oracle.oracle_task(edm_oracle.normalise(t, xq, **kw), lib, pred, 3, k)
    assert np.array_equal(g["nn_idx"], o["nn_idx"])
    assert np.array_equal(g["nn_dist"].view(np.int64), o["nn_dist"].view(np.int64))
    assert np.array_equal(g["predictions"], o["predictions"], equal_nan=True)
    assert np.array_equal(g["kused"], o["kused"])
    if ctx.precision == fedm.PRECISION_MIXED:
        # uncertified points (a few hundred rows under their bound at most)
        # are all settled by the bounded re-scan
        tm = ctx.timing()
        assert tm["fallback_points"] > 0 and tm["exact_points"] == 0


@pytest.mark.parametrize("case", ["over_capacity", "wide_dt"])
@pytest.mark.parametrize("algorithm", ["simplex", "smap"])
def test_uncertified_points_bit_exact(ctx, case, algorithm):
    """Points whose FP32 candidate list cannot be certified are re-scanned
    for the rows under their certified bound, which are scored in FP64 and
    ranked (knn_refine_kernel); past 1024 such rows the point goes to the
    full exact search.  'over_capacity': a two-level series at E = 2, where
    every point has well over a thousand rows at distance zero or one level
    away, so every uncertified point takes the exact search.  'wide_dt': a
    quantised panel series with dt (E_a = 10, the wide kernel), where the
    re-scan settles every uncertified point.  Both give the oracle's bits."""
    if case == "over_capacity":
        t, x, _ = workloads.coupled_logistic(6000, seed=11)
        x = np.round(x * 2) / 2
        lib = np.zeros(6000, bool)
        lib[:4000] = True
        E, kw = 2, dict(E=2, theta=[0.0, 1.5], algorithm=algorithm)
        k = E + 1 + (algorithm == "smap")
    else:
        w = workloads.panel_config(n_panels=24, lo=80, hi=400)
        t, x = w["t"], np.round(w["x"] * 6) / 6
        lib = np.random.default_rng(5).uniform(size=len(t)) < 0.5
        E, kw = 5, dict(panel=w["panel"], E=5, dt=True, theta=[0.5, 2.0], algorithm=algorithm)
        k = 2 * E + 1 + (algorithm == "smap")
    a = fedm.normalise(t, x, **kw)
    usable = fedm.host_usable(a, E)
    lib, pred = lib & usable, ~lib & usable
    g = ctx.run_task(a, lib, pred, E, k)
    o = edm_oracle.oracle_task(edm_oracle.normalise(t, x, **kw), lib, pred, E, k)
    assert np.array_equal(g["nn_idx"], o["nn_idx"])
    assert np.array_equal(g["nn_dist"].view(np.int64), o["nn_dist"].view(np.int64))
    assert np.array_equal(g["predictions"], o["predictions"], equal_nan=True)
    assert np.array_equal(g["kused"], o["kused"])
    if ctx.precision == fedm.PRECISION_MIXED:
        tm = ctx.timing()
        assert tm["fallback_points"] > 500
        assert tm["exact_points"] == (tm["fallback_points"] if case == "over_capacity" else 0)
