"""The reference's golden test blocks (tests/testthat/test-ci.R), restated.

Each case is a function `case(edm)` taking an implementation with the call
shape of the reference's R `edm()` and asserting the same expectations the
reference asserts, against the literal values read from test-ci.R by
tests/golden/make_goldens.py.  The same cases run against the CPU oracle
(pinning it) and against the GB300 library (through its C ABI).
"""
import numpy as np

from rdata import (NA, aggregate_mean_rho, golden, logistic_map, max_abs_err_ok, r_mean, r_sd, seq, tsdiff,
                   tslag, vector)


def check_edm_result(res, rho, co_rho=None):
    """test-ci.R:35-41"""
    assert res["rc"] == 0, res["rc"]
    assert max_abs_err_ok(res["stats"]["rho"], rho), (res["stats"]["rho"], rho)
    if co_rho is not None:
        assert max_abs_err_ok(res["copredStats"]["rho"], co_rho), (res["copredStats"]["rho"], co_rho)


def check_edm_results(res1, res2, rho1, rho2):
    check_edm_result(res1, rho1)
    check_edm_result(res2, rho2)


def check_noisy(res, lo, hi, co_lo=None, co_hi=None):
    """test-ci.R:48-61"""
    assert res["rc"] == 0
    m = aggregate_mean_rho(res["stats"])
    assert np.all((np.asarray(lo) <= m) & (m <= np.asarray(hi))), (m, lo, hi)
    if co_lo is not None:
        m = aggregate_mean_rho(res["copredStats"])
        assert np.all((np.asarray(co_lo) <= m) & (m <= np.asarray(co_hi))), (m, co_lo, co_hi)


def _na(v):
    return np.isnan(np.asarray(v, dtype=float))


# ---------------------------------------------------------------- datasets
def simple_data():
    mx, my = logistic_map(500)
    x, y = mx[299:500], my[299:500]
    t = 299.0 + np.arange(1, len(x) + 1)
    return t, x, y


def missing_data():
    """test-ci.R:221-238"""
    t, x, y = simple_data()
    u = vector("missing_u")
    keep = u >= 0.1
    t, x, y, u = t[keep].copy(), x[keep].copy(), y[keep].copy(), u[keep].copy()
    x[u < 0.2] = NA
    t[np.fmod(t, 19) == 1] = NA
    return t, x, y, u


def bigger_data():
    x, y = logistic_map(100)
    t = np.arange(1, 101, dtype=float)
    return t, x, y, vector("bigger_u"), vector("bigger_u1")


def bigger_missing_data():
    """test-ci.R:319-331"""
    t, x, y, u, u1 = bigger_data()
    keep = u >= 0.1
    t, x, y, u, u1 = (a[keep].copy() for a in (t, x, y, u, u1))
    x[u < 0.2] = NA
    u1[np.fmod(t, 7) == 1] = NA
    t[np.fmod(t, 19) == 1] = NA
    return t, x, y, u, u1


def panel_data():
    x, y = logistic_map(100)
    t = np.arange(1, 101, dtype=float)
    panel = (t > 100 / 3) * 1.0
    return t, x, y, panel


# ---------------------------------------------------------------- cases
def case_no_seed(edm):
    """test-ci.R:66-78"""
    t = np.arange(1, 11, dtype=float)
    x = np.arange(1, 11, dtype=float)
    edm(t, x, shuffle=True)
    old = edm(t, x, full=True, predictWithPast=False, savePredictions=True)
    new = edm(t, x, full=True, predictWithPast=True, savePredictions=True)
    check_edm_result(old, golden(76))
    check_edm_result(new, golden(77))


def case_simple_explore(edm):
    t, x, y = simple_data()
    check_edm_result(edm(t, x, E=list(range(2, 11))), golden(93))          # :91-94
    check_edm_result(edm(t, x, full=True), golden(188))                    # :187-188
    res = edm(t, x, E=[2, 3], theta=[0, 1])                                 # :201-203
    check_edm_result(res, golden(202))
    check_edm_result(edm(t, x, lowMemory=True), golden(207))               # :206-207
    check_edm_result(edm(t, x, verbosity=1), golden(211))                  # :210-211
    check_edm_result(edm(t, x, numThreads=4), golden(215))                 # :214-215


def case_simple_xmap(edm):
    t, x, y = simple_data()
    r1, r2 = edm(t, x, y, k=5), edm(t, y, x, k=5)                          # :97-99
    check_edm_results(r1, r2, *golden(99))
    r1, r2 = edm(t, x, y, E=6, library=8), edm(t, y, x, E=6, library=8)    # :102-104
    check_edm_results(r1, r2, *golden(104))
    r1, r2 = edm(t, x, y), edm(t, y, x)                                    # :194-196
    check_edm_results(r1, r2, *golden(196))
    check_edm_result(edm(t, tslag(t, x), x), golden(184))                  # :183-184


def case_simple_crossfold(edm):
    t, x, y = simple_data()
    res = edm(t, x, k=5, crossfold=10)                                     # :107-108
    assert max_abs_err_ok(np.mean(res["stats"]["rho"]), golden(108)[0])


def case_simple_smap(edm):
    t, x, y = simple_data()
    res = edm(t, x, theta=seq(0.2, 2.0, 0.1), algorithm="smap")            # :111-113
    assert max_abs_err_ok(res["stats"]["rho"][0], golden(112)[1])
    assert max_abs_err_ok(res["stats"]["rho"][-1], golden(113)[0])
    r1 = edm(t, x, y, theta=0.2, algorithm="smap", saveSMAPCoeffs=True)    # :116-123
    r2 = edm(t, y, x, theta=0.2, algorithm="smap", saveSMAPCoeffs=True)
    check_edm_results(r1, r2, *golden(119))
    beta1 = r1["coeffs"]
    assert _na(beta1[0, :]).sum() == beta1.shape[1]
    assert _na(beta1[1:, :]).sum() == 0


def case_simple_predictions(edm):
    t, x, y = simple_data()
    u1 = vector("simple_u1")
    res = edm(t, y, x, savePredictions=True)                               # :126-132
    x2 = res["predictions"][:, 0]
    check_edm_result(res, golden(128))
    assert _na(x2[0]) and _na(x2[1:]).sum() == 0
    res = edm(t, x, copredict=y, saveCoPredictions=True)                   # :135-141
    teste = res["copredictions"][:, 0]
    check_edm_result(res, golden(137)[0], co_rho=golden(137)[1])
    assert _na(teste[0]) and _na(teste[1:]).sum() == 0
    zx = (x - r_mean(x)) / r_sd(x)                                         # :144-146
    check_edm_result(edm(t, zx, p=10), golden(146))
    check_edm_result(edm(t, y, x, p=10), golden(150))                      # :149-150
    res = edm(t, y, x, p=10, copredict=x2, saveCoPredictions=True)         # :153-159
    testx = res["copredictions"][:, 0]
    check_edm_result(res, golden(155)[0], co_rho=golden(155)[1])
    assert _na(testx[:2]).sum() == 2 and _na(testx[2:]).sum() == 0
    ok = ~np.isnan(x2)
    zx2 = (x2 - r_mean(x2[ok])) / r_sd(x2[ok])                            # :162-169
    res = edm(t, y, x, p=10, copredict=zx2, saveCoPredictions=True)
    testx2 = res["copredictions"][:, 0]
    check_edm_result(res, golden(165)[0], co_rho=golden(165)[1])
    assert _na(testx2[:2]).sum() == 2 and _na(testx2[2:]).sum() == 0
    res = edm(t, y, x, extras=[u1], p=10, copredict=zx2, saveCoPredictions=True)  # :172-178
    testx3 = res["copredictions"][:, 0]
    check_edm_result(res, golden(174)[0], co_rho=golden(174)[1])
    assert _na(testx3[:2]).sum() == 2 and _na(testx3[2:]).sum() == 0


def case_missing(edm):
    t, x, y, u = missing_data()
    check_edm_result(edm(t, x), golden(242))
    check_edm_result(edm(t, x, dt=True, saveManifolds=True, dtWeight=1), golden(246))
    check_edm_result(edm(t, x, allowMissing=True), golden(250))
    check_edm_result(edm(t, x, allowMissing=True, missingDistance=1.0), golden(254))
    r1 = edm(t, x, tslag(t, x), allowMissing=True)
    r2 = edm(t, tslag(t, x), x, allowMissing=True)
    check_edm_results(r1, r2, *golden(262))
    kw = dict(extras=[u], dt=True, algorithm="smap", saveSMAPCoeffs=True, E=5)
    r1 = edm(t, x, tslag(t, x), **kw)
    r2 = edm(t, tslag(t, x), x, **kw)
    check_edm_results(r1, r2, *golden(267))
    check_edm_result(edm(t, x, tslag(t, x, 3), **kw), golden(271))
    res = edm(t, x, extras=[u], allowMissing=True, dt=True, crossfold=5)
    assert max_abs_err_ok(np.mean(res["stats"]["rho"]), golden(275)[0])
    check_edm_result(edm(t, tsdiff(t, x), dt=True), golden(279))


def case_missing_reps(edm):
    t, x, y, u = missing_data()
    check_noisy(edm(t, x, numReps=20), *golden(283))
    r1 = edm(t, x, y, library=50, numReps=20)
    r2 = edm(t, y, x, library=50, numReps=20)
    check_noisy(r1, *golden(288))
    check_noisy(r2, *golden(289))


def case_bigger_full(edm):
    t, x, y, u, u1 = bigger_data()
    res = edm(t, x, E=2, crossfold=2, k=float("inf"), allowMissing=True)
    assert max_abs_err_ok(np.mean(res["stats"]["rho"]), golden(308)[0])
    res = edm(t, x, E=2, crossfold=10, k=float("inf"), allowMissing=True)
    assert max_abs_err_ok(np.mean(res["stats"]["rho"]), golden(313)[0])
    res = edm(t, x, E=5, extras=[tsdiff(t, y)], full=True, allowMissing=True)
    check_edm_result(res, golden(317))


def case_bigger_ccm(edm):
    t, x, y, u, u1 = bigger_missing_data()
    libs = seq(10, 70, 5)
    r1 = edm(t, x, y, allowMissing=True, dt=True, library=libs)            # :335-340
    r2 = edm(t, y, x, allowMissing=True, dt=True, library=libs)
    check_edm_results(r1, r2, golden(338), golden(339))
    check_edm_result(edm(t, x, p=-1), golden(346))
    r1, r2 = edm(t, x, y, p=-1), edm(t, y, x, p=-1)
    check_edm_results(r1, r2, *golden(351))


def case_bigger_copredict(edm):
    t, x, y, u, u1 = bigger_missing_data()
    res = edm(t, x, copredict=y)
    check_edm_result(res, golden(357)[0], co_rho=golden(357)[1])
    res = edm(t, x, copredict=y, full=True)
    check_edm_result(res, golden(361)[0], co_rho=golden(361)[1])
    r1, r2 = edm(t, x, y, copredict=u1), edm(t, y, x, copredict=u1)
    check_edm_result(r1, golden(366)[0], co_rho=golden(366)[1])
    check_edm_result(r2, golden(367)[0], co_rho=golden(367)[1])
    res = edm(t, x, E=[2, 3, 4, 5], theta=[0, 1], copredict=y)            # :372-384
    assert res["rc"] == 0
    rho, co_rho = np.array(golden(375)), np.array(golden(376))
    keep = np.arange(8) != 6
    assert np.max(np.abs(res["stats"]["rho"][keep] - rho[keep])) < 1e-4
    assert np.max(np.abs(res["copredStats"]["rho"][keep] - co_rho[keep])) < 1e-4
    r1 = edm(t, x, y, library=[5, 10, 20, 40], copredict=u1)               # :387-396
    r2 = edm(t, y, x, library=[5, 10, 20, 40], copredict=u1)
    check_edm_result(r1, golden(390), golden(391))
    check_edm_result(r2, golden(394), golden(395))


def case_bigger_reps(edm):
    t, x, y, u, u1 = bigger_missing_data()
    check_noisy(edm(t, x, copredict=y, numReps=20), *golden(400))
    r1 = edm(t, x, y, library=[5, 10, 20, 40], copredict=u1, numReps=100)
    r2 = edm(t, y, x, library=[5, 10, 20, 40], copredict=u1, numReps=100)
    check_noisy(r1, golden(406), golden(407), golden(408), golden(409))
    check_noisy(r2, golden(413), golden(414), golden(415), golden(416))


def case_panel(edm):
    t, x, y, panel = panel_data()
    inf = float("inf")
    check_edm_result(edm(t, x, panel=panel, E=40), golden(440))
    check_edm_result(edm(t, x, panel=panel, E=40, allowMissing=True), golden(444))
    check_edm_result(edm(t, x, panel=panel, E=40, panelWeight=inf), golden(448))
    check_edm_result(edm(t, x, panel=panel, E=40, panelWeight=inf, allowMissing=True), golden(452))
    for line, kw in ((457, {}), (462, dict(allowMissing=True)), (467, dict(panelWeight=inf)),
                     (472, dict(panelWeight=inf, allowMissing=True))):
        r1 = edm(t, x, y, panel=panel, E=40, **kw)
        r2 = edm(t, y, x, panel=panel, E=40, **kw)
        check_edm_results(r1, r2, *golden(line))


def case_panel_dropped(edm):
    t, x, y, panel = panel_data()
    keep = np.fmod(t, 7) != 0
    t, x, panel = t[keep], x[keep], panel[keep]
    inf = float("inf")
    for line, kw in ((495, {}), (499, dict(allowMissing=True)), (503, dict(panelWeight=inf)),
                     (507, dict(panelWeight=inf, allowMissing=True)), (511, dict(panelWeight=inf, k=inf)),
                     (517, dict(reldt=True)), (521, dict(reldt=True, allowMissing=True)),
                     (525, dict(panelWeight=inf, reldt=True)),
                     (529, dict(panelWeight=inf, reldt=True, allowMissing=True))):
        check_edm_result(edm(t, x, panel=panel, E=5, **kw), golden(line))


def case_bad_inputs(edm):
    t, x, y = simple_data()
    assert edm(t, x, y, E=NA)["rc"] == 0
    assert edm(t, x, y, E=[2, 3, NA])["rc"] == 0
    assert edm(t, x, y, k=NA)["rc"] == 0


CASES = [
    case_no_seed, case_simple_explore, case_simple_xmap, case_simple_crossfold, case_simple_smap,
    case_simple_predictions, case_missing, case_missing_reps, case_bigger_full, case_bigger_ccm,
    case_bigger_copredict, case_bigger_reps, case_panel, case_panel_dropped, case_bad_inputs,
]
