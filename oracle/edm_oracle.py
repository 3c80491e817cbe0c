"""Python binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

`oracle_edm` mirrors the reference's R entry `edm()` (R/edm.R:232-397): the
same argument names and defaults, the same normalisation (R/edm.R:241-322),
and a result dict shaped like the R list run_command returns
(src/r.cpp:420-457).  Only tests/, bench.py's CPU-baseline leg and
__graft_entry__.smoke() use it; the GB300 library never does.
"""
import ctypes as C
import math
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle_edm.so"
INT_MIN = -(2**31)


class OracleArgs(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("t", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p),
        ("panel", C.c_void_p), ("co_x", C.c_void_p), ("num_extras", C.c_int), ("extras", C.c_void_p),
        ("Es", C.c_void_p), ("nE", C.c_int), ("tau", C.c_int), ("thetas", C.c_void_p), ("n_thetas", C.c_int),
        ("libs", C.c_void_p), ("n_libs", C.c_int), ("k", C.c_int), ("algorithm", C.c_int),
        ("num_reps", C.c_int), ("p", C.c_int), ("crossfold", C.c_int), ("full", C.c_int),
        ("shuffle", C.c_int), ("seed", C.c_int), ("save_predictions", C.c_int),
        ("save_copredictions", C.c_int), ("save_manifolds", C.c_int), ("save_smap_coeffs", C.c_int),
        ("dt", C.c_int), ("reldt", C.c_int), ("dt_weight", C.c_double), ("allow_missing", C.c_int),
        ("missing_distance", C.c_double), ("panel_weight", C.c_double), ("panel_weights", C.c_void_p),
        ("n_panel_weights", C.c_int), ("num_threads", C.c_int), ("low_memory", C.c_int),
        ("predict_with_past", C.c_int),
    ]


class OracleResult(C.Structure):
    _fields_ = [
        ("rc", C.c_int), ("n_stats", C.c_int), ("stat_E", C.POINTER(C.c_int)),
        ("stat_library", C.POINTER(C.c_int)), ("stat_theta", C.POINTER(C.c_double)),
        ("stat_rho", C.POINTER(C.c_double)), ("stat_mae", C.POINTER(C.c_double)),
        ("n_costats", C.c_int), ("costat_E", C.POINTER(C.c_int)), ("costat_library", C.POINTER(C.c_int)),
        ("costat_theta", C.POINTER(C.c_double)), ("costat_rho", C.POINTER(C.c_double)),
        ("costat_mae", C.POINTER(C.c_double)), ("kmin", C.c_int), ("kmax", C.c_int),
        ("pred_rows", C.c_int), ("pred_cols", C.c_int), ("predictions", C.POINTER(C.c_double)),
        ("copred_rows", C.c_int), ("copred_cols", C.c_int), ("copredictions", C.POINTER(C.c_double)),
        ("coeff_rows", C.c_int), ("coeff_cols", C.c_int), ("coeffs", C.POINTER(C.c_double)),
        ("missing_distance", C.c_double), ("dt_weight", C.c_double), ("internal", C.c_void_p),
    ]


class OracleTaskIO(C.Structure):
    _fields_ = [
        ("library_rows", C.c_void_p), ("prediction_rows", C.c_void_p), ("E", C.c_int), ("k", C.c_int),
        ("copredict", C.c_int), ("distance", C.c_int), ("force_compute", C.c_int),
        ("n_pred", C.c_int), ("n_lib", C.c_int), ("e_actual", C.c_int), ("total_nn", C.c_int),
        ("predictions", C.c_void_p), ("coeffs", C.c_void_p), ("rc", C.c_void_p), ("kused", C.c_void_p),
        ("nn_offsets", C.c_void_p), ("nn_idx", C.c_void_p), ("nn_dist", C.c_void_p),
        ("stats_rho", C.c_void_p), ("stats_mae", C.c_void_p), ("lib_point_rows", C.c_void_p),
        ("pred_point_rows", C.c_void_p), ("lib_manifold", C.c_void_p), ("pred_manifold", C.c_void_p),
        ("lib_targets", C.c_void_p), ("pred_targets", C.c_void_p),
        ("missing_distance_used", C.c_double), ("dt_weight_used", C.c_double), ("aspect_ratio", C.c_double),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"oracle library missing: build it with `make -C {HERE}`")
        _lib = C.CDLL(str(LIB_PATH))
        _lib.oracle_run_command.restype = C.POINTER(OracleResult)
        _lib.oracle_run_command.argtypes = [C.POINTER(OracleArgs)]
        _lib.oracle_free_result.argtypes = [C.POINTER(OracleResult)]
        _lib.oracle_task_sizes.argtypes = [C.POINTER(OracleArgs), C.POINTER(OracleTaskIO)]
        _lib.oracle_task_run.argtypes = [C.POINTER(OracleArgs), C.POINTER(OracleTaskIO)]
        _lib.oracle_usable.argtypes = [C.POINTER(OracleArgs), C.c_int, C.c_int, C.c_void_p]
        _lib.oracle_mt_real2.argtypes = [C.c_ulonglong, C.c_longlong, C.c_void_p]
        _lib.oracle_set_exp_mode.argtypes = [C.c_int]
        _lib.oracle_set_pred_stride.argtypes = [C.c_int]
        _lib.oracle_set_sum_mode.argtypes = [C.c_int]
        _lib.oracle_emd_uniform.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _lib.oracle_emd_uniform.restype = C.c_double
        _lib.oracle_smap_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                          C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.oracle_plan.argtypes = [C.POINTER(OracleArgs), C.c_int] + [C.c_void_p] * 7
        _lib.oracle_exp.argtypes = [C.c_double]
        _lib.oracle_exp.restype = C.c_double
    return _lib


def _isnothing(v):
    return v is None or (isinstance(v, float) and math.isnan(v))


def _dvec(v, n=None):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
    if n is not None and a.shape[0] != n:
        raise ValueError("wrong length")
    return a


def _panel_ints(panel):
    p = np.asarray(panel, dtype=np.float64)
    out = np.where(np.isnan(p), INT_MIN, np.trunc(np.nan_to_num(p))).astype(np.int32)
    return np.ascontiguousarray(out)


def normalise(t, x, y=None, panel=None, E=2, tau=1, theta=1, library=None, k=0, algorithm="simplex", p=None,
              crossfold=0, full=False, shuffle=False, seed=0, copredict=None, savePredictions=False,
              saveCoPredictions=False, saveManifolds=False, saveSMAPCoeffs=False, extras=None,
              allowMissing=False, missingDistance=0.0, dt=False, reldt=False, dtWeight=0.0, numReps=1,
              panelWeight=0, panelWeights=None, verbosity=1, showProgressBar=None, numThreads=1,
              lowMemory=False, predictWithPast=False):
    """edm()'s argument handling (R/edm.R:241-322) as a dict of plain values."""
    n = len(t)
    if len(x) != n:
        raise ValueError("The time and x variables should be the same length")
    if y is not None and len(y) > 0 and len(y) != n:
        raise ValueError("The y variable is the wrong length")
    if panel is not None and len(panel) > 0 and len(panel) != n:
        raise ValueError("The panel id variable is the wrong length")
    if copredict is not None and len(copredict) > 0 and len(copredict) != n:
        raise ValueError("Coprediction vector is the wrong length")
    for e in extras or []:
        if len(e) != n:
            raise ValueError("An extra variable is not the right size")
    if numReps > 1:
        shuffle = True
    explore = y is None or len(y) == 0
    p = (1 if explore else 0) if p is None else int(p)
    k = 0 if _isnothing(k) else k
    Es = [E] if not hasattr(E, "__len__") else list(E)
    if len(Es) == 1:
        Es = [2 if _isnothing(Es[0]) else Es[0]]
    else:
        Es = [e for e in Es if not _isnothing(e)]
    k = -1 if k == math.inf else int(k)
    panelWeight = -1.0 if panelWeight == math.inf else float(panelWeight)
    thetas = [theta] if not hasattr(theta, "__len__") else list(theta)
    return dict(
        n=n, t=_dvec(t), x=_dvec(x), y=None if explore else _dvec(y),
        panel=None if panel is None or len(panel) == 0 else _panel_ints(panel),
        co_x=None if copredict is None or len(copredict) == 0 else _dvec(copredict),
        extras=[_dvec(e) for e in (extras or [])], Es=[int(e) for e in Es], tau=int(tau),
        thetas=[float(v) for v in thetas], libs=None if library is None else [int(v) for v in np.atleast_1d(library)],
        k=k, algorithm=1 if algorithm == "smap" else 0, num_reps=int(numReps), p=p, crossfold=int(crossfold),
        full=bool(full), shuffle=bool(shuffle), seed=int(seed), save_predictions=bool(savePredictions),
        save_copredictions=bool(saveCoPredictions), save_manifolds=bool(saveManifolds),
        save_smap_coeffs=bool(saveSMAPCoeffs), dt=bool(dt), reldt=bool(reldt), dt_weight=float(dtWeight),
        allow_missing=bool(allowMissing), missing_distance=float(missingDistance), panel_weight=panelWeight,
        panel_weights=None if panelWeights is None else np.asarray(panelWeights, dtype=np.float64),
        num_threads=int(numThreads), low_memory=bool(lowMemory), predict_with_past=bool(predictWithPast),
        algorithm_name=algorithm,
    )


def make_args(a, keep):
    """Packs a normalised dict into the C struct; `keep` holds the buffers."""
    def ptr(arr, dtype):
        if arr is None:
            return None
        b = np.ascontiguousarray(np.asarray(arr, dtype=dtype))
        keep.append(b)
        return b.ctypes.data

    s = OracleArgs()
    s.n = a["n"]
    s.t, s.x, s.y = ptr(a["t"], np.float64), ptr(a["x"], np.float64), ptr(a["y"], np.float64)
    s.panel = ptr(a["panel"], np.int32)
    s.co_x = ptr(a["co_x"], np.float64)
    s.num_extras = len(a["extras"])
    s.extras = ptr(np.concatenate(a["extras"]) if a["extras"] else None, np.float64)
    s.Es, s.nE = ptr(a["Es"], np.int32), len(a["Es"])
    s.tau = a["tau"]
    s.thetas, s.n_thetas = ptr(a["thetas"], np.float64), len(a["thetas"])
    s.libs = ptr(a["libs"], np.int32)
    s.n_libs = 0 if a["libs"] is None else len(a["libs"])
    for f in ("k", "algorithm", "num_reps", "p", "crossfold", "seed", "num_threads"):
        setattr(s, f, int(a[f]))
    for f in ("full", "shuffle", "save_predictions", "save_copredictions", "save_manifolds", "save_smap_coeffs",
              "dt", "reldt", "allow_missing", "low_memory", "predict_with_past"):
        setattr(s, f, int(bool(a[f])))
    s.dt_weight, s.missing_distance, s.panel_weight = a["dt_weight"], a["missing_distance"], a["panel_weight"]
    if a["panel_weights"] is not None:
        pw = np.asarray(a["panel_weights"], dtype=np.float64)
        s.panel_weights = ptr(pw.flatten(order="F"), np.float64)
        s.n_panel_weights = pw.shape[0]
    return s


def _arr(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n > 0 else np.zeros(0)


def _int_na(v):
    return None if v == INT_MIN else int(v)


def result_to_dict(r):
    out = {"rc": r.rc}
    if r.n_stats or r.n_costats or r.rc == 0:
        out["stats"] = {
            "E": _arr(r.stat_E, r.n_stats), "library": _arr(r.stat_library, r.n_stats),
            "theta": _arr(r.stat_theta, r.n_stats), "rho": _arr(r.stat_rho, r.n_stats),
            "mae": _arr(r.stat_mae, r.n_stats),
        }
        out["kMin"], out["kMax"] = _int_na(r.kmin), _int_na(r.kmax)
        if r.n_costats:
            out["copredStats"] = {
                "E": _arr(r.costat_E, r.n_costats), "library": _arr(r.costat_library, r.n_costats),
                "theta": _arr(r.costat_theta, r.n_costats), "rho": _arr(r.costat_rho, r.n_costats),
                "mae": _arr(r.costat_mae, r.n_costats),
            }
    if r.predictions:
        out["predictions"] = _arr(r.predictions, r.pred_rows * r.pred_cols).reshape(r.pred_cols, r.pred_rows).T
    if r.copredictions:
        out["copredictions"] = _arr(r.copredictions, r.copred_rows * r.copred_cols).reshape(
            r.copred_cols, r.copred_rows).T
    if r.coeffs:
        out["coeffs"] = _arr(r.coeffs, r.coeff_rows * r.coeff_cols).reshape(r.coeff_cols, r.coeff_rows).T
    if not math.isnan(r.missing_distance):
        out["missingdistance"] = r.missing_distance
    if not math.isnan(r.dt_weight):
        out["dtWeight"] = r.dt_weight
    return out


def run_command(a):
    lib = load()
    keep = []
    s = make_args(a, keep)
    rp = lib.oracle_run_command(C.byref(s))
    try:
        return result_to_dict(rp.contents)
    finally:
        lib.oracle_free_result(rp)


def oracle_edm(t, x, y=None, **kw):
    """Same call shape as the reference's R edm()."""
    return run_command(normalise(t, x, y, **kw))


def oracle_task(a, library_rows, prediction_rows, E, k, copredict=False, distance=1, force_compute=True,
                aspect_ratio=0.0):
    """One edm_task on explicit masks; returns predictions, coeffs, rc,
    neighbour lists and the manifolds (numpy arrays).  distance: 0 mean
    absolute error, 1 Euclidean, 2 Wasserstein."""
    lib = load()
    keep = []
    s = make_args(a, keep)
    n = a["n"]
    lr = np.ascontiguousarray(np.asarray(library_rows, dtype=np.uint8))
    pr = np.ascontiguousarray(np.asarray(prediction_rows, dtype=np.uint8))
    io = OracleTaskIO()
    io.library_rows, io.prediction_rows = lr.ctypes.data, pr.ctypes.data
    io.E, io.k, io.copredict, io.distance, io.force_compute = E, k, int(copredict), distance, int(force_compute)
    io.aspect_ratio = float(aspect_ratio)
    rc = lib.oracle_task_sizes(C.byref(s), C.byref(io))
    if rc:
        raise RuntimeError(f"oracle_task_sizes rc={rc}")
    npred, nlib, ea, tot = io.n_pred, io.n_lib, io.e_actual, io.total_nn
    nt = len(a["thetas"])
    out = dict(
        predictions=np.zeros(nt * npred), coeffs=np.zeros(npred * (ea + 1)), rc=np.zeros(nt * npred, np.int32),
        kused=np.zeros(npred, np.int32), nn_offsets=np.zeros(npred + 1, np.int32),
        nn_idx=np.zeros(max(tot, 1), np.int32), nn_dist=np.zeros(max(tot, 1)), stats_rho=np.zeros(nt),
        stats_mae=np.zeros(nt), lib_point_rows=np.zeros(max(nlib, 1), np.int32),
        pred_point_rows=np.zeros(max(npred, 1), np.int32), lib_manifold=np.zeros(max(nlib * ea, 1)),
        pred_manifold=np.zeros(max(npred * ea, 1)), lib_targets=np.zeros(max(nlib, 1)),
        pred_targets=np.zeros(max(npred, 1)),
    )
    for key, arr in out.items():
        setattr(io, key, arr.ctypes.data)
    task_rc = lib.oracle_task_run(C.byref(s), C.byref(io))
    out["predictions"] = out["predictions"].reshape(nt, npred)
    out["coeffs"] = out["coeffs"].reshape(npred, ea + 1)
    out["rc"] = out["rc"].reshape(nt, npred)
    out["nn_idx"] = out["nn_idx"][:tot]
    out["nn_dist"] = out["nn_dist"][:tot]
    out["lib_point_rows"] = out["lib_point_rows"][:nlib]
    out["pred_point_rows"] = out["pred_point_rows"][:npred]
    out["lib_manifold"] = out["lib_manifold"][: nlib * ea].reshape(nlib, ea)
    out["pred_manifold"] = out["pred_manifold"][: npred * ea].reshape(npred, ea)
    out["lib_targets"] = out["lib_targets"][:nlib]
    out["pred_targets"] = out["pred_targets"][:npred]
    out.update(task_rc=task_rc, n_pred=npred, n_lib=nlib, e_actual=ea,
               missing_distance=io.missing_distance_used, dt_weight=io.dt_weight_used)
    return out


def usable(a, maxE, copredict=False):
    lib = load()
    keep = []
    s = make_args(a, keep)
    u = np.zeros(a["n"], np.uint8)
    lib.oracle_usable(C.byref(s), maxE, int(copredict), u.ctypes.data)
    return u.astype(bool)


def mt_real2(seed, count):
    lib = load()
    out = np.zeros(count)
    lib.oracle_mt_real2(seed, count, out.ctypes.data)
    return out


def set_exp_mode(mode):
    """0: std::exp (the reference); 1: the GPU library's IEEE-only exp."""
    load().oracle_set_exp_mode(int(mode))


def exp_rn(x):
    return load().oracle_exp(float(x))


def plan(a):
    """configure_tasks' task list: dict of arrays plus [tasks x n] masks."""
    lib = load()
    keep = []
    s = make_args(a, keep)
    nt = C.c_int()
    lib.oracle_plan(C.byref(s), 0, C.byref(nt), None, None, None, None, None, None)
    m = nt.value
    n = a["n"]
    E, k, L, co = (np.zeros(max(m, 1), np.int32) for _ in range(4))
    lm = np.zeros((max(m, 1), n), np.uint8)
    pm = np.zeros((max(m, 1), n), np.uint8)
    lib.oracle_plan(C.byref(s), m, C.byref(nt), E.ctypes.data, k.ctypes.data, L.ctypes.data, co.ctypes.data,
                    lm.ctypes.data, pm.ctypes.data)
    return dict(E=E[:m], k=k[:m], library=L[:m], copredict=co[:m], lib=lm[:m].astype(bool), pred=pm[:m].astype(bool))


def set_sum_mode(mode):
    """Summation order of the reference's Eigen reductions and scalar loops
    (0: sequential unfused; bits 1/2: Eigen packets of 2/4; 4: fused
    products; 8: FMA-contracted scalar loops)."""
    load().oracle_set_sum_mode(int(mode))


def set_pred_stride(stride):
    """Benchmark sampling: predict every stride-th row of each prediction set."""
    load().oracle_set_pred_stride(int(stride))


def smap_grad(lib, lib_t, pred, pred_t, theta, w, backward=True):
    """CPU FP64 differentiable S-map: (mse, dtheta, dw, yhat)."""
    L = load()
    lib = np.ascontiguousarray(lib, dtype=np.float64)
    pred = np.ascontiguousarray(pred, dtype=np.float64)
    lib_t = np.ascontiguousarray(lib_t, dtype=np.float64)
    pred_t = np.ascontiguousarray(pred_t, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    E = lib.shape[1]
    mse, dth = C.c_double(), C.c_double()
    dw = np.zeros(E)
    yh = np.zeros(pred.shape[0])
    L.oracle_smap_grad(lib.ctypes.data, lib_t.ctypes.data, lib.shape[0], pred.ctypes.data, pred_t.ctypes.data,
                       pred.shape[0], E, float(theta), w.ctypes.data, C.byref(mse),
                       C.byref(dth) if backward else None, dw.ctypes.data if backward else None, yh.ctypes.data)
    return mse.value, (dth.value if backward else None), (dw if backward else None), yh


def emd_uniform(D):
    """Transport cost of the row-major cost matrix D (n1 x n2) with masses
    1/n1 and 1/n2, as the reference's Wasserstein distance takes it from
    EMD_wrap."""
    D = np.ascontiguousarray(np.asarray(D, dtype=np.float64))
    return load().oracle_emd_uniform(D.ctypes.data, D.shape[0], D.shape[1])
