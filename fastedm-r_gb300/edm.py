"""Python binding of libfastedm_gb300.so with the call shape of fastEDM's R API.

`edm()` takes the reference's R arguments (R/edm.R:232-238), applies the
same normalisation (R/edm.R:241-322) and returns the list run_command returns
(src/r.cpp:420-457) as a dict, computed on the GPU through the C ABI
(include/fastedm_gb300.h).  There is no CPU fallback: without the built
library or a CUDA device every call raises.
"""
import ctypes as C
import math
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libfastedm_gb300.so"
INT_MIN = -(2**31)

PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_FAST = 2


class Args(C.Structure):
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


class Result(C.Structure):
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
        ("n_manifolds", C.c_int), ("manifold_rows", C.POINTER(C.c_int)),
        ("pred_manifold_rows", C.POINTER(C.c_int)), ("manifold_cols", C.POINTER(C.c_int)),
        ("manifolds", C.POINTER(C.c_double)), ("pred_manifolds", C.POINTER(C.c_double)),
    ]


class TaskIO(C.Structure):
    _fields_ = [
        ("library_rows", C.c_void_p), ("prediction_rows", C.c_void_p), ("E", C.c_int), ("k", C.c_int),
        ("copredict", C.c_int), ("distance", C.c_int), ("force_compute", C.c_int),
        ("n_pred", C.c_int), ("n_lib", C.c_int), ("e_actual", C.c_int), ("total_nn", C.c_int),
        ("predictions", C.c_void_p), ("coeffs", C.c_void_p), ("rc", C.c_void_p), ("kused", C.c_void_p),
        ("nn_offsets", C.c_void_p), ("nn_idx", C.c_void_p), ("nn_dist", C.c_void_p),
        ("stats_rho", C.c_void_p), ("stats_mae", C.c_void_p), ("aspect_ratio", C.c_double),
    ]


class Timing(C.Structure):
    _fields_ = [
        ("device_ms", C.c_double), ("knn_kernel_ms", C.c_double), ("knn_launches", C.c_int),
        ("host_ms", C.c_double), ("distance_pairs", C.c_longlong), ("predictions", C.c_longlong),
        ("h2d_bytes", C.c_longlong), ("d2h_bytes", C.c_longlong), ("fallback_points", C.c_int),
        ("kernel_launches", C.c_int), ("fp64_ops", C.c_longlong), ("list_wait_ms", C.c_double),
        ("setup_ms", C.c_double), ("finish_ms", C.c_double), ("exact_points", C.c_int),
        ("mixed_form", C.c_int), ("autotune_probes", C.c_int), ("prep_ms", C.c_double),
        ("manifold_ms", C.c_double), ("scan_flops", C.c_longlong), ("forecast_kernel_ms", C.c_double),
        ("forecast_launches", C.c_int), ("tensor_core_tiles", C.c_int), ("manifold_builds", C.c_int),
        ("manifolds_reused", C.c_int), ("scanned_pairs", C.c_longlong), ("grad_cache_level", C.c_int),
    ]


EXPORTS = [
    "fedm_create", "fedm_destroy", "fedm_last_error", "fedm_set_precision", "fedm_set_ctas_per_sm",
    "fedm_set_keep_going",
    "fedm_run_command", "fedm_free_result", "fedm_run_task", "fedm_last_timing", "fedm_measure_peak",
    "fedm_host_usable", "fedm_host_manifold", "fedm_host_mt_real2", "fedm_host_plan",
    "fedm_smap_fwd", "fedm_smap_bwd", "fedm_smap_grad", "fedm_predict_static",
]

_lib = None


def load():
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run fastedm-r_gb300/build.py")
        lib = C.CDLL(str(LIB_PATH))
        lib.fedm_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
        lib.fedm_destroy.argtypes = [C.c_void_p]
        lib.fedm_last_error.argtypes = [C.c_void_p]
        lib.fedm_last_error.restype = C.c_char_p
        lib.fedm_set_precision.argtypes = [C.c_void_p, C.c_int]
        lib.fedm_set_ctas_per_sm.argtypes = [C.c_void_p, C.c_int]
        lib.fedm_set_keep_going.argtypes = [C.c_void_p, C.CFUNCTYPE(C.c_int)]
        lib.fedm_run_command.argtypes = [C.c_void_p, C.POINTER(Args), C.POINTER(C.POINTER(Result))]
        lib.fedm_free_result.argtypes = [C.POINTER(Result)]
        lib.fedm_run_task.argtypes = [C.c_void_p, C.POINTER(Args), C.POINTER(TaskIO)]
        lib.fedm_last_timing.argtypes = [C.c_void_p, C.POINTER(Timing)]
        lib.fedm_measure_peak.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        grad_args = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                     C.c_double, C.c_void_p, C.POINTER(C.c_double)]
        lib.fedm_smap_fwd.argtypes = grad_args + [C.c_void_p]
        lib.fedm_smap_bwd.argtypes = grad_args + [C.POINTER(C.c_double), C.c_void_p]
        lib.fedm_smap_grad.argtypes = grad_args[:-1] + [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                        C.c_void_p, C.c_void_p]
        lib.fedm_host_usable.argtypes = [C.POINTER(Args), C.c_int, C.c_int, C.c_void_p]
        lib.fedm_host_manifold.argtypes = [C.POINTER(Args), C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int)]
        lib.fedm_host_mt_real2.argtypes = [C.c_ulonglong, C.c_longlong, C.c_void_p]
        lib.fedm_host_plan.argtypes = [C.POINTER(Args), C.c_int, C.POINTER(C.c_int)] + [C.c_void_p] * 6
        _lib = lib
    return _lib


class Context:
    """One GPU context (stream + memory pool) of the library."""

    def __init__(self, device=0, precision=PRECISION_MIXED):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.fedm_create(device, C.byref(h))
        if rc != 0 or not h.value:
            raise RuntimeError(f"fedm_create failed (rc={rc}): no usable CUDA device {device}")
        self.h = h
        self.set_precision(precision)

    def set_keep_going(self, fn):
        """fn() -> bool is polled between GPU batches; returning False stops
        the run with rc 1 (BREAK_HIT), like the reference's keep_going()."""
        proto = C.CFUNCTYPE(C.c_int)
        # a NULL function pointer clears the callback
        self._keep_going = proto() if fn is None else proto(lambda: 1 if fn() else 0)
        self.lib.fedm_set_keep_going(self.h, self._keep_going)

    def set_precision(self, precision):
        if self.lib.fedm_set_precision(self.h, precision) != 0:
            raise ValueError("bad precision")
        self.precision = precision

    def set_ctas_per_sm(self, ctas):
        """Caps the mixed kernels' resident CTAs per SM (0: no cap), so that
        calls on other contexts from other threads can share the SMs."""
        if self.lib.fedm_set_ctas_per_sm(self.h, int(ctas)) != 0:
            raise ValueError("bad CTA count")

    def close(self):
        if self.h:
            self.lib.fedm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self):
        return self.lib.fedm_last_error(self.h).decode()

    def timing(self):
        t = Timing()
        self.lib.fedm_last_timing(self.h, C.byref(t))
        return {f: getattr(t, f) for f, _ in Timing._fields_}

    def measure_peak(self, kind):
        """TFLOP/s of kind 0 FP32 FFMA, 1 FP64 DFMA, 2 packed FP32 FFMA2,
        3 FP64 DMUL/DADD without fusion (one flop per instruction)."""
        v = C.c_double()
        if self.lib.fedm_measure_peak(self.h, kind, C.byref(v)) != 0:
            raise RuntimeError(self.last_error())
        return v.value

    def smap_grad(self, lib, lib_t, pred, pred_t, theta, w, backward=True):
        """Differentiable S-map over every library neighbour with per-lag
        weights w: (mse, dmse/dtheta, dmse/dw, predictions)."""
        arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (lib, lib_t, pred, pred_t, w)]
        lib, lib_t, pred, pred_t, w = arrs
        E = lib.shape[1]
        mse = C.c_double()
        if backward:
            dth = C.c_double()
            dw = np.zeros(E)
            rc = self.lib.fedm_smap_bwd(self.h, lib.ctypes.data, lib_t.ctypes.data, lib.shape[0], pred.ctypes.data,
                                        pred_t.ctypes.data, pred.shape[0], E, float(theta), w.ctypes.data,
                                        C.byref(mse), C.byref(dth), dw.ctypes.data)
            if rc != 0:
                raise RuntimeError(f"fedm_smap_bwd rc={rc}: {self.last_error()}")
            return mse.value, dth.value, dw, None
        yh = np.zeros(pred.shape[0])
        rc = self.lib.fedm_smap_fwd(self.h, lib.ctypes.data, lib_t.ctypes.data, lib.shape[0], pred.ctypes.data,
                                    pred_t.ctypes.data, pred.shape[0], E, float(theta), w.ctypes.data, C.byref(mse),
                                    yh.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"fedm_smap_fwd rc={rc}: {self.last_error()}")
        return mse.value, None, None, yh

    def smap_objective_grad(self, lib, lib_t, pred, pred_t, theta, w, objective="mse"):
        """The same pass for a chosen objective, "mse" or "rho" (forecasts
        against targets): (value, dvalue/dtheta, dvalue/dw, predictions)."""
        arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (lib, lib_t, pred, pred_t, w)]
        lib, lib_t, pred, pred_t, w = arrs
        E = lib.shape[1]
        val, dth = C.c_double(), C.c_double()
        dw = np.zeros(E)
        yh = np.zeros(pred.shape[0])
        obj = {"mse": 0, "rho": 1}[objective]
        rc = self.lib.fedm_smap_grad(self.h, lib.ctypes.data, lib_t.ctypes.data, lib.shape[0], pred.ctypes.data,
                                     pred_t.ctypes.data, pred.shape[0], E, float(theta), w.ctypes.data, obj,
                                     C.byref(val), C.byref(dth), dw.ctypes.data, yh.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"fedm_smap_grad rc={rc}: {self.last_error()}")
        return val.value, dth.value, dw, yh

    def run_command(self, a):
        keep = []
        s = make_args(a, keep)
        out = C.POINTER(Result)()
        self.lib.fedm_run_command(self.h, C.byref(s), C.byref(out))
        if not out:
            raise RuntimeError("fedm_run_command returned no result")
        try:
            d = result_to_dict(out.contents)
        finally:
            self.lib.fedm_free_result(out)
        if d["rc"] not in (0, 1) and "stats" not in d:
            d["error"] = self.last_error()
        return d

    def run_task(self, a, library_rows, prediction_rows, E, k, copredict=False, distance=1, force_compute=True,
                 aspect_ratio=0.0):
        """One task on explicit masks; neighbour lists included.  distance: 0
        mean absolute error, 1 Euclidean, 2 Wasserstein (aspect_ratio weights
        its time axis under dt)."""
        keep = []
        s = make_args(a, keep)
        lr = np.ascontiguousarray(np.asarray(library_rows, dtype=np.uint8))
        pr = np.ascontiguousarray(np.asarray(prediction_rows, dtype=np.uint8))
        io = TaskIO()
        io.library_rows, io.prediction_rows = lr.ctypes.data, pr.ctypes.data
        io.E, io.k, io.copredict, io.distance, io.force_compute = E, k, int(copredict), distance, int(force_compute)
        io.aspect_ratio = float(aspect_ratio)
        rc = self.lib.fedm_run_task(self.h, C.byref(s), C.byref(io))
        if rc not in (0, 503, 8000) or (rc and io.n_pred == 0 and io.n_lib == 0):
            raise RuntimeError(f"fedm_run_task sizes rc={rc}: {self.last_error()}")
        npred, nlib, ea, tot = io.n_pred, io.n_lib, io.e_actual, io.total_nn
        nt = len(a["thetas"])
        out = dict(
            predictions=np.zeros(max(nt * npred, 1)), coeffs=np.zeros(max(npred * (ea + 1), 1)),
            rc=np.zeros(max(nt * npred, 1), np.int32), kused=np.zeros(max(npred, 1), np.int32),
            nn_offsets=np.zeros(npred + 1, np.int32), nn_idx=np.zeros(max(tot, 1), np.int32),
            nn_dist=np.zeros(max(tot, 1)), stats_rho=np.zeros(nt), stats_mae=np.zeros(nt),
        )
        for key, arr in out.items():
            setattr(io, key, arr.ctypes.data)
        task_rc = self.lib.fedm_run_task(self.h, C.byref(s), C.byref(io))
        out["predictions"] = out["predictions"][: nt * npred].reshape(nt, npred)
        out["coeffs"] = out["coeffs"][: npred * (ea + 1)].reshape(npred, ea + 1)
        out["rc"] = out["rc"][: nt * npred].reshape(nt, npred)
        out["kused"] = out["kused"][:npred]
        out["nn_idx"] = out["nn_idx"][:tot]
        out["nn_dist"] = out["nn_dist"][:tot]
        out.update(task_rc=task_rc, n_pred=npred, n_lib=nlib, e_actual=ea)
        return out


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _isnothing(v):
    return v is None or (isinstance(v, float) and math.isnan(v))


def _dvec(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64))


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
    """edm()'s argument handling (R/edm.R:241-322)."""
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
        thetas=[float(v) for v in thetas],
        libs=None if library is None else [int(v) for v in np.atleast_1d(library)],
        k=k, algorithm=1 if algorithm == "smap" else (0 if algorithm == "simplex" else 99),
        num_reps=int(numReps), p=p, crossfold=int(crossfold), full=bool(full), shuffle=bool(shuffle),
        seed=int(seed), save_predictions=bool(savePredictions), save_copredictions=bool(saveCoPredictions),
        save_manifolds=bool(saveManifolds), save_smap_coeffs=bool(saveSMAPCoeffs), dt=bool(dt),
        reldt=bool(reldt), dt_weight=float(dtWeight), allow_missing=bool(allowMissing),
        missing_distance=float(missingDistance), panel_weight=panelWeight,
        panel_weights=None if panelWeights is None else np.asarray(panelWeights, dtype=np.float64),
        num_threads=int(numThreads), low_memory=bool(lowMemory), predict_with_past=bool(predictWithPast),
    )


def make_args(a, keep):
    def ptr(arr, dtype):
        if arr is None:
            return None
        b = np.ascontiguousarray(np.asarray(arr, dtype=dtype))
        keep.append(b)
        return b.ctypes.data

    s = Args()
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


def result_to_dict(r):
    out = {"rc": r.rc}
    if r.n_stats or r.n_costats or r.rc == 0:
        out["stats"] = {
            "E": _arr(r.stat_E, r.n_stats), "library": _arr(r.stat_library, r.n_stats),
            "theta": _arr(r.stat_theta, r.n_stats), "rho": _arr(r.stat_rho, r.n_stats),
            "mae": _arr(r.stat_mae, r.n_stats),
        }
        out["kMin"] = None if r.kmin == INT_MIN else int(r.kmin)
        out["kMax"] = None if r.kmax == INT_MIN else int(r.kmax)
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
    if r.n_manifolds:
        # saveManifolds: per task the library (Ms) and prediction (Mps)
        # manifolds, row-major blocks in task order
        rows, prows, cols = (_arr(v, r.n_manifolds) for v in (r.manifold_rows, r.pred_manifold_rows,
                                                              r.manifold_cols))
        man = _arr(r.manifolds, int(np.sum(rows * cols)))
        pman = _arr(r.pred_manifolds, int(np.sum(prows * cols)))
        out["Ms"], out["Mps"] = [], []
        o1 = o2 = 0
        for nr, npr, nc in zip(rows, prows, cols):
            out["Ms"].append(man[o1:o1 + nr * nc].reshape(nr, nc))
            out["Mps"].append(pman[o2:o2 + npr * nc].reshape(npr, nc))
            o1 += nr * nc
            o2 += npr * nc
    if not math.isnan(r.missing_distance):
        out["missingdistance"] = r.missing_distance
    if not math.isnan(r.dt_weight):
        out["dtWeight"] = r.dt_weight
    return out


def edm(t, x, y=None, ctx=None, **kw):
    """The reference's R edm(), on the GPU."""
    ctx = ctx or default_context()
    return ctx.run_command(normalise(t, x, y, **kw))


# ---------------------------------------------------------------- host side
def host_usable(a, maxE, copredict=False):
    lib = load()
    keep = []
    s = make_args(a, keep)
    u = np.zeros(a["n"], np.uint8)
    if lib.fedm_host_usable(C.byref(s), maxE, int(copredict), u.ctypes.data) != 0:
        raise RuntimeError("fedm_host_usable failed")
    return u.astype(bool)


def host_manifold(a, E, copredict=False):
    """Manifold rows of every observation, [n x E_actual]."""
    lib = load()
    keep = []
    s = make_args(a, keep)
    ea = C.c_int()
    lib.fedm_host_manifold(C.byref(s), E, int(copredict), None, C.byref(ea))
    out = np.zeros((a["n"], ea.value))
    if lib.fedm_host_manifold(C.byref(s), E, int(copredict), out.ctypes.data, C.byref(ea)) != 0:
        raise RuntimeError("fedm_host_manifold failed")
    return out


def host_mt_real2(seed, count):
    out = np.zeros(count)
    load().fedm_host_mt_real2(seed, count, out.ctypes.data)
    return out


def host_plan(a):
    lib = load()
    keep = []
    s = make_args(a, keep)
    nt = C.c_int()
    lib.fedm_host_plan(C.byref(s), 0, C.byref(nt), None, None, None, None, None, None)
    m, n = nt.value, a["n"]
    E, k, L, co = (np.zeros(max(m, 1), np.int32) for _ in range(4))
    lm = np.zeros((max(m, 1), n), np.uint8)
    pm = np.zeros((max(m, 1), n), np.uint8)
    lib.fedm_host_plan(C.byref(s), m, C.byref(nt), E.ctypes.data, k.ctypes.data, L.ctypes.data, co.ctypes.data,
                       lm.ctypes.data, pm.ctypes.data)
    return dict(E=E[:m], k=k[:m], library=L[:m], copredict=co[:m], lib=lm[:m].astype(bool), pred=pm[:m].astype(bool))
