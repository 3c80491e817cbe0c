"""The allocation-free entry point, checked against the regular one.

fedm_predict_static serves callers that cannot let the library allocate
device memory (a fixed device-memory budget owned by the host application,
or a pipeline that must not hit the implicit synchronisation of
cudaMalloc/cudaFree).  It keeps its working memory in a static device array,
so this test calls it twice in a row, through the C ABI, on buffers the test
owns, and requires the same forecasts and neighbour counts as fedm_run_task
(the FP64 path: identical operations, so identical bits).  It lives in a file
of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from fedm_loader import fedm, workloads

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.fedm_predict_static
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                  C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _task_inputs(t, x, lib_mask, pred_mask, E):
    """Library rows with an observed one-step target, their targets, and the
    prediction rows, from the library's own host manifold."""
    a = fedm.normalise(t, x, E=E)
    F = fedm.host_manifold(a, E)
    n = len(t)
    lib_rows = [i for i in np.nonzero(lib_mask)[0] if i + 1 < n]
    pred_rows = list(np.nonzero(pred_mask)[0])
    return F[lib_rows], x[np.array(lib_rows) + 1], F[pred_rows]


def test_static_entry_matches_run_task_twice():
    import torch

    lib = fedm.load()
    predict_static = _bind(lib)
    ctx = fedm.Context(0, precision=fedm.PRECISION_FP64)
    t, x, _ = workloads.coupled_logistic(700, seed=21)
    lib_mask = np.zeros(700, bool)
    lib_mask[:350] = True
    pred_mask = ~lib_mask
    pred_mask[:10] = False
    calls = [("simplex", 3, 4, [1.0, 2.5]), ("smap", 4, 7, [0.5]), ("simplex", 2, 3, [0.0])]
    for algorithm, E, k, thetas in calls:
        ref = ctx.run_task(fedm.normalise(t, x, E=E, theta=thetas, algorithm=algorithm), lib_mask, pred_mask, E, k)
        M, tgt, Mp = _task_inputs(t, x, lib_mask, pred_mask, E)
        assert M.shape[0] == ref["n_lib"] and Mp.shape[0] == ref["n_pred"]
        dev = torch.device("cuda:0")
        dM = torch.tensor(M, dtype=torch.float64, device=dev).contiguous()
        dT = torch.tensor(tgt, dtype=torch.float64, device=dev).contiguous()
        dMp = torch.tensor(Mp, dtype=torch.float64, device=dev).contiguous()
        dP = torch.zeros(len(thetas) * Mp.shape[0], dtype=torch.float64, device=dev)
        dK = torch.zeros(Mp.shape[0], dtype=torch.int32, device=dev)
        th = np.ascontiguousarray(np.asarray(thetas, dtype=np.float64))
        torch.cuda.synchronize()
        rc = predict_static(dM.data_ptr(), dT.data_ptr(), M.shape[0], dMp.data_ptr(), Mp.shape[0], M.shape[1], k,
                            1 if algorithm == "smap" else 0, th.ctypes.data, len(thetas), dP.data_ptr(),
                            dK.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == 0
        pred = dP.cpu().numpy().reshape(len(thetas), Mp.shape[0])
        assert np.array_equal(pred, ref["predictions"]), (algorithm, E, k)
        assert np.array_equal(dK.cpu().numpy(), ref["kused"])
    ctx.close()


def test_static_entry_rejects_oversize():
    lib = fedm.load()
    predict_static = _bind(lib)
    th = np.array([1.0])
    big = 1 << 22  # above FEDM_STATIC_MAX_LIB; nothing is launched or read
    rc = predict_static(1, 1, big, 1, 10, 3, 4, 0, th.ctypes.data, 1, 1, None, None)
    assert rc == 908
