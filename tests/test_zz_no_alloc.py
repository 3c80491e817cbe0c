"""The allocation-free entry point, checked against the regular one.

fedm_predict_static serves callers that cannot let the library allocate
device memory: a host application that owns a fixed device-memory budget
(its allocator owns the GPU, so an unplanned cudaMalloc fails or fragments
its pool), or a pipeline that must not hit the implicit synchronisation of
cudaMalloc/cudaFree.  It keeps its working memory in a static device array
shared by every call, so each configuration here is called twice in a row,
through the C ABI, on buffers the test owns, and must give the same
forecasts and neighbour counts as fedm_run_task (the FP64 path: identical
operations, so identical bits) both times.  The cases cover a finite k,
k >= n_lib (every valid library row, in library order), an empty library,
kused = NULL and a non-default stream; free device memory must not change
across calls.  The file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

import edm_oracle
from fedm_loader import fedm, workloads

pytestmark = pytest.mark.gpu

INT_MIN = -(2**31)


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
    lib_rows = np.array([i for i in np.nonzero(lib_mask)[0] if i + 1 < n], dtype=np.int64)
    pred_rows = np.nonzero(pred_mask)[0]
    tgt = x[lib_rows + 1] if len(lib_rows) else np.zeros(0)
    return F[lib_rows].reshape(len(lib_rows), F.shape[1]), tgt, F[pred_rows]


class _Static:
    """Device copies of one task's inputs and outputs, and the call."""

    def __init__(self, predict_static, M, tgt, Mp, thetas, with_kused):
        import torch

        dev = torch.device("cuda:0")
        self.f = predict_static
        # an empty library still passes valid (one-element) buffers
        self.dM = torch.tensor(M if len(M) else np.zeros((1, Mp.shape[1])), dtype=torch.float64, device=dev)
        self.dT = torch.tensor(tgt if len(tgt) else np.zeros(1), dtype=torch.float64, device=dev)
        self.dMp = torch.tensor(Mp, dtype=torch.float64, device=dev).contiguous()
        self.n_lib, self.n_pred, self.ea = M.shape[0], Mp.shape[0], Mp.shape[1]
        self.th = np.ascontiguousarray(np.asarray(thetas, dtype=np.float64))
        self.dP = torch.zeros(len(thetas) * self.n_pred, dtype=torch.float64, device=dev)
        self.dK = torch.zeros(self.n_pred, dtype=torch.int32, device=dev) if with_kused else None

    def __call__(self, k, algorithm, stream=None):
        import torch

        self.dP.fill_(-7.0)  # stale values must be overwritten
        if self.dK is not None:
            self.dK.fill_(-7)
        torch.cuda.synchronize()
        rc = self.f(self.dM.data_ptr(), self.dT.data_ptr(), self.n_lib, self.dMp.data_ptr(), self.n_pred, self.ea, k,
                    algorithm, self.th.ctypes.data, len(self.th), self.dP.data_ptr(),
                    None if self.dK is None else self.dK.data_ptr(),
                    None if stream is None else stream.cuda_stream)
        torch.cuda.synchronize()
        pred = self.dP.cpu().numpy().reshape(len(self.th), self.n_pred)
        kused = None if self.dK is None else self.dK.cpu().numpy()
        return rc, pred, kused


@pytest.mark.parametrize("case", ["simplex_k4", "smap_k7", "simplex_k_all", "smap_k_all", "empty_library",
                                  "no_kused", "side_stream"])
def test_static_entry_matches_run_task_twice(case):
    import torch

    lib = fedm.load()
    predict_static = _bind(lib)
    ctx = fedm.Context(0, precision=fedm.PRECISION_FP64)
    t, x, _ = workloads.coupled_logistic(700, seed=21)
    lib_mask = np.zeros(700, bool)
    lib_mask[:350] = True
    algorithm, E, k, thetas = {
        "simplex_k4": ("simplex", 3, 4, [1.0, 2.5]),
        "smap_k7": ("smap", 4, 7, [0.5]),
        "simplex_k_all": ("simplex", 2, 32, [0.0, 1.0]),
        "smap_k_all": ("smap", 3, 32, [2.0]),
        "empty_library": ("simplex", 2, 3, [1.0]),
        "no_kused": ("smap", 2, 5, [1.0, 3.0]),
        "side_stream": ("simplex", 4, 6, [1.0]),
    }[case]
    if case.endswith("k_all"):
        lib_mask[:] = False
        lib_mask[300:322] = True  # 22 library rows, fewer than k
    if case == "empty_library":
        lib_mask[:] = False
    pred_mask = ~lib_mask
    pred_mask[:10] = False
    try:
        ref = ctx.run_task(fedm.normalise(t, x, E=E, theta=thetas, algorithm=algorithm), lib_mask, pred_mask, E, k)
    finally:
        ctx.close()
    M, tgt, Mp = _task_inputs(t, x, lib_mask, pred_mask, E)
    assert M.shape[0] == ref["n_lib"] and Mp.shape[0] == ref["n_pred"]
    call = _Static(predict_static, M, tgt, Mp, thetas, with_kused=case != "no_kused")
    stream = torch.cuda.Stream() if case == "side_stream" else None
    alg = 1 if algorithm == "smap" else 0
    for _ in range(2):
        rc, pred, kused = call(k, alg, stream)
        assert rc == 0
        assert np.array_equal(pred, ref["predictions"]), case
        if kused is not None:
            assert np.array_equal(kused, ref["kused"])
    if case == "empty_library":
        assert np.all(pred == 1e100) and np.all(kused == INT_MIN)
    if case.endswith("k_all"):
        assert np.all(kused == M.shape[0])


def test_static_entry_against_oracle():
    """One S-map configuration against the CPU oracle directly (the oracle
    evaluates exp with the library's IEEE-only formula for this)."""
    lib = fedm.load()
    predict_static = _bind(lib)
    t, x, _ = workloads.coupled_logistic(900, seed=5)
    lib_mask = np.zeros(900, bool)
    lib_mask[10:500] = True  # rows with every lag observed
    pred_mask = np.zeros(900, bool)
    pred_mask[500:] = True
    E, k, thetas = 3, 5, [0.0, 1.0, 4.0]
    edm_oracle.set_exp_mode(1)
    try:
        o = edm_oracle.oracle_task(edm_oracle.normalise(t, x, E=E, theta=thetas, algorithm="smap"), lib_mask,
                                   pred_mask, E, k)
    finally:
        edm_oracle.set_exp_mode(0)
    M, tgt, Mp = _task_inputs(t, x, lib_mask, pred_mask, E)
    assert np.array_equal(M, o["lib_manifold"]) and np.array_equal(tgt, o["lib_targets"])
    call = _Static(predict_static, M, tgt, Mp, thetas, with_kused=True)
    rc, pred, kused = call(k, 1)
    assert rc == 0
    assert np.array_equal(pred, o["predictions"], equal_nan=True)
    assert np.array_equal(kused, o["kused"])


def test_static_entry_allocates_nothing():
    """After a first call, further calls leave the device's free memory
    unchanged: the entry point takes nothing from the device allocator."""
    import torch

    lib = fedm.load()
    predict_static = _bind(lib)
    t, x, _ = workloads.coupled_logistic(4000, seed=9)
    lib_mask = np.zeros(4000, bool)
    lib_mask[:2000] = True
    M, tgt, Mp = _task_inputs(t, x, lib_mask, ~lib_mask, 4)
    call = _Static(predict_static, M, tgt, Mp, [1.0, 2.0], with_kused=True)
    configs = ((6, 1), (9, 0), (32, 1), (3, 0))
    first = []
    for k, alg in configs:  # every kernel the calls use is loaded by now
        rc, pred, _ = call(k, alg)
        assert rc == 0
        first.append(pred)
    free0 = torch.cuda.mem_get_info()[0]
    for (k, alg), want in zip(configs, first):
        rc, pred, _ = call(k, alg)
        assert rc == 0
        assert torch.cuda.mem_get_info()[0] == free0
        assert np.array_equal(pred, want)


def test_static_entry_rejects_oversize():
    lib = fedm.load()
    predict_static = _bind(lib)
    th = np.array([1.0])
    big = 1 << 22  # above FEDM_STATIC_MAX_LIB; nothing is launched or read
    rc = predict_static(1, 1, big, 1, 10, 3, 4, 0, th.ctypes.data, 1, 1, None, None)
    assert rc == 908
