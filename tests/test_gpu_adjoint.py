"""Differentiable S-map (config 5 shape: Lorenz-63 x with noise, E = 6,
tau = 5, per-lag weights w, every library point a neighbour).

* at w = 1 the forward pass is the library's own S-map with k = all
  (fedm_run_task), up to reduction order;
* dMSE/dtheta and dMSE/dw match the CPU FP64 adjoint and central finite
  differences (h = 1e-5) of the GPU forward pass;
* gradient descent on theta lowers the MSE;
* the full size (50 000 library rows, 20 000 forecasts) runs and its
  gradient matches finite differences.
"""
import numpy as np
import pytest

import edm_oracle
from fedm_loader import fedm, workloads

pytestmark = pytest.mark.gpu
E, TAU = 6, 5


@pytest.fixture(scope="module", autouse=True)
def _device_exp():
    edm_oracle.set_exp_mode(1)
    yield
    edm_oracle.set_exp_mode(0)


@pytest.fixture(scope="module")
def ctx():
    c = fedm.Context(0, precision=fedm.PRECISION_FP64)
    yield c
    c.close()


def lorenz_sets(T, n_lib, n_pred, seed=5):
    w = workloads.lorenz_config(seed=seed, T=T)
    x = w["x"]
    a = fedm.normalise(w["t"], x, E=E, tau=TAU)
    F = fedm.host_manifold(a, E)
    first = (E - 1) * TAU
    lib_rows = np.arange(first, first + n_lib)
    pred_rows = np.arange(first + n_lib, first + n_lib + n_pred)
    return dict(x=x, t=w["t"], a=a, lib=F[lib_rows], lib_t=x[lib_rows + 1], pred=F[pred_rows], pred_t=x[pred_rows + 1],
                lib_rows=lib_rows, pred_rows=pred_rows)


@pytest.fixture(scope="module")
def small():
    return lorenz_sets(T=6000, n_lib=2500, n_pred=300)


def test_forward_matches_smap_all_neighbours(ctx, small):
    s = small
    mse, _, _, yh = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], 1.5, np.ones(E), backward=False)
    n = len(s["x"])
    lib = np.zeros(n, bool)
    lib[s["lib_rows"]] = True
    pred = np.zeros(n, bool)
    pred[s["pred_rows"]] = True
    a = fedm.normalise(s["t"], s["x"], E=E, tau=TAU, theta=1.5, algorithm="smap")
    ref = ctx.run_task(a, lib, pred, E, -1)
    assert np.allclose(yh, ref["predictions"][0], rtol=1e-9, atol=1e-12)
    assert np.isclose(mse, np.mean((ref["predictions"][0] - s["pred_t"]) ** 2), rtol=1e-9)


@pytest.mark.parametrize("theta", [0.0, 0.7, 2.5])
def test_gradient_matches_cpu_fp64(ctx, small, theta):
    s = small
    w = np.linspace(0.8, 1.3, E)
    g = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w)
    o = edm_oracle.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w)
    assert np.isclose(g[0], o[0], rtol=1e-10)
    assert np.isclose(g[1], o[1], rtol=1e-7, atol=1e-12)
    assert np.allclose(g[2], o[2], rtol=1e-7, atol=1e-12)


# Central differences of the GPU forward pass.  With h = 1e-5 the quotient is
# limited by the forward pass's own rounding (the S-map normal equations have
# cond ~1e5 here): about 1e-4 relative on dw, 1e-6 on dtheta.  h = 1e-3 is
# past that noise and agrees to ~1e-6.
@pytest.mark.parametrize("h,rtol_theta,rtol_w", [(1e-5, 2e-5, 2e-3), (1e-3, 1e-6, 2e-5)])
def test_gradient_matches_finite_differences(ctx, small, h, rtol_theta, rtol_w):
    s = small
    theta, w = 1.2, np.ones(E)
    _, gt, gw, _ = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w)

    def f(th, ww):
        return ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], th, ww, backward=False)[0]

    fd_t = (f(theta + h, w) - f(theta - h, w)) / (2 * h)
    assert np.isclose(gt, fd_t, rtol=rtol_theta, atol=1e-13), (gt, fd_t)
    for j in range(E):
        e = np.zeros(E)
        e[j] = h
        fd = (f(theta, w + e) - f(theta, w - e)) / (2 * h)
        assert np.isclose(gw[j], fd, rtol=rtol_w, atol=1e-12), (j, gw[j], fd)


def test_objective_entry_mse_is_the_backward_pass(ctx, small):
    s = small
    w = np.linspace(0.9, 1.2, E)
    m, gt, gw, _ = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], 0.8, w)
    v, vt, vw, yh = ctx.smap_objective_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], 0.8, w, "mse")
    assert v == m and vt == gt and np.array_equal(vw, gw)
    assert np.isclose(v, np.mean((yh - s["pred_t"]) ** 2), rtol=1e-12)


def test_rho_objective_value(ctx, small):
    """rho of the forecasts against the targets, by the reference's
    centred-sum formula (src/stats.cpp:64-80)."""
    s = small
    v, _, _, yh = ctx.smap_objective_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], 1.5, np.ones(E), "rho")
    a, b = yh - yh.mean(), s["pred_t"] - s["pred_t"].mean()
    assert np.isclose(v, np.sum(a * b) / (np.sqrt(np.sum(a * a)) * np.sqrt(np.sum(b * b))), rtol=1e-12)
    assert 0.5 < v < 1.0


@pytest.mark.parametrize("theta", [0.3, 2.0])
def test_rho_gradient_matches_finite_differences(ctx, small, theta):
    """drho/dtheta and drho/dw from the adjoint (drho/dyhat composed on the
    host with the kernel's dyhat/d(.)) against central differences of the
    forward pass, h = 1e-3 (past the forward pass's rounding noise)."""
    s = small
    w = np.linspace(0.8, 1.3, E)
    _, gt, gw, _ = ctx.smap_objective_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w, "rho")

    def f(th, ww):
        return ctx.smap_objective_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], th, ww, "rho")[0]

    h = 1e-3
    fd_t = (f(theta + h, w) - f(theta - h, w)) / (2 * h)
    assert np.isclose(gt, fd_t, rtol=1e-4, atol=1e-9), (gt, fd_t)
    for j in range(E):
        e = np.zeros(E)
        e[j] = h
        fd = (f(theta, w + e) - f(theta, w - e)) / (2 * h)
        assert np.isclose(gw[j], fd, rtol=1e-3, atol=1e-8), (j, gw[j], fd)


def test_gradient_descent_on_theta(ctx, small):
    s = small
    w = np.ones(E)
    theta = 0.0
    m0, g, _, _ = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w)
    m = m0
    lr = 0.5 / max(abs(g), 1e-12) * 0.1
    for _ in range(15):
        m_new, g, _, _ = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w)
        if m_new > m + 1e-15:
            lr *= 0.5
        m = m_new
        theta = max(0.0, theta - lr * g)
    assert m < m0, (m, m0, theta)


def test_full_size_gradient(ctx):
    s = lorenz_sets(T=100000, n_lib=50000, n_pred=20000)
    theta, w = 1.0, np.ones(E)
    mse, gt, gw, _ = ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], theta, w)
    tm = ctx.timing()
    assert np.isfinite(mse) and np.isfinite(gt) and np.all(np.isfinite(gw))
    h = 1e-5
    f = lambda th: ctx.smap_grad(s["lib"], s["lib_t"], s["pred"], s["pred_t"], th, w, backward=False)[0]
    fd = (f(theta + h) - f(theta - h)) / (2 * h)
    assert np.isclose(gt, fd, rtol=1e-4, atol=1e-13), (gt, fd)
    print(f"full-size differentiable S-map: {tm['device_ms']:.1f} ms forward+backward")


@pytest.mark.parametrize("e_actual", [2, 6, 8])
def test_cache_levels_give_the_same_bits(e_actual, monkeypatch):
    """The kernel keeps each point's per-row values in a per-warp cache
    (level 2: distances, weights, reciprocals and per-lag products; level 1:
    distances and weights; level 0: none, every pass recomputes).  The cached
    values are the ones the passes recompute: every level gives the same
    bits for the forecasts, the MSE and its gradient."""
    w = workloads.lorenz_config(seed=8, T=8000)
    a = fedm.normalise(w["t"], w["x"], E=e_actual, tau=3)
    F = fedm.host_manifold(a, e_actual)
    first = (e_actual - 1) * 3
    lib_rows = np.arange(first, first + 3000)
    pred_rows = np.arange(first + 3000, first + 3700)
    lib, lib_t = F[lib_rows], w["x"][lib_rows + 1]
    pred, pred_t = F[pred_rows], w["x"][pred_rows + 1]
    wv = np.linspace(0.7, 1.4, e_actual)
    out = {}
    for level in (2, 1, 0):
        monkeypatch.setenv("FEDM_GRAD_CACHE", str(level))
        c = fedm.Context(0, precision=fedm.PRECISION_FP64)
        try:
            mse, gt, gw, _ = c.smap_grad(lib, lib_t, pred, pred_t, 1.5, wv)
            assert c.timing()["grad_cache_level"] == level
            _, _, _, yh = c.smap_grad(lib, lib_t, pred, pred_t, 1.5, wv, backward=False)
        finally:
            c.close()
        out[level] = np.concatenate([[mse, gt], gw, yh]).view(np.int64)
    assert np.array_equal(out[2], out[1]) and np.array_equal(out[2], out[0])
