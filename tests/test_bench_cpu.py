"""CPU check of bench.py's output contract: with the library context and the
CPU sample replaced by fakes (no GPU here), every mode prints one JSON line
carrying the keys the benchmark line must have."""
import io
import json
import sys
import types
from contextlib import redirect_stdout
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


class FakeContext:
    def __init__(self, device=0, precision=1):
        self.precision = precision

    def set_ctas_per_sm(self, ctas):
        self.ctas = ctas

    def measure_peak(self, kind):
        return {0: 78.0, 1: 1.05, 2: 65.0, 3: 0.53}[kind]

    def run_command(self, args):
        n = len(args["Es"]) * len(args["thetas"])
        out = {"rc": 0, "stats": {"rho": np.linspace(0.1, 0.9, n), "E": np.repeat(args["Es"], len(args["thetas"])),
                                  "theta": np.tile(args["thetas"], len(args["Es"]))}}
        if args["save_manifolds"]:
            out["Ms"] = [np.zeros((args["n"] // 2, args["Es"][0]))]
        return out

    def run_task(self, *a, **k):
        return {}

    def smap_grad(self, *a, **k):
        return 0.0, 0.0, np.zeros(6), None

    def timing(self):
        return dict(device_ms=100.0, knn_kernel_ms=90.0, knn_launches=1, host_ms=101.0, distance_pairs=10**9,
                    predictions=10**6, h2d_bytes=1000, d2h_bytes=100, fallback_points=3, kernel_launches=10,
                    fp64_ops=10**10, list_wait_ms=1.0, setup_ms=2.0, finish_ms=0.5, exact_points=1, mixed_form=1,
                    autotune_probes=0, prep_ms=0.3, manifold_ms=0.2, scan_flops=12 * 10**9,
                    forecast_kernel_ms=80.0, forecast_launches=1, tensor_core_tiles=0, manifold_builds=1,
                    manifolds_reused=0, scanned_pairs=4 * 10**8, grad_cache_level=0)

    def close(self):
        pass


class FakeClocks:
    def __init__(self, device):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def summary(self):
        return {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 1}


@pytest.fixture()
def bench(monkeypatch):
    import bench as b

    fedm, workloads = b.load_pkg()
    fake = types.SimpleNamespace(**{k: getattr(fedm, k) for k in dir(fedm) if not k.startswith("__")})
    fake.Context = FakeContext
    fake.edm = lambda t, x, y=None, ctx=None, **kw: ctx.run_command(fedm.normalise(t, x, y, **kw))
    fake.host_manifold = lambda a, E, copredict=False: np.zeros((a["n"], E))
    monkeypatch.setattr(b, "load_pkg", lambda: (fake, workloads))
    monkeypatch.setattr(b, "flush_l2", lambda d: None)
    monkeypatch.setattr(b, "Clocks", FakeClocks)
    sample = {"value": 3.0e4, "unit": "predictions/s", "cores": 16, "kind": "port", "sample": "fake"}
    monkeypatch.setattr(b, "cpu_baseline", lambda *a, **k: dict(sample))
    return b


def run(bench, monkeypatch, *argv):
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    out = io.StringIO()
    with redirect_stdout(out):
        bench.main()
    lines = [l for l in out.getvalue().splitlines() if l.strip()]
    assert len(lines) == 1
    return json.loads(lines[0])


BASE_KEYS = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline",
             "dtype", "data", "config", "e2e"]


def test_headline_line(bench, monkeypatch):
    d = run(bench, monkeypatch, "--reps", "2", "--steps", "1", "--warmup", "3")
    for k in BASE_KEYS + ["ms_per_step", "gpu_launches", "roofline", "cpu_baseline", "clocks", "fp64_plain",
                          "concurrent_calls"]:
        assert k in d, k
    assert d["warmup"] >= 3 and d["n_gpus"] == 1 and "workload" in d["config"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in d["e2e"], k
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in d["roofline"], k
    assert d["roofline"]["frac"] == pytest.approx(d["roofline"]["achieved"] / d["roofline"]["peak"])
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in d["cpu_baseline"], k
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert d["concurrent_calls"]["value"] > 0 and d["concurrent_calls"]["rho_identical_to_sequential"]


@pytest.mark.parametrize("workload", ["simplex_explore", "smap_sweep", "panels", "panels_independent",
                                      "panels_penalty", "adjoint",
                                      "easy_edm"])
def test_other_workloads_line(bench, monkeypatch, workload):
    # the oracle's CPU sample runs for real on the quick workloads
    quick = workload in ("simplex_explore", "adjoint")
    d = run(bench, monkeypatch, "--workload", workload, "--steps", "1", "--warmup", "3", *([] if quick else ["--no-cpu"]))
    for k in BASE_KEYS + ["ms_per_step", "gpu_launches", "clocks", "roofline", "cpu_baseline"]:
        assert k in d, k
    assert d["value"] > 0 and d["config"]["workload"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic", "kernel_ms_per_step"):
        assert k in d["roofline"], k
    assert d["roofline"]["frac"] == pytest.approx(d["roofline"]["achieved"] / d["roofline"]["peak"])
    if quick:
        for k in ("value", "unit", "cores", "kind", "sample"):
            assert k in d["cpu_baseline"], k
        assert d["cpu_baseline"]["value"] > 0


def test_reference_arm_line(bench, monkeypatch):
    d = run(bench, monkeypatch, "--impl", "reference", "--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference"
    for k in BASE_KEYS + ["cpu_baseline"]:
        assert k in d, k
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] == d["cpu_baseline"]["value"]
