"""Loads the package's Python binding (its directory name is not an identifier)."""
import importlib.util
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent / "fastedm-r_gb300"


def _load(name):
    spec = importlib.util.spec_from_file_location(f"fastedm_gb300_{name}", PKG / f"{name}.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


fedm = _load("edm")
workloads = _load("workloads")
build = _load("build")
