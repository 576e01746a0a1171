"""Shared test set-up: the `gpu` marker and the package loader.

The package directory is named `rive-runtime_gb300` (not an identifier), so it
is loaded under the module name `rive_runtime_gb300`.
"""
import importlib.util
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")


def load_package():
    if "rive_runtime_gb300" in sys.modules:
        return sys.modules["rive_runtime_gb300"]
    root = os.path.join(REPO, "rive-runtime_gb300")
    spec = importlib.util.spec_from_file_location(
        "rive_runtime_gb300", os.path.join(root, "__init__.py"),
        submodule_search_locations=[root])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["rive_runtime_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()
if os.path.join(REPO, "oracle") not in sys.path:
    sys.path.insert(0, os.path.join(REPO, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".cap"))


def load_golden(name):
    from rive_runtime_gb300 import capture
    with open(os.path.join(GOLDEN, name + ".cap"), "rb") as f:
        cap = capture.parse(f.read())
    with open(os.path.join(GOLDEN, name + ".scene"), "rb") as f:
        scene_bytes = f.read()
    return cap, scene_bytes
