"""Shared fixtures.

Libraries under test:
  gpulib     libimagew_gb300.so, the product (built in-tree on first use);
  oracle     the CPU restatement of the reference (oracle/_build/liboracle_iw.so);
  reference  the unmodified reference core compiled from its sources
             (oracle/_ref/libimagew_ref.so) -- only where it was built; tests
             that need it are skipped elsewhere.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# one hardware queue per device lane of the library (read when the CUDA
# context is created, which torch may do before the library loads)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from imageworsener_gb300.iwapi import IWLib, Job  # noqa: E402

ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle_iw.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libimagew_ref.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def oracle() -> IWLib:
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return IWLib(ORACLE_SO)


@pytest.fixture(scope="session")
def reference() -> IWLib:
    if not os.path.exists(REF_SO):
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    return IWLib(REF_SO)


@pytest.fixture(scope="session")
def gpulib() -> IWLib:
    from imageworsener_gb300 import build
    return IWLib(build.build())


def load_grid():
    """The golden grid: (Job, expected digest, expected meta) per case."""
    with open(os.path.join(GOLDEN, "grid.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, "grid.npz"))
    cases = []
    for n, m in enumerate(meta):
        calls = [tuple(tuple(a) if isinstance(a, list) else a for a in c) for c in m["calls"]]
        job = Job(m["imgtype"], m["bit_depth"], m["width"], m["height"], arrays[f"in{n}"].tobytes(), bpr=m["bpr"],
                  calls=calls, sampletype=m["sampletype"], orient=m["orient"])
        cases.append((job, m["result"]["digest"], m))
    return cases


def load_workload_digests():
    with open(os.path.join(GOLDEN, "workloads.json")) as f:
        return json.load(f)
