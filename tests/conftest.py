"""Test configuration: the `gpu` marker and on-demand builds of the CPU
oracle and the C-ABI library (both in-tree, both git-ignored)."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _ensure_built():
    oracle_so = ROOT / "oracle" / "_build" / "liboracle.so"
    if not oracle_so.exists():
        subprocess.run(["bash", str(ROOT / "oracle" / "build_oracle.sh")], check=True)
    lib = ROOT / "tg_gb300" / "libtgx.so"
    if not lib.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("tgx_build", ROOT / "tg_gb300" / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()


_ensure_built()


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    from oracle_lib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def ctx():
    import tg_gb300 as tg
    c = tg.Context(0)
    yield c
    c.close()
