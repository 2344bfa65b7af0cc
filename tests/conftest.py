"""Test configuration: puts the repository root on sys.path, registers the `gpu` marker and
builds the in-tree library and the CPU oracle once per session (a no-op when up to date)."""
import importlib.util
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def _build():
    spec = importlib.util.spec_from_file_location("_dsssp_build", ROOT / "dynamicssspv2_gb300" / "_build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_library()
    mod.build_oracle()


_build()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")
