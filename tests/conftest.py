"""Shared test setup: import paths, the `gpu` marker, on-demand builds."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "msc-thesis_gb300"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def _ensure_built():
    import oracle  # noqa: F401  (builds the restatement on first use)
    lib = os.path.join(ROOT, "msc-thesis_gb300", "libpic.so")
    if not os.path.exists(lib):
        sys.path.insert(0, os.path.join(ROOT, "msc-thesis_gb300"))
        import build_lib
        build_lib.build()


_ensure_built()
