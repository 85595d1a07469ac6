import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # Bring libfmf_gb300.so up to date before any test module imports the
    # package: a library loaded into this process cannot be replaced later.
    # In a child process, so that the stale copy is never loaded here.
    subprocess.run([sys.executable, "-c",
                    "from fast_matched_filter_gb300 import build; build.build()"],
                   cwd=REPO, check=False)
    # The checker libraries too, before collection: tests that pin the oracle
    # against the reference library are skipped when that library is absent.
    subprocess.run([sys.executable, "-c", "from oracle import cpu; cpu.build()"],
                   cwd=REPO, check=False)


@pytest.fixture(scope="session")
def oracle_built():
    """Build the checker libraries once per session (no-op when up to date)."""
    from oracle import cpu
    cpu.build()
    return cpu
