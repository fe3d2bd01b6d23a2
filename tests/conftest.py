import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

_status = {"exit": None}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library through its C ABI")


def pytest_sessionfinish(session, exitstatus):
    _status["exit"] = int(exitstatus)


@pytest.hookimpl(trylast=True)
def pytest_unconfigure(config):
    """The reference built from its sources (oracle/_ref) unloads its modules
    in static destructors at process exit, and with more than one of its
    modules loaded in one process (macadvection3 beside macutility3 or
    macpressuresolver3) that teardown faults after every test has finished.
    When the reference was loaded in this process, the session ends here,
    with pytest's own status, instead of running that teardown."""
    orc = sys.modules.get("oracle")
    if orc is None or getattr(orc, "_ref", None) is None or _status["exit"] is None:
        return
    sys.stdout.flush()
    sys.stderr.flush()
    os._exit(_status["exit"])


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")
