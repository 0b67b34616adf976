import faulthandler
import os
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The descriptor a crash report goes to: the terminal or log the run writes to
# (pytest redirects descriptor 2 to a temporary file while a test runs).
_REPORT_FD = None
_STARTED = {}


def _report(text: str) -> None:
    fd = _REPORT_FD if _REPORT_FD is not None else 2
    try:
        os.write(fd, text.encode())
    except OSError:
        pass


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.hookimpl(trylast=True)
def pytest_sessionstart(session):
    """Crash reports name the test: every test's node id is written, unbuffered,
    to the run's own output before it starts, and a fatal signal dumps the
    faulting thread only (a crash in several native threads at once then
    stays short enough to leave that line in view)."""
    global _REPORT_FD
    fd = None
    try:
        from _pytest.faulthandler import fault_handler_stderr_fd_key
        fd = session.config.stash.get(fault_handler_stderr_fd_key, None)
    except ImportError:
        pass
    if fd is None:
        fd = os.dup(2)
    _REPORT_FD = fd
    faulthandler.enable(file=fd, all_threads=False)


def pytest_runtest_logstart(nodeid, location):
    _STARTED[nodeid] = time.monotonic()
    _report(f"\n[test start] {nodeid}\n")


def pytest_runtest_logfinish(nodeid, location):
    t0 = _STARTED.pop(nodeid, None)
    dt = time.monotonic() - t0 if t0 is not None else 0.0
    _report(f"[test end] {nodeid} ({dt:.1f} s)\n")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def dk_lib():
    from denrimrendererkit_gb300 import build, library
    build.build()
    return library.load()
