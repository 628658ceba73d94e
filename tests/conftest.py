import ctypes
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
TESTS = Path(__file__).resolve().parent
if str(TESTS) not in sys.path:
    sys.path.insert(0, str(TESTS))


def pytest_addoption(parser):
    parser.addoption("--run-long", action="store_true", default=False,
                     help="also run the tests marked long (full-length runs against the oracle)")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "long: a full-length run against the oracle (--run-long)")


def _have_gpu() -> bool:
    try:
        cuda = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    if cuda.cuInit(0) != 0:
        return False
    n = ctypes.c_int(0)
    return cuda.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0


def pytest_collection_modifyitems(config, items):
    if not config.getoption("--run-long"):
        skip_long = pytest.mark.skip(reason="long run: pass --run-long")
        for it in items:
            if it.get_closest_marker("long"):
                it.add_marker(skip_long)
    gpu_items = [it for it in items if it.get_closest_marker("gpu")]
    if gpu_items and not _have_gpu():
        skip = pytest.mark.skip(reason="no CUDA GPU on this machine")
        for it in gpu_items:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build (if stale) and load the CUDA library."""
    import __graft_entry__
    __graft_entry__.build()
    return True


def pytest_terminal_summary(terminalreporter):
    """Print the parity checks that passed through the zero-field fallback
    (test_gpu_parity.FALLBACKS) and the float64 error table collected by
    test_gpu_fp64_error."""
    par = sys.modules.get("test_gpu_parity")
    used = getattr(par, "FALLBACKS", None) if par else None
    if used:
        tr = terminalreporter
        tr.section("parity checks passed through the zero-field fallback")
        for name, e, how in used:
            tr.write_line(f"{name}: {e:.2e} against the float32 oracle; {how}")
    mod = sys.modules.get("test_gpu_fp64_error")
    rows = getattr(mod, "TABLE", None) if mod else None
    if not rows:
        return
    tr = terminalreporter
    tr.section("error against float64 (GPU | float32 oracle)")
    for row in rows:
        cells = [f"{k} {v[0]:.2e} | {v[1]:.2e}" + (" abs" if v[2] == "abs" else "")
                 for k, v in row.items() if k != "config"]
        tr.write_line(f"{row['config']}: " + "; ".join(cells))
