import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C-ABI")


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")


def pytest_terminal_summary(terminalreporter):
    """One line per configuration the GPU parity tests compared with the oracle."""
    from tests import _golden as G

    if not G.REPORT:
        return
    tr = terminalreporter
    tr.section("parity against the FP64 oracle")
    for case in sorted(G.REPORT):
        e = G.REPORT[case]
        nn = f"{e['nn_equal']:,} of {e['nn_total']:,} neighbour indices equal" if e["nn_total"] else "no indices"
        tr.write_line(f"{case}: {e['cubes']} comparisons, max norm err {e['norm_max']:.2e}, L2 {e['l2']:.2e}, "
                      f"max rel (|o| >= 1e-6 max) {e['sig']:.2e}; {nn}")
