import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_terminal_summary(terminalreporter):
    """The max errors every parity test measured, printed at the end of the
    run (also in -q mode), and written as JSON to $FPGB_PARITY_REPORT."""
    import json
    import parity
    for line in parity.summary_lines():
        terminalreporter.write_line(line)
    path = os.environ.get("FPGB_PARITY_REPORT")
    if path and parity.REPORT:
        with open(path, "w") as f:
            json.dump(parity.REPORT, f, indent=1, sort_keys=True)


@pytest.fixture(scope="session")
def oracle_port():
    """The C restatement of the reference (test infrastructure only)."""
    import oracle
    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    import fastpli_gb300
    fastpli_gb300.native_library()
    return torch
