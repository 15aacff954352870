import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def fap_lib():
    from fastapsp_gb300 import build

    build.build()
    import fastapsp_gb300

    fastapsp_gb300.lib()
    return fastapsp_gb300


@pytest.fixture(scope="session")
def gpu(fap_lib):
    if fap_lib.device_count() < 1:
        pytest.fail("no CUDA device visible to the engine")
    return fap_lib


def load_golden(name):
    import numpy as np

    from fastapsp_gb300 import graphs

    z = dict(np.load(ROOT / "tests" / "golden" / f"{name}.npz"))
    g = graphs.csr_from_lines(int(z["n"]), z["lines_src"], z["lines_dst"], z["lines_w"],
                              bool(z["directed"]), bool(z["weighted"]))
    return z, g


GOLDEN = sorted(p.stem for p in (ROOT / "tests" / "golden").glob("*.npz"))
