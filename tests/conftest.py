import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build
    build(with_reference=None)
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.oracle import Reference
    if not Reference.available():
        pytest.skip("reference sources not present here (only the committed fixtures travel)")
    return Reference()


@pytest.fixture(scope="session")
def salty_lib():
    from salty_gb300 import build as b
    b.build()
    import salty_gb300
    return salty_gb300.lib()


@pytest.fixture(scope="session")
def ctx(salty_lib):
    import salty_gb300
    c = salty_gb300.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def soup_1m():
    import salty_gb300
    return salty_gb300.microbench_soup(20260001, 1_000_000)


@pytest.fixture(scope="session")
def gpu_soup_1m(ctx, soup_1m):
    from salty_gb300 import scenes
    sc = scenes.upload(ctx, {"tri_pos": soup_1m, "tri_nrm": None, "tri_mat": None, "materials": [],
                             "light": None, "sun": None, "sky": (0, 0, 0), "camera": None})
    sc.build()
    yield sc
    sc.close()
