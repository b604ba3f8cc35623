import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Monte Carlo agreement of two independent estimates of an image (or of one estimate and
# the exact image), per pixel-channel z = difference / sqrt(sum of variances of the mean):
# under agreement a z beyond 3 in magnitude has probability 0.27 %, so the count beyond 3
# among n pixel-channels is binomial(n, 0.0027); the bound is its mean plus four standard
# deviations plus one, a false alarm about once in 30,000 checks.  The image mean is one
# more normal variable (the summed differences over the root of the summed variances),
# bounded at 4.5.
P_BEYOND_3 = 0.0027


def beyond3_bound(n):
    return n * P_BEYOND_3 + 4.0 * math.sqrt(n * P_BEYOND_3) + 1.0


def assert_within_3_sigma(z, zmax=6.0, zsum=None):
    z = np.asarray(z, float).ravel()
    k = int(np.count_nonzero(np.abs(z) > 3))
    assert k <= beyond3_bound(z.size), f"{k} of {z.size} pixel-channels beyond 3 sigma (at most {beyond3_bound(z.size):.1f})"
    assert float(np.max(np.abs(z))) < zmax, f"max |z| {float(np.max(np.abs(z))):.2f} >= {zmax}"
    if zsum is not None:
        assert abs(zsum) < 4.5, f"image mean {zsum:.2f} sigma apart"


def assert_agree(ma, va, mb, vb, zmax=6.0):
    """Two images (means and variances of the mean) against the bounds above."""
    ma, va, mb, vb = (np.asarray(x, float) for x in (ma, va, mb, vb))
    v = np.maximum(va + vb, 1e-30)
    assert_within_3_sigma((ma - mb) / np.sqrt(v), zmax, zsum=float((ma - mb).sum() / np.sqrt(v.sum())))


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
