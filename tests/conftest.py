import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "mp-sort_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy
    z = numpy.load(os.path.join(REPO, "tests", "golden", "golden.npz"))
    return {k: z[k] for k in z.files}


def golden_cases(golden):
    names = sorted({k.split("__")[0] for k in golden if k.endswith("__orderby")})
    return [(n, golden[n + "__in"], golden[n + "__out"], str(golden[n + "__orderby"]))
            for n in names]
