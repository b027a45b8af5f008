import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "pimc.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def engine_lib():
    import glob

    import pimc
    srcs = glob.glob(os.path.join(ROOT, "pimc.jl_gb300", "csrc", "*")) + \
        [os.path.join(ROOT, "include", "pimc.h")]
    from pimc._native import LIB_CHECK_PATH, check_build_requested
    check = check_build_requested()
    path = LIB_CHECK_PATH if check else pimc.LIB_PATH
    stale = not os.path.exists(path) or \
        max(os.path.getmtime(s) for s in srcs) > os.path.getmtime(path)
    if stale:
        pimc.build(check=check)
    return pimc.load()
