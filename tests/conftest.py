import os
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Builds the product library and the CPU oracle (incremental)."""
    from rayt_gb300 import build
    build.build_library()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def trees(built):
    """Block files of every golden builder case, built by the product builder
    (their bytes are pinned to the reference builder by test_builder_golden)."""
    import rayt_gb300 as R
    from tests.golden.common import BUILDER_CASES
    d = tempfile.mkdtemp(prefix="rayt_trees_")
    out = {}
    for name, case in BUILDER_CASES.items():
        path = os.path.join(d, name + ".tree")
        if case["kind"] == "sphere":
            R.build_sphere_test(path, case["center"], case["radius"], case["depth"], case["nib"])
        else:
            t = case["terrain"]
            R.build_terrain(path, t["depth"], case["nib"], seed=t["seed"], base_cells=t["base_cells"],
                            octaves=t["octaves"], spheres=t["spheres"], sphere_seed=t["sphere_seed"],
                            min_radius=t["min_radius"], max_radius=t["max_radius"])
        out[name] = path
    return out


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)


def libc_srand(seed):
    import ctypes
    ctypes.CDLL(None).srand(ctypes.c_uint(seed))
