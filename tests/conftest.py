import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


INDEX_CASES = sorted(
    os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
    if os.path.basename(p) not in ("encode.npz", "plan.npz") and not os.path.basename(p).startswith("construct_")
)
CONSTRUCT_CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "construct_*.npz")))


class GoldenCase:
    """One reference-built index with the reference's outputs on it."""

    def __init__(self, name, tmpdir):
        self.name = name
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.z = z
        self.params = json.loads(bytes(z["params"]).decode())
        self.index_path = os.path.join(tmpdir, name + ".index")
        with open(self.index_path, "wb") as f:
            f.write(z["index_bytes"].tobytes())
        self.q = z["q"]
        self.plan = [tuple(map(int, r)) for r in z["plan"]]
        self.topk = self.params["topk"]
        self.nprobe = self.params["nprobe"]


@pytest.fixture(scope="session")
def golden_dir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("golden"))


@pytest.fixture(params=INDEX_CASES)
def golden_case(request, golden_dir):
    return GoldenCase(request.param, golden_dir)


@pytest.fixture
def golden_case_by_name(golden_dir):
    """Path of a golden case's reference-format index file, by case name."""
    def get(name):
        path = os.path.join(golden_dir, name + ".index")
        if not os.path.exists(path):
            z = np.load(os.path.join(GOLDEN, name + ".npz"))
            with open(path, "wb") as f:
                f.write(z["index_bytes"].tobytes())
        return path
    return get
