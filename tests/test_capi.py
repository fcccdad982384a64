"""CPU-side checks of the native library: it loads, exports every symbol that
include/saqg.h declares, and its host-only entry points (the planner, error
reporting) behave like the reference without touching a GPU."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "saqg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(saqg_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from saq_gb300 import _native
    return _native.load(build_if_missing=True)


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_covers_header():
    from saq_gb300 import _native
    assert set(declared_symbols()) == set(_native.EXPORTS)


def test_planner_matches_reference(lib):
    from saq_gb300 import ivf
    z = np.load(os.path.join(GOLDEN, "plan.npz"))
    i = 0
    while f"c{i}_var" in z:
        p = ivf.plan(z[f"c{i}_var"], float(z[f"c{i}_avg_bits"]))
        assert p == [tuple(map(int, r)) for r in z[f"c{i}_plan"]]
        i += 1


def test_equal_segmentation_and_no_segmentation(lib):
    from saq_gb300 import ivf
    assert ivf.plan(np.ones(1024, np.float32), 4.0, enable_segmentation=False) == [(1024, 4)]
    assert ivf.plan(np.ones(1024, np.float32), 4.0, seg_eqseg=3) == [(384, 4), (320, 4), (320, 4)]


def test_invalid_arguments_return_status(lib):
    from saq_gb300 import ivf
    from saq_gb300._native import SaqgError
    with pytest.raises(SaqgError, match="multiple of 64"):
        ivf.plan(np.ones(100, np.float32), 4.0)
    assert lib.saqg_version() == 1
