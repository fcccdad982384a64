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


def test_integration_adapter_compiles_and_links(tmp_path, lib):
    """The C++ adapter a reference application uses (include/saqg_ivf.hpp: GpuIVF,
    same member signature as IVF::search) compiles against include/saqg.h and
    links against the library, with a stand-in for the reference's row vector
    and searcher config (only .data() and searcher_vars_bound_m are used)."""
    import shutil
    import subprocess
    from saq_gb300.build import LIB
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "adapter.cpp"
    src.write_text("""#include <vector>
#include "saqg_ivf.hpp"
struct RowVec { std::vector<float> v; const float *data() const { return v.data(); } };
struct Cfg { float searcher_vars_bound_m = 4.0f; };
int main(int argc, char **argv) {
    if (argc < 2) return 0;  // construction needs an index file and a GPU
    GpuIVF ivf(argv[1]);
    RowVec q{std::vector<float>(128, 0.0f)};
    uint32_t ids[10];
    ivf.search(q, 10, 4, Cfg{}, ids);
    ivf.search_batch(q.data(), 1, 10, 4, Cfg{}, ids);
    return 0;
}
""")
    exe = tmp_path / "adapter"
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe), LIB, "-Wl,-rpath," + os.path.dirname(LIB)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert subprocess.run([str(exe)]).returncode == 0
