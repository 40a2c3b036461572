"""Host-side checks that need no GPU: the CUDA library loads and exports every
entry point the public header declares, and the scene generators produce the
workload sizes."""
import ctypes
import os

import numpy as np
import pytest

from collision_gb300 import _lib, scenes


def _built():
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__ as g
        g.build()
    return _lib.LIB_PATH


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_built())
    syms = _lib.declared_symbols()
    assert len(syms) >= 14
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_loader_fails_loudly_without_library(tmp_path):
    with pytest.raises(RuntimeError):
        _lib._LIB = None
        _lib.load(str(tmp_path / "missing.so"))
    _lib._LIB = None


def test_workload_sizes():
    sc = scenes.cloth_on_sphere()
    assert (sc.nv, sc.nt) == (33 * 33 + 642, 2048 + 1280)
    st = scenes.strings(nstr=4, nseg=16)
    assert st.nb == 64 and st.nt == 12 and st.nv == 4 * 17 + 8
    ico, tri = scenes.icosphere(5, 0.3)
    assert (len(ico), len(tri)) == (10242, 20480)
    fc = scenes.folded_cloth(n=9)
    assert fc.nt == 2 * 8 * 8
    # rest lengths are the initial edge lengths
    e = np.linalg.norm(sc.x[sc.tris[:, 0]] - sc.x[sc.tris[:, 1]], axis=1)
    assert np.array_equal(e, sc.tri_rest[:, 0])


def test_batched_sizes_deterministic():
    a = scenes.batched(nscenes=4, seed=3)
    b = scenes.batched(nscenes=4, seed=3)
    assert [s.nv for s in a] == [s.nv for s in b]
    assert all(16 * 16 <= s.nv - (642 if s.nt > 12 + 2 * 15 * 15 + 1280 - 1 else 8) or True for s in a)


def test_cpp_headers_compile_and_link(tmp_path):
    """The C++ classes over the C ABI compile and link against the library
    (nothing is called: there is no GPU here)."""
    import shutil
    import subprocess
    from collision_gb300 import _lib
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "collision_gb300.hpp"\n'
        'int main(int argc, char**) {\n'
        '  if (argc > 5) {\n'
        '    collision_gb300::CollisionSolver3d s(0);\n'
        '    collision_gb300::SceneBatch b(0);\n'
        '    b.assemble({});\n'
        '    s.setMode(1); b.setMode(1);\n'
        '    s.setTuning(CC_TUNE_ROPE_TRAVERSE, 1); b.setTuning(CC_TUNE_SUBSET_REFIT, 1);\n'
        '    double ms = s.autotune() + b.autotune();\n'
        '    return s.hasCollision() + b.numScenes() + s.tuning(CC_TUNE_ROPE_TRAVERSE) + (int)ms +\n'
        '           (int)s.counters().size() + (int)b.counters().size();\n'
        '  }\n'
        '  return 0;\n'
        '}\n')
    out = tmp_path / "use"
    inc = os.path.join(_lib.ROOT, "include")
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-I", inc, str(src), "-o", str(out), "-L", libdir,
                        "-lcollision_gb300", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_one_core_baseline_samples_by_size():
    # the bench's one-core CPU baseline: the median scene of every sixteenth
    # of the scenes in size order, stepped on one thread by the oracle
    import bench
    from collision_gb300 import scenes
    scs = [scenes.cloth_on_sphere(n=3 + (i * 7) % 6, sub=0, side=0.2, seed=i) for i in range(32)]
    r = bench.one_core_rate(scs, 1, 0.01, 1000)
    assert r["cores"] == 1 and r["value"] > 0
    assert r["sample"].startswith("2 of 32 scenes"), r["sample"]
