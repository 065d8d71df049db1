"""The gb300 framework plugin inside NPBench's own harness.

* CPU: the plugin installs into an NPBench tree, ``generate_framework("gb300")``
  returns ``GB300Framework`` and every stencil benchmark resolves to the
  npbench_gb300 kernels with the reference's argument strings plus a device
  synchronisation (framework.py:140-162, cupy_framework.py:32-58).
* GPU: the harness's ``Test.run`` executes each stencil benchmark at preset S
  through the plugin, validates it against the harness's own NumPy run
  (test.py:103-126), reports SUCCESS and writes its timings into the
  harness's ``npbench.db`` (test.py:133-163); ``run_benchmark.py`` does the
  same end to end, line counts included (run_benchmark.py:1-59), and next to NumPy's rows
  ``npbench_gb300.report`` turns the database into plot_results.py's speed-up table and
  heat map.  It uses the NPBench tree that
  ``__graft_entry__.build()`` installs into baseline/_ref/npbench, and is
  skipped where that tree was never built.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUBS = os.path.join(ROOT, "tests", "stubs")
BUILT_TREE = os.path.join(ROOT, "baseline", "_ref", "npbench")


def _npbench_source():
    """An NPBench tree to copy: NPBENCH_SRC, else the tree build() installed."""
    for src in (os.environ.get("NPBENCH_SRC"), BUILT_TREE):
        if src and os.path.isdir(os.path.join(src, "npbench", "infrastructure")):
            return src
    return None


def _run(tree, code, timeout=600):
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([tree, ROOT, STUBS, env.get("PYTHONPATH", "")])
    env["PYTHONDONTWRITEBYTECODE"] = "1"
    return subprocess.run([sys.executable, "-c", code], cwd=tree, env=env, capture_output=True,
                          text=True, timeout=timeout)


def test_plugin_resolves_in_harness(tmp_path):
    src = _npbench_source()
    if src is None:
        pytest.skip("no NPBench source tree available")
    from npbench_gb300.plugin import install
    tree = str(tmp_path / "npbench")
    install.install(tree, copy_from=src)
    code = r"""
from npbench.infrastructure import Benchmark, generate_framework
f = generate_framework("gb300")
assert type(f).__name__ == "GB300Framework"
assert f.version().startswith("npbgb ")
for name, fn, mod in [("jacobi_2d", "kernel", "npbench.benchmarks.polybench.jacobi_2d.jacobi_2d_gb300"),
                      ("heat_3d", "kernel", "npbench.benchmarks.polybench.heat_3d.heat_3d_gb300"),
                      ("hdiff", "hdiff", "npbench.benchmarks.weather_stencils.hdiff.hdiff_gb300"),
                      ("jacobi_1d", "kernel", "npbench.benchmarks.polybench.jacobi_1d.jacobi_1d_gb300"),
                      ("fdtd_2d", "kernel", "npbench.benchmarks.polybench.fdtd_2d.fdtd_2d_gb300"),
                      ("vadv", "vadv", "npbench.benchmarks.weather_stencils.vadv.vadv_gb300"),
                      ("cavity_flow", "cavity_flow",
                       "npbench.benchmarks.cavity_flow.cavity_flow_gb300"),
                      ("channel_flow", "channel_flow",
                       "npbench.benchmarks.channel_flow.channel_flow_gb300")]:
    b = Benchmark(name)
    impl, label = f.implementations(b)[0]
    assert impl.__module__ == mod and impl.__name__ == fn and label == "default", impl
    assert f.exec_str(b).endswith("; torch.cuda.synchronize()"), f.exec_str(b)
    assert f.setup_str(b).endswith("; torch.cuda.synchronize()"), f.setup_str(b)
    assert "__npb_gb_" in f.exec_str(b)
print("OK")
"""
    r = _run(tree, code)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_install_is_idempotent(tmp_path):
    src = _npbench_source()
    if src is None:
        pytest.skip("no NPBench source tree available")
    from npbench_gb300.plugin import install
    tree = str(tmp_path / "npbench")
    install.install(tree, copy_from=src)
    install.install(tree)
    with open(os.path.join(tree, "npbench", "infrastructure", "__init__.py")) as f:
        assert f.read().count("gb300_framework") == 1


@pytest.mark.gpu
@pytest.mark.parametrize("bench", ["jacobi_2d", "heat_3d", "hdiff", "jacobi_1d", "fdtd_2d",
                                   "vadv", "cavity_flow", "channel_flow"])
def test_harness_runs_and_validates_plugin(tmp_path, bench):
    if not os.path.isdir(os.path.join(BUILT_TREE, "npbench", "infrastructure")):
        pytest.skip("baseline/_ref/npbench was not built")
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import shutil
    tree = str(tmp_path / "npbench")
    shutil.copytree(BUILT_TREE, tree)
    code = f"""
from npbench.infrastructure import Benchmark, generate_framework, Test
bench = Benchmark("{bench}")
frmwrk = generate_framework("gb300")
numpy = generate_framework("numpy")
Test(bench, frmwrk, numpy).run("S", True, 2, 300.0, False)
print("HARNESS-DONE")
"""
    r = _run(tree, code)
    out = r.stdout + r.stderr
    assert r.returncode == 0 and "HARNESS-DONE" in r.stdout, out
    assert "validation: SUCCESS" in r.stdout, out
    assert "did not validate" not in out, out
    rows = _results(tree)
    assert len(rows) == 2 and all(v == 1 and t > 0 for _, _, v, t in rows), rows
    assert {fw for _, fw, _, _ in rows} == {"gb300"}, rows


def _results(tree):
    import sqlite3
    with sqlite3.connect(os.path.join(tree, "npbench.db")) as con:
        return con.execute("SELECT benchmark, framework, validated, time FROM results").fetchall()


@pytest.mark.gpu
def test_run_benchmark_writes_results_db(tmp_path):
    """NPBench's own command line with -f gb300: validated timings land in npbench.db."""
    if not os.path.isdir(os.path.join(BUILT_TREE, "npbench", "infrastructure")):
        pytest.skip("baseline/_ref/npbench was not built")
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import shutil
    import sqlite3
    tree = str(tmp_path / "npbench")
    shutil.copytree(BUILT_TREE, tree)
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([tree, ROOT, STUBS, env.get("PYTHONPATH", "")])
    env["PYTHONDONTWRITEBYTECODE"] = "1"
    r = subprocess.run([sys.executable, "run_benchmark.py", "-b", "heat_3d", "-f", "gb300", "-p",
                        "S", "-r", "3"], cwd=tree, env=env, capture_output=True, text=True,
                       timeout=600)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out
    assert "validation: SUCCESS" in r.stdout, out
    rows = _results(tree)
    assert len(rows) == 3, rows
    assert all(b == "heat3d" or b == "heat_3d" for b, _, _, _ in rows), rows
    assert all(fw == "gb300" and v == 1 and t > 0 for _, fw, v, t in rows), rows
    with sqlite3.connect(os.path.join(tree, "npbench.db")) as con:
        lc = con.execute("SELECT framework, count FROM lcounts").fetchall()
    assert any(fw == "gb300" and n > 0 for fw, n in lc), lc
    # NumPy's own rows next to ours, then the speed-up report over the database
    # (the table of plot_results.py, without pandas/matplotlib).
    r = subprocess.run([sys.executable, "run_benchmark.py", "-b", "heat_3d", "-f", "numpy", "-p",
                        "S", "-r", "3"], cwd=tree, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    from npbench_gb300 import report
    table = report.speedup_table(report.load_results(os.path.join(tree, "npbench.db")), "S")
    assert table["frameworks"] == ["gb300", "numpy"], table["frameworks"]
    (bd,) = table["benchmarks"]
    assert 0 < table["ratio"][bd]["gb300"] < 1, table["ratio"]  # faster than NumPy
    svg = os.path.join(tree, "heatmap.svg")
    report.main(["--db", os.path.join(tree, "npbench.db"), "-p", "S", "--svg", svg])
    import xml.etree.ElementTree as ET
    assert ET.parse(svg).getroot().tag.endswith("svg")
