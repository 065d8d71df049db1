"""Install the gb300 framework plugin into an NPBench checkout.

    python -m npbench_gb300.plugin.install NPBENCH_ROOT
    python -m npbench_gb300.plugin.install --copy-from SRC NPBENCH_ROOT

Adds, under NPBENCH_ROOT (the directory holding ``framework_info/``,
``bench_info/`` and ``npbench/``):

* ``framework_info/gb300.json``
* ``npbench/infrastructure/gb300_framework.py``
* ``npbench/benchmarks/polybench/jacobi_2d/jacobi_2d_gb300.py``
* ``npbench/benchmarks/polybench/heat_3d/heat_3d_gb300.py``
* ``npbench/benchmarks/weather_stencils/hdiff/hdiff_gb300.py``
* ``npbench/benchmarks/polybench/jacobi_1d/jacobi_1d_gb300.py``
* ``npbench/benchmarks/polybench/fdtd_2d/fdtd_2d_gb300.py``
* ``npbench/benchmarks/weather_stencils/vadv/vadv_gb300.py``
* ``npbench/benchmarks/cavity_flow/cavity_flow_gb300.py``
* ``npbench/benchmarks/channel_flow/channel_flow_gb300.py``

and appends ``from .gb300_framework import *`` to
``npbench/infrastructure/__init__.py`` (once).  ``--copy-from`` first copies a
read-only NPBench tree to NPBENCH_ROOT.  The harness then runs the plugin with
``python run_benchmark.py -b heat_3d -f gb300`` as long as ``npbench_gb300``
is importable (e.g. its parent directory on PYTHONPATH).
"""
import argparse
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = [
    "framework_info/gb300.json",
    "infrastructure/gb300_framework.py",
    "benchmarks/polybench/jacobi_2d/jacobi_2d_gb300.py",
    "benchmarks/polybench/heat_3d/heat_3d_gb300.py",
    "benchmarks/weather_stencils/hdiff/hdiff_gb300.py",
    "benchmarks/polybench/jacobi_1d/jacobi_1d_gb300.py",
    "benchmarks/polybench/fdtd_2d/fdtd_2d_gb300.py",
    "benchmarks/weather_stencils/vadv/vadv_gb300.py",
    "benchmarks/cavity_flow/cavity_flow_gb300.py",
    "benchmarks/channel_flow/channel_flow_gb300.py",
]
IMPORT_LINE = "from .gb300_framework import *\n"


def _dest(root, rel):
    if rel.startswith("framework_info/"):
        return os.path.join(root, rel)
    return os.path.join(root, "npbench", rel)


def install(root, copy_from=None):
    """Install the plugin files into the NPBench tree at ``root``; returns the written paths."""
    if copy_from is not None:
        if os.path.exists(root):
            shutil.rmtree(root)
        shutil.copytree(copy_from, root, ignore=shutil.ignore_patterns("__pycache__", "*.pyc",
                                                                       ".git"))
        for dirpath, dirnames, filenames in os.walk(root):
            os.chmod(dirpath, 0o755)
            for fn in filenames:
                os.chmod(os.path.join(dirpath, fn), 0o644)
    init = os.path.join(root, "npbench", "infrastructure", "__init__.py")
    if not os.path.exists(init):
        raise FileNotFoundError(f"{root} is not an NPBench checkout (no {init})")
    written = []
    for rel in FILES:
        dst = _dest(root, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(HERE, rel), dst)
        written.append(dst)
    with open(init) as f:
        text = f.read()
    if IMPORT_LINE.strip() not in text:
        with open(init, "a") as f:
            f.write(("" if text.endswith("\n") else "\n") + IMPORT_LINE)
    return written


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("root")
    ap.add_argument("--copy-from", default=None)
    a = ap.parse_args(argv)
    for p in install(a.root, a.copy_from):
        print(p)


if __name__ == "__main__":
    sys.exit(main())
