"""NPBench framework plugin files for npbench_gb300 and their installer.

The files under this directory mirror their destinations in an NPBench
checkout (see ``install.py``): a ``framework_info`` JSON, the
``GB300Framework`` class and one implementation module per stencil, each
keeping the NumPy kernel's signature.
"""
