"""Test-only stand-in for pygount, which NPBench's harness imports for line counts.

npbench/infrastructure/line_count.py:6 imports ``SourceAnalysis``; the harness
import fails without it.  Line counting is not part of the stencil path, so the
plugin tests put this stub on PYTHONPATH.  ``code_count`` counts non-blank,
non-comment lines.
"""


class SourceAnalysis:
    def __init__(self, code_count):
        self.code_count = code_count

    @classmethod
    def from_file(cls, path, group=None, **kwargs):
        n = 0
        with open(path) as f:
            for line in f:
                s = line.strip()
                if s and not s.startswith("#"):
                    n += 1
        return cls(n)
