"""npbench_gb300.report: the speed-up table of NPBench's plot_results.py, restated.

The database is built with the schema and insert statement of
npbench/infrastructure/utilities.py:81-108; the expected values are worked out by
hand from plot_results.py's aggregation (validated rows with a domain, best
details per mode by median, mean over modes, ratio to NumPy, geometric mean).
"""
import math
import sqlite3
import xml.etree.ElementTree as ET

import pytest

from npbench_gb300 import report

SCHEMA = """CREATE TABLE IF NOT EXISTS results (
    id integer PRIMARY KEY, timestamp integer NOT NULL, benchmark text NOT NULL, kind text,
    domain text, dwarf text, preset text NOT NULL, mode text NOT NULL, framework text NOT NULL,
    version text NOT NULL, details text, validated integer, time real);"""
INSERT = """INSERT INTO results(timestamp, benchmark, kind, domain, dwarf, preset, mode,
    framework, version, details, validated, time) VALUES (?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?);"""


def _db(path, rows):
    con = sqlite3.connect(path)
    con.execute(SCHEMA)
    for bench, domain, preset, mode, fw, details, valid, t in rows:
        con.execute(INSERT, (0, bench, "", domain, "", preset, mode, fw, "1", details, valid, t))
    con.commit()
    con.close()


@pytest.fixture
def db(tmp_path):
    rows = []
    # jacobi_2d: numpy 2.0 s (median of 1, 2, 3 -> 2); gb300 best details "fast" median 0.01.
    rows += [("jacobi_2d", "polybench", "S", "main", "numpy", "default", 1, t) for t in (1, 2, 3)]
    rows += [("jacobi_2d", "polybench", "S", "main", "gb300", "fast", 1, t)
             for t in (0.01, 0.009, 0.011)]
    rows += [("jacobi_2d", "polybench", "S", "main", "gb300", "slow", 1, t) for t in (0.5, 0.6)]
    # a failed validation and another preset are ignored
    rows += [("jacobi_2d", "polybench", "S", "main", "gb300", "broken", 0, 0.0001)]
    rows += [("jacobi_2d", "polybench", "M", "main", "gb300", "fast", 1, 0.0001)]
    # heat_3d: numpy 4.0; gb300 two modes, best medians 0.02 and 0.06 -> mean 0.04.
    rows += [("heat_3d", "polybench", "S", "main", "numpy", "default", 1, 4.0)]
    rows += [("heat_3d", "polybench", "S", "main", "gb300", "default", 1, t) for t in (0.02, 0.02)]
    rows += [("heat_3d", "polybench", "S", "other", "gb300", "default", 1, 0.06)]
    # no domain: dropped
    rows += [("hdiff", "", "S", "main", "numpy", "default", 1, 1.0)]
    path = tmp_path / "npbench.db"
    _db(str(path), rows)
    return str(path)


def test_table_follows_plot_results_aggregation(db):
    t = report.speedup_table(report.load_results(db), "S")
    assert t["frameworks"] == ["gb300", "numpy"]
    assert t["benchmarks"] == [("heat_3d", "polybench"), ("jacobi_2d", "polybench")]
    j, h = ("jacobi_2d", "polybench"), ("heat_3d", "polybench")
    assert t["time"][j]["numpy"] == 2.0 and t["time"][j]["gb300"] == pytest.approx(0.01)
    assert t["time"][h]["gb300"] == pytest.approx(0.04)
    assert t["ratio"][j]["gb300"] == pytest.approx(0.005)
    assert t["ratio"][h]["gb300"] == pytest.approx(0.01)
    assert t["ratio"][j]["numpy"] == 1.0
    assert t["total"]["gb300"] == pytest.approx(math.sqrt(0.005 * 0.01))
    assert t["total"]["numpy"] == 1.0
    assert t["ci"][j]["gb300"] >= 0.0


def test_labels():
    assert report.speedup_label(0.5) == "↑2.0"
    assert report.speedup_label(2.0) == "↓2.0"
    assert report.speedup_label(1.0) == "1.0"
    assert report.speedup_label(1 / 250.7) == "↑250.0"
    assert report.speedup_label(1 / 1234.0) == "↑1.2k"
    assert report.speedup_label(math.nan) == ""
    assert report.runtime_label(0.0123) == "12.30 ms"
    assert report.runtime_label(2.5) == "2.50 s"


def test_markdown_and_svg(db, tmp_path, capsys):
    svg = tmp_path / "heat.svg"
    report.main(["--db", db, "-p", "S", "--svg", str(svg)])
    md = capsys.readouterr().out
    assert "| **Total** | ↑141.0 |" in md  # above 100 the label truncates to an integer
    assert "| jacobi_2d | ↑200.0" in md and "2.00 s |" in md
    root = ET.parse(svg).getroot()
    assert root.tag.endswith("svg")
    texts = [e.text for e in root.iter() if e.tag.endswith("text")]
    assert "↑200.0" in " ".join(x or "" for x in texts)


def test_missing_baseline_is_an_error(tmp_path):
    path = tmp_path / "npbench.db"
    _db(str(path), [("jacobi_2d", "polybench", "S", "main", "gb300", "fast", 1, 0.01)])
    with pytest.raises(ValueError):
        report.speedup_table(report.load_results(str(path)), "S")


def test_benchmark_without_numpy_rows_is_blank(tmp_path):
    """A benchmark that NumPy never ran has no ratio (blank cells, no effect on Total)."""
    path = tmp_path / "npbench.db"
    _db(str(path), [("jacobi_2d", "polybench", "S", "main", "numpy", "default", 1, 2.0),
                    ("jacobi_2d", "polybench", "S", "main", "gb300", "fast", 1, 0.02),
                    ("hdiff", "weather", "S", "main", "gb300", "default", 1, 0.5)])
    t = report.speedup_table(report.load_results(str(path)), "S")
    h = ("hdiff", "weather")
    assert math.isnan(t["ratio"][h]["gb300"]) and math.isnan(t["ratio"][h]["numpy"])
    assert t["total"]["gb300"] == pytest.approx(0.01)
    md = report.to_markdown(t)
    assert "| hdiff |  |  |" in md
    ET.fromstring(report.to_svg(t))  # well-formed with blank cells
