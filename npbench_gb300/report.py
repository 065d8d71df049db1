"""Speed-up report over NPBench's results database, without pandas or matplotlib.

    python -m npbench_gb300.report --db npbench.db --preset S [--svg heatmap.svg]

NPBench's ``plot_results.py`` turns the ``results`` table that ``Test.run``
fills (npbench/infrastructure/utilities.py:32-122, test.py:133-163) into a
heat map of each framework's runtime relative to NumPy.  It needs pandas and
matplotlib; this module computes the same table with the standard library and
NumPy and writes the heat map as a plain SVG file.  The aggregation follows
plot_results.py:90-168:

* rows with an empty domain and rows that did not validate are dropped, and
  only the chosen preset is kept;
* per (benchmark, domain, framework, mode, details) the median time is taken;
  per (benchmark, domain, framework, mode) the details with the lowest median
  are the best, and the framework's time for a benchmark is the mean over its
  modes of those best medians (the pivot's default aggregation);
* a framework's entry is its time divided by NumPy's; ``Total`` is the
  geometric mean of a framework's entries over the benchmarks it has;
* the confidence figure is the width of a 95% bootstrap interval of the
  median (300 resamples) over the raw times of the best details, as a percent
  of the median.  The resampling here uses a seeded generator, so a report is
  reproducible (the reference draws from NumPy's global state).

Labels follow plot_results.py:20-40: an entry below 1 is shown as "↑x" (x times
faster than NumPy), above 1 as "↓x"; NumPy's own column shows its runtime.
"""
import argparse
import math
import sqlite3
import statistics
from xml.sax.saxutils import escape

import numpy as np

__all__ = ["load_results", "speedup_table", "speedup_label", "runtime_label", "to_markdown",
           "to_svg", "main"]


def load_results(db_path):
    """The ``results`` table as a list of dicts."""
    con = sqlite3.connect(db_path)
    try:
        con.row_factory = sqlite3.Row
        return [dict(r) for r in con.execute("SELECT * FROM results")]
    finally:
        con.close()


def _bootstrap_ci(times, rng, n_samples=300, alpha=0.05):
    data = np.asarray(times, dtype=np.float64)
    idx = rng.integers(0, data.shape[0], size=(n_samples, data.shape[0]))
    stat = np.sort(np.median(data[idx], axis=1))
    lo, hi = np.round((n_samples - 1) * np.array([alpha / 2, 1 - alpha / 2])).astype(int)
    return float(stat[hi] - stat[lo])


def speedup_table(rows, preset="S", baseline="numpy", seed=0):
    """Aggregates result rows as plot_results.py does.

    Returns a dict with ``frameworks`` (the baseline last), ``benchmarks``
    (sorted (benchmark, domain) pairs), ``time[(b, d)][f]`` (seconds),
    ``ratio[(b, d)][f]`` (time / baseline time), ``ci[(b, d)][f]`` (percent)
    and ``total[f]`` (geometric mean of the ratios).  Raises ValueError when the
    baseline framework has no rows for the preset.
    """
    kept = [r for r in rows
            if r.get("domain") != "" and bool(r.get("validated")) and r.get("preset") == preset
            and r.get("time") is not None]
    groups = {}
    for r in kept:
        key = (r["benchmark"], r["domain"], r["framework"], r["mode"], r["details"])
        groups.setdefault(key, []).append(float(r["time"]))
    best = {}  # (b, d, f, mode) -> (median, details)
    for (b, d, f, mode, det), ts in groups.items():
        med = statistics.median(ts)
        k = (b, d, f, mode)
        if k not in best or med < best[k][0]:
            best[k] = (med, det)
    time, raw = {}, {}
    per_mode = {}
    for (b, d, f, mode), (med, det) in best.items():
        per_mode.setdefault((b, d, f), []).append(med)
        raw.setdefault((b, d, f), []).extend(groups[(b, d, f, mode, det)])
    for (b, d, f), meds in per_mode.items():
        time.setdefault((b, d), {})[f] = sum(meds) / len(meds)
    frameworks = sorted({f for (_, _, f) in per_mode})
    if baseline not in frameworks:
        raise ValueError(f"no validated {baseline!r} rows for preset {preset!r}")
    frameworks.remove(baseline)
    frameworks.append(baseline)
    benchmarks = sorted(time, key=lambda bd: (str(bd[0]), str(bd[1])))
    rng = np.random.default_rng(seed)
    ratio, ci = {}, {}
    for bd in benchmarks:
        base = time[bd].get(baseline)
        ratio[bd] = {f: (time[bd][f] / base if base and f in time[bd] else math.nan)
                     for f in frameworks}
        ci[bd] = {}
        for f in frameworks:
            ts = raw.get((bd[0], bd[1], f))
            if ts:
                ci[bd][f] = 100.0 * _bootstrap_ci(ts, rng) / statistics.median(ts)
    total = {}
    for f in frameworks:
        vals = [ratio[bd][f] for bd in benchmarks if not math.isnan(ratio[bd][f])]
        total[f] = math.exp(sum(math.log(v) for v in vals) / len(vals)) if vals else math.nan
    return {"preset": preset, "frameworks": frameworks, "benchmarks": benchmarks, "time": time,
            "ratio": ratio, "ci": ci, "total": total, "baseline": baseline}


def speedup_label(x):
    """plot_results.py's my_speedup_abbr: ↑ faster than the baseline, ↓ slower."""
    if math.isnan(x):
        return ""
    prefix = ""
    if x < 1:
        prefix, x = "↑", 1 / x
    elif x > 1:
        prefix = "↓"
    if x > 100:
        x = int(x)
    if x > 1000:
        return f"{prefix}{x / 1000:.1f}k"
    return f"{prefix}{x:.1f}"


def runtime_label(seconds):
    """plot_results.py's my_runtime_abbr: milliseconds below 0.1 s."""
    if math.isnan(seconds):
        return ""
    if seconds < 0.1:
        return f"{seconds * 1000:.2f} ms"
    return f"{seconds:.2f} s"


def _cell(table, bd, f):
    if f == table["baseline"]:
        return runtime_label(table["time"][bd].get(f, math.nan))
    label = speedup_label(table["ratio"][bd][f])
    c = table["ci"][bd].get(f)
    if label and c is not None and int(c) > 0:
        label += f" ({int(c)}%)"
    return label


def to_markdown(table):
    fws = table["frameworks"]
    out = ["| benchmark | " + " | ".join(fws) + " |", "|---" * (len(fws) + 1) + "|"]
    out.append("| **Total** | " + " | ".join(
        speedup_label(table["total"][f]) if f != table["baseline"] else "" for f in fws) + " |")
    for bd in table["benchmarks"]:
        out.append(f"| {bd[0]} | " + " | ".join(_cell(table, bd, f) for f in fws) + " |")
    return "\n".join(out)


# ColorBrewer RdYlGn, reversed (green = faster than the baseline, red = slower),
# over plot_results.py's colour range [0, 2].
_RDYLGN_R = ["#006837", "#1a9850", "#66bd63", "#a6d96a", "#d9ef8b", "#ffffbf", "#fee08b",
             "#fdae61", "#f46d43", "#d73027", "#a50026"]


def _colour(x, vmin=0.0, vmax=2.0):
    if math.isnan(x):
        return "#ffffff"
    t = min(max((x - vmin) / (vmax - vmin), 0.0), 1.0) * (len(_RDYLGN_R) - 1)
    i = min(int(t), len(_RDYLGN_R) - 2)
    a, b = _RDYLGN_R[i], _RDYLGN_R[i + 1]
    w = t - i
    rgb = [round(int(a[1 + 2 * c:3 + 2 * c], 16) * (1 - w) + int(b[1 + 2 * c:3 + 2 * c], 16) * w)
           for c in range(3)]
    return "#" + "".join(f"{v:02x}" for v in rgb)


def to_svg(table, cell_w=90, cell_h=26, left=150, top=70):
    """The heat map as an SVG document (benchmarks down, frameworks across,
    a Total row on top; the baseline column shows its runtimes)."""
    fws, bds = table["frameworks"], table["benchmarks"]
    width = left + cell_w * len(fws) + 10
    height = top + cell_h * (len(bds) + 2) + 10
    parts = [f'<svg xmlns="http://www.w3.org/2000/svg" width="{width}" height="{height}" '
             f'font-family="sans-serif" font-size="11">',
             f'<text x="{left}" y="16" font-size="13">Runtime relative to {escape(table["baseline"])}'
             f' (preset {escape(str(table["preset"]))})</text>']
    for j, f in enumerate(fws):
        x = left + j * cell_w + cell_w / 2
        parts.append(f'<text x="{x}" y="{top - 8}" text-anchor="middle">{escape(f)}</text>')

    def row(i, name, values, labels):
        y = top + i * cell_h
        parts.append(f'<text x="{left - 6}" y="{y + cell_h / 2 + 4}" text-anchor="end">'
                     f'{escape(name)}</text>')
        for j, (v, lab) in enumerate(zip(values, labels)):
            x = left + j * cell_w
            fill = _colour(v) if fws[j] != table["baseline"] else "#ffffff"
            parts.append(f'<rect x="{x}" y="{y}" width="{cell_w}" height="{cell_h}" fill="{fill}" '
                         f'stroke="#888888" stroke-width="0.5"/>')
            t = v if not math.isnan(v) else 1.0
            t = 1 / t if t < 1 else t
            colour = "black" if fws[j] == table["baseline"] else ("#555555" if t < 1.3 else "white")
            parts.append(f'<text x="{x + cell_w / 2}" y="{y + cell_h / 2 + 4}" '
                         f'text-anchor="middle" fill="{colour}">{escape(lab)}</text>')

    row(0, "Total", [table["total"][f] for f in fws],
        [speedup_label(table["total"][f]) if f != table["baseline"] else "" for f in fws])
    for i, bd in enumerate(bds, start=2):
        row(i, str(bd[0]), [table["ratio"][bd][f] for f in fws], [_cell(table, bd, f) for f in fws])
    parts.append("</svg>")
    return "\n".join(parts) + "\n"


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--db", default="npbench.db")
    ap.add_argument("-p", "--preset", default="S", choices=["S", "M", "L", "paper"])
    ap.add_argument("--baseline", default="numpy")
    ap.add_argument("--svg", help="write the heat map to this file")
    a = ap.parse_args(argv)
    table = speedup_table(load_results(a.db), a.preset, a.baseline)
    print(to_markdown(table))
    if a.svg:
        with open(a.svg, "w") as f:
            f.write(to_svg(table))


if __name__ == "__main__":
    main()
