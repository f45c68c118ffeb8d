"""Side-by-side tables and plots of reference and GPU runs.

The reference's experiments write results/results_<method>.csv: one line per
run in the 16 columns of reporting() (include/common.h:212-249),

    Method,Payoff,S0,E,r,sigma,T,N,M,Parallel,Nr_of_assets,T_overall,
    T_calculation,Result,Abs_Error,Error

The drop-in programs (pcf_cli) and sweeps.run_sweep() write the same
columns. This module reads two such files, pairs the runs that share their
parameters (Method, Payoff, S0, E, r, sigma, T, N, M, Parallel,
Nr_of_assets; repeated runs of one key are averaged), and writes

  * a table (Markdown or CSV): both results, their difference, both errors
    against the comparison value, both calculation times and the speed-up;
  * SVG line plots, drawn here without a plotting library: calculation time
    against N and absolute error against N, one line per method and side,
    on log axes.

    python -m parcompfin_gb300.results REF.csv GPU.csv --md table.md \\
        --svg-prefix plots/mc_eur
"""
from __future__ import annotations

import argparse
import csv
import math
import os
from xml.sax.saxutils import escape

COLUMNS = ("Method", "Payoff", "S0", "E", "r", "sigma", "T", "N", "M", "Parallel",
           "Nr_of_assets", "T_overall", "T_calculation", "Result", "Abs_Error", "Error")
KEY = ("Method", "Payoff", "S0", "E", "r", "sigma", "T", "N", "M", "Parallel", "Nr_of_assets")
_INT = {"N", "M", "Parallel", "Nr_of_assets"}
_STR = {"Method", "Payoff"}
_VALUES = ("T_overall", "T_calculation", "Result", "Abs_Error", "Error")


def load(path: str) -> list:
    """Rows of a results CSV as dicts with typed values. Lines that repeat
    the header (several sweeps appended to one file) are skipped."""
    rows = []
    with open(path, newline="") as f:
        rd = csv.reader(f)
        header = None
        for rec in rd:
            if not rec or not "".join(rec).strip():
                continue
            if rec[0] == "Method":
                header = rec
                continue
            if header is None:
                header = list(COLUMNS)
            if len(rec) != len(header):
                raise ValueError(f"{path}: {len(rec)} fields where the header has {len(header)}")
            row = {}
            for k, v in zip(header, rec):
                v = v.strip()
                if k in _STR:
                    row[k] = v
                elif k in _INT:
                    row[k] = int(float(v))
                else:
                    row[k] = float(v)
            missing = [k for k in COLUMNS if k not in row]
            if missing:
                raise ValueError(f"{path}: missing columns {missing}")
            rows.append(row)
    return rows


def _key(row) -> tuple:
    return tuple(round(row[k], 12) if isinstance(row[k], float) else row[k] for k in KEY)


def _mean_by_key(rows) -> dict:
    acc = {}
    for r in rows:
        a = acc.setdefault(_key(r), {"n": 0, **{v: 0.0 for v in _VALUES}})
        a["n"] += 1
        for v in _VALUES:
            a[v] += r[v]
    return {k: {"runs": a["n"], **{v: a[v] / a["n"] for v in _VALUES}} for k, a in acc.items()}


def compare(ref_rows, gpu_rows) -> list:
    """One dict per parameter set present in both inputs, in the reference's
    order: the key columns, then ref_* and gpu_* values, the difference of the
    results and the speed-up of the calculation time (ref / gpu)."""
    ref, gpu = _mean_by_key(ref_rows), _mean_by_key(gpu_rows)
    out, seen = [], set()
    for r in ref_rows:
        k = _key(r)
        if k in seen or k not in gpu:
            continue
        seen.add(k)
        a, b = ref[k], gpu[k]
        row = dict(zip(KEY, k))
        for v in _VALUES:
            row["ref_" + v] = a[v]
            row["gpu_" + v] = b[v]
        row["ref_runs"], row["gpu_runs"] = a["runs"], b["runs"]
        row["result_diff"] = b["Result"] - a["Result"]
        row["speedup"] = a["T_calculation"] / b["T_calculation"] if b["T_calculation"] > 0 \
            else math.inf
        out.append(row)
    return out


def unmatched(ref_rows, gpu_rows) -> tuple:
    """Parameter sets found only in the reference file, and only in the GPU file."""
    rk = {_key(r) for r in ref_rows}
    gk = {_key(r) for r in gpu_rows}
    return sorted(rk - gk, key=str), sorted(gk - rk, key=str)


_TABLE = (("Method", "Method", "{}"), ("Payoff", "Payoff", "{}"), ("N", "N", "{}"),
          ("M", "M", "{}"), ("Parallel", "Parallel", "{}"), ("Nr_of_assets", "assets", "{}"),
          ("ref_Result", "ref result", "{:.10g}"), ("gpu_Result", "GPU result", "{:.10g}"),
          ("result_diff", "GPU - ref", "{:.3g}"), ("ref_Abs_Error", "ref abs error", "{:.3g}"),
          ("gpu_Abs_Error", "GPU abs error", "{:.3g}"), ("ref_T_calculation", "ref s", "{:.4g}"),
          ("gpu_T_calculation", "GPU s", "{:.4g}"), ("speedup", "speed-up", "{:.3g}"))


def markdown(rows) -> str:
    head = "| " + " | ".join(h for _, h, _ in _TABLE) + " |"
    rule = "|" + "|".join("---" for _ in _TABLE) + "|"
    lines = [head, rule]
    for r in rows:
        lines.append("| " + " | ".join(f.format(r[k]) for k, _, f in _TABLE) + " |")
    return "\n".join(lines) + "\n"


def write_csv(rows, path: str) -> None:
    if not rows:
        cols = list(KEY)
    else:
        cols = list(rows[0].keys())
    with open(path, "w", newline="") as f:
        w = csv.DictWriter(f, fieldnames=cols)
        w.writeheader()
        for r in rows:
            w.writerow(r)


# ---- SVG line plots ----

_COLORS = ("#1f77b4", "#d62728", "#2ca02c", "#9467bd", "#ff7f0e", "#8c564b", "#e377c2",
           "#7f7f7f", "#bcbd22", "#17becf")


def _ticks(lo: float, hi: float, log: bool) -> list:
    if log:
        a, b = math.floor(math.log10(lo)), math.ceil(math.log10(hi))
        return [10.0 ** e for e in range(a, b + 1)]
    step = 10 ** math.floor(math.log10(max(hi - lo, 1e-300)))
    if (hi - lo) / step < 4:
        step /= 2
    t, out = math.floor(lo / step) * step, []
    while t <= hi + 1e-12 * step:
        out.append(t)
        t += step
    return out


def svg_plot(series: dict, path: str, title: str, xlabel: str, ylabel: str,
             logx: bool = True, logy: bool = True, width: int = 720, height: int = 440) -> None:
    """series: {label: [(x, y), ...]}. Points with a non-positive coordinate
    on a log axis are left out. Writes a standalone SVG file."""
    pts = {k: [(x, y) for x, y in v if (x > 0 or not logx) and (y > 0 or not logy)
               and math.isfinite(x) and math.isfinite(y)] for k, v in series.items()}
    allp = [p for v in pts.values() for p in v]
    ml, mr, mt, mb = 80, 190, 40, 60
    pw, ph = width - ml - mr, height - mt - mb
    out = [f'<svg xmlns="http://www.w3.org/2000/svg" width="{width}" height="{height}" '
           f'font-family="sans-serif" font-size="12">',
           f'<rect width="{width}" height="{height}" fill="white"/>',
           f'<text x="{ml + pw / 2}" y="22" text-anchor="middle" font-size="14">{escape(title)}</text>']
    if allp:
        xs, ys = [p[0] for p in allp], [p[1] for p in allp]
        x0, x1, y0, y1 = min(xs), max(xs), min(ys), max(ys)
        if x1 == x0:
            x0, x1 = (x0 / 2, x0 * 2) if logx else (x0 - 1, x0 + 1)
        if y1 == y0:
            y0, y1 = (y0 / 2, y0 * 2) if logy else (y0 - 1, y0 + 1)
        xt, yt = _ticks(x0, x1, logx), _ticks(y0, y1, logy)
        x0, x1 = min(x0, xt[0]), max(x1, xt[-1])
        y0, y1 = min(y0, yt[0]), max(y1, yt[-1])
        fx = (lambda v: math.log10(v)) if logx else (lambda v: v)
        fy = (lambda v: math.log10(v)) if logy else (lambda v: v)
        X = lambda v: ml + (fx(v) - fx(x0)) / (fx(x1) - fx(x0)) * pw
        Y = lambda v: mt + ph - (fy(v) - fy(y0)) / (fy(y1) - fy(y0)) * ph
        for t in xt:
            out.append(f'<line x1="{X(t):.1f}" y1="{mt}" x2="{X(t):.1f}" y2="{mt + ph}" '
                       f'stroke="#e0e0e0"/>')
            out.append(f'<text x="{X(t):.1f}" y="{mt + ph + 16}" text-anchor="middle">{t:.3g}</text>')
        for t in yt:
            out.append(f'<line x1="{ml}" y1="{Y(t):.1f}" x2="{ml + pw}" y2="{Y(t):.1f}" '
                       f'stroke="#e0e0e0"/>')
            out.append(f'<text x="{ml - 6}" y="{Y(t) + 4:.1f}" text-anchor="end">{t:.3g}</text>')
        for i, (label, v) in enumerate(pts.items()):
            if not v:
                continue
            c = _COLORS[i % len(_COLORS)]
            v = sorted(v)
            d = " ".join(f"{X(x):.1f},{Y(y):.1f}" for x, y in v)
            out.append(f'<polyline points="{d}" fill="none" stroke="{c}" stroke-width="1.5"/>')
            for x, y in v:
                out.append(f'<circle cx="{X(x):.1f}" cy="{Y(y):.1f}" r="2.5" fill="{c}"/>')
            ly = mt + 14 + 18 * i
            out.append(f'<line x1="{ml + pw + 12}" y1="{ly - 4}" x2="{ml + pw + 32}" y2="{ly - 4}" '
                       f'stroke="{c}" stroke-width="2"/>')
            out.append(f'<text x="{ml + pw + 38}" y="{ly}">{escape(label)}</text>')
    out.append(f'<rect x="{ml}" y="{mt}" width="{pw}" height="{ph}" fill="none" stroke="black"/>')
    out.append(f'<text x="{ml + pw / 2}" y="{height - 14}" text-anchor="middle">{escape(xlabel)}</text>')
    out.append(f'<text x="16" y="{mt + ph / 2}" text-anchor="middle" '
               f'transform="rotate(-90 16 {mt + ph / 2})">{escape(ylabel)}</text>')
    out.append("</svg>")
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def _by_method(rows, value: str) -> dict:
    """{(Method, Parallel): [(N, mean value)]} from raw rows."""
    acc = {}
    for r in rows:
        acc.setdefault((r["Method"], r["Parallel"]), {}).setdefault(r["N"], []).append(r[value])
    return {k: sorted((n, sum(v) / len(v)) for n, v in d.items()) for k, d in acc.items()}


def plots(ref_rows, gpu_rows, prefix: str, parallel=None) -> list:
    """Calculation time and absolute error against N, reference and GPU, one
    line per method (and thread / process count, or only `parallel`)."""
    written = []
    for value, name, ylabel in (("T_calculation", "time", "calculation time (s)"),
                                ("Abs_Error", "error", "|result - comparison|")):
        series = {}
        for side, rows in (("ref", ref_rows), ("GPU", gpu_rows)):
            for (method, par), v in sorted(_by_method(rows, value).items()):
                if parallel is not None and par != parallel:
                    continue
                label = f"{side} {method}" + (f" ({par})" if par else "")
                series[label] = v
        path = f"{prefix}_{name}.svg"
        svg_plot(series, path, f"{os.path.basename(prefix)}: {ylabel} against N", "N", ylabel)
        written.append(path)
    return written


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("ref", help="the reference's results CSV")
    ap.add_argument("gpu", help="the GPU programs' results CSV (same columns)")
    ap.add_argument("--md", help="write the side-by-side table as Markdown here")
    ap.add_argument("--csv", help="write the side-by-side table as CSV here")
    ap.add_argument("--svg-prefix", help="write <prefix>_time.svg and <prefix>_error.svg")
    ap.add_argument("--parallel", type=int, default=None,
                    help="plot only this thread / process count")
    ap.add_argument("--method", action="append", default=None,
                    help="keep only runs with this Method label (repeatable)")
    a = ap.parse_args(argv)
    ref, gpu = load(a.ref), load(a.gpu)
    if a.method:
        ref = [r for r in ref if r["Method"] in a.method]
        gpu = [r for r in gpu if r["Method"] in a.method]
    rows = compare(ref, gpu)
    only_ref, only_gpu = unmatched(ref, gpu)
    if a.md:
        with open(a.md, "w") as f:
            f.write(markdown(rows))
    if a.csv:
        write_csv(rows, a.csv)
    if a.svg_prefix:
        plots(ref, gpu, a.svg_prefix, a.parallel)
    if not (a.md or a.csv):
        print(markdown(rows), end="")
    print(f"{len(rows)} parameter sets in both; {len(only_ref)} only in the reference file, "
          f"{len(only_gpu)} only in the GPU file")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
