"""The results pipeline (parcompfin_gb300/results.py): reading files in the
reference's 16-column results format, pairing reference and GPU runs, and the
table and SVG outputs. The inputs are small CSV files written here in that
format (values invented for the test)."""
import math
import xml.etree.ElementTree as ET

import pytest

from parcompfin_gb300 import results

HEADER = ("Method,Payoff,S0,E,r,sigma,T,N,M,Parallel,Nr_of_assets,T_overall,T_calculation,"
          "Result,Abs_Error,Error")

REF = """{h}
Serial,call,100,110,0.02,0.75,1,10000,0,0,1,0.0032,0.0031,26.38,0.2275,-0.2275
Serial,call,100,110,0.02,0.75,1,80000,0,0,1,0.0185,0.0184,26.77,0.1603,0.1603
OMP,call,100,110,0.02,0.75,1,10000,0,8,1,0.0010,0.0008,26.50,0.1100,-0.1100
OMP,call,100,110,0.02,0.75,1,10000,0,8,1,0.0012,0.0010,26.52,0.0900,-0.0900
Serial,call,100,110,0.02,0.75,1,160000,0,0,1,0.0360,0.0358,26.60,0.0100,-0.0100
""".format(h=HEADER)

GPU = """{h}
Serial,call,100,110,0.02,0.75,1,10000,0,0,1,0.2500,0.000155,26.59,0.0215,-0.0215
Serial,call,100,110,0.02,0.75,1,80000,0,0,1,0.2510,0.000184,26.62,0.0089,0.0089
OMP,call,100,110,0.02,0.75,1,10000,0,8,1,0.2490,0.000160,26.60,0.0120,-0.0120
{h}
Serial,call,100,110,0.02,0.75,1,320000,0,0,1,0.2520,0.000190,26.61,0.0012,-0.0012
""".format(h=HEADER)


@pytest.fixture
def files(tmp_path):
    r, g = tmp_path / "ref.csv", tmp_path / "gpu.csv"
    r.write_text(REF)
    g.write_text(GPU)
    return str(r), str(g)


def test_load_types_and_repeated_headers(files):
    ref, gpu = (results.load(p) for p in files)
    assert len(ref) == 5 and len(gpu) == 4  # the second header line is skipped
    r = ref[0]
    assert r["Method"] == "Serial" and r["Payoff"] == "call"
    assert isinstance(r["N"], int) and r["N"] == 10000
    assert isinstance(r["Parallel"], int) and isinstance(r["Nr_of_assets"], int)
    assert r["Result"] == pytest.approx(26.38) and r["Error"] == pytest.approx(-0.2275)


def test_load_rejects_a_short_line(tmp_path):
    p = tmp_path / "bad.csv"
    p.write_text(HEADER + "\nSerial,call,100\n")
    with pytest.raises(ValueError):
        results.load(str(p))


def test_pairs_runs_by_parameters_and_averages_repeats(files):
    ref, gpu = (results.load(p) for p in files)
    rows = results.compare(ref, gpu)
    assert [(r["Method"], r["N"]) for r in rows] == [("Serial", 10000), ("Serial", 80000),
                                                     ("OMP", 10000)]
    omp = rows[2]
    assert omp["ref_runs"] == 2 and omp["gpu_runs"] == 1
    assert omp["ref_Result"] == pytest.approx(26.51)          # mean of the two repeats
    assert omp["ref_T_calculation"] == pytest.approx(0.0009)
    assert omp["result_diff"] == pytest.approx(26.60 - 26.51)
    assert omp["speedup"] == pytest.approx(0.0009 / 0.000160)
    only_ref, only_gpu = results.unmatched(ref, gpu)
    assert len(only_ref) == 1 and len(only_gpu) == 1


def test_markdown_and_csv_tables(files, tmp_path):
    ref, gpu = (results.load(p) for p in files)
    rows = results.compare(ref, gpu)
    md = results.markdown(rows)
    lines = md.strip().splitlines()
    assert len(lines) == 2 + len(rows)
    assert all(l.count("|") == lines[0].count("|") for l in lines)
    out = tmp_path / "t.csv"
    results.write_csv(rows, str(out))
    back = out.read_text().strip().splitlines()
    assert len(back) == 1 + len(rows) and back[0].startswith("Method,")


def test_svg_plots_are_well_formed(files, tmp_path):
    ref, gpu = (results.load(p) for p in files)
    paths = results.plots(ref, gpu, str(tmp_path / "plots" / "mc_eur"))
    assert [p.rsplit("_", 1)[1] for p in paths] == ["time.svg", "error.svg"]
    for p in paths:
        root = ET.parse(p).getroot()
        assert root.tag.endswith("svg")
        ns = "{http://www.w3.org/2000/svg}"
        lines = root.findall(f"{ns}polyline")
        # ref Serial, ref OMP (8), GPU Serial, GPU OMP (8)
        assert len(lines) == 4
        for pl in lines:
            for pt in pl.get("points").split():
                x, y = map(float, pt.split(","))
                assert math.isfinite(x) and math.isfinite(y)


def test_svg_plot_drops_points_a_log_axis_cannot_show(tmp_path):
    p = tmp_path / "p.svg"
    results.svg_plot({"a": [(1, 0.0), (10, 1.0), (100, 2.0)], "b": []}, str(p), "t", "x", "y")
    root = ET.parse(str(p)).getroot()
    pl = root.findall("{http://www.w3.org/2000/svg}polyline")
    assert len(pl) == 1 and len(pl[0].get("points").split()) == 2


def test_command_line(files, tmp_path, capsys):
    md = tmp_path / "t.md"
    assert results.main([files[0], files[1], "--md", str(md), "--svg-prefix",
                         str(tmp_path / "s")]) == 0
    assert md.read_text().startswith("| Method |")
    assert (tmp_path / "s_time.svg").exists() and (tmp_path / "s_error.svg").exists()
    assert "3 parameter sets in both" in capsys.readouterr().out


def test_command_line_method_filter(files, tmp_path, capsys):
    md = tmp_path / "t.md"
    assert results.main([files[0], files[1], "--md", str(md), "--method", "OMP"]) == 0
    body = md.read_text().strip().splitlines()[2:]
    assert len(body) == 1 and body[0].startswith("| OMP |")
