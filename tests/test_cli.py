"""The drop-in command-line programs (parcompfin_gb300/csrc/pcf_cli.cpp), on
the CPU: every reference program name exists, argv errors fail like the
reference's programs (no GPU needed for these)."""
import os
import subprocess

import pytest

from parcompfin_gb300 import build as B


@pytest.fixture(scope="module")
def bindir():
    B.build()
    return B.CLI_BIN


def run(path, *args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([path, *map(str, args)], capture_output=True, text=True, env=e,
                          timeout=120)


def test_every_reference_program_name_is_installed(bindir):
    for stem in ("mc_eur", "mc_eur_multi", "mc_asia", "mc_amer", "binom_embar"):
        for v in ("", "_omp", "_mpi", "_hybrid"):
            p = os.path.join(bindir, stem + v)
            assert os.path.islink(p) and os.access(p, os.X_OK), p


def test_unknown_payoff_is_an_error(bindir):
    # src/mc_eur.cpp:40 throws std::invalid_argument("Unknown payoff function").
    r = run(os.path.join(bindir, "mc_eur"), "straddle", 100, 100, .05, .2, 1, 1000)
    assert r.returncode == 1 and "Unknown payoff function" in r.stderr


def test_missing_arguments_print_usage(bindir):
    r = run(os.path.join(bindir, "mc_asia"), "call", 100, 100, .05, .2, 1, 1000)
    assert r.returncode == 2 and "usage" in r.stderr
    r = run(os.path.join(bindir, "mc_eur_omp"), "call", 100, 100, .05, .2, 1, 1000)
    assert r.returncode == 2  # the OpenMP program takes a thread count
    r = run(B.CLI)
    assert r.returncode == 2


def test_bad_number_is_an_error(bindir):
    r = run(os.path.join(bindir, "binom_embar"), "put", "abc", 100, .05, .2, 1, 1000)
    assert r.returncode == 1


def test_first_argument_selects_the_program(bindir):
    r = run(B.CLI, "mc_amer", "call", 100, 100, .05, .2, 1, 1000, 10, env={"PCF_DEVICE": "0"})
    # Either a GPU priced it (16 columns) or there is none and it says so.
    if r.returncode == 0:
        assert len(r.stdout.strip().split(",")) == 16
    else:
        assert r.returncode == 1 and r.stderr.strip()


def test_sweep_grids_follow_the_reference_scripts():
    from parcompfin_gb300 import sweeps
    # runscript_mc_eur.sh: 18 path counts; serial, 5 thread counts, 5 process
    # counts, 3 hybrid shapes.
    runs = sweeps.commands("mc_eur")
    assert len(runs) == 18 * (1 + 5 + 5 + 3)
    assert runs[0] == ("mc_eur", ["call", "100", "110", "0.02", "0.75", "1", "10000"], 1)
    assert runs[18] == ("mc_eur_omp", ["call", "100", "110", "0.02", "0.75", "1", "10000", "1"], 1)
    assert runs[-1][0] == "mc_eur_hybrid" and runs[-1][2] == 8
    # runscript_mc_asia.sh has its serial loop commented out.
    assert all(p != "mc_asia" for p, _, _ in sweeps.commands("mc_asia"))
    # runscript_binom_embar.sh runs the vanilla lattice beside each serial run.
    b = sweeps.commands("binom_embar", variants=("serial",))
    assert [p for p, _, _ in b[:2]] == ["binom_embar", "binom_vanilla_eur"]
    m = sweeps.commands("mc_eur_multi", max_n=10000, variants=("serial",))
    assert m == [("mc_eur_multi", ["call", "100", "100", "0.1", "0.2", "1", "10000", "4", "0.5"],
                  1)]
