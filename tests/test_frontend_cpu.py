"""The reference's unmodified C front end (src/c/main.c), compiled against its own header
(src/pampa.hxx), links against libpampa_gb300.so: the drop-in needs no source change.

Needs the reference checkout: PAMPA_REFERENCE, else a directory named "reference" next to
this repository; skipped without it.
Without a GPU the solve fails, so the run is checked up to the first solve: the printed
lines match the reference's golden output, and the error is reported through the
reference's convention (a message, then "Error in pampa_solve()." and exit status 1).
"""
import json
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT, gpu_available, materialize_case

REF = os.environ.get("PAMPA_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
MAIN_C = os.path.join(REF, "src", "c", "main.c")


@pytest.mark.skipif(not os.path.exists(MAIN_C), reason="reference checkout not available")
def test_reference_front_end_links_and_runs_to_the_solve(tmp_path):
    import pampa_gb300.build as b
    lib = b.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "pampa_ref_main")
    subprocess.run(["gcc", "-O2", "-I", os.path.join(REF, "src"), MAIN_C, "-L", libdir, "-lpampa_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    case = "slabs/reflected-diffusion"
    path = materialize_case(case, str(tmp_path))
    res = subprocess.run([exe, "input.pmp"], cwd=os.path.dirname(path), capture_output=True, text=True,
                         timeout=300)
    expected = json.load(open(os.path.join(GOLDEN, "check_ref_stdout.json")))[case]
    got = res.stdout.split("\n")
    head = expected.index("Solve steady state...") + 2
    assert got[:head] == expected[:head]
    if gpu_available():
        assert res.returncode == 0
    else:
        assert res.returncode == 1
        assert "Error in pampa_solve()." in res.stdout


def test_own_front_end_compiles_against_the_header(tmp_path):
    import pampa_gb300.build as b
    lib = b.build()
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-O2", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "frontend", "pampa_main.c"), "-L", libdir, "-lpampa_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(tmp_path / "pampa")], check=True)


def test_precursor_golden_case_without_a_gpu(tmp_path):
    """pwr-iaea-benchmark/cartesian-precursors-3d runs the precursor solver alone (steady
    state and four steps; PrecursorSolver.cxx), which needs no GPU: the front end's output
    must equal the reference's printed lines, including "Precursor population: 0.000e+00
    (min), 1.424e-06 (max)." at every step."""
    import pampa_gb300.build as b
    lib = b.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "pampa")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "frontend", "pampa_main.c"), "-L", libdir, "-lpampa_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    case = "pwr-iaea-benchmark/cartesian-precursors-3d"
    path = materialize_case(case, str(tmp_path))
    res = subprocess.run([exe, "input.pmp"], cwd=os.path.dirname(path), capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout[-2000:]
    expected = json.load(open(os.path.join(GOLDEN, "check_ref_stdout.json")))[case]
    strip = lambda ls: ls[:max(i for i, x in enumerate(ls) if x) + 1]  # noqa: E731
    assert strip(res.stdout.split("\n")) == strip(expected)
