"""The reference's own test method, on the GPU library: a C front end runs every golden
input and its standard output is compared line by line with what the reference printed
(test/check_ref.txt, via tests/golden/check_ref_stdout.json).

check.sh runs `pampa input.pmp` in each case's directory and diffs the printed summary
(check.sh:113-117): "Effective multiplication factor" to 6 decimals
(NeutronicSolver.cxx:122), "Power" to 3, and for the 3D cases four transient steps with
"Time step size", "Physical time" and "Power" (Driver.cxx:59-75).  The front end here
(tests/frontend/pampa_main.c) drives the calls in the order of the reference's C front end
(src/c/main.c:16-29) and links against libpampa_gb300.so.  Two golden values come from
the reference's uninitialised least-squares matrix on 2D SN meshes (SNSolver.cxx:247-252);
for those the keff line is checked to 5e-5 and every other line exactly.
"""
import json
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT, materialize_case

pytestmark = pytest.mark.gpu

LS_2D = {"pwr-iaea-benchmark/cartesian-sn", "pwr-iaea-benchmark/unstructured-sn"}
CASES = sorted(json.load(open(os.path.join(GOLDEN, "check_ref_stdout.json"))))


@pytest.fixture(scope="module")
def frontend(tmp_path_factory):
    import pampa_gb300.build as b
    lib = b.build()
    exe = str(tmp_path_factory.mktemp("frontend") / "pampa")
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "frontend", "pampa_main.c"), "-L", libdir, "-lpampa_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


def _strip(lines):
    lines = list(lines)
    while lines and lines[-1] == "":
        lines.pop()
    return lines


@pytest.mark.parametrize("case", CASES)
def test_reference_check_output(case, frontend, tmp_path):
    expected = _strip(json.load(open(os.path.join(GOLDEN, "check_ref_stdout.json")))[case])
    path = materialize_case(case, str(tmp_path))
    res = subprocess.run([frontend, "input.pmp"], cwd=os.path.dirname(path), capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    got = _strip(res.stdout.split("\n"))
    assert len(got) == len(expected), "\n".join(got)
    for g, e in zip(got, expected):
        if case in LS_2D and e.startswith("Effective multiplication factor"):
            kg = float(g.split(":")[1].rstrip("."))
            ke = float(e.split(":")[1].rstrip("."))
            assert abs(kg - ke) <= 5e-5, (g, e)
        else:
            assert g == e
