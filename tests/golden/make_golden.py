"""Regenerate the golden fixtures from the reference project's own test suite.

Reads (only when this script runs, in a container that has the reference checkout):
  <reference>/test/check_ref.txt            -> known_answers.json (printed keff per case)
                                               check_ref_stdout.json (the lines the reference
                                               printed for each case's first run)
  <reference>/test/<case>/input.pmp, mesh   -> cases/<case>/... (gzipped .pmp files)
  <reference>/test/<family>/materials/*.pmp -> cases/<family>/materials/

Usage: python tests/golden/make_golden.py <reference checkout>
       (or with the checkout in the PAMPA_REFERENCE environment variable)
"""
from __future__ import annotations

import gzip
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    "slabs/reflected-diffusion", "slabs/reflected-s2", "slabs/reflected-s4",
    "pwr-iaea-benchmark/cartesian-diffusion", "pwr-iaea-benchmark/cartesian-diffusion-3d",
    "pwr-iaea-benchmark/cartesian-sn", "pwr-iaea-benchmark/unstructured-diffusion",
    "pwr-iaea-benchmark/unstructured-diffusion-3d", "pwr-iaea-benchmark/unstructured-sn",
    "pwr-iaea-benchmark/cartesian-precursors-3d",
]


def parse_check_ref(path: str) -> dict:
    """First 'Effective multiplication factor' printed after each 'Run <case>...' line."""
    out = {}
    case = None
    with open(path) as fh:
        for line in fh:
            m = re.match(r"Run (\S+)\.\.\.", line.strip())
            if m:
                case = m.group(1)
                continue
            m = re.match(r"Effective multiplication factor: ([0-9.]+)\.", line.strip())
            if m and case and case not in out:
                out[case] = float(m.group(1))
    return out


def parse_check_ref_stdout(path: str) -> dict:
    """Lines printed by the reference for the first run of each case (check.sh runs
    `pampa input.pmp` after printing "Run <case>...", and prints "Rerun..." before a second
    run or "Done." once the case is over; neither line is the program's)."""
    lines = open(path).read().split("\n")
    out = {}
    k = 0
    while k < len(lines):
        m = re.match(r"Run (\S+)\.\.\.$", lines[k])
        if not m:
            k += 1
            continue
        case = m.group(1)
        j = k + 1
        while j < len(lines) and lines[j] != "Rerun..." and not re.match(r"Run \S+\.\.\.$", lines[j]):
            j += 1
        block = lines[k + 1:j]
        while block and block[-1] == "":
            block.pop()
        if j >= len(lines) or lines[j] != "Rerun...":
            block.pop()  # check.sh's own "Done." after the case
            while block and block[-1] == "":
                block.pop()
        out[case] = block
        k = j
    return out


def main(ref: str):
    test = os.path.join(ref, "test")
    answers = parse_check_ref(os.path.join(test, "check_ref.txt"))
    stdout = parse_check_ref_stdout(os.path.join(test, "check_ref.txt"))
    cases_dir = os.path.join(HERE, "cases")
    if os.path.isdir(cases_dir):
        shutil.rmtree(cases_dir)
    families = set()
    for case in CASES:
        src = os.path.join(test, case)
        dst = os.path.join(cases_dir, case)
        os.makedirs(dst, exist_ok=True)
        for f in ("input.pmp", "mesh.pmp"):
            with open(os.path.join(src, f), "rb") as fi, gzip.GzipFile(os.path.join(dst, f + ".gz"), "wb", 9, mtime=0) as fo:
                fo.write(fi.read())
        families.add(case.split("/")[0])
    for fam in sorted(families):
        src = os.path.join(test, fam, "materials")
        dst = os.path.join(cases_dir, fam, "materials")
        os.makedirs(dst, exist_ok=True)
        for f in sorted(x for x in os.listdir(src) if x.endswith(".pmp")):
            with open(os.path.join(src, f), "rb") as fi, gzip.GzipFile(os.path.join(dst, f + ".gz"), "wb", 9, mtime=0) as fo:
                fo.write(fi.read())
    with open(os.path.join(HERE, "known_answers.json"), "w") as fh:
        json.dump({c: answers[c] for c in CASES if c in answers}, fh, indent=1, sort_keys=True)
    with open(os.path.join(HERE, "check_ref_stdout.json"), "w") as fh:
        json.dump({c: stdout[c] for c in CASES}, fh, indent=1, sort_keys=True)
    print(f"wrote {len(CASES)} cases")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PAMPA_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set PAMPA_REFERENCE)")
    main(ref)
