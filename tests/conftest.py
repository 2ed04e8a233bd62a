import gzip
import json
import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def known_answers() -> dict:
    with open(os.path.join(GOLDEN, "known_answers.json")) as fh:
        return json.load(fh)


def materialize_case(case: str, dest: str) -> str:
    """Decompress a golden case (and its family's materials) under `dest`; return input path."""
    fam = case.split("/")[0]
    for sub in (case, f"{fam}/materials"):
        src = os.path.join(GOLDEN, "cases", sub)
        out = os.path.join(dest, sub)
        os.makedirs(out, exist_ok=True)
        for f in os.listdir(src):
            if f.endswith(".gz"):
                with gzip.open(os.path.join(src, f), "rb") as fi, open(os.path.join(out, f[:-3]), "wb") as fo:
                    shutil.copyfileobj(fi, fo)
    return os.path.join(dest, case, "input.pmp")


@pytest.fixture
def case_input(tmp_path):
    def make(case: str) -> str:
        return materialize_case(case, str(tmp_path))
    return make


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
