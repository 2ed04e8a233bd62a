"""CPU-only checks of the shipped library: it loads, exports every declared symbol, and
the host half of the drop-in API (parser, meshes, materials) behaves like the reference's
without touching a GPU."""
import ctypes as C
import os
import re

import pytest

import pampa_gb300 as pg
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "pampa_gb300.h")


def declared_functions() -> list[str]:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pampa_\w+|pgpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = pg.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(pg.SYMBOLS), set(names) ^ set(pg.SYMBOLS)


def test_default_options():
    o = pg.default_options()
    assert o.precision == pg.PGPU_FP64 and o.tol_k == 1e-10 and o.max_outer == 5000


@pytest.mark.parametrize("case", ["slabs/reflected-diffusion", "pwr-iaea-benchmark/unstructured-sn",
                                  "pwr-iaea-benchmark/cartesian-diffusion-3d"])
def test_initialize_parses_reference_inputs(case, case_input):
    from oracle import pampa_oracle as po
    path = case_input(case)
    prob = po.read_problem(path)
    with pg.Pampa(path, "-silent") as p:
        phi = p.field("scalar-flux")
        assert phi.size == prob.mesh.n * prob.G
        assert p.field("power").size == prob.mesh.n
        if prob.solver == "sn":
            M = prob.order * (prob.order + 2)
            assert p.field("angular-flux").size == prob.mesh.n * prob.G * M


def test_initialize_reports_errors(tmp_path, capfd):
    bad = tmp_path / "input.pmp"
    bad.write_text("mesh cartesian missing.pmp\n")
    with pytest.raises(pg.PampaError):
        pg.Pampa(str(bad), "-silent")
    out = capfd.readouterr().out
    assert "error: unable to open" in out


def test_set_field_roundtrip(case_input):
    import numpy as np
    with pg.Pampa(case_input("slabs/reflected-diffusion"), "-silent") as p:
        T = np.linspace(300, 900, p.field("temperature").size)
        p.set_field("temperature", T)
        assert np.array_equal(p.field("temperature"), T)
        with pytest.raises(pg.PampaError):
            p.field("no-such-field")


def test_angular_flux_field_before_a_solve_and_set(case_input):
    """The SN angular flux (kept on the device after a solve) reads as zeros before any
    solve, as the reference's new vector, and a value set by the caller reads back."""
    import numpy as np
    with pg.Pampa(case_input("slabs/reflected-s4"), "-silent") as p:
        psi = p.field("angular-flux")
        assert psi.size > 0 and not np.any(psi)
        v = np.arange(psi.size, dtype=np.float64) * 0.5
        p.set_field("angular-flux", v)
        assert np.array_equal(p.field("angular-flux"), v)


@pytest.mark.parametrize("opts,msg", [(["-pgpu_precision", "fp16"], "wrong -pgpu_precision"),
                                      (["-pgpu_shift", "-1"], "wrong -pgpu_shift"),
                                      (["-pgpu_max_outer", "0"], "wrong -pgpu_max_outer"),
                                      (["-pgpu_device", "x"], "wrong -pgpu_device")])
def test_gpu_options_are_checked(opts, msg, case_input, capfd):
    """Bad GPU options fail pampa_initialize with the reference's error convention (a
    file:line: error: message line and *error > 0)."""
    with pytest.raises(pg.PampaError):
        pg.Pampa(case_input("slabs/reflected-diffusion"), "-silent", *opts)
    assert msg in capfd.readouterr().out


@pytest.mark.parametrize("block,msg", [("solver diffusion {\n   energy-groups 0\n}\n", "error"),
                                       ("solver sn {\n   energy-groups 2\n   order 10\n}\n", "error"),
                                       ("solver nothing {\n}\n", "error")])
def test_solver_block_errors(block, msg, case_input, capfd):
    path = case_input("slabs/reflected-diffusion")
    text = open(path).read()
    head = text[:text.index("solver diffusion")]
    with open(path, "w") as fh:
        fh.write(head + block)
    with pytest.raises(pg.PampaError):
        pg.Pampa(path, "-silent")
    assert msg in capfd.readouterr().out
