"""Feedback nuclear data (FeedbackNuclearData.hxx:60-140) in the oracle and the host
parser: linear interpolation between the data sets of the reference temperatures,
clamped outside them, and an operator that follows the temperature field."""
import numpy as np
import pytest

import pampa_gb300 as pg
from helpers import feedback_input, feedback_temperatures
from oracle import pampa_oracle as po


def test_interpolation_rule(tmp_path):
    prob = po.read_problem(feedback_input(str(tmp_path)))
    m = prob.materials[1]
    assert m.tref == [300.0, 600.0, 1200.0]
    s0, s1, s2 = m.sets
    assert np.array_equal(m.at(100.0).st, s0.st)            # below the first: first set
    assert np.array_equal(m.at(5000.0).st, s2.st)           # above the last: last set
    assert np.array_equal(m.at(600.0).st, s1.st)            # on an inner reference value
    assert np.allclose(m.at(450.0).st, 0.5 * s0.st + 0.5 * s1.st, rtol=1e-15)
    assert np.allclose(m.at(1000.0).D, (1 / 3) * s1.D + (2 / 3) * s2.D, rtol=1e-14)


def test_operator_follows_the_temperature_field(tmp_path):
    prob = po.read_problem(feedback_input(str(tmp_path)))
    R0, F0 = po.assemble_diffusion(prob)
    prob.T = feedback_temperatures(prob.mesh.n)
    R1, F1 = po.assemble_diffusion(prob)
    assert abs(R1 - R0).sum() > 0 and abs(F1 - F0).sum() > 0
    k0 = po.solve_problem(po.read_problem(feedback_input(str(tmp_path))))["keff"]
    k1 = po.solve_problem(prob)["keff"]
    assert k1 < k0                                            # hotter fuel: less reactive


def test_host_parser_reads_feedback_materials(tmp_path):
    path = feedback_input(str(tmp_path))
    with pg.Pampa(path, "-silent") as p:
        assert p.field_size("temperature") == 100
        p.set_field("temperature", feedback_temperatures(100))


def test_reference_temperatures_must_match_the_sets(tmp_path, capfd):
    path = feedback_input(str(tmp_path))
    text = open(tmp_path / "mat2.pmp").read().replace("temperature 3", "temperature 2").replace(
        "300.0 600.0 1200.0", "300.0 600.0")
    open(tmp_path / "mat2.pmp", "w").write(text)
    with pytest.raises(pg.PampaError):
        pg.Pampa(path, "-silent")
    assert "one nuclear-data set is needed per reference temperature" in capfd.readouterr().out
