"""Feedback nuclear data on the GPU path against the oracle: the operator is assembled
with every cell's cross sections interpolated at the cell's temperature
(FeedbackNuclearData.hxx:60-140, the "temperature" input field), and is rebuilt when a
caller sets a new temperature field between solves, as a coupled heat-conduction solver
does.  Bars as for the other solves: k within 1e-6, flux within 1e-5 relative L2."""
import pytest

import pampa_gb300 as pg
from helpers import feedback_input, feedback_temperatures, rel_l2
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver", ["diffusion", "sn"])
def test_feedback_cross_sections_follow_the_temperature(solver, tmp_path):
    path = feedback_input(str(tmp_path), solver)
    prob = po.read_problem(path)
    cold = po.solve_problem(prob)
    prob.T = feedback_temperatures(prob.mesh.n)
    hot = po.solve_problem(prob)
    with pg.Pampa(path, "-silent") as p:
        p.solve()                                   # temperature field 0: the first data sets
        assert abs(p.keff - cold["keff"]) <= 1e-6, (p.keff, cold["keff"])
        assert rel_l2(p.field("scalar-flux"), cold["phi"]) <= 1e-5
        p.set_field("temperature", prob.T)
        p.solve()                                   # the operator follows the new field
        assert abs(p.keff - hot["keff"]) <= 1e-6, (p.keff, hot["keff"])
        assert rel_l2(p.field("scalar-flux"), hot["phi"]) <= 1e-5
        assert rel_l2(p.field("power"), hot["q"]) <= 1e-5
    assert hot["keff"] < cold["keff"]
