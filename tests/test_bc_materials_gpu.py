"""Boundary-condition and split materials (Mesh::splitMaterials and removeBCMaterials,
Mesh.cxx:24-204) through the drop-in driver on the GPU, against the oracle: the split
strips become two boundaries with their own conditions, the strips' cells leave the mesh.
"""
import pytest

import pampa_gb300 as pg
from helpers import bc_split_input, rel_l2
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver", ["diffusion", "sn"])
@pytest.mark.parametrize("right", ["reflective", "vacuum"])
def test_split_bc_material(solver, right, tmp_path):
    path = bc_split_input(str(tmp_path), solver, right)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        assert p.field_size("power") == 68
        assert abs(p.keff - ref["keff"]) <= 1e-6, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= 1e-5
        assert rel_l2(p.field("power"), ref["q"]) <= 1e-5
