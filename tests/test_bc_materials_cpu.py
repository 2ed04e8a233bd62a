"""Boundary-condition and split materials in the oracle and the host parser (no GPU).

The oracle's restatement of Mesh::splitMaterials / removeBCMaterials (Mesh.cxx:24-204)
must turn the split strips into the boundaries edge-0 and edge-1 and drop their cells,
and the condition on edge-1 must reach the operator.  The host C++ parser behind
pampa_initialize must build the same reduced mesh (field sizes), without touching a GPU.
"""
import numpy as np

import pampa_gb300 as pg
from helpers import bc_split_input
from oracle import pampa_oracle as po


def test_oracle_splits_and_removes_bc_materials(tmp_path):
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    pa = bc_split_input(str(tmp_path / "a"), right="reflective")
    pb = bc_split_input(str(tmp_path / "b"), right="vacuum")
    prob = po.read_problem(pa)
    assert prob.mesh.n == 68
    assert prob.mesh.boundaries == ["-x", "+x", "-y", "+y", "edge", "edge-0", "edge-1"]
    assert [m.name for m in prob.materials] == ["fuel", "refl", "edge", "edge-0", "edge-1"]
    # the removed strips' neighbours now point at the new boundaries
    nb = prob.mesh.neighbors
    assert np.any(nb == -(prob.mesh.boundaries.index("edge-0") + 1))
    assert np.any(nb == -(prob.mesh.boundaries.index("edge-1") + 1))
    Ra, _ = po.assemble_diffusion(prob)
    Rb, _ = po.assemble_diffusion(po.read_problem(pb))
    assert abs(Ra - Rb).sum() > 0.0       # edge-1 reflective vs vacuum changes the operator


def test_host_parser_builds_the_reduced_mesh(tmp_path):
    path = bc_split_input(str(tmp_path))
    with pg.Pampa(path, "-silent") as p:
        assert p.field_size("power") == 68
        assert p.field_size("scalar-flux") == 68 * 2
