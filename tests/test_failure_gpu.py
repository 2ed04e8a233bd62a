"""Failure detection of the device-side bounded wait, without a GPU fault.

The dataflow sweep's tasks wait for their upwind tiles with a bounded poll.  A wait that
runs out sets an error word, every other wait of the sweep returns at once, the kernel
finishes, and the solve reports PGPU_ERR_TIMEOUT.  PGPU_DEBUG_SWEEP_STALL=t+1 makes task t
also wait (with a bound of a few thousand polls, about a millisecond) for a word that
nothing sets, so that wait runs out on purpose.  The test then checks that the same
problem, in the same process and context, solves correctly once the injection is off.
(The counterpart in the reference is its error propagation: an error code returned up to
the C API, src/utils.hxx:41-81.)
"""
import os

import pytest

import pampa_gb300 as pg
from helpers import rel_l2
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu


def test_sweep_wait_that_runs_out_reports_timeout_and_context_stays_usable(tmp_path, monkeypatch):
    from pampa_gb300 import workloads as wl
    # an 8x8x4 box is swept by the dataflow kernel (4x4x4 tiles): the injection applies
    path = wl.sn_3d(str(tmp_path), nx=8, ny=8, nz=4, order=4, block=2)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        monkeypatch.setenv("PGPU_DEBUG_SWEEP_STALL", "1")   # task 0 of every sweep
        with pytest.raises(pg.PampaError, match="ran out"):
            p.solve()
        monkeypatch.delenv("PGPU_DEBUG_SWEEP_STALL")
        p.solve()                                           # same problem, same context
        assert abs(p.keff - ref["keff"]) <= 1e-6, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= 1e-5
    assert "PGPU_DEBUG_SWEEP_STALL" not in os.environ


def test_injected_stall_of_a_late_task_is_also_reported(tmp_path, monkeypatch):
    """A stalled task in the middle of the sweep: its downwind tasks see the error word
    and return without waiting their own full bound."""
    from pampa_gb300 import workloads as wl
    # 2x2x2 tiles of 8x8x4 cells x 8 octants = 64 tasks; task 39 is on a middle tile diagonal
    path = wl.sn_3d(str(tmp_path), nx=16, ny=16, nz=8, order=2, block=2)
    with pg.Pampa(path, "-silent") as p:
        monkeypatch.setenv("PGPU_DEBUG_SWEEP_STALL", "40")
        with pytest.raises(pg.PampaError, match="ran out"):
            p.solve()
        monkeypatch.delenv("PGPU_DEBUG_SWEEP_STALL")
        p.solve()
        assert p.keff > 0.0


def test_injected_stall_in_an_s8_sweep_with_one_group_per_task(tmp_path, monkeypatch):
    """S8 (ten directions per octant, so one group per task): the same bounded wait and
    the same recovery, and repeated solves give the same k."""
    from pampa_gb300 import workloads as wl
    path = wl.sn_3d(str(tmp_path), nx=16, ny=16, nz=8, order=8, block=2)
    with pg.Pampa(path, "-silent") as p:
        monkeypatch.setenv("PGPU_DEBUG_SWEEP_STALL", "30")
        with pytest.raises(pg.PampaError, match="ran out"):
            p.solve()
        monkeypatch.delenv("PGPU_DEBUG_SWEEP_STALL")
        p.solve()
        k1 = p.keff
        p.solve()
        assert p.keff == k1 and k1 > 0.0


def test_injected_stall_in_the_column_sweep(tmp_path, monkeypatch):
    """A box whose sides are not multiples of 4 is swept by columns: the same bounded
    wait, error word and recovery."""
    from pampa_gb300 import workloads as wl
    path = wl.sn_3d(str(tmp_path), nx=10, ny=6, nz=5, order=4, block=2)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        monkeypatch.setenv("PGPU_DEBUG_SWEEP_STALL", "20")
        with pytest.raises(pg.PampaError, match="ran out"):
            p.solve()
        monkeypatch.delenv("PGPU_DEBUG_SWEEP_STALL")
        p.solve()
        assert abs(p.keff - ref["keff"]) <= 1e-6, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= 1e-5
