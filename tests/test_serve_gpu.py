"""Serving (pgpu_serve_*): requests of uneven sizes and group counts solved concurrently on
one GPU give the same results as each solved alone, and match the oracle.

Bars: every keff and flux bitwise equal alone and in the mix (each solve has its own
device state, its grids are sized by the server's SM share rather than by what else
runs, and the reductions are deterministic); against the oracle |dk| <= 1e-6 and
flux relative L2 <= 1e-5 in FP64, 1 pcm and 1e-4 in mixed precision.
"""
import numpy as np
import pytest

import pampa_gb300 as pg
from helpers import rel_l2
from oracle import pampa_oracle as po
from pampa_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SHAPES = [((6, 5, 4), 2), ((8, 8, 4), 4), ((5, 4, 3), 7), ((12, 8, 6), 2), ((7, 9, 5), 4), ((4, 4, 8), 7),
          ((10, 10, 4), 2), ((6, 6, 6), 4)]


def _requests(seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for (nx, ny, nz), G in SHAPES:
        op, mats, layout = wl.diffusion_request(rng, nx, ny, nz, G, block=2)
        out.append(dict(op=op, mats=mats, layout=layout, shape=(nx, ny, nz), G=G))
    return out


def _solve_all(reqs, slots, precision, one_at_a_time=False):
    res = []
    with pg.Server(slots=slots) as srv:
        opts = pg.default_options(precision=precision)
        if one_at_a_time:  # each request alone on the device: submitted after the previous answer
            for r in reqs:
                res.append(srv.wait(srv.submit_diffusion(r["op"], opts, want_flux=True)))
        else:
            ids = [srv.submit_diffusion(r["op"], opts, want_flux=True) for r in reqs]
            res = [srv.wait(rid) for rid in ids]
    for out in res:
        assert out["status"] == pg.PGPU_OK, out.get("error")
    return res


@pytest.mark.parametrize("precision", [pg.PGPU_FP64, pg.PGPU_MIXED])
def test_alone_equals_in_the_mix(precision):
    reqs = _requests()
    # same server configuration (4 slots, so the same SM share per solve), requests alone
    # on the device, then all eight queued at once
    alone = _solve_all(reqs, 4, precision, one_at_a_time=True)
    mixed = _solve_all(reqs, 4, precision)
    for a, b in zip(alone, mixed):
        assert a["keff"] == b["keff"]
        assert np.array_equal(a["phi"], b["phi"])


def test_served_results_match_oracle(tmp_path):
    reqs = _requests()[:3]
    out64 = _solve_all(reqs, 3, pg.PGPU_FP64)
    out32 = _solve_all(reqs, 3, pg.PGPU_MIXED)
    for k, (r, a, b) in enumerate(zip(reqs, out64, out32)):
        nx, ny, nz = r["shape"]
        path = wl.write_diffusion_input(str(tmp_path / f"r{k}"), nx, ny, nz, 2.0, r["layout"], r["mats"])
        ref = po.run_input(path)
        assert abs(a["keff"] - ref["keff"]) <= 1e-6, (a["keff"], ref["keff"])
        assert abs(b["keff"] - ref["keff"]) <= 1e-5, (b["keff"], ref["keff"])
        # the server returns the normalised scalar flux, as the drop-in's scalar-flux field
        assert rel_l2(a["phi"], ref["phi"]) <= 1e-5
        assert rel_l2(b["phi"], ref["phi"]) <= 1e-4


def test_request_above_the_budget_is_rejected():
    rng = np.random.default_rng(3)
    op, _, _ = wl.diffusion_request(rng, 4, 4, 4, 2)
    with pg.Server(slots=1, hbm_fraction=1e-9) as srv:
        with pytest.raises(pg.PampaError, match="failed"):
            srv.submit_diffusion(op)
