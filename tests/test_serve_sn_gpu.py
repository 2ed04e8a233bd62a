"""Serving SN requests (pgpu_serve_submit_sn): discrete-ordinates solves of uneven sizes,
orders and sweep forms run concurrently on one GPU give the same results as each solved
alone, and match the oracle.

Bars: keff and scalar flux bitwise equal alone and in the mix (each solve has its own
device state and stream; its sweep grid is sized from the device, not from what else
runs; every cell's update is made by one thread in a fixed order and the reductions are
deterministic); against the oracle |dk| <= 1e-6 and flux relative L2 <= 1e-5 in FP64,
1e-5 and 1e-4 in mixed precision.
"""
import numpy as np
import pytest

import pampa_gb300 as pg
from helpers import rel_l2, sn_operator_from_oracle
from oracle import pampa_oracle as po
from pampa_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

# (nx, ny, nz, order): boxes the tile sweep takes (sides multiples of 4) and boxes swept by
# per-cell upwind levels, S2 to S8, and one box given without its Cartesian dimensions
SHAPES = [(8, 8, 4, 4), (12, 8, 6, 2), (16, 16, 8, 8), (6, 5, 4, 4), (10, 6, 5, 6), (16, 8, 8, 2)]


def _requests(tmp_path, shapes=SHAPES):
    out = []
    for k, (nx, ny, nz, order) in enumerate(shapes):
        path = wl.sn_3d(str(tmp_path / f"sn{k}"), nx=nx, ny=ny, nz=nz, order=order, block=2, seed=20 + k)
        prob = po.read_problem(path)
        # the last box is given without its Cartesian dimensions: upwind-level sweep
        cart = (nx, ny, nz) if k != len(shapes) - 1 else (0, 0, 0)
        out.append(dict(path=path, prob=prob, op=sn_operator_from_oracle(prob, cart)))
    return out


def _solve_all(reqs, slots, precision, one_at_a_time=False):
    opts = pg.default_options(precision=precision)
    with pg.Server(slots=slots) as srv:
        if one_at_a_time:
            res = [srv.wait(srv.submit_sn(r["op"], opts, want_flux=True)) for r in reqs]
        else:
            ids = [srv.submit_sn(r["op"], opts, want_flux=True) for r in reqs]
            res = [srv.wait(rid) for rid in ids]
    for out in res:
        assert out["status"] == pg.PGPU_OK, out.get("error")
    return res


def test_operator_arrays_apply_as_the_assembled_matrix(tmp_path):
    """The operator arrays built for serving are the SN operator: R x on the GPU equals
    the oracle's assembled R times x."""
    r = _requests(tmp_path, [(8, 8, 4, 4)])[0]
    R, _, _ = po.assemble_sn(r["prob"])
    x = np.random.default_rng(5).random(R.shape[0])
    arrays = dict(r["op"])
    arrays.pop("cart")
    with pg.SNProblem(**arrays) as p:
        y = p.apply(x)
    assert rel_l2(y, R @ x) <= 1e-13


@pytest.mark.parametrize("precision", [pg.PGPU_FP64, pg.PGPU_MIXED])
def test_sn_alone_equals_in_the_mix(tmp_path, precision):
    reqs = _requests(tmp_path)
    alone = _solve_all(reqs, 3, precision, one_at_a_time=True)
    mixed = _solve_all(reqs, 3, precision)
    for a, b in zip(alone, mixed):
        assert a["keff"] == b["keff"]
        assert np.array_equal(a["phi"], b["phi"])


def test_served_sn_matches_oracle_and_mixes_with_diffusion(tmp_path):
    reqs = _requests(tmp_path, [(8, 8, 4, 4), (6, 5, 4, 2)])
    rng = np.random.default_rng(9)
    dop, _, _ = wl.diffusion_request(rng, 8, 8, 4, 2, block=2)
    for precision, dk, dphi in [(pg.PGPU_FP64, 1e-6, 1e-5), (pg.PGPU_MIXED, 1e-5, 1e-4)]:
        opts = pg.default_options(precision=precision)
        with pg.Server(slots=3) as srv:
            ids = [srv.submit_sn(r["op"], opts, want_flux=True) for r in reqs]
            did = srv.submit_diffusion(dop, opts, want_flux=True)
            outs = [srv.wait(i) for i in ids]
            assert srv.wait(did)["status"] == pg.PGPU_OK
        for r, out in zip(reqs, outs):
            assert out["status"] == pg.PGPU_OK, out.get("error")
            ref = po.run_input(r["path"])
            assert abs(out["keff"] - ref["keff"]) <= dk, (out["keff"], ref["keff"])
            assert rel_l2(out["phi"], ref["phi"]) <= dphi
