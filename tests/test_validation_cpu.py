"""Argument and operator checks of the C-ABI, on CPU.

Every check below happens before the library touches a device, so a malformed request
is refused with PGPU_ERR_INVALID and a message on any machine (the reference's
equivalent is its PETSc/ input-checking error path: `*error > 0` plus a message)."""
import ctypes as C

import numpy as np
import pytest

import pampa_gb300 as pg
from pampa_gb300 import workloads as wl


def _op():
    op, _, _ = wl.diffusion_request(np.random.default_rng(0), 4, 3, 2, 2)
    return op


def test_diffusion_operator_index_checks():
    op = _op()
    bad = dict(op, materials=op["materials"].copy())
    bad["materials"][3] = 9
    with pytest.raises(pg.PampaError, match="material index out of range"):
        pg.DiffusionProblem(**bad)
    nb = op["neighbors"].copy()
    nb[1, 0] = nb.shape[1]
    with pytest.raises(pg.PampaError, match="neighbour index out of range"):
        pg.DiffusionProblem(**dict(op, neighbors=nb))


@pytest.mark.parametrize("n,G,F,nm,msg", [(0, 2, 6, 1, "bad operator sizes"), (4, 0, 6, 1, "bad operator sizes"),
                                          (4, 2, 6, 0, "bad operator sizes"), (1, 17, 0, 1, "more than 16")])
def test_diffusion_operator_size_checks(n, G, F, nm, msg):
    h = C.c_void_p(None)
    op = pg.pgpu_diffusion_operator(n, G, F, nm)
    assert pg.lib().pgpu_diffusion_create(0, C.byref(op), C.byref(h)) == pg.PGPU_ERR_INVALID
    assert msg in pg.last_error()
    assert not h.value


def test_null_arguments():
    h = C.c_void_p(None)
    assert pg.lib().pgpu_diffusion_create(0, None, C.byref(h)) == pg.PGPU_ERR_INVALID
    assert pg.lib().pgpu_sn_create(0, None, C.byref(h)) == pg.PGPU_ERR_INVALID
    assert pg.lib().pgpu_problem_set_sm_share(None, 4) == pg.PGPU_ERR_INVALID


@pytest.mark.parametrize("slots,fraction", [(0, 0.5), (257, 0.5), (4, 0.0), (4, 1.5)])
def test_serving_argument_checks(slots, fraction):
    srv = C.c_void_p(None)
    assert pg.lib().pgpu_serve_create(0, slots, fraction, C.byref(srv)) == pg.PGPU_ERR_INVALID
    assert not srv.value
    assert pg.lib().pgpu_serve_set_sm_share(None, 4) == pg.PGPU_ERR_INVALID
