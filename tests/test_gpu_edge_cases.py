"""Edge cases of the single-model path against the CPU oracle: ragged group
sizes (1, 127, 129, ... elements, not multiples of the 128-element blocks),
several materials and laws in one model, hexas and shells sharing nodes,
a single element; and the C-ABI's refusals of invalid input (returned
status codes, never a device fault)."""
import ctypes as C

import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (s if s > 0 else 1.0))


def compare(m, oracle_lib, ncyc=30, every=10, tol_f=1e-12, tol_x=1e-10):
    """Forces of the first cycles within tol_f; after that, as in the other
    parity tests, forces and trajectories within 1e-10."""
    from openradioss_gb300.engine import Engine
    e = Engine(m)
    o = oracle_lib.OracleModel(m, nthreads=2)
    for _ in range(2):
        e.cycle(1)
        o.cycle(1)
        assert rel(e.forces()["F"], o.nodes()["F"]) < tol_f
    for _ in range(ncyc // every):
        e.cycle(every)
        o.cycle(every)
        fg, fo = e.forces(), o.nodes()
        assert rel(fg["F"], fo["F"]) < 1e-10
        ng = e.nodes()
        assert rel(ng["X"] - m.X, fo["X"] - m.X) < tol_x
    tg, to = e.time(), o.time()
    assert abs(tg["dt2"] - to["dt2"]) <= 1e-12 * to["dt2"]
    assert tg["neltst"] == to["neltst"]
    assert e.status() == 0
    return e, o


def split_groups(m, sizes, mats=None):
    g = m.hexa[0]
    out, k = [], 0
    for i, sz in enumerate(sizes):
        mat = g.mat if mats is None else mats[i % len(mats)]
        out.append(M.HexaGroupSpec(np.ascontiguousarray(g.ixs[:, k:k + sz]), mat, g.geo))
        k += sz
    assert k == g.ixs.shape[1]
    m.hexa = out
    return m


def test_ragged_group_sizes(oracle_lib):
    m = M.bar_impact(n=7)  # 343 elements
    split_groups(m, [1, 127, 129, 86])
    compare(m, oracle_lib)


def test_two_laws_in_one_model(oracle_lib):
    m = M.large_block(n=8, seed=5)  # 512 elements, JC
    law1 = M.law1(7850.0, 210e9, 0.3)
    jc = m.hexa[0].mat
    split_groups(m, [200, 56, 256], mats=[jc, law1])
    compare(m, oracle_lib)


def test_single_element(oracle_lib):
    m = M.bar_impact(n=1)
    compare(m, oracle_lib, ncyc=20)


def test_hexa_and_shells_share_nodes(oracle_lib):
    """A hexa block with a shell skin on its top face (shells after the
    solids in the PARITH/ON slot order)."""
    n = 5
    m = M.large_block(n=n, seed=9)
    X = m.X
    top = np.where(np.isclose(X[2], X[2].max()))[0]
    # top-face quads from the hexa connectivity: nodes 5..8 of the top layer
    ixs = m.hexa[0].ixs
    ztop = X[2, ixs[5] - 1]
    sel = np.isclose(ztop, X[2].max())
    quads = ixs[5:9, sel]
    nel = quads.shape[1]
    ixc = np.zeros((7, nel), np.int32)
    ixc[0] = 2
    ixc[1:5] = quads
    ixc[5] = 2
    ixc[6] = np.arange(10001, 10001 + nel, dtype=np.int32)
    thk = np.full(nel, 1.0e-3)
    mat = M.law2(7850.0, 210e9, 0.3, 350e6, 275e6, 0.36, c=0.022, eps0=1.0)
    ms, inr = M.shell_mass_inertia(X, ixc, thk, 7850.0, ms=m.MS.copy(), inr=np.zeros(m.numnod))
    m.MS = ms
    m.IN = inr
    m.shells = [M.ShellGroupSpec(ixc, mat, M.shell_prop(1.0e-3), thk, 3)]
    assert len(top) > 0
    compare(m, oracle_lib, tol_f=1e-11)


def _ctx():
    from openradioss_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    assert L.rg_ctx_create(0, C.byref(h)) == 0
    return L, h


def test_invalid_input_is_refused():
    L, h = _ctx()
    try:
        m = M.bar_impact(n=2)
        X = np.ascontiguousarray(m.X.T.reshape(-1))
        V = np.ascontiguousarray(m.V.T.reshape(-1))
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        # cycle before set-up
        assert L.rg_cycle(h, 1) == -2
        assert L.rg_mesh_upload(h, m.numnod, p(X), p(V), p(m.MS), None, p(m.icodt)) == 0
        g = m.hexa[0]
        bad = np.ascontiguousarray(g.ixs.T.reshape(-1)).copy()
        bad[1] = m.numnod + 5  # node number out of range
        assert L.rg_hexa_group_add(h, g.ixs.shape[1], p(bad), 1, p(g.mat["pm"]), p(g.geo),
                                   None, None, 4, 1, 0) == -1
        ixs = np.ascontiguousarray(g.ixs.T.reshape(-1))
        # unsupported formulation / law
        assert L.rg_hexa_group_add(h, g.ixs.shape[1], p(ixs), 1, p(g.mat["pm"]), p(g.geo),
                                   None, None, 2, 1, 0) == -4
        assert L.rg_hexa_group_add(h, g.ixs.shape[1], p(ixs), 5, p(g.mat["pm"]), p(g.geo),
                                   None, None, 4, 1, 0) == -4
        assert L.rg_hexa_group_add(h, g.ixs.shape[1], p(ixs), 1, p(g.mat["pm"]), p(g.geo),
                                   None, None, 4, 1, 0) == 0
        assert L.rg_finalize(h, 0.9, 0.9, 1e30, 1e30) == 0
        assert L.rg_cycle(h, -1) == -1
        assert L.rg_finalize(h, 0.9, 0.9, 1e30, 1e30) == -2  # twice
        assert L.rg_cycle(h, 3) == 0
        assert L.rg_synchronize(h) == 0
        assert L.rg_status(h) == 0
    finally:
        L.rg_ctx_destroy(h)


def test_shell_npt_out_of_range_is_refused():
    from openradioss_gb300.engine import Engine, RgError
    m = M.crash_box(n_side=3, n_len=3)
    m.shells[0].npt = 6
    with pytest.raises(RgError):
        Engine(m)
