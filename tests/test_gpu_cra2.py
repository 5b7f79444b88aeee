"""The CUDA path on the reference engine's QA deck CRA2V44 (GPU).

The same deck and reference outputs as tests/test_oracle_cra2.py (768
Belytschko-Tsay shells, /SHFRA/V4 frame, Ithick = 0, NPT = 3 radial return,
rigid link with 500 t added mass, restart without the link; 3375 cycles),
run through the C ABI (Engine -> librg.so):

* FP64 form: the reference's printed cycle table to every printed digit,
  the controlling element of every printed cycle, and the time histories
  within the tolerances the oracle meets;
* mixed form (FP32 element arithmetic): the printed time, time step,
  internal and kinetic energy within the mixed form's accuracy bound
  (1e-4 relative), and the time histories' energies likewise.

The listing record of a cycle is formed from what the C ABI returns: the
element energies (rg_energy), the time record (rg_get_time) and the nodal
velocities before and after the cycle (rg_download_nodes), whose difference
gives the cycle's acceleration for ECRIT's V + DT1/2 A.
"""
import numpy as np
import pytest

from cra2_common import (PART_TOL, check_part_history, check_printed, check_time_history,
                         listing_from_velocities, load_deck, printed_ok, run_both)
from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def deck():
    return load_deck()


def gpu_run(deck, precision):
    from openradioss_gb300.engine import Engine

    m = M.model_from_deck(deck, "cra2")
    e = Engine(m, precision=precision)
    state = {}

    def nodes_of():
        nd = e.nodes()
        state["V0"], state["VR0"] = nd["V"], nd["VR"]
        return nd["D"], nd["V"]

    def step():
        e.part_sums_due()
        e.cycle(1)
        t = e.time()
        en = e.energy()
        nd = e.nodes()
        rec = listing_from_velocities(m.MS, m.IN, state["V0"], nd["V"], state["VR0"], nd["VR"],
                                      t["dt1"], t["dt2"])
        rec.update(tt=t["tt"] - t["dt2"], dt2=t["dt2"], neltst=t["neltst"], eint=en["eint"],
                   ehour=en["ehour"], parts=e.part_sums())
        return rec

    try:
        out = run_both(deck, step, lambda: e.set_link_active(0, False), nodes_of,
                       lambda: e.time()["tt"])
        assert e.status() == 0
    finally:
        e.close()
    return out


@pytest.fixture(scope="module")
def fp64(deck):
    from openradioss_gb300.engine import RG_PREC_FP64

    return gpu_run(deck, RG_PREC_FP64)


@pytest.fixture(scope="module")
def mixed(deck):
    from openradioss_gb300.engine import RG_PREC_MIXED

    return gpu_run(deck, RG_PREC_MIXED)


@pytest.mark.parametrize("phase", [0, 1])
def test_fp64_printed_table(deck, fp64, phase):
    check_printed(deck, fp64[0], phase)


@pytest.mark.parametrize("phase", [0, 1])
def test_fp64_time_history(deck, fp64, phase):
    check_time_history(deck, fp64[0], fp64[1], phase)


@pytest.mark.parametrize("phase", [0, 1])
def test_fp64_part_time_history(deck, fp64, phase):
    """The device's per-part sums (rg_part_sums, taken every cycle here)
    against the reference's /TH/PART outputs, within the oracle's
    tolerances."""
    check_part_history(deck, fp64[0], phase)


@pytest.mark.parametrize("phase", [0, 1])
def test_mixed_part_time_history(deck, mixed, phase):
    """Mixed form: the per-part sums within the mixed form's bound (1e-4
    relative, the mass to its FP64 accuracy: it depends on coordinates and
    the FP64 thickness only).  The mixed run's cycle times stay within
    1e-2 of a step of the reference's (3e-7 relative by t = 4.6)."""
    tol = {k: max(v, 1e-4) for k, v in PART_TOL.items()}
    tol["MASS"] = 1e-6
    check_part_history(deck, mixed[0], phase, tol=tol, tmatch=1e-2)


def test_fp64_cycle_count(deck, fp64):
    # run 1 stops at the same cycle as the reference: the restart's cycle 0
    # is printed at t = 2.501
    assert printed_ok(fp64[0][1][0]["tt"], deck["out2"][0, 1])
    assert len(fp64[0][1]) > int(deck["out2"][-1, 0])


@pytest.mark.parametrize("phase", [0, 1])
def test_mixed_within_bound(deck, mixed, phase):
    """Mixed form against the reference's printed values: time, time step,
    internal and kinetic energy within 1e-4 relative plus the print
    rounding."""
    recs = mixed[0]
    table = deck["out1" if phase == 0 else "out2"]
    for row in table:
        r = recs[phase][int(row[0])]
        for key, col in (("tt", 1), ("dt2", 2), ("eint", 4), ("ekin", 5)):
            ref = row[col]
            half = 0.5 * 10.0 ** (np.floor(np.log10(abs(ref))) - 3) if ref else 5e-4
            assert abs(r[key] - ref) <= 1e-4 * abs(ref) + half, (phase, int(row[0]), key, r[key], ref)


def test_fp64_matches_oracle(deck, fp64):
    """Over the first 200 cycles (before the buckling amplifies round-off)
    the FP64 form and the oracle agree to round-off: energies, time step and
    the per-part sums within 1e-12 relative, time-history node values within
    1e-9."""
    from oracle.oracle import OracleModel

    o = OracleModel(M.model_from_deck(deck, "cra2"))
    o.set_record(True)
    recs, nodes = [], []
    nid = deck["th_node_ids"] - 1
    for c in range(200):
        nd = o.nodes()
        nodes.append(np.concatenate([nd["D"][:, nid].T, nd["V"][:, nid].T], axis=1))
        o.cycle(1)
        r = o.record()
        r["parts"] = o.part_sums()
        recs.append(r)
    g, gn = fp64[0][0], fp64[1][0]
    for c in range(200):
        for key in ("eint", "ekin", "dt2", "ehour", "tt"):
            ref = recs[c][key]
            assert abs(g[c][key] - ref) <= 1e-12 * abs(ref) + 1e-12, (c, key, g[c][key], ref)
        # the controlling element: equal, except between elements whose time
        # steps tie to round-off (the regular mesh has many equal ones)
        if g[c]["neltst"] != recs[c]["neltst"]:
            assert abs(g[c]["dt2"] - recs[c]["dt2"]) <= 1e-13 * recs[c]["dt2"], c
        assert np.abs(gn[c] - nodes[c]).max() <= 1e-9, c
        # per-part sums (chunked fixed-order tree vs sequential sums)
        pg, po = g[c]["parts"], recs[c]["parts"]
        scale = np.maximum(np.abs(po), np.abs(po[:, 2:5]).max(axis=1, keepdims=True))
        assert (np.abs(pg - po) <= 1e-12 * scale + 1e-12).all(), (c, pg, po)
