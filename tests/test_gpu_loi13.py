"""The CUDA path as a drop-in FORINT on the reference engine's QA deck
LOI13/solide (GPU): Johnson-Cook hexas in the co-rotational frame crushed
plastically, beside rigid-material bodies and an imposed velocity.

Every cycle the engine's RESOL (here the oracle's, with the deck's
rigid-material bodies and imposed velocity, fed through or_set_forces)
hands the nodal state to the FORINT-level call (rg_forint_step, host
buffers), which runs the Johnson-Cook group on the device and returns the
PARITH/ON-assembled forces, STIFN and the element time step; the listing
takes the element energies from the device (rg_energy).  The run must
reproduce what the reference engine wrote for the deck
(tests/golden/loi13.npz):

* FP64 form: every printed digit of the 17 printed cycles and the
  801-sample time history within the tolerances the oracle meets
  (energies 1e-6 relative), and the oracle's own run within 1e-9 over the
  1636 cycles;
* mixed form (FP32 element arithmetic): the printed time, step, energies and
  external work within 1e-4 relative plus the print rounding.
"""
import numpy as np
import pytest

from loi13_common import check_printed, check_time_history, load_deck, run
from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def deck():
    return load_deck()


def drop_in_run(deck, precision):
    from openradioss_gb300.engine import Engine
    from oracle.oracle import OracleModel

    m = M.rigid_jc_model_from_deck(deck, "loi13")
    e = Engine(m, precision=precision, elements_only=True)
    o = OracleModel(M.rigid_jc_model_from_deck(deck, "loi13"), nthreads=2)
    o.set_record(True)
    n = m.numnod
    x, v, f, st = np.empty((n, 3)), np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
    for a in (x, v, f, st):
        e.host_register(a)

    def step():
        nd = o.nodes()
        x[:] = nd["X"].T
        v[:] = nd["V"].T
        _, _, dt2t, el = e.forint_step(x, v, o.time()["dt2"], f=f, stifn=st)
        o.set_forces(f, st, dt2t, el)
        o.cycle(1)
        r = o.record()
        en = e.energy()
        r["eint"], r["ehour"] = en["eint"], en["ehour"]
        return r

    try:
        recs = run(deck, step, lambda: o.time()["tt"])
        assert e.status() == 0 and o.error() == 0
        final = o.nodes()
    finally:
        for a in (x, v, f, st):
            e.host_unregister(a)
        e.close()
    return m, recs, final


@pytest.fixture(scope="module")
def fp64(deck):
    from openradioss_gb300.engine import RG_PREC_FP64

    return drop_in_run(deck, RG_PREC_FP64)


def test_fp64_printed_table(deck, fp64):
    m, recs, _ = fp64
    check_printed(deck, m, recs)


def test_fp64_time_history(deck, fp64):
    _, recs, _ = fp64
    check_time_history(deck, recs)


def test_fp64_matches_oracle_run(deck, fp64):
    from oracle.oracle import OracleModel

    m, recs, final = fp64
    o = OracleModel(M.rigid_jc_model_from_deck(deck, "loi13"), nthreads=2)
    o.cycle(len(recs))
    no = o.nodes()
    s = np.abs(no["X"] - m.X).max()
    assert np.abs(final["X"] - no["X"]).max() <= 1e-9 * s
    assert np.abs(final["V"] - no["V"]).max() <= 1e-9 * np.abs(no["V"]).max()
    assert abs(recs[-1]["eint"] - o.energy()["eint"]) <= 1e-9 * o.energy()["eint"]


def test_mixed_within_bound(deck):
    from openradioss_gb300.engine import RG_PREC_MIXED

    m, recs, _ = drop_in_run(deck, RG_PREC_MIXED)
    check_printed(deck, m, recs, rel=1e-4)
