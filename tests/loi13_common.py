"""Shared pieces of the LOI13 parity tests (oracle and CUDA path).

The deck and the reference engine's outputs for it are in
tests/golden/loi13.npz (made by tests/golden/make_loi13.py): a block of 464
Johnson-Cook one-point hexas in the co-rotational frame with three
rigid-material (LAW13) parts, crushed by an imposed-velocity ramp, one
engine run of 1636 cycles.  A run keeps per cycle the listing record
(ECRIT, output/ecrit.F:193-330).
"""
from __future__ import annotations

import os

import numpy as np

from cra2_common import printed_ok

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "loi13.npz")

# time-history tolerances (the file holds float32): relative for the
# energies, step and mass; momenta relative to the momentum's norm
TH_TOL = dict(IE=1e-6, KE=1e-6, EXTW=1e-6, HE=1e-6, DT=1e-6, MASS=1e-7)
TH_KEY = dict(IE="eint", KE="ekin", EXTW="wfext", HE="ehour", DT="dt2", MASS="mass")
MOM_TOL = 1e-6


def load_deck():
    return dict(np.load(FIX))


def run(deck, step, time_of):
    """Drive a stepper to the run's end time; step() advances one cycle and
    returns its listing record."""
    tstop = float(deck["run_tstop"])
    recs = []
    while time_of() < tstop:
        recs.append(step())
    return recs


def jc_elements(model):
    return {int(e) for g in model.hexa for e in g.ixs[10]}


def check_printed(deck, model, recs, rel=None):
    """Every printed cycle: time, time step, internal, kinetic and rotational
    kinetic energy, external work and mass to the printed digits (or within
    rel relative plus the print rounding), the energy error to its printed
    tenth of a percent, and the controlling element one of the Johnson-Cook
    block (at cycle 0 the regular block's elements tie to round-off)."""
    jc = jc_elements(model)
    for row in deck["out"]:
        c = int(row[0])
        r = recs[c]
        for key, col in (("tt", 1), ("dt2", 2), ("eint", 5), ("ekin", 6), ("ekinr", 7),
                         ("wfext", 8), ("mass", 10)):
            ref = row[col]
            if rel is None:
                assert printed_ok(r[key], ref), (c, key, r[key], ref)
            else:
                half = 0.5 * 10.0 ** (np.floor(np.log10(abs(ref))) - 3) if ref else 5e-4
                assert abs(r[key] - ref) <= rel * abs(ref) + half, (c, key, r[key], ref)
        if rel is None and r["wfext"]:
            err = (r["eint"] + r["ekin"] + r["ekinr"]) / r["wfext"] - 1.0
            assert abs(100.0 * err - row[4]) <= 0.0501, (c, 100.0 * err, row[4])
        assert r["neltst"] in jc, (c, r["neltst"])
        if c > 0:
            assert r["neltst"] == int(row[3]), (c, r["neltst"], row[3])


def check_time_history(deck, recs, tol=TH_TOL, mom_tol=MOM_TOL):
    tts = np.array([r["tt"] for r in recs])
    cols = [str(c) for c in deck["th_glob_columns"]]
    ix = [cols.index(k) for k in ("XMOM", "YMOM", "ZMOM")]
    for k, t in enumerate(deck["th_time"]):
        c = int(np.argmin(np.abs(tts - float(t))))
        assert abs(tts[c] - float(t)) <= 1e-3 * recs[c]["dt2"], (k, t, tts[c])
        r = recs[c]
        for name, rel in tol.items():
            ref = float(deck["th_glob"][k][cols.index(name)])
            if ref != 0.0:
                assert abs(r[TH_KEY[name]] - ref) <= rel * abs(ref), (k, name, r[TH_KEY[name]], ref)
        ref = np.array([float(deck["th_glob"][k][i]) for i in ix])
        got = np.array([r["xmom"], r["ymom"], r["zmom"]])
        scale = np.linalg.norm(ref)
        if scale > 0:
            assert np.max(np.abs(got - ref)) <= mom_tol * scale, (k, got, ref)
    assert len(deck["th_time"]) == 801
