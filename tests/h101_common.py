"""Shared pieces of the H101 parity tests (oracle and CUDA path).

The deck and the reference engine's outputs for it are in
tests/golden/h101.npz (made by tests/golden/make_h101.py): six elastic
cantilevers of co-rotational one-point hexas, each with a rigid body at its
tip loaded by a constant concentrated force, one engine run of 848 cycles.
A run keeps per cycle the listing record (ECRIT, output/ecrit.F:193-330,
with RBYCOR's rigid-body corrections) and the displacement and velocity of
the six main nodes as they are when the time history is written (D at the
cycle's time, V half a step before).
"""
from __future__ import annotations

import os

import numpy as np

from cra2_common import printed_ok

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "h101.npz")

# time-history tolerances (relative; the file holds float32): global
# variables, and the main nodes' D and V relative to their largest value
TH_TOL = dict(IE=1e-6, KE=1e-6, RKE=1e-6, EXTW=1e-6, HE=1e-6, DT=1e-6, MASS=1e-7, ZMOM=1e-6)
TH_KEY = dict(IE="eint", KE="ekin", RKE="ekinr", EXTW="wfext", HE="ehour", DT="dt2",
              MASS="mass", ZMOM="zmom")


def load_deck():
    return dict(np.load(FIX))


def run(deck, step, nodes_of, time_of):
    """Drive a stepper to the run's end time.  step() advances one cycle and
    returns its listing record; nodes_of() gives (D, V) of the main nodes
    (3, 6 arrays) before the cycle."""
    tstop = float(deck["run_tstop"])
    recs, nodes = [], []
    while time_of() < tstop:
        D, V = nodes_of()
        nodes.append(np.concatenate([D.T, V.T], axis=1))
        recs.append(step())
    return recs, nodes


def part_of(model):
    return {int(e): int(g.ixs[9][0]) for g in model.hexa for e in g.ixs[10]}


def check_printed(deck, model, recs, rel=None):
    """Every printed cycle: time, time step, internal, kinetic and rotational
    kinetic energy, external work and mass to the printed digits (or within
    rel relative plus the print rounding), the energy error to its printed
    tenth of a percent, and the controlling element: the printed one or one
    of the same part (the parts are regular meshes whose elements' steps tie
    to round-off)."""
    parts = part_of(model)
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
        if rel is None:
            err = (r["eint"] + r["ekin"] + r["ekinr"]) / r["wfext"] - 1.0 if r["wfext"] else 0.0
            assert abs(100.0 * err - row[4]) <= 0.0501, (c, 100.0 * err, row[4])
        assert parts[r["neltst"]] == parts[int(row[3])], (c, r["neltst"], row[3])


def check_time_history(deck, recs, nodes, tol=TH_TOL, ntol=1e-6):
    tts = np.array([r["tt"] for r in recs])
    cols = [str(c) for c in deck["th_glob_columns"]]
    scale = np.abs(deck["th_node"]).max(axis=(0, 1))
    for k, t in enumerate(deck["th_time"]):
        c = int(np.argmin(np.abs(tts - float(t))))
        assert abs(tts[c] - float(t)) <= 1e-3 * recs[c]["dt2"], (k, t, tts[c])
        r = recs[c]
        for name, rel in tol.items():
            ref = float(deck["th_glob"][k][cols.index(name)])
            if ref != 0.0:
                assert abs(r[TH_KEY[name]] - ref) <= rel * abs(ref), (k, name, r[TH_KEY[name]], ref)
        dn = np.abs(nodes[c] - deck["th_node"][k]) / scale
        # VY is two orders below the other components: its own scale
        assert dn[:, [0, 1, 2, 3, 5]].max() <= ntol, (k, dn.max(axis=0))
        assert dn[:, 4].max() <= 1e-4, (k, dn[:, 4].max())
    assert len(deck["th_time"]) == 200
