"""Shared pieces of the CRA2V44 parity tests (oracle and CUDA path).

The deck and the reference engine's outputs for it are in
tests/golden/cra2.npz (made by tests/golden/make_cra2.py).  A run goes
through both engine runs of the QA test: to t = 2.5 with the rigid link,
then (the restart deck has no /VEL card) to t = 5 without it, and keeps per
cycle the quantities the reference writes at that cycle:

* the listing record (ECRIT, output/ecrit.F:193-330): time, time step,
  controlling element, internal energy, kinetic energy and rotational
  kinetic energy of V + DT1/2 A, hourglass energy, momentum, mass;
* the nodal displacement and velocity of the time-history nodes as they are
  when the time history is written (D at the cycle's time, V half a step
  before).
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "cra2.npz")


def load_deck():
    return dict(np.load(FIX))


def printed_ok(ours, ref):
    """ours rounds to the 4-significant-digit value ref printed by ECRIT."""
    if ref == 0.0:
        return abs(ours) < 5e-4
    e = np.floor(np.log10(abs(ref)))
    return abs(ours - ref) <= 0.5 * 10.0 ** (e - 3) * 1.02


def run_both(deck, step, clear_links, nodes_of, time_of):
    """Drive a stepper through the two runs.

    step() advances one cycle and returns its listing record (dict);
    clear_links() drops the rigid link; nodes_of() returns (D, V) arrays
    (3, numnod) of the current state; time_of() the current time."""
    tstop1, tstop2 = (float(t) for t in deck["run_tstop"])
    nid = deck["th_node_ids"] - 1
    recs = ([], [])
    nodes = ([], [])
    phase = 0
    while True:
        tt = time_of()
        if phase == 0 and tt >= tstop1:
            clear_links()
            phase = 1
        if phase == 1 and tt >= tstop2:
            break
        D, V = nodes_of()
        recs[phase].append(step())
        nodes[phase].append(np.concatenate([D[:, nid].T, V[:, nid].T], axis=1))
    return recs, nodes


def check_printed(deck, recs, phase):
    table = deck["out1" if phase == 0 else "out2"]
    for row in table:
        c = int(row[0])
        r = recs[phase][c]
        for key, col in (("tt", 1), ("dt2", 2), ("eint", 4), ("ekin", 5), ("ekinr", 6)):
            assert printed_ok(r[key], row[col]), (phase, c, key, r[key], row[col])
        assert r["neltst"] == int(row[3]), (phase, c, r["neltst"], row[3])


TH_TOL = dict(IE=2e-6, KE=2e-7, XMOM=2e-7, MASS=1e-7, DT=3e-6, RKE=1e-4, HE=1e-5)
TH_KEY = dict(IE="eint", KE="ekin", XMOM="xmom", MASS="mass", DT="dt2", RKE="ekinr", HE="ehour")


def check_time_history(deck, recs, nodes, phase, tol=TH_TOL, dtol=5e-5, vtol=5e-3):
    pre = "th1" if phase == 0 else "th2"
    th_t, th_g, th_n = deck[pre + "_time"], deck[pre + "_glob"], deck[pre + "_node"]
    tts = np.array([r["tt"] for r in recs[phase]])
    cols = [str(c) for c in deck["th_glob_columns"]]
    for k, t in enumerate(th_t):
        # the time-history cycle: the one whose time matches the recorded one
        c = int(np.argmin(np.abs(tts - float(t))))
        assert abs(tts[c] - float(t)) <= 1e-3 * recs[phase][c]["dt2"], (phase, k, t, tts[c])
        r = recs[phase][c]
        for name, rel in tol.items():
            ref = float(th_g[k][cols.index(name)])
            if ref != 0.0:
                assert abs(r[TH_KEY[name]] - ref) <= rel * abs(ref), (phase, k, name, r[TH_KEY[name]], ref)
        dn = np.abs(nodes[phase][c] - th_n[k])
        assert dn[:, :3].max() <= dtol, (phase, k, dn[:, :3].max())
        assert dn[:, 3:].max() <= vtol, (phase, k, dn[:, 3:].max())
    assert len(th_t) == 50


# per-part time history (the 7 sums SBILAN / CBILAN accumulate, relative;
# momentum relative to the part's momentum norm): a few times the oracle's
# differences (IE 8e-7, KE 1.3e-5, momentum 2.2e-5, MASS 3.4e-8, HE 3.7e-6)
PART_TOL = dict(IE=3e-6, KE=5e-5, MOM=1e-4, MASS=1e-7, HE=1.5e-5)


def check_part_history(deck, recs, phase, tol=PART_TOL, tmatch=1e-3):
    """Every time-history output of the part variables IE, KE, XMOM, YMOM,
    ZMOM, MASS, HE against rec["parts"] (npart x 7) of the matching cycle
    (its time within tmatch time steps of the output's)."""
    pre = "th1" if phase == 0 else "th2"
    th_t, th_p = deck[pre + "_time"], deck[pre + "_part"]
    tts = np.array([r["tt"] for r in recs[phase]])
    for k, t in enumerate(th_t):
        c = int(np.argmin(np.abs(tts - float(t))))
        assert abs(tts[c] - float(t)) <= tmatch * recs[phase][c]["dt2"], (phase, k, t, tts[c])
        ours = recs[phase][c]["parts"]
        ref = th_p[k].astype(np.float64)
        assert ours.shape == (ref.shape[0], 7)
        for p in range(ref.shape[0]):
            mom = np.abs(ref[p, 2:5]).max()
            for q, name in enumerate(("IE", "KE", "XMOM", "YMOM", "ZMOM", "MASS", "HE")):
                rel = tol["MOM"] if name.endswith("MOM") else tol[name]
                scale = mom if name.endswith("MOM") else abs(ref[p, q])
                assert abs(ours[p, q] - ref[p, q]) <= rel * scale + 1e-12, (phase, k, p, name,
                                                                             ours[p, q], ref[p, q])


def listing_from_velocities(MS, IN, V0, V1, VR0, VR1, dt1, dt2):
    """ECRIT's kinetic energies from the velocities before (V0 = V at
    t - DT1/2) and after (V1 = V at t + DT2/2) a cycle: the cycle's
    acceleration is (V1 - V0) / DT12, so V + DT1/2 A = V0 + DT1/(DT1 + DT2)
    (V1 - V0).  Also the momentum and mass."""
    w = dt1 / (dt1 + dt2) if dt1 + dt2 > 0 else 0.0
    V = V0 + w * (V1 - V0)
    VR = VR0 + w * (VR1 - VR0)
    ek = float(np.sum(0.5 * MS * np.sum(V * V, axis=0)))
    ekr = float(np.sum(0.5 * IN * np.sum(VR * VR, axis=0)))
    mom = (MS * V).sum(axis=1)
    return dict(ekin=ek, ekinr=ekr, xmom=float(mom[0]), ymom=float(mom[1]), zmom=float(mom[2]),
                mass=float(MS.sum()))
