"""The oracle's per-part sums (SBILAN / CBILAN PARTSAV, CHVIS3's hourglass
energy) on known answers (CPU).

* a rigid translation: every node moving with the same velocity v, each
  element's kinetic energy is 1/2 XMAS |v|^2 and its momentum XMAS v, so a
  part's KE and momentum are 1/2 M |v|^2 and M v with M its element mass --
  RHO0 VOL0 for hexas, RHO AREA THK for shells;
* the parts add up to the model totals of the oracle's energy (internal
  and hourglass energy), for any part map;
* a map that moves elements between parts moves their contributions and
  nothing else.
The reference engine's own per-part outputs pin the sums on CRA2V44
(tests/test_oracle_cra2.py).
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M


def _shell_mass(m):
    out = []
    for g in m.shells:
        n = g.ixc[1:5] - 1
        p = [m.X[:, n[k]] for k in range(4)]
        area = 0.5 * np.linalg.norm(np.cross((p[2] - p[0]).T, (p[3] - p[1]).T), axis=1)
        out.append(g.mat["pm"][0] * area * g.thk)
    return out


@pytest.mark.parametrize("kind", ["hexa", "shell"])
def test_rigid_translation_known_answer(kind):
    from oracle.oracle import OracleModel

    m = (M.hexa_impact_block(3000, seed=1, law="law2") if kind == "hexa"
         else M.crash_box(n_side=4, n_len=10))
    v = np.array([3.0, -1.5, 0.5])
    m.V[:] = v[:, None]
    m.icodt[:] = 0
    m.rwalls = []
    o = OracleModel(m)
    o.set_record(True)
    o.cycle(1)  # the sums of the first cycle's element pass: V(n-1/2) = v
    ps = o.part_sums()
    if kind == "hexa":
        mass = [float(np.sum(g.mat["pm"][0] * M.hexa_volumes(m.X, g.ixs))) for g in m.hexa]
    else:
        mass = [float(x.sum()) for x in _shell_mass(m)]
    assert ps.shape == (len(mass), 7)
    for p, mp in enumerate(mass):
        assert abs(ps[p, 5] - mp) <= 1e-12 * mp
        assert abs(ps[p, 1] - 0.5 * mp * float(v @ v)) <= 1e-12 * mp * float(v @ v)
        assert np.allclose(ps[p, 2:5], mp * v, rtol=1e-12, atol=0)


def test_parts_add_up_and_follow_the_map():
    from oracle.oracle import OracleModel

    m = M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0)
    o = OracleModel(m)
    o.set_record(True)
    o.cycle(120)
    base = o.part_sums()
    en = o.energy()
    assert abs(base[:, 0].sum() - en["eint"]) <= 1e-12 * en["eint"]
    assert abs(base[:, 6].sum() - en["ehour"]) <= 1e-12 * max(en["ehour"], 1e-30)
    # the same state, the elements dealt into 3 parts: the parts add up to
    # the one-part totals, and part p holds exactly its elements' share
    o2 = OracleModel(m)
    o2.set_record(True)
    part = (np.arange(m.numelc) % 3).astype(np.int32)
    o2.set_parts(3, None, part)
    o2.cycle(120)
    three = o2.part_sums()
    assert three.shape == (3, 7)
    tot = base.sum(axis=0)
    scale = np.maximum(np.abs(tot), np.abs(tot[2:5]).max())
    assert (np.abs(three.sum(axis=0) - tot) <= 1e-11 * scale).all()
    assert (three[:, 5] > 0).all() and (three[:, 0] > 0).all()
    with pytest.raises(ValueError):
        o2.set_parts(2, None, np.full(m.numelc, 2, np.int32))
