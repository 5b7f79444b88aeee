"""Per-part element sums (rg_set_parts / rg_part_sums_due / rg_part_sums):
the PARTSAV accumulation of SBILAN (hexas, engine/source/elements/solid/
solide/sbilan.F:118-160) and CBILAN (shells, elements/shell/coque/
cbilan.F:160-190) with CHVIS3's hourglass energy, taken by the cycle they
are asked of between its element pass and its nodal update (GPU).

* FP64 form against the oracle's sums of the same cycles (the oracle takes
  them in every recorded cycle), on a Johnson-Cook hexa block with a part
  map that interleaves the parts and on crash boxes (shells against a rigid
  wall, one part per element group) up to the benchmark's 120,120 shells:
  1e-12 relative (a chunked fixed-order tree against sequential sums);
* mixed form within 1e-4 of the oracle (element state in FP32);
* the parts add up to the model totals of rg_energy (IE, hourglass);
* one request is taken by one cycle; the FORINT-level call takes the sums
  at the same point of the cycle as the device cycle; a restore drops them;
  the sums do not depend on the part map's form (the default map and the
  same map given explicitly give the same bits); bad maps are refused.
The reference engine's own per-part outputs pin the formulas on CRA2V44
(tests/test_oracle_cra2.py, tests/test_gpu_cra2.py).
"""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def _close(g, o, rel):
    """Per part: each quantity within rel of the larger of its own size and
    the part's momentum norm (momentum components can cancel to ~0)."""
    scale = np.maximum(np.abs(o), np.abs(o[:, 2:5]).max(axis=1, keepdims=True))
    return np.abs(g - o) <= rel * scale + 1e-300


def _run_pair(m, precision, cycles_at, hexa_part=None, shell_part=None, npart=None):
    from openradioss_gb300.engine import Engine
    from oracle.oracle import OracleModel

    e = Engine(m, precision=precision)
    o = OracleModel(m)
    o.set_record(True)
    if npart is not None:
        e.set_parts(npart, hexa_part, shell_part)
        o.set_parts(npart, hexa_part, shell_part)
    out = []
    done = 0
    try:
        for c in cycles_at:
            e.cycle(c - 1 - done)
            o.cycle(c - 1 - done)
            e.part_sums_due()
            e.cycle(1)
            o.cycle(1)
            done = c
            out.append((e.part_sums(), o.part_sums(), e.energy()))
        assert e.status() == 0 and o.error() == 0
    finally:
        e.close()
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_hexa_block_interleaved_parts(precision):
    m = M.hexa_impact_block(20000, seed=3, law="law2")
    ne = m.numels
    part = (np.arange(ne) * 7 % 5).astype(np.int32)  # interleaved parts
    res = _run_pair(m, precision, [1, 40, 120], hexa_part=part, npart=5)
    for g, o, en in res:
        assert g.shape == (5, 7)
        assert _close(g, o, 1e-12 if precision == 0 else 1e-4).all(), (g, o)
        # the parts add up to the model totals
        assert abs(g[:, 0].sum() - en["eint"]) <= 1e-12 * max(en["eint"], 1e-300)
        assert abs(g[:, 6].sum() - en["ehour"]) <= 1e-12 * max(en["ehour"], 1e-300)
    # element masses: RHO0 * VOL0 over every element
    assert abs(res[-1][0][:, 5].sum() - res[-1][1][:, 5].sum()) <= 1e-12 * res[-1][1][:, 5].sum()


def test_hexa_default_parts():
    """Without a map each hexa group added is a part, in the oracle too
    (whose groups are split into MVSIZ-long element groups internally)."""
    m = M.hexa_impact_block(20000, seed=3, law="law2")
    res = _run_pair(m, 0, [1, 30])
    for g, o, en in res:
        assert g.shape == o.shape == (len(m.hexa), 7)
        assert _close(g, o, 1e-12).all(), (g, o)


@pytest.mark.parametrize("precision", [0, 1])
def test_crash_box_parts(precision):
    m = M.crash_box(n_side=10, n_len=60, v0=20.0, vpert=1.0)
    res = _run_pair(m, precision, [1, 150, 400])
    for g, o, en in res:
        assert g.shape == (len(m.shells), 7)
        assert _close(g, o, 1e-12 if precision == 0 else 1e-4).all(), (g, o)
        assert abs(g[:, 0].sum() - en["eint"]) <= 1e-12 * max(en["eint"], 1e-300)


def test_crash_box_benchmark_size_parts():
    """The benchmark's crash box (120,120 shells) for a few cycles."""
    m = M.crash_box()
    assert m.numelc == 120120
    res = _run_pair(m, 0, [1, 12])
    for g, o, _ in res:
        assert _close(g, o, 1e-12).all(), (g, o)


def test_request_semantics():
    from openradioss_gb300.engine import Engine, RgError

    m = M.crash_box(n_side=6, n_len=16, v0=20.0, vpert=1.0)
    ng = len(m.shells)
    e = Engine(m, precision=0)
    try:
        with pytest.raises(RgError):
            e.part_sums()  # no cycle has taken them
        x0 = e.nodes()
        e.part_sums_due()
        e.cycle(1)
        s1 = e.part_sums()
        dt1 = e.time()["dt1"]
        e.cycle(5)  # no request: the sums stay those of the first cycle
        assert np.array_equal(e.part_sums(), s1)
        snap = e.snapshot()
        e.part_sums_due()
        e.cycle(1)
        sa = e.part_sums()  # default map: one part per shell group
        e.restore(snap)
        with pytest.raises(RgError):
            e.part_sums()  # a restore drops the sums of a cycle before it
        # the same map given explicitly: the same tables, the same bits
        e.set_parts(ng, None, np.concatenate(
            [np.full(g.ixc.shape[1], k, np.int32) for k, g in enumerate(m.shells)]))
        e.part_sums_due()
        e.cycle(1)
        assert np.array_equal(e.part_sums(), sa)
        # every shell in part 0 of ng + 1 parts: the sum of the groups
        e.restore(snap)
        e.set_parts(ng + 1, None, np.zeros(m.numelc, np.int32))
        e.part_sums_due()
        e.cycle(1)
        one = e.part_sums()
        assert one.shape == (ng + 1, 7) and (one[1:] == 0).all()
        assert _close(one[:1], sa.sum(axis=0, keepdims=True), 1e-12).all(), (one[0], sa.sum(0))
        with pytest.raises(RgError):
            e.set_parts(2, None, np.full(m.numelc, 2, np.int32))  # part out of range
    finally:
        e.close()
    # the FORINT-level call on the first cycle's inputs takes the sums at the
    # same point of the cycle: the same bits
    f = Engine(m, precision=0, elements_only=True)
    try:
        f.part_sums_due()
        f.forint_step(np.ascontiguousarray(x0["X"].T), np.ascontiguousarray(x0["V"].T), dt1,
                      vr=np.ascontiguousarray(x0["VR"].T))
        assert np.array_equal(f.part_sums(), s1)
    finally:
        f.close()
