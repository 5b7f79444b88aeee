"""ctypes front-end of the CPU oracle -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as a checker / reported baseline;
the product never imports it.  See rg_oracle.cpp for what it restates and
its parity status (shell path pinned against the reference engine's own
outputs for its QA deck CRA2V44, hexa path for its QA deck H101; both also
by analytic known-answer tests).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "librg_oracle.so")
_LIB_COUNT = os.path.join(_HERE, "_build", "librg_oracle_count.so")
_lib = None
_lib_count = None

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(force=False):
    """Compile the oracle with its Makefile (g++, -ffp-contract=off); make
    rebuilds it whenever a source is newer than the library, and a failed
    compile raises instead of leaving an older library in use."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = _declare(C.CDLL(_LIB))
    return _lib


def count_lib():
    """The op-counting build of the oracle (rg_opcount.h): same entry points
    plus or_opcount_get / or_opcount_reset; run it with one thread."""
    global _lib_count
    if _lib_count is None:
        subprocess.run(["make", "-s", "-C", _HERE, "opcount"], check=True)
        L = _declare(C.CDLL(_LIB_COUNT))
        L.or_opcount_get.argtypes = [C.c_void_p]
        L.or_opcount_reset.argtypes = []
        _lib_count = L
    return _lib_count


def _declare(L):
    if True:
        vp = C.c_void_p
        L.or_model_new.restype = vp
        L.or_model_new.argtypes = [C.c_int, _dp, _dp, _dp, _ip]
        L.or_model_free.argtypes = [vp]
        L.or_hexa_group_add.argtypes = [vp, C.c_int, _ip, C.c_int, _dp, _dp, _dp, _ip,
                                        C.c_int, C.c_int, C.c_int]
        L.or_shell_group_add.argtypes = [vp, C.c_int, _ip, C.c_int, _dp, _dp, _dp, _ip,
                                         _dp, C.c_int, C.c_int]
        L.or_set_inertia.argtypes = [vp, _dp]
        L.or_rwall_add.argtypes = [vp, _dp, _dp, C.c_double]
        L.or_finalize.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.or_get_skyline.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_cycle.argtypes = [vp, C.c_int]
        L.or_get_nodes.argtypes = [vp] + [C.c_void_p] * 7
        L.or_get_time.argtypes = [vp] + [C.c_void_p] * 5
        L.or_get_hexa_state.argtypes = [vp, C.c_int, C.c_int, _dp]
        L.or_energy.argtypes = [vp] + [C.c_void_p] * 4
        L.or_error.argtypes = [vp]
        L.or_get_shell_state.argtypes = [vp, C.c_int, _dp]
        L.or_shell_frame.argtypes = [vp, C.c_int]
        L.or_rlink_add.argtypes = [vp, C.c_int, _ip, C.c_int, C.c_int]
        L.or_rlink_clear.argtypes = [vp]
        L.or_set_record.argtypes = [vp, C.c_int]
        L.or_set_nodal_dt.argtypes = [vp, C.c_double, C.c_double]
        L.or_set_dtmin.argtypes = [vp, C.c_int, C.c_int, C.c_double]
        L.or_rmat_add.argtypes = [vp, C.c_int, _ip, _dp, C.c_double, _dp, _dp]
        L.or_impvel_add.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_int, _dp, _dp]
        L.or_get_mass.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.or_get_record.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.or_get_wfext.argtypes = [vp, C.c_void_p]
        L.or_rbody_add.argtypes = [vp, C.c_int, C.c_int, _ip, _dp, _dp]
        L.or_set_forces.argtypes = [vp] + [C.c_void_p] * 4 + [C.c_double, C.c_int]
        L.or_cload_add.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                   _dp, _dp]
        L.or_set_parts.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p]
        L.or_get_part_sums.argtypes = [vp, C.c_void_p, C.c_int]
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class OracleModel:
    """A model stepped by the CPU oracle."""

    def __init__(self, model, nthreads=None, library=None):
        L = library or lib()
        self.L = L
        self.model = model
        n = model.numnod
        X = np.ascontiguousarray(model.X.T.reshape(-1))
        V = np.ascontiguousarray(model.V.T.reshape(-1))
        self.h = L.or_model_new(n, X, V, np.ascontiguousarray(model.MS, np.float64),
                                np.ascontiguousarray(model.icodt, np.int32))
        for g in model.hexa:
            r = L.or_hexa_group_add(self.h, g.ixs.shape[1],
                                    np.ascontiguousarray(g.ixs.T.reshape(-1), np.int32),
                                    g.mat["mtn"], g.mat["pm"], g.geo, g.mat["uparam"],
                                    g.mat["iparam"], 4, 1, getattr(g, "jcvt", 0))
            if r < 0:
                raise RuntimeError("or_hexa_group_add failed %d" % r)
        for g in model.shells:
            r = L.or_shell_group_add(self.h, g.ixc.shape[1],
                                     np.ascontiguousarray(g.ixc.T.reshape(-1), np.int32),
                                     g.npt, g.mat["pm"], g.geo, g.mat["uparam"],
                                     g.mat["iparam"], np.ascontiguousarray(g.thk, np.float64),
                                     g.ismstr, g.ithk)
            if r < 0:
                raise RuntimeError("or_shell_group_add failed %d" % r)
        if model.IN is not None:
            L.or_set_inertia(self.h, np.ascontiguousarray(model.IN, np.float64))
        for (main, nodes, axes, inertia) in getattr(model, "rbodies", []):
            r = L.or_rbody_add(self.h, int(main), len(nodes),
                               np.ascontiguousarray(nodes, np.int32),
                               np.ascontiguousarray(axes, np.float64).reshape(-1),
                               np.ascontiguousarray(inertia, np.float64))
            if r < 0:
                raise RuntimeError("or_rbody_add failed %d" % r)
        for (nodes, xg, mass, axes, inertia) in getattr(model, "rmats", []):
            r = L.or_rmat_add(self.h, len(nodes), np.ascontiguousarray(nodes, np.int32),
                              np.ascontiguousarray(xg, np.float64), float(mass),
                              np.ascontiguousarray(axes, np.float64).reshape(-1),
                              np.ascontiguousarray(inertia, np.float64))
            if r < 0:
                raise RuntimeError("or_rmat_add failed %d" % r)
        for (node, dr, facx, fsc, t0, t1, xs, ys) in getattr(model, "impvels", []):
            xs = np.ascontiguousarray(xs, np.float64)
            r = L.or_impvel_add(self.h, int(node), int(dr), float(facx), float(fsc), float(t0),
                                float(t1), len(xs), xs, np.ascontiguousarray(ys, np.float64))
            if r < 0:
                raise RuntimeError("or_impvel_add failed %d" % r)
        for (node, dr, fcx, fcy, xs, ys) in getattr(model, "cloads", []):
            xs = np.ascontiguousarray(xs, np.float64)
            r = L.or_cload_add(self.h, int(node), int(dr), float(fcx), float(fcy), len(xs), xs,
                               np.ascontiguousarray(ys, np.float64))
            if r < 0:
                raise RuntimeError("or_cload_add failed %d" % r)
        for (p0, nrm, ds) in model.rwalls:
            L.or_rwall_add(self.h, np.asarray(p0, np.float64), np.asarray(nrm, np.float64), ds)
        for (nodes, ic, icr) in model.rlinks:
            nodes = np.ascontiguousarray(nodes, np.int32)
            if L.or_rlink_add(self.h, len(nodes), nodes, ic, icr) < 0:
                raise RuntimeError("or_rlink_add failed")
        if L.or_shell_frame(self.h, model.ishfram) != 0:
            raise RuntimeError("or_shell_frame: unsupported ISHFRAM %d" % model.ishfram)
        if getattr(model, "nodal_dt", None):
            if L.or_set_nodal_dt(self.h, float(model.nodal_dt[0]), float(model.nodal_dt[1])) != 0:
                raise RuntimeError("or_set_nodal_dt failed")
        for kind, (idtmin, dtmin) in sorted(getattr(model, "dtmin_actions", {}).items()):
            if L.or_set_dtmin(self.h, int(kind), int(idtmin), float(dtmin)) != 0:
                raise RuntimeError("or_set_dtmin failed")
        nt = nthreads or os.cpu_count() or 1
        r = L.or_finalize(self.h, model.dtfac_solid, model.dtfac_shell, model.dtmx,
                          model.dt2old, nt)
        if r != 0:
            raise RuntimeError("or_finalize failed %d" % r)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_model_free(self.h)
            self.h = None

    def cycle(self, n=1):
        return self.L.or_cycle(self.h, n)

    def skyline(self):
        m = self.model
        adsky = np.zeros(m.numnod + 1, np.int32)
        iads = np.zeros(8 * max(m.numels, 1), np.int32)
        iadc = np.zeros(4 * max(m.numelc, 1), np.int32)
        lsky = np.zeros(1, np.int32)
        self.L.or_get_skyline(self.h, _ptr(adsky), _ptr(iads), _ptr(iadc), _ptr(lsky))
        return adsky, iads[:8 * m.numels], iadc[:4 * m.numelc], int(lsky[0])

    def nodes(self):
        n = self.model.numnod
        out = {k: np.zeros(3 * n) for k in ("X", "V", "D", "VR", "F", "FR")}
        out["STIFN"] = np.zeros(n)
        self.L.or_get_nodes(self.h, _ptr(out["X"]), _ptr(out["V"]), _ptr(out["D"]),
                           _ptr(out["VR"]), _ptr(out["F"]), _ptr(out["STIFN"]),
                           _ptr(out["FR"]))
        for k in ("X", "V", "D", "VR", "F", "FR"):
            out[k] = out[k].reshape(n, 3).T.copy()
        return out

    def time(self):
        tt, dt1, dt2 = (np.zeros(1) for _ in range(3))
        nc, el = np.zeros(1, np.int32), np.zeros(1, np.int32)
        self.L.or_get_time(self.h, _ptr(tt), _ptr(dt1), _ptr(dt2), _ptr(nc), _ptr(el))
        return dict(tt=tt[0], dt1=dt1[0], dt2=dt2[0], ncycle=int(nc[0]), neltst=int(el[0]))

    def hexa_state(self, which):
        ne = self.model.numels
        out = np.zeros(6 * ne if which == 0 else ne)
        self.L.or_get_hexa_state(self.h, 0, which, out)
        return out.reshape(6, ne) if which == 0 else out

    def shell_state(self, which, size):
        out = np.zeros(size)
        self.L.or_get_shell_state(self.h, which, out)
        return out

    def energy(self):
        v = [np.zeros(1) for _ in range(4)]
        self.L.or_energy(self.h, *[_ptr(a) for a in v])
        return dict(eint=v[0][0], ekin=v[1][0], ekinr=v[2][0], ehour=v[3][0])

    def mass(self):
        """Nodal masses and inertias (MS, IN) after any mass scaling."""
        n = self.model.numnod
        ms, inn = np.zeros(n), np.zeros(n)
        self.L.or_get_mass(self.h, _ptr(ms), _ptr(inn))
        return ms, inn

    def wfext(self):
        """External work accumulated so far (loads, rigid walls)."""
        out = np.zeros(1)
        self.L.or_get_wfext(self.h, _ptr(out))
        return float(out[0])

    def error(self):
        return self.L.or_error(self.h)

    def set_forces(self, f, stifn, dt2t, neltst, fr=None, stifr=None):
        """Assembled element forces for the next cycle(1) (F and FR as (N, 3)
        or (3*N,) arrays in node-major order, STIFN, STIFR (N,)), with the
        element time step: the cycle skips its own element groups."""
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.float64).reshape(-1)
        f, stifn, fr, stifr = c(f), c(stifn), c(fr), c(stifr)
        if self.L.or_set_forces(self.h, _ptr(f), _ptr(stifn), _ptr(fr), _ptr(stifr), float(dt2t),
                               int(neltst)) != 0:
            raise RuntimeError("or_set_forces failed")

    def clear_links(self):
        self.L.or_rlink_clear(self.h)

    def set_record(self, on=True):
        self.L.or_set_record(self.h, 1 if on else 0)

    def set_parts(self, npart, hexa_part=None, shell_part=None):
        """Element -> part maps of the per-part sums (0-based, element
        order); without them each element group is a part."""
        hp = np.ascontiguousarray(hexa_part if hexa_part is not None else np.zeros(0), np.int32)
        sp = np.ascontiguousarray(shell_part if shell_part is not None else np.zeros(0), np.int32)
        if self.L.or_set_parts(self.h, int(npart), _ptr(hp), _ptr(sp)) != 0:
            raise ValueError("or_set_parts: a part in [0, npart) for every element")

    def part_sums(self):
        """Per-part sums (SBILAN / CBILAN) of the last recorded cycle:
        (npart, 7) array, columns IE KE XMOM YMOM ZMOM MASS HE."""
        n = self.L.or_get_part_sums(self.h, None, 0)
        out = np.zeros((n, 7))
        self.L.or_get_part_sums(self.h, _ptr(out), n)
        return out

    def record(self):
        """Listing quantities of the last cycle (ECRIT's point of the
        cycle): time, dt, energies (internal, kinetic, rotational kinetic,
        hourglass), momentum, mass, controlling element."""
        out = np.zeros(11)
        el = np.zeros(1, np.int32)
        self.L.or_get_record(self.h, _ptr(out), _ptr(el))
        keys = ("tt", "dt2", "eint", "ekin", "ekinr", "ehour", "xmom", "ymom", "zmom", "mass",
                "wfext")
        r = dict(zip(keys, out.tolist()))
        r["neltst"] = int(el[0])
        return r
