"""Python host mirror of the C ABI (include/rg_api.h).

``Engine`` drives one rg_ctx through ctypes: it uploads a
:class:`openradioss_gb300.model.Model` (the arrays the starter hands to the
engine), advances explicit cycles on the GPU and reads results back.  Every
call goes to librg.so; there is no CPU fallback -- if the library or a CUDA
device is missing, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib

RG_PREC_FP64 = 0
RG_PREC_MIXED = 1

ST_NEGVOL = 1
ST_NAN = 2
ST_SLOT = 4
ST_DTMIN = 8


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class RgError(RuntimeError):
    pass


class Engine:
    """One model resident on one GPU (an rg_ctx)."""

    def __init__(self, model, device=0, precision=RG_PREC_FP64, skyline=None,
                 elements_only=False):
        """elements_only: the model's rigid bodies, rigid-material bodies,
        concentrated loads and imposed velocities (model.rbodies, rmats,
        cloads, impvels), which the CUDA path does not run, are left to the
        caller's own nodal update, and only the FORINT-level call
        (forint_step) is open; without it such a model is refused."""
        if any(getattr(model, k, None) for k in ("rbodies", "rmats", "cloads", "impvels")) \
                and not elements_only:
            raise RgError("rigid bodies, rigid materials, concentrated loads and imposed "
                          "velocities are not on the CUDA path: use elements_only=True with "
                          "forint_step")
        self.elements_only = elements_only
        self.L = _lib.lib()
        self.model = model
        self.precision = precision
        h = C.c_void_p()
        r = self.L.rg_ctx_create(device, C.byref(h))
        if r != 0:
            raise RgError("rg_ctx_create failed (%d): no usable CUDA device %d" % (r, device))
        self.h = h
        try:
            self._setup(model, precision, skyline)
        except Exception:
            self.close()
            raise

    def _chk(self, r, what):
        if r < 0:
            raise RgError("%s failed (%d): %s" % (what, r, self.L.rg_last_error(self.h).decode()))
        return r

    def _setup(self, m, precision, skyline):
        L = self.L
        self._chk(L.rg_set_precision(self.h, precision), "rg_set_precision")
        X = np.ascontiguousarray(m.X.T.reshape(-1), np.float64)
        V = np.ascontiguousarray(m.V.T.reshape(-1), np.float64)
        MS = np.ascontiguousarray(m.MS, np.float64)
        IN = None if m.IN is None else np.ascontiguousarray(m.IN, np.float64)
        ic = np.ascontiguousarray(m.icodt, np.int32)
        self._chk(L.rg_mesh_upload(self.h, m.numnod, _p(X), _p(V), _p(MS), _p(IN), _p(ic)),
                  "rg_mesh_upload")
        for g in m.hexa:
            ixs = np.ascontiguousarray(g.ixs.T.reshape(-1), np.int32)
            self._chk(L.rg_hexa_group_add(self.h, g.ixs.shape[1], _p(ixs), g.mat["mtn"],
                                          _p(g.mat["pm"]), _p(g.geo), _p(g.mat["uparam"]),
                                          _p(g.mat["iparam"]), 4, 1, getattr(g, "jcvt", 0)),
                      "rg_hexa_group_add")
        for g in m.shells:
            ixc = np.ascontiguousarray(g.ixc.T.reshape(-1), np.int32)
            thk = np.ascontiguousarray(g.thk, np.float64)
            self._chk(L.rg_shell_group_add(self.h, g.ixc.shape[1], _p(ixc), g.npt,
                                           _p(g.mat["pm"]), _p(g.geo), _p(g.mat["uparam"]),
                                           _p(g.mat["iparam"]), _p(thk), g.ismstr, g.ithk),
                      "rg_shell_group_add")
        for (p0, nrm, ds) in m.rwalls:
            self._chk(L.rg_rwall_add(self.h, _p(np.asarray(p0, np.float64)),
                                     _p(np.asarray(nrm, np.float64)), float(ds)), "rg_rwall_add")
        for (nodes, ic, icr) in getattr(m, "rlinks", []):
            nodes = np.ascontiguousarray(nodes, np.int32)
            self._chk(L.rg_rlink_add(self.h, len(nodes), _p(nodes), int(ic), int(icr)),
                      "rg_rlink_add")
        if getattr(m, "ishfram", 0):
            self._chk(L.rg_set_shell_frame(self.h, int(m.ishfram)), "rg_set_shell_frame")
        if getattr(m, "nodal_dt", None):
            dtfac, dtmin = m.nodal_dt
            self._chk(L.rg_set_nodal_dt(self.h, float(dtfac), float(dtmin)), "rg_set_nodal_dt")
        for kind, (idtmin, dtmin) in sorted(getattr(m, "dtmin_actions", {}).items()):
            self._chk(L.rg_set_dtmin(self.h, int(kind), int(idtmin), float(dtmin)), "rg_set_dtmin")
        if skyline is not None:
            adsky, iads, iadc = (np.ascontiguousarray(a, np.int32) for a in skyline)
            self._chk(L.rg_skyline_set(self.h, _p(adsky), _p(iads), _p(iadc)), "rg_skyline_set")
        self._chk(L.rg_finalize(self.h, m.dtfac_solid, m.dtfac_shell, m.dtmx, m.dt2old),
                  "rg_finalize")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.rg_ctx_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- stepping --------------------------------------------------------
    def cycle(self, n=1, sync=True):
        if self.elements_only:
            raise RgError("an elements_only engine runs forint_step only")
        self._chk(self.L.rg_cycle(self.h, int(n)), "rg_cycle")
        if sync:
            self.sync()

    def set_link_active(self, link, active):
        """Switch rigid link `link` on or off between cycles."""
        self._chk(self.L.rg_rlink_set_active(self.h, int(link), 1 if active else 0),
                  "rg_rlink_set_active")

    def sync(self):
        self._chk(self.L.rg_synchronize(self.h), "rg_synchronize")

    def status(self):
        return self._chk(self.L.rg_status(self.h), "rg_status")

    def forint_step(self, x, v, dt1, vr=None, f=None, stifn=None, fr=None, stifr=None):
        """FORINT-level call with host buffers: x, v (and vr for shells) as
        X(3,N) arrays (numpy (N,3) row-major == Fortran (3,N)).  Returns
        (f, stifn, dt2t, neltst); moments go to fr / stifr when given."""
        n = self.model.numnod
        if f is None:
            f = np.empty((n, 3))
        if stifn is None:
            stifn = np.empty(n)
        dt2t = C.c_double()
        el = C.c_int()
        self._chk(self.L.rg_forint_step(self.h, _p(x), _p(v), _p(vr), float(dt1), _p(f),
                                        _p(stifn), _p(fr), _p(stifr), C.byref(dt2t),
                                        C.byref(el)), "rg_forint_step")
        return f, stifn, dt2t.value, el.value

    def cycle_host(self, x=None, v=None, vr=None, x_out=None, v_out=None, vr_out=None,
                   d_out=None):
        """One whole cycle with host node buffers (rg_cycle_host): x, v (vr)
        as (N, 3) arrays replace the device's nodes when given; the new
        X, V (VR, D) go to the *_out arrays given.  Returns the cycle's
        step."""
        if self.elements_only:
            raise RgError("an elements_only engine runs forint_step only")
        dt2 = C.c_double()
        self._chk(self.L.rg_cycle_host(self.h, _p(x), _p(v), _p(vr), _p(x_out), _p(v_out),
                                       _p(vr_out), _p(d_out), C.byref(dt2)), "rg_cycle_host")
        return dt2.value

    def host_register(self, a):
        self._chk(self.L.rg_host_register(self.h, _p(a), a.nbytes), "rg_host_register")

    def host_unregister(self, a):
        self._chk(self.L.rg_host_unregister(self.h, _p(a)), "rg_host_unregister")

    # ---- results -----------------------------------------------------------
    def nodes(self):
        n = self.model.numnod
        out = {k: np.zeros(3 * n) for k in ("X", "V", "D", "VR")}
        self._chk(self.L.rg_download_nodes(self.h, _p(out["X"]), _p(out["V"]), _p(out["D"]),
                                           _p(out["VR"])), "rg_download_nodes")
        return {k: a.reshape(n, 3).T.copy() for k, a in out.items()}

    def displacement(self):
        """D(3, N): the nodes' displacement from their initial position."""
        n = self.model.numnod
        d = np.zeros(3 * n)
        self._chk(self.L.rg_download_nodes(self.h, None, None, _p(d), None), "rg_download_nodes")
        return d.reshape(n, 3).T.copy()

    def forces(self):
        n = self.model.numnod
        f, st, fr = np.zeros(3 * n), np.zeros(n), np.zeros(3 * n)
        self._chk(self.L.rg_download_forces(self.h, _p(f), _p(st), _p(fr)), "rg_download_forces")
        return dict(F=f.reshape(n, 3).T.copy(), STIFN=st, FR=fr.reshape(n, 3).T.copy())

    def hexa_state(self, which):
        ne = self.model.numels
        out = np.zeros(6 * ne if which == 0 else ne)
        self._chk(self.L.rg_download_hexa_state(self.h, which, _p(out)), "rg_download_hexa_state")
        return out.reshape(6, ne) if which == 0 else out

    def shell_state(self, which, size):
        out = np.zeros(size)
        self._chk(self.L.rg_download_shell_state(self.h, which, _p(out)), "rg_download_shell_state")
        return out

    def time(self):
        tt, dt1, dt2 = C.c_double(), C.c_double(), C.c_double()
        nc, el = C.c_int(), C.c_int()
        self._chk(self.L.rg_get_time(self.h, C.byref(tt), C.byref(dt1), C.byref(dt2),
                                     C.byref(nc), C.byref(el)), "rg_get_time")
        return dict(tt=tt.value, dt1=dt1.value, dt2=dt2.value, ncycle=nc.value, neltst=el.value)

    def energy(self):
        v = [C.c_double() for _ in range(4)]
        self._chk(self.L.rg_energy(self.h, *[C.byref(x) for x in v]), "rg_energy")
        return dict(eint=v[0].value, ekin=v[1].value, ekinr=v[2].value, ehour=v[3].value)

    BALANCE_KEYS = ("tt", "eint", "ekin", "ekinr", "ehour", "wfext", "entot", "error_pct",
                    "mass", "mass_error", "xmom", "ymom", "zmom")

    def energy_balance(self):
        """The listing cycle line's energy balance (ECRIT): energies, the
        rigid walls' external work, ENTOT, the energy error in percent
        against the cycle-0 total, mass, mass error and momentum."""
        out = np.zeros(len(self.BALANCE_KEYS))
        self._chk(self.L.rg_energy_balance(self.h, _p(out), len(out)), "rg_energy_balance")
        return dict(zip(self.BALANCE_KEYS, out.tolist()))

    PART_KEYS = ("IE", "KE", "XMOM", "YMOM", "ZMOM", "MASS", "HE")

    def set_parts(self, npart, hexa_part=None, shell_part=None):
        """Every element's 0-based part number, in element order (groups in
        the order added); without it each element group is a part."""
        m = self.model
        hp = np.ascontiguousarray(hexa_part if hexa_part is not None else np.zeros(0), np.int32)
        sp = np.ascontiguousarray(shell_part if shell_part is not None else np.zeros(0), np.int32)
        if hp.size != m.numels or sp.size != m.numelc:
            raise ValueError("one part number per hexa and per shell")
        self._chk(self.L.rg_set_parts(self.h, int(npart), _p(hp), _p(sp)), "rg_set_parts")

    def part_count(self):
        n = C.c_int()
        self._chk(self.L.rg_part_count(self.h, C.byref(n)), "rg_part_count")
        return n.value

    def part_sums_due(self):
        """The next cycle takes the per-part sums (between its element pass
        and its nodal update)."""
        self._chk(self.L.rg_part_sums_due(self.h), "rg_part_sums_due")

    def part_sums(self):
        """Per-part sums of the last cycle that took them: (npart, 7) array,
        columns PART_KEYS."""
        n = self.part_count()
        out = np.zeros((n, len(self.PART_KEYS)))
        self._chk(self.L.rg_part_sums(self.h, _p(out), n), "rg_part_sums")
        return out

    def skyline(self):
        m = self.model
        adsky = np.zeros(m.numnod + 1, np.int32)
        iads = np.zeros(max(8 * m.numels, 1), np.int32)
        iadc = np.zeros(max(4 * m.numelc, 1), np.int32)
        lsky = C.c_int()
        self._chk(self.L.rg_skyline_get(self.h, _p(adsky), _p(iads), _p(iadc), C.byref(lsky)),
                  "rg_skyline_get")
        return adsky, iads[:8 * m.numels], iadc[:4 * m.numelc], lsky.value

    def snapshot(self):
        """The model's whole device state as bytes (rg_snapshot), after the
        queued cycles."""
        n = C.c_ulonglong()
        self._chk(self.L.rg_snapshot_size(self.h, C.byref(n)), "rg_snapshot_size")
        buf = np.empty(n.value, np.uint8)
        self._chk(self.L.rg_snapshot(self.h, _p(buf), n.value), "rg_snapshot")
        return buf

    def restore(self, snap):
        """Resume from a snapshot of the same model (this engine or another
        one built from the same model and precision)."""
        snap = np.ascontiguousarray(snap, np.uint8)
        self._chk(self.L.rg_restore(self.h, _p(snap), snap.nbytes), "rg_restore")

    def info(self):
        a = [C.c_int() for _ in range(4)]
        b = C.c_ulonglong()
        self._chk(self.L.rg_info(self.h, *[C.byref(x) for x in a], C.byref(b)), "rg_info")
        return dict(numnod=a[0].value, numels=a[1].value, numelc=a[2].value, lsky=a[3].value,
                    device_bytes=b.value)

    def set_timing(self, on):
        self._chk(self.L.rg_set_timing(self.h, 1 if on else 0), "rg_set_timing")

    def time_cycles_cold(self, n, flush_bytes=256 << 20):
        """Run n cycles, each after overwriting flush_bytes (more than the L2)
        outside the timed span; returns the summed device time in ms."""
        ms = C.c_double()
        self._chk(self.L.rg_time_cycles_cold(self.h, int(n), int(flush_bytes), C.byref(ms)),
                  "rg_time_cycles_cold")
        return ms.value

    def time_cycles(self, n):
        """Run n cycles between two CUDA events on the context stream and
        return the device time in ms."""
        ms = C.c_double()
        self._chk(self.L.rg_time_cycles(self.h, int(n), C.byref(ms)), "rg_time_cycles")
        return ms.value

    def kernel_times(self):
        a = (C.c_double * 4)()
        self._chk(self.L.rg_kernel_times(self.h, a), "rg_kernel_times")
        return dict(hexa=a[0], shell=a[1], dt=a[2], node=a[3])
