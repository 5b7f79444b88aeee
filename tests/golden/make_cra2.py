"""Generate tests/golden/cra2.npz from the OpenRadioss QA deck CRA2V44.

The deck (qa-tests/miniqa/RESTART/cra2 of the OpenRadioss tree) is a U-section
channel of 768 Belytschko-Tsay shells (three parts, Johnson-Cook LAW2) crushed
axially: the 17 nodes of its x = 0 end are tied by an engine rigid link
(/VEL/TRA/XYZ) and carry an added mass of 500 t on node 1 with an initial
velocity of 5 along x; the x = 480 end is held.  The first engine run goes to
t = 2.5 with the link, the restart run to t = 5 without it (its engine file
has no /VEL card).

What this script extracts (numbers only, no text of the deck is kept):

* the starter deck: nodes, shells and their parts, the /MAT/PLAS_JOHNS and
  /PROP/SHELL cards as read, /DEF_SHELL, /SHFRA/V4, /BCS groups,
  /INIVEL/TRA, /ADMAS and the run end times;
* the starter listing (CRA2V44_0000.out): part masses, total mass and the
  smallest shell time step;
* the engine output tables of both runs (CRA2V44_0001.out, _0002.out): cycle,
  time, time step, controlling element, internal, kinetic and rotational
  kinetic energy;
* the time-history files CRA2V44T01 / T02 (big-endian Fortran sequential
  records, /TFILE/4): every 0.05 the 12 global variables, the 8 default
  variables of each part and the 6 default variables (D, V) of nodes 1, 17
  and 33.

The deck is (C) Siemens, licensed CC BY-NC 4.0 (header of CRA2V44_0000.rad);
the fixture carries its numbers for parity testing only.

Usage:  python tests/golden/make_cra2.py [path to the cra2 QA directory]
        (or OPENRADIOSS_SRC=<root of the OpenRadioss tree> python tests/golden/make_cra2.py)
"""
from __future__ import annotations

import os
import re
import struct
import sys

import numpy as np

# inside an OpenRadioss source tree, given by the command line or by the
# OPENRADIOSS_SRC environment variable (the tree's root)
QA_SUBDIR = "qa-tests/miniqa/RESTART/cra2"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cra2.npz")


def qa_dir(subdir):
    """The QA directory to read: the first command-line argument, else
    subdir inside the OpenRadioss tree named by OPENRADIOSS_SRC; neither
    given is an error (no machine path is assumed)."""
    if len(sys.argv) > 1:
        return sys.argv[1]
    root = os.environ.get("OPENRADIOSS_SRC")
    if not root:
        sys.exit("give the QA directory as the first argument, or set OPENRADIOSS_SRC "
                 "to the root of an OpenRadioss source tree")
    return os.path.join(root, subdir)


def read_blocks(path):
    """Keyword blocks of a Radioss block-format deck: {keyword line: [data
    lines]}, comment lines dropped, repeated keywords numbered."""
    blocks = []
    cur = None
    for ln in open(path, encoding="latin1").read().splitlines():
        if ln.startswith("#") or ln.startswith("$"):
            continue
        if ln.startswith("/"):
            cur = [ln.strip(), []]
            blocks.append(cur)
            continue
        if cur is not None and ln.strip():
            cur[1].append(ln)
    return blocks


def nums(line):
    return [float(v) for v in line.split()]


def ints(line):
    return [int(v) for v in line.split()]


def find(blocks, key):
    return [b for b in blocks if b[0] == key]


def one(blocks, key):
    r = find(blocks, key)
    if len(r) != 1:
        raise ValueError("expected one %s, found %d" % (key, len(r)))
    return r[0][1]


def grnod(blocks, gid):
    lines = one(blocks, "/GRNOD/NODE/%d" % gid)
    out = []
    for ln in lines[1:]:  # first line: title
        out += ints(ln)
    return np.array(out, np.int32)


def parse_starter(path):
    b = read_blocks(path)
    d = {}
    nodes = [ints(ln.split()[0]) + nums(" ".join(ln.split()[1:])) for ln in one(b, "/NODE")]
    nodes = np.array(nodes)
    d["node_id"] = nodes[:, 0].astype(np.int32)
    d["X"] = nodes[:, 1:4].astype(np.float64)
    sid, snodes, spart = [], [], []
    parts = sorted(int(k[0].split("/")[2]) for k in b if k[0].startswith("/PART/"))
    part_mat, part_prop = [], []
    for p in parts:
        pl = one(b, "/PART/%d" % p)
        prop, mat = ints(pl[1])[:2]
        part_prop.append(prop)
        part_mat.append(mat)
        for ln in one(b, "/SHELL/%d" % p):
            v = ints(ln)
            sid.append(v[0])
            snodes.append(v[1:5])
            spart.append(p)
    d["shell_id"] = np.array(sid, np.int32)
    d["shell_nodes"] = np.array(snodes, np.int32)
    d["shell_part"] = np.array(spart, np.int32)
    d["part_id"] = np.array(parts, np.int32)
    d["part_mat"] = np.array(part_mat, np.int32)
    d["part_prop"] = np.array(part_prop, np.int32)
    # /MAT/PLAS_JOHNS: rho | E nu Iflag | a b n epsmax sigmax |
    # c eps0 ICC Fsmooth Fcut Chard | m Tmelt rhoCp Tr
    mats = []
    mat_ids = sorted(int(k[0].split("/")[3]) for k in b if k[0].startswith("/MAT/PLAS_JOHNS/"))
    for m in mat_ids:
        ml = one(b, "/MAT/PLAS_JOHNS/%d" % m)
        rho = nums(ml[1])[0]
        e, nu, iflag = nums(ml[2])
        a, bb, n, epsmax, sigmax = nums(ml[3])
        c, eps0, icc, fsm, fcut, chard = nums(ml[4])
        mm, tmelt, rhocp, tr = nums(ml[5])
        mats.append([m, rho, e, nu, iflag, a, bb, n, epsmax, sigmax, c, eps0, icc, fsm, fcut,
                     chard, mm, tmelt, rhocp, tr])
    d["mat"] = np.array(mats)
    d["mat_columns"] = np.array("id rho E nu Iflag a b n epsmax sigmax c eps0 ICC Fsmooth "
                                "Fcut Chard m Tmelt rhoCp Tr".split())
    # /PROP/SHELL: Ishell Ismstr Ish3n Idrill Pthick_fail | hm hf hr dm dn |
    # N Istrain Thick Ashear Ithick Iplas
    props = []
    prop_ids = sorted(int(k[0].split("/")[3]) for k in b if k[0].startswith("/PROP/SHELL/"))
    for p in prop_ids:
        pl = one(b, "/PROP/SHELL/%d" % p)
        r1 = nums(pl[1])
        r2 = nums(pl[2])
        r3 = nums(pl[3])
        props.append([p] + r1[:5] + r2[:5] + r3[:6])
    d["prop"] = np.array(props)
    d["prop_columns"] = np.array("id Ishell Ismstr Ish3n Idrill Pthick_fail hm hf hr dm dn "
                                 "N Istrain Thick Ashear Ithick Iplas".split())
    # /DEF_SHELL: ISHELL ISMSTR ITHICK IPLAS ISTRAIN I_SH3N IDRIL
    d["def_shell"] = np.array(ints(one(b, "/DEF_SHELL")[0]), np.int32)
    d["shfra_v4"] = np.int32(len(find(b, "/SHFRA/V4")))
    # /BCS: "Tra rot skew grnod"
    tra, rot, off, bn = [], [], [0], []
    for k in sorted((k for k in b if k[0].startswith("/BCS/")), key=lambda k: k[0]):
        t, r, skew, g = k[1][1].split()
        if int(skew) != 0:
            raise ValueError("skewed BCS not expected")
        tra.append(t)
        rot.append(r)
        g = grnod(b, int(g))
        bn += g.tolist()
        off.append(len(bn))
    d["bcs_tra"] = np.array(tra)
    d["bcs_rot"] = np.array(rot)
    d["bcs_nodes"] = np.array(bn, np.int32)
    d["bcs_offsets"] = np.array(off, np.int32)
    iv = one(b, "/INIVEL/TRA/1")
    vx, vy, vz, g, skew = nums(iv[1])
    d["inivel"] = np.array([vx, vy, vz])
    d["inivel_nodes"] = grnod(b, int(g))
    am = one(b, "/ADMAS/0/1")
    mass, g = nums(am[1])
    d["admas"] = np.float64(mass)
    d["admas_nodes"] = grnod(b, int(g))
    return d


def parse_engine(path):
    b = read_blocks(path)
    run = [k for k in b if k[0].startswith("/RUN/")]
    tstop = nums(run[0][1][0])[0]
    link = []
    for k in b:
        if k[0].startswith("/VEL/"):
            if k[0] != "/VEL/TRA/XYZ":
                raise ValueError("unexpected %s" % k[0])
            for ln in k[1]:
                link += ints(ln)
    return tstop, np.array(link, np.int32)


ROW = re.compile(r"^\s*(\d+)\s+([-0-9.E+]+)\s+([-0-9.E+]+)\s+SHELL\s+(\d+)\s+"
                 r"([-0-9.]+)%\s+([-0-9.E+]+)\s+([-0-9.E+]+)\s+([-0-9.E+]+)")


def parse_out(path):
    """Printed cycle table: cycle, time, dt, element, I-ENERGY, K-ENERGY T,
    K-ENERGY R."""
    rows = []
    for ln in open(path, encoding="latin1"):
        m = ROW.match(ln)
        if m:
            c, t, dt, el, err, ie, ke, ker = m.groups()
            rows.append([int(c), float(t), float(dt), int(el), float(ie), float(ke), float(ker)])
    return np.array(rows)


def parse_starter_out(path):
    """Starter listing: part masses, total mass (added mass included) and
    the smallest shell element time step."""
    lines = open(path, encoding="latin1").read().splitlines()
    part_mass, total, dt = [], None, None
    for i, ln in enumerate(lines):
        if ln.startswith("PART :"):
            part_mass.append(float(lines[i + 3].split()[0]))
        elif "TOTAL MASS AND MASS CENTER" in ln:
            total = float(lines[i + 4].split()[0])
        elif "SHELL ELEMENTS TIME STEP" in ln and dt is None:
            dt = float(lines[i + 4].split()[0])
    return np.array(part_mass), total, dt


def fortran_records(path):
    data = open(path, "rb").read()
    p, recs = 0, []
    while p < len(data):
        n = struct.unpack(">i", data[p:p + 4])[0]
        recs.append(data[p + 4:p + 4 + n])
        if struct.unpack(">i", data[p + 4 + n:p + 8 + n])[0] != n:
            raise ValueError("bad record marker")
        p += 8 + n
    return recs


def parse_th(path, ngv=12, npart=3, npv=8, nnode=3, nnv=6):
    """Time records of a /TFILE/4 time-history file: after the header, each
    output time is a 4-byte time record, then the global, part and node
    records (big-endian float32)."""
    recs = fortran_records(path)
    sizes = (4, 4 * ngv, 4 * npart * npv, 4 * nnode * nnv)
    start = None
    for i in range(len(recs) - 3):
        if tuple(len(r) for r in recs[i:i + 4]) == sizes:
            start = i
            break
    t, g, pv, nv = [], [], [], []
    i = start
    while i + 3 < len(recs) + 0 and tuple(len(r) for r in recs[i:i + 4]) == sizes:
        t.append(struct.unpack(">f", recs[i])[0])
        g.append(struct.unpack(">%df" % ngv, recs[i + 1]))
        pv.append(np.array(struct.unpack(">%df" % (npart * npv), recs[i + 2])).reshape(npart, npv))
        nv.append(np.array(struct.unpack(">%df" % (nnode * nnv), recs[i + 3])).reshape(nnode, nnv))
        i += 4
    return (np.array(t, np.float32), np.array(g, np.float32), np.array(pv, np.float32),
            np.array(nv, np.float32))


def main():
    qa = qa_dir(QA_SUBDIR)
    dd = os.path.join(qa, "data")
    rd = os.path.join(qa, "reference")
    d = parse_starter(os.path.join(dd, "CRA2V44_0000.rad"))
    t1, link1 = parse_engine(os.path.join(dd, "CRA2V44_0001.rad"))
    t2, link2 = parse_engine(os.path.join(dd, "CRA2V44_0002.rad"))
    d["run_tstop"] = np.array([t1, t2])
    d["rlink_nodes"] = link1
    d["rlink_nodes_run2"] = link2
    pm, total, dt0 = parse_starter_out(os.path.join(rd, "CRA2V44_0000.out"))
    d["starter_part_mass"] = pm
    d["starter_total_mass"] = np.float64(total)
    d["starter_shell_dt"] = np.float64(dt0)
    d["out1"] = parse_out(os.path.join(rd, "CRA2V44_0001.out"))
    d["out2"] = parse_out(os.path.join(rd, "CRA2V44_0002.out"))
    d["out_columns"] = np.array("cycle time dt element IE KE KER".split())
    for k, f in (("th1", "CRA2V44T01"), ("th2", "CRA2V44T02")):
        t, g, pv, nv = parse_th(os.path.join(rd, f))
        d[k + "_time"], d[k + "_glob"], d[k + "_part"], d[k + "_node"] = t, g, pv, nv
    d["th_glob_columns"] = np.array("IE KE XMOM YMOM ZMOM MASS DT RKE EXTW REINT ECONT HE".split())
    d["th_part_columns"] = np.array("IE KE XMOM YMOM ZMOM MASS HE HEAT".split())
    d["th_node_ids"] = np.array([1, 17, 33], np.int32)
    d["th_node_columns"] = np.array("DX DY DZ VX VY VZ".split())
    np.savez_compressed(OUT, **d)
    print("wrote %s: %d nodes, %d shells, %d + %d printed cycles, %d + %d TH times"
          % (OUT, len(d["node_id"]), len(d["shell_id"]), len(d["out1"]), len(d["out2"]),
             len(d["th1_time"]), len(d["th2_time"])))


if __name__ == "__main__":
    main()
