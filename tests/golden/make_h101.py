"""Generate tests/golden/h101.npz from the OpenRadioss QA deck H101.

The deck (qa-tests/miniqa/SOLIDES/nv_elts/poutre_flex/flexion/H101 of the
OpenRadioss tree) holds six elastic cantilevers of one-point hexahedra
(/MAT/ELAST, /PROP/SOLID with every field 0, so /DEF_SOLID's Isolid = 1 and
Iframe = 2 apply) meshed with 1 to 48 elements.  Each cantilever is held at
x = 0 and carries at its x = 10 end a rigid body (/RBODY, no added mass)
whose main node takes a constant concentrated load of 40000 along z
(/CLOAD with /FUNCT 1).  One engine run to t = 0.0020001.

What this script extracts (numbers only, no text of the deck is kept):

* the starter deck: nodes, bricks with their parts, /MAT/ELAST, /PROP/SOLID,
  /DEF_SOLID, /BCS groups, /FUNCT, /CLOAD, /RBODY cards and the run end time;
* the starter listing (CONV_ELS_0000.out): for each rigid body the main
  node position, mass, inertia and principal inertia after the starter's
  rigid-body initialisation; the total mass; the starter's solid time step;
* the engine listing (CONV_ELS_0001.out): cycle, time, time step,
  controlling element, energy error, internal, kinetic, rotational kinetic
  energy, external work and total mass of every printed cycle;
* the time-history file CONV_ELST01 (big-endian Fortran sequential records,
  /TFILE/4, every 1e-5): the 12 global variables and the 6 default variables
  (D, V) of the six main nodes.

The deck is (C) Siemens, licensed CC BY-NC 4.0 (header of
CONV_ELS_0000.rad); the fixture carries its numbers for parity testing only.

Usage:  python tests/golden/make_h101.py [path to the H101 QA directory]
        (or OPENRADIOSS_SRC=<root of the OpenRadioss tree> python tests/golden/make_h101.py)
"""
from __future__ import annotations

import os
import re
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_cra2 import find, fortran_records, grnod, ints, nums, one, qa_dir, read_blocks  # noqa: E402,E501

# inside an OpenRadioss source tree, given by the command line or by the
# OPENRADIOSS_SRC environment variable (the tree's root)
QA_SUBDIR = "qa-tests/miniqa/SOLIDES/nv_elts/poutre_flex/flexion/H101"
OUT = os.path.join(HERE, "h101.npz")


def group_nodes(b, gid):
    """/GRNOD/NODE or /GRNOD/GRNOD (a group of groups) by id."""
    if find(b, "/GRNOD/NODE/%d" % gid):
        return grnod(b, gid)
    lines = one(b, "/GRNOD/GRNOD/%d" % gid)
    out = []
    for ln in lines[1:]:
        for g in ints(ln):
            out += group_nodes(b, g).tolist()
    return np.array(out, np.int32)


def parse_starter(path):
    b = read_blocks(path)
    d = {}
    nodes = np.array([[float(v) for v in ln.split()[:4]] for ln in one(b, "/NODE")])
    d["node_id"] = nodes[:, 0].astype(np.int32)
    d["X"] = nodes[:, 1:4].astype(np.float64)
    parts = sorted(int(k[0].split("/")[2]) for k in b if k[0].startswith("/PART/"))
    bid, bnodes, bpart, part_prop, part_mat = [], [], [], [], []
    for p in parts:
        pl = one(b, "/PART/%d" % p)
        prop, mat = ints(pl[1])[:2]
        part_prop.append(prop)
        part_mat.append(mat)
        for ln in one(b, "/BRICK/%d" % p):
            v = ints(ln)
            bid.append(v[0])
            bnodes.append(v[1:9])
            bpart.append(p)
    d["brick_id"] = np.array(bid, np.int32)
    d["brick_nodes"] = np.array(bnodes, np.int32)
    d["brick_part"] = np.array(bpart, np.int32)
    d["part_id"] = np.array(parts, np.int32)
    d["part_prop"] = np.array(part_prop, np.int32)
    d["part_mat"] = np.array(part_mat, np.int32)
    # /MAT/ELAST: title | rho rho_ref | E nu
    mats = []
    for k in b:
        if k[0].startswith("/MAT/ELAST/"):
            rho = nums(k[1][1])[0]
            e, nu = nums(k[1][2])[:2]
            mats.append([int(k[0].split("/")[3]), rho, e, nu])
    d["mat"] = np.array(mats)
    # /PROP/SOLID: Isolid Ismstr Icpre Inpts Itetra Iframe dn | qa qb h
    # LAMBDA_V MU_V | dt_min istrain IHKT
    props = []
    for k in b:
        if k[0].startswith("/PROP/SOLID/"):
            r1, r2 = nums(k[1][1]), nums(k[1][2])
            props.append([int(k[0].split("/")[3])] + r1[:7] + r2[:3])
    d["prop"] = np.array(props)
    d["prop_columns"] = np.array("id Isolid Ismstr Icpre Inpts Itetra Iframe dn qa qb h".split())
    # /DEF_SOLID: I_SOLID ISMSTR ISTRAIN IFRAME
    d["def_solid"] = np.array(ints(one(b, "/DEF_SOLID")[0]), np.int32)
    tra, rot, off, bn = [], [], [0], []
    for k in sorted((k for k in b if k[0].startswith("/BCS/")), key=lambda k: k[0]):
        t, r, skew, g = k[1][1].split()
        if int(skew) != 0:
            raise ValueError("skewed BCS not expected")
        tra.append(t)
        rot.append(r)
        bn += group_nodes(b, int(g)).tolist()
        off.append(len(bn))
    d["bcs_tra"] = np.array(tra)
    d["bcs_rot"] = np.array(rot)
    d["bcs_nodes"] = np.array(bn, np.int32)
    d["bcs_offsets"] = np.array(off, np.int32)
    # /FUNCT/1: title, then x y pairs
    fl = one(b, "/FUNCT/1")
    d["funct1"] = np.array([nums(ln)[:2] for ln in fl[1:]])
    # /CLOAD: funct Dir skew sensor grnod Ascalex Fscaley
    cl = one(b, "/CLOAD/1")[1].split()
    if int(cl[0]) != 1 or int(cl[2]) != 0 or int(cl[3]) != 0:
        raise ValueError("unexpected /CLOAD card")
    d["cload_dir"] = np.int32("XYZ".index(cl[1]))
    d["cload_nodes"] = group_nodes(b, int(cl[4]))
    d["cload_scale"] = np.array([float(cl[5]), float(cl[6])])
    # /RBODY: RBID ISENS NSKEW ISPHER MASS Gnod IKREM ICOG SURF | J's
    rmain, rsec, roff, rflags = [], [], [0], []
    for k in sorted((k for k in b if k[0].startswith("/RBODY/")), key=lambda k: k[0]):
        v = k[1][1].split()
        main, isens, nskew, ispher = (int(x) for x in v[:4])
        mass = float(v[4])
        g, ikrem, icog, surf = (int(x) for x in v[5:9])
        jj = nums(k[1][2]) + nums(k[1][3])
        if isens or nskew or surf or mass != 0.0 or any(jj):
            raise ValueError("unexpected /RBODY card")
        rmain.append(main)
        rsec += group_nodes(b, g).tolist()
        roff.append(len(rsec))
        rflags.append([ispher, icog, ikrem])
    d["rbody_main"] = np.array(rmain, np.int32)
    d["rbody_nodes"] = np.array(rsec, np.int32)
    d["rbody_offsets"] = np.array(roff, np.int32)
    d["rbody_flags"] = np.array(rflags, np.int32)
    th = one(b, "/TH/NODE/1")
    d["th_node_ids"] = np.array([int(ln[:10]) for ln in th[2:]], np.int32)
    return d


def parse_engine(path):
    b = read_blocks(path)
    run = [k for k in b if k[0].startswith("/RUN/")]
    return nums(run[0][1][0])[0]


F = r"([-0-9.E+]+)"
ROW = re.compile(r"^\s*(\d+)\s+" + F + r"\s+" + F + r"\s+SOLID\s+(\d+)\s+([-0-9.]+)%\s+"
                 + r"\s+".join([F] * 6))


def parse_out(path):
    """Printed cycle table: cycle, time, dt, element, error %, I-ENERGY,
    K-ENERGY T, K-ENERGY R, EXT-WORK, MAS.ERR, TOTAL MASS."""
    rows = []
    for ln in open(path, encoding="latin1"):
        m = ROW.match(ln)
        if m:
            g = m.groups()
            rows.append([int(g[0]), float(g[1]), float(g[2]), int(g[3])] + [float(x) for x in g[4:]])
    return np.array(rows)


def parse_starter_out(path):
    """Rigid-body initialisation blocks (main node id, new position, mass,
    inertia xx yy zz, xy yz zx, principal inertia), the total mass and the
    starter's smallest solid time step."""
    lines = open(path, encoding="latin1").read().splitlines()
    rb, total, dt = [], None, None
    for i, ln in enumerate(lines):
        if ln.strip().startswith("RIGID BODY ID") and "NEW X,Y,Z" in lines[i + 2]:
            main = int(lines[i + 1].split()[-1])
            xyz = [float(v) for v in lines[i + 2].split()[-3:]]
            mass = float(lines[i + 3].split()[-1])
            inr = [float(v) for v in lines[i + 4].split()[-3:]]
            cross = [float(v) for v in lines[i + 5].split()[-3:]]
            pri = [float(v) for v in lines[i + 6].split()[-3:]]
            rb.append([main] + xyz + [mass] + inr + cross + pri)
        elif "TOTAL MASS AND MASS CENTER" in ln:
            total = float(lines[i + 4].split()[0])
        elif "SOLID ELEMENTS TIME STEP" in ln and dt is None:
            dt = float(lines[i + 4].split()[0])
    return np.array(rb), total, dt


def parse_th(path, ngv=12, nnode=6, nnv=6):
    """Time records of the /TFILE/4 file: a 4-byte time record, the global
    record and the node record (big-endian float32) per output time."""
    recs = fortran_records(path)
    sizes = (4, 4 * ngv, 4 * nnode * nnv)
    t, g, nv = [], [], []
    i = 0
    while i + 2 < len(recs):
        if tuple(len(r) for r in recs[i:i + 3]) == sizes:
            t.append(struct.unpack(">f", recs[i])[0])
            g.append(struct.unpack(">%df" % ngv, recs[i + 1]))
            nv.append(np.array(struct.unpack(">%df" % (nnode * nnv), recs[i + 2])).reshape(nnode, nnv))
            i += 3
        else:
            i += 1
    return np.array(t, np.float32), np.array(g, np.float32), np.array(nv, np.float32)


def main():
    qa = qa_dir(QA_SUBDIR)
    dd = os.path.join(qa, "data")
    rd = os.path.join(qa, "reference")
    d = parse_starter(os.path.join(dd, "CONV_ELS_0000.rad"))
    d["run_tstop"] = np.float64(parse_engine(os.path.join(dd, "CONV_ELS_0001.rad")))
    rb, total, dt0 = parse_starter_out(os.path.join(rd, "CONV_ELS_0000.out"))
    d["starter_rbody"] = rb
    d["starter_rbody_columns"] = np.array("main x y z mass Ixx Iyy Izz Ixy Iyz Izx I1 I2 I3".split())
    d["starter_total_mass"] = np.float64(total)
    d["starter_solid_dt"] = np.float64(dt0)
    d["out"] = parse_out(os.path.join(rd, "CONV_ELS_0001.out"))
    d["out_columns"] = np.array("cycle time dt element error IE KE KER EXTW MASERR MASS".split())
    t, g, nv = parse_th(os.path.join(rd, "CONV_ELST01"))
    d["th_time"], d["th_glob"], d["th_node"] = t, g, nv
    d["th_glob_columns"] = np.array("IE KE XMOM YMOM ZMOM MASS DT RKE EXTW REINT ECONT HE".split())
    d["th_node_columns"] = np.array("DX DY DZ VX VY VZ".split())
    np.savez_compressed(OUT, **d)
    print("wrote %s: %d nodes, %d bricks, %d rigid bodies, %d printed cycles, %d TH times"
          % (OUT, len(d["node_id"]), len(d["brick_id"]), len(d["rbody_main"]), len(d["out"]),
             len(d["th_time"])))


if __name__ == "__main__":
    main()
