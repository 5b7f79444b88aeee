"""Generate tests/golden/loi13.npz from the OpenRadioss QA deck LOI13/solide.

The deck (qa-tests/miniqa/LOIS/LOI13/solide of the OpenRadioss tree) holds a
block of 466 one-point hexahedra of a Johnson-Cook material (/MAT/PLAS_JOHNS,
no strain-rate effect, /PROP/SOLID Isolid = 1, Iframe = 2: co-rotational),
and three parts of /MAT/RIGID (LAW13) bricks, each of which the starter makes
a rigid-material body.  The block's bottom face is fixed; its top nodes move
down under an imposed velocity (/IMPVEL, a linear ramp /FUNCT 1) and crush
it plastically.  One engine run to t = 8.01 (1636 cycles).

What this script extracts (numbers only, no text of the deck is kept):

* the starter deck: nodes, bricks with their parts, the materials (Johnson-
  Cook and rigid), /PROP/SOLID, /BCS groups, /IMPVEL, /FUNCT and the run's
  end time and time-step factor from the engine deck;
* the starter listing (MODELE_0000.out): for each rigid-material body its
  secondary nodes, centre of mass and mass; the total mass; the starter's
  smallest solid time step;
* the engine listing (MODELE_0001.out): cycle, time, time step, controlling
  element, energy error, internal, kinetic, rotational kinetic energy,
  external work, mass error and total mass of every printed cycle;
* the time-history file MODELET01 (big-endian Fortran sequential records,
  /TFILE every 0.01): the 12 global variables.

The deck is (C) Siemens, licensed CC BY-NC 4.0 (header of MODELE_0000.rad);
the fixture carries its numbers for parity testing only.

Usage:  python tests/golden/make_loi13.py [path to the LOI13/solide QA directory]
        (or OPENRADIOSS_SRC=<root of the OpenRadioss tree> python tests/golden/make_loi13.py)
"""
from __future__ import annotations

import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_cra2 import fortran_records, grnod, ints, nums, one, qa_dir, read_blocks  # noqa: E402,E501
from make_h101 import parse_out  # noqa: E402

QA_SUBDIR = "qa-tests/miniqa/LOIS/LOI13/solide"
OUT = os.path.join(HERE, "loi13.npz")


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
    # /MAT/PLAS_JOHNS: title | rho rho_ref | E nu | a b n epsmax sigmax |
    # c eps0 Icc Fsmooth Fcut | m Tmelt rhoCp Ti
    jc = None
    rigid = {}
    for k in b:
        if k[0].startswith("/MAT/PLAS_JOHNS/"):
            ln = k[1]
            rho = nums(ln[1])[0]
            e, nu = nums(ln[2])[:2]
            a, bb, n, epsmax, sigmax = nums(ln[3])[:5]
            c, eps0 = nums(ln[4])[:2]
            m, tmelt, rhocp, ti = nums(ln[5])[:4]
            jc = [int(k[0].split("/")[3]), rho, e, nu, a, bb, n, epsmax, sigmax, c, eps0,
                  m, tmelt, rhocp, ti]
        elif k[0].startswith("/MAT/RIGID/"):
            rho = nums(k[1][1])[0]
            e, nu = nums(k[1][2])[:2]
            rigid[int(k[0].split("/")[3])] = [rho, e, nu]
    d["mat_jc"] = np.array(jc)
    d["mat_jc_columns"] = np.array("id rho E nu a b n epsmax sigmax c eps0 m Tmelt rhoCp Ti".split())
    d["mat_rigid"] = np.array([[i] + v for i, v in sorted(rigid.items())])
    # /PROP/SOLID: Isolid Ismstr Icpre Inpts Iframe dn | qa qb h | dtmin
    pr = one(b, "/PROP/SOLID/1")
    d["prop"] = np.array(nums(pr[1])[:6] + nums(pr[2])[:3])
    d["prop_columns"] = np.array("Isolid Ismstr Icpre Inpts Iframe dn qa qb h".split())
    tra, rot, off, bn = [], [], [0], []
    for k in sorted((k for k in b if k[0].startswith("/BCS/")), key=lambda k: k[1][1]):
        t, r, skew, g = k[1][1].split()
        if int(skew) != 0:
            raise ValueError("skewed BCS not expected")
        tra.append(t)
        rot.append(r)
        bn += grnod(b, int(g)).tolist()
        off.append(len(bn))
    d["bcs_tra"] = np.array(tra)
    d["bcs_rot"] = np.array(rot)
    d["bcs_nodes"] = np.array(bn, np.int32)
    d["bcs_offsets"] = np.array(off, np.int32)
    # /IMPVEL: Ifunct DIR Iskew Isensor Gnod Iframe | Ascale_x Fscale_y Tstart Tstop
    iv = one(b, "/IMPVEL/1")
    f, dirn, skew, sens, g, fr = iv[1].split()[:6]
    if int(skew) or int(sens) or int(fr):
        raise ValueError("unexpected /IMPVEL card")
    d["impvel_funct"] = np.int32(f)
    d["impvel_dir"] = np.int32("XYZ".index(dirn))
    d["impvel_nodes"] = grnod(b, int(g))
    d["impvel_scale"] = np.array(nums(iv[2])[:4])
    fl = one(b, "/FUNCT/1")
    d["funct1"] = np.array([nums(ln)[:2] for ln in fl[1:]])
    return d


def parse_engine(path):
    b = read_blocks(path)
    run = [k for k in b if k[0].startswith("/RUN/")]
    dt = [k for k in b if k[0] == "/DT"]
    return nums(run[0][1][0])[0], nums(dt[0][1][0])


def parse_starter_out(path):
    """Rigid-material bodies (RIGID_MAT: number of secondary nodes, centre of
    mass, mass and the secondary node ids), the total mass and the
    starter's smallest solid time step."""
    lines = open(path, encoding="latin1").read().splitlines()
    bodies, total, dt = [], None, None
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.strip().startswith("RIGID BODY ID") and "NUMBER OF SECONDARY NODE" in lines[i + 1]:
            nsl = int(lines[i + 1].split()[-1])
            xyz = [float(v) for v in lines[i + 2].split()[-3:]]
            mass = float(lines[i + 3].split()[-1])
            ids = []
            j = i + 5
            while len(ids) < nsl:
                ids += [int(v) for v in lines[j].split()]
                j += 1
            bodies.append((xyz, mass, ids))
            i = j
            continue
        if "TOTAL MASS AND MASS CENTER" in ln:
            total = float(lines[i + 4].split()[0])
        elif "SOLID ELEMENTS TIME STEP" in ln and dt is None:
            dt = float(lines[i + 4].split()[0])
        i += 1
    return bodies, total, dt


def parse_th(path, ngv=12):
    """Time records of the /TFILE file without /TH groups: a 4-byte time
    record and the global record (big-endian float32) per output time."""
    recs = fortran_records(path)
    t, g = [], []
    i = 0
    while i + 1 < len(recs):
        if len(recs[i]) == 4 and len(recs[i + 1]) == 4 * ngv:
            t.append(struct.unpack(">f", recs[i])[0])
            g.append(struct.unpack(">%df" % ngv, recs[i + 1]))
            i += 2
        else:
            i += 1
    return np.array(t, np.float32), np.array(g, np.float32)


def main():
    qa = qa_dir(QA_SUBDIR)
    dd = os.path.join(qa, "data")
    rd = os.path.join(qa, "reference")
    d = parse_starter(os.path.join(dd, "MODELE_0000.rad"))
    tstop, dtcard = parse_engine(os.path.join(dd, "MODELE_0001.rad"))
    d["run_tstop"] = np.float64(tstop)
    d["run_dt"] = np.array(dtcard)
    bodies, total, dt0 = parse_starter_out(os.path.join(rd, "MODELE_0000.out"))
    d["rm_com"] = np.array([b[0] for b in bodies])
    d["rm_mass"] = np.array([b[1] for b in bodies])
    d["rm_nodes"] = np.array(sum((b[2] for b in bodies), []), np.int32)
    d["rm_offsets"] = np.cumsum([0] + [len(b[2]) for b in bodies]).astype(np.int32)
    d["starter_total_mass"] = np.float64(total if total is not None else np.nan)
    d["starter_solid_dt"] = np.float64(dt0)
    d["out"] = parse_out(os.path.join(rd, "MODELE_0001.out"))
    d["out_columns"] = np.array("cycle time dt element error IE KE KER EXTW MASERR MASS".split())
    t, g = parse_th(os.path.join(rd, "MODELET01"))
    d["th_time"], d["th_glob"] = t, g
    d["th_glob_columns"] = np.array("IE KE XMOM YMOM ZMOM MASS DT RKE EXTW REINT ECONT HE".split())
    np.savez_compressed(OUT, **d)
    print("wrote %s: %d nodes, %d bricks, %d rigid-material bodies, %d printed cycles, "
          "%d TH times" % (OUT, len(d["node_id"]), len(d["brick_id"]), len(bodies),
                           len(d["out"]), len(d["th_time"])))


if __name__ == "__main__":
    main()
