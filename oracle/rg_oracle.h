/*
 * CPU oracle for the OpenRadioss explicit hot path -- TEST INFRASTRUCTURE.
 *
 * This library restates, in plain C++ on the CPU and in FP64, the reference
 * Fortran routines of one explicit cycle (element forces -> PARITH/ON slot
 * assembly -> acceleration -> boundary conditions -> velocity ->
 * displacement -> time step).  It exists only to check the CUDA product and to
 * time the CPU baseline; the product never links, loads or calls it.
 *
 * Parity status: the reference engine cannot be built here (no Fortran
 * compiler).  The shell path (CFORC3, LAW2, PARITH/ON assembly, ACCELE, BCS,
 * rigid link, VELOCITY / DEPLA, time step) is pinned against outputs of the
 * reference engine itself: its QA deck CRA2V44 (768 shells, 3375 cycles over
 * a run and a restart), whose printed cycle table the oracle reproduces to
 * every printed digit and whose time histories to ~1e-6 relative
 * (tests/test_oracle_cra2.py).  The hexa path (LAW1, co-rotational frame,
 * viscous hourglass) is pinned the same way by the QA deck H101 (six
 * cantilevers with rigid-body tips under concentrated loads, 847 cycles:
 * printed table to every digit, energies and tip motions to ~1e-7,
 * tests/test_oracle_h101.py), and by analytic known-answer tests
 * (rigid-body motion, constant-strain patch test, elastic wave speed,
 * energy conservation, Johnson-Cook uniaxial yield).
 *
 * Conventions follow the reference: nodal arrays are X(3,NUMNOD) (xyz
 * interleaved), IXS(11,NUMELS) columns hold {mat, n1..n8 (1-based), prop,
 * user id}, IXC(7,NUMELC) hold {mat, n1..n4, prop, user id}.
 */
#pragma once

// Phase marks of the op-counting build (rg_opcount.h); nothing elsewhere.
#ifndef RG_OPCOUNT_PHASE
#ifdef RG_OPCOUNT
#define RG_OPCOUNT_PHASE(p) (rg_count::phase = (p))
#else
#define RG_OPCOUNT_PHASE(p) ((void)0)
#endif
#endif
#ifdef __cplusplus
extern "C" {
#endif

void *or_model_new(int numnod, const double *x, const double *v,
                   const double *ms, const int *icodt);
void or_model_free(void *m);

/* Hexa group (SFORC3 path).  pm / geo are the material / property columns
 * (PM(1:NPROPM,imat), GEO(1:NPROPG,iprop)); uparam / iparam the LAW2
 * mat_param%uparam(1:12) / iparam(1:4); jcvt 0 (Iframe=1, Jaumann rate) or
 * 1 (co-rotational frame, the default of 8-node Lagrangian bricks).
 * Returns the group index or <0. */
int or_hexa_group_add(void *m, int nel, const int *ixs, int mtn,
                      const double *pm, const double *geo,
                      const double *uparam, const int *iparam, int ismstr,
                      int jhbe, int jcvt);

/* Belytschko-Tsay shell group (CFORC3 path, LAW2). */
int or_shell_group_add(void *m, int nel, const int *ixc, int npt,
                       const double *pm, const double *geo,
                       const double *uparam, const int *iparam,
                       const double *thk0, int ismstr, int ithk);

/* Rotational inertia (shell nodes). */
int or_set_inertia(void *m, const double *in);

/* Planar rigid wall (RGWALL, infinite plane): point, outward normal,
 * sliding (0) ; slave nodes all nodes with distance < dsearch. */
int or_rwall_add(void *m, const double *p0, const double *nrm,
                 double dsearch);

/* Build PARITH/ON tables (FILLCNE order) and finish set-up. */
int or_finalize(void *m, double dtfac_solid, double dtfac_shell, double dtmx,
                double dt2old_init, int nthreads);

/* Skyline tables (after finalize): adsky (numnod+1, 1-based like ADSKY),
 * iads (8*numels), iadc (4*numelc). */
int or_get_skyline(void *m, int *adsky, int *iads, int *iadc, int *lsky);

int or_cycle(void *m, int ncycle);

/* Nodal results: X, V, D (3*numnod each, any may be NULL); F = assembled
 * forces of the last cycle (A before division by mass), STIFN. */
int or_get_nodes(void *m, double *x, double *v, double *d, double *vr,
                 double *f, double *stifn, double *fr);
int or_get_time(void *m, double *tt, double *dt1, double *dt2,
                int *ncycle, int *neltst);
/* Element state: which = 0 sig(6*nel, c*nel+i), 1 eint, 2 rho, 3 qvis,
 * 4 offg, 5 pla, 6 epsd, 7 vol0. */
int or_get_hexa_state(void *m, int group, int which, double *out);
/* Energies: internal, kinetic (translational), kinetic rotational,
 * hourglass (accumulated). */
int or_energy(void *m, double *eint, double *ekin, double *ekinr,
              double *ehour);
int or_error(void *m);

/* Nodal time step (/DT/NODA; DTNODA, time_step/dtnoda.F): elements give
 * only their stiffness, the cycle's step is the minimum over nodes of
 * dtfac*sqrt(2*MS/STIFN) (and 2*IN/STIFR for shell nodes).  Before
 * or_finalize.  Error bits: 8 below dtmin, 32 node without stiffness. */
int or_set_nodal_dt(void *m, double dtfac, double dtmin);
/* /DT time-step actions: kind 3 shells (IDTMIN(3) 1/5 stop flag, 2 delete),
 * kind 11 nodal step (IDTMIN(11) 3/8 mass scaling, else stop flag). */
int or_set_dtmin(void *m, int kind, int idtmin, double dtmin);
/* Rigid-material body (/MAT/RIGID, LAW13) of the starter's RIGID_MAT:
 * 1-based secondary nodes, centre of mass, mass, principal axes (rows, 3x3)
 * and principal inertia.  Before or_finalize. */
int or_rmat_add(void *m, int nsl, const int *nodes, const double *xg, double mass,
                const double *axes, const double *inertia);
/* Imposed velocity (/IMPVEL, IDIS = 1) on a 1-based node along x, y or z
 * (0..2): F((TT + DT2/2) * facx) * fscale between tstart and tstop. */
int or_impvel_add(void *m, int node, int dir, double facx, double fscale, double tstart,
                  double tstop, int npts, const double *x, const double *y);
/* Nodal masses and inertias (after any mass scaling). */
int or_get_mass(void *m, double *ms, double *in);
/* Local shell frame: 0 = symmetric convected frame (default), 2 = the
 * version-4 frame of /SHFRA/V4 (CNVEC3, cnvec3.F:143-170). */
int or_shell_frame(void *m, int ishfram);
/* Rigid link (engine /VEL/TRA|ROT, RLINK1): nodes 1-based, ic / icr the
 * translational / rotational direction bits (4 = x, 2 = y, 1 = z).  Applied
 * after the boundary conditions of every cycle.  or_rlink_clear removes all
 * links (a restart whose engine deck has no /VEL card). */
int or_rlink_add(void *m, int nsn, const int *nodes, int ic, int icr);
int or_rlink_clear(void *m);
/* Rigid body (/RBODY; RBYFOR, RBYVIT, RBYCOR): main node and nsn > 2
 * secondary nodes (1-based); the caller has done the starter's INIRBY: the
 * main node sits at the centre of mass with MS = body mass and IN = the
 * smallest principal inertia; axes = principal directions as rows (RBY(1:9),
 * right-handed), inertia = principal inertia (RBY(10:12)).  Before
 * or_finalize; or_set_inertia must come first.  Error bit 64: a body turns
 * more than one radian in a step. */
int or_rbody_add(void *m, int main, int nsn, const int *nodes,
                 const double *axes, const double *inertia);
/* Concentrated load (/CLOAD; FORCE): node 1-based, dir 0..2 force x/y/z,
 * 3..5 moment; the load curve (npts increasing abscissae, FINTER) is read at
 * TT * fcx and scaled by fcy.  Its external work enters the listing record. */
int or_cload_add(void *m, int node, int dir, double fcx, double fcy, int npts,
                 const double *x, const double *y);
/* Element forces from outside for the next cycle (a FORINT done elsewhere,
 * e.g. by the CUDA path's rg_forint_step): F(3,NUMNOD) and STIFN (FR,
 * STIFR may be NULL) are the assembled element forces, dt2t / neltst the
 * element time step and its element.  The next or_cycle(m, 1) skips its own
 * element groups and slot sums and runs the rest of RESOL (loads, rigid
 * bodies, ACCELE, conditions, listing, VELOCITY, DEPLA) on these. */
int or_set_forces(void *m, const double *f, const double *stifn, const double *fr,
                  const double *stifr, double dt2t, int neltst);
/* Listing record of the last cycle (what ECRIT prints): out[0..10] = TT,
 * DT2, internal energy, kinetic energy and rotational kinetic energy of
 * V + DT1/2 A, hourglass energy, x/y/z momentum, mass, external work of the
 * concentrated loads.  Off by default. */
int or_set_record(void *m, int on);
int or_get_wfext(void *m, double *out);
int or_get_record(void *m, double *out, int *neltst);
/* Shell state: which = 0 FOR (5 x nc), 1 MOM (3 x nc), 2 THK, 3 EINT
 * (2 x nc), 4 OFF, 5 SIG (5 x npt x nc), 6 PLA (npt x nc), 7 HOUR (5 x nc). */
int or_get_shell_state(void *m, int which, double *out);
/* Per-part sums (SBILAN / CBILAN) of the recorded cycles: element -> part
 * maps (0-based) and the sums of the last recorded cycle, out[p * 7 + q]
 * = IE, KE, XMOM, YMOM, ZMOM, MASS, HE; returns the part count. */
int or_set_parts(void *m, int npart, const int *hexa_part, const int *shell_part);
int or_get_part_sums(void *m, double *out, int npart);

#ifdef __cplusplus
}
#endif
