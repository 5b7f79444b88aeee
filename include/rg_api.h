/*
 * rg_api.h -- C ABI of the GB300-native explicit hot path of OpenRadioss.
 *
 * One context (rg_ctx) owns one model resident in the HBM of one GPU: nodes,
 * element groups with their state, the PARITH/ON skyline and the time-step
 * scalars.  All entry points take plain pointers and sizes, copy what they
 * are given (nothing is retained unless stated), and return an int status
 * (RG_OK or a negative RG_E* code; rg_last_error() gives the message).  No
 * entry point calls exit().  Calls on one context are not thread-safe: use one
 * context per host thread.
 *
 * Array conventions follow the reference engine so that a Fortran
 * ISO_C_BINDING module can pass its own arrays unchanged:
 *   X(3,NUMNOD), V(3,NUMNOD), A(3,NUMNOD)    xyz interleaved, FP64
 *   IXS(11,NUMELS)  {mat, n1..n8 (1-based), prop, user id}   int32
 *   IXC(7,NUMELC)   {mat, n1..n4 (1-based), prop, user id}   int32
 *   PM(NPROPM) / GEO(NPROPG)  material / property columns    FP64
 *   ADSKY(NUMNOD+1), IADS(8,NUMELS), IADC(4,NUMELC)  1-based skyline slots
 *   boundary code per node: bit 1/2/4 fixed x/y/z translation,
 *                           bit 8/16/32 fixed x/y/z rotation.
 *
 * The calls mirror the reference's GPU shell driver interface
 * (engine/source/elements/shell/coque/shell_gpu_driver.h:302-477) and its
 * Fortran binding (shell_gpu_mod.F90:292-713), widened to the whole explicit
 * cycle: element groups (FORINT/FORINTC, engine/source/elements/forint.F:95,
 * forintc.F:65), PARITH/ON assembly (ASSPAR4, engine/source/assembly/
 * asspar4.F:41), ACCELE / VELOCITY / DEPLA (assembly/accele.F:29,
 * velocity.F:29, displacement.F:29) and the RESOL time-step logic
 * (engine/source/engine/resol.F:2721, 6123-6127, 6352, 6494-6497).
 */
#ifndef RG_API_H
#define RG_API_H

#ifdef __cplusplus
extern "C" {
#endif

#define RG_OK 0
#define RG_E_ARG (-1)      /* invalid argument / size */
#define RG_E_STATE (-2)    /* call not allowed in the context's state */
#define RG_E_CUDA (-3)     /* CUDA runtime error */
#define RG_E_UNSUP (-4)    /* formulation not supported by this build */
#define RG_E_DEVICE (-5)   /* device-side status raised (see rg_status) */
#define RG_E_MEM (-6)      /* device memory budget exceeded */
#define RG_E_SIZE (-7)     /* size above a fixed no-allocation scratch */

/* device status bits (rg_status) */
#define RG_ST_NEGVOL 1     /* non-positive hexa volume (SCHKJABT3) */
#define RG_ST_NAN 2        /* non-finite nodal acceleration */
#define RG_ST_SLOT 4       /* skyline slot index out of range */
#define RG_ST_DTMIN 8      /* time step below the configured minimum */
#define RG_ST_BARRIER 16   /* batched kernel: grid barrier wait gave up */
#define RG_ST_NODSTIF 32   /* nodal time step: node with no stiffness (DTNODA stop) */

/* precision modes (rg_set_precision) */
#define RG_PREC_FP64 0     /* plain form: everything in FP64 */
#define RG_PREC_MIXED 1    /* FP32 element/material, FP64 nodal + energies */

typedef struct rg_ctx rg_ctx;

/* Create / destroy a context on CUDA device `device`.
 * Replaces shell_gpu_allocate / shell_gpu_global_allocate
 * (shell_gpu_driver.h:302-330). */
int rg_ctx_create(int device, rg_ctx **out);
int rg_ctx_destroy(rg_ctx *ctx);
const char *rg_last_error(rg_ctx *ctx);

/* Select the arithmetic form before rg_finalize. */
int rg_set_precision(rg_ctx *ctx, int mode);

/* Nodes: coordinates, velocities, lumped masses (MS), rotational inertia
 * (IN, may be NULL when no shells), boundary codes (may be NULL).
 * Replaces shell_gpu_global_upload_nodes (shell_gpu_driver.cu:149-185) for
 * the device-resident form; NODES%X/V/MS/IN (nodal_arrays.F90). */
int rg_mesh_upload(rg_ctx *ctx, int numnod, const double *x, const double *v,
                   const double *ms, const double *in, const int *icodt);

/* One-point hexa group (SFORC3, engine/source/elements/solid/solide/
 * sforc3.F:60): nel elements, IXS(11,nel), law mtn (1 = M1LAW elastic,
 * 2 = M2LAW Johnson-Cook), PM / GEO columns (NPROPM >= 100, NPROPG >= 200
 * entries read), LAW2 mat_param%uparam(1:12) / iparam(1:4) (may be NULL for
 * LAW1).  Supported formulation: ISMSTR=4, JHBE=1 (Isolid=1), Lagrangian,
 * jcvt (the starter's JCVT): 0 (Iframe=1, Jaumann rate, SROTA3) or 1
 * (co-rotational frame SRCOOR3 / SRROTA3, the starter's choice for 8-node
 * Lagrangian bricks when Iframe is left to default, sgrtails.F:906-912).
 * Returns the group index (>= 0) or an error. */
int rg_hexa_group_add(rg_ctx *ctx, int nel, const int *ixs, int mtn,
                      const double *pm, const double *geo,
                      const double *uparam, const int *iparam, int ismstr,
                      int jhbe, int jcvt);

/* Belytschko-Tsay 4-node shell group (CFORC3, engine/source/elements/shell/
 * coque/cforc3.F:85) with LAW2 (SIGEPS02C / M2CPLR): IXC(7,nel), npt
 * through-thickness points (1..5), initial thickness per element.
 * Replaces shell_gpu_upload_constant / _upload_ip_state / _set_mat_params /
 * _set_hg_params (shell_gpu_driver.h:330-420). */
int rg_shell_group_add(rg_ctx *ctx, int nel, const int *ixc, int npt,
                       const double *pm, const double *geo,
                       const double *uparam, const int *iparam,
                       const double *thk0, int ismstr, int ithk);

/* Planar rigid wall, infinite plane through p0 with normal nrm, sliding;
 * slave nodes: every node within dsearch of the plane at set-up
 * (RGWAL0/RGWALL, engine/source/constraints/general/rwall/rgwall.F:33). */
int rg_rwall_add(rg_ctx *ctx, const double *p0, const double *nrm,
                 double dsearch);

/* Rigid link between nodes: the engine deck's /VEL/TRA|ROT card, applied by
 * RLINK10 -> RLINK1 (engine/source/constraints/general/rlink/rlink10.F:38,
 * rlink1.F) after the boundary conditions of every cycle (resol.F:7355).
 * The nsn nodes (1-based) take the mass-weighted mean acceleration of the
 * link in the directions of ic and the inertia-weighted mean rotational
 * acceleration in those of icr (bits 4 = x, 2 = y, 1 = z; /VEL/TRA/XYZ is
 * ic = 7).  Before rg_finalize; a node belongs to one link at most.
 * Returns the link index. */
int rg_rlink_add(rg_ctx *ctx, int nsn, const int *nodes, int ic, int icr);

/* Switch link `link` on or off between cycles (a restart whose engine deck
 * no longer has the /VEL card); ordered after the cycles already queued. */
int rg_rlink_set_active(rg_ctx *ctx, int link, int active);

/* Nodal time step (/DT/NODA: DTNODA, engine/source/time_step/dtnoda.F:37,
 * called at resol.F:6066): the elements give only their stiffness (hexa STI
 * of MQVISCB, shell STI / STIR of CHVIS3's nodal branch, no CDT3), and the
 * cycle's step is the minimum over nodes of dtfac*sqrt(2*MS/STIFN) and, for
 * shell models, dtfac*sqrt(2*IN/STIFR) -- dtfac = DTFAC1(11).  NELTST then
 * holds the controlling node's number.  A step below dtmin (DTMIN1(11), 0 =
 * none) raises RG_ST_DTMIN; a node without stiffness RG_ST_NODSTIF.  Before
 * rg_finalize; models with it run alone (not in a batch). */
int rg_set_nodal_dt(rg_ctx *ctx, double dtfac, double dtmin);

/* Time-step actions of /DT (IDTMIN, DTMIN1), before rg_finalize; a model
 * with one runs alone (not in a batch).
 * kind 3 -- shells, IDTMIN(3) in CDT3 (engine/source/elements/shell/coque/
 *   cdt3.F:77-141): an element of OFF = 1 whose step is at or below dtmin
 *   raises RG_ST_DTMIN (idtmin 1 or 5: the engine stops) or is deleted
 *   (idtmin 2: OFF = 0 from that cycle on, out of the step minimum; its
 *   forces of that cycle are still assembled, as CFINT3 does not read OFF).
 * kind 11 -- nodal time step, IDTMIN(11) in DTNODA (dtnoda.F:258-305,
 *   459-500), with rg_set_nodal_dt: a node whose step is below dtmin raises
 *   RG_ST_DTMIN (idtmin 0, 1, 5) or takes the mass (inertia) of a step dtmin:
 *   MS = 1/2 STIFN (dtmin/DTFAC1)^2 * 1.00001 (idtmin 3 or 8), used from
 *   that cycle's ACCELE on; the added mass shows in rg_energy_balance.
 * Other kinds and actions (IDTMIN(3) = 3 small-strain switch, IDTMIN(11) =
 * 4 acceleration scaling) are refused with RG_E_UNSUP.  Solids: a hexa of
 * non-positive volume is always deleted and flagged RG_ST_NEGVOL
 * (SCHKJAB3); the engine stops on the flag or carries on (IDTMIN(1) = 2). */
int rg_set_dtmin(rg_ctx *ctx, int kind, int idtmin, double dtmin);

/* Local shell frame of CNVEC3 (cnvec3.F:117-170): ISHFRAM 0 (symmetric
 * convected frame, default) or 2 (the starter's /SHFRA/V4, contrl.F:495-498).
 * Before rg_finalize. */
int rg_set_shell_frame(rg_ctx *ctx, int ishfram);

/* Optional: PARITH/ON tables from the engine (ADSKY(NUMNOD+1), IADS(8,
 * NUMELS), IADC(4,NUMELC), 1-based; FILLCNE order, starter/source/spmd/
 * domdec2.F:2046).  Without this call rg_finalize builds them in that order. */
int rg_skyline_set(rg_ctx *ctx, const int *adsky, const int *iads,
                   const int *iadc);

/* Finish set-up: builds the skyline if not given, initial element state
 * (volume, density), uploads everything and captures the cycle graph.
 * dtfac_* = DTFAC1(1) / DTFAC1(3), dtmx = DTMX, dt2old = initial DT2OLD. */
int rg_finalize(rg_ctx *ctx, double dtfac_solid, double dtfac_shell,
                double dtmx, double dt2old);

/* Read the PARITH/ON tables in use (any pointer may be NULL). */
int rg_skyline_get(rg_ctx *ctx, int *adsky, int *iads, int *iadc, int *lsky);

/* Advance ncycle explicit cycles on the device (RESOL loop body: element
 * groups -> ASSPAR4 -> dt -> ACCELE -> BCS -> rigid walls -> VELOCITY ->
 * DEPLA).  Asynchronous: returns after enqueueing; rg_synchronize waits. */
int rg_cycle(rg_ctx *ctx, int ncycle);
int rg_synchronize(rg_ctx *ctx);

/* FORINT-level drop-in (host buffers): upload X,V (and VR) for this cycle,
 * run every element group with time step dt1, assemble in PARITH/ON order
 * and return the nodal forces F(3,NUMNOD), STIFN(NUMNOD) (FR, STIFR for
 * shells, may be NULL) and the element time step dt2t (min of DTFAC*DTX).
 * This is the per-cycle call a Fortran engine makes in place of FORINT +
 * ASSPAR4 (resol.F:4138-4858); the engine keeps its own nodal update.
 * Host buffers may be pinned with rg_host_register: registered inputs are
 * read in place, and registered outputs (F, FR aligned to 16 bytes) are
 * written in place by the device.  For a model without rotations FR and
 * STIFR come back zero. */
int rg_forint_step(rg_ctx *ctx, const double *x, const double *v,
                   const double *vr, double dt1, double *f, double *stifn,
                   double *fr, double *stifr, double *dt2t, int *neltst);
/* Whole cycle with host node buffers, for an engine that keeps X, V on the
 * host for its other work (outputs, contact) but lets the device do the
 * complete explicit cycle: x, v (and vr) -- both or neither -- replace the
 * device's node positions and velocities, one cycle of rg_cycle runs
 * (elements, PARITH/ON assembly, RESOL time step, ACCELE, BCS, rigid walls,
 * VELOCITY, DEPLA), and the new X, V (VR, D = displacement) are written to
 * the *_out buffers (any may be NULL; they may alias the inputs), *dt2 = the
 * cycle's step.  Synchronous.  The device keeps the time-step record and the
 * element state.  In the mixed form the element volumes are re-anchored to
 * the given coordinates, as in rg_forint_step.  Registered host buffers
 * (rg_host_register) are read in place, and registered outputs aligned to
 * 16 bytes are written in place by the device.  The reference's GPU shell path
 * moves the same arrays each cycle (shell_gpu_global_upload_nodes,
 * shell_gpu_driver.cu:149-185) but leaves the nodal update on the host. */
int rg_cycle_host(rg_ctx *ctx, const double *x, const double *v, const double *vr,
                  double *x_out, double *v_out, double *vr_out, double *d_out,
                  double *dt2);
int rg_host_register(rg_ctx *ctx, void *ptr, unsigned long long bytes);
int rg_host_unregister(rg_ctx *ctx, void *ptr);

/* Results (synchronous). */
int rg_download_nodes(rg_ctx *ctx, double *x, double *v, double *d,
                      double *vr);
/* Assembled forces of the last cycle (A before division by the mass),
 * STIFN, moments FR (any may be NULL). */
int rg_download_forces(rg_ctx *ctx, double *f, double *stifn, double *fr);
/* Hexa element state over all hexa groups in order: which = 0 SIG (6 x
 * NUMELS, component-major), 1 EINT, 2 RHO, 3 QVIS, 4 OFF, 5 PLA, 6 EPSD,
 * 7 VOL0, 8 accumulated hourglass energy. */
int rg_download_hexa_state(rg_ctx *ctx, int which, double *out);
/* Shell element state: which = 0 FOR (5 x NUMELC), 1 MOM (3 x NUMELC),
 * 2 THK, 3 EINT (2 x NUMELC), 4 OFF, 5 SIG per IP (5 x npt x NUMELC),
 * 6 PLA per IP (npt x NUMELC). */
int rg_download_shell_state(rg_ctx *ctx, int which, double *out);
int rg_get_time(rg_ctx *ctx, double *tt, double *dt1, double *dt2,
                int *ncycle, int *neltst);
/* Energies with fixed-order device reductions: element internal,
 * translational / rotational kinetic, accumulated hourglass. */
int rg_energy(rg_ctx *ctx, double *eint, double *ekin, double *ekinr,
              double *ehour);
/* Energy balance of the listing's cycle line (ECRIT, engine/source/output/
 * ecrit.F:501-517), n <= 13 values: 0 TT, 1 internal energy, 2 kinetic,
 * 3 rotational kinetic, 4 accumulated hourglass, 5 external work of the
 * rigid walls (WFEXT), 6 ENTOT = IE + KE + KE-R, 7 energy error in percent
 * 100 (ENTOT / (ENTOT0 + WFEXT) - 1) clamped to +-99 with ENTOT0 taken at
 * rg_finalize, 8 total nodal mass, 9 mass error (M - M0) / M0, 10-12
 * momentum x, y, z.  The node sums are fixed-order device reductions. */
int rg_energy_balance(rg_ctx *ctx, double *out, int n);

/* Per-part element sums, the PARTSAV accumulation of SBILAN (engine/source/
 * elements/solid/solide/sbilan.F:118-160) and CBILAN (elements/shell/coque/
 * cbilan.F:160-190) plus CHVIS3's hourglass energy (chvis3.F:355-395): the
 * default /TH/PART variables (output/th/hist2.F:377-395) of each part,
 * out[p * RG_PART_NQ + q] with q = 0 IE, 1 KE (element-based: the element
 * mass times the mean square of its nodes' velocities), 2-4 momentum,
 * 5 mass of the elements not switched off, 6 accumulated hourglass energy.
 *
 * rg_set_parts (after rg_finalize) gives every element's 0-based part
 * number, in element order (the groups in the order added); without it
 * each element group is a part (hexa groups first, then shell groups).
 * rg_part_count gives the context's part count.  rg_part_sums_due asks
 * the next cycle -- rg_cycle (its first cycle), rg_cycle_host or
 * rg_forint_step -- to take the sums where the engine does when it prints
 * (IPRI, resol.F): after the element pass, before the nodal update, from
 * X(n), V(n-1/2) and the element state of that cycle.  rg_part_sums reads
 * them (RG_E_STATE before any such cycle; the batched kernel does not take
 * them).  Fixed-order device reductions: the sums do not depend on the
 * launch layout. */
#define RG_PART_NQ 7
int rg_set_parts(rg_ctx *ctx, int npart, const int *hexa_part,
                 const int *shell_part);
int rg_part_count(rg_ctx *ctx, int *npart);
int rg_part_sums_due(rg_ctx *ctx);
int rg_part_sums(rg_ctx *ctx, double *out, int npart);

/* Device status word (RG_ST_* bits), cleared by the read. */
int rg_status(rg_ctx *ctx);

/* Checkpoint / restart of one model, the device-resident counterpart of the
 * engine's restart file (WRRESTP, engine/source/output/restart/
 * wrrestp.F:161): the snapshot holds every device array of the context --
 * nodes, element and point state, PARITH/ON slots, the time-step record,
 * link switches, status -- behind a header naming the model (counts,
 * precision, allocation layout).  rg_snapshot copies after the cycles
 * already queued (synchronous; a context in a batch: after
 * rg_batch_synchronize).  rg_restore accepts a snapshot of the same model
 * set up the same way (this context or a fresh one: a restart in another
 * process) and refuses any other with RG_E_ARG; the run then resumes bit for
 * bit.  Host buffers are plain memory of rg_snapshot_size bytes. */
int rg_snapshot_size(rg_ctx *ctx, unsigned long long *bytes);
int rg_snapshot(rg_ctx *ctx, void *buf, unsigned long long bytes);
int rg_restore(rg_ctx *ctx, const void *buf, unsigned long long bytes);

/* Inspection / benchmarking. */
int rg_info(rg_ctx *ctx, int *numnod, int *numels, int *numelc, int *lsky,
            unsigned long long *device_bytes);
/* Mean device time per launch (ms) of each kernel class over the last
 * rg_cycle call when timing is enabled: [0] hexa, [1] shell, [2] dt (0
 * when the time-step reduction runs inside the element kernels), [3] node.  rg_set_timing(ctx, 1) enables event timing (no graph); once
 * rg_time_cycles_cold has run, each timed cycle starts from cold L2. */
int rg_set_timing(rg_ctx *ctx, int on);
int rg_kernel_times(rg_ctx *ctx, double *ms4);
/* Advance ncycle cycles (graph launches) bracketed by CUDA events recorded
 * on the context's stream; *ms = device time of the whole span. */
int rg_time_cycles(rg_ctx *ctx, int ncycle, double *ms);
/* Same, each cycle preceded by a write of flush_bytes (> L2) to a buffer of
 * the context, outside the timed spans: *ms = sum of the per-cycle device
 * times, every cycle starting from cold L2. */
int rg_time_cycles_cold(rg_ctx *ctx, int ncycle, unsigned long long flush_bytes,
                        double *ms);

/* Kinetic energy 0.5*sum(MS*|V|^2) of caller-owned DEVICE arrays V(3,numnod)
 * and MS(numnod) on CUDA device `device`, without allocating device memory:
 * the per-block partial sums live in a fixed file-scope device scratch of
 * RG_NOALLOC_MAX_BLOCKS doubles, each block covering
 * RG_NOALLOC_NODES_PER_BLOCK nodes, so numnod may be at most
 * RG_NOALLOC_MAX_BLOCKS * RG_NOALLOC_NODES_PER_BLOCK (67,108,864); larger
 * sizes are refused with RG_E_SIZE before any device work.  For callers that
 * must not allocate at that moment (a serving loop whose HBM budget is fully
 * reserved; an engine that accounts its own device memory).  Synchronous, on
 * the legacy default stream, which is not ordered after a context's own
 * (non-blocking) stream: call rg_synchronize(ctx) -- or synchronise whatever
 * stream produced the arrays -- before this call, or it races with the
 * cycles still queued.  Nothing in the scratch needs to start at zero (each
 * call overwrites the partials it reads); the scratch is shared per device,
 * so calls that overlap in time on one device race and must be serialised by
 * the caller.  The first call on a device looks the scratch address up
 * (cudaGetSymbolAddress); with CUDA's default lazy module loading that is
 * when the library's module, and the 512 KB scratch with it, is loaded onto
 * the device, so the first call does take device memory: make one warm-up
 * call per device while there is still room (before reserving the whole HBM
 * budget) and before starting any stream capture on that device; later calls
 * allocate nothing.  No counterpart in the reference (its energy sums are
 * host loops). */
#define RG_NOALLOC_NODES_PER_BLOCK 1024
#define RG_NOALLOC_MAX_BLOCKS 65536
int rg_kinetic_energy_noalloc(int device, int numnod, const double *d_v,
                              const double *d_ms, double *ekin);

/* Measured FP64 fused multiply-add rate of device `device` (thread
 * instructions per second, ~0.1 s of a dedicated kernel): the ceiling of the
 * FP64-pipe roofline of the plain form.  Benchmarking aid; no counterpart in
 * the reference. */
int rg_fp64_peak(int device, double *fma_per_s);

/* ---- Batched jobs -------------------------------------------------------
 * A batch advances many finalized contexts (independent models, "jobs") of
 * the same arithmetic form together: one persistent cooperative kernel per
 * cycle (element tiles of every job -> grid barrier -> per-job time step ->
 * grid barrier -> node tiles of every job), captured in a CUDA graph.  Each
 * job keeps its own state, time step and cycle target.  Within the batched
 * kernel a job's results are bitwise the same under every launch
 * configuration, schedule and batch composition; against rg_cycle on the
 * job alone (separately compiled kernels, whose multiply-add contraction may
 * differ) they agree within 1e-10 (FP64) / 1e-4 (mixed form) of the job's
 * displacement and velocity scales, and the job reaches exactly its cycle
 * target.  While a context is in a batch,
 * only the batch advances it; read its results with the rg_download_* calls
 * after rg_batch_synchronize.  No counterpart in the reference (its engine
 * runs one model per process); the per-job cycle is the RESOL loop body. */
typedef struct rg_batch rg_batch;
int rg_batch_create(int device, rg_batch **out);
int rg_batch_destroy(rg_batch *b);
const char *rg_batch_last_error(rg_batch *b);
/* Add a job; it advances until its Time::ncycle reaches target_ncycle
 * (< 0: no target).  Returns the slot (>= 0) or an error. */
int rg_batch_add(rg_batch *b, rg_ctx *job, int target_ncycle);
int rg_batch_remove(rg_batch *b, int slot);
int rg_batch_set_target(rg_batch *b, int slot, int target_ncycle);
/* Launch configuration: elements per tile = 128*ktile, nodes per tile =
 * 128*knode, resident blocks per SM (0 = occupancy maximum), schedule 0 =
 * one persistent cooperative launch per cycle, 1 = three launches. */
int rg_batch_set_config(rg_batch *b, int ktile, int knode, int blocks_per_sm,
                        int schedule);
/* cfg5 = {ktile, knode, blocks_per_sm, schedule, max blocks per SM}. */
int rg_batch_get_config(rg_batch *b, int *cfg5);
int rg_batch_cycle(rg_batch *b, int ncycle);
int rg_batch_synchronize(rg_batch *b);
int rg_batch_time_cycles(rg_batch *b, int ncycle, double *ms);
/* ncycle[slot] = the job's cycle count after the last batched cycle (-1 for
 * a free slot); bstatus = batch status (RG_ST_BARRIER), cleared. */
int rg_batch_progress(rg_batch *b, int *ncycle, int nslots, int *bstatus);
/* Status word (RG_ST_* bits) of every job's own context after the batch's
 * queued cycles: status[slot], 0 for a free slot; the words are left set
 * (the job's rg_status reads and clears its own).  A job whose word is raised
 * can be removed (rg_batch_remove) while the other jobs go on: jobs share no
 * data.  No counterpart in the reference (one model per process; its
 * engine stops the run, MSTOP / TSTOP, resol.F). */
int rg_batch_job_status(rg_batch *b, int *status, int nslots);
/* Test hook of the batched kernel's bounded grid barrier: spin_limit naps of
 * 64 ns before a waiting block gives up (0 = the default, about a second),
 * and block late_block (-1 = none) made to arrive at every barrier after
 * late_us microseconds (at most 1e6) of sleep.  With a limit shorter than
 * the delay the waits run out: the kernel records RG_ST_BARRIER (read by
 * rg_batch_progress) and returns; the cycle's results are void, the batch
 * stays usable.  Nothing waits without a bound, nothing faults. */
int rg_batch_set_barrier_test(rg_batch *b, unsigned spin_limit, int late_block,
                              unsigned late_us);
/* Autotuner: times each candidate configuration ({ktile, knode,
 * blocks_per_sm, schedule} rows; NULL = built-in list) for trial_cycles on
 * the batch's jobs with their state saved and restored, keeps the fastest.
 * best5 = {ktile, knode, blocks_per_sm, schedule, microseconds per cycle}. */
int rg_batch_autotune(rg_batch *b, int trial_cycles, const int *cand,
                      int ncand, int *best5);

#ifdef __cplusplus
}
#endif
#endif /* RG_API_H */
