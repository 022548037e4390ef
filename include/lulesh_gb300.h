/*
 * lulesh_gb300.h -- C ABI of the GB300 LULESH Lagrange leap-frog path.
 *
 * The reference exposes its hot path as two file-static C++ functions that
 * mutate a host-side Domain in place and are driven by main():
 *   TimeIncrement(Domain&)        lulesh.cc:166
 *   LagrangeLeapFrog(Domain&)     lulesh.cc:2601
 *   main loop                     lulesh.cc:2745-2757
 *   Domain accessors              lulesh.h:263-429
 *   Domain::Domain (problem set-up) lulesh-init.cc:16-194
 *   VerifyAndWriteFinalOutput     lulesh-util.cc:175-230
 * and it reports errors by exit(VolumeError = -1) / exit(QStopError = -2)
 * (lulesh.h:42).  This header replaces that surface with a handle API over a
 * device-resident Domain.  All pointers are plain host pointers; no CUDA or
 * PyTorch types appear in the signatures.
 *
 * Status codes (every entry point returns one):
 *    0  LG_OK
 *   -1  LG_VOLUME_ERROR   (reference exit(VolumeError))
 *   -2  LG_QSTOP_ERROR    (reference exit(QStopError))
 *   >0  API / CUDA errors, see lg_status; lg_last_error() has the text.
 *
 * Threading: one handle per host thread; each handle owns one CUDA stream.
 * Ownership: device memory belongs to the handle; host buffers passed to the
 * get/set calls belong to the caller and are not retained.
 */
#ifndef LULESH_GB300_H
#define LULESH_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lg_domain lg_domain;

enum lg_status {
    LG_OK = 0,
    LG_VOLUME_ERROR = -1,
    LG_QSTOP_ERROR = -2,
    LG_ERR_INVALID = 1,  /* bad argument or unknown name */
    LG_ERR_CUDA = 2,     /* CUDA runtime failure */
    LG_ERR_NOMEM = 3,    /* device or host allocation failed */
    LG_ERR_STATE = 4     /* handle is in an error state from an earlier call */
};

enum lg_precision {
    LG_FP64 = 0,  /* every operation in IEEE double, no FMA contraction */
    LG_FP64_FMA = 1, /* FP64 with fused multiply-add contraction */
    LG_MIXED = 2  /* FP32 stress/hourglass/kinematics/Q, FP64 state, EOS and dt */
};

enum lg_dtype { LG_F64 = 0, LG_I32 = 1 };

/* Command-line options of the reference (lulesh.h:599-609, defaults
 * lulesh.cc:2682-2690) plus the device-path choices. */
typedef struct lg_opts {
    int nx;        /* -s  edge elements (default 30) */
    int numReg;    /* -r  regions (default 11) */
    int balance;   /* -b  region balance (default 1) */
    int cost;      /* -c  extra EOS cost (default 1) */
    int its;       /* -i  cycle limit (default 9999999) */
    int precision; /* enum lg_precision (default LG_FP64) */
    double hgcoef; /* hourglass coefficient, reference constant 3.0 (lulesh-init.cc:25) */
    double einit_factor; /* factor on the deposited origin energy (default 1.0) */
    int device;    /* CUDA device ordinal (default 0) */
} lg_opts;

/* Fill *opts with the reference defaults. */
void lg_default_opts(lg_opts *opts);

/* Build the Sedov problem exactly as Domain::Domain (lulesh-init.cc:16-194)
 * on the host and upload it.  *out receives the handle. */
int lg_create(const lg_opts *opts, lg_domain **out);

void lg_destroy(lg_domain *d);

/* Run at most ncycles iterations of the reference main loop
 * (lulesh.cc:2745-2757): while (time < stoptime && cycle < its)
 * { TimeIncrement; LagrangeLeapFrog; }.  Blocks until done.  Returns the
 * status of the run (0, -1 or -2, or an API error). */
int lg_step(lg_domain *d, int ncycles);

/* lg_step until time >= stoptime or cycle >= its. */
int lg_run(lg_domain *d);

/* Same as lg_step, and reports the device time of the cycles in *ms (CUDA
 * events on the handle's stream). */
int lg_step_timed(lg_domain *d, int ncycles, double *ms);

/* One piece of the cycle, for phase-level checks (same numbering as the
 * oracle): 0 TimeIncrement, 1 LagrangeNodal, 2 LagrangeElements,
 * 3 CalcTimeConstraintsForElems (lulesh.cc:166, 1224, 2432, 2577). */
int lg_phase(lg_domain *d, int phase);

/* Field access by Domain accessor name (lulesh.h:263-367).  Double fields:
 * x y z xd yd zd xdd ydd zdd fx fy fz nodalMass e p q ql qq v volo vnew delv
 * vdov arealg ss elemMass delx_xi delx_eta delx_zeta delv_xi delv_eta
 * delv_zeta.  Integer fields: nodelist lxim lxip letam letap lzetam lzetap
 * elemBC regNumList regElemSize symmX symmY symmZ nodeElemStart
 * nodeElemCornerList.  n is the element count of dst/src and must equal the
 * field length.  Setting nodelist rebuilds the corner list; setting
 * regNumList rebuilds the region sets. */
int lg_field_info(lg_domain *d, const char *name, size_t *count, int *dtype);
int lg_get_field(lg_domain *d, const char *name, void *dst, size_t n);
int lg_set_field(lg_domain *d, const char *name, const void *src, size_t n);

/* Scalars (lulesh.h:377-429): time deltatime dtcourant dthydro stoptime
 * dtmax dtfixed deltatimemultlb deltatimemultub hgcoef cycle its numElem
 * numNode numReg sizeX cost status launches.  launches counts the kernels
 * this handle has queued.  Constants are read-only except hgcoef. */
int lg_get_scalar(lg_domain *d, const char *name, double *value);
int lg_set_scalar(lg_domain *d, const char *name, double value);

/* EOS repetition count of region r (lulesh.cc:2390-2400). */
int lg_region_rep(lg_domain *d, int r, int *rep);

/* Write the reference end-of-run report (lulesh-util.cc:175-230) for the
 * current state into buf (NUL-terminated, truncated to buflen). */
int lg_report(lg_domain *d, double elapsed_seconds, char *buf, size_t buflen);

/* Origin energy and plane-0 symmetry deltas (lulesh-util.cc:197-212),
 * computed on the device: out[0]=e(0), out[1]=MaxAbsDiff,
 * out[2]=TotalAbsDiff, out[3]=MaxRelDiff. */
int lg_verify(lg_domain *d, double out[4]);

/* Per-kernel device time of ncycles cycles (one event pair per launch),
 * without CUDA graphs: ms[i] is the summed time of kernel i and names[i] its
 * name, for i < *nkernels (capacity on input, count on output). */
int lg_profile(lg_domain *d, int ncycles, double *ms, const char **names, int *nkernels);

/* Restore the state built by lg_create (all fields, time-step state and
 * cycle count), so a problem can be rerun without rebuilding it.  Fields set
 * with lg_set_field are not part of that state and are overwritten. */
int lg_reset(lg_domain *d);

/* Issue-rate microbenchmark of one arithmetic pipe on the current device:
 * op 0 = fused multiply-add, 1 = add, 2 = multiply; fp32 != 0 selects FP32,
 * else FP64.  *ginst_per_s receives thread-instructions per second / 1e9.
 * The FP64 leap-frog path is bound by this rate, not by HBM bandwidth. */
int lg_measure_pipe(int op, int fp32, double *ginst_per_s);

/* ---------------------------------------------------------------------------
 * Frozen time steps and the adjoint.  No counterpart in the reference, whose
 * time step always comes from TimeIncrement (lulesh.cc:166-222).
 * ------------------------------------------------------------------------- */

/* Record the time step of every following cycle: cycle c (0-based count of
 * completed cycles when it starts) stores its dt at index c < capacity.
 * capacity 0 stops recording.  lg_dt_get copies the first n entries. */
int lg_dt_record(lg_domain *d, int capacity);
int lg_dt_get(lg_domain *d, double *out, int n);

/* Freeze the time steps: cycle c uses dts[c] (c < n) instead of
 * TimeIncrement's selection.  n = 0 unfreezes.  Survives lg_reset. */
int lg_dt_freeze(lg_domain *d, const double *dts, int n);

/* Reverse-mode gradient of J = sum over elements i with mask[i] != 0 of
 * e_i * volo_i after ncycles cycles (the total internal energy of the
 * masked elements), with respect to the energy field e of the current state
 * (dJ_de0, numElem entries) and the hourglass coefficient (*dJ_dhgcoef).
 * The time steps must be frozen for these cycles (lg_dt_freeze).  Runs the
 * forward cycles with a checkpoint every ckpt_k cycles, recomputes each
 * segment and sweeps it backwards; leaves the handle in the final state and
 * returns *J.  Non-smooth operations: the physical clamps and switches
 * (emin, pmin, eosvmin/eosvmax, the monotonic limiter, vdov > 0, delvc > 0,
 * the sound-speed floors) contribute the derivative of the branch taken; the
 * noise cut-offs (u_cut, p_cut, e_cut, q_cut, v_cut) pass it through.
 * FP64 paths only (LG_FP64, LG_FP64_FMA). */
int lg_adjoint(lg_domain *d, int ncycles, int ckpt_k, const unsigned char *mask, double *J,
               double *dJ_de0, double *dJ_dhgcoef);

/* The general reverse-mode product of the same cycles: given the adjoint of
 * the final state, field by field -- seed[f] for f in x y z xd yd zd
 * (numNode values each) then e p q v ss (numElem each), NULL for a zero
 * seed -- returns the adjoint of the current (initial) state in grad[f]
 * (NULL: not wanted) and dJ/dhgcoef.  For an objective J(final state), seed
 * with dJ/d(final fields).  lg_adjoint is the seed e = mask * volo.  Same
 * frozen-step and precision conditions; leaves the handle in the final
 * state. */
int lg_adjoint_vjp(lg_domain *d, int ncycles, int ckpt_k, const double *const seed[11],
                   double *const grad[11], double *dJ_dhgcoef);

/* ---------------------------------------------------------------------------
 * Ensembles: many independent problems advanced together.  No counterpart in
 * the reference, which runs one problem per process; each member behaves as
 * an lg_create problem with its own options (time step, stop test, cycle
 * count, hourglass coefficient, deposited energy, regions), while every phase
 * of the cycle is one launch over all members.
 * ------------------------------------------------------------------------- */
typedef struct lg_ensemble lg_ensemble;

/* The ensemble study's problem set: nprob option sets drawn from seed with
 * splitmix64 -- nx uniform in 16..64, einit_factor log-uniform in [0.5, 2],
 * hgcoef uniform in [1, 3], numReg uniform in 4..16, balance 1, cost 1,
 * its 300, precision LG_FP64, device 0. */
int lg_ensemble_sample(int nprob, unsigned long long seed, lg_opts *out);

/* Build nprob problems (opts[i] each; precision and device from opts[0]). */
int lg_ensemble_create(int nprob, const lg_opts *opts, lg_ensemble **out);
void lg_ensemble_destroy(lg_ensemble *en);

/* Up to ncycles cycles of every member (each with its own loop test).
 * Returns 0, or the status of the first member in error; per-member status
 * through lg_ensemble_get_scalar(..., "status"). */
int lg_ensemble_step(lg_ensemble *en, int ncycles);
int lg_ensemble_step_timed(lg_ensemble *en, int ncycles, double *ms);

/* Restore every member's set-up state. */
int lg_ensemble_reset(lg_ensemble *en);

/* Total elements and nodes over all members, and kernels queued so far. */
int lg_ensemble_info(lg_ensemble *en, long long *total_elems, long long *total_nodes,
                     long long *launches);

/* Member prob's fields (double accessor fields; nodelist, regNumList, elemBC)
 * and scalars (time deltatime dtcourant dthydro cycle status numElem numNode
 * nx numReg hgcoef einit_factor its). */
int lg_ensemble_get_field(lg_ensemble *en, int prob, const char *name, void *dst, size_t n);
/* Replace member prob's double accessor field `name` (n values from host
 * memory), e.g. the initial energies of a study; nodalMass also updates the
 * mixed path's reciprocal.  Integer topology is fixed at creation. */
int lg_ensemble_set_field(lg_ensemble *en, int prob, const char *name, const void *src, size_t n);
int lg_ensemble_get_scalar(lg_ensemble *en, int prob, const char *name, double *value);

/* Times every block size (64, 128, 256) and grid shape (one pass over the
 * members with resident blocks, or one thread per item) of each kernel for
 * ncycles cycles on this ensemble, keeps the fastest, and restores the
 * set-up state.  block_sizes[4] / persistent[4] receive the choice (either
 * may be NULL). */
int lg_ensemble_autotune(lg_ensemble *en, int ncycles, int *block_sizes, int *persistent);

/* ---------------------------------------------------------------------------
 * Halo exchange of a block decomposition.  The reference runs one Domain per
 * MPI rank on a tp x tp x tp grid of cubes of nx elements (InitMeshDecomp,
 * lulesh-init.cc:676-738; rank = col + row*tp + plane*tp^2) and exchanges
 * boundary values with up to 26 neighbours (6 faces, 12 edges, 8 corners):
 *   LG_HALO_SBN           CommSend + CommSBN (lulesh-comm.cc:357, 848): node
 *                         fields; each neighbour's values at the shared nodes
 *                         are added, message after message (forces,
 *                         lulesh.cc:1109-1133; nodal mass, lulesh.cc:2723-2729)
 *   LG_HALO_SYNC_POS_VEL  CommSend + CommSyncPosVel (357, 1261): node fields;
 *                         shared nodes take the higher-ranked neighbour's
 *                         values (lulesh.cc:2621-2642)
 *   LG_HALO_MONOQ         CommSend + CommMonoQ (357, 1684): element fields of
 *                         the six face neighbours' boundary layers, copied into
 *                         ghost elements after numElem (lulesh.cc:1963-1985)
 * A plan lists one rank's messages in the reference's order and buffer layout
 * (CommRecv/CommSend, lulesh-comm.cc:59-845: faces, edges, corners at
 * pmsg*maxPlaneComm + emsg*maxEdgeComm + cmsg*16 doubles, the fields of a
 * message one after another), so send and receive buffers are
 * interchangeable with the reference's commDataSend / commDataRecv.  Packing
 * and unpacking run on the GPU; moving each message to its peer's receive
 * buffer (MPI, NCCL, peer copies) is the caller's, as MPI_Isend / MPI_Irecv
 * are the reference's.
 * ------------------------------------------------------------------------- */
enum lg_halo_kind { LG_HALO_SBN = 0, LG_HALO_SYNC_POS_VEL = 1, LG_HALO_MONOQ = 2 };

typedef struct lg_halo_plan lg_halo_plan;

typedef struct lg_halo_info {
    size_t buffer_doubles; /* send and receive buffer length: the reference's
                              comBufSize (lulesh-init.cc:358-380) */
    int send_messages, recv_messages;
    int send_values, recv_values; /* values per field, summed over the messages */
    int recv_targets;   /* distinct lattice points (or ghost slots) written */
    int ghost_elems;    /* LG_HALO_MONOQ: ghost elements after numElem */
    int field_length;   /* entries each field array must hold: nodes (nx+1)^3,
                           or numElem + ghost_elems */
} lg_halo_info;

/* The plan of rank `rank` of a tp^3 decomposition of cubes of nx elements
 * for nfields fields (1..6; the reference sends 3 forces, 1 nodal mass, 6
 * positions and velocities, 3 velocity gradients).  Host-only: the plan's
 * device copy is made on the current device by its first pack or unpack. */
int lg_halo_plan_create(int kind, int nx, int tp, int rank, int nfields, lg_halo_plan **out);
void lg_halo_plan_destroy(lg_halo_plan *plan);
int lg_halo_plan_info(const lg_halo_plan *plan, lg_halo_info *info);

/* Message m (in order) of direction dir (0 send, 1 receive): the peer rank,
 * the values per field, and the message's offset in the buffer (doubles);
 * the message occupies nfields * count doubles from there. */
int lg_halo_plan_message(const lg_halo_plan *plan, int dir, int m, int *peer, int *count,
                         size_t *offset);

/* The plan's value list (n = send_values or recv_values): for dir 0, the
 * lattice index packed at buffer position bufpos[k] (field f at bufpos[k] +
 * f*stride[k]); for dir 1, the lattice index (or ghost slot) each received
 * value goes to, grouped by target in the order the values are applied.
 * Any output may be NULL. */
int lg_halo_plan_entries(const lg_halo_plan *plan, int dir, int *index, int *bufpos, int *stride,
                         size_t n);

/* Pack fields[0..nfields) (device arrays of field_length doubles; fields is
 * a host array of device pointers) into send_buf (device, buffer_doubles),
 * on stream (a cudaStream_t or NULL).  Asynchronous. */
int lg_halo_pack(lg_halo_plan *plan, double *const *fields, double *send_buf, void *stream);

/* Apply the received messages in recv_buf (device, buffer_doubles) to the
 * fields in the reference's message order: added for LG_HALO_SBN, copied
 * otherwise.  Deterministic (no atomics).  Asynchronous on stream. */
int lg_halo_unpack(lg_halo_plan *plan, double *const *fields, const double *recv_buf,
                   void *stream);

/* Nodal forces with no device allocation, for callers that own all device
 * memory themselves.  No counterpart in the reference: it exists for codes
 * that cannot let a library allocate behind their back -- hydro codes that
 * carve every device buffer from one pool sized at start-up, processes under
 * a hard per-GPU memory budget, and time-step loops that must not pay for the
 * device-wide synchronisation of cudaFree or an allocation failing mid-run.
 *
 * Computes fx, fy, fz of CalcForceForNodes (stress integration, FB hourglass
 * forces and the ordered per-node corner gather; lulesh.cc:1104-1135) from
 * the caller's device arrays: nodelist (8*numElem, element-major as
 * Domain::nodelist), nodeElemStart (numNode+1) and nodeElemCornerList
 * (8*numElem) as built by lulesh-init.cc:272-337, node fields x..zd
 * (numNode), element fields p q v volo ss elemMass (numElem), hgcoef; writes
 * fx, fy, fz (numNode).  stream is a cudaStream_t or NULL; the call waits for
 * its work to finish and returns 0, -1 (VolumeError: a non-positive volume)
 * or an LG_ERR_* code.
 *
 * It calls no cudaMalloc, cudaFree or allocating routine.  Its per-corner
 * scratch is one fixed static device array of 48 doubles per element for at
 * most 32768 elements (about 12.6 MB, held on every GPU where the call has
 * run until the process exits); larger meshes are rejected with
 * LG_ERR_INVALID.  Every call copies its status word back and synchronises
 * the stream, so it blocks the host until its kernels have finished and no
 * call can be captured into a CUDA graph.  A non-sticky CUDA error left pending by
 * the caller's earlier work is cleared on entry, so that a failure reported
 * here is this call's own.  All calls share the array: calls whose work
 * overlaps on one GPU race and must be serialised by the caller. */
int lg_calc_force_for_nodes_noalloc(int numElem, int numNode, const int *nodelist,
                                    const int *nodeElemStart, const int *nodeElemCornerList,
                                    const double *x, const double *y, const double *z,
                                    const double *xd, const double *yd, const double *zd,
                                    const double *p, const double *q, const double *v,
                                    const double *volo, const double *ss,
                                    const double *elemMass, double hgcoef, double *fx,
                                    double *fy, double *fz, void *stream);

/* Human-readable description of the most recent error on this thread. */
const char *lg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
