/*
 * lulesh_oracle.h -- CPU oracle for the LULESH 2.x Lagrange leap-frog path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C restatement of the
 * reference algorithm (LLNL LULESH 2.x, lulesh.cc / lulesh-init.cc) used as
 * the parity checker for the GPU path and as the timed CPU baseline.  The
 * product (lulesh_gb300) never links, loads or calls it.
 *
 * Semantics follow the reference's OpenMP build run with two or more threads:
 * element forces are written per element corner and gathered per node in
 * ascending element order (lulesh.cc:514-586, 737-990), which makes the result
 * independent of the thread count.  Errors that make the reference call
 * exit() are returned as status codes instead: -1 VolumeError, -2 QStopError
 * (lulesh.h:42).
 */
#ifndef LULESH_ORACLE_H
#define LULESH_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_domain orc_domain;

/* Build the Sedov problem exactly as Domain::Domain (lulesh-init.cc:16-194)
 * for one rank: nx elements per edge, numReg regions, balance, cost. */
orc_domain *orc_create(int nx, int numReg, int balance, int cost);

/* Same, with the two problem parameters the ensemble and the adjoint vary:
 * hgcoef (reference constant 3.0, lulesh-init.cc:25) and a factor applied to
 * the deposited origin energy (lulesh-init.cc:183-192; the initial time step
 * is computed from the scaled energy). */
orc_domain *orc_create_ex(int nx, int numReg, int balance, int cost,
                          double hgcoef, double einit_factor);

void orc_destroy(orc_domain *d);

/* Run at most ncycles iterations of the reference main loop
 * (lulesh.cc:2745-2757): while (time < stoptime && cycle < its) {
 * TimeIncrement; LagrangeLeapFrog; }.  Returns 0, -1 or -2. */
int orc_step(orc_domain *d, int ncycles);

/* One piece of the cycle, for phase-level parity:
 *   0 TimeIncrement        (lulesh.cc:166)
 *   1 LagrangeNodal        (lulesh.cc:1224)
 *   2 LagrangeElements     (lulesh.cc:2432)
 *   3 CalcTimeConstraints  (lulesh.cc:2577)                                */
int orc_phase(orc_domain *d, int phase);

/* Field access by Domain accessor name (lulesh.h:263-367).  Returns a pointer
 * into the oracle's storage and its length, or NULL for an unknown name. */
double *orc_field_f64(orc_domain *d, const char *name, size_t *n);
int    *orc_field_i32(orc_domain *d, const char *name, size_t *n);

/* Scalars: time, deltatime, dtcourant, dthydro, stoptime, dtmax, dtfixed,
 * deltatimemultlb, deltatimemultub, hgcoef, cycle, numElem, numNode, numReg.
 * Unknown names return NaN. */
double orc_get_scalar(orc_domain *d, const char *name);
int    orc_set_scalar(orc_domain *d, const char *name, double value);

/* Number of EOS repetitions for region r (lulesh.cc:2387-2401). */
int orc_region_rep(orc_domain *d, int r);

/* Frozen time steps: cycle c (0-based) uses dts[c] (c < n) instead of
 * TimeIncrement's selection; n = 0 unfreezes.  Recording: every following
 * cycle stores its step at index c < capacity (orc_dt_recorded). */
int orc_dt_freeze(orc_domain *d, const double *dts, int n);
int orc_dt_record(orc_domain *d, int capacity);
const double *orc_dt_recorded(orc_domain *d);

/* Decision tape, for finite differences along one branch of the cycle
 * (compiled into build/liblulesh_oracle_tape.so; the other builds return
 * -1).  orc_tape_record: the next ncycles cycles of orc_step store the
 * outcome of every branch that changes a state value (limiter min/max,
 * vdov and delv*delx switches, eosvmin/eosvmax, delvc > 0, emin, pmin,
 * sound-speed floors) and the offset of every noise cut-off that fired
 * (u_cut, p_cut, e_cut, q_cut, v_cut).  orc_tape_replay: the next cycles of
 * d take src's recorded outcomes and add src's offsets where a cut-off
 * fired -- a smooth map of d's state that equals the plain cycles bitwise
 * on src's trajectory (src must outlive d's use).  orc_tape_stop: plain
 * cycles again. */
int orc_tape_record(orc_domain *d, int ncycles);
int orc_tape_replay(orc_domain *d, const orc_domain *src);
int orc_tape_stop(orc_domain *d);

/* Rebuild the corner-per-node list from the current nodelist
 * (lulesh-init.cc:272-337).  Call after replacing nodelist. */
void orc_rebuild_corner_list(orc_domain *d);

#ifdef __cplusplus
}
#endif

#endif
