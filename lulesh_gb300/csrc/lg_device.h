// lg_device.h -- device-resident Domain: layout shared by host and kernels.
//
// Every field is a separate structure-of-arrays buffer in HBM, 256-byte
// aligned, carved from one allocation.  Kernel-side derived layouts:
//   nodelistT[j*E + e]  element-to-node map transposed to corner-major, so the
//                       eight corner loads of a warp are each coalesced;
//   corner[c][j*E + e]  per-corner forces, c = 0..2 stress x/y/z and
//                       c = 3..5 hourglass x/y/z, written coalesced by the
//                       element kernel and gathered per node (FP32 values in
//                       the same buffer for the mixed path, which also keeps
//                       the monotonic-Q gradients as FP32 in the delx_* and
//                       delv_* buffers);
//   symm[n]             bit 0/1/2 set when node n is in symmX/Y/Z;
//   regPerm[t], regRep[t]  region-sorted element order and the EOS
//                       repetition count of position t (regions with the
//                       most repetitions first, ascending element ids inside
//                       each region, the order of regElemlist).
#pragma once

#include <cstdint>

namespace lg {

// element face boundary-condition bits (lulesh.h:59-87)
enum : int {
    XI_M = 0x00007, XI_M_SYMM = 0x00001, XI_M_FREE = 0x00002, XI_M_COMM = 0x00004,
    XI_P = 0x00038, XI_P_SYMM = 0x00008, XI_P_FREE = 0x00010, XI_P_COMM = 0x00020,
    ETA_M = 0x001c0, ETA_M_SYMM = 0x00040, ETA_M_FREE = 0x00080, ETA_M_COMM = 0x00100,
    ETA_P = 0x00e00, ETA_P_SYMM = 0x00200, ETA_P_FREE = 0x00400, ETA_P_COMM = 0x00800,
    ZETA_M = 0x07000, ZETA_M_SYMM = 0x01000, ZETA_M_FREE = 0x02000, ZETA_M_COMM = 0x04000,
    ZETA_P = 0x38000, ZETA_P_SYMM = 0x08000, ZETA_P_FREE = 0x10000, ZETA_P_COMM = 0x20000,
};


struct Ctl {
    double time, deltatime, dtcourant, dthydro;
    double stoptime, dtmax, dtfixed, dtmultlb, dtmultub;
    int cycle;
    int cycle_limit;   // min(its, cycle at which the current lg_step stops)
    int active;        // 1 while the current cycle is running
    int status;        // 0, -1 (VolumeError) or -2 (QStopError)
    int err_qstop;     // set by the material kernel, merged by its last block
    int err_matvol;
    unsigned int blocks_done;
    int pad;
    // frozen time steps: when non-null, cycle c (0-based) uses dt_frozen[c]
    // (c < dt_frozen_len) instead of TimeIncrement's selection; dt_record[c]
    // receives every cycle's time step when non-null (c < dt_record_len)
    const double *dt_frozen;
    double *dt_record;
    int dt_frozen_len;
    int dt_record_len;
    // the self-check's origin energy, MaxAbsDiff, TotalAbsDiff, MaxRelDiff
    double verify[4];
};

struct Params {
    double e_cut, p_cut, q_cut, v_cut, u_cut, hgcoef, ss4o3, qstop, monoq_max_slope;
    double monoq_limiter_mult, qlc_monoq, qqc_monoq, qqc, eosvmax, eosvmin, pmin, emin;
    double dvovmax, refdens;
};

struct DevState {
    int E, N, nx, numReg;
    // node fields
    double *x, *y, *z, *xd, *yd, *zd, *xdd, *ydd, *zdd, *fx, *fy, *fz, *nodalMass;
    double *invMass;  // RN(1 / nodalMass): the nodal accelerations of every path
    uint8_t *symm;
    int *nodeElemStart, *nodeElemCornerList;
    // element fields
    int *nodelist, *nodelistT, *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elemBC;
    double *e, *p, *q, *ql, *qq, *v, *volo, *vnew, *delv, *vdov, *arealg, *ss, *elemMass;
    double *delx_xi, *delx_eta, *delx_zeta, *delv_xi, *delv_eta, *delv_zeta;
    int *regNumList, *regPerm, *regRep;
    // work items of the material phase: regPerm / regRep hold nItems entries
    // (one per element in region order, regRep its repetitions; or, when the
    // phase runs split, repetition items: an element and a share of its EOS
    // repetitions, regRep > 0 for its writer and < 0 for the others).
    // Ensembles: nItems = E.
    int nItems;
    // 1: the material phase runs split (small meshes; lg::build_material_items):
    // k_material_inputs over the elements, k_material_eos over the nItems
    // repetition items, k_material_finish over the elements, staging the
    // EOS inputs and results in the per-corner scratch (free in that phase)
    int matSplit;
    // block sizes of the single-problem element kernels (k_forces,
    // k_kinematics) and of k_nodes: 32, 64 or 128 (0 means 128), chosen at
    // creation so that small meshes spread evenly over the SMs
    int bs_elem, bs_node;
    // per-corner force scratch, 6 * 8 * E doubles
    double *corner;
    // per-block minima of the time-constraint reduction
    double *dt_partial;
    int dt_blocks;
    Ctl *ctl;  // nprob control blocks
    Params prm;
    // batched problems (nprob > 1): owner of every element and node, each
    // problem's hourglass coefficient, its Courant/hydro minimum slots (bit
    // patterns of positive doubles) and the grid-wide block counter
    int nprob;
    uint16_t *elemProb, *nodeProb;
    double *hgcoefs;
    unsigned long long *dtSlots;
    unsigned int *gridCounter;
};

}  // namespace lg
