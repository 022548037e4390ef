/*
 * lulesh_oracle.c -- CPU oracle for the LULESH 2.x Lagrange leap-frog path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GPU path and the timed
 * CPU baseline ("port").  Nothing in the product links or calls this file.
 *
 * A plain-C restatement of the reference algorithm.  Every floating-point
 * expression keeps the reference's operand order, because the parity bar is
 * rounding-exact agreement with the reference's OpenMP build compiled with
 * -ffp-contract=off.  Each function names the reference lines it follows
 * (paths relative to the LULESH 2.x source tree).
 *
 * Differences from the reference that do not change results:
 *  - state lives in one C struct of arrays instead of class Domain;
 *  - per-call malloc/free temporaries (lulesh.h:110-123) are allocated once;
 *  - region loops that are element-independent (Q limiter, EOS, time
 *    constraints) run per region exactly as the reference does, but errors
 *    are returned as status codes instead of exit().
 */
#include <limits.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#ifdef ORC_LONG_DOUBLE
/* The extended-precision build (liblulesh_oracle_tape_ld.so, a reference for
 * finite differences only): every double of this file and of its API becomes
 * long double, with the long double forms of the math functions.  Not a
 * parity build: its results differ from the reference's in the last bits of
 * double precision. */
#define sqrt sqrtl
#define cbrt cbrtl
#define fabs fabsl
#define pow powl
#define double long double
#endif
#include "lulesh_oracle.h"

/* element face boundary-condition bits (lulesh.h:59-87) */
#define XI_M 0x00007
#define XI_M_SYMM 0x00001
#define XI_M_FREE 0x00002
#define XI_M_COMM 0x00004
#define XI_P 0x00038
#define XI_P_SYMM 0x00008
#define XI_P_FREE 0x00010
#define XI_P_COMM 0x00020
#define ETA_M 0x001c0
#define ETA_M_SYMM 0x00040
#define ETA_M_FREE 0x00080
#define ETA_M_COMM 0x00100
#define ETA_P 0x00e00
#define ETA_P_SYMM 0x00200
#define ETA_P_FREE 0x00400
#define ETA_P_COMM 0x00800
#define ZETA_M 0x07000
#define ZETA_M_SYMM 0x01000
#define ZETA_M_FREE 0x02000
#define ZETA_M_COMM 0x04000
#define ZETA_P 0x38000
#define ZETA_P_SYMM 0x08000
#define ZETA_P_FREE 0x10000
#define ZETA_P_COMM 0x20000

enum { ORC_OK = 0, ORC_VOLUME_ERROR = -1, ORC_QSTOP_ERROR = -2 };

struct orc_domain {
    int nx, numElem, numNode, numReg, cost, balance, cycle;
    /* node-centred (lulesh.h:460-480) */
    double *x, *y, *z, *xd, *yd, *zd, *xdd, *ydd, *zdd, *fx, *fy, *fz, *nodalMass;
    int *symmX, *symmY, *symmZ;
    int nsymm;
    /* element-centred (lulesh.h:484-531) */
    int *nodelist, *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elemBC;
    double *e, *p, *q, *ql, *qq, *v, *volo, *vnew, *delv, *vdov, *arealg, *ss, *elemMass;
    int *regElemSize, *regNumList, **regElemlist;
    int *nodeElemStart, *nodeElemCornerList;
    /* per-cycle temporaries */
    double *fx_elem, *fy_elem, *fz_elem, *determ, *sig;
    double *dvdx, *dvdy, *dvdz, *x8n, *y8n, *z8n;
    double *dxx, *dyy, *dzz;
    double *delx_xi, *delx_eta, *delx_zeta, *delv_xi, *delv_eta, *delv_zeta;
    double *vnewc;
    /* compressed EOS temporaries, sized to the largest region */
    double *eos_tmp;
    /* constants (lulesh-init.cc:20-38) */
    double e_cut, p_cut, q_cut, v_cut, u_cut, hgcoef, ss4o3, qstop, monoq_max_slope,
        monoq_limiter_mult, qlc_monoq, qqc_monoq, qqc, eosvmax, eosvmin, pmin, emin,
        dvovmax, refdens;
    /* time-step state (lulesh-init.cc:146-156) */
    double dtcourant, dthydro, dtfixed, time, deltatime, deltatimemultlb,
        deltatimemultub, dtmax, stoptime;
    /* frozen time steps (cycle c uses dt_frozen[c]) and recorded ones */
    double *dt_frozen, *dt_record;
    int dt_frozen_len, dt_record_len;
    /* decision tape (ORC_TAPE builds only; NULL otherwise) */
    struct orc_tape_state *tape;
};

#define ALLOC(T, n) ((T *)calloc((size_t)(n) > 0 ? (size_t)(n) : 1, sizeof(T)))

/* ------------------------------------------------------------------------ */
/* decision tape                                                             */
/* ------------------------------------------------------------------------ */
/*
 * Built with -DORC_TAPE only (liblulesh_oracle_tape.so); every other build
 * compiles the TAPE_IF / TAPE_CUT sites below to the plain comparisons of
 * the reference, so its arithmetic is unchanged.
 *
 * Record mode stores, per cycle, the outcome of every branch of the cycle
 * that can change a state value (the monotonic limiter's min/max and its
 * vdov and delv*delx switches, the eosvmin/eosvmax clamps of vnewc and of
 * the EOS, the delvc > 0 switches, the emin and pmin clamps, the sound-speed
 * floors) and, for each noise cut-off that fired (|u| < u_cut, |p| < p_cut,
 * |e| < e_cut, |q| < q_cut, |v - 1| < v_cut), the offset it applied.  Replay
 * mode takes the recorded outcomes instead of evaluating the comparisons and
 * adds the recorded offsets where a cut-off fired.  Replayed cycles are a
 * smooth function of the state (compositions of +, *, / and sqrt), equal to
 * the plain cycles bitwise at the recorded trajectory: central differences
 * of a replay resolve the derivative of the branch the recorded run took,
 * the derivative with clamps and switches held and noise cut-offs passed.
 * The Courant/hydro constraints (which only choose time steps) and the error
 * checks are not taped.
 */
enum {
    TB_PHI = 0,        /* 3 directions x 4 limiter comparisons: bits 0-11 */
    TB_VDOV = 12,      /* vdov > 0 */
    TB_DELVX = 13,     /* delv*delx > 0, 3 directions: bits 13-15 */
    TB_VC_MIN = 16, TB_VC_MAX = 17,          /* vnewc clamps */
    TB_EOS_VMIN = 18, TB_EOS_VMAX = 19,      /* EOS compression switches */
    TB_E1_EMIN = 20,
    TB_P_HALF = 21,    /* p_cut, eosvmax, pmin of the half-step pressure: 21-23 */
    TB_Q1_COMP = 24, TB_Q1_FLOOR = 25, TB_E3_CUT = 26, TB_E3_EMIN = 27,
    TB_P_NEW1 = 28,    /* 28-30 */
    TB_QT_COMP = 31, TB_QT_FLOOR = 32, TB_E4_CUT = 33, TB_E4_EMIN = 34,
    TB_P_NEW2 = 35,    /* 35-37 */
    TB_QF_COMP = 38, TB_QF_FLOOR = 39, TB_QF_CUT = 40, TB_SS_FLOOR = 41, TB_V_CUT = 42,
    TB_NODE_U = 0      /* node bits: u_cut of xd, yd, zd: 0-2 */
};
/* slots of the cut-off offsets: 0-6 element sites, 7-9 node sites */
enum {
    TS_P_HALF, TS_E3, TS_P_NEW1, TS_E4, TS_P_NEW2, TS_QF, TS_V, TS_U, TS_NSLOT = TS_U + 3
};

#ifdef ORC_TAPE
struct orc_tape_data {
    int ncyc, E, N;
    uint64_t *eb;      /* ncyc x E decision bits */
    uint8_t *nb;       /* ncyc x N decision bits */
    size_t *off_start; /* ncyc + 1: offsets of cycle c in [off_start[c], off_start[c+1]) */
    int *off_slot, *off_idx;
    double *off_val;
    size_t off_len, off_cap;
};

struct orc_tape_state {
    int mode; /* 1 record, 2 replay */
    int next; /* tape cycle of the next orc_step cycle */
    int cyc;  /* tape cycle running, -1 outside */
    struct orc_tape_data *data;
    int owns;
    double *dense[TS_NSLOT];
};

static inline int tape_bit_e(const orc_domain *d, int bit, int idx, int cond)
{
    const struct orc_tape_state *t = d->tape;
    if (!t || t->cyc < 0) return cond;
    uint64_t *w = &t->data->eb[(size_t)t->cyc * t->data->E + idx];
    if (t->mode == 1) {
        if (cond) *w |= (uint64_t)1 << bit;
        return cond;
    }
    return (int)((*w >> bit) & 1u);
}

static inline int tape_bit_n(const orc_domain *d, int bit, int idx, int cond)
{
    const struct orc_tape_state *t = d->tape;
    if (!t || t->cyc < 0) return cond;
    uint8_t *w = &t->data->nb[(size_t)t->cyc * t->data->N + idx];
    if (t->mode == 1) {
        if (cond) *w |= (uint8_t)(1u << bit);
        return cond;
    }
    return (int)((*w >> bit) & 1u);
}

/* a noise cut-off "x = target when cond": record the offset, replay it */
static inline double tape_cut(const orc_domain *d, int node, int bit, int slot, int idx,
                              double x, int cond, double target)
{
    const struct orc_tape_state *t = d->tape;
    if (!t || t->cyc < 0) return cond ? target : x;
    const int fired = node ? tape_bit_n(d, bit, idx, cond) : tape_bit_e(d, bit, idx, cond);
    if (!fired) return x;
    if (t->mode == 1) {
        t->dense[slot][idx] = target - x;
        return target;
    }
    return x + t->dense[slot][idx];
}

#define TAPE_IF(bit, idx, cond) tape_bit_e(d, (bit), (idx), (cond))
#define TAPE_CUT(bit, slot, idx, x, cond, target) \
    tape_cut(d, 0, (bit), (slot), (idx), (x), (cond), (target))
#define TAPE_CUT_NODE(bit, slot, idx, x, cond, target) \
    tape_cut(d, 1, (bit), (slot), (idx), (x), (cond), (target))

static void tape_free(struct orc_tape_state *t)
{
    if (!t) return;
    if (t->owns && t->data) {
        free(t->data->eb);
        free(t->data->nb);
        free(t->data->off_start);
        free(t->data->off_slot);
        free(t->data->off_idx);
        free(t->data->off_val);
        free(t->data);
    }
    for (int k = 0; k < TS_NSLOT; ++k) free(t->dense[k]);
    free(t);
}

static struct orc_tape_state *tape_new(const orc_domain *d)
{
    struct orc_tape_state *t = (struct orc_tape_state *)calloc(1, sizeof(*t));
    if (!t) return NULL;
    for (int k = 0; k < TS_NSLOT; ++k) {
        const int n = k >= TS_U ? d->numNode : d->numElem;
        t->dense[k] = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
        if (!t->dense[k]) {
            tape_free(t);
            return NULL;
        }
    }
    t->cyc = -1;
    return t;
}

static void tape_begin_cycle(orc_domain *d)
{
    struct orc_tape_state *t = d->tape;
    if (!t) return;
    struct orc_tape_data *D = t->data;
    if (t->next >= D->ncyc) {
        t->cyc = -1;
        return;
    }
    t->cyc = t->next;
    const size_t c = (size_t)t->cyc;
    if (t->mode == 1) {
        memset(D->eb + c * D->E, 0, sizeof(uint64_t) * (size_t)D->E);
        memset(D->nb + c * D->N, 0, (size_t)D->N);
        D->off_start[c] = D->off_len;
    } else {
        for (size_t k = D->off_start[c]; k < D->off_start[c + 1]; ++k)
            t->dense[D->off_slot[k]][D->off_idx[k]] = D->off_val[k];
    }
}

static int tape_push(struct orc_tape_data *D, int slot, int idx, double val)
{
    if (D->off_len == D->off_cap) {
        const size_t cap = D->off_cap ? 2 * D->off_cap : 4096;
        int *s2 = (int *)realloc(D->off_slot, cap * sizeof(int));
        if (s2) D->off_slot = s2;
        int *i2 = (int *)realloc(D->off_idx, cap * sizeof(int));
        if (i2) D->off_idx = i2;
        double *v2 = (double *)realloc(D->off_val, cap * sizeof(double));
        if (v2) D->off_val = v2;
        if (!s2 || !i2 || !v2) return -1;
        D->off_cap = cap;
    }
    D->off_slot[D->off_len] = slot;
    D->off_idx[D->off_len] = idx;
    D->off_val[D->off_len] = val;
    ++D->off_len;
    return 0;
}

static void tape_end_cycle(orc_domain *d)
{
    struct orc_tape_state *t = d->tape;
    if (!t || t->cyc < 0) return;
    struct orc_tape_data *D = t->data;
    const size_t c = (size_t)t->cyc;
    if (t->mode == 1) {
        static const int ebit[TS_U] = {TB_P_HALF, TB_E3_CUT, TB_P_NEW1, TB_E4_CUT,
                                       TB_P_NEW2, TB_QF_CUT, TB_V_CUT};
        const uint64_t *eb = D->eb + c * D->E;
        const uint8_t *nb = D->nb + c * D->N;
        for (int k = 0; k < TS_U; ++k)
            for (int i = 0; i < D->E; ++i)
                if (((eb[i] >> ebit[k]) & 1u) && t->dense[k][i] != 0.0)
                    tape_push(D, k, i, t->dense[k][i]);
        for (int k = 0; k < 3; ++k)
            for (int i = 0; i < D->N; ++i)
                if (((nb[i] >> (TB_NODE_U + k)) & 1u) && t->dense[TS_U + k][i] != 0.0)
                    tape_push(D, TS_U + k, i, t->dense[TS_U + k][i]);
        D->off_start[c + 1] = D->off_len;
    } else {
        for (size_t k = D->off_start[c]; k < D->off_start[c + 1]; ++k)
            t->dense[D->off_slot[k]][D->off_idx[k]] = 0.0;
    }
    t->cyc = -1;
    ++t->next;
}

int orc_tape_record(orc_domain *d, int ncycles)
{
    tape_free(d->tape);
    d->tape = NULL;
    if (ncycles <= 0) return 0;
    struct orc_tape_state *t = tape_new(d);
    struct orc_tape_data *D = (struct orc_tape_data *)calloc(1, sizeof(*D));
    if (!t || !D) {
        free(D);
        tape_free(t);
        return -1;
    }
    t->data = D;
    t->owns = 1;
    t->mode = 1;
    D->ncyc = ncycles;
    D->E = d->numElem;
    D->N = d->numNode;
    D->eb = (uint64_t *)calloc((size_t)ncycles * (size_t)(D->E > 0 ? D->E : 1), sizeof(uint64_t));
    D->nb = (uint8_t *)calloc((size_t)ncycles * (size_t)(D->N > 0 ? D->N : 1), 1);
    D->off_start = (size_t *)calloc((size_t)ncycles + 1, sizeof(size_t));
    if (!D->eb || !D->nb || !D->off_start) {
        tape_free(t);
        return -1;
    }
    d->tape = t;
    return 0;
}

int orc_tape_replay(orc_domain *d, const orc_domain *src)
{
    tape_free(d->tape);
    d->tape = NULL;
    if (!src || !src->tape || src->tape->mode != 1) return -1;
    if (src->numElem != d->numElem || src->numNode != d->numNode) return -1;
    struct orc_tape_state *t = tape_new(d);
    if (!t) return -1;
    t->data = src->tape->data;
    t->owns = 0;
    t->mode = 2;
    d->tape = t;
    return 0;
}

int orc_tape_stop(orc_domain *d)
{
    tape_free(d->tape);
    d->tape = NULL;
    return 0;
}
#else
struct orc_tape_state;
#define TAPE_IF(bit, idx, cond) (cond)
#define TAPE_CUT(bit, slot, idx, x, cond, target) ((cond) ? (target) : (x))
#define TAPE_CUT_NODE(bit, slot, idx, x, cond, target) ((cond) ? (target) : (x))
static inline void tape_free(struct orc_tape_state *t) { (void)t; }
static inline void tape_begin_cycle(orc_domain *d) { (void)d; }
static inline void tape_end_cycle(orc_domain *d) { (void)d; }
int orc_tape_record(orc_domain *d, int ncycles) { (void)d; (void)ncycles; return -1; }
int orc_tape_replay(orc_domain *d, const orc_domain *src) { (void)d; (void)src; return -1; }
int orc_tape_stop(orc_domain *d) { (void)d; return -1; }
#endif

/* ------------------------------------------------------------------------ */
/* setup: Domain::Domain and helpers (lulesh-init.cc)                        */
/* ------------------------------------------------------------------------ */

/* BuildMesh, lulesh-init.cc:218-267 (single rank: col/row/plane loc 0, tp 1) */
static void build_mesh(orc_domain *d)
{
    const int nx = d->nx, edgeNodes = nx + 1, edgeElems = nx;
    int nidx = 0;
    double tz = 1.125 * (double)(0) / (double)(nx);
    for (int plane = 0; plane < edgeNodes; ++plane) {
        double ty = 1.125 * (double)(0) / (double)(nx);
        for (int row = 0; row < edgeNodes; ++row) {
            double tx = 1.125 * (double)(0) / (double)(nx);
            for (int col = 0; col < edgeNodes; ++col) {
                d->x[nidx] = tx;
                d->y[nidx] = ty;
                d->z[nidx] = tz;
                ++nidx;
                tx = 1.125 * (double)(col + 1) / (double)(nx);
            }
            ty = 1.125 * (double)(row + 1) / (double)(nx);
        }
        tz = 1.125 * (double)(plane + 1) / (double)(nx);
    }
    int zidx = 0;
    nidx = 0;
    for (int plane = 0; plane < edgeElems; ++plane) {
        for (int row = 0; row < edgeElems; ++row) {
            for (int col = 0; col < edgeElems; ++col) {
                int *ln = &d->nodelist[8 * zidx];
                ln[0] = nidx;
                ln[1] = nidx + 1;
                ln[2] = nidx + edgeNodes + 1;
                ln[3] = nidx + edgeNodes;
                ln[4] = nidx + edgeNodes * edgeNodes;
                ln[5] = nidx + edgeNodes * edgeNodes + 1;
                ln[6] = nidx + edgeNodes * edgeNodes + edgeNodes + 1;
                ln[7] = nidx + edgeNodes * edgeNodes + edgeNodes;
                ++zidx;
                ++nidx;
            }
            ++nidx;
        }
        nidx += edgeNodes;
    }
}

/* SetupThreadSupportStructures, lulesh-init.cc:272-337 */
void orc_rebuild_corner_list(orc_domain *d)
{
    int *count = ALLOC(int, d->numNode);
    for (int i = 0; i < d->numElem; ++i)
        for (int j = 0; j < 8; ++j) ++count[d->nodelist[8 * i + j]];
    free(d->nodeElemStart);
    free(d->nodeElemCornerList);
    d->nodeElemStart = ALLOC(int, d->numNode + 1);
    d->nodeElemStart[0] = 0;
    for (int i = 1; i <= d->numNode; ++i)
        d->nodeElemStart[i] = d->nodeElemStart[i - 1] + count[i - 1];
    d->nodeElemCornerList = ALLOC(int, d->nodeElemStart[d->numNode]);
    memset(count, 0, sizeof(int) * (size_t)d->numNode);
    for (int i = 0; i < d->numElem; ++i) {
        for (int j = 0; j < 8; ++j) {
            int m = d->nodelist[8 * i + j];
            d->nodeElemCornerList[d->nodeElemStart[m] + count[m]] = 8 * i + j;
            ++count[m];
        }
    }
    free(count);
}

/* CreateRegionIndexSets, lulesh-init.cc:401-510 (rank 0: srand(0), no rotation) */
static void create_regions(orc_domain *d, int nr, int balance)
{
    srand(0);
    const int myRank = 0;
    d->numReg = nr;
    d->regElemSize = ALLOC(int, nr);
    d->regElemlist = ALLOC(int *, nr);
    int nextIndex = 0;
    if (nr == 1) {
        while (nextIndex < d->numElem) {
            d->regNumList[nextIndex] = 1;
            nextIndex++;
        }
        d->regElemSize[0] = 0;
    } else {
        int regionNum, regionVar, lastReg = -1, binSize, elements, runto = 0;
        int costDenominator = 0;
        int *regBinEnd = ALLOC(int, nr);
        for (int i = 0; i < nr; ++i) {
            d->regElemSize[i] = 0;
            costDenominator += pow((i + 1), balance);
            regBinEnd[i] = costDenominator;
        }
        while (nextIndex < d->numElem) {
            regionVar = rand() % costDenominator;
            int i = 0;
            while (regionVar >= regBinEnd[i]) i++;
            regionNum = ((i + myRank) % nr) + 1;
            while (regionNum == lastReg) {
                regionVar = rand() % costDenominator;
                i = 0;
                while (regionVar >= regBinEnd[i]) i++;
                regionNum = ((i + myRank) % nr) + 1;
            }
            binSize = rand() % 1000;
            if (binSize < 773)
                elements = rand() % 15 + 1;
            else if (binSize < 937)
                elements = rand() % 16 + 16;
            else if (binSize < 970)
                elements = rand() % 32 + 32;
            else if (binSize < 974)
                elements = rand() % 64 + 64;
            else if (binSize < 978)
                elements = rand() % 128 + 128;
            else if (binSize < 981)
                elements = rand() % 256 + 256;
            else
                elements = rand() % 1537 + 512;
            runto = elements + nextIndex;
            while (nextIndex < runto && nextIndex < d->numElem) {
                d->regNumList[nextIndex] = regionNum;
                nextIndex++;
            }
            lastReg = regionNum;
        }
        free(regBinEnd);
    }
    for (int i = 0; i < d->numElem; ++i) d->regElemSize[d->regNumList[i] - 1]++;
    for (int i = 0; i < nr; ++i) {
        d->regElemlist[i] = ALLOC(int, d->regElemSize[i]);
        d->regElemSize[i] = 0;
    }
    for (int i = 0; i < d->numElem; ++i) {
        int r = d->regNumList[i] - 1;
        int regndx = d->regElemSize[r]++;
        d->regElemlist[r][regndx] = i;
    }
}

/* SetupSymmetryPlanes, lulesh-init.cc:514-533 */
static void setup_symmetry(orc_domain *d)
{
    const int edgeNodes = d->nx + 1;
    int nidx = 0;
    for (int i = 0; i < edgeNodes; ++i) {
        int planeInc = i * edgeNodes * edgeNodes;
        int rowInc = i * edgeNodes;
        for (int j = 0; j < edgeNodes; ++j) {
            d->symmZ[nidx] = rowInc + j;
            d->symmY[nidx] = planeInc + j;
            d->symmX[nidx] = planeInc + j * edgeNodes;
            ++nidx;
        }
    }
}

/* SetupElementConnectivities, lulesh-init.cc:539-565 */
static void setup_connectivity(orc_domain *d)
{
    const int E = d->numElem, n = d->nx;
    d->lxim[0] = 0;
    for (int i = 1; i < E; ++i) {
        d->lxim[i] = i - 1;
        d->lxip[i - 1] = i;
    }
    d->lxip[E - 1] = E - 1;
    for (int i = 0; i < n; ++i) {
        d->letam[i] = i;
        d->letap[E - n + i] = E - n + i;
    }
    for (int i = n; i < E; ++i) {
        d->letam[i] = i - n;
        d->letap[i - n] = i;
    }
    for (int i = 0; i < n * n; ++i) {
        d->lzetam[i] = i;
        d->lzetap[E - n * n + i] = E - n * n + i;
    }
    for (int i = n * n; i < E; ++i) {
        d->lzetam[i] = i - n * n;
        d->lzetap[i - n * n] = i;
    }
}

/* SetupBoundaryConditions, lulesh-init.cc:569-673 (single rank: min faces
 * symmetric, max faces free) */
static void setup_bc(orc_domain *d)
{
    const int n = d->nx, E = d->numElem;
    for (int i = 0; i < E; ++i) d->elemBC[i] = 0;
    for (int i = 0; i < n; ++i) {
        int planeInc = i * n * n;
        int rowInc = i * n;
        for (int j = 0; j < n; ++j) {
            d->elemBC[rowInc + j] |= ZETA_M_SYMM;
            d->elemBC[rowInc + j + E - n * n] |= ZETA_P_FREE;
            d->elemBC[planeInc + j] |= ETA_M_SYMM;
            d->elemBC[planeInc + j + n * n - n] |= ETA_P_FREE;
            d->elemBC[planeInc + j * n] |= XI_M_SYMM;
            d->elemBC[planeInc + j * n + n - 1] |= XI_P_FREE;
        }
    }
}

/* CalcElemVolume, lulesh.cc:1273-1356 */
static double elem_volume(const double x[8], const double y[8], const double z[8])
{
    const double twelveth = 1.0 / 12.0;
    double dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    double dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    double dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    double dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    double dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    double dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    double dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    double dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    double dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    double dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    double dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    double dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
#define TP(a1, b1, c1, a2, b2, c2, a3, b3, c3) \
    ((a1) * ((b2) * (c3) - (c2) * (b3)) + (a2) * ((c1) * (b3) - (b1) * (c3)) + \
     (a3) * ((b1) * (c2) - (c1) * (b2)))
    double volume = TP(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
                    TP(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
                    TP(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
#undef TP
    volume *= twelveth;
    return volume;
}

/* Domain::Domain, lulesh-init.cc:16-194 */
orc_domain *orc_create_ex(int nx, int numReg, int balance, int cost, double hgcoef,
                          double einit_factor)
{
    if (nx < 1 || numReg < 1) return NULL;
    orc_domain *d = (orc_domain *)calloc(1, sizeof(orc_domain));
    d->e_cut = 1.0e-7;
    d->p_cut = 1.0e-7;
    d->q_cut = 1.0e-7;
    d->v_cut = 1.0e-10;
    d->u_cut = 1.0e-7;
    d->hgcoef = hgcoef;
    d->ss4o3 = 4.0 / 3.0;
    d->qstop = 1.0e+12;
    d->monoq_max_slope = 1.0;
    d->monoq_limiter_mult = 2.0;
    d->qlc_monoq = 0.5;
    d->qqc_monoq = 2.0 / 3.0;
    d->qqc = 2.0;
    d->eosvmax = 1.0e+9;
    d->eosvmin = 1.0e-9;
    d->pmin = 0.;
    d->emin = -1.0e+15;
    d->dvovmax = 0.1;
    d->refdens = 1.0;

    const int edgeElems = nx, edgeNodes = nx + 1;
    d->nx = nx;
    d->cost = cost;
    d->balance = balance;
    d->numElem = edgeElems * edgeElems * edgeElems;
    d->numNode = edgeNodes * edgeNodes * edgeNodes;
    const int E = d->numElem, N = d->numNode;

    d->regNumList = ALLOC(int, E);
#define NA(f) d->f = ALLOC(double, N)
    NA(x); NA(y); NA(z); NA(xd); NA(yd); NA(zd); NA(xdd); NA(ydd); NA(zdd);
    NA(fx); NA(fy); NA(fz); NA(nodalMass);
#undef NA
    d->nodelist = ALLOC(int, 8 * E);
    d->lxim = ALLOC(int, E); d->lxip = ALLOC(int, E);
    d->letam = ALLOC(int, E); d->letap = ALLOC(int, E);
    d->lzetam = ALLOC(int, E); d->lzetap = ALLOC(int, E);
    d->elemBC = ALLOC(int, E);
#define EA(f) d->f = ALLOC(double, E)
    EA(e); EA(p); EA(q); EA(ql); EA(qq); EA(v); EA(volo); EA(vnew); EA(delv); EA(vdov);
    EA(arealg); EA(ss); EA(elemMass);
    EA(determ); EA(sig); EA(dxx); EA(dyy); EA(dzz);
    EA(delx_xi); EA(delx_eta); EA(delx_zeta); EA(delv_xi); EA(delv_eta); EA(delv_zeta);
    EA(vnewc);
#undef EA
#define CA(f) d->f = ALLOC(double, 8 * (size_t)E)
    CA(fx_elem); CA(fy_elem); CA(fz_elem); CA(dvdx); CA(dvdy); CA(dvdz);
    CA(x8n); CA(y8n); CA(z8n);
#undef CA
    d->nsymm = edgeNodes * edgeNodes;
    d->symmX = ALLOC(int, d->nsymm);
    d->symmY = ALLOC(int, d->nsymm);
    d->symmZ = ALLOC(int, d->nsymm);

    for (int i = 0; i < E; ++i) {
        d->e[i] = 0.0;
        d->p[i] = 0.0;
        d->q[i] = 0.0;
        d->ss[i] = 0.0;
        d->v[i] = 1.0;
    }
    build_mesh(d);
    orc_rebuild_corner_list(d);
    create_regions(d, numReg, balance);
    setup_symmetry(d);
    setup_connectivity(d);
    setup_bc(d);

    int maxreg = 0;
    for (int r = 0; r < d->numReg; ++r)
        if (d->regElemSize[r] > maxreg) maxreg = d->regElemSize[r];
    d->eos_tmp = ALLOC(double, 15 * (size_t)maxreg);

    d->dtfixed = -1.0e-6;
    d->stoptime = 1.0e-2;
    d->deltatimemultlb = 1.1;
    d->deltatimemultub = 1.2;
    d->dtcourant = 1.0e+20;
    d->dthydro = 1.0e+20;
    d->dtmax = 1.0e-2;
    d->time = 0.;
    d->cycle = 0;

    for (int i = 0; i < E; ++i) {
        double xl[8], yl[8], zl[8];
        const int *en = &d->nodelist[8 * i];
        for (int l = 0; l < 8; ++l) {
            xl[l] = d->x[en[l]];
            yl[l] = d->y[en[l]];
            zl[l] = d->z[en[l]];
        }
        double volume = elem_volume(xl, yl, zl);
        d->volo[i] = volume;
        d->elemMass[i] = volume;
        for (int j = 0; j < 8; ++j) d->nodalMass[en[j]] += volume / 8.0;
    }

    const double ebase = 3.948746e+7;
    double scale = (nx * 1) / 45.0;
    double einit = ebase * scale * scale * scale;
    einit = einit * einit_factor;
    d->e[0] = einit;
    d->deltatime = (.5 * cbrt(d->volo[0])) / sqrt(2.0 * einit);
    return d;
}

orc_domain *orc_create(int nx, int numReg, int balance, int cost)
{
    return orc_create_ex(nx, numReg, balance, cost, 3.0, 1.0);
}

void orc_destroy(orc_domain *d)
{
    if (!d) return;
    double **fl[] = {&d->x, &d->y, &d->z, &d->xd, &d->yd, &d->zd, &d->xdd, &d->ydd, &d->zdd,
                     &d->fx, &d->fy, &d->fz, &d->nodalMass, &d->e, &d->p, &d->q, &d->ql,
                     &d->qq, &d->v, &d->volo, &d->vnew, &d->delv, &d->vdov, &d->arealg,
                     &d->ss, &d->elemMass, &d->fx_elem, &d->fy_elem, &d->fz_elem,
                     &d->determ, &d->sig, &d->dvdx, &d->dvdy, &d->dvdz, &d->x8n, &d->y8n,
                     &d->z8n, &d->dxx, &d->dyy, &d->dzz, &d->delx_xi, &d->delx_eta,
                     &d->delx_zeta, &d->delv_xi, &d->delv_eta, &d->delv_zeta, &d->vnewc,
                     &d->eos_tmp, &d->dt_frozen, &d->dt_record};
    for (size_t i = 0; i < sizeof(fl) / sizeof(fl[0]); ++i) free(*fl[i]);
    int **il[] = {&d->symmX, &d->symmY, &d->symmZ, &d->nodelist, &d->lxim, &d->lxip,
                  &d->letam, &d->letap, &d->lzetam, &d->lzetap, &d->elemBC,
                  &d->regElemSize, &d->regNumList, &d->nodeElemStart,
                  &d->nodeElemCornerList};
    for (int r = 0; r < d->numReg; ++r) free(d->regElemlist[r]);
    free(d->regElemlist);
    for (size_t i = 0; i < sizeof(il) / sizeof(il[0]); ++i) free(*il[i]);
    tape_free(d->tape);
    free(d);
}

/* ------------------------------------------------------------------------ */
/* time step                                                                 */
/* ------------------------------------------------------------------------ */

/* TimeIncrement, lulesh.cc:166-222 (or the frozen step of this cycle) */
static void time_increment(orc_domain *d)
{
    if (d->dt_frozen && d->cycle < d->dt_frozen_len) {
        d->deltatime = d->dt_frozen[d->cycle];
        d->time += d->deltatime;
        ++d->cycle;
        return;
    }
    double targetdt = d->stoptime - d->time;
    if ((d->dtfixed <= 0.0) && (d->cycle != 0)) {
        double ratio;
        double olddt = d->deltatime;
        double gnewdt = 1.0e+20;
        double newdt;
        if (d->dtcourant < gnewdt) gnewdt = d->dtcourant / 2.0;
        if (d->dthydro < gnewdt) gnewdt = d->dthydro * 2.0 / 3.0;
        newdt = gnewdt;
        ratio = newdt / olddt;
        if (ratio >= 1.0) {
            if (ratio < d->deltatimemultlb)
                newdt = olddt;
            else if (ratio > d->deltatimemultub)
                newdt = olddt * d->deltatimemultub;
        }
        if (newdt > d->dtmax) newdt = d->dtmax;
        d->deltatime = newdt;
    }
    if ((targetdt > d->deltatime) && (targetdt < (4.0 * d->deltatime / 3.0)))
        targetdt = 2.0 * d->deltatime / 3.0;
    if (targetdt < d->deltatime) d->deltatime = targetdt;
    if (d->dt_record && d->cycle < d->dt_record_len) d->dt_record[d->cycle] = d->deltatime;
    d->time += d->deltatime;
    ++d->cycle;
}

int orc_dt_freeze(orc_domain *d, const double *dts, int n)
{
    free(d->dt_frozen);
    d->dt_frozen = NULL;
    d->dt_frozen_len = 0;
    if (n > 0) {
        d->dt_frozen = ALLOC(double, n);
        memcpy(d->dt_frozen, dts, sizeof(double) * (size_t)n);
        d->dt_frozen_len = n;
    }
    return 0;
}

int orc_dt_record(orc_domain *d, int capacity)
{
    free(d->dt_record);
    d->dt_record = NULL;
    d->dt_record_len = 0;
    if (capacity > 0) {
        d->dt_record = ALLOC(double, capacity);
        d->dt_record_len = capacity;
    }
    return 0;
}

const double *orc_dt_recorded(orc_domain *d) { return d->dt_record; }

static inline void gather8(const orc_domain *d, const double *f, const int *en, double o[8])
{
    for (int l = 0; l < 8; ++l) o[l] = f[en[l]];
}

/* CalcElemShapeFunctionDerivatives, lulesh.cc:290-377 */
static void shape_derivs(const double x[8], const double y[8], const double z[8],
                         double b[3][8], double *volume)
{
    const double x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3], x4 = x[4], x5 = x[5],
                 x6 = x[6], x7 = x[7];
    const double y0 = y[0], y1 = y[1], y2 = y[2], y3 = y[3], y4 = y[4], y5 = y[5],
                 y6 = y[6], y7 = y[7];
    const double z0 = z[0], z1 = z[1], z2 = z[2], z3 = z[3], z4 = z[4], z5 = z[5],
                 z6 = z[6], z7 = z[7];
    double fjxxi = .125 * ((x6 - x0) + (x5 - x3) - (x7 - x1) - (x4 - x2));
    double fjxet = .125 * ((x6 - x0) - (x5 - x3) + (x7 - x1) - (x4 - x2));
    double fjxze = .125 * ((x6 - x0) + (x5 - x3) + (x7 - x1) + (x4 - x2));
    double fjyxi = .125 * ((y6 - y0) + (y5 - y3) - (y7 - y1) - (y4 - y2));
    double fjyet = .125 * ((y6 - y0) - (y5 - y3) + (y7 - y1) - (y4 - y2));
    double fjyze = .125 * ((y6 - y0) + (y5 - y3) + (y7 - y1) + (y4 - y2));
    double fjzxi = .125 * ((z6 - z0) + (z5 - z3) - (z7 - z1) - (z4 - z2));
    double fjzet = .125 * ((z6 - z0) - (z5 - z3) + (z7 - z1) - (z4 - z2));
    double fjzze = .125 * ((z6 - z0) + (z5 - z3) + (z7 - z1) + (z4 - z2));
    double cjxxi = (fjyet * fjzze) - (fjzet * fjyze);
    double cjxet = -(fjyxi * fjzze) + (fjzxi * fjyze);
    double cjxze = (fjyxi * fjzet) - (fjzxi * fjyet);
    double cjyxi = -(fjxet * fjzze) + (fjzet * fjxze);
    double cjyet = (fjxxi * fjzze) - (fjzxi * fjxze);
    double cjyze = -(fjxxi * fjzet) + (fjzxi * fjxet);
    double cjzxi = (fjxet * fjyze) - (fjyet * fjxze);
    double cjzet = -(fjxxi * fjyze) + (fjyxi * fjxze);
    double cjzze = (fjxxi * fjyet) - (fjyxi * fjxet);
    b[0][0] = -cjxxi - cjxet - cjxze;
    b[0][1] = cjxxi - cjxet - cjxze;
    b[0][2] = cjxxi + cjxet - cjxze;
    b[0][3] = -cjxxi + cjxet - cjxze;
    b[0][4] = -b[0][2];
    b[0][5] = -b[0][3];
    b[0][6] = -b[0][0];
    b[0][7] = -b[0][1];
    b[1][0] = -cjyxi - cjyet - cjyze;
    b[1][1] = cjyxi - cjyet - cjyze;
    b[1][2] = cjyxi + cjyet - cjyze;
    b[1][3] = -cjyxi + cjyet - cjyze;
    b[1][4] = -b[1][2];
    b[1][5] = -b[1][3];
    b[1][6] = -b[1][0];
    b[1][7] = -b[1][1];
    b[2][0] = -cjzxi - cjzet - cjzze;
    b[2][1] = cjzxi - cjzet - cjzze;
    b[2][2] = cjzxi + cjzet - cjzze;
    b[2][3] = -cjzxi + cjzet - cjzze;
    b[2][4] = -b[2][2];
    b[2][5] = -b[2][3];
    b[2][6] = -b[2][0];
    b[2][7] = -b[2][1];
    *volume = 8. * (fjxet * cjxet + fjyet * cjyet + fjzet * cjzet);
}

/* SumElemFaceNormal, lulesh.cc:381-415 */
static void face_normal(double *nx0, double *ny0, double *nz0, double *nx1, double *ny1,
                        double *nz1, double *nx2, double *ny2, double *nz2, double *nx3,
                        double *ny3, double *nz3, double x0, double y0, double z0, double x1,
                        double y1, double z1, double x2, double y2, double z2, double x3,
                        double y3, double z3)
{
    double bisectX0 = 0.5 * (x3 + x2 - x1 - x0);
    double bisectY0 = 0.5 * (y3 + y2 - y1 - y0);
    double bisectZ0 = 0.5 * (z3 + z2 - z1 - z0);
    double bisectX1 = 0.5 * (x2 + x1 - x3 - x0);
    double bisectY1 = 0.5 * (y2 + y1 - y3 - y0);
    double bisectZ1 = 0.5 * (z2 + z1 - z3 - z0);
    double areaX = 0.25 * (bisectY0 * bisectZ1 - bisectZ0 * bisectY1);
    double areaY = 0.25 * (bisectZ0 * bisectX1 - bisectX0 * bisectZ1);
    double areaZ = 0.25 * (bisectX0 * bisectY1 - bisectY0 * bisectX1);
    *nx0 += areaX; *nx1 += areaX; *nx2 += areaX; *nx3 += areaX;
    *ny0 += areaY; *ny1 += areaY; *ny2 += areaY; *ny3 += areaY;
    *nz0 += areaZ; *nz1 += areaZ; *nz2 += areaZ; *nz3 += areaZ;
}

/* CalcElemNodeNormals, lulesh.cc:419-474 */
static void node_normals(double pfx[8], double pfy[8], double pfz[8], const double x[8],
                         const double y[8], const double z[8])
{
    static const int face[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2},
                                   {2, 6, 7, 3}, {3, 7, 4, 0}, {4, 7, 6, 5}};
    for (int i = 0; i < 8; ++i) pfx[i] = pfy[i] = pfz[i] = 0.0;
    for (int f = 0; f < 6; ++f) {
        const int a = face[f][0], b = face[f][1], c = face[f][2], e = face[f][3];
        face_normal(&pfx[a], &pfy[a], &pfz[a], &pfx[b], &pfy[b], &pfz[b], &pfx[c], &pfy[c],
                    &pfz[c], &pfx[e], &pfy[e], &pfz[e], x[a], y[a], z[a], x[b], y[b], z[b],
                    x[c], y[c], z[c], x[e], y[e], z[e]);
    }
}

/* VoluDer, lulesh.cc:591-619 */
static void volu_der(double x0, double x1, double x2, double x3, double x4, double x5,
                     double y0, double y1, double y2, double y3, double y4, double y5,
                     double z0, double z1, double z2, double z3, double z4, double z5,
                     double *dvdx, double *dvdy, double *dvdz)
{
    const double twelfth = 1.0 / 12.0;
    *dvdx = (y1 + y2) * (z0 + z1) - (y0 + y1) * (z1 + z2) + (y0 + y4) * (z3 + z4) -
            (y3 + y4) * (z0 + z4) - (y2 + y5) * (z3 + z5) + (y3 + y5) * (z2 + z5);
    *dvdy = -(x1 + x2) * (z0 + z1) + (x0 + x1) * (z1 + z2) - (x0 + x4) * (z3 + z4) +
            (x3 + x4) * (z0 + z4) + (x2 + x5) * (z3 + z5) - (x3 + x5) * (z2 + z5);
    *dvdz = -(y1 + y2) * (x0 + x1) + (y0 + y1) * (x1 + x2) - (y0 + y4) * (x3 + x4) +
            (y3 + y4) * (x0 + x4) + (y2 + y5) * (x3 + x5) - (y3 + y5) * (x2 + x5);
    *dvdx *= twelfth;
    *dvdy *= twelfth;
    *dvdz *= twelfth;
}

/* CalcElemVolumeDerivative, lulesh.cc:623-663: corner k uses the six
 * neighbouring nodes listed in row k */
static void volume_derivative(double dvdx[8], double dvdy[8], double dvdz[8],
                              const double x[8], const double y[8], const double z[8])
{
    static const int nb[8][6] = {{1, 2, 3, 4, 5, 7}, {2, 3, 0, 5, 6, 4}, {3, 0, 1, 6, 7, 5},
                                 {0, 1, 2, 7, 4, 6}, {7, 6, 5, 0, 3, 1}, {4, 7, 6, 1, 0, 2},
                                 {5, 4, 7, 2, 1, 3}, {6, 5, 4, 3, 2, 0}};
    for (int k = 0; k < 8; ++k) {
        const int *m = nb[k];
        volu_der(x[m[0]], x[m[1]], x[m[2]], x[m[3]], x[m[4]], x[m[5]], y[m[0]], y[m[1]],
                 y[m[2]], y[m[3]], y[m[4]], y[m[5]], z[m[0]], z[m[1]], z[m[2]], z[m[3]],
                 z[m[4]], z[m[5]], &dvdx[k], &dvdy[k], &dvdz[k]);
    }
}

/* hourglass base vectors, lulesh.cc:743-776 */
static const double GAMMA[4][8] = {{1., 1., -1., -1., -1., -1., 1., 1.},
                                   {1., -1., -1., 1., -1., 1., 1., -1.},
                                   {1., -1., 1., -1., 1., -1., 1., -1.},
                                   {-1., 1., -1., 1., 1., -1., 1., -1.}};

/* CalcElemFBHourglassForce, lulesh.cc:667-706 */
static void fb_hourglass_force(const double *xd, const double *yd, const double *zd,
                               double hourgam[8][4], double coefficient, double *hgfx,
                               double *hgfy, double *hgfz)
{
    const double *vel[3] = {xd, yd, zd};
    double *out[3] = {hgfx, hgfy, hgfz};
    for (int c = 0; c < 3; ++c) {
        const double *u = vel[c];
        double hxx[4];
        for (int i = 0; i < 4; i++)
            hxx[i] = hourgam[0][i] * u[0] + hourgam[1][i] * u[1] + hourgam[2][i] * u[2] +
                     hourgam[3][i] * u[3] + hourgam[4][i] * u[4] + hourgam[5][i] * u[5] +
                     hourgam[6][i] * u[6] + hourgam[7][i] * u[7];
        for (int i = 0; i < 8; i++)
            out[c][i] = coefficient * (hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] +
                                       hourgam[i][2] * hxx[2] + hourgam[i][3] * hxx[3]);
    }
}

/* node gather over nodeElemCornerList, lulesh.cc:565-582 (assign=1) and
 * lulesh.cc:969-986 (assign=0, accumulate) */
static void gather_corner_forces(orc_domain *d, int assign)
{
    const int N = d->numNode;
#pragma omp parallel for schedule(static)
    for (int g = 0; g < N; ++g) {
        const int count = d->nodeElemStart[g + 1] - d->nodeElemStart[g];
        const int *cl = &d->nodeElemCornerList[d->nodeElemStart[g]];
        double fxt = 0.0, fyt = 0.0, fzt = 0.0;
        for (int i = 0; i < count; ++i) {
            const int c = cl[i];
            fxt += d->fx_elem[c];
            fyt += d->fy_elem[c];
            fzt += d->fz_elem[c];
        }
        if (assign) {
            d->fx[g] = fxt;
            d->fy[g] = fyt;
            d->fz[g] = fzt;
        } else {
            d->fx[g] += fxt;
            d->fy[g] += fyt;
            d->fz[g] += fzt;
        }
    }
}

/* CalcVolumeForceForElems, lulesh.cc:1062-1100, with InitStressTermsForElems
 * (273-286), IntegrateStressForElems (494-587), CalcHourglassControlForElems
 * (995-1057) and CalcFBHourglassForceForElems (710-991) */
static int volume_force(orc_domain *d)
{
    const int E = d->numElem;
    if (E == 0) return ORC_OK;
    const double hgcoef = d->hgcoef;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < E; ++i) d->sig[i] = -d->p[i] - d->q[i];

#pragma omp parallel for schedule(static)
    for (int k = 0; k < E; ++k) {
        const int *en = &d->nodelist[8 * k];
        double B[3][8], xl[8], yl[8], zl[8];
        gather8(d, d->x, en, xl);
        gather8(d, d->y, en, yl);
        gather8(d, d->z, en, zl);
        shape_derivs(xl, yl, zl, B, &d->determ[k]);
        node_normals(B[0], B[1], B[2], xl, yl, zl);
        const double s = d->sig[k];
        for (int i = 0; i < 8; ++i) {
            d->fx_elem[8 * k + i] = -(s * B[0][i]);
            d->fy_elem[8 * k + i] = -(s * B[1][i]);
            d->fz_elem[8 * k + i] = -(s * B[2][i]);
        }
    }
    gather_corner_forces(d, 1);

    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int k = 0; k < E; ++k)
        if (d->determ[k] <= 0.0) bad |= 1;
    if (bad) return ORC_VOLUME_ERROR;

    /* CalcHourglassControlForElems */
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < E; ++i) {
        const int *en = &d->nodelist[8 * i];
        double x1[8], y1[8], z1[8], pfx[8], pfy[8], pfz[8];
        gather8(d, d->x, en, x1);
        gather8(d, d->y, en, y1);
        gather8(d, d->z, en, z1);
        volume_derivative(pfx, pfy, pfz, x1, y1, z1);
        for (int ii = 0; ii < 8; ++ii) {
            const int jj = 8 * i + ii;
            d->dvdx[jj] = pfx[ii];
            d->dvdy[jj] = pfy[ii];
            d->dvdz[jj] = pfz[ii];
            d->x8n[jj] = x1[ii];
            d->y8n[jj] = y1[ii];
            d->z8n[jj] = z1[ii];
        }
        d->determ[i] = d->volo[i] * d->v[i];
        if (d->v[i] <= 0.0) bad |= 1;
    }
    if (bad) return ORC_VOLUME_ERROR;
    if (!(hgcoef > 0.)) return ORC_OK;

    /* CalcFBHourglassForceForElems */
#pragma omp parallel for schedule(static)
    for (int i2 = 0; i2 < E; ++i2) {
        const int *en = &d->nodelist[8 * i2];
        const int i3 = 8 * i2;
        double hourgam[8][4], xd1[8], yd1[8], zd1[8], hgfx[8], hgfy[8], hgfz[8];
        double volinv = 1.0 / d->determ[i2];
        for (int i1 = 0; i1 < 4; ++i1) {
            const double *g = GAMMA[i1];
            double hourmodx = d->x8n[i3] * g[0] + d->x8n[i3 + 1] * g[1] +
                              d->x8n[i3 + 2] * g[2] + d->x8n[i3 + 3] * g[3] +
                              d->x8n[i3 + 4] * g[4] + d->x8n[i3 + 5] * g[5] +
                              d->x8n[i3 + 6] * g[6] + d->x8n[i3 + 7] * g[7];
            double hourmody = d->y8n[i3] * g[0] + d->y8n[i3 + 1] * g[1] +
                              d->y8n[i3 + 2] * g[2] + d->y8n[i3 + 3] * g[3] +
                              d->y8n[i3 + 4] * g[4] + d->y8n[i3 + 5] * g[5] +
                              d->y8n[i3 + 6] * g[6] + d->y8n[i3 + 7] * g[7];
            double hourmodz = d->z8n[i3] * g[0] + d->z8n[i3 + 1] * g[1] +
                              d->z8n[i3 + 2] * g[2] + d->z8n[i3 + 3] * g[3] +
                              d->z8n[i3 + 4] * g[4] + d->z8n[i3 + 5] * g[5] +
                              d->z8n[i3 + 6] * g[6] + d->z8n[i3 + 7] * g[7];
            for (int k = 0; k < 8; ++k)
                hourgam[k][i1] = g[k] - volinv * (d->dvdx[i3 + k] * hourmodx +
                                                  d->dvdy[i3 + k] * hourmody +
                                                  d->dvdz[i3 + k] * hourmodz);
        }
        double ss1 = d->ss[i2];
        double mass1 = d->elemMass[i2];
        double volume13 = cbrt(d->determ[i2]);
        gather8(d, d->xd, en, xd1);
        gather8(d, d->yd, en, yd1);
        gather8(d, d->zd, en, zd1);
        double coefficient = -hgcoef * 0.01 * ss1 * mass1 / volume13;
        fb_hourglass_force(xd1, yd1, zd1, hourgam, coefficient, hgfx, hgfy, hgfz);
        for (int k = 0; k < 8; ++k) {
            d->fx_elem[i3 + k] = hgfx[k];
            d->fy_elem[i3 + k] = hgfy[k];
            d->fz_elem[i3 + k] = hgfz[k];
        }
    }
    gather_corner_forces(d, 0);
    return ORC_OK;
}

/* LagrangeNodal, lulesh.cc:1223-1269, with CalcForceForNodes (1104-1135),
 * CalcAccelerationForNodes (1139-1149), ApplyAccelerationBoundaryConditions
 * ForNodes (1153-1179), CalcVelocityForNodes (1183-1205) and
 * CalcPositionForNodes (1209-1219) */
static int lagrange_nodal(orc_domain *d)
{
    const double delt = d->deltatime;
    const double u_cut = d->u_cut;
    const int N = d->numNode;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) d->fx[i] = d->fy[i] = d->fz[i] = 0.0;
    int st = volume_force(d);
    if (st) return st;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        d->xdd[i] = d->fx[i] / d->nodalMass[i];
        d->ydd[i] = d->fy[i] / d->nodalMass[i];
        d->zdd[i] = d->fz[i] / d->nodalMass[i];
    }
    for (int i = 0; i < d->nsymm; ++i) d->xdd[d->symmX[i]] = 0.0;
    for (int i = 0; i < d->nsymm; ++i) d->ydd[d->symmY[i]] = 0.0;
    for (int i = 0; i < d->nsymm; ++i) d->zdd[d->symmZ[i]] = 0.0;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        double xdtmp = d->xd[i] + d->xdd[i] * delt;
        xdtmp = TAPE_CUT_NODE(TB_NODE_U + 0, TS_U + 0, i, xdtmp, fabs(xdtmp) < u_cut, 0.0);
        d->xd[i] = xdtmp;
        double ydtmp = d->yd[i] + d->ydd[i] * delt;
        ydtmp = TAPE_CUT_NODE(TB_NODE_U + 1, TS_U + 1, i, ydtmp, fabs(ydtmp) < u_cut, 0.0);
        d->yd[i] = ydtmp;
        double zdtmp = d->zd[i] + d->zdd[i] * delt;
        zdtmp = TAPE_CUT_NODE(TB_NODE_U + 2, TS_U + 2, i, zdtmp, fabs(zdtmp) < u_cut, 0.0);
        d->zd[i] = zdtmp;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        d->x[i] += d->xd[i] * delt;
        d->y[i] += d->yd[i] * delt;
        d->z[i] += d->zd[i] * delt;
    }
    return ORC_OK;
}

/* AreaFace, lulesh.cc:1370-1390 */
static double area_face(double x0, double x1, double x2, double x3, double y0, double y1,
                        double y2, double y3, double z0, double z1, double z2, double z3)
{
    double fx = (x2 - x0) - (x3 - x1);
    double fy = (y2 - y0) - (y3 - y1);
    double fz = (z2 - z0) - (z3 - z1);
    double gx = (x2 - x0) + (x3 - x1);
    double gy = (y2 - y0) + (y3 - y1);
    double gz = (z2 - z0) + (z3 - z1);
    return (fx * fx + fy * fy + fz * fz) * (gx * gx + gy * gy + gz * gz) -
           (fx * gx + fy * gy + fz * gz) * (fx * gx + fy * gy + fz * gz);
}

/* CalcElemCharacteristicLength, lulesh.cc:1394-1435; std::max(a,b) is
 * (a < b) ? b : a */
static double char_length(const double x[8], const double y[8], const double z[8],
                          double volume)
{
    static const int face[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                   {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
    double cl = 0.0;
    for (int f = 0; f < 6; ++f) {
        const int *m = face[f];
        double a = area_face(x[m[0]], x[m[1]], x[m[2]], x[m[3]], y[m[0]], y[m[1]], y[m[2]],
                             y[m[3]], z[m[0]], z[m[1]], z[m[2]], z[m[3]]);
        cl = (a < cl) ? cl : a;
    }
    return 4.0 * volume / sqrt(cl);
}

/* CalcKinematicsForElems, lulesh.cc:1504-1568 with CalcElemVelocityGradient
 * (1439-1500, only the diagonal terms are kept by the caller), and the strain
 * loop of CalcLagrangeElements (1572-1609) */
static int lagrange_elements_kinematics(orc_domain *d)
{
    const int E = d->numElem;
    const double deltaTime = d->deltatime;
    int bad = 0;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < E; ++k) {
        const int *en = &d->nodelist[8 * k];
        double B[3][8], xl[8], yl[8], zl[8], xdl[8], ydl[8], zdl[8], detJ = 0.0;
        gather8(d, d->x, en, xl);
        gather8(d, d->y, en, yl);
        gather8(d, d->z, en, zl);
        double volume = elem_volume(xl, yl, zl);
        double relativeVolume = volume / d->volo[k];
        d->vnew[k] = relativeVolume;
        d->delv[k] = relativeVolume - d->v[k];
        d->arealg[k] = char_length(xl, yl, zl, volume);
        gather8(d, d->xd, en, xdl);
        gather8(d, d->yd, en, ydl);
        gather8(d, d->zd, en, zdl);
        double dt2 = 0.5 * deltaTime;
        for (int j = 0; j < 8; ++j) {
            xl[j] -= dt2 * xdl[j];
            yl[j] -= dt2 * ydl[j];
            zl[j] -= dt2 * zdl[j];
        }
        shape_derivs(xl, yl, zl, B, &detJ);
        const double inv_detJ = 1.0 / detJ;
        const double *pfx = B[0], *pfy = B[1], *pfz = B[2];
        d->dxx[k] = inv_detJ * (pfx[0] * (xdl[0] - xdl[6]) + pfx[1] * (xdl[1] - xdl[7]) +
                                pfx[2] * (xdl[2] - xdl[4]) + pfx[3] * (xdl[3] - xdl[5]));
        d->dyy[k] = inv_detJ * (pfy[0] * (ydl[0] - ydl[6]) + pfy[1] * (ydl[1] - ydl[7]) +
                                pfy[2] * (ydl[2] - ydl[4]) + pfy[3] * (ydl[3] - ydl[5]));
        d->dzz[k] = inv_detJ * (pfz[0] * (zdl[0] - zdl[6]) + pfz[1] * (zdl[1] - zdl[7]) +
                                pfz[2] * (zdl[2] - zdl[4]) + pfz[3] * (zdl[3] - zdl[5]));
    }
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int k = 0; k < E; ++k) {
        double vdov = d->dxx[k] + d->dyy[k] + d->dzz[k];
        double vdovthird = vdov / 3.0;
        d->vdov[k] = vdov;
        d->dxx[k] -= vdovthird;
        d->dyy[k] -= vdovthird;
        d->dzz[k] -= vdovthird;
        if (d->vnew[k] <= 0.0) bad |= 1;
    }
    return bad ? ORC_VOLUME_ERROR : ORC_OK;
}

/* CalcMonotonicQGradientsForElems, lulesh.cc:1613-1757 */
static void monoq_gradients(orc_domain *d)
{
    const int E = d->numElem;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < E; ++i) {
        const double ptiny = 1.e-36;
        const int *en = &d->nodelist[8 * i];
        double X[8], Y[8], Z[8], XV[8], YV[8], ZV[8];
        gather8(d, d->x, en, X);
        gather8(d, d->y, en, Y);
        gather8(d, d->z, en, Z);
        gather8(d, d->xd, en, XV);
        gather8(d, d->yd, en, YV);
        gather8(d, d->zd, en, ZV);
        double ax, ay, az, dxv, dyv, dzv;
        double vol = d->volo[i] * d->vnew[i];
        double norm = 1.0 / (vol + ptiny);
#define S4(A, a, b, c, e) (A[a] + A[b] + A[c] + A[e])
        double dxj = -0.25 * (S4(X, 0, 1, 5, 4) - S4(X, 3, 2, 6, 7));
        double dyj = -0.25 * (S4(Y, 0, 1, 5, 4) - S4(Y, 3, 2, 6, 7));
        double dzj = -0.25 * (S4(Z, 0, 1, 5, 4) - S4(Z, 3, 2, 6, 7));
        double dxi = 0.25 * (S4(X, 1, 2, 6, 5) - S4(X, 0, 3, 7, 4));
        double dyi = 0.25 * (S4(Y, 1, 2, 6, 5) - S4(Y, 0, 3, 7, 4));
        double dzi = 0.25 * (S4(Z, 1, 2, 6, 5) - S4(Z, 0, 3, 7, 4));
        double dxk = 0.25 * (S4(X, 4, 5, 6, 7) - S4(X, 0, 1, 2, 3));
        double dyk = 0.25 * (S4(Y, 4, 5, 6, 7) - S4(Y, 0, 1, 2, 3));
        double dzk = 0.25 * (S4(Z, 4, 5, 6, 7) - S4(Z, 0, 1, 2, 3));

        ax = dyi * dzj - dzi * dyj;
        ay = dzi * dxj - dxi * dzj;
        az = dxi * dyj - dyi * dxj;
        d->delx_zeta[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm;
        ay *= norm;
        az *= norm;
        dxv = 0.25 * (S4(XV, 4, 5, 6, 7) - S4(XV, 0, 1, 2, 3));
        dyv = 0.25 * (S4(YV, 4, 5, 6, 7) - S4(YV, 0, 1, 2, 3));
        dzv = 0.25 * (S4(ZV, 4, 5, 6, 7) - S4(ZV, 0, 1, 2, 3));
        d->delv_zeta[i] = ax * dxv + ay * dyv + az * dzv;

        ax = dyj * dzk - dzj * dyk;
        ay = dzj * dxk - dxj * dzk;
        az = dxj * dyk - dyj * dxk;
        d->delx_xi[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm;
        ay *= norm;
        az *= norm;
        dxv = 0.25 * (S4(XV, 1, 2, 6, 5) - S4(XV, 0, 3, 7, 4));
        dyv = 0.25 * (S4(YV, 1, 2, 6, 5) - S4(YV, 0, 3, 7, 4));
        dzv = 0.25 * (S4(ZV, 1, 2, 6, 5) - S4(ZV, 0, 3, 7, 4));
        d->delv_xi[i] = ax * dxv + ay * dyv + az * dzv;

        ax = dyk * dzi - dzk * dyi;
        ay = dzk * dxi - dxk * dzi;
        az = dxk * dyi - dyk * dxi;
        d->delx_eta[i] = vol / sqrt(ax * ax + ay * ay + az * az + ptiny);
        ax *= norm;
        ay *= norm;
        az *= norm;
        dxv = -0.25 * (S4(XV, 0, 1, 5, 4) - S4(XV, 3, 2, 6, 7));
        dyv = -0.25 * (S4(YV, 0, 1, 5, 4) - S4(YV, 3, 2, 6, 7));
        dzv = -0.25 * (S4(ZV, 0, 1, 5, 4) - S4(ZV, 3, 2, 6, 7));
        d->delv_eta[i] = ax * dxv + ay * dyv + az * dzv;
#undef S4
    }
}

/* one direction of the monotonic limiter, lulesh.cc:1778-1813 */
static double monoq_phi(const orc_domain *d, const double *delv_dir, int ielem, int bc,
                        int mmask, int msymm, int mfree, int mcomm, int pmask, int psymm,
                        int pfree, int pcomm, int nbm, int nbp, double ptiny, int bit0)
{
    (void)bit0;
    double delvm = 0.0, delvp = 0.0;
    double norm = 1. / (delv_dir[ielem] + ptiny);
    int bm = bc & mmask;
    if (bm == mcomm || bm == 0)
        delvm = delv_dir[nbm];
    else if (bm == msymm)
        delvm = delv_dir[ielem];
    else if (bm == mfree)
        delvm = 0.0;
    else
        delvm = 0;
    int bp = bc & pmask;
    if (bp == pcomm || bp == 0)
        delvp = delv_dir[nbp];
    else if (bp == psymm)
        delvp = delv_dir[ielem];
    else if (bp == pfree)
        delvp = 0.0;
    else
        delvp = 0;
    delvm = delvm * norm;
    delvp = delvp * norm;
    double phi = .5 * (delvm + delvp);
    delvm *= d->monoq_limiter_mult;
    delvp *= d->monoq_limiter_mult;
    if (TAPE_IF(bit0 + 0, ielem, delvm < phi)) phi = delvm;
    if (TAPE_IF(bit0 + 1, ielem, delvp < phi)) phi = delvp;
    if (TAPE_IF(bit0 + 2, ielem, phi < 0.)) phi = 0.;
    if (TAPE_IF(bit0 + 3, ielem, phi > d->monoq_max_slope)) phi = d->monoq_max_slope;
    return phi;
}

/* CalcMonotonicQRegionForElems, lulesh.cc:1761-1921 */
static void monoq_region(orc_domain *d, int r)
{
    const double ptiny = 1.e-36;
    const int len = d->regElemSize[r];
    const int *list = d->regElemlist[r];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < len; ++i) {
        const int ielem = list[i];
        const int bc = d->elemBC[ielem];
        double qlin, qquad;
        double phixi = monoq_phi(d, d->delv_xi, ielem, bc, XI_M, XI_M_SYMM, XI_M_FREE,
                                 XI_M_COMM, XI_P, XI_P_SYMM, XI_P_FREE, XI_P_COMM,
                                 d->lxim[ielem], d->lxip[ielem], ptiny, TB_PHI + 0);
        double phieta = monoq_phi(d, d->delv_eta, ielem, bc, ETA_M, ETA_M_SYMM, ETA_M_FREE,
                                  ETA_M_COMM, ETA_P, ETA_P_SYMM, ETA_P_FREE, ETA_P_COMM,
                                  d->letam[ielem], d->letap[ielem], ptiny, TB_PHI + 4);
        double phizeta = monoq_phi(d, d->delv_zeta, ielem, bc, ZETA_M, ZETA_M_SYMM,
                                   ZETA_M_FREE, ZETA_M_COMM, ZETA_P, ZETA_P_SYMM,
                                   ZETA_P_FREE, ZETA_P_COMM, d->lzetam[ielem],
                                   d->lzetap[ielem], ptiny, TB_PHI + 8);
        if (TAPE_IF(TB_VDOV, ielem, d->vdov[ielem] > 0.)) {
            qlin = 0.;
            qquad = 0.;
        } else {
            double delvxxi = d->delv_xi[ielem] * d->delx_xi[ielem];
            double delvxeta = d->delv_eta[ielem] * d->delx_eta[ielem];
            double delvxzeta = d->delv_zeta[ielem] * d->delx_zeta[ielem];
            if (TAPE_IF(TB_DELVX + 0, ielem, delvxxi > 0.)) delvxxi = 0.;
            if (TAPE_IF(TB_DELVX + 1, ielem, delvxeta > 0.)) delvxeta = 0.;
            if (TAPE_IF(TB_DELVX + 2, ielem, delvxzeta > 0.)) delvxzeta = 0.;
            double rho = d->elemMass[ielem] / (d->volo[ielem] * d->vnew[ielem]);
            qlin = -d->qlc_monoq * rho *
                   (delvxxi * (1. - phixi) + delvxeta * (1. - phieta) +
                    delvxzeta * (1. - phizeta));
            qquad = d->qqc_monoq * rho *
                    (delvxxi * delvxxi * (1. - phixi * phixi) +
                     delvxeta * delvxeta * (1. - phieta * phieta) +
                     delvxzeta * delvxzeta * (1. - phizeta * phizeta));
        }
        d->qq[ielem] = qquad;
        d->ql[ielem] = qlin;
    }
}

/* CalcQForElems, lulesh.cc:1945-2010 */
static int calc_q(orc_domain *d)
{
    if (d->numElem == 0) return ORC_OK;
    monoq_gradients(d);
    for (int r = 0; r < d->numReg; ++r)
        if (d->regElemSize[r] > 0) monoq_region(d, r);
    for (int i = 0; i < d->numElem; ++i)
        if (d->q[i] > d->qstop) return ORC_QSTOP_ERROR;
    return ORC_OK;
}

/* CalcPressureForElems, lulesh.cc:2014-2044 */
static void calc_pressure(const orc_domain *d, int bit0, int slot, double *p_new, double *bvc,
                          double *pbvc, const double *e_old, const double *compression,
                          const double *vnewc, double pmin, double p_cut, double eosvmax,
                          int length, const int *list)
{
    (void)d; (void)bit0; (void)slot;
    for (int i = 0; i < length; ++i) {
        const double c1s = 2.0 / 3.0;
        bvc[i] = c1s * (compression[i] + 1.);
        pbvc[i] = c1s;
    }
    for (int i = 0; i < length; ++i) {
        const int ielem = list[i];
        p_new[i] = bvc[i] * e_old[i];
        p_new[i] = TAPE_CUT(bit0 + 0, slot, ielem, p_new[i], fabs(p_new[i]) < p_cut, 0.0);
        if (TAPE_IF(bit0 + 1, ielem, vnewc[ielem] >= eosvmax)) p_new[i] = 0.0;
        if (TAPE_IF(bit0 + 2, ielem, p_new[i] < pmin)) p_new[i] = pmin;
    }
}

/* sound-speed-like term shared by lulesh.cc:2083-2090, 2126-2133,
 * 2158-2165, 2190-2197 */
static inline double ssc_of(const orc_domain *d, int bit, int idx, double x, double rho0)
{
    (void)d; (void)bit; (void)idx;
    double ssc = x / rho0;
    if (TAPE_IF(bit, idx, ssc <= .1111111e-36))
        ssc = .3333333e-18;
    else
        ssc = sqrt(ssc);
    return ssc;
}

/* EvalEOSForElems (lulesh.cc:2204-2324) with CalcEnergyForElems (2048-2176)
 * and CalcSoundSpeedForElems (2180-2200), evaluated for the elements
 * [lo, hi) of one region's list.  Each element's arithmetic is independent
 * of the others, so chunks of a region can be processed in parallel. */
static void eval_eos_chunk(orc_domain *d, const int *list, int lo, int hi, int rep, double *t)
{
    const int len = hi - lo;
    const int *rl = list + lo;
    double *e_old = t, *delvc = t + len, *p_old = t + 2 * len, *q_old = t + 3 * len,
           *compression = t + 4 * len, *compHalfStep = t + 5 * len, *qq_old = t + 6 * len,
           *ql_old = t + 7 * len, *work = t + 8 * len, *p_new = t + 9 * len,
           *e_new = t + 10 * len, *q_new = t + 11 * len, *bvc = t + 12 * len,
           *pbvc = t + 13 * len, *pHalfStep = t + 14 * len;
    const double e_cut = d->e_cut, p_cut = d->p_cut, q_cut = d->q_cut;
    const double eosvmax = d->eosvmax, eosvmin = d->eosvmin, pmin = d->pmin, emin = d->emin;
    const double rho0 = d->refdens;
    const double *vnewc = d->vnewc;
    for (int j = 0; j < rep; j++) {
        for (int i = 0; i < len; ++i) {
            const int ielem = rl[i];
            e_old[i] = d->e[ielem];
            delvc[i] = d->delv[ielem];
            p_old[i] = d->p[ielem];
            q_old[i] = d->q[ielem];
            qq_old[i] = d->qq[ielem];
            ql_old[i] = d->ql[ielem];
        }
        for (int i = 0; i < len; ++i) {
            const int ielem = rl[i];
            double vchalf;
            compression[i] = 1. / vnewc[ielem] - 1.;
            vchalf = vnewc[ielem] - delvc[i] * .5;
            compHalfStep[i] = 1. / vchalf - 1.;
        }
        if (eosvmin != 0.)
            for (int i = 0; i < len; ++i)
                if (TAPE_IF(TB_EOS_VMIN, rl[i], vnewc[rl[i]] <= eosvmin))
                    compHalfStep[i] = compression[i];
        if (eosvmax != 0.)
            for (int i = 0; i < len; ++i)
                if (TAPE_IF(TB_EOS_VMAX, rl[i], vnewc[rl[i]] >= eosvmax)) {
                    p_old[i] = 0.;
                    compression[i] = 0.;
                    compHalfStep[i] = 0.;
                }
        for (int i = 0; i < len; ++i) work[i] = 0.;

        /* CalcEnergyForElems, lulesh.cc:2048-2176 */
        for (int i = 0; i < len; ++i) {
            e_new[i] = e_old[i] - .5 * delvc[i] * (p_old[i] + q_old[i]) + .5 * work[i];
            if (TAPE_IF(TB_E1_EMIN, rl[i], e_new[i] < emin)) e_new[i] = emin;
        }
        calc_pressure(d, TB_P_HALF, TS_P_HALF, pHalfStep, bvc, pbvc, e_new, compHalfStep, vnewc,
                      pmin, p_cut, eosvmax, len, rl);
        for (int i = 0; i < len; ++i) {
            const int ielem = rl[i];
            (void)ielem;
            double vhalf = 1. / (1. + compHalfStep[i]);
            if (TAPE_IF(TB_Q1_COMP, ielem, delvc[i] > 0.)) {
                q_new[i] = 0.;
            } else {
                double ssc = ssc_of(d, TB_Q1_FLOOR, ielem,
                                    pbvc[i] * e_new[i] + vhalf * vhalf * bvc[i] * pHalfStep[i],
                                    rho0);
                q_new[i] = (ssc * ql_old[i] + qq_old[i]);
            }
            e_new[i] = e_new[i] + .5 * delvc[i] *
                                      (3.0 * (p_old[i] + q_old[i]) -
                                       4.0 * (pHalfStep[i] + q_new[i]));
        }
        for (int i = 0; i < len; ++i) {
            const int ielem = rl[i];
            (void)ielem;
            e_new[i] += .5 * work[i];
            e_new[i] = TAPE_CUT(TB_E3_CUT, TS_E3, ielem, e_new[i], fabs(e_new[i]) < e_cut, 0.);
            if (TAPE_IF(TB_E3_EMIN, ielem, e_new[i] < emin)) e_new[i] = emin;
        }
        calc_pressure(d, TB_P_NEW1, TS_P_NEW1, p_new, bvc, pbvc, e_new, compression, vnewc, pmin,
                      p_cut, eosvmax, len, rl);
        for (int i = 0; i < len; ++i) {
            const double sixth = 1.0 / 6.0;
            const int ielem = rl[i];
            double q_tilde;
            if (TAPE_IF(TB_QT_COMP, ielem, delvc[i] > 0.)) {
                q_tilde = 0.;
            } else {
                double ssc = ssc_of(d, TB_QT_FLOOR, ielem,
                                    pbvc[i] * e_new[i] +
                                        vnewc[ielem] * vnewc[ielem] * bvc[i] * p_new[i],
                                    rho0);
                q_tilde = (ssc * ql_old[i] + qq_old[i]);
            }
            e_new[i] = e_new[i] - (7.0 * (p_old[i] + q_old[i]) -
                                   8.0 * (pHalfStep[i] + q_new[i]) + (p_new[i] + q_tilde)) *
                                      delvc[i] * sixth;
            e_new[i] = TAPE_CUT(TB_E4_CUT, TS_E4, ielem, e_new[i], fabs(e_new[i]) < e_cut, 0.);
            if (TAPE_IF(TB_E4_EMIN, ielem, e_new[i] < emin)) e_new[i] = emin;
        }
        calc_pressure(d, TB_P_NEW2, TS_P_NEW2, p_new, bvc, pbvc, e_new, compression, vnewc, pmin,
                      p_cut, eosvmax, len, rl);
        for (int i = 0; i < len; ++i) {
            const int ielem = rl[i];
            if (TAPE_IF(TB_QF_COMP, ielem, delvc[i] <= 0.)) {
                double ssc = ssc_of(d, TB_QF_FLOOR, ielem,
                                    pbvc[i] * e_new[i] +
                                        vnewc[ielem] * vnewc[ielem] * bvc[i] * p_new[i],
                                    rho0);
                q_new[i] = (ssc * ql_old[i] + qq_old[i]);
                q_new[i] = TAPE_CUT(TB_QF_CUT, TS_QF, ielem, q_new[i], fabs(q_new[i]) < q_cut, 0.);
            }
        }
    }
    for (int i = 0; i < len; ++i) {
        const int ielem = rl[i];
        d->p[ielem] = p_new[i];
        d->e[ielem] = e_new[i];
        d->q[ielem] = q_new[i];
    }
    for (int i = 0; i < len; ++i) {
        const int ielem = rl[i];
        d->ss[ielem] = ssc_of(d, TB_SS_FLOOR, ielem,
                              pbvc[i] * e_new[i] + vnewc[ielem] * vnewc[ielem] * bvc[i] * p_new[i],
                              rho0);
    }
}

int orc_region_rep(orc_domain *d, int r)
{
    /* lulesh.cc:2390-2400 */
    if (r < d->numReg / 2) return 1;
    if (r < (d->numReg - (d->numReg + 15) / 20)) return 1 + d->cost;
    return 10 * (1 + d->cost);
}

/* ApplyMaterialPropertiesForElems, lulesh.cc:2328-2406 */
static int apply_material(orc_domain *d)
{
    const int E = d->numElem;
    if (E == 0) return ORC_OK;
    const double eosvmin = d->eosvmin, eosvmax = d->eosvmax;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int i = 0; i < E; ++i) {
        double vc = d->vnew[i];
        if (eosvmin != 0. && TAPE_IF(TB_VC_MIN, i, vc < eosvmin)) vc = eosvmin;
        if (eosvmax != 0. && TAPE_IF(TB_VC_MAX, i, vc > eosvmax)) vc = eosvmax;
        d->vnewc[i] = vc;
        double v = d->v[i];
        if (eosvmin != 0. && v < eosvmin) v = eosvmin;
        if (eosvmax != 0. && v > eosvmax) v = eosvmax;
        if (v <= 0.) bad |= 1;
    }
    if (bad) return ORC_VOLUME_ERROR;
    const int CH = 2048;
    for (int r = 0; r < d->numReg; r++) {
        const int len = d->regElemSize[r];
        const int rep = orc_region_rep(d, r);
        const int nchunk = (len + CH - 1) / CH;
#pragma omp parallel
        {
            double *t = (double *)malloc(sizeof(double) * 15 * CH);
#pragma omp for schedule(dynamic, 1)
            for (int c = 0; c < nchunk; ++c) {
                int lo = c * CH, hi = lo + CH < len ? lo + CH : len;
                eval_eos_chunk(d, d->regElemlist[r], lo, hi, rep, t);
            }
            free(t);
        }
    }
    return ORC_OK;
}

/* UpdateVolumesForElems, lulesh.cc:2410-2427 */
static void update_volumes(orc_domain *d)
{
    const int E = d->numElem;
    const double v_cut = d->v_cut;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < E; ++i) {
        double tmpV = d->vnew[i];
        tmpV = TAPE_CUT(TB_V_CUT, TS_V, i, tmpV, fabs(tmpV - 1.0) < v_cut, 1.0);
        d->v[i] = tmpV;
    }
}

/* LagrangeElements, lulesh.cc:2431-2443 */
static int lagrange_elements(orc_domain *d)
{
    int st;
    if (d->numElem > 0) {
        st = lagrange_elements_kinematics(d);
        if (st) return st;
    }
    st = calc_q(d);
    if (st) return st;
    st = apply_material(d);
    if (st) return st;
    update_volumes(d);
    return ORC_OK;
}

/* CalcTimeConstraintsForElems, lulesh.cc:2576-2596, with
 * CalcCourantConstraintForElems (2447-2513) and CalcHydroConstraintForElems
 * (2517-2572).  The per-thread minima followed by a serial minimum equal the
 * minimum over all qualifying elements, which is what is computed here. */
static void time_constraints(orc_domain *d)
{
    d->dtcourant = 1.0e+20;
    d->dthydro = 1.0e+20;
    const double qqc2 = 64.0 * d->qqc * d->qqc;
    const double dvovmax = d->dvovmax;
    for (int r = 0; r < d->numReg; ++r) {
        const int len = d->regElemSize[r];
        const int *list = d->regElemlist[r];
        double dtc = d->dtcourant, dth = d->dthydro;
#pragma omp parallel for schedule(static) reduction(min : dtc, dth)
        for (int i = 0; i < len; ++i) {
            const int indx = list[i];
            double dtf = d->ss[indx] * d->ss[indx];
            if (d->vdov[indx] < 0.)
                dtf = dtf + qqc2 * d->arealg[indx] * d->arealg[indx] * d->vdov[indx] * d->vdov[indx];
            dtf = sqrt(dtf);
            dtf = d->arealg[indx] / dtf;
            if (d->vdov[indx] != 0.) {
                if (dtf < dtc) dtc = dtf;
                double dtdvov = dvovmax / (fabs(d->vdov[indx]) + 1.e-20);
                if (dth > dtdvov) dth = dtdvov;
            }
        }
        d->dtcourant = dtc;
        d->dthydro = dth;
    }
}

int orc_phase(orc_domain *d, int phase)
{
    switch (phase) {
    case 0: time_increment(d); return ORC_OK;
    case 1: return lagrange_nodal(d);
    case 2: return lagrange_elements(d);
    case 3: time_constraints(d); return ORC_OK;
    default: return 1;
    }
}

int orc_step(orc_domain *d, int ncycles)
{
    for (int c = 0; c < ncycles && d->time < d->stoptime; ++c) {
        tape_begin_cycle(d);
        time_increment(d);
        int st = lagrange_nodal(d);
        if (st) return st;
        st = lagrange_elements(d);
        if (st) return st;
        time_constraints(d);
        tape_end_cycle(d);
    }
    return ORC_OK;
}

double *orc_field_f64(orc_domain *d, const char *name, size_t *n)
{
    const size_t N = (size_t)d->numNode, E = (size_t)d->numElem;
    struct { const char *nm; double *p; size_t len; } t[] = {
        {"x", d->x, N}, {"y", d->y, N}, {"z", d->z, N}, {"xd", d->xd, N}, {"yd", d->yd, N},
        {"zd", d->zd, N}, {"xdd", d->xdd, N}, {"ydd", d->ydd, N}, {"zdd", d->zdd, N},
        {"fx", d->fx, N}, {"fy", d->fy, N}, {"fz", d->fz, N}, {"nodalMass", d->nodalMass, N},
        {"e", d->e, E}, {"p", d->p, E}, {"q", d->q, E}, {"ql", d->ql, E}, {"qq", d->qq, E},
        {"v", d->v, E}, {"volo", d->volo, E}, {"vnew", d->vnew, E}, {"delv", d->delv, E},
        {"vdov", d->vdov, E}, {"arealg", d->arealg, E}, {"ss", d->ss, E},
        {"elemMass", d->elemMass, E}, {"delx_xi", d->delx_xi, E},
        {"delx_eta", d->delx_eta, E}, {"delx_zeta", d->delx_zeta, E},
        {"delv_xi", d->delv_xi, E}, {"delv_eta", d->delv_eta, E},
        {"delv_zeta", d->delv_zeta, E}, {"dxx", d->dxx, E}, {"dyy", d->dyy, E},
        {"dzz", d->dzz, E}};
    for (size_t i = 0; i < sizeof(t) / sizeof(t[0]); ++i)
        if (!strcmp(t[i].nm, name)) {
            if (n) *n = t[i].len;
            return t[i].p;
        }
    return NULL;
}

int *orc_field_i32(orc_domain *d, const char *name, size_t *n)
{
    const size_t E = (size_t)d->numElem;
    struct { const char *nm; int *p; size_t len; } t[] = {
        {"nodelist", d->nodelist, 8 * E}, {"lxim", d->lxim, E}, {"lxip", d->lxip, E},
        {"letam", d->letam, E}, {"letap", d->letap, E}, {"lzetam", d->lzetam, E},
        {"lzetap", d->lzetap, E}, {"elemBC", d->elemBC, E},
        {"regNumList", d->regNumList, E}, {"regElemSize", d->regElemSize, (size_t)d->numReg},
        {"symmX", d->symmX, (size_t)d->nsymm}, {"symmY", d->symmY, (size_t)d->nsymm},
        {"symmZ", d->symmZ, (size_t)d->nsymm},
        {"nodeElemStart", d->nodeElemStart, (size_t)d->numNode + 1},
        {"nodeElemCornerList", d->nodeElemCornerList, 8 * E}};
    for (size_t i = 0; i < sizeof(t) / sizeof(t[0]); ++i)
        if (!strcmp(t[i].nm, name)) {
            if (n) *n = t[i].len;
            return t[i].p;
        }
    return NULL;
}

#define SCALARS(X)                                                                   \
    X(time) X(deltatime) X(dtcourant) X(dthydro) X(stoptime) X(dtmax) X(dtfixed)     \
    X(deltatimemultlb) X(deltatimemultub) X(hgcoef)

double orc_get_scalar(orc_domain *d, const char *name)
{
#define G(f) if (!strcmp(name, #f)) return d->f;
    SCALARS(G)
#undef G
    if (!strcmp(name, "cycle")) return d->cycle;
    if (!strcmp(name, "numElem")) return d->numElem;
    if (!strcmp(name, "numNode")) return d->numNode;
    if (!strcmp(name, "numReg")) return d->numReg;
    return NAN;
}

int orc_set_scalar(orc_domain *d, const char *name, double value)
{
#define S(f) if (!strcmp(name, #f)) { d->f = value; return 0; }
    SCALARS(S)
#undef S
    if (!strcmp(name, "cycle")) { d->cycle = (int)value; return 0; }
    return 1;
}
