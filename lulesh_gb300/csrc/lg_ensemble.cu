// lg_ensemble.cu -- many independent Sedov problems advanced together.
//
// The problems' fields are concatenated into one set of device arrays (node
// and element ids offset per problem), so each phase of the cycle is ONE
// grid-stride launch over every problem's elements or nodes; each element and
// node knows its problem, each problem keeps its own control block (its own
// time step, cycle count, stop test and error status) and hourglass
// coefficient.  The cycle is replayed from CUDA graphs.  Block size and grid
// shape of each kernel are chosen by a small autotuner that times the
// candidates on the actual problem set and then restores the initial state.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lg_device.h"
#include "lg_kernelset.h"
#include "lg_problem.h"
#include "lulesh_gb300.h"

namespace lg {
int record_error(int code, const char *msg);
cudaError_t device_setup(const DevState &s, int nx, double einit, bool topology,
                         cudaStream_t stream, int eoff, int noff, long long tstride, int pid);
cudaError_t device_inv_mass(const double *m, double *inv, long long n, cudaStream_t stream);
}

namespace {

int err(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int err(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return lg::record_error(code, buf);
}

#define EN_CUDA(call)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return err(LG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),      \
                       __FILE__, __LINE__);                                               \
    } while (0)

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// splitmix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): the ensemble sampler's generator
struct SplitMix64 {
    unsigned long long s;
    unsigned long long next()
    {
        unsigned long long z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
    int uniform_int(int lo, int hi) { return lo + (int)(uniform() * (double)(hi - lo + 1)); }
};

constexpr int kBlockChoices[3] = {64, 128, 256};

}  // namespace

struct lg_ensemble {
    int nprob = 0;
    int precision = LG_FP64;
    int device = 0;
    std::vector<lg_opts> opts;
    std::vector<lg::Problem> prob;
    std::vector<long long> eoff, noff;  // first element / node of each problem
    long long E = 0, N = 0;
    lg::DevState ds{};
    const lg::KernelSet *ks = nullptr;
    void *arena = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<lg::Ctl> h_ctl;
    lg::Ctl *pinned_ctl = nullptr;
    int sms = 1;
    int bs[lg::K_COUNT] = {128, 128, 128, 128};
    bool persistent[lg::K_COUNT] = {true, true, true, true};
    cudaGraphExec_t g1 = nullptr, g16 = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    long long launches = 0;
};

namespace {

int grid_of(lg_ensemble *en, int id)
{
    const long long count = (id == lg::K_NODES) ? en->N : en->E;
    const int b = en->bs[id];
    const long long cover = (count + b - 1) / b;
    if (!en->persistent[id]) return (int)std::max(1LL, cover);
    const long long res = (long long)en->ks->occupancy(id, b) * en->sms;
    return (int)std::max(1LL, std::min(cover, res));
}

void enqueue_cycle(lg_ensemble *en)
{
    for (int id = 0; id < lg::K_COUNT; ++id)
        en->ks->launch_batched(id, en->ds, en->bs[id], grid_of(en, id), en->stream);
}

void drop_graphs(lg_ensemble *en)
{
    if (en->g1) cudaGraphExecDestroy(en->g1);
    if (en->g16) cudaGraphExecDestroy(en->g16);
    en->g1 = en->g16 = nullptr;
}

int capture(lg_ensemble *en, int ncycles, cudaGraphExec_t *out)
{
    cudaGraph_t g = nullptr;
    EN_CUDA(cudaStreamBeginCapture(en->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < ncycles; ++i) enqueue_cycle(en);
    EN_CUDA(cudaStreamEndCapture(en->stream, &g));
    const cudaError_t e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return err(LG_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    return LG_OK;
}

int read_ctl(lg_ensemble *en)
{
    EN_CUDA(cudaMemcpyAsync(en->pinned_ctl, en->ds.ctl, sizeof(lg::Ctl) * en->nprob,
                            cudaMemcpyDeviceToHost, en->stream));
    EN_CUDA(cudaStreamSynchronize(en->stream));
    std::copy(en->pinned_ctl, en->pinned_ctl + en->nprob, en->h_ctl.begin());
    return LG_OK;
}

int write_ctl(lg_ensemble *en)
{
    std::copy(en->h_ctl.begin(), en->h_ctl.end(), en->pinned_ctl);
    EN_CUDA(cudaMemcpyAsync(en->ds.ctl, en->pinned_ctl, sizeof(lg::Ctl) * en->nprob,
                            cudaMemcpyHostToDevice, en->stream));
    EN_CUDA(cudaStreamSynchronize(en->stream));
    return LG_OK;
}

template <typename T>
int put(lg_ensemble *en, T *dst, const std::vector<T> &src)
{
    if (src.empty()) return LG_OK;
    EN_CUDA(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice,
                            en->stream));
    EN_CUDA(cudaStreamSynchronize(en->stream));
    return LG_OK;
}

// node / element double fields of one problem, by accessor name
std::vector<double> *host_f64(lg::Problem &p, const char *name, bool *node)
{
    struct { const char *n; std::vector<double> *v; bool node; } t[] = {
        {"x", &p.x, true}, {"y", &p.y, true}, {"z", &p.z, true}, {"xd", &p.xd, true},
        {"yd", &p.yd, true}, {"zd", &p.zd, true}, {"xdd", &p.xdd, true}, {"ydd", &p.ydd, true},
        {"zdd", &p.zdd, true}, {"fx", &p.fx, true}, {"fy", &p.fy, true}, {"fz", &p.fz, true},
        {"nodalMass", &p.nodalMass, true}, {"e", &p.e, false}, {"p", &p.p, false},
        {"q", &p.q, false}, {"ql", &p.ql, false}, {"qq", &p.qq, false}, {"v", &p.v, false},
        {"volo", &p.volo, false}, {"vnew", &p.vnew, false}, {"delv", &p.delv, false},
        {"vdov", &p.vdov, false}, {"arealg", &p.arealg, false}, {"ss", &p.ss, false},
        {"elemMass", &p.elemMass, false}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) {
            *node = f.node;
            return f.v;
        }
    return nullptr;
}

double *dev_f64(lg::DevState &s, const char *name)
{
    struct { const char *n; double *p; } t[] = {
        {"x", s.x}, {"y", s.y}, {"z", s.z}, {"xd", s.xd}, {"yd", s.yd}, {"zd", s.zd},
        {"xdd", s.xdd}, {"ydd", s.ydd}, {"zdd", s.zdd}, {"fx", s.fx}, {"fy", s.fy},
        {"fz", s.fz}, {"nodalMass", s.nodalMass}, {"e", s.e}, {"p", s.p}, {"q", s.q},
        {"ql", s.ql}, {"qq", s.qq}, {"v", s.v}, {"volo", s.volo}, {"vnew", s.vnew},
        {"delv", s.delv}, {"vdov", s.vdov}, {"arealg", s.arealg}, {"ss", s.ss},
        {"elemMass", s.elemMass}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) return f.p;
    return nullptr;
}

// member i's view of the concatenated arrays: every pointer moved to its
// first element or node, its own sizes
lg::DevState member_view(const lg_ensemble *en, int i)
{
    lg::DevState v = en->ds;
    const long long eo = en->eoff[i], no = en->noff[i];
    v.E = en->prob[i].numElem;
    v.N = en->prob[i].numNode;
    double **nodef[14] = {&v.x, &v.y, &v.z, &v.xd, &v.yd, &v.zd, &v.xdd, &v.ydd, &v.zdd,
                          &v.fx, &v.fy, &v.fz, &v.nodalMass, &v.invMass};
    for (auto f : nodef) *f += no;
    double **elemf[19] = {&v.e, &v.p, &v.q, &v.ql, &v.qq, &v.v, &v.volo, &v.vnew, &v.delv,
                          &v.vdov, &v.arealg, &v.ss, &v.elemMass, &v.delx_xi, &v.delx_eta,
                          &v.delx_zeta, &v.delv_xi, &v.delv_eta, &v.delv_zeta};
    for (auto f : elemf) *f += eo;
    int **conn[7] = {&v.lxim, &v.lxip, &v.letam, &v.letap, &v.lzetam, &v.lzetap, &v.elemBC};
    for (auto c : conn) *c += eo;
    v.nodelist += 8 * eo;
    v.nodelistT += eo;
    v.nodeElemStart += no;
    v.nodeElemCornerList += 8 * eo;
    v.symm += no;
    v.elemProb += eo;
    v.nodeProb += no;
    return v;
}

// every member's set-up state, built on the device (lg_setup.cu): the
// topology too when `topology`; then the dt slots and control blocks
int setup_members(lg_ensemble *en, bool topology)
{
    for (int i = 0; i < en->nprob; ++i) {
        const lg_opts &o = en->opts[i];
        EN_CUDA(lg::device_setup(member_view(en, i), o.nx, lg::sedov_einit(o.nx, o.einit_factor),
                                 topology, en->stream, (int)en->eoff[i], (int)en->noff[i], en->E,
                                 i));
    }
    const unsigned long long big = [] {
        double v = 1.0e+20;
        unsigned long long b;
        memcpy(&b, &v, sizeof b);
        return b;
    }();
    std::vector<unsigned long long> slots(2 * (size_t)en->nprob, big);
    int st;
    if ((st = put(en, en->ds.dtSlots, slots))) return st;
    EN_CUDA(cudaMemsetAsync(en->ds.gridCounter, 0, sizeof(unsigned), en->stream));
    for (int i = 0; i < en->nprob; ++i) {
        const lg::TimeState &t = en->prob[i].t;
        lg::Ctl c;
        memset(&c, 0, sizeof c);
        c.time = t.time;
        c.deltatime = t.deltatime;
        c.dtcourant = t.dtcourant;
        c.dthydro = t.dthydro;
        c.stoptime = t.stoptime;
        c.dtmax = t.dtmax;
        c.dtfixed = t.dtfixed;
        c.dtmultlb = t.deltatimemultlb;
        c.dtmultub = t.deltatimemultub;
        c.cycle = t.cycle;
        en->h_ctl[i] = c;
    }
    return write_ctl(en);
}

// region order over all members (global element ids, each member's regions
// in turn, most EOS repetitions first as in lg::region_visit_order) with the
// EOS repetition counts, and the members' hgcoef
int upload_regions(lg_ensemble *en)
{
    const long long E = en->E;
    std::vector<int> perm(E), rep(E);
    std::vector<double> hg(en->nprob);
    long long pos = 0;
    for (int pi = 0; pi < en->nprob; ++pi) {
        const lg::Problem &p = en->prob[pi];
        const long long eo = en->eoff[pi];
        hg[pi] = p.k.hgcoef;
        for (const int r : lg::region_visit_order(p.numReg, p.cost)) {
            const int rr = lg::region_rep(r, p.numReg, p.cost);
            for (int e : p.regElemlist[r]) {
                perm[pos] = (int)(e + eo);
                rep[pos] = rr;
                ++pos;
            }
        }
    }
    if (pos != E) return err(LG_ERR_INVALID, "region sets do not cover all elements");
    int st;
    if ((st = put(en, en->ds.regPerm, perm)) || (st = put(en, en->ds.regRep, rep)) ||
        (st = put(en, en->ds.hgcoefs, hg)))
        return st;
    return LG_OK;
}

int begin_steps(lg_ensemble *en, int ncycles)
{
    int st;
    if ((st = read_ctl(en))) return st;
    for (int i = 0; i < en->nprob; ++i) {
        lg::Ctl &c = en->h_ctl[i];
        c.cycle_limit = (int)std::min<long long>(en->opts[i].its, (long long)c.cycle + ncycles);
    }
    if ((st = write_ctl(en))) return st;
    if (!en->g1 && (st = capture(en, 1, &en->g1))) return st;
    if (!en->g16 && (st = capture(en, 16, &en->g16))) return st;
    return LG_OK;
}

int launch_cycles(lg_ensemble *en, int ncycles)
{
    en->ks->begin_all(en->ds.ctl, en->nprob, en->stream);
    int left = ncycles;
    while (left >= 16) {
        EN_CUDA(cudaGraphLaunch(en->g16, en->stream));
        left -= 16;
    }
    while (left-- > 0) EN_CUDA(cudaGraphLaunch(en->g1, en->stream));
    EN_CUDA(cudaGetLastError());
    en->launches += 1 + 4LL * ncycles;
    return LG_OK;
}

int first_status(lg_ensemble *en)
{
    for (int i = 0; i < en->nprob; ++i)
        if (en->h_ctl[i].status) return en->h_ctl[i].status;
    return LG_OK;
}

}  // namespace

extern "C" {

int lg_ensemble_sample(int nprob, unsigned long long seed, lg_opts *out)
{
    if (nprob < 1 || !out) return err(LG_ERR_INVALID, "invalid argument");
    SplitMix64 g{seed};
    for (int i = 0; i < nprob; ++i) {
        lg_opts &o = out[i];
        lg_default_opts(&o);
        o.nx = g.uniform_int(16, 64);
        o.einit_factor = std::exp(std::log(0.5) + g.uniform() * (std::log(2.0) - std::log(0.5)));
        o.hgcoef = 1.0 + 2.0 * g.uniform();
        o.numReg = g.uniform_int(4, 16);
        o.balance = 1;
        o.cost = 1;
        o.its = 300;
    }
    return LG_OK;
}

int lg_ensemble_create(int nprob, const lg_opts *opts, lg_ensemble **out)
{
    if (nprob < 1 || nprob > 65535 || !opts || !out) return err(LG_ERR_INVALID, "invalid argument");
    *out = nullptr;
    const lg::KernelSet *ks = nullptr;
    switch (opts[0].precision) {
    case LG_FP64: ks = lg::kernels_fp64_strict(); break;
    case LG_FP64_FMA: ks = lg::kernels_fp64_fma(); break;
    case LG_MIXED: ks = lg::kernels_mixed(); break;
    default: return err(LG_ERR_INVALID, "precision %d not available", opts[0].precision);
    }
    lg_ensemble *en = new lg_ensemble();
    en->nprob = nprob;
    en->precision = opts[0].precision;
    en->device = opts[0].device;
    en->ks = ks;
    en->opts.assign(opts, opts + nprob);
    auto fail = [&](int code) {
        lg_ensemble_destroy(en);
        return code;
    };
    if (cudaSetDevice(en->device) != cudaSuccess)
        return fail(err(LG_ERR_CUDA, "cudaSetDevice(%d) failed", en->device));
    for (int i = 0; i < nprob; ++i) {
        const lg_opts &o = opts[i];
        if (o.nx < 1 || o.numReg < 1 || o.its < 0 || (long long)o.nx * o.nx * o.nx * 8 > 2147483647LL)
            return fail(err(LG_ERR_INVALID, "problem %d: invalid size", i));
        if (o.cost < 0)  // repetition counts 1+cost and 10(1+cost) must be positive
            return fail(err(LG_ERR_INVALID, "problem %d: cost=%d is negative", i, o.cost));
        // sizes, constants, time state and regions; the mesh and fields are
        // built on the device
        en->prob.push_back(lg::build_sedov_scalars(o.nx, o.numReg, o.balance, o.cost, o.hgcoef,
                                                   o.einit_factor));
        en->eoff.push_back(en->E);
        en->noff.push_back(en->N);
        en->E += en->prob.back().numElem;
        en->N += en->prob.back().numNode;
    }
    if (8 * en->E > 2147483647LL)
        return fail(err(LG_ERR_INVALID, "ensemble exceeds the 32-bit corner index range"));
    const long long E = en->E, N = en->N;

    // one arena: the same buffers as a single problem, over all problems
    size_t total = 0;
    auto add = [&](size_t bytes) {
        const size_t off = total;
        total = align256(total + bytes);
        return off;
    };
    size_t o_node[14], o_elem[19];
    for (auto &o : o_node) o = add(8 * N);
    for (auto &o : o_elem) o = add(8 * E);
    const size_t o_corner = add(8 * 48 * E), o_nl = add(4 * 8 * E), o_nlT = add(4 * 8 * E);
    size_t o_conn[7];
    for (auto &o : o_conn) o = add(4 * E);
    const size_t o_perm = add(4 * E), o_rep = add(4 * E), o_nes = add(4 * (N + 1)),
                 o_ncl = add(4 * 8 * E), o_symm = add(N), o_eprob = add(2 * E),
                 o_nprob = add(2 * N), o_hg = add(8 * (size_t)nprob),
                 o_slots = add(16 * (size_t)nprob), o_cnt = add(4),
                 o_ctl = add(sizeof(lg::Ctl) * (size_t)nprob);
    if (cudaMalloc(&en->arena, total) != cudaSuccess)
        return fail(err(LG_ERR_NOMEM, "cudaMalloc(%zu bytes) failed", total));
    char *b = static_cast<char *>(en->arena);
    lg::DevState &s = en->ds;
    s.E = (int)E;
    s.nItems = (int)E;
    s.N = (int)N;
    s.nx = 0;
    s.numReg = 0;
    s.nprob = nprob;
    double **nodef[14] = {&s.x, &s.y, &s.z, &s.xd, &s.yd, &s.zd, &s.xdd, &s.ydd, &s.zdd,
                          &s.fx, &s.fy, &s.fz, &s.nodalMass, &s.invMass};
    for (int i = 0; i < 14; ++i) *nodef[i] = reinterpret_cast<double *>(b + o_node[i]);
    double **elemf[19] = {&s.e, &s.p, &s.q, &s.ql, &s.qq, &s.v, &s.volo, &s.vnew, &s.delv,
                          &s.vdov, &s.arealg, &s.ss, &s.elemMass, &s.delx_xi, &s.delx_eta,
                          &s.delx_zeta, &s.delv_xi, &s.delv_eta, &s.delv_zeta};
    for (int i = 0; i < 19; ++i) *elemf[i] = reinterpret_cast<double *>(b + o_elem[i]);
    s.corner = reinterpret_cast<double *>(b + o_corner);
    s.nodelist = reinterpret_cast<int *>(b + o_nl);
    s.nodelistT = reinterpret_cast<int *>(b + o_nlT);
    int **conn[7] = {&s.lxim, &s.lxip, &s.letam, &s.letap, &s.lzetam, &s.lzetap, &s.elemBC};
    for (int i = 0; i < 7; ++i) *conn[i] = reinterpret_cast<int *>(b + o_conn[i]);
    s.regNumList = nullptr;
    s.regPerm = reinterpret_cast<int *>(b + o_perm);
    s.regRep = reinterpret_cast<int *>(b + o_rep);
    s.nodeElemStart = reinterpret_cast<int *>(b + o_nes);
    s.nodeElemCornerList = reinterpret_cast<int *>(b + o_ncl);
    s.symm = reinterpret_cast<uint8_t *>(b + o_symm);
    s.elemProb = reinterpret_cast<uint16_t *>(b + o_eprob);
    s.nodeProb = reinterpret_cast<uint16_t *>(b + o_nprob);
    s.hgcoefs = reinterpret_cast<double *>(b + o_hg);
    s.dtSlots = reinterpret_cast<unsigned long long *>(b + o_slots);
    s.gridCounter = reinterpret_cast<unsigned *>(b + o_cnt);
    s.ctl = reinterpret_cast<lg::Ctl *>(b + o_ctl);
    s.dt_partial = nullptr;
    s.dt_blocks = 0;
    lg::Constants k;  // shared constants; hgcoef is per problem
    s.prm.e_cut = k.e_cut; s.prm.p_cut = k.p_cut; s.prm.q_cut = k.q_cut;
    s.prm.v_cut = k.v_cut; s.prm.u_cut = k.u_cut; s.prm.hgcoef = k.hgcoef;
    s.prm.ss4o3 = k.ss4o3; s.prm.qstop = k.qstop; s.prm.monoq_max_slope = k.monoq_max_slope;
    s.prm.monoq_limiter_mult = k.monoq_limiter_mult; s.prm.qlc_monoq = k.qlc_monoq;
    s.prm.qqc_monoq = k.qqc_monoq; s.prm.qqc = k.qqc; s.prm.eosvmax = k.eosvmax;
    s.prm.eosvmin = k.eosvmin; s.prm.pmin = k.pmin; s.prm.emin = k.emin;
    s.prm.dvovmax = k.dvovmax; s.prm.refdens = k.refdens;

    en->h_ctl.assign(nprob, lg::Ctl{});
    if (cudaStreamCreateWithFlags(&en->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&en->pinned_ctl, sizeof(lg::Ctl) * nprob) != cudaSuccess ||
        cudaEventCreate(&en->ev0) != cudaSuccess || cudaEventCreate(&en->ev1) != cudaSuccess)
        return fail(err(LG_ERR_CUDA, "stream/event/pinned allocation failed"));
    int dev = en->device, sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    en->sms = sms > 0 ? sms : 1;
    if (cudaMemsetAsync(en->arena, 0, total, en->stream) != cudaSuccess)
        return fail(err(LG_ERR_CUDA, "cudaMemset failed"));
    int st;
    if ((st = upload_regions(en)) || (st = setup_members(en, true))) return fail(st);
    *out = en;
    return LG_OK;
}

void lg_ensemble_destroy(lg_ensemble *en)
{
    if (!en) return;
    cudaSetDevice(en->device);
    if (en->stream) cudaStreamSynchronize(en->stream);
    drop_graphs(en);
    if (en->ev0) cudaEventDestroy(en->ev0);
    if (en->ev1) cudaEventDestroy(en->ev1);
    if (en->pinned_ctl) cudaFreeHost(en->pinned_ctl);
    if (en->arena) cudaFree(en->arena);
    if (en->stream) cudaStreamDestroy(en->stream);
    delete en;
}

int lg_ensemble_step(lg_ensemble *en, int ncycles)
{
    if (!en || ncycles < 0) return err(LG_ERR_INVALID, "invalid argument");
    EN_CUDA(cudaSetDevice(en->device));
    int st;
    if (ncycles == 0) return LG_OK;
    if ((st = begin_steps(en, ncycles)) || (st = launch_cycles(en, ncycles)) ||
        (st = read_ctl(en)))
        return st;
    return first_status(en);
}

int lg_ensemble_step_timed(lg_ensemble *en, int ncycles, double *ms)
{
    if (!en || ncycles < 0 || !ms) return err(LG_ERR_INVALID, "invalid argument");
    EN_CUDA(cudaSetDevice(en->device));
    int st;
    if ((st = begin_steps(en, ncycles))) return st;
    EN_CUDA(cudaEventRecord(en->ev0, en->stream));
    if ((st = launch_cycles(en, ncycles))) return st;
    EN_CUDA(cudaEventRecord(en->ev1, en->stream));
    EN_CUDA(cudaEventSynchronize(en->ev1));
    float f = 0.f;
    EN_CUDA(cudaEventElapsedTime(&f, en->ev0, en->ev1));
    *ms = f;
    if ((st = read_ctl(en))) return st;
    return first_status(en);
}

int lg_ensemble_reset(lg_ensemble *en)
{
    if (!en) return err(LG_ERR_INVALID, "null handle");
    EN_CUDA(cudaSetDevice(en->device));
    EN_CUDA(cudaStreamSynchronize(en->stream));
    return setup_members(en, false);
}

int lg_ensemble_info(lg_ensemble *en, long long *total_elems, long long *total_nodes,
                     long long *launches)
{
    if (!en) return err(LG_ERR_INVALID, "null handle");
    if (total_elems) *total_elems = en->E;
    if (total_nodes) *total_nodes = en->N;
    if (launches) *launches = en->launches;
    return LG_OK;
}

int lg_ensemble_get_field(lg_ensemble *en, int prob, const char *name, void *dst, size_t n)
{
    if (!en || !name || prob < 0 || prob >= en->nprob || (!dst && n))
        return err(LG_ERR_INVALID, "invalid argument");
    EN_CUDA(cudaSetDevice(en->device));
    lg::Problem &p = en->prob[prob];
    bool node = false;
    if (host_f64(p, name, &node)) {
        const size_t cnt = node ? p.numNode : p.numElem;
        if (n != cnt) return err(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name, cnt, n);
        const double *src = dev_f64(en->ds, name) + (node ? en->noff[prob] : en->eoff[prob]);
        EN_CUDA(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToHost,
                                en->stream));
        EN_CUDA(cudaStreamSynchronize(en->stream));
        return LG_OK;
    }
    if (!strcmp(name, "regNumList")) {
        if (n != p.regNumList.size()) return err(LG_ERR_INVALID, "field '%s' size mismatch", name);
        memcpy(dst, p.regNumList.data(), n * sizeof(int));
        return LG_OK;
    }
    // topology, member-local ids (the device arrays hold ensemble-wide ids)
    const bool nl = !strcmp(name, "nodelist");
    if (!nl && strcmp(name, "elemBC") != 0) return err(LG_ERR_INVALID, "unknown field '%s'", name);
    const size_t cnt = (nl ? 8 : 1) * (size_t)p.numElem;
    if (n != cnt) return err(LG_ERR_INVALID, "field '%s' size mismatch", name);
    const int *src = nl ? en->ds.nodelist + 8 * en->eoff[prob] : en->ds.elemBC + en->eoff[prob];
    EN_CUDA(cudaMemcpyAsync(dst, src, cnt * sizeof(int), cudaMemcpyDeviceToHost, en->stream));
    EN_CUDA(cudaStreamSynchronize(en->stream));
    if (nl) {
        int *d = static_cast<int *>(dst);
        for (size_t i = 0; i < cnt; ++i) d[i] -= (int)en->noff[prob];
    }
    return LG_OK;
}

int lg_ensemble_set_field(lg_ensemble *en, int prob, const char *name, const void *src, size_t n)
{
    if (!en || !name || prob < 0 || prob >= en->nprob || (!src && n))
        return err(LG_ERR_INVALID, "invalid argument");
    EN_CUDA(cudaSetDevice(en->device));
    lg::Problem &p = en->prob[prob];
    bool node = false;
    if (!host_f64(p, name, &node))
        return err(LG_ERR_INVALID, "'%s' is not a double field of a member", name);
    const size_t cnt = node ? p.numNode : p.numElem;
    if (n != cnt) return err(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name, cnt, n);
    double *dst = dev_f64(en->ds, name) + (node ? en->noff[prob] : en->eoff[prob]);
    EN_CUDA(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, en->stream));
    if (!strcmp(name, "nodalMass"))  // RN(1 / m) of the member's masses, on the device
        EN_CUDA(lg::device_inv_mass(dst, en->ds.invMass + en->noff[prob], (long long)cnt,
                                    en->stream));
    EN_CUDA(cudaStreamSynchronize(en->stream));
    return LG_OK;
}

int lg_ensemble_get_scalar(lg_ensemble *en, int prob, const char *name, double *value)
{
    if (!en || !name || !value || prob < 0 || prob >= en->nprob)
        return err(LG_ERR_INVALID, "invalid argument");
    EN_CUDA(cudaSetDevice(en->device));
    int st;
    if ((st = read_ctl(en))) return st;
    const lg::Ctl &c = en->h_ctl[prob];
    const lg_opts &o = en->opts[prob];
    struct { const char *n; double v; } t[] = {
        {"time", c.time}, {"deltatime", c.deltatime}, {"dtcourant", c.dtcourant},
        {"dthydro", c.dthydro}, {"cycle", (double)c.cycle}, {"status", (double)c.status},
        {"numElem", (double)en->prob[prob].numElem}, {"numNode", (double)en->prob[prob].numNode},
        {"nx", (double)o.nx}, {"numReg", (double)o.numReg}, {"hgcoef", o.hgcoef},
        {"einit_factor", o.einit_factor}, {"its", (double)o.its}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) {
            *value = f.v;
            return LG_OK;
        }
    return err(LG_ERR_INVALID, "unknown scalar '%s'", name);
}

int lg_ensemble_autotune(lg_ensemble *en, int ncycles, int *block_sizes, int *persistent)
{
    if (!en || ncycles < 1) return err(LG_ERR_INVALID, "invalid argument");
    EN_CUDA(cudaSetDevice(en->device));
    int st;
    if ((st = begin_steps(en, 1 << 30))) return st;  // no stop for the tuning cycles
    en->ks->begin_all(en->ds.ctl, en->nprob, en->stream);
    cudaEvent_t a, b;
    EN_CUDA(cudaEventCreate(&a));
    EN_CUDA(cudaEventCreate(&b));
    // each kernel in turn: every (block size, grid shape) candidate for
    // ncycles cycles, the other kernels at their current choice
    for (int id = 0; id < lg::K_COUNT; ++id) {
        float best = 1e30f;
        int best_bs = en->bs[id];
        bool best_p = en->persistent[id];
        for (int bsi = 0; bsi < 3; ++bsi)
            for (int pers = 0; pers < 2; ++pers) {
                en->bs[id] = kBlockChoices[bsi];
                en->persistent[id] = pers != 0;
                float total = 0.f;
                for (int c = 0; c < ncycles; ++c)
                    for (int k = 0; k < lg::K_COUNT; ++k) {
                        if (k == id) EN_CUDA(cudaEventRecord(a, en->stream));
                        en->ks->launch_batched(k, en->ds, en->bs[k], grid_of(en, k), en->stream);
                        if (k == id) {
                            EN_CUDA(cudaEventRecord(b, en->stream));
                            EN_CUDA(cudaEventSynchronize(b));
                            float ms = 0.f;
                            EN_CUDA(cudaEventElapsedTime(&ms, a, b));
                            total += ms;
                        }
                    }
                if (total < best) {
                    best = total;
                    best_bs = en->bs[id];
                    best_p = en->persistent[id];
                }
            }
        en->bs[id] = best_bs;
        en->persistent[id] = best_p;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    EN_CUDA(cudaGetLastError());
    for (int id = 0; id < lg::K_COUNT; ++id) {
        if (block_sizes) block_sizes[id] = en->bs[id];
        if (persistent) persistent[id] = en->persistent[id] ? 1 : 0;
    }
    drop_graphs(en);
    return lg_ensemble_reset(en);
}

}  // extern "C"
