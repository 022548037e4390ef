// lg_api.cu -- the C ABI (include/lulesh_gb300.h): handle, device memory,
// upload/download, the cycle loop under CUDA graphs, and the report.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lg_device.h"
#include "lg_adjoint.h"
#include "lg_kernelset.h"
#include "lg_problem.h"
#include "lulesh_gb300.h"

namespace {

thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define LG_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t err_ = (call);                                                      \
        if (err_ != cudaSuccess)                                                        \
            return set_error(LG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(err_), \
                             __FILE__, __LINE__);                                       \
    } while (0)

constexpr size_t kAlign = 256;
size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

// Sub-allocations of the single device arena.
struct Layout {
    size_t total = 0;
    template <typename T>
    size_t add(size_t count)
    {
        const size_t off = total;
        total = align_up(total + count * sizeof(T));
        return off;
    }
};

}  // namespace

namespace lg {
int record_error(int code, const char *msg) { return set_error(code, "%s", msg); }
}  // namespace lg

struct lg_domain {
    lg_opts opts{};
    // host mirror: sizes, constants, time state and regions always; the
    // initial double fields when mirror_state (host-only handles), the
    // integer topology when mirror_topo (host-only handles, or downloaded on
    // first use from the device that built it)
    lg::Problem prob;
    bool mirror_state = false, mirror_topo = false;
    lg::DevState ds{};
    const lg::KernelSet *ks = nullptr;
    void *arena = nullptr;
    size_t arena_bytes = 0;
    cudaStream_t stream = nullptr;
    lg::Ctl *h_ctl = nullptr;  // pinned host copy of the control block
    cudaGraphExec_t graph1 = nullptr, graph16 = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int its = 9999999;
    // k_material's work items: threads one wave of it keeps resident, and the
    // capacity of regPerm / regRep (upload_regions)
    int resident = 0, item_cap = 0;
    bool host_only = false;  // device < 0: problem set-up only, no GPU
    long long launches = 0;  // kernels queued by this handle
    // frozen / recorded time steps (lg_dt_freeze, lg_dt_record)
    double *d_dtfrozen = nullptr, *d_dtrec = nullptr;
    int dtfrozen_len = 0, dtrec_len = 0;
    std::vector<double> h_dtfrozen;
};

namespace lg {
cudaError_t device_setup(const DevState &s, int nx, double einit, bool topology,
                         cudaStream_t stream, int eoff = 0, int noff = 0, long long tstride = 0,
                         int pid = 0);
cudaError_t device_verify(const double *e, int nx, double *scratch, double *out,
                          cudaStream_t stream);
cudaError_t device_inv_mass(const double *m, double *inv, long long n, cudaStream_t stream);
}  // namespace lg

namespace {

int ensure_device(lg_domain *d)
{
    if (d->host_only)
        return set_error(LG_ERR_STATE, "handle was created host-only (device < 0)");
    LG_CUDA(cudaSetDevice(d->opts.device));
    return LG_OK;
}

void drop_graphs(lg_domain *d)
{
    if (d->graph1) cudaGraphExecDestroy(d->graph1);
    if (d->graph16) cudaGraphExecDestroy(d->graph16);
    d->graph1 = d->graph16 = nullptr;
}

lg::Params make_params(const lg::Constants &k)
{
    lg::Params p;
    p.e_cut = k.e_cut; p.p_cut = k.p_cut; p.q_cut = k.q_cut; p.v_cut = k.v_cut;
    p.u_cut = k.u_cut; p.hgcoef = k.hgcoef; p.ss4o3 = k.ss4o3; p.qstop = k.qstop;
    p.monoq_max_slope = k.monoq_max_slope; p.monoq_limiter_mult = k.monoq_limiter_mult;
    p.qlc_monoq = k.qlc_monoq; p.qqc_monoq = k.qqc_monoq; p.qqc = k.qqc;
    p.eosvmax = k.eosvmax; p.eosvmin = k.eosvmin; p.pmin = k.pmin; p.emin = k.emin;
    p.dvovmax = k.dvovmax; p.refdens = k.refdens;
    return p;
}

template <typename T>
int upload(lg_domain *d, T *dst, const std::vector<T> &src)
{
    if (src.empty()) return LG_OK;
    LG_CUDA(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice,
                            d->stream));
    return LG_OK;
}

// invMass = RN(1 / nodalMass) from the masses on the device (the nodal
// accelerations of every path)
int refresh_inv_mass(lg_domain *d)
{
    LG_CUDA(lg::device_inv_mass(d->ds.nodalMass, d->ds.invMass, d->ds.N, d->stream));
    return LG_OK;
}

// regNumList and the material phase's work items (DevState::nItems), built
// on the host by lg::build_material_items.  Large meshes: one item per
// element in region order, the regions with the most EOS repetitions first,
// each region's elements in their ascending regElemlist order.  Small
// meshes, where the costly regions would fill too few blocks to keep every
// SM's FP64 pipe busy (at s=30 the 8,445 elements with 20 repetitions make 66
// blocks for 152 SMs), run the phase split (DevState::matSplit): repetition
// items of equal shares carry the EOS work, and the per-element parts run
// once per element.  The work done and the results are the same either way.
int upload_regions(lg_domain *d)
{
    const lg::Problem &p = d->prob;
    std::vector<int> perm, rep;
    const bool split = lg::build_material_items(p, d->resident, perm, rep);
    if (!split && (int)perm.size() != p.numElem)
        return set_error(LG_ERR_INVALID, "region sets do not cover all elements");
    if ((long long)perm.size() > d->item_cap)
        return set_error(LG_ERR_STATE, "%zu work items exceed the capacity %d", perm.size(),
                         d->item_cap);
    int st;
    if ((st = upload(d, d->ds.regNumList, p.regNumList))) return st;
    if ((st = upload(d, d->ds.regPerm, perm))) return st;
    if ((st = upload(d, d->ds.regRep, rep))) return st;
    // the graphs hold the kernel arguments (nItems) and the material kernels
    // chosen for them
    if (d->ds.nItems != (int)perm.size() || d->ds.matSplit != (int)split) drop_graphs(d);
    d->ds.nItems = (int)perm.size();
    d->ds.matSplit = split ? 1 : 0;
    LG_CUDA(cudaStreamSynchronize(d->stream));
    return LG_OK;
}

// Kernel-side layouts derived from the host mirror's integer fields (see
// lg_device.h).
int upload_topology(lg_domain *d)
{
    const lg::Problem &p = d->prob;
    const int E = p.numElem, N = p.numNode;
    std::vector<int> nlT(8 * (size_t)E);
    for (int e = 0; e < E; ++e)
        for (int j = 0; j < 8; ++j) nlT[(size_t)j * E + e] = p.nodelist[8 * (size_t)e + j];
    std::vector<uint8_t> symm(N, 0);
    for (int n : p.symmX) symm[n] |= 1;
    for (int n : p.symmY) symm[n] |= 2;
    for (int n : p.symmZ) symm[n] |= 4;
    int st;
    if ((st = upload(d, d->ds.nodelist, p.nodelist))) return st;
    if ((st = upload(d, d->ds.nodelistT, nlT))) return st;
    if ((st = upload(d, d->ds.symm, symm))) return st;
    if ((st = upload(d, d->ds.nodeElemStart, p.nodeElemStart))) return st;
    if ((st = upload(d, d->ds.nodeElemCornerList, p.nodeElemCornerList))) return st;
    if ((st = upload(d, d->ds.lxim, p.lxim))) return st;
    if ((st = upload(d, d->ds.lxip, p.lxip))) return st;
    if ((st = upload(d, d->ds.letam, p.letam))) return st;
    if ((st = upload(d, d->ds.letap, p.letap))) return st;
    if ((st = upload(d, d->ds.lzetam, p.lzetam))) return st;
    if ((st = upload(d, d->ds.lzetap, p.lzetap))) return st;
    if ((st = upload(d, d->ds.elemBC, p.elemBC))) return st;
    return upload_regions(d);
}

template <typename T>
int download(lg_domain *d, std::vector<T> &dst, const T *src, size_t n)
{
    dst.resize(n);
    if (n) LG_CUDA(cudaMemcpyAsync(dst.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost,
                                   d->stream));
    return LG_OK;
}

// The integer topology in the host mirror: downloaded from the device that
// built it, once (afterwards the mirror is the master copy: lg_set_field
// edits it and uploads it).
int ensure_topology_mirror(lg_domain *d)
{
    if (d->host_only || d->mirror_topo) return LG_OK;
    lg::Problem &p = d->prob;
    const lg::DevState &s = d->ds;
    const size_t E = p.numElem, N = p.numNode;
    int st;
    if ((st = download(d, p.nodelist, s.nodelist, 8 * E))) return st;
    if ((st = download(d, p.lxim, s.lxim, E))) return st;
    if ((st = download(d, p.lxip, s.lxip, E))) return st;
    if ((st = download(d, p.letam, s.letam, E))) return st;
    if ((st = download(d, p.letap, s.letap, E))) return st;
    if ((st = download(d, p.lzetam, s.lzetam, E))) return st;
    if ((st = download(d, p.lzetap, s.lzetap, E))) return st;
    if ((st = download(d, p.elemBC, s.elemBC, E))) return st;
    if ((st = download(d, p.nodeElemStart, s.nodeElemStart, N + 1))) return st;
    if ((st = download(d, p.nodeElemCornerList, s.nodeElemCornerList, 8 * E))) return st;
    std::vector<uint8_t> symm;
    if ((st = download(d, symm, s.symm, N))) return st;
    LG_CUDA(cudaStreamSynchronize(d->stream));
    p.symmX.clear();
    p.symmY.clear();
    p.symmZ.clear();
    for (size_t n = 0; n < N; ++n) {  // ascending node order, as SetupSymmetryPlanes lists them
        if (symm[n] & 1) p.symmX.push_back((int)n);
        if (symm[n] & 2) p.symmY.push_back((int)n);
        if (symm[n] & 4) p.symmZ.push_back((int)n);
    }
    d->mirror_topo = true;
    return LG_OK;
}

// double fields that live on the device
bool find_f64(lg_domain *d, const char *name, double **ptr, size_t *count)
{
    lg::DevState &s = d->ds;
    const size_t N = s.N, E = s.E;
    struct { const char *n; double *p; size_t c; } t[] = {
        {"x", s.x, N}, {"y", s.y, N}, {"z", s.z, N}, {"xd", s.xd, N}, {"yd", s.yd, N},
        {"zd", s.zd, N}, {"xdd", s.xdd, N}, {"ydd", s.ydd, N}, {"zdd", s.zdd, N},
        {"fx", s.fx, N}, {"fy", s.fy, N}, {"fz", s.fz, N}, {"nodalMass", s.nodalMass, N},
        {"e", s.e, E}, {"p", s.p, E}, {"q", s.q, E}, {"ql", s.ql, E}, {"qq", s.qq, E},
        {"v", s.v, E}, {"volo", s.volo, E}, {"vnew", s.vnew, E}, {"delv", s.delv, E},
        {"vdov", s.vdov, E}, {"arealg", s.arealg, E}, {"ss", s.ss, E},
        {"elemMass", s.elemMass, E}, {"delx_xi", s.delx_xi, E}, {"delx_eta", s.delx_eta, E},
        {"delx_zeta", s.delx_zeta, E}, {"delv_xi", s.delv_xi, E}, {"delv_eta", s.delv_eta, E},
        {"delv_zeta", s.delv_zeta, E}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) {
            *ptr = f.p;
            *count = f.c;
            return true;
        }
    return false;
}

// double fields of the host mirror (the state built by set-up)
std::vector<double> *find_f64_host(lg_domain *d, const char *name)
{
    lg::Problem &p = d->prob;
    struct { const char *n; std::vector<double> *v; } t[] = {
        {"x", &p.x}, {"y", &p.y}, {"z", &p.z}, {"xd", &p.xd}, {"yd", &p.yd}, {"zd", &p.zd},
        {"xdd", &p.xdd}, {"ydd", &p.ydd}, {"zdd", &p.zdd}, {"fx", &p.fx}, {"fy", &p.fy},
        {"fz", &p.fz}, {"nodalMass", &p.nodalMass}, {"e", &p.e}, {"p", &p.p}, {"q", &p.q},
        {"ql", &p.ql}, {"qq", &p.qq}, {"v", &p.v}, {"volo", &p.volo}, {"vnew", &p.vnew},
        {"delv", &p.delv}, {"vdov", &p.vdov}, {"arealg", &p.arealg}, {"ss", &p.ss},
        {"elemMass", &p.elemMass}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) return f.v;
    return nullptr;
}

// integer fields, served from the host mirror
std::vector<int> *find_i32(lg_domain *d, const char *name)
{
    lg::Problem &p = d->prob;
    struct { const char *n; std::vector<int> *v; } t[] = {
        {"nodelist", &p.nodelist}, {"lxim", &p.lxim}, {"lxip", &p.lxip},
        {"letam", &p.letam}, {"letap", &p.letap}, {"lzetam", &p.lzetam},
        {"lzetap", &p.lzetap}, {"elemBC", &p.elemBC}, {"regNumList", &p.regNumList},
        {"regElemSize", &p.regElemSize}, {"symmX", &p.symmX}, {"symmY", &p.symmY},
        {"symmZ", &p.symmZ}, {"nodeElemStart", &p.nodeElemStart},
        {"nodeElemCornerList", &p.nodeElemCornerList}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) return f.v;
    return nullptr;
}

int read_ctl(lg_domain *d)
{
    LG_CUDA(cudaMemcpyAsync(d->h_ctl, d->ds.ctl, sizeof(lg::Ctl), cudaMemcpyDeviceToHost,
                            d->stream));
    LG_CUDA(cudaStreamSynchronize(d->stream));
    return LG_OK;
}

int write_ctl(lg_domain *d)
{
    LG_CUDA(cudaMemcpyAsync(d->ds.ctl, d->h_ctl, sizeof(lg::Ctl), cudaMemcpyHostToDevice,
                            d->stream));
    LG_CUDA(cudaStreamSynchronize(d->stream));
    return LG_OK;
}

// kernels one cycle launches: four, or six when the material phase runs split
int kernels_per_cycle(const lg_domain *d) { return d->ds.matSplit ? 6 : 4; }

void enqueue_cycle(lg_domain *d)
{
    d->ks->launch(lg::K_FORCES, d->ds, 0, d->stream);
    d->ks->launch(lg::K_NODES, d->ds, 0, d->stream);
    d->ks->launch(lg::K_KINEMATICS, d->ds, 0, d->stream);
    d->ks->launch(lg::K_MATERIAL, d->ds, 2, d->stream);
}

int capture(lg_domain *d, int ncycles, cudaGraphExec_t *out)
{
    cudaGraph_t g = nullptr;
    LG_CUDA(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < ncycles; ++i) enqueue_cycle(d);
    LG_CUDA(cudaStreamEndCapture(d->stream, &g));
    cudaError_t err = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess)
        return set_error(LG_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(err));
    return LG_OK;
}

int ensure_graphs(lg_domain *d)
{
    int st;
    if (!d->graph1 && (st = capture(d, 1, &d->graph1))) return st;
    if (!d->graph16 && (st = capture(d, 16, &d->graph16))) return st;
    return LG_OK;
}

// Queue ncycles cycles behind a k_begin that evaluates the loop test.
int enqueue_cycles(lg_domain *d, int ncycles)
{
    int st;
    if ((st = read_ctl(d))) return st;
    if (d->h_ctl->status != 0) return d->h_ctl->status;
    const long long limit = std::min<long long>(d->its, (long long)d->h_ctl->cycle + ncycles);
    const int lim = (int)limit;
    LG_CUDA(cudaMemcpyAsync(&d->ds.ctl->cycle_limit, &lim, sizeof(int), cudaMemcpyHostToDevice,
                            d->stream));
    LG_CUDA(cudaStreamSynchronize(d->stream));
    if ((st = ensure_graphs(d))) return st;
    d->ks->begin(d->ds.ctl, d->stream);
    int left = ncycles;
    while (left >= 16) {
        LG_CUDA(cudaGraphLaunch(d->graph16, d->stream));
        left -= 16;
    }
    while (left-- > 0) LG_CUDA(cudaGraphLaunch(d->graph1, d->stream));
    LG_CUDA(cudaGetLastError());
    d->launches += 1 + (long long)kernels_per_cycle(d) * ncycles;
    return LG_OK;
}

// Put the set-up state on the device: the initial fields (uploaded from the
// host mirror where it holds them, else rebuilt by the set-up kernels), the
// topology where the host mirror holds it (at creation without a mirror the
// set-up kernels build it), and the time-step state.
int upload_initial_state(lg_domain *d, bool creating)
{
    lg::Problem &p = d->prob;
    int st;
    if (d->mirror_state) {
        double *fld;
        size_t cnt;
        std::vector<double> *hostf[26] = {&p.x, &p.y, &p.z, &p.xd, &p.yd, &p.zd, &p.xdd, &p.ydd,
                                          &p.zdd, &p.fx, &p.fy, &p.fz, &p.nodalMass, &p.e, &p.p,
                                          &p.q, &p.ql, &p.qq, &p.v, &p.volo, &p.vnew, &p.delv,
                                          &p.vdov, &p.arealg, &p.ss, &p.elemMass};
        const char *names[26] = {"x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy",
                                 "fz", "nodalMass", "e", "p", "q", "ql", "qq", "v", "volo", "vnew",
                                 "delv", "vdov", "arealg", "ss", "elemMass"};
        for (int i = 0; i < 26; ++i) {
            find_f64(d, names[i], &fld, &cnt);
            if ((st = upload(d, fld, *hostf[i]))) return st;
        }
        if ((st = refresh_inv_mass(d))) return st;
    } else {
        LG_CUDA(lg::device_setup(d->ds, p.nx, lg::sedov_einit(p.nx, d->opts.einit_factor),
                                 creating && !d->mirror_topo, d->stream));
    }
    if (d->mirror_topo) {
        if ((st = upload_topology(d))) return st;
    } else if (creating) {
        if ((st = upload_regions(d))) return st;
    }

    lg::Ctl &c = *d->h_ctl;
    memset(&c, 0, sizeof(c));
    c.time = p.t.time;
    c.deltatime = p.t.deltatime;
    c.dtcourant = p.t.dtcourant;
    c.dthydro = p.t.dthydro;
    c.stoptime = p.t.stoptime;
    c.dtmax = p.t.dtmax;
    c.dtfixed = p.t.dtfixed;
    c.dtmultlb = p.t.deltatimemultlb;
    c.dtmultub = p.t.deltatimemultub;
    c.cycle = p.t.cycle;
    c.cycle_limit = 0;
    c.dt_frozen = d->d_dtfrozen;
    c.dt_frozen_len = d->dtfrozen_len;
    c.dt_record = d->d_dtrec;
    c.dt_record_len = d->dtrec_len;
    return write_ctl(d);
}

}  // namespace

extern "C" {

const char *lg_last_error(void) { return g_last_error.c_str(); }

void lg_default_opts(lg_opts *o)
{
    if (!o) return;
    o->nx = 30;
    o->numReg = 11;
    o->balance = 1;
    o->cost = 1;
    o->its = 9999999;
    o->precision = LG_FP64;
    o->hgcoef = 3.0;
    o->einit_factor = 1.0;
    o->device = 0;
}

// Block size of a one-thread-per-unit kernel over `units` threads.  Every
// FP64 warp instruction holds an SM's FP64 pipe for the same time, so a
// kernel lasts about as long as its busiest SM's warps take: blocks spread
// over the SMs, the busiest gets ceil(blocks / SMs) of them.  Smaller blocks
// are taken when they cut that warp count by more than 3 %, which happens on
// small meshes only (s=30: 8 warps with blocks of 128, 6 with 64); results
// do not depend on the block size.
static int pick_block(long long units, int sms)
{
    auto busiest = [&](int bs) {
        const long long blocks = (units + bs - 1) / bs;
        return (double)((blocks + sms - 1) / sms) * (bs / 32);
    };
    int best = 128;
    double best_cost = busiest(128);
    for (const int bs : {64, 32}) {
        const double c = busiest(bs);
        if (c < 0.97 * best_cost) {
            best = bs;
            best_cost = c;
        }
    }
    return best;
}

int lg_create(const lg_opts *opts, lg_domain **out)
{
    if (!opts || !out) return set_error(LG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (opts->nx < 1 || opts->numReg < 1 || opts->its < 0)
        return set_error(LG_ERR_INVALID, "invalid problem size (nx=%d numReg=%d its=%d)",
                         opts->nx, opts->numReg, opts->its);
    if ((long long)opts->nx * opts->nx * opts->nx * 8 > 2147483647LL)
        return set_error(LG_ERR_INVALID, "nx=%d exceeds the 32-bit corner index range", opts->nx);
    // A negative cost makes a region's EOS repetition count 0 or negative
    // (lulesh.cc:2390-2400); the reference then stores pressures and energies
    // its repetition loop never computed (lulesh.cc:2296-2308), so no result
    // is defined to match.
    if (opts->cost < 0)
        return set_error(LG_ERR_INVALID, "cost=%d: the EOS repetition count 1+cost must be "
                         "positive", opts->cost);
    const lg::KernelSet *ks = nullptr;
    switch (opts->precision) {
    case LG_FP64: ks = lg::kernels_fp64_strict(); break;
    case LG_FP64_FMA: ks = lg::kernels_fp64_fma(); break;
    case LG_MIXED: ks = lg::kernels_mixed(); break;
    default: return set_error(LG_ERR_INVALID, "precision %d not available", opts->precision);
    }
    lg_domain *d = new lg_domain();
    d->opts = *opts;
    d->its = opts->its;
    d->ks = ks;
    d->host_only = opts->device < 0;
    int st;
    if (!d->host_only && (st = ensure_device(d))) {
        delete d;
        return st;
    }
    if (d->host_only) {
        d->prob = lg::build_sedov(opts->nx, opts->numReg, opts->balance, opts->cost,
                                  opts->hgcoef, opts->einit_factor);
        d->mirror_state = d->mirror_topo = true;
    } else {
        // sizes, constants, time state and regions on the host; the mesh and
        // the fields are built on the device (lg_setup.cu)
        d->prob = lg::build_sedov_scalars(opts->nx, opts->numReg, opts->balance, opts->cost,
                                          opts->hgcoef, opts->einit_factor);
    }
    lg::Problem &p = d->prob;
    if (d->host_only) {
        d->ds.E = p.numElem;
        d->ds.N = p.numNode;
        d->ds.prm = make_params(p.k);
        *out = d;
        return LG_OK;
    }
    const size_t E = p.numElem, N = p.numNode;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opts->device) != cudaSuccess ||
        sms < 1)
        sms = 1;
    d->resident = sms * 8 * 128;  // 8 blocks of 128 threads per SM (64 registers)
    // split material phase: at most E + 4 x resident repetition items (each
    // element's count rounded up, the total bounded by 4 x resident shares)
    d->item_cap = (int)(E + 4 * (size_t)d->resident);
    const int eblocks = (int)((d->item_cap + 127) / 128);

    Layout L;
    size_t o_node[14], o_elem[19];
    for (auto &o : o_node) o = L.add<double>(N);
    for (auto &o : o_elem) o = L.add<double>(E);
    const size_t o_corner = L.add<double>(48 * E);
    const size_t o_nl = L.add<int>(8 * E), o_nlT = L.add<int>(8 * E);
    size_t o_conn[7];
    for (auto &o : o_conn) o = L.add<int>(E);
    const size_t o_regnum = L.add<int>(E), o_perm = L.add<int>(d->item_cap),
                 o_rep = L.add<int>(d->item_cap);
    const size_t o_nes = L.add<int>(N + 1), o_ncl = L.add<int>(8 * E);
    const size_t o_symm = L.add<uint8_t>(N);
    const size_t o_part = L.add<double>(2 * (size_t)eblocks);
    const size_t o_ctl = L.add<lg::Ctl>(1);

    cudaError_t err = cudaMalloc(&d->arena, L.total);
    if (err != cudaSuccess) {
        delete d;
        return set_error(LG_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", L.total, cudaGetErrorString(err));
    }
    d->arena_bytes = L.total;
    char *base = static_cast<char *>(d->arena);
    lg::DevState &s = d->ds;
    s.E = (int)E;
    s.N = (int)N;
    s.nItems = (int)E;
    s.nx = p.nx;
    s.numReg = p.numReg;
    double **nodef[14] = {&s.x, &s.y, &s.z, &s.xd, &s.yd, &s.zd, &s.xdd, &s.ydd, &s.zdd,
                          &s.fx, &s.fy, &s.fz, &s.nodalMass, &s.invMass};
    for (int i = 0; i < 14; ++i) *nodef[i] = reinterpret_cast<double *>(base + o_node[i]);
    double **elemf[19] = {&s.e, &s.p, &s.q, &s.ql, &s.qq, &s.v, &s.volo, &s.vnew, &s.delv,
                          &s.vdov, &s.arealg, &s.ss, &s.elemMass, &s.delx_xi, &s.delx_eta,
                          &s.delx_zeta, &s.delv_xi, &s.delv_eta, &s.delv_zeta};
    for (int i = 0; i < 19; ++i) *elemf[i] = reinterpret_cast<double *>(base + o_elem[i]);
    s.corner = reinterpret_cast<double *>(base + o_corner);
    s.nodelist = reinterpret_cast<int *>(base + o_nl);
    s.nodelistT = reinterpret_cast<int *>(base + o_nlT);
    int **conn[7] = {&s.lxim, &s.lxip, &s.letam, &s.letap, &s.lzetam, &s.lzetap, &s.elemBC};
    for (int i = 0; i < 7; ++i) *conn[i] = reinterpret_cast<int *>(base + o_conn[i]);
    s.regNumList = reinterpret_cast<int *>(base + o_regnum);
    s.regPerm = reinterpret_cast<int *>(base + o_perm);
    s.regRep = reinterpret_cast<int *>(base + o_rep);
    s.nodeElemStart = reinterpret_cast<int *>(base + o_nes);
    s.nodeElemCornerList = reinterpret_cast<int *>(base + o_ncl);
    s.symm = reinterpret_cast<uint8_t *>(base + o_symm);
    s.dt_partial = reinterpret_cast<double *>(base + o_part);
    s.dt_blocks = eblocks;
    s.bs_elem = pick_block((long long)E, sms);
    s.bs_node = pick_block((long long)N, sms);
    s.ctl = reinterpret_cast<lg::Ctl *>(base + o_ctl);
    s.prm = make_params(p.k);

    auto fail = [&](int code) {
        lg_destroy(d);
        return code;
    };
    if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&d->h_ctl, sizeof(lg::Ctl)) != cudaSuccess ||
        cudaEventCreate(&d->ev0) != cudaSuccess || cudaEventCreate(&d->ev1) != cudaSuccess)
        return fail(set_error(LG_ERR_CUDA, "stream/event/pinned allocation failed"));
    if (cudaMemsetAsync(d->arena, 0, L.total, d->stream) != cudaSuccess)
        return fail(set_error(LG_ERR_CUDA, "cudaMemset failed"));

    if ((st = upload_initial_state(d, true))) return fail(st);
    *out = d;
    return LG_OK;
}

int lg_reset(lg_domain *d)
{
    if (!d) return set_error(LG_ERR_INVALID, "null handle");
    int st;
    if ((st = ensure_device(d))) return st;
    LG_CUDA(cudaStreamSynchronize(d->stream));
    return upload_initial_state(d, false);
}

void lg_destroy(lg_domain *d)
{
    if (!d) return;
    if (d->host_only) {
        delete d;
        return;
    }
    cudaSetDevice(d->opts.device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    drop_graphs(d);
    if (d->d_dtfrozen) cudaFree(d->d_dtfrozen);
    if (d->d_dtrec) cudaFree(d->d_dtrec);
    if (d->ev0) cudaEventDestroy(d->ev0);
    if (d->ev1) cudaEventDestroy(d->ev1);
    if (d->h_ctl) cudaFreeHost(d->h_ctl);
    if (d->arena) cudaFree(d->arena);
    if (d->stream) cudaStreamDestroy(d->stream);
    delete d;
}

int lg_step(lg_domain *d, int ncycles)
{
    if (!d || ncycles < 0) return set_error(LG_ERR_INVALID, "invalid argument");
    int st;
    if ((st = ensure_device(d))) return st;
    if (ncycles == 0) return LG_OK;
    if ((st = enqueue_cycles(d, ncycles))) return st;
    if ((st = read_ctl(d))) return st;
    return d->h_ctl->status;
}

int lg_step_timed(lg_domain *d, int ncycles, double *ms)
{
    if (!d || ncycles < 0 || !ms) return set_error(LG_ERR_INVALID, "invalid argument");
    int st;
    if ((st = ensure_device(d))) return st;
    if ((st = ensure_graphs(d))) return st;
    LG_CUDA(cudaStreamSynchronize(d->stream));
    // the control-block write of enqueue_cycles happens before ev0
    if ((st = read_ctl(d))) return st;
    if (d->h_ctl->status != 0) return d->h_ctl->status;
    const long long limit = std::min<long long>(d->its, (long long)d->h_ctl->cycle + ncycles);
    const int lim = (int)limit;
    LG_CUDA(cudaMemcpyAsync(&d->ds.ctl->cycle_limit, &lim, sizeof(int), cudaMemcpyHostToDevice,
                            d->stream));
    LG_CUDA(cudaStreamSynchronize(d->stream));
    LG_CUDA(cudaEventRecord(d->ev0, d->stream));
    d->ks->begin(d->ds.ctl, d->stream);
    int left = ncycles;
    while (left >= 16) {
        LG_CUDA(cudaGraphLaunch(d->graph16, d->stream));
        left -= 16;
    }
    while (left-- > 0) LG_CUDA(cudaGraphLaunch(d->graph1, d->stream));
    LG_CUDA(cudaEventRecord(d->ev1, d->stream));
    d->launches += 1 + (long long)kernels_per_cycle(d) * ncycles;
    LG_CUDA(cudaEventSynchronize(d->ev1));
    float f = 0.f;
    LG_CUDA(cudaEventElapsedTime(&f, d->ev0, d->ev1));
    *ms = f;
    if ((st = read_ctl(d))) return st;
    return d->h_ctl->status;
}

int lg_run(lg_domain *d)
{
    if (!d) return set_error(LG_ERR_INVALID, "null handle");
    int st;
    if ((st = ensure_device(d))) return st;
    if ((st = read_ctl(d))) return st;
    for (;;) {
        const lg::Ctl &c = *d->h_ctl;
        if (c.status) return c.status;
        if (!(c.time < c.stoptime && c.cycle < d->its)) return LG_OK;
        // chunks of at most 64 cycles; lg_step leaves h_ctl current
        const int n = (int)std::min<long long>(64, (long long)d->its - c.cycle);
        if ((st = lg_step(d, n))) return st;
    }
}

int lg_phase(lg_domain *d, int phase)
{
    if (!d) return set_error(LG_ERR_INVALID, "null handle");
    int st;
    if ((st = ensure_device(d))) return st;
    switch (phase) {
    case 0: d->ks->time_increment(d->ds.ctl, d->stream); break;
    case 1:
        d->ks->set_active(d->ds.ctl, d->stream);
        d->ks->launch(lg::K_FORCES, d->ds, 0, d->stream);
        d->ks->launch(lg::K_NODES, d->ds, 0, d->stream);
        break;
    case 2:
        d->ks->set_active(d->ds.ctl, d->stream);
        d->ks->launch(lg::K_KINEMATICS, d->ds, 0, d->stream);
        d->ks->launch(lg::K_MATERIAL, d->ds, 0, d->stream);
        break;
    case 3:
        d->ks->set_active(d->ds.ctl, d->stream);
        d->ks->launch(lg::K_MATERIAL, d->ds, 1, d->stream);
        break;
    default: return set_error(LG_ERR_INVALID, "unknown phase %d", phase);
    }
    LG_CUDA(cudaGetLastError());
    if ((st = read_ctl(d))) return st;
    return d->h_ctl->status;
}

int lg_field_info(lg_domain *d, const char *name, size_t *count, int *dtype)
{
    if (!d || !name) return set_error(LG_ERR_INVALID, "null argument");
    double *p;
    size_t c;
    if (find_f64(d, name, &p, &c)) {
        if (count) *count = c;
        if (dtype) *dtype = LG_F64;
        return LG_OK;
    }
    int st;
    if ((st = ensure_topology_mirror(d))) return st;
    if (std::vector<int> *v = find_i32(d, name)) {
        if (count) *count = v->size();
        if (dtype) *dtype = LG_I32;
        return LG_OK;
    }
    return set_error(LG_ERR_INVALID, "unknown field '%s'", name);
}

int lg_get_field(lg_domain *d, const char *name, void *dst, size_t n)
{
    if (!d || !name || (!dst && n)) return set_error(LG_ERR_INVALID, "null argument");
    int st;
    if (d->host_only) {
        if (std::vector<double> *hv = find_f64_host(d, name)) {
            if (n != hv->size())
                return set_error(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name,
                                 hv->size(), n);
            memcpy(dst, hv->data(), n * sizeof(double));
            return LG_OK;
        }
    } else if ((st = ensure_device(d))) {
        return st;
    }
    double *p;
    size_t c;
    if (d->opts.precision == LG_MIXED && !strncmp(name, "del", 3) && strcmp(name, "delv") != 0)
        return set_error(LG_ERR_INVALID, "'%s' is held in FP32 by the mixed path", name);
    if (!d->host_only && find_f64(d, name, &p, &c)) {
        if (n != c) return set_error(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name, c, n);
        LG_CUDA(cudaMemcpyAsync(dst, p, c * sizeof(double), cudaMemcpyDeviceToHost, d->stream));
        LG_CUDA(cudaStreamSynchronize(d->stream));
        return LG_OK;
    }
    if ((st = ensure_topology_mirror(d))) return st;
    if (std::vector<int> *v = find_i32(d, name)) {
        if (n != v->size())
            return set_error(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name, v->size(), n);
        if (n) memcpy(dst, v->data(), n * sizeof(int));
        return LG_OK;
    }
    return set_error(LG_ERR_INVALID, "unknown field '%s'", name);
}

int lg_set_field(lg_domain *d, const char *name, const void *src, size_t n)
{
    if (!d || !name || (!src && n)) return set_error(LG_ERR_INVALID, "null argument");
    int st;
    if ((st = ensure_device(d))) return st;
    double *p;
    size_t c;
    if (find_f64(d, name, &p, &c)) {
        if (n != c) return set_error(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name, c, n);
        LG_CUDA(cudaMemcpyAsync(p, src, c * sizeof(double), cudaMemcpyHostToDevice, d->stream));
        if (!strcmp(name, "nodalMass") && (st = refresh_inv_mass(d))) return st;
        LG_CUDA(cudaStreamSynchronize(d->stream));
        return LG_OK;
    }
    if ((st = ensure_topology_mirror(d))) return st;
    std::vector<int> *v = find_i32(d, name);
    if (!v) return set_error(LG_ERR_INVALID, "unknown field '%s'", name);
    if (n != v->size())
        return set_error(LG_ERR_INVALID, "field '%s' has %zu entries, not %zu", name, v->size(), n);
    lg::Problem &pr = d->prob;
    const int *in = static_cast<const int *>(src);
    if (!strcmp(name, "regElemSize") || !strcmp(name, "nodeElemStart") ||
        !strcmp(name, "nodeElemCornerList") || !strcmp(name, "symmX") ||
        !strcmp(name, "symmY") || !strcmp(name, "symmZ"))
        return set_error(LG_ERR_INVALID, "field '%s' is derived and read-only", name);
    if (!strcmp(name, "nodelist")) {
        for (size_t i = 0; i < n; ++i)
            if (in[i] < 0 || in[i] >= pr.numNode)
                return set_error(LG_ERR_INVALID, "nodelist entry %zu out of range", i);
    } else if (!strcmp(name, "regNumList")) {
        for (size_t i = 0; i < n; ++i)
            if (in[i] < 1 || in[i] > pr.numReg)
                return set_error(LG_ERR_INVALID, "regNumList entry %zu out of range", i);
    } else if (strcmp(name, "elemBC") != 0) {
        for (size_t i = 0; i < n; ++i)
            if (in[i] < 0 || in[i] >= pr.numElem)
                return set_error(LG_ERR_INVALID, "%s entry %zu out of range", name, i);
    }
    std::copy(in, in + n, v->begin());
    if (!strcmp(name, "nodelist")) lg::build_corner_list(pr);
    if (!strcmp(name, "regNumList")) lg::build_region_sets(pr);
    return upload_topology(d);
}

int lg_get_scalar(lg_domain *d, const char *name, double *value)
{
    if (!d || !name || !value) return set_error(LG_ERR_INVALID, "null argument");
    int st;
    lg::Ctl hc{};
    if (d->host_only) {
        const lg::TimeState &t = d->prob.t;
        hc.time = t.time; hc.deltatime = t.deltatime; hc.dtcourant = t.dtcourant;
        hc.dthydro = t.dthydro; hc.stoptime = t.stoptime; hc.dtmax = t.dtmax;
        hc.dtfixed = t.dtfixed; hc.dtmultlb = t.deltatimemultlb;
        hc.dtmultub = t.deltatimemultub; hc.cycle = t.cycle;
    } else {
        if ((st = ensure_device(d))) return st;
        if ((st = read_ctl(d))) return st;
        hc = *d->h_ctl;
    }
    const lg::Ctl &c = hc;
    const lg::Problem &p = d->prob;
    struct { const char *n; double v; } t[] = {
        {"time", c.time}, {"deltatime", c.deltatime}, {"dtcourant", c.dtcourant},
        {"dthydro", c.dthydro}, {"stoptime", c.stoptime}, {"dtmax", c.dtmax},
        {"dtfixed", c.dtfixed}, {"deltatimemultlb", c.dtmultlb},
        {"deltatimemultub", c.dtmultub}, {"hgcoef", d->ds.prm.hgcoef},
        {"cycle", (double)c.cycle}, {"its", (double)d->its}, {"numElem", (double)p.numElem},
        {"numNode", (double)p.numNode}, {"numReg", (double)p.numReg},
        {"sizeX", (double)p.nx}, {"cost", (double)p.cost}, {"status", (double)c.status},
        {"launches", (double)d->launches}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) {
            *value = f.v;
            return LG_OK;
        }
    return set_error(LG_ERR_INVALID, "unknown scalar '%s'", name);
}

int lg_set_scalar(lg_domain *d, const char *name, double value)
{
    if (!d || !name) return set_error(LG_ERR_INVALID, "null argument");
    int st;
    if ((st = ensure_device(d))) return st;
    if (!strcmp(name, "hgcoef")) {
        d->ds.prm.hgcoef = value;
        drop_graphs(d);  // the kernel arguments are baked into the graphs
        return LG_OK;
    }
    if (!strcmp(name, "its")) {
        d->its = (int)value;
        return LG_OK;
    }
    if ((st = read_ctl(d))) return st;
    lg::Ctl &c = *d->h_ctl;
    struct { const char *n; double *v; } t[] = {
        {"time", &c.time}, {"deltatime", &c.deltatime}, {"dtcourant", &c.dtcourant},
        {"dthydro", &c.dthydro}, {"stoptime", &c.stoptime}, {"dtmax", &c.dtmax},
        {"dtfixed", &c.dtfixed}, {"deltatimemultlb", &c.dtmultlb},
        {"deltatimemultub", &c.dtmultub}};
    for (auto &f : t)
        if (!strcmp(f.n, name)) {
            *f.v = value;
            return write_ctl(d);
        }
    if (!strcmp(name, "cycle")) {
        c.cycle = (int)value;
        return write_ctl(d);
    }
    if (!strcmp(name, "status")) {  // clear a recorded error
        c.status = (int)value;
        return write_ctl(d);
    }
    return set_error(LG_ERR_INVALID, "unknown or read-only scalar '%s'", name);
}

int lg_region_rep(lg_domain *d, int r, int *rep)
{
    if (!d || !rep || r < 0 || r >= d->prob.numReg) return set_error(LG_ERR_INVALID, "invalid region");
    *rep = lg::region_rep(r, d->prob.numReg, d->prob.cost);
    return LG_OK;
}

int lg_verify(lg_domain *d, double out[4])
{
    if (!d || !out) return set_error(LG_ERR_INVALID, "null argument");
    int st;
    if ((st = ensure_device(d))) return st;
    // lulesh-util.cc:189-218 on the device (lg_setup.cu), into the control
    // block; the per-corner scratch, idle between cycles, holds the pairs
    LG_CUDA(lg::device_verify(d->ds.e, d->prob.nx, d->ds.corner, d->ds.ctl->verify, d->stream));
    if ((st = read_ctl(d))) return st;
    for (int i = 0; i < 4; ++i) out[i] = d->h_ctl->verify[i];
    return LG_OK;
}

int lg_report(lg_domain *d, double elapsed, char *buf, size_t buflen)
{
    if (!d || !buf || !buflen) return set_error(LG_ERR_INVALID, "null argument");
    double v[4];
    int st;
    if ((st = lg_verify(d, v))) return st;
    if ((st = read_ctl(d))) return st;
    const std::string s = lg::format_report(d->prob.nx, d->h_ctl->cycle, v[0], v[1], v[2], v[3],
                                            elapsed);
    snprintf(buf, buflen, "%s", s.c_str());
    return LG_OK;
}

int lg_dt_record(lg_domain *d, int capacity)
{
    if (!d || capacity < 0) return set_error(LG_ERR_INVALID, "invalid argument");
    int st;
    if ((st = ensure_device(d))) return st;
    LG_CUDA(cudaStreamSynchronize(d->stream));
    if (d->d_dtrec) cudaFree(d->d_dtrec);
    d->d_dtrec = nullptr;
    d->dtrec_len = 0;
    if (capacity > 0) {
        LG_CUDA(cudaMalloc(&d->d_dtrec, sizeof(double) * (size_t)capacity));
        LG_CUDA(cudaMemsetAsync(d->d_dtrec, 0, sizeof(double) * (size_t)capacity, d->stream));
        d->dtrec_len = capacity;
    }
    if ((st = read_ctl(d))) return st;
    d->h_ctl->dt_record = d->d_dtrec;
    d->h_ctl->dt_record_len = d->dtrec_len;
    return write_ctl(d);
}

int lg_dt_get(lg_domain *d, double *out, int n)
{
    if (!d || !out || n < 0 || n > d->dtrec_len) return set_error(LG_ERR_INVALID, "invalid argument");
    int st;
    if ((st = ensure_device(d))) return st;
    if (n == 0) return LG_OK;
    LG_CUDA(cudaMemcpyAsync(out, d->d_dtrec, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost,
                            d->stream));
    LG_CUDA(cudaStreamSynchronize(d->stream));
    return LG_OK;
}

int lg_dt_freeze(lg_domain *d, const double *dts, int n)
{
    if (!d || n < 0 || (n > 0 && !dts)) return set_error(LG_ERR_INVALID, "invalid argument");
    int st;
    if ((st = ensure_device(d))) return st;
    LG_CUDA(cudaStreamSynchronize(d->stream));
    if (d->d_dtfrozen) cudaFree(d->d_dtfrozen);
    d->d_dtfrozen = nullptr;
    d->dtfrozen_len = 0;
    d->h_dtfrozen.assign(dts, dts + n);
    if (n > 0) {
        LG_CUDA(cudaMalloc(&d->d_dtfrozen, sizeof(double) * (size_t)n));
        LG_CUDA(cudaMemcpyAsync(d->d_dtfrozen, dts, sizeof(double) * (size_t)n,
                                cudaMemcpyHostToDevice, d->stream));
        d->dtfrozen_len = n;
    }
    if ((st = read_ctl(d))) return st;
    d->h_ctl->dt_frozen = d->d_dtfrozen;
    d->h_ctl->dt_frozen_len = d->dtfrozen_len;
    return write_ctl(d);
}

namespace {

// lg_adjoint and lg_adjoint_vjp: checks, then the checkpointed sweep
int run_adjoint(lg_domain *d, int ncycles, int ckpt_k, const unsigned char *mask,
                const double *const *seed, double *const *grad, double *J, double *dJ_dhgcoef)
{
    if (d->opts.precision == LG_MIXED)
        return set_error(LG_ERR_INVALID, "the adjoint differentiates the FP64 paths only");
    int st;
    if ((st = ensure_device(d))) return st;
    if ((st = read_ctl(d))) return st;
    if (d->h_ctl->status != 0) return d->h_ctl->status;
    const int c0 = d->h_ctl->cycle;
    if (!d->d_dtfrozen || c0 + ncycles > d->dtfrozen_len)
        return set_error(LG_ERR_STATE, "the adjoint needs frozen time steps for cycles %d..%d "
                                       "(lg_dt_freeze)", c0, c0 + ncycles - 1);
    drop_graphs(d);  // the adjoint launches its own cycles
    if ((st = ensure_topology_mirror(d))) return st;
    const lg::Problem &p = d->prob;
    lg::AdjointIO io{&d->ds, d->ks, d->stream, d->h_ctl, d->h_dtfrozen.data() + c0, ncycles,
                     ckpt_k, mask, seed, grad, d->ds.prm.hgcoef, &p.lxim, &p.lxip, &p.letam,
                     &p.letap, &p.lzetam, &p.lzetap, &p.elemBC};
    st = lg::adjoint_run(io, J, dJ_dhgcoef);
    d->launches += 10LL * ncycles;
    return st;
}

}  // namespace

int lg_adjoint(lg_domain *d, int ncycles, int ckpt_k, const unsigned char *mask, double *J,
               double *dJ_de0, double *dJ_dhgcoef)
{
    if (!d || ncycles < 1 || ckpt_k < 1 || !mask || !J || !dJ_de0 || !dJ_dhgcoef)
        return set_error(LG_ERR_INVALID, "invalid argument");
    double *grad[lg::kAdjFields] = {};
    grad[6] = dJ_de0;
    return run_adjoint(d, ncycles, ckpt_k, mask, nullptr, grad, J, dJ_dhgcoef);
}

int lg_adjoint_vjp(lg_domain *d, int ncycles, int ckpt_k, const double *const seed[11],
                   double *const grad[11], double *dJ_dhgcoef)
{
    if (!d || ncycles < 1 || ckpt_k < 1 || !seed || !grad || !dJ_dhgcoef)
        return set_error(LG_ERR_INVALID, "invalid argument");
    return run_adjoint(d, ncycles, ckpt_k, nullptr, seed, grad, nullptr, dJ_dhgcoef);
}

int lg_profile(lg_domain *d, int ncycles, double *ms, const char **names, int *nkernels)
{
    if (!d || !ms || !nkernels || *nkernels < lg::K_COUNT)
        return set_error(LG_ERR_INVALID, "invalid argument");
    int st;
    if ((st = ensure_device(d))) return st;
    if ((st = read_ctl(d))) return st;
    if (d->h_ctl->status != 0) return d->h_ctl->status;
    const int lim = (int)std::min<long long>(d->its, (long long)d->h_ctl->cycle + ncycles);
    LG_CUDA(cudaMemcpyAsync(&d->ds.ctl->cycle_limit, &lim, sizeof(int), cudaMemcpyHostToDevice,
                            d->stream));
    std::vector<cudaEvent_t> ev(2 * lg::K_COUNT * (size_t)ncycles);
    for (auto &e : ev) LG_CUDA(cudaEventCreate(&e));
    d->ks->begin(d->ds.ctl, d->stream);
    for (int c = 0; c < ncycles; ++c)
        for (int k = 0; k < lg::K_COUNT; ++k) {
            LG_CUDA(cudaEventRecord(ev[2 * (c * lg::K_COUNT + k)], d->stream));
            d->ks->launch(k, d->ds, k == lg::K_MATERIAL ? 2 : 0, d->stream);
            LG_CUDA(cudaEventRecord(ev[2 * (c * lg::K_COUNT + k) + 1], d->stream));
        }
    LG_CUDA(cudaStreamSynchronize(d->stream));
    for (int k = 0; k < lg::K_COUNT; ++k) {
        ms[k] = 0.0;
        if (names) names[k] = d->ks->kernel_names[k];
    }
    for (int c = 0; c < ncycles; ++c)
        for (int k = 0; k < lg::K_COUNT; ++k) {
            float f = 0.f;
            LG_CUDA(cudaEventElapsedTime(&f, ev[2 * (c * lg::K_COUNT + k)],
                                         ev[2 * (c * lg::K_COUNT + k) + 1]));
            ms[k] += f;
        }
    for (auto &e : ev) cudaEventDestroy(e);
    *nkernels = lg::K_COUNT;
    if ((st = read_ctl(d))) return st;
    return d->h_ctl->status;
}

}  // extern "C"
