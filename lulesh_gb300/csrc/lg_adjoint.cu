// lg_adjoint.cu -- checkpointed reverse-mode adjoint of the FP64 leap-frog
// cycle with the time-step sequence frozen.
//
// The cycle c maps the state S_c = (x, y, z, xd, yd, zd, e, p, q, v, ss) to
// S_{c+1} with the frozen step dt_c.  Its adjoint runs the forward phases
// backwards, one kernel per phase, each element or node recomputing the
// forward values it needs (lg_adjoint_math.h) from stored states:
//   ka_material   EOS (one repetition: the repetitions recompute identical
//                 values) and monotonic-Q limiter, from the adjoints of
//                 e, p, q, ss, v of S_{c+1}
//   ka_qslots     the limiter's neighbour reads, transposed into a gather
//   ka_kinematics Q gradients and the element volume (vnew = V / volo)
//   ka_nodes      position/velocity update, a = F / m, boundary conditions
//   ka_forces     stress and FB hourglass forces
//   ka_gather     the element -> node corner sums of the two element phases
// Scatter adjoints become gathers through the corner scratch and the node
// corner lists, as in the forward path: no atomics, deterministic sums.
// S_c is checkpointed every k cycles in a first forward pass; each segment is
// recomputed from its checkpoint storing S_c and the per-cycle temporaries
// (vnew, vdov and the six Q gradients), then swept backwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lg_adjoint.h"
#include "lg_adjoint_cycle.h"
#include "lg_device.h"
#include "lg_kernelset.h"

namespace lg {
int record_error(int code, const char *msg);
}

#include "lulesh_gb300.h"

namespace {

constexpr int kB = 128;
using namespace ::lg::adj;

__global__ void __launch_bounds__(kB) ka_material(lg::DevState s, AdjArgs a)
{
    const int k = blockIdx.x * kB + threadIdx.x;
    if (k < s.E) adj_material(s, a, k);
}

__global__ void __launch_bounds__(kB) ka_qslots(lg::DevState s, AdjArgs a)
{
    const int k = blockIdx.x * kB + threadIdx.x;
    if (k < s.E) adj_qslots(s, a, k);
}

__global__ void __launch_bounds__(kB) ka_kinematics(lg::DevState s, AdjArgs a)
{
    const int k = blockIdx.x * kB + threadIdx.x;
    if (k < s.E) adj_kinematics(s, a, k);
}

__global__ void __launch_bounds__(kB) ka_nodes(lg::DevState s, AdjArgs a)
{
    const int n = blockIdx.x * kB + threadIdx.x;
    if (n < s.N) adj_nodes(s, a, n);
}

__global__ void __launch_bounds__(kB) ka_forces(lg::DevState s, AdjArgs a)
{
    const int k = blockIdx.x * kB + threadIdx.x;
    const double hgb = (k < s.E) ? adj_forces(s, a, k) : 0.;
    // block sum of the hourglass-coefficient adjoint (fixed order)
    __shared__ double red[kB];
    red[threadIdx.x] = hgb;
    __syncthreads();
    for (int w = kB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.hgPart[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(kB) ka_gather(lg::DevState s, AdjArgs a)
{
    const int n = blockIdx.x * kB + threadIdx.x;
    if (n < s.N) adj_gather(s, a, n);
}

// Adds the per-block hourglass-coefficient partials of one reverse cycle to
// acc: one block, each thread summing a strided subset in index order, then
// a pairwise tree in shared memory.  The order is fixed, so the sum is the
// same on every run; one thread reading them in turn waited on each load.
__global__ void __launch_bounds__(kB) ka_hg_sum(const double *part, int nparts, double *acc)
{
    __shared__ double red[kB];
    double t = 0.;
    for (int i = threadIdx.x; i < nparts; i += kB) t += part[i];
    red[threadIdx.x] = t;
    __syncthreads();
    for (int w = kB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *acc += red[0];
}

int err(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return lg::record_error(code, buf);
}

#define AD_CUDA(call)                                                                    \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return err(LG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                       __FILE__, __LINE__);                                              \
    } while (0)

}  // namespace

namespace lg {

int adjoint_run(const AdjointIO &io, double *J, double *dJdhg)
{
    const DevState &S = *io.ds;
    const int E = S.E, N = S.N;
    const int K = std::max(1, std::min(io.ckpt_k, io.ncycles));
    const int nseg = (io.ncycles + K - 1) / K;
    const size_t snapD = 6 * (size_t)N + 5 * (size_t)E, tempD = 8 * (size_t)E;
    cudaStream_t st = io.stream;

    // reverse neighbour map of the limiter (element j reads element k)
    std::vector<int> revCount(E + 1, 0), revStart(E + 1, 0), revEntry;
    {
        const std::vector<int> *nb[6] = {io.lxim, io.lxip, io.letam, io.letap, io.lzetam, io.lzetap};
        const int mmask[3] = {XI_M, ETA_M, ZETA_M}, msym[3] = {XI_M_SYMM, ETA_M_SYMM, ZETA_M_SYMM},
                  mfree[3] = {XI_M_FREE, ETA_M_FREE, ZETA_M_FREE};
        const int pmask[3] = {XI_P, ETA_P, ZETA_P}, psym[3] = {XI_P_SYMM, ETA_P_SYMM, ZETA_P_SYMM},
                  pfree[3] = {XI_P_FREE, ETA_P_FREE, ZETA_P_FREE};
        auto uses = [](int bits, int mask, int sym, int fr) {
            const int b = bits & mask;
            return b == 0 || (b != sym && b != fr && b == (mask & ~(sym | fr)));
        };
        std::vector<std::vector<int>> lists(E);
        for (int j = 0; j < E; ++j) {
            const int bc = (*io.elemBC)[j];
            for (int d = 0; d < 3; ++d) {
                if (uses(bc, mmask[d], msym[d], mfree[d])) lists[(*nb[2 * d])[j]].push_back(j * 6 + 2 * d);
                if (uses(bc, pmask[d], psym[d], pfree[d])) lists[(*nb[2 * d + 1])[j]].push_back(j * 6 + 2 * d + 1);
            }
        }
        for (int k = 0; k < E; ++k) {
            revStart[k + 1] = revStart[k] + (int)lists[k].size();
            revEntry.insert(revEntry.end(), lists[k].begin(), lists[k].end());
        }
        if (revEntry.empty()) revEntry.push_back(0);
    }

    // one arena for checkpoints, the segment store and the adjoint arrays
    const int eb = (E + kB - 1) / kB, nbk = (N + kB - 1) / kB;
    const size_t dbl = (size_t)(nseg + 1) * snapD + (size_t)(K + 1) * snapD + (size_t)K * tempD +
                       6 * (size_t)N + 5 * (size_t)E + 7 * (size_t)E + 6 * (size_t)E +
                       48 * (size_t)E + 3 * (size_t)N + eb + 1;
    char *arena = nullptr;
    const size_t bytes = dbl * sizeof(double) + (size_t)(E + 1 + revEntry.size()) * sizeof(int) + 4096;
    if (cudaMalloc(&arena, bytes) != cudaSuccess)
        return err(LG_ERR_NOMEM, "adjoint: cudaMalloc(%zu bytes) failed", bytes);
    struct Free {
        char *p;
        ~Free() { cudaFree(p); }
    } guard{arena};
    double *p = reinterpret_cast<double *>(arena);
    auto take = [&](size_t n) {
        double *r = p;
        p += n;
        return r;
    };
    double *ckpt = take((size_t)(nseg + 1) * snapD);
    double *seg = take((size_t)(K + 1) * snapD);
    double *tmp = take((size_t)K * tempD);
    double *nbar = take(6 * (size_t)N);
    double *ebar = take(5 * (size_t)E);
    double *vnewb = take(E), *dxb = take(3 * (size_t)E), *dvb = take(3 * (size_t)E);
    double *slot = take(6 * (size_t)E), *corner = take(48 * (size_t)E), *fb = take(3 * (size_t)N);
    double *hgPart = take(eb), *hgAcc = take(1);
    int *d_revStart = reinterpret_cast<int *>(p);
    int *d_revEntry = d_revStart + (E + 1);
    AD_CUDA(cudaMemcpyAsync(d_revStart, revStart.data(), sizeof(int) * (E + 1), cudaMemcpyHostToDevice, st));
    AD_CUDA(cudaMemcpyAsync(d_revEntry, revEntry.data(), sizeof(int) * revEntry.size(), cudaMemcpyHostToDevice, st));

    double *const live_n[6] = {S.x, S.y, S.z, S.xd, S.yd, S.zd};
    double *const live_e[5] = {S.e, S.p, S.q, S.v, S.ss};
    double *const live_t[8] = {S.vnew, S.vdov, S.delx_xi, S.delx_eta, S.delx_zeta,
                               S.delv_xi, S.delv_eta, S.delv_zeta};
    auto snap_at = [&](double *base) {
        Snap s;
        for (int i = 0; i < 6; ++i) s.n[i] = base + (size_t)i * N;
        for (int i = 0; i < 5; ++i) s.el[i] = base + 6 * (size_t)N + (size_t)i * E;
        return s;
    };
    auto save = [&](double *base) -> int {
        const Snap s = snap_at(base);
        for (int i = 0; i < 6; ++i)
            AD_CUDA(cudaMemcpyAsync(s.n[i], live_n[i], 8 * (size_t)N, cudaMemcpyDeviceToDevice, st));
        for (int i = 0; i < 5; ++i)
            AD_CUDA(cudaMemcpyAsync(s.el[i], live_e[i], 8 * (size_t)E, cudaMemcpyDeviceToDevice, st));
        return LG_OK;
    };
    auto restore = [&](const double *base) -> int {
        const Snap s = snap_at(const_cast<double *>(base));
        for (int i = 0; i < 6; ++i)
            AD_CUDA(cudaMemcpyAsync(live_n[i], s.n[i], 8 * (size_t)N, cudaMemcpyDeviceToDevice, st));
        for (int i = 0; i < 5; ++i)
            AD_CUDA(cudaMemcpyAsync(live_e[i], s.el[i], 8 * (size_t)E, cudaMemcpyDeviceToDevice, st));
        return LG_OK;
    };
    auto read_ctl = [&](Ctl *out) -> int {
        AD_CUDA(cudaMemcpyAsync(io.h_ctl, S.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        AD_CUDA(cudaStreamSynchronize(st));
        *out = *io.h_ctl;
        return LG_OK;
    };
    auto write_ctl = [&](const Ctl &c) -> int {
        *io.h_ctl = c;
        AD_CUDA(cudaMemcpyAsync(S.ctl, io.h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
        AD_CUDA(cudaStreamSynchronize(st));
        return LG_OK;
    };
    auto cycle = [&]() {
        for (int id = 0; id < K_COUNT; ++id) io.ks->launch(id, S, id == K_MATERIAL ? 2 : 0, st);
    };

    // forward pass: checkpoints at cycles 0, K, 2K, ...
    std::vector<Ctl> ckctl(nseg + 1);
    Ctl c0;
    int rc;
    if ((rc = read_ctl(&c0))) return rc;
    c0.cycle_limit = c0.cycle + io.ncycles;
    if ((rc = write_ctl(c0))) return rc;
    io.ks->begin(S.ctl, st);
    for (int c = 0; c < io.ncycles; ++c) {
        if (c % K == 0) {
            if ((rc = save(ckpt + (size_t)(c / K) * snapD))) return rc;
            if ((rc = read_ctl(&ckctl[c / K]))) return rc;
        }
        cycle();
    }
    AD_CUDA(cudaGetLastError());
    Ctl cend;
    if ((rc = read_ctl(&cend))) return rc;
    if (cend.status != 0) return cend.status;
    if ((rc = save(ckpt + (size_t)nseg * snapD))) return rc;

    // the adjoint of the final state: the masked terminal energy sum(e * volo)
    // seeds e with volo on the masked elements; otherwise the caller's seeds
    AD_CUDA(cudaMemsetAsync(nbar, 0, 8 * 6 * (size_t)N, st));
    AD_CUDA(cudaMemsetAsync(ebar, 0, 8 * 5 * (size_t)E, st));
    AD_CUDA(cudaMemsetAsync(hgAcc, 0, 8, st));
    if (io.mask) {
        std::vector<double> e(E), volo(E);
        AD_CUDA(cudaMemcpyAsync(e.data(), S.e, 8 * (size_t)E, cudaMemcpyDeviceToHost, st));
        AD_CUDA(cudaMemcpyAsync(volo.data(), S.volo, 8 * (size_t)E, cudaMemcpyDeviceToHost, st));
        AD_CUDA(cudaStreamSynchronize(st));
        double j = 0.;
        std::vector<double> eb0(E, 0.);
        for (int i = 0; i < E; ++i)
            if (io.mask[i]) {
                j += e[i] * volo[i];
                eb0[i] = volo[i];
            }
        if (J) *J = j;
        AD_CUDA(cudaMemcpyAsync(ebar, eb0.data(), 8 * (size_t)E, cudaMemcpyHostToDevice, st));
    } else {
        for (int f = 0; f < kAdjFields; ++f) {
            if (!io.seed || !io.seed[f]) continue;
            double *dst = f < 6 ? nbar + (size_t)f * N : ebar + (size_t)(f - 6) * E;
            AD_CUDA(cudaMemcpyAsync(dst, io.seed[f], 8 * (size_t)(f < 6 ? N : E),
                                    cudaMemcpyHostToDevice, st));
        }
        AD_CUDA(cudaStreamSynchronize(st));  // the seeds are the caller's memory
    }

    AdjArgs A;
    for (int i = 0; i < 6; ++i) A.nb[i] = nbar + (size_t)i * N;
    A.eb = ebar;
    A.pb = ebar + E;
    A.qb = ebar + 2 * (size_t)E;
    A.vb = ebar + 3 * (size_t)E;
    A.ssb = ebar + 4 * (size_t)E;
    A.vnewb = vnewb;
    for (int d = 0; d < 3; ++d) {
        A.delxb[d] = dxb + (size_t)d * E;
        A.delvb[d] = dvb + (size_t)d * E;
    }
    A.slot = slot;
    A.corner = corner;
    A.fb = fb;
    A.hgPart = hgPart;
    A.revStart = d_revStart;
    A.revEntry = d_revEntry;
    A.hg = io.hgcoef;

    // backward over segments
    for (int sg = nseg - 1; sg >= 0; --sg) {
        const int cb = sg * K, ce = std::min(cb + K, io.ncycles);
        if ((rc = restore(ckpt + (size_t)sg * snapD))) return rc;
        Ctl cs = ckctl[sg];
        cs.cycle_limit = c0.cycle + ce;  // absolute, like the cycle counter
        if ((rc = write_ctl(cs))) return rc;
        for (int c = cb; c < ce; ++c) {
            if ((rc = save(seg + (size_t)(c - cb) * snapD))) return rc;
            cycle();
            for (int t = 0; t < 8; ++t)
                AD_CUDA(cudaMemcpyAsync(tmp + (size_t)(c - cb) * tempD + (size_t)t * E, live_t[t],
                                        8 * (size_t)E, cudaMemcpyDeviceToDevice, st));
        }
        if ((rc = save(seg + (size_t)(ce - cb) * snapD))) return rc;
        Ctl cr;
        if ((rc = read_ctl(&cr))) return rc;
        if (cr.status != 0 || cr.cycle != c0.cycle + ce)
            return err(LG_ERR_STATE, "adjoint: the recomputed segment ended at cycle %d (status %d), "
                                     "not %d", cr.cycle, cr.status, c0.cycle + ce);
        for (int c = ce - 1; c >= cb; --c) {
            A.s0 = snap_at(seg + (size_t)(c - cb) * snapD);
            A.s1 = snap_at(seg + (size_t)(c - cb + 1) * snapD);
            for (int t = 0; t < 8; ++t) A.tc.t[t] = tmp + (size_t)(c - cb) * tempD + (size_t)t * E;
            A.dt = io.dts[c];
            ka_material<<<eb, kB, 0, st>>>(S, A);
            ka_qslots<<<eb, kB, 0, st>>>(S, A);
            ka_kinematics<<<eb, kB, 0, st>>>(S, A);
            ka_nodes<<<nbk, kB, 0, st>>>(S, A);
            ka_forces<<<eb, kB, 0, st>>>(S, A);
            ka_gather<<<nbk, kB, 0, st>>>(S, A);
            ka_hg_sum<<<1, kB, 0, st>>>(hgPart, eb, hgAcc);
        }
        AD_CUDA(cudaGetLastError());
    }
    for (int f = 0; f < kAdjFields; ++f) {
        if (!io.grad || !io.grad[f]) continue;
        const double *src = f < 6 ? nbar + (size_t)f * N : ebar + (size_t)(f - 6) * E;
        AD_CUDA(cudaMemcpyAsync(io.grad[f], src, 8 * (size_t)(f < 6 ? N : E),
                                cudaMemcpyDeviceToHost, st));
    }
    AD_CUDA(cudaMemcpyAsync(dJdhg, hgAcc, 8, cudaMemcpyDeviceToHost, st));
    // leave the handle in the final forward state
    if ((rc = restore(ckpt + (size_t)nseg * snapD))) return rc;
    if ((rc = write_ctl(cend))) return rc;
    AD_CUDA(cudaStreamSynchronize(st));
    return LG_OK;
}

}  // namespace lg
