// lg_halo.cu -- halo pack/unpack of a block decomposition on the GPU.
//
// The reference runs one Domain per MPI rank on a tp x tp x tp grid of cubes
// of nx elements (InitMeshDecomp, lulesh-init.cc:676-738) and exchanges the
// cubes' boundary values three ways (lulesh-comm.cc):
//   CommSBN         node fields (forces, nodal mass): each neighbour's values
//                   at shared nodes are added, message after message (848)
//   CommSyncPosVel  positions and velocities: the shared nodes take the
//                   higher-ranked neighbour's values (1261)
//   CommMonoQ       element velocity gradients of the neighbours' boundary
//                   layers, copied into ghost elements after numElem (1684)
// CommSend (357) packs up to 26 messages per rank (6 faces, 12 edges, 8
// corners), CommRecv (59) posts their receive buffers, and MPI moves them.
//
// Here a plan, built once per (kind, nx, tp, rank, nfields) on the host,
// describes every message of one rank by its neighbour direction d =
// (dcol, drow, dplane): the message's values are the rank's lattice points
// with coordinate 0 on axes where d is -1, the last coordinate where d is +1,
// and every coordinate where d is 0, plane (z) slowest and x fastest -- the
// order of the reference's packing loops.  Messages keep the reference's
// sequence and buffer layout (faces, then edges, then corners, at
// pmsg*maxPlaneComm + emsg*maxEdgeComm + cmsg*16 doubles, fields one after
// another within a message), so the buffers are interchangeable with the
// reference's commDataSend / commDataRecv and a rank of this code can
// exchange messages with a rank of the reference.
//
// Kernels (no atomics, deterministic):
//   k_halo_pack    one thread per packed value: buf[pos + f*count] = field_f[index]
//   k_halo_unpack  one thread per receiving lattice point, which applies its
//                  messages' values in the reference's message order: added
//                  (CommSBN: ((v + a1) + a2) ..., the reference's rounding),
//                  or copied (the last message wins, as in CommSyncPosVel;
//                  CommMonoQ's ghost slots get exactly one value each)
// Moving the messages between ranks (MPI, NCCL, peer copies) is the caller's:
// lg_halo_plan_message gives each message's peer, length and offset.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "lulesh_gb300.h"

namespace lg {
// lg_api.cu: records the text lg_last_error() returns on this thread.
int record_error(int code, const char *msg);
}  // namespace lg

struct lg_halo_plan {
    int kind = 0, nx = 0, tp = 0, rank = 0, nfields = 0;
    lg_halo_info info{};
    struct Msg {
        int peer, count;
        size_t offset;
    };
    std::vector<Msg> send, recv;
    // send entries in buffer order; receive entries grouped by target in the
    // order they are applied
    std::vector<int> s_index, s_pos, s_stride;
    std::vector<int> r_target, r_start, r_pos, r_stride;
    // device copies, made on first use
    int device = -1;
    int *d_s_index = nullptr, *d_s_pos = nullptr, *d_s_stride = nullptr;
    int *d_r_target = nullptr, *d_r_start = nullptr, *d_r_pos = nullptr, *d_r_stride = nullptr;
};

namespace {

constexpr int kMaxHaloFields = 6;  // MAX_FIELDS_PER_MPI_COMM (lulesh.h:94)
constexpr int kPad = 16;           // CACHE_COHERENCE_PAD_REAL doubles (lulesh.h:98)

int fail(int code, const char *msg) { return lg::record_error(code, msg); }

size_t align_pad(size_t n) { return (n + kPad - 1) & ~(size_t)(kPad - 1); }

struct Dir {
    int c, r, p;  // dcol, drow, dplane
};
// The reference's message sequence: faces (planeMin, planeMax, rowMin,
// rowMax, colMin, colMax), edges, corners (lulesh-comm.cc:407-842).
const Dir kOrder[26] = {
    {0, 0, -1},  {0, 0, 1},   {0, -1, 0},  {0, 1, 0},   {-1, 0, 0},  {1, 0, 0},
    {-1, -1, 0}, {0, -1, -1}, {-1, 0, -1}, {1, 1, 0},   {0, 1, 1},   {1, 0, 1},
    {-1, 1, 0},  {0, -1, 1},  {-1, 0, 1},  {1, -1, 0},  {0, 1, -1},  {1, 0, -1},
    {-1, -1, -1}, {-1, -1, 1}, {1, -1, -1}, {1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},
    {1, 1, -1},  {1, 1, 1}};

int nonzero(const Dir &d) { return (d.c != 0) + (d.r != 0) + (d.p != 0); }

// +1 when the neighbour in direction d has the higher rank (the first
// non-zero of dplane, drow, dcol is positive), -1 when it has the lower.
int rank_side(const Dir &d) { return d.p ? d.p : d.r ? d.r : d.c; }

// Lattice indices of the box toward d on an n^3 lattice, plane slowest.
void box(const Dir &d, int n, std::vector<int> &out)
{
    auto range = [n](int dd, int &lo, int &hi) {
        lo = dd > 0 ? n - 1 : 0;
        hi = dd < 0 ? 1 : n;
    };
    int x0, x1, y0, y1, z0, z1;
    range(d.c, x0, x1);
    range(d.r, y0, y1);
    range(d.p, z0, z1);
    out.clear();
    for (int z = z0; z < z1; ++z)
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) out.push_back(x + n * (y + n * z));
}

int build(lg_halo_plan &pl)
{
    const int tp = pl.tp, nx = pl.nx, nf = pl.nfields;
    const int col = pl.rank % tp, row = (pl.rank / tp) % tp, plane = pl.rank / (tp * tp);
    // the call sites: CalcForceForNodes (lulesh.cc:1109-1133) and the nodal
    // mass (2723-2729) send both ways on the node lattice; the position /
    // velocity sync (2621-2642) sends only to lower ranks and receives only
    // from higher ones; CalcQForElems (1963-1985) sends the six faces of the
    // element lattice
    const bool nodes = pl.kind != LG_HALO_MONOQ;
    const int n = nodes ? nx + 1 : nx;
    const bool one_way = pl.kind == LG_HALO_SYNC_POS_VEL;
    const int max_classes = pl.kind == LG_HALO_MONOQ ? 1 : 3;
    const size_t max_plane = (size_t)nf * align_pad((size_t)(nx + 1) * (nx + 1));
    const size_t max_edge = (size_t)nf * align_pad((size_t)nx + 1);

    size_t cnt_send[3] = {0, 0, 0}, cnt_recv[3] = {0, 0, 0};
    size_t ghost = (size_t)nx * nx * nx;
    int nbr_faces = 0, nbr_edges = 0, nbr_corners = 0;
    std::vector<int> idx;
    struct RecvEntry {
        int target, seq, pos, stride;
    };
    std::vector<RecvEntry> rents;
    int seq = 0;
    for (const Dir &d : kOrder) {
        const int cls = nonzero(d) - 1;  // 0 face, 1 edge, 2 corner
        const int nc = col + d.c, nr = row + d.r, np = plane + d.p;
        if (nc < 0 || nc >= tp || nr < 0 || nr >= tp || np < 0 || np >= tp) continue;
        (cls == 0 ? nbr_faces : cls == 1 ? nbr_edges : nbr_corners)++;
        if (cls >= max_classes) continue;
        const int peer = nc + tp * (nr + tp * np);
        box(d, n, idx);
        const int count = (int)idx.size();
        const int side = rank_side(d);
        if (!one_way || side < 0) {
            const size_t off = cnt_send[0] * max_plane + cnt_send[1] * max_edge + cnt_send[2] * kPad;
            ++cnt_send[cls];
            pl.send.push_back({peer, count, off});
            for (int i = 0; i < count; ++i) {
                pl.s_index.push_back(idx[i]);
                pl.s_pos.push_back((int)(off + i));
                pl.s_stride.push_back(count);
            }
        }
        if (!one_way || side > 0) {
            const size_t off = cnt_recv[0] * max_plane + cnt_recv[1] * max_edge + cnt_recv[2] * kPad;
            ++cnt_recv[cls];
            pl.recv.push_back({peer, count, off});
            for (int i = 0; i < count; ++i) {
                const int target = nodes ? idx[i] : (int)(ghost + i);
                rents.push_back({target, seq++, (int)(off + i), count});
            }
            if (!nodes) ghost += count;
        }
    }
    // group the receive entries by target, keeping the message order
    std::stable_sort(rents.begin(), rents.end(),
                     [](const RecvEntry &a, const RecvEntry &b) { return a.target < b.target; });
    for (size_t i = 0; i < rents.size(); ++i) {
        if (i == 0 || rents[i].target != rents[i - 1].target) {
            pl.r_target.push_back(rents[i].target);
            pl.r_start.push_back((int)i);
        }
        pl.r_pos.push_back(rents[i].pos);
        pl.r_stride.push_back(rents[i].stride);
    }
    pl.r_start.push_back((int)rents.size());

    lg_halo_info &in = pl.info;
    // SetupCommBuffers' comBufSize (lulesh-init.cc:358-380), which sizes for
    // MAX_FIELDS_PER_MPI_COMM fields whatever the call site sends
    in.buffer_doubles = (size_t)nbr_faces * align_pad((size_t)(nx + 1) * (nx + 1)) * kMaxHaloFields +
                        (size_t)nbr_edges * align_pad((size_t)nx + 1) * kMaxHaloFields +
                        (size_t)nbr_corners * kPad;
    in.send_messages = (int)pl.send.size();
    in.recv_messages = (int)pl.recv.size();
    in.send_values = (int)pl.s_index.size();
    in.recv_values = (int)pl.r_pos.size();
    in.recv_targets = (int)pl.r_target.size();
    in.ghost_elems = nodes ? 0 : (int)(ghost - (size_t)nx * nx * nx);
    in.field_length = nodes ? (nx + 1) * (nx + 1) * (nx + 1) : nx * nx * nx + in.ghost_elems;
    return LG_OK;
}

struct Fields {
    double *f[kMaxHaloFields];
};

__global__ void k_halo_pack(int n, int nf, Fields fl, const int *__restrict__ index,
                            const int *__restrict__ pos, const int *__restrict__ stride,
                            double *__restrict__ buf)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int i = index[e], p = pos[e], s = stride[e];
    for (int f = 0; f < nf; ++f) buf[p + (size_t)f * s] = fl.f[f][i];
}

template <bool ADD>
__global__ void k_halo_unpack(int nt, int nf, Fields fl, const int *__restrict__ target,
                              const int *__restrict__ start, const int *__restrict__ pos,
                              const int *__restrict__ stride, const double *__restrict__ buf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int i = target[t], b = start[t], e = start[t + 1];
    for (int f = 0; f < nf; ++f) {
        double v = fl.f[f][i];
        for (int k = b; k < e; ++k) {
            const double m = buf[pos[k] + (size_t)f * stride[k]];
            v = ADD ? __dadd_rn(v, m) : m;
        }
        fl.f[f][i] = v;
    }
}

template <typename T>
int upload(T **dst, const std::vector<T> &src)
{
    const size_t bytes = std::max<size_t>(1, src.size()) * sizeof(T);
    if (cudaMalloc((void **)dst, bytes) != cudaSuccess) return LG_ERR_NOMEM;
    if (!src.empty() &&
        cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return LG_ERR_CUDA;
    return LG_OK;
}

void free_device(lg_halo_plan *p)
{
    int *ptrs[] = {p->d_s_index, p->d_s_pos, p->d_s_stride, p->d_r_target,
                   p->d_r_start, p->d_r_pos,  p->d_r_stride};
    for (int *q : ptrs)
        if (q) cudaFree(q);
    p->d_s_index = p->d_s_pos = p->d_s_stride = nullptr;
    p->d_r_target = p->d_r_start = p->d_r_pos = p->d_r_stride = nullptr;
    p->device = -1;
}

// device copies of the plan on the current device, made by the first pack or
// unpack; a plan serves one device
int ensure_device(lg_halo_plan *p)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(LG_ERR_CUDA, "no CUDA device");
    if (p->device == dev) return LG_OK;
    if (p->device >= 0)
        return fail(LG_ERR_INVALID, "halo plan: first used on another device");
    int st;
    if ((st = upload(&p->d_s_index, p->s_index)) || (st = upload(&p->d_s_pos, p->s_pos)) ||
        (st = upload(&p->d_s_stride, p->s_stride)) ||
        (st = upload(&p->d_r_target, p->r_target)) ||
        (st = upload(&p->d_r_start, p->r_start)) || (st = upload(&p->d_r_pos, p->r_pos)) ||
        (st = upload(&p->d_r_stride, p->r_stride))) {
        free_device(p);
        return fail(st, "halo plan: device upload failed");
    }
    p->device = dev;
    return LG_OK;
}

int get_fields(const lg_halo_plan *p, double *const *fields, Fields &fl)
{
    if (!fields) return fail(LG_ERR_INVALID, "halo: null field array");
    std::memset(&fl, 0, sizeof fl);
    for (int f = 0; f < p->nfields; ++f) {
        if (!fields[f]) return fail(LG_ERR_INVALID, "halo: null field pointer");
        fl.f[f] = fields[f];
    }
    return LG_OK;
}

}  // namespace

extern "C" {

int lg_halo_plan_create(int kind, int nx, int tp, int rank, int nfields, lg_halo_plan **out)
{
    if (!out) return fail(LG_ERR_INVALID, "lg_halo_plan_create: null output");
    *out = nullptr;
    if (kind < LG_HALO_SBN || kind > LG_HALO_MONOQ)
        return fail(LG_ERR_INVALID, "lg_halo_plan_create: unknown kind");
    if (nx < 1 || tp < 1 || rank < 0 || rank >= tp * tp * tp)
        return fail(LG_ERR_INVALID, "lg_halo_plan_create: invalid nx, tp or rank");
    if (nfields < 1 || nfields > kMaxHaloFields)
        return fail(LG_ERR_INVALID, "lg_halo_plan_create: nfields must be 1..6");
    // every buffer position and lattice index must fit in an int
    if ((long long)(nx + 1) * (nx + 1) * (nx + 1) * 2 > 2147483647LL ||
        (long long)26 * kMaxHaloFields * (nx + 16) * (nx + 16) > 2147483647LL)
        return fail(LG_ERR_INVALID, "lg_halo_plan_create: nx too large");
    lg_halo_plan *p = new lg_halo_plan();
    p->kind = kind;
    p->nx = nx;
    p->tp = tp;
    p->rank = rank;
    p->nfields = nfields;
    build(*p);
    *out = p;
    return LG_OK;
}

void lg_halo_plan_destroy(lg_halo_plan *p)
{
    if (!p) return;
    if (p->device >= 0) {
        int cur = -1;
        cudaGetDevice(&cur);
        cudaSetDevice(p->device);
        free_device(p);
        if (cur >= 0) cudaSetDevice(cur);
    }
    delete p;
}

int lg_halo_plan_info(const lg_halo_plan *p, lg_halo_info *info)
{
    if (!p || !info) return fail(LG_ERR_INVALID, "lg_halo_plan_info: null argument");
    *info = p->info;
    return LG_OK;
}

int lg_halo_plan_message(const lg_halo_plan *p, int dir, int m, int *peer, int *count,
                         size_t *offset)
{
    if (!p || (dir != 0 && dir != 1)) return fail(LG_ERR_INVALID, "lg_halo_plan_message: bad argument");
    const auto &v = dir == 0 ? p->send : p->recv;
    if (m < 0 || m >= (int)v.size()) return fail(LG_ERR_INVALID, "lg_halo_plan_message: no such message");
    if (peer) *peer = v[m].peer;
    if (count) *count = v[m].count;
    if (offset) *offset = v[m].offset;
    return LG_OK;
}

int lg_halo_plan_entries(const lg_halo_plan *p, int dir, int *index, int *bufpos, int *stride,
                         size_t n)
{
    if (!p || (dir != 0 && dir != 1)) return fail(LG_ERR_INVALID, "lg_halo_plan_entries: bad argument");
    const size_t want = dir == 0 ? p->s_index.size() : p->r_pos.size();
    if (n != want) return fail(LG_ERR_INVALID, "lg_halo_plan_entries: n must equal the value count");
    for (size_t k = 0; k < n; ++k) {
        if (dir == 0) {
            if (index) index[k] = p->s_index[k];
            if (bufpos) bufpos[k] = p->s_pos[k];
            if (stride) stride[k] = p->s_stride[k];
        } else {
            if (bufpos) bufpos[k] = p->r_pos[k];
            if (stride) stride[k] = p->r_stride[k];
        }
    }
    if (dir == 1 && index)  // the target of every entry, in application order
        for (size_t t = 0; t + 1 < p->r_start.size(); ++t)
            for (int k = p->r_start[t]; k < p->r_start[t + 1]; ++k) index[k] = p->r_target[t];
    return LG_OK;
}

int lg_halo_pack(lg_halo_plan *p, double *const *fields, double *send_buf, void *stream)
{
    if (!p) return fail(LG_ERR_INVALID, "lg_halo_pack: null plan");
    const int n = p->info.send_values;
    if (n == 0) return LG_OK;  // no neighbour (tp = 1): nothing to pack
    if (!send_buf) return fail(LG_ERR_INVALID, "lg_halo_pack: null buffer");
    Fields fl;
    int st;
    if ((st = get_fields(p, fields, fl)) || (st = ensure_device(p))) return st;
    (void)cudaGetLastError();
    k_halo_pack<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        n, p->nfields, fl, p->d_s_index, p->d_s_pos, p->d_s_stride, send_buf);
    if (cudaGetLastError() != cudaSuccess) return fail(LG_ERR_CUDA, "lg_halo_pack: launch failed");
    return LG_OK;
}

int lg_halo_unpack(lg_halo_plan *p, double *const *fields, const double *recv_buf, void *stream)
{
    if (!p) return fail(LG_ERR_INVALID, "lg_halo_unpack: null plan");
    const int nt = p->info.recv_targets;
    if (nt == 0) return LG_OK;  // no neighbour: nothing received
    if (!recv_buf) return fail(LG_ERR_INVALID, "lg_halo_unpack: null buffer");
    Fields fl;
    int st;
    if ((st = get_fields(p, fields, fl)) || (st = ensure_device(p))) return st;
    (void)cudaGetLastError();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int grid = (nt + 255) / 256;
    if (p->kind == LG_HALO_SBN)
        k_halo_unpack<true><<<grid, 256, 0, s>>>(nt, p->nfields, fl, p->d_r_target, p->d_r_start,
                                                  p->d_r_pos, p->d_r_stride, recv_buf);
    else
        k_halo_unpack<false><<<grid, 256, 0, s>>>(nt, p->nfields, fl, p->d_r_target, p->d_r_start,
                                                   p->d_r_pos, p->d_r_stride, recv_buf);
    if (cudaGetLastError() != cudaSuccess) return fail(LG_ERR_CUDA, "lg_halo_unpack: launch failed");
    return LG_OK;
}

}  // extern "C"
