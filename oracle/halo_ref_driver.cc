// halo_ref_driver.cc -- the reference's own halo exchange (lulesh-comm.cc,
// unchanged) run for every rank of a tp x tp x tp decomposition inside one
// process, over the in-process MPI stand-in of mpi_stub/mpi.h.  Test
// infrastructure only (it pins the halo restatement halo_oracle.py and the
// GPU halo kernels to the reference): compiled by `make -C oracle halo` from
// the reference sources where they lie, with -DUSE_MPI=1.
//
// Entry points (extern "C"):
//   hr_create(tp, nx)         tp^3 Domains as main() builds them on each rank
//                             (InitMeshDecomp + Domain::Domain, lulesh.cc:2710-2716)
//   hr_field(rank, name, &n)  a Domain field array (x y z xd yd zd fx fy fz
//                             nodalMass; delv_xi delv_eta delv_zeta with their
//                             ghost elements after hr_alloc_gradients)
//   hr_alloc_gradients()      Domain::AllocateGradients with the ghost count of
//                             CalcQForElems (lulesh.cc:1955-1960) on every rank
//   hr_exchange(kind)         0: CommRecv/CommSend/CommSBN of fx fy fz
//                             (lulesh.cc:1109-1133); 1: of CommSyncPosVel's x y z
//                             xd yd zd (lulesh.cc:2621-2642); 2: CommMonoQ of
//                             delv_xi/eta/zeta (lulesh.cc:1963-1985); 3: CommSBN
//                             of nodalMass alone (lulesh.cc:2723-2729)
//   hr_send_buffer / hr_recv_buffer(rank, &n)   commDataSend / commDataRecv
//   hr_destroy()
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "lulesh.h"

// ---------------------------------------------------------------- MPI stand-in
static int g_rank = 0;

namespace {
struct PendingRecv {
    void *buf;
    size_t bytes;
    int source, dest, tag;
};
std::map<std::tuple<int, int, int>, std::vector<std::vector<char>>> g_mailbox;
std::vector<PendingRecv> g_recvs;

[[noreturn]] void die(const char *what)
{
    std::fprintf(stderr, "mpi stand-in: %s\n", what);
    std::abort();
}
size_t type_size(MPI_Datatype t) { return t == MPI_FLOAT ? 4 : 8; }
}  // namespace

extern "C" {
int MPI_Comm_rank(MPI_Comm, int *rank)
{
    *rank = g_rank;
    return 0;
}
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm,
              MPI_Request *req)
{
    const char *p = static_cast<const char *>(buf);
    g_mailbox[std::make_tuple(g_rank, dest, tag)].emplace_back(p, p + count * type_size(type));
    *req = MPI_REQUEST_NULL;
    return 0;
}
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm,
              MPI_Request *req)
{
    g_recvs.push_back({buf, count * type_size(type), source, g_rank, tag});
    *req = (int)g_recvs.size() - 1;
    return 0;
}
int MPI_Wait(MPI_Request *req, MPI_Status *)
{
    if (*req == MPI_REQUEST_NULL) return 0;
    if (*req < 0 || *req >= (int)g_recvs.size()) die("unknown request");
    PendingRecv &r = g_recvs[*req];
    auto it = g_mailbox.find(std::make_tuple(r.source, r.dest, r.tag));
    if (it == g_mailbox.end() || it->second.empty()) die("no matching message");
    std::vector<char> msg = std::move(it->second.front());
    it->second.erase(it->second.begin());
    if (msg.size() != r.bytes) die("message size mismatch");
    std::memcpy(r.buf, msg.data(), msg.size());
    *req = MPI_REQUEST_NULL;
    return 0;
}
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *)
{
    for (int i = 0; i < n; ++i)
        if (reqs[i] != MPI_REQUEST_NULL && reqs[i] >= 0) MPI_Wait(&reqs[i], nullptr);
    return 0;
}
int MPI_Abort(MPI_Comm, int code)
{
    std::fprintf(stderr, "MPI_Abort(%d)\n", code);
    std::exit(code);
}
int MPI_Init(int *, char ***) { die("MPI_Init is not part of the halo exchange"); }
int MPI_Init_thread(int *, char ***, int, int *) { die("MPI_Init_thread called"); }
int MPI_Comm_size(MPI_Comm, int *) { die("MPI_Comm_size called"); }
int MPI_Barrier(MPI_Comm) { die("MPI_Barrier called"); }
int MPI_Finalize(void) { die("MPI_Finalize called"); }
double MPI_Wtime(void) { die("MPI_Wtime called"); }
int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm)
{
    die("MPI_Allreduce called");
}
int MPI_Reduce(const void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm)
{
    die("MPI_Reduce called");
}
}

// ---------------------------------------------------------------- the driver
namespace {
std::vector<Domain *> g_doms;
int g_tp = 0;
bool g_gradients = false;  // AllocateGradients has run on every Domain

void post_all(int kind)
{
    const int nr = (int)g_doms.size();
    Domain_member fx[3] = {&Domain::fx, &Domain::fy, &Domain::fz};
    Domain_member pv[6] = {&Domain::x, &Domain::y, &Domain::z,
                           &Domain::xd, &Domain::yd, &Domain::zd};
    Domain_member dq[3] = {&Domain::delv_xi, &Domain::delv_eta, &Domain::delv_zeta};
    Domain_member nm[1] = {&Domain::nodalMass};
    // every rank posts its receives, then every rank sends, then every rank
    // unpacks: the order main() reaches these calls on each rank
    for (int r = 0; r < nr; ++r) {
        g_rank = r;
        Domain &d = *g_doms[r];
        const Index_t nx = d.sizeX() + 1, ny = d.sizeY() + 1, nz = d.sizeZ() + 1;
        switch (kind) {
        case 0: CommRecv(d, MSG_COMM_SBN, 3, nx, ny, nz, true, false); break;
        case 1: CommRecv(d, MSG_SYNC_POS_VEL, 6, nx, ny, nz, false, false); break;
        case 2: CommRecv(d, MSG_MONOQ, 3, d.sizeX(), d.sizeY(), d.sizeZ(), true, true); break;
        case 3: CommRecv(d, MSG_COMM_SBN, 1, nx, ny, nz, true, false); break;
        }
    }
    for (int r = 0; r < nr; ++r) {
        g_rank = r;
        Domain &d = *g_doms[r];
        const Index_t nx = d.sizeX() + 1, ny = d.sizeY() + 1, nz = d.sizeZ() + 1;
        switch (kind) {
        case 0: CommSend(d, MSG_COMM_SBN, 3, fx, nx, ny, nz, true, false); break;
        case 1: CommSend(d, MSG_SYNC_POS_VEL, 6, pv, nx, ny, nz, false, false); break;
        case 2: CommSend(d, MSG_MONOQ, 3, dq, d.sizeX(), d.sizeY(), d.sizeZ(), true, true); break;
        case 3: CommSend(d, MSG_COMM_SBN, 1, nm, nx, ny, nz, true, false); break;
        }
    }
    for (int r = 0; r < nr; ++r) {
        g_rank = r;
        Domain &d = *g_doms[r];
        switch (kind) {
        case 0: CommSBN(d, 3, fx); break;
        case 1: CommSyncPosVel(d); break;
        case 2: CommMonoQ(d); break;
        case 3: CommSBN(d, 1, nm); break;
        }
    }
    g_recvs.clear();
    for (auto &kv : g_mailbox)
        if (!kv.second.empty()) die("unreceived message");
    g_mailbox.clear();
}
}  // namespace

extern "C" {
void hr_destroy()
{
    for (Domain *d : g_doms) {
        if (g_gradients) d->DeallocateGradients();
        delete d;
    }
    g_doms.clear();
    g_gradients = false;
}

int hr_create(int tp, int nx)
{
    hr_destroy();
    g_tp = tp;
    const int nranks = tp * tp * tp;
    for (int r = 0; r < nranks; ++r) {
        g_rank = r;
        Int_t col, row, plane, side;
        InitMeshDecomp(nranks, r, &col, &row, &plane, &side);
        g_doms.push_back(new Domain(nranks, col, row, plane, nx, side, 11, 1, 1));
    }
    return nranks;
}

void hr_alloc_gradients()
{
    for (Domain *d : g_doms) {
        const Int_t numElem = d->numElem();
        const Int_t allElem = numElem + 2 * d->sizeX() * d->sizeY() +
                              2 * d->sizeX() * d->sizeZ() + 2 * d->sizeY() * d->sizeZ();
        d->AllocateGradients(numElem, allElem);
    }
    g_gradients = true;
}

double *hr_field(int rank, const char *name, size_t *n)
{
    Domain &d = *g_doms[rank];
    const size_t N = d.numNode(), E = d.numElem();
    const size_t G = E + 2 * d.sizeX() * d.sizeY() + 2 * d.sizeX() * d.sizeZ() +
                     2 * d.sizeY() * d.sizeZ();
    struct { const char *nm; Domain_member m; size_t len; } t[] = {
        {"x", &Domain::x, N},   {"y", &Domain::y, N},   {"z", &Domain::z, N},
        {"xd", &Domain::xd, N}, {"yd", &Domain::yd, N}, {"zd", &Domain::zd, N},
        {"fx", &Domain::fx, N}, {"fy", &Domain::fy, N}, {"fz", &Domain::fz, N},
        {"nodalMass", &Domain::nodalMass, N}, {"delv_xi", &Domain::delv_xi, G},
        {"delv_eta", &Domain::delv_eta, G}, {"delv_zeta", &Domain::delv_zeta, G}};
    for (auto &f : t)
        if (!std::strcmp(f.nm, name)) {
            *n = f.len;
            return &(d.*f.m)(0);
        }
    *n = 0;
    return nullptr;
}

int hr_loc(int rank, int *col, int *row, int *plane)
{
    Domain &d = *g_doms[rank];
    *col = d.colLoc();
    *row = d.rowLoc();
    *plane = d.planeLoc();
    return d.sizeX();
}

void hr_exchange(int kind) { post_all(kind); }

static size_t comm_doubles(Domain &d)
{
    // SetupCommBuffers' comBufSize (lulesh-init.cc:358-380)
    const int rmn = d.rowLoc() != 0, rmx = d.rowLoc() != g_tp - 1, cmn = d.colLoc() != 0,
              cmx = d.colLoc() != g_tp - 1, pmn = d.planeLoc() != 0, pmx = d.planeLoc() != g_tp - 1;
    size_t s = (size_t)(rmn + rmx + cmn + cmx + pmn + pmx) * d.maxPlaneSize() *
               MAX_FIELDS_PER_MPI_COMM;
    s += (size_t)((rmn & cmn) + (rmn & pmn) + (cmn & pmn) + (rmx & cmx) + (rmx & pmx) +
                  (cmx & pmx) + (rmx & cmn) + (rmn & pmx) + (cmn & pmx) + (rmn & cmx) +
                  (rmx & pmn) + (cmx & pmn)) *
         d.maxEdgeSize() * MAX_FIELDS_PER_MPI_COMM;
    s += (size_t)((rmn & cmn & pmn) + (rmn & cmn & pmx) + (rmn & cmx & pmn) +
                  (rmn & cmx & pmx) + (rmx & cmn & pmn) + (rmx & cmn & pmx) +
                  (rmx & cmx & pmn) + (rmx & cmx & pmx)) *
         CACHE_COHERENCE_PAD_REAL;
    return s;
}

double *hr_send_buffer(int rank, size_t *n)
{
    *n = comm_doubles(*g_doms[rank]);
    return g_doms[rank]->commDataSend;
}

double *hr_recv_buffer(int rank, size_t *n)
{
    *n = comm_doubles(*g_doms[rank]);
    return g_doms[rank]->commDataRecv;
}
}
