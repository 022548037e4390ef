// lg_setup.cu -- the Sedov set-up of Domain::Domain built on the device.
//
// The structured mesh of one rank (lulesh-init.cc:16-194, 218-673) is a
// function of the node and element indices, so every array follows from its
// index in one pass, instead of being built by the host loops and uploaded:
//   k_setup_topology  nodelist (element- and corner-major), the six
//                     neighbour lists, elemBC, the symmetry-plane bits and
//                     the node -> element-corner CSR (nodeElemStart,
//                     nodeElemCornerList), lulesh-init.cc:218-337, 514-673;
//   k_setup_elems     the element fields: volo and elemMass from the corner
//                     coordinates (CalcElemVolume), the deposited energy in
//                     element 0, v = 1, everything else zero;
//   k_setup_nodes     the node fields: BuildMesh coordinates, zero
//                     velocities, accelerations and forces, and nodalMass,
//                     the sum of volo / 8 over the node's elements in
//                     ascending element order (the reference's serial
//                     accumulation order, lulesh-init.cc:159-178).
// The region draw stays on the host: it follows the reference's sequential
// random stream (lulesh-init.cc:401-490) and is uploaded.
//
// An ensemble member is set up through a view of the concatenated arrays
// (every pointer moved to the member's first element or node): the ids it
// writes are shifted by the member's first element and node, the
// corner-major nodelist keeps the ensemble's stride, and each element and
// node records its member.
//
// Compiled without FMA contraction: coordinates, volumes and masses must
// round as the host set-up's do, bit for bit.  The state kernels derive the
// mesh from the indices, not from the nodelist array, so a reset restores the
// original set-up state even after a caller replaced the topology.
#include <cuda_runtime.h>

#include <cstdint>

#include "lg_device.h"
#include "lg_geometry.cuh"

namespace lg {
namespace {

constexpr int kSetupBlock = 256;

// BuildMesh coordinate of grid line i (lulesh-init.cc:229-245)
__device__ __forceinline__ double grid(int i, int nx)
{
    return 1.125 * double(i) / double(nx);
}

// corner number of the node at offset (di, dj, dk) from an element's first
// node (lulesh-init.cc:251-258)
__device__ __forceinline__ int corner_of(int di, int dj, int dk)
{
    return dk * 4 + (dj ? (di ? 2 : 3) : (di ? 1 : 0));
}

// number of corners on grid line i of nx elements: 1 on the faces, 2 inside
__device__ __forceinline__ long long corners_on(int i, int nx)
{
    return (i == 0 || i == nx) ? 1 : 2;
}

// corners on grid lines 0..i-1
__device__ __forceinline__ long long corners_before(int i)
{
    return i == 0 ? 0 : 2LL * i - 1;
}

__global__ void k_setup_topology(DevState s, int nx, int eoff, int noff, long long tstride,
                                 int pid)
{
    const int n = nx, en = nx + 1;
    const int E = s.E, N = s.N;
    const long long nn = (long long)n * n;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        const int i = e % n, j = (e / n) % n, k = e / (int)nn;
        const int b = (k * en + j) * en + i;
        const int ln[8] = {b, b + 1, b + en + 1, b + en, b + en * en, b + en * en + 1,
                           b + en * en + en + 1, b + en * en + en};
        for (int c = 0; c < 8; ++c) {
            s.nodelist[8 * (size_t)e + c] = ln[c] + noff;
            s.nodelistT[(size_t)c * tstride + e] = ln[c] + noff;
        }
        // SetupElementConnectivities, lulesh-init.cc:539-565
        s.lxim[e] = (e == 0 ? 0 : e - 1) + eoff;
        s.lxip[e] = (e == E - 1 ? E - 1 : e + 1) + eoff;
        s.letam[e] = (e < n ? e : e - n) + eoff;
        s.letap[e] = (e >= E - n ? e : e + n) + eoff;
        s.lzetam[e] = (e < nn ? e : e - (int)nn) + eoff;
        s.lzetap[e] = (e >= E - nn ? e : e + (int)nn) + eoff;
        if (s.elemProb) s.elemProb[e] = (uint16_t)pid;
        // SetupBoundaryConditions, lulesh-init.cc:569-673 (one rank: the
        // minimum faces are symmetry planes, the maximum faces free)
        int bc = 0;
        if (k == 0) bc |= ZETA_M_SYMM;
        if (k == n - 1) bc |= ZETA_P_FREE;
        if (j == 0) bc |= ETA_M_SYMM;
        if (j == n - 1) bc |= ETA_P_FREE;
        if (i == 0) bc |= XI_M_SYMM;
        if (i == n - 1) bc |= XI_P_FREE;
        s.elemBC[e] = bc;
    }
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
        const int i = v % en, j = (v / en) % en, k = v / (en * en);
        // SetupSymmetryPlanes, lulesh-init.cc:514-533
        s.symm[v] = (uint8_t)((i == 0 ? 1 : 0) | (j == 0 ? 2 : 0) | (k == 0 ? 4 : 0));
        // SetupThreadSupportStructures, lulesh-init.cc:272-337: corners of
        // the nodes before this one (plane-major order), then this node's
        // corners in ascending element order
        const long long line = 2LL * n;  // corners on all lines of one axis
        const long long start = corners_before(k) * line * line +
                                corners_on(k, n) * corners_before(j) * line +
                                corners_on(k, n) * corners_on(j, n) * corners_before(i);
        s.nodeElemStart[v] = (int)(start + 8LL * eoff);
        if (v == N - 1) s.nodeElemStart[N] = 8 * (E + eoff);
        if (s.nodeProb) s.nodeProb[v] = (uint16_t)pid;
        int m = 0;
        for (int ek = k - 1; ek <= k; ++ek)
            for (int ej = j - 1; ej <= j; ++ej)
                for (int ei = i - 1; ei <= i; ++ei) {
                    if (ek < 0 || ek >= n || ej < 0 || ej >= n || ei < 0 || ei >= n) continue;
                    const int el = (ek * n + ej) * n + ei;
                    s.nodeElemCornerList[start + m++] =
                        8 * (el + eoff) + corner_of(i - ei, j - ej, k - ek);
                }
    }
}

__global__ void k_setup_elems(DevState s, int nx, double einit)
{
    const int n = nx;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < s.E; e += gridDim.x * blockDim.x) {
        const int i = e % n, j = (e / n) % n, k = e / (n * n);
        const double x0 = grid(i, n), x1 = grid(i + 1, n);
        const double y0 = grid(j, n), y1 = grid(j + 1, n);
        const double z0 = grid(k, n), z1 = grid(k + 1, n);
        const double xs[8] = {x0, x1, x1, x0, x0, x1, x1, x0};
        const double ys[8] = {y0, y0, y1, y1, y0, y0, y1, y1};
        const double zs[8] = {z0, z0, z0, z0, z1, z1, z1, z1};
        const double vol = geom::elem_volume<double>(xs, ys, zs);
        s.volo[e] = vol;
        s.elemMass[e] = vol;
        s.e[e] = e == 0 ? einit : 0.0;
        s.v[e] = 1.0;
        s.p[e] = s.q[e] = s.ql[e] = s.qq[e] = 0.0;
        s.vnew[e] = s.delv[e] = s.vdov[e] = s.arealg[e] = s.ss[e] = 0.0;
        s.delx_xi[e] = s.delx_eta[e] = s.delx_zeta[e] = 0.0;
        s.delv_xi[e] = s.delv_eta[e] = s.delv_zeta[e] = 0.0;
    }
}

__global__ void k_setup_nodes(DevState s, int nx)
{
    const int n = nx, en = nx + 1;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < s.N; v += gridDim.x * blockDim.x) {
        const int i = v % en, j = (v / en) % en, k = v / (en * en);
        s.x[v] = grid(i, n);
        s.y[v] = grid(j, n);
        s.z[v] = grid(k, n);
        s.xd[v] = s.yd[v] = s.zd[v] = 0.0;
        s.xdd[v] = s.ydd[v] = s.zdd[v] = 0.0;
        s.fx[v] = s.fy[v] = s.fz[v] = 0.0;
        double mass = 0.0;
        for (int ek = k - 1; ek <= k; ++ek)
            for (int ej = j - 1; ej <= j; ++ej)
                for (int ei = i - 1; ei <= i; ++ei) {
                    if (ek < 0 || ek >= n || ej < 0 || ej >= n || ei < 0 || ei >= n) continue;
                    mass += s.volo[(ek * n + ej) * n + ei] / 8.0;
                }
        s.nodalMass[v] = mass;
        s.invMass[v] = 1.0 / mass;
    }
}

// The end-of-run self-check of lulesh-util.cc:189-218 on the device: the
// symmetry of e across the x = y diagonal of plane 0.  k_verify_pairs writes
// each pair (j, k > j)'s |e(j,k) - e(k,j)| and that over e(k,j) in the
// reference's loop order; k_verify_reduce takes the maxima (kept only when
// strictly greater, as the reference keeps them, so 0/0 pairs drop out) and
// sums the differences serially in that order, so the report's values are
// the reference's to the bit.
__device__ __forceinline__ long long pair_pos(int j, int k, int nx)
{
    return (long long)j * nx - (long long)j * (j + 1) / 2 + (k - j - 1);
}

__global__ void k_verify_pairs(const double *e, int nx, double *absd, double *reld)
{
    const long long total = (long long)nx * nx;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / nx), k = (int)(idx % nx);
        if (k <= j) continue;
        const double a = fabs(e[(size_t)j * nx + k] - e[(size_t)k * nx + j]);
        const long long p = pair_pos(j, k, nx);
        absd[p] = a;
        reld[p] = a / e[(size_t)k * nx + j];
    }
}

__global__ void k_verify_reduce(const double *e, int nx, const double *absd, const double *reld,
                                double *out)
{
    __shared__ double sa[kSetupBlock], sr[kSetupBlock];
    const long long pairs = (long long)nx * (nx - 1) / 2;
    double ma = 0.0, mr = 0.0;
    for (long long p = threadIdx.x; p < pairs; p += blockDim.x) {
        if (ma < absd[p]) ma = absd[p];
        if (mr < reld[p]) mr = reld[p];
    }
    sa[threadIdx.x] = ma;
    sr[threadIdx.x] = mr;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int t = 1; t < blockDim.x; ++t) {
            if (ma < sa[t]) ma = sa[t];
            if (mr < sr[t]) mr = sr[t];
        }
        double total = 0.0;
        for (long long p = 0; p < pairs; ++p) total += absd[p];
        out[0] = e[0];
        out[1] = ma;
        out[2] = total;
        out[3] = mr;
    }
}

int blocks_for(long long n)
{
    const long long b = (n + kSetupBlock - 1) / kSetupBlock;
    return (int)(b < 1 ? 1 : (b > 65535LL * 32 ? 65535LL * 32 : b));
}

}  // namespace

__global__ void k_inv_mass(const double *m, double *inv, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) inv[i] = 1.0 / m[i];  // the IEEE quotient, as the host's
}

// Queue inv[i] = RN(1 / m[i]) for n nodal masses already on the device.
cudaError_t device_inv_mass(const double *m, double *inv, long long n, cudaStream_t stream)
{
    if (n > 0) k_inv_mass<<<blocks_for(n), kSetupBlock, 0, stream>>>(m, inv, n);
    return cudaGetLastError();
}

// Queue the self-check of the energy field e of an nx^3 mesh: out[0..3] =
// origin energy, MaxAbsDiff, TotalAbsDiff, MaxRelDiff.  scratch holds at
// least nx * nx doubles.
cudaError_t device_verify(const double *e, int nx, double *scratch, double *out,
                          cudaStream_t stream)
{
    const long long pairs = (long long)nx * (nx - 1) / 2;
    double *absd = scratch, *reld = scratch + (pairs > 0 ? pairs : 1);
    k_verify_pairs<<<blocks_for((long long)nx * nx), kSetupBlock, 0, stream>>>(e, nx, absd, reld);
    k_verify_reduce<<<1, kSetupBlock, 0, stream>>>(e, nx, absd, reld, out);
    return cudaGetLastError();
}

// Queue the set-up on `stream`: the topology when `topology`, the initial
// element and node fields always.  s must hold a structured nx^3 mesh's
// arrays (E = nx^3, N = (nx+1)^3), or be an ensemble member's view of them:
// eoff / noff its first element / node, tstride the ensemble's element count
// (0: s.E), pid its member number.
cudaError_t device_setup(const DevState &s, int nx, double einit, bool topology,
                         cudaStream_t stream, int eoff, int noff, long long tstride, int pid)
{
    const long long items = s.E > s.N ? s.E : s.N;
    if (topology)
        k_setup_topology<<<blocks_for(items), kSetupBlock, 0, stream>>>(
            s, nx, eoff, noff, tstride > 0 ? tstride : s.E, pid);
    k_setup_elems<<<blocks_for(s.E), kSetupBlock, 0, stream>>>(s, nx, einit);
    k_setup_nodes<<<blocks_for(s.N), kSetupBlock, 0, stream>>>(s, nx);
    return cudaGetLastError();
}

}  // namespace lg
