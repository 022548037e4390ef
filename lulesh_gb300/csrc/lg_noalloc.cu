// lg_noalloc.cu -- nodal forces into caller-owned device buffers, with no
// device allocation of any kind.
//
// Some callers cannot let a library allocate device memory behind their
// back: hydro codes that carve every device buffer out of one pool sized at
// start-up so their memory high-water mark is known, processes running under
// a hard per-GPU memory budget, and time-stepping loops that must not pay
// for cudaFree (which synchronises the whole device) or risk an allocation
// failing half-way through a run.  lg_calc_force_for_nodes_noalloc serves
// them: every input and output is a device pointer the caller already owns,
// and the only scratch it needs -- the per-corner forces that keep the node
// sums in the reference's order -- lives in the fixed file-scope array below.
//
// That array is a static device symbol: every GPU on which this code is
// loaded (at the latest on the first call made there) keeps it, about
// 12.6 MB, until the process exits.  Its size caps the
// mesh at kNoAllocMaxElem elements.  All calls share the one array, which
// keeps whatever the previous call left in it; calls whose kernels overlap on
// the same GPU (different streams or host threads) race on it and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#define LG_NS noalloc
#include "lg_kernels.cuh"
#include "lulesh_gb300.h"

namespace lg {
// lg_api.cu: records the text lg_last_error() returns on this thread.
int record_error(int code, const char *msg);
}  // namespace lg

constexpr int kNoAllocMaxElem = 32768;  // s <= 32 for the Sedov cube
constexpr int kMaxDevices = 64;

// Six per-corner force components (stress x/y/z, hourglass x/y/z), corner
// major: scratch[(c * 8 + j) * numElem + e], then one status word.
constexpr size_t kScratchDoubles = 48 * (size_t)kNoAllocMaxElem;
static __device__ __align__(256) double g_corner_scratch[kScratchDoubles + 32];

namespace {

struct DeviceSlot {
    std::once_flag once;
    cudaError_t err = cudaSuccess;
    double *scratch = nullptr;  // device address of g_corner_scratch
};
DeviceSlot g_slots[kMaxDevices];

int fail(int code, const char *msg) { return lg::record_error(code, msg); }

// Variant of k_forces (lg_kernels.cuh) that reads the element-major
// Domain::nodelist and writes the per-corner forces into the static scratch.
__global__ void __launch_bounds__(lg::noalloc::kBlock)
k_forces_static(int E, const int *__restrict__ nodelist, const double *__restrict__ xs,
                const double *__restrict__ ys, const double *__restrict__ zs,
                const double *__restrict__ xds, const double *__restrict__ yds,
                const double *__restrict__ zds, const double *__restrict__ ps,
                const double *__restrict__ qs, const double *__restrict__ vs,
                const double *__restrict__ volos, const double *__restrict__ sss,
                const double *__restrict__ masses, double hourg, double *cs, int *status)
{
    using namespace lg::noalloc;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= E) return;
    const size_t E8 = 8 * (size_t)E;
    int nd[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) nd[j] = nodelist[8 * (size_t)k + j];
    double x[8], y[8], z[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        x[j] = xs[nd[j]];
        y[j] = ys[nd[j]];
        z[j] = zs[nd[j]];
    }
    {
        // InitStressTermsForElems + IntegrateStressForElems (lulesh.cc:273-587)
        const double sig = -ps[k] - qs[k];
        const double determ = jacobian_det(x, y, z);
        double pfx[8], pfy[8], pfz[8];
        node_normals(pfx, pfy, pfz, x, y, z);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            cs[0 * E8 + (size_t)j * E + k] = -(sig * pfx[j]);
            cs[1 * E8 + (size_t)j * E + k] = -(sig * pfy[j]);
            cs[2 * E8 + (size_t)j * E + k] = -(sig * pfz[j]);
        }
        if (determ <= 0.0) atomicCAS(status, 0, -1);
    }
    // CalcHourglassControlForElems / CalcFBHourglassForceForElems
    // (lulesh.cc:710-1057)
    const double vk = vs[k];
    const double determ = volos[k] * vk;
    if (vk <= 0.0) atomicCAS(status, 0, -1);
    if (!(hourg > 0.)) return;
    double hourgam[8][4];
    {
        double dvdx[8], dvdy[8], dvdz[8];
        volume_derivative(x, y, z, dvdx, dvdy, dvdz);
        const double volinv = 1.0 / determ;
#pragma unroll
        for (int i1 = 0; i1 < 4; ++i1) {
            const double hourmodx = x[0] * gam(i1, 0) + x[1] * gam(i1, 1) + x[2] * gam(i1, 2) +
                                    x[3] * gam(i1, 3) + x[4] * gam(i1, 4) + x[5] * gam(i1, 5) +
                                    x[6] * gam(i1, 6) + x[7] * gam(i1, 7);
            const double hourmody = y[0] * gam(i1, 0) + y[1] * gam(i1, 1) + y[2] * gam(i1, 2) +
                                    y[3] * gam(i1, 3) + y[4] * gam(i1, 4) + y[5] * gam(i1, 5) +
                                    y[6] * gam(i1, 6) + y[7] * gam(i1, 7);
            const double hourmodz = z[0] * gam(i1, 0) + z[1] * gam(i1, 1) + z[2] * gam(i1, 2) +
                                    z[3] * gam(i1, 3) + z[4] * gam(i1, 4) + z[5] * gam(i1, 5) +
                                    z[6] * gam(i1, 6) + z[7] * gam(i1, 7);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                hourgam[kk][i1] = gam(i1, kk) - volinv * (dvdx[kk] * hourmodx +
                                                          dvdy[kk] * hourmody +
                                                          dvdz[kk] * hourmodz);
        }
    }
    const double coefficient = -hourg * 0.01 * sss[k] * masses[k] / cbrt(determ);
    const double *vel[3] = {xds, yds, zds};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double u[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) u[j] = vel[c][nd[j]];
        double hxx[4];
#pragma unroll
        for (int i = 0; i < 4; i++)
            hxx[i] = hourgam[0][i] * u[0] + hourgam[1][i] * u[1] + hourgam[2][i] * u[2] +
                     hourgam[3][i] * u[3] + hourgam[4][i] * u[4] + hourgam[5][i] * u[5] +
                     hourgam[6][i] * u[6] + hourgam[7][i] * u[7];
#pragma unroll
        for (int i = 0; i < 8; i++)
            cs[(3 + c) * E8 + (size_t)i * E + k] =
                coefficient * (hourgam[i][0] * hxx[0] + hourgam[i][1] * hxx[1] +
                               hourgam[i][2] * hxx[2] + hourgam[i][3] * hxx[3]);
    }
}

// Ordered corner gather of lulesh.cc:565-582 (stress, assigned) and 969-986
// (hourglass, added), into the caller's force arrays.
__global__ void __launch_bounds__(lg::noalloc::kBlock)
k_gather_static(int E, int N, const int *__restrict__ start, const int *__restrict__ corners,
                bool hg, const double *__restrict__ cs, double *fxo, double *fyo, double *fzo)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const size_t E8 = 8 * (size_t)E;
    double fx = 0.0, fy = 0.0, fz = 0.0, hx = 0.0, hy = 0.0, hz = 0.0;
    for (int i = start[n]; i < start[n + 1]; ++i) {
        const int c = corners[i];
        const size_t idx = (size_t)(c & 7) * E + (c >> 3);
        fx += cs[0 * E8 + idx];
        fy += cs[1 * E8 + idx];
        fz += cs[2 * E8 + idx];
        if (hg) {
            hx += cs[3 * E8 + idx];
            hy += cs[4 * E8 + idx];
            hz += cs[5 * E8 + idx];
        }
    }
    if (hg) {
        fx += hx;
        fy += hy;
        fz += hz;
    }
    fxo[n] = fx;
    fyo[n] = fy;
    fzo[n] = fz;
}

}  // namespace

extern "C" int lg_calc_force_for_nodes_noalloc(
    int numElem, int numNode, const int *nodelist, const int *nodeElemStart,
    const int *nodeElemCornerList, const double *x, const double *y, const double *z,
    const double *xd, const double *yd, const double *zd, const double *p, const double *q,
    const double *v, const double *volo, const double *ss, const double *elemMass,
    double hgcoef, double *fx, double *fy, double *fz, void *stream)
{
    if (numElem < 1 || numNode < 1)
        return fail(LG_ERR_INVALID, "lg_calc_force_for_nodes_noalloc: empty mesh");
    if (numElem > kNoAllocMaxElem)
        return fail(LG_ERR_INVALID,
                    "lg_calc_force_for_nodes_noalloc: numElem exceeds the fixed scratch "
                    "capacity of 32768 elements; use the lg_create/lg_step path");
    const void *ptrs[] = {nodelist, nodeElemStart, nodeElemCornerList, x, y, z, xd, yd, zd,
                          p, q, v, volo, ss, elemMass, fx, fy, fz};
    for (const void *ptr : ptrs)
        if (!ptr) return fail(LG_ERR_INVALID, "lg_calc_force_for_nodes_noalloc: null pointer");

    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(LG_ERR_CUDA, "lg_calc_force_for_nodes_noalloc: no usable current device");
    // One-time set-up per device, on the first call made with that device
    // current: the device address of the static scratch.
    DeviceSlot &slot = g_slots[dev];
    std::call_once(slot.once, [&]() {
        void *ptr = nullptr;
        slot.err = cudaGetSymbolAddress(&ptr, g_corner_scratch);
        slot.scratch = static_cast<double *>(ptr);
    });
    if (slot.err != cudaSuccess || !slot.scratch)
        return fail(LG_ERR_CUDA, "lg_calc_force_for_nodes_noalloc: cudaGetSymbolAddress failed");

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *cs = slot.scratch;
    int *status = reinterpret_cast<int *>(cs + kScratchDoubles);
    // A launch error left pending by unrelated earlier work of the caller is
    // not this call's failure: clear it so that the check after the launches
    // below sees only these kernels.  (A sticky error cannot be cleared; the
    // status reset then fails and is reported as such.)
    (void)cudaGetLastError();
    // the status word must start at zero; the corner values are all rewritten
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess)
        return fail(LG_ERR_CUDA, "lg_calc_force_for_nodes_noalloc: status reset failed");
    const int kb = lg::noalloc::kBlock;
    k_forces_static<<<(numElem + kb - 1) / kb, kb, 0, st>>>(
        numElem, nodelist, x, y, z, xd, yd, zd, p, q, v, volo, ss, elemMass, hgcoef, cs, status);
    k_gather_static<<<(numNode + kb - 1) / kb, kb, 0, st>>>(
        numElem, numNode, nodeElemStart, nodeElemCornerList, hgcoef > 0., cs, fx, fy, fz);
    if (cudaGetLastError() != cudaSuccess)
        return fail(LG_ERR_CUDA, "lg_calc_force_for_nodes_noalloc: kernel launch failed");
    int h_status = 0;
    if (cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return fail(LG_ERR_CUDA, "lg_calc_force_for_nodes_noalloc: status read-back failed");
    if (cudaStreamSynchronize(st) != cudaSuccess)
        return fail(LG_ERR_CUDA,
                    "lg_calc_force_for_nodes_noalloc: the kernels failed while running");
    return h_status;  // 0, or -1 (VolumeError) as the reference's exit code
}
