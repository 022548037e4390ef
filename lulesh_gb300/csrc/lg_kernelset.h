// lg_kernelset.h -- launch entry points of one compiled copy of the kernels.
//
// The FP64 kernels are compiled twice from lg_kernels.cuh: once with
// --fmad=false (the parity build) and once with --fmad=true.  Each copy
// exports a KernelSet; the handle picks one at creation.
#pragma once

#include <cuda_runtime.h>

#include "lg_device.h"

namespace lg {

enum KernelId { K_FORCES = 0, K_NODES, K_KINEMATICS, K_MATERIAL, K_COUNT };

struct KernelSet {
    const char *name;
    void (*begin)(Ctl *ctl, cudaStream_t st);           // loop test + TimeIncrement
    void (*time_increment)(Ctl *ctl, cudaStream_t st);  // TimeIncrement alone
    void (*set_active)(Ctl *ctl, cudaStream_t st);
    // id < K_COUNT; mode selects the k_material variant (0, 1 or 2)
    void (*launch)(int id, const DevState &s, int mode, cudaStream_t st);
    // batched problems (DevState::nprob > 1)
    void (*launch_batched)(int id, const DevState &s, int bs, int grid, cudaStream_t st);
    void (*begin_all)(Ctl *ctl, int nprob, cudaStream_t st);
    int (*occupancy)(int id, int bs);
    const char *kernel_names[K_COUNT];
    int material_blocks(int E) const { return (E + 127) / 128; }
};

const KernelSet *kernels_fp64_strict();
const KernelSet *kernels_fp64_fma();
const KernelSet *kernels_mixed();

}  // namespace lg
