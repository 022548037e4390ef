// lg_adjoint.h -- the checkpointed adjoint's internal entry point (lg_adjoint.cu),
// called by the C ABI (lg_api.cu), which owns the handle.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "lg_device.h"
#include "lg_kernelset.h"

namespace lg {

// The state fields the adjoint carries, in the order of its seed and
// gradient arrays: node x y z xd yd zd, element e p q v ss.
constexpr int kAdjFields = 11;

struct AdjointIO {
    const DevState *ds;
    const KernelSet *ks;
    cudaStream_t stream;
    Ctl *h_ctl;                 // pinned host copy of the control block
    const double *dts;          // host: frozen time steps of the cycles run
    int ncycles, ckpt_k;
    // the objective: either the masked terminal energy (mask non-null; E
    // entries) or the adjoint of the final state given field by field
    // (seed[f], host, NULL for zero)
    const unsigned char *mask;
    const double *const *seed;
    // host outputs: dJ / d(initial field f), NULL when not wanted (with a
    // mask, grad[6] receives dJ/de)
    double *const *grad;
    double hgcoef;
    const std::vector<int> *lxim, *lxip, *letam, *letap, *lzetam, *lzetap, *elemBC;
};

// Runs the forward cycles with checkpoints, then the reverse sweep; *J (mask
// mode) receives the objective, *dJdhg dJ/dhgcoef; leaves the state at the
// final cycle.
int adjoint_run(const AdjointIO &io, double *J, double *dJdhg);

}  // namespace lg
