// lg_kernels_fp64.cu -- FP64 parity build of the cycle kernels (--fmad=false).
#define LG_NS fp64_strict
#define LG_NS_NAME "fp64"
#include "lg_kernels.cuh"
#include "lg_kernelset.inc"
namespace lg {
const KernelSet *kernels_fp64_strict() { return &fp64_strict::kKernelSet; }
}
