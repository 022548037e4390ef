// lg_kernels_fma.cu -- FP64 build of the cycle kernels with FMA contraction.
#define LG_NS fp64_fma
#define LG_NS_NAME "fp64_fma"
#define LG_REASSOC 1
#include "lg_kernels.cuh"
#include "lg_kernelset.inc"
namespace lg {
const KernelSet *kernels_fp64_fma() { return &fp64_fma::kKernelSet; }
}
