// Instantiations of the fused sweep kernel (sweep_kern.cuh): native FP64 sweeps, 512 x 1 and 256 x 2.
#define PQC_SWEEP_INSTANTIATE
#include "sweep_kern.cuh"

namespace pqc {

PQC_SWEEP_SHAPE(ArithF64, 512, 1)
PQC_SWEEP_SHAPE(ArithF64, 256, 2)

}  // namespace pqc
