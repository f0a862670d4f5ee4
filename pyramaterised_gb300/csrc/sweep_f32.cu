// Instantiations of the fused sweep kernel (sweep_kern.cuh): complex64 sampling-mode sweeps, every shape.
#define PQC_SWEEP_INSTANTIATE
#include "sweep_kern.cuh"

namespace pqc {

PQC_SWEEP_SHAPE(ArithF32, 512, 1)
PQC_SWEEP_SHAPE(ArithF32, 256, 2)
PQC_SWEEP_SHAPE(ArithF32, 256, 3)
PQC_SWEEP_SHAPE(ArithF32, 128, 3)

}  // namespace pqc
