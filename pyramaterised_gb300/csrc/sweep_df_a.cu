// Instantiations of the fused sweep kernel (sweep_kern.cuh): double-float sweeps, 512 x 1 and 256 x 2.
#define PQC_SWEEP_INSTANTIATE
#include "sweep_kern.cuh"

namespace pqc {

PQC_SWEEP_SHAPE(ArithDF, 512, 1)
PQC_SWEEP_SHAPE(ArithDF, 256, 2)

}  // namespace pqc
