// Instantiations of the fused sweep kernel (sweep_kern.cuh): double-float sweeps, 256 x 3 and 128 x 3.
#define PQC_SWEEP_INSTANTIATE
#include "sweep_kern.cuh"

namespace pqc {

PQC_SWEEP_SHAPE(ArithDF, 256, 3)
PQC_SWEEP_SHAPE(ArithDF, 128, 3)

}  // namespace pqc
