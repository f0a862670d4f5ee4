// Instantiations of the dual sweep kernel (sweep_kern.cuh): double-float sweeps of relabelled plans with an
// unrelabelled twin, for runs with per-row op limits or starts and for derivative runs.
#define PQC_DUAL_SWEEP_INSTANTIATE
#include "sweep_kern.cuh"

namespace pqc {

PQC_DUAL_SWEEP_SHAPE(ArithDF, 512, 1)
PQC_DUAL_SWEEP_SHAPE(ArithDF, 256, 2)
PQC_DUAL_SWEEP_SHAPE(ArithDF, 256, 3)
PQC_DUAL_SWEEP_SHAPE(ArithDF, 128, 3)

}  // namespace pqc
