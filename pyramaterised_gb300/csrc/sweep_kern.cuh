// The fused sweep kernel (one template over arithmetic and launch shape) and its launchers.  The
// instantiations are spread over sweep_df_a.cu, sweep_df_b.cu, sweep_f32.cu and sweep_f64.cu, which the
// build compiles in parallel; sweep.cu, which plans and issues the launches, only declares them.
#pragma once
#include "sweep_body.cuh"

namespace pqc {

// the per-launch arguments of a sweep launch besides its descriptor
struct SweepArgs {
  const DOp* ops;
  const int64_t* offs;
  const float2* rowcoef;
  int coef_stride;
  const float2* consts;
  const double2* psi0;
  int64_t psi0_index;
  void* psi;
  int n_qubits;
  int64_t tiles;
  int64_t row0;
  RowCtl ctl;
  const uint16_t* lazy_cols;
  int* status;
};

// launch sweep sd over `grid` CTAs (THREADS threads, MINB resident per SM) with `smem` bytes of dynamic
// shared memory; count_launch + error check included
template <class A, int THREADS, int MINB>
int launch_sweep(const SweepDesc& sd, const SweepArgs& a, unsigned grid, size_t smem, cudaStream_t stream);

// allow the kernel the device's opt-in dynamic shared memory (less its static use)
template <class A, int THREADS, int MINB>
int allow_sweep_smem();

// launch sweep `sd` of a relabelled plan whose unrelabelled twin holds the same sweep as plain_sd with ops
// plain_ops: each CTA takes the relabelled sweep when its row applies every op of it (start <= min_fwd and
// limit > max_fwd), the twin otherwise.  The relabelled sweeps may hold derivative generators.
template <class A, int THREADS, int MINB>
int launch_dual_sweep(const SweepDesc& sd, const SweepDesc& plain_sd, const DOp* plain_ops, const SweepArgs& a,
                      unsigned grid, size_t smem, cudaStream_t stream);

template <class A, int THREADS, int MINB>
int allow_dual_sweep_smem();

#ifdef PQC_SWEEP_INSTANTIATE
template <class A, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) sweep_kernel(const __grid_constant__ SweepDesc sd, const DOp* __restrict__ ops,
                                                    const int64_t* __restrict__ offs_g,
                                                    const float2* __restrict__ rowcoef, int coef_stride,
                                                    const float2* __restrict__ consts,
                                                    const double2* __restrict__ psi0, int64_t psi0_index, void* psi,
                                                    int n_qubits, int64_t tiles, int64_t row0, const RowCtl ctl,
                                                    const uint16_t* __restrict__ lazy_cols, int* __restrict__ status) {
  sweep_body<A, THREADS, MINB>(sd, op_list(sd), ops, offs_g, rowcoef, coef_stride, consts, psi0, psi0_index, psi, n_qubits, tiles,
                               row0, ctl, lazy_cols, status, (int64_t)blockIdx.x);
}

template <class A, int THREADS, int MINB>
int launch_sweep(const SweepDesc& sd, const SweepArgs& a, unsigned grid, size_t smem, cudaStream_t stream) {
  sweep_kernel<A, THREADS, MINB><<<grid, THREADS, smem, stream>>>(sd, a.ops, a.offs, a.rowcoef, a.coef_stride,
                                                                  a.consts, a.psi0, a.psi0_index, a.psi, a.n_qubits,
                                                                  a.tiles, a.row0, a.ctl, a.lazy_cols, a.status);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

template <class A, int THREADS, int MINB>
int allow_sweep_smem() {
  int dev = 0, optin = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  PQC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  PQC_CUDA(cudaFuncGetAttributes(&fa, sweep_kernel<A, THREADS, MINB>));
  PQC_CUDA(cudaFuncSetAttribute(sweep_kernel<A, THREADS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                optin - (int)fa.sharedSizeBytes));
  return PQC_OK;
}

#define PQC_SWEEP_SHAPE(A, T, MB)                                                                                 \
  template int launch_sweep<A, T, MB>(const SweepDesc&, const SweepArgs&, unsigned, size_t, cudaStream_t);       \
  template int allow_sweep_smem<A, T, MB>();
#endif

#ifdef PQC_DUAL_SWEEP_INSTANTIATE
// sd: the relabelled sweep; plain_begin / plain_n: the op list of its unrelabelled twin (same geometry) in
// plain_ops.  Each CTA picks one by its row's start and limit; the descriptor's geometry serves both.
template <class A, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) dual_sweep_kernel(const __grid_constant__ SweepDesc sd,
                                                         int plain_begin, int plain_n,
                                                         const DOp* __restrict__ ops,
                                                         const DOp* __restrict__ plain_ops,
                                                         const int64_t* __restrict__ offs_g,
                                                         const float2* __restrict__ rowcoef, int coef_stride,
                                                         const float2* __restrict__ consts,
                                                         const double2* __restrict__ psi0, int64_t psi0_index,
                                                         void* psi, int n_qubits, int64_t tiles, int64_t row0,
                                                         const RowCtl ctl, const uint16_t* __restrict__ lazy_cols,
                                                         int* __restrict__ status) {
  const int64_t row = row0 + (int64_t)blockIdx.x / tiles;
  const int st = ctl.start ? ctl.start[row] : 0;
  const int lim = ctl.limit ? ctl.limit[row] : 0x7fffffff;
  const bool full = st <= sd.min_fwd && lim > sd.max_fwd;
  const OpList ol = full ? op_list(sd) : OpList{plain_begin, plain_n, 0, 0};
  sweep_body<A, THREADS, MINB, true>(sd, ol, full ? ops : plain_ops, offs_g, rowcoef, coef_stride, consts, psi0,
                                     psi0_index, psi, n_qubits, tiles, row0, ctl, lazy_cols, status,
                                     (int64_t)blockIdx.x);
}

template <class A, int THREADS, int MINB>
int launch_dual_sweep(const SweepDesc& sd, const SweepDesc& plain_sd, const DOp* plain_ops, const SweepArgs& a,
                      unsigned grid, size_t smem, cudaStream_t stream) {
  dual_sweep_kernel<A, THREADS, MINB><<<grid, THREADS, smem, stream>>>(
      sd, plain_sd.op_begin, plain_sd.n_ops, a.ops, plain_ops, a.offs, a.rowcoef, a.coef_stride, a.consts, a.psi0,
      a.psi0_index, a.psi, a.n_qubits, a.tiles, a.row0, a.ctl, a.lazy_cols, a.status);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

template <class A, int THREADS, int MINB>
int allow_dual_sweep_smem() {
  int dev = 0, optin = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  PQC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  PQC_CUDA(cudaFuncGetAttributes(&fa, dual_sweep_kernel<A, THREADS, MINB>));
  PQC_CUDA(cudaFuncSetAttribute(dual_sweep_kernel<A, THREADS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                optin - (int)fa.sharedSizeBytes));
  return PQC_OK;
}

#define PQC_DUAL_SWEEP_SHAPE(A, T, MB)                                                                         \
  template int launch_dual_sweep<A, T, MB>(const SweepDesc&, const SweepDesc&, const DOp*, const SweepArgs&,   \
                                           unsigned, size_t, cudaStream_t);                                   \
  template int allow_dual_sweep_smem<A, T, MB>();
#endif

}  // namespace pqc
