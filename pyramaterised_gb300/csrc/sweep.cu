// Fused shared-memory sweeps: the forward hot path.
//
// Replaces `PQC.run` (pyramaterised/circuit.py:118-125), which multiplies the
// state by one full 2^N x 2^N QuTiP operator per gate.  Here the planner
// (program.cu) groups the op list into sweeps; one sweep is one HBM pass in
// which every CTA gathers a tile of 2^k amplitudes (the k "active" bit
// positions, the lowest c of them contiguous so each gather row is a run of
// 2^c consecutive amplitudes), applies all of the sweep's ops to it in shared
// memory and writes it back.  Diagonal ops and controls on non-active
// positions use the tile's fixed bits; tile-constant phases are folded into
// one multiply at write-out.
//
// Arithmetic: ArithDF keeps every real as a double-float (hi + lo floats,
// ~48-bit significand) and runs on the FP32 pipes; between sweeps the state
// is stored in the output buffer in that format (16 B per amplitude, the
// same size as complex128) and converted to complex128 by the last sweep.
// ArithF32 is the complex64 sampling mode; ArithF64 runs the same plan in native FP64 (the comparison arm).
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "sweep_kern.cuh"

namespace pqc {

// The native FP64 arm is instantiated in two shapes only, (512, 1) at 2^13-amplitude tiles and (256, 2)
// below: it is bound by the FP64 pipe, not by latency, and its loops want the larger register budget.  The
// kernel instantiations live in sweep_df_a.cu, sweep_df_b.cu, sweep_f32.cu and sweep_f64.cu (compiled in
// parallel); sweep_kern.cuh declares them.
template <class A>
constexpr bool kFp64 = std::is_same<A, ArithF64>::value;

template <class A>
static int set_sweep_attrs() {
  int rc = allow_sweep_smem<A, 512, 1>();
  if (!rc) rc = allow_sweep_smem<A, 256, 2>();
  if constexpr (!kFp64<A>) {
    if (!rc) rc = allow_sweep_smem<A, 256, 3>();
    if (!rc) rc = allow_sweep_smem<A, 128, 3>();
  }
  return rc;
}

// launch shape of a sweep of 2^k-amplitude tiles over `ctas` tiles: (512, 1) at k = 13, else the program's
// setting.  Untuned programs take 3 CTAs per SM with 128 threads on grids of at least 2048 tiles (the N = 20,
// 256-row batches and the QFIM's derivative states ran fastest so) and 256 threads on smaller grids (the
// 64-row forward pass of the N = 16 gradient did).
static void sweep_shape(const pqc_program* prog, int k, int64_t ctas, int& threads, int& minb) {
  if (k >= 13) {
    threads = 512;
    minb = 1;
    return;
  }
  minb = prog->ctas_per_sm == 2 ? 2 : 3;
  if (minb == 2)
    threads = 256;
  else if (prog->sweep_threads != 0)
    threads = prog->sweep_threads;
  else
    threads = ctas >= 2048 ? 128 : 256;
}

// dynamic shared memory of a sweep launch (sweep_body's layout): the tile, the gather offsets, the phase and
// index tables, and one chunk of staged ops with their coefficients
size_t sweep_smem_bytes(const SweepDesc& sd, size_t amp_bytes) {
  return amp_bytes * ((size_t)1 << sd.k) + ((sizeof(int64_t) * ((size_t)1 << (sd.k - sd.c)) + 15) & ~(size_t)15) +
         amp_bytes * 256 + 512 + ((sizeof(DOp) * (size_t)std::min(sd.n_ops, kOpChunk) + 15) & ~(size_t)15) +
         sizeof(float2) * 4 * (size_t)std::min(sd.n_ops, kOpChunk);
}

// the forward plan a multi-program item takes: the relabelled plan, or its unrelabelled twin when rows have op
// limits or starts (the multi-program kernel has no dual form)
const Plan& run_plan_for(const pqc_program* prog, bool row_controls) {
  return (prog->fwd_lazy && row_controls) ? prog->fwd_lim : prog->fwd;
}

template <class A>
static int set_dual_sweep_attrs() {
  int rc = allow_dual_sweep_smem<A, 512, 1>();
  if (!rc) rc = allow_dual_sweep_smem<A, 256, 2>();
  if (!rc) rc = allow_dual_sweep_smem<A, 256, 3>();
  if (!rc) rc = allow_dual_sweep_smem<A, 128, 3>();
  return rc;
}

// twin: the unrelabelled twin of a relabelled plan (same sweeps).  With a twin, each sweep runs as the dual
// kernel: rows that apply every op of the sweep take the relabelled sweep, the others (a start or limit inside
// the sweep) the twin's.  Forward runs with row controls pair the relabelled plan with fwd_lim so; without the
// double-float dual kernels they take fwd_lim alone.
template <class A>
static int run_plan_impl(const pqc_program* prog, const Plan& plan_in, int coef_stride, const float2* rowcoef,
                         const float2* consts, int64_t rows, const void* psi0, int64_t psi0_index, void* psi,
                         cudaStream_t stream, const int32_t* row_limit, const RowCtl* ctl_in = nullptr,
                         const Plan* twin = nullptr) {
  RowCtl ctl = ctl_in ? *ctl_in : RowCtl{};
  if (row_limit) ctl.limit = row_limit;
  constexpr bool kDual = std::is_same<A, ArithDF>::value;
  const bool controls = ctl.limit || ctl.start || ctl.psi0_row;
  if (&plan_in == &prog->fwd && prog->fwd_lazy && controls && kDual) twin = &prog->fwd_lim;
  const Plan& plan =
      (&plan_in == &prog->fwd && prog->fwd_lazy && controls && !kDual) ? prog->fwd_lim : plan_in;
  if (twin && twin->sweeps.size() != plan.sweeps.size()) return fail(PQC_ERR_INVALID, "plan twins differ");
  using Amp = typename A::Amp;
  const int N = prog->n_qubits;
  static int attr_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    int rc = set_sweep_attrs<A>();
    if constexpr (kDual) {
      if (!rc) rc = set_dual_sweep_attrs<A>();
    }
    if (rc) return rc;
    attr_dev = dev;
  }
  for (size_t si = 0; si < plan.sweeps.size(); ++si) {
    const SweepDesc& sd = plan.sweeps[si];
    const int64_t tiles = 1ll << (N - sd.k);
    const size_t smem = twin ? std::max(sweep_smem_bytes(sd, sizeof(Amp)), sweep_smem_bytes(twin->sweeps[si],
                                                                                            sizeof(Amp)))
                             : sweep_smem_bytes(sd, sizeof(Amp));
    const int64_t max_rows = std::max<int64_t>(1, (int64_t)0x7fffffff / tiles);
    for (int64_t r0 = 0; r0 < rows; r0 += max_rows) {
      const int64_t nr = std::min(max_rows, rows - r0);
      const unsigned grid = (unsigned)(nr * tiles);
      int threads = 256, minb = 2;
      sweep_shape(prog, sd.k, (int64_t)grid, threads, minb);
      if constexpr (kFp64<A>) {
        if (threads != 512) {
          threads = 256;
          minb = 2;
        }
      }
      const SweepArgs args{plan.d_ops, plan.d_offs, rowcoef, coef_stride, consts, (const double2*)psi0, psi0_index,
                           psi, N, tiles, r0, ctl, plan.d_lazy_cols, prog->d_status};
      int lrc;
      if constexpr (kDual) {
        if (twin && sd.lazy) {  // an unrelabelled sweep holds the same ops as its twin: the plain kernel runs it
          const SweepDesc& psd = twin->sweeps[si];
          if (threads == 512)
            lrc = launch_dual_sweep<A, 512, 1>(sd, psd, twin->d_ops, args, grid, smem, stream);
          else if (threads == 256 && minb == 2)
            lrc = launch_dual_sweep<A, 256, 2>(sd, psd, twin->d_ops, args, grid, smem, stream);
          else if (threads == 128)
            lrc = launch_dual_sweep<A, 128, 3>(sd, psd, twin->d_ops, args, grid, smem, stream);
          else
            lrc = launch_dual_sweep<A, 256, 3>(sd, psd, twin->d_ops, args, grid, smem, stream);
          if (lrc) return lrc;
          continue;
        }
      }
      if (threads == 512) {
        lrc = launch_sweep<A, 512, 1>(sd, args, grid, smem, stream);
      } else if (threads == 256 && minb == 2) {
        lrc = launch_sweep<A, 256, 2>(sd, args, grid, smem, stream);
      } else {
        if constexpr (!kFp64<A>) {
          if (threads == 128)
            lrc = launch_sweep<A, 128, 3>(sd, args, grid, smem, stream);
          else
            lrc = launch_sweep<A, 256, 3>(sd, args, grid, smem, stream);
        } else {
          lrc = fail(PQC_ERR_INVALID, "no FP64 sweep shape");
        }
      }
      if (lrc) return lrc;
      count_launch();
      PQC_CUDA(cudaGetLastError());
    }
  }
  return PQC_OK;
}

int run_plan_df(const pqc_program* prog, const Plan& plan, int coef_stride, const float2* rowcoef,
                const float2* consts, int64_t rows, const void* psi0, int64_t psi0_index, void* psi,
                cudaStream_t stream, const int32_t* row_limit, const RowCtl* ctl, const Plan* twin) {
  return run_plan_impl<ArithDF>(prog, plan, coef_stride, rowcoef, consts, rows, psi0, psi0_index, psi, stream,
                                row_limit, ctl, twin);
}

// Workspace layout: [row coefs f64 | row coefs df | consts df]
// (SIZE_MAX when the sizes overflow: no workspace is then large enough)
static size_t coef_ws(size_t rows, size_t n_slots, size_t n_consts) {
  const size_t per_row = n_slots * 4 * (sizeof(double) + sizeof(float2));
  if ((n_slots != 0 && rows > (SIZE_MAX / 2) / per_row) || n_consts > (SIZE_MAX / 4) / sizeof(float2)) return SIZE_MAX;
  size_t a = align_up(rows * n_slots * 4 * sizeof(double), 256);
  size_t b = align_up(rows * n_slots * 4 * sizeof(float2), 256);
  size_t c = align_up(std::max<size_t>(n_consts, 4) * sizeof(float2), 256);
  return a + b + c;
}

struct CoefBufs {
  double* c64;
  float2* cdf;
  float2* kdf;
};

static CoefBufs carve_coefs(void* ws, size_t rows, size_t n_slots) {
  char* w = (char*)ws;
  CoefBufs b;
  b.c64 = (double*)w;
  b.cdf = (float2*)(w + align_up(rows * n_slots * 4 * sizeof(double), 256));
  b.kdf = (float2*)((char*)b.cdf + align_up(rows * n_slots * 4 * sizeof(float2), 256));
  return b;
}

// theta rows -> df coefficient tables for table t
static int prepare_coefs(const OpTable& t, const double* theta, int64_t theta_stride, int64_t rows, void* ws,
                         CoefBufs& b, cudaStream_t stream) {
  b = carve_coefs(ws, rows, t.specs.size());
  int rc = launch_row_coefs(t, theta, theta_stride, rows, b.c64, stream);
  if (rc) return rc;
  rc = launch_to_df(b.c64, b.cdf, rows * (int64_t)t.specs.size() * 4, stream);
  if (rc) return rc;
  return launch_to_df(t.d_consts, b.kdf, (int64_t)t.consts.size(), stream);
}

template <class A>
static int run_entry(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                     const void* psi0, int64_t psi0_index, void* psi, void* ws, size_t ws_bytes, void* stream_v,
                     const int32_t* row_limit = nullptr) {
  if (!prog) return fail(PQC_ERR_INVALID, "program is NULL");
  if (batch < 0) return fail(PQC_ERR_INVALID, "batch < 0");
  if (batch == 0) return PQC_OK;
  if (!psi) return fail(PQC_ERR_INVALID, "psi is NULL");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  if (theta_stride < 0) return fail(PQC_ERR_INVALID, "theta_stride < 0");
  if (theta_stride > 0 && theta_stride < prog->n_params) return fail(PQC_ERR_INVALID, "theta_stride < n_params");
  const size_t need = coef_ws(batch, prog->fwd_t.specs.size(), prog->fwd_t.consts.size());
  if (!ws || ws_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  cudaStream_t stream = (cudaStream_t)stream_v;
  CoefBufs b;
  int rc = prepare_coefs(prog->fwd_t, theta, theta_stride, batch, ws, b, stream);
  if (rc) return rc;
  if constexpr (kFp64<A>)  // the FP64 tables, one double per 8-byte element (ArithF64::ld)
    return run_plan_impl<A>(prog, prog->fwd, (int)prog->fwd_t.specs.size(), (const float2*)b.c64,
                            (const float2*)prog->fwd_t.d_consts, batch, psi0, psi0_index, psi, stream, row_limit);
  return run_plan_impl<A>(prog, prog->fwd, (int)prog->fwd_t.specs.size(), b.cdf, b.kdf, batch, psi0, psi0_index,
                          psi, stream, row_limit);
}

// sum derivative runs into their output rows: out[row_of[r]] += runs[r]
__global__ void scatter_add_rows(const double2* __restrict__ runs, const int32_t* __restrict__ row_of, int n_runs,
                                 double2* __restrict__ out, int n_qubits, int n_rows) {
  const int64_t D = 1ll << n_qubits;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= D) return;
  const int row = blockIdx.y;
  double2 acc = make_double2(0.0, 0.0);
  for (int r = 0; r < n_runs; ++r)
    if (row_of[r] == row) {
      double2 v = runs[(int64_t)r * D + i];
      acc.x += v.x;
      acc.y += v.y;
    }
  out[(int64_t)row * D + i] = acc;
}

}  // namespace pqc

using namespace pqc;

extern "C" size_t pqc_run_workspace_size(const pqc_program* prog, int64_t batch) {
  if (!prog || batch < 0) return 0;
  return coef_ws(batch, prog->fwd_t.specs.size(), prog->fwd_t.consts.size());
}

extern "C" int pqc_run(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                       const void* psi0, int64_t psi0_index, void* psi, void* workspace, size_t workspace_bytes,
                       void* stream) {
  return run_entry<ArithDF>(prog, theta, theta_stride, batch, psi0, psi0_index, psi, workspace, workspace_bytes,
                            stream);
}

extern "C" int pqc_run_limited(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                               const void* psi0, int64_t psi0_index, const int32_t* row_limit, void* psi,
                               void* workspace, size_t workspace_bytes, void* stream) {
  return run_entry<ArithDF>(prog, theta, theta_stride, batch, psi0, psi0_index, psi, workspace, workspace_bytes,
                            stream, row_limit);
}

extern "C" int pqc_run_fp64(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                            const void* psi0, int64_t psi0_index, void* psi, void* workspace, size_t workspace_bytes,
                            void* stream) {
  return run_entry<ArithF64>(prog, theta, theta_stride, batch, psi0, psi0_index, psi, workspace, workspace_bytes,
                             stream);
}

extern "C" int pqc_run_c64(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                           const void* psi0, int64_t psi0_index, void* psi_c64, void* workspace,
                           size_t workspace_bytes, void* stream) {
  return run_entry<ArithF32>(prog, theta, theta_stride, batch, psi0, psi0_index, psi_c64, workspace,
                             workspace_bytes, stream);
}

static bool identity_rows(const pqc_op* gens, int n_runs, int n_rows) {
  if (n_runs != n_rows) return false;
  for (int r = 0; r < n_runs; ++r)
    if (gens[r].sel != r) return false;
  return true;
}

extern "C" size_t pqc_derivative_states_workspace_size(const pqc_program* prog, int32_t n_runs, int32_t n_rows) {
  if (!prog || n_runs < 0) return 0;
  // coefficient tables for the generator-inserted program (one shared theta row)
  size_t n_slots = prog->fwd_t.specs.size() + (size_t)n_runs * 1;  // generators carry at most one slot each
  size_t n_consts = prog->fwd_t.consts.size() + (size_t)n_runs * 32;
  size_t ws = coef_ws(1, n_slots, n_consts);
  // run buffer + row map, used when runs do not map 1:1 onto output rows
  size_t D = (size_t)1 << prog->n_qubits;
  ws += align_up((size_t)n_runs * D * 16, 256);
  (void)n_rows;
  return ws;
}

static int derivative_runs(pqc_program* prog, const double* theta, const void* psi0, int64_t psi0_index,
                           const pqc_op* gens, const int32_t* gen_after, int32_t n_runs, int32_t n_rows,
                           const RowCtl& ctl, void* dpsi, void* workspace, size_t workspace_bytes,
                           cudaStream_t stream) {
  if (n_runs < 0 || n_rows < 0) return fail(PQC_ERR_INVALID, "negative count");
  if (n_runs == 0 || n_rows == 0) return PQC_OK;
  if (!gens || !gen_after || !dpsi) return fail(PQC_ERR_INVALID, "NULL argument");
  for (int r = 0; r < n_runs; ++r)
    if (gens[r].sel < 0 || gens[r].sel >= n_rows) return fail(PQC_ERR_INVALID, "gens[r].sel outside [0, n_rows)");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  const size_t need = pqc_derivative_states_workspace_size(prog, n_runs, n_rows);
  if (!workspace || workspace_bytes < need)
    return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  int rc = ensure_deriv(prog, gens, gen_after, n_runs);
  if (rc) return rc;
  CoefBufs b;
  rc = prepare_coefs(prog->deriv_t, theta, 0, 1, workspace, b, stream);
  if (rc) return rc;
  const size_t cw = coef_ws(1, prog->deriv_t.specs.size(), prog->deriv_t.consts.size());
  // relabelled derivative sweeps for the runs that apply every op of a sweep (PQC_NO_LAZY_DERIV=1: the
  // unrelabelled plan for every run)
  const bool no_lazy = std::getenv("PQC_NO_LAZY_DERIV") != nullptr;
  const bool lazy = prog->deriv_lazy_ok && !no_lazy;
  if (identity_rows(gens, n_runs, n_rows))
    return run_plan_df(prog, lazy ? prog->deriv_lazy : prog->deriv_plan, 0, b.cdf, b.kdf, n_runs, psi0, psi0_index,
                       dpsi, stream, nullptr, &ctl, lazy ? &prog->deriv_plan : nullptr);
  char* runs = (char*)workspace + cw;
  const int32_t* row_of = prog->d_run_row;  // uploaded with the cached plan
  rc = run_plan_df(prog, lazy ? prog->deriv_lazy : prog->deriv_plan, 0, b.cdf, b.kdf, n_runs, psi0, psi0_index, runs,
                   stream, nullptr, &ctl, lazy ? &prog->deriv_plan : nullptr);
  if (rc) return rc;
  dim3 grid((unsigned)((D + 255) / 256), (unsigned)n_rows);
  scatter_add_rows<<<grid, 256, 0, stream>>>((const double2*)runs, row_of, n_runs, (double2*)dpsi, prog->n_qubits,
                                             n_rows);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" int pqc_derivative_states(const pqc_program* prog_c, const double* theta, const void* psi0,
                                     int64_t psi0_index, const pqc_op* gens, const int32_t* gen_after, int32_t n_runs,
                                     int32_t n_rows, const int32_t* row_limit, void* dpsi, void* workspace,
                                     size_t workspace_bytes, void* stream_v) {
  if (!prog_c) return fail(PQC_ERR_INVALID, "program is NULL");
  RowCtl ctl;
  ctl.limit = row_limit;
  return derivative_runs(const_cast<pqc_program*>(prog_c), theta, psi0, psi0_index, gens, gen_after, n_runs, n_rows,
                         ctl, dpsi, workspace, workspace_bytes, (cudaStream_t)stream_v);
}

extern "C" int pqc_derivative_states_from(const pqc_program* prog_c, const double* theta, const void* psi0_rows,
                                          const int32_t* run_psi0, const int32_t* run_start, const pqc_op* gens,
                                          const int32_t* gen_after, int32_t n_runs, int32_t n_rows, void* dpsi,
                                          void* workspace, size_t workspace_bytes, void* stream_v) {
  if (!prog_c) return fail(PQC_ERR_INVALID, "program is NULL");
  if (!psi0_rows || !run_psi0 || !run_start) return fail(PQC_ERR_INVALID, "NULL checkpoint argument");
  RowCtl ctl;
  ctl.start = run_start;
  ctl.psi0_row = run_psi0;
  return derivative_runs(const_cast<pqc_program*>(prog_c), theta, psi0_rows, 0, gens, gen_after, n_runs, n_rows, ctl,
                         dpsi, workspace, workspace_bytes, (cudaStream_t)stream_v);
}
