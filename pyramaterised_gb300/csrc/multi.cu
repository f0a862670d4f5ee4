// pqc_run_multi: forward evaluation of several programs -- circuits of different qubit counts, depths and
// gate lists -- in one sequence of launches.
//
// The reference evaluates every circuit on its own (`PQC.run`, pyramaterised/circuit.py:118-125), and so does
// pqc_run, one program per call: a call costs at least three launches (coefficients, their double-float
// split, one sweep per HBM pass) however small the circuit.  For many small circuits (a serving loop's mix of
// families) those launches, not the arithmetic, set the time.  Here the work of all items shares the launches:
// one coefficient launch and one conversion launch for every item, then one launch per sweep index s that
// runs sweep s of every item that has one (circuits of up to 13 qubits are a single sweep, so a mix of them
// is three launches in total).  Each CTA of a sweep launch finds its item from the running CTA totals, copies
// that item's sweep descriptor into shared memory and runs the same per-tile body as the single-program
// kernel (sweep_body.cuh), so every row's state is bit-identical to pqc_run's.
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "sweep_body.cuh"

namespace pqc {

struct MultiItem {
  const SweepDesc* sd;  // device copy of the item's sweep descriptor
  const DOp* ops;
  const int64_t* offs;
  const float2* rowcoef;
  int coef_stride;
  int n_qubits;
  const float2* consts;
  const double2* psi0;
  int64_t psi0_index;
  void* psi;
  int64_t tiles;
  RowCtl ctl;
  const uint16_t* lazy_cols;
  int* status;
};

struct MultiLaunch {
  int n;
  int64_t end[kMultiMax];  // running CTA totals: item j owns CTAs [end[j-1], end[j])
  MultiItem it[kMultiMax];
};

// (256 threads, 2 CTAs per SM): tiles of up to 2^12 amplitudes run two per SM, 2^13 one
template <class A>
__global__ void __launch_bounds__(256, 2) multi_sweep_kernel(const __grid_constant__ MultiLaunch L) {
  __shared__ SweepDesc s_sd;
  __shared__ int s_item;
  if (threadIdx.x == 0) {
    const int64_t b = blockIdx.x;
    int lo = 0, hi = L.n - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (b < L.end[mid]) hi = mid; else lo = mid + 1;
    }
    s_item = lo;
    s_sd = *L.it[lo].sd;
  }
  __syncthreads();
  const int j = s_item;
  const MultiItem& m = L.it[j];
  const int64_t blk = (int64_t)blockIdx.x - (j ? L.end[j - 1] : 0);
  sweep_body<A, 256, 2>(s_sd, op_list(s_sd), m.ops, m.offs, m.rowcoef, m.coef_stride, m.consts, m.psi0, m.psi0_index, m.psi,
                        m.n_qubits, m.tiles, 0, m.ctl, m.lazy_cols, m.status, blk);
}

// workspace of one item: [row coefficients f64 | row coefficients double-float | constants double-float]
static size_t item_ws(const pqc_run_item& it) {
  const size_t ns = it.prog->fwd_t.specs.size(), nc = it.prog->fwd_t.consts.size(), rows = (size_t)it.batch;
  if (ns != 0 && rows > ((size_t)1 << 40) / (ns * 64)) return SIZE_MAX;
  return align_up(rows * ns * 4 * sizeof(double), 256) + align_up(rows * ns * 4 * sizeof(float2), 256) +
         align_up(std::max<size_t>(nc, 4) * sizeof(float2), 256);
}

}  // namespace pqc

using namespace pqc;

extern "C" size_t pqc_run_multi_workspace_size(const pqc_run_item* items, int32_t n_items) {
  if (!items || n_items < 0) return 0;
  size_t ws = 0;
  for (int i = 0; i < n_items; ++i) {
    if (!items[i].prog || items[i].batch < 0) return 0;
    const size_t w = item_ws(items[i]);
    if (w == SIZE_MAX || ws > SIZE_MAX - w) return SIZE_MAX;
    ws += w;
  }
  return std::max<size_t>(ws, 256);
}

extern "C" int pqc_run_multi(const pqc_run_item* items, int32_t n_items, void* workspace, size_t workspace_bytes,
                             void* stream_v) {
  if (n_items < 0 || (n_items > 0 && !items)) return fail(PQC_ERR_INVALID, "bad item array");
  cudaStream_t stream = (cudaStream_t)stream_v;
  // validate, and give each item its workspace share
  std::vector<CoefJob> jobs;
  std::vector<int> live;  // items with rows
  char* w = (char*)workspace;
  size_t used = 0;
  int dev = -1;
  for (int i = 0; i < n_items; ++i) {
    const pqc_run_item& it = items[i];
    const std::string tag = "item " + std::to_string(i) + ": ";
    if (!it.prog) return fail(PQC_ERR_INVALID, tag + "program is NULL");
    if (it.batch < 0) return fail(PQC_ERR_INVALID, tag + "batch < 0");
    if (it.batch == 0) continue;
    if (!it.psi) return fail(PQC_ERR_INVALID, tag + "psi is NULL");
    const int64_t D = 1ll << it.prog->n_qubits;
    if (!it.psi0 && (it.psi0_index < 0 || it.psi0_index >= D))
      return fail(PQC_ERR_INVALID, tag + "psi0_index out of range");
    if (it.theta_stride < 0 || (it.theta_stride > 0 && it.theta_stride < it.prog->n_params))
      return fail(PQC_ERR_INVALID, tag + "bad theta_stride");
    if (dev < 0) dev = it.prog->device;
    if (it.prog->device != dev) return fail(PQC_ERR_INVALID, tag + "programs live on different devices");
    const size_t need = item_ws(it);
    if (need == SIZE_MAX || !workspace || used + need > workspace_bytes)
      return fail(PQC_ERR_WORKSPACE,
                  "workspace too small: need " + std::to_string(pqc_run_multi_workspace_size(items, n_items)));
    const size_t ns = it.prog->fwd_t.specs.size(), nc = it.prog->fwd_t.consts.size(), rows = (size_t)it.batch;
    CoefJob j;
    j.specs = it.prog->fwd_t.d_specs;
    j.n_slots = (int)ns;
    j.n_consts = (int)nc;
    j.theta = it.theta;
    j.theta_stride = it.theta_stride;
    j.rows = it.batch;
    j.coef = (double*)(w + used);
    j.coef_df = (float2*)(w + used + align_up(rows * ns * 4 * sizeof(double), 256));
    j.consts = it.prog->fwd_t.d_consts;
    j.consts_df = (float2*)((char*)j.coef_df + align_up(rows * ns * 4 * sizeof(float2), 256));
    jobs.push_back(j);
    live.push_back(i);
    used += need;
  }
  if (live.empty()) return PQC_OK;
  int rc = launch_coefs_multi(jobs.data(), (int)jobs.size(), stream);
  if (rc) return rc;
  static int attr_dev = -1;
  int cur = 0;
  PQC_CUDA(cudaGetDevice(&cur));
  if (attr_dev != cur) {
    int optin = 0;
    PQC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, cur));
    cudaFuncAttributes fa;
    PQC_CUDA(cudaFuncGetAttributes(&fa, multi_sweep_kernel<ArithDF>));
    PQC_CUDA(cudaFuncSetAttribute(multi_sweep_kernel<ArithDF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes));
    attr_dev = cur;
  }
  // sweep launches: launch s runs sweep s of every item that has one, kMultiMax items per launch
  size_t max_sweeps = 0;
  for (int i : live)
    max_sweeps = std::max(max_sweeps, run_plan_for(items[i].prog, items[i].row_limit != nullptr).sweeps.size());
  for (size_t s = 0; s < max_sweeps; ++s) {
    MultiLaunch L;
    L.n = 0;
    int64_t ctas = 0;
    size_t smem = 0;
    auto flush = [&]() -> int {
      if (L.n == 0) return PQC_OK;
      multi_sweep_kernel<ArithDF><<<(unsigned)ctas, 256, smem, stream>>>(L);
      count_launch();
      PQC_CUDA(cudaGetLastError());
      L.n = 0;
      ctas = 0;
      smem = 0;
      return PQC_OK;
    };
    for (size_t q = 0; q < live.size(); ++q) {
      const pqc_run_item& it = items[live[q]];
      const Plan& plan = run_plan_for(it.prog, it.row_limit != nullptr);
      if (s >= plan.sweeps.size()) continue;
      const SweepDesc& sd = plan.sweeps[s];
      const int64_t tiles = 1ll << (it.prog->n_qubits - sd.k);
      if (it.batch * tiles > (int64_t)0x7fffffff - ctas) {
        rc = flush();
        if (rc) return rc;
        if (it.batch * tiles > (int64_t)0x7fffffff) return fail(PQC_ERR_UNSUPPORTED, "item too large for one launch");
      }
      MultiItem& m = L.it[L.n];
      m.sd = plan.d_sweeps + s;
      m.ops = plan.d_ops;
      m.offs = plan.d_offs;
      m.rowcoef = jobs[q].coef_df;
      m.coef_stride = jobs[q].n_slots;
      m.n_qubits = it.prog->n_qubits;
      m.consts = jobs[q].consts_df;
      m.psi0 = (const double2*)it.psi0;
      m.psi0_index = it.psi0_index;
      m.psi = it.psi;
      m.tiles = tiles;
      m.ctl = RowCtl{};
      m.ctl.limit = it.row_limit;
      m.lazy_cols = plan.d_lazy_cols;
      m.status = it.prog->d_status;
      ctas += it.batch * tiles;
      L.end[L.n] = ctas;
      smem = std::max(smem, sweep_smem_bytes(sd, sizeof(cdf)));
      if (++L.n == kMultiMax) {
        rc = flush();
        if (rc) return rc;
      }
    }
    rc = flush();
    if (rc) return rc;
  }
  return PQC_OK;
}
