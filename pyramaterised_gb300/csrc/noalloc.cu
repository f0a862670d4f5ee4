// pqc_run_static: the forward evaluation without any device allocation.
//
// pqc_run asks its caller for a workspace (the per-row sine/cosine tables of
// the circuit's angles).  Some callers cannot provide one: a host application
// or plugin framework that owns every byte of device memory and forbids the
// libraries it loads from calling cudaMalloc, or a latency-critical loop that
// must never risk an allocation failing or stalling.  This entry point keeps
// that scratch in a fixed array compiled into the library instead.
//
// Contract (also in include/pyramaterised_gb300.h):
//   * Scratch is the file-scope array `g_static_scratch` below, kStaticScratchBytes
//     (16 MiB) large.  Every GPU that loads the library holds it until the process
//     exits.  A call whose tables do not fit returns PQC_ERR_UNSUPPORTED naming the
//     required and available sizes.
//   * The first call on each device looks up the array's device address with
//     cudaGetSymbolAddress, with that device current, once; make that first call
//     before any stream capture.  The address is kept per CUDA context (keyed by the
//     driver's context id): after cudaDeviceReset the next call on that device is a
//     first call again and looks the address up anew.
//   * All calls share the one array and it keeps the last call's contents.  The
//     tables are rewritten completely before they are read, so nothing has to start
//     at zero; but calls that overlap on the GPU (different streams, or different
//     host threads) race on the array and must be serialised by the caller.
//   * No cudaMalloc, cudaFree or allocating library routine is called.
#include <algorithm>
#include <mutex>
#include <string>

#include "engine.cuh"

namespace pqc {

constexpr size_t kStaticScratchBytes = (size_t)16 << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static std::mutex g_static_mu;
struct StaticSlot {
  unsigned long long ctx_id = 0;  // driver context id the address belongs to (0: unknown)
  void* ptr = nullptr;
};
static StaticSlot g_static_slot[64];

// The current context's unique id (cuCtxGetId through the runtime's driver entry points, so the library
// does not link the driver library itself); 0 when the driver does not provide it.
static unsigned long long current_context_id() {
  typedef int (*get_current_t)(void**);
  typedef int (*get_id_t)(void*, unsigned long long*);
  static get_current_t get_current = nullptr;
  static get_id_t get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_static_mu
    looked_up = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (get_current_t)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (get_id_t)f;
    cudaGetLastError();
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of g_static_scratch on the current device, looked up once per device (and context).
static int static_scratch(void** out) {
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(PQC_ERR_UNSUPPORTED, "device ordinal >= 64");
  std::lock_guard<std::mutex> lock(g_static_mu);
  const unsigned long long id = current_context_id();
  StaticSlot& s = g_static_slot[dev];
  if (!s.ptr || (id != 0 && id != s.ctx_id)) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
    s.ptr = p;
    s.ctx_id = id;
  }
  *out = s.ptr;
  return PQC_OK;
}

}  // namespace pqc

using namespace pqc;

extern "C" size_t pqc_run_static_capacity(void) { return kStaticScratchBytes; }

extern "C" int pqc_run_static(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                              const void* psi0, int64_t psi0_index, void* psi, void* stream_v) {
  if (!prog) return fail(PQC_ERR_INVALID, "program is NULL");
  if (batch < 0) return fail(PQC_ERR_INVALID, "batch < 0");
  if (batch == 0) return PQC_OK;
  if (!psi) return fail(PQC_ERR_INVALID, "psi is NULL");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  if (theta_stride < 0) return fail(PQC_ERR_INVALID, "theta_stride < 0");
  if (theta_stride > 0 && theta_stride < prog->n_params) return fail(PQC_ERR_INVALID, "theta_stride < n_params");
  const size_t n_slots = prog->fwd_t.specs.size();
  const size_t n_consts = prog->fwd_t.consts.size();
  // reject before the size arithmetic below can overflow: every row takes n_slots x 4 x (8 + 8) bytes
  if (n_slots > 0 && (uint64_t)batch > kStaticScratchBytes / (n_slots * 4 * (sizeof(double) + sizeof(float2))))
    return fail(PQC_ERR_UNSUPPORTED, "pqc_run_static: a batch of " + std::to_string(batch) +
                                         " rows needs more scratch than the static array holds (" +
                                         std::to_string(kStaticScratchBytes) + " bytes); use pqc_run or a smaller batch");
  // scratch layout: [row coefficients f64 | row coefficients double-float | constants double-float]
  const size_t a = align_up((size_t)batch * n_slots * 4 * sizeof(double), 256);
  const size_t b = align_up((size_t)batch * n_slots * 4 * sizeof(float2), 256);
  const size_t c = align_up(std::max<size_t>(n_consts, 4) * sizeof(float2), 256);
  if (a + b + c > kStaticScratchBytes)
    return fail(PQC_ERR_UNSUPPORTED, "pqc_run_static: this batch needs " + std::to_string(a + b + c) +
                                         " bytes of scratch but the static array holds " +
                                         std::to_string(kStaticScratchBytes) + "; use pqc_run or a smaller batch");
  void* base = nullptr;
  int rc = static_scratch(&base);
  if (rc) return rc;
  cudaStream_t stream = (cudaStream_t)stream_v;
  char* w = (char*)base;
  double* coef64 = (double*)w;
  float2* coefdf = (float2*)(w + a);
  float2* constdf = (float2*)(w + a + b);
  rc = launch_row_coefs(prog->fwd_t, theta, theta_stride, batch, coef64, stream);
  if (rc) return rc;
  rc = launch_to_df(coef64, coefdf, batch * (int64_t)n_slots * 4, stream);
  if (rc) return rc;
  rc = launch_to_df(prog->fwd_t.d_consts, constdf, (int64_t)n_consts, stream);
  if (rc) return rc;
  return run_plan_df(prog, prog->fwd, (int)n_slots, coefdf, constdf, batch, psi0, psi0_index, psi, stream);
}
