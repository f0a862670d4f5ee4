// The counts-only fidelity Gram on the tensor cores (tcgen05.mma, kind::tf32).
//
// Replaces the O(S^2) Qobj.overlap loop of _gen_f_samples (measure.py:123-137, 409-419) when only the
// histogram counts of the pair fidelities are wanted and S <= 256.  The states are split into planar
// real / imaginary parts rounded to TF32, G = <a|b> is formed as four real products per amplitude slice
//   Re G = Ar Br^T + Ai Bi^T,   Im G = Ar Bi^T - Ai Br^T
// with the accumulators in tensor memory, and every CTA writes the FP32 partial Gram of its amplitude slice.
// The partials are summed in FP64 (tc_reduce).  Each component of G is then within
//   delta = (2^-10 + Ks 2^-21) ||a|| ||b||
// of the exact value: 2^-10 from the TF32 rounding of both inputs (unit roundoff 2^-11 each), and Ks 2^-21
// for the FP32 accumulation of a slice of Ks amplitudes inside the tensor core (each of the 2 Ks / 8
// accumulation steps of a component, modelled as aligning its 8 exact products and the accumulator to the
// largest exponent and truncating, errs by at most 9 x 2^-23 of the running sum of magnitudes; the bound
// uses 4 x 2^-23 per amplitude, 1.8 times that).  measures.cu certifies each pair's bin with that delta and
// recomputes the undecided pairs exactly, so the counts are those of the exact path.
//
// One CTA: a 128-row block of G (rows 128 mt ..) against all 256 columns, over one amplitude slice.
// Warp 0 issues the TMA tile loads (cp.async.bulk.tensor, 128-byte swizzle, three stages), warp 1 the
// MMAs (one elected thread), and all four warps read the 128 x 512 accumulator columns back with
// tcgen05.ld.  Every wait is bounded; a CTA that times out raises the caller's fallback flag (the exact
// double-float recount then runs) and frees its tensor memory after its copies and MMAs are done.
#include <cuda.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>

#include "engine.cuh"
#include "sweep_ops.cuh"

namespace pqc {

namespace {
constexpr int kTcRows = 256;                       // columns of G (states); rows are two 128-row blocks
constexpr int kTcK = 32;                           // amplitudes per stage: 128-byte rows, the swizzle span
constexpr int kTcStages = 3;
constexpr unsigned kTcPart = kTcRows * kTcK * 4;   // one part (re or im) of a stage: 32 KiB
constexpr unsigned kTcStage = 2 * kTcPart;
constexpr size_t kTcSmem = 1024 + (size_t)kTcStages * kTcStage + 256;
constexpr uint64_t kTcWaitNs = 1000000000ull;      // 1 s
constexpr int kTcCols = 512;                       // tensor-memory columns: Re G (0..255), Im G (256..511)
}  // namespace

// ------------------------------------------------------------------ tcgen05 / TMA primitives
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_init1(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// 2-D tiled TMA load of box {32 amplitudes, 256 states} at (x, y) into 1024-byte aligned shared memory
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle (rows of 128 B, 8-row groups 1 KiB
// apart), descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc_sw128(unsigned saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3ffffu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                             // leading byte offset (unused by swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                   // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                             // version
  d |= (uint64_t)2 << 61;                             // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major, M = 128, N = 256 (neg: -A)
__host__ __device__ constexpr uint32_t umma_idesc_tf32(bool neg) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((neg ? 1u : 0u) << 13) | ((uint32_t)(256 >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(unsigned d_tmem, uint64_t a, uint64_t b, uint32_t idesc, unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

// arrives on the mbarrier once every MMA this thread issued before it has completed
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_addr(bar))
               : "memory");
}

// 32 consecutive accumulator columns of this warp's 32 lanes (one lane, i.e. one row, per thread)
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// ------------------------------------------------------------------ kernels
// complex128 states -> planar TF32 (round to nearest, ties away) real and imaginary parts
__global__ void split_tf32(const double2* __restrict__ X, float* __restrict__ yr, float* __restrict__ yi, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = X[i];
    uint32_t r, m;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(__double2float_rn(v.x)));
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(m) : "f"(__double2float_rn(v.y)));
    yr[i] = __uint_as_float(r);
    yi[i] = __uint_as_float(m);
  }
}

// partial[slice][row][col] = the slice's FP32 <row|col> (rows 128 blockIdx.x .., all 256 columns)
__global__ void __launch_bounds__(128, 1)
    gram_tc_kernel(const __grid_constant__ CUtensorMap map_re, const __grid_constant__ CUtensorMap map_im, int64_t D,
                   int64_t slice, float2* __restrict__ partial, int* __restrict__ fallback) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // stage buffers on 1024-byte boundaries of the shared window (the 128-byte swizzle repeats every 1 KiB)
  unsigned char* smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kTcStages * kTcStage);
  uint64_t* empty = full + kTcStages;
  uint64_t* done = empty + kTcStages;
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(done + 1);
  volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* issued = fail + 1;  // stages whose loads the producer issued
  volatile int* used = fail + 2;    // stages the MMA thread consumed
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x;
  const int64_t k0 = (int64_t)blockIdx.y * slice;
  const int64_t k1 = min(D, k0 + slice);
  const int nst = (int)((k1 - k0 + kTcK - 1) / kTcK);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      mbar_init1(&full[s]);
      mbar_init1(&empty[s]);
    }
    mbar_init1(done);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *fail = 0;
    *issued = 0;
    *used = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tmem_slot)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: stage it holds amplitudes [k0 + 32 it, +32) of all 256 states (rows >= S read as zeros)
    for (int it = 0; it < nst; ++it) {
      const int s = it % kTcStages;
      if (it >= kTcStages && !mbar_wait(&empty[s], (unsigned)((it / kTcStages - 1) & 1), kTcWaitNs)) {
        *fail = 1;
        break;
      }
      if (*fail) break;
      unsigned char* st = smem + (size_t)s * kTcStage;
      mbar_expect(&full[s], kTcStage);
      const int x = (int)(k0 + (int64_t)it * kTcK);
      tma_load_2d(st, &map_re, x, 0, &full[s]);
      tma_load_2d(st + kTcPart, &map_im, x, 0, &full[s]);
      *issued = it + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: per stage and 8-amplitude step, Re += Ar Br + Ai Bi, Im += Ar Bi - Ai Br
    constexpr uint32_t kPos = umma_idesc_tf32(false), kNeg = umma_idesc_tf32(true);
    for (int it = 0; it < nst; ++it) {
      const int s = it % kTcStages;
      if (*fail || !mbar_wait(&full[s], (unsigned)((it / kTcStages) & 1), kTcWaitNs)) {
        *fail = 1;
        break;
      }
      tc_fence_after();
      const unsigned re = smem_addr(smem + (size_t)s * kTcStage), im = re + kTcPart;
      const unsigned a_off = (unsigned)mt * 128u * 128u;  // rows 128 mt .. of the panel: 128 rows of 128 B
#pragma unroll
      for (int kk = 0; kk < kTcK / 8; ++kk) {
        const unsigned kb = (unsigned)kk * 32u;
        const uint64_t ar = umma_desc_sw128(re + a_off + kb), ai = umma_desc_sw128(im + a_off + kb);
        const uint64_t br = umma_desc_sw128(re + kb), bi = umma_desc_sw128(im + kb);
        const unsigned first = (it == 0 && kk == 0) ? 0u : 1u;
        umma_tf32(tmem, ar, br, kPos, first);
        umma_tf32(tmem, ai, bi, kPos, 1u);
        umma_tf32(tmem + 256, ar, bi, kPos, first);
        umma_tf32(tmem + 256, ai, br, kNeg, 1u);
      }
      umma_commit(&empty[s]);  // the stage's buffers are free once these MMAs have read them
      *used = it + 1;
    }
    umma_commit(done);
  }
  __syncwarp();

  // epilogue: warp w reads tensor-memory lanes 32 w .. 32 w + 31 (rows 128 mt + 32 w + lane)
  bool ok = mbar_wait(done, 0u, kTcWaitNs);
  tc_fence_after();
  // tcgen05.ld is warp-collective: the whole warp reads or none of it does
  if (__all_sync(0xffffffffu, ok && !*fail)) {
    const int row = mt * 128 + warp * 32 + lane;
    float2* out = partial + ((int64_t)blockIdx.y * kTcRows + row) * kTcRows;
    const unsigned lane_addr = tmem + ((unsigned)(warp * 32) << 16);
    for (int c = 0; c < 256; c += 32) {
      float vr[32], vi[32];
      tmem_ld32(lane_addr + (unsigned)c, vr);
      tmem_ld32(lane_addr + 256u + (unsigned)c, vi);
#pragma unroll
      for (int j = 0; j < 32; ++j) out[c + j] = make_float2(vr[j], vi[j]);
    }
  }
  if (!ok) *fail = 1;
  tc_fence_before();
  __syncthreads();
  if (*fail) {
    if (threadIdx.x == 0) {
      atomicExch(fallback, 1);
      // let the issued copies land and the committed MMAs finish before the buffers and columns go away
      for (int it = *used; it < *issued; ++it)
        mbar_wait(&full[it % kTcStages], (unsigned)((it / kTcStages) & 1), kTcWaitNs);
      mbar_wait(done, 0u, kTcWaitNs);
    }
    __syncthreads();
  }
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcCols) : "memory");
  }
}

// G[a][b] = sum over the slices of partial[slice][a][b], in FP64 and a fixed order
__global__ void tc_reduce(const float2* __restrict__ partial, int n_slices, double2* __restrict__ G) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kTcRows * kTcRows) return;
  double re = 0.0, im = 0.0;
  for (int s = 0; s < n_slices; ++s) {
    const float2 p = partial[(int64_t)s * kTcRows * kTcRows + i];
    re += (double)p.x;
    im += (double)p.y;
  }
  G[i] = make_double2(re, im);
}

// ------------------------------------------------------------------ host
namespace {
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static std::once_flag once;
  static EncodeTiled fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

void tc_geometry(int64_t S, int n_qubits, int& n_mt, int& n_slices, int64_t& slice) {
  const int64_t D = 1ll << n_qubits;
  n_mt = S > 128 ? 2 : 1;
  // about two waves of one CTA per SM; slices of whole stages
  const int64_t want = (2 * 152 + n_mt - 1) / n_mt;
  slice = (D + want - 1) / want;
  slice = (slice + kTcK - 1) / kTcK * kTcK;
  n_slices = (int)((D + slice - 1) / slice);
}
}  // namespace

bool gram_tc_usable(int64_t S, int n_qubits) {
  if (S < 2 || S > kTcRows || n_qubits < 13 || n_qubits > 30) return false;
  if (std::getenv("PQC_NO_TENSOR_GRAM")) return false;
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return major == 10 && minor == 3 && encode_fn() != nullptr;
}

size_t gram_tc_ws(int64_t S, int n_qubits) {
  int n_mt, n_slices;
  int64_t slice;
  tc_geometry(S, n_qubits, n_mt, n_slices, slice);
  return align_up((size_t)n_slices * kTcRows * kTcRows * sizeof(float2), 256) +
         align_up((size_t)kTcRows * kTcRows * sizeof(double2), 256);
}

int launch_gram_tc(const double2* psi, int64_t S, int n_qubits, float* planes, void* ws, double2** G_out,
                   double* delta_factor, int* fallback, cudaStream_t stream) {
  const int64_t D = 1ll << n_qubits;
  int n_mt, n_slices;
  int64_t slice;
  tc_geometry(S, n_qubits, n_mt, n_slices, slice);
  float2* partial = static_cast<float2*>(ws);
  double2* G = reinterpret_cast<double2*>(static_cast<char*>(ws) +
                                          align_up((size_t)n_slices * kTcRows * kTcRows * sizeof(float2), 256));
  float* yr = planes;
  float* yi = planes + S * D;
  const int64_t n = S * D;
  split_tf32<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, stream>>>(psi, yr, yi, n);
  count_launch();
  PQC_CUDA(cudaGetLastError());

  EncodeTiled enc = encode_fn();
  if (!enc) return fail(PQC_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  CUtensorMap maps[2];
  for (int part = 0; part < 2; ++part) {
    const cuuint64_t dims[2] = {(cuuint64_t)D, (cuuint64_t)S};
    const cuuint64_t strides[1] = {(cuuint64_t)D * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)kTcRows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(&maps[part], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, part ? (void*)yi : (void*)yr, dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(PQC_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  }
  static int attr_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    PQC_CUDA(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    attr_dev = dev;
  }
  gram_tc_kernel<<<dim3((unsigned)n_mt, (unsigned)n_slices), 128, kTcSmem, stream>>>(maps[0], maps[1], D, slice,
                                                                                      partial, fallback);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  tc_reduce<<<kTcRows * kTcRows / 256, 256, 0, stream>>>(partial, n_slices, G);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  *G_out = G;
  *delta_factor = 1.0 / 1024.0 + (double)slice / (double)(1 << 21);
  return PQC_OK;
}

// G[a][b] for a, b < S from the 256 x 256 reduction (NaN everywhere when a CTA timed out)
__global__ void tc_extract(const double2* __restrict__ G, int64_t S, const int* __restrict__ fallback,
                           double2* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= S * S) return;
  const int64_t a = i / S, b = i - a * S;
  out[i] = *fallback ? make_double2(__longlong_as_double(0x7ff8000000000000ll), __longlong_as_double(0x7ff8000000000000ll))
                     : G[a * kTcRows + b];
}

}  // namespace pqc

using namespace pqc;

extern "C" size_t pqc_gram_tf32_workspace_size(int64_t S, int32_t n_qubits) {
  if (S < 1 || n_qubits < 1 || n_qubits > 30) return 256;
  return gram_tc_ws(S, n_qubits) + align_up((size_t)S * ((size_t)1 << n_qubits) * 2 * sizeof(float), 256) + 256;
}

extern "C" int pqc_gram_tf32(const void* psi, int64_t S, int32_t n_qubits, void* G, double* delta_factor,
                             void* workspace, size_t workspace_bytes, void* stream_v) {
  if (!psi || !G || !delta_factor) return fail(PQC_ERR_INVALID, "psi, G and delta_factor must not be NULL");
  if (!gram_tc_usable(S, n_qubits))
    return fail(PQC_ERR_UNSUPPORTED, "the tensor-core Gram needs 2 <= S <= 256, 13 <= n_qubits <= 30 and sm_103");
  const size_t need = pqc_gram_tf32_workspace_size(S, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  cudaStream_t stream = (cudaStream_t)stream_v;
  char* w = static_cast<char*>(workspace);
  void* gws = w;
  w += gram_tc_ws(S, n_qubits);
  float* planes = reinterpret_cast<float*>(w);
  w += align_up((size_t)S * ((size_t)1 << n_qubits) * 2 * sizeof(float), 256);
  int* fb = reinterpret_cast<int*>(w);
  PQC_CUDA(cudaMemsetAsync(fb, 0, sizeof(int), stream));
  double2* Gt = nullptr;
  int rc = launch_gram_tc(static_cast<const double2*>(psi), S, n_qubits, planes, gws, &Gt, delta_factor, fb, stream);
  if (rc) return rc;
  tc_extract<<<(unsigned)((S * S + 255) / 256), 256, 0, stream>>>(Gt, S, fb, static_cast<double2*>(G));
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}
