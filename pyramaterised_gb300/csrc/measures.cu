// Capacity measures on device states (complex128 [rows, 2^n]).
//
//   pqc_overlaps       Qobj.overlap                    measure.py:52,58; circuit.py:141
//   pqc_fidelity_hist  _gen_f_samples + _gen_histo     measure.py:123-159, 409-419
//   pqc_expr_kl        expr (KL vs Haar)               measure.py:161-180
//   pqc_mw             single_Q                        measure.py:226-237
//   pqc_expect         qt.expect                       circuit.py:132-137
//   pqc_magic          renyi_entropy_fast / gkp_fast   measure.py:318-368
//   pqc_qfim           get_QFI                         measure.py:33-71
//
// Reductions are two-stage (per-block partials in the caller's workspace,
// then a fixed-order final pass), so every result is bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "df.cuh"
#include "dfacc.cuh"
#include "reduce.cuh"

namespace pqc {

// ------------------------------------------------------------------ overlaps
__global__ void overlap_partial(const double2* __restrict__ a, const double2* __restrict__ b,
                                const int64_t* __restrict__ ia, const int64_t* __restrict__ ib, int n_qubits,
                                int64_t chunk, int64_t k0, double2* __restrict__ partial) {
  __shared__ double scratch[32];
  const int64_t D = 1ll << n_qubits;
  const int64_t k = k0 + blockIdx.y;
  const double2* x = a + ia[k] * D;
  const double2* y = b + ib[k] * D;
  const int64_t s0 = blockIdx.x * chunk, s1 = min(D, s0 + chunk);
  double re = 0.0, im = 0.0;
  for (int64_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
    double2 u = x[i], v = y[i];
    re = fma(u.x, v.x, fma(u.y, v.y, re));
    im = fma(u.x, v.y, fma(-u.y, v.x, im));
  }
  re = block_sum(re, scratch);
  im = block_sum(im, scratch);
  if (threadIdx.x == 0) partial[k * gridDim.x + blockIdx.x] = make_double2(re, im);
}

__global__ void overlap_final(const double2* __restrict__ partial, int nblk, int64_t n, double2* __restrict__ out) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  double re = 0.0, im = 0.0;
  for (int j = 0; j < nblk; ++j) {
    double2 p = partial[k * nblk + j];
    re += p.x;
    im += p.y;
  }
  out[k] = make_double2(re, im);
}

static int overlap_blocks(int n_qubits, int64_t n) {
  const int64_t D = 1ll << n_qubits;
  int64_t want = std::max<int64_t>(1, 2048 / std::max<int64_t>(n, 1));
  int64_t cap = std::max<int64_t>(1, D / 2048);
  return (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(want, cap), 1024));
}

// ------------------------------------------------------------------ Gram tiles
// Overlaps <x_a|x_b> of many states in double-float arithmetic on the FP32
// pipes (GB300's FP64 rate is 1/72 of FP32).  A CTA owns a 32 x 32 tile of
// (a, b) pairs over one chunk of the amplitude axis; each thread accumulates
// 2 x 2 pairs.  Every product hi*hi is split exactly (FMA), its high part is
// summed with TwoSum and the low-order terms are gathered in a float, so the
// absolute error is a small multiple of 2^-48 * sum |a_i||b_i|.
constexpr int TS = 32;  // states per tile side
constexpr int KS = 16;  // amplitudes per smem slice

// partial[chunk][ta][tb][32][32] = sum over the chunk of conj(x_a) y_b (real part only when real_only); with
// sym (Y == X) only the tiles ta <= tb are computed
__global__ void __launch_bounds__(256) gram_partial(const double2* __restrict__ X, int64_t SA,
                                                    const double2* __restrict__ Y, int64_t SB, int n_qubits,
                                                    int64_t chunk, int real_only, int sym,
                                                    double2* __restrict__ partial,
                                                    const int* __restrict__ run_if = nullptr) {
  const int ta = blockIdx.x, tb = blockIdx.y;
  if (sym && ta > tb) return;
  if (run_if && *run_if == 0) return;
  __shared__ float4 As[TS][KS + 1];
  __shared__ float4 Bs[KS][TS];
  const int64_t D = 1ll << n_qubits;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t a0 = (int64_t)ta * TS, b0 = (int64_t)tb * TS;
  const int64_t s0 = blockIdx.z * chunk, s1 = min(D, s0 + chunk);
  Acc re[2][2], im[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) re[i][j] = im[i][j] = Acc{0.f, 0.f};
  for (int64_t base = s0; base < s1; base += KS) {
    for (int e = threadIdx.x; e < TS * KS; e += 256) {
      const int r = e / KS, kk = e % KS;
      const int64_t i = base + kk;
      const int64_t ra = a0 + r, rb = b0 + r;
      double2 u = (ra < SA && i < s1) ? X[ra * D + i] : make_double2(0.0, 0.0);
      double2 v = (rb < SB && i < s1) ? Y[rb * D + i] : make_double2(0.0, 0.0);
      const float2 ur = split_double(u.x), ui = split_double(u.y);
      const float2 vr = split_double(v.x), vi = split_double(v.y);
      As[r][kk] = make_float4(ur.x, ur.y, ui.x, ui.y);
      Bs[kk][r] = make_float4(vr.x, vr.y, vi.x, vi.y);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < KS; ++kk) {
      const float4 u[2] = {As[ty][kk], As[ty + 16][kk]};
      const float4 v[2] = {Bs[kk][tx], Bs[kk][tx + 16]};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          // conj(u) v = (ur vr + ui vi) + i (ur vi - ui vr)
          acc_mul(re[i][j], u[i].x, u[i].y, v[j].x, v[j].y);
          acc_mul(re[i][j], u[i].z, u[i].w, v[j].z, v[j].w);
          if (!real_only) {
            acc_mul(im[i][j], u[i].x, u[i].y, v[j].z, v[j].w);
            acc_mul(im[i][j], -u[i].z, -u[i].w, v[j].x, v[j].y);
          }
        }
    }
    __syncthreads();
  }
  double2* out = partial + (((int64_t)blockIdx.z * gridDim.x + ta) * gridDim.y + tb) * (TS * TS);
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
      out[(ty + 16 * i) * TS + tx + 16 * j] =
          make_double2((double)re[i][j].h + (double)re[i][j].l, (double)im[i][j].h + (double)im[i][j].l);
}

// The same tiles in native FP64 (complex128 products and sums on the FP64 pipe): the QFIM's Gram at the
// reference's precision (pqc_qfim_fp64).  Same layout of `partial` as gram_partial.
__global__ void __launch_bounds__(256) gram_partial_f64(const double2* __restrict__ X, int64_t SA, int n_qubits,
                                                        int64_t chunk, int real_only, double2* __restrict__ partial) {
  const int ta = blockIdx.x, tb = blockIdx.y;
  if (ta > tb) return;
  __shared__ double2 As[TS][KS + 1];
  __shared__ double2 Bs[KS][TS];
  const int64_t D = 1ll << n_qubits;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t a0 = (int64_t)ta * TS, b0 = (int64_t)tb * TS;
  const int64_t s0 = blockIdx.z * chunk, s1 = min(D, s0 + chunk);
  double re[2][2] = {{0.0, 0.0}, {0.0, 0.0}}, im[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int64_t base = s0; base < s1; base += KS) {
    for (int e = threadIdx.x; e < TS * KS; e += 256) {
      const int r = e / KS, kk = e % KS;
      const int64_t i = base + kk;
      const int64_t ra = a0 + r, rb = b0 + r;
      As[r][kk] = (ra < SA && i < s1) ? X[ra * D + i] : make_double2(0.0, 0.0);
      Bs[kk][r] = (rb < SA && i < s1) ? X[rb * D + i] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < KS; ++kk) {
      const double2 u[2] = {As[ty][kk], As[ty + 16][kk]};
      const double2 v[2] = {Bs[kk][tx], Bs[kk][tx + 16]};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          re[i][j] = fma(u[i].x, v[j].x, fma(u[i].y, v[j].y, re[i][j]));
          if (!real_only) im[i][j] = fma(u[i].x, v[j].y, fma(-u[i].y, v[j].x, im[i][j]));
        }
    }
    __syncthreads();
  }
  double2* out = partial + (((int64_t)blockIdx.z * gridDim.x + ta) * gridDim.y + tb) * (TS * TS);
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) out[(ty + 16 * i) * TS + tx + 16 * j] = make_double2(re[i][j], im[i][j]);
}

__device__ __forceinline__ double2 gram_entry(const double2* __restrict__ partial, int nchunk, int nt, int64_t a,
                                              int64_t b) {
  const int ta = (int)(a / TS), tb = (int)(b / TS);
  const int ty = (int)(a % TS), tx = (int)(b % TS);
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    double2 p = partial[(((int64_t)c * nt + ta) * nt + tb) * (TS * TS) + ty * TS + tx];
    re += p.x;
    im += p.y;
  }
  return make_double2(re, im);
}

// numpy's np.histogram(range=(first, last)) index rule for equal bins
__device__ __forceinline__ int np_bin(double f, const double* __restrict__ edges, int nbins) {
  const double first = edges[0], last = edges[nbins];
  if (!(f >= first) || !(f <= last)) return -1;
  double fi = ((f - first) / (last - first)) * (double)nbins;
  int64_t idx = (int64_t)fi;
  if (idx == nbins) idx -= 1;
  if (f < edges[idx])
    idx -= 1;
  else if (f >= edges[idx + 1] && idx != nbins - 1)
    idx += 1;
  return (int)idx;
}

// fidelities for a < b in itertools.combinations order + histogram
__device__ __forceinline__ void pair_of(int64_t k, int64_t S, int64_t& a, int64_t& b) {
  // invert k = a*(2S-a-1)/2 + (b-a-1)
  const double Sd = (double)S;
  a = (int64_t)floor(((2.0 * Sd - 1.0) - sqrt((2.0 * Sd - 1.0) * (2.0 * Sd - 1.0) - 8.0 * (double)k)) / 2.0);
  if (a < 0) a = 0;
  while (a > 0 && a * (2 * S - a - 1) / 2 > k) --a;
  while ((a + 1) * (2 * S - a - 2) / 2 <= k) ++a;
  b = k - a * (2 * S - a - 1) / 2 + a + 1;
}

__global__ void fid_final(const double2* __restrict__ partial, int nchunk, int nt, int64_t S,
                          const double* __restrict__ edges, int nbins, double* __restrict__ F,
                          unsigned long long* __restrict__ counts, const int* __restrict__ run_if = nullptr) {
  const int64_t M = S * (S - 1) / 2;
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= M) return;
  if (run_if && *run_if == 0) return;
  int64_t a, b;
  pair_of(k, S, a, b);
  double2 g = gram_entry(partial, nchunk, nt, a, b);
  double f = g.x * g.x + g.y * g.y;
  if (F) F[k] = f;
  if (counts) {
    int bin = np_bin(f, edges, nbins);
    if (bin >= 0) atomicAdd(&counts[bin], 1ull);
  }
}

// CTAs of gram_partial resident on the whole GPU at once (SMs x CTAs per SM; 152 x 4 without a device)
static int64_t gram_slots() {
  static int64_t slots = 0;
  if (slots == 0) {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms < 1)
      sms = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, gram_partial, 256, 0) != cudaSuccess || per < 1) per = 4;
    cudaGetLastError();
    slots = (int64_t)sms * per;
  }
  return slots;
}

// Tiles of TS x TS states (nt per side; with SB, nt x ntb tiles, else the nt (nt + 1) / 2 of the upper triangle)
// times nchunk chunks of the amplitude axis.  Every working CTA does the same work, so the GPU is busy for
// ceil(W / slots) waves of W = tiles x nchunk CTAs; nchunk is the smallest count whose waves are filled within
// 0.5 % of the best fill over the candidates (at P = 256: 36 tiles x 21 chunks = 756 CTAs for 760 slots, where
// the old choice of 17 chunks left a fifth wave of 4 CTAs on 4 SMs), with chunks of at least 4 KS amplitudes
// and the partial sums within 256 MiB.
static void gram_geometry(int64_t S, int n_qubits, int& nt, int& nchunk, int64_t& chunk, int64_t SB = -1) {
  const int64_t D = 1ll << n_qubits;
  nt = (int)((S + TS - 1) / TS);
  const int ntb = SB < 0 ? nt : (int)((SB + TS - 1) / TS);
  const int64_t pairs = SB < 0 ? (int64_t)nt * (nt + 1) / 2 : (int64_t)nt * ntb;
  const int64_t slots = gram_slots();
  const int64_t maxc = std::max<int64_t>(1, D / (4 * KS));
  const int64_t mem_cap = std::max<int64_t>(1, ((int64_t)256 << 20) / ((int64_t)nt * ntb * TS * TS * 16));
  const int64_t top = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(maxc, mem_cap), std::min<int64_t>(
                                               65535, 2 * ((slots + pairs - 1) / pairs) + 8)));
  auto realised = [&](int64_t n) {  // chunk count after rounding the chunk length up to KS
    int64_t c = (D + n - 1) / n;
    c = (c + KS - 1) / KS * KS;
    return (D + c - 1) / c;
  };
  auto fill = [&](int64_t n) {
    const int64_t w = pairs * realised(n);
    return (double)w / (double)(((w + slots - 1) / slots) * slots);
  };
  double best = 0.0;
  for (int64_t n = 1; n <= top; ++n) best = std::max(best, fill(n));
  int64_t pick = top;
  for (int64_t n = 1; n <= top; ++n)
    if (fill(n) >= best - 0.005) {
      pick = n;
      break;
    }
  chunk = (D + pick - 1) / pick;
  chunk = (chunk + KS - 1) / KS * KS;
  nchunk = (int)((D + chunk - 1) / chunk);
}

static size_t gram_ws(int64_t S, int n_qubits) {
  int nt, nchunk;
  int64_t chunk;
  gram_geometry(S, n_qubits, nt, nchunk, chunk);
  return align_up((size_t)nchunk * nt * nt * TS * TS * sizeof(double2), 256);
}

static int launch_gram(const double2* X, int64_t S, int n_qubits, double2* partial, int& nt, int& nchunk,
                       cudaStream_t stream, int real_only = 0, bool fp64 = false) {
  int64_t chunk;
  gram_geometry(S, n_qubits, nt, nchunk, chunk);
  dim3 grid(nt, nt, nchunk);
  if (fp64)
    gram_partial_f64<<<grid, 256, 0, stream>>>(X, S, n_qubits, chunk, real_only, partial);
  else
    gram_partial<<<grid, 256, 0, stream>>>(X, S, X, S, n_qubits, chunk, real_only, 1, partial);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

// ------------------------------------------------------------------ certified histogram counts
// When only the bin counts of the pair fidelities are wanted, the Gram is first formed with FP32
// products: amplitudes truncated to 24 significand bits, 64-term FP32 FMA sums per slice (32 amplitudes,
// two products each), slices accumulated in double-float.  Each component of <a|b> is then within
//   delta = 5e-6 ||a|| ||b||
// of the exact value (2 x 2^-23 from the truncated inputs plus gamma_64 = 64 x 2^-24 of the slice sums
// = 4.05e-6, with margin), so F = |<a|b>|^2 is within e = 2.83 |G| delta + 2 delta^2.  A pair whose interval
// [F - e, F + e] lies inside one bin is counted directly; the others are listed and recomputed exactly in
// double-float, and if more than the list holds, every pair is recomputed by the double-float Gram.
// The counts equal those of the exact path.
constexpr int kRefineCap = 4096;

// 64 x 64 pair tiles (4 x 4 per thread) and 32-amplitude slices: 64-term FP32 sums, within the same delta
// (2 x 2^-23 + 64 x 2^-24 = 4.05e-6 < 5e-6).
constexpr int TSF = 64, KSF = 32;

static void gram_fast_geometry(int64_t S, int n_qubits, int& nt, int& nchunk, int64_t& chunk) {
  const int64_t D = 1ll << n_qubits;
  nt = (int)((S + TSF - 1) / TSF);
  const int64_t pairs = (int64_t)nt * (nt + 1) / 2;
  const int64_t want = std::max<int64_t>(1, (152 * 4 + pairs - 1) / pairs);
  const int64_t maxc = std::max<int64_t>(1, D / (4 * KSF));
  nchunk = (int)std::min<int64_t>(std::min<int64_t>(want, maxc), 65535);
  chunk = (D + nchunk - 1) / nchunk;
  chunk = (chunk + KSF - 1) / KSF * KSF;
  nchunk = (int)((D + chunk - 1) / chunk);
}

static size_t gram_fast_ws(int64_t S, int n_qubits) {
  int nt, nchunk;
  int64_t chunk;
  gram_fast_geometry(S, n_qubits, nt, nchunk, chunk);
  return align_up((size_t)nchunk * nt * nt * TSF * TSF * sizeof(double2), 256);
}

__device__ __forceinline__ double2 gram_fast_entry(const double2* __restrict__ partial, int nchunk, int nt, int64_t a,
                                                   int64_t b) {
  const int ta = (int)(a / TSF), tb = (int)(b / TSF);
  const int ty = (int)(a % TSF), tx = (int)(b % TSF);
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    const double2 p = partial[(((int64_t)c * nt + ta) * nt + tb) * (TSF * TSF) + ty * TSF + tx];
    re += p.x;
    im += p.y;
  }
  return make_double2(re, im);
}

// The states as truncated FP32 (the top 24 significand bits of each component), the fast Gram's input.
__global__ void trunc_to_f32(const double2* __restrict__ X, float2* __restrict__ Y, int64_t n,
                             const int* __restrict__ gate = nullptr) {
  if (gate && !*gate) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = X[i];
    Y[i] = make_float2(split_double(v.x).x, split_double(v.y).x);
  }
}

// 16-byte asynchronous copy; src_bytes 0 zero-fills the destination without reading
__device__ __forceinline__ void cp_async16(void* s, const void* g, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(g), "r"(src_bytes) : "memory");
}

// Panels of 64 states x 32 amplitudes, double-buffered with cp.async (the next slice loads while the current
// one is multiplied).  Rows of 34 float2 keep every copy 16-byte aligned.
constexpr int KSP = KSF + 2;
constexpr size_t kGramFastSmem = 2 * 2 * TSF * KSP * sizeof(float2);

// One CTA's 64 x 64 pair tile over its amplitude chunk.  NJ: 16-state column blocks that hold states (< S);
// DIAG: a diagonal tile (rows = columns), of which only the blocks i <= j are needed (a pair a < b of the
// tile never has its row block above its column block).  Blocks that are not needed are neither computed
// nor written; fid_certify reads only pairs a < b and the diagonal of states < S.
template <int NJ, bool DIAG>
__device__ __forceinline__ void gram_fast_tile(const float2* __restrict__ Y, int64_t S, int64_t D, int64_t a0,
                                               int64_t b0, int64_t s0, int64_t s1, unsigned char* smem,
                                               double2* __restrict__ out) {
  constexpr int NI = DIAG ? NJ : 4;
  float2(*As)[TSF][KSP] = reinterpret_cast<float2(*)[TSF][KSP]>(smem);
  float2(*Bs)[TSF][KSP] = reinterpret_cast<float2(*)[TSF][KSP]>(smem + 2 * TSF * KSP * sizeof(float2));
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int nsl = (int)((s1 - s0 + KSF - 1) / KSF);
  auto issue = [&](int sl, int st) {
    const int64_t base = s0 + (int64_t)sl * KSF;
    for (int e = threadIdx.x; e < TSF * KSF / 2; e += 256) {
      const int r = e / (KSF / 2), q = e % (KSF / 2);
      const int64_t i = base + 2 * q;  // s1 is even: a 2-amplitude copy never straddles it
      const int64_t ra = a0 + r, rb = b0 + r;
      const bool oa = ra < S && i < s1, ob = rb < S && i < s1;
      cp_async16(&As[st][r][2 * q], Y + (oa ? ra * D + i : 0), oa ? 16 : 0);
      cp_async16(&Bs[st][r][2 * q], Y + (ob ? rb * D + i : 0), ob ? 16 : 0);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  Acc re[NI][NJ], im[NI][NJ];
#pragma unroll
  for (int i = 0; i < NI; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j) re[i][j] = im[i][j] = Acc{0.f, 0.f};
  issue(0, 0);
  for (int sl = 0; sl < nsl; ++sl) {
    const int st = sl & 1;
    if (sl + 1 < nsl) {
      issue(sl + 1, st ^ 1);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();
    float sr[NI][NJ], si[NI][NJ];
#pragma unroll
    for (int i = 0; i < NI; ++i)
#pragma unroll
      for (int j = 0; j < NJ; ++j) sr[i][j] = si[i][j] = 0.f;
#pragma unroll 4
    for (int kk = 0; kk < KSF; ++kk) {
      float2 u[NI], v[NJ];
#pragma unroll
      for (int i = 0; i < NI; ++i) u[i] = As[st][ty + 16 * i][kk];
#pragma unroll
      for (int j = 0; j < NJ; ++j) v[j] = Bs[st][tx + 16 * j][kk];
#pragma unroll
      for (int i = 0; i < NI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
          if (DIAG && i > j) continue;
          sr[i][j] = __fmaf_rn(u[i].x, v[j].x, sr[i][j]);
          sr[i][j] = __fmaf_rn(u[i].y, v[j].y, sr[i][j]);
          si[i][j] = __fmaf_rn(u[i].x, v[j].y, si[i][j]);
          si[i][j] = __fmaf_rn(-u[i].y, v[j].x, si[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < NI; ++i)
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        if (DIAG && i > j) continue;
        acc_add(re[i][j], sr[i][j], 0.f);
        acc_add(im[i][j], si[i][j], 0.f);
      }
    __syncthreads();  // the stage is refilled by the next iteration's issue
  }
#pragma unroll
  for (int i = 0; i < NI; ++i)
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      if (DIAG && i > j) continue;
      out[(ty + 16 * i) * TSF + tx + 16 * j] =
          make_double2((double)re[i][j].h + (double)re[i][j].l, (double)im[i][j].h + (double)im[i][j].l);
    }
}

__global__ void __launch_bounds__(256, 2) gram_fast_partial(const float2* __restrict__ Y, int64_t S, int n_qubits,
                                                            int64_t chunk, double2* __restrict__ partial,
                                                            const int* __restrict__ gate = nullptr) {
  const int ta = blockIdx.x, tb = blockIdx.y;
  if (ta > tb || (gate && !*gate)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t D = 1ll << n_qubits;
  const int64_t a0 = (int64_t)ta * TSF, b0 = (int64_t)tb * TSF;
  const int64_t s0 = blockIdx.z * chunk, s1 = min(D, s0 + chunk);
  double2* out = partial + (((int64_t)blockIdx.z * gridDim.x + ta) * gridDim.y + tb) * (TSF * TSF);
  const int64_t left = S - b0;  // states in the column tile (>= 1)
  const int nj = left >= 64 ? 4 : (int)((left + 15) / 16);
  if (ta == tb) {
    switch (nj) {
      case 1: gram_fast_tile<1, true>(Y, S, D, a0, b0, s0, s1, smem, out); break;
      case 2: gram_fast_tile<2, true>(Y, S, D, a0, b0, s0, s1, smem, out); break;
      case 3: gram_fast_tile<3, true>(Y, S, D, a0, b0, s0, s1, smem, out); break;
      default: gram_fast_tile<4, true>(Y, S, D, a0, b0, s0, s1, smem, out); break;
    }
  } else {
    switch (nj) {
      case 1: gram_fast_tile<1, false>(Y, S, D, a0, b0, s0, s1, smem, out); break;
      case 2: gram_fast_tile<2, false>(Y, S, D, a0, b0, s0, s1, smem, out); break;
      case 3: gram_fast_tile<3, false>(Y, S, D, a0, b0, s0, s1, smem, out); break;
      default: gram_fast_tile<4, false>(Y, S, D, a0, b0, s0, s1, smem, out); break;
    }
  }
}

// ctl[0]: number of listed pairs, ctl[1]: 1 when the list overflowed
__global__ void fid_certify(const double2* __restrict__ partial, int nchunk, int nt, int64_t S,
                            const double* __restrict__ edges, int nbins, unsigned long long* __restrict__ counts,
                            int64_t* __restrict__ list, int* __restrict__ ctl, const int* __restrict__ gate = nullptr) {
  const int64_t M = S * (S - 1) / 2;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= M || (gate && !*gate)) return;
  int64_t a, b;
  pair_of(k, S, a, b);
  const double2 g = gram_fast_entry(partial, nchunk, nt, a, b);
  const double na = sqrt(fmax(gram_fast_entry(partial, nchunk, nt, a, a).x, 0.0) * 1.00001);
  const double nb = sqrt(fmax(gram_fast_entry(partial, nchunk, nt, b, b).x, 0.0) * 1.00001);
  const double delta = 5e-6 * na * nb + 1e-300;
  const double f = g.x * g.x + g.y * g.y;
  const double e = 2.83 * sqrt(f) * delta + 2.0 * delta * delta;
  const int lo = np_bin(fmax(f - e, 0.0), edges, nbins), hi = np_bin(f + e, edges, nbins);
  if (lo == hi) {
    if (lo >= 0) atomicAdd(&counts[lo], 1ull);
    return;
  }
  const int slot = atomicAdd(&ctl[0], 1);
  if (slot < kRefineCap)
    list[slot] = k;
  else
    atomicExch(&ctl[1], 1);
}

// The same certification from the tensor-core Gram G (double2 [256][256], gram_tc.cu), each component
// within dfac ||a|| ||b||.  More undecided pairs than the list holds raise ctl[2]: the FP32 tier then runs.
__global__ void fid_certify_tc(const double2* __restrict__ G, int64_t S, double dfac, const double* __restrict__ edges,
                               int nbins, unsigned long long* __restrict__ counts, int64_t* __restrict__ list,
                               int* __restrict__ ctl) {
  const int64_t M = S * (S - 1) / 2;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= M) return;
  int64_t a, b;
  pair_of(k, S, a, b);
  const double2 g = G[a * 256 + b];
  // G_aa >= ||a||^2 (1 - dfac): an upper bound of the norms
  const double na = sqrt(fmax(G[a * 257].x, 0.0) / (1.0 - dfac));
  const double nb = sqrt(fmax(G[b * 257].x, 0.0) / (1.0 - dfac));
  const double delta = dfac * na * nb + 1e-300;
  const double f = g.x * g.x + g.y * g.y;
  const double e = 2.83 * sqrt(f) * delta + 2.0 * delta * delta;
  const int lo = np_bin(fmax(f - e, 0.0), edges, nbins), hi = np_bin(f + e, edges, nbins);
  if (lo == hi) {
    if (lo >= 0) atomicAdd(&counts[lo], 1ull);
    return;
  }
  const int slot = atomicAdd(&ctl[0], 1);
  if (slot < kRefineCap)
    list[slot] = k;
  else
    atomicExch(&ctl[2], 1);
}

// after a tensor-core tier that left too many pairs undecided: clear its counts and list for the FP32 tier
__global__ void tc_tier_reset(int* __restrict__ ctl, unsigned long long* __restrict__ counts, int nbins) {
  if (!ctl[2]) return;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) counts[i] = 0;
  if (threadIdx.x == 0) ctl[0] = 0;
}

// exact double-float |<a|b>|^2 of each listed pair (one CTA per pair) into the counts
__global__ void __launch_bounds__(256) fid_refine(const double2* __restrict__ X, int64_t S, int n_qubits,
                                                  const double* __restrict__ edges, int nbins,
                                                  unsigned long long* __restrict__ counts,
                                                  const int64_t* __restrict__ list, const int* __restrict__ ctl) {
  if (ctl[1] || (int)blockIdx.x >= ctl[0]) return;
  __shared__ float2 ws[8][2];
  int64_t a, b;
  pair_of(list[blockIdx.x], S, a, b);
  const int64_t D = 1ll << n_qubits;
  const double2* u = X + a * D;
  const double2* v = X + b * D;
  Acc sr{0.f, 0.f}, si{0.f, 0.f};
  for (int64_t i = threadIdx.x; i < D; i += blockDim.x) {
    const double2 p = u[i], q = v[i];
    const float2 ur = split_double(p.x), ui = split_double(p.y), vr = split_double(q.x), vi = split_double(q.y);
    acc_mul(sr, ur.x, ur.y, vr.x, vr.y);
    acc_mul(sr, ui.x, ui.y, vi.x, vi.y);
    acc_mul(si, ur.x, ur.y, vi.x, vi.y);
    acc_mul(si, -ui.x, -ui.y, vr.x, vr.y);
  }
  sr = warp_sum_df(sr);
  si = warp_sum_df(si);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    ws[wid][0] = make_float2(sr.h, sr.l);
    ws[wid][1] = make_float2(si.h, si.l);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Acc x{0.f, 0.f}, y{0.f, 0.f};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      acc_add(x, ws[w][0].x, ws[w][0].y);
      acc_add(y, ws[w][1].x, ws[w][1].y);
    }
    const double gr = (double)x.h + (double)x.l, gi = (double)y.h + (double)y.l;
    const int bin = np_bin(gr * gr + gi * gi, edges, nbins);
    if (bin >= 0) atomicAdd(&counts[bin], 1ull);
  }
}

__global__ void clear_counts_if(const int* __restrict__ ctl, unsigned long long* __restrict__ counts, int nbins) {
  if (!ctl[1]) return;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) counts[i] = 0;
}

// histogram of arbitrary samples with the same numpy index rule
__global__ void hist_kernel(const double* __restrict__ F, int64_t M, const double* __restrict__ edges, int nbins,
                            unsigned long long* __restrict__ counts) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= M) return;
  int bin = np_bin(F[k], edges, nbins);
  if (bin >= 0) atomicAdd(&counts[bin], 1ull);
}

// ------------------------------------------------------------------ KL (expr)
__device__ double kl_div_dev(double x, double y) {
  if (isnan(x) || isnan(y)) return nan("");
  if (x > 0 && y > 0) return x * log(x / y) - x + y;
  if (x == 0 && y >= 0) return y;
  return INFINITY;
}

__global__ void expr_kl_kernel(const unsigned long long* __restrict__ counts, int nbins,
                               const double* __restrict__ edges, double d, double* out) {
  __shared__ double haar[1024];
  __shared__ double hsum;
  __shared__ unsigned long long tot;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
    const double F = (edges[i] + edges[i + 1]) / 2;
    haar[i] = (d - 1) * pow(1 - F, d - 2);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double h = 0.0;
    unsigned long long t = 0;
    for (int i = 0; i < nbins; ++i) {
      h += haar[i];
      t += counts[i];
    }
    hsum = h;
    tot = t;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
    const double p = (double)counts[i] / (double)tot;
    haar[i] = kl_div_dev(p, haar[i] / hsum);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int i = 0; i < nbins; ++i) sum += haar[i];
    out[0] = sum;
  }
}

// ------------------------------------------------------------------ Meyer-Wallach
// Per state and qubit q: p1_q = sum_{bit q = 1} |a_i|^2 and
// c_q = sum_{bit q = 0} a_i conj(a_{i | bit q}); tr rho_q^2 = p0^2 + p1^2 + 2|c_q|^2.
// A CTA gathers a tile of 2^k amplitudes (the same active-bit gather as the
// sweeps), splits them to double-float and reduces, for every active bit, the
// pairs inside the tile.  N <= 13 is one pass; otherwise pass A (the low k bits)
// gives p1 for every qubit (a fixed bit adds the whole tile) and c for the low
// qubits, and pass B (a tile that contains the high bits) gives c for the rest.

// partial[row][tile][N + 1][3]: (p1, Re c, Im c) per qubit, then (tile total, 0, 0)
__global__ void __launch_bounds__(512) mw_tile_kernel(const __grid_constant__ SweepDesc sd,
                                                      const double2* __restrict__ psi, int n_qubits, int64_t tiles,
                                                      uint32_t c_bits, int with_p1, double* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem[];
  // warp partials: [quantity 0..2][local bit 0..12][warp 0..15] plus the tile total [warp]
  __shared__ float2 wpart[3][13][16];
  __shared__ float2 wtot[16];
  __shared__ double res[3 * 13 + 1];
  const int k = sd.k, c = sd.c;
  const int nloc = 1 << k;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float4* x = reinterpret_cast<float4*>(smem);
  float2* w = reinterpret_cast<float2*>(smem + sizeof(float4) * (size_t)nloc);
  int64_t* offs = reinterpret_cast<int64_t*>(smem + (sizeof(float4) + sizeof(float2)) * (size_t)nloc);
  const int64_t tile = blockIdx.x % tiles;
  const int64_t row = blockIdx.x / tiles;
  const int64_t D = 1ll << n_qubits;
  int64_t base = 0;
  for (int i = 0; i < sd.n_free; ++i)
    if ((tile >> i) & 1) base |= 1ll << sd.free_pos[i];
  // gather offsets of the tile's high local bits: offs[h] = sum over set bits j of h of 2^(position of local bit c+j)
  __shared__ int8_t pos_of[kMaxQubits];
  if (threadIdx.x < kMaxQubits && sd.local_of[threadIdx.x] >= 0) pos_of[sd.local_of[threadIdx.x]] = (int8_t)threadIdx.x;
  __syncthreads();
  for (int i = threadIdx.x; i < (1 << (k - c)); i += blockDim.x) {
    int64_t off = 0;
    for (int j = 0; j < k - c; ++j)
      if ((i >> j) & 1) off |= 1ll << pos_of[c + j];
    offs[i] = off;
  }
  __syncthreads();
  const int cmask = (1 << c) - 1;
  Acc tot{0.f, 0.f};
  for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
    const double2 v = psi[row * D + base + offs[l >> c] + (l & cmask)];
    const float2 re = split_double(v.x), im = split_double(v.y);
    x[l] = make_float4(re.x, re.y, im.x, im.y);
    Acc a{0.f, 0.f};
    acc_mul(a, re.x, re.y, re.x, re.y);
    acc_mul(a, im.x, im.y, im.x, im.y);
    w[l] = make_float2(a.h, a.l);
    acc_add(tot, a.h, a.l);
  }
  tot = warp_sum_df(tot);
  if (lane == 0) wtot[wid] = make_float2(tot.h, tot.l);
  __syncthreads();
  const int half = nloc >> 1;
  for (int j = 0; j < k; ++j) {
    const bool want_c = (c_bits >> j) & 1;
    Acc a1{0.f, 0.f}, ar{0.f, 0.f}, ai{0.f, 0.f};
    for (int t = threadIdx.x; t < half; t += blockDim.x) {
      const int i0 = ((t >> j) << (j + 1)) | (t & ((1 << j) - 1)), i1 = i0 | (1 << j);
      if (with_p1) {
        const float2 w1 = w[i1];
        acc_add(a1, w1.x, w1.y);
      }
      if (want_c) {
        const float4 u = x[i0], v = x[i1];
        // u conj(v) = (ur vr + ui vi) + i (ui vr - ur vi)
        acc_mul(ar, u.x, u.y, v.x, v.y);
        acc_mul(ar, u.z, u.w, v.z, v.w);
        acc_mul(ai, u.z, u.w, v.x, v.y);
        acc_mul(ai, -u.x, -u.y, v.z, v.w);
      }
    }
    a1 = warp_sum_df(a1);
    ar = warp_sum_df(ar);
    ai = warp_sum_df(ai);
    if (lane == 0) {
      wpart[0][j][wid] = make_float2(a1.h, a1.l);
      wpart[1][j][wid] = make_float2(ar.h, ar.l);
      wpart[2][j][wid] = make_float2(ai.h, ai.l);
    }
  }
  __syncthreads();
  // one thread per (quantity, bit) combines the warp partials in a fixed order
  if (threadIdx.x < 3 * k + 1) {
    Acc sacc{0.f, 0.f};
    if (threadIdx.x == 3 * k) {
      for (int q = 0; q < nw; ++q) acc_add(sacc, wtot[q].x, wtot[q].y);
    } else {
      const int qn = threadIdx.x / k, j = threadIdx.x % k;
      for (int q = 0; q < nw; ++q) acc_add(sacc, wpart[qn][j][q].x, wpart[qn][j][q].y);
    }
    res[threadIdx.x] = (double)sacc.h + (double)sacc.l;
  }
  __syncthreads();
  double* out = partial + ((row * tiles + tile) * (n_qubits + 1)) * 3;
  const double total = res[3 * k];
  for (int q = threadIdx.x; q <= n_qubits; q += blockDim.x) {
    double p1 = 0.0, cr = 0.0, ci = 0.0;
    if (q == n_qubits) {
      p1 = with_p1 ? total : 0.0;
    } else {
      const int p = n_qubits - 1 - q;
      const int j = sd.local_of[p];
      if (j < 0) {
        p1 = (with_p1 && ((base >> p) & 1)) ? total : 0.0;
      } else {
        p1 = with_p1 ? res[j] : 0.0;
        if ((c_bits >> j) & 1) {
          cr = res[k + j];
          ci = res[2 * k + j];
        }
      }
    }
    out[q * 3 + 0] = p1;
    out[q * 3 + 1] = cr;
    out[q * 3 + 2] = ci;
  }
}

// The same reduction for 12 <= N <= 22 with 2^11-amplitude tiles: a CTA takes a run of `tpc` tiles of one
// state and keeps its per-bit sums in registers across the run (bits unrolled), so the block reductions
// happen once per run instead of once per tile; two CTAs per SM.  partial[row][run][N + 1][3] as above.
constexpr int kMwRunBits = 11;
template <bool WP1>
__global__ void __launch_bounds__(256, 2) mw_run_kernel(const __grid_constant__ SweepDesc sd,
                                                        const double2* __restrict__ psi, int n_qubits, int64_t tiles,
                                                        int tpc, int64_t runs, uint32_t c_bits,
                                                        double* __restrict__ partial) {
  constexpr int K = kMwRunBits, NL = 1 << K, NT = 256, PER = NL / NT;
  extern __shared__ __align__(16) unsigned char smem[];
  float4* x = reinterpret_cast<float4*>(smem);
  float2* w = reinterpret_cast<float2*>(smem + sizeof(float4) * NL);
  int64_t* offs = reinterpret_cast<int64_t*>(smem + (sizeof(float4) + sizeof(float2)) * NL);
  // the next tile's amplitudes, copied asynchronously while the current one is reduced (each thread converts
  // exactly the amplitudes it copied, so the staging needs no block barrier)
  double2* stg = reinterpret_cast<double2*>(smem + (sizeof(float4) + sizeof(float2) + sizeof(int64_t)) * NL);
  __shared__ float2 tnorm[16][NT / 32];  // per tile of the run, per warp
  __shared__ float2 wpart[3 * K][NT / 32];
  __shared__ double res[3 * K];
  __shared__ double tot[16];
  __shared__ int8_t pos_of[kMaxQubits];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t row = blockIdx.x / runs, run = blockIdx.x - row * runs;
  const int64_t t0 = run * tpc, t1 = min(tiles, t0 + tpc);
  const int64_t D = 1ll << n_qubits;
  const int c = sd.c;
  if (threadIdx.x < kMaxQubits && sd.local_of[threadIdx.x] >= 0) pos_of[sd.local_of[threadIdx.x]] = (int8_t)threadIdx.x;
  __syncthreads();
  for (int i = threadIdx.x; i < (1 << (K - c)); i += NT) {
    int64_t off = 0;
    for (int j = 0; j < K - c; ++j)
      if ((i >> j) & 1) off |= 1ll << pos_of[c + j];
    offs[i] = off;
  }
  const int cmask = (1 << c) - 1;
  Acc a1[K], ar[K], ai[K];
#pragma unroll
  for (int j = 0; j < K; ++j) a1[j] = ar[j] = ai[j] = Acc{0.f, 0.f};
  auto issue = [&](int64_t tile) {
    int64_t base = 0;
    for (int i = 0; i < sd.n_free; ++i)
      if ((tile >> i) & 1) base |= 1ll << sd.free_pos[i];
    const double2* src = psi + row * D + base;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int l = threadIdx.x + NT * i;
      cp_async16(stg + l, src + offs[l >> c] + (l & cmask), 16);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  __syncthreads();  // offs ready
  if (t0 < t1) issue(t0);
  for (int64_t tile = t0; tile < t1; ++tile) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    Acc tn{0.f, 0.f};
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int l = threadIdx.x + NT * i;
      const double2 v = stg[l];
      const float2 re = split_double(v.x), im = split_double(v.y);
      x[l] = make_float4(re.x, re.y, im.x, im.y);
      Acc a{0.f, 0.f};
      acc_mul(a, re.x, re.y, re.x, re.y);
      acc_mul(a, im.x, im.y, im.x, im.y);
      w[l] = make_float2(a.h, a.l);
      acc_add(tn, a.h, a.l);
    }
    if (tile + 1 < t1) issue(tile + 1);
    tn = warp_sum_df(tn);
    if (lane == 0) tnorm[tile - t0][wid] = make_float2(tn.h, tn.l);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool want_c = (c_bits >> j) & 1;
#pragma unroll
      for (int u = 0; u < NL / 2 / NT; ++u) {
        const int t = threadIdx.x + NT * u;
        const int i0 = ((t >> j) << (j + 1)) | (t & ((1 << j) - 1)), i1 = i0 | (1 << j);
        if (WP1) {
          const float2 w1 = w[i1];
          acc_add(a1[j], w1.x, w1.y);
        }
        if (want_c) {
          const float4 p = x[i0], q = x[i1];
          // p conj(q) = (pr qr + pi qi) + i (pi qr - pr qi)
          acc_mul(ar[j], p.x, p.y, q.x, q.y);
          acc_mul(ar[j], p.z, p.w, q.z, q.w);
          acc_mul(ai[j], p.z, p.w, q.x, q.y);
          acc_mul(ai[j], -p.x, -p.y, q.z, q.w);
        }
      }
    }
    __syncthreads();  // the next tile's conversion overwrites x and w
  }
  // block sums of the run, combined in a fixed order
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const Acc s1 = warp_sum_df(a1[j]), sr = warp_sum_df(ar[j]), si = warp_sum_df(ai[j]);
    if (lane == 0) {
      wpart[j][wid] = make_float2(s1.h, s1.l);
      wpart[K + j][wid] = make_float2(sr.h, sr.l);
      wpart[2 * K + j][wid] = make_float2(si.h, si.l);
    }
  }
  __syncthreads();
  if (threadIdx.x < 3 * K) {
    Acc sacc{0.f, 0.f};
    for (int q = 0; q < NT / 32; ++q) acc_add(sacc, wpart[threadIdx.x][q].x, wpart[threadIdx.x][q].y);
    res[threadIdx.x] = (double)sacc.h + (double)sacc.l;
  } else if (threadIdx.x >= 64 && threadIdx.x < 64 + t1 - t0) {
    const int i = threadIdx.x - 64;
    Acc sacc{0.f, 0.f};
    for (int q = 0; q < NT / 32; ++q) acc_add(sacc, tnorm[i][q].x, tnorm[i][q].y);
    tot[i] = (double)sacc.h + (double)sacc.l;
  }
  __syncthreads();
  double* out = partial + ((row * runs + run) * (n_qubits + 1)) * 3;
  for (int q = threadIdx.x; q <= n_qubits; q += NT) {
    double p1 = 0.0, cr = 0.0, ci = 0.0;
    if (q == n_qubits) {
      if (WP1)
        for (int64_t t = t0; t < t1; ++t) p1 += tot[t - t0];
    } else {
      const int pos = n_qubits - 1 - q;
      const int j = sd.local_of[pos];
      if (j < 0) {
        if (WP1) {
          int fb = 0;  // index of pos among the free positions
          while (sd.free_pos[fb] != pos) ++fb;
          for (int64_t t = t0; t < t1; ++t)
            if ((t >> fb) & 1) p1 += tot[t - t0];
        }
      } else {
        p1 = WP1 ? res[j] : 0.0;
        if ((c_bits >> j) & 1) {
          cr = res[K + j];
          ci = res[2 * K + j];
        }
      }
    }
    out[q * 3 + 0] = p1;
    out[q * 3 + 1] = cr;
    out[q * 3 + 2] = ci;
  }
}

__global__ void mw_final(const double* __restrict__ pa, int64_t tiles_a, const double* __restrict__ pb,
                         int64_t tiles_b, int n_qubits, double* __restrict__ Q) {
  __shared__ double pur[64];
  const int64_t row = blockIdx.x;
  const int W = (n_qubits + 1) * 3;
  const int q = threadIdx.x;
  if (q < n_qubits) {
    double total = 0.0, p1 = 0.0, cr = 0.0, ci = 0.0;
    for (int64_t t = 0; t < tiles_a; ++t) {
      const double* o = pa + (row * tiles_a + t) * W;
      total += o[n_qubits * 3];
      p1 += o[q * 3 + 0];
      cr += o[q * 3 + 1];
      ci += o[q * 3 + 2];
    }
    for (int64_t t = 0; t < tiles_b; ++t) {
      const double* o = pb + (row * tiles_b + t) * W + q * 3;
      cr += o[1];
      ci += o[2];
    }
    const double p0 = total - p1;
    pur[q] = p0 * p0 + p1 * p1 + 2.0 * (cr * cr + ci * ci);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double summand = 0.0;
    for (int i = 0; i < n_qubits; ++i) summand += pur[i];
    Q[row] = 2.0 * (1.0 - (1.0 / n_qubits) * summand);
  }
}

// Two host-built tile descriptors for the MW passes.
struct MWPlan {
  SweepDesc a, b;
  bool two;
  std::vector<int64_t> offs;
};

static void mw_desc(int N, uint64_t active, SweepDesc& sd, std::vector<int64_t>& offs) {
  memset(&sd, 0, sizeof(sd));
  int act[64], na = 0;
  for (int p = 0; p < kMaxQubits; ++p) sd.local_of[p] = -1;
  for (int p = 0; p < N; ++p)
    if (active >> p & 1) act[na++] = p;
  sd.k = na;
  int c = 0;
  while (c < na && act[c] == c) ++c;
  sd.c = c;
  for (int j = 0; j < na; ++j) sd.local_of[act[j]] = (int8_t)j;
  sd.n_free = 0;
  for (int p = 0; p < N; ++p)
    if (!(active >> p & 1)) sd.free_pos[sd.n_free++] = (int8_t)p;
  sd.offs_begin = (int64_t)offs.size();
  for (int h = 0; h < (1 << (na - c)); ++h) {
    int64_t off = 0;
    for (int j = 0; j < na - c; ++j)
      if (h >> j & 1) off |= 1ll << act[c + j];
    offs.push_back(off);
  }
}

static MWPlan mw_plan(int N, int kmax = 13) {
  MWPlan m;
  const int k = N < kmax ? N : kmax;
  mw_desc(N, (k >= 64 ? ~0ull : ((1ull << k) - 1)), m.a, m.offs);
  m.two = N > k;
  if (m.two) {
    const int h = N - k;  // high positions k..N-1, filled up with the lowest positions
    uint64_t act = 0;
    for (int p = k; p < N; ++p) act |= 1ull << p;
    for (int p = 0; p < k - h; ++p) act |= 1ull << p;
    mw_desc(N, act, m.b, m.offs);
  }
  return m;
}

static size_t mw_smem(const SweepDesc& sd) {
  return (sizeof(float4) + sizeof(float2)) * ((size_t)1 << sd.k) + sizeof(int64_t) * ((size_t)1 << (sd.k - sd.c));
}

// ------------------------------------------------------------------ expectation
__global__ void expect_partial(const double2* __restrict__ psi, int n_qubits, const pqc_pauli_term* __restrict__ terms,
                               int n_terms, int64_t chunk, double* __restrict__ partial) {
  __shared__ double scratch[32];
  const int64_t D = 1ll << n_qubits;
  const int64_t row = blockIdx.y;
  const double2* x = psi + row * D;
  const int64_t s0 = blockIdx.x * chunk, s1 = min(D, s0 + chunk);
  double acc = 0.0;
  for (int64_t j = s0 + threadIdx.x; j < s1; j += blockDim.x) {
    const double2 u = x[j];
    double hr = 0.0, hi = 0.0;
    for (int t = 0; t < n_terms; ++t) {
      const pqc_pauli_term T = terms[t];
      const int64_t src = j ^ (int64_t)T.xmask;
      double2 v = x[src];
      double c = (__popcll((uint64_t)src & T.zmask) & 1) ? -T.coef : T.coef;
      double vr = v.x, vi = v.y;
      for (int q = 0; q < (T.n_y & 3); ++q) {
        double tmp = vr;
        vr = -vi;
        vi = tmp;
      }
      hr = fma(c, vr, hr);
      hi = fma(c, vi, hi);
    }
    acc = fma(u.x, hr, fma(u.y, hi, acc));  // Re(conj(u) h)
  }
  acc = block_sum(acc, scratch);
  if (threadIdx.x == 0) partial[row * gridDim.x + blockIdx.x] = acc;
}

__global__ void sum_rows_final(const double* __restrict__ partial, int nblk, int64_t rows, double* __restrict__ out) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= rows) return;
  double s = 0.0;
  for (int j = 0; j < nblk; ++j) s += partial[row * nblk + j];
  out[row] = s;
}

// ------------------------------------------------------------------ magic (WHT)
// partial[row][k] = sum_i |r_i|^{2 alpha}, r = WHT_j(conj(c_j) c_{j^k})
__global__ void magic_partial(const double2* __restrict__ psi, int n_qubits, double alpha,
                              double* __restrict__ partial) {
  extern __shared__ double2 v[];
  __shared__ double scratch[32];
  const int D = 1 << n_qubits;
  const int64_t row = blockIdx.y;
  const int k = blockIdx.x;
  const double2* c = psi + row * (int64_t)D;
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    double2 a = c[j], b = c[j ^ k];
    v[j] = make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);  // conj(a) * b
  }
  __syncthreads();
  for (int h = 1; h < D; h <<= 1) {
    for (int t = threadIdx.x; t < (D >> 1); t += blockDim.x) {
      const int i = ((t / h) * 2 * h) + (t % h);
      double2 a = v[i], b = v[i + h];
      v[i] = make_double2(a.x + b.x, a.y + b.y);
      v[i + h] = make_double2(a.x - b.x, a.y - b.y);
    }
    __syncthreads();
  }
  double acc = 0.0;
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    double m2 = v[j].x * v[j].x + v[j].y * v[j].y;
    acc += (alpha == 2.0) ? m2 * m2 : (alpha == 0.5 ? sqrt(m2) : pow(m2, alpha));
  }
  acc = block_sum(acc, scratch);
  if (threadIdx.x == 0) partial[row * gridDim.x + k] = acc;
}

// Renyi-2 (alpha = 2) in double-float on the FP32 pipes: the same transform per (state, shift k), with the
// products conj(c_j) c_{j^k} and the butterflies in double-float and sum_z |r_z|^4 accumulated in
// double-float.  GB300 runs FP64 at 1/72 of FP32, so the FP64 form above is bound by its DADDs.
__global__ void __launch_bounds__(256) magic2_partial_df(const double2* __restrict__ psi, int n_qubits,
                                                         double* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char magic_smem[];
  cdf* v = reinterpret_cast<cdf*>(magic_smem);
  __shared__ float2 ws[8];
  const int D = 1 << n_qubits;
  const int64_t row = blockIdx.y;
  const int k = blockIdx.x;
  const double2* c = psi + row * (int64_t)D;
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    const double2 a = c[j], b = c[j ^ k];
    const float2 ar = split_double(a.x), ai = split_double(a.y), br = split_double(b.x), bi = split_double(b.y);
    // conj(a) b = (ar br + ai bi) + i (ar bi - ai br)
    const df re = dot2(df{ar.x, ar.y}, df{br.x, br.y}, df{ai.x, ai.y}, df{bi.x, bi.y});
    const df im = dot2(df{ar.x, ar.y}, df{bi.x, bi.y}, df{-ai.x, -ai.y}, df{br.x, br.y});
    v[j] = cdf{re.h, re.l, im.h, im.l};
  }
  __syncthreads();
  for (int lh = 0; lh < n_qubits; ++lh) {
    const int h = 1 << lh;
    for (int t = threadIdx.x; t < (D >> 1); t += blockDim.x) {
      const int i = ((t >> lh) << (lh + 1)) | (t & (h - 1));
      const cdf a = v[i], b = v[i | h];
      v[i] = cadd(a, b);
      v[i | h] = cadd(a, cneg(b));
    }
    __syncthreads();
  }
  Acc acc{0.f, 0.f};
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    const cdf r = v[j];
    const df m2 = dot2(re(r), re(r), im(r), im(r));
    acc_mul(acc, m2.h, m2.l, m2.h, m2.l);
  }
  acc = warp_sum_df(acc);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = make_float2(acc.h, acc.l);
  __syncthreads();
  if (threadIdx.x == 0) {
    Acc t{0.f, 0.f};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) acc_add(t, ws[w].x, ws[w].y);
    partial[row * gridDim.x + k] = (double)t.h + (double)t.l;
  }
}

// The same Renyi-2 partial sum with the Walsh-Hadamard transform in radix 16: a CTA of D / 16 threads (used at N = 13),
// each thread holding 16 elements whose indices differ in the four bits of the current pass, so four butterfly
// stages run in registers between shared-memory round trips (ceil(N / 4) passes and barriers instead of N).  Pass
// p covers index bits [4p, 4p + w); element (t, m) of a pass is the index whose pass bits are the low w bits of m
// and whose other bits are (t << (4 - w)) | (m >> w).  The products conj(c_j) c_{j^k} are formed in the first pass
// and the sum of |r|^4 in the last, which stores nothing.  Shared memory is padded by one element in 16 so that
// the first pass (16 consecutive elements per thread) is free of bank conflicts.  The butterflies, their order
// and the double-float arithmetic are those of magic2_partial_df.
__device__ __forceinline__ int magic_pad(int i) { return i + (i >> 4); }

__device__ __forceinline__ int magic_elem(int t, int m, int lo, int w) {
  const int rest = (t << (4 - w)) | (m >> w);
  return (rest & ((1 << lo) - 1)) | ((m & ((1 << w) - 1)) << lo) | ((rest >> lo) << (lo + w));
}

__global__ void __launch_bounds__(512) magic2_radix16_df(const double2* __restrict__ psi, int n_qubits,
                                                         double* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char magic_smem[];
  cdf* v = reinterpret_cast<cdf*>(magic_smem);
  __shared__ float2 ws[16];
  const int D = 1 << n_qubits;
  const int64_t row = blockIdx.y;
  const int k = blockIdx.x;
  const int t = threadIdx.x;
  const double2* c = psi + row * (int64_t)D;
  const int passes = (n_qubits + 3) >> 2;
  Acc acc{0.f, 0.f};
  for (int p = 0; p < passes; ++p) {
    const int lo = 4 * p, w = min(4, n_qubits - lo);
    cdf a[16];
    if (p == 0) {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int j = magic_elem(t, m, lo, w);
        const double2 x = c[j], y = c[j ^ k];
        const float2 xr = split_double(x.x), xi = split_double(x.y), yr = split_double(y.x), yi = split_double(y.y);
        const df re = dot2(df{xr.x, xr.y}, df{yr.x, yr.y}, df{xi.x, xi.y}, df{yi.x, yi.y});
        const df im = dot2(df{xr.x, xr.y}, df{yi.x, yi.y}, df{-xi.x, -xi.y}, df{yr.x, yr.y});
        a[m] = cdf{re.h, re.l, im.h, im.l};
      }
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) a[m] = v[magic_pad(magic_elem(t, m, lo, w))];
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      if (s >= w) break;
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        if (m & (1 << s)) continue;
        const cdf x = a[m], y = a[m | (1 << s)];
        a[m] = cadd(x, y);
        a[m | (1 << s)] = cadd(x, cneg(y));
      }
    }
    if (p + 1 < passes) {
      // a thread reads and writes only its own elements within a pass; the next pass reads other threads' ones
#pragma unroll
      for (int m = 0; m < 16; ++m) v[magic_pad(magic_elem(t, m, lo, w))] = a[m];
      __syncthreads();
    } else {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const df m2 = dot2(re(a[m]), re(a[m]), im(a[m]), im(a[m]));
        acc_mul(acc, m2.h, m2.l, m2.h, m2.l);
      }
    }
  }
  acc = warp_sum_df(acc);
  if ((t & 31) == 0) ws[t >> 5] = make_float2(acc.h, acc.l);
  __syncthreads();
  if (t == 0) {
    Acc tot{0.f, 0.f};
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) acc_add(tot, ws[q].x, ws[q].y);
    partial[row * gridDim.x + k] = (double)tot.h + (double)tot.l;
  }
}

__global__ void magic_final(const double* __restrict__ partial, int n_qubits, double alpha, int64_t rows,
                            double* __restrict__ M) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= rows) return;
  const int D = 1 << n_qubits;
  double s = 0.0;
  for (int k = 0; k < D; ++k) s += partial[row * D + k];
  // |2^{-N/2} r|^{2 alpha} = 2^{-N alpha} |r|^{2 alpha}
  s *= exp2(-(double)n_qubits * alpha);
  M[row] = 1.0 / (1.0 - alpha) * log(s) - log(exp2((double)n_qubits));
}

// ------------------------------------------------------------------ cross Gram
// G[a][b] = <x_a|y_b> summed over the chunk partials
__global__ void gram_cross_final(const double2* __restrict__ partial, int nchunk, int nta, int ntb, int64_t SA,
                                 int64_t SB, double2* __restrict__ G) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= SA * SB) return;
  const int64_t a = idx / SB, b = idx % SB;
  const int ta = (int)(a / TS), tb = (int)(b / TS);
  const int ty = (int)(a % TS), tx = (int)(b % TS);
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    const double2 p = partial[(((int64_t)c * nta + ta) * ntb + tb) * (TS * TS) + ty * TS + tx];
    re += p.x;
    im += p.y;
  }
  G[idx] = make_double2(re, im);
}

// ------------------------------------------------------------------ QFIM
// overlap pairs (0, p) of the reference state with every derivative state
__global__ void qfim_pairs(int64_t* __restrict__ idx, int64_t P) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= P) return;
  idx[p] = 0;
  idx[P + p] = p;
}

__global__ void qfim_final(const double2* __restrict__ partial, int nchunk, int nt, int64_t P,
                           const double2* __restrict__ v, double* __restrict__ F) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= P * P) return;
  int64_t p = idx / P, q = idx % P;
  int64_t a = p < q ? p : q, b = p < q ? q : p;  // upper triangle, copied to the lower one
  double2 g = gram_entry(partial, nchunk, nt, a, b);
  double2 va = v[a], vb = v[b];
  // Re(conj(va) vb)
  double rhs = va.x * vb.x + va.y * vb.y;
  F[idx] = 4.0 * (g.x - rhs);
}

}  // namespace pqc

using namespace pqc;

extern "C" size_t pqc_overlaps_workspace_size(int64_t n, int32_t n_qubits) {
  if (n <= 0) return 256;
  return align_up((size_t)n * overlap_blocks(n_qubits, n) * sizeof(double2), 256);
}

extern "C" int pqc_overlaps(const void* a, const void* b, const int64_t* ia, const int64_t* ib, int64_t n,
                            int32_t n_qubits, void* out, void* workspace, size_t workspace_bytes, void* stream_v) {
  if (n < 0) return fail(PQC_ERR_INVALID, "n < 0");
  if (n == 0) return PQC_OK;
  if (!a || !b || !ia || !ib || !out) return fail(PQC_ERR_INVALID, "NULL argument");
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  const size_t need = pqc_overlaps_workspace_size(n, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  cudaStream_t stream = (cudaStream_t)stream_v;
  const int nblk = overlap_blocks(n_qubits, n);
  const int64_t D = 1ll << n_qubits;
  const int64_t chunk = (D + nblk - 1) / nblk;
  double2* partial = (double2*)workspace;
  for (int64_t k0 = 0; k0 < n; k0 += 65535) {
    const int64_t nk = std::min<int64_t>(65535, n - k0);
    overlap_partial<<<dim3(nblk, (unsigned)nk), 256, 0, stream>>>((const double2*)a, (const double2*)b, ia, ib,
                                                                  n_qubits, chunk, k0, partial);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  overlap_final<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(partial, nblk, n, (double2*)out);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

// the partial-sum region shared by the three Grams (double-float, FP32, tensor cores)
static size_t hist_partial_ws(int64_t S, int n_qubits) {
  return std::max(std::max(gram_ws(S, n_qubits), gram_fast_ws(S, n_qubits)), gram_tc_ws(S, n_qubits));
}

extern "C" size_t pqc_fidelity_hist_workspace_size(int64_t S, int32_t n_qubits) {
  if (S < 2) return 256;
  // partials (either Gram) | refine list | control words | the states as truncated FP32
  return hist_partial_ws(S, n_qubits) + align_up(kRefineCap * sizeof(int64_t), 256) + 256 +
         align_up((size_t)S * ((size_t)1 << n_qubits) * sizeof(float2), 256);
}

extern "C" int pqc_fidelity_hist(const void* psi, int64_t S, int32_t n_qubits, int32_t nbins, const double* edges,
                                 double* F, int64_t* counts, void* workspace, size_t workspace_bytes, void* stream_v) {
  if (S < 0) return fail(PQC_ERR_INVALID, "S < 0");
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  if (counts && (nbins < 1 || !edges)) return fail(PQC_ERR_INVALID, "histogram needs nbins >= 1 and edges");
  cudaStream_t stream = (cudaStream_t)stream_v;
  if (counts) PQC_CUDA(cudaMemsetAsync(counts, 0, nbins * sizeof(int64_t), stream));
  if (S < 2) return PQC_OK;
  if (!psi) return fail(PQC_ERR_INVALID, "psi is NULL");
  const size_t need = pqc_fidelity_hist_workspace_size(S, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  int nt, nchunk;
  double2* partial = (double2*)workspace;
  const int64_t M = S * (S - 1) / 2;
  if (F || !counts) {  // the fidelities themselves: the double-float Gram for every pair
    int rc = launch_gram((const double2*)psi, S, n_qubits, partial, nt, nchunk, stream);
    if (rc) return rc;
    fid_final<<<(unsigned)((M + 255) / 256), 256, 0, stream>>>(partial, nchunk, nt, S, edges, nbins, F,
                                                               (unsigned long long*)counts);
    count_launch();
    PQC_CUDA(cudaGetLastError());
    return PQC_OK;
  }
  // counts only: a certified low-precision Gram (tensor cores for S <= 256 and n >= 13, else FP32 products;
  // the FP32 tier also runs when the tensor-core tier leaves more pairs undecided than the list holds), exact
  // recomputation of the undecided pairs, and the double-float recount of every pair when the list overflows.
  // ctl[0]: listed pairs, ctl[1]: recount every pair, ctl[2]: run the FP32 tier after the tensor-core tier.
  int64_t* list = (int64_t*)((char*)workspace + hist_partial_ws(S, n_qubits));
  int* ctl = (int*)((char*)list + align_up(kRefineCap * sizeof(int64_t), 256));
  unsigned long long* cnt = (unsigned long long*)counts;
  PQC_CUDA(cudaMemsetAsync(ctl, 0, 3 * sizeof(int), stream));
  float2* y = (float2*)((char*)ctl + 256);
  const bool tc = gram_tc_usable(S, n_qubits);
  if (tc) {
    double2* G = nullptr;
    double dfac = 0.0;
    int rc = launch_gram_tc((const double2*)psi, S, n_qubits, (float*)y, partial, &G, &dfac, ctl + 1, stream);
    if (rc) return rc;
    fid_certify_tc<<<(unsigned)((M + 255) / 256), 256, 0, stream>>>(G, S, dfac, edges, nbins, cnt, list, ctl);
    count_launch();
    tc_tier_reset<<<1, 256, 0, stream>>>(ctl, cnt, nbins);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  const int* gate = tc ? ctl + 2 : nullptr;
  static int fast_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (fast_dev != dev) {
    PQC_CUDA(cudaFuncSetAttribute(gram_fast_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGramFastSmem));
    fast_dev = dev;
  }
  const int64_t n_amp = S << n_qubits;
  trunc_to_f32<<<(unsigned)std::min<int64_t>((n_amp + 255) / 256, 152 * 16), 256, 0, stream>>>((const double2*)psi, y,
                                                                                              n_amp, gate);
  count_launch();
  int ntf, nchunkf;
  int64_t chunk;
  gram_fast_geometry(S, n_qubits, ntf, nchunkf, chunk);
  gram_fast_partial<<<dim3(ntf, ntf, nchunkf), 256, kGramFastSmem, stream>>>(y, S, n_qubits, chunk, partial, gate);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  fid_certify<<<(unsigned)((M + 255) / 256), 256, 0, stream>>>(partial, nchunkf, ntf, S, edges, nbins, cnt, list,
                                                               ctl, gate);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  fid_refine<<<(unsigned)std::min<int64_t>(M, kRefineCap), 256, 0, stream>>>((const double2*)psi, S, n_qubits,
                                                                              edges, nbins, cnt, list, ctl);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  // overflow: clear and recount every pair with the double-float Gram (these kernels exit at once otherwise)
  clear_counts_if<<<1, 256, 0, stream>>>(ctl, cnt, nbins);
  count_launch();
  gram_geometry(S, n_qubits, nt, nchunk, chunk);
  gram_partial<<<dim3(nt, nt, nchunk), 256, 0, stream>>>((const double2*)psi, S, (const double2*)psi, S, n_qubits,
                                                          chunk, 0, 1, partial, ctl + 1);
  count_launch();
  fid_final<<<(unsigned)((M + 255) / 256), 256, 0, stream>>>(partial, nchunk, nt, S, edges, nbins, nullptr, cnt,
                                                             ctl + 1);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" int pqc_histogram(const double* F, int64_t M, int32_t nbins, const double* edges, int64_t* counts,
                             void* stream_v) {
  if (M < 0 || nbins < 1 || !edges || !counts || (M > 0 && !F)) return fail(PQC_ERR_INVALID, "bad arguments");
  cudaStream_t stream = (cudaStream_t)stream_v;
  PQC_CUDA(cudaMemsetAsync(counts, 0, nbins * sizeof(int64_t), stream));
  if (M == 0) return PQC_OK;
  hist_kernel<<<(unsigned)((M + 255) / 256), 256, 0, stream>>>(F, M, edges, nbins, (unsigned long long*)counts);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" int pqc_expr_kl(const int64_t* counts, int32_t nbins, const double* edges, double d, double* out,
                           void* stream_v) {
  if (!counts || !edges || !out || nbins < 1) return fail(PQC_ERR_INVALID, "bad arguments");
  cudaStream_t stream = (cudaStream_t)stream_v;
  if (nbins > 1024) return fail(PQC_ERR_UNSUPPORTED, "at most 1024 bins");
  expr_kl_kernel<<<1, 256, 0, stream>>>((const unsigned long long*)counts, nbins, edges, d, out);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" size_t pqc_mw_workspace_size(int64_t batch, int32_t n_qubits) {
  if (batch <= 0 || n_qubits < 1 || n_qubits > kMaxQubits) return 256;
  const int k = n_qubits < 13 ? n_qubits : 13;
  const size_t tiles = (size_t)1 << (n_qubits - k);
  const size_t per = (size_t)batch * tiles * (n_qubits + 1) * 3 * sizeof(double);
  return 2 * align_up(per, 256);
}

extern "C" int pqc_mw(const void* psi, int64_t batch, int32_t n_qubits, double* Q, void* workspace,
                      size_t workspace_bytes, void* stream_v) {
  if (batch < 0) return fail(PQC_ERR_INVALID, "batch < 0");
  if (batch == 0) return PQC_OK;
  if (!psi || !Q) return fail(PQC_ERR_INVALID, "NULL argument");
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  const size_t need = pqc_mw_workspace_size(batch, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  cudaStream_t stream = (cudaStream_t)stream_v;
  static int attr_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    PQC_CUDA(cudaFuncSetAttribute(mw_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_dev = dev;
  }
  const size_t half = pqc_mw_workspace_size(batch, n_qubits) / 2;
  char* w = (char*)workspace;
  double* pa = (double*)w;
  double* pb = (double*)(w + half);
  if (n_qubits >= 12 && n_qubits <= 2 * kMwRunBits) {
    // runs of 2^11-amplitude tiles (two passes); runs of at least 4 tiles keep the partials within the
    // workspace sized for 2^13-amplitude tiles, at most 16 fit the per-tile norms
    static int run_dev = -1;
    if (run_dev != dev) {
      PQC_CUDA(cudaFuncSetAttribute(mw_run_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
      PQC_CUDA(cudaFuncSetAttribute(mw_run_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
      run_dev = dev;
    }
    const MWPlan m = mw_plan(n_qubits, kMwRunBits);
    const int64_t tiles = 1ll << (n_qubits - kMwRunBits);
    const int tpc = (int)std::max<int64_t>(4, std::min<int64_t>(16, tiles * batch / (152 * 8)));
    const int64_t runs = (tiles + tpc - 1) / tpc;
    const int64_t max_rows = std::max<int64_t>(1, (int64_t)0x7fffffff / runs);
    for (int pass = 0; pass < 2; ++pass) {
      const SweepDesc& sd = pass == 0 ? m.a : m.b;
      uint32_t cbits = 0;
      for (int p = 0; p < n_qubits; ++p) {
        const int j = sd.local_of[p];
        if (j >= 0 && (pass == 0 ? (p < kMwRunBits) : (p >= kMwRunBits))) cbits |= 1u << j;
      }
      // tile, |a|^2, gather offsets (at most 2^11) and the staging of the next tile
      const size_t smem = (sizeof(float4) + sizeof(float2) + sizeof(int64_t) + sizeof(double2)) << kMwRunBits;
      for (int64_t r0 = 0; r0 < batch; r0 += max_rows) {
        const int64_t nr = std::min(max_rows, batch - r0);
        const double2* src = (const double2*)psi + (r0 << n_qubits);
        double* out = (pass == 0 ? pa : pb) + r0 * runs * (n_qubits + 1) * 3;
        if (pass == 0)
          mw_run_kernel<true><<<(unsigned)(nr * runs), 256, smem, stream>>>(sd, src, n_qubits, tiles, tpc, runs, cbits,
                                                                             out);
        else
          mw_run_kernel<false><<<(unsigned)(nr * runs), 256, smem, stream>>>(sd, src, n_qubits, tiles, tpc, runs,
                                                                              cbits, out);
        count_launch();
        PQC_CUDA(cudaGetLastError());
      }
    }
    mw_final<<<(unsigned)batch, 64, 0, stream>>>(pa, runs, pb, runs, n_qubits, Q);
    count_launch();
    PQC_CUDA(cudaGetLastError());
    return PQC_OK;
  }
  MWPlan m = mw_plan(n_qubits);
  const int k = m.a.k;
  const int64_t tiles = 1ll << (n_qubits - k);
  const int64_t max_rows = std::max<int64_t>(1, (int64_t)0x7fffffff / tiles);
  for (int pass = 0; pass < (m.two ? 2 : 1); ++pass) {
    const SweepDesc& sd = pass == 0 ? m.a : m.b;
    uint32_t cbits = 0;
    for (int p = 0; p < n_qubits; ++p) {
      const int j = sd.local_of[p];
      if (j >= 0 && (pass == 0 ? (p < k) : (p >= k))) cbits |= 1u << j;
    }
    for (int64_t r0 = 0; r0 < batch; r0 += max_rows) {
      const int64_t nr = std::min(max_rows, batch - r0);
      mw_tile_kernel<<<(unsigned)(nr * tiles), 512, mw_smem(sd), stream>>>(
          sd, (const double2*)psi + (r0 << n_qubits), n_qubits, tiles, cbits, pass == 0 ? 1 : 0,
          (pass == 0 ? pa : pb) + r0 * tiles * (n_qubits + 1) * 3);
      count_launch();
      PQC_CUDA(cudaGetLastError());
    }
  }
  mw_final<<<(unsigned)batch, 64, 0, stream>>>(pa, tiles, pb, m.two ? tiles : 0, n_qubits, Q);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

static int expect_blocks(int n_qubits, int64_t rows) {
  const int64_t D = 1ll << n_qubits;
  int64_t want = std::max<int64_t>(1, 1216 / std::max<int64_t>(rows, 1));
  int64_t cap = std::max<int64_t>(1, D / 1024);
  return (int)std::min<int64_t>(std::min<int64_t>(want, cap), 1024);
}

extern "C" size_t pqc_expect_workspace_size(int64_t batch, int32_t n_qubits, int32_t n_terms) {
  (void)n_terms;
  if (batch <= 0 || n_qubits < 1) return 256;
  return align_up((size_t)batch * expect_blocks(n_qubits, batch) * sizeof(double), 256);
}

extern "C" int pqc_expect(const void* psi, int64_t batch, int32_t n_qubits, const pqc_pauli_term* terms,
                          int32_t n_terms, double* E, void* workspace, size_t workspace_bytes, void* stream_v) {
  if (batch < 0 || n_terms < 0) return fail(PQC_ERR_INVALID, "negative count");
  if (batch == 0) return PQC_OK;
  if (!psi || !E || (n_terms > 0 && !terms)) return fail(PQC_ERR_INVALID, "NULL argument");
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  const size_t need = pqc_expect_workspace_size(batch, n_qubits, n_terms);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  cudaStream_t stream = (cudaStream_t)stream_v;
  const int nblk = expect_blocks(n_qubits, batch);
  const int64_t D = 1ll << n_qubits;
  const int64_t chunk = (D + nblk - 1) / nblk;
  double* partial = (double*)workspace;
  for (int64_t r0 = 0; r0 < batch; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, batch - r0);
    expect_partial<<<dim3(nblk, (unsigned)nr), 256, 0, stream>>>((const double2*)psi + r0 * D, n_qubits, terms,
                                                                 n_terms, chunk, partial + r0 * nblk);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  sum_rows_final<<<(unsigned)((batch + 127) / 128), 128, 0, stream>>>(partial, nblk, batch, E);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" size_t pqc_magic_workspace_size(int64_t batch, int32_t n_qubits) {
  if (batch <= 0 || n_qubits < 1 || n_qubits > 13) return 256;
  return align_up((size_t)batch * ((size_t)1 << n_qubits) * sizeof(double), 256);
}

extern "C" int pqc_magic(const void* psi, int64_t batch, int32_t n_qubits, double alpha, double* M, void* workspace,
                         size_t workspace_bytes, void* stream_v) {
  if (batch < 0) return fail(PQC_ERR_INVALID, "batch < 0");
  if (batch == 0) return PQC_OK;
  if (!psi || !M) return fail(PQC_ERR_INVALID, "NULL argument");
  if (n_qubits < 1 || n_qubits > 13) return fail(PQC_ERR_UNSUPPORTED, "magic supports 1 <= n_qubits <= 13");
  if (alpha == 1.0) return fail(PQC_ERR_INVALID, "alpha = 1 is singular in the Renyi formula");
  const size_t need = pqc_magic_workspace_size(batch, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  cudaStream_t stream = (cudaStream_t)stream_v;
  const int D = 1 << n_qubits;
  const size_t smem = (size_t)D * sizeof(double2);
  const bool df2 = alpha == 2.0;
  // radix 16 at N = 13 only: there the one-stage kernel's 128 KiB tile allows one 256-thread CTA per SM and the
  // radix-16 CTA of 512 threads ran 27 % faster; at N <= 12 the one-stage kernel keeps several CTAs per SM and was
  // faster (4 % at N = 12, 29 % at N = 10)
  const bool radix16 = df2 && n_qubits == 13;
  const size_t smem16 = (size_t)(D + D / 16) * sizeof(cdf);
  if (radix16 && smem16 > 48 * 1024)
    PQC_CUDA(cudaFuncSetAttribute(magic2_radix16_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem16));
  if (!radix16 && smem > 48 * 1024) {  // opt in to exactly what this launch needs (the kernels also have static scratch)
    if (df2)
      PQC_CUDA(cudaFuncSetAttribute(magic2_partial_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    else
      PQC_CUDA(cudaFuncSetAttribute(magic_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  double* partial = (double*)workspace;
  for (int64_t r0 = 0; r0 < batch; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, batch - r0);
    if (radix16)
      magic2_radix16_df<<<dim3(D, (unsigned)nr), D / 16, smem16, stream>>>((const double2*)psi + r0 * D, n_qubits,
                                                                           partial + r0 * D);
    else if (df2)
      magic2_partial_df<<<dim3(D, (unsigned)nr), 256, smem, stream>>>((const double2*)psi + r0 * D, n_qubits,
                                                                      partial + r0 * D);
    else
      magic_partial<<<dim3(D, (unsigned)nr), 256, smem, stream>>>((const double2*)psi + r0 * D, n_qubits, alpha,
                                                                  partial + r0 * D);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  magic_final<<<(unsigned)((batch + 127) / 128), 128, 0, stream>>>(partial, n_qubits, alpha, batch, M);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" size_t pqc_qfim_workspace_size(int64_t P, int32_t n_qubits) {
  if (P <= 0) return 256;
  return gram_ws(P, n_qubits) + align_up((size_t)P * sizeof(double2), 256) + align_up(P * 2 * sizeof(int64_t), 256) +
         pqc_overlaps_workspace_size(P, n_qubits);
}

static int qfim_impl(const void* state, const void* dpsi, int64_t P, int32_t n_qubits, double* F, void* workspace,
                     size_t workspace_bytes, void* stream_v, bool fp64) {
  if (P < 0) return fail(PQC_ERR_INVALID, "P < 0");
  if (P == 0) return PQC_OK;
  if (!state || !dpsi || !F) return fail(PQC_ERR_INVALID, "NULL argument");
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  const size_t need = pqc_qfim_workspace_size(P, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  cudaStream_t stream = (cudaStream_t)stream_v;
  char* w = (char*)workspace;
  double2* partial = (double2*)w;
  w += gram_ws(P, n_qubits);
  double2* v = (double2*)w;
  w += align_up((size_t)P * sizeof(double2), 256);
  int64_t* idx = (int64_t*)w;
  w += align_up(P * 2 * sizeof(int64_t), 256);
  void* ows = w;
  // v_p = <state|d_p>: pairs (0, p)
  qfim_pairs<<<(unsigned)((P + 255) / 256), 256, 0, stream>>>(idx, P);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  int rc = pqc_overlaps(state, dpsi, idx, idx + P, P, n_qubits, v, ows, pqc_overlaps_workspace_size(P, n_qubits),
                        stream);
  if (rc) return rc;
  int nt, nchunk;
  rc = launch_gram((const double2*)dpsi, P, n_qubits, partial, nt, nchunk, stream, 1, fp64);
  if (rc) return rc;
  qfim_final<<<(unsigned)((P * P + 255) / 256), 256, 0, stream>>>(partial, nchunk, nt, P, v, F);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" int pqc_qfim(const void* state, const void* dpsi, int64_t P, int32_t n_qubits, double* F, void* workspace,
                        size_t workspace_bytes, void* stream) {
  return qfim_impl(state, dpsi, P, n_qubits, F, workspace, workspace_bytes, stream, false);
}

extern "C" int pqc_qfim_fp64(const void* state, const void* dpsi, int64_t P, int32_t n_qubits, double* F,
                             void* workspace, size_t workspace_bytes, void* stream) {
  return qfim_impl(state, dpsi, P, n_qubits, F, workspace, workspace_bytes, stream, true);
}

extern "C" size_t pqc_gram_cross_workspace_size(int64_t na, int64_t nb, int32_t n_qubits) {
  if (na <= 0 || nb <= 0 || n_qubits < 1 || n_qubits > kMaxQubits) return 256;
  int nt, nchunk;
  int64_t chunk;
  gram_geometry(na, n_qubits, nt, nchunk, chunk, nb);
  const int ntb = (int)((nb + TS - 1) / TS);
  return align_up((size_t)nchunk * nt * ntb * TS * TS * sizeof(double2), 256);
}

extern "C" int pqc_gram_cross(const void* a, int64_t na, const void* b, int64_t nb, int32_t n_qubits, void* G,
                              void* workspace, size_t workspace_bytes, void* stream_v) {
  if (na < 0 || nb < 0) return fail(PQC_ERR_INVALID, "negative count");
  if (na == 0 || nb == 0) return PQC_OK;
  if (!a || !b || !G) return fail(PQC_ERR_INVALID, "NULL argument");
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  const size_t need = pqc_gram_cross_workspace_size(na, nb, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  cudaStream_t stream = (cudaStream_t)stream_v;
  int nt, nchunk;
  int64_t chunk;
  gram_geometry(na, n_qubits, nt, nchunk, chunk, nb);
  const int ntb = (int)((nb + TS - 1) / TS);
  double2* partial = (double2*)workspace;
  gram_partial<<<dim3(nt, ntb, nchunk), 256, 0, stream>>>((const double2*)a, na, (const double2*)b, nb, n_qubits,
                                                          chunk, 0, 0, partial);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  gram_cross_final<<<(unsigned)((na * nb + 255) / 256), 256, 0, stream>>>(partial, nchunk, nt, ntb, na, nb,
                                                                          (double2*)G);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}
