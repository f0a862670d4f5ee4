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

#include "engine.cuh"
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
constexpr int TS = 16;  // states per tile side
constexpr int KS = 32;  // amplitudes per smem slice

// partial[chunk][ta][tb][16][16] = sum over the chunk of conj(x_a) x_b
__global__ void __launch_bounds__(256) gram_partial(const double2* __restrict__ X, int64_t S, int n_qubits,
                                                    int64_t chunk, double2* __restrict__ partial) {
  const int ta = blockIdx.x, tb = blockIdx.y;
  if (ta > tb) return;
  __shared__ double2 As[TS][KS + 1];
  __shared__ double2 Bs[KS][TS];
  const int64_t D = 1ll << n_qubits;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t a0 = (int64_t)ta * TS, b0 = (int64_t)tb * TS;
  const int64_t s0 = blockIdx.z * chunk, s1 = min(D, s0 + chunk);
  double re = 0.0, im = 0.0;
  for (int64_t base = s0; base < s1; base += KS) {
    for (int e = threadIdx.x; e < TS * KS; e += 256) {
      int r = e / KS, kk = e % KS;
      int64_t i = base + kk;
      int64_t ra = a0 + r, rb = b0 + r;
      As[r][kk] = (ra < S && i < s1) ? X[ra * D + i] : make_double2(0.0, 0.0);
      Bs[kk][r] = (rb < S && i < s1) ? X[rb * D + i] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < KS; ++kk) {
      double2 u = As[ty][kk], v = Bs[kk][tx];
      re = fma(u.x, v.x, fma(u.y, v.y, re));
      im = fma(u.x, v.y, fma(-u.y, v.x, im));
    }
    __syncthreads();
  }
  const int nt = gridDim.x;
  partial[(((int64_t)blockIdx.z * nt + ta) * nt + tb) * 256 + ty * 16 + tx] = make_double2(re, im);
}

__device__ __forceinline__ double2 gram_entry(const double2* __restrict__ partial, int nchunk, int nt, int64_t a,
                                              int64_t b) {
  const int ta = (int)(a / TS), tb = (int)(b / TS);
  const int ty = (int)(a % TS), tx = (int)(b % TS);
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    double2 p = partial[(((int64_t)c * nt + ta) * nt + tb) * 256 + ty * 16 + tx];
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
__global__ void fid_final(const double2* __restrict__ partial, int nchunk, int nt, int64_t S,
                          const double* __restrict__ edges, int nbins, double* __restrict__ F,
                          unsigned long long* __restrict__ counts) {
  const int64_t M = S * (S - 1) / 2;
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= M) return;
  // invert k = a*(2S-a-1)/2 + (b-a-1)
  double Sd = (double)S;
  int64_t a = (int64_t)floor(((2.0 * Sd - 1.0) - sqrt((2.0 * Sd - 1.0) * (2.0 * Sd - 1.0) - 8.0 * (double)k)) / 2.0);
  if (a < 0) a = 0;
  while (a > 0 && a * (2 * S - a - 1) / 2 > k) --a;
  while ((a + 1) * (2 * S - a - 2) / 2 <= k) ++a;
  const int64_t b = k - a * (2 * S - a - 1) / 2 + a + 1;
  double2 g = gram_entry(partial, nchunk, nt, a, b);
  double f = g.x * g.x + g.y * g.y;
  if (F) F[k] = f;
  if (counts) {
    int bin = np_bin(f, edges, nbins);
    if (bin >= 0) atomicAdd(&counts[bin], 1ull);
  }
}

static void gram_geometry(int64_t S, int n_qubits, int& nt, int& nchunk, int64_t& chunk) {
  const int64_t D = 1ll << n_qubits;
  nt = (int)((S + TS - 1) / TS);
  const int64_t pairs = (int64_t)nt * (nt + 1) / 2;
  int64_t want = std::max<int64_t>(1, (152 * 6 + pairs - 1) / pairs);
  int64_t maxc = std::max<int64_t>(1, D / (4 * KS));
  nchunk = (int)std::min<int64_t>(std::min<int64_t>(want, maxc), 65535);
  chunk = (D + nchunk - 1) / nchunk;
  chunk = (chunk + KS - 1) / KS * KS;
  nchunk = (int)((D + chunk - 1) / chunk);
}

static size_t gram_ws(int64_t S, int n_qubits) {
  int nt, nchunk;
  int64_t chunk;
  gram_geometry(S, n_qubits, nt, nchunk, chunk);
  return align_up((size_t)nchunk * nt * nt * 256 * sizeof(double2), 256);
}

static int launch_gram(const double2* X, int64_t S, int n_qubits, double2* partial, int& nt, int& nchunk,
                       cudaStream_t stream) {
  int64_t chunk;
  gram_geometry(S, n_qubits, nt, nchunk, chunk);
  dim3 grid(nt, nt, nchunk);
  gram_partial<<<grid, 256, 0, stream>>>(X, S, n_qubits, chunk, partial);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
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
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long tot = 0;
  for (int i = 0; i < nbins; ++i) tot += counts[i];
  double hsum = 0.0;
  for (int i = 0; i < nbins; ++i) {
    double F = (edges[i] + edges[i + 1]) / 2;
    hsum += (d - 1) * pow(1 - F, d - 2);
  }
  double s = 0.0;
  for (int i = 0; i < nbins; ++i) {
    double F = (edges[i] + edges[i + 1]) / 2;
    double p = (double)counts[i] / (double)tot;
    double h = (d - 1) * pow(1 - F, d - 2) / hsum;
    s += kl_div_dev(p, h);
  }
  out[0] = s;
}

// ------------------------------------------------------------------ Meyer-Wallach
// partial[row][blk][q][4] = (p0, p1, Re c, Im c) over this block's pair chunk
__global__ void mw_partial(const double2* __restrict__ psi, int n_qubits, int64_t chunk,
                           double* __restrict__ partial) {
  __shared__ double scratch[32];
  const int64_t D = 1ll << n_qubits, half = D >> 1;
  const int64_t row = blockIdx.y;
  const double2* x = psi + row * D;
  const int64_t t0 = blockIdx.x * chunk, t1 = min(half, t0 + chunk);
  for (int q = 0; q < n_qubits; ++q) {
    const int p = n_qubits - 1 - q;
    double p0 = 0.0, p1 = 0.0, cr = 0.0, ci = 0.0;
    for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
      const int64_t i0 = ((t >> p) << (p + 1)) | (t & ((1ll << p) - 1));
      const int64_t i1 = i0 | (1ll << p);
      double2 u = x[i0], v = x[i1];
      p0 = fma(u.x, u.x, fma(u.y, u.y, p0));
      p1 = fma(v.x, v.x, fma(v.y, v.y, p1));
      // rho_01 = sum u conj(v)
      cr = fma(u.x, v.x, fma(u.y, v.y, cr));
      ci = fma(u.y, v.x, fma(-u.x, v.y, ci));
    }
    p0 = block_sum(p0, scratch);
    p1 = block_sum(p1, scratch);
    cr = block_sum(cr, scratch);
    ci = block_sum(ci, scratch);
    if (threadIdx.x == 0) {
      double* o = partial + ((row * gridDim.x + blockIdx.x) * n_qubits + q) * 4;
      o[0] = p0;
      o[1] = p1;
      o[2] = cr;
      o[3] = ci;
    }
  }
}

__global__ void mw_final(const double* __restrict__ partial, int nblk, int n_qubits, int64_t rows,
                         double* __restrict__ Q) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= rows) return;
  double summand = 0.0;
  for (int q = 0; q < n_qubits; ++q) {
    double p0 = 0.0, p1 = 0.0, cr = 0.0, ci = 0.0;
    for (int j = 0; j < nblk; ++j) {
      const double* o = partial + ((row * nblk + j) * n_qubits + q) * 4;
      p0 += o[0];
      p1 += o[1];
      cr += o[2];
      ci += o[3];
    }
    summand += p0 * p0 + p1 * p1 + 2.0 * (cr * cr + ci * ci);
  }
  Q[row] = 2.0 * (1.0 - (1.0 / n_qubits) * summand);
}

static int mw_blocks(int n_qubits, int64_t rows) {
  const int64_t half = (1ll << n_qubits) >> 1;
  int64_t want = std::max<int64_t>(1, 1216 / std::max<int64_t>(rows, 1));
  int64_t cap = std::max<int64_t>(1, half / 1024);
  return (int)std::min<int64_t>(std::min<int64_t>(want, cap), 1024);
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

// ------------------------------------------------------------------ QFIM
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

extern "C" size_t pqc_fidelity_hist_workspace_size(int64_t S, int32_t n_qubits) {
  if (S < 2) return 256;
  return gram_ws(S, n_qubits);
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
  const size_t need = gram_ws(S, n_qubits);
  if (!workspace || workspace_bytes < need) return fail(PQC_ERR_WORKSPACE, "workspace too small");
  int nt, nchunk;
  double2* partial = (double2*)workspace;
  int rc = launch_gram((const double2*)psi, S, n_qubits, partial, nt, nchunk, stream);
  if (rc) return rc;
  const int64_t M = S * (S - 1) / 2;
  fid_final<<<(unsigned)((M + 255) / 256), 256, 0, stream>>>(partial, nchunk, nt, S, edges, nbins, F,
                                                             (unsigned long long*)counts);
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
  expr_kl_kernel<<<1, 32, 0, stream>>>((const unsigned long long*)counts, nbins, edges, d, out);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

extern "C" size_t pqc_mw_workspace_size(int64_t batch, int32_t n_qubits) {
  if (batch <= 0 || n_qubits < 1) return 256;
  return align_up((size_t)batch * mw_blocks(n_qubits, batch) * n_qubits * 4 * sizeof(double), 256);
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
  const int nblk = mw_blocks(n_qubits, batch);
  const int64_t half = (1ll << n_qubits) >> 1;
  const int64_t chunk = std::max<int64_t>(1, (half + nblk - 1) / nblk);
  double* partial = (double*)workspace;
  for (int64_t r0 = 0; r0 < batch; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, batch - r0);
    mw_partial<<<dim3(nblk, (unsigned)nr), 256, 0, stream>>>((const double2*)psi + (r0 << n_qubits), n_qubits, chunk,
                                                             partial + r0 * nblk * n_qubits * 4);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  mw_final<<<(unsigned)((batch + 127) / 128), 128, 0, stream>>>(partial, nblk, n_qubits, batch, Q);
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
  if (smem > 48 * 1024)  // opt in to exactly what this launch needs (the kernel also has static scratch)
    PQC_CUDA(cudaFuncSetAttribute(magic_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  double* partial = (double*)workspace;
  for (int64_t r0 = 0; r0 < batch; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, batch - r0);
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

extern "C" int pqc_qfim(const void* state, const void* dpsi, int64_t P, int32_t n_qubits, double* F, void* workspace,
                        size_t workspace_bytes, void* stream_v) {
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
  std::vector<int64_t> h(2 * P);
  for (int64_t p = 0; p < P; ++p) {
    h[p] = 0;
    h[P + p] = p;
  }
  PQC_CUDA(cudaMemcpyAsync(idx, h.data(), 2 * P * sizeof(int64_t), cudaMemcpyHostToDevice, stream));
  int rc = pqc_overlaps(state, dpsi, idx, idx + P, P, n_qubits, v, ows, pqc_overlaps_workspace_size(P, n_qubits),
                        stream);
  if (rc) return rc;
  int nt, nchunk;
  rc = launch_gram((const double2*)dpsi, P, n_qubits, partial, nt, nchunk, stream);
  if (rc) return rc;
  qfim_final<<<(unsigned)((P * P + 255) / 256), 256, 0, stream>>>(partial, nchunk, nt, P, v, F);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  // the pageable index array must outlive its copy
  PQC_CUDA(cudaStreamSynchronize(stream));
  return PQC_OK;
}
