// The plain path: one FP64 kernel launch per op, straight from the program
// order -- the per-gate structure of pyramaterised/circuit.py:123-124
// (`for g in self.gates: circuit_state = g * circuit_state`), minus the
// operator rebuild.  It is the comparison point for the fused sweeps and the
// engine of the adjoint gradient (which needs U^dagger of every op).
#include <algorithm>
#include <vector>

#include "engine.cuh"
#include "reduce.cuh"

namespace pqc {

__device__ __forceinline__ int64_t pins0(int64_t t, int j) {
  return ((t >> j) << (j + 1)) | (t & ((1ll << j) - 1));
}
__device__ __forceinline__ int64_t pins00(int64_t t, int ja, int jb) {
  int lo = ja < jb ? ja : jb, hi = ja < jb ? jb : ja;
  return pins0(pins0(t, lo), hi);
}
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zneg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
// c*x - i*s*y
__device__ __forceinline__ double2 zrx(double c, double2 x, double s, double2 y) {
  return make_double2(c * x.x + s * y.y, c * x.y - s * y.x);
}

// One op on every row of psi.  `inv` applies U^dagger.  Work item t indexes
// pairs / quads / elements depending on the kind; blockIdx.y is the row.
__global__ void plain_op_kernel(DOp op, double2* __restrict__ psi, int n_qubits, int64_t row0,
                                const double* __restrict__ rowcoef, int n_slots, const double* __restrict__ consts,
                                int inv, int64_t n_items, const int32_t* __restrict__ row_limit) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n_items) return;
  const int64_t row = row0 + blockIdx.y;
  if (op.sel >= 0 && op.sel != row) return;
  if (row_limit && op.gidx >= row_limit[row]) return;
  double2* x = psi + (row << n_qubits);
  const double* cf = op.slot >= 0 ? rowcoef + ((size_t)row * n_slots + op.slot) * 4 : consts + (-op.slot - 1);
  const int j0 = op.p0, j1 = op.p1;
  switch (op.kind) {
    case K_RY:
    case K_REAL2: {
      double a, b, c, d;
      if (op.kind == K_RY) {
        a = cf[0];
        b = -cf[1];
        c = cf[1];
        d = cf[0];
      } else {
        a = cf[0];
        b = cf[1];
        c = cf[2];
        d = cf[3];
      }
      if (inv) {  // real orthogonal: inverse = transpose
        double tmp = b;
        b = c;
        c = tmp;
      }
      int64_t i0 = pins0(t, j0), i1 = i0 | (1ll << j0);
      double2 u = x[i0], v = x[i1];
      x[i0] = make_double2(a * u.x + b * v.x, a * u.y + b * v.y);
      x[i1] = make_double2(c * u.x + d * v.x, c * u.y + d * v.y);
      break;
    }
    case K_RX: {
      double c = cf[0], s = inv ? -cf[1] : cf[1];
      int64_t i0 = pins0(t, j0), i1 = i0 | (1ll << j0);
      double2 u = x[i0], v = x[i1];
      x[i0] = zrx(c, u, s, v);
      x[i1] = zrx(c, v, s, u);
      break;
    }
    case K_RZ:
    case K_DIAG1: {
      double2 p0, p1;
      if (op.kind == K_RZ) {
        p0 = make_double2(cf[0], -cf[1]);
        p1 = make_double2(cf[0], cf[1]);
      } else {
        p0 = make_double2(cf[0], cf[1]);
        p1 = make_double2(cf[2], cf[3]);
      }
      if (inv) {
        p0 = zconj(p0);
        p1 = zconj(p1);
      }
      int b = (int)((t >> j0) & 1);
      x[t] = zmul(b ? p1 : p0, x[t]);
      break;
    }
    case K_GEN1: {
      double2 m00 = make_double2(cf[0], cf[1]), m01 = make_double2(cf[2], cf[3]);
      double2 m10 = make_double2(cf[4], cf[5]), m11 = make_double2(cf[6], cf[7]);
      if (inv) {
        double2 t01 = m01;
        m00 = zconj(m00);
        m11 = zconj(m11);
        m01 = zconj(m10);
        m10 = zconj(t01);
      }
      int64_t i0 = pins0(t, j0), i1 = i0 | (1ll << j0);
      double2 u = x[i0], v = x[i1];
      x[i0] = zadd(zmul(m00, u), zmul(m01, v));
      x[i1] = zadd(zmul(m10, u), zmul(m11, v));
      break;
    }
    case K_X: {
      int64_t i0 = pins0(t, j0), i1 = i0 | (1ll << j0);
      double2 u = x[i0];
      x[i0] = x[i1];
      x[i1] = u;
      break;
    }
    case K_CNOT: {
      int64_t i0 = pins00(t, j0, j1) | (1ll << j0), i1 = i0 | (1ll << j1);
      double2 u = x[i0];
      x[i0] = x[i1];
      x[i1] = u;
      break;
    }
    case K_CZ: {
      int64_t i = pins00(t, j0, j1) | (1ll << j0) | (1ll << j1);
      x[i] = zneg(x[i]);
      break;
    }
    case K_RZZ: {
      double c = cf[0], s = inv ? -cf[1] : cf[1];
      int par = (int)(((t >> j0) ^ (t >> j1)) & 1);
      x[t] = zmul(par ? make_double2(c, s) : make_double2(c, -s), x[t]);
      break;
    }
    case K_RXX:
    case K_RYY: {
      double c = cf[0], s = inv ? -cf[1] : cf[1];
      int64_t mm = (1ll << j0) | (1ll << j1);
      int64_t i = pins0(t, j0), p = i ^ mm;
      double sp = (op.kind == K_RXX) ? s : (((i >> j1) & 1) ? s : -s);
      double2 a = x[i], b = x[p];
      x[i] = zrx(c, a, sp, b);
      x[p] = zrx(c, b, sp, a);
      break;
    }
    case K_MIX2: {
      double c = cf[0], s = inv ? -cf[1] : cf[1];
      double2 p11 = make_double2(cf[2], inv ? -cf[3] : cf[3]);
      int64_t i00 = pins00(t, j0, j1);
      int64_t i01 = i00 | (1ll << j1), i10 = i00 | (1ll << j0), i11 = i01 | i10;
      double2 a = x[i01], b = x[i10];
      x[i01] = zrx(c, a, s, b);
      x[i10] = zrx(c, b, s, a);
      x[i11] = zmul(p11, x[i11]);
      break;
    }
    case K_GEN2: {
      int64_t i00 = pins00(t, j0, j1);
      int64_t idx[4] = {i00, i00 | (1ll << j1), i00 | (1ll << j0), i00 | (1ll << j0) | (1ll << j1)};
      double2 v[4] = {x[idx[0]], x[idx[1]], x[idx[2]], x[idx[3]]};
      for (int r = 0; r < 4; ++r) {
        double2 acc = make_double2(0.0, 0.0);
        for (int cc = 0; cc < 4; ++cc) {
          double2 m = inv ? zconj(make_double2(cf[2 * (4 * cc + r)], cf[2 * (4 * cc + r) + 1]))
                          : make_double2(cf[2 * (4 * r + cc)], cf[2 * (4 * r + cc) + 1]);
          acc = zadd(acc, zmul(m, v[cc]));
        }
        x[idx[r]] = acc;
      }
      break;
    }
    case K_PAULI: {
      // generators are never inverted; applied in place as coef * P
      const int l0 = op.aux & 0xff, l1 = (op.aux >> 8) & 0xff;
      double2 w = make_double2(cf[0], cf[1]);
      const int ny = (l0 == 2) + (l1 == 2);
      for (int q = 0; q < ny; ++q) w = make_double2(-w.y, w.x);
      int64_t xm = ((l0 == 1 || l0 == 2) ? (1ll << j0) : 0) | ((l1 == 1 || l1 == 2) ? (1ll << j1) : 0);
      int64_t zm = ((l0 == 2 || l0 == 3) ? (1ll << j0) : 0) | ((l1 == 2 || l1 == 3) ? (1ll << j1) : 0);
      if (xm == 0) {
        double2 v = zmul(w, x[t]);
        x[t] = (__popcll(t & zm) & 1) ? zneg(v) : v;
      } else {
        int lb = __ffsll(xm) - 1;
        int64_t j = pins0(t, lb), p = j ^ xm;
        double2 a = x[j], b = x[p];
        double2 nb = zmul(w, b), na = zmul(w, a);
        x[j] = (__popcll(p & zm) & 1) ? zneg(nb) : nb;
        x[p] = (__popcll(j & zm) & 1) ? zneg(na) : na;
      }
      break;
    }
    default:
      break;
  }
}

static int64_t plain_items(const DOp& op, int n_qubits) {
  const int64_t D = 1ll << n_qubits;
  switch (op.kind) {
    case K_RZ:
    case K_DIAG1:
    case K_RZZ:
      return D;
    case K_CNOT:
    case K_CZ:
    case K_MIX2:
    case K_GEN2:
      return D >> 2;
    case K_PAULI: {
      const int l0 = op.aux & 0xff, l1 = (op.aux >> 8) & 0xff;
      bool mv = (l0 == 1 || l0 == 2) || (l1 == 1 || l1 == 2);
      return mv ? D >> 1 : D;
    }
    default:
      return D >> 1;
  }
}

int launch_plain_op(const DOp& op, double2* psi, int n_qubits, int64_t rows, const double* rowcoef, int n_slots,
                    const double* consts, int inv, cudaStream_t stream, const int32_t* row_limit) {
  const int64_t items = plain_items(op, n_qubits);
  const int threads = 256;
  const int64_t bx = (items + threads - 1) / threads;
  for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, rows - r0);
    dim3 grid((unsigned)bx, (unsigned)nr);
    plain_op_kernel<<<grid, threads, 0, stream>>>(op, psi, n_qubits, r0, rowcoef, n_slots, consts, inv, items,
                                                  row_limit);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  return PQC_OK;
}

// psi[b] <- psi0 (or the basis state) for every row
__global__ void init_rows_kernel(double2* __restrict__ psi, const double2* __restrict__ psi0, int64_t idx,
                                 int n_qubits, int64_t rows) {
  const int64_t D = 1ll << n_qubits;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= D * rows) return;
  int64_t g = i & (D - 1);
  psi[i] = psi0 ? psi0[g] : make_double2(g == idx ? 1.0 : 0.0, 0.0);
}

int init_rows(double2* psi, const void* psi0, int64_t idx, int n_qubits, int64_t rows, cudaStream_t stream) {
  const int64_t n = rows << n_qubits;
  init_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(psi, (const double2*)psi0, idx, n_qubits, rows);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

// ---------------------------------------------------------------- adjoint
// out[b][j] = sum_t coef_t i^{ny_t} (-1)^{popc((j ^ x_t) & z_t)} psi[b][j ^ x_t]   (H|psi>)
__global__ void pauli_sum_apply(const double2* __restrict__ psi, double2* __restrict__ out,
                                const pqc_pauli_term* __restrict__ terms, int n_terms, int n_qubits) {
  const int64_t D = 1ll << n_qubits;
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= D) return;
  const int64_t row = blockIdx.y;
  const double2* x = psi + row * D;
  double ar = 0.0, ai = 0.0;
  for (int t = 0; t < n_terms; ++t) {
    const pqc_pauli_term T = terms[t];
    const int64_t src = j ^ (int64_t)T.xmask;
    double2 v = x[src];
    double sgn = (__popcll((uint64_t)src & T.zmask) & 1) ? -T.coef : T.coef;
    // multiply by i^{n_y}
    double vr = v.x, vi = v.y;
    for (int q = 0; q < (T.n_y & 3); ++q) {
      double tmp = vr;
      vr = -vi;
      vi = tmp;
    }
    ar += sgn * vr;
    ai += sgn * vi;
  }
  out[row * D + j] = make_double2(ar, ai);
}

// partial[row][blk] = sum over this block's chunk of conj(a) * b  (complex)
__global__ void row_dot_partial(const double2* __restrict__ a, const double2* __restrict__ b, int n_qubits,
                                int64_t chunk, double2* __restrict__ partial) {
  __shared__ double scratch[32];
  const int64_t D = 1ll << n_qubits;
  const int64_t row = blockIdx.y;
  const int64_t s0 = blockIdx.x * chunk;
  const int64_t s1 = min(D, s0 + chunk);
  const double2* x = a + row * D;
  const double2* y = b + row * D;
  double re = 0.0, im = 0.0;
  for (int64_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
    double2 u = x[i], v = y[i];
    re += u.x * v.x + u.y * v.y;
    im += u.x * v.y - u.y * v.x;
  }
  re = block_sum(re, scratch);
  im = block_sum(im, scratch);
  if (threadIdx.x == 0) partial[row * gridDim.x + blockIdx.x] = make_double2(re, im);
}

// mode 0: out[row] = Re(sum);  mode 1: out[row * stride + col] += scale * Re(sum)
__global__ void row_dot_finalize(const double2* __restrict__ partial, int nblk, int64_t rows, double* __restrict__ out,
                                 int mode, int64_t stride, int col, double scale) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= rows) return;
  double s = 0.0;
  for (int k = 0; k < nblk; ++k) s += partial[row * nblk + k].x;
  if (mode == 0)
    out[row] = s;
  else
    out[row * stride + col] += scale * s;
}

static int row_dot(const double2* a, const double2* b, int n_qubits, int64_t rows, double2* partial, int nblk,
                   double* out, int mode, int64_t stride, int col, double scale, cudaStream_t stream) {
  const int64_t D = 1ll << n_qubits;
  const int64_t chunk = (D + nblk - 1) / nblk;
  for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, rows - r0);
    row_dot_partial<<<dim3(nblk, (unsigned)nr), 256, 0, stream>>>(a + r0 * D, b + r0 * D, n_qubits, chunk,
                                                                   partial + r0 * nblk);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  row_dot_finalize<<<(unsigned)((rows + 127) / 128), 128, 0, stream>>>(partial, nblk, rows, out, mode, stride, col,
                                                                       scale);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

static int dot_blocks(int n_qubits) {
  const int64_t D = 1ll << n_qubits;
  int64_t b = D / 4096;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 256));
}

static size_t grad_ws(const pqc_program* p, int64_t rows, int n_gen_slots) {
  const size_t D = (size_t)1 << p->n_qubits;
  size_t ws = align_up(rows * p->fwd_t.specs.size() * 4 * sizeof(double), 256);
  ws += align_up(rows * (size_t)std::max(n_gen_slots, 1) * 4 * sizeof(double), 256);
  ws += 3 * align_up(rows * D * 16, 256);
  ws += align_up(rows * (size_t)dot_blocks(p->n_qubits) * 16, 256);
  return ws;
}

}  // namespace pqc

using namespace pqc;

extern "C" int pqc_run_plain(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                             const void* psi0, int64_t psi0_index, void* psi, void* workspace, size_t workspace_bytes,
                             void* stream_v) {
  if (!prog) return fail(PQC_ERR_INVALID, "program is NULL");
  if (batch <= 0) return batch == 0 ? PQC_OK : fail(PQC_ERR_INVALID, "batch < 0");
  if (!psi) return fail(PQC_ERR_INVALID, "psi is NULL");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  const size_t need = align_up(batch * prog->fwd_t.specs.size() * 4 * sizeof(double), 256);
  if (need && (!workspace || workspace_bytes < need))
    return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  cudaStream_t stream = (cudaStream_t)stream_v;
  double* coef = (double*)workspace;
  int rc = launch_row_coefs(prog->fwd_t, theta, theta_stride, batch, coef, stream);
  if (!rc) rc = init_rows((double2*)psi, psi0, psi0_index, prog->n_qubits, batch, stream);
  for (size_t i = 0; !rc && i < prog->fwd_t.dops.size(); ++i)
    rc = launch_plain_op(prog->fwd_t.dops[i], (double2*)psi, prog->n_qubits, batch, coef,
                         (int)prog->fwd_t.specs.size(), prog->fwd_t.d_consts, 0, stream);
  return rc;
}

// workspace of the fused adjoint: [coef f64 | coef df | consts df | psi | lambda | dot partials | measure partials]
static size_t fused_grad_ws(const pqc_program* p, int64_t rows, int n_gens) {
  const size_t D = (size_t)1 << p->n_qubits;
  const size_t slots = p->fwd_t.specs.size();
  const size_t n_consts = std::max<size_t>(p->fwd_t.consts.size(), p->adj_valid ? p->adj_t.consts.size() : 0);
  // the inverse program has the forward's constants plus 4 per generator
  const size_t consts_bound = std::max(n_consts, p->fwd_t.consts.size() + 4 * (size_t)n_gens) + 4;
  const int k = std::min(kAdjTileQubits, (int)p->n_qubits);
  const size_t tiles = (size_t)1 << (p->n_qubits - k);
  size_t ws = align_up(rows * slots * 4 * sizeof(double), 256);
  ws += align_up(rows * slots * 4 * sizeof(float2), 256);
  ws += align_up(consts_bound * sizeof(float2), 256);
  ws += 2 * align_up(rows * D * 16, 256);
  ws += align_up(rows * (size_t)dot_blocks(p->n_qubits) * 16, 256);
  ws += align_up(rows * (size_t)std::max(n_gens, 1) * tiles * sizeof(double), 256);
  return ws;
}

static bool all_pauli(const pqc_op* gens, int n) {
  for (int t = 0; t < n; ++t)
    if (gens[t].kind != PQC_OP_PAULI) return false;
  return true;
}

extern "C" size_t pqc_energy_grad_workspace_size(const pqc_program* prog, int64_t batch, int32_t n_gens,
                                                 int32_t n_cols) {
  if (!prog || batch < 0 || n_gens < 0) return 0;
  (void)n_cols;
  return std::max(grad_ws(prog, batch, n_gens), fused_grad_ws(prog, batch, n_gens));
}

// FP64 adjoint, one kernel per op: used for generators that are not Pauli terms.
static int energy_grad_plain(pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                             const void* psi0, int64_t psi0_index, const pqc_pauli_term* terms, int32_t n_terms,
                             const pqc_op* gens, const int32_t* gen_after, int32_t n_gens, int32_t n_cols, double* E,
                             double* grad, void* workspace, size_t workspace_bytes, cudaStream_t stream) {
  const int64_t D = 1ll << prog->n_qubits;
  int rc = ensure_deriv(prog, gens, gen_after, n_gens);
  if (rc) return rc;
  const int n_gslots = (int)prog->gen_t.specs.size();
  const size_t need = grad_ws(prog, batch, n_gslots);
  if (!workspace || workspace_bytes < need)
    return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  const int N = prog->n_qubits;
  char* w = (char*)workspace;
  double* coef = (double*)w;
  w += align_up(batch * prog->fwd_t.specs.size() * 4 * sizeof(double), 256);
  double* gcoef = (double*)w;
  w += align_up(batch * (size_t)std::max(n_gslots, 1) * 4 * sizeof(double), 256);
  double2* psi = (double2*)w;
  w += align_up(batch * D * 16, 256);
  double2* lam = (double2*)w;
  w += align_up(batch * D * 16, 256);
  double2* tmp = (double2*)w;
  w += align_up(batch * D * 16, 256);
  double2* partial = (double2*)w;
  const int nblk = dot_blocks(N);
  rc = launch_row_coefs(prog->fwd_t, theta, theta_stride, batch, coef, stream);
  if (!rc) rc = launch_row_coefs(prog->gen_t, theta, theta_stride, batch, gcoef, stream);
  if (rc) return rc;
  // forward: psi = U psi0
  rc = init_rows(psi, psi0, psi0_index, N, batch, stream);
  const int n_slots = (int)prog->fwd_t.specs.size();
  const std::vector<DOp>& ops = prog->fwd_t.dops;
  for (size_t i = 0; !rc && i < ops.size(); ++i)
    rc = launch_plain_op(ops[i], psi, N, batch, coef, n_slots, prog->fwd_t.d_consts, 0, stream);
  if (rc) return rc;
  // lambda = H psi ; E = <psi|lambda>
  for (int64_t r0 = 0; r0 < batch; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, batch - r0);
    pauli_sum_apply<<<dim3((unsigned)((D + 255) / 256), (unsigned)nr), 256, 0, stream>>>(psi + r0 * D, lam + r0 * D,
                                                                                      terms, n_terms, N);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  if (E) {
    rc = row_dot(psi, lam, N, batch, partial, nblk, E, 0, 0, 0, 1.0, stream);
    if (rc) return rc;
  }
  if (n_cols > 0) PQC_CUDA(cudaMemsetAsync(grad, 0, batch * n_cols * sizeof(double), stream));
  // generators grouped by insertion point
  std::vector<std::vector<int>> at(ops.size() + 1);
  for (int t = 0; t < n_gens; ++t) at[gen_after[t] + 1].push_back(t);
  for (int64_t i = (int64_t)ops.size() - 1; i >= -1; --i) {
    for (int t : at[i + 1]) {
      // tmp = G_t psi ; grad[:, sel] += 2 Re <lambda|tmp>
      PQC_CUDA(cudaMemcpyAsync(tmp, psi, batch * D * 16, cudaMemcpyDeviceToDevice, stream));
      DOp g = prog->gen_t.dops[t];
      const int col = g.sel;
      g.sel = -1;
      rc = launch_plain_op(g, tmp, N, batch, gcoef, n_gslots, prog->gen_t.d_consts, 0, stream);
      if (!rc) rc = row_dot(lam, tmp, N, batch, partial, nblk, grad, 1, n_cols, col, 2.0, stream);
      if (rc) return rc;
    }
    if (i >= 0) {
      rc = launch_plain_op(ops[i], psi, N, batch, coef, n_slots, prog->fwd_t.d_consts, 1, stream);
      if (!rc) rc = launch_plain_op(ops[i], lam, N, batch, coef, n_slots, prog->fwd_t.d_consts, 1, stream);
      if (rc) return rc;
    }
  }
  return PQC_OK;
}

// Fused double-float adjoint: forward sweeps, lambda = H psi, then the reverse
// sweeps over psi and lambda with the generator measures (adjoint.cu).
static int energy_grad_fused(pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                             const void* psi0, int64_t psi0_index, const pqc_pauli_term* terms, int32_t n_terms,
                             const pqc_op* gens, const int32_t* gen_after, int32_t n_gens, int32_t n_cols, double* E,
                             double* grad, const int32_t* row_limit, void* workspace, size_t workspace_bytes,
                             cudaStream_t stream) {
  int rc = ensure_adjoint(prog, gens, gen_after, n_gens, n_cols);
  if (rc) return rc;
  const size_t need = fused_grad_ws(prog, batch, n_gens);
  if (!workspace || workspace_bytes < need)
    return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  const int N = prog->n_qubits;
  const size_t D = (size_t)1 << N;
  const size_t slots = prog->fwd_t.specs.size();
  if (prog->adj_t.specs.size() != slots) return fail(PQC_ERR_INVALID, "adjoint coefficient slots differ from the forward program");
  const size_t consts_bound =
      std::max(std::max(prog->fwd_t.consts.size(), prog->adj_t.consts.size()),
               prog->fwd_t.consts.size() + 4 * (size_t)n_gens) + 4;
  const int64_t tiles = adjoint_tiles(prog);
  char* w = (char*)workspace;
  double* coef64 = (double*)w;
  w += align_up(batch * slots * 4 * sizeof(double), 256);
  float2* coefdf = (float2*)w;
  w += align_up(batch * slots * 4 * sizeof(float2), 256);
  float2* constdf = (float2*)w;
  w += align_up(consts_bound * sizeof(float2), 256);
  double2* psi = (double2*)w;
  w += align_up(batch * D * 16, 256);
  double2* lam = (double2*)w;
  w += align_up(batch * D * 16, 256);
  double2* partial = (double2*)w;
  w += align_up(batch * (size_t)dot_blocks(N) * 16, 256);
  double* mpart = (double*)w;
  // forward
  rc = launch_row_coefs(prog->fwd_t, theta, theta_stride, batch, coef64, stream);
  if (!rc) rc = launch_to_df(coef64, coefdf, batch * (int64_t)slots * 4, stream);
  if (!rc) rc = launch_to_df(prog->fwd_t.d_consts, constdf, (int64_t)prog->fwd_t.consts.size(), stream);
  if (!rc)
    rc = run_plan_df(prog, prog->fwd, (int)slots, coefdf, constdf, batch, psi0, psi0_index, psi, stream, row_limit);
  if (rc) return rc;
  // lambda = H psi ; E = <psi|lambda>
  for (int64_t r0 = 0; r0 < batch; r0 += 65535) {
    const int64_t nr = std::min<int64_t>(65535, batch - r0);
    pauli_sum_apply<<<dim3((unsigned)((D + 255) / 256), (unsigned)nr), 256, 0, stream>>>(psi + r0 * D, lam + r0 * D,
                                                                                      terms, n_terms, N);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  if (E) {
    rc = row_dot(psi, lam, N, batch, partial, dot_blocks(N), E, 0, 0, 0, 1.0, stream);
    if (rc) return rc;
  }
  if (n_cols == 0 || n_gens == 0) {
    if (n_cols > 0) PQC_CUDA(cudaMemsetAsync(grad, 0, batch * n_cols * sizeof(double), stream));
    return PQC_OK;
  }
  // reverse pass
  rc = launch_row_coefs(prog->adj_t, theta, theta_stride, batch, coef64, stream);
  if (!rc) rc = launch_to_df(coef64, coefdf, batch * (int64_t)slots * 4, stream);
  if (!rc) rc = launch_to_df(prog->adj_t.d_consts, constdf, (int64_t)prog->adj_t.consts.size(), stream);
  if (rc) return rc;
  PQC_CUDA(cudaMemsetAsync(mpart, 0, batch * (size_t)n_gens * tiles * sizeof(double), stream));
  rc = run_adjoint_sweeps(prog, coefdf, constdf, batch, psi, lam, row_limit, mpart, stream);
  if (!rc) rc = launch_adj_final(prog, mpart, batch, grad, stream);
  return rc;
}

extern "C" int pqc_energy_grad(const pqc_program* prog_c, const double* theta, int64_t theta_stride, int64_t batch,
                               const void* psi0, int64_t psi0_index, const pqc_pauli_term* terms, int32_t n_terms,
                               const pqc_op* gens, const int32_t* gen_after, int32_t n_gens, int32_t n_cols,
                               double* E, double* grad, const int32_t* row_limit, void* workspace,
                               size_t workspace_bytes, void* stream_v) {
  pqc_program* prog = const_cast<pqc_program*>(prog_c);
  if (!prog) return fail(PQC_ERR_INVALID, "program is NULL");
  if (batch <= 0) return batch == 0 ? PQC_OK : fail(PQC_ERR_INVALID, "batch < 0");
  if (n_terms < 0 || (n_terms > 0 && !terms)) return fail(PQC_ERR_INVALID, "bad Hamiltonian terms");
  if (n_gens < 0 || (n_gens > 0 && (!gens || !gen_after))) return fail(PQC_ERR_INVALID, "bad generator list");
  if (n_cols < 0 || (n_cols > 0 && !grad)) return fail(PQC_ERR_INVALID, "bad gradient output");
  for (int t = 0; t < n_gens; ++t) {
    if (gens[t].sel < 0 || gens[t].sel >= n_cols) return fail(PQC_ERR_INVALID, "gens[t].sel outside [0, n_cols)");
    if (gen_after[t] < -1 || gen_after[t] >= (int)prog->ops.size())
      return fail(PQC_ERR_INVALID, "gen_after[t] outside [-1, n_ops)");
  }
  if (theta_stride < 0 || (theta_stride > 0 && theta_stride < prog->n_params))
    return fail(PQC_ERR_INVALID, "theta_stride < n_params");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  cudaStream_t stream = (cudaStream_t)stream_v;
  if (all_pauli(gens, n_gens))
    return energy_grad_fused(prog, theta, theta_stride, batch, psi0, psi0_index, terms, n_terms, gens, gen_after,
                             n_gens, n_cols, E, grad, row_limit, workspace, workspace_bytes, stream);
  if (row_limit) return fail(PQC_ERR_UNSUPPORTED, "row_limit needs Pauli-term generators");
  return energy_grad_plain(prog, theta, theta_stride, batch, psi0, psi0_index, terms, n_terms, gens, gen_after,
                           n_gens, n_cols, E, grad, workspace, workspace_bytes, stream);
}

// ------------------------------------------------------------ plain baselines
// The one-kernel-per-op FP64 paths, exposed for comparison (serving, benchmarks)
// and as an independent cross-check of the fused sweeps.

extern "C" int pqc_energy_grad_plain(const pqc_program* prog_c, const double* theta, int64_t theta_stride,
                                     int64_t batch, const void* psi0, int64_t psi0_index,
                                     const pqc_pauli_term* terms, int32_t n_terms, const pqc_op* gens,
                                     const int32_t* gen_after, int32_t n_gens, int32_t n_cols, double* E,
                                     double* grad, void* workspace, size_t workspace_bytes, void* stream_v) {
  pqc_program* prog = const_cast<pqc_program*>(prog_c);
  if (!prog) return fail(PQC_ERR_INVALID, "program is NULL");
  if (batch <= 0) return batch == 0 ? PQC_OK : fail(PQC_ERR_INVALID, "batch < 0");
  if (n_terms < 0 || (n_terms > 0 && !terms)) return fail(PQC_ERR_INVALID, "bad Hamiltonian terms");
  if (n_gens < 0 || (n_gens > 0 && (!gens || !gen_after))) return fail(PQC_ERR_INVALID, "bad generator list");
  if (n_cols < 0 || (n_cols > 0 && !grad)) return fail(PQC_ERR_INVALID, "bad gradient output");
  for (int t = 0; t < n_gens; ++t) {
    if (gens[t].sel < 0 || gens[t].sel >= n_cols) return fail(PQC_ERR_INVALID, "gens[t].sel outside [0, n_cols)");
    if (gen_after[t] < -1 || gen_after[t] >= (int)prog->ops.size())
      return fail(PQC_ERR_INVALID, "gen_after[t] outside [-1, n_ops)");
  }
  if (theta_stride < 0 || (theta_stride > 0 && theta_stride < prog->n_params))
    return fail(PQC_ERR_INVALID, "theta_stride < n_params");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  return energy_grad_plain(prog, theta, theta_stride, batch, psi0, psi0_index, terms, n_terms, gens, gen_after,
                           n_gens, n_cols, E, grad, workspace, workspace_bytes, (cudaStream_t)stream_v);
}

extern "C" size_t pqc_derivative_states_plain_workspace_size(const pqc_program* prog, int32_t n_runs) {
  if (!prog || n_runs < 0) return 0;
  const size_t slots = prog->fwd_t.specs.size() + (size_t)n_runs;
  return align_up(std::max<size_t>(1, (size_t)n_runs) * slots * 4 * sizeof(double), 256);
}

extern "C" int pqc_derivative_states_plain(const pqc_program* prog_c, const double* theta, const void* psi0,
                                           int64_t psi0_index, const pqc_op* gens, const int32_t* gen_after,
                                           int32_t n_runs, void* dpsi, void* workspace, size_t workspace_bytes,
                                           void* stream_v) {
  pqc_program* prog = const_cast<pqc_program*>(prog_c);
  if (!prog) return fail(PQC_ERR_INVALID, "program is NULL");
  if (n_runs < 0) return fail(PQC_ERR_INVALID, "negative count");
  if (n_runs == 0) return PQC_OK;
  if (!gens || !gen_after || !dpsi) return fail(PQC_ERR_INVALID, "NULL argument");
  for (int r = 0; r < n_runs; ++r)
    if (gens[r].sel != r) return fail(PQC_ERR_UNSUPPORTED, "plain derivative states need gens[r].sel == r");
  const int64_t D = 1ll << prog->n_qubits;
  if (!psi0 && (psi0_index < 0 || psi0_index >= D)) return fail(PQC_ERR_INVALID, "psi0_index out of range");
  int rc = ensure_deriv(prog, gens, gen_after, n_runs);
  if (rc) return rc;
  const size_t slots = prog->deriv_t.specs.size();
  const size_t need = align_up((size_t)n_runs * std::max<size_t>(slots, 1) * 4 * sizeof(double), 256);
  if (slots && (!workspace || workspace_bytes < need))
    return fail(PQC_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need));
  cudaStream_t stream = (cudaStream_t)stream_v;
  double* coef = (double*)workspace;
  rc = launch_row_coefs(prog->deriv_t, theta, 0, n_runs, coef, stream);  // stride 0: every run shares theta
  if (!rc) rc = init_rows((double2*)dpsi, psi0, psi0_index, prog->n_qubits, n_runs, stream);
  if (rc) return rc;
  // program order with each generator right after its op; a generator's sel limits it to its own run
  const int n_fwd = (int)prog->ops.size();
  std::vector<std::vector<int>> at(n_fwd + 1);
  for (int r = 0; r < n_runs; ++r) at[gen_after[r] + 1].push_back(r);
  const std::vector<DOp>& ops = prog->deriv_t.dops;
  for (int i = -1; !rc && i < n_fwd; ++i) {
    if (i >= 0)
      rc = launch_plain_op(ops[i], (double2*)dpsi, prog->n_qubits, n_runs, coef, (int)slots, prog->deriv_t.d_consts,
                           0, stream);
    for (size_t q = 0; !rc && q < at[i + 1].size(); ++q)
      rc = launch_plain_op(ops[n_fwd + at[i + 1][q]], (double2*)dpsi, prog->n_qubits, n_runs, coef, (int)slots,
                           prog->deriv_t.d_consts, 0, stream);
  }
  return rc;
}
