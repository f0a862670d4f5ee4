// Program creation: classification of ops, the sweep planner, the
// per-row coefficient kernel and the error plumbing of the C ABI.
//
// Replaces the reference's per-gate operator construction: every
// `set_theta` in pyramaterised/gates.py:129-131 rebuilds a full 2^N x 2^N
// QuTiP operator; here a gate is lowered once to a small op record whose
// 2x2/4x4 coefficients are computed per parameter row on the device.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <set>
#include <unordered_map>

#include "engine.cuh"

namespace pqc {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return PQC_ERR_CUDA;
}

// ---------------------------------------------------------------- coefficients
// (c, s, x, y) for a parameterised op, shared by host (fixed angles) and device.
__host__ __device__ inline void op_coefs(int kind, double a, double a2, double out[4]) {
  switch (kind) {
    case PQC_OP_RX:
    case PQC_OP_RY: {
      // (cos, sin, tan, 0) of a/2: the sweeps' scaled rotations apply cos * [[1, -tan], [tan, 1]]
      const double c = cos(a / 2), s = sin(a / 2);
      out[0] = c;
      out[1] = s;
      out[2] = c != 0.0 ? s / c : 0.0;
      out[3] = 0.0;
      break;
    }
    case PQC_OP_RZ:
    case PQC_OP_RXX:
    case PQC_OP_RYY:
    case PQC_OP_RZZ:
      out[0] = cos(a / 2);
      out[1] = sin(a / 2);
      out[2] = 0.0;
      out[3] = 0.0;
      break;
    case PQC_OP_FSIM:  // gates.py:598-606
      out[0] = cos(a);
      out[1] = sin(a);
      out[2] = cos(a2);
      out[3] = -sin(a2);
      break;
    case PQC_OP_FIXED_FSIM:  // gates.py:708-716
      out[0] = cos(a);
      out[1] = sin(a);
      out[2] = 1.0;
      out[3] = 0.0;
      break;
    case PQC_OP_FSIM_DTHETA:  // gates.py:619-627: middle block [[-s,-ic],[-ic,-s]]
      out[0] = -sin(a);
      out[1] = cos(a);
      out[2] = cos(a2);
      out[3] = -sin(a2);
      break;
    case PQC_OP_FSIM_DPHI:  // gates.py:640-648: |11> gets -i e^{-i phi}
      out[0] = cos(a);
      out[1] = sin(a);
      out[2] = -sin(a2);
      out[3] = -cos(a2);
      break;
    case PQC_OP_FIXED_FSIM_DTHETA:  // gates.py:729-737
      out[0] = -sin(a);
      out[1] = cos(a);
      out[2] = 1.0;
      out[3] = 0.0;
      break;
    default:
      out[0] = out[1] = out[2] = out[3] = 0.0;
  }
}

__global__ void row_coef_kernel(const RowCoefSpec* __restrict__ specs, int n_slots, const double* __restrict__ theta,
                                int64_t theta_stride, int64_t rows, double* __restrict__ coef) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t n = rows * n_slots;
  if (i >= n) return;
  int64_t row = i / n_slots;
  int slot = (int)(i - row * n_slots);
  RowCoefSpec s = specs[slot];
  const double* th = theta + row * theta_stride;
  double a = s.param >= 0 ? s.scale * th[s.param] + s.offset : s.offset;
  double a2 = s.param2 >= 0 ? s.scale2 * th[s.param2] + s.offset2 : s.offset2;
  double out[4];
  op_coefs(s.kind, a, a2, out);
  double2* o = reinterpret_cast<double2*>(coef) + 2 * i;
  o[0] = make_double2(out[0], out[1]);
  o[1] = make_double2(out[2], out[3]);
}

int launch_row_coefs(const OpTable& t, const double* theta, int64_t theta_stride, int64_t rows, double* coef,
                     cudaStream_t stream) {
  int n_slots = (int)t.specs.size();
  if (n_slots == 0 || rows == 0) return PQC_OK;
  if (!theta) return fail(PQC_ERR_INVALID, "theta is NULL but the program has parameterised ops");
  int64_t n = rows * n_slots;
  int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  row_coef_kernel<<<(unsigned)blocks, threads, 0, stream>>>(t.d_specs, n_slots, theta, theta_stride, rows, coef);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

// Multi-program coefficient launches: the jobs' records travel as kernel parameters; a thread finds its job
// from the running totals `end` (job j covers items [end[j-1], end[j]) of the launch).
struct CoefLaunch {
  int n;
  int64_t end[kMultiMax];
  CoefJob job[kMultiMax];
};

__device__ __forceinline__ int find_job(const CoefLaunch& L, int64_t i) {
  int lo = 0, hi = L.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (i < L.end[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

__global__ void row_coef_multi_kernel(const __grid_constant__ CoefLaunch L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L.end[L.n - 1]) return;
  const int j = find_job(L, i);
  const CoefJob& b = L.job[j];
  const int64_t k = i - (j ? L.end[j - 1] : 0);
  const int64_t row = k / b.n_slots;
  const int slot = (int)(k - row * b.n_slots);
  const RowCoefSpec s = b.specs[slot];
  const double* th = b.theta + row * b.theta_stride;
  const double a = s.param >= 0 ? s.scale * th[s.param] + s.offset : s.offset;
  const double a2 = s.param2 >= 0 ? s.scale2 * th[s.param2] + s.offset2 : s.offset2;
  double out[4];
  op_coefs(s.kind, a, a2, out);
  double2* o = reinterpret_cast<double2*>(b.coef) + 2 * k;
  o[0] = make_double2(out[0], out[1]);
  o[1] = make_double2(out[2], out[3]);
}

// job j converts its 4 rows x n_slots coefficients, then its n_consts constants
__global__ void to_df_multi_kernel(const __grid_constant__ CoefLaunch L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L.end[L.n - 1]) return;
  const int j = find_job(L, i);
  const CoefJob& b = L.job[j];
  const int64_t k = i - (j ? L.end[j - 1] : 0);
  const int64_t nc = 4 * b.rows * b.n_slots;
  const double v = k < nc ? b.coef[k] : b.consts[k - nc];
  const float h = __double2float_rn(v);
  const float l = __double2float_rn(v - (double)h);
  (k < nc ? b.coef_df[k] : b.consts_df[k - nc]) = make_float2(h, l);
}

int launch_coefs_multi(const CoefJob* jobs, int n_jobs, cudaStream_t stream) {
  for (int j0 = 0; j0 < n_jobs; j0 += kMultiMax) {
    CoefLaunch a, b;
    a.n = b.n = std::min(kMultiMax, n_jobs - j0);
    int64_t na = 0, nb = 0;
    for (int j = 0; j < a.n; ++j) {
      const CoefJob& c = jobs[j0 + j];
      if (c.n_slots > 0 && c.rows > 0 && !c.theta)
        return fail(PQC_ERR_INVALID, "theta is NULL but a program has parameterised ops");
      a.job[j] = b.job[j] = c;
      na += c.rows * c.n_slots;
      nb += 4 * c.rows * c.n_slots + c.n_consts;
      a.end[j] = na;
      b.end[j] = nb;
    }
    if (na > 0) {
      row_coef_multi_kernel<<<(unsigned)((na + 255) / 256), 256, 0, stream>>>(a);
      count_launch();
      PQC_CUDA(cudaGetLastError());
    }
    if (nb > 0) {
      to_df_multi_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, stream>>>(b);
      count_launch();
      PQC_CUDA(cudaGetLastError());
    }
  }
  return PQC_OK;
}

// doubles -> double-float (hi, lo) pairs
__global__ void to_df_kernel(const double* __restrict__ in, float2* __restrict__ out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = in[i];
  float h = __double2float_rn(v);
  float l = __double2float_rn(v - (double)h);
  out[i] = make_float2(h, l);
}

int launch_to_df(const double* in, float2* out, int64_t n, cudaStream_t stream) {
  if (n <= 0) return PQC_OK;
  to_df_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(in, out, n);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

// ---------------------------------------------------------------- lowering
static bool is_param_kind(int k) {
  return k == PQC_OP_RX || k == PQC_OP_RY || k == PQC_OP_RZ || k == PQC_OP_RXX || k == PQC_OP_RYY ||
         k == PQC_OP_RZZ || k == PQC_OP_FSIM || k == PQC_OP_FIXED_FSIM || k == PQC_OP_FSIM_DTHETA ||
         k == PQC_OP_FSIM_DPHI || k == PQC_OP_FIXED_FSIM_DTHETA;
}

int lower_ops(const pqc_op* ops, int n_ops, int n_qubits, OpTable& t) {
  std::vector<DOp>& dops = t.dops;
  std::vector<RowCoefSpec>& row_specs = t.specs;
  std::vector<double>& consts = t.consts;
  dops.clear();
  row_specs.clear();
  consts.clear();
  auto pos = [&](int q) { return n_qubits - 1 - q; };
  for (int i = 0; i < n_ops; ++i) {
    const pqc_op& o = ops[i];
    bool two = o.kind == PQC_OP_CNOT || o.kind == PQC_OP_CZ || o.kind == PQC_OP_RXX || o.kind == PQC_OP_RYY ||
               o.kind == PQC_OP_RZZ || o.kind == PQC_OP_MAT2 || o.kind == PQC_OP_FSIM || o.kind == PQC_OP_FIXED_FSIM ||
               o.kind == PQC_OP_FSIM_DTHETA || o.kind == PQC_OP_FSIM_DPHI || o.kind == PQC_OP_FIXED_FSIM_DTHETA;
    if (o.q0 < 0 || o.q0 >= n_qubits)
      return fail(PQC_ERR_INVALID, "op " + std::to_string(i) + ": qubit q0 out of range");
    if (two || (o.kind == PQC_OP_PAULI && o.q1 >= 0)) {
      if (o.q1 < 0 || o.q1 >= n_qubits || o.q1 == o.q0)
        return fail(PQC_ERR_INVALID, "op " + std::to_string(i) + ": second qubit invalid");
    }
    DOp d;
    d.sel = o.sel;
    d.p0 = pos(o.q0);
    d.p1 = (two || (o.kind == PQC_OP_PAULI && o.q1 >= 0)) ? pos(o.q1) : -1;
    d.aux = 0;
    d.slot = 0;
    d.gidx = i;
    if (is_param_kind(o.kind)) {
      if (o.param >= 0 || o.param2 >= 0) {
        RowCoefSpec s;
        s.kind = o.kind;
        s.param = o.param;
        s.param2 = o.param2;
        s.pad = 0;
        s.scale = o.scale;
        s.offset = o.offset;
        s.scale2 = o.scale2;
        s.offset2 = o.offset2;
        d.slot = (int)row_specs.size();
        row_specs.push_back(s);
      } else {
        double c[4];
        op_coefs(o.kind, o.offset, o.offset2, c);
        d.slot = -(int)consts.size() - 1;
        consts.insert(consts.end(), c, c + 4);
      }
      switch (o.kind) {
        case PQC_OP_RX: d.kind = K_RX; break;
        case PQC_OP_RY: d.kind = K_RY; break;
        case PQC_OP_RZ: d.kind = K_RZ; break;
        case PQC_OP_RXX: d.kind = K_RXX; break;
        case PQC_OP_RYY: d.kind = K_RYY; break;
        case PQC_OP_RZZ: d.kind = K_RZZ; break;
        default: d.kind = K_MIX2; break;
      }
    } else if (o.kind == PQC_OP_MAT1) {
      const double* m = o.m;  // m00 = (m[0], m[1]), m01 = (m[2], m[3]), m10 = (m[4], m[5]), m11 = (m[6], m[7])
      bool diag = m[2] == 0 && m[3] == 0 && m[4] == 0 && m[5] == 0;
      bool xg = m[0] == 0 && m[1] == 0 && m[6] == 0 && m[7] == 0 && m[2] == 1 && m[3] == 0 && m[4] == 1 && m[5] == 0;
      bool real = m[1] == 0 && m[3] == 0 && m[5] == 0 && m[7] == 0;
      d.slot = -(int)consts.size() - 1;
      if (xg) {
        d.kind = K_X;
      } else if (diag) {
        d.kind = K_DIAG1;
        consts.insert(consts.end(), {m[0], m[1], m[6], m[7]});
      } else if (real) {
        d.kind = K_REAL2;
        consts.insert(consts.end(), {m[0], m[2], m[4], m[6]});
      } else {
        d.kind = K_GEN1;
        consts.insert(consts.end(), m, m + 8);
      }
    } else if (o.kind == PQC_OP_CNOT) {
      d.kind = K_CNOT;
    } else if (o.kind == PQC_OP_CZ) {
      d.kind = K_CZ;
    } else if (o.kind == PQC_OP_MAT2) {
      const double* m = o.m;  // entry (r, c) at m[2*(4r+c)]
      auto re = [&](int r, int c) { return m[2 * (4 * r + c)]; };
      auto imv = [&](int r, int c) { return m[2 * (4 * r + c) + 1]; };
      bool mix = true;
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
          bool inblock = (r == 1 || r == 2) && (c == 1 || c == 2);
          bool keep = inblock || (r == c);
          if (!keep && (re(r, c) != 0 || imv(r, c) != 0)) mix = false;
        }
      if (mix && !(re(0, 0) == 1 && imv(0, 0) == 0)) mix = false;
      // block [[a, b], [b, a]] with a real, b imaginary: c = a, s = -Im(b)
      if (mix && !(imv(1, 1) == 0 && imv(2, 2) == 0 && re(1, 1) == re(2, 2) && re(1, 2) == 0 && re(2, 1) == 0 &&
                   imv(1, 2) == imv(2, 1)))
        mix = false;
      d.slot = -(int)consts.size() - 1;
      if (mix) {
        d.kind = K_MIX2;
        consts.insert(consts.end(), {re(1, 1), -imv(1, 2), re(3, 3), imv(3, 3)});
      } else {
        d.kind = K_GEN2;
        consts.insert(consts.end(), m, m + 32);
      }
    } else if (o.kind == PQC_OP_PAULI) {
      d.kind = K_PAULI;
      d.aux = o.pauli & 0xffff;
      int l0 = o.pauli & 0xff, l1 = (o.pauli >> 8) & 0xff;
      if (l0 > 3 || l1 > 3) return fail(PQC_ERR_INVALID, "op " + std::to_string(i) + ": bad Pauli letter");
      if (o.q1 < 0 && l1 != 0) return fail(PQC_ERR_INVALID, "op " + std::to_string(i) + ": Pauli letter on q1 = -1");
      d.slot = -(int)consts.size() - 1;
      consts.insert(consts.end(), {o.m[0], o.m[1], 0.0, 0.0});
    } else {
      return fail(PQC_ERR_UNSUPPORTED, "op " + std::to_string(i) + ": unsupported kind " + std::to_string(o.kind));
    }
    dops.push_back(d);
  }
  return PQC_OK;
}

// ---------------------------------------------------------------- planner
struct Masks {
  uint64_t move, touch;
  bool diag;
};

static Masks op_masks(const DOp& o) {
  uint64_t b0 = 1ull << o.p0, b1 = o.p1 >= 0 ? 1ull << o.p1 : 0ull;
  switch (o.kind) {
    case K_RY:
    case K_RX:
    case K_REAL2:
    case K_GEN1:
    case K_X:
      return {b0, b0, false};
    case K_RZ:
    case K_DIAG1:
      return {0, b0, true};
    case K_CNOT:
      return {b1, b0 | b1, false};
    case K_CZ:
    case K_RZZ:
      return {0, b0 | b1, true};
    case K_PAULI:
    case K_MEASURE: {
      int l0 = o.aux & 0xff, l1 = (o.aux >> 8) & 0xff;
      uint64_t mv = ((l0 == 1 || l0 == 2) ? b0 : 0) | ((l1 == 1 || l1 == 2) ? b1 : 0);
      uint64_t tc = (l0 ? b0 : 0) | (l1 ? b1 : 0);
      return {mv, tc, mv == 0};
    }
    default:
      return {b0 | b1, b0 | b1, false};
  }
}

static int popc(uint64_t x) { return __builtin_popcountll(x); }

// What the planner's searches read of each op, computed once per search: its masks and its cost class (0: CNOT or
// X, free in a relabelled sweep; 1: a single-qubit rotation that can pair; 2: any other non-diagonal op).
struct OpInfo {
  uint64_t move, touch;
  bool diag;
  uint8_t cat;
};

static std::vector<OpInfo> op_infos(const std::vector<DOp>& dops) {
  std::vector<OpInfo> info(dops.size());
  for (size_t i = 0; i < dops.size(); ++i) {
    const DOp& o = dops[i];
    const Masks m = op_masks(o);
    const uint8_t cat = (o.kind == K_CNOT || o.kind == K_X)                                             ? 0
                        : (o.kind == K_RY || o.kind == K_RX || o.kind == K_REAL2 || o.kind == K_GEN1) ? 1
                                                                                                        : 2;
    info[i] = {m.move, m.touch, m.diag, cat};
  }
  return info;
}

// An op is blocked (must wait for a later sweep) when an earlier pending op that stays pending touches one of
// its qubits, unless both are diagonal.  `applied` receives the ops a sweep with active set S applies, in
// order (nullptr: only count them).
static int split_pending(const std::vector<OpInfo>& info, const std::vector<int>& pending, uint64_t S,
                         std::vector<int>* applied, std::vector<int>* deferred) {
  uint64_t bAny = 0, bND = 0;
  int n = 0;
  for (int idx : pending) {
    const OpInfo& m = info[idx];
    const bool blocked = m.diag ? (m.touch & bND) != 0 : (m.touch & bAny) != 0;
    if (!blocked && (m.move & ~S) == 0) {
      ++n;
      if (applied) applied->push_back(idx);
    } else {
      if (deferred) deferred->push_back(idx);
      bAny |= m.touch;
      if (!m.diag) bND |= m.touch;
    }
  }
  return n;
}

// Greedy active set: S grows by the moving positions of the pending ops in program order (the ops of `seed`
// first, when >= 0) while they fit in k positions; ops that cannot join block the later ops they touch.
static uint64_t greedy_active(const std::vector<OpInfo>& info, const std::vector<int>& pending, uint64_t S, int k,
                              int seed) {
  if (seed >= 0) S |= info[seed].move;
  uint64_t bAny = 0, bND = 0;
  for (int idx : pending) {
    if (popc(S) >= k) break;  // full: no later op can add a position
    const OpInfo& m = info[idx];
    const bool blocked = m.diag ? (m.touch & bND) != 0 : (m.touch & bAny) != 0;
    if (!blocked) {
      if ((m.move & ~S) == 0) continue;
      if (popc(S | m.move) <= k) {
        S |= m.move;
        continue;
      }
    }
    bAny |= m.touch;
    if (!m.diag) bND |= m.touch;
  }
  return S;
}

// Candidate active sets of the next sweep: the greedy set in program order, the greedy sets seeded with each of
// the first kMaxSeeds unblocked pending ops that move positions outside `base`, and the windows of k - c0
// consecutive positions above `base` (the windows follow nearest-neighbour entanglers), without repeats.
static std::vector<uint64_t> active_candidates(const std::vector<OpInfo>& info, const std::vector<int>& pending,
                                               int N, int k, int c0) {
  constexpr int kMaxSeeds = 64;
  const uint64_t base = (1ull << c0) - 1;
  auto fill = [&](uint64_t S) {
    for (int p = 0; p < N && popc(S) < k; ++p) S |= 1ull << p;
    return S;
  };
  std::vector<uint64_t> cands;
  auto add = [&](uint64_t S) {
    if (std::find(cands.begin(), cands.end(), S) == cands.end()) cands.push_back(S);
  };
  add(fill(greedy_active(info, pending, base, k, -1)));
  uint64_t bAny = 0, bND = 0;
  int seeds = 0;
  for (int idx : pending) {
    const OpInfo& m = info[idx];
    const bool blocked = m.diag ? (m.touch & bND) != 0 : (m.touch & bAny) != 0;
    if (blocked) {
      bAny |= m.touch;
      if (!m.diag) bND |= m.touch;
      continue;
    }
    if ((m.move & ~base) != 0 && popc(base | m.move) <= k) {
      add(fill(greedy_active(info, pending, base, k, idx)));
      if (++seeds >= kMaxSeeds) break;
    }
  }
  const int w = k - c0;
  for (int a = c0; w > 0 && a + w <= N; ++a) add(base | (((1ull << w) - 1) << a));
  return cands;
}

// Estimated cost of one sweep that applies `applied` (in order), in units of a rotation-pair pass over the tile:
// the sweep's own load and write-out (kSweepCost), one pass per pair of consecutive single-qubit rotations
// (CNOTs and X gates in between cost nothing: the sweep relabels the tile index), one phase-table pass per run
// of diagonal ops, one pass per other op.  The weights follow the N = 20 hardware-efficient batch (2^13-amplitude
// tiles): about 0.57 ms per rotation-pair pass, 0.87 ms per phase-table pass and 2 ms of load and write-out per
// 256-row sweep.
constexpr double kSweepCost = 3.5, kPairCost = 1.0, kPhaseCost = 1.5;

static double sweep_cost(const std::vector<OpInfo>& info, const std::vector<int>& applied) {
  double cost = kSweepCost;
  int rot = 0;
  bool diag = false;
  auto flush = [&] {
    cost += kPairCost * ((rot + 1) / 2) + (diag ? kPhaseCost : 0.0);
    rot = 0;
    diag = false;
  };
  for (int idx : applied) {
    const OpInfo& m = info[idx];
    if (m.cat == 0) continue;
    if (m.diag) {
      if (rot) flush();
      diag = true;
    } else if (m.cat == 1) {
      if (diag) flush();
      ++rot;
    } else {
      flush();
      cost += kPairCost;
    }
  }
  flush();
  return cost;
}

// Estimated cost of the ops still pending, at the rates a good plan of the hardware-efficient ladder reaches:
// 1.84 rotations per rotation-pair pass, 7 diagonal ops per phase-table pass and 2.6 k rotations per sweep.
static double pending_cost(const std::vector<OpInfo>& info, const std::vector<int>& pending, int k) {
  int rot = 0, diag = 0;
  for (int idx : pending) {
    const OpInfo& m = info[idx];
    if (m.cat == 0) continue;
    if (m.diag)
      ++diag;
    else
      ++rot;
  }
  return kPairCost * rot / 1.84 + kPhaseCost * diag / 7.0 + kSweepCost * rot / (2.6 * k);
}

// One beam search over sweep sequences: every candidate set extends each of the `width` partial plans kept at the
// previous level by one sweep.  by_cost false keeps the plans with the fewest pending ops (width 1 is the per-sweep
// greedy choice of the set that applies the most ops); by_cost true keeps the lowest estimated total cost (cost so
// far plus pending_cost).  Returns the cheapest complete plan found (ties: the earlier one) and its cost.
static std::vector<uint64_t> beam_plan(const std::vector<OpInfo>& info, int N, int k, int c0, size_t width,
                                       bool by_cost, double* cost_out) {
  struct Node {
    std::vector<int> pending;
    std::vector<uint64_t> seq;
    double cost, f;
    uint64_t hash;
  };
  auto hash_of = [](const std::vector<int>& v) {
    uint64_t h = 1469598103934665603ull;
    for (int x : v) h = (h ^ (uint64_t)(uint32_t)x) * 1099511628211ull;
    return h ^ (uint64_t)v.size();
  };
  std::vector<Node> beam(1);
  beam[0].pending.resize(info.size());
  for (size_t i = 0; i < info.size(); ++i) beam[0].pending[i] = (int)i;
  beam[0].cost = 0.0;
  beam[0].f = pending_cost(info, beam[0].pending, k);
  beam[0].hash = hash_of(beam[0].pending);
  std::vector<uint64_t> best;
  double best_cost = 1e300;
  for (size_t level = 0; level <= info.size() && !beam.empty(); ++level) {
    std::vector<Node> next;
    for (const Node& nd : beam) {
      if (by_cost && nd.f >= best_cost) continue;
      for (uint64_t S : active_candidates(info, nd.pending, N, k, c0)) {
        std::vector<int> applied, deferred;
        applied.reserve(nd.pending.size());
        deferred.reserve(nd.pending.size());
        split_pending(info, nd.pending, S, &applied, &deferred);
        if (applied.empty()) continue;
        Node ch{std::move(deferred), nd.seq, nd.cost + sweep_cost(info, applied), 0.0, 0};
        ch.seq.push_back(S);
        if (ch.pending.empty()) {
          if (ch.cost < best_cost) {
            best_cost = ch.cost;
            best = ch.seq;
          }
          continue;
        }
        ch.f = ch.cost + pending_cost(info, ch.pending, k);
        if (by_cost && ch.f >= best_cost) continue;
        ch.hash = hash_of(ch.pending);
        bool dup = false;
        for (Node& o : next)
          if (o.hash == ch.hash && o.pending == ch.pending) {
            if (ch.cost < o.cost) o = std::move(ch);  // the same pending ops, reached more cheaply
            dup = true;
            break;
          }
        if (!dup) next.push_back(std::move(ch));
      }
    }
    if (by_cost)
      std::stable_sort(next.begin(), next.end(), [](const Node& x, const Node& y) { return x.f < y.f; });
    else
      std::stable_sort(next.begin(), next.end(),
                       [](const Node& x, const Node& y) { return x.pending.size() < y.pending.size(); });
    if (next.size() > width) next.resize(width);
    beam = std::move(next);
    if (!by_cost && !best.empty()) break;  // the fewest sweeps this beam reaches
  }
  *cost_out = best_cost;
  return best;
}

// The active sets of all sweeps: the cheapest (by sweep_cost) of the per-sweep greedy plan, the plan of a beam
// that keeps the partial plans with the fewest pending ops, and the plan of a beam ranked by estimated cost.  On
// the hardware-efficient ladder at N = 20, L = 20 the greedy plan leaves two sweeps that apply one rotation and
// five CNOTs, while the fewest sweeps are not always the cheapest plan either: narrow bands of many layers split
// each layer's diagonal ops over more phase-table passes.
constexpr int kPlanSearch = 3;  // 1: greedy only, 2: + fewest-pending beam, 3: + cost-ranked beam

static std::vector<uint64_t> search_active_sets(const std::vector<DOp>& dops, int N, int k, int c0);

// The searches depend only on the ops' kinds, positions and Pauli letters: plans of identical op lists (the
// families of a serving loop, programs rebuilt by a caller) come from a process-wide cache.
static std::vector<uint64_t> plan_active_sets(const std::vector<DOp>& dops, int N, int k, int c0) {
  if (dops.empty()) return {};
  uint64_t key = 1469598103934665603ull;
  auto mix = [&](int64_t v) { key = (key ^ (uint64_t)v) * 1099511628211ull; };
  mix(N);
  mix(k);
  mix(c0);
  for (const DOp& o : dops) {
    mix(o.kind);
    mix(o.p0);
    mix(o.p1);
    mix(o.aux);
  }
  static std::mutex mu;
  static std::unordered_map<uint64_t, std::pair<std::vector<DOp>, std::vector<uint64_t>>> cache;
  auto same = [&](const std::vector<DOp>& a) {
    if (a.size() != dops.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
      if (a[i].kind != dops[i].kind || a[i].p0 != dops[i].p0 || a[i].p1 != dops[i].p1 || a[i].aux != dops[i].aux)
        return false;
    return true;
  };
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end() && same(it->second.first)) return it->second.second;
  }
  std::vector<uint64_t> seq = search_active_sets(dops, N, k, c0);
  std::lock_guard<std::mutex> lock(mu);
  if (cache.size() >= 1024) cache.clear();
  cache[key] = {dops, seq};
  return seq;
}

static std::vector<uint64_t> search_active_sets(const std::vector<DOp>& dops, int N, int k, int c0) {
  double c1 = 1e300, c2 = 1e300, c3 = 1e300;
  const std::vector<OpInfo> info = op_infos(dops);
  std::vector<uint64_t> best = beam_plan(info, N, k, c0, 1, false, &c1);
  double best_cost = c1;
  // beams of 16 partial plans up to about 1500 ops, narrower above (the search time grows with both)
  const size_t width = std::max<size_t>(4, std::min<size_t>(16, 16 * 1500 / std::max<size_t>(dops.size(), 1)));
  if (kPlanSearch >= 2) {
    std::vector<uint64_t> p = beam_plan(info, N, k, c0, width, false, &c2);
    if (!p.empty() && c2 < best_cost) best = std::move(p), best_cost = c2;
  }
  if (kPlanSearch >= 3) {
    std::vector<uint64_t> p = beam_plan(info, N, k, c0, width, true, &c3);
    if (!p.empty() && c3 < best_cost) best = std::move(p), best_cost = c3;
  }
  return best;
}

int build_plan(const std::vector<DOp>& dops, int n_qubits, int k, int cmin, Plan& plan) {
  plan.sweeps.clear();
  plan.ops.clear();
  plan.offs.clear();
  plan.lazy_cols.clear();
  const int N = n_qubits;
  if (k <= 0 || k > N) k = N;
  const uint64_t all = (N >= 64) ? ~0ull : ((1ull << N) - 1);
  int c0 = std::min(cmin, k);
  if (k < N && k - c0 < 2) c0 = std::max(0, k - 2);
  std::vector<int> pending(dops.size());
  for (size_t i = 0; i < dops.size(); ++i) pending[i] = (int)i;
  bool first = true;
  const std::vector<uint64_t> seq = (k == N) ? std::vector<uint64_t>() : plan_active_sets(dops, N, k, c0);
  if (k < N && !dops.empty() && seq.empty()) return fail(PQC_ERR_INVALID, "planner made no progress");
  const std::vector<OpInfo> info = op_infos(dops);
  size_t step = 0;
  do {
    const uint64_t S = (k == N) ? all : seq[std::min(step++, seq.size() - 1)];
    std::vector<int> applied, deferred;
    split_pending(info, pending, S, &applied, &deferred);
    if (applied.empty() && !pending.empty()) return fail(PQC_ERR_INVALID, "planner made no progress");
    SweepDesc sd;
    memset(&sd, 0, sizeof(sd));
    sd.k = k;
    int act[64], na = 0;
    for (int p = 0; p < N; ++p) {
      sd.local_of[p] = -1;
      if (S >> p & 1) act[na++] = p;
    }
    for (int p = N; p < kMaxQubits; ++p) sd.local_of[p] = -1;
    if (na != k) return fail(PQC_ERR_INVALID, "planner: active set size mismatch");
    int c = 0;
    while (c < k && act[c] == c) ++c;
    if (k >= 9 && c > 4) c = 4;  // the low 4 positions keep global rows coalesced; the rest may be reordered
    // Local bits above the low c in order of use: the positions that the sweep's non-element-wise ops touch
    // most get the lowest local bits, the least used the top ones.  With warp-blocked loops the kernels
    // need a CTA-wide barrier only around ops on the top local bits (those that span warps).
    {
      int uses[64] = {0};
      for (int idx : applied) {
        const DOp& o = dops[idx];
        if (o.kind == K_RZ || o.kind == K_DIAG1 || o.kind == K_RZZ) continue;
        if (o.p0 >= 0) ++uses[o.p0];
        if (o.p1 >= 0) ++uses[o.p1];
      }
      std::stable_sort(act + c, act + k, [&](int a, int b) { return uses[a] > uses[b]; });
    }
    sd.c = c;
    for (int j = 0; j < k; ++j) sd.local_of[act[j]] = (int8_t)j;
    sd.n_free = 0;
    for (int p = 0; p < N; ++p)
      if (!(S >> p & 1)) sd.free_pos[sd.n_free++] = (int8_t)p;
    sd.offs_begin = (int64_t)plan.offs.size();
    int nhi = 1 << (k - c);
    for (int h = 0; h < nhi; ++h) {
      int64_t off = 0;
      for (int j = 0; j < k - c; ++j)
        if (h >> j & 1) off |= 1ll << act[c + j];
      plan.offs.push_back(off);
    }
    sd.op_begin = (int)plan.ops.size();
    sd.n_ops = (int)applied.size();
    if (sd.n_ops > kMaxSweepOps) {
      // split very long sweeps so one launch stays bounded; same active set
      int done = 0;
      while (done < sd.n_ops) {
        SweepDesc part = sd;
        part.op_begin = (int)plan.ops.size();
        part.n_ops = std::min(kMaxSweepOps, sd.n_ops - done);
        for (int j = 0; j < part.n_ops; ++j) plan.ops.push_back(dops[applied[done + j]]);
        part.first = first ? 1 : 0;
        first = false;
        part.last = 0;
        plan.sweeps.push_back(part);
        done += part.n_ops;
      }
    } else {
      for (int idx : applied) plan.ops.push_back(dops[idx]);
      sd.first = first ? 1 : 0;
      first = false;
      sd.last = 0;
      plan.sweeps.push_back(sd);
    }
    pending.swap(deferred);
  } while (!pending.empty());
  plan.sweeps.back().last = 1;
  // verify: every op's moving positions are active in its sweep
  for (const SweepDesc& sd : plan.sweeps)
    for (int j = 0; j < sd.n_ops; ++j) {
      Masks m = op_masks(plan.ops[sd.op_begin + j]);
      for (int p = 0; p < N; ++p)
        if ((m.move >> p & 1) && sd.local_of[p] < 0) return fail(PQC_ERR_INVALID, "planner: moving bit not active");
    }
  return PQC_OK;
}

// Insert a K_PHASEBLK marker before every run of >= 2 consecutive diagonal ops
// (RZ, DIAG1, CZ, RZZ; applied to every row) inside a sweep.  Diagonal ops
// commute, so the kernel may multiply the whole run in at the marker.
static bool fusable_diag(const DOp& o) {
  return o.sel < 0 && (o.kind == K_RZ || o.kind == K_DIAG1 || o.kind == K_CZ || o.kind == K_RZZ);
}

static bool fusable_rot(const DOp& o) {
  return o.sel < 0 && (o.kind == K_RY || o.kind == K_RX || o.kind == K_REAL2);
}

// After fuse_diagonal_runs: consecutive pairs of single-qubit rotations on different
// positions become [K_ROT2, a, b], applied in one pass over amplitude quads (half the
// shared-memory traffic and barriers of two passes).  Phase blocks are kept intact.
void fuse_rotation_pairs(Plan& plan) {
  std::vector<DOp> ops;
  ops.reserve(plan.ops.size() + plan.ops.size() / 2 + 1);
  for (SweepDesc& sd : plan.sweeps) {
    const int begin = (int)ops.size();
    int j = 0;
    while (j < sd.n_ops) {
      const DOp& o = plan.ops[sd.op_begin + j];
      if (o.kind == K_PHASEBLK) {
        for (int r = 0; r <= o.aux; ++r) ops.push_back(plan.ops[sd.op_begin + j + r]);
        j += o.aux + 1;
        continue;
      }
      if (j + 1 < sd.n_ops && fusable_rot(o)) {
        const DOp& q = plan.ops[sd.op_begin + j + 1];
        const bool distinct = sd.lazy ? (q.c0 != o.c0) : (q.p0 != o.p0);
        if (fusable_rot(q) && distinct) {
          DOp m;
          m.kind = K_ROT2;
          m.sel = -1;
          m.p0 = o.p0;
          m.p1 = q.p0;
          m.slot = 0;
          m.aux = 2;
          m.gidx = -1;
          if (sd.lazy) {
            // pivot bits (q0, q1) on which the two masks form an invertible 2 x 2 block: enumerating the
            // slots with both pivots clear visits every quad {p, p^c0, p^c1, p^c0^c1} once
            const unsigned a = (uint16_t)o.c0, b = (uint16_t)q.c0;
            const int p0 = __builtin_ctz(a);
            const unsigned b2 = ((b >> p0) & 1) ? (b ^ a) : b;
            m.q0 = (int8_t)p0;
            m.q1 = (int8_t)__builtin_ctz(b2);
          }
          ops.push_back(m);
          ops.push_back(o);
          ops.push_back(q);
          j += 2;
          continue;
        }
      }
      ops.push_back(o);
      ++j;
    }
    sd.op_begin = begin;
    sd.n_ops = (int)ops.size() - begin;
  }
  plan.ops.swap(ops);
}

// Relabelled sweeps: a CNOT with both qubits in the tile permutes the tile index linearly over GF(2)
// (l -> l ^ (l_c << t)); instead of moving amplitudes, the sweep keeps logical index l at physical slot
// A l ^ b and folds each CNOT into A (and each X, or CNOT with a control outside the tile, into the offset
// b).  Every later op of the sweep then addresses its pairs and parities through masks of A, and the
// write-out reads logical index l from slot A l ^ b.  A sweep is relabelled when it holds at least one
// CNOT/X and only kinds with a masked form (rotations, diagonal ops, CZ, phase blocks); the others run
// as before.
static bool relabel_supported(const DOp& o, bool measures, bool gens) {
  if (o.kind == K_MEASURE) return measures;
  if (o.kind == K_PAULI) return gens;  // derivative generators (one row each)
  if (o.sel >= 0) return false;
  switch (o.kind) {
    case K_RY: case K_RX: case K_REAL2: case K_GEN1: case K_RZ: case K_DIAG1: case K_RZZ: case K_CZ:
    case K_CNOT: case K_X:
      return true;
    default:
      return false;
  }
}

static uint16_t inverse_columns_bit(const uint16_t* row, int k, int i) {
  uint16_t v = 0;
  for (int j = 0; j < k; ++j)
    if ((row[j] >> i) & 1) v |= (uint16_t)(1u << j);
  return v;
}

void relabel_cnots(Plan& plan, bool measures, bool gens) {
  std::vector<DOp> ops;
  ops.reserve(plan.ops.size());
  for (SweepDesc& sd : plan.sweeps) {
    const int begin = (int)ops.size();
    const DOp* src = plan.ops.data() + sd.op_begin;
    bool eligible = sd.k <= 13, any = false;
    int n_folded = 0, n_diag_single = 0;
    for (int j = 0; eligible && j < sd.n_ops; ++j) {
      const DOp& o = src[j];
      if (o.kind == K_PHASEBLK) {  // members are diagonal kinds
        j += o.aux;
        continue;
      }
      if (!relabel_supported(o, measures, gens)) eligible = false;
      if (o.kind == K_RZ || o.kind == K_DIAG1 || o.kind == K_RZZ || o.kind == K_CZ) ++n_diag_single;
      if (o.kind == K_CNOT && sd.local_of[o.p0] >= 0 && sd.local_of[o.p1] >= 0) ++n_folded;
      if (o.kind == K_CNOT && sd.local_of[o.p1] >= 0) any = true;
      if (o.kind == K_X) any = true;
      if (o.kind == K_CNOT && sd.local_of[o.p1] < 0) eligible = false;
    }
    // A relabelled sweep recomputes the logical bits of every amplitude for each single diagonal op, so a
    // derivative sweep stays unrelabelled unless it folds at least 4 CNOTs per such op (TFIM-style CNOT-RZ-CNOT
    // ladders, 2 per op: 4.59 ms for the N = 16 derivative states unrelabelled, 4.87 ms relabelled; the HE
    // ladder's sweeps, 30 per op: 6.05 against 7.19 ms from the initial state).
    if (gens && n_diag_single * 4 > n_folded) eligible = false;
    if (!eligible || !any) {
      for (int j = 0; j < sd.n_ops; ++j) ops.push_back(src[j]);
      sd.op_begin = begin;
      sd.lazy = 0;
      continue;
    }
    const int k = sd.k;
    uint16_t col[16], row[16];
    for (int j = 0; j < 16; ++j) col[j] = row[j] = (uint16_t)(j < k ? (1u << j) : 0);
    auto masks = [&](DOp& o) {
      const int j0 = sd.local_of[o.p0];
      const int j1 = o.p1 >= 0 ? sd.local_of[o.p1] : -1;
      o.c0 = (int16_t)(j0 >= 0 ? col[j0] : 0);
      o.c1 = (int16_t)(j1 >= 0 ? col[j1] : 0);
      o.r0 = (int16_t)(j0 >= 0 ? row[j0] : 0);
      o.r1 = (int16_t)(j1 >= 0 ? row[j1] : 0);
      o.q0 = (int8_t)(o.c0 ? __builtin_ctz((unsigned)(uint16_t)o.c0) : 0);
    };
    int j = 0;
    while (j < sd.n_ops) {
      DOp o = src[j];
      if (o.kind == K_PHASEBLK) {
        // record the columns of A^-1 (physical bit i -> logical mask) for the block's index tables
        o.slot = (int32_t)(plan.lazy_cols.size() / kLazyRec);
        for (int i = 0; i < kLazyRec; ++i)
          plan.lazy_cols.push_back(i < k ? inverse_columns_bit(row, k, i) : (uint16_t)0);
        ops.push_back(o);
        for (int r = 1; r <= src[j].aux; ++r) {
          DOp m = src[j + r];
          masks(m);
          ops.push_back(m);
        }
        j += src[j].aux + 1;
        continue;
      }
      const int j0 = sd.local_of[o.p0];
      const int j1 = o.p1 >= 0 ? sd.local_of[o.p1] : -1;
      if (o.kind == K_CNOT && j0 >= 0) {
        // A' = A C: column c picks up column t; (A')^-1 = C A^-1: row t picks up row c
        col[j0] ^= col[j1];
        row[j1] ^= row[j0];
        ++j;
        continue;
      }
      if (o.kind == K_CNOT || o.kind == K_X) {
        DOp f = o;
        const int t = o.kind == K_CNOT ? j1 : j0;
        f.kind = K_OFFSET;
        f.c0 = (int16_t)col[t];
        f.aux = o.kind == K_CNOT ? 1 : 0;  // CNOT: only where the control (outside the tile) is set
        f.slot = 0;
        ops.push_back(f);
        ++j;
        continue;
      }
      masks(o);
      ops.push_back(o);
      ++j;
    }
    sd.out_rec = (int32_t)(plan.lazy_cols.size() / kLazyRec);
    for (int i = 0; i < kLazyRec; ++i) plan.lazy_cols.push_back(i < k ? col[i] : (uint16_t)0);
    sd.lazy = 1;
    sd.op_begin = begin;
    sd.n_ops = (int)ops.size() - begin;
  }
  plan.ops.swap(ops);
}

void finalize_plan(Plan& plan) {
  for (SweepDesc& sd : plan.sweeps) {
    int m = -1, lo = INT32_MAX, hi = -1;
    for (int j = 0; j < sd.n_ops; ++j) {
      const DOp& o = plan.ops[sd.op_begin + j];
      m = std::max(m, (int)o.gidx);
      if (o.sel < 0 && o.gidx >= 0) {
        lo = std::min(lo, (int)o.gidx);
        hi = std::max(hi, (int)o.gidx);
      }
    }
    sd.max_gidx = m;
    sd.min_fwd = lo;
    sd.max_fwd = hi;
  }
}

// A relabelled plan folds CNOTs into its index maps, so its sweeps' op ranges come from the unrelabelled twin
// (same sweeps, same ops before relabelling).
void copy_sweep_ranges(Plan& lazy, const Plan& plain) {
  for (size_t i = 0; i < lazy.sweeps.size() && i < plain.sweeps.size(); ++i) {
    lazy.sweeps[i].max_gidx = plain.sweeps[i].max_gidx;
    lazy.sweeps[i].min_fwd = plain.sweeps[i].min_fwd;
    lazy.sweeps[i].max_fwd = plain.sweeps[i].max_fwd;
  }
}

void fuse_diagonal_runs(Plan& plan) {
  std::vector<DOp> ops;
  ops.reserve(plan.ops.size() + plan.sweeps.size() * 8);
  for (SweepDesc& sd : plan.sweeps) {
    const int begin = (int)ops.size();
    int j = 0;
    while (j < sd.n_ops) {
      const DOp& o = plan.ops[sd.op_begin + j];
      int run = 0;
      while (j + run < sd.n_ops && run < kOpChunk - 1 && fusable_diag(plan.ops[sd.op_begin + j + run])) ++run;
      if (run >= 2) {
        // members ordered by where they act (diagonal ops commute): tile-constant, low half of the local
        // bits, high half, both halves; the kernels build one phase table per half from these ranges.  The
        // low half is the first kl bits, kl near k / 2 with the fewest members straddling the halves (each
        // such member costs an extra pass) and both tables within the kernels' 256-entry table space.
        auto cls_of = [&](const DOp& q, int kl) {
          const int j0 = sd.local_of[q.p0];
          const int j1 = q.p1 >= 0 ? sd.local_of[q.p1] : -1;
          const int h0 = j0 < 0 ? -1 : (j0 < kl ? 0 : 1);
          const int h1 = j1 < 0 ? -1 : (j1 < kl ? 0 : 1);
          return (h0 < 0 && h1 < 0) ? 0 : (h0 <= 0 && h1 <= 0) ? 1 : (h0 != 0 && h1 != 0) ? 2 : 3;
        };
        int kl = sd.k >> 1, best = -1;
        for (int cand : {sd.k >> 1, (sd.k >> 1) - 1, (sd.k >> 1) + 1}) {
          if (cand < 1 || cand >= sd.k || (1 << cand) + (1 << (sd.k - cand)) > 256) continue;
          int straddle = 0;
          for (int r = 0; r < run; ++r) straddle += cls_of(plan.ops[sd.op_begin + j + r], cand) == 3;
          if (best < 0 || straddle < best) {
            best = straddle;
            kl = cand;
          }
        }
        std::vector<DOp> cls[4];
        for (int r = 0; r < run; ++r) {
          const DOp& q = plan.ops[sd.op_begin + j + r];
          cls[cls_of(q, kl)].push_back(q);
        }
        DOp m;
        m.kind = K_PHASEBLK;
        m.sel = -1;
        m.p0 = 0;
        m.p1 = -1;
        m.slot = 0;
        m.aux = run;
        m.gidx = -1;
        m.c0 = (int16_t)cls[0].size();
        m.c1 = (int16_t)cls[1].size();
        m.r0 = (int16_t)cls[2].size();
        m.r1 = (int16_t)cls[3].size();
        m.q0 = (int8_t)kl;
        ops.push_back(m);
        for (int c = 0; c < 4; ++c)
          for (const DOp& q : cls[c]) ops.push_back(q);
        j += run;
      } else {
        ops.push_back(o);
        ++j;
      }
    }
    sd.op_begin = begin;
    sd.n_ops = (int)ops.size() - begin;
  }
  plan.ops.swap(ops);
}

int upload_plan(Plan& plan) {
  if (!plan.lazy_cols.empty()) {
    PQC_CUDA(cudaMalloc(&plan.d_lazy_cols, plan.lazy_cols.size() * sizeof(uint16_t)));
    PQC_CUDA(cudaMemcpy(plan.d_lazy_cols, plan.lazy_cols.data(), plan.lazy_cols.size() * sizeof(uint16_t),
                        cudaMemcpyHostToDevice));
  }
  size_t nb = plan.ops.size() * sizeof(DOp);
  if (nb) {
    PQC_CUDA(cudaMalloc(&plan.d_ops, nb));
    PQC_CUDA(cudaMemcpy(plan.d_ops, plan.ops.data(), nb, cudaMemcpyHostToDevice));
  }
  size_t no = plan.offs.size() * sizeof(int64_t);
  PQC_CUDA(cudaMalloc(&plan.d_offs, no));
  PQC_CUDA(cudaMemcpy(plan.d_offs, plan.offs.data(), no, cudaMemcpyHostToDevice));
  if (!plan.sweeps.empty()) {  // the descriptors, for the multi-program kernel (pqc_run_multi)
    const size_t ns = plan.sweeps.size() * sizeof(SweepDesc);
    PQC_CUDA(cudaMalloc(&plan.d_sweeps, ns));
    PQC_CUDA(cudaMemcpy(plan.d_sweeps, plan.sweeps.data(), ns, cudaMemcpyHostToDevice));
  }
  return PQC_OK;
}

void free_plan(Plan& plan) {
  if (plan.d_ops) cudaFree(plan.d_ops);
  if (plan.d_offs) cudaFree(plan.d_offs);
  if (plan.d_lazy_cols) cudaFree(plan.d_lazy_cols);
  if (plan.d_sweeps) cudaFree(plan.d_sweeps);
  plan.d_ops = nullptr;
  plan.d_offs = nullptr;
  plan.d_lazy_cols = nullptr;
  plan.d_sweeps = nullptr;
}

int upload_table(OpTable& t) {
  if (!t.specs.empty()) {
    PQC_CUDA(cudaMalloc(&t.d_specs, t.specs.size() * sizeof(RowCoefSpec)));
    PQC_CUDA(cudaMemcpy(t.d_specs, t.specs.data(), t.specs.size() * sizeof(RowCoefSpec), cudaMemcpyHostToDevice));
  }
  size_t nc = std::max<size_t>(t.consts.size(), 4);
  PQC_CUDA(cudaMalloc(&t.d_consts, nc * sizeof(double)));
  if (!t.consts.empty())
    PQC_CUDA(cudaMemcpy(t.d_consts, t.consts.data(), t.consts.size() * sizeof(double), cudaMemcpyHostToDevice));
  if (!t.dops.empty()) {
    PQC_CUDA(cudaMalloc(&t.d_dops, t.dops.size() * sizeof(DOp)));
    PQC_CUDA(cudaMemcpy(t.d_dops, t.dops.data(), t.dops.size() * sizeof(DOp), cudaMemcpyHostToDevice));
  }
  return PQC_OK;
}

void free_table(OpTable& t) {
  if (t.d_specs) cudaFree(t.d_specs);
  if (t.d_consts) cudaFree(t.d_consts);
  if (t.d_dops) cudaFree(t.d_dops);
  t.d_specs = nullptr;
  t.d_consts = nullptr;
  t.d_dops = nullptr;
}

// N <= 13: one sweep over the whole state; above that 2^12-amplitude tiles with 256 threads and two
// CTAs per SM measured faster than 2^13 tiles with one (11.2 vs 14.7 ms per sweep at N=20, B=256)
int default_tile_qubits(int n_qubits) { return n_qubits <= 13 ? n_qubits : 12; }

static bool same_op(const pqc_op& a, const pqc_op& b) { return memcmp(&a, &b, sizeof(pqc_op)) == 0; }

// Build (or reuse) the generator-inserted plan: run r applies gens[r]
// (with sel = r) right after forward op after[r].
// A reordering of forward ops (sel < 0) that keeps every pair of ops that may not commute in its order: two
// ops commute here when they act on disjoint positions or are both diagonal.  Ops are placed one at a time from
// those whose earlier non-commuting ops are all placed; the next op extends the current run when it can (a
// rotation after a rotation, on another qubit when the two would pair; a diagonal op after a diagonal op, so that
// they share a phase-block pass), and is otherwise the earliest op in the original order.  A sequence that is
// already grouped comes back unchanged.  Rows with op limits or starts stay correct, because each row applies the
// ops it selects (by op index) in an order that differs from the original only by swaps of commuting ops.
std::vector<DOp> schedule_for_fusion(const std::vector<DOp>& d) {
  const int n = (int)d.size();
  auto diag = [](const DOp& o) { return fusable_diag(o); };
  std::vector<std::vector<int>> succ(n);
  std::vector<int> indeg(n, 0);
  std::vector<int> last_nondiag(kMaxQubits + 1, -1);
  std::vector<std::vector<int>> diag_since(kMaxQubits + 1);
  auto edge = [&](int a, int b) {
    if (a < 0) return;
    succ[a].push_back(b);
    ++indeg[b];
  };
  for (int i = 0; i < n; ++i) {
    const DOp& o = d[i];
    if (o.sel >= 0) return d;  // generators and per-row ops keep their places
    const int qs[2] = {o.p0, o.p1};
    for (int t = 0; t < 2; ++t) {
      const int q = qs[t];
      if (q < 0) continue;
      if (q > kMaxQubits) return d;
      if (diag(o)) {
        edge(last_nondiag[q], i);
        diag_since[q].push_back(i);
      } else {
        edge(last_nondiag[q], i);
        for (int j : diag_since[q]) edge(j, i);
        diag_since[q].clear();
        last_nondiag[q] = i;
      }
    }
  }
  // an edge may repeat (both qubits shared): indeg counts each, and placing the source removes each
  std::set<int> ready;
  for (int i = 0; i < n; ++i)
    if (indeg[i] == 0) ready.insert(i);
  std::vector<DOp> out;
  out.reserve(n);
  int prev = -1;
  bool pair_open = false;  // the last op is a rotation that starts a pair
  while (!ready.empty()) {
    int pick = *ready.begin();
    if (prev >= 0) {
      const DOp& l = d[prev];
      for (int c : ready) {
        if ((diag(l) && diag(d[c])) || (fusable_rot(l) && fusable_rot(d[c]) && (!pair_open || d[c].p0 != l.p0))) {
          pick = c;
          break;
        }
      }
    }
    ready.erase(pick);
    const bool rot = fusable_rot(d[pick]);
    pair_open = rot && !(pair_open && prev >= 0 && fusable_rot(d[prev]) && d[prev].p0 != d[pick].p0);
    prev = pick;
    out.push_back(d[pick]);
    for (int c : succ[pick])
      if (--indeg[c] == 0) ready.insert(c);
  }
  if ((int)out.size() != n) return d;  // cannot happen: the edges run forward in the original order
  return out;
}

// Whether generator g (a Pauli term on one or two positions, run by one row) commutes with forward op o: they
// act on disjoint positions, both are diagonal, o is the rotation (or X gate) about the generator's own single
// axis, or o is a CNOT that the generator's letters pass (Z on the control, X on the target).
static bool generator_commutes(const DOp& g, const DOp& o) {
  if (g.kind != K_PAULI || o.sel >= 0) return false;
  const bool g2 = g.p1 >= 0, o2 = o.p1 >= 0;
  const bool share = g.p0 == o.p0 || (o2 && g.p0 == o.p1) || (g2 && (g.p1 == o.p0 || (o2 && g.p1 == o.p1)));
  if (!share) return true;
  const int l0 = g.aux & 0xff, l1 = (g.aux >> 8) & 0xff;  // 0 I, 1 X, 2 Y, 3 Z
  const bool gdiag = (l0 == 0 || l0 == 3) && (!g2 || l1 == 0 || l1 == 3);
  if (gdiag && fusable_diag(o)) return true;
  if (!g2 && !o2 && g.p0 == o.p0)
    return (o.kind == K_RY && l0 == 2) || ((o.kind == K_RX || o.kind == K_X) && l0 == 1);
  if (!g2 && o.kind == K_CNOT) return (g.p0 == o.p0 && l0 == 3) || (g.p0 == o.p1 && l0 == 1);
  return false;
}

// Whether forward ops a and b, adjacent in the sequence, may fuse into one pass (a rotation pair or a member
// run of a phase block); a generator placed between them would split that pass.
static bool fusing_neighbours(const DOp& a, const DOp& b) {
  return (fusable_diag(a) && fusable_diag(b)) || (fusable_rot(a) && fusable_rot(b) && a.p0 != b.p0);
}

// Where each generator enters the forward op sequence (before forward op pos[r]).  Generator r belongs right
// after forward op after[r]; it may move later past forward ops it commutes with without changing its row's
// state.  A position splits a fused pass when it falls inside a run of diagonal ops (one phase-block pass) or
// between two rotations that would pair; the generator takes the first position of its window that splits none,
// or stays where it belongs when the window has none.  Two tests of "between two rotations that would pair":
// parity 0 counts any two adjacent rotations; parity 1 only the pairs that form when each run of rotations pairs
// greedily from its start (as the planner pairs them when no sweep boundary falls inside the run).  A generator
// never moves earlier: a sweep that gained a generator from a later sweep could no longer be skipped by rows that
// start from a checkpoint after the sweep's forward ops.  A row that stops at a limit above after[r] still applies
// the window's forward ops and the generator, in an order that gives the same state; the generator keeps its op
// index, so row starts and limits select it as before.
void deriv_insert_positions(const std::vector<DOp>& fwd, const DOp* gens, const int32_t* after, int n_gens,
                            bool parity, std::vector<int>& pos) {
  const int n_fwd = (int)fwd.size();
  std::vector<char> pair_first(n_fwd + 1, 0);  // fwd[i] pairs with fwd[i + 1]
  for (int i = 0; i + 1 < n_fwd;) {
    if (fusable_rot(fwd[i]) && fusing_neighbours(fwd[i], fwd[i + 1])) {
      pair_first[i] = 1;
      i += 2;
    } else {
      ++i;
    }
  }
  auto splits = [&](int j) {
    if (j <= 0 || j >= n_fwd) return false;
    if (fusable_diag(fwd[j - 1]) && fusable_diag(fwd[j])) return true;
    return parity ? pair_first[j - 1] != 0 : fusing_neighbours(fwd[j - 1], fwd[j]);
  };
  pos.assign(n_gens, 0);
  for (int r = 0; r < n_gens; ++r) {
    const int home = after[r] + 1;
    int j = home;
    while (splits(j) && j < n_fwd && generator_commutes(gens[r], fwd[j])) ++j;
    pos[r] = splits(j) ? home : j;
  }
}

// Passes over a tile that one row of a plan makes: a load and a store per sweep, one per fused block and per
// other op; generators (one row each) and the index-offset updates of relabelled sweeps count nothing.
static long plan_passes(const Plan& plan) {
  long n = 0;
  for (const SweepDesc& sd : plan.sweeps) {
    n += 2;
    for (int j = 0; j < sd.n_ops; ++j) {
      const DOp& o = plan.ops[sd.op_begin + j];
      if (o.kind == K_PHASEBLK) j += o.aux;
      if (o.kind == K_ROT2) j += 2;
      if (o.sel < 0 && o.kind != K_OFFSET) ++n;
    }
  }
  return n;
}

// The forward plans of op sequence seq: sweeps with phase blocks, relabelled CNOTs and rotation pairs (fwd), and
// the same without relabelling (lim, kept only when some sweep is relabelled; lazy says whether one is).  A
// relabelled sweep folds its CNOTs into the tile index for every row, so runs with per-row op limits or starts
// take lim.
static int make_forward_plans(const std::vector<DOp>& seq, int n_qubits, int k, Plan& fwd, Plan& lim, bool& lazy) {
  Plan f;
  int rc = build_plan(seq, n_qubits, k, 4, f);
  if (rc) return rc;
  fuse_diagonal_runs(f);
  Plan l = f;
  relabel_cnots(f);
  lazy = false;
  for (const SweepDesc& sd : f.sweeps) lazy = lazy || sd.lazy;
  fuse_rotation_pairs(f);
  finalize_plan(f);
  if (lazy) {
    fuse_rotation_pairs(l);
    finalize_plan(l);
    copy_sweep_ranges(f, l);
  } else {
    l = Plan();
  }
  fwd = std::move(f);
  lim = std::move(l);
  return PQC_OK;
}

// The forward plans of seq or of its schedule_for_fusion order, whichever makes fewer passes over the tiles (seq
// is replaced by the order taken; a schedule that changes nothing is not planned again).
static int choose_forward_plans(std::vector<DOp>& seq, int n_qubits, int k, Plan& fwd, Plan& lim, bool& lazy) {
  int rc = make_forward_plans(seq, n_qubits, k, fwd, lim, lazy);
  if (rc) return rc;
  std::vector<DOp> alt = schedule_for_fusion(seq);
  bool same_order = true;
  for (size_t i = 0; same_order && i < seq.size(); ++i) same_order = alt[i].gidx == seq[i].gidx;
  if (same_order) return PQC_OK;
  Plan b, bl;
  bool bz = false;
  rc = make_forward_plans(alt, n_qubits, k, b, bl, bz);
  if (rc) return rc;
  if (plan_passes(b) < plan_passes(fwd)) {
    seq.swap(alt);
    fwd = std::move(b);
    lim = std::move(bl);
    lazy = bz;
  }
  return PQC_OK;
}

// The derivative plan of forward ops fwd with generators gens (gen r after forward op after[r]; sel = its run):
// the sequence with each generator at its position, planned and fused.  The forward ops run in their own order
// or in the order of schedule_for_fusion (generator r then follows op after[r] where that op now stands, which
// gives the same state: an op that moved across op after[r] commutes with it, so also with its generator, whose
// positions are a subset of the op's and which is diagonal when the op is).  Of these orders and the placements
// (every generator where it belongs, and the two split tests of deriv_insert_positions) the plan with the fewest
// passes is kept (out).  lazy_out receives its twin with relabelled sweeps (same sweeps; lazy_ok says whether any
// sweep is relabelled), which the rows that apply every op of a sweep take.
int build_deriv_plan(const std::vector<DOp>& fwd_in, const DOp* gens, const int32_t* after_in, int n_gens,
                     int n_qubits, int tile_qubits, Plan& out, Plan& lazy_out, bool& lazy_ok) {
  const int n_fwd = (int)fwd_in.size();
  long best = -1;
  Plan best_base;
  const std::vector<DOp> scheduled = schedule_for_fusion(fwd_in);
  bool same_order = true;
  for (int i = 0; same_order && i < n_fwd; ++i) same_order = scheduled[i].gidx == fwd_in[i].gidx;
  for (int order = 0; order < (same_order ? 1 : 2); ++order) {  // a schedule that changes nothing is not re-planned
    const std::vector<DOp>& fwd = order ? scheduled : fwd_in;
    std::vector<int> where(n_fwd);  // original op index -> position in fwd
    for (int i = 0; i < n_fwd; ++i) where[fwd[i].gidx] = i;
    std::vector<int32_t> after(n_gens);
    for (int r = 0; r < n_gens; ++r) after[r] = after_in[r] < 0 ? -1 : where[after_in[r]];
    std::vector<std::vector<int>> tried;  // generator positions already planned with this order
    for (int strategy = 0; strategy < 3; ++strategy) {
      std::vector<int> pos(n_gens);
      if (strategy == 0)
        for (int r = 0; r < n_gens; ++r) pos[r] = after[r] + 1;
      else
        deriv_insert_positions(fwd, gens, after.data(), n_gens, strategy == 2, pos);
      if (std::find(tried.begin(), tried.end(), pos) != tried.end()) continue;  // the same sequence again
      tried.push_back(pos);
      std::vector<std::vector<int>> at(n_fwd + 1);
      for (int r = 0; r < n_gens; ++r) at[pos[r]].push_back(r);
      std::vector<DOp> seq;
      seq.reserve(n_fwd + n_gens);
      for (int r : at[0]) seq.push_back(gens[r]);
      for (int i = 0; i < n_fwd; ++i) {
        seq.push_back(fwd[i]);
        for (int r : at[i + 1]) seq.push_back(gens[r]);
      }
      Plan base;
      int rc = build_plan(seq, n_qubits, tile_qubits, 4, base);
      if (rc) return rc;
      fuse_diagonal_runs(base);
      Plan plan = base;
      fuse_rotation_pairs(plan);
      const long n = plan_passes(plan);
      if (best < 0 || n < best) {
        best = n;
        out = std::move(plan);
        best_base = std::move(base);
      }
    }
  }
  finalize_plan(out);
  relabel_cnots(best_base, false, true);
  lazy_ok = false;
  for (const SweepDesc& sd : best_base.sweeps) lazy_ok = lazy_ok || sd.lazy;
  if (lazy_ok) {
    fuse_rotation_pairs(best_base);
    finalize_plan(best_base);
    copy_sweep_ranges(best_base, out);
    lazy_out = std::move(best_base);
  } else {
    lazy_out = Plan();
  }
  return PQC_OK;
}

int ensure_deriv(pqc_program* p, const pqc_op* gens, const int32_t* after, int n_gens) {
  if (p->deriv_valid && (int)p->d_gens.size() == n_gens) {
    bool same = true;
    for (int i = 0; same && i < n_gens; ++i) same = same_op(p->d_gens[i], gens[i]) && p->d_after[i] == after[i];
    if (same) return PQC_OK;
  }
  const int n_fwd = (int)p->ops.size();
  for (int i = 0; i < n_gens; ++i)
    if (after[i] < -1 || after[i] >= n_fwd) return fail(PQC_ERR_INVALID, "gen_after out of range");
  free_table(p->deriv_t);
  free_plan(p->deriv_plan);
  free_plan(p->deriv_lazy);
  p->deriv_lazy_ok = false;
  free_table(p->gen_t);
  if (p->d_run_row) cudaFree(p->d_run_row);
  p->d_run_row = nullptr;
  p->deriv_valid = false;
  std::vector<pqc_op> all(p->ops);
  std::vector<pqc_op> g(gens, gens + n_gens);
  for (int r = 0; r < n_gens; ++r) g[r].sel = r;  // run index
  all.insert(all.end(), g.begin(), g.end());
  int rc = lower_ops(all.data(), (int)all.size(), p->n_qubits, p->deriv_t);
  if (rc) return rc;
  rc = lower_ops(gens, n_gens, p->n_qubits, p->gen_t);
  if (rc) return rc;
  for (int r = 0; r < n_gens; ++r) p->deriv_t.dops[n_fwd + r].gidx = after[r];
  const std::vector<DOp> fwd_ops(p->deriv_t.dops.begin(), p->deriv_t.dops.begin() + n_fwd);
  rc = build_deriv_plan(fwd_ops, p->deriv_t.dops.data() + n_fwd, after, n_gens, p->n_qubits, p->tile_qubits,
                        p->deriv_plan, p->deriv_lazy, p->deriv_lazy_ok);
  if (rc) return rc;
  rc = upload_table(p->deriv_t);
  if (!rc) rc = upload_table(p->gen_t);
  if (!rc) rc = upload_plan(p->deriv_plan);
  if (!rc && p->deriv_lazy_ok) rc = upload_plan(p->deriv_lazy);
  if (rc) return rc;
  if (n_gens > 0) {
    std::vector<int32_t> rows(n_gens);
    for (int r = 0; r < n_gens; ++r) rows[r] = gens[r].sel;
    PQC_CUDA(cudaMalloc(&p->d_run_row, n_gens * sizeof(int32_t)));
    PQC_CUDA(cudaMemcpy(p->d_run_row, rows.data(), n_gens * sizeof(int32_t), cudaMemcpyHostToDevice));
  }
  p->d_gens = g;
  for (int r = 0; r < n_gens; ++r) p->d_gens[r] = gens[r];
  p->d_after.assign(after, after + n_gens);
  p->deriv_valid = true;
  return PQC_OK;
}

}  // namespace pqc

using namespace pqc;

extern "C" int pqc_abi_version(void) { return PQC_ABI_VERSION; }

extern "C" const char* pqc_last_error(void) { return g_last_error.c_str(); }

extern "C" long long pqc_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

// CNOT(c, t) RZ_t(theta) CNOT(c, t) = exp(-i theta/2 Z_c Z_t): the conjugated rotation is diagonal, so the
// triple becomes one K_RZZ on (c, t) with the RZ's coefficient slot.  Diagonal ops need no active bits and
// fuse into phase-table passes, so ansatze built from CNOT-RZ-CNOT (the TFIM-style ZZ layer) lose both the
// CNOT passes and most of their sweeps.  The fused op carries the index of the triple's last op; the
// indices inside a triple are recorded, because a per-row op limit may not cut a triple.
static std::vector<DOp> fuse_zz_conjugations(const std::vector<DOp>& d, std::vector<int32_t>& interior) {
  std::vector<DOp> out;
  out.reserve(d.size());
  size_t i = 0;
  while (i < d.size()) {
    if (i + 2 < d.size()) {
      const DOp &a = d[i], &r = d[i + 1], &b = d[i + 2];
      if (a.kind == K_CNOT && b.kind == K_CNOT && r.kind == K_RZ && a.sel < 0 && r.sel < 0 && b.sel < 0 &&
          a.p0 == b.p0 && a.p1 == b.p1 && r.p0 == a.p1) {
        DOp z = r;
        z.kind = K_RZZ;
        z.p0 = a.p0;
        z.p1 = a.p1;
        z.gidx = b.gidx;
        out.push_back(z);
        interior.push_back(a.gidx + 1);
        interior.push_back(a.gidx + 2);
        i += 3;
        continue;
      }
    }
    out.push_back(d[i]);
    ++i;
  }
  return out;
}

extern "C" int pqc_program_limit_ok(const pqc_program* p, int32_t limit) {
  if (!p) return 0;
  return std::binary_search(p->fused_interior.begin(), p->fused_interior.end(), limit) ? 0 : 1;
}

static int alloc_status(pqc_program* p) {
  PQC_CUDA(cudaMalloc(&p->d_status, sizeof(int32_t)));
  PQC_CUDA(cudaMemset(p->d_status, 0, sizeof(int32_t)));
  return PQC_OK;
}

extern "C" int pqc_program_create(const pqc_op* ops, int32_t n_ops, int32_t n_qubits, int32_t n_params,
                                  int32_t tile_qubits, pqc_program** out) {
  if (!out) return fail(PQC_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (n_qubits < 1 || n_qubits > kMaxQubits)
    return fail(PQC_ERR_UNSUPPORTED, "n_qubits must be in [1, " + std::to_string(kMaxQubits) + "]");
  if (n_ops < 0 || (n_ops > 0 && !ops)) return fail(PQC_ERR_INVALID, "bad op array");
  if (n_params < 0) return fail(PQC_ERR_INVALID, "n_params < 0");
  for (int i = 0; i < n_ops; ++i) {
    if (ops[i].param >= n_params || ops[i].param2 >= n_params)
      return fail(PQC_ERR_INVALID, "op " + std::to_string(i) + ": parameter column out of range");
    if (ops[i].sel != -1) return fail(PQC_ERR_INVALID, "op " + std::to_string(i) + ": forward ops must have sel = -1");
  }
  pqc_program* p = new (std::nothrow) pqc_program();
  if (!p) return fail(PQC_ERR_NOMEM, "host allocation failed");
  p->n_qubits = n_qubits;
  p->n_params = n_params;
  p->ops.assign(ops, ops + n_ops);
  int rc = lower_ops(ops, n_ops, n_qubits, p->fwd_t);
  if (rc) {
    delete p;
    return rc;
  }
  int k = tile_qubits > 0 ? std::min<int>(tile_qubits, n_qubits) : default_tile_qubits(n_qubits);
  if (k > 13) {
    delete p;
    return fail(PQC_ERR_UNSUPPORTED, "tile_qubits > 13 does not fit shared memory");
  }
  p->tile_qubits = k;
  std::vector<DOp> seq = fuse_zz_conjugations(p->fwd_t.dops, p->fused_interior);
  rc = choose_forward_plans(seq, n_qubits, k, p->fwd, p->fwd_lim, p->fwd_lazy);
  if (rc) {
    delete p;
    return rc;
  }
  cudaGetDevice(&p->device);
  rc = upload_table(p->fwd_t);
  if (!rc) rc = upload_plan(p->fwd);
  if (!rc && p->fwd_lazy) rc = upload_plan(p->fwd_lim);
  if (!rc) rc = alloc_status(p);
  if (rc) {
    pqc_program_destroy(p);
    return rc;
  }
  *out = p;
  return PQC_OK;
}

extern "C" int pqc_program_status(pqc_program* prog, int32_t* flags) {
  if (!prog || !flags) return fail(PQC_ERR_INVALID, "NULL argument");
  int32_t v = 0;
  PQC_CUDA(cudaMemcpy(&v, prog->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost));
  PQC_CUDA(cudaMemset(prog->d_status, 0, sizeof(int32_t)));
  *flags = v;
  return PQC_OK;
}

extern "C" void pqc_program_destroy(pqc_program* p) {
  if (!p) return;
  free_plan(p->fwd);
  free_plan(p->fwd_lim);
  free_table(p->fwd_t);
  free_plan(p->deriv_plan);
  free_plan(p->deriv_lazy);
  free_table(p->deriv_t);
  free_table(p->gen_t);
  if (p->d_run_row) cudaFree(p->d_run_row);
  if (p->d_status) cudaFree(p->d_status);
  free_adjoint(p);
  delete p;
}

extern "C" int pqc_plan_order(const pqc_op* ops, int32_t n_ops, int32_t n_qubits, int32_t tile_qubits,
                              int32_t* order, int32_t* sweep_of, int32_t* n_sweeps) {
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  if (n_ops < 0 || (n_ops > 0 && (!ops || !order || !sweep_of))) return fail(PQC_ERR_INVALID, "bad arguments");
  OpTable t;
  int rc = lower_ops(ops, n_ops, n_qubits, t);
  if (rc) return rc;
  // tag each op with its index through the otherwise unused `aux` bits above the Pauli letters
  std::vector<DOp> tagged = t.dops;
  for (int i = 0; i < n_ops; ++i) tagged[i].aux |= (i + 1) << 16;
  int k = tile_qubits > 0 ? std::min<int>(tile_qubits, n_qubits) : default_tile_qubits(n_qubits);
  if (k > 13) return fail(PQC_ERR_UNSUPPORTED, "tile_qubits > 13 does not fit shared memory");
  {
    Plan f, l;
    bool z = false;
    rc = choose_forward_plans(tagged, n_qubits, k, f, l, z);
    if (rc) return rc;
  }
  Plan plan;
  rc = build_plan(tagged, n_qubits, k, 4, plan);
  if (rc) return rc;
  int pos = 0;
  for (size_t s = 0; s < plan.sweeps.size(); ++s)
    for (int j = 0; j < plan.sweeps[s].n_ops; ++j) {
      order[pos] = (plan.ops[plan.sweeps[s].op_begin + j].aux >> 16) - 1;
      sweep_of[pos] = (int32_t)s;
      ++pos;
    }
  if (n_sweeps) *n_sweeps = (int32_t)plan.sweeps.size();
  return PQC_OK;
}

extern "C" int pqc_derivative_plan_order(const pqc_op* ops, int32_t n_ops, const pqc_op* gens,
                                         const int32_t* gen_after, int32_t n_gens, int32_t n_qubits,
                                         int32_t tile_qubits, int32_t* order, int32_t* n_sweeps) {
  if (n_qubits < 1 || n_qubits > kMaxQubits) return fail(PQC_ERR_UNSUPPORTED, "n_qubits out of range");
  if (n_ops < 0 || n_gens < 0 || (n_ops > 0 && !ops) || (n_gens > 0 && (!gens || !gen_after)) ||
      (n_ops + n_gens > 0 && !order))
    return fail(PQC_ERR_INVALID, "bad arguments");
  if (n_ops + n_gens > 32767) return fail(PQC_ERR_UNSUPPORTED, "more than 32767 ops and generators");
  for (int r = 0; r < n_gens; ++r)
    if (gen_after[r] < -1 || gen_after[r] >= n_ops) return fail(PQC_ERR_INVALID, "gen_after out of range");
  std::vector<pqc_op> all(ops, ops + n_ops);
  for (int r = 0; r < n_gens; ++r) {
    pqc_op g = gens[r];
    g.sel = r;
    all.push_back(g);
  }
  OpTable t;
  int rc = lower_ops(all.data(), (int)all.size(), n_qubits, t);
  if (rc) return rc;
  // tag each op and generator with its index through the `aux` bits above the Pauli letters
  for (int i = 0; i < n_ops + n_gens; ++i) t.dops[i].aux |= (i + 1) << 16;
  for (int r = 0; r < n_gens; ++r) t.dops[n_ops + r].gidx = gen_after[r];
  const int k = tile_qubits > 0 ? std::min<int>(tile_qubits, n_qubits) : default_tile_qubits(n_qubits);
  if (k > 13) return fail(PQC_ERR_UNSUPPORTED, "tile_qubits > 13 does not fit shared memory");
  const std::vector<DOp> fwd(t.dops.begin(), t.dops.begin() + n_ops);
  Plan plan, lazy;
  bool lazy_ok = false;
  rc = build_deriv_plan(fwd, t.dops.data() + n_ops, gen_after, n_gens, n_qubits, k, plan, lazy, lazy_ok);
  if (rc) return rc;
  int pos = 0;
  for (const SweepDesc& sd : plan.sweeps)
    for (int j = 0; j < sd.n_ops; ++j) {
      const DOp& o = plan.ops[sd.op_begin + j];
      if (o.kind == K_PHASEBLK || o.kind == K_ROT2) continue;  // markers of fused blocks
      const int tag = (o.aux >> 16) - 1;
      order[pos++] = tag < n_ops ? tag : -(tag - n_ops + 1);
    }
  if (pos != n_ops + n_gens) return fail(PQC_ERR_INVALID, "derivative plan lost an op");
  if (n_sweeps) *n_sweeps = (int32_t)plan.sweeps.size();
  return PQC_OK;
}

extern "C" int pqc_program_info(const pqc_program* p, int32_t* n_sweeps, int32_t* tile_qubits) {
  if (!p) return fail(PQC_ERR_INVALID, "program is NULL");
  if (n_sweeps) *n_sweeps = (int32_t)p->fwd.sweeps.size();
  if (tile_qubits) *tile_qubits = p->tile_qubits;
  return PQC_OK;
}

extern "C" int pqc_program_set_occupancy(pqc_program* p, int32_t ctas_per_sm) {
  return pqc_program_set_launch(p, ctas_per_sm, 0);
}

extern "C" int pqc_program_set_launch(pqc_program* p, int32_t ctas_per_sm, int32_t threads) {
  if (!p) return fail(PQC_ERR_INVALID, "program is NULL");
  if (ctas_per_sm != 0 && ctas_per_sm != 2 && ctas_per_sm != 3)
    return fail(PQC_ERR_INVALID, "ctas_per_sm must be 0 (default), 2 or 3");
  if (threads != 0 && threads != 256 && !(threads == 128 && ctas_per_sm == 3))
    return fail(PQC_ERR_INVALID, "threads must be 0 (default), 256, or 128 with 3 CTAs per SM");
  p->ctas_per_sm = ctas_per_sm;
  p->sweep_threads = threads;
  return PQC_OK;
}
