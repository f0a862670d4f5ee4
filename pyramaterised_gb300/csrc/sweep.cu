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

#include "sweep_ops.cuh"

namespace pqc {

// Launch shapes: THREADS per CTA and MINB resident CTAs per SM -- (512, 1) for 2^13-amplitude tiles, (256, 2),
// (256, 3) and (128, 3).  The register budget 65536 / (THREADS x MINB) sets the loops' ILP: 4 pairs (2 quads)
// per iteration at 128 registers or more, 2 pairs (1 quad) below.  Fewer threads per tile give each thread more
// amplitudes per op, which amortises the per-op dispatch; more CTAs per SM hide latency.
template <class A, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) sweep_kernel(const __grid_constant__ SweepDesc sd, const DOp* __restrict__ ops,
                                                    const int64_t* __restrict__ offs_g,
                                                    const float2* __restrict__ rowcoef, int coef_stride,
                                                    const float2* __restrict__ consts,
                                                    const double2* __restrict__ psi0, int64_t psi0_index, void* psi,
                                                    int n_qubits, int64_t tiles, int64_t row0, const RowCtl ctl,
                                                    const uint16_t* __restrict__ lazy_cols, int* __restrict__ status) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t s_bar;  // completion of the bulk tile load
  // Tile-constant state, kept by thread 0 in shared memory (registers are the kernel's limit): the pending
  // product of the scaled rotations' factors (see Rot) and the tile phase (ops on fixed bits only).
  __shared__ R s_scale, s_phr, s_phi;
  __shared__ int s_ph;
  const int k = sd.k, c = sd.c;
  const int nloc = 1 << k;
  Amp* x = reinterpret_cast<Amp*>(smem);
  int64_t* offs = reinterpret_cast<int64_t*>(smem + sizeof(Amp) * (size_t)nloc);
  Amp* tab = reinterpret_cast<Amp*>(smem + sizeof(Amp) * (size_t)nloc +
                                    ((sizeof(int64_t) * ((size_t)1 << (k - c)) + 15) & ~(size_t)15));
  uint16_t* itab = reinterpret_cast<uint16_t*>(reinterpret_cast<unsigned char*>(tab) + sizeof(Amp) * 256);
  DOp* sops = reinterpret_cast<DOp*>(reinterpret_cast<unsigned char*>(itab) + 512);
  float2* scf = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(sops) +
                                          ((sizeof(DOp) * (size_t)min(sd.n_ops, kOpChunk) + 15) & ~(size_t)15));
  const int64_t blk = blockIdx.x;
  const int64_t rloc = blk / tiles;
  const int64_t tile = blk - rloc * tiles;
  const int64_t row = row0 + rloc;
  const int64_t D = 1ll << n_qubits;
  const int lim = ctl.limit ? ctl.limit[row] : 0x7fffffff;
  const int st = ctl.start ? ctl.start[row] : 0;
  // a row that starts after every op of this middle sweep keeps its tile as it is in psi
  if (!sd.first && !sd.last && st > sd.max_gidx + 1) return;
  int64_t base = 0;
  for (int i = 0; i < sd.n_free; ++i)
    if ((tile >> i) & 1) base |= 1ll << sd.free_pos[i];
  const int nhi = 1 << (k - c);
  const int cmask = (1 << c) - 1;
  for (int i = threadIdx.x; i < nhi; i += blockDim.x) offs[i] = offs_g[sd.offs_begin + i];
  // Mid-circuit double-float tiles arrive as bulk copies on the TMA engine, one per run of 2^m amplitudes that
  // is contiguous both in the state and in the tile (local bits 0..m-1 are positions 0..m-1).  The complex64
  // mode keeps per-thread cp.async copies: bulk copies of its half-size tiles measured 14 % slower.
  int m = c;
  while (m < k && sd.local_of[m] == m) ++m;
  const unsigned run_bytes = (unsigned)sizeof(Amp) << m;
  const bool bulk = !sd.first && sizeof(Amp) == 16 && run_bytes >= 256;
  if (threadIdx.x == 0) {
    s_scale = A::rone();
    s_phr = A::rone();
    s_phi = A::rzero();
    s_ph = 0;
    if (bulk) mbar_init_expect(&s_bar, (unsigned)sizeof(Amp) << k);
  }
  // the first chunk of the sweep's ops (kOpChunk at a time, see stage_ops)
  int cb = 0, cn = min(kOpChunk, sd.n_ops);
  stage_ops(ops, sd.op_begin, cn, sops, scf, rowcoef, row, coef_stride, consts);
  __syncthreads();
  if (sd.first) {
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
      const int64_t g = base + offs[l >> c] + (l & cmask);
      x[l] = psi0 ? A::load_initial(psi0 + (ctl.psi0_row ? (int64_t)ctl.psi0_row[row] * D : 0), g)
                  : (g == psi0_index ? A::one() : A::zero());
    }
  } else if (bulk) {
    const Amp* src = reinterpret_cast<const Amp*>(psi) + row * D + base;
    for (int i = threadIdx.x; i < (1 << (k - m)); i += blockDim.x)
      bulk_g2s(x + ((size_t)i << m), src + offs[i << (m - c)], run_bytes, &s_bar);
    // bounded wait (1 s); a timeout is flagged and waited out once more; if the tile is still incomplete the
    // CTA leaves it as it is in psi (no compute, no write-back) and the status word reports the failed run
    const bool late = !mbar_wait(&s_bar, 0, 1000000000ull);
    if (__syncthreads_or(late)) {
      if (threadIdx.x == 0) atomicOr(status, PQC_STATUS_LOAD_TIMEOUT);
      const bool still_late = !mbar_wait(&s_bar, 0, 1000000000ull);
      if (__syncthreads_or(still_late)) return;
    }
  } else {
    const Amp* src = reinterpret_cast<const Amp*>(psi) + row * D + base;
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) cp_async<sizeof(Amp)>(x + l, src + offs[l >> c] + (l & cmask));
    cp_async_wait_all();
  }
  __syncthreads();
  // a phase that an op gave the whole tile: every thread computes it, thread 0 records it
  auto tile_phase = [&](R tr, R ti, bool tp) {
    if (tp && threadIdx.x == 0) {
      A::cacc(s_phr, s_phi, tr, ti);
      s_ph = 1;
    }
  };
  // log2 bound of the growth of the unscaled amplitudes since the pending factor was last applied; the
  // scaled rotations stop at 2^60 (amplitudes and the factor stay well inside the float range)
  constexpr int kMaxScaledGrowth = 60;
  int growth = 0;
  // Warp-blocked loops (see Split) when every warp owns at least 32 amplitude quads: ops on local bits
  // below S then stay inside one warp's sub-tile, and two such ops in a row need only __syncwarp.
  const int lognw = 31 - __clz((int)(blockDim.x >> 5));
  const int wl = (k - 2 - lognw >= 5) ? lognw : -1;
  const int S = wl >= 0 ? k - lognw : 0;
  bool prev_cross = false;
  auto fence = [&](bool cross) {
    if (cross || prev_cross)
      __syncthreads();
    else
      __syncwarp();
    prev_cross = cross;
  };
  int b = 0;  // relabelled sweeps: the tile's index offset
  for (int o = 0; o < sd.n_ops; ++o) {
    if (o >= cb + cn || o + op_extent(sops[o - cb]) > cb + cn) {  // stage the chunk that starts at op o
      __syncthreads();
      cb = o;
      cn = min(kOpChunk, sd.n_ops - o);
      stage_ops(ops, sd.op_begin + o, cn, sops, scf, rowcoef, row, coef_stride, consts);
      __syncthreads();
    }
    const int so = o - cb;  // op o in the staged chunk
    const DOp op = sops[so];
    if (sd.lazy) {
      if (op.kind == K_PHASEBLK) {
        fence(true);
        R tr = A::rone(), ti = A::rzero();
        bool tp = false;
        if (phase_block<A, true>(op, sops + so + 1, scf + 4 * (so + 1), sd, x, k, base, tab, itab,
                                 lazy_cols + (size_t)op.slot * kLazyRec, b, tr, ti, tp, lim, st, &s_scale))
          growth = 0;
        tile_phase(tr, ti, tp);
        o += op.aux;
        continue;
      }
      if (op.kind == K_ROT2) {
        const DOp m0 = sops[so + 1], m1 = sops[so + 2];
        Rot<A> r0, r1;
        const bool act0 = m0.gidx < lim && m0.gidx >= st, act1 = m1.gidx < lim && m1.gidx >= st;
        const int g = Rot<A>::scaled_growth(scf + 4 * (so + 1), act0) + Rot<A>::scaled_growth(scf + 4 * (so + 2), act1);
        if (Rot<A>::scalable(m0, act0) && Rot<A>::scalable(m1, act1) && growth + g <= kMaxScaledGrowth) {
          growth += g;
          r0.load_scaled(m0, scf + 4 * (so + 1), act0, threadIdx.x == 0 ? &s_scale : nullptr);
          r1.load_scaled(m1, scf + 4 * (so + 2), act1, threadIdx.x == 0 ? &s_scale : nullptr);
        } else {
          r0.load(m0, scf + 4 * (so + 1), act0);
          r1.load(m1, scf + 4 * (so + 2), act1);
        }
        fence((((int)(uint16_t)m0.c0 | (int)(uint16_t)m1.c0) >> S) != 0);
        rot2_lazy<A, (65536 / (THREADS * MINB) >= 128 ? 2 : 1)>(x, k, op, m0, m1, r0, r1, b, wl);
        o += 2;
        continue;
      }
      if (op.gidx >= lim || op.gidx < st) continue;
      if (op.kind == K_OFFSET) {
        if (op.aux == 0 || ((base >> op.p0) & 1)) b ^= (int)(uint16_t)op.c0;
        continue;
      }
      const float2* cf = op.kind == K_GEN1
                             ? (op.slot >= 0 ? rowcoef + ((size_t)row * coef_stride + op.slot) * 4
                                             : consts + (-op.slot - 1))
                             : scf + 4 * so;
      const int j0 = sd.local_of[op.p0];
      const int j1 = op.p1 >= 0 ? sd.local_of[op.p1] : -1;
      const int f0 = j0 < 0 ? (int)((base >> op.p0) & 1) : 0;
      const int f1 = (op.p1 >= 0 && j1 < 0) ? (int)((base >> op.p1) & 1) : 0;
      if (j0 < 0 && j1 < 0) {  // only the tile phase changes
        R tr = A::rone(), ti = A::rzero();
        bool tp = false;
        apply_op<A, 2>(op, x, k, j0, j1, f0, f1, cf, tr, ti, tp, wl);
        tile_phase(tr, ti, tp);
        continue;
      }
      const bool elementwise = op.kind == K_RZ || op.kind == K_DIAG1 || op.kind == K_RZZ || op.kind == K_CZ;
      fence(!elementwise && ((((int)(uint16_t)op.c0 | (int)(uint16_t)op.c1) >> S) != 0));
      apply_op_lazy<A, (65536 / (THREADS * MINB) >= 128 ? 4 : 2)>(op, x, k, j0, j1, f0, f1, cf, b, wl);
      continue;
    }
    if (op.kind == K_PHASEBLK) {
      fence(true);
      R tr = A::rone(), ti = A::rzero();
      bool tp = false;
      if (phase_block<A, false>(op, sops + so + 1, scf + 4 * (so + 1), sd, x, k, base, tab, itab, nullptr, 0, tr, ti,
                                tp, lim, st, &s_scale))
        growth = 0;
      tile_phase(tr, ti, tp);
      o += op.aux;
      continue;
    }
    if (op.kind == K_ROT2) {
      const DOp m0 = sops[so + 1], m1 = sops[so + 2];
      const int ja = sd.local_of[m0.p0], jb = sd.local_of[m1.p0];
      Rot<A> r0, r1;
      const bool act0 = m0.gidx < lim && m0.gidx >= st, act1 = m1.gidx < lim && m1.gidx >= st;
      const int g = Rot<A>::scaled_growth(scf + 4 * (so + 1), act0) + Rot<A>::scaled_growth(scf + 4 * (so + 2), act1);
      if (Rot<A>::scalable(m0, act0) && Rot<A>::scalable(m1, act1) && growth + g <= kMaxScaledGrowth) {
        growth += g;
        r0.load_scaled(m0, scf + 4 * (so + 1), act0, threadIdx.x == 0 ? &s_scale : nullptr);
        r1.load_scaled(m1, scf + 4 * (so + 2), act1, threadIdx.x == 0 ? &s_scale : nullptr);
      } else {
        r0.load(m0, scf + 4 * (so + 1), act0);
        r1.load(m1, scf + 4 * (so + 2), act1);
      }
      fence(ja >= S || jb >= S);
      rot2<A, (65536 / (THREADS * MINB) >= 128 ? 2 : 1)>(x, k, ja, jb, r0, r1, wl);
      o += 2;
      continue;
    }
    // generators (sel >= 0) sit between op gidx and op gidx + 1
    if ((op.sel >= 0 && op.sel != row) || op.gidx >= lim || op.gidx + (op.sel >= 0 ? 1 : 0) < st) continue;
    const float2* cf = (op.kind == K_GEN1 || op.kind == K_GEN2)
                           ? (op.slot >= 0 ? rowcoef + ((size_t)row * coef_stride + op.slot) * 4 : consts + (-op.slot - 1))
                           : scf + 4 * so;
    const int j0 = sd.local_of[op.p0];
    const int j1 = op.p1 >= 0 ? sd.local_of[op.p1] : -1;
    const int f0 = j0 < 0 ? (int)((base >> op.p0) & 1) : 0;
    const int f1 = (op.p1 >= 0 && j1 < 0) ? (int)((base >> op.p1) & 1) : 0;
    // element-wise kinds touch each amplitude from the thread that owns it; the others cross warps when
    // one of their local bits is at or above S
    const bool elementwise = op.kind == K_RZ || op.kind == K_DIAG1 || op.kind == K_RZZ;
    fence(!elementwise && (j0 >= S || j1 >= S));
    R tr = A::rone(), ti = A::rzero();
    bool tp = false;
    apply_op<A, (65536 / (THREADS * MINB) >= 128 ? 4 : 2)>(op, x, k, j0, j1, f0, f1, cf, tr, ti, tp, wl);
    tile_phase(tr, ti, tp);
  }
  __syncthreads();
  // the pending factor of scaled rotations joins the tile phase, or is a real scale at write-out
  const R scale = s_scale;
  R phr = s_phr, phi = s_phi;
  const bool ph = s_ph != 0;
  const bool sc = !A::is_unit(scale);
  if (sc && ph) {
    phr = A::rmul(phr, scale);
    phi = A::rmul(phi, scale);
  }
  if (sd.lazy) {  // logical index l lives at slot A l ^ b
    build_index_tables(lazy_cols + (size_t)sd.out_rec * kLazyRec, k, itab);
    __syncthreads();
  }
  for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
    const int64_t g = base + offs[l >> c] + (l & cmask);
    Amp v = x[sd.lazy ? (map_index(itab, l) ^ b) : l];
    if (ph)
      v = A::cm(phr, phi, v);
    else if (sc)
      v = A::scale(scale, v);
    if (sd.last)
      A::store_final(psi, row * D + g, v);
    else
      A::store_mid(psi, row * D + g, v);
  }
}

// the opt-in dynamic shared memory limit of a kernel: the device's per-block maximum less its static use
template <class K>
static int allow_max_dynamic_smem(K kernel) {
  int dev = 0, optin = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  PQC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  PQC_CUDA(cudaFuncGetAttributes(&fa, kernel));
  PQC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  return PQC_OK;
}

// The native FP64 arm is instantiated in two shapes only, (512, 1) at 2^13-amplitude tiles and (256, 2)
// below: it is bound by the FP64 pipe, not by latency, and its loops want the larger register budget.
template <class A>
constexpr bool kFp64 = std::is_same<A, ArithF64>::value;

template <class A>
static int set_sweep_attrs() {
  int rc = allow_max_dynamic_smem(sweep_kernel<A, 512, 1>);
  if (!rc) rc = allow_max_dynamic_smem(sweep_kernel<A, 256, 2>);
  if constexpr (!kFp64<A>) {
    if (!rc) rc = allow_max_dynamic_smem(sweep_kernel<A, 256, 3>);
    if (!rc) rc = allow_max_dynamic_smem(sweep_kernel<A, 128, 3>);
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

template <class A>
static int run_plan_impl(const pqc_program* prog, const Plan& plan_in, int coef_stride, const float2* rowcoef,
                         const float2* consts, int64_t rows, const void* psi0, int64_t psi0_index, void* psi,
                         cudaStream_t stream, const int32_t* row_limit, const RowCtl* ctl_in = nullptr) {
  RowCtl ctl = ctl_in ? *ctl_in : RowCtl{};
  if (row_limit) ctl.limit = row_limit;
  const Plan& plan =
      (&plan_in == &prog->fwd && prog->fwd_lazy && (ctl.limit || ctl.start || ctl.psi0_row)) ? prog->fwd_lim : plan_in;
  using Amp = typename A::Amp;
  const int N = prog->n_qubits;
  static int attr_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    int rc = set_sweep_attrs<A>();
    if (rc) return rc;
    attr_dev = dev;
  }
  for (size_t si = 0; si < plan.sweeps.size(); ++si) {
    const SweepDesc& sd = plan.sweeps[si];
    const int64_t tiles = 1ll << (N - sd.k);
    const size_t smem = sizeof(Amp) * ((size_t)1 << sd.k) +
                        ((sizeof(int64_t) * ((size_t)1 << (sd.k - sd.c)) + 15) & ~(size_t)15) + sizeof(Amp) * 256 +
                        512 + ((sizeof(DOp) * (size_t)std::min(sd.n_ops, kOpChunk) + 15) & ~(size_t)15) +
                        sizeof(float2) * 4 * (size_t)std::min(sd.n_ops, kOpChunk);
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
#define PQC_SWEEP_LAUNCH(T, MB)                                                                            \
  sweep_kernel<A, T, MB><<<grid, T, smem, stream>>>(sd, plan.d_ops, plan.d_offs, rowcoef, coef_stride, consts,   \
                                                    (const double2*)psi0, psi0_index, psi, N, tiles, r0, ctl,    \
                                                    plan.d_lazy_cols, prog->d_status)
      if (threads == 512) {
        PQC_SWEEP_LAUNCH(512, 1);
      } else if (threads == 256 && minb == 2) {
        PQC_SWEEP_LAUNCH(256, 2);
      } else {
        if constexpr (!kFp64<A>) {
          if (threads == 128)
            PQC_SWEEP_LAUNCH(128, 3);
          else
            PQC_SWEEP_LAUNCH(256, 3);
        }
      }
#undef PQC_SWEEP_LAUNCH
      count_launch();
      PQC_CUDA(cudaGetLastError());
    }
  }
  return PQC_OK;
}

int run_plan_df(const pqc_program* prog, const Plan& plan, int coef_stride, const float2* rowcoef,
                const float2* consts, int64_t rows, const void* psi0, int64_t psi0_index, void* psi,
                cudaStream_t stream, const int32_t* row_limit, const RowCtl* ctl) {
  return run_plan_impl<ArithDF>(prog, plan, coef_stride, rowcoef, consts, rows, psi0, psi0_index, psi, stream,
                                row_limit, ctl);
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
  if (identity_rows(gens, n_runs, n_rows))
    return run_plan_df(prog, prog->deriv_plan, 0, b.cdf, b.kdf, n_runs, psi0, psi0_index, dpsi, stream, nullptr,
                       &ctl);
  char* runs = (char*)workspace + cw;
  const int32_t* row_of = prog->d_run_row;  // uploaded with the cached plan
  rc = run_plan_df(prog, prog->deriv_plan, 0, b.cdf, b.kdf, n_runs, psi0, psi0_index, runs, stream, nullptr, &ctl);
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
