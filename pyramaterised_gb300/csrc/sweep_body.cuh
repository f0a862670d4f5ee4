// The body of the fused shared-memory sweep (one CTA = one tile of one row), shared by the single-program
// sweep kernel (sweep.cu) and the multi-program kernel (multi.cu).  See sweep.cu for the method.
#pragma once
#include "sweep_ops.cuh"

namespace pqc {

// Launch shapes: THREADS per CTA and MINB resident CTAs per SM -- (512, 1) for 2^13-amplitude tiles, (256, 2),
// (256, 3) and (128, 3).  The register budget 65536 / (THREADS x MINB) sets the loops' ILP: 4 pairs (2 quads)
// per iteration at 128 registers or more, 2 pairs (1 quad) below.  Fewer threads per tile give each thread more
// amplitudes per op, which amortises the per-op dispatch; more CTAs per SM hide latency.
//
// sweep_body is the whole work of one CTA: tile `blk` (rows x tiles of a launch, row-major) of sweep `sd`.  The
// single-program kernel (sweep.cu) passes its __grid_constant__ descriptor; the multi-program kernel (multi.cu)
// a shared-memory copy of the descriptor of the program its CTA serves.
//
// ol_arg: the op list the dual kernel's CTA runs, sd's own or that of the sweep's unrelabelled twin (same
// geometry); the other kernels read sd's (GENS false).  GENS: the relabelled sweeps may hold derivative generators (K_PAULI ops run by one row,
// placed after op gidx); only the dual kernels are instantiated with it.
struct OpList {
  int32_t op_begin, n_ops, lazy, out_rec;
};
__device__ __forceinline__ OpList op_list(const SweepDesc& sd) {
  return {sd.op_begin, sd.n_ops, sd.lazy, sd.out_rec};
}

template <class A, int THREADS, int MINB, bool GENS = false>
__device__ __forceinline__ void sweep_body(const SweepDesc& sd, const OpList ol_arg, const DOp* __restrict__ ops,
                                           const int64_t* __restrict__ offs_g, const float2* __restrict__ rowcoef,
                                           int coef_stride, const float2* __restrict__ consts,
                                           const double2* __restrict__ psi0, int64_t psi0_index, void* psi,
                                           int n_qubits, int64_t tiles, int64_t row0, const RowCtl& ctl,
                                           const uint16_t* __restrict__ lazy_cols, int* __restrict__ status,
                                           int64_t blk) {
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
  const int n_staged = min((GENS ? ol_arg.n_ops : sd.n_ops), kOpChunk);
  float2* scf = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(sops) +
                                          ((sizeof(DOp) * (size_t)n_staged + 15) & ~(size_t)15));
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
  int cb = 0, cn = min(kOpChunk, (GENS ? ol_arg.n_ops : sd.n_ops));
  stage_ops(ops, (GENS ? ol_arg.op_begin : sd.op_begin), cn, sops, scf, rowcoef, row, coef_stride, consts);
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
  for (int o = 0; o < (GENS ? ol_arg.n_ops : sd.n_ops); ++o) {
    if (o >= cb + cn || o + op_extent(sops[o - cb]) > cb + cn) {  // stage the chunk that starts at op o
      __syncthreads();
      cb = o;
      cn = min(kOpChunk, (GENS ? ol_arg.n_ops : sd.n_ops) - o);
      stage_ops(ops, (GENS ? ol_arg.op_begin : sd.op_begin) + o, cn, sops, scf, rowcoef, row, coef_stride, consts);
      __syncthreads();
    }
    const int so = o - cb;  // op o in the staged chunk
    const DOp op = sops[so];
    if ((GENS ? ol_arg.lazy : sd.lazy)) {
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
      if constexpr (GENS) {
        if ((op.sel >= 0 && op.sel != row) || op.gidx >= lim || op.gidx + (op.sel >= 0 ? 1 : 0) < st) continue;
      } else {
        if (op.gidx >= lim || op.gidx < st) continue;
      }
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
      if constexpr (GENS) {
        if (op.kind == K_PAULI) {
          apply_pauli_lazy<A>(op, x, k, j0, j1, f0, f1, cf, b, wl);
          continue;
        }
      }
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
      if (!act0 && !act1) {  // the row's start or limit excludes both rotations
        o += 2;
        continue;
      }
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
  if ((GENS ? ol_arg.lazy : sd.lazy)) {  // logical index l lives at slot A l ^ b
    build_index_tables(lazy_cols + (size_t)(GENS ? ol_arg.out_rec : sd.out_rec) * kLazyRec, k, itab);
    __syncthreads();
  }
  for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
    const int64_t g = base + offs[l >> c] + (l & cmask);
    Amp v = x[(GENS ? ol_arg.lazy : sd.lazy) ? (map_index(itab, l) ^ b) : l];
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

}  // namespace pqc
