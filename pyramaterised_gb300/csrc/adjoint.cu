// Adjoint energy gradient with fused double-float sweeps.
//
// Replaces `Measurements.get_gradient_vector` (pyramaterised/measure.py:461-471),
// which builds every derivative state |d_j psi> by re-running the circuit with
// the gate replaced by `deriv * gate` (circuit.py:149-192) and then takes
// 2 Re <psi|H|d_j psi>.  Here, with psi the final state and lambda = H psi:
//   dE/dtheta_j = sum over the generator terms G of column j, inserted after
//                 forward op i, of 2 Re <lambda_i| G |psi_i>,
//   psi_{i-1} = U_i^dagger psi_i,  lambda_{i-1} = U_i^dagger lambda_i.
// The reverse pass is the forward machinery run on the inverse program
// (reversed ops, negated angles, conjugate-transposed fixed matrices) over
// psi and lambda tiles together, with "measure" ops at the generator points
// that reduce <lambda|G|psi> over each tile in double-float.
#include <algorithm>

#include <cstring>
#include <string>

#include "dfacc.cuh"
#include "sweep_ops.cuh"

namespace pqc {

// U^dagger of a forward op.
static int inverse_op(const pqc_op& o, pqc_op& inv) {
  inv = o;
  switch (o.kind) {
    case PQC_OP_RX:
    case PQC_OP_RY:
    case PQC_OP_RZ:
    case PQC_OP_RXX:
    case PQC_OP_RYY:
    case PQC_OP_RZZ:
    case PQC_OP_FSIM:  // fsim(t, p)^dagger = fsim(-t, -p)
    case PQC_OP_FIXED_FSIM:
      inv.scale = -o.scale;
      inv.offset = -o.offset;
      inv.scale2 = -o.scale2;
      inv.offset2 = -o.offset2;
      return PQC_OK;
    case PQC_OP_MAT1:
    case PQC_OP_MAT2: {
      const int n = o.kind == PQC_OP_MAT1 ? 2 : 4;
      for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
          inv.m[2 * (n * r + c)] = o.m[2 * (n * c + r)];
          inv.m[2 * (n * r + c) + 1] = -o.m[2 * (n * c + r) + 1];
        }
      return PQC_OK;
    }
    case PQC_OP_CNOT:
    case PQC_OP_CZ:
      return PQC_OK;
    default:
      return fail(PQC_ERR_UNSUPPORTED, "adjoint: no inverse for op kind " + std::to_string(o.kind));
  }
}

static bool same_ops(const std::vector<pqc_op>& a, const pqc_op* b, int n) {
  if ((int)a.size() != n) return false;
  for (int i = 0; i < n; ++i)
    if (memcmp(&a[i], &b[i], sizeof(pqc_op)) != 0) return false;
  return true;
}

void free_adjoint(pqc_program* p) {
  free_table(p->adj_t);
  free_plan(p->adj_plan);
  free_plan(p->adj_plan_lim);
  p->adj_lazy = false;
  if (p->d_adj_cols) cudaFree(p->d_adj_cols);
  if (p->d_adj_start) cudaFree(p->d_adj_start);
  p->d_adj_cols = p->d_adj_start = nullptr;
  p->adj_valid = false;
}

int64_t adjoint_tiles(const pqc_program* p) {
  return p->adj_plan.sweeps.empty() ? 1 : (1ll << (p->n_qubits - p->adj_plan.sweeps[0].k));
}

static bool z_type(const DOp& d) {
  const int l0 = d.aux & 0xff, l1 = (d.aux >> 8) & 0xff;
  return d.kind == K_MEASURE && (l0 == 0 || l0 == 3) && (l1 == 0 || l1 == 3);
}

// Runs of consecutive measures become groups of up to 4 reduced in one pass: [K_MEASZ(n), m_1 .. m_n]
// when all are Z-type (they share the products conj(lambda_j) psi_j), else [K_MEASG(n), ...].
static void group_z_measures(Plan& plan) {
  std::vector<DOp> ops;
  ops.reserve(plan.ops.size() + plan.ops.size() / 4 + 1);
  for (SweepDesc& sd : plan.sweeps) {
    const int begin = (int)ops.size();
    int j = 0;
    while (j < sd.n_ops) {
      const DOp& o = plan.ops[sd.op_begin + j];
      if (o.kind == K_PHASEBLK || o.kind == K_ROT2) {
        const int n = o.kind == K_PHASEBLK ? o.aux : 2;
        for (int r = 0; r <= n; ++r) ops.push_back(plan.ops[sd.op_begin + j + r]);
        j += n + 1;
        continue;
      }
      int run = 0;
      bool all_z = true;
      while (j + run < sd.n_ops && run < 4 && plan.ops[sd.op_begin + j + run].kind == K_MEASURE) {
        all_z = all_z && z_type(plan.ops[sd.op_begin + j + run]);
        ++run;
      }
      if (run >= 2) {
        DOp m;
        m.kind = all_z ? K_MEASZ : K_MEASG;
        m.sel = -1;
        m.p0 = 0;
        m.p1 = -1;
        m.slot = 0;
        m.aux = run;
        m.gidx = -1;
        ops.push_back(m);
        for (int r = 0; r < run; ++r) ops.push_back(plan.ops[sd.op_begin + j + r]);
        j += run;
        continue;
      }
      ops.push_back(o);
      ++j;
    }
    sd.op_begin = begin;
    sd.n_ops = (int)ops.size() - begin;
  }
  plan.ops.swap(ops);
}

// Build (or reuse) the reverse plan for generators `gens` (PQC_OP_PAULI, sel = column).
int ensure_adjoint(pqc_program* p, const pqc_op* gens, const int32_t* after, int n_gens, int n_cols) {
  if (p->adj_valid && same_ops(p->adj_gens, gens, n_gens) &&
      std::equal(p->adj_after.begin(), p->adj_after.end(), after) && p->adj_ncols == n_cols)
    return PQC_OK;
  const int n = (int)p->ops.size();
  for (int t = 0; t < n_gens; ++t) {
    if (gens[t].kind != PQC_OP_PAULI) return fail(PQC_ERR_UNSUPPORTED, "adjoint generators must be Pauli terms");
    if (after[t] < -1 || after[t] >= n) return fail(PQC_ERR_INVALID, "gen_after out of range");
    if (gens[t].sel < 0 || gens[t].sel >= n_cols) return fail(PQC_ERR_INVALID, "gens[t].sel outside [0, n_cols)");
  }
  free_adjoint(p);
  std::vector<pqc_op> all(n + n_gens);
  for (int i = 0; i < n; ++i) {
    int rc = inverse_op(p->ops[i], all[i]);
    if (rc) return rc;
  }
  for (int t = 0; t < n_gens; ++t) {
    all[n + t] = gens[t];
    all[n + t].sel = -1;
  }
  int rc = lower_ops(all.data(), (int)all.size(), p->n_qubits, p->adj_t);
  if (rc) return rc;
  for (int i = 0; i < n; ++i) p->adj_t.dops[i].gidx = i;
  for (int t = 0; t < n_gens; ++t) {
    DOp& d = p->adj_t.dops[n + t];
    d.kind = K_MEASURE;
    d.sel = t;
    d.gidx = after[t];
  }
  std::vector<std::vector<int>> at(n + 1);
  for (int t = 0; t < n_gens; ++t) at[after[t] + 1].push_back(t);
  std::vector<DOp> seq;
  seq.reserve(all.size());
  for (int i = n - 1; i >= -1; --i) {
    for (int t : at[i + 1]) seq.push_back(p->adj_t.dops[n + t]);
    if (i >= 0) seq.push_back(p->adj_t.dops[i]);
  }
  // A measure reads psi and lambda without changing them, and an op U applied to both tiles leaves
  // <lambda|P|psi> unchanged when U commutes with P: ops on other qubits, and diagonal ops when P is
  // Z-type.  Two passes regroup the measures so that they share passes and stop splitting the runs of
  // ops that fuse: (1) each measure sinks (moves later) past the ops that commute with it; when an op
  // does not commute with one of the waiting measures, all of them are emitted before it.  Z-type
  // measures thereby gather behind runs of diagonal ops.  (2) each measure then rises (moves earlier)
  // past single-qubit rotations on other qubits, so consecutive rotations are no longer split.
  {
    auto qubits = [](const DOp& d) {
      uint64_t m = 1ull << d.p0;
      if (d.p1 >= 0) m |= 1ull << d.p1;
      return m;
    };
    auto diagonal = [](const DOp& d) {
      return d.kind == K_RZ || d.kind == K_DIAG1 || d.kind == K_CZ || d.kind == K_RZZ;
    };
    auto z_only = [](const DOp& d) {
      const int l0 = d.aux & 0xff, l1 = (d.aux >> 8) & 0xff;
      return (l0 == 0 || l0 == 3) && (l1 == 0 || l1 == 3);
    };
    auto commute = [&](const DOp& m, const DOp& d) {
      return (qubits(m) & qubits(d)) == 0 || (z_only(m) && diagonal(d));
    };
    std::vector<DOp> sunk, waiting;
    sunk.reserve(seq.size());
    for (const DOp& d : seq) {
      if (d.kind == K_MEASURE) {
        waiting.push_back(d);
        continue;
      }
      bool ok = true;
      for (const DOp& m : waiting) ok = ok && commute(m, d);
      if (!ok) {
        sunk.insert(sunk.end(), waiting.begin(), waiting.end());
        waiting.clear();
      }
      sunk.push_back(d);
    }
    sunk.insert(sunk.end(), waiting.begin(), waiting.end());
    auto rotation = [](const DOp& d) {
      return d.sel < 0 && d.p1 < 0 && (d.kind == K_RY || d.kind == K_RX || d.kind == K_REAL2 || d.kind == K_GEN1);
    };
    std::vector<DOp> risen;
    risen.reserve(sunk.size());
    for (const DOp& d : sunk) {
      size_t pos = risen.size();
      if (d.kind == K_MEASURE)
        while (pos > 0 && rotation(risen[pos - 1]) && commute(d, risen[pos - 1])) --pos;
      risen.insert(risen.begin() + pos, d);
    }
    seq.swap(risen);
  }
  // A measure of a Z-type Pauli string is unchanged by diagonal ops applied to both tiles
  // (<D lambda|Z|D psi> = <lambda|Z|psi>), so inside every run of diagonal ops and Z-type measures the
  // measures move to the front; the diagonal ops then stay adjacent and fuse into one phase-table pass.
  {
    auto diag_op = [](const DOp& d) {
      return d.sel < 0 && (d.kind == K_RZ || d.kind == K_DIAG1 || d.kind == K_CZ || d.kind == K_RZZ);
    };
    auto z_measure = [](const DOp& d) {
      const int l0 = d.aux & 0xff, l1 = (d.aux >> 8) & 0xff;
      return d.kind == K_MEASURE && (l0 == 0 || l0 == 3) && (l1 == 0 || l1 == 3);
    };
    size_t i = 0;
    while (i < seq.size()) {
      size_t j = i;
      while (j < seq.size() && (diag_op(seq[j]) || z_measure(seq[j]))) ++j;
      if (j > i + 1) std::stable_partition(seq.begin() + i, seq.begin() + j, z_measure);
      i = j > i ? j : i + 1;
    }
  }
  const int k = std::min(kAdjTileQubits, (int)p->n_qubits);
  rc = build_plan(seq, p->n_qubits, k, 4, p->adj_plan);
  if (rc) return rc;
  for (const SweepDesc& sd : p->adj_plan.sweeps)
    if (sd.k != k) return fail(PQC_ERR_INVALID, "adjoint plan: sweeps of different widths");
  fuse_diagonal_runs(p->adj_plan);
  p->adj_plan_lim = p->adj_plan;
  relabel_cnots(p->adj_plan, true);
  for (const SweepDesc& sd : p->adj_plan.sweeps) p->adj_lazy = p->adj_lazy || sd.lazy;
  for (Plan* pl : {&p->adj_plan, &p->adj_plan_lim}) {
    fuse_rotation_pairs(*pl);
    group_z_measures(*pl);
    finalize_plan(*pl);
  }
  if (!p->adj_lazy) p->adj_plan_lim = Plan();
  rc = upload_table(p->adj_t);
  if (!rc) rc = upload_plan(p->adj_plan);
  if (!rc && p->adj_lazy) rc = upload_plan(p->adj_plan_lim);
  if (rc) return rc;
  // measures grouped by column (CSR)
  std::vector<int32_t> start(n_cols + 1, 0), order;
  for (int t = 0; t < n_gens; ++t) start[gens[t].sel + 1]++;
  for (int c = 0; c < n_cols; ++c) start[c + 1] += start[c];
  order.resize(n_gens);
  std::vector<int32_t> fill(start.begin(), start.end() - 1);
  for (int t = 0; t < n_gens; ++t) order[fill[gens[t].sel]++] = t;
  PQC_CUDA(cudaMalloc(&p->d_adj_cols, std::max<size_t>(1, order.size()) * sizeof(int32_t)));
  PQC_CUDA(cudaMalloc(&p->d_adj_start, start.size() * sizeof(int32_t)));
  if (!order.empty())
    PQC_CUDA(cudaMemcpy(p->d_adj_cols, order.data(), order.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  PQC_CUDA(cudaMemcpy(p->d_adj_start, start.data(), start.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  p->adj_gens.assign(gens, gens + n_gens);
  p->adj_after.assign(after, after + n_gens);
  p->adj_ncols = n_cols;
  p->adj_valid = true;
  return PQC_OK;
}

// One reverse sweep over psi and lambda tiles.  mpart[row][t][tile] receives
// 2 Re(w_t <lambda|P_t|psi>) for each measure t of this sweep (w_t = coef i^{n_y}).
__global__ void __launch_bounds__(256, 3)
    adj_sweep_kernel(const __grid_constant__ SweepDesc sd, const DOp* __restrict__ ops,
                     const int64_t* __restrict__ offs_g, const float2* __restrict__ rowcoef, int coef_stride,
                     const float2* __restrict__ consts, const double* __restrict__ dconsts, void* psi, void* lam,
                     int n_qubits, int64_t tiles, int64_t row0, const int32_t* __restrict__ row_limit, int n_meas,
                     double* __restrict__ mpart, const uint16_t* __restrict__ lazy_cols) {
  using A = ArithDF;
  using Amp = cdf;
  using R = df;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float2 wsum[8][2];
  __shared__ float2 gsum[8][4][2];
  const int k = sd.k, c = sd.c;
  const int nloc = 1 << k;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  size_t off = 0;
  Amp* x = reinterpret_cast<Amp*>(smem);
  off += sizeof(Amp) * (size_t)nloc;
  Amp* y = reinterpret_cast<Amp*>(smem + off);
  off += sizeof(Amp) * (size_t)nloc;
  int64_t* offs = reinterpret_cast<int64_t*>(smem + off);
  off += (sizeof(int64_t) * ((size_t)1 << (k - c)) + 15) & ~(size_t)15;
  Amp* tab = reinterpret_cast<Amp*>(smem + off);
  off += sizeof(Amp) * 256;
  uint16_t* itab = reinterpret_cast<uint16_t*>(smem + off);
  off += 512;
  DOp* sops = reinterpret_cast<DOp*>(smem + off);
  off += (sizeof(DOp) * (size_t)min(sd.n_ops, kOpChunk) + 15) & ~(size_t)15;
  float2* scf = reinterpret_cast<float2*>(smem + off);

  const int64_t blk = blockIdx.x;
  const int64_t rloc = blk / tiles;
  const int64_t tile = blk - rloc * tiles;
  const int64_t row = row0 + rloc;
  const int64_t D = 1ll << n_qubits;
  int64_t base = 0;
  for (int i = 0; i < sd.n_free; ++i)
    if ((tile >> i) & 1) base |= 1ll << sd.free_pos[i];
  const int nhi = 1 << (k - c);
  const int cmask = (1 << c) - 1;
  for (int i = threadIdx.x; i < nhi; i += blockDim.x) offs[i] = offs_g[sd.offs_begin + i];
  // the first chunk of the sweep's ops (kOpChunk at a time, see stage_ops)
  int cb = 0, cn = min(kOpChunk, sd.n_ops);
  stage_ops(ops, sd.op_begin, cn, sops, scf, rowcoef, row, coef_stride, consts);
  __syncthreads();
  if (sd.first) {
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
      const int64_t g = row * D + base + offs[l >> c] + (l & cmask);
      x[l] = A::load_initial((const double2*)psi, g);
      y[l] = A::load_initial((const double2*)lam, g);
    }
  } else {
    const Amp* sx = reinterpret_cast<const Amp*>(psi) + row * D + base;
    const Amp* sy = reinterpret_cast<const Amp*>(lam) + row * D + base;
    for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
      const int64_t g = offs[l >> c] + (l & cmask);
      cp_async<sizeof(Amp)>(x + l, sx + g);
      cp_async<sizeof(Amp)>(y + l, sy + g);
    }
    cp_async_wait_all();
  }
  __syncthreads();
  R pxr = A::rone(), pxi = A::rzero(), pyr = A::rone(), pyi = A::rzero();
  bool phx = false, phy = false;
  const int lim = row_limit ? row_limit[row] : 0x7fffffff;
  // relabelled sweeps (SweepDesc::lazy): logical index l of both tiles lives at slot A l ^ b; bx is b in
  // that mode and 0 otherwise, so the measures below read parities of (slot ^ bx)
  const bool lz = sd.lazy != 0;
  int b = 0;
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
    const int bx = lz ? b : 0;
    if (op.kind == K_PHASEBLK) {
      // one pair of phase tables serves both tiles
      const PhaseSplit ps = phase_split(op);
      const DOp* blk = sops + so + 1;
      const float2* bcf = scf + 4 * (so + 1);
      R cr = A::rone(), ci = A::rzero();
      bool cph = false;
      const int use = phase_tables<A>(blk, bcf, ps, sd, k, base, tab, cr, ci, cph, lim, 0);
      if (cph) {
        A::cacc(pxr, pxi, cr, ci);
        A::cacc(pyr, pyi, cr, ci);
        phx = phy = true;
      }
      if (use) {
        if (lz) build_index_tables(lazy_cols + (size_t)op.slot * kLazyRec, k, itab);
        __syncthreads();
        // one copy of each loop for both tiles (the kernel's size, not its arithmetic, is at stake)
#pragma unroll 1
        for (int w = 0; w < 2; ++w) {
          if (lz)
            phase_apply<A, true>(w ? y : x, k, ps.kl, tab, use, itab, b);
          else
            phase_apply<A, false>(w ? y : x, k, ps.kl, tab, use, itab, b);
        }
      }
#pragma unroll 1
      for (int w = 0; w < 2; ++w) {
        R& qr = w ? pyr : pxr;
        R& qi = w ? pyi : pxi;
        bool& qh = w ? phy : phx;
        if (lz)
          phase_mid<A, true>(blk, bcf, ps, sd, w ? y : x, k, b, qr, qi, qh, lim, 0);
        else
          phase_mid<A, false>(blk, bcf, ps, sd, w ? y : x, k, b, qr, qi, qh, lim, 0);
      }
      o += op.aux;
      __syncthreads();
      continue;
    }
    if (op.kind == K_ROT2) {
      const DOp m0 = sops[so + 1], m1 = sops[so + 2];
      const int ja = sd.local_of[m0.p0], jb = sd.local_of[m1.p0];
      Rot<A> r0, r1;
      r0.load(m0, scf + 4 * (so + 1), m0.gidx < lim);
      r1.load(m1, scf + 4 * (so + 2), m1.gidx < lim);
#pragma unroll 1
      for (int w = 0; w < 2; ++w) {
        if (lz)
          rot2_lazy<A, 1, true>(w ? y : x, k, op, m0, m1, r0, r1, b, -1);
        else
          rot2<A, 1, true>(w ? y : x, k, ja, jb, r0, r1);
      }
      o += 2;
      __syncthreads();
      continue;
    }
    if (op.kind == K_OFFSET) {  // relabelled sweeps only; measures of skipped rows do not depend on it
      if (op.aux == 0 || ((base >> op.p0) & 1)) b ^= (int)(uint16_t)op.c0;
      continue;
    }
    if (op.kind == K_MEASZ) {
      // up to 4 Z-type measures: S_t = sum_j (-1)^{parity(j & z_t) ^ zf_t} conj(y_j) x_j
      const int n = op.aux;
      int zl[4], zf[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        zl[t] = 0;
        zf[t] = 0;
        if (t < n) {
          const DOp m = sops[so + 1 + t];
          const int l0 = m.aux & 0xff, l1 = (m.aux >> 8) & 0xff;
          const int a0 = sd.local_of[m.p0], a1 = m.p1 >= 0 ? sd.local_of[m.p1] : -1;
          if (l0 == 3) {
            if (a0 >= 0) zl[t] ^= lz ? (int)(uint16_t)m.r0 : (1 << a0);
            else zf[t] ^= (int)((base >> m.p0) & 1);
          }
          if (l1 == 3) {
            if (a1 >= 0) zl[t] ^= lz ? (int)(uint16_t)m.r1 : (1 << a1);
            else zf[t] ^= (int)((base >> m.p1) & 1);
          }
        }
      }
      Acc ar[4], ai[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) ar[t] = ai[t] = Acc{0.f, 0.f};
      for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
        const Amp u = y[j], v = x[j];
        const int jb = j ^ bx;
        Acc wr{0.f, 0.f}, wi{0.f, 0.f};
        acc_mul(wr, u.rh, u.rl, v.rh, v.rl);
        acc_mul(wr, u.ih, u.il, v.ih, v.il);
        acc_mul(wi, u.rh, u.rl, v.ih, v.il);
        acc_mul(wi, -u.ih, -u.il, v.rh, v.rl);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (t >= n) break;
          const bool neg = (__popc(jb & zl[t]) & 1) ^ zf[t];
          acc_add(ar[t], neg ? -wr.h : wr.h, neg ? -wr.l : wr.l);
          acc_add(ai[t], neg ? -wi.h : wi.h, neg ? -wi.l : wi.l);
        }
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (t >= n) break;
        ar[t] = warp_sum_df(ar[t]);
        ai[t] = warp_sum_df(ai[t]);
        if (lane == 0) {
          gsum[wid][t][0] = make_float2(ar[t].h, ar[t].l);
          gsum[wid][t][1] = make_float2(ai[t].h, ai[t].l);
        }
      }
      __syncthreads();
      if (threadIdx.x < n) {
        const int t = threadIdx.x;
        const DOp m = sops[so + 1 + t];
        if (m.gidx < lim) {
          Acc a{0.f, 0.f}, b{0.f, 0.f};
          for (int w = 0; w < nw; ++w) {
            acc_add(a, gsum[w][t][0].x, gsum[w][t][0].y);
            acc_add(b, gsum[w][t][1].x, gsum[w][t][1].y);
          }
          const double Sr = (double)a.h + (double)a.l, Si = (double)b.h + (double)b.l;
          const double* cd = dconsts + (-m.slot - 1);
          mpart[((int64_t)row * n_meas + m.sel) * tiles + tile] = 2.0 * (cd[0] * Sr - cd[1] * Si);
        }
      }
      __syncthreads();
      o += n;
      continue;
    }
    if (op.kind == K_MEASG) {
      // up to 4 measures of any Pauli type: S_t = sum_j conj(y_j) (-1)^{parity(src & z_t) ^ zf_t} x_src,
      // src = j ^ xm_t
      const int n = op.aux;
      int xm[4], zl[4], zf[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        xm[t] = zl[t] = zf[t] = 0;
        if (t < n) {
          const DOp m = sops[so + 1 + t];
          const int l0 = m.aux & 0xff, l1 = (m.aux >> 8) & 0xff;
          const int a0 = sd.local_of[m.p0], a1 = m.p1 >= 0 ? sd.local_of[m.p1] : -1;
          // moving letters are on active bits (planner)
          if (l0 == 1 || l0 == 2) xm[t] ^= lz ? (int)(uint16_t)m.c0 : (1 << a0);
          if (l1 == 1 || l1 == 2) xm[t] ^= lz ? (int)(uint16_t)m.c1 : (1 << a1);
          if (l0 == 2 || l0 == 3) {
            if (a0 >= 0) zl[t] ^= lz ? (int)(uint16_t)m.r0 : (1 << a0);
            else zf[t] ^= (int)((base >> m.p0) & 1);
          }
          if (l1 == 2 || l1 == 3) {
            if (a1 >= 0) zl[t] ^= lz ? (int)(uint16_t)m.r1 : (1 << a1);
            else zf[t] ^= (int)((base >> m.p1) & 1);
          }
        }
      }
      Acc ar[4], ai[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) ar[t] = ai[t] = Acc{0.f, 0.f};
      for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
        const Amp u = y[j];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (t >= n) break;
          const int src = j ^ xm[t];
          Amp v = x[src];
          if ((__popc((src ^ bx) & zl[t]) & 1) ^ zf[t]) v = cneg(v);
          acc_mul(ar[t], u.rh, u.rl, v.rh, v.rl);
          acc_mul(ar[t], u.ih, u.il, v.ih, v.il);
          acc_mul(ai[t], u.rh, u.rl, v.ih, v.il);
          acc_mul(ai[t], -u.ih, -u.il, v.rh, v.rl);
        }
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (t >= n) break;
        ar[t] = warp_sum_df(ar[t]);
        ai[t] = warp_sum_df(ai[t]);
        if (lane == 0) {
          gsum[wid][t][0] = make_float2(ar[t].h, ar[t].l);
          gsum[wid][t][1] = make_float2(ai[t].h, ai[t].l);
        }
      }
      __syncthreads();
      if (threadIdx.x < n) {
        const int t = threadIdx.x;
        const DOp m = sops[so + 1 + t];
        if (m.gidx < lim) {
          Acc a{0.f, 0.f}, b{0.f, 0.f};
          for (int w = 0; w < nw; ++w) {
            acc_add(a, gsum[w][t][0].x, gsum[w][t][0].y);
            acc_add(b, gsum[w][t][1].x, gsum[w][t][1].y);
          }
          const double Sr = (double)a.h + (double)a.l, Si = (double)b.h + (double)b.l;
          const double* cd = dconsts + (-m.slot - 1);
          double wr = cd[0], wi = cd[1];
          const int ny = ((m.aux & 0xff) == 2) + (((m.aux >> 8) & 0xff) == 2);
          for (int q = 0; q < ny; ++q) {
            const double tmp = wr;
            wr = -wi;
            wi = tmp;
          }
          mpart[((int64_t)row * n_meas + m.sel) * tiles + tile] = 2.0 * (wr * Sr - wi * Si);
        }
      }
      __syncthreads();
      o += n;
      continue;
    }
    if (op.gidx >= lim || (op.kind != K_MEASURE && op.sel >= 0 && op.sel != row)) continue;
    const int j0 = sd.local_of[op.p0];
    const int j1 = op.p1 >= 0 ? sd.local_of[op.p1] : -1;
    const int f0 = j0 < 0 ? (int)((base >> op.p0) & 1) : 0;
    const int f1 = (op.p1 >= 0 && j1 < 0) ? (int)((base >> op.p1) & 1) : 0;
    if (op.kind == K_MEASURE) {
      // S = sum_j conj(y_j) (-1)^{parity(src & z) ^ zf} x_src,  src = j ^ xm.  Both tiles carry the same pending
      // tile phase (the same ops were applied to both), which cancels in conj(y) x.
      const int l0 = op.aux & 0xff, l1 = (op.aux >> 8) & 0xff;
      const bool mv0 = (l0 == 1 || l0 == 2), mv1 = (l1 == 1 || l1 == 2);
      const bool z0 = (l0 == 2 || l0 == 3), z1 = (l1 == 2 || l1 == 3);
      const int xm = lz ? ((mv0 ? (int)(uint16_t)op.c0 : 0) ^ (mv1 ? (int)(uint16_t)op.c1 : 0))
                        : ((mv0 ? (1 << j0) : 0) | (mv1 ? (1 << j1) : 0));
      const int zl = lz ? (((z0 && j0 >= 0) ? (int)(uint16_t)op.r0 : 0) ^ ((z1 && j1 >= 0) ? (int)(uint16_t)op.r1 : 0))
                        : (((z0 && j0 >= 0) ? (1 << j0) : 0) | ((z1 && j1 >= 0) ? (1 << j1) : 0));
      const int zf = ((z0 && j0 < 0) ? f0 : 0) ^ ((z1 && j1 < 0) ? f1 : 0);
      Acc sr{0.f, 0.f}, si{0.f, 0.f};
      for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
        const int src = j ^ xm;
        const Amp u = y[j];
        Amp v = x[src];
        if ((__popc((src ^ bx) & zl) & 1) ^ zf) v = cneg(v);
        acc_mul(sr, u.rh, u.rl, v.rh, v.rl);
        acc_mul(sr, u.ih, u.il, v.ih, v.il);
        acc_mul(si, u.rh, u.rl, v.ih, v.il);
        acc_mul(si, -u.ih, -u.il, v.rh, v.rl);
      }
      sr = warp_sum_df(sr);
      si = warp_sum_df(si);
      if (lane == 0) {
        wsum[wid][0] = make_float2(sr.h, sr.l);
        wsum[wid][1] = make_float2(si.h, si.l);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        Acc a{0.f, 0.f}, b{0.f, 0.f};
        for (int w = 0; w < nw; ++w) {
          acc_add(a, wsum[w][0].x, wsum[w][0].y);
          acc_add(b, wsum[w][1].x, wsum[w][1].y);
        }
        const double Sr = (double)a.h + (double)a.l, Si = (double)b.h + (double)b.l;
        const double* cd = dconsts + (-op.slot - 1);
        double wr = cd[0], wi = cd[1];
        const int ny = (l0 == 2) + (l1 == 2);
        for (int q = 0; q < ny; ++q) {
          const double t = wr;
          wr = -wi;
          wi = t;
        }
        mpart[((int64_t)row * n_meas + op.sel) * tiles + tile] = 2.0 * (wr * Sr - wi * Si);
      }
      __syncthreads();
      continue;
    }
    const float2* cf = (op.kind == K_GEN1 || op.kind == K_GEN2)
                           ? (op.slot >= 0 ? rowcoef + ((size_t)row * coef_stride + op.slot) * 4 : consts + (-op.slot - 1))
                           : scf + 4 * so;
#pragma unroll 1
    for (int w = 0; w < 2; ++w) {
      if (lz && (j0 >= 0 || j1 >= 0)) {
        apply_op_lazy<A, 2>(op, w ? y : x, k, j0, j1, f0, f1, cf, b, -1);
      } else {
        R& qr = w ? pyr : pxr;
        R& qi = w ? pyi : pxi;
        bool& qh = w ? phy : phx;
        apply_op<A, 2>(op, w ? y : x, k, j0, j1, f0, f1, cf, qr, qi, qh);
      }
    }
    __syncthreads();
  }
  if (sd.last) return;  // the uncomputed initial states are not needed
  if (lz) {  // logical index l lives at slot A l ^ b
    build_index_tables(lazy_cols + (size_t)sd.out_rec * kLazyRec, k, itab);
    __syncthreads();
  }
  for (int l = threadIdx.x; l < nloc; l += blockDim.x) {
    const int64_t g = row * D + base + offs[l >> c] + (l & cmask);
    const int sl = lz ? (map_index(itab, l) ^ b) : l;
    Amp v = x[sl], w = y[sl];
    if (phx) v = A::cm(pxr, pxi, v);
    if (phy) w = A::cm(pyr, pyi, w);
    A::store_mid(psi, g, v);
    A::store_mid(lam, g, w);
  }
}

// grad[row][col] = sum over the measures t of col and the tiles of mpart[row][t][tile]
__global__ void adj_grad_final(const double* __restrict__ mpart, int n_meas, int64_t tiles,
                               const int32_t* __restrict__ order, const int32_t* __restrict__ start, int n_cols,
                               int64_t rows, double* __restrict__ grad) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= rows * n_cols) return;
  const int64_t row = i / n_cols;
  const int col = (int)(i - row * n_cols);
  double s = 0.0;
  for (int q = start[col]; q < start[col + 1]; ++q) {
    const double* m = mpart + ((int64_t)row * n_meas + order[q]) * tiles;
    for (int64_t t = 0; t < tiles; ++t) s += m[t];
  }
  grad[i] = s;
}

static size_t adj_smem(const SweepDesc& sd) {
  size_t s = 2 * sizeof(cdf) * ((size_t)1 << sd.k);
  s += (sizeof(int64_t) * ((size_t)1 << (sd.k - sd.c)) + 15) & ~(size_t)15;
  s += sizeof(cdf) * 256 + 512;
  s += (sizeof(DOp) * (size_t)std::min(sd.n_ops, kOpChunk) + 15) & ~(size_t)15;
  s += sizeof(float2) * 4 * (size_t)std::min(sd.n_ops, kOpChunk);
  return s;
}

int run_adjoint_sweeps(const pqc_program* prog, const float2* rowcoef, const float2* consts, int64_t rows,
                       void* psi, void* lam, const int32_t* row_limit, double* mpart, cudaStream_t stream) {
  static int attr_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    PQC_CUDA(cudaFuncSetAttribute(adj_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    attr_dev = dev;
  }
  const int N = prog->n_qubits;
  const int n_meas = (int)prog->adj_gens.size();
  const int coef_stride = (int)prog->adj_t.specs.size();
  // relabelled sweeps apply their CNOTs to every row: per-row limits take the plan without relabelling
  const Plan& plan = (row_limit && prog->adj_lazy) ? prog->adj_plan_lim : prog->adj_plan;
  for (const SweepDesc& sd : plan.sweeps) {
    const int64_t tiles = 1ll << (N - sd.k);
    const size_t smem = adj_smem(sd);
    if (smem > 220 * 1024) return fail(PQC_ERR_UNSUPPORTED, "adjoint sweep needs too much shared memory");
    const int64_t max_rows = std::max<int64_t>(1, (int64_t)0x7fffffff / tiles);
    for (int64_t r0 = 0; r0 < rows; r0 += max_rows) {
      const int64_t nr = std::min(max_rows, rows - r0);
      adj_sweep_kernel<<<(unsigned)(nr * tiles), 256, smem, stream>>>(
          sd, plan.d_ops, plan.d_offs, rowcoef, coef_stride, consts, prog->adj_t.d_consts, psi, lam, N, tiles, r0,
          row_limit, n_meas, mpart, plan.d_lazy_cols);
      count_launch();
      PQC_CUDA(cudaGetLastError());
    }
  }
  return PQC_OK;
}

int launch_adj_final(const pqc_program* prog, const double* mpart, int64_t rows, double* grad, cudaStream_t stream) {
  const int n_cols = prog->adj_ncols;
  if (n_cols == 0) return PQC_OK;
  const int64_t tiles = adjoint_tiles(prog);
  const int64_t n = rows * n_cols;
  adj_grad_final<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(mpart, (int)prog->adj_gens.size(), tiles,
                                                                  prog->d_adj_cols, prog->d_adj_start, n_cols, rows,
                                                                  grad);
  count_launch();
  PQC_CUDA(cudaGetLastError());
  return PQC_OK;
}

}  // namespace pqc
