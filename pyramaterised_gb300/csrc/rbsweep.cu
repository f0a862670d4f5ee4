// Register-blocked sweeps: the forward hot path for tiles of k >= 9 bits.
//
// Same HBM pass as sweep.cu (gather a 2^k-amplitude tile, apply the sweep's
// ops, scatter it back), but inside the tile each of the 2^(k-4) threads keeps
// 16 amplitudes in registers: those whose local index agrees with the thread
// on every bit except the phase's 4 "register bits".  Every op whose moving
// bits are register bits (and every diagonal op, whatever its bits) is applied
// to the registers with 8 independent pairs per thread; shared memory is
// touched only when the next phase selects other register bits.  The ops and
// their coefficients are staged in shared memory once per CTA, and the tile is
// stored with an XOR swizzle so the phase re-partitions hit distinct banks.
#include <algorithm>

#include "sweep_ops.cuh"

namespace pqc {

// local-index offset of register slot pattern v: bit q of v goes to position bq
struct VOff {
  int m0, m1, m2, m3;
  __device__ __forceinline__ int operator()(int v) const {
    return ((v & 1) ? m0 : 0) | ((v & 2) ? m1 : 0) | ((v & 4) ? m2 : 0) | ((v & 8) ? m3 : 0);
  }
};

__device__ __forceinline__ int swz(int l) {
  const int u = l >> 3;
  return l ^ ((u ^ (u >> 3) ^ (u >> 6) ^ (u >> 9)) & 7);
}

template <int Q, class Amp, class F>
__device__ __forceinline__ void rp1(Amp (&r)[16], F& f) {
#pragma unroll
  for (int v = 0; v < 16; ++v)
    if (!((v >> Q) & 1)) f(v, r[v], r[v | (1 << Q)]);
}

// pairs (v, v | 1 << q) of register slots, q < 4
template <class Amp, class F>
__device__ __forceinline__ void rpairs(int q, Amp (&r)[16], F f) {
  switch (q) {
    case 0: rp1<0>(r, f); break;
    case 1: rp1<1>(r, f); break;
    case 2: rp1<2>(r, f); break;
    default: rp1<3>(r, f); break;
  }
}

template <int Q0, int Q1, class Amp, class F>
__device__ __forceinline__ void rq2(Amp (&r)[16], F& f) {
#pragma unroll
  for (int v = 0; v < 16; ++v)
    if (!((v >> Q0) & 1) && !((v >> Q1) & 1))
      f(v, r[v], r[v | (1 << Q1)], r[v | (1 << Q0)], r[v | (1 << Q0) | (1 << Q1)]);
}

// quads (00, 01, 10, 11) of slots (q0 = first tensor factor, q1 = second)
template <class Amp, class F>
__device__ __forceinline__ void rquads(int q0, int q1, Amp (&r)[16], F f) {
  switch (q0 * 4 + q1) {
    case 1: rq2<0, 1>(r, f); break;
    case 2: rq2<0, 2>(r, f); break;
    case 3: rq2<0, 3>(r, f); break;
    case 4: rq2<1, 0>(r, f); break;
    case 6: rq2<1, 2>(r, f); break;
    case 7: rq2<1, 3>(r, f); break;
    case 8: rq2<2, 0>(r, f); break;
    case 9: rq2<2, 1>(r, f); break;
    case 11: rq2<2, 3>(r, f); break;
    case 12: rq2<3, 0>(r, f); break;
    case 13: rq2<3, 1>(r, f); break;
    case 14: rq2<3, 2>(r, f); break;
    default: break;
  }
}

__device__ __forceinline__ const float2* rop_coefs(const ROp& op, const float2* __restrict__ rowcoef, int coef_stride,
                                                   const float2* __restrict__ consts, int64_t row) {
  return op.slot >= 0 ? rowcoef + ((size_t)row * coef_stride + op.slot) * 4 : consts + (-op.slot - 1);
}

__device__ __forceinline__ bool rop_has_coefs(int kind) {
  return kind != K_PHASEBLK && kind != K_X && kind != K_CNOT && kind != K_CZ;
}

// One phase-table pass over a diagonal run, applied to the registers.
template <class A>
__device__ __forceinline__ void rb_phase_block(const ROp* __restrict__ blk, const float2* __restrict__ bcf, int n, int k,
                                               int64_t base, int tb, const VOff& voff, typename A::Amp (&r)[16],
                                               typename A::Amp* tab, typename A::R& phr, typename A::R& phi, bool& ph,
                                               int lim) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  const int kl = k >> 1, kh = k - kl;
  const int nlo = 1 << kl, nhi = 1 << kh;
  bool any_lo = false, any_hi = false, any_mid = false;
  for (int t = 0; t < n; ++t) {
    const ROp& op = blk[t];
    if (op.gidx >= lim) continue;
    const int cls = phase_class(op.j0, op.j1, kl);
    any_lo |= cls == 0;
    any_hi |= cls == 1;
    any_mid |= cls == 2;
    if (cls == -1) {
      const int f0 = (int)((base >> op.p0) & 1);
      const int f1 = op.p1 >= 0 ? (int)((base >> op.p1) & 1) : 0;
      DOp d{op.kind, op.sel, op.p0, op.p1, op.slot, op.aux, op.gidx};
      diag_phase<A>(d, bcf + 4 * t, f0, f1, phr, phi);
      ph = true;
    }
  }
  if (any_lo || any_hi) {
    for (int i = threadIdx.x; i < nlo + nhi; i += blockDim.x) {
      const bool lo = i < nlo;
      const int idx = lo ? i : i - nlo;
      const int shift = lo ? 0 : kl;
      R pr = A::rone(), pi = A::rzero();
      for (int t = 0; t < n; ++t) {
        const ROp& op = blk[t];
        if (op.gidx >= lim || phase_class(op.j0, op.j1, kl) != (lo ? 0 : 1)) continue;
        const int b0 = op.j0 >= 0 ? (idx >> (op.j0 - shift)) & 1 : (int)((base >> op.p0) & 1);
        const int b1 = op.p1 < 0 ? 0 : (op.j1 >= 0 ? (idx >> (op.j1 - shift)) & 1 : (int)((base >> op.p1) & 1));
        DOp d{op.kind, op.sel, op.p0, op.p1, op.slot, op.aux, op.gidx};
        diag_phase<A>(d, bcf + 4 * t, b0, b1, pr, pi);
      }
      tab[i] = A::cplx(pr, pi);
    }
    __syncthreads();
#pragma unroll
    for (int v = 0; v < 16; ++v) {
      const int l = tb | voff(v);
      if (any_lo) {
        const Amp t = tab[l & (nlo - 1)];
        r[v] = A::cm(A::real(t), A::imag(t), r[v]);
      }
      if (any_hi) {
        const Amp u = tab[nlo + (l >> kl)];
        r[v] = A::cm(A::real(u), A::imag(u), r[v]);
      }
    }
    __syncthreads();
  }
  if (any_mid) {
    for (int t = 0; t < n; ++t) {
      const ROp& op = blk[t];
      if (op.gidx >= lim || phase_class(op.j0, op.j1, kl) != 2) continue;
      DOp d{op.kind, op.sel, op.p0, op.p1, op.slot, op.aux, op.gidx};
#pragma unroll
      for (int v = 0; v < 16; ++v) {
        const int l = tb | voff(v);
        R pr = A::rone(), pi = A::rzero();
        diag_phase<A>(d, bcf + 4 * t, (l >> op.j0) & 1, (l >> op.j1) & 1, pr, pi);
        r[v] = A::cm(pr, pi, r[v]);
      }
    }
  }
}

// Apply one (non-block) op to the registers.
template <class A>
__device__ __forceinline__ void rb_apply(const ROp& op, const float2* __restrict__ cf, const float2* __restrict__ gcf,
                                         int64_t base, int tb, const VOff& voff, typename A::Amp (&r)[16],
                                         typename A::R& phr, typename A::R& phi, bool& ph) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  const int f0 = op.j0 < 0 ? (int)((base >> op.p0) & 1) : 0;
  const int f1 = (op.p1 >= 0 && op.j1 < 0) ? (int)((base >> op.p1) & 1) : 0;
  switch (op.kind) {
    case K_RY: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      rpairs(op.q0, r, [&](int, Amp& a, Amp& b) {
        const Amp na = A::lin(c, a, ns, b);
        b = A::lin(s, a, c, b);
        a = na;
      });
      break;
    }
    case K_REAL2: {
      const R a0 = A::ld(cf[0]), b0 = A::ld(cf[1]), c0 = A::ld(cf[2]), d0 = A::ld(cf[3]);
      rpairs(op.q0, r, [&](int, Amp& u, Amp& w) {
        const Amp nu = A::lin(a0, u, b0, w);
        w = A::lin(c0, u, d0, w);
        u = nu;
      });
      break;
    }
    case K_RX: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]);
      rpairs(op.q0, r, [&](int, Amp& a, Amp& b) {
        const Amp na = A::rxc(c, a, s, b);
        b = A::rxc(c, b, s, a);
        a = na;
      });
      break;
    }
    case K_GEN1: {
      const R a0 = A::ld(gcf[0]), a1 = A::ld(gcf[1]), b0 = A::ld(gcf[2]), b1 = A::ld(gcf[3]);
      const R c0 = A::ld(gcf[4]), c1 = A::ld(gcf[5]), d0 = A::ld(gcf[6]), d1 = A::ld(gcf[7]);
      rpairs(op.q0, r, [&](int, Amp& u, Amp& w) {
        const Amp nu = A::cd(a0, a1, u, b0, b1, w);
        w = A::cd(c0, c1, u, d0, d1, w);
        u = nu;
      });
      break;
    }
    case K_X:
      rpairs(op.q0, r, [&](int, Amp& a, Amp& b) {
        const Amp t = a;
        a = b;
        b = t;
      });
      break;
    case K_RZ:
    case K_DIAG1: {
      R p0r, p0i, p1r, p1i;
      if (op.kind == K_RZ) {
        const R c = A::ld(cf[0]), s = A::ld(cf[1]);
        p0r = c;
        p0i = A::rneg(s);
        p1r = c;
        p1i = s;
      } else {
        p0r = A::ld(cf[0]);
        p0i = A::ld(cf[1]);
        p1r = A::ld(cf[2]);
        p1i = A::ld(cf[3]);
      }
      if (op.j0 < 0) {
        if (f0)
          A::cacc(phr, phi, p1r, p1i);
        else
          A::cacc(phr, phi, p0r, p0i);
        ph = true;
      } else {
#pragma unroll
        for (int v = 0; v < 16; ++v) {
          const int b = ((tb | voff(v)) >> op.j0) & 1;
          r[v] = A::cm(b ? p1r : p0r, b ? p1i : p0i, r[v]);
        }
      }
      break;
    }
    case K_CNOT: {
      if (op.q0 >= 0) {
        rquads(op.q0, op.q1, r, [&](int, Amp&, Amp&, Amp& a10, Amp& a11) {
          const Amp t = a10;
          a10 = a11;
          a11 = t;
        });
      } else {
        const int ctrl = op.j0 >= 0 ? (tb >> op.j0) & 1 : f0;
        if (ctrl)
          rpairs(op.q1, r, [&](int, Amp& a, Amp& b) {
            const Amp t = a;
            a = b;
            b = t;
          });
      }
      break;
    }
    case K_CZ: {
      if (op.j0 < 0 && op.j1 < 0) {
        if (f0 & f1) {
          phr = A::rneg(phr);
          phi = A::rneg(phi);
          ph = true;
        }
      } else {
#pragma unroll
        for (int v = 0; v < 16; ++v) {
          const int l = tb | voff(v);
          const int b0 = op.j0 >= 0 ? (l >> op.j0) & 1 : f0;
          const int b1 = op.j1 >= 0 ? (l >> op.j1) & 1 : f1;
          if (b0 & b1) r[v] = A::neg(r[v]);
        }
      }
      break;
    }
    case K_RZZ: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      if (op.j0 < 0 && op.j1 < 0) {
        A::cacc(phr, phi, c, (f0 ^ f1) ? s : ns);
        ph = true;
      } else {
#pragma unroll
        for (int v = 0; v < 16; ++v) {
          const int l = tb | voff(v);
          const int b0 = op.j0 >= 0 ? (l >> op.j0) & 1 : f0;
          const int b1 = op.j1 >= 0 ? (l >> op.j1) & 1 : f1;
          r[v] = A::cm(c, (b0 ^ b1) ? s : ns, r[v]);
        }
      }
      break;
    }
    case K_RXX:
    case K_RYY: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      // RXX: c x - i s x';  RYY: c x + i s sigma x', sigma = +1 when the two bits agree
      const R s_eq = op.kind == K_RXX ? s : ns;
      const R s_ne = s;
      rquads(op.q0, op.q1, r, [&](int, Amp& a00, Amp& a01, Amp& a10, Amp& a11) {
        const Amp n00 = A::rxc(c, a00, s_eq, a11);
        a11 = A::rxc(c, a11, s_eq, a00);
        a00 = n00;
        const Amp n01 = A::rxc(c, a01, s_ne, a10);
        a10 = A::rxc(c, a10, s_ne, a01);
        a01 = n01;
      });
      break;
    }
    case K_MIX2: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), pr = A::ld(cf[2]), pi = A::ld(cf[3]);
      const bool one11 = A::is_one(pr, pi);
      rquads(op.q0, op.q1, r, [&](int, Amp&, Amp& a01, Amp& a10, Amp& a11) {
        const Amp n01 = A::rxc(c, a01, s, a10);
        a10 = A::rxc(c, a10, s, a01);
        a01 = n01;
        if (!one11) a11 = A::cm(pr, pi, a11);
      });
      break;
    }
    case K_PAULI: {
      // out[j] = w (-1)^{parity((j ^ xm) & z)} x[j ^ xm],  w = coef * i^{n_y}
      const int l0 = op.aux & 0xff, l1 = (op.aux >> 8) & 0xff;
      R wr = A::ld(cf[0]), wi = A::ld(cf[1]);
      const int ny = (l0 == 2) + (l1 == 2);
      for (int q = 0; q < ny; ++q) {
        const R t = wr;
        wr = A::rneg(wi);
        wi = t;
      }
      const bool mv0 = (l0 == 1 || l0 == 2), mv1 = (l1 == 1 || l1 == 2);
      const bool z0 = (l0 == 2 || l0 == 3), z1 = (l1 == 2 || l1 == 3);
      const int zl = ((z0 && op.j0 >= 0) ? (1 << op.j0) : 0) | ((z1 && op.j1 >= 0) ? (1 << op.j1) : 0);
      const int zf = ((z0 && op.j0 < 0) ? f0 : 0) ^ ((z1 && op.j1 < 0) ? f1 : 0);
      auto sgn = [&](int v) { return (__popc((tb | voff(v)) & zl) & 1) ^ zf; };
      auto term = [&](int vsrc, const Amp& src) {
        const Amp t = A::cm(wr, wi, src);
        return sgn(vsrc) ? A::neg(t) : t;
      };
      if (!mv0 && !mv1) {
#pragma unroll
        for (int v = 0; v < 16; ++v) r[v] = term(v, r[v]);
      } else if (mv0 && mv1) {
        rquads(op.q0, op.q1, r, [&](int v, Amp& a00, Amp& a01, Amp& a10, Amp& a11) {
          const int m1 = 1 << op.q1, m0 = 1 << op.q0;
          const Amp n00 = term(v | m0 | m1, a11), n11 = term(v, a00);
          const Amp n01 = term(v | m0, a10), n10 = term(v | m1, a01);
          a00 = n00;
          a11 = n11;
          a01 = n01;
          a10 = n10;
        });
      } else {
        const int q = mv0 ? op.q0 : op.q1;
        rpairs(q, r, [&](int v, Amp& a, Amp& b) {
          const Amp na = term(v | (1 << q), b), nb = term(v, a);
          a = na;
          b = nb;
        });
      }
      break;
    }
    default:
      break;
  }
}

// general 4x4 on local bits (j0 first tensor factor) over the swizzled tile
template <class A>
__device__ __forceinline__ void smem_gen2(typename A::Amp* x, int k, int j0, int j1, const float2* __restrict__ cf) {
  using Amp = typename A::Amp;
  const int quarter = 1 << (k - 2);
  const int m0 = 1 << j0, m1 = 1 << j1;
  for (int t = threadIdx.x; t < quarter; t += blockDim.x) {
    const int i00 = ins00(t, j0, j1);
    const int idx[4] = {swz(i00), swz(i00 | m1), swz(i00 | m0), swz(i00 | m0 | m1)};
    const Amp v[4] = {x[idx[0]], x[idx[1]], x[idx[2]], x[idx[3]]};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float2* row = cf + 8 * q;
      const Amp u = A::cd(A::ld(row[0]), A::ld(row[1]), v[0], A::ld(row[2]), A::ld(row[3]), v[1]);
      const Amp w = A::cd(A::ld(row[4]), A::ld(row[5]), v[2], A::ld(row[6]), A::ld(row[7]), v[3]);
      x[idx[q]] = A::add(u, w);
    }
  }
}

template <class A>
__global__ void __launch_bounds__(512, 1)
    rb_sweep_kernel(const __grid_constant__ SweepDesc sd, const RPhase* __restrict__ phases, int phase_begin,
                    int n_phases, const ROp* __restrict__ rops, int rop_begin, int n_rops,
                    const int64_t* __restrict__ offs_g, const float2* __restrict__ rowcoef, int coef_stride,
                    const float2* __restrict__ consts, const double2* __restrict__ psi0, int64_t psi0_index, void* psi,
                    int n_qubits, int64_t tiles, int64_t row0, const int32_t* __restrict__ row_limit) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  extern __shared__ __align__(16) unsigned char smem[];
  const int k = sd.k, c = sd.c;
  const int nloc = 1 << k;
  const int tid = threadIdx.x, nt = blockDim.x;
  size_t off = sizeof(Amp) * (size_t)nloc;
  Amp* x = reinterpret_cast<Amp*>(smem);
  int64_t* offs = reinterpret_cast<int64_t*>(smem + off);
  off += (sizeof(int64_t) * ((size_t)1 << (k - c)) + 15) & ~(size_t)15;
  Amp* tab = reinterpret_cast<Amp*>(smem + off);
  off += sizeof(Amp) * 256;
  ROp* sops = reinterpret_cast<ROp*>(smem + off);
  off += (sizeof(ROp) * (size_t)n_rops + 15) & ~(size_t)15;
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
  for (int i = tid; i < nhi; i += nt) offs[i] = offs_g[sd.offs_begin + i];
  for (int i = tid; i < n_rops; i += nt) {
    const ROp o = rops[rop_begin + i];
    sops[i] = o;
    if (rop_has_coefs(o.kind)) {
      const float2* cf = rop_coefs(o, rowcoef, coef_stride, consts, row);
#pragma unroll
      for (int q = 0; q < 4; ++q) scf[4 * i + q] = cf[q];
    }
  }
  __syncthreads();
  for (int l = tid; l < nloc; l += nt) {
    const int64_t g = base + offs[l >> c] + (l & cmask);
    Amp v;
    if (sd.first)
      v = psi0 ? A::load_initial(psi0, g) : (g == psi0_index ? A::one() : A::zero());
    else
      v = A::load_mid(psi, row * D + g);
    x[swz(l)] = v;
  }
  __syncthreads();
  R phr = A::rone(), phi = A::rzero();
  bool ph = false;
  const int allmask = nloc - 1;
  const int lim = row_limit ? row_limit[row] : 0x7fffffff;
  for (int p = 0; p < n_phases; ++p) {
    const RPhase P = phases[phase_begin + p];
    // register positions b0 < b1 < b2 < b3 and this thread's share of the other bits
    uint32_t rb = P.rb;
    const int b0 = __ffs(rb) - 1;
    rb &= rb - 1;
    const int b1 = __ffs(rb) - 1;
    rb &= rb - 1;
    const int b2 = __ffs(rb) - 1;
    rb &= rb - 1;
    const int b3 = __ffs(rb) - 1;
    int tb = 0;
    {
      uint32_t comp = (uint32_t)allmask & ~P.rb;
      int t = tid;
      while (comp) {
        const int b = __ffs(comp) - 1;
        comp &= comp - 1;
        tb |= (t & 1) << b;
        t >>= 1;
      }
    }
    const VOff voff{1 << b0, 1 << b1, 1 << b2, 1 << b3};
    Amp r[16];
#pragma unroll
    for (int v = 0; v < 16; ++v) r[v] = x[swz(tb | voff(v))];
    const int o_end = P.op_begin - rop_begin + P.n_ops;
    for (int o = P.op_begin - rop_begin; o < o_end; ++o) {
      const ROp& op = sops[o];
      if (op.kind == K_PHASEBLK) {
        rb_phase_block<A>(sops + o + 1, scf + 4 * (o + 1), op.aux, k, base, tb, voff, r, tab, phr, phi, ph, lim);
        o += op.aux;
        continue;
      }
      if ((op.sel >= 0 && op.sel != row) || op.gidx >= lim) continue;
      const float2* gcf = (op.kind == K_GEN1 || op.kind == K_GEN2) ? rop_coefs(op, rowcoef, coef_stride, consts, row)
                                                                   : nullptr;
      if (op.kind == K_GEN2) {  // general 4x4: through shared memory (keeps register pressure down)
#pragma unroll
        for (int v = 0; v < 16; ++v) x[swz(tb | voff(v))] = r[v];
        __syncthreads();
        smem_gen2<A>(x, k, op.j0, op.j1, gcf);
        __syncthreads();
#pragma unroll
        for (int v = 0; v < 16; ++v) r[v] = x[swz(tb | voff(v))];
        continue;
      }
      rb_apply<A>(op, scf + 4 * o, gcf, base, tb, voff, r, phr, phi, ph);
    }
#pragma unroll
    for (int v = 0; v < 16; ++v) x[swz(tb | voff(v))] = r[v];
    __syncthreads();
  }
  for (int l = tid; l < nloc; l += nt) {
    const int64_t g = base + offs[l >> c] + (l & cmask);
    Amp v = x[swz(l)];
    if (ph) v = A::cm(phr, phi, v);
    if (sd.last)
      A::store_final(psi, row * D + g, v);
    else
      A::store_mid(psi, row * D + g, v);
  }
}

size_t rb_smem_bytes(const SweepDesc& sd, int n_rops) {
  const size_t amp = sizeof(cdf);
  size_t s = amp * ((size_t)1 << sd.k);
  s += (sizeof(int64_t) * ((size_t)1 << (sd.k - sd.c)) + 15) & ~(size_t)15;
  s += amp * 256;
  s += (sizeof(ROp) * (size_t)n_rops + 15) & ~(size_t)15;
  s += sizeof(float2) * 4 * (size_t)n_rops;
  return s;
}

// Launch one register-blocked sweep; returns 1 when the sweep must use the
// shared-memory kernel instead (tile too small or too many ops to stage).
int launch_rb_sweep(const pqc_program* prog, const Plan& plan, size_t si, int coef_stride, const float2* rowcoef,
                    const float2* consts, int64_t rows, const void* psi0, int64_t psi0_index, void* psi,
                    cudaStream_t stream, const int32_t* row_limit) {
  const SweepDesc& sd = plan.sweeps[si];
  if (sd.k < 9 || plan.sweep_n_phases.empty() || plan.sweep_n_phases[si] == 0) return 1;
  const int pb = plan.sweep_phase_begin[si], np = plan.sweep_n_phases[si];
  const RPhase& first = plan.phases[pb];
  const RPhase& last = plan.phases[pb + np - 1];
  const int rop_begin = first.op_begin;
  const int n_rops = last.op_begin + last.n_ops - rop_begin;
  const size_t smem = rb_smem_bytes(sd, n_rops);
  if (smem > 227 * 1024) return 1;
  static int attr_dev = -1;
  int dev = 0;
  PQC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    PQC_CUDA(cudaFuncSetAttribute(rb_sweep_kernel<ArithDF>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    attr_dev = dev;
  }
  const int N = prog->n_qubits;
  const int64_t tiles = 1ll << (N - sd.k);
  const int threads = 1 << (sd.k - kRegBits);
  const int64_t max_rows = std::max<int64_t>(1, (int64_t)0x7fffffff / tiles);
  for (int64_t r0 = 0; r0 < rows; r0 += max_rows) {
    const int64_t nr = std::min(max_rows, rows - r0);
    rb_sweep_kernel<ArithDF><<<(unsigned)(nr * tiles), threads, smem, stream>>>(
        sd, plan.d_phases, pb, np, plan.d_rops, rop_begin, n_rops, plan.d_offs, rowcoef, coef_stride, consts,
        (const double2*)psi0, psi0_index, psi, N, tiles, r0, row_limit);
    count_launch();
    PQC_CUDA(cudaGetLastError());
  }
  return 0;
}

}  // namespace pqc
