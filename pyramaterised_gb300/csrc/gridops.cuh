// Grid double-float: the forward sweeps' rotation and phase passes with the high word of every amplitude
// kept on a fixed grid.
//
// A double-float product-and-add x + t y needs an exact TwoProd and an exact TwoSum (12 FP32 instructions in
// the lazy form, df.cuh).  When the high words of a tile all lie on one grid -- multiples of a quantum
// Q = 2^(E-23) with every value below 2^(E-1) in magnitude -- the sum needs no TwoSum: with G = 1.5 * 2^E,
//
//     X = x_hi + G            exact (x_hi is a multiple of Q, |x_hi| < 2^(E-1))
//     U = fma(t_hi, y_hi, X)  rounds x_hi + t_hi y_hi to the grid (U stays in [2^E, 2^(E+1)), ulp Q)
//     h = U - G               the new high word, a multiple of Q (exact)
//     r = fma(t_hi, y_hi, X - U)   the rounding residual (X - U exact by Sterbenz; |r| <= Q/2)
//
// and the low word collects r, t_hi y_lo, t_lo y_hi and x_lo: 8 instructions per output instead of 12.  The
// price is that the high word carries absolute precision Q, set by a bound on the tile's magnitudes rather
// than by each amplitude: every amplitude of the tile is at most the tile's 2-norm, so the grid is chosen from
// an upper bound on that norm (tracked exactly through the unitary ops of a forward sweep), and the low word's
// rounding error is ~2^-24 of |lo| <= ~Q per op.  Measured against the FP64 oracle this gives ~1e-13 absolute
// amplitude error on the 20-qubit benchmark circuits (1e-12 when the whole state is one tile), against ~3e-15
// for the relative-precision double-float passes; both far inside the 1e-10 the parity tests demand.
//
// Rotations use the scaled form with |t| <= 1 by choosing, per row, between
//     form A (|cos| >= |sin|):  R = cos * [[1, -tan], [tan, 1]]      (RY; RX likewise with -i tan)
//     form B (|sin| >  |cos|):  R = sin * [[cot, -1], [1, cot]]      (RY),   RX(a) = -i sin * (...)(swap)
// so that the unscaled tile norm grows by sqrt(1 + t^2) <= sqrt(2) per rotation (half a bit at most, 0.16 on
// average for uniform angles); the factor cos or sin joins the tile's pending real scale, which the next phase
// block folds into its tables (restoring the norm), and RX in form B adds a -i to the tile phase.  Form B reads
// the pair crosswise: both forms run the same arithmetic
//
//     o0 = sg p + t0 q,   o1 = q + t1 p        (p, q: the pair's members as loaded; o0 -> logical 0, o1 -> 1)
//
// with p loaded from the logical-1 member in form B (an index XOR on the load, none on the store) and sg = -1
// for RY in form B.  A pass that starts from high words not on the current grid (after a load, a non-grid op,
// or when the norm bound outgrows the grid and a coarser one is chosen) takes the regrid variant, which also
// moves the rounding error of x_hi + G into the low word (3 more instructions per output; kept out of line).
//
// Phase blocks multiply by table entries onto a freshly chosen grid (their inputs need not be on any grid),
// folding the low word back into the high word on the last multiply.
#pragma once
#include "sweep_ops.cuh"

namespace pqc {

// Grid state of a tile (uniform across the CTA).
struct GridState {
  float G;     // 1.5 * 2^E
  float lim2;  // largest squared tile norm the grid admits (2^(2E-2) less a margin)
  float tb2;   // upper bound of the squared 2-norm of the stored (unscaled) tile
  bool ok;     // every high word is a multiple of the grid's quantum
};

// Grid for a tile whose squared norm is at most tb2, with `head` bits of headroom for the growth of the
// rotations that follow.  E is the smallest exponent with 4^(E-1) > tb2 * 4^head (1 + 2^-10); tb2 is clamped
// to [2^-120, 2^100] (the caller leaves grid mode before the upper end).
__device__ __forceinline__ void grid_set(GridState& g, float tb2, int head) {
  const float v = fminf(fmaxf(tb2 * 1.0009765625f, 0x1p-120f), 0x1p100f);
  const int e2 = (int)((__float_as_uint(v) >> 23) & 0xffu) - 127 + 2 * head;  // v * 4^head < 2^(e2 + 1)
  const int m = (e2 + 2) >> 1;                                                 // 4^m >= 2^(e2 + 1)
  g.G = __uint_as_float((unsigned)(m + 1 + 127) << 23 | 0x400000u);            // 1.5 * 2^(m + 1)
  g.lim2 = __uint_as_float((unsigned)(2 * m + 127) << 23) * (1.f - 0x1p-11f);  // 4^m (1 - 2^-11)
  g.tb2 = tb2;
  g.ok = false;
}

// Upper bound of the squared 2-norm of the tile x[0, 2^k): the first 128 threads sum fixed interleaved
// slices in order and thread 0 adds the 128 partial sums in order, so the result does not depend on the
// launch shape (every shape has at least 128 threads).  CTA-wide; the caller synchronises before and after.
template <class Amp>
__device__ __forceinline__ void tile_norm2(const Amp* x, int n, float* out, float* part) {
  if (threadIdx.x < 128) {
    float s0 = 0.f, s1 = 0.f;
    int l = threadIdx.x;
    for (; l + 128 < n; l += 256) {
      const Amp a = x[l], b = x[l + 128];
      s0 = __fmaf_rn(a.rh, a.rh, __fmaf_rn(a.ih, a.ih, s0));
      s1 = __fmaf_rn(b.rh, b.rh, __fmaf_rn(b.ih, b.ih, s1));
    }
    if (l < n) {
      const Amp a = x[l];
      s0 = __fmaf_rn(a.rh, a.rh, __fmaf_rn(a.ih, a.ih, s0));
    }
    part[threadIdx.x] = __fadd_rn(s0, s1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < 128; ++i) s = __fadd_rn(s, part[i]);
    *out = s;
  }
}

// One rotation of a grid pass: o0 = sg p + t0 q, o1 = q + t1 p (see above); RX pairs (p.re, q.im) with
// (t0, t1) and (p.im, q.re) with (t1, t0).
struct GRot {
  float sg;
  df t0, t1;
  df f;        // the rotation's factor (cos or sin of the half angle; 1 when inactive)
  float grow;  // bound of the squared-norm growth factor 1 + t^2 (rounded up)
  bool swap;   // form B: p is the logical-1 member
  bool rx;
  bool active;
  // kinds with a grid form (an inactive op is the identity)
  static __device__ __forceinline__ bool usable(const DOp& op, bool active) {
    return !active || op.kind == K_RY || op.kind == K_RX;
  }
  // cf: (cos, sin, tan, cot) of the half angle as double-float pairs
  __device__ __forceinline__ void load(const DOp& op, const float2* cf, bool act) {
    active = act;
    rx = act && op.kind == K_RX;
    if (!act) {
      sg = 1.f;
      t0 = t1 = df{0.f, 0.f};
      f = df{1.f, 0.f};
      grow = 1.f;
      swap = false;
      return;
    }
    swap = fabsf(cf[1].x) > fabsf(cf[0].x);
    f = swap ? df{cf[1].x, cf[1].y} : df{cf[0].x, cf[0].y};
    if (rx) {
      const df tau = swap ? dneg(df{cf[3].x, cf[3].y}) : df{cf[2].x, cf[2].y};
      sg = 1.f;
      t0 = tau;
      t1 = dneg(tau);
    } else if (swap) {
      sg = -1.f;
      t0 = t1 = df{cf[3].x, cf[3].y};
    } else {
      sg = 1.f;
      t1 = df{cf[2].x, cf[2].y};
      t0 = dneg(t1);
    }
    grow = __fmaf_rn(t0.h, t0.h, 1.f) * (1.f + 0x1p-20f);
  }
  // one thread of the CTA: the factor into the tile's pending scale, RX's -i (form B) into its phase
  __device__ __forceinline__ void fold(df* scale, df* phr, df* phi, int* ph) const {
    if (!active) return;
    *scale = df_mul(*scale, f);
    if (rx && swap) {
      ArithDF::cacc(*phr, *phi, df{0.f, 0.f}, df{-1.f, 0.f});
      *ph = 1;
    }
  }
};

// Grid single rotation dispatch (both variants out of line: single rotations are a minority of passes)
template <bool LAZY, bool REGRID>
__device__ __noinline__ void grot1_out(cdf* x, int k, int q, int m, int r, int b, const GRot g, float G, int wl);

template <bool LAZY>
__device__ __forceinline__ void grot1(cdf* x, int k, int q, int m, int r, int b, const GRot& g, float G, bool regrid,
                                      int wl) {
  if (regrid)
    grot1_out<LAZY, true>(x, k, q, m, r, b, g, G, wl);
  else
    grot1_out<LAZY, false>(x, k, q, m, r, b, g, G, wl);
}

// Headroom (bits of the tile norm) of a freshly chosen grid: one bit lets a few rotations grow the norm
// before a coarser grid is needed, and costs one bit of the low word's absolute precision.
constexpr int kGridHead = 1;

// Admits a grid pass whose rotations grow the squared norm bound by `grow`: false when the bound would leave
// the range grid_set handles (the caller then takes the unscaled general form).  Otherwise updates the bound,
// moves to a coarser grid when the current one no longer admits it, and returns in *regrid whether the pass
// must take the regrid variant.
__device__ __forceinline__ bool grid_admit(GridState& gs, float grow, bool* regrid) {
  const float tb2n = gs.tb2 * grow;
  if (!(tb2n < 0x1p100f)) return false;
  *regrid = !gs.ok;
  if (tb2n > gs.lim2) {
    grid_set(gs, tb2n, kGridHead);
    *regrid = true;
  }
  gs.tb2 = tb2n;
  return true;
}

// o0 = sg p + t0 q, o1 = q + t1 p for one real component pair, high words on the grid G
template <bool REGRID>
__device__ __forceinline__ void gpair(float& ph, float& pl, float& qh, float& ql, float sg, df t0, df t1, float G) {
  const float x0 = __fmaf_rn(sg, ph, G), x1 = __fadd_rn(qh, G);
  float e0 = 0.f, e1 = 0.f;
  if (REGRID) {  // the rounding of p_hi + G and q_hi + G (exact residuals) joins the low words
    e0 = __fmaf_rn(sg, ph, -__fsub_rn(x0, G));
    e1 = __fsub_rn(qh, __fsub_rn(x1, G));
  }
  const float u0 = __fmaf_rn(t0.h, qh, x0), u1 = __fmaf_rn(t1.h, ph, x1);
  const float r0 = __fmaf_rn(t0.h, qh, __fsub_rn(x0, u0)), r1 = __fmaf_rn(t1.h, ph, __fsub_rn(x1, u1));
  float l0 = __fmaf_rn(t0.l, qh, r0), l1 = __fmaf_rn(t1.l, ph, r1);
  l0 = __fmaf_rn(t0.h, ql, l0);
  l1 = __fmaf_rn(t1.h, pl, l1);
  l0 = __fmaf_rn(sg, pl, l0);
  l1 = __fadd_rn(l1, ql);
  if (REGRID) {
    l0 = __fadd_rn(l0, e0);
    l1 = __fadd_rn(l1, e1);
  }
  ph = __fsub_rn(u0, G);
  pl = l0;
  qh = __fsub_rn(u1, G);
  ql = l1;
}

template <bool RX, bool REGRID>
__device__ __forceinline__ void grot(cdf& p, cdf& q, const GRot& g, float G) {
  if (RX) {
    gpair<REGRID>(p.rh, p.rl, q.ih, q.il, 1.f, g.t0, g.t1, G);
    gpair<REGRID>(p.ih, p.il, q.rh, q.rl, 1.f, g.t1, g.t0, G);
  } else {
    gpair<REGRID>(p.rh, p.rl, q.rh, q.rl, g.sg, g.t0, g.t1, G);
    gpair<REGRID>(p.ih, p.il, q.ih, q.il, g.sg, g.t0, g.t1, G);
  }
}

// Two rotations on different local bits in one pass over amplitude quads.  LAZY: relabelled sweep (slots
// from the ops' physical masks and parity rows, see rot2_lazy_impl); otherwise local bits ja, jb.  The loads
// are permuted by the rotations' form-B flags; the stores are not.
template <bool LAZY, bool RX0, bool RX1, bool REGRID>
__device__ __forceinline__ void grot2_impl(cdf* x, int k, int pa, int pb, int c0, int c1, int s0, int s1, int b,
                                           const GRot& g0, const GRot& g1, float G, int wl) {
  const int lo = pa < pb ? pa : pb, hi = pa < pb ? pb : pa;
  const int f = (g0.swap ? c0 : 0) ^ (g1.swap ? c1 : 0);
  const Split sp(1 << (k - 2), wl);
  for (int t = sp.s; t < sp.e; t += sp.st) {
    const int p = ins0(ins0(t, lo), hi);
    const int base = LAZY ? p ^ (parity((p ^ b) & s0) ? c0 : 0) ^ (parity((p ^ b) & s1) ? c1 : 0) : p;
    const int lb = base ^ f;
    cdf a0 = x[lb], a1 = x[lb ^ c0], a2 = x[lb ^ c1], a3 = x[lb ^ c0 ^ c1];
    grot<RX0, REGRID>(a0, a1, g0, G);
    grot<RX0, REGRID>(a2, a3, g0, G);
    grot<RX1, REGRID>(a0, a2, g1, G);
    grot<RX1, REGRID>(a1, a3, g1, G);
    x[base] = a0;
    x[base ^ c0] = a1;
    x[base ^ c1] = a2;
    x[base ^ c0 ^ c1] = a3;
  }
}

template <bool LAZY, bool REGRID>
__device__ __forceinline__ void grot2_dispatch(cdf* x, int k, int pa, int pb, int c0, int c1, int s0, int s1, int b,
                                               const GRot& g0, const GRot& g1, float G, int wl) {
  if (g0.rx) {
    if (g1.rx)
      grot2_impl<LAZY, true, true, REGRID>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
    else
      grot2_impl<LAZY, true, false, REGRID>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
  } else {
    if (g1.rx)
      grot2_impl<LAZY, false, true, REGRID>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
    else
      grot2_impl<LAZY, false, false, REGRID>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
  }
}

// the regrid passes are rare (one per sweep and tile, plus grid changes): out of line
template <bool LAZY>
__device__ __noinline__ void grot2_regrid(cdf* x, int k, int pa, int pb, int c0, int c1, int s0, int s1, int b,
                                          const GRot g0, const GRot g1, float G, int wl) {
  grot2_dispatch<LAZY, true>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
}

// Rotation pair (the K_ROT2 marker mk and members m0, m1) on the grid G.  Relabelled sweeps take the
// members' physical masks, parity rows and the marker's pivots; plain sweeps the local bits ja, jb.
template <bool LAZY>
__device__ __forceinline__ void grot2(cdf* x, int k, const DOp& mk, const DOp& m0, const DOp& m1, int ja, int jb,
                                      int b, const GRot& g0, const GRot& g1, float G, bool regrid, int wl) {
  const int pa = LAZY ? mk.q0 : ja, pb = LAZY ? mk.q1 : jb;
  const int c0 = LAZY ? (int)(uint16_t)m0.c0 : 1 << ja, c1 = LAZY ? (int)(uint16_t)m1.c0 : 1 << jb;
  const int s0 = LAZY ? (int)(uint16_t)m0.r0 : 0, s1 = LAZY ? (int)(uint16_t)m1.r0 : 0;
  if (regrid)
    grot2_regrid<LAZY>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
  else
    grot2_dispatch<LAZY, false>(x, k, pa, pb, c0, c1, s0, s1, b, g0, g1, G, wl);
}

// One rotation over amplitude pairs (pivot q, physical mask m, parity row r in a relabelled sweep; local bit
// j otherwise: q = j, m = 1 << j, r unused).
template <bool LAZY, bool RX, bool REGRID>
__device__ __forceinline__ void grot1_impl(cdf* x, int k, int q, int m, int r, int b, const GRot& g, float G, int wl) {
  const int f = g.swap ? m : 0;
  const Split sp(1 << (k - 1), wl);
  const int nt = sp.st;
  int t = sp.s;
  for (; t + nt < sp.e; t += 2 * nt) {
    const int p = ins0(t, q), p2 = ins0(t + nt, q);
    const int i0 = LAZY ? (parity((p ^ b) & r) ? (p ^ m) : p) : p;
    const int i2 = LAZY ? (parity((p2 ^ b) & r) ? (p2 ^ m) : p2) : p2;
    cdf a = x[i0 ^ f], c = x[i0 ^ m ^ f], a2 = x[i2 ^ f], c2 = x[i2 ^ m ^ f];
    grot<RX, REGRID>(a, c, g, G);
    grot<RX, REGRID>(a2, c2, g, G);
    x[i0] = a;
    x[i0 ^ m] = c;
    x[i2] = a2;
    x[i2 ^ m] = c2;
  }
  if (t < sp.e) {
    const int p = ins0(t, q);
    const int i0 = LAZY ? (parity((p ^ b) & r) ? (p ^ m) : p) : p;
    cdf a = x[i0 ^ f], c = x[i0 ^ m ^ f];
    grot<RX, REGRID>(a, c, g, G);
    x[i0] = a;
    x[i0 ^ m] = c;
  }
}

template <bool LAZY, bool REGRID>
__device__ __noinline__ void grot1_out(cdf* x, int k, int q, int m, int r, int b, const GRot g, float G, int wl) {
  if (g.rx)
    grot1_impl<LAZY, true, REGRID>(x, k, q, m, r, b, g, G, wl);
  else
    grot1_impl<LAZY, false, REGRID>(x, k, q, m, r, b, g, G, wl);
}

// a x + b y with the high word on the grid G; RENORM also folds the low word into the high word
template <bool RENORM>
__device__ __forceinline__ df gdot(df a, df x, df b, df y, float G) {
  const float u1 = __fmaf_rn(a.h, x.h, G);
  const float r1 = __fmaf_rn(a.h, x.h, __fsub_rn(G, u1));
  const float u2 = __fmaf_rn(b.h, y.h, u1);
  const float r2 = __fmaf_rn(b.h, y.h, __fsub_rn(u1, u2));
  float lo = __fmaf_rn(a.h, x.l, r1);
  lo = __fmaf_rn(a.l, x.h, lo);
  lo = __fmaf_rn(b.h, y.l, lo);
  lo = __fmaf_rn(b.l, y.h, lo);
  lo = __fadd_rn(lo, r2);
  if (RENORM) {
    const float u3 = __fadd_rn(u2, lo);
    lo = __fsub_rn(lo, __fsub_rn(u3, u2));
    return {__fsub_rn(u3, G), lo};
  }
  return {__fsub_rn(u2, G), lo};
}

template <bool RENORM>
__device__ __forceinline__ cdf gcm(const cdf& t, const cdf& v, float G) {
  const df tr = re(t), ti = im(t), vr = re(v), vi = im(v);
  return mk(gdot<RENORM>(tr, vr, dneg(ti), vi, G), gdot<RENORM>(tr, vi, ti, vr, G));
}

// phase_apply on the grid G: x[p] *= the tables' entries at the logical index of slot p
template <bool LAZY, int U = 4>
__device__ __forceinline__ void phase_apply_grid(cdf* x, int k, int kl, const cdf* __restrict__ tab, int use,
                                                 const uint16_t* __restrict__ itab, int b, float G) {
  const int nlo = 1 << kl, n = 1 << k, nt = blockDim.x;
  const int lb = LAZY ? map_index(itab, b) : 0;
  int p = threadIdx.x;
  for (; p + (U - 1) * nt < n; p += U * nt) {
    cdf v[U];
    int l[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      l[u] = LAZY ? (map_index(itab, p + u * nt) ^ lb) : p + u * nt;
      v[u] = x[p + u * nt];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (use == 3) {
        v[u] = gcm<false>(tab[l[u] & (nlo - 1)], v[u], G);
        v[u] = gcm<true>(tab[nlo + (l[u] >> kl)], v[u], G);
      } else {
        v[u] = gcm<true>(tab[use == 1 ? (l[u] & (nlo - 1)) : nlo + (l[u] >> kl)], v[u], G);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) x[p + u * nt] = v[u];
  }
  for (; p < n; p += nt) {
    const int l = LAZY ? (map_index(itab, p) ^ lb) : p;
    cdf v = x[p];
    if (use == 3) {
      v = gcm<false>(tab[l & (nlo - 1)], v, G);
      v = gcm<true>(tab[nlo + (l >> kl)], v, G);
    } else {
      v = gcm<true>(tab[use == 1 ? (l & (nlo - 1)) : nlo + (l >> kl)], v, G);
    }
    x[p] = v;
  }
}

// One phase block on the grid: the tables (with the pending scale `fold` folded in) as in phase_block, then
// the multiply onto a grid chosen for the folded norm bound.  Straddling members run afterwards as plain
// element-wise ops, which leave the tile off the grid.  Returns the tables in use.
template <bool LAZY>
__device__ __forceinline__ int phase_block_grid(const DOp& mk, const DOp* __restrict__ blk,
                                                const float2* __restrict__ bcf, const SweepDesc& sd, cdf* x, int k,
                                                int64_t base, cdf* tab, uint16_t* itab,
                                                const uint16_t* __restrict__ rec, int b, df& phr, df& phi, bool& ph,
                                                int lim, int st, df* scale, GridState& gs, int head) {
  const PhaseSplit ps = phase_split(mk);
  const df fold = *scale;
  const int use = phase_tables<ArithDF>(blk, bcf, ps, sd, k, base, tab, phr, phi, ph, lim, st, fold);
  if (use) {
    if (LAZY) build_index_tables(rec, k, itab);
    __syncthreads();
    if (threadIdx.x == 0) *scale = ArithDF::rone();
    grid_set(gs, gs.tb2 * fold.h * fold.h * (1.f + 0x1p-20f), head);
    phase_apply_grid<LAZY>(x, k, ps.kl, tab, use, itab, b, gs.G);
    gs.ok = true;
  }
  if (ps.nmid > 0) {
    phase_mid<ArithDF, LAZY>(blk, bcf, ps, sd, x, k, b, phr, phi, ph, lim, st);
    gs.ok = false;
  }
  return use;
}

}  // namespace pqc
