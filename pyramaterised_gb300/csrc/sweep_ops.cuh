// Shared device helpers of the sweep kernels: arithmetic traits (double-float
// and FP32), tile index helpers, and the per-op shared-memory updates.
#pragma once
#include "df.cuh"
#include "dfacc.cuh"
#include "engine.cuh"

namespace pqc {

constexpr int kSweepThreads = 512;

__device__ __forceinline__ int ins0(int t, int j) { return ((t >> j) << (j + 1)) | (t & ((1 << j) - 1)); }
__device__ __forceinline__ int ins00(int t, int ja, int jb) {
  int lo = ja < jb ? ja : jb, hi = ja < jb ? jb : ja;
  return ins0(ins0(t, lo), hi);
}

struct ArithDF {
  using Amp = cdf;
  using R = df;
  static __device__ __forceinline__ R ld(float2 v) { return {v.x, v.y}; }
  static __device__ __forceinline__ int log2_abs(float2 v) {
    return (int)((__float_as_uint(v.x) >> 23) & 0xffu) - 127;
  }
  static __device__ __forceinline__ R rneg(R a) { return dneg(a); }
  static __device__ __forceinline__ Amp zero() { return {0.f, 0.f, 0.f, 0.f}; }
  static __device__ __forceinline__ Amp one() { return {1.f, 0.f, 0.f, 0.f}; }
#ifdef PQC_DF_STRICT
  static __device__ __forceinline__ df d2(df a, df x, df b, df y) { return dot2(a, x, b, y); }
#else
  static __device__ __forceinline__ df d2(df a, df x, df b, df y) { return dot2_lazy(a, x, b, y); }
#endif
  static __device__ __forceinline__ Amp lin(R a, Amp x, R b, Amp y) {
    return mk(d2(a, re(x), b, re(y)), d2(a, im(x), b, im(y)));
  }
  // c*x - i*s*y
  static __device__ __forceinline__ Amp rxc(R c, Amp x, R s, Amp y) {
    return mk(d2(c, re(x), s, im(y)), d2(c, im(x), dneg(s), re(y)));
  }
  static __device__ __forceinline__ Amp cm(R pr, R pi, Amp x) {
    const df xr = re(x), xi = im(x);
    return mk(d2(pr, xr, dneg(pi), xi), d2(pr, xi, pi, xr));
  }
  static __device__ __forceinline__ Amp cd(R ar, R ai, Amp x, R br, R bi, Amp y) { return cdot2(ar, ai, x, br, bi, y); }
#ifdef PQC_DF_STRICT
  static __device__ __forceinline__ df ax(df x, df t, df y) {
    const df r = axpy_lazy(x, t, y);
    return fast_two_sum(r.h, r.l);
  }
#else
  static __device__ __forceinline__ df ax(df x, df t, df y) { return axpy_lazy(x, t, y); }
#endif
  // x + t y and x - i t y for a real t
  static __device__ __forceinline__ Amp axpy(Amp x, R t, Amp y) { return mk(ax(re(x), t, re(y)), ax(im(x), t, im(y))); }
  static __device__ __forceinline__ Amp axpy_mi(Amp x, R t, Amp y) {
    return mk(ax(re(x), t, im(y)), ax(im(x), dneg(t), re(y)));
  }
  // -i x
  static __device__ __forceinline__ Amp mul_mi(Amp x) { return {x.ih, x.il, -x.rh, -x.rl}; }
  static __device__ __forceinline__ bool ge_abs(R a, R b) { return fabsf(a.h) >= fabsf(b.h); }
  static __device__ __forceinline__ R rmul(R a, R b) { return df_mul(a, b); }
  static __device__ __forceinline__ bool is_unit(R a) { return a.h == 1.f && a.l == 0.f; }
  static __device__ __forceinline__ Amp scale(R f, Amp x) {
    const df r = df_mul_lazy(f, re(x)), i = df_mul_lazy(f, im(x));
    return mk(r, i);
  }
  static __device__ __forceinline__ Amp add(Amp a, Amp b) { return cadd(a, b); }
  static __device__ __forceinline__ Amp neg(Amp a) { return cneg(a); }
  static __device__ __forceinline__ bool is_one(R pr, R pi) {
    return pr.h == 1.f && pr.l == 0.f && pi.h == 0.f && pi.l == 0.f;
  }
  static __device__ __forceinline__ void cacc(R& pr, R& pi, R qr, R qi) {
    R nr = dot2(pr, qr, dneg(pi), qi);
    R ni = dot2(pr, qi, pi, qr);
    pr = nr;
    pi = ni;
  }
  static __device__ __forceinline__ R rone() { return {1.f, 0.f}; }
  static __device__ __forceinline__ R rzero() { return {0.f, 0.f}; }
  static __device__ __forceinline__ Amp cplx(R r, R i) { return mk(r, i); }
  static __device__ __forceinline__ R real(Amp a) { return re(a); }
  static __device__ __forceinline__ R imag(Amp a) { return im(a); }
  // storage
  // complex128 -> double-float with integer operations only (split_double: the top 24 and next 23
  // significand bits), which keeps the conversion off GB300's slow FP64 pipe
  static __device__ __forceinline__ Amp load_initial(const double2* p, int64_t i) {
    const double2 v = p[i];
    const float2 r = split_double(v.x), m = split_double(v.y);
    return {r.x, r.y, m.x, m.y};
  }
  static __device__ __forceinline__ Amp load_mid(const void* p, int64_t i) {
    float4 v = reinterpret_cast<const float4*>(p)[i];
    return {v.x, v.y, v.z, v.w};
  }
  static __device__ __forceinline__ void store_mid(void* p, int64_t i, Amp a) {
    reinterpret_cast<float4*>(p)[i] = make_float4(a.rh, a.rl, a.ih, a.il);
  }
  static __device__ __forceinline__ void store_final(void* p, int64_t i, Amp a) {
    reinterpret_cast<double2*>(p)[i] = cdf_to(a);
  }
};

struct ArithF32 {
  using Amp = float2;
  using R = float;
  static __device__ __forceinline__ R ld(float2 v) { return v.x + v.y; }
  static __device__ __forceinline__ int log2_abs(float2 v) {
    return (int)((__float_as_uint(v.x + v.y) >> 23) & 0xffu) - 127;
  }
  static __device__ __forceinline__ R rneg(R a) { return -a; }
  static __device__ __forceinline__ Amp zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ Amp one() { return make_float2(1.f, 0.f); }
  static __device__ __forceinline__ Amp lin(R a, Amp x, R b, Amp y) {
    return make_float2(fmaf(a, x.x, b * y.x), fmaf(a, x.y, b * y.y));
  }
  static __device__ __forceinline__ Amp rxc(R c, Amp x, R s, Amp y) {
    return make_float2(fmaf(c, x.x, s * y.y), fmaf(c, x.y, -s * y.x));
  }
  static __device__ __forceinline__ Amp cm(R pr, R pi, Amp x) {
    return make_float2(fmaf(pr, x.x, -pi * x.y), fmaf(pr, x.y, pi * x.x));
  }
  static __device__ __forceinline__ Amp cd(R ar, R ai, Amp x, R br, R bi, Amp y) {
    Amp u = cm(ar, ai, x), v = cm(br, bi, y);
    return make_float2(u.x + v.x, u.y + v.y);
  }
  static __device__ __forceinline__ Amp axpy(Amp x, R t, Amp y) { return make_float2(fmaf(t, y.x, x.x), fmaf(t, y.y, x.y)); }
  static __device__ __forceinline__ Amp axpy_mi(Amp x, R t, Amp y) {
    return make_float2(fmaf(t, y.y, x.x), fmaf(-t, y.x, x.y));
  }
  static __device__ __forceinline__ Amp mul_mi(Amp x) { return make_float2(x.y, -x.x); }
  static __device__ __forceinline__ bool ge_abs(R a, R b) { return fabsf(a) >= fabsf(b); }
  static __device__ __forceinline__ R rmul(R a, R b) { return a * b; }
  static __device__ __forceinline__ bool is_unit(R a) { return a == 1.f; }
  static __device__ __forceinline__ Amp scale(R f, Amp x) { return make_float2(f * x.x, f * x.y); }
  static __device__ __forceinline__ Amp add(Amp a, Amp b) { return make_float2(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ Amp neg(Amp a) { return make_float2(-a.x, -a.y); }
  static __device__ __forceinline__ bool is_one(R pr, R pi) { return pr == 1.f && pi == 0.f; }
  static __device__ __forceinline__ void cacc(R& pr, R& pi, R qr, R qi) {
    R nr = pr * qr - pi * qi, ni = pr * qi + pi * qr;
    pr = nr;
    pi = ni;
  }
  static __device__ __forceinline__ R rone() { return 1.f; }
  static __device__ __forceinline__ R rzero() { return 0.f; }
  static __device__ __forceinline__ Amp cplx(R r, R i) { return make_float2(r, i); }
  static __device__ __forceinline__ R real(Amp a) { return a.x; }
  static __device__ __forceinline__ R imag(Amp a) { return a.y; }
  static __device__ __forceinline__ Amp load_initial(const double2* p, int64_t i) {
    double2 v = p[i];
    return make_float2((float)v.x, (float)v.y);
  }
  static __device__ __forceinline__ Amp load_mid(const void* p, int64_t i) {
    return reinterpret_cast<const float2*>(p)[i];
  }
  static __device__ __forceinline__ void store_mid(void* p, int64_t i, Amp a) { reinterpret_cast<float2*>(p)[i] = a; }
  static __device__ __forceinline__ void store_final(void* p, int64_t i, Amp a) {
    reinterpret_cast<float2*>(p)[i] = a;
  }
};

// Native FP64 (complex128) arithmetic: the reference's precision, on GB300's FP64 pipe (1/64 of the FP32
// rate).  The coefficient tables passed to the FP64 kernels are the FP64 tables themselves, one double per
// float2 element (same 8-byte stride), so ld() reinterprets the element's bits.
struct ArithF64 {
  using Amp = double2;
  using R = double;
  static __device__ __forceinline__ R ld(float2 v) {
    return __hiloint2double(__float_as_int(v.y), __float_as_int(v.x));
  }
  static __device__ __forceinline__ int log2_abs(float2 v) { return ilogb(ld(v)); }
  static __device__ __forceinline__ R rneg(R a) { return -a; }
  static __device__ __forceinline__ Amp zero() { return make_double2(0.0, 0.0); }
  static __device__ __forceinline__ Amp one() { return make_double2(1.0, 0.0); }
  static __device__ __forceinline__ Amp lin(R a, Amp x, R b, Amp y) {
    return make_double2(fma(a, x.x, b * y.x), fma(a, x.y, b * y.y));
  }
  static __device__ __forceinline__ Amp rxc(R c, Amp x, R s, Amp y) {
    return make_double2(fma(c, x.x, s * y.y), fma(c, x.y, -s * y.x));
  }
  static __device__ __forceinline__ Amp cm(R pr, R pi, Amp x) {
    return make_double2(fma(pr, x.x, -pi * x.y), fma(pr, x.y, pi * x.x));
  }
  static __device__ __forceinline__ Amp cd(R ar, R ai, Amp x, R br, R bi, Amp y) {
    Amp u = cm(ar, ai, x), v = cm(br, bi, y);
    return make_double2(u.x + v.x, u.y + v.y);
  }
  static __device__ __forceinline__ Amp axpy(Amp x, R t, Amp y) { return make_double2(fma(t, y.x, x.x), fma(t, y.y, x.y)); }
  static __device__ __forceinline__ Amp axpy_mi(Amp x, R t, Amp y) {
    return make_double2(fma(t, y.y, x.x), fma(-t, y.x, x.y));
  }
  static __device__ __forceinline__ Amp mul_mi(Amp x) { return make_double2(x.y, -x.x); }
  static __device__ __forceinline__ bool ge_abs(R a, R b) { return fabs(a) >= fabs(b); }
  static __device__ __forceinline__ R rmul(R a, R b) { return a * b; }
  static __device__ __forceinline__ bool is_unit(R a) { return a == 1.0; }
  static __device__ __forceinline__ Amp scale(R f, Amp x) { return make_double2(f * x.x, f * x.y); }
  static __device__ __forceinline__ Amp add(Amp a, Amp b) { return make_double2(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ Amp neg(Amp a) { return make_double2(-a.x, -a.y); }
  static __device__ __forceinline__ bool is_one(R pr, R pi) { return pr == 1.0 && pi == 0.0; }
  static __device__ __forceinline__ void cacc(R& pr, R& pi, R qr, R qi) {
    R nr = pr * qr - pi * qi, ni = pr * qi + pi * qr;
    pr = nr;
    pi = ni;
  }
  static __device__ __forceinline__ R rone() { return 1.0; }
  static __device__ __forceinline__ R rzero() { return 0.0; }
  static __device__ __forceinline__ Amp cplx(R r, R i) { return make_double2(r, i); }
  static __device__ __forceinline__ R real(Amp a) { return a.x; }
  static __device__ __forceinline__ R imag(Amp a) { return a.y; }
  static __device__ __forceinline__ Amp load_initial(const double2* p, int64_t i) { return p[i]; }
  static __device__ __forceinline__ Amp load_mid(const void* p, int64_t i) {
    return reinterpret_cast<const double2*>(p)[i];
  }
  static __device__ __forceinline__ void store_mid(void* p, int64_t i, Amp a) { reinterpret_cast<double2*>(p)[i] = a; }
  static __device__ __forceinline__ void store_final(void* p, int64_t i, Amp a) {
    reinterpret_cast<double2*>(p)[i] = a;
  }
};

__device__ __forceinline__ int parity(int x) { return __popc(x) & 1; }

// ops of a fused block starting at op (the marker and its members)
__device__ __forceinline__ int op_extent(const DOp& op) {
  return 1 + ((op.kind == K_PHASEBLK || op.kind == K_MEASZ || op.kind == K_MEASG) ? op.aux
                                                                                  : op.kind == K_ROT2 ? 2 : 0);
}

__device__ __forceinline__ bool has_coefs(int kind) {
  return kind != K_PHASEBLK && kind != K_ROT2 && kind != K_MEASZ && kind != K_MEASG && kind != K_X &&
         kind != K_CNOT && kind != K_CZ && kind != K_OFFSET;
}

// CTA-wide: ops[first, first + n) and their coefficients into sops / scf (the caller synchronises).
__device__ __forceinline__ void stage_ops(const DOp* __restrict__ ops, int first, int n, DOp* sops, float2* scf,
                                          const float2* __restrict__ rowcoef, int64_t row, int coef_stride,
                                          const float2* __restrict__ consts) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const DOp o = ops[first + i];
    sops[i] = o;
    if (has_coefs(o.kind)) {
      const float2* cf = o.slot >= 0 ? rowcoef + ((size_t)row * coef_stride + o.slot) * 4 : consts + (-o.slot - 1);
#pragma unroll
      for (int q = 0; q < 4; ++q) scf[4 * i + q] = cf[q];
    }
  }
}

// Asynchronous global -> shared copy of one stored amplitude (16 B double-float, 8 B complex64) without
// register staging, so that a thread keeps all of its tile's loads in flight; cp_async_wait_all completes
// the calling thread's copies.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* s, const void* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Bulk tile loads on the TMA engine: one cp.async.bulk per contiguous tile row, completion counted in bytes
// on a shared-memory mbarrier.  The waits are bounded in time (the caller flags a timeout).
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// one thread: init for one arrival and announce `bytes` of incoming copies (before the CTA barrier that
// precedes the copies)
__device__ __forceinline__ void mbar_init_expect(uint64_t* bar, unsigned bytes) {
  const unsigned a = smem_addr(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes) : "memory");
}

// global -> shared bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait for phase `parity` of the mbarrier; false after `limit_ns` nanoseconds
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  const unsigned a = smem_addr(bar);
  const uint64_t t0 = global_ns();
  while (true) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Work split of a loop over M items among the CTA's threads.  Strided (wl < 0): thread i takes the items
// i, i + nt, ...  Warp-blocked (wl = log2 of the warp count, M >> wl a multiple of 32): warp w takes the
// contiguous range [w M / nw, (w + 1) M / nw), 32 items at a time, so an op on local bits below k - wl
// touches only warp w's sub-tile and needs no CTA-wide barrier against other such ops.
struct Split {
  int s, e, st;
  __device__ __forceinline__ Split(int M, int wl) {
    if (wl >= 0) {
      const int per = M >> wl, lane = threadIdx.x & 31;
      s = (threadIdx.x >> 5) * per + lane;
      e = s - lane + per;
      st = 32;
    } else {
      s = threadIdx.x;
      e = M;
      st = blockDim.x;
    }
  }
};

// Loops over the tile with U independent items per iteration: all items'
// shared-memory loads are issued before any store, so their double-float
// dependency chains interleave.
template <int U = 4, class Amp, class F>
__device__ __forceinline__ void pairs1(Amp* x, int half, int j, F f, int wl = -1) {
  const int m = 1 << j;
  const Split sp(half, wl);
  const int nt = sp.st;
  int t = sp.s;
  for (; t + (U - 1) * nt < sp.e; t += U * nt) {
    int i0[U], i1[U];
    Amp a[U], b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      i0[u] = ins0(t + u * nt, j);
      i1[u] = i0[u] | m;
      a[u] = x[i0[u]];
      b[u] = x[i1[u]];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) f(a[u], b[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      x[i0[u]] = a[u];
      x[i1[u]] = b[u];
    }
  }
  for (; t < sp.e; t += nt) {
    const int i0 = ins0(t, j), i1 = i0 | m;
    Amp a = x[i0], b = x[i1];
    f(a, b);
    x[i0] = a;
    x[i1] = b;
  }
}

// pairs (i, i ^ mm) over the items with bit j of i clear
template <class Amp, class F>
__device__ __forceinline__ void pairs_mask(Amp* x, int half, int j, int mm, F f, int wl = -1) {
  const Split sp(half, wl);
  const int nt = sp.st;
  int t = sp.s;
  for (; t + nt < sp.e; t += 2 * nt) {
    const int i0 = ins0(t, j), i1 = i0 ^ mm, k0 = ins0(t + nt, j), k1 = k0 ^ mm;
    Amp a = x[i0], b = x[i1], c = x[k0], d = x[k1];
    f(i0, a, b);
    f(k0, c, d);
    x[i0] = a;
    x[i1] = b;
    x[k0] = c;
    x[k1] = d;
  }
  if (t < sp.e) {
    const int i0 = ins0(t, j), i1 = i0 ^ mm;
    Amp a = x[i0], b = x[i1];
    f(i0, a, b);
    x[i0] = a;
    x[i1] = b;
  }
}

// single elements l of the tile
template <int U = 4, class Amp, class F>
__device__ __forceinline__ void elems(Amp* x, int n, F f, int wl = -1) {
  const Split sp(n, wl);
  const int nt = sp.st;
  int l = sp.s;
  for (; l + (U - 1) * nt < sp.e; l += U * nt) {
    Amp a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) a[u] = x[l + u * nt];
#pragma unroll
    for (int u = 0; u < U; ++u) f(l + u * nt, a[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) x[l + u * nt] = a[u];
  }
  for (; l < sp.e; l += nt) {
    Amp a = x[l];
    f(l, a);
    x[l] = a;
  }
}

// Two-by-two rotation of one amplitude pair (u at bit 0, v at bit 1): kind K_RX uses (c, s) =
// (cf[0], cf[1]); K_RY and K_REAL2 are real [[a, b], [c, d]] (K_RY: a = d = cos, c = -b = sin).  An
// inactive rotation (cut off by a row limit) becomes the real identity, which the double-float
// arithmetic applies exactly.
//
// Scaled form (load_scaled, K_RY and K_RX): the map is c * M with M = [[1, -t], [t, 1]] (RY) or
// [[1, -it], [-it, 1]] (RX), t = s / c, so each output is one multiply-add x + t y (12 instructions in
// double-float instead of 16 for a two-term dot product).  load_scaled multiplies c into the pending
// factor *scale (when scale is not null: one thread of the CTA keeps it, in shared memory), which the
// caller applies to the tile later (folded into a phase table or the write-out).  The unscaled amplitudes
// grow by at most 1 + |t| <= 2^(1 - ilogb|c|) per rotation; the caller bounds that growth
// (scaled_growth) and takes the general form for a rotation that would exceed it.  The scaled form keeps
// t in c.
template <class A>
struct Rot {
  typename A::R a, b, c, d;
  bool rx, scaled;
  // kinds with a scaled form (an inactive op is the identity: t = 0, factor 1)
  static __device__ __forceinline__ bool scalable(const DOp& op, bool active) {
    return !active || op.kind == K_RY || op.kind == K_RX;
  }
  // log2 bound of the growth of a scaled rotation with coefficients cf (1 - ilogb|c|; large when c = 0)
  static __device__ __forceinline__ int scaled_growth(const float2* cf, bool active) {
    if (!active) return 0;
    const int e = A::log2_abs(cf[0]);
    return e >= 0 ? 1 : (e < -1000 ? 1 << 20 : 1 - e);
  }
  __device__ __forceinline__ void load(const DOp& op, const float2* cf, bool active) {
    rx = active && op.kind == K_RX;
    scaled = false;
    if (!active) {
      a = d = A::rone();
      b = c = A::rzero();
    } else if (op.kind == K_RY) {
      a = d = A::ld(cf[0]);
      c = A::ld(cf[1]);
      b = A::rneg(c);
    } else {
      a = A::ld(cf[0]);
      b = A::ld(cf[1]);
      c = A::ld(cf[2]);
      d = A::ld(cf[3]);
    }
  }
  // scalable ops only; cf[2] of K_RY / K_RX holds s / c
  __device__ __forceinline__ void load_scaled(const DOp& op, const float2* cf, bool active, typename A::R* scale) {
    scaled = true;
    rx = active && op.kind == K_RX;
    c = active ? A::ld(cf[2]) : A::rzero();
    if (active && scale) *scale = A::rmul(*scale, A::ld(cf[0]));
  }
  template <bool RX>
  __device__ __forceinline__ void apply(typename A::Amp& u, typename A::Amp& v) const {
    if (RX) {
      const typename A::Amp nu = A::rxc(a, u, b, v);
      v = A::rxc(a, v, b, u);
      u = nu;
    } else {
      const typename A::Amp nu = A::lin(a, u, b, v);
      v = A::lin(c, u, d, v);
      u = nu;
    }
  }
  // Loop kind: 0 general real (lin), 1 general RX (rxc), 2 scaled RY, 3 scaled RX (the kernels instantiate
  // one loop per pair of kinds)
  __device__ __forceinline__ int mode() const { return (scaled ? 2 : 0) + (rx ? 1 : 0); }
  template <int M>
  __device__ __forceinline__ void run(typename A::Amp& u, typename A::Amp& v) const {
    if (M == 0 || M == 1) {
      apply<M == 1>(u, v);
    } else if (M == 2) {  // u - t v, v + t u
      const typename A::Amp nu = A::axpy(u, A::rneg(c), v);
      v = A::axpy(v, c, u);
      u = nu;
    } else {  // u - i t v, v - i t u
      const typename A::Amp nu = A::axpy_mi(u, c, v);
      v = A::axpy_mi(v, c, u);
      u = nu;
    }
  }
};

// Calls F::template go<M0, M1>() for the loop kinds of (r0, r1), both scaled (SCALED) or both general.
template <class A, bool SCALED, class F>
__device__ __forceinline__ void rot2_dispatch(const Rot<A>& r0, const Rot<A>& r1, const F& f) {
  constexpr int s = SCALED ? 2 : 0;
  if (r0.rx) {
    if (r1.rx)
      f.template go<s + 1, s + 1>();
    else
      f.template go<s + 1, s>();
  } else {
    if (r1.rx)
      f.template go<s, s + 1>();
    else
      f.template go<s, s>();
  }
}

// Rotation r0 on local bit j0 followed by r1 on local bit j1 (j0 != j1), one pass over the
// quads {i, i|m0, i|m1, i|m0|m1} of the tile, Q (1 or 2) quads per iteration.  The rotation
// kinds are template arguments so that the inner loop holds one arithmetic path.
template <class A, int Q, int M0, int M1>
__device__ __forceinline__ void rot2_impl(typename A::Amp* x, int k, int j0, int j1, const Rot<A>& r0,
                                          const Rot<A>& r1, int wl) {
  using Amp = typename A::Amp;
  const int quarter = 1 << (k - 2);
  const int lo = j0 < j1 ? j0 : j1, hi = j0 < j1 ? j1 : j0;
  const int m0 = 1 << j0, m1 = 1 << j1;
  const Split sp(quarter, wl);
  const int nt = sp.st;
  int t = sp.s;
  for (; Q == 2 && t + nt < sp.e; t += 2 * nt) {
    const int i = ins0(ins0(t, lo), hi), q = ins0(ins0(t + nt, lo), hi);
    Amp a0 = x[i], a1 = x[i | m0], a2 = x[i | m1], a3 = x[i | m0 | m1];
    Amp b0 = x[q], b1 = x[q | m0], b2 = x[q | m1], b3 = x[q | m0 | m1];
    r0.template run<M0>(a0, a1);
    r0.template run<M0>(b0, b1);
    r0.template run<M0>(a2, a3);
    r0.template run<M0>(b2, b3);
    r1.template run<M1>(a0, a2);
    r1.template run<M1>(b0, b2);
    r1.template run<M1>(a1, a3);
    r1.template run<M1>(b1, b3);
    x[i] = a0;
    x[i | m0] = a1;
    x[i | m1] = a2;
    x[i | m0 | m1] = a3;
    x[q] = b0;
    x[q | m0] = b1;
    x[q | m1] = b2;
    x[q | m0 | m1] = b3;
  }
  for (; t < sp.e; t += nt) {
    const int i = ins0(ins0(t, lo), hi);
    Amp a0 = x[i], a1 = x[i | m0], a2 = x[i | m1], a3 = x[i | m0 | m1];
    r0.template run<M0>(a0, a1);
    r0.template run<M0>(a2, a3);
    r1.template run<M1>(a0, a2);
    r1.template run<M1>(a1, a3);
    x[i] = a0;
    x[i | m0] = a1;
    x[i | m1] = a2;
    x[i | m0 | m1] = a3;
  }
}

template <class A, int Q>
struct Rot2Go {
  typename A::Amp* x;
  int k, j0, j1, wl;
  const Rot<A>& r0;
  const Rot<A>& r1;
  template <int M0, int M1>
  __device__ __forceinline__ void go() const {
    rot2_impl<A, Q, M0, M1>(x, k, j0, j1, r0, r1, wl);
  }
};

// The general loops (pairs that are not both scaled: fixed real rotations, or growth past the bound) are
// kept out of line: inlined next to the scaled ones they push the sweep kernel past its register budget.
template <class A, int Q>
__device__ __noinline__ void rot2_general(typename A::Amp* x, int k, int j0, int j1, const Rot<A> r0, const Rot<A> r1,
                                          int wl) {
  rot2_dispatch<A, false>(r0, r1, Rot2Go<A, Q>{x, k, j0, j1, wl, r0, r1});
}

// GENERAL_ONLY: the caller loads no scaled rotations (the general loops are then inlined).
template <class A, int Q = 2, bool GENERAL_ONLY = false>
__device__ __forceinline__ void rot2(typename A::Amp* x, int k, int j0, int j1, const Rot<A>& r0, const Rot<A>& r1,
                                     int wl = -1) {
  if (GENERAL_ONLY)
    rot2_dispatch<A, false>(r0, r1, Rot2Go<A, Q>{x, k, j0, j1, wl, r0, r1});
  else if (r0.scaled)
    rot2_dispatch<A, true>(r0, r1, Rot2Go<A, Q>{x, k, j0, j1, wl, r0, r1});
  else
    rot2_general<A, Q>(x, k, j0, j1, r0, r1, wl);
}

// Dense two-qubit op (16 complex double-float coefficients).  Kept out of line: its
// coefficient registers would otherwise raise the register pressure of the whole
// sweep kernel and force spills into the paths every circuit runs.
template <class A>
__device__ __noinline__ void apply_gen2(typename A::Amp* x, int quarter, int j0, int j1, const float2* cf, int wl) {
  using Amp = typename A::Amp;
  const int m0 = 1 << j0, m1 = 1 << j1;
  const Split sp(quarter, wl);
  for (int t = sp.s; t < sp.e; t += sp.st) {
    int i00 = ins00(t, j0, j1);
    int idx[4] = {i00, i00 | m1, i00 | m0, i00 | m0 | m1};
    Amp v[4] = {x[idx[0]], x[idx[1]], x[idx[2]], x[idx[3]]};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float2* row = cf + 8 * r;
      Amp u = A::cd(A::ld(row[0]), A::ld(row[1]), v[0], A::ld(row[2]), A::ld(row[3]), v[1]);
      Amp w = A::cd(A::ld(row[4]), A::ld(row[5]), v[2], A::ld(row[6]), A::ld(row[7]), v[3]);
      x[idx[r]] = A::add(u, w);
    }
  }
}

// Apply one op to the tile x[0 .. 2^k).  j0/j1: local bits (-1 if the
// position is fixed in this tile, then f0/f1 hold the fixed bit values).
// wl: the loops' work split (see Split).
template <class A, int U = 4>
__device__ __forceinline__ void apply_op(const DOp& op, typename A::Amp* x, int k, int j0, int j1, int f0, int f1,
                                         const float2* __restrict__ cf, typename A::R& phr, typename A::R& phi,
                                         bool& ph, int wl = -1) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  const int n = 1 << k, half = n >> 1, quarter = n >> 2;
  const Split sh(half, wl), sq(quarter, wl), sn(n, wl);
  switch (op.kind) {
    case K_RY: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      pairs1<U>(x, half, j0, [&](Amp& a, Amp& b) {
        const Amp na = A::lin(c, a, ns, b);
        b = A::lin(s, a, c, b);
        a = na;
      }, wl);
      break;
    }
    case K_REAL2: {
      const R a0 = A::ld(cf[0]), b0 = A::ld(cf[1]), c0 = A::ld(cf[2]), d0 = A::ld(cf[3]);
      pairs1<U>(x, half, j0, [&](Amp& u, Amp& v) {
        const Amp nu = A::lin(a0, u, b0, v);
        v = A::lin(c0, u, d0, v);
        u = nu;
      }, wl);
      break;
    }
    case K_RX: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]);
      pairs1<U>(x, half, j0, [&](Amp& a, Amp& b) {
        const Amp na = A::rxc(c, a, s, b);
        b = A::rxc(c, b, s, a);
        a = na;
      }, wl);
      break;
    }
    case K_RZ:
    case K_DIAG1: {
      R p0r, p0i, p1r, p1i;
      if (op.kind == K_RZ) {
        R c = A::ld(cf[0]), s = A::ld(cf[1]);
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
      if (j0 >= 0) {
        const bool one0 = A::is_one(p0r, p0i), one1 = A::is_one(p1r, p1i);
        elems<U>(x, n, [&](int l, Amp& v) {
          const int b = (l >> j0) & 1;
          if (b ? one1 : one0) return;
          const R pr = b ? p1r : p0r, pi = b ? p1i : p0i;
          v = A::cm(pr, pi, v);
        }, wl);
      } else {
        if (f0)
          A::cacc(phr, phi, p1r, p1i);
        else
          A::cacc(phr, phi, p0r, p0i);
        ph = true;
      }
      break;
    }
    case K_GEN1: {
      const R a0 = A::ld(cf[0]), a1 = A::ld(cf[1]), b0 = A::ld(cf[2]), b1 = A::ld(cf[3]);
      const R c0 = A::ld(cf[4]), c1 = A::ld(cf[5]), d0 = A::ld(cf[6]), d1 = A::ld(cf[7]);
      pairs1<U>(x, half, j0, [&](Amp& u, Amp& v) {
        const Amp nu = A::cd(a0, a1, u, b0, b1, v);
        v = A::cd(c0, c1, u, d0, d1, v);
        u = nu;
      }, wl);
      break;
    }
    case K_X: {
      const int m = 1 << j0;
      for (int t = sh.s; t < sh.e; t += sh.st) {
        int i0 = ins0(t, j0), i1 = i0 | m;
        Amp u = x[i0];
        x[i0] = x[i1];
        x[i1] = u;
      }
      break;
    }
    case K_CNOT: {
      const int mt = 1 << j1;
      if (j0 >= 0) {
        const int mc = 1 << j0;
        for (int t = sq.s; t < sq.e; t += sq.st) {
          int i0 = ins00(t, j0, j1) | mc, i1 = i0 | mt;
          Amp u = x[i0];
          x[i0] = x[i1];
          x[i1] = u;
        }
      } else if (f0) {
        for (int t = sh.s; t < sh.e; t += sh.st) {
          int i0 = ins0(t, j1), i1 = i0 | mt;
          Amp u = x[i0];
          x[i0] = x[i1];
          x[i1] = u;
        }
      }
      break;
    }
    case K_CZ: {
      if (j0 >= 0 && j1 >= 0) {
        const int mm = (1 << j0) | (1 << j1);
        for (int t = sq.s; t < sq.e; t += sq.st) {
          int i = ins00(t, j0, j1) | mm;
          x[i] = A::neg(x[i]);
        }
      } else if (j0 >= 0 || j1 >= 0) {
        const int ja = j0 >= 0 ? j0 : j1;
        const int fb = j0 >= 0 ? f1 : f0;
        if (fb) {
          for (int t = sh.s; t < sh.e; t += sh.st) {
            int i = ins0(t, ja) | (1 << ja);
            x[i] = A::neg(x[i]);
          }
        }
      } else if (f0 && f1) {
        phr = A::rneg(phr);
        phi = A::rneg(phi);
        ph = true;
      }
      break;
    }
    case K_RZZ: {
      R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      if (j0 < 0 && j1 < 0) {
        if (f0 ^ f1)
          A::cacc(phr, phi, c, s);
        else
          A::cacc(phr, phi, c, ns);
        ph = true;
      } else {
        elems<U>(x, n, [&](int l, Amp& v) {
          const int b0 = j0 >= 0 ? (l >> j0) & 1 : f0;
          const int b1 = j1 >= 0 ? (l >> j1) & 1 : f1;
          v = A::cm(c, (b0 ^ b1) ? s : ns, v);
        }, wl);
      }
      break;
    }
    case K_RXX:
    case K_RYY: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      const int mm = (1 << j0) | (1 << j1);
      const bool yy = op.kind == K_RYY;
      // RXX: c x - i s x';  RYY: c x + i s sigma x', sigma = +1 when the two bits agree
      pairs_mask(x, half, j0, mm, [&](int i, Amp& a, Amp& b) {
        const R sp = (!yy) ? s : (((i >> j1) & 1) ? s : ns);
        const Amp na = A::rxc(c, a, sp, b);
        b = A::rxc(c, b, sp, a);
        a = na;
      }, wl);
      break;
    }
    case K_MIX2: {
      R c = A::ld(cf[0]), s = A::ld(cf[1]), pr = A::ld(cf[2]), pi = A::ld(cf[3]);
      const bool one11 = A::is_one(pr, pi);
      const int m0 = 1 << j0, m1 = 1 << j1;
      for (int t = sq.s; t < sq.e; t += sq.st) {
        int i00 = ins00(t, j0, j1);
        int i01 = i00 | m1, i10 = i00 | m0, i11 = i00 | m0 | m1;
        Amp a = x[i01], b = x[i10];
        x[i01] = A::rxc(c, a, s, b);
        x[i10] = A::rxc(c, b, s, a);
        if (!one11) x[i11] = A::cm(pr, pi, x[i11]);
      }
      break;
    }
    case K_GEN2:
      apply_gen2<A>(x, quarter, j0, j1, cf, wl);
      break;
    case K_PAULI: {
      const int l0 = op.aux & 0xff, l1 = (op.aux >> 8) & 0xff;
      R wr = A::ld(cf[0]), wi = A::ld(cf[1]);
      const int ny = (l0 == 2) + (l1 == 2);
      for (int q = 0; q < ny; ++q) {  // w *= i
        R t = wr;
        wr = A::rneg(wi);
        wi = t;
      }
      const bool mv0 = (l0 == 1 || l0 == 2), mv1 = (l1 == 1 || l1 == 2);
      const bool z0 = (l0 == 2 || l0 == 3), z1 = (l1 == 2 || l1 == 3);
      const int xm = (mv0 ? (1 << j0) : 0) | (mv1 ? (1 << j1) : 0);
      const int zl = ((z0 && j0 >= 0) ? (1 << j0) : 0) | ((z1 && j1 >= 0) ? (1 << j1) : 0);
      const int zf = ((z0 && j0 < 0) ? f0 : 0) ^ ((z1 && j1 < 0) ? f1 : 0);
      if (xm == 0) {
        for (int l = sn.s; l < sn.e; l += sn.st) {
          Amp v = A::cm(wr, wi, x[l]);
          x[l] = (parity(l & zl) ^ zf) ? A::neg(v) : v;
        }
      } else {
        const int lb = __ffs(xm) - 1;
        for (int t = sh.s; t < sh.e; t += sh.st) {
          int j = ins0(t, lb), p = j ^ xm;
          Amp a = x[j], b = x[p];
          Amp nb = A::cm(wr, wi, b), na = A::cm(wr, wi, a);
          x[j] = (parity(p & zl) ^ zf) ? A::neg(nb) : nb;
          x[p] = (parity(j & zl) ^ zf) ? A::neg(na) : na;
        }
      }
      break;
    }
    default:
      break;
  }
}

// Phase of one diagonal op for bit values (b0, b1), multiplied into (pr, pi).
template <class A>
__device__ __forceinline__ void diag_phase(const DOp& op, const float2* __restrict__ cf, int b0, int b1,
                                           typename A::R& pr, typename A::R& pi) {
  using R = typename A::R;
  switch (op.kind) {
    case K_RZ: {
      R c = A::ld(cf[0]), s = A::ld(cf[1]);
      A::cacc(pr, pi, c, b0 ? s : A::rneg(s));
      break;
    }
    case K_DIAG1:
      if (b0)
        A::cacc(pr, pi, A::ld(cf[2]), A::ld(cf[3]));
      else
        A::cacc(pr, pi, A::ld(cf[0]), A::ld(cf[1]));
      break;
    case K_CZ:
      if (b0 & b1) {
        pr = A::rneg(pr);
        pi = A::rneg(pi);
      }
      break;
    case K_RZZ: {
      R c = A::ld(cf[0]), s = A::ld(cf[1]);
      A::cacc(pr, pi, c, (b0 ^ b1) ? s : A::rneg(s));
      break;
    }
    default:
      break;
  }
}

// ------------------------------------------------------------------ relabelled sweeps
// The tile holds logical index l at physical slot A l ^ b (see DOp::c0).  Logical bit j of slot p is
// parity((p ^ b) & r_j); flipping logical bit j moves from p to p ^ c_j.

// pairs {p, p ^ m} (m = c_j), enumerated with the pivot q (a set bit of m) clear; u is the member whose
// logical bit is 0
template <int U, class Amp, class F>
__device__ __forceinline__ void pairs_lazy(Amp* x, int half, int q, int m, int r, int b, F f, int wl) {
  const Split sp(half, wl);
  const int nt = sp.st;
  int t = sp.s;
  for (; t + (U - 1) * nt < sp.e; t += U * nt) {
    int iu[U];
    Amp a[U], c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = ins0(t + u * nt, q);
      iu[u] = parity((p ^ b) & r) ? (p ^ m) : p;
      a[u] = x[iu[u]];
      c[u] = x[iu[u] ^ m];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) f(a[u], c[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      x[iu[u]] = a[u];
      x[iu[u] ^ m] = c[u];
    }
  }
  for (; t < sp.e; t += nt) {
    const int p = ins0(t, q);
    const int i0 = parity((p ^ b) & r) ? (p ^ m) : p;
    Amp a = x[i0], c = x[i0 ^ m];
    f(a, c);
    x[i0] = a;
    x[i0 ^ m] = c;
  }
}

// The phase of a diagonal op for the bit values (b0, b1); false when it is the identity.
template <class A>
__device__ __forceinline__ bool diag_coef(const DOp& op, const float2* __restrict__ cf, int b0, int b1,
                                          typename A::R& pr, typename A::R& pi) {
  switch (op.kind) {
    case K_RZ: {
      pr = A::ld(cf[0]);
      const typename A::R s = A::ld(cf[1]);
      pi = b0 ? s : A::rneg(s);
      return true;
    }
    case K_DIAG1:
      pr = A::ld(cf[b0 ? 2 : 0]);
      pi = A::ld(cf[b0 ? 3 : 1]);
      return !A::is_one(pr, pi);
    case K_RZZ: {
      pr = A::ld(cf[0]);
      const typename A::R s = A::ld(cf[1]);
      pi = (b0 ^ b1) ? s : A::rneg(s);
      return true;
    }
    case K_CZ:
      pr = (b0 & b1) ? A::rneg(A::rone()) : A::rone();
      pi = A::rzero();
      return b0 & b1;
    default:
      pr = A::rone();
      pi = A::rzero();
      return false;
  }
}

// A Pauli generator (w P, w = m[0] + i m[1], P on one or two qubits) in a relabelled sweep: logical index l lives
// at slot A l ^ b, so an X or Y letter on logical bit j flips the slot bits c_j (column j of A), and the sign of a
// Z or Y letter is logical bit j of the source slot, parity((p ^ b) & r_j) (row j of A^-1), or the fixed bit for
// a qubit outside the tile.  Each Y adds a factor i.  Same arithmetic as the K_PAULI case of apply_op.
template <class A>
__device__ __forceinline__ void apply_pauli_lazy(const DOp& op, typename A::Amp* x, int k, int j0, int j1, int f0,
                                                 int f1, const float2* __restrict__ cf, int b, int wl) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  const int n = 1 << k, half = n >> 1;
  const int l0 = op.aux & 0xff, l1 = (op.aux >> 8) & 0xff;
  R wr = A::ld(cf[0]), wi = A::ld(cf[1]);
  const int ny = (l0 == 2) + (l1 == 2);
  for (int q = 0; q < ny; ++q) {  // w *= i
    const R t = wr;
    wr = A::rneg(wi);
    wi = t;
  }
  const bool mv0 = l0 == 1 || l0 == 2, mv1 = l1 == 1 || l1 == 2;
  const bool z0 = l0 == 2 || l0 == 3, z1 = l1 == 2 || l1 == 3;
  const int xm = (mv0 ? (int)(uint16_t)op.c0 : 0) ^ (mv1 ? (int)(uint16_t)op.c1 : 0);
  const int zl = ((z0 && j0 >= 0) ? (int)(uint16_t)op.r0 : 0) ^ ((z1 && j1 >= 0) ? (int)(uint16_t)op.r1 : 0);
  const int zf = ((z0 && j0 < 0) ? f0 : 0) ^ ((z1 && j1 < 0) ? f1 : 0);
  if (xm == 0) {
    const Split sn(n, wl);
    for (int p = sn.s; p < sn.e; p += sn.st) {
      const Amp v = A::cm(wr, wi, x[p]);
      x[p] = (parity((p ^ b) & zl) ^ zf) ? A::neg(v) : v;
    }
  } else {
    const int lb = __ffs(xm) - 1;
    const Split sh(half, wl);
    for (int t = sh.s; t < sh.e; t += sh.st) {
      const int j = ins0(t, lb), p = j ^ xm;
      const Amp a = x[j], c = x[p];
      const Amp nc = A::cm(wr, wi, c), na = A::cm(wr, wi, a);
      x[j] = (parity((p ^ b) & zl) ^ zf) ? A::neg(nc) : nc;
      x[p] = (parity((j ^ b) & zl) ^ zf) ? A::neg(na) : na;
    }
  }
}

// One op of a relabelled sweep with at least one local bit (ops on fixed bits only go through apply_op:
// they only change the tile phase).  Rotations and dense single-qubit ops run over masked pairs; diagonal
// ops element by element with parity bits.
template <class A, int U>
__device__ __forceinline__ void apply_op_lazy(const DOp& op, typename A::Amp* x, int k, int j0, int j1, int f0,
                                              int f1, const float2* __restrict__ cf, int b, int wl) {
  using Amp = typename A::Amp;
  using R = typename A::R;
  const int n = 1 << k, half = n >> 1;
  switch (op.kind) {
    case K_RY: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]), ns = A::rneg(s);
      pairs_lazy<U>(x, half, op.q0, op.c0, op.r0, b, [&](Amp& a, Amp& v) {
        const Amp na = A::lin(c, a, ns, v);
        v = A::lin(s, a, c, v);
        a = na;
      }, wl);
      break;
    }
    case K_REAL2: {
      const R a0 = A::ld(cf[0]), b0 = A::ld(cf[1]), c0 = A::ld(cf[2]), d0 = A::ld(cf[3]);
      pairs_lazy<U>(x, half, op.q0, op.c0, op.r0, b, [&](Amp& u, Amp& v) {
        const Amp nu = A::lin(a0, u, b0, v);
        v = A::lin(c0, u, d0, v);
        u = nu;
      }, wl);
      break;
    }
    case K_RX: {
      const R c = A::ld(cf[0]), s = A::ld(cf[1]);
      pairs_lazy<U>(x, half, op.q0, op.c0, op.r0, b, [&](Amp& a, Amp& v) {
        const Amp na = A::rxc(c, a, s, v);
        v = A::rxc(c, v, s, a);
        a = na;
      }, wl);
      break;
    }
    case K_GEN1: {
      const R a0 = A::ld(cf[0]), a1 = A::ld(cf[1]), b0 = A::ld(cf[2]), b1 = A::ld(cf[3]);
      const R c0 = A::ld(cf[4]), c1 = A::ld(cf[5]), d0 = A::ld(cf[6]), d1 = A::ld(cf[7]);
      pairs_lazy<U>(x, half, op.q0, op.c0, op.r0, b, [&](Amp& u, Amp& v) {
        const Amp nu = A::cd(a0, a1, u, b0, b1, v);
        v = A::cd(c0, c1, u, d0, d1, v);
        u = nu;
      }, wl);
      break;
    }
    case K_RZ:
    case K_DIAG1:
    case K_RZZ:
    case K_CZ: {
      const int r0 = op.r0, r1 = op.r1;
      elems<U>(x, n, [&](int p, Amp& v) {
        const int bb0 = j0 >= 0 ? parity((p ^ b) & r0) : f0;
        const int bb1 = op.p1 < 0 ? 0 : (j1 >= 0 ? parity((p ^ b) & r1) : f1);
        R pr, pi;
        if (diag_coef<A>(op, cf, bb0, bb1, pr, pi)) v = A::cm(pr, pi, v);
      }, wl);
      break;
    }
    default:
      break;
  }
}

template <class A, int Q, int M0, int M1>
__device__ __forceinline__ void rot2_lazy_impl(typename A::Amp* x, int k, const DOp& mk, const DOp& m0,
                                               const DOp& m1, const Rot<A>& r0, const Rot<A>& r1, int b, int wl) {
  using Amp = typename A::Amp;
  const int quarter = 1 << (k - 2);
  const int lo = mk.q0 < mk.q1 ? mk.q0 : mk.q1, hi = mk.q0 < mk.q1 ? mk.q1 : mk.q0;
  const int c0 = m0.c0, c1 = m1.c0, s0 = m0.r0, s1 = m1.r0;
  const Split sp(quarter, wl);
  const int nt = sp.st;
  for (int t = sp.s; t < sp.e; t += nt) {
    const int p = ins0(ins0(t, lo), hi);
    const int base = p ^ (parity((p ^ b) & s0) ? c0 : 0) ^ (parity((p ^ b) & s1) ? c1 : 0);
    Amp a0 = x[base], a1 = x[base ^ c0], a2 = x[base ^ c1], a3 = x[base ^ c0 ^ c1];
    r0.template run<M0>(a0, a1);
    r0.template run<M0>(a2, a3);
    r1.template run<M1>(a0, a2);
    r1.template run<M1>(a1, a3);
    x[base] = a0;
    x[base ^ c0] = a1;
    x[base ^ c1] = a2;
    x[base ^ c0 ^ c1] = a3;
  }
}

template <class A, int Q>
struct Rot2LazyGo {
  typename A::Amp* x;
  int k;
  const DOp& mk;
  const DOp& m0;
  const DOp& m1;
  const Rot<A>& r0;
  const Rot<A>& r1;
  int b, wl;
  template <int M0, int M1>
  __device__ __forceinline__ void go() const {
    rot2_lazy_impl<A, Q, M0, M1>(x, k, mk, m0, m1, r0, r1, b, wl);
  }
};

template <class A, int Q>
__device__ __noinline__ void rot2_lazy_general(typename A::Amp* x, int k, const DOp mk, const DOp m0, const DOp m1,
                                               const Rot<A> r0, const Rot<A> r1, int b, int wl) {
  rot2_dispatch<A, false>(r0, r1, Rot2LazyGo<A, Q>{x, k, mk, m0, m1, r0, r1, b, wl});
}

template <class A, int Q, bool GENERAL_ONLY = false>
__device__ __forceinline__ void rot2_lazy(typename A::Amp* x, int k, const DOp& mk, const DOp& m0, const DOp& m1,
                                          const Rot<A>& r0, const Rot<A>& r1, int b, int wl) {
  if (GENERAL_ONLY)
    rot2_dispatch<A, false>(r0, r1, Rot2LazyGo<A, Q>{x, k, mk, m0, m1, r0, r1, b, wl});
  else if (r0.scaled)
    rot2_dispatch<A, true>(r0, r1, Rot2LazyGo<A, Q>{x, k, mk, m0, m1, r0, r1, b, wl});
  else
    rot2_lazy_general<A, Q>(x, k, mk, m0, m1, r0, r1, b, wl);
}

// Index tables of a column record (physical bit i -> mask cols[i]): lo[x] for bits 0..5, hi[y] for bits 6..
// of an index; the mapped index is lo[v & 63] ^ hi[v >> 6].  Built by the whole CTA (caller syncs).
__device__ __forceinline__ void build_index_tables(const uint16_t* __restrict__ cols, int k, uint16_t* tabs) {
  const int nl = k < 6 ? k : 6, nh = k - nl;
  for (int i = threadIdx.x; i < 64 + 128; i += blockDim.x) {
    const bool lo = i < 64;
    const int v = lo ? i : i - 64;
    const int nb = lo ? nl : nh, sh = lo ? 0 : 6;
    uint16_t m = 0;
    for (int t = 0; t < nb; ++t)
      if ((v >> t) & 1) m ^= cols[sh + t];
    tabs[i] = m;
  }
}

__device__ __forceinline__ int map_index(const uint16_t* tabs, int v) { return tabs[v & 63] ^ tabs[64 + (v >> 6)]; }

// Phase blocks.  The planner orders a block's members tile-constant | low half | high half | both halves
// of the k local (logical) bits, the low half being the first kl bits (kl chosen near k / 2 to leave the
// fewest members straddling the halves), and stores the four counts in the marker's c0, c1, r0, r1 and kl
// in its q0.  The block is applied as x[l] *= T_lo[l mod 2^kl] * T_hi[l >> kl], each table the product of
// the phases of the members living in that half; the tile-constant members are folded into T_lo, and
// members straddling both halves run afterwards as element-wise ops.
struct PhaseSplit {
  int nc, nlo, nhi, nmid, kl;
};
__device__ __forceinline__ PhaseSplit phase_split(const DOp& m) {
  return {(int)m.c0, (int)m.c1, (int)m.r0, (int)m.r1, (int)m.q0};
}

// Builds T_lo at tab[0, 2^kl) and T_hi at tab[2^kl, 2^kl + 2^(k - kl)) (the caller syncs before reading them).
// Returns the tables in use (bit 0: T_lo, bit 1: T_hi).  The tile-constant members go into the tables in
// use, split between them so that their product chains are about equally long; one thread builds each
// entry.  A block of tile-constant members only builds no table: their phase goes into the tile phase
// (phr, phi).  The real factor `fold` is multiplied into T_lo, or into T_hi when T_lo is not in use.
template <class A>
__device__ __forceinline__ int phase_tables(const DOp* __restrict__ blk, const float2* __restrict__ bcf,
                                            const PhaseSplit& ps, const SweepDesc& sd, int k, int64_t base,
                                            typename A::Amp* tab, typename A::R& phr, typename A::R& phi,
                                            bool& ph, int lim, int st, typename A::R fold = A::rone()) {
  using R = typename A::R;
  if (ps.nlo == 0 && ps.nhi == 0) {
    for (int t = 0; t < ps.nc; ++t) {
      const DOp op = blk[t];
      if (op.gidx >= lim || op.gidx < st) continue;
      const int f0 = (int)((base >> op.p0) & 1);
      const int f1 = op.p1 >= 0 ? (int)((base >> op.p1) & 1) : 0;
      diag_phase<A>(op, bcf + 4 * t, f0, f1, phr, phi);
      ph = true;
    }
    return 0;
  }
  const int kl = ps.kl, nlo = 1 << kl, nhi = 1 << (k - kl);
  const int use = (ps.nlo > 0 ? 1 : 0) | (ps.nhi > 0 ? 2 : 0);
  // tile-constant members [0, a) into T_lo, [a, nc) into T_hi
  int a = use == 1 ? ps.nc : use == 2 ? 0 : (ps.nc + ps.nhi - ps.nlo) / 2;
  a = a < 0 ? 0 : (a > ps.nc ? ps.nc : a);
  const int t_lo = ps.nc, t_hi = ps.nc + ps.nlo;
  for (int i = threadIdx.x; i < nlo + nhi; i += blockDim.x) {
    const bool lo = i < nlo;
    if (!(use & (lo ? 1 : 2))) continue;
    R pr = A::rone(), pi = A::rzero();
    {
      const int idx = lo ? i : i - nlo;
      const int shift = lo ? 0 : kl;
      // this table's members: [s1, s1 + n1) then [s2, ...)
      const int s1 = lo ? 0 : a, n1 = lo ? a : ps.nc - a;
      const int s2 = lo ? t_lo : t_hi, nn = n1 + (lo ? ps.nlo : ps.nhi);
#pragma unroll 1
      for (int u = 0; u < nn; ++u) {
        const int t = u < n1 ? s1 + u : s2 + (u - n1);
        const DOp op = blk[t];
        if (op.gidx >= lim || op.gidx < st) continue;
        const int j0 = sd.local_of[op.p0];
        const int j1 = op.p1 >= 0 ? sd.local_of[op.p1] : -1;
        const int b0 = j0 >= 0 ? (idx >> (j0 - shift)) & 1 : (int)((base >> op.p0) & 1);
        const int b1 = op.p1 < 0 ? 0 : (j1 >= 0 ? (idx >> (j1 - shift)) & 1 : (int)((base >> op.p1) & 1));
        diag_phase<A>(op, bcf + 4 * t, b0, b1, pr, pi);
      }
    }
    if (lo || !(use & 1)) {
      pr = A::rmul(pr, fold);
      pi = A::rmul(pi, fold);
    }
    tab[i] = A::cplx(pr, pi);
  }
  return use;
}

// x[p] *= the tables' phases at the logical index of slot p (p itself, or A^-1 (p ^ b) in a relabelled
// sweep, from the block's index tables itab)
template <class A, bool LAZY, int U = 4>
__device__ __forceinline__ void phase_apply(typename A::Amp* x, int k, int kl, const typename A::Amp* __restrict__ tab,
                                            int use, const uint16_t* __restrict__ itab, int b) {
  using Amp = typename A::Amp;
  const int nlo = 1 << kl, n = 1 << k, nt = blockDim.x;
  const int lb = LAZY ? map_index(itab, b) : 0;
  int p = threadIdx.x;
  for (; p + (U - 1) * nt < n; p += U * nt) {
    Amp v[U];
    int l[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      l[u] = LAZY ? (map_index(itab, p + u * nt) ^ lb) : p + u * nt;
      v[u] = x[p + u * nt];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (use & 1) {
        const Amp t = tab[l[u] & (nlo - 1)];
        v[u] = A::cm(A::real(t), A::imag(t), v[u]);
      }
      if (use & 2) {
        const Amp t = tab[nlo + (l[u] >> kl)];
        v[u] = A::cm(A::real(t), A::imag(t), v[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) x[p + u * nt] = v[u];
  }
  for (; p < n; p += nt) {
    const int l = LAZY ? (map_index(itab, p) ^ lb) : p;
    Amp v = x[p];
    if (use & 1) {
      const Amp t = tab[l & (nlo - 1)];
      v = A::cm(A::real(t), A::imag(t), v);
    }
    if (use & 2) {
      const Amp t = tab[nlo + (l >> kl)];
      v = A::cm(A::real(t), A::imag(t), v);
    }
    x[p] = v;
  }
}

// The block's members that straddle both halves, one element-wise pass each (block-wide barrier first).
template <class A, bool LAZY>
__device__ __forceinline__ void phase_mid(const DOp* __restrict__ blk, const float2* __restrict__ bcf,
                                          const PhaseSplit& ps, const SweepDesc& sd, typename A::Amp* x, int k,
                                          int b, typename A::R& phr, typename A::R& phi, bool& ph, int lim, int st) {
  const int t0 = ps.nc + ps.nlo + ps.nhi;
  for (int t = t0; t < t0 + ps.nmid; ++t) {
    const DOp op = blk[t];
    if (op.gidx >= lim || op.gidx < st) continue;
    const int j0 = sd.local_of[op.p0];
    const int j1 = op.p1 >= 0 ? sd.local_of[op.p1] : -1;
    __syncthreads();
    if (LAZY)
      apply_op_lazy<A, 2>(op, x, k, j0, j1, 0, 0, bcf + 4 * t, b, -1);
    else
      apply_op<A>(op, x, k, j0, j1, 0, 0, bcf + 4 * t, phr, phi, ph);
  }
}

// One phase block on one tile (rec: the block's index record in a relabelled sweep).  The caller has
// synchronised the CTA since the previous block's tables were read (and since *scale, the pending real
// factor of scaled rotations, was last written).  *scale is folded into the tables when the block builds
// any, and then reset to 1.  Returns whether it was (the tables in use).
template <class A, bool LAZY>
__device__ __forceinline__ int phase_block(const DOp& mk, const DOp* __restrict__ blk, const float2* __restrict__ bcf,
                                            const SweepDesc& sd, typename A::Amp* x, int k, int64_t base,
                                            typename A::Amp* tab, uint16_t* itab, const uint16_t* __restrict__ rec,
                                            int b, typename A::R& phr, typename A::R& phi, bool& ph, int lim,
                                            int st, typename A::R* scale) {
  const PhaseSplit ps = phase_split(mk);
  const int use = phase_tables<A>(blk, bcf, ps, sd, k, base, tab, phr, phi, ph, lim, st, *scale);
  if (use) {
    if (LAZY) build_index_tables(rec, k, itab);
    __syncthreads();
    if (threadIdx.x == 0) *scale = A::rone();  // folded into the tables
    phase_apply<A, LAZY>(x, k, ps.kl, tab, use, itab, b);
  }
  phase_mid<A, LAZY>(blk, bcf, ps, sd, x, k, b, phr, phi, ph, lim, st);
  return use;
}

}  // namespace pqc
