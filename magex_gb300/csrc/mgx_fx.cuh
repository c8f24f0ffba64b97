// Fixed-point integer gather shared by the LLG (mgx_llg_fx.cu) and Monte Carlo (mgx_mc.cu) kernels:
// spins and couplings as fixed-point values in two balanced int32 halves, products and sums exact in
// int64 accumulators with 32x32->64-bit multiply-adds.
#pragma once

#include "mgx_internal.cuh"

namespace mgx {

// Two fixed-point formats: LIMB = 24 (MGX_PRECISION_INT48_GATHER, 48-bit values, FP32-pair tail) and
// LIMB = 28 (MGX_PRECISION_FP64_FIXED_GATHER, 56-bit values, FP64 tail).  A value is v = round(x 2^(2 LIMB))
// held as v = hi 2^LIMB + lo with hi = round(v / 2^LIMB) and lo in [-2^(LIMB-1), 2^(LIMB-1)): balanced
// halves, so that the dropped lo x lo products have zero mean.
template <int LIMB>
__device__ __forceinline__ int2 fx_halves(long long v) {
  const long long hi = (v + (1LL << (LIMB - 1))) >> LIMB;
  return make_int2((int)hi, (int)(v - (hi << LIMB)));
}

// round(x 2^(2 LIMB)) (ties to even) in two halves, on the integer pipes
template <int LIMB>
__device__ __forceinline__ int2 fx_split(double x) {
  return fx_halves<LIMB>(double_to_ll_scaled(x, 2 * LIMB));
}

// the same, with the hardware conversion when hw (x 2^(2 LIMB) is exact, a power-of-two scaling)
template <int LIMB>
__device__ __forceinline__ int2 fx_split(double x, int hw) {
  return hw ? fx_halves<LIMB>(__double2ll_rn(x * (double)(1LL << (2 * LIMB)))) : fx_split<LIMB>(x);
}

// c + a b exactly (64-bit two's complement), as a carry chain on the 32-bit halves: the low word of
// the product added with carry out, then the signed high word with that carry in.  Timed against
// `mad.wide.s32` on the bcc 128^3 step (CUDA events, 100 steps, identical spins): 1.089 against
// 1.185 ms per step, with fewer spilled registers.
__device__ __forceinline__ long long mad_wide(int a, int b, long long c) {
  long long d;
  asm("{\n\t"
      ".reg .u32 lo, hi;\n\t"
      "mov.b64 {lo, hi}, %3;\n\t"
      "mad.lo.cc.u32 lo, %1, %2, lo;\n\t"
      "madc.hi.s32 hi, %1, %2, hi;\n\t"
      "mov.b64 %0, {lo, hi};\n\t"
      "}"
      : "=l"(d)
      : "r"(a), "r"(b), "l"(c));
  return d;
}

struct FxAcc {
  long long hh[3] = {0, 0, 0};   // sum J_hi e_hi             (units 2^(sigma - 2 LIMB))
  long long x[3] = {0, 0, 0};    // sum J_hi e_lo + J_lo e_hi (units 2^(sigma - 3 LIMB))
};

// acc += M x for a 3x3 fixed-point tensor M (10 (hi, lo) int pairs, 80 B) and a fixed-point spin x
__device__ __forceinline__ void fx_mat(const int4* __restrict__ T, int2 x0, int2 x1, int2 x2, FxAcc& a) {
  const int4 t01 = __ldg(T), t23 = __ldg(T + 1), t45 = __ldg(T + 2), t67 = __ldg(T + 3), t89 = __ldg(T + 4);
  const int2 m[9] = {make_int2(t01.x, t01.y), make_int2(t01.z, t01.w), make_int2(t23.x, t23.y),
                     make_int2(t23.z, t23.w), make_int2(t45.x, t45.y), make_int2(t45.z, t45.w),
                     make_int2(t67.x, t67.y), make_int2(t67.z, t67.w), make_int2(t89.x, t89.y)};
  const int2 xv[3] = {x0, x1, x2};
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int2 j = m[3 * c + d];
      a.hh[c] = mad_wide(j.x, xv[d].x, a.hh[c]);
      a.x[c] = mad_wide(j.x, xv[d].y, mad_wide(j.y, xv[d].x, a.x[c]));
    }
}

// Accumulate the exchange (+ on-site) sum of lattice index q = (s, c0, c1, c2) from the fixed-point
// field xs into a (hh in units of F.scale[s], x in units 2^-LIMB of that).  Interior cells (whole
// stencil inside the supercell along axes 0 and 1) index neighbours as q + a per-coupling constant,
// corrected for the periodic seam of axis 2.
__device__ __forceinline__ void fx_accumulate(const DevLattice& L, const DevFX& F, const int2* __restrict__ xs,
                                              long long q, int s, int c0, int c1, int c2, FxAcc& a) {
  const long long N = L.N;
  const int b0 = __ldg(L.bond_off + s), b1 = __ldg(L.bond_off + s + 1);
  const int4 r = F.reach[s];
  const bool inner01 = c0 >= r.x && c0 < L.L0 - r.x && c1 >= r.y && c1 < L.L1 - r.y;
  const bool inner2 = L.pbc2 ? r.z < L.L2 : (c2 >= r.z && c2 < L.L2 - r.z);
  if (inner01 && inner2) {
    // 32-bit index arithmetic (N < 2^31 for every lattice this path accepts)
    const int2* __restrict__ x0 = xs;
    const int2* __restrict__ x1 = xs + N;
    const int2* __restrict__ x2 = xs + 2 * N;
    const int qi = (int)q, L2 = L.L2;
    for (int b = b0; b < b1; ++b) {
      const int2 li = __ldg(F.lin + b);
      const int n2 = c2 + li.y;
      const int j = qi + li.x + (n2 < 0 ? L2 : 0) - (n2 >= L2 ? L2 : 0);
      fx_mat(F.J + 5 * b, __ldg(x0 + j), __ldg(x1 + j), __ldg(x2 + j), a);
    }
  } else {
    for (int b = b0; b < b1; ++b) {
      const int4 g = __ldg(L.bond_geo + b);
      int n0 = c0 + g.y, n1 = c1 + g.z, n2 = c2 + g.w;
      bool ok = true;
      if (L.pbc0) { n0 -= (n0 >= L.L0) ? L.L0 : 0; } else { ok &= (unsigned)n0 < (unsigned)L.L0; }
      if (L.pbc1) { n1 -= (n1 >= L.L1) ? L.L1 : 0; } else { ok &= (unsigned)n1 < (unsigned)L.L1; }
      if (L.pbc2) { n2 -= (n2 >= L.L2) ? L.L2 : 0; } else { ok &= (unsigned)n2 < (unsigned)L.L2; }
      if (!ok) continue;
      const long long j = (long long)g.x * L.ncell + ((long long)n0 * L.L1 + n1) * L.L2 + n2;
      fx_mat(F.J + (long long)b * 5, __ldg(xs + j), __ldg(xs + N + j), __ldg(xs + 2 * N + j), a);
    }
  }
  if (F.A) fx_mat(F.A + 5 * s, __ldg(xs + q), __ldg(xs + N + q), __ldg(xs + 2 * N + q), a);
}

// Tables of a lattice model for the fixed-point gather (host): couplings as 3x3 fixed-point tensors at a
// per-sublattice scale, the interior fast-path offsets, and `ncopies` (3, N) split arrays of spins.
// field_scaled: couplings 2 J / (mu mu_B) plus the on-site -2 A / (mu mu_B) as a self-coupling (the
// LLG field, tesla); otherwise the plain couplings J (the exchange field h of energy differences, meV).
mgx_status fx_build(const Model* m, int limb, bool field_scaled, int ncopies, DevFX* fx, void** block);
// Fixed-point split of n doubles x into xs (limb 24 or 28).
void enqueue_fx_split_n(const double* x, int2* xs, long long n, int limb, cudaStream_t st);

}  // namespace mgx
