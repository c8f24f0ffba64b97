// Per-site bodies of the fixed-point-gather step forms (MGX_PRECISION_INT48_GATHER and
// MGX_PRECISION_FP64_FIXED_GATHER), shared by the single-lattice kernels (mgx_llg_fx.cu) and the
// batched ensemble (mgx_batch.cu).  See mgx_llg_fx.cu for the arithmetic.
#pragma once

#include "mgx_dfp.cuh"
#include "mgx_fx.cuh"
#include "mgx_step.cuh"

namespace mgx {

// 48-bit form: field as (hi, lo) float pairs in tesla
__device__ __forceinline__ void fx_gather(const DevLattice& L, const DevFX& F, const int2* __restrict__ xs,
                                          long long q, int s, int c0, int c1, int c2, dfp h[3]) {
  FxAcc a;
  fx_accumulate(L, F, xs, q, s, c0, c1, c2, a);
  const float sc = (float)F.scale[s];            // >= 2^-100 (checked when the tables are built)
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // value = (hh + x 2^-24) 2^(sigma - 48); fold x in with rounding, then split into two floats
    const long long v = a.hh[c] + ((a.x[c] + (1LL << 23)) >> 24);
    const float hi = __ll2float_rn(v);
    const float lo = __ll2float_rn(v - __float2ll_rn(hi));
    h[c] = {__fmul_rn(hi, sc), __fmul_rn(lo, sc)};
  }
}

// Where the conversions of the fixed-point forms run (DevFX::hw_convert): HWC = 2 reads the plan's
// flag at run time; 0 / 1 fix the integer pipes / the hardware converters at compile time (kernels
// that carry no branch for it: the batched stages and the adjoint's recomputation, capped at few
// registers, keep the integer pipes).
template <int HWC>
__device__ __forceinline__ bool fx_hw(const DevFX& F) {
  return HWC == 2 ? F.hw_convert != 0 : HWC == 1;
}

// 56-bit form: field in FP64 = (hh + x 2^-28) 2^(sigma - 56): x rounded to units of 2^(sigma - 56)
// in integer arithmetic (|t| < 2^58), then t converted to FP64 and scaled by the power of two in one
// rounding, on the integer pipes or the hardware converter (the same value)
template <int HWC = 2>
__device__ __forceinline__ void fx_gather64(const DevLattice& L, const DevFX& F, const int2* __restrict__ xs,
                                            long long q, int s, int c0, int c1, int c2, double h[3]) {
  FxAcc a;
  fx_accumulate(L, F, xs, q, s, c0, c1, c2, a);
  const int e2 = F.scale_exp[s];
  const double sc = F.scale[s];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const long long t = a.hh[c] + ((a.x[c] + (1LL << 27)) >> 28);
    h[c] = fx_hw<HWC>(F) ? __ll2double_rn(t) * sc : ll_to_double_scaled(t, e2);   // the same rounding
  }
}

// spin of the site as a (hi, lo) float pair from its fixed-point halves (exact)
__device__ __forceinline__ dfp fx_spin(int2 v) {
  return {__fmul_rn((float)v.x, 5.9604644775390625e-8f), __fmul_rn((float)v.y, 3.552713678800501e-15f)};
}

template <int NOISE>
__device__ __forceinline__ void fx_thermal(const DevLattice& L, const DevLLG& P, const DevFX& F,
                                           const double* __restrict__ noise, long long q, int s, uint64_t step,
                                           dfp B[3]) {
  if (NOISE == MGX_NOISE_NONE) return;
  double g[3];
  if (NOISE == MGX_NOISE_HOST) {
    g[0] = __ldg(noise + q);
    g[1] = __ldg(noise + L.N + q);
    g[2] = __ldg(noise + 2 * L.N + q);
  } else {
    philox_normal3(P.seed, magex_site(L, q, s), step, g[0], g[1], g[2]);   // FP32 draws: exact as floats
  }
  if (NOISE == MGX_NOISE_PHILOX && !P.sigma_site) {
    const dfp sg = dfp_of(F.sig[s]);
#pragma unroll
    for (int c = 0; c < 3; ++c) B[c] = dfp_add(B[c], dfp_mul(sg, {(float)g[c], 0.f}));
  } else {
    const double sig = P.sigma_site ? __ldg(P.sigma_site + q) : __ldg(P.sigma_sub + s);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 b = split_double(sig * g[c]);
      B[c] = dfp_add(B[c], {b.x, b.y});
    }
  }
}

template <int NOISE>
__device__ __forceinline__ void fx_rhs(const DevLattice& L, const DevLLG& P, const DevFX& F,
                                       const int2* __restrict__ xs, const double* __restrict__ noise, long long q,
                                       int s, int c0, int c1, int c2, uint64_t step, double f[3]) {
  dfp B[3], e[3], fd[3];
  fx_gather(L, F, xs, q, s, c0, c1, c2, B);
#pragma unroll
  for (int c = 0; c < 3; ++c) B[c] = dfp_add(B[c], dfp_of(F.B[c]));
  fx_thermal<NOISE>(L, P, F, noise, q, s, step, B);
  const long long N = L.N;
  e[0] = fx_spin(xs[q]);
  e[1] = fx_spin(xs[N + q]);
  e[2] = fx_spin(xs[2 * N + q]);
  dfp_rhs(e, B, dfp_of(F.alpha[s]), dfp_of(F.pre[s]), P.precession != 0, fd);
#pragma unroll
  for (int c = 0; c < 3; ++c) f[c] = dfp_double(fd[c]);
}

// FP64 field of the site from the integer gather (+ Zeeman and thermal): the 56-bit form's field, and
// the field of the Depondt integrator for both forms.  HIGHER (56-bit form only, a separate
// instantiation) adds the cubic and higher-uniaxial fields at the site's FP64 spin (sx, sy, sz), in the
// place the FP64 kernels add them: after the effective field, before the thermal field.
// NC (Philox noise of the 56-bit form): 1 draws the normals and stores them in F.nz, 2 reads them
// back from F.nz (the corrector of the same step), 0 draws them.
template <int NOISE, int PREC, bool HIGHER = false, int HWC = 2, int NC = 0>
__device__ __forceinline__ void fx_field64(const DevLattice& L, const DevLLG& P, const DevFX& F,
                                           const int2* __restrict__ xs, const double* __restrict__ noise,
                                           long long q, int s, int c0, int c1, int c2, uint64_t step, double& bx,
                                           double& by, double& bz, double sx = 0.0, double sy = 0.0,
                                           double sz = 0.0) {
  double h[3];
  if (PREC == MGX_PRECISION_FP64_FIXED_GATHER) {
    fx_gather64<HWC>(L, F, xs, q, s, c0, c1, c2, h);
  } else {
    dfp hp[3];
    fx_gather(L, F, xs, q, s, c0, c1, c2, hp);
    h[0] = dfp_double(hp[0]);
    h[1] = dfp_double(hp[1]);
    h[2] = dfp_double(hp[2]);
  }
  bx = h[0] + L.B0;
  by = h[1] + L.B1;
  bz = h[2] + L.B2;
  if (HIGHER) add_higher_onsite(L, q, s, sx, sy, sz, bx, by, bz);
  if (NOISE == MGX_NOISE_PHILOX && NC != 0) {
    const long long N = L.N;
    float f0, f1, f2;
    if (NC == 1) {
      philox_normal3f(P.seed, magex_site(L, q, s), step, f0, f1, f2);
      F.nz[q] = f0; F.nz[N + q] = f1; F.nz[2 * N + q] = f2;
    } else {
      f0 = F.nz[q]; f1 = F.nz[N + q]; f2 = F.nz[2 * N + q];
    }
    const bool hw = fx_hw<HWC>(F);
    const double sig = P.sigma_site ? __ldg(P.sigma_site + q) : __ldg(P.sigma_sub + s);
    bx = fma(sig, hw ? (double)f0 : f32_to_f64(f0), bx);
    by = fma(sig, hw ? (double)f1 : f32_to_f64(f1), by);
    bz = fma(sig, hw ? (double)f2 : f32_to_f64(f2), bz);
  } else {
    add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz, PREC == MGX_PRECISION_FP64_FIXED_GATHER && fx_hw<HWC>(F));
  }
}

// Predictor of site q (0 <= q < L.N) of the fixed-point forms: writes P.ep, P.k1 and the split F.eps at q.
// HIGHER: the 56-bit form with the model's cubic / higher-uniaxial terms.  The adjoint's recomputation
// (56-bit Heun form) also stores the total field (Hout) and the inverse norm of the predictor (rout).
template <int NOISE, int INTEG, int PREC, bool HIGHER = false, int HWC = 2, bool NCACHE = false>
__device__ __forceinline__ void fx_predict_site(const DevLattice& L, const DevLLG& P, const DevFX& F,
                                                const double* __restrict__ e, const double* __restrict__ noise,
                                                long long q, uint64_t step, double* __restrict__ Hout = nullptr,
                                                double* __restrict__ rout = nullptr) {
  constexpr int LIMB = PREC == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24;
  const long long N = L.N;
  const double ex = e[q], ey = e[N + q], ez = e[2 * N + q];
  if (L.pinned && L.pinned[q]) {
    P.ep[q] = ex; P.ep[N + q] = ey; P.ep[2 * N + q] = ez;
    P.k1[q] = 0.0; P.k1[N + q] = 0.0; P.k1[2 * N + q] = 0.0;
    F.eps[q] = F.es[q]; F.eps[N + q] = F.es[N + q]; F.eps[2 * N + q] = F.es[2 * N + q];
    if (Hout) {
      Hout[q] = 0.0; Hout[N + q] = 0.0; Hout[2 * N + q] = 0.0;
    }
    return;
  }
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double f[3], x, y, z;
  if (INTEG == MGX_INTEGRATOR_HEUN) {
    if (PREC == MGX_PRECISION_FP64_FIXED_GATHER) {
      double bx, by, bz;
      fx_field64<NOISE, PREC, HIGHER, HWC, NCACHE ? 1 : 0>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, bx, by, bz, ex, ey, ez);
      if (Hout) {
        Hout[q] = bx; Hout[N + q] = by; Hout[2 * N + q] = bz;
      }
      llg_rhs(ex, ey, ez, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, f[0], f[1],
              f[2]);
    } else {
      fx_rhs<NOISE>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, f);
    }
    x = fma(P.dt, f[0], ex);
    y = fma(P.dt, f[1], ey);
    z = fma(P.dt, f[2], ez);
    const double r = rsqrt(x * x + y * y + z * z);
    if (rout) rout[q] = r;
    x *= r; y *= r; z *= r;
  } else {
    double bx, by, bz;
    fx_field64<NOISE, PREC, HIGHER, HWC, NCACHE ? 1 : 0>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, bx, by, bz, ex, ey, ez);
    double fx, fy, fz;
    llg_rhs(ex, ey, ez, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, fx, fy, fz);
    f[0] = ey * fz - ez * fy; f[1] = ez * fx - ex * fz; f[2] = ex * fy - ey * fx;
    x = ex; y = ey; z = ez;
    rotate(x, y, z, P.dt * f[0], P.dt * f[1], P.dt * f[2]);
  }
  P.ep[q] = x; P.ep[N + q] = y; P.ep[2 * N + q] = z;
  P.k1[q] = f[0]; P.k1[N + q] = f[1]; P.k1[2 * N + q] = f[2];
  F.eps[q] = fx_split<LIMB>(x, fx_hw<HWC>(F)); F.eps[N + q] = fx_split<LIMB>(y, fx_hw<HWC>(F));
  F.eps[2 * N + q] = fx_split<LIMB>(z, fx_hw<HWC>(F));
}

// the new spins of lattice site q (stencil layout) as row cell*ns + s of a magex-order (N, 3) array
__device__ __forceinline__ void store_site_row(const DevLattice& L, double* __restrict__ rows, long long q, int s,
                                               double x, double y, double z) {
  double* r = rows + 3 * ((q - (long long)s * L.ncell) * L.ns + s);
  r[0] = x; r[1] = y; r[2] = z;
}

// Corrector of site q: reads the neighbours' F.eps, P.k1 and e at q, writes e and its split F.es at q
// (the new spins to eout instead of e when given; Hout and rout as in fx_predict_site).  With rows
// (the last stage of a step on host buffers, stencil layout) the new spins go to the magex-order rows
// `rows` only, and neither e nor its split is written.
template <int NOISE, int INTEG, int PREC, bool HIGHER = false, int HWC = 2, bool NCACHE = false>
__device__ __forceinline__ void fx_correct_site(const DevLattice& L, const DevLLG& P, const DevFX& F,
                                                double* __restrict__ e, const double* __restrict__ noise, long long q,
                                                uint64_t step, double* __restrict__ Hout = nullptr,
                                                double* __restrict__ eout = nullptr,
                                                double* __restrict__ rout = nullptr,
                                                double* __restrict__ rows = nullptr) {
  constexpr int LIMB = PREC == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24;
  if (L.pinned && L.pinned[q]) {                       // e and its split stay as they are
    if (rows) store_site_row(L, rows, q, (int)(q / L.ncell), e[q], e[L.N + q], e[2 * L.N + q]);
    if (eout) {
      eout[q] = e[q]; eout[L.N + q] = e[L.N + q]; eout[2 * L.N + q] = e[2 * L.N + q];
    }
    if (Hout) {
      Hout[q] = 0.0; Hout[L.N + q] = 0.0; Hout[2 * L.N + q] = 0.0;
    }
    return;
  }
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  const double k1x = P.k1[q], k1y = P.k1[N + q], k1z = P.k1[2 * N + q];
  double x = e[q], y = e[N + q], z = e[2 * N + q];
  if (INTEG == MGX_INTEGRATOR_HEUN) {
    double f[3];
    if (PREC == MGX_PRECISION_FP64_FIXED_GATHER) {
      const double px = P.ep[q], py = P.ep[N + q], pz = P.ep[2 * N + q];
      double bx, by, bz;
      fx_field64<NOISE, PREC, HIGHER, HWC, NCACHE ? 2 : 0>(L, P, F, F.eps, noise, q, s, c0, c1, c2, step, bx, by, bz, px, py, pz);
      if (Hout) {
        Hout[q] = bx; Hout[N + q] = by; Hout[2 * N + q] = bz;
      }
      llg_rhs(px, py, pz, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, f[0], f[1],
              f[2]);
    } else {
      fx_rhs<NOISE>(L, P, F, F.eps, noise, q, s, c0, c1, c2, step, f);
    }
    x = fma(P.half_dt, k1x + f[0], x);
    y = fma(P.half_dt, k1y + f[1], y);
    z = fma(P.half_dt, k1z + f[2], z);
  } else {
    const double px = P.ep[q], py = P.ep[N + q], pz = P.ep[2 * N + q];
    double bx, by, bz;
    fx_field64<NOISE, PREC, HIGHER, HWC, NCACHE ? 2 : 0>(L, P, F, F.eps, noise, q, s, c0, c1, c2, step, bx, by, bz, px, py, pz);
    double fx, fy, fz;
    llg_rhs(px, py, pz, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, fx, fy, fz);
    const double wx = py * fz - pz * fy, wy = pz * fx - px * fz, wz = px * fy - py * fx;
    rotate(x, y, z, P.half_dt * (k1x + wx), P.half_dt * (k1y + wy), P.half_dt * (k1z + wz));
  }
  const double r = rsqrt(x * x + y * y + z * z);
  if (rout) rout[q] = r;
  x *= r; y *= r; z *= r;
  if (rows) {
    store_site_row(L, rows, q, s, x, y, z);
    return;
  }
  double* o = eout ? eout : e;
  o[q] = x; o[N + q] = y; o[2 * N + q] = z;
  F.es[q] = fx_split<LIMB>(x, fx_hw<HWC>(F)); F.es[N + q] = fx_split<LIMB>(y, fx_hw<HWC>(F));
  F.es[2 * N + q] = fx_split<LIMB>(z, fx_hw<HWC>(F));
}

}  // namespace mgx
