// Heun / Depondt step with the exchange gather as exact integer arithmetic (MGX_PRECISION_INT48_GATHER).
//
// On GB300 the INT32 multiply-add pipe runs 64 operations per clock per SM and the FP64 pipe 2, so
// h = sum_j J_ij e_j (9 z multiply-adds per site and stage) is evaluated in fixed point:
//   * every spin component is held as v = round(e 2^48) (|v| <= 2^48) in two int32 halves,
//     v = hi 2^24 + lo with lo in [-2^23, 2^23), written by the stage that produces the spins;
//   * every coupling entry (pre-scaled by 2 / (mu mu_B) of the receiving sublattice) and the on-site
//     tensor -2 A / (mu mu_B) likewise, at a power-of-two scale 2^sigma_s >= their largest magnitude;
//   * J e = [J_hi e_hi 2^48 + (J_hi e_lo + J_lo e_hi) 2^24 + J_lo e_lo] 2^(sigma - 96): the first
//     two terms are accumulated exactly with 32x32->64-bit multiply-adds (mad.wide.s32) in two int64
//     accumulators (at most 2^55 and 2^56 for 26 neighbours); the last (|J_lo e_lo| <= 2^46, zero
//     mean with balanced halves) is dropped.
// The sum is exact; the only errors are the 2^-49 roundings of the spins and couplings to fixed point,
// about 1e-11 T in the field of the 26-neighbour bcc workload (FP64's own rounding of the gather is
// of the same order).  The accumulators are turned into (hi, lo) float pairs, the Zeeman and thermal
// fields and the right-hand side are evaluated on pairs (mgx_dfp.cuh) and the integration,
// renormalisation and fixed-point split of the new spins are FP64.  The Depondt form keeps an FP64
// tail after the integer gather.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

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

// 56-bit form: field in FP64, (hh + x 2^-28) 2^(sigma - 56) with one final rounding
__device__ __forceinline__ void fx_gather64(const DevLattice& L, const DevFX& F, const int2* __restrict__ xs,
                                            long long q, int s, int c0, int c1, int c2, double h[3]) {
  FxAcc a;
  fx_accumulate(L, F, xs, q, s, c0, c1, c2, a);
  const double sc = F.scale[s];
#pragma unroll
  for (int c = 0; c < 3; ++c) h[c] = fma((double)a.x[c], 3.7252902984619141e-9, (double)a.hh[c]) * sc;
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
// the field of the Depondt integrator for both forms
template <int NOISE, int PREC>
__device__ __forceinline__ void fx_field64(const DevLattice& L, const DevLLG& P, const DevFX& F,
                                           const int2* __restrict__ xs, const double* __restrict__ noise,
                                           long long q, int s, int c0, int c1, int c2, uint64_t step, double& bx,
                                           double& by, double& bz) {
  double h[3];
  if (PREC == MGX_PRECISION_FP64_FIXED_GATHER) {
    fx_gather64(L, F, xs, q, s, c0, c1, c2, h);
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
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
}

template <int PREC>
__global__ void __launch_bounds__(256) k_fx_split(const double* __restrict__ x, int2* __restrict__ xs, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xs[i] = fx_split<PREC == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24>(x[i]);
}

template <int NOISE, int INTEG, int PREC>
__global__ void __launch_bounds__(256, 4) k_predict_fx(const DevLattice L, const DevLLG P, const DevFX F,
                                                       const double* __restrict__ e, const double* __restrict__ noise,
                                                       uint64_t step) {
  constexpr int LIMB = PREC == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const long long N = L.N;
  const double ex = e[q], ey = e[N + q], ez = e[2 * N + q];
  if (L.pinned && L.pinned[q]) {
    P.ep[q] = ex; P.ep[N + q] = ey; P.ep[2 * N + q] = ez;
    P.k1[q] = 0.0; P.k1[N + q] = 0.0; P.k1[2 * N + q] = 0.0;
    F.eps[q] = F.es[q]; F.eps[N + q] = F.es[N + q]; F.eps[2 * N + q] = F.es[2 * N + q];
    return;
  }
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double f[3], x, y, z;
  if (INTEG == MGX_INTEGRATOR_HEUN) {
    if (PREC == MGX_PRECISION_FP64_FIXED_GATHER) {
      double bx, by, bz;
      fx_field64<NOISE, PREC>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, bx, by, bz);
      llg_rhs(ex, ey, ez, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, f[0], f[1],
              f[2]);
    } else {
      fx_rhs<NOISE>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, f);
    }
    x = fma(P.dt, f[0], ex);
    y = fma(P.dt, f[1], ey);
    z = fma(P.dt, f[2], ez);
    const double r = rsqrt(x * x + y * y + z * z);
    x *= r; y *= r; z *= r;
  } else {
    double bx, by, bz;
    fx_field64<NOISE, PREC>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, bx, by, bz);
    double fx, fy, fz;
    llg_rhs(ex, ey, ez, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, fx, fy, fz);
    f[0] = ey * fz - ez * fy; f[1] = ez * fx - ex * fz; f[2] = ex * fy - ey * fx;
    x = ex; y = ey; z = ez;
    rotate(x, y, z, P.dt * f[0], P.dt * f[1], P.dt * f[2]);
  }
  P.ep[q] = x; P.ep[N + q] = y; P.ep[2 * N + q] = z;
  P.k1[q] = f[0]; P.k1[N + q] = f[1]; P.k1[2 * N + q] = f[2];
  F.eps[q] = fx_split<LIMB>(x); F.eps[N + q] = fx_split<LIMB>(y); F.eps[2 * N + q] = fx_split<LIMB>(z);
}

template <int NOISE, int INTEG, int PREC>
__global__ void __launch_bounds__(256, 4) k_correct_fx(const DevLattice L, const DevLLG P, const DevFX F,
                                                       double* __restrict__ e, const double* __restrict__ noise,
                                                       uint64_t step) {
  constexpr int LIMB = PREC == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  if (L.pinned && L.pinned[q]) return;                 // e and its split stay as they are
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
      fx_field64<NOISE, PREC>(L, P, F, F.eps, noise, q, s, c0, c1, c2, step, bx, by, bz);
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
    fx_field64<NOISE, PREC>(L, P, F, F.eps, noise, q, s, c0, c1, c2, step, bx, by, bz);
    double fx, fy, fz;
    llg_rhs(px, py, pz, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, fx, fy, fz);
    const double wx = py * fz - pz * fy, wy = pz * fx - px * fz, wz = px * fy - py * fx;
    rotate(x, y, z, P.half_dt * (k1x + wx), P.half_dt * (k1y + wy), P.half_dt * (k1z + wz));
  }
  const double r = rsqrt(x * x + y * y + z * z);
  x *= r; y *= r; z *= r;
  e[q] = x; e[N + q] = y; e[2 * N + q] = z;
  F.es[q] = fx_split<LIMB>(x); F.es[N + q] = fx_split<LIMB>(y); F.es[2 * N + q] = fx_split<LIMB>(z);
}

template <int NOISE, int INTEG, int PREC>
static void launch_fx(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st) {
  const DevLattice& L = pl->model->d;
  DevFX F = pl->fx;
  F.B[0] = split_host(L.B0);
  F.B[1] = split_host(L.B1);
  F.B[2] = split_host(L.B2);
  const int tpb = site_block_size(L.N);
  const unsigned grid = (unsigned)((L.N + tpb - 1) / tpb);
  if (stages & 1) k_predict_fx<NOISE, INTEG, PREC><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step);
  if (stages & 2) k_correct_fx<NOISE, INTEG, PREC><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step);
}

template <int NOISE, int PREC>
static void fx_integ(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st) {
  if (pl->p.integrator == MGX_INTEGRATOR_DEPONDT)
    launch_fx<NOISE, MGX_INTEGRATOR_DEPONDT, PREC>(pl, e, noise, step, stages, st);
  else
    launch_fx<NOISE, MGX_INTEGRATOR_HEUN, PREC>(pl, e, noise, step, stages, st);
}

template <int PREC>
static void fx_noise(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st) {
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  switch (mode) {
    case MGX_NOISE_HOST: fx_integ<MGX_NOISE_HOST, PREC>(pl, e, noise, step, stages, st); break;
    case MGX_NOISE_PHILOX: fx_integ<MGX_NOISE_PHILOX, PREC>(pl, e, noise, step, stages, st); break;
    default: fx_integ<MGX_NOISE_NONE, PREC>(pl, e, noise, step, stages, st); break;
  }
}

void enqueue_fx_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages) {
  if (pl->precision == MGX_PRECISION_FP64_FIXED_GATHER)
    fx_noise<MGX_PRECISION_FP64_FIXED_GATHER>(pl, e, noise, step, stages, st);
  else
    fx_noise<MGX_PRECISION_INT48_GATHER>(pl, e, noise, step, stages, st);
}

void enqueue_fx_split(const LLGPlan* pl, const double* e, cudaStream_t st) {
  const long long n = 3 * pl->model->d.N;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (pl->precision == MGX_PRECISION_FP64_FIXED_GATHER)
    k_fx_split<MGX_PRECISION_FP64_FIXED_GATHER><<<grid, 256, 0, st>>>(e, pl->fx.es, n);
  else
    k_fx_split<MGX_PRECISION_INT48_GATHER><<<grid, 256, 0, st>>>(e, pl->fx.es, n);
}

// balanced (hi, lo) int32 halves of round(v 2^(2 limb - sigma)), |v| <= 2^sigma
static int2 fx_host(double v, int sigma, int limb) {
  const long long w = std::llround(std::ldexp(v, 2 * limb - sigma));
  const long long hi = (w + (1LL << (limb - 1))) >> limb;
  return make_int2((int)hi, (int)(w - (hi << limb)));
}

mgx_status fx_build(const Model* m, int limb, bool field_scaled, int ncopies, DevFX* fx, void** block) {
  const DevLattice& d = m->d;
  if (d.layout != 0) return set_error(MGX_ERR_UNSUPPORTED, "the integer gather needs a lattice stencil model");
  if (d.N >= (1LL << 31)) return set_error(MGX_ERR_UNSUPPORTED, "the integer gather indexes at most 2^31 - 1 sites");
  if (d.A_site || d.mu_site) return set_error(MGX_ERR_UNSUPPORTED, "the integer gather needs per-sublattice A and mu");
  const int ns = d.ns, nb = m->nbond, W = d.width;
  const long long N = d.N;
  std::vector<int> off(ns + 1);
  std::vector<double> J((size_t)std::max(nb, 1) * W), A(9 * ns), inv(ns);
  std::vector<int4> geo((size_t)std::max(nb, 1));
  MGX_CUDA_TRY(cudaMemcpy(off.data(), d.bond_off, sizeof(int) * (ns + 1), cudaMemcpyDeviceToHost));
  if (nb > 0) {
    MGX_CUDA_TRY(cudaMemcpy(J.data(), d.bond_J, sizeof(double) * nb * W, cudaMemcpyDeviceToHost));
    MGX_CUDA_TRY(cudaMemcpy(geo.data(), d.bond_geo, sizeof(int4) * nb, cudaMemcpyDeviceToHost));
  }
  MGX_CUDA_TRY(cudaMemcpy(A.data(), d.A_sub, sizeof(double) * 9 * ns, cudaMemcpyDeviceToHost));
  MGX_CUDA_TRY(cudaMemcpy(inv.data(), d.inv_mu_sub, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  // 3x3 tensors of the receiving sublattice
  std::vector<double> M((size_t)std::max(nb, 1) * 9, 0.0), nA(9 * ns, 0.0);
  for (int s = 0; s < ns; ++s)
    for (int b = off[s]; b < off[s + 1]; ++b) {
      const double* t = J.data() + (size_t)b * W;
      double T[9];
      if (W == 1) {
        for (int k = 0; k < 9; ++k) T[k] = (k % 4 == 0) ? t[0] : 0.0;
      } else if (W == 4) {   // J I + antisymmetric part with (J^A e) = e x D
        T[0] = t[0]; T[1] = t[3]; T[2] = -t[2];
        T[3] = -t[3]; T[4] = t[0]; T[5] = t[1];
        T[6] = t[2]; T[7] = -t[1]; T[8] = t[0];
      } else {
        for (int k = 0; k < 9; ++k) T[k] = t[k];
      }
      const double f = field_scaled ? 2.0 * inv[s] : 1.0;
      for (int k = 0; k < 9; ++k) M[(size_t)b * 9 + k] = f * T[k];
    }
  bool hasA = false;
  if (field_scaled)
    for (int s = 0; s < ns; ++s)
      for (int k = 0; k < 9; ++k) {
        nA[9 * s + k] = -2.0 * inv[s] * A[9 * s + k];
        hasA |= A[9 * s + k] != 0.0;
      }
  // per-sublattice scale 2^sigma.  48-bit form: 2^sigma >= every magnitude (every half fits 25 bits;
  // every product is below 2^48, so the accumulators hold 2^14 terms per component).  56-bit form:
  // 2^sigma >= the sum of all magnitudes of the sublattice, so that |sum J_hi e_hi| <= 2^56 sum |J|
  // / 2^sigma <= 2^62 whatever the number of couplings: no int64 accumulator can overflow.
  std::vector<int> sigma(ns, 0);
  for (int s = 0; s < MGX_MAX_SUBLATTICES; ++s) fx->scale[s] = 0.0;
  for (int s = 0; s < ns; ++s) {
    double mx = 0.0, sum = 0.0;
    for (int b = off[s]; b < off[s + 1]; ++b)
      for (int k = 0; k < 9; ++k) {
        mx = std::max(mx, std::fabs(M[(size_t)b * 9 + k]));
        sum += std::fabs(M[(size_t)b * 9 + k]);
      }
    for (int k = 0; k < 9; ++k) {
      mx = std::max(mx, std::fabs(nA[9 * s + k]));
      sum += std::fabs(nA[9 * s + k]);
    }
    const double bound = limb == 28 ? sum : mx;
    int e = 0;
    if (bound > 0.0) std::frexp(bound, &e);      // bound < 2^e
    if (e < -50 || e > 900)
      return set_error(MGX_ERR_UNSUPPORTED, "couplings of sublattice %d (scale 2^%d) are outside the range of the "
                       "fixed-point gather", s, e);
    sigma[s] = e;
    fx->scale[s] = std::ldexp(1.0, e - 2 * limb);
  }
  std::vector<int2> Jq((size_t)std::max(nb, 1) * 10, make_int2(0, 0)), Aq((size_t)ns * 10, make_int2(0, 0));
  for (int s = 0; s < ns; ++s) {
    for (int b = off[s]; b < off[s + 1]; ++b)
      for (int k = 0; k < 9; ++k) Jq[(size_t)b * 10 + k] = fx_host(M[(size_t)b * 9 + k], sigma[s], limb);
    for (int k = 0; k < 9; ++k) Aq[(size_t)s * 10 + k] = fx_host(nA[9 * s + k], sigma[s], limb);
  }
  // interior fast path: signed offsets, linear neighbour offset and reach per receiving sublattice
  std::vector<int2> lin((size_t)std::max(nb, 1), make_int2(0, 0));
  const int Ls[3] = {d.L0, d.L1, d.L2}, pbc[3] = {d.pbc0, d.pbc1, d.pbc2};
  for (int s = 0; s < MGX_MAX_SUBLATTICES; ++s) fx->reach[s] = make_int4(0, 0, 0, 0);
  for (int s = 0; s < ns; ++s)
    for (int b = off[s]; b < off[s + 1]; ++b) {
      int R[3] = {geo[b].y, geo[b].z, geo[b].w};
      for (int a = 0; a < 3; ++a)
        if (pbc[a] && R[a] > Ls[a] / 2) R[a] -= Ls[a];
      lin[b] = make_int2((geo[b].x - s) * d.ncell + (R[0] * d.L1 + R[1]) * d.L2 + R[2], R[2]);
      int4& r = fx->reach[s];
      r.x = std::max(r.x, std::abs(R[0]));
      r.y = std::max(r.y, std::abs(R[1]));
      r.z = std::max(r.z, std::abs(R[2]));
    }
  const size_t nJ = sizeof(int2) * Jq.size(), nA2 = sizeof(int2) * Aq.size(), nL = sizeof(int2) * lin.size();
  const size_t o_A = (nJ + 15) / 16 * 16, o_L = (o_A + nA2 + 15) / 16 * 16, o_es = (o_L + nL + 15) / 16 * 16;
  const size_t n_split = sizeof(int2) * 3 * (size_t)N;
  MGX_CUDA_TRY(cudaMalloc(block, o_es + (size_t)ncopies * n_split));
  char* base = (char*)*block;
  MGX_CUDA_TRY(cudaMemcpy(base, Jq.data(), nJ, cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(base + o_A, Aq.data(), nA2, cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(base + o_L, lin.data(), nL, cudaMemcpyHostToDevice));
  fx->J = (const int4*)base;
  fx->A = hasA ? (const int4*)(base + o_A) : nullptr;
  fx->lin = (const int2*)(base + o_L);
  fx->es = (int2*)(base + o_es);
  fx->eps = ncopies > 1 ? (int2*)(base + o_es + n_split) : nullptr;
  return MGX_OK;
}

mgx_status build_fx_tables(LLGPlan* pl) {
  if (pl->p.alpha_site || pl->p.sigma_site)
    return set_error(MGX_ERR_UNSUPPORTED, "the integer gather needs uniform damping");
  const int limb = pl->precision == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24;
  const mgx_status st = fx_build(pl->model, limb, true, 2, &pl->fx, &pl->fx_block);
  if (st != MGX_OK) return st;
  const int ns = pl->model->d.ns;
  std::vector<double> ap(2 * ns);
  MGX_CUDA_TRY(cudaMemcpy(ap.data(), pl->p.alpha_sub, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  MGX_CUDA_TRY(cudaMemcpy(ap.data() + ns, pl->p.pre_sub, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  for (int s = 0; s < ns; ++s) {
    pl->fx.alpha[s] = split_host(ap[s]);
    pl->fx.pre[s] = split_host(ap[ns + s]);
  }
  return MGX_OK;
}

void enqueue_fx_split_n(const double* x, int2* xs, long long n, int limb, cudaStream_t st) {
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (limb == 28)
    k_fx_split<MGX_PRECISION_FP64_FIXED_GATHER><<<grid, 256, 0, st>>>(x, xs, n);
  else
    k_fx_split<MGX_PRECISION_INT48_GATHER><<<grid, 256, 0, st>>>(x, xs, n);
}

}  // namespace mgx
