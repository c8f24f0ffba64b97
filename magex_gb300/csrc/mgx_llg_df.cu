// Heun / Depondt step with the exchange gather in compensated FP32 pairs (MGX_PRECISION_DF32_GATHER).
//
// GB300 runs FP64 FMAs at 2 per clock per SM and FP32 FMAs at 128; the FP64 step is bound by the
// 9 z FP64 multiply-adds of the gather (234 of ~290 FP64 instructions per site and stage for the
// 26-neighbour bcc workload).  This form evaluates h = sum_j J_ij e_j with error-free transformations
// on FP32 pairs:
//   * couplings (pre-scaled by 2 / (mu mu_B)) and neighbour spins are stored as (hi, lo) floats with
//     hi + lo equal to the double to ~2^-48;
//   * each product J e is split into its rounded value p = J_hi e_hi and the exact error
//     fma(J_hi, e_hi, -p) (Dekker / Ogita-Rump-Oishi TwoProduct with an FMA), plus the cross terms
//     J_hi e_lo + J_lo e_hi;
//   * p is added to the high accumulator with TwoSum (Knuth), the rounding error, the product error
//     and the cross terms go to the low accumulator, and the pair is renormalised with TwoSum after
//     every coupling so the low part never grows.
// For the Heun integrator the rest of the field (Zeeman, on-site, thermal) and the right-hand side
// f = pre [e x B + alpha e x (e x B)] stay on pairs too; the integration e + dt f, the renormalisation
// and the (hi, lo) splits of the new spins are FP64.  The Depondt form keeps an FP64 tail.  The
// result carries about 44 significant bits in B and f: for the bcc workload a relative error near
// 1e-13 in the field, far below the 1e-12-per-step parity tolerance against magex.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "mgx_dfp.cuh"
#include "mgx_step.cuh"

namespace mgx {

// (S, T) += J * v for J = (J.x + J.y), v = (v.x + v.y)
__device__ __forceinline__ void df_mac(float2 J, float2 v, float& S, float& T) {
  const float p = __fmul_rn(J.x, v.x);
  const float pe = __fmaf_rn(J.x, v.x, -p);
  const float s = __fadd_rn(S, p);
  const float bp = __fsub_rn(s, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bp)), __fsub_rn(p, bp));
  S = s;
  T = __fmaf_rn(J.x, v.y, __fmaf_rn(J.y, v.x, __fadd_rn(T, __fadd_rn(pe, err))));
}

// renormalise so that |T| <= ulp(S) / 2 (TwoSum, valid for any magnitudes)
__device__ __forceinline__ void df_renorm(float& S, float& T) {
  const float s = __fadd_rn(S, T);
  const float bp = __fsub_rn(s, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bp)), __fsub_rn(T, bp));
  S = s;
  T = err;
}

// (S, T) += M_b x_j for the 3x3 coupling b (10 (hi, lo) pairs, 80 B) and neighbour split spin x_j
__device__ __forceinline__ void df_bond(const float4* __restrict__ T, float2 ax, float2 ay, float2 az, float& Sx,
                                        float& Tx, float& Sy, float& Ty, float& Sz, float& Tz) {
  const float4 t01 = __ldg(T), t23 = __ldg(T + 1), t45 = __ldg(T + 2), t67 = __ldg(T + 3), t89 = __ldg(T + 4);
  df_mac(make_float2(t01.x, t01.y), ax, Sx, Tx); df_mac(make_float2(t01.z, t01.w), ay, Sx, Tx);
  df_mac(make_float2(t23.x, t23.y), az, Sx, Tx);
  df_mac(make_float2(t23.z, t23.w), ax, Sy, Ty); df_mac(make_float2(t45.x, t45.y), ay, Sy, Ty);
  df_mac(make_float2(t45.z, t45.w), az, Sy, Ty);
  df_mac(make_float2(t67.x, t67.y), ax, Sz, Tz); df_mac(make_float2(t67.z, t67.w), ay, Sz, Tz);
  df_mac(make_float2(t89.x, t89.y), az, Sz, Tz);
  df_renorm(Sx, Tx);
  df_renorm(Sy, Ty);
  df_renorm(Sz, Tz);
}

// h' = sum_j (2 J_ij / (mu_i mu_B)) x_j at lattice index q = site (s, c0, c1, c2) from the split field xs.
// Cells whose whole stencil stays inside the supercell along axes 0 and 1 take the fast path: the
// neighbour index is q plus a per-coupling constant, corrected only for the periodic seam of axis 2.
__device__ __forceinline__ void df_gather_pairs(const DevLattice& L, const DevDF& F, const float2* __restrict__ xs,
                                                long long q, int s, int c0, int c1, int c2, float& Sx, float& Tx,
                                                float& Sy, float& Ty, float& Sz, float& Tz) {
  const long long N = L.N;
  const int b0 = __ldg(L.bond_off + s), b1 = __ldg(L.bond_off + s + 1);
  const int4 r = F.reach[s];
  const bool inner01 = c0 >= r.x && c0 < L.L0 - r.x && c1 >= r.y && c1 < L.L1 - r.y;
  const bool inner2 = L.pbc2 ? r.z < L.L2 : (c2 >= r.z && c2 < L.L2 - r.z);
  if (inner01 && inner2) {
    for (int b = b0; b < b1; ++b) {
      const int2 li = __ldg(F.lin + b);
      const int n2 = c2 + li.y;
      const long long j = q + li.x + (n2 < 0 ? L.L2 : 0) - (n2 >= L.L2 ? L.L2 : 0);
      df_bond(F.J + (long long)b * 5, __ldg(xs + j), __ldg(xs + N + j), __ldg(xs + 2 * N + j), Sx, Tx, Sy, Ty, Sz,
              Tz);
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
      df_bond(F.J + (long long)b * 5, __ldg(xs + j), __ldg(xs + N + j), __ldg(xs + 2 * N + j), Sx, Tx, Sy, Ty, Sz,
              Tz);
    }
  }
}

__device__ __forceinline__ void df_gather(const DevLattice& L, const DevDF& F, const float2* __restrict__ xs,
                                          long long q, int s, int c0, int c1, int c2, double& hx, double& hy,
                                          double& hz) {
  float Sx = 0.f, Tx = 0.f, Sy = 0.f, Ty = 0.f, Sz = 0.f, Tz = 0.f;
  df_gather_pairs(L, F, xs, q, s, c0, c1, c2, Sx, Tx, Sy, Ty, Sz, Tz);
  hx = (double)Sx + (double)Tx;
  hy = (double)Sy + (double)Ty;
  hz = (double)Sz + (double)Tz;
}

// B_eff = h' - 2 A e / (mu mu_B) + B_ext (T), with h' already scaled by 2 / (mu mu_B)
__device__ __forceinline__ void df_field(const DevLattice& L, const DevDF& F, const float2* __restrict__ xs,
                                         long long q, int s, int c0, int c1, int c2, double ex, double ey, double ez,
                                         double& bx, double& by, double& bz) {
  double hx, hy, hz;
  df_gather(L, F, xs, q, s, c0, c1, c2, hx, hy, hz);
  bx = hx + L.B0;
  by = hy + L.B1;
  bz = hz + L.B2;
  if (F.hasA) {
    const double* a = F.nA2 + 9 * s;
    if (F.diagA) {
      bx = fma(__ldg(a + 0), ex, bx);
      by = fma(__ldg(a + 4), ey, by);
      bz = fma(__ldg(a + 8), ez, bz);
    } else {
      bx = fma(__ldg(a + 0), ex, fma(__ldg(a + 1), ey, fma(__ldg(a + 2), ez, bx)));
      by = fma(__ldg(a + 3), ex, fma(__ldg(a + 4), ey, fma(__ldg(a + 5), ez, by)));
      bz = fma(__ldg(a + 6), ex, fma(__ldg(a + 7), ey, fma(__ldg(a + 8), ez, bz)));
    }
  }
}

// B = h' + B_ext - 2 A e / (mu mu_B) + sigma g (T) on pairs; x: (hi, lo) of the spin at the site
template <int NOISE>
__device__ __forceinline__ void dfp_field(const DevLattice& L, const DevLLG& P, const DevDF& F,
                                          const float2* __restrict__ xs, const double* __restrict__ noise,
                                          long long q, int s, int c0, int c1, int c2, uint64_t step, dfp x[3],
                                          dfp B[3]) {
  float Sx = 0.f, Tx = 0.f, Sy = 0.f, Ty = 0.f, Sz = 0.f, Tz = 0.f;
  df_gather_pairs(L, F, xs, q, s, c0, c1, c2, Sx, Tx, Sy, Ty, Sz, Tz);
  B[0] = dfp_add({Sx, Tx}, dfp_of(F.B[0]));
  B[1] = dfp_add({Sy, Ty}, dfp_of(F.B[1]));
  B[2] = dfp_add({Sz, Tz}, dfp_of(F.B[2]));
  if (F.hasA) {
    const float2* a = F.nA2f + 9 * s;
    if (F.diagA) {
#pragma unroll
      for (int c = 0; c < 3; ++c) B[c] = dfp_add(B[c], dfp_mul(dfp_of(__ldg(a + 4 * c)), x[c]));
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < 3; ++k) B[c] = dfp_add(B[c], dfp_mul(dfp_of(__ldg(a + 3 * c + k)), x[k]));
    }
  }
  if (NOISE != MGX_NOISE_NONE) {
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
}

__global__ void __launch_bounds__(256) k_split(const double* __restrict__ x, float2* __restrict__ xs, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xs[i] = split_double(x[i]);
}

template <int NOISE, int INTEG>
__global__ void __launch_bounds__(256) k_predict_df(const DevLattice L, const DevLLG P, const DevDF F,
                                                    const double* __restrict__ e, const double* __restrict__ noise,
                                                    uint64_t step_arg) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const uint64_t step = P.step_base ? *P.step_base + step_arg : step_arg;
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
  double fx, fy, fz;
  if (INTEG == MGX_INTEGRATOR_HEUN) {
    dfp xe[3] = {dfp_of(F.es[q]), dfp_of(F.es[N + q]), dfp_of(F.es[2 * N + q])}, B[3], f[3];
    dfp_field<NOISE>(L, P, F, F.es, noise, q, s, c0, c1, c2, step, xe, B);
    dfp_rhs(xe, B, dfp_of(F.alpha[s]), dfp_of(F.pre[s]), P.precession != 0, f);
    fx = dfp_double(f[0]);
    fy = dfp_double(f[1]);
    fz = dfp_double(f[2]);
  } else {
    double bx, by, bz;
    df_field(L, F, F.es, q, s, c0, c1, c2, ex, ey, ez, bx, by, bz);
    add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
    llg_rhs(ex, ey, ez, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, fx, fy, fz);
  }
  double x, y, z;
  if (INTEG == MGX_INTEGRATOR_DEPONDT) {
    const double wx = ey * fz - ez * fy, wy = ez * fx - ex * fz, wz = ex * fy - ey * fx;
    x = ex; y = ey; z = ez;
    rotate(x, y, z, P.dt * wx, P.dt * wy, P.dt * wz);
    fx = wx; fy = wy; fz = wz;
  } else {
    x = fma(P.dt, fx, ex);
    y = fma(P.dt, fy, ey);
    z = fma(P.dt, fz, ez);
    const double r = rsqrt(x * x + y * y + z * z);
    x *= r; y *= r; z *= r;
  }
  P.ep[q] = x; P.ep[N + q] = y; P.ep[2 * N + q] = z;
  P.k1[q] = fx; P.k1[N + q] = fy; P.k1[2 * N + q] = fz;
  F.eps[q] = split_double(x); F.eps[N + q] = split_double(y); F.eps[2 * N + q] = split_double(z);
}

template <int NOISE, int INTEG>
__global__ void __launch_bounds__(256) k_correct_df(const DevLattice L, const DevLLG P, const DevDF F,
                                                    double* __restrict__ e, const double* __restrict__ noise,
                                                    uint64_t step_arg) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const uint64_t step = P.step_base ? *P.step_base + step_arg : step_arg;
  if (L.pinned && L.pinned[q]) return;                 // e and its split stay as they are
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double px = 0.0, py = 0.0, pz = 0.0;
  double fx, fy, fz;
  if (INTEG == MGX_INTEGRATOR_HEUN) {
    dfp xe[3] = {dfp_of(F.eps[q]), dfp_of(F.eps[N + q]), dfp_of(F.eps[2 * N + q])}, B[3], f[3];
    dfp_field<NOISE>(L, P, F, F.eps, noise, q, s, c0, c1, c2, step, xe, B);
    dfp_rhs(xe, B, dfp_of(F.alpha[s]), dfp_of(F.pre[s]), P.precession != 0, f);
    fx = dfp_double(f[0]);
    fy = dfp_double(f[1]);
    fz = dfp_double(f[2]);
  } else {
    px = P.ep[q]; py = P.ep[N + q]; pz = P.ep[2 * N + q];
    double bx, by, bz;
    df_field(L, F, F.eps, q, s, c0, c1, c2, px, py, pz, bx, by, bz);
    add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
    llg_rhs(px, py, pz, bx, by, bz, __ldg(P.alpha_sub + s), __ldg(P.pre_sub + s), P.precession != 0, fx, fy, fz);
  }
  const double k1x = P.k1[q], k1y = P.k1[N + q], k1z = P.k1[2 * N + q];
  double x = e[q], y = e[N + q], z = e[2 * N + q];
  if (INTEG == MGX_INTEGRATOR_DEPONDT) {
    const double wx = py * fz - pz * fy, wy = pz * fx - px * fz, wz = px * fy - py * fx;
    rotate(x, y, z, P.half_dt * (k1x + wx), P.half_dt * (k1y + wy), P.half_dt * (k1z + wz));
  } else {
    x = fma(P.half_dt, k1x + fx, x);
    y = fma(P.half_dt, k1y + fy, y);
    z = fma(P.half_dt, k1z + fz, z);
  }
  const double r = rsqrt(x * x + y * y + z * z);
  x *= r; y *= r; z *= r;
  e[q] = x; e[N + q] = y; e[2 * N + q] = z;
  F.es[q] = split_double(x); F.es[N + q] = split_double(y); F.es[2 * N + q] = split_double(z);
}

template <int NOISE, int INTEG>
static void launch_df(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st) {
  const DevLattice& L = pl->model->d;
  DevDF F = pl->df;
  F.B[0] = split_host(L.B0);
  F.B[1] = split_host(L.B1);
  F.B[2] = split_host(L.B2);
  const int tpb = site_block_size(L.N);
  const unsigned grid = (unsigned)((L.N + tpb - 1) / tpb);
  if (stages & 1) k_predict_df<NOISE, INTEG><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step);
  if (stages & 2) k_correct_df<NOISE, INTEG><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step);
}

template <int NOISE>
static void df_integ(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st) {
  if (pl->p.integrator == MGX_INTEGRATOR_DEPONDT) launch_df<NOISE, MGX_INTEGRATOR_DEPONDT>(pl, e, noise, step, stages, st);
  else launch_df<NOISE, MGX_INTEGRATOR_HEUN>(pl, e, noise, step, stages, st);
}

void enqueue_df_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages) {
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  switch (mode) {
    case MGX_NOISE_HOST: df_integ<MGX_NOISE_HOST>(pl, e, noise, step, stages, st); break;
    case MGX_NOISE_PHILOX: df_integ<MGX_NOISE_PHILOX>(pl, e, noise, step, stages, st); break;
    default: df_integ<MGX_NOISE_NONE>(pl, e, noise, step, stages, st); break;
  }
}

void enqueue_df_split(const LLGPlan* pl, const double* e, cudaStream_t st) {
  const long long n = 3 * pl->model->d.N;
  k_split<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(e, pl->df.es, n);
}

mgx_status build_df_tables(LLGPlan* pl) {
  const Model* m = pl->model;
  const DevLattice& d = m->d;
  if (d.layout != 0) return set_error(MGX_ERR_UNSUPPORTED, "the compensated-FP32 gather needs a lattice stencil model");
  if (d.A_site || d.mu_site) return set_error(MGX_ERR_UNSUPPORTED, "the compensated-FP32 gather needs per-sublattice A and mu");
  if (pl->p.alpha_site || pl->p.sigma_site) return set_error(MGX_ERR_UNSUPPORTED, "the compensated-FP32 gather needs uniform damping");
  const int ns = d.ns, nb = m->nbond, W = d.width;
  const long long N = d.N;
  std::vector<int> off(ns + 1);
  std::vector<double> J((size_t)std::max(nb, 1) * W), A(9 * ns), inv(ns);
  MGX_CUDA_TRY(cudaMemcpy(off.data(), d.bond_off, sizeof(int) * (ns + 1), cudaMemcpyDeviceToHost));
  if (nb > 0) MGX_CUDA_TRY(cudaMemcpy(J.data(), d.bond_J, sizeof(double) * nb * W, cudaMemcpyDeviceToHost));
  MGX_CUDA_TRY(cudaMemcpy(A.data(), d.A_sub, sizeof(double) * 9 * ns, cudaMemcpyDeviceToHost));
  MGX_CUDA_TRY(cudaMemcpy(inv.data(), d.inv_mu_sub, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  std::vector<float2> Jf((size_t)std::max(nb, 1) * 10, make_float2(0.f, 0.f));
  std::vector<int4> geo((size_t)std::max(nb, 1));
  if (nb > 0) MGX_CUDA_TRY(cudaMemcpy(geo.data(), d.bond_geo, sizeof(int4) * nb, cudaMemcpyDeviceToHost));
  // signed cell offsets (periodic axes store R mod L), the linear offset of an interior neighbour and
  // the reach of every receiving sublattice's stencil
  std::vector<int2> lin((size_t)std::max(nb, 1), make_int2(0, 0));
  const int Ls[3] = {d.L0, d.L1, d.L2}, pbc[3] = {d.pbc0, d.pbc1, d.pbc2};
  for (int s = 0; s < MGX_MAX_SUBLATTICES; ++s) pl->df.reach[s] = make_int4(0, 0, 0, 0);
  for (int s = 0; s < ns; ++s)
    for (int b = off[s]; b < off[s + 1]; ++b) {
      int R[3] = {geo[b].y, geo[b].z, geo[b].w};
      for (int a = 0; a < 3; ++a)
        if (pbc[a] && R[a] > Ls[a] / 2) R[a] -= Ls[a];
      lin[b] = make_int2((geo[b].x - s) * d.ncell + (R[0] * d.L1 + R[1]) * d.L2 + R[2], R[2]);
      int4& r = pl->df.reach[s];
      r.x = std::max(r.x, std::abs(R[0]));
      r.y = std::max(r.y, std::abs(R[1]));
      r.z = std::max(r.z, std::abs(R[2]));
    }
  for (int s = 0; s < ns; ++s)
    for (int b = off[s]; b < off[s + 1]; ++b) {
      double M[9];
      const double* t = J.data() + (size_t)b * W;
      if (W == 1) {
        for (int k = 0; k < 9; ++k) M[k] = (k % 4 == 0) ? t[0] : 0.0;
      } else if (W == 4) {   // J I + antisymmetric part with (J^A e) = e x D
        M[0] = t[0]; M[1] = t[3]; M[2] = -t[2];
        M[3] = -t[3]; M[4] = t[0]; M[5] = t[1];
        M[6] = t[2]; M[7] = -t[1]; M[8] = t[0];
      } else {
        for (int k = 0; k < 9; ++k) M[k] = t[k];
      }
      for (int k = 0; k < 9; ++k) {
        const double v = 2.0 * inv[s] * M[k];
        const float hi = (float)v;
        Jf[(size_t)b * 10 + k] = make_float2(hi, (float)(v - (double)hi));
      }
    }
  std::vector<double> nA2(9 * ns);
  bool hasA = false, diag = true;
  for (int s = 0; s < ns; ++s)
    for (int k = 0; k < 9; ++k) {
      nA2[9 * s + k] = -2.0 * inv[s] * A[9 * s + k];
      hasA |= A[9 * s + k] != 0.0;
      if (k % 4 != 0) diag &= A[9 * s + k] == 0.0;
    }
  std::vector<float2> nA2f(nA2.size());
  for (size_t k = 0; k < nA2.size(); ++k) nA2f[k] = split_host(nA2[k]);
  std::vector<double> ap(2 * ns);
  MGX_CUDA_TRY(cudaMemcpy(ap.data(), pl->p.alpha_sub, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  MGX_CUDA_TRY(cudaMemcpy(ap.data() + ns, pl->p.pre_sub, sizeof(double) * ns, cudaMemcpyDeviceToHost));
  for (int s = 0; s < ns; ++s) {
    pl->df.alpha[s] = split_host(ap[s]);
    pl->df.pre[s] = split_host(ap[ns + s]);
  }
  const size_t nJ = sizeof(float2) * Jf.size(), nA = sizeof(double) * nA2.size(), nL = sizeof(int2) * lin.size();
  const size_t nAf = sizeof(float2) * nA2f.size();
  const size_t o_A = (nJ + 15) / 16 * 16, o_L = (o_A + nA + 15) / 16 * 16, o_Af = (o_L + nL + 15) / 16 * 16;
  const size_t o_es = (o_Af + nAf + 15) / 16 * 16;
  const size_t n_split = sizeof(float2) * 3 * (size_t)N;
  const size_t total = o_es + 2 * n_split;
  MGX_CUDA_TRY(cudaMalloc(&pl->df_block, total));
  char* base = (char*)pl->df_block;
  MGX_CUDA_TRY(cudaMemcpy(base, Jf.data(), nJ, cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(base + o_A, nA2.data(), nA, cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(base + o_L, lin.data(), nL, cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(base + o_Af, nA2f.data(), nAf, cudaMemcpyHostToDevice));
  pl->df.nA2f = (const float2*)(base + o_Af);
  pl->df.J = (const float4*)base;
  pl->df.lin = (const int2*)(base + o_L);
  pl->df.nA2 = (const double*)(base + o_A);
  pl->df.hasA = hasA ? 1 : 0;
  pl->df.diagA = diag ? 1 : 0;
  pl->df.es = (float2*)(base + o_es);
  pl->df.eps = (float2*)(base + o_es + n_split);
  return MGX_OK;
}

}  // namespace mgx
