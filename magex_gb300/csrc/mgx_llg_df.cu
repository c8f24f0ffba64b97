// Heun / Depondt step with the exchange gather in compensated FP32 pairs (MGX_PRECISION_DF32_GATHER).
//
// GB300 runs FP64 FMAs at 2 per clock per SM and FP32 FMAs at 128; the FP64 step is bound by the
// 9 z FP64 multiply-adds of the gather (234 of ~290 FP64 instructions per site and stage for the
// 26-neighbour bcc workload).  This form keeps the spins, the on-site and Zeeman terms, the LLG
// right-hand side, the integration and the normalisation in FP64, and evaluates only
// h = sum_j J_ij e_j with error-free transformations on FP32 pairs:
//   * couplings (pre-scaled by 2 / (mu mu_B)) and neighbour spins are stored as (hi, lo) floats with
//     hi + lo equal to the double to ~2^-48;
//   * each product J e is split into its rounded value p = J_hi e_hi and the exact error
//     fma(J_hi, e_hi, -p) (Dekker / Ogita-Rump-Oishi TwoProduct with an FMA), plus the cross terms
//     J_hi e_lo + J_lo e_hi;
//   * p is added to the high accumulator with TwoSum (Knuth), the rounding error, the product error
//     and the cross terms go to the low accumulator, and the pair is renormalised with TwoSum after
//     every coupling so the low part never grows.
// The field then carries about 44 significant bits instead of 53: for the bcc workload a relative
// error near 1e-13 in B_eff, far below the 1e-12-per-step parity tolerance against magex.
#include <cmath>
#include <vector>

#include "mgx_step.cuh"

namespace mgx {

__device__ __forceinline__ float2 split_double(double x) {
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - (double)hi);
  return make_float2(hi, lo);
}

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

// h' = sum_j (2 J_ij / (mu_i mu_B)) x_j at site (s, c0, c1, c2) from the split field xs.
__device__ __forceinline__ void df_gather(const DevLattice& L, const DevDF& F, const float2* __restrict__ xs, int s,
                                          int c0, int c1, int c2, double& hx, double& hy, double& hz) {
  float Sx = 0.f, Tx = 0.f, Sy = 0.f, Ty = 0.f, Sz = 0.f, Tz = 0.f;
  const long long N = L.N;
  const int b0 = __ldg(L.bond_off + s), b1 = __ldg(L.bond_off + s + 1);
  for (int b = b0; b < b1; ++b) {
    const int4 g = __ldg(L.bond_geo + b);
    int n0 = c0 + g.y, n1 = c1 + g.z, n2 = c2 + g.w;
    bool ok = true;
    if (L.pbc0) { n0 -= (n0 >= L.L0) ? L.L0 : 0; } else { ok &= (unsigned)n0 < (unsigned)L.L0; }
    if (L.pbc1) { n1 -= (n1 >= L.L1) ? L.L1 : 0; } else { ok &= (unsigned)n1 < (unsigned)L.L1; }
    if (L.pbc2) { n2 -= (n2 >= L.L2) ? L.L2 : 0; } else { ok &= (unsigned)n2 < (unsigned)L.L2; }
    if (!ok) continue;
    const long long j = (long long)g.x * L.ncell + ((long long)n0 * L.L1 + n1) * L.L2 + n2;
    const float2 ax = __ldg(xs + j), ay = __ldg(xs + N + j), az = __ldg(xs + 2 * N + j);
    const float2* T = F.J + (long long)b * 9;
    df_mac(__ldg(T + 0), ax, Sx, Tx); df_mac(__ldg(T + 1), ay, Sx, Tx); df_mac(__ldg(T + 2), az, Sx, Tx);
    df_mac(__ldg(T + 3), ax, Sy, Ty); df_mac(__ldg(T + 4), ay, Sy, Ty); df_mac(__ldg(T + 5), az, Sy, Ty);
    df_mac(__ldg(T + 6), ax, Sz, Tz); df_mac(__ldg(T + 7), ay, Sz, Tz); df_mac(__ldg(T + 8), az, Sz, Tz);
    df_renorm(Sx, Tx);
    df_renorm(Sy, Ty);
    df_renorm(Sz, Tz);
  }
  hx = (double)Sx + (double)Tx;
  hy = (double)Sy + (double)Ty;
  hz = (double)Sz + (double)Tz;
}

// B_eff = h' - 2 A e / (mu mu_B) + B_ext (T), with h' already scaled by 2 / (mu mu_B)
__device__ __forceinline__ void df_field(const DevLattice& L, const DevDF& F, const float2* __restrict__ xs,
                                         int s, int c0, int c1, int c2, double ex, double ey, double ez,
                                         double& bx, double& by, double& bz) {
  double hx, hy, hz;
  df_gather(L, F, xs, s, c0, c1, c2, hx, hy, hz);
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

__global__ void __launch_bounds__(256) k_split(const double* __restrict__ x, float2* __restrict__ xs, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xs[i] = split_double(x[i]);
}

template <int NOISE, int INTEG>
__global__ void __launch_bounds__(256) k_predict_df(const DevLattice L, const DevLLG P, const DevDF F,
                                                    const double* __restrict__ e, const double* __restrict__ noise,
                                                    uint64_t step) {
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
  double bx, by, bz;
  df_field(L, F, F.es, s, c0, c1, c2, ex, ey, ez, bx, by, bz);
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
  const double a = __ldg(P.alpha_sub + s);
  const double pre = __ldg(P.pre_sub + s);
  double fx, fy, fz;
  llg_rhs(ex, ey, ez, bx, by, bz, a, pre, P.precession != 0, fx, fy, fz);
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
                                                    uint64_t step) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  if (L.pinned && L.pinned[q]) return;                 // e and its split stay as they are
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  const double px = P.ep[q], py = P.ep[N + q], pz = P.ep[2 * N + q];
  double bx, by, bz;
  df_field(L, F, F.eps, s, c0, c1, c2, px, py, pz, bx, by, bz);
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
  const double a = __ldg(P.alpha_sub + s);
  const double pre = __ldg(P.pre_sub + s);
  double fx, fy, fz;
  llg_rhs(px, py, pz, bx, by, bz, a, pre, P.precession != 0, fx, fy, fz);
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
  const int tpb = site_block_size(L.N);
  const unsigned grid = (unsigned)((L.N + tpb - 1) / tpb);
  if (stages & 1) k_predict_df<NOISE, INTEG><<<grid, tpb, 0, st>>>(L, pl->p, pl->df, e, noise, step);
  if (stages & 2) k_correct_df<NOISE, INTEG><<<grid, tpb, 0, st>>>(L, pl->p, pl->df, e, noise, step);
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
  std::vector<float2> Jf((size_t)std::max(nb, 1) * 9, make_float2(0.f, 0.f));
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
        Jf[(size_t)b * 9 + k] = make_float2(hi, (float)(v - (double)hi));
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
  const size_t nJ = sizeof(float2) * Jf.size(), nA = sizeof(double) * nA2.size();
  const size_t o_A = (nJ + 15) / 16 * 16, o_es = (o_A + nA + 15) / 16 * 16;
  const size_t n_split = sizeof(float2) * 3 * (size_t)N;
  const size_t total = o_es + 2 * n_split;
  MGX_CUDA_TRY(cudaMalloc(&pl->df_block, total));
  char* base = (char*)pl->df_block;
  MGX_CUDA_TRY(cudaMemcpy(base, Jf.data(), nJ, cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(base + o_A, nA2.data(), nA, cudaMemcpyHostToDevice));
  pl->df.J = (const float2*)base;
  pl->df.nA2 = (const double*)(base + o_A);
  pl->df.hasA = hasA ? 1 : 0;
  pl->df.diagA = diag ? 1 : 0;
  pl->df.es = (float2*)(base + o_es);
  pl->df.eps = (float2*)(base + o_es + n_split);
  return MGX_OK;
}

}  // namespace mgx
