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

#include "mgx_fx_step.cuh"

namespace mgx {

template <int PREC>
__global__ void __launch_bounds__(256) k_fx_split(const double* __restrict__ x, int2* __restrict__ xs, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xs[i] = fx_split<PREC == MGX_PRECISION_FP64_FIXED_GATHER ? 28 : 24>(x[i]);
}

// Sites begin + i (i < count) of sublattice blockIdx.y: the whole lattice is one row of N sites
// (gridDim.y = 1, begin = 0), a range of cells one row of `count` cells per sublattice.
// Philox noise of the 56-bit form in the five-block kernels (the plans of many couplings per site): the
// predictor stores its normal draws (DevFX::nz) and the corrector of the same step reads them back, 12 B
// per site each way instead of a second Philox block and Box-Muller per site.  bcc 128^3: 1.047 ->
// 1.029 ms per step; on the triangular film 2048^2 (FP64-bound, four blocks) it cost 6.8 %, so the
// four-block kernels draw the normals in both stages.
template <int NOISE, int PREC, int BLK>
constexpr bool kNoiseCache = NOISE == MGX_NOISE_PHILOX && PREC == MGX_PRECISION_FP64_FIXED_GATHER && BLK == 5;

// BLK: resident blocks per SM of the stage kernels.  5 (48 registers, ~100 B of spills per thread)
// for stencils of at least 16 couplings per site without the higher on-site terms (the plans whose
// conversions run on the hardware converters, DevFX::hw_convert), 4 (64 registers) otherwise.  Timed
// with CUDA events over 100 steps: bcc 128^3 (26 couplings) 1.046 ms per step at 5, 1.076 at 4,
// 1.124 at 6; the triangular film 2048^2 (6 couplings) 0.698 ms at 4, 0.704 at 5, and small films,
// whose plans are launch- and latency-bound, about 8 % slower at 5.
template <int NOISE, int INTEG, int PREC, bool HIGHER, int BLK>
__global__ void __launch_bounds__(256, BLK) k_predict_fx(const DevLattice L, const DevLLG P, const DevFX F,
                                                         const double* __restrict__ e, const double* __restrict__ noise,
                                                         uint64_t step, long long begin, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count)
    fx_predict_site<NOISE, INTEG, PREC, HIGHER, 2, kNoiseCache<NOISE, PREC, BLK>>(
        L, P, F, e, noise, (long long)blockIdx.y * L.ncell + begin + i, P.step_base ? *P.step_base + step : step);
}

// ROWS (the slabs of a step on host buffers): the new spins go to the magex-order rows `rows` only.
// A separate instantiation: the device step's corrector carries no branch for it (a run-time pointer
// cost 2.3 % of the bcc 128^3 step).
template <int NOISE, int INTEG, int PREC, bool HIGHER, int BLK, bool ROWS = false>
__global__ void __launch_bounds__(256, BLK) k_correct_fx(const DevLattice L, const DevLLG P, const DevFX F,
                                                         double* __restrict__ e, const double* __restrict__ noise,
                                                         uint64_t step, long long begin, long long count,
                                                         double* __restrict__ rows) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count)
    fx_correct_site<NOISE, INTEG, PREC, HIGHER, 2, kNoiseCache<NOISE, PREC, BLK>>(
        L, P, F, e, noise, (long long)blockIdx.y * L.ncell + begin + i, P.step_base ? *P.step_base + step : step,
        nullptr, nullptr, nullptr, ROWS ? rows : nullptr);
}

// Magex-order rows [begin, begin + count) of an (N, 3) array -> lattice layout (3, N) and its fixed-point
// split, in one pass (the input slabs of a step on host buffers)
template <int LIMB>
__global__ void __launch_bounds__(256) k_pack_split(const double* __restrict__ rows, double* __restrict__ lat,
                                                    int2* __restrict__ xs, int ns, int ncell, long long N,
                                                    long long begin, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const long long site = begin + i;
  const long long cell = site / ns;
  const int s = (int)(site - cell * ns);
  const long long q = (long long)s * ncell + cell;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double v = rows[3 * site + c];
    lat[c * N + q] = v;
    xs[c * N + q] = fx_split<LIMB>(v);
  }
}

template <int NOISE, int INTEG, int PREC, bool HIGHER, int BLK>
static void launch_stages(const LLGPlan* pl, const DevFX& F, double* e, const double* noise, uint64_t step,
                          int stages, cudaStream_t st, dim3 grid, int tpb, long long cb, long long count,
                          double* rows) {
  const DevLattice& L = pl->model->d;
  if (stages & 1)
    k_predict_fx<NOISE, INTEG, PREC, HIGHER, BLK><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step, cb, count);
  if ((stages & 2) && rows)
    k_correct_fx<NOISE, INTEG, PREC, HIGHER, BLK, true><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step, cb, count,
                                                                              rows);
  else if (stages & 2)
    k_correct_fx<NOISE, INTEG, PREC, HIGHER, BLK><<<grid, tpb, 0, st>>>(L, pl->p, F, e, noise, step, cb, count,
                                                                        nullptr);
}

template <int NOISE, int INTEG, int PREC>
static void launch_fx(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st,
                      long long cb, long long cn, double* rows) {
  const DevLattice& L = pl->model->d;
  DevFX F = pl->fx;
  F.B[0] = split_host(L.B0);
  F.B[1] = split_host(L.B1);
  F.B[2] = split_host(L.B2);
  const bool whole = cb == 0 && cn == L.ncell;
  // the slabs of a step on host buffers keep the conversions on the integer pipes: there the slab
  // kernels share the GPU with each other and with the packing (bcc 128^3: 1.343 ms per call against
  // 1.352 with the hardware converters; the same kernel, so the same values either way)
  if (!whole) F.hw_convert = 0;
  const long long count = whole ? L.N : cn;
  const int tpb = site_block_size(whole ? L.N : cn * L.ns);
  const dim3 grid((unsigned)((count + tpb - 1) / tpb), whole ? 1u : (unsigned)L.ns);
  // cubic / higher-uniaxial terms (56-bit form only): a separate instantiation, so that the plain
  // kernels keep their registers; five blocks per SM for the stencils with many couplings (BLK above,
  // chosen from the plan's tables: the slabs of a host-buffer step run the device step's kernels)
  if constexpr (PREC == MGX_PRECISION_FP64_FIXED_GATHER) {
    if (has_higher_onsite(L))
      launch_stages<NOISE, INTEG, PREC, true, 4>(pl, F, e, noise, step, stages, st, grid, tpb, cb, count, rows);
    else if (pl->fx.hw_convert)
      launch_stages<NOISE, INTEG, PREC, false, 5>(pl, F, e, noise, step, stages, st, grid, tpb, cb, count, rows);
    else
      launch_stages<NOISE, INTEG, PREC, false, 4>(pl, F, e, noise, step, stages, st, grid, tpb, cb, count, rows);
  } else {
    launch_stages<NOISE, INTEG, PREC, false, 4>(pl, F, e, noise, step, stages, st, grid, tpb, cb, count, rows);
  }
}

template <int NOISE, int PREC>
static void fx_integ(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st,
                     long long cb, long long cn, double* rows) {
  if (pl->p.integrator == MGX_INTEGRATOR_DEPONDT)
    launch_fx<NOISE, MGX_INTEGRATOR_DEPONDT, PREC>(pl, e, noise, step, stages, st, cb, cn, rows);
  else
    launch_fx<NOISE, MGX_INTEGRATOR_HEUN, PREC>(pl, e, noise, step, stages, st, cb, cn, rows);
}

template <int PREC>
static void fx_noise(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages, cudaStream_t st,
                     long long cb, long long cn, double* rows) {
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  switch (mode) {
    case MGX_NOISE_HOST: fx_integ<MGX_NOISE_HOST, PREC>(pl, e, noise, step, stages, st, cb, cn, rows); break;
    case MGX_NOISE_PHILOX: fx_integ<MGX_NOISE_PHILOX, PREC>(pl, e, noise, step, stages, st, cb, cn, rows); break;
    default: fx_integ<MGX_NOISE_NONE, PREC>(pl, e, noise, step, stages, st, cb, cn, rows); break;
  }
}

void enqueue_fx_range(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages,
                      long long cb, long long cn, double* rows) {
  if (pl->precision == MGX_PRECISION_FP64_FIXED_GATHER)
    fx_noise<MGX_PRECISION_FP64_FIXED_GATHER>(pl, e, noise, step, stages, st, cb, cn, rows);
  else
    fx_noise<MGX_PRECISION_INT48_GATHER>(pl, e, noise, step, stages, st, cb, cn, rows);
}

void enqueue_fx_pack_split(const LLGPlan* pl, const double* rows, double* lat, long long begin, long long count,
                           cudaStream_t st) {
  const DevLattice& L = pl->model->d;
  if (count <= 0) return;
  const unsigned grid = (unsigned)((count + 255) / 256);
  if (pl->precision == MGX_PRECISION_FP64_FIXED_GATHER)
    k_pack_split<28><<<grid, 256, 0, st>>>(rows, lat, pl->fx.es, L.ns, L.ncell, L.N, begin, count);
  else
    k_pack_split<24><<<grid, 256, 0, st>>>(rows, lat, pl->fx.es, L.ns, L.ncell, L.N, begin, count);
}

void enqueue_fx_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages) {
  enqueue_fx_range(pl, e, noise, step, st, stages, 0, pl->model->d.ncell);
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
  // conversions on the hardware converters for stencils of at least 16 couplings per site without the
  // cubic / higher-uniaxial terms, whose FP64 work makes the FP64 pipe the busier side (see DevFX)
  int zmax = 0;
  for (int s = 0; s < ns; ++s) zmax = std::max(zmax, off[s + 1] - off[s]);
  fx->hw_convert = zmax >= 16 && !has_higher_onsite(d) ? 1 : 0;
  fx->nz = nullptr;
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
  // 2^sigma >= the sum S of all magnitudes of the sublattice, so |w| = |round(J 2^(56 - sigma))| and
  // |v| = |round(e 2^56)| are at most 2^56 and their halves |w_hi|, |v_hi| <= 2^28, |w_lo|, |v_lo| <= 2^27.
  // Per field component, with n couplings (on-site included) and unit spins (sum_d |v_hi,d| <=
  // sqrt(3) 2^28 + 2):  |sum w_hi v_hi| <= (2^28 + 1)(sum |w| 2^-28 + 1.5 n) < 2^57, and
  // |sum (w_hi v_lo + w_lo v_hi)| <= 2^27 (2^28 + 1.5 n) + 2^27 n (sqrt(3) 2^28 + 2) < 2^55 (1 + 1.74 n),
  // below 2^63 for n <= 146: the 56-bit form takes at most 128 couplings per receiving sublattice.
  if (limb == 28)
    for (int s = 0; s < ns; ++s)
      if (off[s + 1] - off[s] + 1 > 128)
        return set_error(MGX_ERR_UNSUPPORTED, "sublattice %d has %d couplings: the 56-bit fixed-point sum takes at "
                         "most 127 couplings per site (plus the on-site term)", s, off[s + 1] - off[s]);
  std::vector<int> sigma(ns, 0);
  for (int s = 0; s < MGX_MAX_SUBLATTICES; ++s) {
    fx->scale[s] = 0.0;
    fx->scale_exp[s] = 0;
  }
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
    fx->scale_exp[s] = e - 2 * limb;
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
  // the normal-draw cache of the five-block kernels (the plans whose stages run five blocks per SM)
  if (limb == 28 && pl->fx.hw_convert && !has_higher_onsite(pl->model->d)) {
    MGX_CUDA_TRY(cudaMalloc(&pl->fx_noise, sizeof(float) * 3 * (size_t)pl->model->d.N));
    pl->fx.nz = pl->fx_noise;
  }
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
