// Adjoint (reverse-mode derivative) of the stochastic Heun step, with step checkpointing.
//
// Forward step (magex/llg.py:216-227), per site i, with H = B_eff + b:
//   H1 = H(e), f1 = f(e, H1), x = e + dt f1, p = x / |x|,
//   H2 = H(p), f2 = f(p, H2), y = e + dt/2 (f1 + f2), e' = y / |y|,
//   H(v)_i = (2 sum_j J_ij v_j - 2 A_i v_i) / (mu_i mu_B) + B + b_i,
//   f(e, H) = pre [e x H + alpha e x (e x H)].
// The reference has no gradients; this file supplies d loss / d e and the parameter gradients for
// a trajectory.  Given ebar' = dL/de' one backward step is three kernel bodies (the last one of a
// step and the first one of the step before it run as one kernel):
//   k_adj_local   (site-local) ybar, f1bar = f2bar = dt/2 ybar, H2bar and pbar from the rhs adjoint at
//                 (p, H2), g2 = 2 H2bar / (mu mu_B), local A term; A and B gradients of stage 2;
//   k_adj_mid     pbar += sum_rev J^T g2 (transposed stencil gather), xbar through the normalisation,
//                 f1bar += dt xbar, H1bar and ebar from the rhs adjoint at (e, H1), g1; J gradients of
//                 stage 2 (g2_i (x) p_j per coupling group); A and B gradients of stage 1;
//   k_adj_final   ebar = acc + sum_rev J^T g1; J gradients of stage 1 (g1_i (x) e_j).
// The transposed gather uses a second stencil (the reverse couplings j -> i with J_ij^T), so the
// adjoint is exact also when a coupling set does not satisfy J_ji = J_ij^T.
// Parameter gradients accumulate per site (deterministic, no atomics) and are summed at the end.
// States of a segment of steps are recomputed from a checkpoint and stored (e, p, H1, H2 and the two
// inverse norms); a caller may keep several segments resident (mgx_adjoint_set_storage) and skip
// their recomputation.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mgx_fx_step.cuh"
#include "mgx_observe.cuh"

namespace mgx {

struct AdjDev {
  DevLattice F;           // forward stencil
  DevLattice R;           // reverse stencil (transposed tensors), bonds sorted by (src, group, transposed)
  const int2* group;      // [nbond_rev] (parameter group, transposed flag) of the reverse couplings
  int ngroups;
  double dt, half_dt;
  double pre, alpha;      // uniform damping
  int precession;
  double* PG;             // [ngroups*9][N] coupling-group gradients per site
  double* PA;             // [9][N] single-ion gradients per site
  double* PB;             // [3][N] field gradients per site
  double* PH;             // [3][N] gradients w.r.t. the sites' Kc, K2, K3 (cubic / higher uniaxial), or nullptr
  // which parameter gradients are accumulated (mgx_adjoint_set_needs): coupling groups (PG), single-ion
  // tensors (PA), field (PB); the spins' adjoint is always computed
  int need_G = 1, need_A = 1, need_B = 1;
  // fixed-point transposed gathers (the plan's forward uses the fixed-point sum): the reverse
  // couplings as 56-bit fixed-point tensors, and per stage (0: g1, 1: g2) each site's g as 56-bit
  // fixed point at a power-of-two scale of its own (block floating point: gs = round(g 2^(56 - ge)))
  int fixed = 0;
  DevFX RF;
  int2* gs[2] = {nullptr, nullptr};   // [3][N] each
  int* ge[2] = {nullptr, nullptr};    // [N] each
};

struct AdjPlan {
  const Model* fwd = nullptr;
  const Model* rev = nullptr;
  AdjDev d;
  DevLLG P;               // forward parameters; ep / k1 re-pointed per step
  int seg_cap = 0;
  int noise = MGX_NOISE_NONE;
  double* seg = nullptr;  // current segment storage (one of own_seg or caller storage)
  // two plan-owned storages: a caller may recompute one segment into one while the backward pass
  // runs through the other (the second is allocated on first use)
  double* own_seg[2] = {nullptr, nullptr};
  double* work = nullptr; // eacc | pbar | f1bar | g1 | g2 (5 x 3N)
  double* k1 = nullptr;
  double* grads = nullptr;  // reduction output on device
  double* PH = nullptr;     // [3][N] Kc | K2 | K3 gradient accumulators (used when the model has those terms)
  int2* d_group = nullptr;
  void* sub = nullptr;
  int seg_steps = 0;
  // captured step loops of the plan's own segment storage (the recomputed segments): the forward of
  // `fwd_steps` steps (Philox step index from the device counter d_step) and the backward of
  // `bwd_steps` steps into `bwd_ebar`; dropped when the models change (kernel arguments hold the
  // stencils, fields included, by value)
  cudaStream_t cap_stream = nullptr;
  unsigned long long* d_step = nullptr;
  // (one pair per own storage)
  cudaGraphExec_t fwd_graph[2] = {nullptr, nullptr}, bwd_graph[2] = {nullptr, nullptr};
  int fwd_steps[2] = {0, 0}, bwd_steps[2] = {0, 0};
  const double* bwd_ebar[2] = {nullptr, nullptr};
  // forward (and recomputation) with the exact 56-bit fixed-point exchange sum (MGX_PRECISION_FP64_FIXED_GATHER):
  // tables of the current couplings and the split copies of e / ep
  bool fixed = false;
  DevFX fx{};
  void* fx_block = nullptr;
  void* rfx_block = nullptr;       // fixed-point tables of the reverse stencil (transposed gathers)
  void* gsplit_block = nullptr;    // g1 / g2 in block floating point
};

// Lattices up to this size replay captured graphs for recomputed segments (larger ones are bound by
// the kernels, not by their launches).
constexpr long long kAdjGraphMaxSites = 1LL << 21;

__device__ __forceinline__ void cross3(double ax, double ay, double az, double bx, double by, double bz, double& cx,
                                       double& cy, double& cz) {
  cx = ay * bz - az * by;
  cy = az * bx - ax * bz;
  cz = ax * by - ay * bx;
}

// rhs adjoint for f = pre [e x H + a e x (e x H)]: given fbar,
//   Hbar = pre [fbar x e + a e x (e x fbar)] = pre [-(e x fbar) + a (e (e.fbar) - fbar)],
//   ebar = pre [H x fbar + a ((e x H) x fbar - H x (e x fbar))]
//        = pre [H x fbar + a (H (e.fbar) + fbar (H.e) - 2 e (H.fbar))],
// using the triple-product identities and |e| = 1 (e and p are unit vectors to rounding);
// without precession the e x H terms (H x fbar, e x fbar) are dropped.
__device__ __forceinline__ void rhs_adjoint(double ex, double ey, double ez, double Hx, double Hy, double Hz,
                                            double fbx, double fby, double fbz, double a, double pre, bool prec,
                                            double& Hbx, double& Hby, double& Hbz, double& ebx, double& eby,
                                            double& ebz) {
  const double ef = ex * fbx + ey * fby + ez * fbz;
  const double He = Hx * ex + Hy * ey + Hz * ez;
  const double m2Hf = -2.0 * (Hx * fbx + Hy * fby + Hz * fbz);
  Hbx = a * fma(ex, ef, -fbx);
  Hby = a * fma(ey, ef, -fby);
  Hbz = a * fma(ez, ef, -fbz);
  ebx = a * fma(ex, m2Hf, fma(fbx, He, Hx * ef));
  eby = a * fma(ey, m2Hf, fma(fby, He, Hy * ef));
  ebz = a * fma(ez, m2Hf, fma(fbz, He, Hz * ef));
  if (prec) {
    double ux, uy, uz, hx, hy, hz;
    cross3(ex, ey, ez, fbx, fby, fbz, ux, uy, uz);     // e x fbar
    cross3(Hx, Hy, Hz, fbx, fby, fbz, hx, hy, hz);     // H x fbar
    Hbx -= ux; Hby -= uy; Hbz -= uz;
    ebx += hx; eby += hy; ebz += hz;
  }
  Hbx *= pre; Hby *= pre; Hbz *= pre;
  ebx *= pre; eby *= pre; ebz *= pre;
}

__device__ __forceinline__ void onsite_tensor(const DevLattice& L, long long q, int s, double* a) {
  if (L.A_site) {
    for (int k = 0; k < 9; ++k) a[k] = L.A_site[(long long)k * L.N + q];
  } else {
    for (int k = 0; k < 9; ++k) a[k] = L.A_sub[s * 9 + k];
  }
}

__device__ __forceinline__ void load3(const double* x, long long N, long long q, double& a, double& b, double& c) {
  a = x[q];
  b = x[N + q];
  c = x[2 * N + q];
}
__device__ __forceinline__ void store3(double* x, long long N, long long q, double a, double b, double c) {
  x[q] = a;
  x[N + q] = b;
  x[2 * N + q] = c;
}

// Per-site gradient accumulators are K cells N apart: all K loads are issued before any store (the
// compiler cannot prove that cells N apart do not alias, so a cell-by-cell read-modify-write would
// wait a full memory round trip per cell).
template <int K>
__device__ __forceinline__ void load_cells(const double* p, long long N, double* v) {
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = p[(long long)k * N];
}
template <int K>
__device__ __forceinline__ void store_cells(double* p, long long N, const double* v) {
#pragma unroll
  for (int k = 0; k < K; ++k) p[(long long)k * N] = v[k];
}

// PA -= g (x) v (single-ion gradient of one stage) and PB += Hbar (field gradient), as far as requested
__device__ __forceinline__ void accumulate_onsite(const AdjDev& A, long long N, long long q, bool hasA, double gx,
                                                  double gy, double gz, double vx, double vy, double vz, double Hbx,
                                                  double Hby, double Hbz) {
  hasA = hasA && A.need_A;
  if (!A.need_B) {
    if (!hasA) return;
    double pa[9];
    load_cells<9>(A.PA + q, N, pa);
    const double gv[3] = {gx, gy, gz}, v[3] = {vx, vy, vz};
#pragma unroll
    for (int k = 0; k < 9; ++k) pa[k] -= gv[k / 3] * v[k % 3];
    store_cells<9>(A.PA + q, N, pa);
    return;
  }
  double pa[9], pb[3];
  if (hasA) load_cells<9>(A.PA + q, N, pa);
  load_cells<3>(A.PB + q, N, pb);
  if (hasA) {
    const double gv[3] = {gx, gy, gz}, v[3] = {vx, vy, vz};
#pragma unroll
    for (int k = 0; k < 9; ++k) pa[k] -= gv[k / 3] * v[k % 3];
    store_cells<9>(A.PA + q, N, pa);
  }
  pb[0] += Hbx;
  pb[1] += Hby;
  pb[2] += Hbz;
  store_cells<3>(A.PB + q, N, pb);
}

// Adjoint of the cubic and higher-uniaxial fields at a site with spin v (magex/terms.py:35-75):
// B_h = -grad E_h(v) / (mu mu_B), so with g = 2 Hbar / (mu mu_B) the spin adjoint gains
// (dB_h/dv)^T Hbar = -Hess E_h(v) g / 2 (returned in ox, oy, oz) and the parameter accumulators
// PH[Kc | K2 | K3] gain Hbar . dB_h/dK = -(g / 2) . d(grad E_h)/dK.
//   cubic, a = C v, S = |a|^2:  dE/da_i = 2 Kc a_i (S - a_i^2),
//     (Hess_a w)_i = 2 Kc [(S - a_i^2) w_i + 2 a_i (a.w - a_i w_i)],  Hess_v = C^T Hess_a C;
//   uniaxial, c = v.u:  grad E = (-4 K2 c^3 - 6 K3 c^5) u,  Hess = (-12 K2 c^2 - 30 K3 c^4) u u^T.
__device__ __forceinline__ void higher_onsite_adjoint(const AdjDev& A, long long q, double vx, double vy, double vz,
                                                      double gx, double gy, double gz, double& ox, double& oy,
                                                      double& oz) {
  const DevLattice& L = A.F;
  const long long N = L.N;
  ox = oy = oz = 0.0;
  const double hx = 0.5 * gx, hy = 0.5 * gy, hz = 0.5 * gz;       // Hbar / (mu mu_B)
  double ph[3];
  load_cells<3>(A.PH + q, N, ph);
  if (L.Kc_site) {
    const double* C = L.C;
    const double a1 = C[0] * vx + C[1] * vy + C[2] * vz;
    const double a2 = C[3] * vx + C[4] * vy + C[5] * vz;
    const double a3 = C[6] * vx + C[7] * vy + C[8] * vz;
    const double w1 = C[0] * hx + C[1] * hy + C[2] * hz;              // w = C h
    const double w2 = C[3] * hx + C[4] * hy + C[5] * hz;
    const double w3 = C[6] * hx + C[7] * hy + C[8] * hz;
    const double q1 = a1 * a1, q2 = a2 * a2, q3 = a3 * a3, S = q1 + q2 + q3;
    const double aw = a1 * w1 + a2 * w2 + a3 * w3;
    const double kc = L.Kc_site[q];
    // -(h . d grad / dKc) = -(w . d), d_i = 2 a_i (S - a_i^2)
    ph[0] -= 2.0 * (w1 * a1 * (S - q1) + w2 * a2 * (S - q2) + w3 * a3 * (S - q3));
    const double t1 = 2.0 * kc * ((S - q1) * w1 + 2.0 * a1 * (aw - a1 * w1));
    const double t2 = 2.0 * kc * ((S - q2) * w2 + 2.0 * a2 * (aw - a2 * w2));
    const double t3 = 2.0 * kc * ((S - q3) * w3 + 2.0 * a3 * (aw - a3 * w3));
    ox -= C[0] * t1 + C[3] * t2 + C[6] * t3;                           // -C^T Hess_a C h
    oy -= C[1] * t1 + C[4] * t2 + C[7] * t3;
    oz -= C[2] * t1 + C[5] * t2 + C[8] * t3;
  }
  if (L.K2_site) {
    const double* u = L.u;
    const double c = vx * u[0] + vy * u[1] + vz * u[2], c2 = c * c;
    const double hu = hx * u[0] + hy * u[1] + hz * u[2];
    ph[1] += 4.0 * c2 * c * hu;
    ph[2] += 6.0 * c2 * c2 * c * hu;
    const double f = -(-12.0 * L.K2_site[q] * c2 - 30.0 * L.K3_site[q] * c2 * c2) * hu;
    ox += f * u[0];
    oy += f * u[1];
    oz += f * u[2];
  }
  store_cells<3>(A.PH + q, N, ph);
}

// Transposed gather sum_rev J^T g_nbr at site q of the reverse stencil, with the parameter-gradient
// outer products added to PG once per group run: a forward coupling with tensor T_g contributes
// g_nbr (x) v, one with T_g^T contributes v (x) g_nbr (v = own p or e), so each run keeps the sums of
// g_nbr over its plain and its transposed couplings and flushes 9 values per group.  Couplings are
// taken in chunks of ADJ_CHUNK: the neighbour values of a chunk are all loaded before any of them is
// used, so a site waits one memory round trip per chunk instead of one per coupling (small lattices,
// a few warps per SM, are bound by that latency).
constexpr int ADJ_CHUNK = 6;

__device__ __forceinline__ void adjoint_gather(const AdjDev& A, const double* __restrict__ g, long long q, int s,
                                               int c0, int c1, int c2, double vx, double vy, double vz,
                                               double& ox, double& oy, double& oz) {
  const DevLattice& L = A.R;
  const long long N = L.N;
  ox = oy = oz = 0.0;
  const int b0 = __ldg(L.bond_off + s), b1 = __ldg(L.bond_off + s + 1);
  int cur_g = -1;
  double sx = 0.0, sy = 0.0, sz = 0.0;      // sum of g over couplings with tensor T_g
  double tx = 0.0, ty = 0.0, tz = 0.0;      // sum of g over couplings with tensor T_g^T
  const double vv[3] = {vx, vy, vz};
  auto flush = [&]() {
    if (cur_g < 0 || !A.need_G) return;
    double* P = A.PG + (long long)cur_g * 9 * N + q;
    const double gs[3] = {sx, sy, sz}, gt[3] = {tx, ty, tz};
    double acc[9];
    load_cells<9>(P, N, acc);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) acc[3 * a + b] = fma(vv[a], gt[b], fma(gs[a], vv[b], acc[3 * a + b]));
    store_cells<9>(P, N, acc);
  };
  for (int c = b0; c < b1; c += ADJ_CHUNK) {
    double gx[ADJ_CHUNK], gy[ADJ_CHUNK], gz[ADJ_CHUNK];
#pragma unroll
    for (int k = 0; k < ADJ_CHUNK; ++k) {
      gx[k] = gy[k] = gz[k] = 0.0;
      const int b = c + k;
      if (b >= b1) continue;
      const int4 geo = __ldg(L.bond_geo + b);
      int n0 = c0 + geo.y, n1 = c1 + geo.z, n2 = c2 + geo.w;
      bool ok = true;
      if (L.pbc0) { n0 -= (n0 >= L.L0) ? L.L0 : 0; } else { ok &= (unsigned)n0 < (unsigned)L.L0; }
      if (L.pbc1) { n1 -= (n1 >= L.L1) ? L.L1 : 0; } else { ok &= (unsigned)n1 < (unsigned)L.L1; }
      if (L.pbc2) { n2 -= (n2 >= L.L2) ? L.L2 : 0; } else { ok &= (unsigned)n2 < (unsigned)L.L2; }
      if (!ok) continue;                    // a dropped coupling contributes a zero g
      const long long j = (long long)geo.x * L.ncell + ((long long)n0 * L.L1 + n1) * L.L2 + n2;
      gx[k] = __ldg(g + j);
      gy[k] = __ldg(g + N + j);
      gz[k] = __ldg(g + 2 * N + j);
    }
#pragma unroll
    for (int k = 0; k < ADJ_CHUNK; ++k) {
      const int b = c + k;
      if (b >= b1) break;
      const int2 gr = __ldg(A.group + b);
      if (gr.x != cur_g) {
        flush();
        cur_g = gr.x;
        sx = sy = sz = 0.0;
        tx = ty = tz = 0.0;
      }
      const double* T = L.bond_J + (long long)b * 9;
      ox = fma(__ldg(T + 0), gx[k], ox); ox = fma(__ldg(T + 1), gy[k], ox); ox = fma(__ldg(T + 2), gz[k], ox);
      oy = fma(__ldg(T + 3), gx[k], oy); oy = fma(__ldg(T + 4), gy[k], oy); oy = fma(__ldg(T + 5), gz[k], oy);
      oz = fma(__ldg(T + 6), gx[k], oz); oz = fma(__ldg(T + 7), gy[k], oz); oz = fma(__ldg(T + 8), gz[k], oz);
      if (gr.y) {
        tx += gx[k]; ty += gy[k]; tz += gz[k];
      } else {
        sx += gx[k]; sy += gy[k]; sz += gz[k];
      }
    }
  }
  flush();
}

// ---------------------------------------------------------------- forward recomputation (stores states)
// (step index: P.step_base[0] + step inside a captured segment, step otherwise)
// (HIGHER: the EXTRA bodies, which add the cubic / higher-uniaxial fields; the adjoint's forward
// parameters carry no spin-orbit torque or extra field)
template <int NOISE, bool HIGHER>
__global__ void __launch_bounds__(256) k_fwd_pred(const DevLattice L, const DevLLG P, const double* __restrict__ e,
                                                  uint64_t step, double* __restrict__ H1, double* __restrict__ R) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < L.N)
    predict_site<9, NOISE, MGX_INTEGRATOR_HEUN, HIGHER>(L, P, e, nullptr, q, P.step_base ? *P.step_base + step : step,
                                                        H1, R);
}

template <int NOISE, bool HIGHER>
__global__ void __launch_bounds__(256) k_fwd_corr(const DevLattice L, const DevLLG P, double* __restrict__ e,
                                                  uint64_t step, double* __restrict__ H2, double* __restrict__ eout,
                                                  double* __restrict__ R) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < L.N)
    correct_site<9, NOISE, MGX_INTEGRATOR_HEUN, HIGHER>(L, P, e, nullptr, q, P.step_base ? *P.step_base + step : step,
                                                        H2, eout, nullptr, R + L.N);
}

// the same with the exact fixed-point exchange sum: the split of E is in F.es (written by the previous
// corrector, or by the split kernel before the first step); the corrector writes E_next and its split
template <int NOISE, bool HIGHER>
__global__ void __launch_bounds__(256, 4) k_fwd_pred_fx(const DevLattice L, const DevLLG P, const DevFX F,
                                                        const double* __restrict__ e, uint64_t step,
                                                        double* __restrict__ H1, double* __restrict__ R) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < L.N)
    fx_predict_site<NOISE, MGX_INTEGRATOR_HEUN, MGX_PRECISION_FP64_FIXED_GATHER, HIGHER, 0>(
        L, P, F, e, nullptr, q, P.step_base ? *P.step_base + step : step, H1, R);
}

template <int NOISE, bool HIGHER>
__global__ void __launch_bounds__(256, 4) k_fwd_corr_fx(const DevLattice L, const DevLLG P, const DevFX F,
                                                        double* __restrict__ e, uint64_t step, double* __restrict__ H2,
                                                        double* __restrict__ eout, double* __restrict__ R) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < L.N)
    fx_correct_site<NOISE, MGX_INTEGRATOR_HEUN, MGX_PRECISION_FP64_FIXED_GATHER, HIGHER, 0>(
        L, P, F, e, nullptr, q, P.step_base ? *P.step_base + step : step, H2, eout, R + L.N);
}

__global__ void k_adj_step_set(unsigned long long* c, unsigned long long v) { *c = v; }

// ---------------------------------------------------------------- fixed-point transposed gather
// g of site q in block floating point: the exponent tau with max_c |g_c| < 2^tau (from the bit pattern
// of the largest component) and round(g_c 2^(56 - tau)) in balanced 28-bit halves, all on the integer
// pipes.
__device__ __forceinline__ void store_g_split(const AdjDev& A, int which, long long N, long long q, double gx,
                                              double gy, double gz) {
  const unsigned long long mask = 0x7FFFFFFFFFFFFFFFULL;
  const unsigned long long ax = (unsigned long long)__double_as_longlong(gx) & mask;
  const unsigned long long ay = (unsigned long long)__double_as_longlong(gy) & mask;
  const unsigned long long az = (unsigned long long)__double_as_longlong(gz) & mask;
  const unsigned long long m = ax > ay ? (ax > az ? ax : az) : (ay > az ? ay : az);
  const int E = (int)(m >> 52);
  const int tau = (E == 0 ? 1 : E) - 1022;
  int2* gs = A.gs[which];
  gs[q] = fx_halves<28>(double_to_ll_scaled(gx, 56 - tau));
  gs[N + q] = fx_halves<28>(double_to_ll_scaled(gy, 56 - tau));
  gs[2 * N + q] = fx_halves<28>(double_to_ll_scaled(gz, 56 - tau));
  A.ge[which][q] = tau;
}

// a 56-bit fixed-point value (two halves) at exponent tau_j, re-expressed at exponent tau_j + d
// (rounded, d >= 0)
__device__ __forceinline__ long long fx_align(int2 h, int d) {
  const long long v = ((long long)h.x << 28) + (long long)h.y;
  if (d <= 0) return v;
  if (d > 62) return 0;
  return (v + (1LL << (d - 1))) >> d;
}

// t 2^e2 as FP64 (ll_to_double_scaled, with a plain fallback where the result would leave the normal
// range: the adjoint field of a site whose neighbours' g are all tiny)
__device__ __forceinline__ double fx_to_double(long long t, int e2) {
  if (t == 0) return 0.0;
  const unsigned long long a = t < 0 ? 0ULL - (unsigned long long)t : (unsigned long long)t;
  const int msb = 63 - __clzll((long long)a);
  if (msb + e2 + 1023 < 2 || msb + e2 + 1023 > 2045) return ldexp((double)t, e2);
  return ll_to_double_scaled(t, e2);
}

// The transposed gather of adjoint_gather on the integer pipes: the neighbours' g (block floating
// point, stage `which`) are aligned to the largest exponent among them and multiplied by the
// fixed-point J^T exactly (the sum of products is exact; each aligned term is rounded to 2^-57 of the
// largest); the group sums for the parameter gradients are exact integer sums too.  The coupling
// gradients' outer products stay FP64.
__device__ __forceinline__ void adjoint_gather_fx(const AdjDev& A, int which, long long q, int s, int c0, int c1,
                                                  int c2, double vx, double vy, double vz, double& ox, double& oy,
                                                  double& oz) {
  const DevLattice& L = A.R;
  const long long N = L.N;
  const int2* __restrict__ gs = A.gs[which];
  const int* __restrict__ ge = A.ge[which];
  const int b0 = __ldg(L.bond_off + s), b1 = __ldg(L.bond_off + s + 1);
  auto nbr = [&](int b) -> long long {
    const int4 geo = __ldg(L.bond_geo + b);
    int n0 = c0 + geo.y, n1 = c1 + geo.z, n2 = c2 + geo.w;
    bool ok = true;
    if (L.pbc0) { n0 -= (n0 >= L.L0) ? L.L0 : 0; } else { ok &= (unsigned)n0 < (unsigned)L.L0; }
    if (L.pbc1) { n1 -= (n1 >= L.L1) ? L.L1 : 0; } else { ok &= (unsigned)n1 < (unsigned)L.L1; }
    if (L.pbc2) { n2 -= (n2 >= L.L2) ? L.L2 : 0; } else { ok &= (unsigned)n2 < (unsigned)L.L2; }
    return ok ? (long long)geo.x * L.ncell + ((long long)n0 * L.L1 + n1) * L.L2 + n2 : -1LL;
  };
  int tmax = -2000;
  for (int b = b0; b < b1; ++b) {
    const long long j = nbr(b);
    if (j >= 0) tmax = max(tmax, __ldg(ge + j));
  }
  FxAcc acc;
  long long ss[3] = {0, 0, 0}, tt[3] = {0, 0, 0};   // exact sums of g over plain / transposed couplings
  int cur_g = -1;
  const double vv[3] = {vx, vy, vz};
  auto flush = [&]() {
    if (cur_g < 0 || !A.need_G) return;
    double* P = A.PG + (long long)cur_g * 9 * N + q;
    double gsd[3], gtd[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      gsd[c] = fx_to_double(ss[c], tmax - 56);
      gtd[c] = fx_to_double(tt[c], tmax - 56);
    }
    double accp[9];
    load_cells<9>(P, N, accp);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) accp[3 * a + b] = fma(vv[a], gtd[b], fma(gsd[a], vv[b], accp[3 * a + b]));
    store_cells<9>(P, N, accp);
  };
  for (int b = b0; b < b1; ++b) {
    const int2 gr = __ldg(A.group + b);
    if (gr.x != cur_g) {
      flush();
      cur_g = gr.x;
      ss[0] = ss[1] = ss[2] = 0;
      tt[0] = tt[1] = tt[2] = 0;
    }
    const long long j = nbr(b);
    if (j < 0) continue;
    const int d = tmax - __ldg(ge + j);
    const long long v0 = fx_align(__ldg(gs + j), d), v1 = fx_align(__ldg(gs + N + j), d),
                    v2 = fx_align(__ldg(gs + 2 * N + j), d);
    fx_mat(A.RF.J + 5 * b, fx_halves<28>(v0), fx_halves<28>(v1), fx_halves<28>(v2), acc);
    if (gr.y) {
      tt[0] += v0; tt[1] += v1; tt[2] += v2;
    } else {
      ss[0] += v0; ss[1] += v1; ss[2] += v2;
    }
  }
  flush();
  const int e2 = A.RF.scale_exp[s] + tmax;
  ox = fx_to_double(acc.hh[0] + ((acc.x[0] + (1LL << 27)) >> 28), e2);
  oy = fx_to_double(acc.hh[1] + ((acc.x[1] + (1LL << 27)) >> 28), e2);
  oz = fx_to_double(acc.hh[2] + ((acc.x[2] + (1LL << 27)) >> 28), e2);
}

// ---------------------------------------------------------------- backward kernels
// Site-local part of the backward step (first kernel body of step n): ybar from zbar = dL/de' through
// the corrector normalisation (e' = y |y|^-1 and |y|^-1 are stored), the rhs adjoint at (p, H2), g2
// and the stage-2 single-ion and field gradients.
__device__ __forceinline__ void adj_local_site(const AdjDev& A, long long q, const double* __restrict__ Z,
                                               const double* __restrict__ Pp, const double* __restrict__ H2,
                                               const double* __restrict__ R, double zbx, double zby, double zbz,
                                               double* __restrict__ eacc, double* __restrict__ pbar,
                                               double* __restrict__ f1bar, double* __restrict__ g2) {
  const DevLattice& L = A.F;
  const long long N = L.N;
  if (L.pinned && L.pinned[q]) {
    store3(eacc, N, q, zbx, zby, zbz);
    store3(pbar, N, q, 0.0, 0.0, 0.0);
    store3(f1bar, N, q, 0.0, 0.0, 0.0);
    store3(g2, N, q, 0.0, 0.0, 0.0);
    if (A.fixed) store_g_split(A, 1, N, q, 0.0, 0.0, 0.0);
    return;
  }
  const int s = (int)(q / L.ncell);
  double zx, zy, zz, px, py, pz, h2x, h2y, h2z;
  load3(Z, N, q, zx, zy, zz);
  load3(Pp, N, q, px, py, pz);
  load3(H2, N, q, h2x, h2y, h2z);
  const double inv_ny = R[N + q];
  const bool prec = A.precession != 0;
  const double zd = zx * zbx + zy * zby + zz * zbz;
  const double ybx = fma(-zx, zd, zbx) * inv_ny, yby = fma(-zy, zd, zby) * inv_ny, ybz = fma(-zz, zd, zbz) * inv_ny;
  const double fbx = A.half_dt * ybx, fby = A.half_dt * yby, fbz = A.half_dt * ybz;
  double Hbx, Hby, Hbz, pbx, pby, pbz;
  rhs_adjoint(px, py, pz, h2x, h2y, h2z, fbx, fby, fbz, A.alpha, A.pre, prec, Hbx, Hby, Hbz, pbx, pby, pbz);
  const double inv2 = 2.0 * (L.inv_mu_site ? L.inv_mu_site[q] : L.inv_mu_sub[s]);
  const double gx = Hbx * inv2, gy = Hby * inv2, gz = Hbz * inv2;
  if (L.has_A) {
    double a[9];
    onsite_tensor(L, q, s, a);
    pbx -= a[0] * gx + a[3] * gy + a[6] * gz;     // -A^T g
    pby -= a[1] * gx + a[4] * gy + a[7] * gz;
    pbz -= a[2] * gx + a[5] * gy + a[8] * gz;
  }
  if (A.PH) {
    double hx, hy, hz;
    higher_onsite_adjoint(A, q, px, py, pz, gx, gy, gz, hx, hy, hz);
    pbx += hx;
    pby += hy;
    pbz += hz;
  }
  accumulate_onsite(A, N, q, L.has_A != 0, gx, gy, gz, px, py, pz, Hbx, Hby, Hbz);
  store3(eacc, N, q, ybx, yby, ybz);
  store3(pbar, N, q, pbx, pby, pbz);
  store3(f1bar, N, q, fbx, fby, fbz);
  store3(g2, N, q, gx, gy, gz);
  if (A.fixed) store_g_split(A, 1, N, q, gx, gy, gz);
}

__global__ void __launch_bounds__(256) k_adj_local(const AdjDev A, const double* __restrict__ Z,
                                                   const double* __restrict__ Pp, const double* __restrict__ H2,
                                                   const double* __restrict__ R, const double* __restrict__ ebar,
                                                   double* __restrict__ eacc, double* __restrict__ pbar,
                                                   double* __restrict__ f1bar, double* __restrict__ g2) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= A.F.N) return;
  double zbx, zby, zbz;
  load3(ebar, A.F.N, q, zbx, zby, zbz);
  adj_local_site(A, q, Z, Pp, H2, R, zbx, zby, zbz, eacc, pbar, f1bar, g2);
}

// Resident blocks per SM asked of the adjoint kernels in the fixed-point form: their FP64 work is
// about two thirds of the all-FP64 form's, so occupancy (80 registers, a few spills) pays there; the
// FP64 instantiations keep their registers (about 126) and stay bound by the FP64 pipe.  Measured on
// the 1024^2 film (200 steps, fixed-point form): backward 213.5 -> 190.2 ms.
constexpr int kAdjFxBlocks = 3;

// Second kernel of step n: pbar += sum_rev J^T g2, xbar through the predictor normalisation
// (p = x |x|^-1, both stored), the rhs adjoint at (e, H1), g1; stage-2 coupling and stage-1 single-ion
// and field gradients.
template <bool FX>
__device__ __forceinline__ void adj_mid_site(
    const AdjDev& A, const double* __restrict__ E, const double* __restrict__ Pp, const double* __restrict__ H1,
    const double* __restrict__ R, double* __restrict__ eacc, const double* __restrict__ pbar,
    const double* __restrict__ f1bar, const double* __restrict__ g2, double* __restrict__ g1) {
  const DevLattice& L = A.F;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double px, py, pz;
  load3(Pp, N, q, px, py, pz);
  double tx, ty, tz;
  if (FX)
    adjoint_gather_fx(A, 1, q, s, c0, c1, c2, px, py, pz, tx, ty, tz);
  else
    adjoint_gather(A, g2, q, s, c0, c1, c2, px, py, pz, tx, ty, tz);
  double pbx, pby, pbz;
  load3(pbar, N, q, pbx, pby, pbz);
  pbx += tx;
  pby += ty;
  pbz += tz;
  double ax, ay, az;
  load3(eacc, N, q, ax, ay, az);
  if (L.pinned && L.pinned[q]) {          // p = e on pinned sites
    store3(eacc, N, q, ax + pbx, ay + pby, az + pbz);
    store3(g1, N, q, 0.0, 0.0, 0.0);
    if (FX) store_g_split(A, 0, N, q, 0.0, 0.0, 0.0);
    return;
  }
  double ex, ey, ez, h1x, h1y, h1z;
  load3(E, N, q, ex, ey, ez);
  load3(H1, N, q, h1x, h1y, h1z);
  const double inv_nx = R[q];
  const bool prec = A.precession != 0;
  const double ud = px * pbx + py * pby + pz * pbz;
  const double xbx = fma(-px, ud, pbx) * inv_nx, xby = fma(-py, ud, pby) * inv_nx, xbz = fma(-pz, ud, pbz) * inv_nx;
  ax += xbx;
  ay += xby;
  az += xbz;
  double fbx, fby, fbz;
  load3(f1bar, N, q, fbx, fby, fbz);
  fbx = fma(A.dt, xbx, fbx);
  fby = fma(A.dt, xby, fby);
  fbz = fma(A.dt, xbz, fbz);
  double Hbx, Hby, Hbz, ebx, eby, ebz;
  rhs_adjoint(ex, ey, ez, h1x, h1y, h1z, fbx, fby, fbz, A.alpha, A.pre, prec, Hbx, Hby, Hbz, ebx, eby, ebz);
  const double inv2 = 2.0 * (L.inv_mu_site ? L.inv_mu_site[q] : L.inv_mu_sub[s]);
  const double gx = Hbx * inv2, gy = Hby * inv2, gz = Hbz * inv2;
  ax += ebx;
  ay += eby;
  az += ebz;
  if (L.has_A) {
    double a[9];
    onsite_tensor(L, q, s, a);
    ax -= a[0] * gx + a[3] * gy + a[6] * gz;
    ay -= a[1] * gx + a[4] * gy + a[7] * gz;
    az -= a[2] * gx + a[5] * gy + a[8] * gz;
  }
  if (A.PH) {
    double hx, hy, hz;
    higher_onsite_adjoint(A, q, ex, ey, ez, gx, gy, gz, hx, hy, hz);
    ax += hx;
    ay += hy;
    az += hz;
  }
  accumulate_onsite(A, N, q, L.has_A != 0, gx, gy, gz, ex, ey, ez, Hbx, Hby, Hbz);
  store3(eacc, N, q, ax, ay, az);
  store3(g1, N, q, gx, gy, gz);
  if (FX) store_g_split(A, 0, N, q, gx, gy, gz);
}

// Last kernel of step n: ebar_n = acc + sum_rev J^T g1 (and the stage-1 coupling gradients).  With
// FUSE the site-local body of step n - 1 follows in the same thread on ebar_n, which is then never
// stored; otherwise ebar_n is written out.
template <bool FUSE, bool FX>
__device__ __forceinline__ void adj_final_site(
    const AdjDev& A, const double* __restrict__ E, double* __restrict__ eacc, const double* __restrict__ g1,
    double* __restrict__ ebar, const double* __restrict__ Pprev, const double* __restrict__ H2prev,
    const double* __restrict__ Rprev, double* __restrict__ pbar, double* __restrict__ f1bar, double* __restrict__ g2) {
  const DevLattice& L = A.F;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double ex, ey, ez;
  load3(E, N, q, ex, ey, ez);
  double tx, ty, tz;
  if (FX)
    adjoint_gather_fx(A, 0, q, s, c0, c1, c2, ex, ey, ez, tx, ty, tz);
  else
    adjoint_gather(A, g1, q, s, c0, c1, c2, ex, ey, ez, tx, ty, tz);
  double ax, ay, az;
  load3(eacc, N, q, ax, ay, az);
  if (FUSE) {
    // step n - 1 ends in e(n) = E: its corrector output z is this step's input spins
    adj_local_site(A, q, E, Pprev, H2prev, Rprev, ax + tx, ay + ty, az + tz, eacc, pbar, f1bar, g2);
  } else {
    store3(ebar, N, q, ax + tx, ay + ty, az + tz);
  }
}

// The adjoint kernels: the FP64 form unbounded in registers, the fixed-point form at kAdjFxBlocks
// blocks per SM.
#define MGX_MID_PARAMS                                                                                          \
  const AdjDev A, const double* __restrict__ E, const double* __restrict__ Pp, const double* __restrict__ H1,    \
      const double* __restrict__ R, double* __restrict__ eacc, const double* __restrict__ pbar,                 \
      const double* __restrict__ f1bar, const double* __restrict__ g2, double* __restrict__ g1
#define MGX_FINAL_PARAMS                                                                                        \
  const AdjDev A, const double* __restrict__ E, double* __restrict__ eacc, const double* __restrict__ g1,        \
      double* __restrict__ ebar, const double* __restrict__ Pprev, const double* __restrict__ H2prev,           \
      const double* __restrict__ Rprev, double* __restrict__ pbar, double* __restrict__ f1bar,                  \
      double* __restrict__ g2
__global__ void __launch_bounds__(256) k_adj_mid(MGX_MID_PARAMS) {
  adj_mid_site<false>(A, E, Pp, H1, R, eacc, pbar, f1bar, g2, g1);
}
__global__ void __launch_bounds__(256, kAdjFxBlocks) k_adj_mid_fx(MGX_MID_PARAMS) {
  adj_mid_site<true>(A, E, Pp, H1, R, eacc, pbar, f1bar, g2, g1);
}
template <bool FUSE>
__global__ void __launch_bounds__(256) k_adj_final(MGX_FINAL_PARAMS) {
  adj_final_site<FUSE, false>(A, E, eacc, g1, ebar, Pprev, H2prev, Rprev, pbar, f1bar, g2);
}
template <bool FUSE>
__global__ void __launch_bounds__(256, kAdjFxBlocks) k_adj_final_fx(MGX_FINAL_PARAMS) {
  adj_final_site<FUSE, true>(A, E, eacc, g1, ebar, Pprev, H2prev, Rprev, pbar, f1bar, g2);
}
#undef MGX_MID_PARAMS
#undef MGX_FINAL_PARAMS

// out[r] = sum of x[r*stride .. r*stride + len)  (one block per row, fixed-order tree)
__global__ void __launch_bounds__(256) k_sum_rows(const double* __restrict__ x, long long len, long long stride,
                                                  double* __restrict__ out) {
  const double* row = x + (long long)blockIdx.x * stride;
  double acc = 0.0;
  for (long long i = threadIdx.x; i < len; i += blockDim.x) acc += row[i];
  __shared__ double red[8];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w];
    out[blockIdx.x] = s;
  }
}

constexpr int SEG_E = 0, SEG_P = 1, SEG_H1 = 2, SEG_H2 = 3, SEG_R = 4;

// Segment storage: per step [e | ep | H1 | H2] (3N doubles each) and [1/|x| | 1/|y|] (2N) of the
// predictor and corrector normalisations, then one more e slot for the spins after the last step.
static size_t seg_stride(const AdjPlan* a) { return 14 * (size_t)a->fwd->d.N; }
static size_t seg_doubles(const AdjPlan* a) { return seg_stride(a) * a->seg_cap + 3 * (size_t)a->fwd->d.N; }

static double* seg_ptr(const AdjPlan* a, int n, int k) {
  const size_t N = (size_t)a->fwd->d.N;
  if (k == SEG_E && n == a->seg_cap) return a->seg + seg_stride(a) * a->seg_cap;   // tail slot
  return a->seg + seg_stride(a) * n + (size_t)k * 3 * N;
}

// The kernels of a forward segment of nsteps steps from the spins in storage slot 0 (step index
// step0 + n, or the device counter plus n when P.step_base is set).
template <int NOISE, bool HIGHER>
static void launch_adj_step_fx(const AdjPlan* a, const DevLLG& P, double* E, uint64_t step, double* H1, double* H2,
                               double* E1, double* R, unsigned grid, int tpb, cudaStream_t st) {
  const DevLattice& L = a->fwd->d;
  k_fwd_pred_fx<NOISE, HIGHER><<<grid, tpb, 0, st>>>(L, P, a->fx, E, step, H1, R);
  k_fwd_corr_fx<NOISE, HIGHER><<<grid, tpb, 0, st>>>(L, P, a->fx, E, step, H2, E1, R);
}

static void enqueue_adj_forward(const AdjPlan* a, const DevLLG& P0, int nsteps, uint64_t step0, cudaStream_t st) {
  const DevLattice& L = a->fwd->d;
  const long long N = L.N;
  const int tpb = site_block_size(N);
  const unsigned grid = (unsigned)((N + tpb - 1) / tpb);
  if (a->fixed) {
    // the split of the first spins; every corrector then writes the split of the spins it produces
    enqueue_fx_split_n(seg_ptr(a, 0, SEG_E), a->fx.es, 3 * N, 28, st);
    const bool hi = has_higher_onsite(L);
    for (int n = 0; n < nsteps; ++n) {
      DevLLG P = P0;
      P.ep = seg_ptr(a, n, SEG_P);
      double* E = seg_ptr(a, n, SEG_E);
      double* R = seg_ptr(a, n, SEG_R);
      double* H1 = seg_ptr(a, n, SEG_H1);
      double* H2 = seg_ptr(a, n, SEG_H2);
      double* E1 = seg_ptr(a, n + 1, SEG_E);
      const uint64_t step = step0 + (uint64_t)n;
      if (a->noise == MGX_NOISE_PHILOX)
        hi ? launch_adj_step_fx<MGX_NOISE_PHILOX, true>(a, P, E, step, H1, H2, E1, R, grid, tpb, st)
           : launch_adj_step_fx<MGX_NOISE_PHILOX, false>(a, P, E, step, H1, H2, E1, R, grid, tpb, st);
      else
        hi ? launch_adj_step_fx<MGX_NOISE_NONE, true>(a, P, E, step, H1, H2, E1, R, grid, tpb, st)
           : launch_adj_step_fx<MGX_NOISE_NONE, false>(a, P, E, step, H1, H2, E1, R, grid, tpb, st);
    }
    return;
  }
  for (int n = 0; n < nsteps; ++n) {
    DevLLG P = P0;
    P.ep = seg_ptr(a, n, SEG_P);
    double* E = seg_ptr(a, n, SEG_E);
    double* R = seg_ptr(a, n, SEG_R);
    const uint64_t step = step0 + (uint64_t)n;
    double* H1 = seg_ptr(a, n, SEG_H1);
    double* H2 = seg_ptr(a, n, SEG_H2);
    double* E1 = seg_ptr(a, n + 1, SEG_E);
    const bool hi = has_higher_onsite(L);
    if (a->noise == MGX_NOISE_PHILOX) {
      if (hi) {
        k_fwd_pred<MGX_NOISE_PHILOX, true><<<grid, tpb, 0, st>>>(L, P, E, step, H1, R);
        k_fwd_corr<MGX_NOISE_PHILOX, true><<<grid, tpb, 0, st>>>(L, P, E, step, H2, E1, R);
      } else {
        k_fwd_pred<MGX_NOISE_PHILOX, false><<<grid, tpb, 0, st>>>(L, P, E, step, H1, R);
        k_fwd_corr<MGX_NOISE_PHILOX, false><<<grid, tpb, 0, st>>>(L, P, E, step, H2, E1, R);
      }
    } else {
      if (hi) {
        k_fwd_pred<MGX_NOISE_NONE, true><<<grid, tpb, 0, st>>>(L, P, E, step, H1, R);
        k_fwd_corr<MGX_NOISE_NONE, true><<<grid, tpb, 0, st>>>(L, P, E, step, H2, E1, R);
      } else {
        k_fwd_pred<MGX_NOISE_NONE, false><<<grid, tpb, 0, st>>>(L, P, E, step, H1, R);
        k_fwd_corr<MGX_NOISE_NONE, false><<<grid, tpb, 0, st>>>(L, P, E, step, H2, E1, R);
      }
    }
  }
}

// The kernels of the backward pass through a segment of nsteps steps (ebar in: dL/de after the last
// step; out: dL/de before the first).
static void enqueue_adj_backward(const AdjPlan* a, double* ebar, int nsteps, cudaStream_t st) {
  const long long N = a->fwd->d.N;
  const size_t n3 = 3 * (size_t)N;
  const int tpb = site_block_size(N);
  const unsigned grid = (unsigned)((N + tpb - 1) / tpb);
  double* eacc = a->work;
  double* pbar = a->work + n3;
  double* f1bar = a->work + 2 * n3;
  double* g1 = a->work + 3 * n3;
  double* g2 = a->work + 4 * n3;
  const int last = nsteps - 1;
  k_adj_local<<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, last + 1, SEG_E), seg_ptr(a, last, SEG_P),
                                    seg_ptr(a, last, SEG_H2), seg_ptr(a, last, SEG_R), ebar, eacc, pbar, f1bar, g2);
  for (int n = last; n >= 0; --n) {
    if (a->d.fixed)
      k_adj_mid_fx<<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, n, SEG_E), seg_ptr(a, n, SEG_P), seg_ptr(a, n, SEG_H1),
                                            seg_ptr(a, n, SEG_R), eacc, pbar, f1bar, g2, g1);
    else
      k_adj_mid<<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, n, SEG_E), seg_ptr(a, n, SEG_P), seg_ptr(a, n, SEG_H1),
                                             seg_ptr(a, n, SEG_R), eacc, pbar, f1bar, g2, g1);
    if (n > 0) {
      if (a->d.fixed)
        k_adj_final_fx<true><<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, n, SEG_E), eacc, g1, nullptr,
                                                      seg_ptr(a, n - 1, SEG_P), seg_ptr(a, n - 1, SEG_H2),
                                                      seg_ptr(a, n - 1, SEG_R), pbar, f1bar, g2);
      else
        k_adj_final<true><<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, n, SEG_E), eacc, g1, nullptr,
                                                       seg_ptr(a, n - 1, SEG_P), seg_ptr(a, n - 1, SEG_H2),
                                                       seg_ptr(a, n - 1, SEG_R), pbar, f1bar, g2);
    } else {
      if (a->d.fixed)
        k_adj_final_fx<false><<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, 0, SEG_E), eacc, g1, ebar, nullptr, nullptr,
                                                       nullptr, nullptr, nullptr, nullptr);
      else
        k_adj_final<false><<<grid, tpb, 0, st>>>(a->d, seg_ptr(a, 0, SEG_E), eacc, g1, ebar, nullptr, nullptr,
                                                        nullptr, nullptr, nullptr, nullptr);
    }
  }
}

// (Re)build the fixed-point tables from the forward model's current couplings and on-site tensors
// (called at creation and whenever the models change), keeping two split arrays of 3 N.
static mgx_status build_adj_fx(AdjPlan* a) {
  if (!a->fixed) return MGX_OK;
  if (a->fx_block) cudaFree(a->fx_block);
  if (a->rfx_block) cudaFree(a->rfx_block);
  a->fx_block = a->rfx_block = nullptr;
  mgx_status st = fx_build(a->fwd, 28, true, 2, &a->fx, &a->fx_block);
  if (st == MGX_OK) st = fx_build(a->rev, 28, false, 0, &a->d.RF, &a->rfx_block);
  if (st != MGX_OK) return st;
  if (!a->gsplit_block) {
    const size_t N = (size_t)a->fwd->d.N;
    MGX_CUDA_TRY(cudaMalloc(&a->gsplit_block, 2 * (sizeof(int2) * 3 * N + sizeof(int) * N)));
    char* p = (char*)a->gsplit_block;
    for (int k = 0; k < 2; ++k) {
      a->d.gs[k] = (int2*)p;
      p += sizeof(int2) * 3 * N;
    }
    for (int k = 0; k < 2; ++k) {
      a->d.ge[k] = (int*)p;
      p += sizeof(int) * N;
    }
  }
  a->d.fixed = 1;
  return MGX_OK;
}

static void drop_adj_graphs(AdjPlan* a) {
  for (int k = 0; k < 2; ++k) {
    if (a->fwd_graph[k]) cudaGraphExecDestroy(a->fwd_graph[k]);
    if (a->bwd_graph[k]) cudaGraphExecDestroy(a->bwd_graph[k]);
    a->fwd_graph[k] = a->bwd_graph[k] = nullptr;
    a->fwd_steps[k] = a->bwd_steps[k] = 0;
    a->bwd_ebar[k] = nullptr;
  }
}

// Index of the current storage among the plan's own storages, or -1 for caller storage.
static int own_index(const AdjPlan* a) {
  for (int k = 0; k < 2; ++k)
    if (a->own_seg[k] && a->seg == a->own_seg[k]) return k;
  return -1;
}

// Capture the kernels that `enqueue` puts on a stream into *exec.
template <typename F>
static mgx_status capture_adj(AdjPlan* a, cudaGraphExec_t* exec, F enqueue) {
  if (!a->cap_stream) MGX_CUDA_TRY(cudaStreamCreateWithFlags(&a->cap_stream, cudaStreamNonBlocking));
  MGX_CUDA_TRY(cudaStreamBeginCapture(a->cap_stream, cudaStreamCaptureModeThreadLocal));
  enqueue(a->cap_stream);
  cudaGraph_t g = nullptr;
  cudaError_t err = cudaStreamEndCapture(a->cap_stream, &g);
  if (err != cudaSuccess) return cuda_error(err, "adjoint segment capture");
  err = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (err != cudaSuccess) {
    *exec = nullptr;
    return cuda_error(err, "adjoint segment instantiate");
  }
  return MGX_OK;
}

}  // namespace mgx

using namespace mgx;

extern "C" {

mgx_status mgx_adjoint_create(const mgx_model* fwd, const mgx_model* rev, const int32_t* rev_group,
                              const int32_t* rev_transposed, int32_t ngroups, const mgx_llg_params* p,
                              int32_t seg_steps, mgx_adjoint** out) {
  const Model* F = reinterpret_cast<const Model*>(fwd);
  const Model* R = reinterpret_cast<const Model*>(rev);
  if (!F || !R || !p || !out) return set_error(MGX_ERR_INVALID, "mgx_adjoint_create: null argument");
  *out = nullptr;
  if (F->d.layout != 0 || R->d.layout != 0)
    return set_error(MGX_ERR_UNSUPPORTED, "the adjoint is implemented for lattice stencils, not neighbour lists");
  if (F->d.width != 9 || R->d.width != 9)
    return set_error(MGX_ERR_INVALID, "the adjoint needs full-tensor (width 9) forward and reverse models");
  if (F->d.ns != R->d.ns || F->d.L0 != R->d.L0 || F->d.L1 != R->d.L1 || F->d.L2 != R->d.L2 ||
      F->d.pbc0 != R->d.pbc0 || F->d.pbc1 != R->d.pbc1 || F->d.pbc2 != R->d.pbc2)
    return set_error(MGX_ERR_INVALID, "forward and reverse models must describe the same supercell");
  if (F->nbond != R->nbond) return set_error(MGX_ERR_INVALID, "the reverse stencil must have one coupling per forward coupling");
  if (F->d.A_site) return set_error(MGX_ERR_UNSUPPORTED, "the adjoint supports single-ion tensors per sublattice only");
  if (ngroups < 1 || ngroups > 4096) return set_error(MGX_ERR_INVALID, "ngroups must be in 1..4096");
  if (R->nbond > 0 && (!rev_group || !rev_transposed)) return set_error(MGX_ERR_INVALID, "group arrays are required");
  if (p->alpha_site) return set_error(MGX_ERR_UNSUPPORTED, "the adjoint supports a uniform damping only");
  if (p->precision != MGX_PRECISION_FP64 && p->precision != MGX_PRECISION_FP64_FIXED_GATHER)
    return set_error(MGX_ERR_UNSUPPORTED, "the adjoint runs its forward in the FP64 form (0) or the FP64 form with "
                     "the exact fixed-point exchange sum (3)");
  if (p->integrator != MGX_INTEGRATOR_HEUN) return set_error(MGX_ERR_UNSUPPORTED, "the adjoint is implemented for heun");
  if (p->noise == MGX_NOISE_HOST) return set_error(MGX_ERR_UNSUPPORTED, "the adjoint recomputes noise: use none or philox");
  if (!(p->dt > 0.0)) return set_error(MGX_ERR_INVALID, "dt must be positive");
  if (seg_steps < 1) return set_error(MGX_ERR_INVALID, "seg_steps must be >= 1");
  std::vector<int2> grp(std::max(R->nbond, 1));
  for (int b = 0; b < R->nbond; ++b) {
    if (rev_group[b] < 0 || rev_group[b] >= ngroups) return set_error(MGX_ERR_INVALID, "group of bond %d out of range", b);
    grp[b] = make_int2(rev_group[b], rev_transposed[b] ? 1 : 0);
  }
  AdjPlan* a = new AdjPlan();
  a->fwd = F;
  a->rev = R;
  a->seg_cap = seg_steps;
  a->noise = p->noise;
  a->fixed = p->precision == MGX_PRECISION_FP64_FIXED_GATHER;
  const long long N = F->d.N;
  const int ns = F->d.ns;
  const double gamma = 0.1760859630;
  const double pre = -gamma / (1.0 + p->alpha * p->alpha);
  const size_t n3 = 3 * (size_t)N;
  cudaError_t err = cudaMalloc(&a->own_seg[0], sizeof(double) * seg_doubles(a));
  a->seg = a->own_seg[0];
  if (err == cudaSuccess) err = cudaMalloc(&a->work, sizeof(double) * n3 * 5);
  if (err == cudaSuccess) err = cudaMalloc(&a->k1, sizeof(double) * n3);
  if (err == cudaSuccess) err = cudaMalloc(&a->d_group, sizeof(int2) * grp.size());
  if (err == cudaSuccess) err = cudaMalloc(&a->d.PG, sizeof(double) * 9 * (size_t)ngroups * N);
  if (err == cudaSuccess) err = cudaMalloc(&a->d.PA, sizeof(double) * 9 * (size_t)N);
  if (err == cudaSuccess) err = cudaMalloc(&a->d.PB, sizeof(double) * 3 * (size_t)N);
  if (err == cudaSuccess) err = cudaMalloc(&a->PH, sizeof(double) * 3 * (size_t)N);
  if (err == cudaSuccess) err = cudaMemset(a->PH, 0, sizeof(double) * 3 * (size_t)N);
  if (err == cudaSuccess) err = cudaMalloc(&a->grads, sizeof(double) * (9 * (size_t)ngroups + 9 * ns + 3));
  if (err == cudaSuccess) err = cudaMalloc(&a->sub, sizeof(double) * 3 * ns);
  if (err == cudaSuccess) err = cudaMalloc(&a->d_step, sizeof(unsigned long long));
  if (err == cudaSuccess) err = cudaMemcpy(a->d_group, grp.data(), sizeof(int2) * grp.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    std::vector<double> sub(3 * ns, 0.0);
    for (int s = 0; s < ns; ++s) {
      sub[s] = p->alpha;
      sub[ns + s] = pre;
    }
    err = cudaMemcpy(a->sub, sub.data(), sizeof(double) * sub.size(), cudaMemcpyHostToDevice);
  }
  if (err == cudaSuccess) err = cudaMemset(a->d.PG, 0, sizeof(double) * 9 * (size_t)ngroups * N);
  if (err == cudaSuccess) err = cudaMemset(a->d.PA, 0, sizeof(double) * 9 * (size_t)N);
  if (err == cudaSuccess) err = cudaMemset(a->d.PB, 0, sizeof(double) * 3 * (size_t)N);
  if (err != cudaSuccess) {
    mgx_adjoint_destroy(reinterpret_cast<mgx_adjoint*>(a));
    return cuda_error(err, "mgx_adjoint_create");
  }
  AdjDev& d = a->d;
  d.F = F->d;
  d.R = R->d;
  d.PH = has_higher_onsite(F->d) ? a->PH : nullptr;
  d.group = a->d_group;
  d.ngroups = ngroups;
  d.dt = p->dt;
  d.half_dt = 0.5 * p->dt;
  d.alpha = p->alpha;
  d.pre = pre;
  d.precession = p->precession ? 1 : 0;
  DevLLG& P = a->P;
  P.dt = p->dt;
  P.half_dt = 0.5 * p->dt;
  P.precession = p->precession ? 1 : 0;
  P.noise = p->noise;
  P.integrator = MGX_INTEGRATOR_HEUN;
  P.seed = p->seed;
  P.alpha_sub = (const double*)a->sub;
  P.pre_sub = P.alpha_sub + ns;
  P.sigma_sub = P.alpha_sub + 2 * ns;
  P.alpha_site = P.pre_site = P.sigma_site = nullptr;
  P.ep = nullptr;
  P.k1 = a->k1;
  const mgx_status fs = build_adj_fx(a);
  if (fs != MGX_OK) {
    mgx_adjoint_destroy(reinterpret_cast<mgx_adjoint*>(a));
    return fs;
  }
  *out = reinterpret_cast<mgx_adjoint*>(a);
  return MGX_OK;
}

mgx_status mgx_adjoint_destroy(mgx_adjoint* aa) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a) return MGX_OK;
  drop_adj_graphs(a);
  if (a->fx_block) cudaFree(a->fx_block);
  if (a->rfx_block) cudaFree(a->rfx_block);
  if (a->gsplit_block) cudaFree(a->gsplit_block);
  if (a->cap_stream) cudaStreamDestroy(a->cap_stream);
  cudaFree(a->d_step);
  cudaFree(a->own_seg[0]);
  cudaFree(a->own_seg[1]);
  cudaFree(a->work);
  cudaFree(a->k1);
  cudaFree(a->d_group);
  cudaFree(a->d.PG);
  cudaFree(a->d.PA);
  cudaFree(a->d.PB);
  cudaFree(a->PH);
  cudaFree(a->grads);
  cudaFree(a->sub);
  delete a;
  return MGX_OK;
}

mgx_status mgx_adjoint_set_sigma(mgx_adjoint* aa, const double* sigma_sub) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a || !sigma_sub) return set_error(MGX_ERR_INVALID, "mgx_adjoint_set_sigma: null argument");
  const int ns = a->fwd->d.ns;
  for (int s = 0; s < ns; ++s)
    if (!std::isfinite(sigma_sub[s]) || sigma_sub[s] < 0.0) return set_error(MGX_ERR_INVALID, "sigma must be finite and >= 0");
  MGX_CUDA_TRY(cudaMemcpy((double*)a->sub + 2 * ns, sigma_sub, sizeof(double) * ns, cudaMemcpyHostToDevice));
  return MGX_OK;
}

mgx_status mgx_adjoint_sync_models(mgx_adjoint* aa) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a) return set_error(MGX_ERR_INVALID, "mgx_adjoint_sync_models: null argument");
  a->d.F = a->fwd->d;
  a->d.R = a->rev->d;
  a->d.PH = has_higher_onsite(a->fwd->d) ? a->PH : nullptr;
  drop_adj_graphs(a);
  return build_adj_fx(a);
}

int64_t mgx_adjoint_storage_doubles(const mgx_adjoint* aa) {
  const AdjPlan* a = reinterpret_cast<const AdjPlan*>(aa);
  return a ? (int64_t)seg_doubles(a) : -1;
}

mgx_status mgx_adjoint_set_storage(mgx_adjoint* aa, double* storage) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a) return set_error(MGX_ERR_INVALID, "mgx_adjoint_set_storage: null adjoint");
  if (storage && ((uintptr_t)storage % 16) != 0) return set_error(MGX_ERR_INVALID, "storage must be 16-byte aligned");
  a->seg = storage ? storage : a->own_seg[0];
  return MGX_OK;
}

mgx_status mgx_adjoint_forward(mgx_adjoint* aa, const double* e0, int32_t nsteps, uint64_t step0, double* e_out,
                               void* stream) {
  NvtxRange nvtx_range("mgx_adjoint_forward");
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a || !e0) return set_error(MGX_ERR_INVALID, "mgx_adjoint_forward: null argument");
  if (nsteps < 1 || nsteps > a->seg_cap)
    return set_error(MGX_ERR_INVALID, "nsteps = %d outside 1..%d (segment capacity)", nsteps, a->seg_cap);
  cudaStream_t st = (cudaStream_t)stream;
  const long long N = a->fwd->d.N;
  if (e0 != seg_ptr(a, 0, SEG_E))
    MGX_CUDA_TRY(cudaMemcpyAsync(seg_ptr(a, 0, SEG_E), e0, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, st));
  const int own = own_index(a);
  if (own >= 0 && N <= kAdjGraphMaxSites) {
    // recomputed segments of a small lattice: one graph replay (the step index from the counter)
    if (!a->fwd_graph[own] || a->fwd_steps[own] != nsteps) {
      if (a->fwd_graph[own]) cudaGraphExecDestroy(a->fwd_graph[own]);
      a->fwd_graph[own] = nullptr;
      DevLLG P = a->P;
      P.step_base = a->d_step;
      const mgx_status cs = capture_adj(a, &a->fwd_graph[own], [&](cudaStream_t cst) {
        enqueue_adj_forward(a, P, nsteps, 0, cst);
      });
      if (cs != MGX_OK) return cs;
      a->fwd_steps[own] = nsteps;
    }
    k_adj_step_set<<<1, 1, 0, st>>>(a->d_step, (unsigned long long)step0);
    MGX_CUDA_TRY(cudaGraphLaunch(a->fwd_graph[own], st));
  } else {
    enqueue_adj_forward(a, a->P, nsteps, step0, st);
  }
  if (e_out)
    MGX_CUDA_TRY(cudaMemcpyAsync(e_out, seg_ptr(a, nsteps, SEG_E), sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, st));
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_adjoint_backward(mgx_adjoint* aa, double* ebar, int32_t nsteps, void* stream) {
  NvtxRange nvtx_range("mgx_adjoint_backward");
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a || !ebar) return set_error(MGX_ERR_INVALID, "mgx_adjoint_backward: null argument");
  if (nsteps < 1 || nsteps > a->seg_cap)
    return set_error(MGX_ERR_INVALID, "nsteps = %d outside 1..%d (segment capacity)", nsteps, a->seg_cap);
  cudaStream_t st = (cudaStream_t)stream;
  const long long N = a->fwd->d.N;
  const int own = own_index(a);
  if (own >= 0 && N <= kAdjGraphMaxSites) {
    if (!a->bwd_graph[own] || a->bwd_steps[own] != nsteps || a->bwd_ebar[own] != ebar) {
      if (a->bwd_graph[own]) cudaGraphExecDestroy(a->bwd_graph[own]);
      a->bwd_graph[own] = nullptr;
      const mgx_status cs = capture_adj(a, &a->bwd_graph[own], [&](cudaStream_t cst) {
        enqueue_adj_backward(a, ebar, nsteps, cst);
      });
      if (cs != MGX_OK) return cs;
      a->bwd_steps[own] = nsteps;
      a->bwd_ebar[own] = ebar;
    }
    MGX_CUDA_TRY(cudaGraphLaunch(a->bwd_graph[own], st));
  } else {
    enqueue_adj_backward(a, ebar, nsteps, st);
  }
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_adjoint_zero_grads(mgx_adjoint* aa, void* stream) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a) return set_error(MGX_ERR_INVALID, "mgx_adjoint_zero_grads: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const long long N = a->fwd->d.N;
  MGX_CUDA_TRY(cudaMemsetAsync(a->d.PG, 0, sizeof(double) * 9 * (size_t)a->d.ngroups * N, st));
  MGX_CUDA_TRY(cudaMemsetAsync(a->d.PA, 0, sizeof(double) * 9 * (size_t)N, st));
  MGX_CUDA_TRY(cudaMemsetAsync(a->d.PB, 0, sizeof(double) * 3 * (size_t)N, st));
  MGX_CUDA_TRY(cudaMemsetAsync(a->PH, 0, sizeof(double) * 3 * (size_t)N, st));
  return MGX_OK;
}

mgx_status mgx_adjoint_grads(mgx_adjoint* aa, double* out, void* stream) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a || !out) return set_error(MGX_ERR_INVALID, "mgx_adjoint_grads: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const DevLattice& L = a->fwd->d;
  const long long N = L.N;
  const int G = a->d.ngroups, ns = L.ns;
  k_sum_rows<<<9 * G, 256, 0, st>>>(a->d.PG, N, N, out);
  k_sum_rows<<<9 * ns, 256, 0, st>>>(a->d.PA, L.ncell, L.ncell, out + 9 * G);   // rows (component k, sublattice s)
  k_sum_rows<<<3, 256, 0, st>>>(a->d.PB, N, N, out + 9 * G + 9 * ns);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_adjoint_select_own_storage(mgx_adjoint* aa, int32_t which) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a) return set_error(MGX_ERR_INVALID, "mgx_adjoint_select_own_storage: null adjoint");
  if (which != 0 && which != 1) return set_error(MGX_ERR_INVALID, "own storage %d is not 0 or 1", which);
  if (!a->own_seg[which]) MGX_CUDA_TRY(cudaMalloc(&a->own_seg[which], sizeof(double) * seg_doubles(a)));
  a->seg = a->own_seg[which];
  return MGX_OK;
}

mgx_status mgx_adjoint_set_needs(mgx_adjoint* aa, int32_t couplings, int32_t onsite, int32_t field) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a) return set_error(MGX_ERR_INVALID, "mgx_adjoint_set_needs: null adjoint");
  const int g = couplings ? 1 : 0, o = onsite ? 1 : 0, f = field ? 1 : 0;
  if (g != a->d.need_G || o != a->d.need_A || f != a->d.need_B) {
    a->d.need_G = g;
    a->d.need_A = o;
    a->d.need_B = f;
    drop_adj_graphs(a);                 // captured kernels hold the flags by value
  }
  return MGX_OK;
}

mgx_status mgx_adjoint_grads_onsite_higher(mgx_adjoint* aa, double* out, void* stream) {
  AdjPlan* a = reinterpret_cast<AdjPlan*>(aa);
  if (!a || !out) return set_error(MGX_ERR_INVALID, "mgx_adjoint_grads_onsite_higher: null argument");
  const long long N = a->fwd->d.N;
  k_sum_rows<<<3, 256, 0, (cudaStream_t)stream>>>(a->PH, N, N, out);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

}  // extern "C"
