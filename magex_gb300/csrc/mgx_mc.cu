// Monte Carlo colour sweeps on the GB300: magex/montecarlo.py:71-230 (MetropolisMC.sweep and its
// NumPy moves), magex/fast.py:393-490 (_mc_group) and magex/cuda_backend.py:220-304,380-418 (_k_mc,
// CudaMC).
//
// Sites are split into colour classes of mutually non-interacting sites (first-fit greedy colouring
// in magex site order, magex/montecarlo.py:35-48, computed on the host by mgx_colour_stencil /
// mgx_colour_graph).  All sites of one class are updated at once by one kernel launch: thread t owns
// site sites[t], gathers its exchange field with the same stencil / neighbour-list code as the LLG
// kernels, proposes a move (Gaussian cone, uniform direction, heat bath of the linear field, Hinzke
// mixture, or an over-relaxation reflection about the exchange field), evaluates the energy change
// of magex's _dE (magex/montecarlo.py:136-147) and accepts with the Metropolis rule.  Because no two
// sites of a class interact, the order of updates inside a class does not matter and the result is
// the sequential sweep's.
//
// Random numbers: counter-based Philox keyed by (seed, magex site, sweep, pass), or host-supplied
// buffers with exactly the draws of the NumPy sweep in its order, so that a sweep reproduces magex's
// own trajectory (the layout is documented at mgx_mc_sweep in include/mgx.h).
#include <cmath>
#include <vector>

#include "mgx_fx.cuh"

namespace mgx {

constexpr double kMuB = 5.7883818060e-2;     // meV / T (magex/spinmodel.py:28)

// Chains of an ensemble (mgx_mc_set_chains): per-chain Philox key, inverse temperature, cone width and
// accept counter; seed == nullptr for the plan's single chain.
struct McChains {
  const uint64_t* seed;
  const double* beta;
  const double* sigma;
  unsigned long long* acc;
};

struct McPlan {
  const Model* model = nullptr;
  int move = 0;
  int overrelax = 0;
  int rng = 0;
  double sigma = 0.6;
  uint64_t seed = 0;
  uint64_t sweep = 0;
  int ngroups = 0;
  std::vector<long long> gsize, goff;
  std::vector<int> hb_ok;                  // heat bath usable in group g (every beta finite)
  long long* sites = nullptr;              // device [sum gsize] lattice indices, grouped
  double* beta = nullptr;                  // device [ns] per-sublattice beta
  double* beta_site = nullptr;             // device [N] per-site beta (lattice layout), or nullptr
  unsigned long long* acc = nullptr;       // device accepted-move counter
  unsigned long long tried = 0;
  std::vector<long long> sites_host;
  bool fixed = false;                      // exchange field from the exact 56-bit fixed-point gather
  DevFX fx{};
  void* fx_block = nullptr;
  bool share = false;                      // small classes split a site over kShare lanes (see launch_pass)
  // ensemble (mgx_mc_set_chains): nchains > 1 or chain_block set
  int nchains = 1;
  void* chain_block = nullptr;             // device: seed | beta | sigma | acc, nchains each
  McChains chains{};
};

// ------------------------------------------------------------------ random numbers
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {       // [0, 1), 53 random bits
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * 1.1102230246251565e-16;
}

struct McRandom {
  // one Philox block per (site, sweep, pass, slot)
  __device__ static uint4 block(uint64_t seed, uint64_t site, uint64_t sweep, int pass, int slot) {
    return philox4x32_10(make_uint4((uint32_t)site, (uint32_t)(site >> 32), (uint32_t)sweep,
                                    ((uint32_t)(sweep >> 32) << 12) | ((uint32_t)pass << 4) | (uint32_t)slot),
                         make_uint2((uint32_t)(seed ^ 0x4d43u), (uint32_t)(seed >> 32)));
  }
  // three N(0, 1) draws by Box-Muller from the block of slot, in FP32 as the LLG thermal field: the
  // proposal's precision does not enter the acceptance test, and FP64 log / sincos would be about half
  // of a trial move's FP64 instructions (slot + 1 stays reserved)
  __device__ static void normal3(uint64_t seed, uint64_t site, uint64_t sweep, int pass, int slot, double& g0,
                                 double& g1, double& g2) {
    const uint4 r = block(seed, site, sweep, pass, slot);
    const float tw = 2.3283064365386963e-10f;                 // 2^-32
    const float u1 = fmaf((float)r.x, tw, 0.5f * tw);          // (0, 1]
    const float u3 = fmaf((float)r.z, tw, 0.5f * tw);
    const float m1 = sqrtf(-2.0f * logf(u1));
    const float m3 = sqrtf(-2.0f * logf(u3));
    float s1, c1;
    sincospif(2.0f * ((float)r.y * tw), &s1, &c1);
    g0 = (double)(m1 * c1);
    g1 = (double)(m1 * s1);
    g2 = (double)(m3 * cospif(2.0f * ((float)r.w * tw)));
  }
};

// u < exp(x) for -700 <= x <= 0 with u a multiple of 2^-53 (Philox u53 or NumPy's random()): the
// decision of the FP64 comparison, taken in FP32 unless exp(x) is within 1e-5 of u (the FP32
// exponential of the rounded argument is within 3e-6 of exp(x) for x >= -40).  Below -40, exp(x)
// < 2^-53 <= every nonzero u.
__device__ __forceinline__ bool below_exp(double u, double x) {
  if (x < -40.0) return u == 0.0;
  const double ef = (double)expf((float)x);
  if (u < ef * (1.0 - 1e-5)) return true;
  if (u >= ef * (1.0 + 1e-5)) return false;
  return u < exp(x);
}

__device__ __forceinline__ void normalise3(double& x, double& y, double& z) {
  const double n = sqrt(x * x + y * y + z * z);       // magex normalize: e / |e| (magex/spinmodel.py:553)
  x /= n;
  y /= n;
  z /= n;
}

// e.A.e at lattice index q (sublattice s)
__device__ __forceinline__ double onsite(const DevLattice& L, long long q, int s, double x, double y, double z) {
  double a[9];
  if (L.A_site) {
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = __ldg(L.A_site + (long long)k * L.N + q);
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = __ldg(L.A_sub + s * 9 + k);
  }
  return x * (a[0] * x + a[1] * y + a[2] * z) + y * (a[3] * x + a[4] * y + a[5] * z) +
         z * (a[6] * x + a[7] * y + a[8] * z);
}

enum { MC_GAUSSIAN = 0, MC_UNIFORM = 1, MC_HEATBATH = 2, MC_HINZKE = 3, MC_OVERRELAX = 4 };

// This lane's share of the exchange field h = sum_j J_ij x_j when LANES lanes split a site's
// couplings: couplings lane, lane + LANES, ... (the shares are summed by the caller).  Same per-coupling
// arithmetic and open-boundary skips as exchange_field.
template <int W, int LANES>
__device__ __forceinline__ void exchange_field_share(const DevLattice& L, const double* __restrict__ x, int s, int c0,
                                                     int c1, int c2, int lane, double& hx, double& hy, double& hz) {
  hx = hy = hz = 0.0;
  const long long N = L.N;
  const int b0 = __ldg(L.bond_off + s), b1 = __ldg(L.bond_off + s + 1);
  for (int b = b0 + lane; b < b1; b += LANES) {
    const int4 g = __ldg(L.bond_geo + b);
    int n0 = c0 + g.y, n1 = c1 + g.z, n2 = c2 + g.w;
    bool ok = true;
    if (L.pbc0) { n0 -= (n0 >= L.L0) ? L.L0 : 0; } else { ok &= (unsigned)n0 < (unsigned)L.L0; }
    if (L.pbc1) { n1 -= (n1 >= L.L1) ? L.L1 : 0; } else { ok &= (unsigned)n1 < (unsigned)L.L1; }
    if (L.pbc2) { n2 -= (n2 >= L.L2) ? L.L2 : 0; } else { ok &= (unsigned)n2 < (unsigned)L.L2; }
    if (!ok) continue;
    const long long j = (long long)g.x * L.ncell + ((long long)n0 * L.L1 + n1) * L.L2 + n2;
    const double ex = __ldg(x + j), ey = __ldg(x + N + j), ez = __ldg(x + 2 * N + j);
    const double* T = L.bond_J + (long long)b * W;
    if (W == 1) {
      const double J = __ldg(T);
      hx = fma(J, ex, hx);
      hy = fma(J, ey, hy);
      hz = fma(J, ez, hz);
    } else if (W == 4) {
      const double J = __ldg(T), Dx = __ldg(T + 1), Dy = __ldg(T + 2), Dz = __ldg(T + 3);
      hx = fma(J, ex, hx); hx = fma(ey, Dz, hx); hx = fma(-ez, Dy, hx);
      hy = fma(J, ey, hy); hy = fma(ez, Dx, hy); hy = fma(-ex, Dz, hy);
      hz = fma(J, ez, hz); hz = fma(ex, Dy, hz); hz = fma(-ey, Dx, hz);
    } else {
      hx = fma(__ldg(T + 0), ex, hx); hx = fma(__ldg(T + 1), ey, hx); hx = fma(__ldg(T + 2), ez, hx);
      hy = fma(__ldg(T + 3), ex, hy); hy = fma(__ldg(T + 4), ey, hy); hy = fma(__ldg(T + 5), ez, hy);
      hz = fma(__ldg(T + 6), ex, hz); hz = fma(__ldg(T + 7), ey, hz); hz = fma(__ldg(T + 8), ez, hz);
    }
  }
}

// One pass over the n sites of a colour class (of chain blockIdx.y of an ensemble).  hr: host-supplied
// draws of this pass (RNG_HOST), laid out as documented at mgx_mc_sweep; otherwise Philox with counter
// (site, sweep, pass).
// LANES > 1 (stencil FP64 plans, small classes): LANES consecutive lanes share one site; each sums its
// share of the couplings, the shares are added across the group, every lane of the group then runs the
// same move and test and lane 0 writes the site.  This shortens each thread's serial chain when a class
// is too small to fill the GPU with one thread per site.
template <int W, int MOVE, bool HOSTRNG, bool FIXED, int LANES>
__global__ void __launch_bounds__(128) k_mc_pass(const DevLattice L, double* __restrict__ e,
                                                 const long long* __restrict__ sites, long long n,
                                                 const double* __restrict__ beta_sub,
                                                 const double* __restrict__ beta_site, double sigma,
                                                 const double* __restrict__ hr, uint64_t seed, uint64_t sweep,
                                                 int pass, unsigned long long* acc, const DevFX F,
                                                 const McChains chains) {
  const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / LANES;
  const int lane = (int)(threadIdx.x % LANES);
  double chain_beta = 0.0;
  if (chains.seed) {
    const int k = blockIdx.y;
    e += (long long)k * 3 * L.N;
    seed = chains.seed[k];
    sigma = chains.sigma[k];
    chain_beta = chains.beta[k];
    acc = chains.acc + k;
  }
  bool ok = false;
  const bool active = t < n;
  long long q = 0;
  int s = 0, c0 = 0, c1 = 0, c2 = 0;
  double hx = 0.0, hy = 0.0, hz = 0.0;
  if (LANES > 1) {
    if (active) {
      q = __ldg(sites + t);
      site_coords(L, q, s, c0, c1, c2);
      exchange_field_share<W, LANES>(L, e, s, c0, c1, c2, lane, hx, hy, hz);
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) {          // every lane of the warp takes part
      hx += __shfl_xor_sync(0xffffffffu, hx, o);
      hy += __shfl_xor_sync(0xffffffffu, hy, o);
      hz += __shfl_xor_sync(0xffffffffu, hz, o);
    }
  }
  if (active) {
    const long long N = L.N;
    if (LANES == 1) {
      q = __ldg(sites + t);
      site_coords(L, q, s, c0, c1, c2);
      if (FIXED) {
        // exact 56-bit fixed-point sum h = sum_j J_ij e_j, rounded once to FP64
        FxAcc a;
        fx_accumulate(L, F, F.es, q, s, c0, c1, c2, a);
        const double sc = F.scale[s];
        hx = fma((double)a.x[0], 3.7252902984619141e-9, (double)a.hh[0]) * sc;
        hy = fma((double)a.x[1], 3.7252902984619141e-9, (double)a.hh[1]) * sc;
        hz = fma((double)a.x[2], 3.7252902984619141e-9, (double)a.hh[2]) * sc;
      } else {
        exchange_field<W>(L, e, s, c0, c1, c2, hx, hy, hz);
      }
    }
    const long long m = (L.layout == 1) ? q : (long long)(q - (long long)s * L.ncell) * L.ns + s;
    const double ox = e[q], oy = e[N + q], oz = e[2 * N + q];
    const double mu = L.mu_site ? __ldg(L.mu_site + q) : __ldg(L.mu_sub + s);
    const double bt = chains.seed ? chain_beta : (beta_site ? __ldg(beta_site + q) : __ldg(beta_sub + s));
    double nx, ny, nz, ua;
    double extra = 0.0;                       // heat bath: (en - eo).H is added back (nonlinear part only)
    if (MOVE == MC_OVERRELAX) {
      // reflection about the exchange field h (magex/montecarlo.py:200-210)
      const double hh = hx * hx + hy * hy + hz * hz;
      nx = ox; ny = oy; nz = oz;
      if (hh > 1e-14) {
        const double p = 2.0 * ((ox * hx + oy * hy + oz * hz) / hh);
        nx = p * hx - ox;
        ny = p * hy - oy;
        nz = p * hz - oz;
      }
      normalise3(nx, ny, nz);
      ua = HOSTRNG ? __ldg(hr + t) : [&] { const uint4 r = McRandom::block(seed, m, sweep, pass, 0);
                                           return u53(r.x, r.y); }();
    } else if (MOVE == MC_HEATBATH) {
      // exp(beta H.e) on the unit sphere for the linear field H = 2h + mu_B mu B (magex/montecarlo.py:51-68)
      const double zf = kMuB * mu;
      const double Hx = 2.0 * hx + zf * L.B0, Hy = 2.0 * hy + zf * L.B1, Hz = 2.0 * hz + zf * L.B2;
      double u1, u2;
      if (HOSTRNG) {
        u1 = __ldg(hr + t);
        u2 = __ldg(hr + n + t);
        ua = __ldg(hr + 2 * n + t);
      } else {
        const uint4 r = McRandom::block(seed, m, sweep, pass, 0);
        u1 = u53(r.x, r.y);
        u2 = u53(r.z, r.w);
        const uint4 r2 = McRandom::block(seed, m, sweep, pass, 1);
        ua = u53(r2.x, r2.y);
      }
      const double Hn = sqrt(Hx * Hx + Hy * Hy + Hz * Hz);
      const double x = bt * Hn;
      const bool small = x < 1e-8;
      double c = small ? 2.0 * u1 - 1.0 : 1.0 + log1p(-u1 * (-expm1(-2.0 * x))) / x;
      c = fmin(1.0, fmax(-1.0, c));
      const double ph = 2.0 * M_PI * u2;
      double zx = 0.0, zy = 0.0, zz = 1.0;
      if (!small) {
        const double d = Hn > 0 ? Hn : 1.0;
        zx = Hx / d; zy = Hy / d; zz = Hz / d;
      }
      const bool ax = fabs(zx) < 0.9;             // a = x-hat, else y-hat
      double t1x = ax ? 0.0 : -zz, t1y = ax ? zz : 0.0, t1z = ax ? -zy : zx;
      normalise3(t1x, t1y, t1z);
      const double t2x = zy * t1z - zz * t1y, t2y = zz * t1x - zx * t1z, t2z = zx * t1y - zy * t1x;
      const double sn = sqrt(1.0 - c * c);
      const double cp = cos(ph), sp = sin(ph);
      nx = c * zx + sn * (cp * t1x + sp * t2x);
      ny = c * zy + sn * (cp * t1y + sp * t2y);
      nz = c * zz + sn * (cp * t1z + sp * t2z);
      normalise3(nx, ny, nz);
      extra = (nx - ox) * Hx + (ny - oy) * Hy + (nz - oz) * Hz;
    } else {
      double g0, g1, g2;
      if (HOSTRNG) {
        const long long o = (MOVE == MC_HINZKE) ? n : 0;
        g0 = __ldg(hr + o + 3 * t);
        g1 = __ldg(hr + o + 3 * t + 1);
        g2 = __ldg(hr + o + 3 * t + 2);
      } else {
        McRandom::normal3(seed, m, sweep, pass, 0, g0, g1, g2);
      }
      if (MOVE == MC_UNIFORM) {
        nx = g0; ny = g1; nz = g2;
      } else {
        nx = ox + sigma * g0; ny = oy + sigma * g1; nz = oz + sigma * g2;
      }
      normalise3(nx, ny, nz);
      if (MOVE == MC_HINZKE) {
        // k = 0: Gaussian cone, 1: uniform direction, 2: spin flip (magex/montecarlo.py:217-224)
        int k;
        double f0, f1, f2;
        if (HOSTRNG) {
          k = (int)__ldg(hr + t);
          f0 = __ldg(hr + 4 * n + 3 * t);
          f1 = __ldg(hr + 4 * n + 3 * t + 1);
          f2 = __ldg(hr + 4 * n + 3 * t + 2);
          ua = __ldg(hr + 7 * n + t);
        } else {
          McRandom::normal3(seed, m, sweep, pass, 2, f0, f1, f2);
          const uint4 r2 = McRandom::block(seed, m, sweep, pass, 4);
          k = (int)(((unsigned long long)r2.z * 3ull) >> 32);
          ua = u53(r2.x, r2.y);
        }
        if (k == 1) {
          normalise3(f0, f1, f2);
          nx = f0; ny = f1; nz = f2;
        } else if (k == 2) {
          nx = -ox; ny = -oy; nz = -oz;
        }
      } else {
        if (HOSTRNG) {
          ua = __ldg(hr + 3 * n + t);
        } else {
          const uint4 r = McRandom::block(seed, m, sweep, pass, 2);
          ua = u53(r.x, r.y);
        }
      }
    }
    // energy change of magex/montecarlo.py:136-147
    const double dx = nx - ox, dy = ny - oy, dz = nz - oz;
    double dE = -2.0 * (dx * hx + dy * hy + dz * hz) - kMuB * mu * (dx * L.B0 + dy * L.B1 + dz * L.B2);
    if (L.has_A) dE += onsite(L, q, s, nx, ny, nz) - onsite(L, q, s, ox, oy, oz);
    if (L.Kc_site) dE += cubic_energy(L, q, nx, ny, nz) - cubic_energy(L, q, ox, oy, oz);
    if (L.K2_site) dE += uniaxial_higher_energy(L, q, nx, ny, nz) - uniaxial_higher_energy(L, q, ox, oy, oz);
    dE += extra;
    const double thr = (MOVE == MC_OVERRELAX) ? 1e-12 : 0.0;
    ok = dE <= thr;
    if (!ok) {
      const double a = dE * bt;
      ok = below_exp(ua, -(a < 700.0 ? a : 700.0));
    }
    if (ok && lane == 0) {
      e[q] = nx;
      e[N + q] = ny;
      e[2 * N + q] = nz;
      if (FIXED) {
        F.es[q] = fx_split<28>(nx);
        F.es[N + q] = fx_split<28>(ny);
        F.es[2 * N + q] = fx_split<28>(nz);
      }
    }
  }
  const int cnt = __syncthreads_count(ok && lane == 0);
  if (MOVE != MC_OVERRELAX && threadIdx.x == 0 && cnt) atomicAdd(acc, (unsigned long long)cnt);
}

// Classes of at most kShareMaxSites sites of stencil FP64 plans with many couplings per site run with
// kShare lanes per site (the choice depends on the class alone, so a chain's trajectory is the same in
// an ensemble and on its own).  Measured on bcc (26 couplings): a single chain gains 2x at every class
// size up to ~1000 sites, a 16-chain ensemble gains 2x at ~60 sites per class, 1.2x at ~200 and
// loses beyond (the lanes repeat the move's arithmetic), so sharing stops at 256.
constexpr long long kShareMaxSites = 256;
constexpr int kShare = 16;

template <int W, int MOVE>
static void launch_pass(const McPlan* mc, double* e, int g, const double* hr, int pass, cudaStream_t st) {
  const DevLattice& L = mc->model->d;
  const long long n = mc->gsize[g];
  if (n == 0) return;
  const long long* sites = mc->sites + mc->goff[g];
  const bool share = mc->share && n <= kShareMaxSites;
  const long long threads = n * (share ? kShare : 1);
  // small classes in small blocks, so that they still spread over the SMs
  const int tpb = threads > 152LL * 128 ? 128 : (threads > 152LL * 64 ? 64 : 32);
  const dim3 grid((unsigned)((threads + tpb - 1) / tpb), (unsigned)mc->nchains);
  if (share) {
    if (hr)
      k_mc_pass<W, MOVE, true, false, kShare><<<grid, tpb, 0, st>>>(L, e, sites, n, mc->beta, mc->beta_site,
                                                                     mc->sigma, hr, mc->seed, mc->sweep, pass,
                                                                     mc->acc, mc->fx, mc->chains);
    else
      k_mc_pass<W, MOVE, false, false, kShare><<<grid, tpb, 0, st>>>(L, e, sites, n, mc->beta, mc->beta_site,
                                                                      mc->sigma, nullptr, mc->seed, mc->sweep,
                                                                      pass, mc->acc, mc->fx, mc->chains);
  } else if (mc->fixed) {
    if (hr)
      k_mc_pass<W, MOVE, true, true, 1><<<grid, tpb, 0, st>>>(L, e, sites, n, mc->beta, mc->beta_site, mc->sigma, hr,
                                                              mc->seed, mc->sweep, pass, mc->acc, mc->fx, mc->chains);
    else
      k_mc_pass<W, MOVE, false, true, 1><<<grid, tpb, 0, st>>>(L, e, sites, n, mc->beta, mc->beta_site, mc->sigma,
                                                               nullptr, mc->seed, mc->sweep, pass, mc->acc, mc->fx,
                                                               mc->chains);
  } else {
    if (hr)
      k_mc_pass<W, MOVE, true, false, 1><<<grid, tpb, 0, st>>>(L, e, sites, n, mc->beta, mc->beta_site, mc->sigma,
                                                               hr, mc->seed, mc->sweep, pass, mc->acc, mc->fx,
                                                               mc->chains);
    else
      k_mc_pass<W, MOVE, false, false, 1><<<grid, tpb, 0, st>>>(L, e, sites, n, mc->beta, mc->beta_site, mc->sigma,
                                                                nullptr, mc->seed, mc->sweep, pass, mc->acc, mc->fx,
                                                                mc->chains);
  }
}

template <int W>
static void launch_move(const McPlan* mc, int move, double* e, int g, const double* hr, int pass, cudaStream_t st) {
  switch (move) {
    case MC_UNIFORM: launch_pass<W, MC_UNIFORM>(mc, e, g, hr, pass, st); break;
    case MC_HEATBATH: launch_pass<W, MC_HEATBATH>(mc, e, g, hr, pass, st); break;
    case MC_HINZKE: launch_pass<W, MC_HINZKE>(mc, e, g, hr, pass, st); break;
    case MC_OVERRELAX: launch_pass<W, MC_OVERRELAX>(mc, e, g, hr, pass, st); break;
    default: launch_pass<W, MC_GAUSSIAN>(mc, e, g, hr, pass, st); break;
  }
}

static void launch_any(const McPlan* mc, int move, double* e, int g, const double* hr, int pass, cudaStream_t st) {
  switch (mc->model->d.width) {
    case 1: launch_move<1>(mc, move, e, g, hr, pass, st); break;
    case 4: launch_move<4>(mc, move, e, g, hr, pass, st); break;
    default: launch_move<9>(mc, move, e, g, hr, pass, st); break;
  }
}

// doubles of host draws for group g in the move pass
static long long move_draws(const McPlan* mc, int g) {
  const long long n = mc->gsize[g];
  const int mv = (mc->move == MC_HEATBATH && !mc->hb_ok[g]) ? MC_GAUSSIAN : mc->move;
  switch (mv) {
    case MC_HEATBATH: return 3 * n;
    case MC_HINZKE: return 8 * n;
    default: return 4 * n;
  }
}

// ------------------------------------------------------------------ host colouring
// First-fit greedy colouring in vertex order (magex/montecarlo.py:35-48): vertex v takes the smallest
// colour not used by an already coloured neighbour.
template <class Nbrs>
static int32_t first_fit(int64_t N, Nbrs nbrs, int32_t* colour) {
  for (int64_t v = 0; v < N; ++v) colour[v] = -1;
  std::vector<int64_t> mark;                  // mark[c] == v: colour c is used around v
  int32_t ncol = 0;
  for (int64_t v = 0; v < N; ++v) {
    nbrs(v, [&](int64_t w) {
      const int32_t c = colour[w];
      if (c >= 0) {
        if ((size_t)c >= mark.size()) mark.resize((size_t)c + 1, -1);
        mark[c] = v;
      }
    });
    int32_t c = 0;
    while ((size_t)c < mark.size() && mark[c] == v) ++c;
    colour[v] = c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  return ncol;
}

// sigma <- clip(sigma * 0.5 / max(1 - a, 0.05), 0.02, 4) with a = accepted / tried, counts reset: the
// arithmetic of magex's adaptation (magex/montecarlo.py:257-261), operation for operation
__global__ void k_mc_adapt(double* __restrict__ sigma, unsigned long long* __restrict__ acc, int n,
                           unsigned long long tried) {
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double a = (double)acc[k] / (double)(tried > 0 ? tried : 1ull);
    const double x = sigma[k] * 0.5 / fmax(1.0 - a, 0.05);
    sigma[k] = fmin(fmax(x, 0.02), 4.0);
    acc[k] = 0;
  }
}

}  // namespace mgx

using namespace mgx;

struct mgx_mc {};

extern "C" mgx_status mgx_colour_stencil(const mgx_lattice_desc* lat, int32_t* colour, int32_t* ncolours) {
  if (!lat || !colour || !ncolours) return set_error(MGX_ERR_INVALID, "mgx_colour_stencil: null argument");
  const int ns = lat->ns, nb = lat->nbond;
  if (ns < 1 || ns > MGX_MAX_SUBLATTICES || nb < 0 || nb > MGX_MAX_BONDS)
    return set_error(MGX_ERR_INVALID, "mgx_colour_stencil: ns %d or nbond %d out of range", ns, nb);
  for (int a = 0; a < 3; ++a)
    if (lat->L[a] < 1) return set_error(MGX_ERR_INVALID, "mgx_colour_stencil: L[%d] = %d", a, lat->L[a]);
  if (nb > 0 && (!lat->bond_src || !lat->bond_dst || !lat->bond_R))
    return set_error(MGX_ERR_INVALID, "mgx_colour_stencil: null bond arrays");
  for (int b = 0; b < nb; ++b)
    if (lat->bond_src[b] < 0 || lat->bond_src[b] >= ns || lat->bond_dst[b] < 0 || lat->bond_dst[b] >= ns)
      return set_error(MGX_ERR_INVALID, "mgx_colour_stencil: bond %d sublattice out of range", b);
  const long long L0 = lat->L[0], L1 = lat->L[1], L2 = lat->L[2];
  const int64_t N = L0 * L1 * L2 * ns;
  // neighbours of v: forward bonds from its sublattice and reverse bonds into it (adj + adj^T)
  auto nbrs = [&](int64_t v, auto&& visit) {
    const int s = (int)(v % ns);
    const long long cell = v / ns;
    const long long c[3] = {cell / (L1 * L2), (cell / L2) % L1, cell % L2};
    const long long Ls[3] = {L0, L1, L2};
    for (int b = 0; b < nb; ++b) {
      for (int dir = 0; dir < 2; ++dir) {
        const int from = dir == 0 ? lat->bond_src[b] : lat->bond_dst[b];
        if (from != s) continue;
        const int to = dir == 0 ? lat->bond_dst[b] : lat->bond_src[b];
        long long t[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
          long long x = c[a] + (dir == 0 ? lat->bond_R[3 * b + a] : -lat->bond_R[3 * b + a]);
          if (lat->pbc[a]) {
            x %= Ls[a];
            if (x < 0) x += Ls[a];
          } else if (x < 0 || x >= Ls[a]) {
            ok = false;
          }
          t[a] = x;
        }
        if (!ok) continue;
        const int64_t w = ((t[0] * L1 + t[1]) * L2 + t[2]) * ns + to;
        if (w != v) visit(w);
      }
    }
  };
  *ncolours = first_fit(N, nbrs, colour);
  return MGX_OK;
}

extern "C" mgx_status mgx_colour_graph(int64_t N, const int64_t* ptr, const int32_t* nbr, int32_t* colour,
                                       int32_t* ncolours) {
  if (N < 0 || !ptr || !colour || !ncolours || (N > 0 && ptr[N] > 0 && !nbr))
    return set_error(MGX_ERR_INVALID, "mgx_colour_graph: bad argument");
  for (int64_t v = 0; v < N; ++v)
    if (ptr[v + 1] < ptr[v]) return set_error(MGX_ERR_INVALID, "mgx_colour_graph: ptr is not monotone at %lld",
                                               (long long)v);
  for (int64_t k = 0; k < ptr[N]; ++k)
    if (nbr[k] < 0 || nbr[k] >= N) return set_error(MGX_ERR_INVALID, "mgx_colour_graph: neighbour %lld out of range",
                                                    (long long)k);
  auto nbrs = [&](int64_t v, auto&& visit) {
    for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k)
      if (nbr[k] != v) visit(nbr[k]);
  };
  *ncolours = first_fit(N, nbrs, colour);
  return MGX_OK;
}

static void mc_free(McPlan* mc) {
  if (!mc) return;
  cudaFree(mc->fx_block);
  cudaFree(mc->sites);
  cudaFree(mc->beta);
  cudaFree(mc->beta_site);
  cudaFree(mc->acc);
  cudaFree(mc->chain_block);
  delete mc;
}

extern "C" mgx_status mgx_mc_create(const mgx_model* mm, const mgx_mc_params* p, const int64_t* group_sites,
                                    const int64_t* group_sizes, int32_t ngroups, mgx_mc** out) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !p || !out || ngroups < 0 || (ngroups > 0 && (!group_sites || !group_sizes)))
    return set_error(MGX_ERR_INVALID, "mgx_mc_create: bad argument");
  if (p->move < MC_GAUSSIAN || p->move > MC_HINZKE)
    return set_error(MGX_ERR_INVALID, "mgx_mc_create: move %d is not gaussian (0), uniform (1), heatbath (2) or "
                                      "hinzke (3)", p->move);
  if (p->overrelax < 0) return set_error(MGX_ERR_INVALID, "mgx_mc_create: overrelax must be >= 0");
  if (p->rng != MGX_MC_RNG_PHILOX && p->rng != MGX_MC_RNG_HOST)
    return set_error(MGX_ERR_INVALID, "mgx_mc_create: rng %d is not philox (0) or host (1)", p->rng);
  if (p->precision != MGX_PRECISION_FP64 && p->precision != MGX_PRECISION_FP64_FIXED_GATHER)
    return set_error(MGX_ERR_INVALID, "mgx_mc_create: precision %d is not fp64 (0) or fp64-fixed-gather (3)",
                     p->precision);
  const DevLattice& d = m->d;
  const long long N = d.N;
  McPlan* mc = new McPlan();
  mc->model = m;
  mc->move = p->move;
  mc->overrelax = p->overrelax;
  mc->rng = p->rng;
  mc->sigma = p->sigma;
  mc->seed = p->seed;
  mc->ngroups = ngroups;
  long long total = 0;
  for (int g = 0; g < ngroups; ++g) {
    if (group_sizes[g] < 0) {
      mc_free(mc);
      return set_error(MGX_ERR_INVALID, "mgx_mc_create: negative group size");
    }
    mc->goff.push_back(total);
    mc->gsize.push_back(group_sizes[g]);
    total += group_sizes[g];
  }
  // magex site index -> lattice index; each site at most once
  std::vector<unsigned char> seen((size_t)N, 0);
  mc->sites_host.resize((size_t)total);
  for (long long k = 0; k < total; ++k) {
    const long long v = group_sites[k];
    if (v < 0 || v >= N || seen[(size_t)v]) {
      mc_free(mc);
      return set_error(MGX_ERR_INVALID, "mgx_mc_create: site %lld out of range or listed twice", v);
    }
    seen[(size_t)v] = 1;
    mc->sites_host[(size_t)k] = (d.layout == 1) ? v : (v % d.ns) * (long long)d.ncell + v / d.ns;
  }
  mc->hb_ok.assign((size_t)ngroups, 1);
  cudaError_t err = cudaMalloc(&mc->sites, sizeof(long long) * (size_t)std::max(total, 1LL));
  if (err == cudaSuccess && total)
    err = cudaMemcpy(mc->sites, mc->sites_host.data(), sizeof(long long) * (size_t)total, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMalloc(&mc->beta, sizeof(double) * MGX_MAX_SUBLATTICES);
  if (err == cudaSuccess) err = cudaMalloc(&mc->acc, sizeof(unsigned long long));
  if (err == cudaSuccess) err = cudaMemset(mc->acc, 0, sizeof(unsigned long long));
  if (err == cudaSuccess) err = cudaMemset(mc->beta, 0, sizeof(double) * MGX_MAX_SUBLATTICES);
  if (err != cudaSuccess) {
    mc_free(mc);
    return cuda_error(err, "mgx_mc_create");
  }
  // many couplings per site (at least 12 per cell and sublattice) on the stencil layout: sites of small
  // classes are shared by kShare lanes
  mc->share = d.layout == 0 && p->precision == MGX_PRECISION_FP64 && m->nbond >= 12 * d.ns;
  if (p->precision == MGX_PRECISION_FP64_FIXED_GATHER) {
    const mgx_status st = fx_build(m, 28, false, 1, &mc->fx, &mc->fx_block);
    if (st != MGX_OK) {
      mc_free(mc);
      return st;
    }
    mc->fixed = true;
  }
  *out = reinterpret_cast<mgx_mc*>(mc);
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_destroy(mgx_mc* h) {
  mc_free(reinterpret_cast<McPlan*>(h));
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_set_beta(mgx_mc* h, const double* beta_sub, const double* beta_site) {
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc || (!beta_sub && !beta_site)) return set_error(MGX_ERR_INVALID, "mgx_mc_set_beta: bad argument");
  const DevLattice& d = mc->model->d;
  const long long N = d.N;
  std::vector<double> bq;
  if (beta_site) {
    bq.resize((size_t)N);
    for (long long v = 0; v < N; ++v) {
      const long long q = (d.layout == 1) ? v : (v % d.ns) * (long long)d.ncell + v / d.ns;
      bq[(size_t)q] = beta_site[v];
    }
    if (!mc->beta_site) MGX_CUDA_TRY(cudaMalloc(&mc->beta_site, sizeof(double) * (size_t)N));
    MGX_CUDA_TRY(cudaMemcpy(mc->beta_site, bq.data(), sizeof(double) * (size_t)N, cudaMemcpyHostToDevice));
  } else {
    MGX_CUDA_TRY(cudaMemcpy(mc->beta, beta_sub, sizeof(double) * d.ns, cudaMemcpyHostToDevice));
    cudaFree(mc->beta_site);
    mc->beta_site = nullptr;
  }
  // heat bath only where every beta of the class is finite, else Gaussian moves (magex/montecarlo.py:191-197)
  for (int g = 0; g < mc->ngroups; ++g) {
    int okg = 1;
    for (long long k = mc->goff[g]; k < mc->goff[g] + mc->gsize[g] && okg; ++k) {
      const long long q = mc->sites_host[(size_t)k];
      int s = (d.layout == 1) ? 0 : (int)(q / d.ncell);
      const double b = beta_site ? bq[(size_t)q] : beta_sub[s];
      okg = std::isfinite(b) ? 1 : 0;
    }
    mc->hb_ok[(size_t)g] = okg;
  }
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_set_sigma(mgx_mc* h, double sigma) {
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc || !(sigma > 0.0)) return set_error(MGX_ERR_INVALID, "mgx_mc_set_sigma: sigma must be positive");
  mc->sigma = sigma;
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_host_draws(const mgx_mc* h, int64_t* ndoubles) {
  const McPlan* mc = reinterpret_cast<const McPlan*>(h);
  if (!mc || !ndoubles) return set_error(MGX_ERR_INVALID, "mgx_mc_host_draws: bad argument");
  long long n = 0;
  for (int g = 0; g < mc->ngroups; ++g) n += move_draws(mc, g) + mc->overrelax * mc->gsize[g];
  *ndoubles = n;
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_sweep(mgx_mc* h, double* e, int64_t nsweeps, const double* host_draws, void* stream) {
  NvtxRange nvtx_range("mgx_mc_sweep");
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc || !e || nsweeps < 0) return set_error(MGX_ERR_INVALID, "mgx_mc_sweep: bad argument");
  if (mc->rng == MGX_MC_RNG_HOST && (nsweeps > 1 || (nsweeps == 1 && !host_draws)))
    return set_error(MGX_ERR_INVALID, "mgx_mc_sweep: host draws cover one sweep per call");
  cudaStream_t st = (cudaStream_t)stream;
  if (mc->fixed && nsweeps > 0) enqueue_fx_split_n(e, mc->fx.es, 3 * mc->model->d.N, 28, st);
  for (int64_t k = 0; k < nsweeps; ++k) {
    const double* hr = mc->rng == MGX_MC_RNG_HOST ? host_draws : nullptr;
    long long off = 0;
    for (int g = 0; g < mc->ngroups; ++g) {
      const int mv = (mc->move == MC_HEATBATH && !mc->hb_ok[(size_t)g]) ? MC_GAUSSIAN : mc->move;
      launch_any(mc, mv, e, g, hr ? hr + off : nullptr, 0, st);
      off += move_draws(mc, g);
      mc->tried += (unsigned long long)mc->gsize[g];
    }
    for (int r = 0; r < mc->overrelax; ++r)
      for (int g = 0; g < mc->ngroups; ++g) {
        launch_any(mc, MC_OVERRELAX, e, g, hr ? hr + off : nullptr, 1 + r, st);
        off += mc->gsize[g];
      }
    MGX_CUDA_TRY(cudaGetLastError());
    ++mc->sweep;
  }
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_counts(mgx_mc* h, uint64_t* accepted, uint64_t* tried, int32_t reset, void* stream) {
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc || !accepted || !tried) return set_error(MGX_ERR_INVALID, "mgx_mc_counts: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long a = 0;
  MGX_CUDA_TRY(cudaMemcpyAsync(&a, mc->acc, sizeof(a), cudaMemcpyDeviceToHost, st));
  MGX_CUDA_TRY(cudaStreamSynchronize(st));
  *accepted = a;
  *tried = mc->tried;
  if (reset) {
    MGX_CUDA_TRY(cudaMemsetAsync(mc->acc, 0, sizeof(unsigned long long), st));
    mc->tried = 0;
  }
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_set_chains(mgx_mc* h, int32_t nchains, const uint64_t* seeds, const double* beta,
                                        const double* sigma) {
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc) return set_error(MGX_ERR_INVALID, "mgx_mc_set_chains: null plan");
  if (nchains < 1 || nchains > 65535) return set_error(MGX_ERR_INVALID, "nchains = %d outside 1..65535", nchains);
  if (nchains == 1 && !seeds && !beta && !sigma) {
    cudaFree(mc->chain_block);
    mc->chain_block = nullptr;
    mc->chains = McChains{};
    mc->nchains = 1;
    mc->tried = 0;
    return MGX_OK;
  }
  if (!seeds || !beta || !sigma) return set_error(MGX_ERR_INVALID, "mgx_mc_set_chains: null array");
  if (mc->rng != MGX_MC_RNG_PHILOX || mc->fixed || mc->beta_site)
    return set_error(MGX_ERR_UNSUPPORTED, "chains need a Philox FP64 plan without site temperatures");
  for (int k = 0; k < nchains; ++k) {
    if (!(beta[k] > 0.0) || !std::isfinite(beta[k]))
      return set_error(MGX_ERR_INVALID, "beta of chain %d must be finite and > 0", k);
    if (!(sigma[k] > 0.0) || !std::isfinite(sigma[k]))
      return set_error(MGX_ERR_INVALID, "sigma of chain %d must be finite and > 0", k);
  }
  const size_t n = (size_t)nchains;
  void* block = nullptr;
  cudaError_t err = cudaMalloc(&block, 32 * n);
  char* b = (char*)block;
  if (err == cudaSuccess) err = cudaMemcpy(b, seeds, 8 * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(b + 8 * n, beta, 8 * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(b + 16 * n, sigma, 8 * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(b + 24 * n, 0, 8 * n);
  if (err != cudaSuccess) {
    cudaFree(block);
    return cuda_error(err, "mgx_mc_set_chains");
  }
  cudaFree(mc->chain_block);
  mc->chain_block = block;
  mc->chains = McChains{(const uint64_t*)b, (const double*)(b + 8 * n), (const double*)(b + 16 * n),
                        (unsigned long long*)(b + 24 * n)};
  mc->nchains = nchains;
  mc->tried = 0;
  mc->hb_ok.assign((size_t)mc->ngroups, 1);          // every beta finite
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_chain_counts(mgx_mc* h, uint64_t* accepted, uint64_t* tried, double* sigma,
                                          int32_t reset, void* stream) {
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc || !accepted || !tried) return set_error(MGX_ERR_INVALID, "mgx_mc_chain_counts: bad argument");
  if (!mc->chain_block) return set_error(MGX_ERR_INVALID, "mgx_mc_chain_counts: no chains set");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)mc->nchains;
  std::vector<unsigned long long> a(n);
  MGX_CUDA_TRY(cudaMemcpyAsync(a.data(), mc->chains.acc, 8 * n, cudaMemcpyDeviceToHost, st));
  if (sigma) MGX_CUDA_TRY(cudaMemcpyAsync(sigma, mc->chains.sigma, 8 * n, cudaMemcpyDeviceToHost, st));
  MGX_CUDA_TRY(cudaStreamSynchronize(st));
  for (size_t k = 0; k < n; ++k) accepted[k] = a[k];
  *tried = mc->tried;
  if (reset) {
    MGX_CUDA_TRY(cudaMemsetAsync(mc->chains.acc, 0, 8 * n, st));
    mc->tried = 0;
  }
  return MGX_OK;
}

extern "C" mgx_status mgx_mc_adapt_sigma(mgx_mc* h, void* stream) {
  McPlan* mc = reinterpret_cast<McPlan*>(h);
  if (!mc) return set_error(MGX_ERR_INVALID, "mgx_mc_adapt_sigma: null plan");
  if (!mc->chain_block) return set_error(MGX_ERR_INVALID, "mgx_mc_adapt_sigma: no chains set");
  mgx::k_mc_adapt<<<1, 256, 0, (cudaStream_t)stream>>>(const_cast<double*>(mc->chains.sigma), mc->chains.acc, mc->nchains,
                                                  (unsigned long long)mc->tried);
  MGX_CUDA_TRY(cudaGetLastError());
  mc->tried = 0;
  return MGX_OK;
}
