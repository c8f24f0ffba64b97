// Internal declarations shared by the translation units of libmgx (GB300, sm_103a).
//
// Device data layout ("lattice layout"): for a supercell of ncell = L0*L1*L2 cells and ns
// sublattices, site (s, cell) has lattice index q = s*ncell + cell and component c of a spin field
// lives at x[c*N + q].  Threads of a warp therefore read consecutive cells of one sublattice, and
// a neighbour at a fixed cell offset is again a consecutive run: every gather load is coalesced.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/mgx.h"

namespace mgx {

// ------------------------------------------------------------------ error reporting (host)
mgx_status set_error(mgx_status code, const char* fmt, ...);
mgx_status cuda_error(cudaError_t err, const char* where);

#define MGX_CUDA_TRY(call)                                   \
  do {                                                       \
    cudaError_t err__ = (call);                              \
    if (err__ != cudaSuccess) return ::mgx::cuda_error(err__, #call); \
  } while (0)

// ------------------------------------------------------------------ device-side lattice view
struct DevLattice {
  int ns;
  int L0, L1, L2;
  int ncell;
  long long N;
  int pbc0, pbc1, pbc2;
  int width;                     // 1, 4 or 9 doubles per coupling
  const int* bond_off;           // [ns+1] range of couplings per receiving sublattice
  const int4* bond_geo;          // [nbond] (dst sublattice, d0, d1, d2); d = R mod L if periodic else R
  const double* bond_J;          // [nbond*width]
  int has_A;
  const double* A_sub;           // [ns*9]
  const double* inv_mu_sub;      // [ns] 1/(mu mu_B)
  const double* mu_sub;          // [ns]
  const double* sign_sub;        // [ns]
  const double* A_site;          // [9][N] lattice layout, or nullptr
  const double* inv_mu_site;     // [N] or nullptr
  const double* mu_site;         // [N] or nullptr
  const uint8_t* pinned;         // [N] or nullptr
  double B0, B1, B2;
  // neighbour-list layout (arbitrary lattices): ns = 1, ncell = N, site q has couplings
  // csr_ptr[q] .. csr_ptr[q+1] to csr_nbr[k] with tensor bond_J[csr_typ[k]]
  int layout;                    // 0 stencil, 1 csr
  const long long* csr_ptr;      // [N+1]
  const int* csr_nbr;            // [nnz]
  const int* csr_typ;            // [nnz]
  const double* sign_site;       // [N] order-parameter signs, or nullptr
  // slab of a larger supercell (mgx_model_set_partition): Philox counters use cell + cell_offset as
  // the cell of the whole lattice; observables sum only cells with own0_begin <= c0 < own0_end
  long long cell_offset;
  int own0_begin, own0_end;
  // cubic anisotropy E = Kc (a1^2 a2^2 + a2^2 a3^2 + a3^2 a1^2), a = C e (magex/terms.py:35-55), and
  // higher uniaxial anisotropy E = -K2 (e.u)^4 - K3 (e.u)^6 (magex/terms.py:58-75): per-site
  // constants in the lattice layout, nullptr when the model has none
  const double* Kc_site;         // [N] or nullptr
  const double* K2_site;         // [N] or nullptr (with K3_site)
  const double* K3_site;         // [N]
  double C[9];                   // cubic axes, rows
  double u[3];                   // uniaxial axis (unit)
};

struct Model {
  DevLattice d;
  int nbond;
  // device allocations owned by the model
  void* dev_block = nullptr;     // tables and per-sublattice constants
  double* A_site = nullptr;
  double* inv_mu_site = nullptr;
  double* mu_site = nullptr;
  uint8_t* pinned = nullptr;
  double* higher_site = nullptr; // Kc | K2 | K3 (lattice layout) of the higher on-site terms
  double* partials = nullptr;    // reduction scratch for observables
  int partial_cap = 0;           // number of 8-double slots
  int* slot_of_bond = nullptr;   // host [nbond]: position of input coupling b in the device table
  void* csr_block = nullptr;     // ptr | nbr | typ (neighbour-list layout)
  double* sign_site = nullptr;
  int reach0 = -1;               // largest |R_0| of a coupling in layers (stencil layout), -1 for the list layout
};

// ------------------------------------------------------------------ LLG plan (mgx_llg.cu)
struct DevLLG {
  double dt, half_dt;
  int precession;
  int noise;
  int integrator;
  uint64_t seed;
  const double* alpha_sub;   // [ns]
  const double* pre_sub;     // [ns]  -gamma / (1 + alpha^2)
  const double* sigma_sub;   // [ns]
  const double* alpha_site;  // [N] or nullptr
  const double* pre_site;    // [N] or nullptr
  const double* sigma_site;  // [N] or nullptr
  double* ep;                // [3][N] predicted spins
  double* k1;                // [3][N] predictor slope (Heun) or rotation rate (Depondt)
  // CUDA-graph replays: the Philox step index is *step_base + the launch's step argument
  const unsigned long long* step_base = nullptr;
  // caller-supplied per-site field added to the effective field of both stages ([3][N], lattice
  // layout; mgx_llg_set_extra_field), or nullptr
  const double* B_add = nullptr;
  // spin-orbit torque as effective fields B_DL e x p + B_FL p (mgx_llg_set_sot): device
  // [p0, p1, p2, B_DL, B_FL], or nullptr
  const double* sot = nullptr;
};

// Tables of the compensated-FP32 gather (MGX_PRECISION_DF32_GATHER): every coupling as 9 (hi, lo)
// float pairs pre-scaled by 2 / (mu mu_B) of the receiving sublattice, -2 A / (mu mu_B) per
// sublattice, and the (hi, lo) copies of the spin fields that the gather reads.
struct DevDF {
  const float4* J;               // [nbond*5]: the 9 (hi, lo) pairs of a coupling padded to 10 (80 B)
  const int2* lin;               // [nbond] (linear offset of the neighbour of an interior cell, signed R2)
  int4 reach[MGX_MAX_SUBLATTICES];  // per receiving sublattice: max |R| along each axis
  float2 alpha[MGX_MAX_SUBLATTICES], pre[MGX_MAX_SUBLATTICES], sig[MGX_MAX_SUBLATTICES];  // (hi, lo) splits
  float2 B[3];                   // (hi, lo) split of the external field, refreshed at every launch
  const float2* nA2f;            // [ns*9] (hi, lo) split of nA2
  const double* nA2;             // [ns*9]
  int hasA, diagA;
  float2* es;                    // [3][N] split of e
  float2* eps;                   // [3][N] split of ep
};

// Tables of the fixed-point integer gather (MGX_PRECISION_INT48_GATHER): couplings and on-site
// tensors as 48-bit fixed-point numbers in two balanced int32 halves (v = hi 2^24 + lo, |lo| <= 2^23)
// at a per-sublattice power-of-two scale, and the fixed-point copies of the spin fields.
struct DevFX {
  const int4* J;                 // [nbond*5]: 9 (hi, lo) pairs of a coupling padded to 10 (80 B)
  const int4* A;                 // [ns*5]: -2 A / (mu mu_B) in the same format, or nullptr
  const int2* lin;               // [nbond] (linear offset of the neighbour of an interior cell, signed R2)
  int4 reach[MGX_MAX_SUBLATTICES];
  double scale[MGX_MAX_SUBLATTICES];  // 2^(sigma_s - 2 limb): value of one unit of the accumulator
  int scale_exp[MGX_MAX_SUBLATTICES];  // sigma_s - 2 limb (the same scale as a power of two)
  float2 alpha[MGX_MAX_SUBLATTICES], pre[MGX_MAX_SUBLATTICES], sig[MGX_MAX_SUBLATTICES];
  float2 B[3];                   // (hi, lo) split of the external field, refreshed at every launch
  // 1: the conversions between the fixed-point values and FP64 (and of the FP32 noise draws) use the
  // hardware converters, which run on the FP64 pipe; 0: exact bit manipulation on the integer pipes.
  // Set by fx_build from the couplings per site: where there are many, the integer pipes are the
  // busier side and the FP64 pipe has room (bcc 128^3, 26 couplings: 1.089 -> 1.071 ms per step);
  // where there are few, the FP64 pipe is (triangular film 2048^2, 6 couplings: 0.697 -> 0.840 ms
  // with every conversion on the hardware), and so it is with the cubic / higher-uniaxial terms.
  // Read at run time by the single-lattice kernels only (fx_hw<2>).
  int hw_convert;
  // [3][N] the FP32 normal draws of the current step (Philox noise, the five-block single-lattice stage
  // kernels): the predictor stores them and the corrector reads them back instead of drawing them again
  float* nz;
  int2* es;                      // [3][N] fixed-point split of e
  int2* eps;                     // [3][N] fixed-point split of ep
};

// Axis-0 slabs a host-buffer step is split into (copies of one overlap the stages of another).
#define MGX_HOST_CHUNKS 32
#define MGX_LLG_GRAPHS 4

// one captured loop of `steps` Heun steps, valid for the spin buffer, noise mode, external field and
// cell offset it was captured with (kernel parameters are captured by value)
struct LLGGraph {
  cudaGraphExec_t exec = nullptr;
  int steps = 0, mode = -1;
  const double* e = nullptr;
  double B[3] = {0.0, 0.0, 0.0};
  long long offset = 0;
  unsigned long long used = 0;
};

struct LLGPlan {
  const Model* model;
  DevLLG p;
  bool sigma_zero = true;        // every thermal amplitude is 0: the noise-free kernels are used
  int precision = 0;
  DevDF df{};
  void* df_block = nullptr;
  DevFX fx{};
  void* fx_block = nullptr;
  float* fx_noise = nullptr;     // DevFX::nz of the 56-bit plans
  void* sub_block = nullptr;     // alpha_sub | pre_sub | sigma_sub
  double* site_block = nullptr;  // alpha_site | pre_site
  double* sigma_site = nullptr;
  double* scratch = nullptr;     // ep | k1
  // captured step loops of mgx_llg_run (small lattices, where launches dominate): a few graphs of
  // different step counts, the least recently used one replaced
  cudaStream_t cap_stream = nullptr;
  LLGGraph graphs[MGX_LLG_GRAPHS];
  unsigned long long graph_clock = 0;
  long long last_tail = -1;      // step count of the previous call's ungraphed tail
  unsigned long long* d_step = nullptr;
  // step on host buffers (mgx_llg_step_host): device copies of the spins, the copy stream (copies in)
  // and a second compute stream (consecutive slabs run on alternate streams so each fills the other's
  // tail), a pack stream (the copies in run back to back on the copy stream while each landed slab is
  // packed into the lattice layout), two corrector streams (the corrector of a slab starts once the
  // predictors of the slabs it gathers from are done, while the predictors of later slabs still run)
  // and an out stream (each finished slab goes back to the host while the copies in still run: the
  // two directions overlap)
  cudaStream_t copy_stream = nullptr, aux_stream = nullptr, pack_stream = nullptr, out_stream = nullptr;
  cudaStream_t corr_stream[2] = {nullptr, nullptr};
  double* host_lat = nullptr;    // [3][N] lattice layout
  double* host_aos = nullptr;    // [N][3] magex order (staging of the copies)
  // in[c] (packed) | out[c] (corrected) | copied[c] | predicted[c] | start | done | joined aux | joined out
  cudaEvent_t host_ev[4 * MGX_HOST_CHUNKS + 4] = {};
  // the slab pipeline of a host-buffer step captured as a graph (step index from d_step), for the
  // last two (input, output) buffer pairs: replaying it costs one launch instead of ~250 API calls
  LLGGraph host_graphs[2];
  const double* host_in[2] = {nullptr, nullptr};
  const double* host_noise[2] = {nullptr, nullptr};
  double* sot_block = nullptr;   // device [5] spin-orbit torque parameters
};

// Threads per block of the one-site-per-thread kernels: 256, or fewer for small lattices so that the
// grid still spreads over every SM (a 16k-site film gives 256 blocks of 64 instead of 64 of 256).
inline int site_block_size(long long N) {
  if (N >= 152LL * 8 * 256) return 256;
  if (N >= 152LL * 4 * 128) return 128;
  return 64;
}

// (hi, lo) float pair of a double: hi = float(x), lo = float(x - hi)
inline float2 split_host(double x) {
  const float hi = (float)x;
  return make_float2(hi, (float)(x - (double)hi));
}

// magex-order (N, 3) rows [begin, begin + count) to / from the lattice layout, on st (mgx_model.cu).
void enqueue_pack(const Model* m, const double* aos, double* lat, long long begin, long long count, cudaStream_t st);
void enqueue_unpack(const Model* m, const double* lat, double* aos, long long begin, long long count, cudaStream_t st);
// Enqueue the predictor (stages & 1) and / or the corrector (stages & 2) of one step on st.
void enqueue_llg_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages);
// Compensated-FP32 gather form (mgx_llg_df.cu): tables built at plan creation, the split copy of e
// refreshed at the start of every library call, then predictor / corrector as above.
mgx_status build_df_tables(LLGPlan* pl);
void enqueue_df_split(const LLGPlan* pl, const double* e, cudaStream_t st);
void enqueue_df_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages);
// Fixed-point integer gather form (mgx_llg_fx.cu), organised the same way.
mgx_status build_fx_tables(LLGPlan* pl);
void enqueue_fx_split(const LLGPlan* pl, const double* e, cudaStream_t st);
void enqueue_fx_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages);
// The same stages on cells [cb, cb + cn) of every sublattice (the slabs of mgx_llg_step_host); with
// `rows` the corrector writes the new spins of those cells to the magex-order (N, 3) rows only.  The
// fused packing of magex-order rows [begin, begin + count) into e and its fixed-point split.
void enqueue_fx_range(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st, int stages,
                      long long cb, long long cn, double* rows = nullptr);
void enqueue_fx_pack_split(const LLGPlan* pl, const double* rows, double* lat, long long begin, long long count,
                           cudaStream_t st);

// Host-side NVTX range over one library call (named in profiler timelines; a no-op without a tool).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// ------------------------------------------------------------------ small device helpers
__device__ __forceinline__ void site_coords(const DevLattice& L, long long q, int& s, int& c0, int& c1, int& c2) {
  s = (int)(q / L.ncell);
  int cell = (int)(q - (long long)s * L.ncell);
  c2 = cell % L.L2;
  int t = cell / L.L2;
  c1 = t % L.L1;
  c0 = t / L.L1;
}

// Exchange field h = sum_j J_ij x_j at site (s, c0, c1, c2) of field x (lattice layout).
// Couplings whose neighbour lies outside an open boundary are skipped, as magex drops them
// when it builds the supercell (magex/spinmodel.py:218-223).
template <int W>
__device__ __forceinline__ void exchange_field(const DevLattice& L, const double* __restrict__ x, int s, int c0,
                                               int c1, int c2, double& hx, double& hy, double& hz) {
  hx = 0.0;
  hy = 0.0;
  hz = 0.0;
  const long long N = L.N;
  if (L.layout == 1) {
    // per-site neighbour list (magex/fast.py:87-120 layout): q = c2 when ns = 1 and ncell = N
    const long long q = c2;
    const long long k1 = __ldg(L.csr_ptr + q + 1);
    for (long long k = __ldg(L.csr_ptr + q); k < k1; ++k) {
      const long long j = __ldg(L.csr_nbr + k);
      const double ex = __ldg(x + j), ey = __ldg(x + N + j), ez = __ldg(x + 2 * N + j);
      const double* T = L.bond_J + (long long)__ldg(L.csr_typ + k) * W;
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
    return;
  }
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
    const double ex = __ldg(x + j), ey = __ldg(x + N + j), ez = __ldg(x + 2 * N + j);
    const double* T = L.bond_J + (long long)b * W;
    if (W == 1) {
      const double J = __ldg(T);
      hx = fma(J, ex, hx);
      hy = fma(J, ey, hy);
      hz = fma(J, ez, hz);
    } else if (W == 4) {
      // J e_j + e_j x D  (antisymmetric part with e_i.J^A.e_j = D.(e_i x e_j)), magex/fast.py:102-111
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

// Effective field B = (2h - dE_onsite/de) / (mu mu_B) + B_ext (T) at lattice index q with spin (x,y,z):
// magex/fast.py:309-317 and magex/spinmodel.py:458-473 (dE/de of e.A.e is 2 A e).
template <int W>
__device__ __forceinline__ void effective_field(const DevLattice& L, const double* __restrict__ x, long long q, int s,
                                                int c0, int c1, int c2, double ex, double ey, double ez,
                                                double& bx, double& by, double& bz) {
  double hx, hy, hz;
  exchange_field<W>(L, x, s, c0, c1, c2, hx, hy, hz);
  double gx = 0.0, gy = 0.0, gz = 0.0;
  if (L.has_A) {
    double a[9];
    if (L.A_site) {
#pragma unroll
      for (int k = 0; k < 9; ++k) a[k] = __ldg(L.A_site + (long long)k * L.N + q);
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) a[k] = __ldg(L.A_sub + s * 9 + k);
    }
    gx = 2.0 * fma(a[0], ex, fma(a[1], ey, a[2] * ez));
    gy = 2.0 * fma(a[3], ex, fma(a[4], ey, a[5] * ez));
    gz = 2.0 * fma(a[6], ex, fma(a[7], ey, a[8] * ez));
  }
  const double inv = L.inv_mu_site ? __ldg(L.inv_mu_site + q) : __ldg(L.inv_mu_sub + s);
  bx = fma(fma(2.0, hx, -gx), inv, L.B0);
  by = fma(fma(2.0, hy, -gy), inv, L.B1);
  bz = fma(fma(2.0, hz, -gz), inv, L.B2);
}

inline bool has_higher_onsite(const DevLattice& L) { return L.Kc_site || L.K2_site; }

// energies of the cubic and the higher uniaxial term at site q (magex/terms.py:41-43,61-63)
__device__ __forceinline__ double cubic_energy(const DevLattice& L, long long q, double x, double y, double z) {
  const double a1 = L.C[0] * x + L.C[1] * y + L.C[2] * z;
  const double a2 = L.C[3] * x + L.C[4] * y + L.C[5] * z;
  const double a3 = L.C[6] * x + L.C[7] * y + L.C[8] * z;
  const double q1 = a1 * a1, q2 = a2 * a2, q3 = a3 * a3;
  return L.Kc_site[q] * (q1 * q2 + q2 * q3 + q3 * q1);
}

__device__ __forceinline__ double uniaxial_higher_energy(const DevLattice& L, long long q, double x, double y,
                                                         double z) {
  const double c = x * L.u[0] + y * L.u[1] + z * L.u[2];
  const double c2 = c * c;
  return -L.K2_site[q] * c2 * c2 - L.K3_site[q] * c2 * c2 * c2;
}

// dE/de of the higher on-site terms at site q (magex/fast.py:39-64 order: cubic, then uniaxial)
__device__ __forceinline__ void higher_onsite_grad(const DevLattice& L, long long q, double x, double y, double z,
                                                   double& gx, double& gy, double& gz) {
  // every rounding explicit (fma, or __dmul_rn / __dadd_rn where nothing may be fused), so that each
  // kernel that inlines this gives the same bits whatever the compiler fuses around it
  gx = gy = gz = 0.0;
  const double* C = L.C;
  if (L.Kc_site) {
    const double a1 = fma(C[0], x, fma(C[1], y, __dmul_rn(C[2], z)));
    const double a2 = fma(C[3], x, fma(C[4], y, __dmul_rn(C[5], z)));
    const double a3 = fma(C[6], x, fma(C[7], y, __dmul_rn(C[8], z)));
    const double q1 = __dmul_rn(a1, a1), q2 = __dmul_rn(a2, a2), q3 = __dmul_rn(a3, a3);
    const double kc2 = __dmul_rn(2.0, L.Kc_site[q]);
    const double d1 = __dmul_rn(__dmul_rn(kc2, a1), __dadd_rn(q2, q3));
    const double d2 = __dmul_rn(__dmul_rn(kc2, a2), __dadd_rn(q1, q3));
    const double d3 = __dmul_rn(__dmul_rn(kc2, a3), __dadd_rn(q1, q2));
    gx = fma(d3, C[6], fma(d2, C[3], __dmul_rn(d1, C[0])));
    gy = fma(d3, C[7], fma(d2, C[4], __dmul_rn(d1, C[1])));
    gz = fma(d3, C[8], fma(d2, C[5], __dmul_rn(d1, C[2])));
  }
  if (L.K2_site) {
    const double* u = L.u;
    const double c = fma(x, u[0], fma(y, u[1], __dmul_rn(z, u[2])));
    const double c2 = __dmul_rn(c, c), c3 = __dmul_rn(c2, c);
    const double f = fma(__dmul_rn(-4.0, L.K2_site[q]), c3, __dmul_rn(__dmul_rn(-6.0, L.K3_site[q]), __dmul_rn(c2, c3)));
    gx = fma(f, u[0], gx);
    gy = fma(f, u[1], gy);
    gz = fma(f, u[2], gz);
  }
}

// B -= dE_higher/de / (mu mu_B) at site q of sublattice s
__device__ __forceinline__ void add_higher_onsite(const DevLattice& L, long long q, int s, double x, double y,
                                                  double z, double& bx, double& by, double& bz) {
  if (!L.Kc_site && !L.K2_site) return;
  double gx, gy, gz;
  higher_onsite_grad(L, q, x, y, z, gx, gy, gz);
  const double inv = L.inv_mu_site ? L.inv_mu_site[q] : L.inv_mu_sub[s];
  bx = fma(-gx, inv, bx);
  by = fma(-gy, inv, by);
  bz = fma(-gz, inv, bz);
}

// LLG right-hand side f = pre [e x B + alpha e x (e x B)], pre = -gamma / (1 + alpha^2)
// (magex/llg.py:21-28, magex/fast.py:225-236); precession=false drops the e x B term.
__device__ __forceinline__ void llg_rhs(double ex, double ey, double ez, double bx, double by, double bz, double a,
                                        double pre, bool precession, double& fx, double& fy, double& fz) {
  const double cx = ey * bz - ez * by;
  const double cy = ez * bx - ex * bz;
  const double cz = ex * by - ey * bx;
  const double dx = ey * cz - ez * cy;
  const double dy = ez * cx - ex * cz;
  const double dz = ex * cy - ey * cx;
  if (precession) {
    fx = pre * fma(a, dx, cx);
    fy = pre * fma(a, dy, cy);
    fz = pre * fma(a, dz, cz);
  } else {
    fx = pre * (a * dx);
    fy = pre * (a * dy);
    fz = pre * (a * dz);
  }
}

// ------------------------------------------------------------------ Philox4x32-10 (Salmon et al., SC'11)
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

// Three N(0,1) draws for (site, step) by Box-Muller on one Philox block.  The draws are computed
// in fp32 (their statistical quality, not their rounding, matters) and widened to fp64.
// ------------------------------------------------------------------ exact conversions on the integer pipes
// GB300 runs FP64-width conversions (I2F.F64, F2I.F64, F2F.F64) on its FP64 pipe, 16 cycles per warp
// instruction like a DFMA.  These do the same conversions with integer instructions on the bit
// patterns (IEEE 754 binary32 / binary64), with the same rounding (to nearest, ties to even).

// float -> double, exactly (normal floats by moving exponent and mantissa; zero and subnormals, which
// a Box-Muller draw almost never yields, through the hardware conversion)
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int ex = (b >> 23) & 0xFFu;
  if (ex == 0u || ex == 0xFFu) return (double)f;
  const unsigned long long bits = ((unsigned long long)(b >> 31) << 63) | ((unsigned long long)(ex + 896u) << 52) |
                                  ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}

// (double)t * 2^e2 rounded to nearest even, for |t| < 2^63 and a normal result
__device__ __forceinline__ double ll_to_double_scaled(long long t, int e2) {
  if (t == 0) return 0.0;
  const unsigned long long sgn = t < 0 ? (1ULL << 63) : 0ULL;
  const unsigned long long a = t < 0 ? 0ULL - (unsigned long long)t : (unsigned long long)t;
  int msb = 63 - __clzll((long long)a);
  unsigned long long m;
  if (msb <= 52) {
    m = a << (52 - msb);
  } else {
    const int sh = msb - 52;
    m = a >> sh;
    const unsigned long long rem = a & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    m += (rem > half || (rem == half && (m & 1ULL))) ? 1ULL : 0ULL;
    if (m >> 53) {
      m >>= 1;
      ++msb;
    }
  }
  return __longlong_as_double(
      (long long)(sgn | ((unsigned long long)(msb + e2 + 1023) << 52) | (m & ((1ULL << 52) - 1))));
}

// round(x * 2^k) to nearest even, for |x 2^k| < 2^62 (the fixed-point spins: |x| <= 1 + 2^-52)
__device__ __forceinline__ long long double_to_ll_scaled(double x, int k) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((u >> 52) & 0x7FF);
  if (E == 0) return 0;                                  // zero or subnormal: |x 2^k| < 1/2
  const unsigned long long m = (u & ((1ULL << 52) - 1)) | (1ULL << 52);
  const int sh = E - 1075 + k;                           // |x 2^k| = m 2^sh
  unsigned long long v;
  if (sh >= 0) {
    v = m << sh;
  } else if (sh < -54) {
    v = 0;
  } else {
    const int r = -sh;
    const unsigned long long q = m >> r, rem = m & ((1ULL << r) - 1), half = 1ULL << (r - 1);
    v = q + ((rem > half || (rem == half && (q & 1ULL))) ? 1ULL : 0ULL);
  }
  return (u >> 63) ? -(long long)v : (long long)v;
}

// three standard normal FP32 draws of (seed, site, step): one Philox block, Box-Muller in FP32
__device__ __forceinline__ void philox_normal3f(uint64_t seed, uint64_t site, uint64_t step, float& f0, float& f1,
                                                float& f2) {
  const uint4 r = philox4x32_10(make_uint4((uint32_t)site, (uint32_t)(site >> 32), (uint32_t)step,
                                           (uint32_t)(step >> 32)),
                                make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  const float tw = 2.3283064365386963e-10f;                 // 2^-32
  const float u1 = fmaf((float)r.x, tw, 0.5f * tw);          // (0, 1]
  const float u3 = fmaf((float)r.z, tw, 0.5f * tw);
  const float v1 = (float)r.y * tw, v3 = (float)r.w * tw;    // [0, 1)
  const float m1 = sqrtf(-2.0f * logf(u1));
  const float m3 = sqrtf(-2.0f * logf(u3));
  float s1, c1;
  sincospif(2.0f * v1, &s1, &c1);
  f0 = m1 * c1;
  f1 = m1 * s1;
  f2 = m3 * cospif(2.0f * v3);
}

// the same draws in FP64 (exact); hw: widened by the hardware conversion instead of on the integer
// pipes (the same values)
__device__ __forceinline__ void philox_normal3(uint64_t seed, uint64_t site, uint64_t step, double& g0, double& g1,
                                               double& g2, bool hw = false) {
  float f0, f1, f2;
  philox_normal3f(seed, site, step, f0, f1, f2);
  g0 = hw ? (double)f0 : f32_to_f64(f0);
  g1 = hw ? (double)f1 : f32_to_f64(f1);
  g2 = hw ? (double)f2 : f32_to_f64(f2);
}

}  // namespace mgx
