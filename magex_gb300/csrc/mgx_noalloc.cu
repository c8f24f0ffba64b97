// mgx_llg_step_noalloc: the stochastic Heun step without any device allocation.
//
// Why it exists: some callers of this library cannot allocate GPU memory when they step the spins.
// A host framework that owns every byte of the device through its own pool allocator and hands a
// plugin only the input and output buffers, or a real-time driver loop that must never block on
// the allocator, needs a step that only reads its inputs and writes its outputs.  mgx_llg_step
// needs a plan from mgx_llg_create, which allocates the predictor scratch (ep and k1, 6 doubles per
// site) with cudaMalloc; this entry point keeps that scratch in one file-scope device array
// instead, allocated by the CUDA runtime when the library's device code is loaded on a GPU and held
// until the process exits.
//
// Rules for callers (also in include/mgx.h):
//   - at most MGX_NOALLOC_MAX_SITES sites; larger models are rejected with MGX_ERR_INVALID;
//   - uniform damping only (params->alpha_site must be NULL);
//   - thermal noise only with one moment per sublattice: a model whose moments differ site by site
//     (per-site mu from a structure edit) needs per-site amplitudes, which only a plan carries, and
//     is rejected with MGX_ERR_UNSUPPORTED unless the noise mode is none;
//   - every call on a device shares the same array: calls whose work overlaps on that GPU (other
//     streams, other host threads) race and must be serialised by the caller;
//   - the first call on a device looks the array's device address up with cudaGetSymbolAddress
//     (with that device current); make that first call before any stream capture begins.
#include <cmath>
#include <mutex>

#include "mgx_internal.cuh"

namespace mgx {

constexpr long long kNoallocMaxSites = MGX_NOALLOC_MAX_SITES;
constexpr int kParamSlots = 3 * MGX_MAX_SUBLATTICES;        // alpha | pre | sigma per sublattice

// [alpha, pre, sigma per sublattice (48 doubles) | pad to 64 | ep (3 N_max) | k1 (3 N_max)]
constexpr long long kNoallocDoubles = 64 + 6 * kNoallocMaxSites;
static __device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

struct SubParams {
  double v[kParamSlots];
};

// Writes the per-sublattice constants into the head of the scratch array (passed by value, so no
// host->device copy and no allocation is needed).
__global__ void k_noalloc_params(double* head, SubParams p, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) head[i] = p.v[i];
}

static std::mutex g_setup_mutex;
static double* g_scratch_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device, looked up once per device.
static mgx_status scratch_address(double** out) {
  int dev = 0;
  MGX_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(MGX_ERR_INVALID, "device ordinal %d outside 0..63", dev);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return cuda_error(err, "cudaGetSymbolAddress(g_noalloc_scratch)");
    if (!p) return set_error(MGX_ERR_CUDA, "cudaGetSymbolAddress returned a null address");
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return MGX_OK;
}

}  // namespace mgx

using namespace mgx;

extern "C" mgx_status mgx_llg_step_noalloc(const mgx_model* mm, const mgx_llg_params* p, const double* sigma_sub,
                                           double* e, const double* noise, uint64_t step, void* stream) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !p || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: null argument");
  const long long N = m->d.N;
  const int ns = m->d.ns;
  if (N > kNoallocMaxSites)
    return set_error(MGX_ERR_INVALID,
                     "mgx_llg_step_noalloc: %lld sites exceed the fixed scratch of %lld sites "
                     "(MGX_NOALLOC_MAX_SITES); use mgx_llg_create / mgx_llg_step for larger models",
                     N, kNoallocMaxSites);
  if (p->alpha_site)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: per-site damping (alpha_site) needs a plan; "
                                      "pass a uniform alpha");
  if (p->precision != MGX_PRECISION_FP64)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: only the FP64 gather (precision 0) is available");
  if (!(p->dt > 0.0) || !std::isfinite(p->dt)) return set_error(MGX_ERR_INVALID, "dt must be a positive number");
  if (!std::isfinite(p->alpha) || p->alpha < 0.0)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: alpha must be finite and >= 0");
  if (p->integrator != MGX_INTEGRATOR_HEUN && p->integrator != MGX_INTEGRATOR_DEPONDT)
    return set_error(MGX_ERR_INVALID, "integrator %d is not heun (0) or depondt (1)", p->integrator);
  if (p->noise < MGX_NOISE_NONE || p->noise > MGX_NOISE_PHILOX)
    return set_error(MGX_ERR_INVALID, "noise mode %d is not none (0), host (1) or philox (2)", p->noise);
  if (p->noise == MGX_NOISE_HOST && !noise)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: host-noise mode needs a noise buffer");
  if (p->noise != MGX_NOISE_NONE && !sigma_sub)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: thermal noise needs sigma_sub");
  if (p->noise != MGX_NOISE_NONE && m->d.inv_mu_site)
    return set_error(MGX_ERR_UNSUPPORTED,
                     "mgx_llg_step_noalloc: the model's moments differ site by site, so the thermal amplitude "
                     "does too; per-site amplitudes need a plan (mgx_llg_create + mgx_llg_set_sigma)");
  if (p->noise != MGX_NOISE_NONE)
    for (int s = 0; s < ns; ++s)
      if (!std::isfinite(sigma_sub[s]) || sigma_sub[s] < 0.0)
        return set_error(MGX_ERR_INVALID, "mgx_llg_step_noalloc: sigma_sub must be finite and >= 0");

  double* base = nullptr;
  mgx_status st = scratch_address(&base);
  if (st != MGX_OK) return st;

  SubParams sp;
  const double gamma = 0.1760859630;
  for (int k = 0; k < kParamSlots; ++k) sp.v[k] = 0.0;
  for (int s = 0; s < ns; ++s) {
    sp.v[s] = p->alpha;
    sp.v[ns + s] = -gamma / (1.0 + p->alpha * p->alpha);
    sp.v[2 * ns + s] = (p->noise != MGX_NOISE_NONE) ? sigma_sub[s] : 0.0;
  }
  cudaStream_t cs = (cudaStream_t)stream;
  k_noalloc_params<<<1, 64, 0, cs>>>(base, sp, 3 * ns);
  MGX_CUDA_TRY(cudaGetLastError());

  LLGPlan view;                        // host-side descriptor only; owns nothing
  view.model = m;
  view.sigma_zero = true;
  for (int s = 0; s < ns; ++s) view.sigma_zero &= sp.v[2 * ns + s] == 0.0;
  DevLLG& d = view.p;
  d.dt = p->dt;
  d.half_dt = 0.5 * p->dt;
  d.precession = p->precession ? 1 : 0;
  d.noise = p->noise;
  d.integrator = p->integrator;
  d.seed = p->seed;
  d.alpha_sub = base;
  d.pre_sub = base + ns;
  d.sigma_sub = base + 2 * ns;
  d.alpha_site = d.pre_site = d.sigma_site = nullptr;
  d.ep = base + 64;                    // the predictor writes every site of ep and k1 before the
  d.k1 = base + 64 + 3 * N;            // corrector reads them, so no clearing is needed
  enqueue_llg_step(&view, e, noise, step, cs, 3);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}
