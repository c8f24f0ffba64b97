// Fused stochastic Heun (and Depondt) LLG step on the lattice stencil: predictor and corrector kernels.
//
// Reference behaviour: magex/llg.py:216-227 (NumPy Heun), magex/fast.py:336-390 (fused predictor /
// corrector, numba), magex/cuda_backend.py:144-218 (numba.cuda twins).  One thread owns one site.
// The predictor gathers the exchange field from e, adds on-site, Zeeman and thermal fields, stores
// k1 and the normalised predicted spin ep; the corrector gathers from ep and writes e in place
// (it reads only its own e, so the in-place update is race-free).
#include <cmath>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx {

// magex site number of lattice index q (layout-independent Philox counter)
__device__ __forceinline__ uint64_t magex_site(const DevLattice& L, long long q, int s) {
  return (uint64_t)(q - (long long)s * L.ncell) * (uint64_t)L.ns + (uint64_t)s;
}

// Rodrigues rotation of (x,y,z) by the rotation vector w (angle |w|), magex/fast.py:271-282
__device__ __forceinline__ void rotate(double& x, double& y, double& z, double wx, double wy, double wz) {
  const double th = sqrt(wx * wx + wy * wy + wz * wz);
  if (th < 1e-14) return;
  const double kx = wx / th, ky = wy / th, kz = wz / th;
  double s, c;
  sincos(th, &s, &c);
  const double kd = kx * x + ky * y + kz * z;
  const double cx = ky * z - kz * y, cy = kz * x - kx * z, cz = kx * y - ky * x;
  const double omc = 1.0 - c;
  const double nx = x * c + cx * s + kx * kd * omc;
  const double ny = y * c + cy * s + ky * kd * omc;
  const double nz = z * c + cz * s + kz * kd * omc;
  x = nx;
  y = ny;
  z = nz;
}

template <int NOISE>
__device__ __forceinline__ void add_thermal(const DevLattice& L, const DevLLG& P, const double* __restrict__ noise,
                                            long long q, int s, uint64_t step, double& bx, double& by, double& bz) {
  if (NOISE == MGX_NOISE_NONE) return;
  const double sig = P.sigma_site ? __ldg(P.sigma_site + q) : __ldg(P.sigma_sub + s);
  double g0, g1, g2;
  if (NOISE == MGX_NOISE_HOST) {
    g0 = __ldg(noise + q);
    g1 = __ldg(noise + L.N + q);
    g2 = __ldg(noise + 2 * L.N + q);
  } else {
    philox_normal3(P.seed, magex_site(L, q, s), step, g0, g1, g2);
  }
  bx = fma(sig, g0, bx);
  by = fma(sig, g1, by);
  bz = fma(sig, g2, bz);
}

template <int W, int NOISE, int INTEG>
__global__ void __launch_bounds__(256) k_predict(const DevLattice L, const DevLLG P, const double* __restrict__ e,
                                                 const double* __restrict__ noise, uint64_t step) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const long long N = L.N;
  const double ex = e[q], ey = e[N + q], ez = e[2 * N + q];
  if (L.pinned && L.pinned[q]) {
    P.ep[q] = ex; P.ep[N + q] = ey; P.ep[2 * N + q] = ez;
    P.k1[q] = 0.0; P.k1[N + q] = 0.0; P.k1[2 * N + q] = 0.0;
    return;
  }
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double bx, by, bz;
  effective_field<W>(L, e, q, s, c0, c1, c2, ex, ey, ez, bx, by, bz);
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
  const double a = P.alpha_site ? __ldg(P.alpha_site + q) : __ldg(P.alpha_sub + s);
  const double pre = P.pre_site ? __ldg(P.pre_site + q) : __ldg(P.pre_sub + s);
  double fx, fy, fz;
  llg_rhs(ex, ey, ez, bx, by, bz, a, pre, P.precession != 0, fx, fy, fz);
  if (INTEG == MGX_INTEGRATOR_DEPONDT) {
    // rotation rate w = e x f (de/dt = w x e for a tangent f); the rotated predictor is used
    // without renormalisation, as magex/fast.py:284-288,359-362 and magex/llg.py:237-238
    const double wx = ey * fz - ez * fy, wy = ez * fx - ex * fz, wz = ex * fy - ey * fx;
    double x = ex, y = ey, z = ez;
    rotate(x, y, z, P.dt * wx, P.dt * wy, P.dt * wz);
    P.ep[q] = x; P.ep[N + q] = y; P.ep[2 * N + q] = z;
    P.k1[q] = wx; P.k1[N + q] = wy; P.k1[2 * N + q] = wz;
    return;
  }
  const double x = fma(P.dt, fx, ex);
  const double y = fma(P.dt, fy, ey);
  const double z = fma(P.dt, fz, ez);
  const double r = rsqrt(x * x + y * y + z * z);
  P.ep[q] = x * r; P.ep[N + q] = y * r; P.ep[2 * N + q] = z * r;
  P.k1[q] = fx; P.k1[N + q] = fy; P.k1[2 * N + q] = fz;
}

template <int W, int NOISE, int INTEG>
__global__ void __launch_bounds__(256) k_correct(const DevLattice L, const DevLLG P, double* __restrict__ e,
                                                 const double* __restrict__ noise, uint64_t step) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  if (L.pinned && L.pinned[q]) return;
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  const double px = P.ep[q], py = P.ep[N + q], pz = P.ep[2 * N + q];
  double bx, by, bz;
  effective_field<W>(L, P.ep, q, s, c0, c1, c2, px, py, pz, bx, by, bz);
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
  const double a = P.alpha_site ? __ldg(P.alpha_site + q) : __ldg(P.alpha_sub + s);
  const double pre = P.pre_site ? __ldg(P.pre_site + q) : __ldg(P.pre_sub + s);
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
  e[q] = x * r; e[N + q] = y * r; e[2 * N + q] = z * r;
}

// stages: bit 0 = predictor, bit 1 = corrector
template <int W, int NOISE, int INTEG>
static void launch_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages,
                        cudaStream_t st) {
  const DevLattice& L = pl->model->d;
  const int tpb = 256;
  const unsigned grid = (unsigned)((L.N + tpb - 1) / tpb);
  if (stages & 1) k_predict<W, NOISE, INTEG><<<grid, tpb, 0, st>>>(L, pl->p, e, noise, step);
  if (stages & 2) k_correct<W, NOISE, INTEG><<<grid, tpb, 0, st>>>(L, pl->p, e, noise, step);
}

template <int W, int NOISE>
static void dispatch_integ(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages,
                           cudaStream_t st) {
  if (pl->p.integrator == MGX_INTEGRATOR_DEPONDT)
    launch_step<W, NOISE, MGX_INTEGRATOR_DEPONDT>(pl, e, noise, step, stages, st);
  else
    launch_step<W, NOISE, MGX_INTEGRATOR_HEUN>(pl, e, noise, step, stages, st);
}

template <int W>
static void dispatch_noise(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages,
                           cudaStream_t st) {
  switch (pl->p.noise) {
    case MGX_NOISE_HOST: dispatch_integ<W, MGX_NOISE_HOST>(pl, e, noise, step, stages, st); break;
    case MGX_NOISE_PHILOX: dispatch_integ<W, MGX_NOISE_PHILOX>(pl, e, noise, step, stages, st); break;
    default: dispatch_integ<W, MGX_NOISE_NONE>(pl, e, noise, step, stages, st); break;
  }
}

void enqueue_llg_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st,
                      int stages) {
  switch (pl->model->d.width) {
    case 1: dispatch_noise<1>(pl, e, noise, step, stages, st); break;
    case 4: dispatch_noise<4>(pl, e, noise, step, stages, st); break;
    default: dispatch_noise<9>(pl, e, noise, step, stages, st); break;
  }
}

template <typename T>
static std::vector<T> site_to_lattice(const T* src, int ns, int ncell) {
  const long long N = (long long)ns * ncell;
  std::vector<T> out(N);
  for (long long site = 0; site < N; ++site) {
    const long long cell = site / ns;
    const int s = (int)(site - cell * ns);
    out[(long long)s * ncell + cell] = src[site];
  }
  return out;
}

}  // namespace mgx

using namespace mgx;

extern "C" {

mgx_status mgx_llg_create(const mgx_model* mm, const mgx_llg_params* p, mgx_llg** out) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !p || !out) return set_error(MGX_ERR_INVALID, "mgx_llg_create: null argument");
  *out = nullptr;
  if (!(p->dt > 0.0) || !std::isfinite(p->dt)) return set_error(MGX_ERR_INVALID, "dt must be a positive number");
  if (p->integrator != MGX_INTEGRATOR_HEUN && p->integrator != MGX_INTEGRATOR_DEPONDT)
    return set_error(MGX_ERR_INVALID, "integrator %d is not heun (0) or depondt (1)", p->integrator);
  if (p->noise < MGX_NOISE_NONE || p->noise > MGX_NOISE_PHILOX)
    return set_error(MGX_ERR_INVALID, "noise mode %d is not none (0), host (1) or philox (2)", p->noise);
  const int ns = m->d.ns;
  const long long N = m->d.N;
  LLGPlan* pl = new LLGPlan();
  pl->model = m;
  DevLLG& d = pl->p;
  d.dt = p->dt;
  d.half_dt = 0.5 * p->dt;
  d.precession = p->precession ? 1 : 0;
  d.noise = p->noise;
  d.integrator = p->integrator;
  d.seed = p->seed;
  const double gamma = 0.1760859630;
  std::vector<double> sub(3 * ns, 0.0);
  for (int s = 0; s < ns; ++s) {
    sub[s] = p->alpha;
    sub[ns + s] = -gamma / (1.0 + p->alpha * p->alpha);
  }
  cudaError_t err = cudaMalloc(&pl->sub_block, sizeof(double) * sub.size());
  if (err == cudaSuccess) err = cudaMemcpy(pl->sub_block, sub.data(), sizeof(double) * sub.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMalloc(&pl->scratch, sizeof(double) * 6 * N);
  if (err != cudaSuccess) {
    mgx_llg_destroy(reinterpret_cast<mgx_llg*>(pl));
    return cuda_error(err, "mgx_llg_create");
  }
  d.alpha_sub = (const double*)pl->sub_block;
  d.pre_sub = d.alpha_sub + ns;
  d.sigma_sub = d.alpha_sub + 2 * ns;
  d.ep = pl->scratch;
  d.k1 = pl->scratch + 3 * N;
  if (p->alpha_site) {
    std::vector<double> a = site_to_lattice(p->alpha_site, ns, m->d.ncell);
    std::vector<double> both(2 * N);
    for (long long q = 0; q < N; ++q) {
      if (!std::isfinite(a[q]) || a[q] < 0.0) {
        mgx_llg_destroy(reinterpret_cast<mgx_llg*>(pl));
        return set_error(MGX_ERR_INVALID, "alpha_site must be finite and >= 0");
      }
      both[q] = a[q];
      both[N + q] = -gamma / (1.0 + a[q] * a[q]);
    }
    err = cudaMalloc(&pl->site_block, sizeof(double) * 2 * N);
    if (err == cudaSuccess) err = cudaMemcpy(pl->site_block, both.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
      mgx_llg_destroy(reinterpret_cast<mgx_llg*>(pl));
      return cuda_error(err, "mgx_llg_create alpha_site");
    }
    d.alpha_site = pl->site_block;
    d.pre_site = pl->site_block + N;
  }
  *out = reinterpret_cast<mgx_llg*>(pl);
  return MGX_OK;
}

mgx_status mgx_llg_destroy(mgx_llg* pp) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl) return MGX_OK;
  cudaFree(pl->sub_block);
  cudaFree(pl->site_block);
  cudaFree(pl->sigma_site);
  cudaFree(pl->scratch);
  delete pl;
  return MGX_OK;
}

mgx_status mgx_llg_set_sigma(mgx_llg* pp, const double* sigma_sub, const double* sigma_site) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl) return set_error(MGX_ERR_INVALID, "mgx_llg_set_sigma: null plan");
  const int ns = pl->model->d.ns;
  const long long N = pl->model->d.N;
  if (sigma_sub) {
    for (int s = 0; s < ns; ++s)
      if (!std::isfinite(sigma_sub[s]) || sigma_sub[s] < 0.0)
        return set_error(MGX_ERR_INVALID, "sigma_sub must be finite and >= 0");
    MGX_CUDA_TRY(cudaMemcpy((double*)pl->sub_block + 2 * ns, sigma_sub, sizeof(double) * ns, cudaMemcpyHostToDevice));
  }
  if (sigma_site) {
    std::vector<double> v = site_to_lattice(sigma_site, ns, pl->model->d.ncell);
    for (double x : v)
      if (!std::isfinite(x) || x < 0.0) return set_error(MGX_ERR_INVALID, "sigma_site must be finite and >= 0");
    if (!pl->sigma_site) MGX_CUDA_TRY(cudaMalloc(&pl->sigma_site, sizeof(double) * N));
    MGX_CUDA_TRY(cudaMemcpy(pl->sigma_site, v.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    pl->p.sigma_site = pl->sigma_site;
  } else {
    pl->p.sigma_site = nullptr;
  }
  return MGX_OK;
}

mgx_status mgx_llg_step(mgx_llg* pp, double* e, const double* noise, uint64_t step, void* stream) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_step: null argument");
  if (pl->p.noise == MGX_NOISE_HOST && !noise)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step: host-noise plan needs a noise buffer");
  enqueue_llg_step(pl, e, noise, step, (cudaStream_t)stream, 3);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_llg_stage(mgx_llg* pp, int32_t stage, double* e, const double* noise, uint64_t step, void* stream) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_stage: null argument");
  if (stage != 0 && stage != 1) return set_error(MGX_ERR_INVALID, "stage %d is not 0 (predictor) or 1 (corrector)", stage);
  if (pl->p.noise == MGX_NOISE_HOST && !noise)
    return set_error(MGX_ERR_INVALID, "mgx_llg_stage: host-noise plan needs a noise buffer");
  enqueue_llg_step(pl, e, noise, step, (cudaStream_t)stream, stage == 0 ? 1 : 2);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_llg_run(mgx_llg* pp, double* e, int64_t nsteps, uint64_t step0, void* stream) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_run: null argument");
  if (nsteps < 0) return set_error(MGX_ERR_INVALID, "nsteps must be >= 0");
  if (pl->p.noise == MGX_NOISE_HOST)
    return set_error(MGX_ERR_INVALID, "mgx_llg_run: host-noise plans step one at a time (mgx_llg_step)");
  for (int64_t n = 0; n < nsteps; ++n) enqueue_llg_step(pl, e, nullptr, step0 + (uint64_t)n, (cudaStream_t)stream, 3);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

}  // extern "C"
