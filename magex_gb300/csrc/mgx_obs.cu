// Observables of a spin configuration: energy, magnetisation, order parameter, max torque, effective
// field and topological charge.  Reductions are two-pass and fixed-shape (warp shuffles, then one
// block over the per-block partials), so the sums do not depend on scheduling.
#include <cmath>

#include "mgx_observe.cuh"

namespace mgx {

constexpr int OBS_TPB = 256;


// Per site: E_i = e.A.e - e.h - mu_B mu e.B (magex/spinmodel.py:475-484), e, s e, |e x B_eff|.
// blockIdx.y selects one of several lattices stored one after the other (3 N doubles each); every
// lattice gets its own partials and the same reduction shape as a single one.
template <int W>
__global__ void __launch_bounds__(OBS_TPB) k_observe(const DevLattice L, const double* __restrict__ e,
                                                     double* __restrict__ partial) {
  e += (long long)blockIdx.y * 3 * L.N;
  partial += (long long)blockIdx.y * gridDim.x * OBS_NV;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v[OBS_NV] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (q < L.N) observe_site<W>(L, e, q, v);
  __shared__ double red[OBS_TPB / 32][OBS_NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < OBS_NV - 1; ++k) v[k] = warp_sum(v[k]);
  v[7] = warp_max(v[7]);
  if (lane == 0)
    for (int k = 0; k < OBS_NV; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < OBS_NV) {
    const int k = threadIdx.x;
    double acc = red[0][k];
    for (int w = 1; w < OBS_TPB / 32; ++w) acc = (k == 7) ? fmax(acc, red[w][k]) : acc + red[w][k];
    partial[(long long)blockIdx.x * OBS_NV + k] = acc;
  }
}

__global__ void __launch_bounds__(OBS_TPB) k_finish(const double* __restrict__ partial, int nblk, double* out) {
  partial += (long long)blockIdx.x * nblk * OBS_NV;
  out += (long long)blockIdx.x * OBS_NV;
  double v[OBS_NV] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblk; b += OBS_TPB)
    for (int k = 0; k < OBS_NV; ++k) {
      const double x = partial[(long long)b * OBS_NV + k];
      v[k] = (k == 7) ? fmax(v[k], x) : v[k] + x;
    }
  __shared__ double red[OBS_TPB / 32][OBS_NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < OBS_NV - 1; ++k) v[k] = warp_sum(v[k]);
  v[7] = warp_max(v[7]);
  if (lane == 0)
    for (int k = 0; k < OBS_NV; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < OBS_NV) {
    const int k = threadIdx.x;
    double acc = red[0][k];
    for (int w = 1; w < OBS_TPB / 32; ++w) acc = (k == 7) ? fmax(acc, red[w][k]) : acc + red[w][k];
    out[k] = acc;
  }
}

template <int W>
__global__ void __launch_bounds__(256) k_field(const DevLattice L, const double* __restrict__ e,
                                               double* __restrict__ B) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= L.N) return;
  const long long N = L.N;
  if (L.pinned && L.pinned[q]) {
    B[q] = 0.0; B[N + q] = 0.0; B[2 * N + q] = 0.0;
    return;
  }
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double bx, by, bz;
  effective_field<W>(L, e, q, s, c0, c1, c2, e[q], e[N + q], e[2 * N + q], bx, by, bz);
  add_higher_onsite(L, q, s, e[q], e[N + q], e[2 * N + q], bx, by, bz);
  B[q] = bx; B[N + q] = by; B[2 * N + q] = bz;
}

__global__ void __launch_bounds__(OBS_TPB) k_solid_angle(long long N, const double* __restrict__ e,
                                                         const int* __restrict__ tri,
                                                         const double* __restrict__ orient, long long ntri,
                                                         double* __restrict__ partial) {
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ntri;
       t += (long long)gridDim.x * blockDim.x) {
    acc += solid_angle(e, N, tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]) * orient[t];
  }
  __shared__ double red[OBS_TPB / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < OBS_TPB / 32; ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void k_solid_finish(const double* __restrict__ partial, int nblk, double* out) {
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += partial[b];
  out[0] = s / (4.0 * 3.14159265358979323846);
}

static mgx_status ensure_partials(Model* m, int need) {
  if (m->partial_cap >= need) return MGX_OK;
  cudaFree(m->partials);
  m->partials = nullptr;
  m->partial_cap = 0;
  MGX_CUDA_TRY(cudaMalloc(&m->partials, sizeof(double) * OBS_NV * (size_t)need));
  m->partial_cap = need;
  return MGX_OK;
}

}  // namespace mgx

using namespace mgx;

extern "C" {

mgx_status mgx_observables_n(const mgx_model* mm, const double* e, int32_t nlat, double* out, void* stream) {
  Model* m = const_cast<Model*>(reinterpret_cast<const Model*>(mm));
  if (!m || !e || !out) return set_error(MGX_ERR_INVALID, "mgx_observables: null argument");
  if (nlat < 1 || nlat > 65535) return set_error(MGX_ERR_INVALID, "mgx_observables_n: nlat = %d outside 1..65535", nlat);
  const long long nblk_ll = (m->d.N + OBS_TPB - 1) / OBS_TPB;
  if (nblk_ll * nlat > 0x7fffffffLL) return set_error(MGX_ERR_INVALID, "lattice too large for mgx_observables");
  const int nblk = (int)nblk_ll;
  mgx_status st = ensure_partials(m, nblk * nlat);
  if (st != MGX_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 grid(nblk, nlat);
  switch (m->d.width) {
    case 1: k_observe<1><<<grid, OBS_TPB, 0, s>>>(m->d, e, m->partials); break;
    case 4: k_observe<4><<<grid, OBS_TPB, 0, s>>>(m->d, e, m->partials); break;
    default: k_observe<9><<<grid, OBS_TPB, 0, s>>>(m->d, e, m->partials); break;
  }
  k_finish<<<nlat, OBS_TPB, 0, s>>>(m->partials, nblk, out);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_observables(const mgx_model* mm, const double* e, double* out, void* stream) {
  return mgx_observables_n(mm, e, 1, out, stream);
}

mgx_status mgx_effective_field(const mgx_model* mm, const double* e, double* B, void* stream) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !e || !B) return set_error(MGX_ERR_INVALID, "mgx_effective_field: null argument");
  const unsigned grid = (unsigned)((m->d.N + 255) / 256);
  cudaStream_t s = (cudaStream_t)stream;
  switch (m->d.width) {
    case 1: k_field<1><<<grid, 256, 0, s>>>(m->d, e, B); break;
    case 4: k_field<4><<<grid, 256, 0, s>>>(m->d, e, B); break;
    default: k_field<9><<<grid, 256, 0, s>>>(m->d, e, B); break;
  }
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_topological_charge(const mgx_model* mm, const double* e, const int32_t* tri, const double* orient,
                                  int64_t ntri, double* out, void* stream) {
  Model* m = const_cast<Model*>(reinterpret_cast<const Model*>(mm));
  if (!m || !e || !out || (ntri > 0 && (!tri || !orient)))
    return set_error(MGX_ERR_INVALID, "mgx_topological_charge: null argument");
  if (ntri < 0) return set_error(MGX_ERR_INVALID, "ntri must be >= 0");
  const int nblk = 4 * 152;
  mgx_status st = ensure_partials(m, (nblk + OBS_NV - 1) / OBS_NV);
  if (st != MGX_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  k_solid_angle<<<nblk, OBS_TPB, 0, s>>>(m->d.N, e, tri, orient, (long long)ntri, m->partials);
  k_solid_finish<<<1, 32, 0, s>>>(m->partials, nblk, out);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

}  // extern "C"
