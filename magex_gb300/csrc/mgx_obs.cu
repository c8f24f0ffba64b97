// Observables of a spin configuration: energy, magnetisation, order parameter, max torque, effective
// field and topological charge.  Reductions are two-pass and fixed-shape (warp shuffles, then one
// block over the per-block partials), so the sums do not depend on scheduling.
#include <cmath>

#include "mgx_internal.cuh"

namespace mgx {

constexpr int OBS_TPB = 256;
constexpr int OBS_NV = 8;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Per site: E_i = e.A.e - e.h - mu_B mu e.B (magex/spinmodel.py:475-484), e, s e, |e x B_eff|.
template <int W>
__global__ void __launch_bounds__(OBS_TPB) k_observe(const DevLattice L, const double* __restrict__ e,
                                                     double* __restrict__ partial) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v[OBS_NV] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (q < L.N) {
    const long long N = L.N;
    const double ex = e[q], ey = e[N + q], ez = e[2 * N + q];
    int s, c0, c1, c2;
    site_coords(L, q, s, c0, c1, c2);
    double hx, hy, hz;
    exchange_field<W>(L, e, s, c0, c1, c2, hx, hy, hz);
    double Ae[3] = {0.0, 0.0, 0.0};
    if (L.has_A) {
      double a[9];
      if (L.A_site) {
        for (int k = 0; k < 9; ++k) a[k] = L.A_site[(long long)k * N + q];
      } else {
        for (int k = 0; k < 9; ++k) a[k] = L.A_sub[s * 9 + k];
      }
      Ae[0] = a[0] * ex + a[1] * ey + a[2] * ez;
      Ae[1] = a[3] * ex + a[4] * ey + a[5] * ez;
      Ae[2] = a[6] * ex + a[7] * ey + a[8] * ez;
    }
    const double mu = L.mu_site ? L.mu_site[q] : L.mu_sub[s];
    const double inv = L.inv_mu_site ? L.inv_mu_site[q] : L.inv_mu_sub[s];
    const double eAe = ex * Ae[0] + ey * Ae[1] + ez * Ae[2];
    const double eh = ex * hx + ey * hy + ez * hz;
    const double eB = ex * L.B0 + ey * L.B1 + ez * L.B2;
    v[0] = eAe - eh - 5.7883818060e-2 * mu * eB;
    v[1] = ex;
    v[2] = ey;
    v[3] = ez;
    const double sg = L.sign_sub[s];
    v[4] = sg * ex;
    v[5] = sg * ey;
    v[6] = sg * ez;
    if (!(L.pinned && L.pinned[q])) {
      const double bx = (2.0 * hx - 2.0 * Ae[0]) * inv + L.B0;
      const double by = (2.0 * hy - 2.0 * Ae[1]) * inv + L.B1;
      const double bz = (2.0 * hz - 2.0 * Ae[2]) * inv + L.B2;
      const double tx = ey * bz - ez * by, ty = ez * bx - ex * bz, tz = ex * by - ey * bx;
      v[7] = sqrt(tx * tx + ty * ty + tz * tz);
    }
  }
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
  B[q] = bx; B[N + q] = by; B[2 * N + q] = bz;
}

// solid angle of each triangle, magex/texture.py:55-60
__global__ void __launch_bounds__(OBS_TPB) k_solid_angle(long long N, const double* __restrict__ e,
                                                         const int* __restrict__ tri,
                                                         const double* __restrict__ orient, long long ntri,
                                                         double* __restrict__ partial) {
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ntri;
       t += (long long)gridDim.x * blockDim.x) {
    const int a = tri[3 * t], b = tri[3 * t + 1], c = tri[3 * t + 2];
    const double ax = e[a], ay = e[N + a], az = e[2 * N + a];
    const double bx = e[b], by = e[N + b], bz = e[2 * N + b];
    const double cx = e[c], cy = e[N + c], cz = e[2 * N + c];
    const double num = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
    const double den = 1.0 + (ax * bx + ay * by + az * bz) + (bx * cx + by * cy + bz * cz) + (cx * ax + cy * ay + cz * az);
    acc += 2.0 * atan2(num, den) * orient[t];
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

mgx_status mgx_observables(const mgx_model* mm, const double* e, double* out, void* stream) {
  Model* m = const_cast<Model*>(reinterpret_cast<const Model*>(mm));
  if (!m || !e || !out) return set_error(MGX_ERR_INVALID, "mgx_observables: null argument");
  const long long nblk_ll = (m->d.N + OBS_TPB - 1) / OBS_TPB;
  if (nblk_ll > 0x7fffffffLL) return set_error(MGX_ERR_INVALID, "lattice too large for mgx_observables");
  const int nblk = (int)nblk_ll;
  mgx_status st = ensure_partials(m, nblk);
  if (st != MGX_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  switch (m->d.width) {
    case 1: k_observe<1><<<nblk, OBS_TPB, 0, s>>>(m->d, e, m->partials); break;
    case 4: k_observe<4><<<nblk, OBS_TPB, 0, s>>>(m->d, e, m->partials); break;
    default: k_observe<9><<<nblk, OBS_TPB, 0, s>>>(m->d, e, m->partials); break;
  }
  k_finish<<<1, OBS_TPB, 0, s>>>(m->partials, nblk, out);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
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
