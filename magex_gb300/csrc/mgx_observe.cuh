// Per-site observables shared by the single-lattice and batched reductions.
#pragma once

#include "mgx_internal.cuh"

namespace mgx {

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

// Solid angle 2 atan2(s1.(s2 x s3), 1 + s1.s2 + s2.s3 + s3.s1) of a spin triangle (magex/texture.py:55-60).
__device__ __forceinline__ double solid_angle(const double* __restrict__ e, long long N, int a, int b, int c) {
  const double ax = e[a], ay = e[N + a], az = e[2 * N + a];
  const double bx = e[b], by = e[N + b], bz = e[2 * N + b];
  const double cx = e[c], cy = e[N + c], cz = e[2 * N + c];
  const double num = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
  const double den = 1.0 + (ax * bx + ay * by + az * bz) + (bx * cx + by * cy + bz * cz) + (cx * ax + cy * ay + cz * az);
  return 2.0 * atan2(num, den);
}

// v[0] = E_i = e.A.e - e.h - mu_B mu e.B (magex/spinmodel.py:475-484), v[1..3] = e,
// v[4..6] = s e (magex/spinmodel.py:517-519), v[7] = |e x B_eff| (magex/llg.py:250-252; 0 if pinned).
template <int W>
__device__ __forceinline__ void observe_site(const DevLattice& L, const double* __restrict__ e, long long q,
                                             double* v) {
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  if (c0 < L.own0_begin || c0 >= L.own0_end) return;      // halo layer of a slab: owned elsewhere
  const double ex = e[q], ey = e[N + q], ez = e[2 * N + q];
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
  double Ghx = 0.0, Ghy = 0.0, Ghz = 0.0;       // higher on-site terms (magex/terms.py:41-43,66-68)
  if (L.Kc_site) v[0] += cubic_energy(L, q, ex, ey, ez);
  if (L.K2_site) v[0] += uniaxial_higher_energy(L, q, ex, ey, ez);
  if (L.Kc_site || L.K2_site) higher_onsite_grad(L, q, ex, ey, ez, Ghx, Ghy, Ghz);
  v[1] = ex;
  v[2] = ey;
  v[3] = ez;
  const double sg = L.sign_site ? L.sign_site[q] : L.sign_sub[s];
  v[4] = sg * ex;
  v[5] = sg * ey;
  v[6] = sg * ez;
  if (!(L.pinned && L.pinned[q])) {
    const double bx = (2.0 * hx - 2.0 * Ae[0] - Ghx) * inv + L.B0;
    const double by = (2.0 * hy - 2.0 * Ae[1] - Ghy) * inv + L.B1;
    const double bz = (2.0 * hz - 2.0 * Ae[2] - Ghz) * inv + L.B2;
    const double tx = ey * bz - ez * by, ty = ez * bx - ex * bz, tz = ex * by - ey * bx;
    v[7] = sqrt(tx * tx + ty * ty + tz * tz);
  }
}

}  // namespace mgx
