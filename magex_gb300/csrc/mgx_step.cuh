// Per-site bodies of the Heun / Depondt predictor and corrector, shared by the single-lattice
// kernels (mgx_llg.cu) and the batched ensemble kernels (mgx_batch.cu).
//
// Reference behaviour: magex/llg.py:216-227 (NumPy Heun), magex/fast.py:336-390 (fused predictor /
// corrector, numba), magex/cuda_backend.py:144-218 (numba.cuda twins).
#pragma once

#include "mgx_internal.cuh"

namespace mgx {

// magex site number of lattice index q (layout-independent Philox counter)
__device__ __forceinline__ uint64_t magex_site(const DevLattice& L, long long q, int s) {
  return (uint64_t)(q - (long long)s * L.ncell + L.cell_offset) * (uint64_t)L.ns + (uint64_t)s;
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

// B += the caller's per-site field of this stage (magex's extra_field, magex/llg.py:131-132)
__device__ __forceinline__ void add_extra(const DevLLG& P, long long N, long long q, double& bx, double& by,
                                          double& bz) {
  if (!P.B_add) return;
  bx += __ldg(P.B_add + q);
  by += __ldg(P.B_add + N + q);
  bz += __ldg(P.B_add + 2 * N + q);
}

// B += B_DL e x p + B_FL p at the stage's spin e (spin-orbit torque as effective fields,
// magex/llg.py:126-128,158-160)
__device__ __forceinline__ void add_sot(const DevLLG& P, double x, double y, double z, double& bx, double& by,
                                        double& bz) {
  if (!P.sot) return;
  const double p0 = __ldg(P.sot), p1 = __ldg(P.sot + 1), p2 = __ldg(P.sot + 2);
  const double dl = __ldg(P.sot + 3), fl = __ldg(P.sot + 4);
  bx += fma(dl, y * p2 - z * p1, fl * p0);
  by += fma(dl, z * p0 - x * p2, fl * p1);
  bz += fma(dl, x * p1 - y * p0, fl * p2);
}

template <int NOISE>
__device__ __forceinline__ void add_thermal(const DevLattice& L, const DevLLG& P, const double* __restrict__ noise,
                                            long long q, int s, uint64_t step, double& bx, double& by, double& bz,
                                            bool hw_convert = false) {
  if (NOISE == MGX_NOISE_NONE) return;
  const double sig = P.sigma_site ? __ldg(P.sigma_site + q) : __ldg(P.sigma_sub + s);
  double g0, g1, g2;
  if (NOISE == MGX_NOISE_HOST) {
    g0 = __ldg(noise + q);
    g1 = __ldg(noise + L.N + q);
    g2 = __ldg(noise + 2 * L.N + q);
  } else {
    philox_normal3(P.seed, magex_site(L, q, s), step, g0, g1, g2, hw_convert);
  }
  bx = fma(sig, g0, bx);
  by = fma(sig, g1, by);
  bz = fma(sig, g2, bz);
}

// Predictor of site q (0 <= q < L.N): writes P.ep and P.k1 at q.  With Hout != nullptr the total
// field (effective + thermal) of the site is stored there too (adjoint recomputation).  EXTRA adds the
// spin-orbit torque fields and the caller's per-site field (a separate instantiation, so the plain
// kernels carry neither).
template <int W, int NOISE, int INTEG, bool EXTRA = false>
__device__ __forceinline__ void predict_site(const DevLattice& L, const DevLLG& P, const double* __restrict__ e,
                                             const double* __restrict__ noise, long long q, uint64_t step,
                                             double* __restrict__ Hout = nullptr, double* __restrict__ rout = nullptr) {
  const long long N = L.N;
  const double ex = e[q], ey = e[N + q], ez = e[2 * N + q];
  if (L.pinned && L.pinned[q]) {
    P.ep[q] = ex; P.ep[N + q] = ey; P.ep[2 * N + q] = ez;
    P.k1[q] = 0.0; P.k1[N + q] = 0.0; P.k1[2 * N + q] = 0.0;
    if (Hout) {
      Hout[q] = 0.0; Hout[N + q] = 0.0; Hout[2 * N + q] = 0.0;
    }
    return;
  }
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  double bx, by, bz;
  effective_field<W>(L, e, q, s, c0, c1, c2, ex, ey, ez, bx, by, bz);
  if (EXTRA) {
    add_higher_onsite(L, q, s, ex, ey, ez, bx, by, bz);
    add_sot(P, ex, ey, ez, bx, by, bz);
    add_extra(P, N, q, bx, by, bz);
  }
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
  if (Hout) {
    Hout[q] = bx; Hout[N + q] = by; Hout[2 * N + q] = bz;
  }
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
  if (rout) rout[q] = r;
  P.ep[q] = x * r; P.ep[N + q] = y * r; P.ep[2 * N + q] = z * r;
  P.k1[q] = fx; P.k1[N + q] = fy; P.k1[2 * N + q] = fz;
}

// Corrector of site q (0 <= q < L.N): reads P.ep (neighbours), P.k1 and e at q, writes e at q
// (or eout at q when given; the adjoint recomputation keeps e).  Hout as in predict_site.
template <int W, int NOISE, int INTEG, bool EXTRA = false>
__device__ __forceinline__ void correct_site(const DevLattice& L, const DevLLG& P, double* __restrict__ e,
                                             const double* __restrict__ noise, long long q, uint64_t step,
                                             double* __restrict__ Hout = nullptr, double* __restrict__ eout = nullptr,
                                             double* __restrict__ fout = nullptr, double* __restrict__ rout = nullptr) {
  if (L.pinned && L.pinned[q]) {
    if (eout) {
      eout[q] = e[q]; eout[L.N + q] = e[L.N + q]; eout[2 * L.N + q] = e[2 * L.N + q];
    }
    if (Hout) {
      Hout[q] = 0.0; Hout[L.N + q] = 0.0; Hout[2 * L.N + q] = 0.0;
    }
    if (fout) {
      fout[q] = 0.0; fout[L.N + q] = 0.0; fout[2 * L.N + q] = 0.0;
    }
    return;
  }
  const long long N = L.N;
  int s, c0, c1, c2;
  site_coords(L, q, s, c0, c1, c2);
  const double px = P.ep[q], py = P.ep[N + q], pz = P.ep[2 * N + q];
  double bx, by, bz;
  effective_field<W>(L, P.ep, q, s, c0, c1, c2, px, py, pz, bx, by, bz);
  if (EXTRA) {
    add_higher_onsite(L, q, s, px, py, pz, bx, by, bz);
    add_sot(P, px, py, pz, bx, by, bz);
    add_extra(P, N, q, bx, by, bz);
  }
  add_thermal<NOISE>(L, P, noise, q, s, step, bx, by, bz);
  if (Hout) {
    Hout[q] = bx; Hout[N + q] = by; Hout[2 * N + q] = bz;
  }
  const double a = P.alpha_site ? __ldg(P.alpha_site + q) : __ldg(P.alpha_sub + s);
  const double pre = P.pre_site ? __ldg(P.pre_site + q) : __ldg(P.pre_sub + s);
  double fx, fy, fz;
  llg_rhs(px, py, pz, bx, by, bz, a, pre, P.precession != 0, fx, fy, fz);
  if (fout) {
    fout[q] = fx; fout[N + q] = fy; fout[2 * N + q] = fz;
  }
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
  if (rout) rout[q] = r;
  double* o = eout ? eout : e;
  o[q] = x * r; o[N + q] = y * r; o[2 * N + q] = z * r;
}

}  // namespace mgx
