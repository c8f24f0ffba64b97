/*
 * heun_ref.c -- CPU restatement of magex's LLG hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the oracle the GB300 kernels are checked against and the CPU baseline that
 * bench.py times.  Nothing in the product (magex_gb300/) loads it.
 *
 * What it restates (operation order of the reference's fused CPU kernels):
 *   oracle_step         magex/fast.py:336-390  (_fused1 predictor, _fused2 corrector; Heun and
 *   oracle_stage        Depondt; oracle_stage runs one of the two), with the field of magex/fast.py:87-120,309-317 and the right-hand
 *                       side of magex/fast.py:225-236; the thermal field b is an input (already
 *                       scaled by sigma), as in magex's extras path magex/llg.py:200-208.
 *   oracle_observables  magex/spinmodel.py:475-484 (energy), :517-519 (order parameter),
 *                       magex/llg.py:250-252,265 (max torque, mean spin).
 *   oracle_gauss3       magex/fast.py:123-200 (xorshift64* streams over 256 fixed chunks and the
 *                       128-layer Marsaglia-Tsang ziggurat), the reference's multithreaded noise.
 *   oracle_greedy_colour, oracle_mc_group
 *                       magex/montecarlo.py:35-48,181-227 (colour classes and the NumPy Monte Carlo
 *                       sweep with its moves), at the end of this file.
 *
 * Neighbour data is magex's per-site block list (magex/fast.py:587-627): ptr (N+1), nbr, typ and a
 * coupling table of width 1 (J), 4 (J, D) or 9 (3x3 row-major), in magex site order.
 * Build: see oracle/Makefile (gcc -O2 -fopenmp, plain C99, no target-specific flags).
 */
#define _DEFAULT_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MU_B 5.7883818060e-2
#define GAMMA 0.1760859630

typedef struct oracle_model {
  int64_t N;
  const int64_t* ptr;
  const int32_t* nbr;
  const int32_t* typ;
  const double* table;
  int32_t width;
  const double* A;        /* N*9 or NULL (no on-site terms) */
  const double* mu;       /* N */
  double B[3];
  const uint8_t* pinned;  /* N or NULL */
  /* cubic anisotropy Kc (N or NULL) with axes C (rows), higher uniaxial K2, K3 (N or NULL) along u:
   * the Kc, C, K2, K3, u, has_c, has_u kernel arguments of magex/fast.py:640-672 */
  const double* Kc;
  double C[9];
  const double* K2;
  const double* K3;
  double u[3];
} oracle_model;

static void hfield(const oracle_model* m, int64_t i, const double* e, double* h) {
  double hx = 0.0, hy = 0.0, hz = 0.0;
  const int w = m->width;
  for (int64_t k = m->ptr[i]; k < m->ptr[i + 1]; ++k) {
    const int64_t j = m->nbr[k];
    const double* T = m->table + (int64_t)m->typ[k] * w;
    const double ex = e[3 * j], ey = e[3 * j + 1], ez = e[3 * j + 2];
    if (w == 1) {
      hx += T[0] * ex;
      hy += T[0] * ey;
      hz += T[0] * ez;
    } else if (w == 4) {
      hx += T[0] * ex + (ey * T[3] - ez * T[2]);
      hy += T[0] * ey + (ez * T[1] - ex * T[3]);
      hz += T[0] * ez + (ex * T[2] - ey * T[1]);
    } else {
      hx += T[0] * ex + T[1] * ey + T[2] * ez;
      hy += T[3] * ex + T[4] * ey + T[5] * ez;
      hz += T[6] * ex + T[7] * ey + T[8] * ez;
    }
  }
  h[0] = hx;
  h[1] = hy;
  h[2] = hz;
}

static void onsite_grad(const oracle_model* m, int64_t i, const double* v, double* g) {
  g[0] = g[1] = g[2] = 0.0;
  if (!m->A) return;
  const double* A = m->A + 9 * i;
  g[0] = 2.0 * (A[0] * v[0] + A[1] * v[1] + A[2] * v[2]);
  g[1] = 2.0 * (A[3] * v[0] + A[4] * v[1] + A[5] * v[2]);
  g[2] = 2.0 * (A[6] * v[0] + A[7] * v[1] + A[8] * v[2]);
}

/* adds dE/de of the cubic and higher uniaxial terms (magex/fast.py:50-63, magex/terms.py:45-49,65-67) */
static void higher_grad(const oracle_model* m, int64_t i, const double* v, double* g) {
  if (m->Kc) {
    const double* C = m->C;
    const double a1 = C[0] * v[0] + C[1] * v[1] + C[2] * v[2];
    const double a2 = C[3] * v[0] + C[4] * v[1] + C[5] * v[2];
    const double a3 = C[6] * v[0] + C[7] * v[1] + C[8] * v[2];
    const double q1 = a1 * a1, q2 = a2 * a2, q3 = a3 * a3;
    const double d1 = 2 * a1 * (q2 + q3) * m->Kc[i], d2 = 2 * a2 * (q1 + q3) * m->Kc[i],
                 d3 = 2 * a3 * (q1 + q2) * m->Kc[i];
    g[0] += d1 * C[0] + d2 * C[3] + d3 * C[6];
    g[1] += d1 * C[1] + d2 * C[4] + d3 * C[7];
    g[2] += d1 * C[2] + d2 * C[5] + d3 * C[8];
  }
  if (m->K2) {
    const double c = v[0] * m->u[0] + v[1] * m->u[1] + v[2] * m->u[2];
    const double f = -4.0 * m->K2[i] * c * c * c - 6.0 * m->K3[i] * c * c * c * c * c;
    g[0] += f * m->u[0];
    g[1] += f * m->u[1];
    g[2] += f * m->u[2];
  }
}

/* energies of the cubic and the higher uniaxial term at site i (magex/terms.py:41-43,61-63) */
static double cubic_energy(const oracle_model* m, int64_t i, const double* v) {
  const double* C = m->C;
  const double a1 = C[0] * v[0] + C[1] * v[1] + C[2] * v[2];
  const double a2 = C[3] * v[0] + C[4] * v[1] + C[5] * v[2];
  const double a3 = C[6] * v[0] + C[7] * v[1] + C[8] * v[2];
  const double q1 = a1 * a1, q2 = a2 * a2, q3 = a3 * a3;
  return m->Kc[i] * (q1 * q2 + q2 * q3 + q3 * q1);
}

static double uniaxial_energy(const oracle_model* m, int64_t i, const double* v) {
  const double c = v[0] * m->u[0] + v[1] * m->u[1] + v[2] * m->u[2];
  return -m->K2[i] * c * c * c * c - m->K3[i] * c * c * c * c * c * c;
}

static double higher_energy(const oracle_model* m, int64_t i, const double* v) {
  return (m->Kc ? cubic_energy(m, i, v) : 0.0) + (m->K2 ? uniaxial_energy(m, i, v) : 0.0);
}

/* B_eff of site i for spins e (T) */
static void bloc(const oracle_model* m, int64_t i, const double* e, double* B) {
  double h[3], g[3];
  hfield(m, i, e, h);
  onsite_grad(m, i, e + 3 * i, g);
  higher_grad(m, i, e + 3 * i, g);
  const double inv = 1.0 / (m->mu[i] * MU_B);
  B[0] = (2 * h[0] - g[0]) * inv + m->B[0];
  B[1] = (2 * h[1] - g[1]) * inv + m->B[1];
  B[2] = (2 * h[2] - g[2]) * inv + m->B[2];
}

static void rhs(const double* e, const double* b, double a, int prec, double* f) {
  const double cx = e[1] * b[2] - e[2] * b[1];
  const double cy = e[2] * b[0] - e[0] * b[2];
  const double cz = e[0] * b[1] - e[1] * b[0];
  const double dx = e[1] * cz - e[2] * cy;
  const double dy = e[2] * cx - e[0] * cz;
  const double dz = e[0] * cy - e[1] * cx;
  const double pre = -GAMMA / (1.0 + a * a);
  if (prec) {
    f[0] = pre * (cx + a * dx);
    f[1] = pre * (cy + a * dy);
    f[2] = pre * (cz + a * dz);
  } else {
    f[0] = pre * a * dx;
    f[1] = pre * a * dy;
    f[2] = pre * a * dz;
  }
}

static void rot(double* v, double wx, double wy, double wz) {
  const double th = sqrt(wx * wx + wy * wy + wz * wz);
  if (th < 1e-14) return;
  const double kx = wx / th, ky = wy / th, kz = wz / th;
  const double c = cos(th), s = sin(th);
  const double kd = kx * v[0] + ky * v[1] + kz * v[2];
  const double cx = ky * v[2] - kz * v[1], cy = kz * v[0] - kx * v[2], cz = kx * v[1] - ky * v[0];
  const double x = v[0] * c + cx * s + kx * kd * (1 - c);
  const double y = v[1] * c + cy * s + ky * kd * (1 - c);
  const double z = v[2] * c + cz * s + kz * kd * (1 - c);
  v[0] = x;
  v[1] = y;
  v[2] = z;
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* One stage of a Heun (depondt = 0) or Depondt (depondt = 1) step (magex order, N*3 arrays):
 * stage 0 (predictor) reads e and writes ep and k1; stage 1 (corrector) reads ep and k1 and updates e
 * in place.  alpha: N damping values; b: N*3 thermal field (T) or NULL. */
void oracle_stage(const oracle_model* m, const double* alpha, double dt, int prec, int depondt, const double* b,
                  double* e, double* ep, double* k1, int stage, int nthreads) {
  const int64_t N = m->N;
  set_threads(nthreads);
  if (stage != 0) goto corrector;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    if (m->pinned && m->pinned[i]) {
      ep[3 * i] = e[3 * i];
      ep[3 * i + 1] = e[3 * i + 1];
      ep[3 * i + 2] = e[3 * i + 2];
      k1[3 * i] = k1[3 * i + 1] = k1[3 * i + 2] = 0.0;
      continue;
    }
    double B[3], f[3];
    bloc(m, i, e, B);
    if (b) {
      B[0] += b[3 * i];
      B[1] += b[3 * i + 1];
      B[2] += b[3 * i + 2];
    }
    rhs(e + 3 * i, B, alpha[i], prec, f);
    if (depondt) {
      const double* v = e + 3 * i;
      const double wx = v[1] * f[2] - v[2] * f[1], wy = v[2] * f[0] - v[0] * f[2], wz = v[0] * f[1] - v[1] * f[0];
      k1[3 * i] = wx;
      k1[3 * i + 1] = wy;
      k1[3 * i + 2] = wz;
      double r[3] = {v[0], v[1], v[2]};
      rot(r, dt * wx, dt * wy, dt * wz);
      ep[3 * i] = r[0];
      ep[3 * i + 1] = r[1];
      ep[3 * i + 2] = r[2];
    } else {
      k1[3 * i] = f[0];
      k1[3 * i + 1] = f[1];
      k1[3 * i + 2] = f[2];
      const double x = e[3 * i] + dt * f[0], y = e[3 * i + 1] + dt * f[1], z = e[3 * i + 2] + dt * f[2];
      const double q = 1.0 / sqrt(x * x + y * y + z * z);
      ep[3 * i] = x * q;
      ep[3 * i + 1] = y * q;
      ep[3 * i + 2] = z * q;
    }
  }
  return;
corrector:
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    if (m->pinned && m->pinned[i]) continue;
    double B[3], f[3], x, y, z;
    bloc(m, i, ep, B);
    if (b) {
      B[0] += b[3 * i];
      B[1] += b[3 * i + 1];
      B[2] += b[3 * i + 2];
    }
    rhs(ep + 3 * i, B, alpha[i], prec, f);
    if (depondt) {
      const double* p = ep + 3 * i;
      const double wx = p[1] * f[2] - p[2] * f[1], wy = p[2] * f[0] - p[0] * f[2], wz = p[0] * f[1] - p[1] * f[0];
      double r[3] = {e[3 * i], e[3 * i + 1], e[3 * i + 2]};
      rot(r, 0.5 * dt * (k1[3 * i] + wx), 0.5 * dt * (k1[3 * i + 1] + wy), 0.5 * dt * (k1[3 * i + 2] + wz));
      x = r[0];
      y = r[1];
      z = r[2];
    } else {
      x = e[3 * i] + 0.5 * dt * (k1[3 * i] + f[0]);
      y = e[3 * i + 1] + 0.5 * dt * (k1[3 * i + 1] + f[1]);
      z = e[3 * i + 2] + 0.5 * dt * (k1[3 * i + 2] + f[2]);
    }
    const double q = 1.0 / sqrt(x * x + y * y + z * z);
    e[3 * i] = x * q;
    e[3 * i + 1] = y * q;
    e[3 * i + 2] = z * q;
  }
}

/* One full step in place on e: both stages. */
void oracle_step(const oracle_model* m, const double* alpha, double dt, int prec, int depondt, const double* b,
                 double* e, double* ep, double* k1, int nthreads) {
  oracle_stage(m, alpha, dt, prec, depondt, b, e, ep, k1, 0, nthreads);
  oracle_stage(m, alpha, dt, prec, depondt, b, e, ep, k1, 1, nthreads);
}

/* out[8] = E, sum e (3), sum s e (3), max |e x B_eff| (pinned sites have zero field). */
void oracle_observables(const oracle_model* m, const double* e, const double* signs, double* out, int nthreads) {
  const int64_t N = m->N;
  double E = 0, mx = 0, my = 0, mz = 0, ox = 0, oy = 0, oz = 0, tmax = 0;
  set_threads(nthreads);
#pragma omp parallel for schedule(static) reduction(+ : E, mx, my, mz, ox, oy, oz) reduction(max : tmax)
  for (int64_t i = 0; i < N; ++i) {
    const double* v = e + 3 * i;
    double h[3], g[3];
    hfield(m, i, e, h);
    onsite_grad(m, i, v, g);
    E += 0.5 * (v[0] * g[0] + v[1] * g[1] + v[2] * g[2]) - (v[0] * h[0] + v[1] * h[1] + v[2] * h[2]) -
         MU_B * m->mu[i] * (v[0] * m->B[0] + v[1] * m->B[1] + v[2] * m->B[2]) + higher_energy(m, i, v);
    higher_grad(m, i, v, g);
    mx += v[0];
    my += v[1];
    mz += v[2];
    const double s = signs ? signs[i] : 1.0;
    ox += s * v[0];
    oy += s * v[1];
    oz += s * v[2];
    if (!(m->pinned && m->pinned[i])) {
      const double inv = 1.0 / (m->mu[i] * MU_B);
      const double bx = (2 * h[0] - g[0]) * inv + m->B[0];
      const double by = (2 * h[1] - g[1]) * inv + m->B[1];
      const double bz = (2 * h[2] - g[2]) * inv + m->B[2];
      const double tx = v[1] * bz - v[2] * by, ty = v[2] * bx - v[0] * bz, tz = v[0] * by - v[1] * bx;
      const double t = sqrt(tx * tx + ty * ty + tz * tz);
      if (t > tmax) tmax = t;
    }
  }
  out[0] = E;
  out[1] = mx;
  out[2] = my;
  out[3] = mz;
  out[4] = ox;
  out[5] = oy;
  out[6] = oz;
  out[7] = tmax;
}

/* ---------------------------------------------------------------- reference noise generator */
static double ZKN[128], ZWN[128], ZFN[128];
static int zig_ready = 0;

static void zig_tables(void) {
  /* 128-layer ziggurat for the standard normal (Marsaglia & Tsang, J. Stat. Softw. 5(8), 2000),
   * same right-tail point and layer area as magex/fast.py:137-158 */
  double dn = 3.442619855899, tn = dn;
  const double vn = 9.91256303526217e-3, m1 = 2147483648.0;
  const double q = vn / exp(-0.5 * dn * dn);
  ZKN[0] = (dn / q) * m1;
  ZKN[1] = 0.0;
  ZWN[0] = q / m1;
  ZWN[127] = dn / m1;
  ZFN[0] = 1.0;
  ZFN[127] = exp(-0.5 * dn * dn);
  for (int i = 126; i >= 1; --i) {
    dn = sqrt(-2.0 * log(vn / dn + exp(-0.5 * dn * dn)));
    ZKN[i + 1] = (dn / tn) * m1;
    tn = dn;
    ZFN[i] = exp(-0.5 * dn * dn);
    ZWN[i] = dn / m1;
  }
  zig_ready = 1;
}

static inline uint64_t xs_next(uint64_t* s) {
  uint64_t x = *s;
  x ^= x >> 12;
  x ^= x << 25;
  x ^= x >> 27;
  *s = x;
  return x * 2685821657736338717ULL;
}

static inline double xs_unif(uint64_t* s) { return (double)(xs_next(s) >> 11) * (1.0 / 9007199254740992.0); }

static inline int64_t xs_hz(uint64_t* s) { return (int64_t)(int32_t)(uint32_t)(xs_next(s) >> 32); }

static double znorm(uint64_t* s) {
  int64_t hz = xs_hz(s);
  int64_t iz = hz & 127;
  if ((double)llabs(hz) < ZKN[iz]) return (double)hz * ZWN[iz];
  const double r = 3.442619855899;
  for (;;) {
    double x = (double)hz * ZWN[iz];
    if (iz == 0) {
      double y;
      do {
        double u = xs_unif(s);
        x = -log(u > 1e-300 ? u : 1e-300) * 0.2904764;
        u = xs_unif(s);
        y = -log(u > 1e-300 ? u : 1e-300);
      } while (!(y + y >= x * x));
      return hz > 0 ? r + x : -r - x;
    }
    if (ZFN[iz] + xs_unif(s) * (ZFN[iz - 1] - ZFN[iz]) < exp(-0.5 * x * x)) return x;
    hz = xs_hz(s);
    iz = hz & 127;
    if ((double)llabs(hz) < ZKN[iz]) return (double)hz * ZWN[iz];
  }
}

/* out[i, c] = scale[i] * N(0,1) over nc fixed chunks (stream c owns chunk c), pinned sites 0:
 * magex/fast.py:189-200.  The draws do not depend on the number of threads. */
void oracle_gauss3(double* out, uint64_t* states, int nc, const double* scale, const uint8_t* pinned, int64_t N,
                   int nthreads) {
  if (!zig_ready) zig_tables();
  const int64_t chunk = (N + nc - 1) / nc;
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    const int64_t lo = (int64_t)c * chunk, hi = lo + chunk < N ? lo + chunk : N;
    for (int64_t i = lo; i < hi; ++i)
      for (int comp = 0; comp < 3; ++comp) {
        const double g = znorm(&states[c]);
        out[3 * i + comp] = (pinned && pinned[i]) ? 0.0 : scale[i] * g;
      }
  }
}

/* ---------------------------------------------------------------- neighbour list for a stencil */
/* Per-site neighbour list of a periodic / open supercell in magex site order, neighbours in the
 * given coupling order (cell offsets R, sublattices src -> dst, coupling type typ_of_bond).
 * ptr must hold N+1 entries; nbr / typ hold ptr[N] entries (call once with nbr == NULL to size). */
int64_t oracle_stencil_csr(int ns, const int32_t* L, const int32_t* pbc, int nbond, const int32_t* src,
                           const int32_t* dst, const int32_t* R, const int32_t* typ_of_bond, int64_t* ptr,
                           int32_t* nbr, int32_t* typ) {
  const int64_t ncell = (int64_t)L[0] * L[1] * L[2], N = ncell * ns;
  ptr[0] = 0;
  for (int64_t site = 0; site < N; ++site) {
    const int64_t cell = site / ns;
    const int s = (int)(site - cell * ns);
    const int c[3] = {(int)(cell / ((int64_t)L[1] * L[2])), (int)((cell / L[2]) % L[1]), (int)(cell % L[2])};
    int64_t n = ptr[site];
    for (int b = 0; b < nbond; ++b) {
      if (src[b] != s) continue;
      int t[3], ok = 1;
      for (int a = 0; a < 3; ++a) {
        int x = c[a] + R[3 * b + a];
        if (pbc[a]) {
          x %= L[a];
          if (x < 0) x += L[a];
        } else if (x < 0 || x >= L[a]) {
          ok = 0;
        }
        t[a] = x;
      }
      if (!ok) continue;
      if (nbr) {
        nbr[n] = (int32_t)(((((int64_t)t[0] * L[1] + t[1]) * L[2]) + t[2]) * ns + dst[b]);
        typ[n] = typ_of_bond[b];
      }
      ++n;
    }
    ptr[site + 1] = n;
  }
  return ptr[N];
}

/* ================================================================ Monte Carlo colour sweeps
 * oracle_greedy_colour  magex/montecarlo.py:35-48: first-fit greedy colouring in site order of the
 *                       graph adj + adj^T (self-loops ignored).
 * oracle_mc_group       one group update of MetropolisMC.sweep (magex/montecarlo.py:181-210) with
 *                       its NumPy moves (magex/montecarlo.py:51-68,136-147,212-227), consuming draws
 *                       that the caller made with magex's generator in magex's order:
 *                         move 0 gaussian / 1 uniform: normal (n,3), uniform (n)
 *                         move 2 heat bath:            uniform (n), uniform (n), uniform (n)
 *                         move 3 hinzke:               k (n), normal (n,3), normal (n,3), uniform (n)
 *                         move 4 over-relaxation:      uniform (n)
 *                       Returns the number of accepted moves.  All sites of the group see the spins
 *                       of before the pass, as in magex's vectorised update. */
int32_t oracle_greedy_colour(int64_t N, const int64_t* ptr, const int32_t* nbr, int32_t* colour) {
  int64_t* tptr = (int64_t*)calloc((size_t)N + 1, sizeof(int64_t));
  int32_t* tnbr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ptr[N] > 0 ? ptr[N] : 1));
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N > 0 ? N : 1));
  for (int64_t k = 0; k < ptr[N]; ++k) tptr[nbr[k] + 1]++;
  for (int64_t v = 0; v < N; ++v) tptr[v + 1] += tptr[v];
  for (int64_t v = 0; v < N; ++v) fill[v] = tptr[v];
  for (int64_t v = 0; v < N; ++v)
    for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k) tnbr[fill[nbr[k]]++] = (int32_t)v;
  int32_t ncol = 0, cap = 64;
  int64_t* mark = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
  for (int32_t c = 0; c < cap; ++c) mark[c] = -1;
  for (int64_t v = 0; v < N; ++v) colour[v] = -1;
  for (int64_t v = 0; v < N; ++v) {
    for (int pass = 0; pass < 2; ++pass) {
      const int64_t* p = pass ? tptr : ptr;
      const int32_t* q = pass ? tnbr : nbr;
      for (int64_t k = p[v]; k < p[v + 1]; ++k) {
        const int32_t c = colour[q[k]];
        if (q[k] == v || c < 0) continue;
        while (c >= cap) {
          mark = (int64_t*)realloc(mark, sizeof(int64_t) * (size_t)cap * 2);
          for (int32_t x = cap; x < 2 * cap; ++x) mark[x] = -1;
          cap *= 2;
        }
        mark[c] = v;
      }
    }
    int32_t c = 0;
    while (c < cap && mark[c] == v) ++c;
    colour[v] = c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  free(mark);
  free(fill);
  free(tnbr);
  free(tptr);
  return ncol;
}

static void nrm3(double* v) {
  const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= n;
  v[1] /= n;
  v[2] /= n;
}

static double eAe(const oracle_model* m, int64_t i, const double* v) {
  const double* A = m->A + 9 * i;
  return v[0] * (A[0] * v[0] + A[1] * v[1] + A[2] * v[2]) + v[1] * (A[3] * v[0] + A[4] * v[1] + A[5] * v[2]) +
         v[2] * (A[6] * v[0] + A[7] * v[1] + A[8] * v[2]);
}

int64_t oracle_mc_group(const oracle_model* m, const int64_t* idx, int64_t n, int move, const double* beta,
                        double sigma, const double* draws, double* e, int nthreads) {
  double* en = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
  unsigned char* acc = (unsigned char*)malloc((size_t)(n > 0 ? n : 1));
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < n; ++t) {
    const int64_t i = idx[t];
    double h[3];
    hfield(m, i, e, h);
    const double* eo = e + 3 * i;
    double* v = en + 3 * t;
    const double mu = m->mu[i], bt = beta[i];
    double extra = 0.0, ua;
    if (move == 4) {                                    /* reflection about the exchange field */
      const double hh = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
      v[0] = eo[0]; v[1] = eo[1]; v[2] = eo[2];
      if (hh > 1e-14) {
        const double p = 2.0 * ((eo[0] * h[0] + eo[1] * h[1] + eo[2] * h[2]) / hh);
        v[0] = p * h[0] - eo[0];
        v[1] = p * h[1] - eo[1];
        v[2] = p * h[2] - eo[2];
      }
      nrm3(v);
      ua = draws[t];
    } else if (move == 2) {                             /* heat bath of H = 2h + mu_B mu B */
      const double zf = MU_B * mu;
      const double H[3] = {2.0 * h[0] + zf * m->B[0], 2.0 * h[1] + zf * m->B[1], 2.0 * h[2] + zf * m->B[2]};
      const double u1 = draws[t], u2 = draws[n + t];
      ua = draws[2 * n + t];
      const double Hn = sqrt(H[0] * H[0] + H[1] * H[1] + H[2] * H[2]);
      const double x = bt * Hn;
      const int small = x < 1e-8;
      double c = small ? 2.0 * u1 - 1.0 : 1.0 + log1p(-u1 * (-expm1(-2.0 * x))) / x;
      if (c > 1.0) c = 1.0;
      if (c < -1.0) c = -1.0;
      const double ph = 2.0 * M_PI * u2;
      double z[3] = {0.0, 0.0, 1.0};
      if (!small) {
        const double d = Hn > 0 ? Hn : 1.0;
        z[0] = H[0] / d; z[1] = H[1] / d; z[2] = H[2] / d;
      }
      const double a[3] = {fabs(z[0]) < 0.9 ? 1.0 : 0.0, fabs(z[0]) < 0.9 ? 0.0 : 1.0, 0.0};
      double t1[3] = {z[1] * a[2] - z[2] * a[1], z[2] * a[0] - z[0] * a[2], z[0] * a[1] - z[1] * a[0]};
      nrm3(t1);
      const double t2[3] = {z[1] * t1[2] - z[2] * t1[1], z[2] * t1[0] - z[0] * t1[2], z[0] * t1[1] - z[1] * t1[0]};
      const double s = sqrt(1.0 - c * c), cp = cos(ph), sp = sin(ph);
      for (int k = 0; k < 3; ++k) v[k] = c * z[k] + s * (cp * t1[k] + sp * t2[k]);
      nrm3(v);
      extra = (v[0] - eo[0]) * H[0] + (v[1] - eo[1]) * H[1] + (v[2] - eo[2]) * H[2];
    } else {
      const double* g = draws + (move == 3 ? n : 0) + 3 * t;
      if (move == 1) {
        v[0] = g[0]; v[1] = g[1]; v[2] = g[2];
      } else {
        v[0] = eo[0] + sigma * g[0]; v[1] = eo[1] + sigma * g[1]; v[2] = eo[2] + sigma * g[2];
      }
      nrm3(v);
      if (move == 3) {
        const int k = (int)draws[t];
        if (k == 1) {
          const double* f = draws + 4 * n + 3 * t;
          v[0] = f[0]; v[1] = f[1]; v[2] = f[2];
          nrm3(v);
        } else if (k == 2) {
          v[0] = -eo[0]; v[1] = -eo[1]; v[2] = -eo[2];
        }
        ua = draws[7 * n + t];
      } else {
        ua = draws[3 * n + t];
      }
    }
    const double d[3] = {v[0] - eo[0], v[1] - eo[1], v[2] - eo[2]};
    double dE = -2.0 * (d[0] * h[0] + d[1] * h[1] + d[2] * h[2]) -
                MU_B * mu * (d[0] * m->B[0] + d[1] * m->B[1] + d[2] * m->B[2]);
    if (m->A) dE += eAe(m, i, v) - eAe(m, i, eo);
    if (m->Kc) dE += cubic_energy(m, i, v) - cubic_energy(m, i, eo);      /* magex/montecarlo.py:136-137 */
    if (m->K2) dE += uniaxial_energy(m, i, v) - uniaxial_energy(m, i, eo);
    dE += extra;
    int ok = dE <= (move == 4 ? 1e-12 : 0.0);
    if (!ok) {
      double a = dE * bt;
      if (a > 700.0) a = 700.0;
      ok = ua < exp(-a);
    }
    acc[t] = (unsigned char)ok;
  }
  int64_t nacc = 0;
  for (int64_t t = 0; t < n; ++t)
    if (acc[t]) {
      const int64_t i = idx[t];
      e[3 * i] = en[3 * t];
      e[3 * i + 1] = en[3 * t + 1];
      e[3 * i + 2] = en[3 * t + 2];
      ++nacc;
    }
  free(acc);
  free(en);
  return nacc;
}
