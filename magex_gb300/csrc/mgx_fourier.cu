// Device-side Fourier projection of the spins for S(q, w) sampling (magex/spectra.py:49-66):
//
//     m_q = N^-1/2 sum_i e_i exp(-i q.r_i),   r_i = (c0 a0 + c1 a1 + c2 a2) + p_s
//
// magex builds the dense (N, nq) phase matrix and multiplies it on the host every sample.  On a
// supercell the phase factorises, exp(-i q.r) = exp(-i q.p_s) w0(c0) w1(c1) w2(c2) with
// w_a(c) = exp(-2 pi i f_a c) (f = fractional coordinates of q), so the projection is a pruned
// separable DFT evaluated only at the requested wave vectors:
//   stage 1 (k_fourier_rows): P[v][comp][row] = sum_c2 e[comp][row, c2] w2_v(c2) for every distinct
//            f_2 value v, one thread per (chunk of f_2 values, row, comp), twiddles broadcast;
//   stage 2 (k_fourier_q):    m_q[comp] = N^-1/2 sum_{s, c0, c1} exp(-i q.p_s) w0(c0) w1(c1)
//            P[v2(q)][comp][s, c0, c1], one block per q.
// Spins never leave HBM; a sample costs one read of e plus O(nq ns L0 L1) work.
#include <cmath>
#include <map>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx {

struct FourierPlan {
  const Model* model = nullptr;
  int nq = 0;
  int nv2 = 0;
  double2* w0 = nullptr;        // [nv0][L0]
  double2* w1 = nullptr;        // [nv1][L1]
  double2* w2 = nullptr;        // [nv2][L2]
  int4* qidx = nullptr;         // [nq] (v0, v1, v2, 0)
  double2* sub = nullptr;       // [nq][ns] exp(-i q.p_s)
  double2* P = nullptr;         // [nv2][3][rows]
  void* block = nullptr;
};

constexpr int kVChunk = 8;      // f_2 values per pass of stage 1 (accumulators held in registers)

// Stage 1: one thread per (chunk of f_2 values, component, row) walks the row's L2 spins once.  The
// twiddles w2[v][c] are the same for every thread of a warp (one broadcast load); the other chunks'
// threads read the row again from L2.  No cross-lane reduction: two FMAs per (spin, f_2).
__global__ void __launch_bounds__(128) k_fourier_rows(const double* __restrict__ e, long long N, int rows, int L2,
                                                      const double2* __restrict__ w2, int nv2,
                                                      double2* __restrict__ P) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per_chunk = 3LL * rows;
  const int chunk = (int)(t / per_chunk);
  const int v0 = chunk * kVChunk;
  if (v0 >= nv2) return;
  const long long r = t - (long long)chunk * per_chunk;
  const int comp = (int)(r / rows), row = (int)(r - (long long)comp * rows);
  const double* x = e + (long long)comp * N + (long long)row * L2;
  double re[kVChunk], im[kVChunk];
#pragma unroll
  for (int k = 0; k < kVChunk; ++k) re[k] = im[k] = 0.0;
  for (int c = 0; c < L2; ++c) {
    const double xv = __ldg(x + c);
#pragma unroll
    for (int k = 0; k < kVChunk; ++k) {
      if (v0 + k < nv2) {
        const double2 w = __ldg(w2 + (long long)(v0 + k) * L2 + c);
        re[k] = fma(xv, w.x, re[k]);
        im[k] = fma(xv, w.y, im[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kVChunk; ++k)
    if (v0 + k < nv2) P[((long long)(v0 + k) * 3 + comp) * rows + row] = make_double2(re[k], im[k]);
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void __launch_bounds__(256) k_fourier_q(const double2* __restrict__ P, int rows, int ns, int L0, int L1,
                                                   const double2* __restrict__ w0, const double2* __restrict__ w1,
                                                   const int4* __restrict__ qidx, const double2* __restrict__ sub,
                                                   double scale, double* __restrict__ mq) {
  const int q = blockIdx.x;
  const int4 v = qidx[q];
  const double2* Pq = P + (long long)v.z * 3 * rows;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int row = threadIdx.x; row < rows; row += blockDim.x) {
    const int s = row / (L0 * L1);
    const int r = row - s * L0 * L1;
    const int c0 = r / L1, c1 = r - c0 * L1;
    const double2 ph = cmul(cmul(__ldg(sub + (long long)q * ns + s), __ldg(w0 + (long long)v.x * L0 + c0)),
                            __ldg(w1 + (long long)v.y * L1 + c1));
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      const double2 p = __ldg(Pq + (long long)comp * rows + row);
      const double2 t = cmul(ph, p);
      acc[2 * comp] += t.x;
      acc[2 * comp + 1] += t.y;
    }
  }
  __shared__ double red[6][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double a = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[k][wid] = a;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double a = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[threadIdx.x][w];
    mq[(long long)q * 6 + threadIdx.x] = a * scale;
  }
}

}  // namespace mgx

using namespace mgx;

struct mgx_fourier {};

static void fourier_free(FourierPlan* f) {
  if (!f) return;
  cudaFree(f->block);
  cudaFree(f->P);
  delete f;
}

extern "C" mgx_status mgx_fourier_create(const mgx_model* mm, int32_t nq, const double* qfrac, const double* sub_phase,
                                         mgx_fourier** out) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || nq < 1 || !qfrac || !sub_phase || !out) return set_error(MGX_ERR_INVALID, "mgx_fourier_create: bad argument");
  const DevLattice& d = m->d;
  if (d.layout != 0)
    return set_error(MGX_ERR_UNSUPPORTED, "mgx_fourier_create: the separable projection needs a lattice (stencil) model");
  const int L[3] = {d.L0, d.L1, d.L2};
  // distinct fractional coordinates per axis and their phase tables w_a(c) = exp(-2 pi i f c)
  std::vector<std::vector<double>> vals(3);
  std::vector<int4> qi((size_t)nq);
  for (int a = 0; a < 3; ++a) {
    std::map<double, int> index;
    for (int q = 0; q < nq; ++q) {
      const double f = qfrac[3 * q + a];
      if (!std::isfinite(f)) return set_error(MGX_ERR_INVALID, "mgx_fourier_create: q %d is not finite", q);
      auto it = index.find(f);
      int id;
      if (it == index.end()) {
        id = (int)vals[a].size();
        index[f] = id;
        vals[a].push_back(f);
      } else {
        id = it->second;
      }
      (&qi[(size_t)q].x)[a] = id;
    }
  }
  std::vector<double2> tab[3];
  for (int a = 0; a < 3; ++a) {
    tab[a].resize(vals[a].size() * (size_t)L[a]);
    for (size_t v = 0; v < vals[a].size(); ++v)
      for (int c = 0; c < L[a]; ++c) {
        // reduce f c modulo 1 before taking the angle so that large c keep full accuracy
        const double x = vals[a][v] * (double)c;
        const double frac = x - std::floor(x);
        const double ang = -2.0 * M_PI * frac;
        tab[a][v * (size_t)L[a] + (size_t)c] = make_double2(std::cos(ang), std::sin(ang));
      }
  }
  std::vector<double2> sub((size_t)nq * d.ns);
  for (size_t k = 0; k < sub.size(); ++k) sub[k] = make_double2(sub_phase[2 * k], sub_phase[2 * k + 1]);
  FourierPlan* f = new FourierPlan();
  f->model = m;
  f->nq = nq;
  f->nv2 = (int)vals[2].size();
  const size_t n0 = tab[0].size(), n1 = tab[1].size(), n2 = tab[2].size();
  const size_t bytes = sizeof(double2) * (n0 + n1 + n2 + sub.size()) + sizeof(int4) * (size_t)nq;
  cudaError_t err = cudaMalloc(&f->block, bytes);
  const int rows = d.ns * d.L0 * d.L1;
  if (err == cudaSuccess) err = cudaMalloc(&f->P, sizeof(double2) * (size_t)f->nv2 * 3 * rows);
  if (err != cudaSuccess) {
    fourier_free(f);
    return cuda_error(err, "mgx_fourier_create");
  }
  double2* p = (double2*)f->block;
  f->w0 = p;
  f->w1 = p + n0;
  f->w2 = p + n0 + n1;
  f->sub = p + n0 + n1 + n2;
  f->qidx = (int4*)(p + n0 + n1 + n2 + sub.size());
  err = cudaMemcpy(f->w0, tab[0].data(), sizeof(double2) * n0, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(f->w1, tab[1].data(), sizeof(double2) * n1, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(f->w2, tab[2].data(), sizeof(double2) * n2, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(f->sub, sub.data(), sizeof(double2) * sub.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(f->qidx, qi.data(), sizeof(int4) * (size_t)nq, cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    fourier_free(f);
    return cuda_error(err, "mgx_fourier_create");
  }
  *out = reinterpret_cast<mgx_fourier*>(f);
  return MGX_OK;
}

extern "C" mgx_status mgx_fourier_project(mgx_fourier* h, const double* e, double* mq, void* stream) {
  NvtxRange nvtx_range("mgx_fourier_project");
  FourierPlan* f = reinterpret_cast<FourierPlan*>(h);
  if (!f || !e || !mq) return set_error(MGX_ERR_INVALID, "mgx_fourier_project: null argument");
  const DevLattice& d = f->model->d;
  const int rows = d.ns * d.L0 * d.L1;
  cudaStream_t st = (cudaStream_t)stream;
  const long long threads = 3LL * rows * ((f->nv2 + kVChunk - 1) / kVChunk);
  if (threads > 0)
    k_fourier_rows<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(e, d.N, rows, d.L2, f->w2, f->nv2, f->P);
  k_fourier_q<<<f->nq, 256, 0, st>>>(f->P, rows, d.ns, d.L0, d.L1, f->w0, f->w1, f->qidx, f->sub,
                                     1.0 / std::sqrt((double)d.N), mq);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

extern "C" mgx_status mgx_fourier_destroy(mgx_fourier* h) {
  fourier_free(reinterpret_cast<FourierPlan*>(h));
  return MGX_OK;
}
