// Batched ensemble: many independent lattices of uneven size stepped by one persistent launch per
// Heun stage, with a per-system descriptor table and a (system, first site) tile list.
//
// Each system keeps its own stencil, field, damping, thermal amplitude and Philox key, so one batch
// can hold replicas, temperature / field scans and different lattices.  A CTA loops over tiles
// (persistent grid), a tile is `threads` consecutive sites of one system, so the system descriptor
// and the coupling width are uniform inside a block.  Spins of system k occupy the (3, N_k)
// lattice-layout block starting at 3 * offset_k doubles of one device array.
//
// The step loop can be captured into a CUDA graph (chunks of G steps); the Philox step index is
// then read from a device counter that a one-thread kernel at the end of each chunk advances, so
// replays of the same graph draw fresh noise.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "mgx_fx_step.cuh"
#include "mgx_observe.cuh"

namespace mgx {

struct BatchSys {
  DevLattice L;
  DevLLG P;
  long long off3;   // offset of the system's spin block in doubles (3 * site offset)
  DevFX F;          // fixed-point gather tables and split arrays (MGX_PRECISION_FP64_FIXED_GATHER)
};

struct StepArg {
  const unsigned long long* base;   // device counter (graph replays) or nullptr
  unsigned long long add;
  __device__ __forceinline__ uint64_t value() const { return (base ? *base : 0ull) + add; }
};

struct Batch {
  int nsys = 0;
  std::vector<const Model*> models;
  std::vector<BatchSys> host_sys;
  std::vector<long long> offset;      // site offsets, nsys + 1
  long long ntot = 0;
  int noise = MGX_NOISE_NONE;
  int integrator = MGX_INTEGRATOR_HEUN;
  int threads = 256;
  int ctas_per_sm = 0;                // 0: one CTA per tile (no persistence)
  int sms = 152;
  BatchSys* d_sys = nullptr;
  int2* d_tiles = nullptr;
  int ntiles = 0;
  std::vector<int> tile_begin;        // first tile of each system, nsys + 1
  int* d_tile_begin = nullptr;
  double* scratch = nullptr;          // ep | k1 of all systems (6 * ntot)
  double* sub = nullptr;              // per system: alpha | pre | sigma per sublattice (3 * 16)
  unsigned long long* d_step = nullptr;
  double* partials = nullptr;
  int partial_cap = 0;
  // topological charge
  int* d_tri = nullptr;
  double* d_orient = nullptr;
  long long ntri = 0;
  int2* d_tri_tiles = nullptr;
  int* d_tri_tile_begin = nullptr;
  long long* d_tri_off = nullptr;
  int ntri_tiles = 0;
  double* tri_partials = nullptr;
  // captured step loop
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_chunk = 0;
  const double* graph_e = nullptr;
  int graph_threads = 0, graph_grid = 0;
  // exact fixed-point exchange sums (every system of the batch, or none)
  bool fixed = false;
  // cubic / higher-uniaxial terms in at least one system: the HIGHER stage instantiation
  bool higher = false;
  std::vector<void*> fx_blocks;
  int2* fx_split = nullptr;           // es | eps of all systems (2 * 3 * ntot)
};

constexpr int BATCH_MAX_THREADS = 512;

// HIGHER: a separate instantiation for batches with cubic / higher-uniaxial terms (in any system), so
// that the plain stage kernels keep their registers.
// At least two CTAs of the largest tile per SM, i.e. at most 64 registers: the fixed-point-sum bodies
// otherwise take 86-98 registers, and the occupancy lost costs more than the few spills (measured on
// the 256-film ensemble: 1.26 against 1.68 ms per step; the FP64 bodies use 64 either way).
template <int STAGE, int NOISE, int INTEG, bool FIXED, bool HIGHER>
__global__ void __launch_bounds__(BATCH_MAX_THREADS, 2) k_batch_stage(const BatchSys* __restrict__ sys,
                                                                   const int2* __restrict__ tiles, int ntiles,
                                                                   double* __restrict__ e,
                                                                   const double* __restrict__ noise, StepArg step) {
  const uint64_t st = step.value();
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int2 tl = tiles[t];
    const BatchSys& S = sys[tl.x];
    const long long q = (long long)tl.y + threadIdx.x;
    if (q >= S.L.N) continue;
    double* es = e + S.off3;
    const double* ns = noise ? noise + S.off3 : nullptr;
    if (FIXED) {
      if (STAGE == 0)
        fx_predict_site<NOISE, INTEG, MGX_PRECISION_FP64_FIXED_GATHER, HIGHER, 0>(S.L, S.P, S.F, es, ns, q, st);
      else
        fx_correct_site<NOISE, INTEG, MGX_PRECISION_FP64_FIXED_GATHER, HIGHER, 0>(S.L, S.P, S.F, es, ns, q, st);
      continue;
    }
    // the EXTRA bodies add the higher on-site fields (the spin-orbit torque and per-site extra field
    // pointers of a batched system are null)
    const int W = S.L.width;
    if (STAGE == 0) {
      if (W == 1) predict_site<1, NOISE, INTEG, HIGHER>(S.L, S.P, es, ns, q, st);
      else if (W == 4) predict_site<4, NOISE, INTEG, HIGHER>(S.L, S.P, es, ns, q, st);
      else predict_site<9, NOISE, INTEG, HIGHER>(S.L, S.P, es, ns, q, st);
    } else {
      if (W == 1) correct_site<1, NOISE, INTEG, HIGHER>(S.L, S.P, es, ns, q, st);
      else if (W == 4) correct_site<4, NOISE, INTEG, HIGHER>(S.L, S.P, es, ns, q, st);
      else correct_site<9, NOISE, INTEG, HIGHER>(S.L, S.P, es, ns, q, st);
    }
  }
}

__global__ void k_step_set(unsigned long long* c, unsigned long long v) { *c = v; }
__global__ void k_step_advance(unsigned long long* c, unsigned long long n) { *c += n; }

// per-tile partial observables (one block per tile, blockDim == tile size)
__global__ void __launch_bounds__(BATCH_MAX_THREADS) k_batch_observe(const BatchSys* __restrict__ sys,
                                                                     const int2* __restrict__ tiles,
                                                                     const double* __restrict__ e,
                                                                     double* __restrict__ partial) {
  const int2 tl = tiles[blockIdx.x];
  const BatchSys& S = sys[tl.x];
  const long long q = (long long)tl.y + threadIdx.x;
  double v[OBS_NV] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (q < S.L.N) {
    const double* es = e + S.off3;
    if (S.L.width == 1) observe_site<1>(S.L, es, q, v);
    else if (S.L.width == 4) observe_site<4>(S.L, es, q, v);
    else observe_site<9>(S.L, es, q, v);
  }
  __shared__ double red[BATCH_MAX_THREADS / 32][OBS_NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < OBS_NV - 1; ++k) v[k] = warp_sum(v[k]);
  v[7] = warp_max(v[7]);
  if (lane == 0)
    for (int k = 0; k < OBS_NV; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < OBS_NV) {
    const int k = threadIdx.x;
    double acc = red[0][k];
    for (int w = 1; w < nw; ++w) acc = (k == 7) ? fmax(acc, red[w][k]) : acc + red[w][k];
    partial[(long long)blockIdx.x * OBS_NV + k] = acc;
  }
}

// one block per system: reduce its tiles in order
__global__ void __launch_bounds__(256) k_batch_obs_finish(const int* __restrict__ tile_begin,
                                                          const double* __restrict__ partial, double* out) {
  const int sys = blockIdx.x;
  const int t0 = tile_begin[sys], t1 = tile_begin[sys + 1];
  double v[OBS_NV] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x)
    for (int k = 0; k < OBS_NV; ++k) {
      const double x = partial[(long long)t * OBS_NV + k];
      v[k] = (k == 7) ? fmax(v[k], x) : v[k] + x;
    }
  __shared__ double red[8][OBS_NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < OBS_NV - 1; ++k) v[k] = warp_sum(v[k]);
  v[7] = warp_max(v[7]);
  if (lane == 0)
    for (int k = 0; k < OBS_NV; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < OBS_NV) {
    const int k = threadIdx.x;
    double acc = red[0][k];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) acc = (k == 7) ? fmax(acc, red[w][k]) : acc + red[w][k];
    out[(long long)sys * OBS_NV + k] = acc;
  }
}

// per-tile solid-angle sums: tile = 256 consecutive triangles of one system
__global__ void __launch_bounds__(256) k_batch_solid(const BatchSys* __restrict__ sys, const int2* __restrict__ tiles,
                                                     const long long* __restrict__ tri_off,
                                                     const int* __restrict__ tri, const double* __restrict__ orient,
                                                     const double* __restrict__ e, double* __restrict__ partial) {
  const int2 tl = tiles[blockIdx.x];
  const BatchSys& S = sys[tl.x];
  const long long t = tri_off[tl.x] + tl.y + threadIdx.x;
  double acc = 0.0;
  if (t < tri_off[tl.x + 1])
    acc = solid_angle(e + S.off3, S.L.N, tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]) * orient[t];
  __shared__ double red[8];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void k_batch_solid_reduce(const int* __restrict__ tile_begin, const double* __restrict__ partial,
                                     int nsys, double* out) {
  const int sys = blockIdx.x * blockDim.x + threadIdx.x;
  if (sys >= nsys) return;
  double s = 0.0;
  for (int t = tile_begin[sys]; t < tile_begin[sys + 1]; ++t) s += partial[t];
  out[sys] = s / (4.0 * 3.14159265358979323846);
}

static mgx_status build_tiles(Batch* b) {
  std::vector<int2> tiles;
  b->tile_begin.assign(b->nsys + 1, 0);
  for (int k = 0; k < b->nsys; ++k) {
    b->tile_begin[k] = (int)tiles.size();
    const long long N = b->host_sys[k].L.N;
    for (long long s0 = 0; s0 < N; s0 += b->threads) tiles.push_back(make_int2(k, (int)s0));
  }
  b->tile_begin[b->nsys] = (int)tiles.size();
  cudaFree(b->d_tiles);
  cudaFree(b->d_tile_begin);
  b->d_tiles = nullptr;
  b->d_tile_begin = nullptr;
  b->ntiles = (int)tiles.size();
  MGX_CUDA_TRY(cudaMalloc(&b->d_tiles, sizeof(int2) * std::max<size_t>(tiles.size(), 1)));
  MGX_CUDA_TRY(cudaMalloc(&b->d_tile_begin, sizeof(int) * (b->nsys + 1)));
  MGX_CUDA_TRY(cudaMemcpy(b->d_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(b->d_tile_begin, b->tile_begin.data(), sizeof(int) * (b->nsys + 1), cudaMemcpyHostToDevice));
  return MGX_OK;
}

static int grid_size(const Batch* b) {
  if (b->ctas_per_sm <= 0) return std::max(b->ntiles, 1);
  return std::max(1, std::min(b->ntiles, b->ctas_per_sm * b->sms));
}

template <int NOISE, int INTEG, bool FIXED, bool HIGHER>
static void enqueue_batch_form(const Batch* b, double* e, const double* noise, StepArg step, cudaStream_t st) {
  const int grid = grid_size(b);
  k_batch_stage<0, NOISE, INTEG, FIXED, HIGHER><<<grid, b->threads, 0, st>>>(b->d_sys, b->d_tiles, b->ntiles, e,
                                                                             noise, step);
  k_batch_stage<1, NOISE, INTEG, FIXED, HIGHER><<<grid, b->threads, 0, st>>>(b->d_sys, b->d_tiles, b->ntiles, e,
                                                                             noise, step);
}

template <int NOISE, int INTEG>
static void enqueue_batch(const Batch* b, double* e, const double* noise, StepArg step, cudaStream_t st) {
  if (b->fixed) {
    if (b->higher) enqueue_batch_form<NOISE, INTEG, true, true>(b, e, noise, step, st);
    else enqueue_batch_form<NOISE, INTEG, true, false>(b, e, noise, step, st);
  } else {
    if (b->higher) enqueue_batch_form<NOISE, INTEG, false, true>(b, e, noise, step, st);
    else enqueue_batch_form<NOISE, INTEG, false, false>(b, e, noise, step, st);
  }
}

static void enqueue_batch_step(const Batch* b, double* e, const double* noise, StepArg step, cudaStream_t st) {
  const bool dep = b->integrator == MGX_INTEGRATOR_DEPONDT;
  switch (b->noise) {
    case MGX_NOISE_HOST:
      dep ? enqueue_batch<MGX_NOISE_HOST, MGX_INTEGRATOR_DEPONDT>(b, e, noise, step, st)
          : enqueue_batch<MGX_NOISE_HOST, MGX_INTEGRATOR_HEUN>(b, e, noise, step, st);
      break;
    case MGX_NOISE_PHILOX:
      dep ? enqueue_batch<MGX_NOISE_PHILOX, MGX_INTEGRATOR_DEPONDT>(b, e, noise, step, st)
          : enqueue_batch<MGX_NOISE_PHILOX, MGX_INTEGRATOR_HEUN>(b, e, noise, step, st);
      break;
    default:
      dep ? enqueue_batch<MGX_NOISE_NONE, MGX_INTEGRATOR_DEPONDT>(b, e, noise, step, st)
          : enqueue_batch<MGX_NOISE_NONE, MGX_INTEGRATOR_HEUN>(b, e, noise, step, st);
      break;
  }
}

static void drop_graph(Batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_chunk = 0;
  b->graph_e = nullptr;
}

static mgx_status upload_sys(Batch* b) {
  MGX_CUDA_TRY(cudaMemcpy(b->d_sys, b->host_sys.data(), sizeof(BatchSys) * b->nsys, cudaMemcpyHostToDevice));
  return MGX_OK;
}

}  // namespace mgx

using namespace mgx;

extern "C" {

mgx_status mgx_batch_create(const mgx_model* const* models, const mgx_llg_params* params, int32_t nsys,
                            mgx_batch** out) {
  if (!models || !params || !out || nsys <= 0) return set_error(MGX_ERR_INVALID, "mgx_batch_create: bad argument");
  *out = nullptr;
  for (int k = 0; k < nsys; ++k) {
    if (!models[k]) return set_error(MGX_ERR_INVALID, "mgx_batch_create: model %d is null", k);
    const mgx_llg_params& p = params[k];
    if (!(p.dt > 0.0)) return set_error(MGX_ERR_INVALID, "system %d: dt must be positive", k);
    if (p.alpha_site) return set_error(MGX_ERR_INVALID, "system %d: batched systems take a uniform alpha", k);
    if (p.precision != params[0].precision)
      return set_error(MGX_ERR_INVALID, "all systems of a batch share the precision form");
    if (p.precision != MGX_PRECISION_FP64 && p.precision != MGX_PRECISION_FP64_FIXED_GATHER)
      return set_error(MGX_ERR_UNSUPPORTED, "batched systems use the FP64 (0) or FP64 fixed-point-gather (3) form");
    if (p.noise != params[0].noise || p.integrator != params[0].integrator)
      return set_error(MGX_ERR_INVALID, "all systems of a batch share the noise mode and the integrator");
    if (p.integrator != MGX_INTEGRATOR_HEUN && p.integrator != MGX_INTEGRATOR_DEPONDT)
      return set_error(MGX_ERR_INVALID, "integrator %d is not heun (0) or depondt (1)", p.integrator);
    if (p.noise < MGX_NOISE_NONE || p.noise > MGX_NOISE_PHILOX)
      return set_error(MGX_ERR_INVALID, "noise mode %d is not none, host or philox", p.noise);
  }
  Batch* b = new Batch();
  b->nsys = nsys;
  b->noise = params[0].noise;
  b->integrator = params[0].integrator;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  b->offset.assign(nsys + 1, 0);
  for (int k = 0; k < nsys; ++k) {
    const Model* m = reinterpret_cast<const Model*>(models[k]);
    b->models.push_back(m);
    b->offset[k + 1] = b->offset[k] + m->d.N;
    b->higher |= has_higher_onsite(m->d);
  }
  b->ntot = b->offset[nsys];
  const double gamma = 0.1760859630;
  std::vector<double> sub((size_t)nsys * 3 * MGX_MAX_SUBLATTICES, 0.0);
  cudaError_t err = cudaMalloc(&b->scratch, sizeof(double) * 6 * (size_t)b->ntot);
  if (err == cudaSuccess) err = cudaMalloc(&b->sub, sizeof(double) * sub.size());
  if (err == cudaSuccess) err = cudaMalloc(&b->d_sys, sizeof(BatchSys) * nsys);
  if (err == cudaSuccess) err = cudaMalloc(&b->d_step, sizeof(unsigned long long));
  if (err != cudaSuccess) {
    mgx_batch_destroy(reinterpret_cast<mgx_batch*>(b));
    return cuda_error(err, "mgx_batch_create");
  }
  b->host_sys.resize(nsys);
  for (int k = 0; k < nsys; ++k) {
    const Model* m = b->models[k];
    const mgx_llg_params& p = params[k];
    BatchSys& S = b->host_sys[k];
    S.L = m->d;
    S.off3 = 3 * b->offset[k];
    double* sk = b->sub + (size_t)k * 3 * MGX_MAX_SUBLATTICES;
    for (int s = 0; s < m->d.ns; ++s) {
      sub[(size_t)k * 3 * MGX_MAX_SUBLATTICES + s] = p.alpha;
      sub[(size_t)k * 3 * MGX_MAX_SUBLATTICES + MGX_MAX_SUBLATTICES + s] = -gamma / (1.0 + p.alpha * p.alpha);
    }
    DevLLG& d = S.P;
    d.dt = p.dt;
    d.half_dt = 0.5 * p.dt;
    d.precession = p.precession ? 1 : 0;
    d.noise = p.noise;
    d.integrator = p.integrator;
    d.seed = p.seed;
    d.alpha_sub = sk;
    d.pre_sub = sk + MGX_MAX_SUBLATTICES;
    d.sigma_sub = sk + 2 * MGX_MAX_SUBLATTICES;
    d.alpha_site = d.pre_site = d.sigma_site = nullptr;
    d.ep = b->scratch + 3 * b->offset[k];
    d.k1 = b->scratch + 3 * b->ntot + 3 * b->offset[k];
  }
  err = cudaMemcpy(b->sub, sub.data(), sizeof(double) * sub.size(), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    mgx_batch_destroy(reinterpret_cast<mgx_batch*>(b));
    return cuda_error(err, "mgx_batch_create params");
  }
  if (params[0].precision == MGX_PRECISION_FP64_FIXED_GATHER) {
    b->fixed = true;
    err = cudaMalloc(&b->fx_split, sizeof(int2) * 6 * (size_t)b->ntot);
    if (err != cudaSuccess) {
      mgx_batch_destroy(reinterpret_cast<mgx_batch*>(b));
      return cuda_error(err, "mgx_batch_create fixed-point split");
    }
    for (int k = 0; k < nsys; ++k) {
      BatchSys& S = b->host_sys[k];
      void* blk = nullptr;
      const mgx_status fst = fx_build(b->models[k], 28, true, 0, &S.F, &blk);
      if (blk) b->fx_blocks.push_back(blk);
      if (fst != MGX_OK) {
        mgx_batch_destroy(reinterpret_cast<mgx_batch*>(b));
        return fst;
      }
      S.F.es = b->fx_split + 3 * b->offset[k];
      S.F.eps = b->fx_split + 3 * b->ntot + 3 * b->offset[k];
    }
  }
  mgx_status st = upload_sys(b);
  if (st == MGX_OK) st = build_tiles(b);
  if (st != MGX_OK) {
    mgx_batch_destroy(reinterpret_cast<mgx_batch*>(b));
    return st;
  }
  *out = reinterpret_cast<mgx_batch*>(b);
  return MGX_OK;
}

mgx_status mgx_batch_destroy(mgx_batch* bb) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b) return MGX_OK;
  drop_graph(b);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  cudaFree(b->d_sys);
  cudaFree(b->d_tiles);
  cudaFree(b->d_tile_begin);
  cudaFree(b->scratch);
  cudaFree(b->sub);
  cudaFree(b->d_step);
  cudaFree(b->partials);
  cudaFree(b->d_tri);
  cudaFree(b->d_orient);
  cudaFree(b->d_tri_tiles);
  cudaFree(b->d_tri_tile_begin);
  cudaFree(b->d_tri_off);
  cudaFree(b->tri_partials);
  for (void* p : b->fx_blocks) cudaFree(p);
  cudaFree(b->fx_split);
  delete b;
  return MGX_OK;
}

int64_t mgx_batch_nsites(const mgx_batch* bb) {
  const Batch* b = reinterpret_cast<const Batch*>(bb);
  return b ? (int64_t)b->ntot : -1;
}

int64_t mgx_batch_offset(const mgx_batch* bb, int32_t sys) {
  const Batch* b = reinterpret_cast<const Batch*>(bb);
  if (!b || sys < 0 || sys > b->nsys) return -1;
  return (int64_t)b->offset[sys];
}

mgx_status mgx_batch_set_sigma(mgx_batch* bb, int32_t sys, const double* sigma_sub) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b || !sigma_sub || sys < 0 || sys >= b->nsys) return set_error(MGX_ERR_INVALID, "mgx_batch_set_sigma: bad argument");
  const int ns = b->host_sys[sys].L.ns;
  for (int s = 0; s < ns; ++s)
    if (!std::isfinite(sigma_sub[s]) || sigma_sub[s] < 0.0)
      return set_error(MGX_ERR_INVALID, "sigma_sub must be finite and >= 0");
  MGX_CUDA_TRY(cudaMemcpy(b->sub + (size_t)sys * 3 * MGX_MAX_SUBLATTICES + 2 * MGX_MAX_SUBLATTICES, sigma_sub,
                          sizeof(double) * ns, cudaMemcpyHostToDevice));
  return MGX_OK;
}

mgx_status mgx_batch_sync_models(mgx_batch* bb) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b) return set_error(MGX_ERR_INVALID, "mgx_batch_sync_models: null batch");
  for (int k = 0; k < b->nsys; ++k) b->host_sys[k].L = b->models[k]->d;
  return upload_sys(b);
}

mgx_status mgx_batch_set_launch(mgx_batch* bb, int32_t threads, int32_t ctas_per_sm) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b) return set_error(MGX_ERR_INVALID, "mgx_batch_set_launch: null batch");
  if (threads != 64 && threads != 128 && threads != 256 && threads != 512)
    return set_error(MGX_ERR_INVALID, "threads per tile must be 64, 128, 256 or 512");
  if (ctas_per_sm < 0 || ctas_per_sm > 64) return set_error(MGX_ERR_INVALID, "ctas_per_sm must be in 0..64");
  drop_graph(b);
  b->ctas_per_sm = ctas_per_sm;
  if (threads != b->threads) {
    b->threads = threads;
    mgx_status st = build_tiles(b);
    if (st != MGX_OK) return st;
  }
  return MGX_OK;
}

mgx_status mgx_batch_step(mgx_batch* bb, double* e, const double* noise, uint64_t step, void* stream) {
  NvtxRange nvtx_range("mgx_batch_step");
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b || !e) return set_error(MGX_ERR_INVALID, "mgx_batch_step: null argument");
  if (b->noise == MGX_NOISE_HOST && !noise) return set_error(MGX_ERR_INVALID, "host-noise batch needs a noise buffer");
  if (b->fixed) enqueue_fx_split_n(e, b->fx_split, 3 * b->ntot, 28, (cudaStream_t)stream);
  enqueue_batch_step(b, e, noise, StepArg{nullptr, step}, (cudaStream_t)stream);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_batch_run(mgx_batch* bb, double* e, int64_t nsteps, uint64_t step0, int32_t graph_chunk, void* stream) {
  NvtxRange nvtx_range("mgx_batch_run");
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b || !e) return set_error(MGX_ERR_INVALID, "mgx_batch_run: null argument");
  if (nsteps < 0) return set_error(MGX_ERR_INVALID, "nsteps must be >= 0");
  if (b->noise == MGX_NOISE_HOST) return set_error(MGX_ERR_INVALID, "host-noise batches step one at a time");
  cudaStream_t st = (cudaStream_t)stream;
  if (b->fixed && nsteps > 0) enqueue_fx_split_n(e, b->fx_split, 3 * b->ntot, 28, st);
  int64_t done = 0;
  if (graph_chunk > 0 && nsteps >= graph_chunk) {
    if (!b->graph || b->graph_chunk != graph_chunk || b->graph_e != e || b->graph_threads != b->threads ||
        b->graph_grid != grid_size(b)) {
      drop_graph(b);
      if (!b->cap_stream) MGX_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
      MGX_CUDA_TRY(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < graph_chunk; ++k) enqueue_batch_step(b, e, nullptr, StepArg{b->d_step, (unsigned long long)k}, b->cap_stream);
      k_step_advance<<<1, 1, 0, b->cap_stream>>>(b->d_step, (unsigned long long)graph_chunk);
      cudaGraph_t g = nullptr;
      cudaError_t err = cudaStreamEndCapture(b->cap_stream, &g);
      if (err != cudaSuccess) return cuda_error(err, "mgx_batch_run capture");
      err = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (err != cudaSuccess) { b->graph = nullptr; return cuda_error(err, "mgx_batch_run instantiate"); }
      b->graph_chunk = graph_chunk;
      b->graph_e = e;
      b->graph_threads = b->threads;
      b->graph_grid = grid_size(b);
    }
    k_step_set<<<1, 1, 0, st>>>(b->d_step, (unsigned long long)step0);
    for (; done + graph_chunk <= nsteps; done += graph_chunk) MGX_CUDA_TRY(cudaGraphLaunch(b->graph, st));
  }
  for (; done < nsteps; ++done) enqueue_batch_step(b, e, nullptr, StepArg{nullptr, step0 + (uint64_t)done}, st);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_batch_observables(mgx_batch* bb, const double* e, double* out, void* stream) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b || !e || !out) return set_error(MGX_ERR_INVALID, "mgx_batch_observables: null argument");
  if (b->partial_cap < b->ntiles) {
    cudaFree(b->partials);
    b->partials = nullptr;
    b->partial_cap = 0;
    MGX_CUDA_TRY(cudaMalloc(&b->partials, sizeof(double) * OBS_NV * (size_t)b->ntiles));
    b->partial_cap = b->ntiles;
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_batch_observe<<<b->ntiles, b->threads, 0, st>>>(b->d_sys, b->d_tiles, e, b->partials);
  k_batch_obs_finish<<<b->nsys, 256, 0, st>>>(b->d_tile_begin, b->partials, out);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_batch_set_triangles(mgx_batch* bb, const int32_t* tri, const double* orient, const int64_t* tri_off) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b || !tri_off) return set_error(MGX_ERR_INVALID, "mgx_batch_set_triangles: null argument");
  if (tri_off[0] != 0) return set_error(MGX_ERR_INVALID, "triangle offsets must start at 0");
  const long long ntri = tri_off[b->nsys];
  if (ntri > 0 && (!tri || !orient)) return set_error(MGX_ERR_INVALID, "mgx_batch_set_triangles: null triangle arrays");
  std::vector<int2> tiles;
  std::vector<int> tb(b->nsys + 1, 0);
  for (int k = 0; k < b->nsys; ++k) {
    if (tri_off[k + 1] < tri_off[k]) return set_error(MGX_ERR_INVALID, "triangle offsets must be non-decreasing");
    for (long long t = tri_off[k]; t < tri_off[k + 1]; ++t)
      for (int v = 0; v < 3; ++v)
        if (tri[3 * t + v] < 0 || tri[3 * t + v] >= b->host_sys[k].L.N)
          return set_error(MGX_ERR_INVALID, "triangle %lld of system %d has a vertex outside the system", t, k);
    tb[k] = (int)tiles.size();
    for (long long s0 = 0; s0 < tri_off[k + 1] - tri_off[k]; s0 += 256) tiles.push_back(make_int2(k, (int)s0));
  }
  tb[b->nsys] = (int)tiles.size();
  cudaFree(b->d_tri);
  cudaFree(b->d_orient);
  cudaFree(b->d_tri_tiles);
  cudaFree(b->d_tri_tile_begin);
  cudaFree(b->d_tri_off);
  cudaFree(b->tri_partials);
  b->d_tri = nullptr;
  b->d_orient = nullptr;
  b->d_tri_tiles = nullptr;
  b->d_tri_tile_begin = nullptr;
  b->d_tri_off = nullptr;
  b->tri_partials = nullptr;
  b->ntri = ntri;
  b->ntri_tiles = (int)tiles.size();
  MGX_CUDA_TRY(cudaMalloc(&b->d_tri, sizeof(int) * 3 * std::max(ntri, 1LL)));
  MGX_CUDA_TRY(cudaMalloc(&b->d_orient, sizeof(double) * std::max(ntri, 1LL)));
  MGX_CUDA_TRY(cudaMalloc(&b->d_tri_tiles, sizeof(int2) * std::max<size_t>(tiles.size(), 1)));
  MGX_CUDA_TRY(cudaMalloc(&b->d_tri_tile_begin, sizeof(int) * (b->nsys + 1)));
  MGX_CUDA_TRY(cudaMalloc(&b->d_tri_off, sizeof(long long) * (b->nsys + 1)));
  MGX_CUDA_TRY(cudaMalloc(&b->tri_partials, sizeof(double) * std::max<size_t>(tiles.size(), 1)));
  if (ntri > 0) {
    MGX_CUDA_TRY(cudaMemcpy(b->d_tri, tri, sizeof(int) * 3 * ntri, cudaMemcpyHostToDevice));
    MGX_CUDA_TRY(cudaMemcpy(b->d_orient, orient, sizeof(double) * ntri, cudaMemcpyHostToDevice));
  }
  if (!tiles.empty())
    MGX_CUDA_TRY(cudaMemcpy(b->d_tri_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice));
  MGX_CUDA_TRY(cudaMemcpy(b->d_tri_tile_begin, tb.data(), sizeof(int) * (b->nsys + 1), cudaMemcpyHostToDevice));
  static_assert(sizeof(long long) == sizeof(int64_t), "offsets are 64-bit");
  MGX_CUDA_TRY(cudaMemcpy(b->d_tri_off, tri_off, sizeof(long long) * (b->nsys + 1), cudaMemcpyHostToDevice));
  return MGX_OK;
}

mgx_status mgx_batch_topological_charge(mgx_batch* bb, const double* e, double* out, void* stream) {
  Batch* b = reinterpret_cast<Batch*>(bb);
  if (!b || !e || !out) return set_error(MGX_ERR_INVALID, "mgx_batch_topological_charge: null argument");
  if (!b->d_tri_off) return set_error(MGX_ERR_INVALID, "mgx_batch_topological_charge: call mgx_batch_set_triangles first");
  cudaStream_t st = (cudaStream_t)stream;
  if (b->ntri_tiles > 0)
    k_batch_solid<<<b->ntri_tiles, 256, 0, st>>>(b->d_sys, b->d_tri_tiles, b->d_tri_off, b->d_tri, b->d_orient, e,
                                                  b->tri_partials);
  k_batch_solid_reduce<<<(b->nsys + 127) / 128, 128, 0, st>>>(b->d_tri_tile_begin, b->tri_partials, b->nsys, out);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

}  // extern "C"
