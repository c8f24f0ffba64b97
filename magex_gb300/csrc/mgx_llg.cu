// Fused stochastic Heun (and Depondt) LLG step on the lattice stencil: predictor and corrector kernels.
//
// Reference behaviour: magex/llg.py:216-227 (NumPy Heun), magex/fast.py:336-390 (fused predictor /
// corrector, numba), magex/cuda_backend.py:144-218 (numba.cuda twins).  One thread owns one site.
// The predictor gathers the exchange field from e, adds on-site, Zeeman and thermal fields, stores
// k1 and the normalised predicted spin ep; the corrector gathers from ep and writes e in place
// (it reads only its own e, so the in-place update is race-free).
#include <algorithm>
#include <cmath>
#include <vector>

#include "mgx_step.cuh"

namespace mgx {

// Sites begin + i (i < count) of sublattice blockIdx.y: the whole lattice is one row of N sites
// (gridDim.y = 1, begin = 0), a range of cells one row of `count` cells per sublattice.
template <int W, int NOISE, int INTEG, bool EXTRA>
__global__ void __launch_bounds__(256) k_predict(const DevLattice L, const DevLLG P, const double* __restrict__ e,
                                                 const double* __restrict__ noise, uint64_t step, long long begin,
                                                 long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count)
    predict_site<W, NOISE, INTEG, EXTRA>(L, P, e, noise, (long long)blockIdx.y * L.ncell + begin + i,
                                  P.step_base ? *P.step_base + step : step);
}

template <int W, int NOISE, int INTEG, bool EXTRA>
__global__ void __launch_bounds__(256) k_correct(const DevLattice L, const DevLLG P, double* __restrict__ e,
                                                 const double* __restrict__ noise, uint64_t step, long long begin,
                                                 long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count)
    correct_site<W, NOISE, INTEG, EXTRA>(L, P, e, noise, (long long)blockIdx.y * L.ncell + begin + i,
                                  P.step_base ? *P.step_base + step : step);
}

// Cells [cb, cb + cn) of every sublattice (cn = ncell: the whole lattice in one row).
struct CellRange {
  long long cb, cn;
};

// stages: bit 0 = predictor, bit 1 = corrector
template <int W, int NOISE, int INTEG>
static void launch_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages,
                        cudaStream_t st, CellRange r) {
  const DevLattice& L = pl->model->d;
  const bool whole = r.cb == 0 && r.cn == L.ncell;
  const long long count = whole ? L.N : r.cn;
  const int tpb = site_block_size(whole ? L.N : r.cn * L.ns);
  const dim3 grid((unsigned)((count + tpb - 1) / tpb), whole ? 1u : (unsigned)L.ns);
  if (pl->p.sot || pl->p.B_add || has_higher_onsite(L)) {
    if (stages & 1) k_predict<W, NOISE, INTEG, true><<<grid, tpb, 0, st>>>(L, pl->p, e, noise, step, r.cb, count);
    if (stages & 2) k_correct<W, NOISE, INTEG, true><<<grid, tpb, 0, st>>>(L, pl->p, e, noise, step, r.cb, count);
  } else {
    if (stages & 1) k_predict<W, NOISE, INTEG, false><<<grid, tpb, 0, st>>>(L, pl->p, e, noise, step, r.cb, count);
    if (stages & 2) k_correct<W, NOISE, INTEG, false><<<grid, tpb, 0, st>>>(L, pl->p, e, noise, step, r.cb, count);
  }
}

template <int W, int NOISE>
static void dispatch_integ(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages,
                           cudaStream_t st, CellRange r) {
  if (pl->p.integrator == MGX_INTEGRATOR_DEPONDT)
    launch_step<W, NOISE, MGX_INTEGRATOR_DEPONDT>(pl, e, noise, step, stages, st, r);
  else
    launch_step<W, NOISE, MGX_INTEGRATOR_HEUN>(pl, e, noise, step, stages, st, r);
}

template <int W>
static void dispatch_noise(const LLGPlan* pl, double* e, const double* noise, uint64_t step, int stages,
                           cudaStream_t st, CellRange r) {
  // sigma = 0 everywhere: the thermal field is exactly zero, skip generating it
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  switch (mode) {
    case MGX_NOISE_HOST: dispatch_integ<W, MGX_NOISE_HOST>(pl, e, noise, step, stages, st, r); break;
    case MGX_NOISE_PHILOX: dispatch_integ<W, MGX_NOISE_PHILOX>(pl, e, noise, step, stages, st, r); break;
    default: dispatch_integ<W, MGX_NOISE_NONE>(pl, e, noise, step, stages, st, r); break;
  }
}

// FP64 stages on the cells [r.cb, r.cb + r.cn) of every sublattice
static void enqueue_fp64_range(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st,
                               int stages, CellRange r) {
  switch (pl->model->d.width) {
    case 1: dispatch_noise<1>(pl, e, noise, step, stages, st, r); break;
    case 4: dispatch_noise<4>(pl, e, noise, step, stages, st, r); break;
    default: dispatch_noise<9>(pl, e, noise, step, stages, st, r); break;
  }
}

void enqueue_llg_step(const LLGPlan* pl, double* e, const double* noise, uint64_t step, cudaStream_t st,
                      int stages) {
  if (pl->precision == MGX_PRECISION_INT48_GATHER || pl->precision == MGX_PRECISION_FP64_FIXED_GATHER) {
    enqueue_fx_step(pl, e, noise, step, st, stages);
    return;
  }
  if (pl->precision == MGX_PRECISION_DF32_GATHER) {
    enqueue_df_step(pl, e, noise, step, st, stages);
    return;
  }
  enqueue_fp64_range(pl, e, noise, step, st, stages, CellRange{0, pl->model->d.ncell});
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

// Small lattices are launch-bound: mgx_llg_run replays CUDA graphs of kGraphChunk steps whose kernels
// read the Philox step index from a device counter (advanced by a one-thread kernel at the end of the
// graph), so every replay draws fresh noise and the trajectory equals the directly launched one.  A
// shorter tail of k >= kGraphMinTail steps is captured as a graph of its own once the same k comes
// twice in a row (callers that step in fixed chunks of a few steps between checks or samples).
constexpr long long kGraphMaxSites = 1LL << 21;
constexpr int kGraphChunk = 32;
constexpr int kGraphMinTail = 4;

__global__ void k_llg_step_set(unsigned long long* c, unsigned long long v) { *c = v; }
__global__ void k_llg_step_advance(unsigned long long* c, unsigned long long n) { *c += n; }

static void drop_llg_graph(LLGPlan* pl) {
  for (LLGGraph& g : pl->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = LLGGraph{};
  }
  for (int k = 0; k < 2; ++k) {
    if (pl->host_graphs[k].exec) cudaGraphExecDestroy(pl->host_graphs[k].exec);
    pl->host_graphs[k] = LLGGraph{};
    pl->host_in[k] = pl->host_noise[k] = nullptr;
  }
  pl->last_tail = -1;
}

static bool graph_matches(const LLGGraph& g, int steps, const double* e, int mode, const DevLattice& L) {
  return g.exec && g.steps == steps && g.e == e && g.mode == mode && g.B[0] == L.B0 && g.B[1] == L.B1 &&
         g.B[2] == L.B2 && g.offset == L.cell_offset;
}

static const LLGGraph* find_llg_graph(LLGPlan* pl, int steps, const double* e) {
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  for (LLGGraph& g : pl->graphs)
    if (graph_matches(g, steps, e, mode, pl->model->d)) return &g;
  return nullptr;
}

// the graph of `steps` steps on spins e (captured now if no current one matches)
static mgx_status llg_graph(LLGPlan* pl, double* e, int steps, cudaGraphExec_t* out) {
  const DevLattice& L = pl->model->d;
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  LLGGraph* slot = nullptr;
  for (LLGGraph& g : pl->graphs) {
    if (graph_matches(g, steps, e, mode, L)) {
      g.used = ++pl->graph_clock;
      *out = g.exec;
      return MGX_OK;
    }
    if (!slot || !g.exec || (slot->exec && g.used < slot->used)) slot = &g;
  }
  if (slot->exec) cudaGraphExecDestroy(slot->exec);
  *slot = LLGGraph{};
  if (!pl->d_step) MGX_CUDA_TRY(cudaMalloc(&pl->d_step, sizeof(unsigned long long)));
  if (!pl->cap_stream) MGX_CUDA_TRY(cudaStreamCreateWithFlags(&pl->cap_stream, cudaStreamNonBlocking));
  MGX_CUDA_TRY(cudaStreamBeginCapture(pl->cap_stream, cudaStreamCaptureModeThreadLocal));
  pl->p.step_base = pl->d_step;
  for (int k = 0; k < steps; ++k) enqueue_llg_step(pl, e, nullptr, (uint64_t)k, pl->cap_stream, 3);
  pl->p.step_base = nullptr;
  k_llg_step_advance<<<1, 1, 0, pl->cap_stream>>>(pl->d_step, (unsigned long long)steps);
  cudaGraph_t g = nullptr;
  cudaError_t err = cudaStreamEndCapture(pl->cap_stream, &g);
  if (err != cudaSuccess) return cuda_error(err, "mgx_llg_run capture");
  err = cudaGraphInstantiate(&slot->exec, g, 0);
  cudaGraphDestroy(g);
  if (err != cudaSuccess) {
    slot->exec = nullptr;
    return cuda_error(err, "mgx_llg_run instantiate");
  }
  slot->steps = steps;
  slot->e = e;
  slot->mode = mode;
  slot->B[0] = L.B0;
  slot->B[1] = L.B1;
  slot->B[2] = L.B2;
  slot->offset = L.cell_offset;
  slot->used = ++pl->graph_clock;
  *out = slot->exec;
  return MGX_OK;
}

static bool pinned_host(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

static void drop_host_buffers(LLGPlan* pl) {
  for (int k = 0; k < 2; ++k) {
    if (pl->host_graphs[k].exec) cudaGraphExecDestroy(pl->host_graphs[k].exec);
    pl->host_graphs[k] = LLGGraph{};
  }
  cudaFree(pl->host_lat);
  cudaFree(pl->host_aos);
  pl->host_lat = pl->host_aos = nullptr;
  for (cudaEvent_t& ev : pl->host_ev) {
    if (ev) cudaEventDestroy(ev);
    ev = nullptr;
  }
  if (pl->copy_stream) cudaStreamDestroy(pl->copy_stream);
  if (pl->aux_stream) cudaStreamDestroy(pl->aux_stream);
  if (pl->pack_stream) cudaStreamDestroy(pl->pack_stream);
  if (pl->out_stream) cudaStreamDestroy(pl->out_stream);
  pl->copy_stream = pl->aux_stream = pl->pack_stream = pl->out_stream = nullptr;
  for (cudaStream_t& cst : pl->corr_stream) {
    if (cst) cudaStreamDestroy(cst);
    cst = nullptr;
  }
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
  if (p->precision < MGX_PRECISION_FP64 || p->precision > MGX_PRECISION_FP64_FIXED_GATHER)
    return set_error(MGX_ERR_INVALID, "precision %d is not fp64 (0), df32-gather (1), int48-gather (2) or "
                     "fp64-fixed-gather (3)", p->precision);
  if (has_higher_onsite(m->d) && p->precision != MGX_PRECISION_FP64 && p->precision != MGX_PRECISION_FP64_FIXED_GATHER)
    return set_error(MGX_ERR_UNSUPPORTED, "cubic / higher uniaxial anisotropy need the FP64 form (precision 0) or "
                     "the FP64 form with the fixed-point exchange sum (precision 3)");
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
  if (p->precision != MGX_PRECISION_FP64) {
    pl->precision = p->precision;
    const mgx_status st = p->precision == MGX_PRECISION_DF32_GATHER ? build_df_tables(pl) : build_fx_tables(pl);
    if (st != MGX_OK) {
      mgx_llg_destroy(reinterpret_cast<mgx_llg*>(pl));
      return st;
    }
  }
  *out = reinterpret_cast<mgx_llg*>(pl);
  return MGX_OK;
}

mgx_status mgx_llg_set_extra_field(mgx_llg* pp, const double* B_add) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl) return set_error(MGX_ERR_INVALID, "mgx_llg_set_extra_field: null plan");
  if (B_add && pl->precision != MGX_PRECISION_FP64)
    return set_error(MGX_ERR_UNSUPPORTED, "a per-site extra field needs an FP64 plan");
  if (B_add != pl->p.B_add) drop_llg_graph(pl);      // captured launches hold the pointer by value
  pl->p.B_add = B_add;
  return MGX_OK;
}

mgx_status mgx_llg_set_sot(mgx_llg* pp, const double p[3], double B_DL, double B_FL) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !p) return set_error(MGX_ERR_INVALID, "mgx_llg_set_sot: null argument");
  const double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  const bool on = B_DL != 0.0 || B_FL != 0.0;
  if (on && !(n > 0.0 && std::isfinite(n) && std::isfinite(B_DL) && std::isfinite(B_FL)))
    return set_error(MGX_ERR_INVALID, "mgx_llg_set_sot: p must be a finite non-zero vector, B_DL and B_FL finite");
  if (on && pl->precision != MGX_PRECISION_FP64)
    return set_error(MGX_ERR_UNSUPPORTED, "spin-orbit torque needs an FP64 plan");
  drop_llg_graph(pl);                                 // captured launches hold the pointer by value
  if (!on) {
    pl->p.sot = nullptr;
    return MGX_OK;
  }
  if (!pl->sot_block) MGX_CUDA_TRY(cudaMalloc(&pl->sot_block, 5 * sizeof(double)));
  const double v[5] = {p[0] / n, p[1] / n, p[2] / n, B_DL, B_FL};
  MGX_CUDA_TRY(cudaMemcpy(pl->sot_block, v, sizeof(v), cudaMemcpyHostToDevice));
  pl->p.sot = pl->sot_block;
  return MGX_OK;
}

mgx_status mgx_llg_predicted(mgx_llg* pp, double** ep) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !ep) return set_error(MGX_ERR_INVALID, "mgx_llg_predicted: null argument");
  *ep = pl->p.ep;
  return MGX_OK;
}

mgx_status mgx_llg_predicted_split(mgx_llg* pp, void** eps) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !eps) return set_error(MGX_ERR_INVALID, "mgx_llg_predicted_split: null argument");
  *eps = nullptr;
  if (pl->precision == MGX_PRECISION_DF32_GATHER) *eps = pl->df.eps;
  if (pl->precision == MGX_PRECISION_INT48_GATHER || pl->precision == MGX_PRECISION_FP64_FIXED_GATHER) *eps = pl->fx.eps;
  return MGX_OK;
}

mgx_status mgx_llg_destroy(mgx_llg* pp) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl) return MGX_OK;
  cudaFree(pl->sub_block);
  cudaFree(pl->site_block);
  cudaFree(pl->sigma_site);
  cudaFree(pl->scratch);
  cudaFree(pl->df_block);
  cudaFree(pl->fx_block);
  cudaFree(pl->fx_noise);
  drop_llg_graph(pl);
  if (pl->cap_stream) cudaStreamDestroy(pl->cap_stream);
  cudaFree(pl->d_step);
  drop_host_buffers(pl);
  cudaFree(pl->sot_block);
  delete pl;
  return MGX_OK;
}

mgx_status mgx_llg_set_sigma(mgx_llg* pp, const double* sigma_sub, const double* sigma_site) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl) return set_error(MGX_ERR_INVALID, "mgx_llg_set_sigma: null plan");
  const int ns = pl->model->d.ns;
  const long long N = pl->model->d.N;
  bool zero = true;
  if (sigma_sub) {
    for (int s = 0; s < ns; ++s) {
      if (!std::isfinite(sigma_sub[s]) || sigma_sub[s] < 0.0)
        return set_error(MGX_ERR_INVALID, "sigma_sub must be finite and >= 0");
      zero &= sigma_sub[s] == 0.0;
    }
    MGX_CUDA_TRY(cudaMemcpy((double*)pl->sub_block + 2 * ns, sigma_sub, sizeof(double) * ns, cudaMemcpyHostToDevice));
    for (int s = 0; s < ns; ++s) pl->df.sig[s] = pl->fx.sig[s] = split_host(sigma_sub[s]);
  } else {
    std::vector<double> cur(ns);
    MGX_CUDA_TRY(cudaMemcpy(cur.data(), (double*)pl->sub_block + 2 * ns, sizeof(double) * ns, cudaMemcpyDeviceToHost));
    for (double x : cur) zero &= x == 0.0;
    for (int s = 0; s < ns; ++s) pl->df.sig[s] = pl->fx.sig[s] = split_host(cur[s]);
  }
  if (sigma_site) {
    std::vector<double> v = site_to_lattice(sigma_site, ns, pl->model->d.ncell);
    for (double x : v) {
      if (!std::isfinite(x) || x < 0.0) return set_error(MGX_ERR_INVALID, "sigma_site must be finite and >= 0");
      zero &= x == 0.0;
    }
    if (!pl->sigma_site) MGX_CUDA_TRY(cudaMalloc(&pl->sigma_site, sizeof(double) * N));
    MGX_CUDA_TRY(cudaMemcpy(pl->sigma_site, v.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    pl->p.sigma_site = pl->sigma_site;
  } else {
    pl->p.sigma_site = nullptr;
  }
  pl->sigma_zero = zero;
  // the captured step loop holds the amplitudes' splits and the per-site pointer by value
  drop_llg_graph(pl);
  return MGX_OK;
}

// The reduced-arithmetic forms gather from a split copy of the spins: refresh it from e at the start
// of every library call (the caller may have changed e in between).
static void enqueue_reduced_split(const LLGPlan* pl, const double* e, cudaStream_t st) {
  if (pl->precision == MGX_PRECISION_DF32_GATHER) enqueue_df_split(pl, e, st);
  if (pl->precision == MGX_PRECISION_INT48_GATHER || pl->precision == MGX_PRECISION_FP64_FIXED_GATHER)
    enqueue_fx_split(pl, e, st);
}

mgx_status mgx_llg_step(mgx_llg* pp, double* e, const double* noise, uint64_t step, void* stream) {
  NvtxRange nvtx_range("mgx_llg_step");
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_step: null argument");
  if (pl->p.noise == MGX_NOISE_HOST && !noise)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step: host-noise plan needs a noise buffer");
  enqueue_reduced_split(pl, e, (cudaStream_t)stream);
  enqueue_llg_step(pl, e, noise, step, (cudaStream_t)stream, 3);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

// The work of one host-buffer step on stream ms (nc slabs, or one piece when nc == 1): copies in on
// the copy stream, packing (and the fixed-point split), predictors, correctors, unpacking and copies
// out; every stream it forks from ms joins ms again at the end, so it can also be captured.
static mgx_status enqueue_host_step(LLGPlan* pl, const double* e_in, double* e_out, const double* noise,
                                    uint64_t step, cudaStream_t ms, int nc) {
  const Model* m = pl->model;
  const DevLattice& L = m->d;
  const long long N = L.N;
  const bool fx = pl->precision == MGX_PRECISION_FP64_FIXED_GATHER || pl->precision == MGX_PRECISION_INT48_GATHER;
  cudaStream_t cs = pl->copy_stream, ps = pl->pack_stream;
  cudaEvent_t* ev_in = pl->host_ev;
  cudaEvent_t* ev_out = pl->host_ev + MGX_HOST_CHUNKS;
  cudaEvent_t* ev_copied = pl->host_ev + 2 * MGX_HOST_CHUNKS;
  cudaEvent_t* ev_pred = pl->host_ev + 3 * MGX_HOST_CHUNKS;
  cudaEvent_t ev_start = pl->host_ev[4 * MGX_HOST_CHUNKS], ev_done = pl->host_ev[4 * MGX_HOST_CHUNKS + 1];
  cudaEvent_t ev_join_aux = pl->host_ev[4 * MGX_HOST_CHUNKS + 2], ev_join_out = pl->host_ev[4 * MGX_HOST_CHUNKS + 3];
  const long long layer = (long long)L.L1 * L.L2;
  auto cell0 = [&](int c) { return (long long)L.L0 * c / nc * layer; };    // first cell of slab c
  MGX_CUDA_TRY(cudaEventRecord(ev_start, ms));
  MGX_CUDA_TRY(cudaStreamWaitEvent(cs, ev_start, 0));
  if (nc > 1) MGX_CUDA_TRY(cudaStreamWaitEvent(ps, ev_start, 0));
  for (int c = 0; c < nc; ++c) {
    const long long sb = (nc == 1 ? 0 : cell0(c) * L.ns), se = (nc == 1 ? N : cell0(c + 1) * L.ns);
    MGX_CUDA_TRY(cudaMemcpyAsync(pl->host_aos + 3 * sb, e_in + 3 * sb, sizeof(double) * 3 * (se - sb),
                                 cudaMemcpyDefault, cs));
    if (nc == 1) {
      enqueue_pack(m, pl->host_aos, pl->host_lat, sb, se - sb, cs);
      MGX_CUDA_TRY(cudaEventRecord(ev_in[c], cs));
      continue;
    }
    // slabs: the next copy does not wait for this slab's packing (pack stream)
    MGX_CUDA_TRY(cudaEventRecord(ev_copied[c], cs));
    MGX_CUDA_TRY(cudaStreamWaitEvent(ps, ev_copied[c], 0));
    if (fx)
      enqueue_fx_pack_split(pl, pl->host_aos, pl->host_lat, sb, se - sb, ps);
    else
      enqueue_pack(m, pl->host_aos, pl->host_lat, sb, se - sb, ps);
    MGX_CUDA_TRY(cudaEventRecord(ev_in[c], ps));
  }
  double* lat = pl->host_lat;
  if (nc == 1) {
    MGX_CUDA_TRY(cudaStreamWaitEvent(ms, ev_in[0], 0));
    enqueue_reduced_split(pl, lat, ms);
    enqueue_llg_step(pl, lat, noise, step, ms, 3);
    enqueue_unpack(m, lat, pl->host_aos, 0, N, ms);
    MGX_CUDA_TRY(cudaEventRecord(ev_out[0], ms));
    MGX_CUDA_TRY(cudaStreamWaitEvent(cs, ev_out[0], 0));
    MGX_CUDA_TRY(cudaMemcpyAsync(e_out, pl->host_aos, sizeof(double) * 3 * N, cudaMemcpyDefault, cs));
  } else {
    cudaStream_t run[2] = {ms, pl->aux_stream}, os = pl->out_stream;
    MGX_CUDA_TRY(cudaStreamWaitEvent(run[1], ev_start, 0));
    MGX_CUDA_TRY(cudaStreamWaitEvent(os, ev_start, 0));
    // predictors: slab c gathers from slabs c-1 .. c+1 (cyclically when axis 0 is periodic); the
    // copies land in slab order, so waiting for the last slab needed is enough
    const bool ring = L.pbc0 != 0;
    for (int k = 0; k < nc; ++k) {
      const int c = ring ? (k + 1) % nc : k;
      cudaStream_t st = run[k & 1];
      MGX_CUDA_TRY(cudaStreamWaitEvent(st, ev_in[c == 0 && ring ? nc - 1 : std::min(c + 1, nc - 1)], 0));
      if (fx)
        enqueue_fx_range(pl, lat, noise, step, st, 1, cell0(c), cell0(c + 1) - cell0(c));
      else
        enqueue_fp64_range(pl, lat, noise, step, st, 1, CellRange{cell0(c), cell0(c + 1) - cell0(c)});
      MGX_CUDA_TRY(cudaEventRecord(ev_pred[c], st));
    }
    // the corrector of slab c gathers the predicted spins of slabs c-1 .. c+1 and overwrites the spins
    // (and their fixed-point copy) of slab c, which the predictors of c-1 and c+1 read: it waits for
    // those three predictors only, on streams of its own, so it overlaps the later predictors
    for (int k = 0; k < nc; ++k) {
      const int c = ring ? (k + 2) % nc : k;
      cudaStream_t st = pl->corr_stream[k & 1];
      for (int d = -1; d <= 1; ++d) {
        const int n = c + d;
        if (n >= 0 && n < nc) MGX_CUDA_TRY(cudaStreamWaitEvent(st, ev_pred[n], 0));
        else if (ring) MGX_CUDA_TRY(cudaStreamWaitEvent(st, ev_pred[(n + nc) % nc], 0));
      }
      const long long sb = cell0(c) * L.ns, se = cell0(c + 1) * L.ns;
      if (fx) {
        // the corrector writes the slab's new spins straight into the (N, 3) staging rows
        enqueue_fx_range(pl, lat, noise, step, st, 2, cell0(c), cell0(c + 1) - cell0(c), pl->host_aos);
      } else {
        enqueue_fp64_range(pl, lat, noise, step, st, 2, CellRange{cell0(c), cell0(c + 1) - cell0(c)});
        enqueue_unpack(m, lat, pl->host_aos, sb, se - sb, st);
      }
      MGX_CUDA_TRY(cudaEventRecord(ev_out[c], st));
      MGX_CUDA_TRY(cudaStreamWaitEvent(os, ev_out[c], 0));
      MGX_CUDA_TRY(cudaMemcpyAsync(e_out + 3 * sb, pl->host_aos + 3 * sb, sizeof(double) * 3 * (se - sb),
                                   cudaMemcpyDefault, os));
    }
  }
  // the out stream waited for every slab of the corrector streams; the copy stream joins it, the pack
  // stream and the second predictor stream: `ms` continues after all of it
  if (nc > 1) {
    MGX_CUDA_TRY(cudaEventRecord(ev_copied[0], ps));
    MGX_CUDA_TRY(cudaStreamWaitEvent(cs, ev_copied[0], 0));
    MGX_CUDA_TRY(cudaEventRecord(ev_join_aux, pl->aux_stream));
    MGX_CUDA_TRY(cudaStreamWaitEvent(cs, ev_join_aux, 0));
    MGX_CUDA_TRY(cudaEventRecord(ev_join_out, pl->out_stream));
    MGX_CUDA_TRY(cudaStreamWaitEvent(cs, ev_join_out, 0));
  }
  MGX_CUDA_TRY(cudaEventRecord(ev_done, cs));
  MGX_CUDA_TRY(cudaStreamWaitEvent(ms, ev_done, 0));
  return MGX_OK;
}


// Copies of host buffers inside one step.  The input goes to the device in axis-0 slabs on the plan's
// copy stream (each packed into the lattice layout as it lands, and for the fixed-point-gather forms
// split into its fixed-point copy in the same pass); the predictor of a slab starts once
// the slabs it gathers from (its own and its neighbours', every slab at least as thick as the
// couplings' reach) are in; the corrector runs slab by slab (the fixed-point forms' corrector writes
// the new spins straight into the (N, 3) staging rows) and each finished slab goes back to the host on
// the out stream while the next ones are computed.  Consecutive slabs alternate between the caller's stream and
// a second compute stream, so the blocks of one slab fill the tail of the previous one.  The
// predictor and corrector kernels, and so the result, are those of mgx_llg_step: only the launch grid
// is split.
mgx_status mgx_llg_step_host(mgx_llg* pp, const double* e_in, double* e_out, const double* noise, uint64_t step,
                             void* stream) {
  NvtxRange nvtx_range("mgx_llg_step_host");
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e_in || !e_out) return set_error(MGX_ERR_INVALID, "mgx_llg_step_host: null argument");
  if (pl->p.noise == MGX_NOISE_HOST && !noise)
    return set_error(MGX_ERR_INVALID, "mgx_llg_step_host: host-noise plan needs a noise buffer");
  const Model* m = pl->model;
  const DevLattice& L = m->d;
  const long long N = L.N;
  cudaStream_t ms = (cudaStream_t)stream;
  if (!pl->copy_stream) {
    // all or nothing: a failed allocation leaves the plan without host buffers
    cudaError_t err = cudaMalloc(&pl->host_lat, sizeof(double) * 3 * N);
    if (err == cudaSuccess) err = cudaMalloc(&pl->host_aos, sizeof(double) * 3 * N);
    for (cudaEvent_t& ev : pl->host_ev)
      if (err == cudaSuccess) err = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&pl->aux_stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&pl->pack_stream, cudaStreamNonBlocking);
    for (cudaStream_t& cst : pl->corr_stream)
      if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&pl->out_stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&pl->copy_stream, cudaStreamNonBlocking);
    if (err != cudaSuccess) {
      drop_host_buffers(pl);
      return cuda_error(err, "mgx_llg_step_host buffers");
    }
  }
  // slabs: FP64 and fixed-point-gather stencil plans of at least 2^20 sites with both buffers
  // page-locked; otherwise one piece
  const bool fx = pl->precision == MGX_PRECISION_FP64_FIXED_GATHER || pl->precision == MGX_PRECISION_INT48_GATHER;
  int nc = 1;
  if ((pl->precision == MGX_PRECISION_FP64 || fx) && L.layout == 0 && m->reach0 >= 0 && N >= (1LL << 20) &&
      pinned_host(e_in) && pinned_host(e_out)) {
    nc = std::min(MGX_HOST_CHUNKS, L.L0 / std::max(m->reach0, 1));
    if (nc < 3) nc = 1;
  }
  if (nc == 1) {
    const mgx_status st = enqueue_host_step(pl, e_in, e_out, noise, step, ms, 1);
    if (st != MGX_OK) return st;
    MGX_CUDA_TRY(cudaGetLastError());
    return MGX_OK;
  }
  // the slab pipeline: replay the graph captured for these buffers (capture it on first use)
  const int mode = pl->sigma_zero ? MGX_NOISE_NONE : pl->p.noise;
  int slot = -1;
  for (int k = 0; k < 2; ++k) {
    const LLGGraph& g = pl->host_graphs[k];
    if (g.exec && g.e == e_out && pl->host_in[k] == e_in && pl->host_noise[k] == noise &&
        graph_matches(g, nc, e_out, mode, L))
      slot = k;
  }
  if (slot < 0) {
    slot = (pl->host_graphs[0].used <= pl->host_graphs[1].used) ? 0 : 1;
    LLGGraph& g = pl->host_graphs[slot];
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = LLGGraph{};
    if (!pl->d_step) MGX_CUDA_TRY(cudaMalloc(&pl->d_step, sizeof(unsigned long long)));
    if (!pl->cap_stream) MGX_CUDA_TRY(cudaStreamCreateWithFlags(&pl->cap_stream, cudaStreamNonBlocking));
    MGX_CUDA_TRY(cudaStreamBeginCapture(pl->cap_stream, cudaStreamCaptureModeThreadLocal));
    pl->p.step_base = pl->d_step;
    const mgx_status es = enqueue_host_step(pl, e_in, e_out, noise, 0, pl->cap_stream, nc);
    pl->p.step_base = nullptr;
    cudaGraph_t graph = nullptr;
    const cudaError_t err = cudaStreamEndCapture(pl->cap_stream, &graph);
    if (es != MGX_OK) {
      if (graph) cudaGraphDestroy(graph);
      return es;
    }
    if (err != cudaSuccess) return cuda_error(err, "mgx_llg_step_host capture");
    const cudaError_t ierr = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ierr != cudaSuccess) {
      g.exec = nullptr;
      return cuda_error(ierr, "mgx_llg_step_host instantiate");
    }
    g.steps = nc;
    g.e = e_out;
    g.mode = mode;
    g.B[0] = L.B0;
    g.B[1] = L.B1;
    g.B[2] = L.B2;
    g.offset = L.cell_offset;
    pl->host_in[slot] = e_in;
    pl->host_noise[slot] = noise;
  }
  pl->host_graphs[slot].used = ++pl->graph_clock;
  k_llg_step_set<<<1, 1, 0, ms>>>(pl->d_step, (unsigned long long)step);
  MGX_CUDA_TRY(cudaGraphLaunch(pl->host_graphs[slot].exec, ms));
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_llg_stage(mgx_llg* pp, int32_t stage, double* e, const double* noise, uint64_t step, void* stream) {
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_stage: null argument");
  if (stage != 0 && stage != 1) return set_error(MGX_ERR_INVALID, "stage %d is not 0 (predictor) or 1 (corrector)", stage);
  if (pl->p.noise == MGX_NOISE_HOST && !noise)
    return set_error(MGX_ERR_INVALID, "mgx_llg_stage: host-noise plan needs a noise buffer");
  if (stage == 0) enqueue_reduced_split(pl, e, (cudaStream_t)stream);
  enqueue_llg_step(pl, e, noise, step, (cudaStream_t)stream, stage == 0 ? 1 : 2);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_llg_run(mgx_llg* pp, double* e, int64_t nsteps, uint64_t step0, void* stream) {
  NvtxRange nvtx_range("mgx_llg_run");
  LLGPlan* pl = reinterpret_cast<LLGPlan*>(pp);
  if (!pl || !e) return set_error(MGX_ERR_INVALID, "mgx_llg_run: null argument");
  if (nsteps < 0) return set_error(MGX_ERR_INVALID, "nsteps must be >= 0");
  if (pl->p.noise == MGX_NOISE_HOST)
    return set_error(MGX_ERR_INVALID, "mgx_llg_run: host-noise plans step one at a time (mgx_llg_step)");
  cudaStream_t st = (cudaStream_t)stream;
  if (nsteps > 0) enqueue_reduced_split(pl, e, st);
  int64_t done = 0;
  if (pl->model->d.N <= kGraphMaxSites) {
    bool counter_set = false;
    cudaGraphExec_t exec = nullptr;
    if (nsteps >= 2 * kGraphChunk) {
      const mgx_status gs = llg_graph(pl, e, kGraphChunk, &exec);
      if (gs != MGX_OK) return gs;
      k_llg_step_set<<<1, 1, 0, st>>>(pl->d_step, (unsigned long long)step0);
      counter_set = true;
      for (; done + kGraphChunk <= nsteps; done += kGraphChunk) MGX_CUDA_TRY(cudaGraphLaunch(exec, st));
    }
    const long long tail = nsteps - done;
    if (tail >= kGraphMinTail && tail < 2 * kGraphChunk &&
        (tail == pl->last_tail || find_llg_graph(pl, (int)tail, e))) {
      const mgx_status gs = llg_graph(pl, e, (int)tail, &exec);
      if (gs != MGX_OK) return gs;
      if (!counter_set) k_llg_step_set<<<1, 1, 0, st>>>(pl->d_step, (unsigned long long)(step0 + done));
      MGX_CUDA_TRY(cudaGraphLaunch(exec, st));
      done = nsteps;
    }
    pl->last_tail = tail;
  }
  for (; done < nsteps; ++done) enqueue_llg_step(pl, e, nullptr, step0 + (uint64_t)done, st, 3);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

}  // extern "C"
