/*
 * mgx.h -- C ABI of the GB300 (sm_103a) atomistic stochastic LLG step.
 *
 * This library replaces the kernel layer behind magex's LLG integrator:
 *   - the NumPy Heun step         magex/llg.py:216-227 (LLGSolver.step, integrator "heun")
 *   - its effective field          magex/spinmodel.py:454-473 (exchange_field, gradient, effective_field)
 *   - the fused CPU kernels        magex/fast.py:336-390 (_fused1 predictor, _fused2 corrector)
 *   - the numba.cuda kernels       magex/cuda_backend.py:144-218 (_k_pred, _k_corr)
 *   - the kernel argument tuple    magex/fast.py:669-672 (FastModel.args)
 *   - the observables of the run   magex/spinmodel.py:475-484,517-519, magex/llg.py:250-252
 *
 * Conventions
 *   - Plain C types only.  Pointers documented "device" point to GPU memory owned by the caller;
 *     "host" pointers are read during the call only.  A stream is a cudaStream_t passed as void*
 *     (NULL = legacy default stream).  All device work of a call is enqueued on that stream;
 *     no call synchronises the device unless it says so.
 *   - Spins on the device use the lattice layout: component-major, then sublattice, then cell
 *     (c0, c1, c2 row-major): x[c * N + s * ncell + cell].  mgx_pack_spins / mgx_unpack_spins
 *     convert from / to magex's (N, 3) row-major array with site = cell * ns + s
 *     (magex/spinmodel.py:197-204).
 *   - Units as magex: time ps, field T, energy meV, moments mu_B.
 *   - Every entry point returns an mgx_status; on failure mgx_last_error() gives a message.
 *     No C++ exception crosses the ABI.  Objects are not thread-safe; distinct objects are.
 */
#ifndef MGX_H
#define MGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGX_VERSION 1

#define MGX_MAX_SUBLATTICES 16
#define MGX_MAX_BONDS 256          /* stencil couplings per unit cell after self-image folding */

typedef int32_t mgx_status;
enum {
  MGX_OK = 0,
  MGX_ERR_INVALID = 1,       /* bad argument (maps to ValueError) */
  MGX_ERR_UNSUPPORTED = 2,   /* feature outside the kernels (maps to NotImplementedError) */
  MGX_ERR_CUDA = 3,          /* CUDA runtime error (maps to RuntimeError) */
  MGX_ERR_NOMEM = 4          /* device allocation failed (maps to MemoryError) */
};

enum { MGX_INTEGRATOR_HEUN = 0, MGX_INTEGRATOR_DEPONDT = 1 };
enum { MGX_NOISE_NONE = 0, MGX_NOISE_HOST = 1, MGX_NOISE_PHILOX = 2 };
/* Arithmetic of the exchange gather: FP64 (default); compensated FP32 pairs (hi + lo, about 44
 * significant bits); or exact integer products and sums of fixed-point couplings and spins on the
 * INT32 multiply-add pipe (wide multiply-adds at ~28 per clock per SM against 2 FP64 FMAs).  The
 * 48-bit integer and the FP32-pair forms keep the integration and renormalisation in FP64 and the rest
 * of the field and the right-hand side on FP32 pairs (Heun).  MGX_PRECISION_FP64_FIXED_GATHER keeps
 * every floating-point operation FP64 and evaluates the exchange and on-site sums exactly on 56-bit
 * fixed-point values: the inputs are quantised 2^-57 below their scale and the sum is rounded once,
 * so its error stays below that of an FP64 FMA chain.  GB300 runs FP64 at 1/61 of its FP32 rate. */
enum { MGX_PRECISION_FP64 = 0, MGX_PRECISION_DF32_GATHER = 1, MGX_PRECISION_INT48_GATHER = 2,
       MGX_PRECISION_FP64_FIXED_GATHER = 3 };

typedef struct mgx_model mgx_model;
typedef struct mgx_llg mgx_llg;
typedef struct mgx_batch mgx_batch;
typedef struct mgx_adjoint mgx_adjoint;

/* Supercell of a unit-cell model, described by its per-cell coupling list ("stencil").
 * Replaces the 3N x 3N CSR matrix of magex/spinmodel.py:240 and the per-site neighbour blocks of
 * magex/fast.py:587-627: site (cell c, sublattice src) couples to (wrap(c + R), dst) with the
 * coupling tensor of the bond.  Self-image couplings must already be folded into A_sub. */
typedef struct mgx_lattice_desc {
  int32_t ns;                /* sublattices per cell, 1..MGX_MAX_SUBLATTICES */
  int32_t L[3];              /* supercell size in cells */
  int32_t pbc[3];            /* 1 = periodic, 0 = open */
  int32_t nbond;             /* couplings per cell, 0..MGX_MAX_BONDS */
  const int32_t* bond_src;   /* host [nbond] sublattice of the site receiving the field */
  const int32_t* bond_dst;   /* host [nbond] sublattice of the neighbour */
  const int32_t* bond_R;     /* host [nbond*3] cell offset of the neighbour */
  int32_t width;             /* doubles per coupling: 1 (J), 4 (J, Dx, Dy, Dz) or 9 (row-major 3x3) */
  const double* bond_table;  /* host [nbond*width] */
  const double* A_sub;       /* host [ns*9] single-ion tensors (row-major), or NULL for none */
  const double* mu_sub;      /* host [ns] moments in mu_B */
  const double* sign_sub;    /* host [ns] order-parameter signs (+-1), or NULL for all +1 */
  double B[3];               /* external field (T) */
} mgx_lattice_desc;

/* Optional per-site overrides in magex site order (host arrays of N entries, or NULL).
 * They mirror SpinSystem.A / mu / pinned after magex.structure edits
 * (magex/structure.py:160-207).  Pinned sites keep their spin, as magex/fast.py:346-350. */
typedef struct mgx_site_desc {
  const double* A_site;      /* host [N*9] or NULL */
  const double* mu_site;     /* host [N] or NULL */
  const uint8_t* pinned;     /* host [N] (0/1) or NULL */
} mgx_site_desc;

/* Integrator parameters; mirror LLGSolver(alpha, dt, precession, integrator) of magex/llg.py:49-50. */
typedef struct mgx_llg_params {
  double dt;                 /* time step (ps) */
  double alpha;              /* Gilbert damping, used when alpha_site == NULL */
  const double* alpha_site;  /* host [N] per-site damping in magex order, or NULL */
  int32_t precession;        /* 1: full LLG; 0: damping term only (magex/llg.py:21-28) */
  int32_t integrator;        /* MGX_INTEGRATOR_HEUN or MGX_INTEGRATOR_DEPONDT */
  int32_t noise;             /* MGX_NOISE_NONE / _HOST (caller supplies N(0,1) draws) / _PHILOX */
  uint64_t seed;             /* Philox key (MGX_NOISE_PHILOX) */
  int32_t precision;         /* MGX_PRECISION_FP64, _DF32_GATHER, _INT48_GATHER or _FP64_FIXED_GATHER (not FP64:
                              * stencil models with per-sublattice moments and single-ion tensors; the
                              * couplings are snapshotted when the plan is created) */
} mgx_llg_params;

/* ---------------------------------------------------------------- library */
int32_t mgx_version(void);
/* Copy the last error message of the calling thread into buf (always NUL-terminated). */
void mgx_last_error(char* buf, size_t len);

/* ---------------------------------------------------------------- model
 * mgx_model_create replaces FastModel(system) (magex/fast.py:630-657) and _Device (magex/cuda_backend.py:307-335):
 * it validates the stencil and uploads tables and per-site arrays to the current device. */
mgx_status mgx_model_create(const mgx_lattice_desc* lat, const mgx_site_desc* sites, mgx_model** out);

/* Arbitrary lattice (carved shapes, vacancies, edited exchange): per-site neighbour lists in magex site
 * order, the argument list of magex's fused kernels (FastModel.args, magex/fast.py:669-672: ptr, nbr,
 * (typ, table), A, mu, B, pinned) built by neighbour_blocks (magex/fast.py:587-627).  Spins of such a
 * model use the identity layout: x[c * N + site]. */
typedef struct mgx_csr_desc {
  int64_t nsites;
  const int64_t* ptr;        /* host [N+1] */
  const int32_t* nbr;        /* host [ptr[N]] */
  const int32_t* typ;        /* host [ptr[N]] coupling type of each neighbour */
  int32_t ntypes;
  int32_t width;             /* 1, 4 or 9 doubles per type (as mgx_lattice_desc) */
  const double* table;       /* host [ntypes*width] */
  const double* A_site;      /* host [N*9] or NULL */
  const double* mu_site;     /* host [N] */
  const double* sign_site;   /* host [N] or NULL */
  const uint8_t* pinned;     /* host [N] or NULL */
  double B[3];
} mgx_csr_desc;
mgx_status mgx_model_create_csr(const mgx_csr_desc* csr, mgx_model** out);
mgx_status mgx_model_destroy(mgx_model* m);
mgx_status mgx_model_set_field(mgx_model* m, const double B[3]);   /* SpinSystem.set_field, magex/spinmodel.py:451-452 */
int64_t mgx_model_nsites(const mgx_model* m);
/* Replace the coupling tensors (host [nbond*width], the order given at creation) or the
 * per-sublattice single-ion tensors (host [ns*9]); synchronous.  Used to evaluate a trajectory at new
 * parameters (magex rebuilds FastModel after editing couplings, magex/fast.py:631). */
mgx_status mgx_model_set_couplings(mgx_model* m, const double* bond_table);
mgx_status mgx_model_set_onsite(mgx_model* m, const double* A_sub);
/* Cubic anisotropy E_i = Kc_i (a1^2 a2^2 + a2^2 a3^2 + a3^2 a1^2), a = C e_i (C: 3x3 axes, rows), and
 * higher uniaxial anisotropy E_i = -K2_i (e_i.u)^4 - K3_i (e_i.u)^6: the Kc, C, K2, K3, u, has_c, has_u
 * members of magex's kernel arguments (magex/fast.py:640-672, magex/terms.py:35-75, from
 * magex/structure.py:188-193).  Host per-site arrays [N] in magex site order (NULL: term absent; K3
 * NULL with K2: zeros); synchronous; call before creating plans.  The FP64 LLG step, the field and
 * the observables and the Monte Carlo sweep include them; the reduced LLG forms, batched systems and
 * the adjoint refuse such a model with MGX_ERR_UNSUPPORTED. */
mgx_status mgx_model_set_onsite_higher(mgx_model* m, const double* Kc, const double* C, const double* K2,
                                       const double* K3, const double* u);
/* Slab decomposition of one supercell along axis 0 (the halo-exchange path of magex/mpi_spin.py:
 * 150-180): this model is a slab of the whole lattice.  In-kernel Philox counters use local cell +
 * cell_offset as the cell index of the whole lattice (so the noise equals the unsplit run's), and
 * mgx_observables sums only cells with own_begin <= c0 < own_end (the halo layers are owned by the
 * neighbouring slabs).  Lattice (stencil) models only. */
mgx_status mgx_model_set_partition(mgx_model* m, int64_t cell_offset, int32_t own_begin, int32_t own_end);
/* Copy the c0 layers [c0_begin, c0_end) of a (3, N) lattice-layout field x (device) into a packed buffer
 * buf (3 * ns * (c0_end - c0_begin) * L1 * L2 doubles, component-major then sublattice; device or
 * pinned host) when to_buffer != 0, or back from it into x: the halo messages of a slab decomposition. */
mgx_status mgx_lattice_layers(const mgx_model* m, double* x, int32_t c0_begin, int32_t c0_end, double* buf,
                              int32_t to_buffer, void* stream);

/* (N,3) magex-order device array <-> lattice-layout device array (3*N doubles each). */
mgx_status mgx_pack_spins(const mgx_model* m, const double* aos, double* lat, void* stream);
mgx_status mgx_unpack_spins(const mgx_model* m, const double* lat, double* aos, void* stream);

/* ---------------------------------------------------------------- LLG plan
 * Replaces LLGSolver's fast-path state (magex/llg.py:89-98) and CudaLLG.__init__ (magex/cuda_backend.py:341-360).
 * Allocates the predictor scratch (6*N doubles) on the current device. */
mgx_status mgx_llg_create(const mgx_model* m, const mgx_llg_params* p, mgx_llg** out);
mgx_status mgx_llg_destroy(mgx_llg* plan);
/* Device pointer of the plan's predicted spins ep ((3, N) lattice layout), written by stage 0 and read
 * by stage 1: a slab decomposition exchanges its halo layers between the two stages. */
mgx_status mgx_llg_predicted(mgx_llg* plan, double** ep);
/* The reduced and fixed-point forms gather the corrector's neighbours from a split copy of ep ((3, N)
 * elements of 8 bytes: float pairs or int32 halves), written by stage 0; a slab decomposition
 * exchanges its halo layers too.  NULL for the FP64 form. */
mgx_status mgx_llg_predicted_split(mgx_llg* plan, void** eps);
/* Thermal-field amplitude sigma_i = sqrt(2 alpha_i k_B T_i / (gamma mu_i mu_B dt)) (magex/llg.py:111):
 * per sublattice (host [ns]) or per site (host [N] magex order, overrides).  Zero means no noise. */
mgx_status mgx_llg_set_sigma(mgx_llg* plan, const double* sigma_sub, const double* sigma_site);
/* Per-site field (T) added to the effective field of both stages from now on: device [3*N], lattice
 * layout, read at every launch (the caller rewrites it between stages for a field that depends on the
 * spins, as magex evaluates extra_field(e) at e and at the predicted spins, magex/llg.py:124-137);
 * NULL removes it.  FP64 plans (MGX_ERR_UNSUPPORTED otherwise). */
mgx_status mgx_llg_set_extra_field(mgx_llg* plan, const double* B_add);
/* Spin-orbit torque as effective fields B_DL e x p + B_FL p at each stage's spins, p normalised here
 * (LLGSolver(sot={p, B_DL, B_FL}), magex/llg.py:84-86,126-128); B_DL = B_FL = 0 removes it.  FP64
 * plans (MGX_ERR_UNSUPPORTED otherwise).  Synchronous: call it while no step of the plan is in flight. */
mgx_status mgx_llg_set_sot(mgx_llg* plan, const double p[3], double B_DL, double B_FL);

/* One stochastic Heun step in place on e (device, lattice layout):
 *   b = sigma * xi;  k1 = f(e, B(e) + b);  ep = |e + dt k1|^-1 (e + dt k1);
 *   k2 = f(ep, B(ep) + b);  e <- normalise(e + dt/2 (k1 + k2))
 * as magex/llg.py:216-227 and magex/fast.py:336-390.  xi is read from noise (device, lattice
 * layout, 3*N N(0,1) draws) in MGX_NOISE_HOST mode, generated by Philox4x32-10 keyed by
 * (seed, site, step) in MGX_NOISE_PHILOX mode, and ignored in MGX_NOISE_NONE mode. */
mgx_status mgx_llg_step(mgx_llg* plan, double* e, const double* noise, uint64_t step, void* stream);
/* nsteps Heun steps (noise NONE or PHILOX), steps step0 .. step0+nsteps-1. */
mgx_status mgx_llg_run(mgx_llg* plan, double* e, int64_t nsteps, uint64_t step0, void* stream);
/* One half of mgx_llg_step: stage 0 = predictor (reads e, writes the plan's ep and k1), stage 1 =
 * corrector (reads ep, k1 and e, writes e).  For callers that exchange halos between the stages,
 * as magex's slab decomposition does (magex/mpi_spin.py:160-174: _fused1, halo(ep), _fused2, halo(e)). */
mgx_status mgx_llg_stage(mgx_llg* plan, int32_t stage, double* e, const double* noise, uint64_t step, void* stream);
/* One step of mgx_llg_step on host buffers: e_in and e_out are (N, 3) float64 spins in magex site
 * order (the arrays magex's LLGSolver.step takes and returns, magex/llg.py:216-227; e_out may equal
 * e_in).  Replaces the copy in, step and copy out that a Python caller would make, with the copies
 * overlapping the stages when both buffers are page-locked (pinned) and the plan is an FP64 or
 * fixed-point-sum stencil plan of at least 2^20 sites: the input then goes to the device in axis-0
 * slabs on a copy stream of the plan, each slab is packed (and split) as it lands, the slabs'
 * predictors and correctors run on streams of the plan as soon as the slabs they gather from are
 * ready, and each finished slab goes back on an out stream while the rest is computed; the whole
 * pipeline is replayed as a CUDA graph per (e_in, e_out) pair.  Work enqueued on `stream` after
 * this call, and a synchronisation of `stream`, follow all of it.  noise as for mgx_llg_step
 * (device, lattice layout).  The plan keeps two device copies of the spins for this (6 N doubles)
 * from the first call on. */
mgx_status mgx_llg_step_host(mgx_llg* plan, const double* e_in, double* e_out, const double* noise, uint64_t step,
                             void* stream);

/* ---------------------------------------------------------------- batched ensemble
 * Many independent systems (replicas, temperature / field scans, different lattices, uneven sizes)
 * stepped together: one persistent launch per Heun stage over a (system, first site) tile list,
 * optionally replayed from a CUDA graph.  The reference steps one system per LLGSolver
 * (magex/llg.py:216-227); a batch step equals nsys such steps (the kernels share the per-site
 * code of mgx_llg_step, so each system's result is the same as its own plan's).
 * Spins of system k are the (3, N_k) lattice-layout block at 3 * mgx_batch_offset(b, k) doubles of
 * one device array of 3 * mgx_batch_nsites(b) doubles.  The models must outlive the batch. */
mgx_status mgx_batch_create(const mgx_model* const* models, const mgx_llg_params* params, int32_t nsys,
                            mgx_batch** out);   /* params[k]: per system; uniform alpha; one noise mode and integrator */
mgx_status mgx_batch_destroy(mgx_batch* b);
int64_t mgx_batch_nsites(const mgx_batch* b);
int64_t mgx_batch_offset(const mgx_batch* b, int32_t sys);        /* site offset of system sys (sys = nsys: total) */
mgx_status mgx_batch_set_sigma(mgx_batch* b, int32_t sys, const double* sigma_sub);   /* host [ns] */
/* Re-read every model's field (after mgx_model_set_field) into the batch. */
mgx_status mgx_batch_sync_models(mgx_batch* b);
/* Launch shape: threads = sites per tile and threads per CTA (64, 128, 256, 512); ctas_per_sm = resident
 * CTAs per SM of the persistent grid (0 = one CTA per tile).  Chosen by the autotuner of magex_gb300.batched. */
mgx_status mgx_batch_set_launch(mgx_batch* b, int32_t threads, int32_t ctas_per_sm);
mgx_status mgx_batch_step(mgx_batch* b, double* e, const double* noise, uint64_t step, void* stream);
/* nsteps steps (noise NONE or PHILOX) from step index step0; graph_chunk > 0 captures graph_chunk steps
 * into a CUDA graph once (per spin pointer and launch shape) and replays it. */
mgx_status mgx_batch_run(mgx_batch* b, double* e, int64_t nsteps, uint64_t step0, int32_t graph_chunk, void* stream);
/* Per-system observables: out (device) [nsys*8], 8 values per system as mgx_observables. */
mgx_status mgx_batch_observables(mgx_batch* b, const double* e, double* out, void* stream);
/* Per-system triangle lists for the topological charge: tri (host) [3*ntri] lattice indices local to each
 * system, orient (host) [ntri], tri_off (host) [nsys+1] triangle offsets (tri_off[0] = 0). */
mgx_status mgx_batch_set_triangles(mgx_batch* b, const int32_t* tri, const double* orient, const int64_t* tri_off);
mgx_status mgx_batch_topological_charge(mgx_batch* b, const double* e, double* out, void* stream);  /* out [nsys] */

/* ---------------------------------------------------------------- adjoint of the Heun step
 * No counterpart in the reference (magex has no gradients).  Reverse-mode derivative of a Heun
 * trajectory (noise NONE or PHILOX, uniform alpha, per-sublattice single-ion tensors):
 *   mgx_adjoint_forward  recomputes nsteps (<= seg_steps) steps from e0 (device, lattice layout),
 *                        storing e, ep and both total fields of every step (a checkpointed segment);
 *                        writes the final spins to e_out when not NULL;
 *   mgx_adjoint_backward maps ebar = dL/de(end of segment) to dL/de(start of segment) in place and adds
 *                        the segment's parameter gradients to per-site accumulators;
 *   mgx_adjoint_grads    sums the accumulators into out (device) [9*ngroups + 9*ns + 3]:
 *                        dL/dT_g (row-major 3x3 per coupling group g), dL/dA (component-major:
 *                        out[9G + k*ns + s] = dL/dA_s[k]), dL/dB.
 * fwd is the forward stencil model (width 9); rev is the reverse stencil: for every forward coupling
 * (i -> j, R, J) one coupling (j -> i, -R, J^T) of the same supercell, in an order grouped by receiving
 * sublattice and then by rev_group.  rev_group[b] names the parameter tensor T_g that
 * the forward coupling uses, rev_transposed[b] = 1 when that coupling is T_g^T.  */
mgx_status mgx_adjoint_create(const mgx_model* fwd, const mgx_model* rev, const int32_t* rev_group,
                              const int32_t* rev_transposed, int32_t ngroups, const mgx_llg_params* p,
                              int32_t seg_steps, mgx_adjoint** out);
mgx_status mgx_adjoint_destroy(mgx_adjoint* a);
mgx_status mgx_adjoint_set_sigma(mgx_adjoint* a, const double* sigma_sub);
mgx_status mgx_adjoint_sync_models(mgx_adjoint* a);      /* after mgx_model_set_couplings / _set_onsite / _set_field */
/* Segment storage: mgx_adjoint_storage_doubles(a) doubles per segment (14 N per step + 3 N).  By default
 * the adjoint uses one storage it owns; mgx_adjoint_set_storage switches to caller storage (device,
 * 16-byte aligned; NULL = the own one), so that segments kept resident need no recomputation. */
int64_t mgx_adjoint_storage_doubles(const mgx_adjoint* a);
mgx_status mgx_adjoint_set_storage(mgx_adjoint* a, double* storage);
/* The plan owns two storages (the second is allocated on first selection); selecting one makes it
 * the current storage.  A caller can recompute one segment into one storage on a second stream
 * while mgx_adjoint_backward runs through the other: the two share no device memory (ordering of
 * the two calls on their streams, with events, is the caller's). */
mgx_status mgx_adjoint_select_own_storage(mgx_adjoint* a, int32_t which);
mgx_status mgx_adjoint_forward(mgx_adjoint* a, const double* e0, int32_t nsteps, uint64_t step0, double* e_out,
                               void* stream);
/* nsteps: the length of the segment held by the current storage. */
mgx_status mgx_adjoint_backward(mgx_adjoint* a, double* ebar, int32_t nsteps, void* stream);
mgx_status mgx_adjoint_zero_grads(mgx_adjoint* a, void* stream);
mgx_status mgx_adjoint_grads(mgx_adjoint* a, double* out, void* stream);
/* Cubic and higher-uniaxial terms (magex/terms.py:35-75, magex/fast.py:39-64) enter the adjoint
 * through their Hessian; their parameter gradients, summed over the sites, go to out (device) [3]:
 * dL/dKc, dL/dK2, dL/dK3 (derivatives with respect to a change of every site's constant by the same
 * amount; zero when the model has none of those terms). */
mgx_status mgx_adjoint_grads_onsite_higher(mgx_adjoint* a, double* out, void* stream);
/* Which parameter gradients mgx_adjoint_backward accumulates (all three by default): the coupling
 * groups, the single-ion tensors, the field (non-zero = accumulate).  The spins' adjoint and the
 * cubic / higher-uniaxial gradients are always computed.  Skipping the ones a caller does not need
 * saves their per-site reads and writes (torch.autograd asks only for the inputs that require grad). */
mgx_status mgx_adjoint_set_needs(mgx_adjoint* a, int32_t couplings, int32_t onsite, int32_t field);

/* ---------------------------------------------------------------- step without allocation
 * No counterpart in the reference.  One Heun / Depondt step like mgx_llg_step, for callers that
 * cannot allocate GPU memory while they step: a host framework that owns all device memory through
 * its own pool and only hands the plugin its input and output buffers, or a real-time loop that must
 * never wait on the allocator.  It needs no plan: the predictor scratch (ep, k1) and the
 * per-sublattice constants live in one static device array of 64 + 6 * MGX_NOALLOC_MAX_SITES doubles
 * (12 MiB) that every GPU loading the library holds until the process exits; the call itself
 * allocates nothing.
 *   - m: a model from mgx_model_create (created beforehand) with at most MGX_NOALLOC_MAX_SITES sites;
 *     larger models are rejected with MGX_ERR_INVALID.  Cubic and higher uniaxial on-site terms of
 *     the model are stepped as in mgx_llg_step.
 *   - p: dt (finite, > 0), uniform alpha (finite, >= 0; p->alpha_site must be NULL), precession,
 *     integrator, noise mode, seed; p->precision must be MGX_PRECISION_FP64.
 *   - sigma_sub: host [ns] thermal amplitudes (finite, >= 0; read during the call), required unless
 *     p->noise is MGX_NOISE_NONE; e, noise and step as for mgx_llg_step.  A model whose moments differ
 *     site by site has per-site amplitudes, which only a plan carries: with noise it is rejected
 *     with MGX_ERR_UNSUPPORTED.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress, with that
 * device current); make that first call before any stream capture begins.  All calls on a device
 * share the array, which keeps the last call's contents: calls whose GPU work overlaps (other
 * streams or host threads) race on it and must be serialised by the caller. */
#define MGX_NOALLOC_MAX_SITES 262144
mgx_status mgx_llg_step_noalloc(const mgx_model* m, const mgx_llg_params* p, const double* sigma_sub, double* e,
                                const double* noise, uint64_t step, void* stream);

/* ---------------------------------------------------------------- observables
 * Writes 8 doubles to out (device):
 *   [0] E total (meV)  = sum_i e.A.e - e.h - mu_B mu e.B      (magex/spinmodel.py:475-484)
 *   [1..3] sum_i e_i                                          (magex/llg.py:265, e.mean(0) * N)
 *   [4..6] sum_i s_i e_i                                      (magex/spinmodel.py:517-519)
 *   [7] max_i |e_i x B_eff,i| (T)                             (magex/llg.py:250-252)
 * The sums are deterministic (fixed-shape tree reduction). */
mgx_status mgx_observables(const mgx_model* m, const double* e, double* out, void* stream);
/* The same for nlat lattices stored one after the other (lattice k at e + 3 N k, e.g. the chains of a
 * Monte Carlo ensemble): out [nlat*8]; lattice k's values equal mgx_observables of lattice k. */
mgx_status mgx_observables_n(const mgx_model* m, const double* e, int32_t nlat, double* out, void* stream);
/* Effective field B_eff (T) of spins e into B (device, lattice layout) (magex/spinmodel.py:471-473). */
mgx_status mgx_effective_field(const mgx_model* m, const double* e, double* B, void* stream);

/* Berg-Luscher topological charge over a triangle list (magex/texture.py:30-63):
 * Q = hand/(4 pi) sum_t orient_t * 2 atan2(s1.(s2 x s3), 1 + s1.s2 + s2.s3 + s3.s1).
 * tri: device [ntri*3] lattice-layout site indices; orient: device [ntri] (+-1, hand folded in).
 * Writes Q to out (device, 1 double). */
mgx_status mgx_topological_charge(const mgx_model* m, const double* e, const int32_t* tri,
                                  const double* orient, int64_t ntri, double* out, void* stream);

/* ---------------------------------------------------------------- diagnostics
 * No counterpart in the reference.  Measures the device's sustained FP64 fused multiply-add rate
 * (FLOP/s, 2 per FMA) with a register-resident DFMA loop on every SM; synchronises the device.
 * The LLG kernels are bound by this rate on GB300, so it is the denominator of their roofline. */
mgx_status mgx_measure_fp64_peak(double* flops_per_s);

/* ---------------------------------------------------------------- Monte Carlo colour sweeps
 * Replace MetropolisMC (magex/montecarlo.py:71-230) with its NumPy moves, the numba colour pass
 * _mc_group (magex/fast.py:393-490) and CudaMC / _k_mc (magex/cuda_backend.py:220-304,380-418).
 *
 * First-fit greedy colouring in magex site order (magex/montecarlo.py:35-48, the graph of every
 * coupling in both directions): host-only, no GPU needed.  colour: host [N] output. */
mgx_status mgx_colour_stencil(const mgx_lattice_desc* lat, int32_t* colour, int32_t* ncolours);
/* The same for an explicit adjacency (host CSR over magex site indices; self-loops are ignored). */
mgx_status mgx_colour_graph(int64_t nsites, const int64_t* ptr, const int32_t* nbr, int32_t* colour,
                            int32_t* ncolours);

typedef struct mgx_mc mgx_mc;
enum { MGX_MC_GAUSSIAN = 0, MGX_MC_UNIFORM = 1, MGX_MC_HEATBATH = 2, MGX_MC_HINZKE = 3 };
enum { MGX_MC_RNG_PHILOX = 0, MGX_MC_RNG_HOST = 1 };
typedef struct mgx_mc_params {
  int32_t move;              /* MGX_MC_* trial move of MetropolisMC(move=...) */
  int32_t overrelax;         /* over-relaxation passes per sweep (MetropolisMC(overrelax=...)) */
  int32_t rng;               /* MGX_MC_RNG_PHILOX (key seed) or MGX_MC_RNG_HOST (draws per sweep) */
  double sigma;              /* Gaussian cone width (adapted by the caller, magex/montecarlo.py:257-261) */
  uint64_t seed;
  int32_t precision;         /* MGX_PRECISION_FP64, or MGX_PRECISION_FP64_FIXED_GATHER: the exchange field
                              * of every trial move as an exact 56-bit fixed-point sum (stencil models
                              * with per-sublattice A and mu) */
} mgx_mc_params;
/* group_sites: host, magex site indices of every colour class in update order, concatenated
 * (group_sizes[g] each; pinned sites left out, as magex/montecarlo.py:93-99). */
mgx_status mgx_mc_create(const mgx_model* m, const mgx_mc_params* p, const int64_t* group_sites,
                         const int64_t* group_sizes, int32_t ngroups, mgx_mc** out);
mgx_status mgx_mc_destroy(mgx_mc* mc);
/* Inverse temperatures 1 / (k_B T) (1/meV; +inf at T = 0): host [ns] per sublattice, or host [N] per
 * site in magex order (site temperatures, magex/montecarlo.py:149-154).  Synchronous. */
mgx_status mgx_mc_set_beta(mgx_mc* mc, const double* beta_sub, const double* beta_site);
mgx_status mgx_mc_set_sigma(mgx_mc* mc, double sigma);
/* Doubles of host draws one sweep consumes (MGX_MC_RNG_HOST). */
mgx_status mgx_mc_host_draws(const mgx_mc* mc, int64_t* ndoubles);
/* nsweeps sweeps of the lattice-layout spins e (device): one pass of the trial move over every class
 * in order, then `overrelax` reflection passes over every class (magex/montecarlo.py:181-210).
 * MGX_MC_RNG_HOST: nsweeps = 1 and host_draws (device) holds, class after class, the draws of the
 * NumPy sweep in its order: gaussian / uniform: normal (n, 3) then uniform (n); heatbath: uniform (n),
 * uniform (n), uniform (n); hinzke: integer k in {0,1,2} (n, as doubles), normal (n, 3), normal (n, 3),
 * uniform (n); classes where some beta is infinite use the gaussian layout; then per over-relaxation
 * pass and class: uniform (n). */
mgx_status mgx_mc_sweep(mgx_mc* mc, double* e, int64_t nsweeps, const double* host_draws, void* stream);
/* Accepted trial moves and tried moves since the last reset (MetropolisMC.acceptance); synchronises
 * the stream. */
mgx_status mgx_mc_counts(mgx_mc* mc, uint64_t* accepted, uint64_t* tried, int32_t reset, void* stream);

/* Ensemble of independent chains on the plan's lattice, swept together: magex runs its (L, T) points
 * as separate processes (magex/montecarlo.py:390-401, _point :248-291); here every pass of a sweep is
 * one launch over the class's sites of all chains.  Chain k's spins are the lattice-layout block at
 * e + 3 N k; it has its own Philox key seeds[k], inverse temperature beta[k] (1/meV, finite, > 0)
 * and cone width sigma[k] (host arrays of nchains).  Each chain's trajectory equals that of a
 * one-chain plan with its key, beta and sigma.  Philox FP64 plans without site temperatures;
 * nchains = 1 with all arrays NULL returns to the plan's own single chain.  Resets the counts. */
mgx_status mgx_mc_set_chains(mgx_mc* mc, int32_t nchains, const uint64_t* seeds, const double* beta,
                             const double* sigma);
/* Per-chain accepted moves since the last reset (host [nchains]) and the tried moves (the same for
 * every chain); the cone widths (host [nchains]) when sigma is not NULL.  Synchronises the stream. */
mgx_status mgx_mc_chain_counts(mgx_mc* mc, uint64_t* accepted, uint64_t* tried, double* sigma, int32_t reset,
                               void* stream);
/* Cone-width adaptation of every chain from its acceptance a since the last reset, on the device:
 * sigma <- clip(sigma * 0.5 / max(1 - a, 0.05), 0.02, 4) (magex/montecarlo.py:257-261); resets the
 * counts. */
mgx_status mgx_mc_adapt_sigma(mgx_mc* mc, void* stream);

/* ---------------------------------------------------------------- S(q, w) sampling
 * Device-side Fourier projection m_q = N^-1/2 sum_i e_i exp(-i q.r_i) of lattice-layout spins, the
 * per-sample product ph^T e of magex/spectra.py:53-66 (structure_factor).  qfrac: host [nq*3]
 * fractional coordinates of q in the reciprocal lattice of the unit cell (any q, commensurate or not);
 * sub_phase: host [nq*ns*2] exp(-i q.p_s) of the sublattice positions as (re, im).  Stencil models. */
typedef struct mgx_fourier mgx_fourier;
mgx_status mgx_fourier_create(const mgx_model* m, int32_t nq, const double* qfrac, const double* sub_phase,
                              mgx_fourier** out);
/* mq: device [nq*3*2] output, (re, im) of m_q^x, m_q^y, m_q^z per q. */
mgx_status mgx_fourier_project(mgx_fourier* f, const double* e, double* mq, void* stream);
mgx_status mgx_fourier_destroy(mgx_fourier* f);

/* ---------------------------------------------------------------- outputs at scale (host only)
 * The text writers of magex/observables.py:122-161 and magex/llg.py:286-297, formatted in parallel;
 * the files are byte-for-byte those of magex's Python writers.  All arrays are host arrays in magex
 * site order: pos [n*3] (Angstrom), spins [n*3], mu [n], sublattice [n] indexing names[nnames]. */
mgx_status mgx_write_xyz(const char* path, int64_t n, const double* pos, const double* spins, const double* mu,
                         const int32_t* sublattice, const char* const* names, int32_t nnames, const char* comment,
                         int32_t append);
/* scalars [nscalars*n] written as "SCALARS name double 1" blocks after the spin vectors */
mgx_status mgx_write_vtk(const char* path, int64_t n, const double* pos, const double* spins, const double* scalars,
                         const char* const* scalar_names, int32_t nscalars);
mgx_status mgx_write_ovf(const char* path, int64_t n, const double* pos, const double* spins);
/* numpy.savetxt(path, values (nrows, ncols), delimiter=",", fmt=fmt, header=header, comments="") for
 * fmt one of "%.6f", "%.8g", "%.6g", "%.8e"; header may be NULL. */
mgx_status mgx_write_csv(const char* path, int64_t nrows, int32_t ncols, const double* values, const char* fmt,
                         const char* header);

#ifdef __cplusplus
}
#endif
#endif /* MGX_H */
