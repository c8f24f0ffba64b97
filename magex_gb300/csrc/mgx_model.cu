// Model creation (stencil tables, per-site overrides), spin layout conversion and error state.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx {

static thread_local std::string g_last_error;

mgx_status set_error(mgx_status code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

mgx_status cuda_error(cudaError_t err, const char* where) {
  const mgx_status code = (err == cudaErrorMemoryAllocation) ? MGX_ERR_NOMEM : MGX_ERR_CUDA;
  return set_error(code, "CUDA error %s (%s) in %s", cudaGetErrorName(err), cudaGetErrorString(err), where);
}

// magex site order (cell*ns + s) -> lattice index (s*ncell + cell): magex-order (N, 3) rows [begin, begin + count) <-> lattice layout (3, N)
__global__ void k_pack(const double* __restrict__ aos, double* __restrict__ lat, int ns, int ncell, long long N,
                       long long begin, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const long long site = begin + i;
  const long long cell = site / ns;
  const int s = (int)(site - cell * ns);
  const long long q = (long long)s * ncell + cell;
  lat[q] = aos[3 * site];
  lat[N + q] = aos[3 * site + 1];
  lat[2 * N + q] = aos[3 * site + 2];
}

__global__ void k_unpack(const double* __restrict__ lat, double* __restrict__ aos, int ns, int ncell, long long N,
                         long long begin, long long count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const long long site = begin + i;
  const long long cell = site / ns;
  const int s = (int)(site - cell * ns);
  const long long q = (long long)s * ncell + cell;
  aos[3 * site] = lat[q];
  aos[3 * site + 1] = lat[N + q];
  aos[3 * site + 2] = lat[2 * N + q];
}

void enqueue_pack(const Model* m, const double* aos, double* lat, long long begin, long long count, cudaStream_t st) {
  if (count <= 0) return;
  k_pack<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(aos, lat, m->d.ns, m->d.ncell, m->d.N, begin, count);
}

void enqueue_unpack(const Model* m, const double* lat, double* aos, long long begin, long long count, cudaStream_t st) {
  if (count <= 0) return;
  k_unpack<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(lat, aos, m->d.ns, m->d.ncell, m->d.N, begin, count);
}

template <typename T>
static std::vector<T> to_lattice_order(const T* src, int per_site, int ns, int ncell) {
  const long long N = (long long)ns * ncell;
  std::vector<T> out((size_t)N * per_site);
  for (long long site = 0; site < N; ++site) {
    const long long cell = site / ns;
    const int s = (int)(site - cell * ns);
    const long long q = (long long)s * ncell + cell;
    for (int k = 0; k < per_site; ++k) out[(size_t)k * N + q] = src[(size_t)site * per_site + k];
  }
  return out;
}

}  // namespace mgx

using namespace mgx;

extern "C" {

int32_t mgx_version(void) { return MGX_VERSION; }

void mgx_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return;
  const size_t n = std::min(len - 1, g_last_error.size());
  std::memcpy(buf, g_last_error.data(), n);
  buf[n] = '\0';
}

mgx_status mgx_model_create(const mgx_lattice_desc* lat, const mgx_site_desc* sites, mgx_model** out) {
  if (!lat || !out) return set_error(MGX_ERR_INVALID, "mgx_model_create: null argument");
  *out = nullptr;
  const int ns = lat->ns;
  if (ns < 1 || ns > MGX_MAX_SUBLATTICES)
    return set_error(MGX_ERR_INVALID, "ns = %d outside 1..%d", ns, MGX_MAX_SUBLATTICES);
  for (int a = 0; a < 3; ++a)
    if (lat->L[a] < 1) return set_error(MGX_ERR_INVALID, "supercell L[%d] = %d must be >= 1", a, lat->L[a]);
  const long long ncell_ll = (long long)lat->L[0] * lat->L[1] * lat->L[2];
  if (ncell_ll * ns > (1LL << 40) || ncell_ll > 0x7fffffffLL)
    return set_error(MGX_ERR_INVALID, "supercell too large (%lld cells)", ncell_ll);
  const int nb = lat->nbond;
  if (nb < 0 || nb > MGX_MAX_BONDS) return set_error(MGX_ERR_INVALID, "nbond = %d outside 0..%d", nb, MGX_MAX_BONDS);
  const int W = lat->width;
  if (W != 1 && W != 4 && W != 9) return set_error(MGX_ERR_INVALID, "coupling width %d must be 1, 4 or 9", W);
  if (nb > 0 && (!lat->bond_src || !lat->bond_dst || !lat->bond_R || !lat->bond_table))
    return set_error(MGX_ERR_INVALID, "bond arrays must not be null");
  if (!lat->mu_sub) return set_error(MGX_ERR_INVALID, "mu_sub must not be null");

  // couplings grouped by receiving sublattice, keeping their given order inside a group
  std::vector<int> off(ns + 1, 0);
  for (int b = 0; b < nb; ++b) {
    const int i = lat->bond_src[b], j = lat->bond_dst[b];
    if (i < 0 || i >= ns || j < 0 || j >= ns)
      return set_error(MGX_ERR_INVALID, "bond %d: sublattices (%d, %d) outside 0..%d", b, i, j, ns - 1);
    off[i + 1]++;
  }
  for (int s = 0; s < ns; ++s) off[s + 1] += off[s];
  std::vector<int> fill(off.begin(), off.end() - 1);
  std::vector<int> slot_of(std::max(nb, 1), 0);
  std::vector<int4> geo(std::max(nb, 1));
  std::vector<double> J((size_t)std::max(nb, 1) * W, 0.0);
  int reach0 = 0;
  for (int b = 0; b < nb; ++b) {
    const int i = lat->bond_src[b];
    const int slot = fill[i]++;
    slot_of[b] = slot;
    int d[3];
    bool self = (lat->bond_dst[b] == i);
    for (int a = 0; a < 3; ++a) {
      const int R = lat->bond_R[3 * b + a];
      const int La = lat->L[a];
      if (lat->pbc[a]) {
        d[a] = ((R % La) + La) % La;
        self &= (d[a] == 0);
      } else {
        if (R <= -La || R >= La) { d[a] = La; }   // never inside the box: coupling has no partner
        else d[a] = R;
        self &= (R == 0);
      }
    }
    if (self)
      return set_error(MGX_ERR_INVALID,
                       "bond %d couples a site to its own periodic image; fold it into A_sub first", b);
    geo[slot] = make_int4(lat->bond_dst[b], d[0], d[1], d[2]);
    const int R0 = lat->bond_R[3 * b];
    reach0 = std::max(reach0, lat->pbc[0] ? std::min(d[0], lat->L[0] - d[0]) : (d[0] == lat->L[0] ? 0 : std::abs(R0)));
    for (int k = 0; k < W; ++k) J[(size_t)slot * W + k] = lat->bond_table[(size_t)b * W + k];
  }

  std::vector<double> A(ns * 9, 0.0), inv_mu(ns), mu(ns), sgn(ns, 1.0);
  bool has_A = false;
  for (int s = 0; s < ns; ++s) {
    mu[s] = lat->mu_sub[s];
    if (!(mu[s] > 0.0)) return set_error(MGX_ERR_INVALID, "moment of sublattice %d must be > 0", s);
    inv_mu[s] = 1.0 / (mu[s] * 5.7883818060e-2);
    if (lat->sign_sub) sgn[s] = lat->sign_sub[s];
    if (lat->A_sub)
      for (int k = 0; k < 9; ++k) {
        A[s * 9 + k] = lat->A_sub[s * 9 + k];
        has_A |= (A[s * 9 + k] != 0.0);
      }
  }

  Model* m = new Model();
  m->slot_of_bond = new int[std::max(nb, 1)];
  std::copy(slot_of.begin(), slot_of.end(), m->slot_of_bond);
  DevLattice& d = m->d;
  d.ns = ns;
  d.L0 = lat->L[0];
  d.cell_offset = 0;
  d.own0_begin = 0;
  d.own0_end = lat->L[0];
  d.L1 = lat->L[1];
  d.L2 = lat->L[2];
  d.ncell = (int)ncell_ll;
  d.N = ncell_ll * ns;
  d.pbc0 = lat->pbc[0] != 0;
  d.pbc1 = lat->pbc[1] != 0;
  d.pbc2 = lat->pbc[2] != 0;
  d.width = W;
  d.B0 = lat->B[0];
  d.B1 = lat->B[1];
  d.B2 = lat->B[2];
  m->nbond = nb;
  m->reach0 = reach0;

  // one device block for all small tables: [off | geo | J | A | inv_mu | mu | sign]
  const size_t s_off = 0, n_off = sizeof(int) * (ns + 1);
  const size_t s_geo = (s_off + n_off + 15) / 16 * 16, n_geo = sizeof(int4) * geo.size();
  const size_t s_J = (s_geo + n_geo + 15) / 16 * 16, n_J = sizeof(double) * J.size();
  const size_t s_A = (s_J + n_J + 15) / 16 * 16, n_A = sizeof(double) * A.size();
  const size_t s_inv = s_A + n_A, n_sub = sizeof(double) * ns;
  const size_t s_mu = s_inv + n_sub, s_sg = s_mu + n_sub, total = s_sg + n_sub;
  std::vector<char> host(total, 0);
  std::memcpy(host.data() + s_off, off.data(), n_off);
  std::memcpy(host.data() + s_geo, geo.data(), n_geo);
  std::memcpy(host.data() + s_J, J.data(), n_J);
  std::memcpy(host.data() + s_A, A.data(), n_A);
  std::memcpy(host.data() + s_inv, inv_mu.data(), n_sub);
  std::memcpy(host.data() + s_mu, mu.data(), n_sub);
  std::memcpy(host.data() + s_sg, sgn.data(), n_sub);
  cudaError_t err = cudaMalloc(&m->dev_block, total);
  if (err == cudaSuccess) err = cudaMemcpy(m->dev_block, host.data(), total, cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    mgx_model_destroy(reinterpret_cast<mgx_model*>(m));
    return cuda_error(err, "mgx_model_create tables");
  }
  char* base = (char*)m->dev_block;
  d.bond_off = (const int*)(base + s_off);
  d.bond_geo = (const int4*)(base + s_geo);
  d.bond_J = (const double*)(base + s_J);
  d.A_sub = (const double*)(base + s_A);
  d.inv_mu_sub = (const double*)(base + s_inv);
  d.mu_sub = (const double*)(base + s_mu);
  d.sign_sub = (const double*)(base + s_sg);
  d.has_A = has_A ? 1 : 0;

  if (sites) {
    const long long N = d.N;
    if (sites->A_site) {
      std::vector<double> v = to_lattice_order(sites->A_site, 9, ns, d.ncell);
      for (double x : v) has_A |= (x != 0.0);
      err = cudaMalloc(&m->A_site, sizeof(double) * v.size());
      if (err == cudaSuccess) err = cudaMemcpy(m->A_site, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice);
      if (err != cudaSuccess) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return cuda_error(err, "mgx_model_create A_site"); }
      d.A_site = m->A_site;
      d.has_A = has_A ? 1 : 0;
    }
    if (sites->mu_site) {
      std::vector<double> v = to_lattice_order(sites->mu_site, 1, ns, d.ncell), inv(N);
      for (long long q = 0; q < N; ++q) {
        if (!(v[q] > 0.0)) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return set_error(MGX_ERR_INVALID, "mu_site must be > 0"); }
        inv[q] = 1.0 / (v[q] * 5.7883818060e-2);
      }
      err = cudaMalloc(&m->mu_site, sizeof(double) * N);
      if (err == cudaSuccess) err = cudaMalloc(&m->inv_mu_site, sizeof(double) * N);
      if (err == cudaSuccess) err = cudaMemcpy(m->mu_site, v.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
      if (err == cudaSuccess) err = cudaMemcpy(m->inv_mu_site, inv.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
      if (err != cudaSuccess) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return cuda_error(err, "mgx_model_create mu_site"); }
      d.mu_site = m->mu_site;
      d.inv_mu_site = m->inv_mu_site;
    }
    if (sites->pinned) {
      std::vector<uint8_t> v = to_lattice_order(sites->pinned, 1, ns, d.ncell);
      bool any = false;
      for (auto& x : v) { x = x ? 1 : 0; any |= x != 0; }
      if (any) {
        err = cudaMalloc(&m->pinned, N);
        if (err == cudaSuccess) err = cudaMemcpy(m->pinned, v.data(), N, cudaMemcpyHostToDevice);
        if (err != cudaSuccess) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return cuda_error(err, "mgx_model_create pinned"); }
        d.pinned = m->pinned;
      }
    }
  }
  *out = reinterpret_cast<mgx_model*>(m);
  return MGX_OK;
}

mgx_status mgx_model_create_csr(const mgx_csr_desc* c, mgx_model** out) {
  if (!c || !out) return set_error(MGX_ERR_INVALID, "mgx_model_create_csr: null argument");
  *out = nullptr;
  const long long N = c->nsites;
  if (N < 1 || N > 0x7fffffffLL) return set_error(MGX_ERR_INVALID, "nsites = %lld outside 1..2^31-1", N);
  const int W = c->width;
  if (W != 1 && W != 4 && W != 9) return set_error(MGX_ERR_INVALID, "coupling width %d must be 1, 4 or 9", W);
  if (!c->ptr || !c->mu_site) return set_error(MGX_ERR_INVALID, "ptr and mu_site must not be null");
  if (c->ptr[0] != 0) return set_error(MGX_ERR_INVALID, "ptr[0] must be 0");
  for (long long i = 0; i < N; ++i)
    if (c->ptr[i + 1] < c->ptr[i]) return set_error(MGX_ERR_INVALID, "ptr must be non-decreasing (site %lld)", i);
  const long long nnz = c->ptr[N];
  if (nnz > 0 && (!c->nbr || !c->typ || !c->table)) return set_error(MGX_ERR_INVALID, "nbr, typ and table must not be null");
  if (c->ntypes < (nnz > 0 ? 1 : 0)) return set_error(MGX_ERR_INVALID, "ntypes must be >= 1");
  for (long long k = 0; k < nnz; ++k) {
    if (c->nbr[k] < 0 || c->nbr[k] >= N) return set_error(MGX_ERR_INVALID, "nbr[%lld] = %d outside 0..N-1", k, c->nbr[k]);
    if (c->typ[k] < 0 || c->typ[k] >= c->ntypes) return set_error(MGX_ERR_INVALID, "typ[%lld] = %d outside 0..ntypes-1", k, c->typ[k]);
  }
  std::vector<double> inv(N);
  for (long long i = 0; i < N; ++i) {
    if (!(c->mu_site[i] > 0.0)) return set_error(MGX_ERR_INVALID, "mu_site[%lld] must be > 0", i);
    inv[i] = 1.0 / (c->mu_site[i] * 5.7883818060e-2);
  }
  Model* m = new Model();
  DevLattice& d = m->d;
  d.ns = 1;
  d.L0 = 1;
  d.cell_offset = 0;
  d.own0_begin = 0;
  d.own0_end = 1;
  d.L1 = 1;
  d.L2 = (int)N;
  d.ncell = (int)N;
  d.N = N;
  d.pbc0 = d.pbc1 = d.pbc2 = 1;
  d.width = W;
  d.B0 = c->B[0];
  d.B1 = c->B[1];
  d.B2 = c->B[2];
  d.layout = 1;
  m->nbond = 0;
  m->slot_of_bond = new int[1];
  const int nt = std::max(c->ntypes, 1);
  // dev_block: [off (2 ints) | J (nt*W) | A_sub (9) | inv_mu | mu | sign (1 each)]
  const size_t s_J = 16, n_J = sizeof(double) * (size_t)nt * W;
  const size_t s_A = s_J + n_J, s_inv = s_A + 9 * sizeof(double), s_mu = s_inv + 8, s_sg = s_mu + 8, total = s_sg + 8;
  std::vector<char> host(total, 0);
  if (c->ntypes > 0) std::memcpy(host.data() + s_J, c->table, sizeof(double) * (size_t)c->ntypes * W);
  const double one = 1.0;
  std::memcpy(host.data() + s_inv, &one, 8);
  std::memcpy(host.data() + s_mu, &one, 8);
  std::memcpy(host.data() + s_sg, &one, 8);
  const size_t c_ptr = 0, c_nbr = sizeof(long long) * (N + 1), c_typ = c_nbr + sizeof(int) * (size_t)std::max(nnz, 1LL);
  const size_t c_total = c_typ + sizeof(int) * (size_t)std::max(nnz, 1LL);
  cudaError_t err = cudaMalloc(&m->dev_block, total);
  if (err == cudaSuccess) err = cudaMemcpy(m->dev_block, host.data(), total, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMalloc(&m->csr_block, c_total);
  if (err == cudaSuccess) err = cudaMemcpy((char*)m->csr_block + c_ptr, c->ptr, sizeof(long long) * (N + 1), cudaMemcpyHostToDevice);
  if (err == cudaSuccess && nnz > 0) err = cudaMemcpy((char*)m->csr_block + c_nbr, c->nbr, sizeof(int) * nnz, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && nnz > 0) err = cudaMemcpy((char*)m->csr_block + c_typ, c->typ, sizeof(int) * nnz, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMalloc(&m->mu_site, sizeof(double) * N);
  if (err == cudaSuccess) err = cudaMalloc(&m->inv_mu_site, sizeof(double) * N);
  if (err == cudaSuccess) err = cudaMemcpy(m->mu_site, c->mu_site, sizeof(double) * N, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(m->inv_mu_site, inv.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    mgx_model_destroy(reinterpret_cast<mgx_model*>(m));
    return cuda_error(err, "mgx_model_create_csr");
  }
  char* base = (char*)m->dev_block;
  d.bond_off = (const int*)base;
  d.bond_geo = nullptr;
  d.bond_J = (const double*)(base + s_J);
  d.A_sub = (const double*)(base + s_A);
  d.inv_mu_sub = (const double*)(base + s_inv);
  d.mu_sub = (const double*)(base + s_mu);
  d.sign_sub = (const double*)(base + s_sg);
  d.mu_site = m->mu_site;
  d.inv_mu_site = m->inv_mu_site;
  d.csr_ptr = (const long long*)((char*)m->csr_block + c_ptr);
  d.csr_nbr = (const int*)((char*)m->csr_block + c_nbr);
  d.csr_typ = (const int*)((char*)m->csr_block + c_typ);
  d.has_A = 0;
  if (c->A_site) {
    bool any = false;
    for (long long k = 0; k < 9 * N; ++k) any |= c->A_site[k] != 0.0;
    if (any) {
      std::vector<double> v((size_t)9 * N);
      for (long long i = 0; i < N; ++i)
        for (int k = 0; k < 9; ++k) v[(size_t)k * N + i] = c->A_site[(size_t)i * 9 + k];
      err = cudaMalloc(&m->A_site, sizeof(double) * v.size());
      if (err == cudaSuccess) err = cudaMemcpy(m->A_site, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice);
      if (err != cudaSuccess) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return cuda_error(err, "A_site"); }
      d.A_site = m->A_site;
      d.has_A = 1;
    }
  }
  if (c->sign_site) {
    err = cudaMalloc(&m->sign_site, sizeof(double) * N);
    if (err == cudaSuccess) err = cudaMemcpy(m->sign_site, c->sign_site, sizeof(double) * N, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return cuda_error(err, "sign_site"); }
    d.sign_site = m->sign_site;
  }
  if (c->pinned) {
    bool any = false;
    for (long long i = 0; i < N; ++i) any |= c->pinned[i] != 0;
    if (any) {
      std::vector<uint8_t> v(N);
      for (long long i = 0; i < N; ++i) v[i] = c->pinned[i] ? 1 : 0;
      err = cudaMalloc(&m->pinned, N);
      if (err == cudaSuccess) err = cudaMemcpy(m->pinned, v.data(), N, cudaMemcpyHostToDevice);
      if (err != cudaSuccess) { mgx_model_destroy(reinterpret_cast<mgx_model*>(m)); return cuda_error(err, "pinned"); }
      d.pinned = m->pinned;
    }
  }
  *out = reinterpret_cast<mgx_model*>(m);
  return MGX_OK;
}

mgx_status mgx_model_set_onsite_higher(mgx_model* mm, const double* Kc, const double* C, const double* K2,
                                       const double* K3, const double* u) {
  Model* m = reinterpret_cast<Model*>(mm);
  if (!m) return set_error(MGX_ERR_INVALID, "mgx_model_set_onsite_higher: null model");
  if ((Kc && !C) || (K2 && !u))
    return set_error(MGX_ERR_INVALID, "mgx_model_set_onsite_higher: Kc needs the cubic axes C, K2 the axis u");
  DevLattice& d = m->d;
  const long long N = d.N, ncell = d.ncell;
  const int ns = d.ns;
  cudaFree(m->higher_site);
  m->higher_site = nullptr;
  d.Kc_site = d.K2_site = d.K3_site = nullptr;
  if (!Kc && !K2) return MGX_OK;
  // magex site i = cell * ns + s  ->  lattice index s * ncell + cell
  std::vector<double> h(3 * (size_t)N, 0.0);
  for (long long i = 0; i < N; ++i) {
    const long long q = (i % ns) * ncell + i / ns;
    if (Kc) h[q] = Kc[i];
    if (K2) {
      h[N + q] = K2[i];
      h[2 * N + q] = K3 ? K3[i] : 0.0;
    }
  }
  MGX_CUDA_TRY(cudaMalloc(&m->higher_site, sizeof(double) * 3 * N));
  MGX_CUDA_TRY(cudaMemcpy(m->higher_site, h.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
  if (Kc) {
    d.Kc_site = m->higher_site;
    for (int k = 0; k < 9; ++k) d.C[k] = C[k];
  }
  if (K2) {
    d.K2_site = m->higher_site + N;
    d.K3_site = m->higher_site + 2 * N;
    for (int k = 0; k < 3; ++k) d.u[k] = u[k];
  }
  return MGX_OK;
}

mgx_status mgx_model_destroy(mgx_model* mm) {
  Model* m = reinterpret_cast<Model*>(mm);
  if (!m) return MGX_OK;
  cudaFree(m->dev_block);
  cudaFree(m->A_site);
  cudaFree(m->inv_mu_site);
  cudaFree(m->mu_site);
  cudaFree(m->pinned);
  cudaFree(m->partials);
  cudaFree(m->csr_block);
  cudaFree(m->sign_site);
  cudaFree(m->higher_site);
  delete[] m->slot_of_bond;
  delete m;
  return MGX_OK;
}

mgx_status mgx_model_set_couplings(mgx_model* mm, const double* bond_table) {
  Model* m = reinterpret_cast<Model*>(mm);
  if (!m || (!bond_table && m->nbond > 0)) return set_error(MGX_ERR_INVALID, "mgx_model_set_couplings: null argument");
  const int W = m->d.width, nb = m->nbond;
  std::vector<double> J((size_t)std::max(nb, 1) * W, 0.0);
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < W; ++k) {
      const double v = bond_table[(size_t)b * W + k];
      if (!std::isfinite(v)) return set_error(MGX_ERR_INVALID, "coupling %d is not finite", b);
      J[(size_t)m->slot_of_bond[b] * W + k] = v;
    }
  if (nb > 0)
    MGX_CUDA_TRY(cudaMemcpy(const_cast<double*>(m->d.bond_J), J.data(), sizeof(double) * nb * W, cudaMemcpyHostToDevice));
  return MGX_OK;
}

mgx_status mgx_model_set_onsite(mgx_model* mm, const double* A_sub) {
  Model* m = reinterpret_cast<Model*>(mm);
  if (!m || !A_sub) return set_error(MGX_ERR_INVALID, "mgx_model_set_onsite: null argument");
  if (m->d.A_site) return set_error(MGX_ERR_INVALID, "the model has per-site single-ion tensors");
  bool has_A = false;
  for (int k = 0; k < 9 * m->d.ns; ++k) {
    if (!std::isfinite(A_sub[k])) return set_error(MGX_ERR_INVALID, "single-ion tensor is not finite");
    has_A |= A_sub[k] != 0.0;
  }
  MGX_CUDA_TRY(cudaMemcpy(const_cast<double*>(m->d.A_sub), A_sub, sizeof(double) * 9 * m->d.ns, cudaMemcpyHostToDevice));
  m->d.has_A = has_A ? 1 : 0;
  return MGX_OK;
}

mgx_status mgx_model_set_field(mgx_model* mm, const double B[3]) {
  Model* m = reinterpret_cast<Model*>(mm);
  if (!m || !B) return set_error(MGX_ERR_INVALID, "mgx_model_set_field: null argument");
  m->d.B0 = B[0];
  m->d.B1 = B[1];
  m->d.B2 = B[2];
  return MGX_OK;
}

mgx_status mgx_model_set_partition(mgx_model* mm, int64_t cell_offset, int32_t own_begin, int32_t own_end) {
  Model* m = reinterpret_cast<Model*>(mm);
  if (!m) return set_error(MGX_ERR_INVALID, "mgx_model_set_partition: null model");
  if (m->d.layout != 0) return set_error(MGX_ERR_UNSUPPORTED, "mgx_model_set_partition: lattice (stencil) models only");
  if (own_begin < 0 || own_end > m->d.L0 || own_begin > own_end)
    return set_error(MGX_ERR_INVALID, "mgx_model_set_partition: owned range [%d, %d) outside [0, %d)", own_begin,
                     own_end, m->d.L0);
  m->d.cell_offset = cell_offset;
  m->d.own0_begin = own_begin;
  m->d.own0_end = own_end;
  return MGX_OK;
}

mgx_status mgx_lattice_layers(const mgx_model* mm, double* x, int32_t c0_begin, int32_t c0_end, double* buf,
                              int32_t to_buffer, void* stream) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !x || !buf) return set_error(MGX_ERR_INVALID, "mgx_lattice_layers: null argument");
  if (m->d.layout != 0) return set_error(MGX_ERR_UNSUPPORTED, "mgx_lattice_layers: lattice (stencil) models only");
  if (c0_begin < 0 || c0_end > m->d.L0 || c0_begin > c0_end)
    return set_error(MGX_ERR_INVALID, "mgx_lattice_layers: layers [%d, %d) outside [0, %d)", c0_begin, c0_end, m->d.L0);
  if (c0_begin == c0_end) return MGX_OK;
  // the layers of every (component, sublattice) block are one contiguous run: one strided 2D copy
  const size_t layer = (size_t)m->d.L1 * m->d.L2;
  const size_t width = sizeof(double) * layer * (size_t)(c0_end - c0_begin);
  const size_t pitch = sizeof(double) * (size_t)m->d.ncell;
  const size_t rows = 3 * (size_t)m->d.ns;
  double* field = x + layer * (size_t)c0_begin;
  if (to_buffer)
    MGX_CUDA_TRY(cudaMemcpy2DAsync(buf, width, field, pitch, width, rows, cudaMemcpyDefault, (cudaStream_t)stream));
  else
    MGX_CUDA_TRY(cudaMemcpy2DAsync(field, pitch, buf, width, width, rows, cudaMemcpyDefault, (cudaStream_t)stream));
  return MGX_OK;
}

int64_t mgx_model_nsites(const mgx_model* mm) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  return m ? (int64_t)m->d.N : -1;
}

mgx_status mgx_pack_spins(const mgx_model* mm, const double* aos, double* lat, void* stream) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !aos || !lat) return set_error(MGX_ERR_INVALID, "mgx_pack_spins: null argument");
  if (aos == lat) return set_error(MGX_ERR_INVALID, "mgx_pack_spins: in-place conversion is not supported");
  enqueue_pack(m, aos, lat, 0, m->d.N, (cudaStream_t)stream);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

mgx_status mgx_unpack_spins(const mgx_model* mm, const double* lat, double* aos, void* stream) {
  const Model* m = reinterpret_cast<const Model*>(mm);
  if (!m || !aos || !lat) return set_error(MGX_ERR_INVALID, "mgx_unpack_spins: null argument");
  if (aos == lat) return set_error(MGX_ERR_INVALID, "mgx_unpack_spins: in-place conversion is not supported");
  enqueue_unpack(m, lat, aos, 0, m->d.N, (cudaStream_t)stream);
  MGX_CUDA_TRY(cudaGetLastError());
  return MGX_OK;
}

}  // extern "C"
