// C ABI for cases: boundary tables, SST wall data, and the residual / JVP entry points.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>

#include "internal.cuh"

size_t fv_residual_work_bytes(int dim, int turb, long nc, long nf, int sweeps, int advection);
size_t fv_adjoint_work_bytes(int dim, int turb, long nc, long nf, int sweeps, int advection);
size_t fv_aux_bytes(int dim, int turb, long nf);
extern "C" int fv_dot_f64(long n, const double* x, const double* y, double* out, void* stream);
int fv_residual_init_constants();

namespace {

template <class X>
int upload_face_table(const FvMesh* m, const X* host, int width, X fill, X** dev, cudaStream_t s) {
  // reference face order (nf, width) row-major -> internal order (width, nf)
  std::vector<X> h((size_t)m->nf * width, fill);
  if (host) {
    for (int i = 0; i < m->nf; ++i) {
      int r = m->h_face_old[i];
      for (int j = 0; j < width; ++j) h[(size_t)j * m->nf + i] = host[(size_t)r * width + j];
    }
  }
  FV_CUDA_TRY(cudaMalloc(dev, sizeof(X) * h.size()));
  FV_CUDA_TRY(cudaMemcpyAsync(*dev, h.data(), sizeof(X) * h.size(), cudaMemcpyHostToDevice, s));
  return FV_OK;
}

// ---- log-solved turbulence scalars (LogScalars, aquaflux/turbulence/coupled.py:178-207)
// The kernels run in the physical fields; the entry points below map the solved state to them
// (phi = exp(w) on the transformed blocks, the tangent by the chain factor phi) and scale the
// state cotangents and Jacobian columns they return by the same chain factor d(phi)/d(w) = phi.
__device__ __forceinline__ bool log_field(int f, int kf, int tr) {
  return (f == kf && (tr & 1)) || (f == kf + 1 && (tr & 2));
}

__global__ void k_to_physical(long nc, int nfld, int kf, int tr, const double* s, double* p) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)nfld * nc) return;
  p[i] = log_field((int)(i / nc), kf, tr) ? exp(s[i]) : s[i];
}

__global__ void k_tangent_to_physical(long nc, int nfld, int kf, int tr, const double* p,
                                      const double* t, double* pt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)nfld * nc) return;
  pt[i] = log_field((int)(i / nc), kf, tr) ? p[i] * t[i] : t[i];
}

// v *= phi on the transformed blocks (a state cotangent / partial derivative)
__global__ void k_chain_state(long nc, int kf, int tr, const double* p, double* v) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * nc) return;
  const long j = (long)kf * nc + i;
  if (log_field((int)(j / nc), kf, tr)) v[j] *= p[j];
}

// Jacobian columns of the transformed fields times phi of the column cell (BSR, nfld x nfld
// row-major blocks, one thread per block row of cell c and field q).
template <class V>
__global__ void k_chain_bsr(int nc, int nfld, int kf, int tr, const int* indptr, const int* indices,
                            const double* p, V* values) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nfld * nc) return;
  const int c = (int)(t % nc), q = (int)(t / nc);
  for (int b = indptr[c]; b < indptr[c + 1]; ++b) {
    const int j = indices[b];
    V* row = values + ((long)b * nfld + q) * nfld;
    for (int r = kf; r <= kf + 1; ++r)
      if (log_field(r, kf, tr)) row[r] = (V)(row[r] * p[(long)r * nc + j]);
  }
}

__global__ void k_axpy_shift(long n, const double* shift, const double* v, double* out) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += shift[i] * v[i];
}

__global__ void k_inv_distance(int nc, const double* wd, double* inv) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double r = wd[c] > 0.0 ? 1.0 / wd[c] : 0.0;
  inv[c] = r;
  inv[nc + c] = r * r;
}

__global__ void k_cell_to_rowmajor(int nc, int dim, const double* in, double* out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int j = 0; j < dim; ++j) out[(long)c * dim + j] = in[(long)j * nc + c];
}

}  // namespace

// The physical state of a log-transformed case (written into c->phys), or `state` itself.
static const double* physical_state(FvCase* c, const double* state, cudaStream_t s) {
  if (!c->desc.scalar_transform) return state;
  const long nc = c->mesh->nc;
  k_to_physical<<<fv_blocks((long)c->nfld * nc, 256), 256, 0, s>>>(
      nc, c->nfld, c->mesh->dim + 1, c->desc.scalar_transform, state, c->phys);
  return c->phys;
}

// The physical tangent of `t` at the state last mapped by physical_state (into c->tphys).
static const double* physical_tangent(FvCase* c, const double* t, cudaStream_t s) {
  if (!c->desc.scalar_transform || !t) return t;
  const long nc = c->mesh->nc;
  k_tangent_to_physical<<<fv_blocks((long)c->nfld * nc, 256), 256, 0, s>>>(
      nc, c->nfld, c->mesh->dim + 1, c->desc.scalar_transform, c->phys, t, c->tphys);
  return c->tphys;
}

static void chain_state(FvCase* c, double* v, cudaStream_t s) {
  if (!c->desc.scalar_transform || !v) return;
  const long nc = c->mesh->nc;
  k_chain_state<<<fv_blocks(2 * nc, 256), 256, 0, s>>>(nc, c->mesh->dim + 1,
                                                        c->desc.scalar_transform, c->phys, v);
}


// Warp-coherent order of the cell stages.  The control flow of a cell-centric stage follows the
// cell's face list: at each position an interior face the cell owns, an interior face it is the
// neighbour of, or a boundary face with its (flow, k, omega, SST-wall) table entry.  Cells with
// the same pattern take the same branches, so the order groups them: patterns ascending, natural
// order inside a group.  On a renumbered mesh the natural order interleaves the few boundary and
// wall patterns with the interior one in nearly every warp, and a diverged warp issues the
// floating-point work of every branch its lanes take.
static int build_cell_order(FvCase* c, const signed char* flow_kind, const signed char* k_kind,
                     const signed char* omega_kind, const unsigned char* sst_wall,
                     cudaStream_t s) {
  const FvMesh* m = c->mesh;
  const int nc = m->nc, nfi = m->nfi, nf = m->nf;
  std::map<uint32_t, int> types;  // boundary table entry -> pattern symbol 2, 3, ... (max 15)
  std::vector<unsigned char> bsym(nf - nfi);
  for (int i = nfi; i < nf; ++i) {
    const int r = m->h_face_old[i];
    const uint32_t key = (uint32_t)(unsigned char)flow_kind[r] |
                         (uint32_t)(unsigned char)(k_kind ? k_kind[r] : -1) << 8 |
                         (uint32_t)(unsigned char)(omega_kind ? omega_kind[r] : -1) << 16 |
                         (uint32_t)(sst_wall && sst_wall[r] ? 1 : 0) << 24;
    const int id = types.emplace(key, (int)types.size()).first->second;
    bsym[i - nfi] = (unsigned char)std::min(2 + id, 15);
  }
  // pattern code: face count in the top byte, 4 bits per position for the first 14 faces
  std::vector<uint64_t> code(nc);
  for (int cell = 0; cell < nc; ++cell) {
    const int b = m->h_cf_ptr[cell], e = m->h_cf_ptr[cell + 1];
    uint64_t v = (uint64_t)std::min(e - b, 255) << 56;
    for (int p = 0; p < e - b && p < 14; ++p) {
      const unsigned ent = m->h_cf_face[b + p];
      const int f = (int)(ent & ~FV_NB_BIT);
      const uint64_t sym = f < nfi ? ((ent & FV_NB_BIT) ? 1 : 0) : bsym[f - nfi];
      v |= sym << (4 * p);
    }
    code[cell] = v;
  }
  std::unordered_map<uint64_t, int> cls;
  for (int cell = 0; cell < nc; ++cell) cls.emplace(code[cell], 0);
  std::vector<uint64_t> keys;
  keys.reserve(cls.size());
  for (const auto& kv : cls) keys.push_back(kv.first);
  std::sort(keys.begin(), keys.end());
  for (size_t i = 0; i < keys.size(); ++i) cls[keys[i]] = (int)i;
  std::vector<int> start(keys.size() + 1, 0), cid(nc);
  for (int cell = 0; cell < nc; ++cell) {
    cid[cell] = cls[code[cell]];
    start[cid[cell] + 1]++;
  }
  for (size_t i = 0; i < keys.size(); ++i) start[i + 1] += start[i];
  std::vector<int> order(nc);
  for (int cell = 0; cell < nc; ++cell) order[start[cid[cell]]++] = cell;
  if (!c->sched) FV_CUDA_TRY(cudaMalloc(&c->sched, sizeof(int) * nc));
  FV_CUDA_TRY(cudaMemcpyAsync(c->sched, order.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  c->n_cell_classes = (int)keys.size();
  return FV_OK;
}

extern "C" int fv_case_create(const FvMesh* mesh, const FvCaseDesc* desc,
                              const signed char* flow_kind, const double* flow_vel,
                              const double* flow_p, const signed char* k_kind, const double* k_val,
                              const signed char* omega_kind, const double* omega_val,
                              const unsigned char* sst_wall, void* stream, FvCase** out) {
  if (!mesh || !desc || !out || !flow_kind) {
    fv_set_error("fv_case_create: bad arguments");
    return FV_ERR_ARG;
  }
  if (!(desc->rho > 0.0) || !(desc->mu > 0.0)) {
    fv_set_error("fv_case_create: viscosity and density must be positive");
    return FV_ERR_ARG;
  }
  if (desc->pressure_pin >= mesh->nc || desc->pressure_pin < -1) {
    fv_set_error("fv_case_create: pressure pin %d out of range", desc->pressure_pin);
    return FV_ERR_ARG;
  }
  if (desc->gradient_sweeps < 0 ||
      (desc->gradient_sweeps >= 1 &&
       !(desc->gradient_relaxation > 0.0 && desc->gradient_relaxation <= 1.0))) {
    fv_set_error("fv_case_create: gradient sweeps must be >= 0 and the relaxation in (0, 1]");
    return FV_ERR_ARG;
  }
  if (desc->advection < 0 || desc->advection > 2 ||
      (desc->advection == 2 && !(desc->limiter_k > 0.0))) {
    fv_set_error("fv_case_create: advection must be 0 (upwind), 1 (linear upwind) or 2 "
                 "(Venkatakrishnan-limited, limiter_k > 0)");
    return FV_ERR_ARG;
  }
  if (desc->scalar_advection < 0 || desc->scalar_advection > 3 ||
      (desc->scalar_advection != 0 && !desc->turbulent) ||
      (desc->scalar_advection == 3 && !(desc->scalar_limiter_k > 0.0))) {
    fv_set_error("fv_case_create: scalar_advection must be 0 (the momentum scheme), 1 (upwind), 2 "
                 "(linear upwind) or 3 (Venkatakrishnan-limited, scalar_limiter_k > 0), for "
                 "turbulent cases only");
    return FV_ERR_ARG;
  }
  if (desc->scalar_transform < 0 || desc->scalar_transform > 3 ||
      (desc->scalar_transform != 0 && !desc->turbulent)) {
    fv_set_error("fv_case_create: scalar_transform must be a bit set in [0, 3] (bit 0 log k, "
                 "bit 1 log omega), for turbulent cases only");
    return FV_ERR_ARG;
  }
  if (desc->turbulent && (!k_kind || !omega_kind || !sst_wall)) {
    fv_set_error("fv_case_create: a turbulent case needs k / omega boundary tables and SST walls");
    return FV_ERR_ARG;
  }
  if (fv_residual_init_constants() != FV_OK) return FV_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  FvMesh* m = const_cast<FvMesh*>(mesh);
  FvCase* c = new FvCase();
  c->mesh = m;
  c->desc = *desc;
  c->mu = desc->mu;
  c->inlet_scale = 1.0;
  c->nfld = m->dim + 1 + (desc->turbulent ? 2 : 0);
  int rc = FV_OK;
  rc |= upload_face_table<signed char>(m, flow_kind, 1, (signed char)-1, &c->fkind, s);
  rc |= upload_face_table<double>(m, flow_vel, m->dim, 0.0, &c->fvel, s);
  rc |= upload_face_table<double>(m, flow_p, 1, 0.0, &c->fp, s);
  rc |= upload_face_table<signed char>(m, k_kind, 1, (signed char)-1, &c->kkind, s);
  rc |= upload_face_table<double>(m, k_val, 1, 0.0, &c->kval, s);
  rc |= upload_face_table<signed char>(m, omega_kind, 1, (signed char)-1, &c->wkind, s);
  rc |= upload_face_table<double>(m, omega_val, 1, 0.0, &c->wval, s);
  rc |= upload_face_table<unsigned char>(m, sst_wall, 1, (unsigned char)0, &c->swall, s);
  if (rc != FV_OK) {
    fv_case_destroy(c);
    return FV_ERR_CUDA;
  }
  // SST wall cells: owners of SST wall faces (aquaflux/turbulence/transport.py:226-227)
  std::vector<unsigned char> wcell(m->nc, 0);
  int n_wall = 0;
  if (desc->turbulent) {
    for (int i = 0; i < m->nf; ++i) {
      int r = m->h_face_old[i];
      if (sst_wall[r]) {
        if (m->h_nb[i] >= 0) {
          fv_set_error("fv_case_create: SST wall face %d is an interior face", r);
          fv_case_destroy(c);
          return FV_ERR_ARG;
        }
        wcell[m->h_owner[i]] = 1;
        ++n_wall;
      }
    }
  }
  FV_CUDA_TRY(cudaMalloc(&c->wcell, m->nc));
  FV_CUDA_TRY(cudaMemcpyAsync(c->wcell, wcell.data(), m->nc, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMalloc(&c->wd, sizeof(double) * m->nc));
  FV_CUDA_TRY(cudaMalloc(&c->wdg, sizeof(double) * m->nc * m->dim));
  FV_CUDA_TRY(cudaMemsetAsync(c->wd, 0, sizeof(double) * m->nc, s));
  FV_CUDA_TRY(cudaMemsetAsync(c->wdg, 0, sizeof(double) * m->nc * m->dim, s));
  FV_CUDA_TRY(cudaMalloc(&c->inv_wd, sizeof(double) * 2 * m->nc));
  FV_CUDA_TRY(cudaMemsetAsync(c->inv_wd, 0, sizeof(double) * 2 * m->nc, s));
  if (desc->turbulent) {
    FV_CUDA_TRY(cudaMalloc(&c->wnear, sizeof(int) * m->nc));
    if (n_wall > 0) {
      rc = fv_wall_distance_compute(m, c->swall, n_wall, c->wd, c->wdg, desc->gradient_sweeps,
                                    desc->gradient_relaxation, c->wnear, s);
      if (rc != FV_OK) {
        fv_case_destroy(c);
        return rc;
      }
      k_inv_distance<<<fv_blocks(m->nc, 256), 256, 0, s>>>(m->nc, c->wd, c->inv_wd);
    } else {
      // no SST wall face on this mesh (a partition's local mesh away from the walls): the caller
      // supplies the distance with fv_case_set_wall_distance before any evaluation
      c->wd_missing = true;
    }
  }
  // effective schemes: momentum (0 upwind, 1 linear, 2 limited) and k, omega likewise
  const int sadv = desc->scalar_advection == 0 ? desc->advection : desc->scalar_advection - 1;
  const double sK = desc->scalar_advection == 0 ? desc->limiter_k : desc->scalar_limiter_k;
  const int rec_any = (desc->advection >= 1 || (desc->turbulent && sadv >= 1)) ? 1 : 0;
  c->work_bytes = fv_residual_work_bytes(m->dim, desc->turbulent, m->nc, m->nf,
                                        desc->gradient_sweeps, rec_any);
  FV_CUDA_TRY(cudaMalloc(&c->work, c->work_bytes));
  FV_CUDA_TRY(cudaMalloc(&c->tmp, sizeof(double) * (size_t)c->nfld * m->nc));
  FV_CUDA_TRY(cudaMalloc(&c->tmp2, sizeof(double) * (size_t)c->nfld * m->nc));
  FV_CUDA_TRY(cudaMalloc(&c->adj, fv_adjoint_work_bytes(m->dim, desc->turbulent, m->nc, m->nf,
                                                        desc->gradient_sweeps, rec_any)));
  FV_CUDA_TRY(cudaMalloc(&c->aux, fv_aux_bytes(m->dim, desc->turbulent, m->nf)));
  FV_CUDA_TRY(cudaMalloc(&c->dscalar, sizeof(double) * 4));
  if (desc->scalar_transform) {
    FV_CUDA_TRY(cudaMalloc(&c->phys, sizeof(double) * (size_t)c->nfld * m->nc));
    FV_CUDA_TRY(cudaMalloc(&c->tphys, sizeof(double) * (size_t)c->nfld * m->nc));
  }
  rc = build_cell_order(c, flow_kind, desc->turbulent ? k_kind : nullptr,
                        desc->turbulent ? omega_kind : nullptr, desc->turbulent ? sst_wall : nullptr,
                        s);
  if (rc != FV_OK) {
    fv_case_destroy(c);
    return rc;
  }
  CaseView& v = c->view;
  v.log_w = (desc->scalar_transform & 2) != 0;
  v.rec_mom = desc->advection >= 1;
  v.rec_sca = desc->turbulent && sadv >= 1;
  v.lim_km = desc->advection == 2 ? desc->limiter_k : 0.0;
  v.lim_ks = (desc->turbulent && sadv == 2) ? sK : 0.0;
  v.turb = desc->turbulent;
  v.rho = desc->rho;
  v.pin = desc->pressure_pin;
  v.pin_value = desc->pressure_pin_value;
  v.fkind = c->fkind;
  v.fvel = c->fvel;
  v.fp = c->fp;
  v.kkind = c->kkind;
  v.kval = c->kval;
  v.wkind = c->wkind;
  v.wval = c->wval;
  v.swall = c->swall;
  v.wcell = c->wcell;
  v.wd = c->wd;
  v.wdg = c->wdg;
  v.inv_wd = c->inv_wd;
  v.inv_wd2 = c->inv_wd + m->nc;
  v.mu_cell = nullptr;
  v.sched = c->sched;
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  *out = c;
  return FV_OK;
}

extern "C" int fv_case_destroy(FvCase* c) {
  if (!c) return FV_OK;
  cudaFree(c->fkind);
  cudaFree(c->fvel);
  cudaFree(c->fp);
  cudaFree(c->kkind);
  cudaFree(c->kval);
  cudaFree(c->wkind);
  cudaFree(c->wval);
  cudaFree(c->swall);
  cudaFree(c->wcell);
  cudaFree(c->wd);
  cudaFree(c->wdg);
  cudaFree(c->inv_wd);
  cudaFree(c->work);
  cudaFree(c->tmp);
  cudaFree(c->tmp2);
  cudaFree(c->adj);
  cudaFree(c->aux);
  cudaFree(c->dscalar);
  cudaFree(c->jac_face);
  cudaFree(c->wnear);
  cudaFree(c->sched);
  cudaFree(c->lin_aux);
  cudaFree(c->lin_fl);
  cudaFree(c->lin_ac);
  cudaFree(c->lin_g);
  cudaFree(c->lin_r);
  cudaFree(c->lin_cl);
  cudaFree(c->lin_cc);
  cudaFree(c->lin_src);
  fv_node_adjoint_free(c);
  cudaFree(c->flx);
  cudaFree(c->mu_cell);
  cudaFree(c->red);
  cudaFree(c->phys);
  cudaFree(c->tphys);
  cudaFree(c->f32);
  cudaFree(c->f_state);
  cudaFree(c->f_tangent);
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  delete c;
  return FV_OK;
}

extern "C" int fv_case_set_params(FvCase* c, double mu, double inlet_scale) {
  if (!c || !(mu > 0.0)) {
    fv_set_error("fv_case_set_params: viscosity must be positive");
    return FV_ERR_ARG;
  }
  c->mu = mu;
  c->inlet_scale = inlet_scale;
  c->lin_valid = 0;
  c->fwd_valid = 0;
  return FV_OK;
}

extern "C" int fv_case_set_viscosity_field(FvCase* c, const double* mu_cell, void* stream) {
  if (!c) {
    fv_set_error("fv_case_set_viscosity_field: null case");
    return FV_ERR_ARG;
  }
  c->lin_valid = 0;
  c->fwd_valid = 0;
  if (!mu_cell) {
    c->view.mu_cell = nullptr;
    return FV_OK;
  }
  if (c->desc.turbulent) {
    fv_set_error("fv_case_set_viscosity_field: a per-cell viscosity applies to laminar cases");
    return FV_ERR_ARG;
  }
  if (!c->mu_cell) FV_CUDA_TRY(cudaMalloc(&c->mu_cell, sizeof(double) * c->mesh->nc));
  FV_CUDA_TRY(cudaMemcpyAsync(c->mu_cell, mu_cell, sizeof(double) * c->mesh->nc,
                              cudaMemcpyDefault, (cudaStream_t)stream));
  c->view.mu_cell = c->mu_cell;
  return FV_OK;
}

extern "C" int fv_case_autotune(FvCase* c, const double* state, const double* w, double* out,
                                void* stream, int* best) {
  if (!c || !state || !w || !out) {
    fv_set_error("fv_case_autotune: bad arguments");
    return FV_ERR_ARG;
  }
  if (c->prof_max_runs) {
    fv_set_error("fv_case_autotune: a stage profile (fv_case_profile_begin) is open");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  // every stage at each candidate, timed stage by stage through the profiling marks; each stage
  // keeps its own fastest (the uniform fastest is returned)
  const int cand[4] = {32, 64, 96, 128};
  const int persistent = c->persistent;
  c->persistent = 0;
  float best_total = 1e30f, stage_best[FV_MAX_STAGES];
  int best_tb = c->tb, stage_tb[FV_MAX_STAGES];
  for (int j = 0; j < FV_MAX_STAGES; ++j) {
    stage_best[j] = 1e30f;
    stage_tb[j] = c->tbs[j];
  }
  int rc = FV_OK;
  for (int k = 0; k < 4 && rc == FV_OK; ++k) {
    c->tb = cand[k];
    for (int j = 0; j < FV_MAX_STAGES; ++j) c->tbs[j] = cand[k];
    rc = fv_case_vjp_run(c, state, w, nullptr, out, s);  // warm-up
    if (rc != FV_OK) break;
    rc = fv_case_profile_begin(c, 3);
    for (int r = 0; r < 3 && rc == FV_OK; ++r) rc = fv_case_vjp_run(c, state, w, nullptr, out, s);
    float ms[FV_MAX_STAGES];
    int runs = 0;
    const int rc2 = fv_case_profile_end(c, ms, FV_MAX_STAGES, &runs);
    if (rc == FV_OK) rc = rc2;
    if (rc != FV_OK) break;
    float total = 0.0f;
    for (int j = 0; j < FV_MAX_STAGES; ++j) {
      total += ms[j];
      if (ms[j] < stage_best[j]) {
        stage_best[j] = ms[j];
        stage_tb[j] = cand[k];
      }
    }
    if (total < best_total) {
      best_total = total;
      best_tb = cand[k];
    }
  }
  c->persistent = persistent;
  c->tb = best_tb;
  for (int j = 0; j < FV_MAX_STAGES; ++j) c->tbs[j] = stage_tb[j];
  if (rc != FV_OK) return rc;
  if (best) *best = best_tb;
  return FV_OK;
}

extern "C" int fv_case_block_sizes(const FvCase* c, int* threads, int n) {
  if (!c || !threads || n <= 0) {
    fv_set_error("fv_case_block_sizes: bad arguments");
    return FV_ERR_ARG;
  }
  for (int j = 0; j < n && j < FV_MAX_STAGES; ++j) threads[j] = c->tbs[j];
  return FV_OK;
}

extern "C" int fv_case_set_cell_order(FvCase* c, int coherent, int* n_classes) {
  if (!c) {
    fv_set_error("fv_case_set_cell_order: bad arguments");
    return FV_ERR_ARG;
  }
  c->view.sched = coherent ? c->sched : nullptr;
  if (n_classes) *n_classes = c->n_cell_classes;
  return FV_OK;
}

extern "C" int fv_case_set_persistent(FvCase* c, int enable, int block, int chunk) {
  if (!c || (enable && (block < 32 || block > 128 || block % 32 != 0 || chunk < 1 || chunk > 64))) {
    fv_set_error("fv_case_set_persistent: block must be a multiple of 32 in [32, 128] and chunk "
                 "in [1, 64]");
    return FV_ERR_ARG;
  }
  c->persistent = enable ? 1 : 0;
  if (enable) {
    c->pblock = block;
    c->pchunk = chunk;
  }
  return FV_OK;
}

extern "C" int fv_case_autotune_persistent(FvCase* c, const double* state, const double* w,
                                           double* out, void* stream, int* best_block,
                                           int* best_chunk, float* best_ms) {
  if (!c || !state || !w || !out) {
    fv_set_error("fv_case_autotune_persistent: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  const int blocks[2] = {64, 128};
  const int chunks[4] = {1, 2, 4, 8};
  cudaEvent_t e0, e1;
  FV_CUDA_TRY(cudaEventCreate(&e0));
  FV_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  int bb = 128, bc = 1;
  const int was = c->persistent;
  c->persistent = 1;
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 4; ++k) {
      c->pblock = blocks[i];
      c->pchunk = chunks[k];
      int rc = fv_case_vjp_run(c, state, w, nullptr, out, s);  // warm-up
      if (rc != FV_OK) {
        c->persistent = was;
        return rc;
      }
      cudaEventRecord(e0, s);
      for (int r = 0; r < 3; ++r) {
        rc = fv_case_vjp_run(c, state, w, nullptr, out, s);
        if (rc != FV_OK) {
          c->persistent = was;
          return rc;
        }
      }
      cudaEventRecord(e1, s);
      FV_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        bb = blocks[i];
        bc = chunks[k];
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->pblock = bb;
  c->pchunk = bc;
  c->persistent = was;
  if (best_block) *best_block = bb;
  if (best_chunk) *best_chunk = bc;
  if (best_ms) *best_ms = best / 3.0f;
  return FV_OK;
}

extern "C" int fv_case_set_block_size(FvCase* c, int threads) {
  if (!c || threads < 32 || threads > 128 || threads % 32 != 0) {
    fv_set_error("fv_case_set_block_size: threads must be a multiple of 32 in [32, 128]");
    return FV_ERR_ARG;
  }
  c->tb = threads;
  for (int j = 0; j < FV_MAX_STAGES; ++j) c->tbs[j] = threads;
  return FV_OK;
}

extern "C" int fv_case_refresh_geometry(FvCase* c, void* stream) {
  if (!c) {
    fv_set_error("fv_case_refresh_geometry: null case");
    return FV_ERR_ARG;
  }
  c->lin_valid = 0;
  c->fwd_valid = 0;
  if (!c->desc.turbulent) return FV_OK;
  if (c->wd_external) {
    fv_set_error("fv_case_refresh_geometry: the wall distance was set by the caller "
                 "(fv_case_set_wall_distance); set it again for the moved nodes");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FvMesh* m = c->mesh;
  int rc = fv_wall_distance_refresh(m, c->swall, c->wnear, c->wd, c->wdg, c->desc.gradient_sweeps,
                                    c->desc.gradient_relaxation, s);
  if (rc != FV_OK) return rc;
  k_inv_distance<<<fv_blocks(m->nc, 256), 256, 0, s>>>(m->nc, c->wd, c->inv_wd);
  FV_CUDA_TRY(cudaGetLastError());
  if (c->f32) {  // the fp32 mirrors of the wall distance, its gradient and reciprocals
    const long nc = m->nc, dim = m->dim;
    float* p = c->f32;
    if ((rc = fv_d2f(nc, c->wd, p, s)) != FV_OK) return rc;
    if ((rc = fv_d2f(dim * nc, c->wdg, p + nc, s)) != FV_OK) return rc;
    if ((rc = fv_d2f(2 * nc, c->inv_wd, p + (1 + dim) * nc, s)) != FV_OK) return rc;
  }
  return FV_OK;
}

extern "C" int fv_case_set_wall_distance(FvCase* c, const double* distance, void* stream) {
  if (!c || !distance || !c->desc.turbulent) {
    fv_set_error("fv_case_set_wall_distance: bad arguments (turbulent cases only)");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FvMesh* m = c->mesh;
  c->lin_valid = 0;
  c->fwd_valid = 0;
  FV_CUDA_TRY(cudaMemcpyAsync(c->wd, distance, sizeof(double) * m->nc, cudaMemcpyDeviceToDevice, s));
  int rc = fv_wall_distance_gradient(m, c->swall, c->wd, c->wdg, c->desc.gradient_sweeps,
                                     c->desc.gradient_relaxation, s);
  if (rc != FV_OK) return rc;
  k_inv_distance<<<fv_blocks(m->nc, 256), 256, 0, s>>>(m->nc, c->wd, c->inv_wd);
  FV_CUDA_TRY(cudaGetLastError());
  if (c->f32) {
    const long nc = m->nc, dim = m->dim;
    float* p = c->f32;
    if ((rc = fv_d2f(nc, c->wd, p, s)) != FV_OK) return rc;
    if ((rc = fv_d2f(dim * nc, c->wdg, p + nc, s)) != FV_OK) return rc;
    if ((rc = fv_d2f(2 * nc, c->inv_wd, p + (1 + dim) * nc, s)) != FV_OK) return rc;
  }
  c->wd_external = true;
  c->wd_missing = false;
  return FV_OK;
}

extern "C" int fv_case_wall_distance(const FvCase* c, double* distance, double* gradient,
                                     void* stream) {
  if (!c) {
    fv_set_error("fv_case_wall_distance: null case");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nc = c->mesh->nc, dim = c->mesh->dim;
  if (distance) FV_CUDA_TRY(cudaMemcpyAsync(distance, c->wd, sizeof(double) * nc, cudaMemcpyDeviceToDevice, s));
  if (gradient) k_cell_to_rowmajor<<<fv_blocks(nc, 256), 256, 0, s>>>(nc, dim, c->wdg, gradient);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" long fv_case_n_unknowns(const FvCase* c) {
  return c ? (long)c->nfld * c->mesh->nc : -1;
}

extern "C" int fv_residual(FvCase* c, const double* state, double* residual, void* stream) {
  if (!c || !state || !residual) {
    fv_set_error("fv_residual: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return fv_case_run(c, physical_state(c, state, s), nullptr, FV_TAN_NONE, residual, nullptr, s);
}

extern "C" int fv_eddy_viscosity(FvCase* c, const double* state, double* nut, void* stream) {
  if (!c || !state || !nut || !c->desc.turbulent) {
    fv_set_error("fv_eddy_viscosity: bad arguments (turbulent cases only)");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return fv_case_eddy_viscosity(c, physical_state(c, state, s), nut, s);
}

extern "C" int fv_jvp(FvCase* c, const double* state, const double* v, double* residual,
                      double* jv, void* stream) {
  if (!c || !state || !v || !jv) {
    fv_set_error("fv_jvp: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  return fv_case_run(c, state, physical_tangent(c, v, s), FV_TAN_STATE, residual, jv, s);
}

extern "C" int fv_linearise(FvCase* c, const double* state, double* residual, void* stream) {
  if (!c || !state) {
    fv_set_error("fv_linearise: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return fv_case_linearise(c, physical_state(c, state, s), residual ? residual : c->tmp2, s);
}

extern "C" int fv_jvp_linearised(FvCase* c, const double* state, const double* v,
                                 double* residual, double* jv, void* stream) {
  if (!c || !state || !v || !jv) {
    fv_set_error("fv_jvp_linearised: bad arguments");
    return FV_ERR_ARG;
  }
  if (!c->lin_valid) {
    fv_set_error("fv_jvp_linearised: no linearisation held; call fv_linearise at this state "
                 "(again after any parameter, viscosity-field or geometry change)");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  c->lin_use = 1;
  const int rc = fv_case_run(c, state, physical_tangent(c, v, s), FV_TAN_STATE, nullptr, jv, s);
  c->lin_use = 0;
  if (rc != FV_OK || !residual) return rc;
  FV_CUDA_TRY(cudaMemcpyAsync(residual, c->lin_r, sizeof(double) * c->nfld * c->mesh->nc,
                              cudaMemcpyDeviceToDevice, s));
  return FV_OK;
}

extern "C" int fv_jvp_frozen(FvCase* c, const double* state, const double* v, double* jv,
                             void* stream) {
  if (!c || !state || !v || !jv) {
    fv_set_error("fv_jvp_frozen: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  return fv_case_run(c, state, physical_tangent(c, v, s), FV_TAN_FROZEN, nullptr, jv, s);
}

namespace {
// values[q][a][field] = jv[a * n + i] for every block q = (i, j) of the pattern whose column cell
// j has colour `colour_id` (one coloured probe of column field `field`).
__global__ void k_probe_scatter(int n, int b, const int* ptr, const int* idx, const int* colour,
                                int colour_id, int field, const double* jv, double* values) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long bb = (long)b * b;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    if (colour[idx[q]] != colour_id) continue;
    double* blk = values + (long)q * bb;
    for (int a = 0; a < b; ++a) blk[(long)a * b + field] = jv[(long)a * n + i];
  }
}
// seed[f * n + c] = 1 where colour[c] == colour_id and f == field, else 0
__global__ void k_probe_seed(int n, int b, const int* colour, int colour_id, int field, double* seed) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * b) return;
  int f = (int)(t / n), c = (int)(t % n);
  seed[t] = (f == field && colour[c] == colour_id) ? 1.0 : 0.0;
}
}  // namespace

extern "C" int fv_probe_jacobian(FvCase* c, const double* state, int frozen, const int* colour,
                                 int n_colours, const int* indptr, const int* indices,
                                 double* values, void* stream) {
  if (!c || !state || !colour || n_colours <= 0 || !indptr || !indices || !values) {
    fv_set_error("fv_probe_jacobian: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int n = c->mesh->nc, b = c->nfld;
  const long len = (long)n * b;
  state = physical_state(c, state, s);
  for (int field = 0; field < b; ++field) {
    for (int col = 0; col < n_colours; ++col) {
      k_probe_seed<<<fv_blocks(len, 256), 256, 0, s>>>(n, b, colour, col, field, c->tmp);
      int rc = fv_case_run(c, state, physical_tangent(c, c->tmp, s),
                           frozen ? FV_TAN_FROZEN : FV_TAN_STATE, nullptr, c->tmp2, s);
      if (rc != FV_OK) return rc;
      k_probe_scatter<<<fv_blocks(n, 256), 256, 0, s>>>(n, b, indptr, indices, colour, col, field,
                                                          c->tmp2, values);
    }
  }
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

namespace {
int assemble_jacobian(FvCase* c, const double* state, const int* indptr, const int* indices,
                      void* values, int fp32, void* stream) {
  if (!c || !state || !indptr || !indices || !values) {
    fv_set_error("fv_assemble_jacobian: bad arguments");
    return FV_ERR_ARG;
  }
  if (!c->jac_face) {
    FV_CUDA_TRY(cudaMalloc(&c->jac_face,
                           fv_jac_face_bytes(c->mesh->dim, c->desc.turbulent, c->mesh->nf)));
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = fv_case_assemble_frozen(c, physical_state(c, state, s), indptr, indices, values,
                                   c->jac_face, fp32, s);
  if (rc == FV_OK && c->desc.scalar_transform) {
    if (fp32)
      k_chain_bsr<float><<<fv_blocks((long)c->nfld * c->mesh->nc, 128), 128, 0, s>>>(
          c->mesh->nc, c->nfld, c->mesh->dim + 1, c->desc.scalar_transform, indptr, indices,
          c->phys, (float*)values);
    else
      k_chain_bsr<double><<<fv_blocks((long)c->nfld * c->mesh->nc, 128), 128, 0, s>>>(
          c->mesh->nc, c->nfld, c->mesh->dim + 1, c->desc.scalar_transform, indptr, indices,
          c->phys, (double*)values);
    FV_CUDA_TRY(cudaGetLastError());
  }
  return rc;
}
}  // namespace

extern "C" int fv_assemble_jacobian(FvCase* c, const double* state, const int* indptr,
                                    const int* indices, double* values, void* stream) {
  return assemble_jacobian(c, state, indptr, indices, values, 0, stream);
}

extern "C" int fv_assemble_jacobian_f32(FvCase* c, const double* state, const int* indptr,
                                        const int* indices, float* values, void* stream) {
  return assemble_jacobian(c, state, indptr, indices, values, 1, stream);
}

extern "C" int fv_jvp_f32(FvCase* c, const double* state, const double* v, double* jv,
                          void* stream) {
  if (!c || !state || !v || !jv) {
    fv_set_error("fv_jvp_f32: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  return fv_case_run(c, state, physical_tangent(c, v, s), FV_TAN_STATE32, nullptr, jv, s);
}

extern "C" int fv_jvp_batch(FvCase* c, const double* state, const double* v, int k, double* jv,
                            void* stream) {
  if (!c || !state || !v || !jv || k < 0) {
    fv_set_error("fv_jvp_batch: bad arguments");
    return FV_ERR_ARG;
  }
  const long n = fv_case_n_unknowns(c);
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  for (int i = 0; i < k; ++i) {
    int rc = fv_case_run(c, state, physical_tangent(c, v + (long)i * n, s), FV_TAN_STATE, nullptr,
                         jv + (long)i * n, s);
    if (rc != FV_OK) return rc;
  }
  return FV_OK;
}

extern "C" int fv_jvp_shift(FvCase* c, const double* state, const double* v, const double* shift,
                            double* jv, void* stream) {
  if (!c || !state || !v || !shift || !jv) {
    fv_set_error("fv_jvp_shift: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  int rc = fv_case_run(c, state, physical_tangent(c, v, s), FV_TAN_STATE, nullptr, jv, s);
  if (rc != FV_OK) return rc;
  long n = fv_case_n_unknowns(c);
  k_axpy_shift<<<fv_blocks(n, 256), 256, 0, s>>>(n, shift, v, jv);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_param_jvp(FvCase* c, const double* state, double* out_mu, double* out_inlet,
                            void* stream) {
  if (!c || !state) {
    fv_set_error("fv_param_jvp: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  state = physical_state(c, state, s);
  if (out_mu) {
    int rc = fv_case_run(c, state, nullptr, FV_TAN_MU, nullptr, out_mu, s);
    if (rc != FV_OK) return rc;
  }
  if (out_inlet) {
    int rc = fv_case_run(c, state, nullptr, FV_TAN_INLET, nullptr, out_inlet, s);
    if (rc != FV_OK) return rc;
  }
  return FV_OK;
}

extern "C" int fv_vjp(FvCase* c, const double* state, const double* w, double* residual,
                      double* vjp, void* stream) {
  if (!c || !state || !w || !vjp) {
    fv_set_error("fv_vjp: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = fv_case_vjp_run(c, physical_state(c, state, s), w, residual, vjp, s);
  if (rc == FV_OK) chain_state(c, vjp, s);
  return rc;
}

extern "C" int fv_hold_forward(FvCase* c, const double* state, double* residual, void* stream) {
  if (!c || !state) {
    fv_set_error("fv_hold_forward: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return fv_case_hold_forward(c, physical_state(c, state, s), residual, s);
}

extern "C" int fv_vjp_held(FvCase* c, const double* state, const double* w, double* vjp,
                           void* stream) {
  if (!c || !state || !w || !vjp) {
    fv_set_error("fv_vjp_held: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = fv_case_vjp_held(c, physical_state(c, state, s), w, vjp, s);
  if (rc == FV_OK) chain_state(c, vjp, s);
  return rc;
}

extern "C" int fv_node_vjp(FvCase* c, const double* state, const double* w, double* dnodes,
                           void* stream) {
  if (!c || !state || !w || !dnodes) {
    fv_set_error("fv_node_vjp: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return fv_case_node_vjp(c, physical_state(c, state, s), w, dnodes, s);
}

extern "C" int fv_face_functional(FvCase* c, const double* state, const double* weights,
                                  int viscous_only, double* value, double* dstate,
                                  double* dparams, double* dnodes, void* stream) {
  if (!c || !state || !weights || !value || !dstate) {
    fv_set_error("fv_face_functional: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = fv_case_face_functional(c, physical_state(c, state, s), weights, viscous_only, value,
                                   dstate, dparams, dnodes, s);
  if (rc == FV_OK) chain_state(c, dstate, s);
  return rc;
}

extern "C" int fv_param_vjp(FvCase* c, const double* state, const double* w, double* out,
                            void* stream) {
  if (!c || !state || !w || !out) {
    fv_set_error("fv_param_vjp: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  long n = fv_case_n_unknowns(c);
  state = physical_state(c, state, s);
  int rc = fv_case_run(c, state, nullptr, FV_TAN_MU, nullptr, c->tmp2, s);
  if (rc == FV_OK) rc = fv_dot_f64(n, w, c->tmp2, out, stream);
  if (rc == FV_OK) rc = fv_case_run(c, state, nullptr, FV_TAN_INLET, nullptr, c->tmp2, s);
  if (rc == FV_OK) rc = fv_dot_f64(n, w, c->tmp2, out + 1, stream);
  return rc;
}

// ------------------------------------------------------------------------------ profiling
void fv_prof_mark(FvCase* c, int k, cudaStream_t s) {
  if (c->prof_max_runs == 0 || c->prof_runs >= c->prof_max_runs) return;
  if (k + 1 > c->prof_stages) c->prof_stages = k + 1;
  if (k + 1 > c->prof_run_marks[c->prof_runs]) c->prof_run_marks[c->prof_runs] = k + 1;
  cudaEventRecord(c->prof_events[(size_t)c->prof_runs * (FV_MAX_STAGES + 1) + k], s);
}
void fv_prof_end_run(FvCase* c) {
  if (c->prof_max_runs == 0 || c->prof_runs >= c->prof_max_runs) return;
  c->prof_runs++;
}

extern "C" int fv_case_profile_begin(FvCase* c, int max_runs) {
  if (!c || max_runs <= 0 || max_runs > 4096) {
    fv_set_error("fv_case_profile_begin: bad arguments");
    return FV_ERR_ARG;
  }
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  c->prof_events.assign((size_t)max_runs * (FV_MAX_STAGES + 1), nullptr);
  for (auto& e : c->prof_events) FV_CUDA_TRY(cudaEventCreate(&e));
  c->prof_max_runs = max_runs;
  c->prof_runs = 0;
  c->prof_stages = 0;
  c->prof_run_marks.assign(max_runs, 0);
  return FV_OK;
}

extern "C" int fv_case_profile_end(FvCase* c, float* stage_ms, int n_stages, int* n_runs) {
  if (!c || !stage_ms || n_stages <= 0) {
    fv_set_error("fv_case_profile_end: bad arguments");
    return FV_ERR_ARG;
  }
  for (int k = 0; k < n_stages; ++k) stage_ms[k] = 0.0f;
  for (int r = 0; r < c->prof_runs; ++r) {
    cudaEvent_t* ev = &c->prof_events[(size_t)r * (FV_MAX_STAGES + 1)];
    const int marks = c->prof_run_marks[r];
    if (marks < 2) continue;
    FV_CUDA_TRY(cudaEventSynchronize(ev[marks - 1]));
    for (int k = 0; k + 1 < marks && k < n_stages; ++k) {
      float ms = 0.0f;
      FV_CUDA_TRY(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
      stage_ms[k] += ms;
    }
  }
  if (n_runs) *n_runs = c->prof_runs;
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  c->prof_events.clear();
  c->prof_max_runs = c->prof_runs = c->prof_stages = 0;
  return FV_OK;
}
