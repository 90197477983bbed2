// Mesh upload, internal face renumbering, cell->face incidence and the GPU geometry pipeline.
//
// Geometry follows aquaflux/mesh/mesh.py:366-387 (_fused_geometry): unoriented face geometry
// (2D edge: aquaflux/mesh/face.py:217-230; 3D centre fan: face.py:292-349), approximate cell
// centroids as the mean of the face centroids (aquaflux/mesh/cell.py:84-108), the owner-outward
// flip (face.py:196-211) and the recentred divergence-theorem volume / centroid
// (cell.py:124-170).  Face-to-cell sums run per cell over its faces in ascending face order, so
// they are deterministic without atomics.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "geom.cuh"
#include "internal.cuh"

namespace {

constexpr int kThreads = 256;

template <int DIM>
__global__ void k_face_geometry(MeshView m, double* area, double* normal, double* xf) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nf = m.nf;
  const int b = m.fn_ptr[f], e = m.fn_ptr[f + 1];
  auto P = [&](int i, int j) -> double { return m.nodes[(long)DIM * m.fn_idx[b + i] + j]; };
  double a, n[DIM], x[DIM];
  face_geom<double, DIM>(e - b, P, a, n, x);
  area[f] = a;
  for (int j = 0; j < DIM; ++j) {
    normal[j * nf + f] = n[j];
    xf[j * nf + f] = x[j];
  }
}

template <int DIM>
__global__ void k_approx_centroid(MeshView m, const double* xf, double* approx) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  double s[DIM];
  for (int j = 0; j < DIM; ++j) s[j] = 0.0;
  int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
    for (int j = 0; j < DIM; ++j) s[j] += xf[j * m.nf + f];
  }
  double inv = 1.0 / (double)(e - b);
  for (int j = 0; j < DIM; ++j) approx[j * m.nc + c] = s[j] * inv;
}

template <int DIM>
__global__ void k_orient(MeshView m, const double* xf, const double* approx, double* normal) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  int o = m.owner[f];
  double proj = 0.0;
  for (int j = 0; j < DIM; ++j)
    proj += (xf[j * m.nf + f] - approx[j * m.nc + o]) * normal[j * m.nf + f];
  if (proj < 0.0)
    for (int j = 0; j < DIM; ++j) normal[j * m.nf + f] = -normal[j * m.nf + f];
}

template <int DIM>
__global__ void k_cell_geometry(MeshView m, const double* area, const double* normal,
                                const double* xf, double* vol, double* xc, double* inv_vol) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  auto F = [&](int i, double& A, double* n, double* x, bool& isnb) {
    const unsigned ent = m.cf_face[b + i];
    const int f = (int)(ent & ~FV_NB_BIT);
    A = area[f];
    for (int j = 0; j < DIM; ++j) {
      n[j] = normal[j * m.nf + f];
      x[j] = xf[j * m.nf + f];
    }
    isnb = (ent & FV_NB_BIT) != 0;
  };
  double volume, x[DIM];
  cell_geom<double, DIM>(e - b, F, volume, x);
  vol[c] = volume;
  inv_vol[c] = 1.0 / volume;
  for (int j = 0; j < DIM; ++j) xc[j * m.nc + c] = x[j];
}

template <int DIM>
__global__ void k_face_factors(MeshView m, double* g, double* nd, double* dpn, double* dnn,
                               double* dvec, double* skew, double* tP, double* tN, double* nn2,
                               double* inv_nd, double* inv_dpn, double* ns) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nf = m.nf, nc = m.nc;
  const int o = m.owner[f];
  const bool interior = f < m.nfi;
  const int n = interior ? m.nb[f] : o;
  double n_[DIM], x[DIM], xo[DIM], xn[DIM];
  for (int j = 0; j < DIM; ++j) {
    n_[j] = m.normal[j * nf + f];
    x[j] = m.xf[j * nf + f];
    xo[j] = m.xc[j * nc + o];
    xn[j] = m.xc[j * nc + n];
  }
  FaceFactors<double, DIM> F;
  face_factors<double, DIM>(n_, x, xo, xn, interior, F);
  g[f] = F.g;
  nd[f] = F.nd;
  dpn[f] = F.dpn;
  dnn[f] = F.dnn;
  nn2[f] = F.nn2;
  inv_nd[f] = F.inv_nd;
  inv_dpn[f] = F.inv_dpn;
  for (int j = 0; j < DIM; ++j) {
    dvec[j * nf + f] = F.dvec[j];
    skew[j * nf + f] = F.skew[j];
    tP[j * nf + f] = F.tP[j];
    tN[j * nf + f] = F.tN[j];
  }
  for (int j = 0; j < DIM * DIM; ++j) ns[(long)j * nf + f] = F.ns[j];
}

// Scatter an internal-order face array (dim, nf) SoA to reference order (nf, dim) row-major.
__global__ void k_face_out(int nf, int dim, const int* face_old, const double* in, double* out) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  int r = face_old[f];
  for (int j = 0; j < dim; ++j) out[(long)r * dim + j] = in[(long)j * nf + f];
}

__global__ void k_cell_out(int nc, int dim, const double* in, double* out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int j = 0; j < dim; ++j) out[(long)c * dim + j] = in[(long)j * nc + c];
}

// Nearest SST-wall face centroid per cell (aquaflux/mesh/distance.py:52-84: exact nearest
// neighbour), by a brute-force search over the wall-face centroids staged through shared memory.
template <int DIM>
__global__ void k_wall_distance(MeshView m, const double* wall_xf, int n_wall, double* wd,
                                const int* slot_face, int* nearest) {
  __shared__ double tile[DIM][256];
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  double x[DIM];
  bool live = c < m.nc;
  for (int j = 0; j < DIM; ++j) x[j] = live ? m.xc[j * m.nc + c] : 0.0;
  double best = 1.0 / 0.0;
  int arg = 0;
  for (int base = 0; base < n_wall; base += 256) {
    int cnt = min(256, n_wall - base);
    __syncthreads();
    if (threadIdx.x < cnt)
      for (int j = 0; j < DIM; ++j) tile[j][threadIdx.x] = wall_xf[(long)j * n_wall + base + threadIdx.x];
    __syncthreads();
    for (int t = 0; t < cnt; ++t) {
      double s = 0.0;
      for (int j = 0; j < DIM; ++j) {
        double dd = x[j] - tile[j][t];
        s += dd * dd;
      }
      if (s < best) {
        best = s;
        arg = base + t;
      }
    }
  }
  if (live) {
    wd[c] = sqrt(best);
    if (nearest) nearest[c] = slot_face[arg];
  }
}

// Distance from each cell centroid to the centroid of its kept nearest SST-wall face (the
// geometry has moved; the nearest face found at case creation is held, as the mesh-coordinate
// adjoint differentiates it).
template <int DIM>
__global__ void k_wall_distance_near(MeshView m, const int* nearest, double* wd) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int f = nearest[c];
  double s = 0.0;
  for (int j = 0; j < DIM; ++j) {
    double dd = m.xc[(long)j * m.nc + c] - m.xf[(long)j * m.nf + f];
    s += dd * dd;
  }
  wd[c] = sqrt(s);
}

__global__ void k_gather_wall_xf(int nf, int dim, const unsigned char* swall, const int* slot,
                                 const double* xf, double* wall_xf, int n_wall) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf || !swall[f]) return;
  int s = slot[f];
  for (int j = 0; j < dim; ++j) wall_xf[(long)j * n_wall + s] = xf[(long)j * nf + f];
}

// Compact Green-Gauss gradient of the wall distance with Dirichlet 0 on the SST walls and zero
// gradient (owner value) elsewhere: aquaflux/turbulence/transport.py:86-111.
// With num non-null (corrected scheme) num receives the numerator B d and wdg rel * B d / V.
template <int DIM>
__global__ void k_wall_distance_gradient(MeshView m, const unsigned char* swall, const double* wd,
                                         double* wdg, double* num, double rel) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  double acc[DIM];
  for (int j = 0; j < DIM; ++j) acc[j] = 0.0;
  double phic = wd[c];
  int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    unsigned ent = m.cf_face[i];
    int f = (int)(ent & ~FV_NB_BIT);
    double phif;
    if (f < m.nfi) {
      double g = m.g[f];
      int o = m.owner[f], n = m.nb[f];
      phif = (1.0 - g) * wd[o] + g * wd[n];
    } else {
      phif = swall[f] ? 0.0 : phic;
    }
    double s = (ent & FV_NB_BIT) ? -phif : phif;
    for (int j = 0; j < DIM; ++j) acc[j] += (m.normal[j * m.nf + f] * m.area[f]) * s;
  }
  double inv = 1.0 / m.vol[c];
  if (num || rel != 1.0) {
    const double iv = m.inv_vol[c];
    for (int j = 0; j < DIM; ++j) {
      if (num) num[j * m.nc + c] = acc[j];
      wdg[j * m.nc + c] = rel * (acc[j] * iv);
    }
  } else {
    for (int j = 0; j < DIM; ++j) wdg[j * m.nc + c] = acc[j] * inv;
  }
}

thread_local char g_err[1024] = "";
thread_local long g_err_index = -1;

}  // namespace

void fv_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void fv_set_error_index(long i) { g_err_index = i; }

extern "C" const char* fv_last_error(void) { return g_err; }
extern "C" long fv_last_error_index(void) { return g_err_index; }
extern "C" const char* fv_version(void) { return "fvgb 0.1 (sm_103a)"; }

int fv_mesh_compute_geometry(FvMesh* m, cudaStream_t s) {
  MeshView v = m->view;
  double* area = const_cast<double*>(v.area);
  double* normal = const_cast<double*>(v.normal);
  double* xf = const_cast<double*>(v.xf);
  double* vol = const_cast<double*>(v.vol);
  double* xc = const_cast<double*>(v.xc);
  int bf = fv_blocks(m->nf, kThreads), bc = fv_blocks(m->nc, kThreads);
  if (m->dim == 2) {
    k_face_geometry<2><<<bf, kThreads, 0, s>>>(v, area, normal, xf);
    k_approx_centroid<2><<<bc, kThreads, 0, s>>>(v, xf, m->approx);
    k_orient<2><<<bf, kThreads, 0, s>>>(v, xf, m->approx, normal);
    k_cell_geometry<2><<<bc, kThreads, 0, s>>>(v, area, normal, xf, vol, xc,
                                                 const_cast<double*>(v.inv_vol));
    k_face_factors<2><<<bf, kThreads, 0, s>>>(
        v, const_cast<double*>(v.g), const_cast<double*>(v.nd), const_cast<double*>(v.dpn),
        const_cast<double*>(v.dnn), const_cast<double*>(v.dvec), const_cast<double*>(v.skew),
        const_cast<double*>(v.tP), const_cast<double*>(v.tN), const_cast<double*>(v.nn2),
        const_cast<double*>(v.inv_nd), const_cast<double*>(v.inv_dpn), const_cast<double*>(v.ns));
  } else {
    k_face_geometry<3><<<bf, kThreads, 0, s>>>(v, area, normal, xf);
    k_approx_centroid<3><<<bc, kThreads, 0, s>>>(v, xf, m->approx);
    k_orient<3><<<bf, kThreads, 0, s>>>(v, xf, m->approx, normal);
    k_cell_geometry<3><<<bc, kThreads, 0, s>>>(v, area, normal, xf, vol, xc,
                                                 const_cast<double*>(v.inv_vol));
    k_face_factors<3><<<bf, kThreads, 0, s>>>(
        v, const_cast<double*>(v.g), const_cast<double*>(v.nd), const_cast<double*>(v.dpn),
        const_cast<double*>(v.dnn), const_cast<double*>(v.dvec), const_cast<double*>(v.skew),
        const_cast<double*>(v.tP), const_cast<double*>(v.tN), const_cast<double*>(v.nn2),
        const_cast<double*>(v.inv_nd), const_cast<double*>(v.inv_dpn), const_cast<double*>(v.ns));
  }
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

namespace {
// Green-Gauss gradient of the wall distance (compact, or corrected with `sweeps` sweeps).
int wall_distance_gradient(FvMesh* m, const unsigned char* swall_dev, const double* wd,
                           double* wdg, int sweeps, double rel, cudaStream_t s) {
  int bc = fv_blocks(m->nc, kThreads);
  // corrected scheme: B d, the other sweep iterate and the face scratch
  double *num = nullptr, *galt = nullptr, *wface = nullptr;
  double* x0 = wdg;
  if (sweeps >= 2) {
    FV_CUDA_TRY(cudaMalloc(&num, sizeof(double) * (size_t)m->dim * m->nc));
    FV_CUDA_TRY(cudaMalloc(&galt, sizeof(double) * (size_t)m->dim * m->nc));
    FV_CUDA_TRY(cudaMalloc(&wface, sizeof(double) * (size_t)m->nf));
    if ((sweeps - 1) % 2 != 0) x0 = galt;
  }
  const double r0 = sweeps >= 1 ? rel : 1.0;
  if (m->dim == 2)
    k_wall_distance_gradient<2><<<bc, kThreads, 0, s>>>(m->view, swall_dev, wd, x0, num, r0);
  else
    k_wall_distance_gradient<3><<<bc, kThreads, 0, s>>>(m->view, swall_dev, wd, x0, num, r0);
  int rc = FV_OK;
  if (sweeps >= 2)
    rc = fv_gg_sweeps_scalar(m->view, sweeps, rel, num, x0, x0 == wdg ? galt : wdg, wface, s);
  FV_CUDA_TRY(cudaGetLastError());
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  cudaFree(num);
  cudaFree(galt);
  cudaFree(wface);
  return rc;
}
}  // namespace

int fv_wall_distance_compute(FvMesh* m, const unsigned char* swall_dev, int n_wall, double* wd,
                             double* wdg, int sweeps, double rel, int* nearest, cudaStream_t s) {
  if (n_wall <= 0) {
    fv_set_error("a turbulent case needs at least one SST wall face");
    return FV_ERR_ARG;
  }
  // slot of each wall face in the compacted centroid list (internal face order)
  std::vector<unsigned char> h_sw(m->nf);
  FV_CUDA_TRY(cudaMemcpyAsync(h_sw.data(), swall_dev, m->nf, cudaMemcpyDeviceToHost, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<int> slot(m->nf, -1), slot_face;
  int k = 0;
  for (int f = 0; f < m->nf; ++f)
    if (h_sw[f]) {
      slot[f] = k++;
      slot_face.push_back(f);
    }
  int* d_slot = nullptr;
  int* d_slot_face = nullptr;
  double* d_wxf = nullptr;
  FV_CUDA_TRY(cudaMalloc(&d_slot, sizeof(int) * m->nf));
  FV_CUDA_TRY(cudaMalloc(&d_slot_face, sizeof(int) * std::max(k, 1)));
  FV_CUDA_TRY(cudaMalloc(&d_wxf, sizeof(double) * (size_t)k * m->dim));
  FV_CUDA_TRY(cudaMemcpyAsync(d_slot, slot.data(), sizeof(int) * m->nf, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(d_slot_face, slot_face.data(), sizeof(int) * k,
                              cudaMemcpyHostToDevice, s));
  int bf = fv_blocks(m->nf, kThreads), bc = fv_blocks(m->nc, kThreads);
  k_gather_wall_xf<<<bf, kThreads, 0, s>>>(m->nf, m->dim, swall_dev, d_slot, m->view.xf, d_wxf, k);
  if (m->dim == 2)
    k_wall_distance<2><<<bc, 256, 0, s>>>(m->view, d_wxf, k, wd, d_slot_face, nearest);
  else
    k_wall_distance<3><<<bc, 256, 0, s>>>(m->view, d_wxf, k, wd, d_slot_face, nearest);
  int rc = wall_distance_gradient(m, swall_dev, wd, wdg, sweeps, rel, s);
  cudaFree(d_slot);
  cudaFree(d_slot_face);
  cudaFree(d_wxf);
  return rc;
}

int fv_wall_distance_gradient(FvMesh* m, const unsigned char* swall_dev, const double* wd,
                              double* wdg, int sweeps, double rel, cudaStream_t s) {
  return wall_distance_gradient(m, swall_dev, wd, wdg, sweeps, rel, s);
}

int fv_wall_distance_refresh(FvMesh* m, const unsigned char* swall_dev, const int* nearest,
                             double* wd, double* wdg, int sweeps, double rel, cudaStream_t s) {
  int bc = fv_blocks(m->nc, kThreads);
  if (m->dim == 2)
    k_wall_distance_near<2><<<bc, kThreads, 0, s>>>(m->view, nearest, wd);
  else
    k_wall_distance_near<3><<<bc, kThreads, 0, s>>>(m->view, nearest, wd);
  FV_CUDA_TRY(cudaGetLastError());
  return wall_distance_gradient(m, swall_dev, wd, wdg, sweeps, rel, s);
}

extern "C" int fv_mesh_create(int dim, int n_cells, int n_faces, int n_nodes, const double* nodes,
                              const int* fn_offsets, const int* fn_indices, const int* owner,
                              const int* neighbour, void* stream, FvMesh** out) {
  if (!out || (dim != 2 && dim != 3) || n_cells <= 0 || n_faces <= 0 || n_nodes <= 0 || !nodes ||
      !fn_offsets || !fn_indices || !owner || !neighbour) {
    fv_set_error("fv_mesh_create: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FvMesh* m = new FvMesh();
  m->dim = dim;
  m->nc = n_cells;
  m->nf = n_faces;
  m->nn = n_nodes;
  // validate the topology the kernels rely on (aquaflux/mesh/mesh.py:208-319)
  for (int f = 0; f < n_faces; ++f) {
    int cnt = fn_offsets[f + 1] - fn_offsets[f];
    if (owner[f] < 0 || owner[f] >= n_cells || neighbour[f] < -1 || neighbour[f] >= n_cells ||
        neighbour[f] == owner[f] || (dim == 2 && cnt != 2) || (dim == 3 && cnt < 3)) {
      fv_set_error("fv_mesh_create: invalid face %d", f);
      delete m;
      return FV_ERR_ARG;
    }
  }
  if (fn_offsets[0] != 0) {
    fv_set_error("fv_mesh_create: fn_offsets[0] must be 0");
    delete m;
    return FV_ERR_ARG;
  }
  // internal face order: interior by (owner, neighbour), then boundary by owner
  std::vector<int> order(n_faces);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    bool ia = neighbour[a] >= 0, ib = neighbour[b] >= 0;
    if (ia != ib) return ia;
    if (owner[a] != owner[b]) return owner[a] < owner[b];
    if (ia) return neighbour[a] < neighbour[b];
    return false;
  });
  m->h_face_old = order;
  m->h_face_new.assign(n_faces, 0);
  for (int i = 0; i < n_faces; ++i) m->h_face_new[order[i]] = i;
  m->nfi = 0;
  for (int f = 0; f < n_faces; ++f) m->nfi += neighbour[f] >= 0;
  m->h_owner.resize(n_faces);
  m->h_nb.resize(n_faces);
  std::vector<int> fptr(n_faces + 1, 0), fidx;
  fidx.reserve(fn_offsets[n_faces]);
  for (int i = 0; i < n_faces; ++i) {
    int r = order[i];
    m->h_owner[i] = owner[r];
    m->h_nb[i] = neighbour[r];
    for (int q = fn_offsets[r]; q < fn_offsets[r + 1]; ++q) {
      int nidx = fn_indices[q];
      if (nidx < 0 || nidx >= n_nodes) {
        fv_set_error("fv_mesh_create: node index out of range at face %d", r);
        delete m;
        return FV_ERR_ARG;
      }
      fidx.push_back(nidx);
    }
    fptr[i + 1] = (int)fidx.size();
  }
  // cell -> face incidence, ascending internal face index
  std::vector<int> cnt(n_cells + 1, 0);
  for (int f = 0; f < n_faces; ++f) {
    cnt[m->h_owner[f] + 1]++;
    if (m->h_nb[f] >= 0) cnt[m->h_nb[f] + 1]++;
  }
  for (int c = 0; c < n_cells; ++c) {
    if (cnt[c + 1] == 0) {
      fv_set_error("fv_mesh_create: cell %d is not referenced by any face", c);
      delete m;
      return FV_ERR_ARG;
    }
    cnt[c + 1] += cnt[c];
  }
  m->h_cf_ptr = cnt;
  m->h_cf_face.assign(cnt[n_cells], 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int f = 0; f < n_faces; ++f) {  // ascending f -> each list is sorted
    m->h_cf_face[fill[m->h_owner[f]]++] = (unsigned)f;
    if (m->h_nb[f] >= 0) m->h_cf_face[fill[m->h_nb[f]]++] = (unsigned)f | FV_NB_BIT;
  }
  // device upload
  size_t nf = n_faces, nc = n_cells;
  FV_CUDA_TRY(cudaMalloc(&m->owner, sizeof(int) * nf));
  FV_CUDA_TRY(cudaMalloc(&m->nb, sizeof(int) * nf));
  FV_CUDA_TRY(cudaMalloc(&m->cf_ptr, sizeof(int) * (nc + 1)));
  FV_CUDA_TRY(cudaMalloc(&m->cf_face, sizeof(unsigned) * m->h_cf_face.size()));
  FV_CUDA_TRY(cudaMalloc(&m->fn_ptr, sizeof(int) * (nf + 1)));
  FV_CUDA_TRY(cudaMalloc(&m->fn_idx, sizeof(int) * fidx.size()));
  FV_CUDA_TRY(cudaMalloc(&m->face_old, sizeof(int) * nf));
  FV_CUDA_TRY(cudaMalloc(&m->nodes, sizeof(double) * (size_t)n_nodes * dim));
  FV_CUDA_TRY(cudaMalloc(&m->approx, sizeof(double) * nc * dim));
  // geometry block: area, dpn, dnn, g, nd, nn2 (6 nf) + normal, xf, dvec, skew, tP, tN (6 dim nf)
  // + vol (nc) + xc (dim nc)
  size_t geo_n = 8 * nf + 6 * (size_t)dim * nf + (size_t)dim * dim * nf + 2 * nc +
                 (size_t)dim * nc;
  m->geo_n = geo_n;
  FV_CUDA_TRY(cudaMalloc(&m->geo, sizeof(double) * geo_n));
  FV_CUDA_TRY(cudaMemcpyAsync(m->owner, m->h_owner.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->nb, m->h_nb.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->cf_ptr, m->h_cf_ptr.data(), sizeof(int) * (nc + 1), cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->cf_face, m->h_cf_face.data(), sizeof(unsigned) * m->h_cf_face.size(), cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->fn_ptr, fptr.data(), sizeof(int) * (nf + 1), cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->fn_idx, fidx.data(), sizeof(int) * fidx.size(), cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->face_old, order.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(m->nodes, nodes, sizeof(double) * (size_t)n_nodes * dim, cudaMemcpyHostToDevice, s));
  double* p = m->geo;
  MeshView& v = m->view;
  v.dim = dim;
  v.nc = n_cells;
  v.nf = n_faces;
  v.nfi = m->nfi;
  v.nn = n_nodes;
  v.owner = m->owner;
  v.nb = m->nb;
  v.cf_ptr = m->cf_ptr;
  v.cf_face = m->cf_face;
  v.fn_ptr = m->fn_ptr;
  v.fn_idx = m->fn_idx;
  v.nodes = m->nodes;
  v.area = p; p += nf;
  v.dpn = p; p += nf;
  v.dnn = p; p += nf;
  v.g = p; p += nf;
  v.nd = p; p += nf;
  v.nn2 = p; p += nf;
  v.inv_nd = p; p += nf;
  v.inv_dpn = p; p += nf;
  v.ns = p; p += dim * dim * nf;
  v.normal = p; p += dim * nf;
  v.xf = p; p += dim * nf;
  v.dvec = p; p += dim * nf;
  v.skew = p; p += dim * nf;
  v.tP = p; p += dim * nf;
  v.tN = p; p += dim * nf;
  v.vol = p; p += nc;
  v.inv_vol = p; p += nc;
  v.xc = p; p += dim * nc;
  int rc = fv_mesh_compute_geometry(m, s);
  if (rc != FV_OK) {
    fv_mesh_destroy(m);
    return rc;
  }
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  *out = m;
  return FV_OK;
}

extern "C" int fv_mesh_destroy(FvMesh* m) {
  if (!m) return FV_OK;
  cudaFree(m->owner);
  cudaFree(m->nb);
  cudaFree(m->cf_ptr);
  cudaFree(m->cf_face);
  cudaFree(m->fn_ptr);
  cudaFree(m->fn_idx);
  cudaFree(m->face_old);
  cudaFree(m->nodes);
  cudaFree(m->geo);
  cudaFree(m->geo_f);
  cudaFree(m->approx);
  delete m;
  return FV_OK;
}

__global__ void k_to_f32(long n, const double* in, float* out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

int fv_d2f(long n, const double* in, float* out, cudaStream_t s) {
  if (n <= 0) return FV_OK;
  k_to_f32<<<fv_blocks(n, kThreads), kThreads, 0, s>>>(n, in, out);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

// The fp32 mirror of the geometry block (same layout), made on first use and refreshed whenever
// the geometry is recomputed.
int fv_mesh_ensure_f32(FvMesh* m, cudaStream_t s) {
  if (m->geo_f) return FV_OK;
  FV_CUDA_TRY(cudaMalloc(&m->geo_f, sizeof(float) * m->geo_n));
  MeshView& v = m->view;
  auto mirror = [&](const double* p) { return (const float*)(m->geo_f + (p - m->geo)); };
  v.f_area = mirror(v.area);
  v.f_normal = mirror(v.normal);
  v.f_xf = mirror(v.xf);
  v.f_vol = mirror(v.vol);
  v.f_xc = mirror(v.xc);
  v.f_g = mirror(v.g);
  v.f_nd = mirror(v.nd);
  v.f_dpn = mirror(v.dpn);
  v.f_dnn = mirror(v.dnn);
  v.f_dvec = mirror(v.dvec);
  v.f_skew = mirror(v.skew);
  v.f_tP = mirror(v.tP);
  v.f_tN = mirror(v.tN);
  v.f_nn2 = mirror(v.nn2);
  v.f_inv_nd = mirror(v.inv_nd);
  v.f_inv_dpn = mirror(v.inv_dpn);
  v.f_ns = mirror(v.ns);
  v.f_inv_vol = mirror(v.inv_vol);
  return fv_d2f((long)m->geo_n, m->geo, m->geo_f, s);
}

extern "C" int fv_mesh_set_nodes(FvMesh* m, const double* nodes_device, void* stream) {
  if (!m || !nodes_device) {
    fv_set_error("fv_mesh_set_nodes: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FV_CUDA_TRY(cudaMemcpyAsync(m->nodes, nodes_device, sizeof(double) * (size_t)m->nn * m->dim,
                              cudaMemcpyDeviceToDevice, s));
  int rc = fv_mesh_compute_geometry(m, s);
  if (rc == FV_OK && m->geo_f) rc = fv_d2f((long)m->geo_n, m->geo, m->geo_f, s);
  return rc;
}

extern "C" int fv_mesh_geometry(const FvMesh* m, double* area, double* normal,
                                double* face_centroid, double* volume, double* cell_centroid,
                                void* stream) {
  if (!m) {
    fv_set_error("fv_mesh_geometry: null mesh");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int bf = fv_blocks(m->nf, kThreads), bc = fv_blocks(m->nc, kThreads);
  if (area) k_face_out<<<bf, kThreads, 0, s>>>(m->nf, 1, m->face_old, m->view.area, area);
  if (normal) k_face_out<<<bf, kThreads, 0, s>>>(m->nf, m->dim, m->face_old, m->view.normal, normal);
  if (face_centroid)
    k_face_out<<<bf, kThreads, 0, s>>>(m->nf, m->dim, m->face_old, m->view.xf, face_centroid);
  if (volume) FV_CUDA_TRY(cudaMemcpyAsync(volume, m->view.vol, sizeof(double) * m->nc, cudaMemcpyDeviceToDevice, s));
  if (cell_centroid) k_cell_out<<<bc, kThreads, 0, s>>>(m->nc, m->dim, m->view.xc, cell_centroid);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_mesh_sizes(const FvMesh* m, int* dim, int* n_cells, int* n_faces, int* n_nodes) {
  if (!m) {
    fv_set_error("fv_mesh_sizes: null mesh");
    return FV_ERR_ARG;
  }
  if (dim) *dim = m->dim;
  if (n_cells) *n_cells = m->nc;
  if (n_faces) *n_faces = m->nf;
  if (n_nodes) *n_nodes = m->nn;
  return FV_OK;
}
