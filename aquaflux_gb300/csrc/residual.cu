// The finite-volume residual pipeline (laminar Rhie-Chow momentum/continuity, optionally coupled
// to k-omega SST), written once as templates over the scalar type:
//   T = double -> R(state)
//   T = Dual   -> R(state) and J v (forward-mode tangent through the same arithmetic)
//
// Pipeline (each stage one kernel; face stages run one thread per face in the internal face
// order, cell stages one thread per cell summing its faces in ascending order, so every
// face-to-cell accumulation is deterministic without atomics):
//   k_grad      cell  compact Green-Gauss gradients of every field
//               (aquaflux/schemes/gradient.py:129-153 with the leading-order boundary values of
//               aquaflux/flow/momentum.py:445-469 / discretization/residual.py:252-291)
//   k_closure   cell  SST closure: strain with the wall-cell log-layer blend, imposed wall-cell
//               omega gradient, F1, nu_t, wall shear rate (aquaflux/turbulence/transport.py:369-579)
//   k_apcoef    face  momentum-diagonal face coefficients: flux-continuous viscous conductance +
//               upwind part of the lagged mass-flux estimate, boundary closures
//               (aquaflux/flow/momentum.py:556-693, aquaflux/flow/rhie_chow.py:81-271)
//   k_dcoeff    cell  a_P and d = V / a_P
//   k_flux      face  Rhie-Chow mass flux (rhie_chow.py:274-353, flow/boundary.py:381-435), face
//               pressure, momentum diffusion + pressure + upwind advection fluxes, k / omega
//               advection + diffusion fluxes (discretization/diffusion.py:163-199,
//               advection.py:99-187, turbulence/transport.py:581-718)
//   k_sum       cell  conservative face-to-cell sums, pressure pin, SST sources and the omega
//               wall-cell fixation (turbulence/sources.py:60-412, fixed_value.py:124-158)
#include <cooperative_groups.h>
#include <type_traits>

#include "geom.cuh"
#include "internal.cuh"

namespace {

// SST constants, aquaflux/turbulence/sst.py:69-82 and sources.py:52-57.
constexpr double A1 = 0.31, BETA_STAR = 0.09, ALPHA_1 = 5.0 / 9.0, BETA_1 = 3.0 / 40.0;
constexpr double SIGMA_K1 = 0.85, SIGMA_W1 = 0.5, ALPHA_2 = 0.44, BETA_2 = 0.0828;
constexpr double SIGMA_K2 = 1.0, SIGMA_W2 = 0.856, KAPPA = 0.41, E_WALL = 9.8;
constexpr double CROSS_FLOOR = 1e-10, PROD_RATIO = 10.0, NUT_FLOOR = 1e-30;

struct SstConst {
  double bs4;   // beta_star ** 0.25
  double ylam;  // laminar-sublayer y* (fixed point of y = ln(E y) / kappa, 10 sweeps from 11)
};
__constant__ SstConst c_sst;

// fp32 passes (T = DualF) read the fp32 mirrors of the geometry and of the state, so that their
// arithmetic stays off the fp64 pipe; GS<T> is the scalar type of the geometry a pass reads.
template <class T>
struct IsF32 : std::false_type {};
template <>
struct IsF32<DualF> : std::true_type {};
template <class T>
using GS = typename std::conditional<IsF32<T>::value, float, double>::type;
// The cell a thread of a cell-centric stage evaluates.  With the case's warp-coherent order the
// threads walk the cells grouped by the pattern of their face lists (owner / neighbour / boundary
// kind at each position), so the 32 lanes of a warp take the same branches; without it, the
// natural order.  A cell's arithmetic does not depend on which thread runs it, so both orders give
// bitwise the same result.  The fp32 dual-number passes keep the natural order: they are not
// bound by the floating-point issue rate that divergence wastes, and the indirection costs them.
template <class T = double>
__device__ __forceinline__ int stage_cell(const MeshView& m, const CaseView& cv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if constexpr (IsF32<T>::value) return t;
  else return (cv.sched != nullptr && t < m.nc) ? __ldg(cv.sched + t) : t;
}

template <class T>
__device__ __forceinline__ GS<T> gx(const double* d, const float* f, long i) {
  if constexpr (IsF32<T>::value) return f[i];
  else return d[i];
}
template <class T>
__device__ __forceinline__ GS<T> rho_of(const CaseView& cv) {
  if constexpr (IsF32<T>::value) return cv.f_rho;
  else return cv.rho;
}

template <class T>
struct Src;
template <>
struct Src<double> {
  const double* v;
  __device__ __forceinline__ double operator()(long i) const { return v[i]; }
};
template <>
struct Src<Dual> {
  const double* v;
  const double* t;  // may be null: zero tangent
  __device__ __forceinline__ Dual operator()(long i) const { return {v[i], t ? t[i] : 0.0}; }
};
template <>
struct Src<DualF> {
  const float* v;  // the fp32 copy of the state
  const float* t;  // of the tangent; may be null: zero tangent
  __device__ __forceinline__ DualF operator()(long i) const { return {v[i], t ? t[i] : 0.0f}; }
};

template <class T>
struct Par {
  T mu;      // molecular dynamic viscosity
  T iscale;  // inlet-velocity factor
  T nu;      // molecular kinematic viscosity mu / rho
};

template <class T>
__device__ __forceinline__ void put(double* r, double* t, long i, const T& x);
template <>
__device__ __forceinline__ void put<double>(double* r, double*, long i, const double& x) {
  r[i] = x;
}
template <>
__device__ __forceinline__ void put<Dual>(double* r, double* t, long i, const Dual& x) {
  if (r) r[i] = x.v;
  t[i] = x.d;
}
template <>
__device__ __forceinline__ void put<DualF>(double* r, double* t, long i, const DualF& x) {
  if (r) r[i] = x.v;
  t[i] = x.d;
}

// ---------------------------------------------------------------- SST wall functions
// aquaflux/turbulence/boundary.py:45-589.
template <class T, class D>
__device__ __forceinline__ T y_star(T nu, D d, T k) {
  return c_sst.bs4 * safe_sqrt(pos(k)) * d / nu;
}
template <class T, class D>
__device__ __forceinline__ T wall_weight(T nu, D d, T k) {
  T r = y_star(nu, d, k) / c_sst.ylam;
  T r2 = r * r;
  return fv_tanh(r2 * r2);
}
template <class T, class D>
__device__ __forceinline__ T log_shear(D d, T k) {
  return c_sst.bs4 * safe_sqrt(pos(k)) / (KAPPA * d);
}
template <class T, class D>
__device__ __forceinline__ T omega_wall(T nu, D d, T k) {
  T vis = 6.0 * nu / (BETA_1 * (d * d));
  T lg = safe_sqrt(pos(k)) / (c_sst.bs4 * KAPPA * d);
  T m = fv_max(vis, lg);
  T ra = vis / m, rb = lg / m;
  T bt = val(rb) > 0.0 ? rb * rb : cst(0.0, rb);
  return m * fv_sqrt(ra * ra + bt);
}
template <class T, class D>
__device__ __forceinline__ T nut_wall(T nu, D d, T k) {
  T ys = y_star(nu, d, k);
  T arg = E_WALL * fv_max(ys, cst(c_sst.ylam, ys));
  T ratio = ys * KAPPA / fv_log(arg) - 1.0;
  return val(ys) > c_sst.ylam ? nu * ratio : cst(0.0, ys);
}
// d omega_wall / d d and d omega_wall / d k in closed form (the reference obtains them with
// jax.grad, boundary.py:585-589); written in T so the JVP differentiates them once more.
template <class T, class D>
__device__ __forceinline__ void omega_wall_partials(T nu, D d, T k, T* dwdd, T* dwdk) {
  T vis = 6.0 * nu / (BETA_1 * (d * d));
  T kp = pos(k);
  T sk = safe_sqrt(kp);
  double c = c_sst.bs4 * KAPPA;
  T lg = sk / (c * d);
  T w = omega_wall(nu, d, k);
  T dvis_dd = -2.0 * vis / d;
  T dlog_dd = -lg / d;
  T dsk = val(kp) > 0.0 ? 0.5 / sk : cst(0.0, sk);
  T dlog_dk = dsk / (c * d);
  T a = vis / w, b = lg / w;
  *dwdd = a * dvis_dd + b * dlog_dd;
  *dwdk = b * dlog_dk;
}

// ---------------------------------------------------------------- boundary values
// Leading-order flow boundary velocity / pressure (aquaflux/flow/boundary.py:43-120, 278-446).
template <class T>
__device__ __forceinline__ T bvel(const CaseView& cv, int nf, int f, int j, signed char kind,
                                  T u_owner, const Par<T>& par) {
  if (kind == 1) return cst(cv.fvel[(long)j * nf + f], u_owner);
  if (kind == 2) return cv.fvel[(long)j * nf + f] * par.iscale;
  if (kind == 3) return u_owner;
  return cst(0.0, u_owner);
}
template <class T>
__device__ __forceinline__ T bpress(const CaseView& cv, int f, signed char kind, T p_owner) {
  if (kind == 3) return cst(cv.fp[f], p_owner);
  if (kind >= 0) return p_owner;
  return cst(0.0, p_owner);
}
// Scalar closure Dirichlet / ZeroGradient (aquaflux/boundary/conditions.py:111-160); `corr` is
// the tangential correction (zero for the leading-order values used by the gradient).
template <class T>
__device__ __forceinline__ T bscalar(signed char kind, double value, T phi_owner, T corr) {
  if (kind == 0) return cst(value, phi_owner);
  if (kind == 1) return phi_owner + corr;
  return cst(0.0, phi_owner);
}

// ---------------------------------------------------------------- geometry accessors
// The face and cell formulas read the mesh geometry through an accessor: GeoPlain returns the
// stored doubles; GeoSeed returns dual numbers whose tangent is 1 on one geometric input (one
// component, on every face / cell or on one of them), which lets the mesh-coordinate adjoint
// differentiate the same formulas with respect to the geometry by local forward mode.
enum GeoFace {
  GF_AREA = 0, GF_NORMAL = 1, GF_TP = 4, GF_TN = 7, GF_G = 10, GF_DVEC = 11, GF_SKEW = 14,
  GF_NN2 = 17, GF_INV_ND = 18, GF_INV_DPN = 19, GF_DPN = 20, GF_DNN = 21, GF_NS = 22,
  GF_COUNT = 31
};
enum GeoCell { GC_VOL = 0, GC_WD = 1, GC_INV_WD = 2, GC_INV_WD2 = 3, GC_WDG = 4, GC_COUNT = 7 };
// Centroid seeds (not stored per-factor cotangent rows): face centroid component j of the seeded
// face (fcomp = GF_XF + j), cell centroid component j of the seeded cell (ccomp = GC_XC + j).
enum GeoCentroid { GF_XF = 40, GC_XC = 50 };

struct GeoPlain {
  __device__ __forceinline__ double area(const MeshView& m, int f) const { return m.area[f]; }
  __device__ __forceinline__ double normal(const MeshView& m, int j, int f) const {
    return m.normal[(long)j * m.nf + f];
  }
  __device__ __forceinline__ double tP(const MeshView& m, int j, int f) const {
    return m.tP[(long)j * m.nf + f];
  }
  __device__ __forceinline__ double tN(const MeshView& m, int j, int f) const {
    return m.tN[(long)j * m.nf + f];
  }
  __device__ __forceinline__ double g(const MeshView& m, int f) const { return m.g[f]; }
  __device__ __forceinline__ double dvec(const MeshView& m, int j, int f) const {
    return m.dvec[(long)j * m.nf + f];
  }
  __device__ __forceinline__ double skew(const MeshView& m, int j, int f) const {
    return m.skew[(long)j * m.nf + f];
  }
  __device__ __forceinline__ double nn2(const MeshView& m, int f) const { return m.nn2[f]; }
  __device__ __forceinline__ double inv_nd(const MeshView& m, int f) const { return m.inv_nd[f]; }
  __device__ __forceinline__ double inv_dpn(const MeshView& m, int f) const {
    return m.inv_dpn[f];
  }
  __device__ __forceinline__ double dpn(const MeshView& m, int f) const { return m.dpn[f]; }
  __device__ __forceinline__ double dnn(const MeshView& m, int f) const { return m.dnn[f]; }
  __device__ __forceinline__ double ns(const MeshView& m, int jq, int f) const {
    return m.ns[(long)jq * m.nf + f];
  }
  __device__ __forceinline__ double vol(const MeshView& m, int c) const { return m.vol[c]; }
  __device__ __forceinline__ double wd(const CaseView& cv, int c) const { return cv.wd[c]; }
  __device__ __forceinline__ double inv_wd(const CaseView& cv, int c) const {
    return cv.inv_wd[c];
  }
  __device__ __forceinline__ double inv_wd2(const CaseView& cv, int c) const {
    return cv.inv_wd2[c];
  }
  __device__ __forceinline__ double wdg(const CaseView& cv, int nc, int j, int c) const {
    return cv.wdg[(long)j * nc + c];
  }
  __device__ __forceinline__ double xf(const MeshView& m, int j, int f) const {
    return m.xf[(long)j * m.nf + f];
  }
  __device__ __forceinline__ double xc(const MeshView& m, int j, int c) const {
    return m.xc[(long)j * m.nc + c];
  }
};

// The fp32 mirror (fp32 passes).
struct GeoPlainF {
  __device__ __forceinline__ float area(const MeshView& m, int f) const { return m.f_area[f]; }
  __device__ __forceinline__ float normal(const MeshView& m, int j, int f) const {
    return m.f_normal[(long)j * m.nf + f];
  }
  __device__ __forceinline__ float tP(const MeshView& m, int j, int f) const {
    return m.f_tP[(long)j * m.nf + f];
  }
  __device__ __forceinline__ float tN(const MeshView& m, int j, int f) const {
    return m.f_tN[(long)j * m.nf + f];
  }
  __device__ __forceinline__ float g(const MeshView& m, int f) const { return m.f_g[f]; }
  __device__ __forceinline__ float dvec(const MeshView& m, int j, int f) const {
    return m.f_dvec[(long)j * m.nf + f];
  }
  __device__ __forceinline__ float skew(const MeshView& m, int j, int f) const {
    return m.f_skew[(long)j * m.nf + f];
  }
  __device__ __forceinline__ float nn2(const MeshView& m, int f) const { return m.f_nn2[f]; }
  __device__ __forceinline__ float inv_nd(const MeshView& m, int f) const { return m.f_inv_nd[f]; }
  __device__ __forceinline__ float inv_dpn(const MeshView& m, int f) const {
    return m.f_inv_dpn[f];
  }
  __device__ __forceinline__ float dpn(const MeshView& m, int f) const { return m.f_dpn[f]; }
  __device__ __forceinline__ float dnn(const MeshView& m, int f) const { return m.f_dnn[f]; }
  __device__ __forceinline__ float ns(const MeshView& m, int jq, int f) const {
    return m.f_ns[(long)jq * m.nf + f];
  }
  __device__ __forceinline__ float vol(const MeshView& m, int c) const { return m.f_vol[c]; }
  __device__ __forceinline__ float wd(const CaseView& cv, int c) const { return cv.f_wd[c]; }
  __device__ __forceinline__ float inv_wd(const CaseView& cv, int c) const {
    return cv.f_inv_wd[c];
  }
  __device__ __forceinline__ float inv_wd2(const CaseView& cv, int c) const {
    return cv.f_inv_wd2[c];
  }
  __device__ __forceinline__ float wdg(const CaseView& cv, int nc, int j, int c) const {
    return cv.f_wdg[(long)j * nc + c];
  }
  __device__ __forceinline__ float xf(const MeshView& m, int j, int f) const {
    return m.f_xf[(long)j * m.nf + f];
  }
  __device__ __forceinline__ float xc(const MeshView& m, int j, int c) const {
    return m.f_xc[(long)j * m.nc + c];
  }
};

// The plain accessor of a pass's scalar type.
template <class T>
struct GeoOf {
  using type = GeoPlain;
};
template <>
struct GeoOf<DualF> {
  using type = GeoPlainF;
};

struct GeoSeed {
  int fcomp;  // seeded face component (GeoFace), -1 for none
  int ccomp;  // seeded cell component (GeoCell), -1 for none
  int face;   // the one seeded face, -1 for every face
  int cell;   // the one seeded cell, -1 for every cell
  __device__ __forceinline__ double hf(int id, int f) const {
    return (fcomp == id && (face < 0 || face == f)) ? 1.0 : 0.0;
  }
  __device__ __forceinline__ double hc(int id, int c) const {
    return (ccomp == id && (cell < 0 || cell == c)) ? 1.0 : 0.0;
  }
  __device__ __forceinline__ Dual area(const MeshView& m, int f) const {
    return {m.area[f], hf(GF_AREA, f)};
  }
  __device__ __forceinline__ Dual normal(const MeshView& m, int j, int f) const {
    return {m.normal[(long)j * m.nf + f], hf(GF_NORMAL + j, f)};
  }
  __device__ __forceinline__ Dual tP(const MeshView& m, int j, int f) const {
    return {m.tP[(long)j * m.nf + f], hf(GF_TP + j, f)};
  }
  __device__ __forceinline__ Dual tN(const MeshView& m, int j, int f) const {
    return {m.tN[(long)j * m.nf + f], hf(GF_TN + j, f)};
  }
  __device__ __forceinline__ Dual g(const MeshView& m, int f) const { return {m.g[f], hf(GF_G, f)}; }
  __device__ __forceinline__ Dual dvec(const MeshView& m, int j, int f) const {
    return {m.dvec[(long)j * m.nf + f], hf(GF_DVEC + j, f)};
  }
  __device__ __forceinline__ Dual skew(const MeshView& m, int j, int f) const {
    return {m.skew[(long)j * m.nf + f], hf(GF_SKEW + j, f)};
  }
  __device__ __forceinline__ Dual nn2(const MeshView& m, int f) const {
    return {m.nn2[f], hf(GF_NN2, f)};
  }
  __device__ __forceinline__ Dual inv_nd(const MeshView& m, int f) const {
    return {m.inv_nd[f], hf(GF_INV_ND, f)};
  }
  __device__ __forceinline__ Dual inv_dpn(const MeshView& m, int f) const {
    return {m.inv_dpn[f], hf(GF_INV_DPN, f)};
  }
  __device__ __forceinline__ Dual dpn(const MeshView& m, int f) const {
    return {m.dpn[f], hf(GF_DPN, f)};
  }
  __device__ __forceinline__ Dual dnn(const MeshView& m, int f) const {
    return {m.dnn[f], hf(GF_DNN, f)};
  }
  __device__ __forceinline__ Dual ns(const MeshView& m, int jq, int f) const {
    return {m.ns[(long)jq * m.nf + f], hf(GF_NS + jq, f)};
  }
  __device__ __forceinline__ Dual vol(const MeshView& m, int c) const {
    return {m.vol[c], hc(GC_VOL, c)};
  }
  __device__ __forceinline__ Dual wd(const CaseView& cv, int c) const {
    return {cv.wd[c], hc(GC_WD, c)};
  }
  __device__ __forceinline__ Dual inv_wd(const CaseView& cv, int c) const {
    return {cv.inv_wd[c], hc(GC_INV_WD, c)};
  }
  __device__ __forceinline__ Dual inv_wd2(const CaseView& cv, int c) const {
    return {cv.inv_wd2[c], hc(GC_INV_WD2, c)};
  }
  __device__ __forceinline__ Dual wdg(const CaseView& cv, int nc, int j, int c) const {
    return {cv.wdg[(long)j * nc + c], hc(GC_WDG + j, c)};
  }
  __device__ __forceinline__ Dual xf(const MeshView& m, int j, int f) const {
    return {m.xf[(long)j * m.nf + f], hf(GF_XF + j, f)};
  }
  __device__ __forceinline__ Dual xc(const MeshView& m, int j, int c) const {
    return {m.xc[(long)j * m.nc + c], hc(GC_XC + j, c)};
  }
};

template <int DIM, bool TURB>
struct Layout {
  static constexpr int NFLD = DIM + 1 + (TURB ? 2 : 0);
  static constexpr int P = DIM, K = DIM + 1, W = DIM + 2;
};

// ---------------------------------------------------------------- workspace
// Forward workspace of one residual evaluation (elements of type T), carved from FvCase::work.
template <class T>
struct Work {
  T* G;      // (NF, DIM, nc) gradients
  T* cl;     // (7, nc) strain, F1, nu_t, wall shear rate, k diffusivity, omega diffusivity, F2
  T* Gwi;    // (DIM, nc) omega gradient with the wall-cell value imposed
  T* acown;  // (nf) momentum-diagonal coefficient, owner side
  T* acnb;   // (nf) neighbour side
  T* dco;    // (nc) d = V / a_P
  T* psi;    // (NA, nc) slope limiter of each advected field (limited upwind only)
  T* me;     // (nf) lagged mass-flux estimate (rho u)_f . n A
  T* FL;     // (NF, nf) face fluxes (also the face scratch of the gradient sweeps)
  T* Bg;     // (NF, DIM, nc) corrected Green-Gauss right-hand side B phi (swept cases only)
  T* Galt;   // (NF, DIM, nc) second iterate buffer of the sweeps (swept cases only)
};
// Number of advected fields (the momentum components, and k and omega) and the limiter storage a
// case needs (limited linear upwind only).
template <int DIM, bool TURB>
__host__ __device__ constexpr int n_advected() {
  return DIM + (TURB ? 2 : 0);
}
template <int DIM, bool TURB>
long psi_count(const FvCase* cs) {
  return (cs->view.rec_mom || cs->view.rec_sca) ? (long)n_advected<DIM, TURB>() * cs->mesh->nc : 0;
}

template <class T, int DIM, bool TURB>
Work<T> work_layout(void* base, long nc, long nf, long npsi = 0) {
  constexpr int NF = Layout<DIM, TURB>::NFLD;
  T* p = (T*)base;
  Work<T> w;
  w.G = p; p += (long)NF * DIM * nc;
  w.cl = p; p += 7 * nc;
  w.Gwi = p; p += DIM * nc;
  w.acown = p; p += nf;
  w.acnb = p; p += nf;
  w.dco = p; p += nc;
  w.psi = p; p += npsi;
  w.me = p; p += nf;
  w.FL = p; p += (long)NF * nf;
  w.Bg = p; p += (long)NF * DIM * nc;
  w.Galt = p;
  return w;
}

// ---------------------------------------------------------------- k_grad
// G = rel * (B phi / V) with B phi the compact Green-Gauss numerator; Bg (may be null) receives
// B phi itself (the right-hand side of the corrected scheme's sweeps).  rel = 1 and Bg = null is
// the compact scheme.
template <class T, int DIM, bool TURB>
__device__ __forceinline__ void k_grad_at(const int c, MeshView m, CaseView cv, Src<T> st, Par<T> par, T* G,
                                              T* Bg, double rel) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  T phic[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q) phic[q] = st((long)q * nc + c);
  T acc[NF][DIM];
#pragma unroll
  for (int q = 0; q < NF; ++q)
#pragma unroll
    for (int j = 0; j < DIM; ++j) acc[q][j] = cst(0.0, phic[0]);
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
    const GS<T> af = gx<T>(m.area, m.f_area, f);
    const GS<T> A = isnb ? -af : af;  // the neighbour takes -S_f phi_f
    GS<T> S[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) S[j] = gx<T>(m.normal, m.f_normal, (long)j * nf + f) * A;
    T phif[NF];
    if (f < m.nfi) {
      const GS<T> g = gx<T>(m.g, m.f_g, f);
      const int other = isnb ? m.owner[f] : m.nb[f];
      // owner value first: the operands are selected, not the interpolation (one code path for
      // both sides of a face, no if-converted duplicate of the dual-number arithmetic)
#pragma unroll
      for (int q = 0; q < NF; ++q) {
        const T po = st((long)q * nc + other);
        phif[q] = lerp(isnb ? po : phic[q], isnb ? phic[q] : po, g);
      }
    } else {
      const signed char kind = cv.fkind[f];
#pragma unroll
      for (int j = 0; j < DIM; ++j) phif[j] = bvel(cv, nf, f, j, kind, phic[j], par);
      phif[L::P] = bpress(cv, f, kind, phic[L::P]);
      if (TURB) {
        T z = cst(0.0, phic[0]);
        phif[L::K] = bscalar(cv.kkind[f], cv.kval[f], phic[L::K], z);
        phif[L::W] = bscalar(cv.wkind[f], cv.wval[f], phic[L::W], z);
      }
    }
#pragma unroll
    for (int q = 0; q < NF; ++q)
#pragma unroll
      for (int j = 0; j < DIM; ++j) acc[q][j] += S[j] * phif[q];
  }
  const GS<T> inv = gx<T>(m.inv_vol, m.f_inv_vol, c);
  if (Bg) {
#pragma unroll
    for (int q = 0; q < NF; ++q)
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        Bg[((long)q * DIM + j) * nc + c] = acc[q][j];
        G[((long)q * DIM + j) * nc + c] = rel * (acc[q][j] * inv);
      }
  } else if (rel != 1.0) {
#pragma unroll
    for (int q = 0; q < NF; ++q)
#pragma unroll
      for (int j = 0; j < DIM; ++j) G[((long)q * DIM + j) * nc + c] = rel * (acc[q][j] * inv);
  } else {
#pragma unroll
    for (int q = 0; q < NF; ++q)
#pragma unroll
      for (int j = 0; j < DIM; ++j) G[((long)q * DIM + j) * nc + c] = acc[q][j] * inv;
  }
}

template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_grad(MeshView m, CaseView cv, Src<T> st, Par<T> par, T* G,
                                              T* Bg, double rel) {
  k_grad_at<T, DIM, TURB>(stage_cell<T>(m, cv), m, cv, st, par, G, Bg, rel);
}

// ---------------------------------------------------------------- corrected Green-Gauss sweeps
// CorrectedGreenGauss (aquaflux/schemes/gradient.py:1122-1337) by SweptGradientSolve
// (gradient.py:618-705): A_g G = V G - C(G), C(G)_c = sum over the interior faces of c of
// +-S_f w_f, w_f = (1 - g) skew . G_P + g skew . G_N; every sweep after the peeled first one is
// X <- X + rel (B phi - A_g X) / V.  Gradients are field-major (NQ, DIM, nc).
//
// w_f for every field (face pass, interior faces).
template <class T, int DIM, int NQ>
__global__ void __launch_bounds__(128) k_gg_skew(MeshView m, const T* X, T* w) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nfi) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f], n = m.nb[f];
  const GS<T> g = gx<T>(m.g, m.f_g, f);
  GS<T> sk[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) sk[j] = gx<T>(m.skew, m.f_skew, (long)j * nf + f);
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    T so = sk[0] * X[((long)q * DIM) * nc + o];
    T sn = sk[0] * X[((long)q * DIM) * nc + n];
#pragma unroll
    for (int j = 1; j < DIM; ++j) {
      so = so + sk[j] * X[((long)q * DIM + j) * nc + o];
      sn = sn + sk[j] * X[((long)q * DIM + j) * nc + n];
    }
    w[(long)q * nf + f] = (GS<T>(1) - g) * so + g * sn;
  }
}

// One sweep (cell pass): Xn = X + rel (Bg - (V X - C(X))) / V.
template <class T, int DIM, int NQ>
__global__ void __launch_bounds__(128) k_gg_sweep(MeshView m, const T* Bg, const T* X, const T* w,
                                                  double rel, T* Xn) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  T corr[NQ][DIM];
  bool first = true;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    if (f >= m.nfi) continue;  // the correction vanishes on boundary faces
    const GS<T> af = gx<T>(m.area, m.f_area, f);
    const GS<T> A = (ent & FV_NB_BIT) ? -af : af;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const T wq = w[(long)q * nf + f];
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        const T x = (gx<T>(m.normal, m.f_normal, (long)j * nf + f) * A) * wq;
        corr[q][j] = first ? x : corr[q][j] + x;
      }
    }
    first = false;
  }
  const GS<T> V = gx<T>(m.vol, m.f_vol, c), inv = gx<T>(m.inv_vol, m.f_inv_vol, c);
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const long k = ((long)q * DIM + j) * nc + c;
      const T x = X[k];
      const T ax = first ? x * V : x * V - corr[q][j];
      Xn[k] = x + rel * ((Bg[k] - ax) * inv);
    }
}

// The swept gradients of NQ fields: on entry G0 holds rel * B phi / V and Bg holds B phi; the
// iterates alternate between G0 and Galt so that the last one lands in G (= G0 or Galt, chosen by
// the caller from the parity of the sweep count).
template <class T, int DIM, int NQ>
void gg_sweeps(const MeshView& m, int sweeps, double rel, const T* Bg, T* G0, T* Galt, T* wface,
               cudaStream_t s) {
  constexpr int TB = 128;
  const int bc = fv_blocks(m.nc, TB), bfi = fv_blocks(m.nfi > 0 ? m.nfi : 1, TB);
  T* cur = G0;
  T* nxt = Galt;
  for (int it = 1; it < sweeps; ++it) {
    if (m.nfi > 0) k_gg_skew<T, DIM, NQ><<<bfi, TB, 0, s>>>(m, cur, wface);
    k_gg_sweep<T, DIM, NQ><<<bc, TB, 0, s>>>(m, Bg, cur, wface, rel, nxt);
    T* t = cur;
    cur = nxt;
    nxt = t;
  }
}

// ---------------------------------------------------------------- k_closure (SST)
// The closure of cell c: out = (S, F1, nu_t, wall shear rate, k diffusivity, omega diffusivity,
// F2), gw = the omega gradient with the wall-cell value imposed.
template <class T, int DIM, class S_, class GV>
__device__ __forceinline__ void closure_cell(const MeshView& m, const CaseView& cv, const S_& st,
                                             const Par<T>& par, const T* G, int c, const GV& gv,
                                             T* out, T* gw) {
  using L = Layout<DIM, true>;
  using GT = decltype(gv.area(m, 0));
  const int nc = m.nc, nf = m.nf;
  T gu[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) gu[i][j] = G[((long)i * DIM + j) * nc + c];
  T sum = cst(0.0, gu[0][0]);
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      T sij = 0.5 * (gu[i][j] + gu[j][i]);
      sum += sij * sij;
    }
  T S = safe_sqrt(2.0 * sum);
  const T k = st((long)L::K * nc + c);
  const T w = st((long)L::W * nc + c);
  const T nu = par.nu;
  const GT d = gv.wd(cv, c), id = gv.inv_wd(cv, c), id2 = gv.inv_wd2(cv, c);
  T gk[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    gk[j] = G[((long)L::K * DIM + j) * nc + c];
    gw[j] = G[((long)L::W * DIM + j) * nc + c];
  }
  T shear = cst(0.0, k);
  if (cv.wcell[c]) {
    T wgt = wall_weight(nu, d, k);
    S = (1.0 - wgt) * S + wgt * log_shear(d, k);
    T dwdd, dwdk;
    omega_wall_partials(nu, d, k, &dwdd, &dwdk);
#pragma unroll
    for (int j = 0; j < DIM; ++j) gw[j] = gv.wdg(cv, nc, j, c) * dwdd + gk[j] * dwdk;
    T num = cst(0.0, k);
    GT den{};
    T u[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) u[j] = st((long)j * nc + c);
    const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
    for (int i = b; i < e; ++i) {
      const int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
      if (f < m.nfi || !cv.swall[f]) continue;
      const signed char kind = cv.fkind[f];
      T s2 = cst(0.0, k);
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        T sl = u[j] - bvel(cv, nf, f, j, kind, u[j], par);
        s2 += sl * sl;
      }
      const GT af = gv.area(m, f);
      num += safe_sqrt(s2) * af;
      den += af;
    }
    shear = num * (id / den);
  }
  // F1 (sst.py:166-202) and the eddy viscosity with F2 (sst.py:152-164, 204-239)
  const T kp = pos(k);
  const T iw = 1.0 / w;
  T dot_kw = gk[0] * gw[0];
#pragma unroll
  for (int j = 1; j < DIM; ++j) dot_kw += gk[j] * gw[j];
  const T cd = fv_max((2.0 * SIGMA_W2) * dot_kw * iw, cst(CROSS_FLOOR, w));
  const T sk = safe_sqrt(kp);
  const T vt = (500.0 * id2) * nu * iw;
  const T c1 = sk * iw * (id / BETA_STAR);
  const T arg1 = fv_min(fv_max(c1, vt), (4.0 * SIGMA_W2 * id2) * kp / cd);
  const T a1sq = arg1 * arg1;
  const T F1 = fv_tanh(a1sq * a1sq);
  const T arg2 = fv_max(2.0 * c1, vt);
  const T F2 = fv_tanh(arg2 * arg2);
  const T nut = A1 * kp / fv_max(A1 * w, S * F2);
  out[0] = S;
  out[1] = F1;
  out[2] = nut;
  out[3] = shear;
  out[4] = nu + (SIGMA_K2 + F1 * (SIGMA_K1 - SIGMA_K2)) * nut;
  out[5] = nu + (SIGMA_W2 + F1 * (SIGMA_W1 - SIGMA_W2)) * nut;
  out[6] = F2;
}

template <class T, int DIM>
__device__ __forceinline__ void k_closure_at(const int c, MeshView m, CaseView cv, Src<T> st, Par<T> par,
                                                 const T* G, T* cl, T* Gwi) {
  if (c >= m.nc) return;
  const int nc = m.nc;
  T out[7], gw[DIM];
  closure_cell<T, DIM>(m, cv, st, par, G, c, typename GeoOf<T>::type{}, out, gw);
#pragma unroll
  for (int i = 0; i < 7; ++i) cl[(long)i * nc + c] = out[i];
#pragma unroll
  for (int j = 0; j < DIM; ++j) Gwi[(long)j * nc + c] = gw[j];
}

template <class T, int DIM>
__global__ void __launch_bounds__(128) k_closure(MeshView m, CaseView cv, Src<T> st, Par<T> par,
                                                 const T* G, T* cl, T* Gwi) {
  k_closure_at<T, DIM>(stage_cell<T>(m, cv), m, cv, st, par, G, cl, Gwi);
}

// effective dynamic viscosity mu + rho nu_t (aquaflux/flow/momentum.py:357-368)
// molecular viscosity of cell c: the case constant, or a per-cell field (laminar batched
// instances) whose tangent under the viscosity seed is the constant's
__device__ __forceinline__ double mu_at(const Par<double>& par, const CaseView& cv, int c) {
  return cv.mu_cell ? cv.mu_cell[c] : par.mu;
}
__device__ __forceinline__ Dual mu_at(const Par<Dual>& par, const CaseView& cv, int c) {
  return cv.mu_cell ? Dual{cv.mu_cell[c], par.mu.d} : par.mu;
}
__device__ __forceinline__ DualF mu_at(const Par<DualF>& par, const CaseView& cv, int c) {
  return cv.mu_cell ? DualF{cv.f_mu_cell[c], par.mu.d} : par.mu;
}
template <class T, bool TURB>
__device__ __forceinline__ T mu_eff(const Par<T>& par, const CaseView& cv, GS<T> rho, const T* cl,
                                    int nc, int c) {
  if (TURB) return par.mu + rho * cl[2L * nc + c];
  return mu_at(par, cv, c);
}

// lagged advective momentum flux (rho u)_f . n with the skew-corrected face value
// (aquaflux/flow/rhie_chow.py:220-271): rho (sum_j n_j u_j,f + sum_jq n_j skew_q (grad u)_jq,f)
template <class T, int DIM, bool TURB, class S, class GV, class GT>
__device__ __forceinline__ T mom_normal(const MeshView& m, const S& st, const T* G, GS<T> rho,
                                        int f, int o, int n, GT g, const GV& gv) {
  const int nc = m.nc;
  T mn = cst(0.0, st(o));
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    mn += gv.normal(m, j, f) * lerp(st((long)j * nc + o), st((long)j * nc + n), g);
#pragma unroll
    for (int q = 0; q < DIM; ++q)
      mn += gv.ns(m, j * DIM + q, f) *
            lerp(G[((long)j * DIM + q) * nc + o], G[((long)j * DIM + q) * nc + n], g);
  }
  return rho * mn;
}

// flux-continuous conductance g_o A / (dpn - g_o / g_n dnn), one division
// (aquaflux/discretization/diffusion.py:85-134)
template <class T, class GT>
__device__ __forceinline__ T conductance(T go, T gn, GT A, GT dpn, GT dnn) {
  return go * gn * A / (dpn * gn - go * dnn);
}

// ---------------------------------------------------------------- slope limiter
// VenkatakrishnanLimiter.limit (aquaflux/schemes/limiter.py:78-117) of one field at cell c:
// psi = clip(min over the cell's faces of psi_face, 0, 1), psi_face from the unlimited increment
// dm = grad . (x_f - x_c) (regularised away from 0) and the headroom to the extrema over the cell
// and its face neighbours, eps^2 = V K^3.  phi(cell) and grad(j) read the field (either may carry
// a tangent).
template <class T, int DIM, class PhiFn, class GradFn, class GV = typename GeoOf<T>::type>
__device__ __forceinline__ T limiter_cell(const MeshView& m, int c, double K, const PhiFn& phi,
                                          const GradFn& grad, const GV& gv = GV{}) {
  const int nc = m.nc, nf = m.nf;
  const T pc = phi(c);
  T pmax = pc, pmin = pc;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    if (f >= m.nfi) continue;
    const T po = phi((ent & FV_NB_BIT) ? m.owner[f] : m.nb[f]);
    pmax = fv_max(pmax, po);
    pmin = fv_min(pmin, po);
  }
  using GT = decltype(gv.vol(m, 0));
  using KT = typename std::conditional<std::is_same<GT, float>::value, float, double>::type;
  const GT e2 = gv.vol(m, c) * KT(K * K * K);
  T psi = cst(1.0, pc);
  for (int i = b; i < e; ++i) {
    const int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
    T dm = grad(0) * (gv.xf(m, 0, f) - gv.xc(m, 0, c));
#pragma unroll
    for (int j = 1; j < DIM; ++j) dm = dm + grad(j) * (gv.xf(m, j, f) - gv.xc(m, j, c));
    const double sign = val(dm) >= 0.0 ? 1.0 : -1.0;
    dm = sign * (fv_abs(dm) + 1e-12);
    const T head = val(dm) > 0.0 ? pmax - pc : pmin - pc;
    const T num = (head * head + e2) * dm + 2.0 * (dm * dm) * head;
    const T den = (head * head + 2.0 * (dm * dm) + head * dm + e2) * dm;
    const T pf = num / den;
    psi = i == b ? pf : fv_min(psi, pf);
  }
  return fv_min(fv_max(psi, cst(0.0, psi)), cst(1.0, psi));
}

// Field index of advected field a: the momentum components, then k and omega.
template <int DIM, bool TURB>
__device__ __forceinline__ int advected_field(int a) {
  return a < DIM ? a : (a == DIM ? Layout<DIM, TURB>::K : Layout<DIM, TURB>::W);
}

// Km / Ks: the limiter constants of the momentum components / of k and omega (0: psi = 1).
template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_limiter(MeshView m, Src<T> st, const T* G, double Km,
                                                 double Ks, T* psi) {
  constexpr int NA = n_advected<DIM, TURB>();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
#pragma unroll 1
  for (int a = 0; a < NA; ++a) {
    const int q = advected_field<DIM, TURB>(a);
    const double K = a < DIM ? Km : Ks;
    T v;
    if (K > 0.0) {
      auto phi = [&](int cell) { return st((long)q * nc + cell); };
      auto grad = [&](int j) { return G[((long)q * DIM + j) * nc + c]; };
      v = limiter_cell<T, DIM>(m, c, K, phi, grad);
    } else {
      v = cst(1.0, st((long)q * nc + c));
    }
    psi[(long)a * nc + c] = v;
  }
}

// The advected face value of field q through face f from the upwind cell cu (upwind_value, the
// cell value; with a limiter, plus psi grad . (x_f - x_cu)).
template <class T, int DIM, class GV>
__device__ __forceinline__ T upwind_rec(const MeshView& m, const T* G, const T* psi, int a, int q,
                                        int f, int cu, const T& value, const GV& gv) {
  if (!psi) return value;
  const int nc = m.nc;
  T d = G[((long)q * DIM) * nc + cu] * (gv.xf(m, 0, f) - gv.xc(m, 0, cu));
#pragma unroll
  for (int j = 1; j < DIM; ++j)
    d = d + G[((long)q * DIM + j) * nc + cu] * (gv.xf(m, j, f) - gv.xc(m, j, cu));
  return value + psi[(long)a * nc + cu] * d;
}

// ---------------------------------------------------------------- k_apcoef
// The momentum-diagonal face coefficients of face f (owner side, neighbour side) and the lagged
// mass-flux estimate me.
template <class T, int DIM, bool TURB, class S_, class GV>
__device__ __forceinline__ void apcoef_face(const MeshView& m, const CaseView& cv, const S_& st,
                                            const Par<T>& par, const T* G, const T* cl, int f,
                                            const GV& gv, T& ac_own, T& ac_nb, T& me) {
  using L = Layout<DIM, TURB>;
  using GT = decltype(gv.area(m, 0));
  const int nc = m.nc;
  const int o = m.owner[f];
  const bool interior = f < m.nfi;
  const int n = interior ? m.nb[f] : o;
  const GT g = gv.g(m, f), A = gv.area(m, f);
  const GS<T> rho = rho_of<T>(cv);
  const T mdot = mom_normal<T, DIM, TURB>(m, st, G, rho, f, o, n, g, gv) * A;
  me = mdot;
  const T mo = mu_eff<T, TURB>(par, cv, rho, cl, nc, o);
  if (interior) {
    const T mnb = mu_eff<T, TURB>(par, cv, rho, cl, nc, n);
    const T visc = conductance(mo, mnb, A, gv.dpn(m, f), gv.dnn(m, f));
    ac_own = visc + pos(mdot);
    ac_nb = visc + pos(-mdot);
  } else {
    const signed char kind = cv.fkind[f];
    T bv = mo;
    if (TURB && (kind == 0 || kind == 1)) {
      T nutw = cst(0.0, mo);
      if (cv.swall[f]) nutw = nut_wall(par.nu, gv.wd(cv, o), st((long)L::K * nc + o));
      bv = par.mu + rho * nutw;
    }
    const T vo = bv * (A * gv.inv_nd(m, f));
    const T conv = pos(mdot);
    ac_own = kind == 0 || kind == 1 ? vo : (kind == 2 ? vo + conv : (kind == 3 ? conv : cst(0.0, vo)));
    ac_nb = cst(0.0, vo);
  }
}

template <class T, int DIM, bool TURB>
__device__ __forceinline__ void k_apcoef_at(const int f, MeshView m, CaseView cv, Src<T> st, Par<T> par,
                                                const T* G, const T* cl, T* ac_own, T* ac_nb,
                                                T* me) {
  if (f >= m.nf) return;
  T ao, an, mf;
  apcoef_face<T, DIM, TURB>(m, cv, st, par, G, cl, f, typename GeoOf<T>::type{}, ao, an, mf);
  ac_own[f] = ao;
  ac_nb[f] = an;
  me[f] = mf;
}

template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_apcoef(MeshView m, CaseView cv, Src<T> st, Par<T> par,
                                                const T* G, const T* cl, T* ac_own, T* ac_nb,
                                                T* me, int face0 = 0) {
  k_apcoef_at<T, DIM, TURB>(face0 + blockIdx.x * blockDim.x + threadIdx.x, m, cv, st, par, G, cl, ac_own, ac_nb, me);
}

// The interior faces' momentum-diagonal coefficients and mass-flux estimate of a state-tangent
// dual-number pass at a held linearisation: the momentum-normal flux is linear in the velocities
// and their gradients, the conductance's tangent comes from its kept partial derivatives in the
// cell viscosities, max(., 0) follows the kept sign of the estimate (JAX's tie rule); the primal
// values are the kept ones (lin: owner coefficient, neighbour coefficient, estimate).
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_apcoef_tangent(MeshView m, CaseView cv, Src<Dual> st,
                                                        const Dual* G, const Dual* cl,
                                                        const double* aux, const double* lin,
                                                        Dual* ac_own, Dual* ac_nb, Dual* me) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nfi) return;
  const long nc = m.nc, nf = m.nf;
  const int o = m.owner[f], n = m.nb[f];
  const double g = m.g[f], A = m.area[f], rho = cv.rho;
  double mn_t = 0.0;
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    mn_t += m.normal[(long)j * nf + f] * lerp(st((long)j * nc + o).d, st((long)j * nc + n).d, g);
#pragma unroll
    for (int q = 0; q < DIM; ++q)
      mn_t += m.ns[(long)(j * DIM + q) * nf + f] *
              lerp(G[((long)j * DIM + q) * nc + o].d, G[((long)j * DIM + q) * nc + n].d, g);
  }
  const double me_t = (rho * mn_t) * A;
  const double mo_t = TURB ? rho * cl[2L * nc + o].d : 0.0;
  const double mn_c = TURB ? rho * cl[2L * nc + n].d : 0.0;
  const double visc_t = aux[4L * nf + f] * mo_t + aux[5L * nf + f] * mn_c;
  const double e = lin[2L * nf + f];
  const double pp = e > 0.0 ? me_t : (e < 0.0 ? 0.0 : 0.5 * me_t);
  const double pm = e < 0.0 ? -me_t : (e > 0.0 ? 0.0 : 0.5 * -me_t);
  ac_own[f] = Dual{lin[f], visc_t + pp};
  ac_nb[f] = Dual{lin[(long)nf + f], visc_t + pm};
  me[f] = Dual{e, me_t};
}

// The compact Green-Gauss gradients of a state-tangent dual-number pass at a held linearisation:
// the scheme is linear, so the tangents are the face-value tangents' gradients (boundary values by
// the dual-number closures) and the primal gradients are the kept ones.
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_grad_tangent(MeshView m, CaseView cv, Src<Dual> st,
                                                      Par<Dual> par, const double* Gp, Dual* G) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  const int c = stage_cell<Dual>(m, cv);
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  Dual phic[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q) phic[q] = st((long)q * nc + c);
  double acc[NF][DIM];
#pragma unroll
  for (int q = 0; q < NF; ++q)
#pragma unroll
    for (int j = 0; j < DIM; ++j) acc[q][j] = 0.0;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
    const double af = m.area[f];
    const double A = isnb ? -af : af;
    double S[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) S[j] = m.normal[(long)j * nf + f] * A;
    double phif[NF];
    if (f < m.nfi) {
      const double g = m.g[f];
      const int other = isnb ? m.owner[f] : m.nb[f];
#pragma unroll
      for (int q = 0; q < NF; ++q) {
        const double po = st((long)q * nc + other).d;
        phif[q] = lerp(isnb ? po : phic[q].d, isnb ? phic[q].d : po, g);
      }
    } else {
      const signed char kind = cv.fkind[f];
#pragma unroll
      for (int j = 0; j < DIM; ++j) phif[j] = bvel(cv, nf, f, j, kind, phic[j], par).d;
      phif[L::P] = bpress(cv, f, kind, phic[L::P]).d;
      if (TURB) {
        const Dual z = cst(0.0, phic[0]);
        phif[L::K] = bscalar(cv.kkind[f], cv.kval[f], phic[L::K], z).d;
        phif[L::W] = bscalar(cv.wkind[f], cv.wval[f], phic[L::W], z).d;
      }
    }
#pragma unroll
    for (int q = 0; q < NF; ++q)
#pragma unroll
      for (int j = 0; j < DIM; ++j) acc[q][j] += S[j] * phif[q];
  }
  const double inv = m.inv_vol[c];
#pragma unroll
  for (int q = 0; q < NF; ++q)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const long k = ((long)q * DIM + j) * nc + c;
      G[k] = Dual{Gp[k], acc[q][j] * inv};
    }
}

// ---------------------------------------------------------------- k_dcoeff
template <class T>
__device__ __forceinline__ void k_dcoeff_at(const int c, MeshView m, const T* ac_own, const T* ac_nb, T* dco) {
  if (c >= m.nc) return;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  T a;
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    T x = (ent & FV_NB_BIT) ? ac_nb[f] : ac_own[f];
    a = i == b ? x : a + x;
  }
  dco[c] = gx<T>(m.vol, m.f_vol, c) / a;
}

template <class T>
__global__ void k_dcoeff(MeshView m, const T* ac_own, const T* ac_nb, T* dco) {
  k_dcoeff_at<T>(blockIdx.x * blockDim.x + threadIdx.x, m, ac_own, ac_nb, dco);
}

// ---------------------------------------------------------------- k_flux
// Face intermediates kept for the adjoint (double forward pass only), (FV_AUX_N, nf):
//   0 mdot, 1 damping, 2 dhat, 3 c (momentum conductance), 4 dc/dm_o, 5 dc/dm_n,
//   6.. 6+DIM-1 diffusion numerators of the velocity components, then for k and omega:
//   conductance, d/dgamma_o, d/dgamma_n, numerator.
template <int DIM, bool TURB>
struct Aux {
  static constexpr int N = 6 + DIM + (TURB ? 8 : 0);
  static constexpr int CPN = 6, S0 = 6 + DIM;
};

// The fluxes of face f, handed to wr(q, flux_q) for every field q.  `st` reads the state (Src, or
// a seeded accessor in the Jacobian assembly); aux (double only) receives the face intermediates.
template <class T, int DIM, bool TURB, class S, class Wr, class GV = typename GeoOf<T>::type>
__device__ __forceinline__ void flux_face(const MeshView& m, const CaseView& cv, const S& st,
                                          const Par<T>& par, const T* G, const T* cl, const T* dco,
                                          const T* me, const T* psi, bool recompute_me, int f,
                                          const Wr& wr, double* aux, const GV& gv = GV{}) {
  using GT = decltype(gv.area(m, 0));
  constexpr bool KEEP = std::is_same<T, double>::value && std::is_same<GT, double>::value;
  using L = Layout<DIM, TURB>;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f];
  const GT A = gv.area(m, f);
  const GS<T> rho = rho_of<T>(cv), irho = GS<T>(1) / rho;
  GT nrm[DIM], tP[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    nrm[j] = gv.normal(m, j, f);
    tP[j] = gv.tP(m, j, f);
  }
  const T po = st((long)L::P * nc + o);
  const T mo = mu_eff<T, TURB>(par, cv, rho, cl, nc, o);
  if (f < m.nfi) {
    const int n = m.nb[f];
    const GT g = gv.g(m, f);
    GT tN[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) tN[j] = gv.tN(m, j, f);
    const T pn = st((long)L::P * nc + n);
    const T mest = recompute_me ? mom_normal<T, DIM, TURB>(m, st, G, rho, f, o, n, g, gv) * A : me[f];
    T gd = cst(0.0, po), gs = cst(0.0, po);
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const T gpf = lerp(G[((long)L::P * DIM + j) * nc + o], G[((long)L::P * DIM + j) * nc + n], g);
      gd += gpf * gv.dvec(m, j, f);
      gs += gpf * gv.skew(m, j, f);
    }
    const T dhat = gv.nn2(m, f) * lerp(dco[o], dco[n], g);
    const T damping = ((pn - po) - gd) * gv.inv_nd(m, f);
    const T mdot = mest - (rho * A) * dhat * damping;
    const T pf = lerp(po, pn, g) + gs;
    const T mnb = mu_eff<T, TURB>(par, cv, rho, cl, nc, n);
    const T iden = 1.0 / (gv.dpn(m, f) * mnb - mo * gv.dnn(m, f));
    const T cmo = mo * mnb * A * iden;
    const bool out = val(mdot) >= 0.0;
    const T pA = pf * A;
    using AX = Aux<DIM, TURB>;
    if constexpr (KEEP) {
      if (aux) {
        aux[0L * nf + f] = mdot;
        aux[1L * nf + f] = damping;
        aux[2L * nf + f] = dhat;
        aux[3L * nf + f] = cmo;
        aux[4L * nf + f] = (mnb * A * iden) * (1.0 + mo * m.dnn[f] * iden);
        aux[5L * nf + f] = (mo * A * iden) * (1.0 - mnb * m.dpn[f] * iden);
      }
    }
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      const T uo = st((long)i * nc + o), un = st((long)i * nc + n);
      T cpn = (un - uo);
#pragma unroll
      for (int j = 0; j < DIM; ++j)
        cpn += G[((long)i * DIM + j) * nc + n] * tN[j] - G[((long)i * DIM + j) * nc + o] * tP[j];
      const T* pm = cv.rec_mom ? psi : nullptr;
      const T up = out ? upwind_rec<T, DIM>(m, G, pm, i, i, f, o, uo, gv)
                       : upwind_rec<T, DIM>(m, G, pm, i, i, f, n, un, gv);
      wr(i, (pA * nrm[i] - cmo * cpn) + mdot * up);
      if constexpr (KEEP) {
        if (aux) aux[(long)(AX::CPN + i) * nf + f] = cpn;
      }
    }
    wr(L::P, mdot);
    if (TURB) {
      const T vflux = mdot * irho;
      const bool vout = val(vflux) >= 0.0;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int q = s == 0 ? L::K : L::W;
        const T go = cl[(4L + s) * nc + o], gn = cl[(4L + s) * nc + n];
        const T phio = st((long)q * nc + o), phin = st((long)q * nc + n);
        T cpn = (phin - phio);
#pragma unroll
        for (int j = 0; j < DIM; ++j)
          cpn += G[((long)q * DIM + j) * nc + n] * tN[j] - G[((long)q * DIM + j) * nc + o] * tP[j];
        const T idn = 1.0 / (gv.dpn(m, f) * gn - go * gv.dnn(m, f));
        const T cs_ = go * gn * A * idn;
        const T* ps = cv.rec_sca ? psi : nullptr;
        const T up = vout ? upwind_rec<T, DIM>(m, G, ps, DIM + s, q, f, o, phio, gv)
                          : upwind_rec<T, DIM>(m, G, ps, DIM + s, q, f, n, phin, gv);
        wr(q, vflux * up - cs_ * cpn);
        if constexpr (KEEP) {
          if (aux) {
            const long b0 = AX::S0 + 4 * s;
            aux[b0 * nf + f] = cs_;
            aux[(b0 + 1) * nf + f] = (gn * A * idn) * (1.0 + go * m.dnn[f] * idn);
            aux[(b0 + 2) * nf + f] = (go * A * idn) * (1.0 - gn * m.dpn[f] * idn);
            aux[(b0 + 3) * nf + f] = cpn;
          }
        }
      }
    }
  } else {
    const signed char kind = cv.fkind[f];
    T uo[DIM], bu[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      uo[j] = st((long)j * nc + o);
      bu[j] = bvel(cv, nf, f, j, kind, uo[j], par);
    }
    T mdot;
    if (kind == 2) {
      T un = bu[0] * nrm[0];
#pragma unroll
      for (int j = 1; j < DIM; ++j) un += bu[j] * nrm[j];
      mdot = (rho * A) * un;
    } else if (kind == 3) {
      T un = uo[0] * nrm[0];
      T interp = G[((long)L::P * DIM) * nc + o] * nrm[0];
#pragma unroll
      for (int j = 1; j < DIM; ++j) {
        un += uo[j] * nrm[j];
        interp += G[((long)L::P * DIM + j) * nc + o] * nrm[j];
      }
      const T dh = gv.nn2(m, f) * dco[o];
      const T compact = (cv.fp[f] - po) * gv.inv_nd(m, f);
      mdot = (rho * A) * (un - dh * (compact - interp));
    } else {
      mdot = cst(0.0, po);
    }
    const T pf = bpress(cv, f, kind, po);
    T gb = mo;
    if (TURB && (kind == 0 || kind == 1)) {
      T nutw = cst(0.0, mo);
      if (cv.swall[f]) nutw = nut_wall(par.nu, gv.wd(cv, o), st((long)L::K * nc + o));
      gb = par.mu + rho * nutw;
    }
    const T gA = gb * (A * gv.inv_dpn(m, f));
    const bool out = val(mdot) >= 0.0;
    const T pA = pf * A;
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      T cp = G[((long)i * DIM) * nc + o] * tP[0];
#pragma unroll
      for (int j = 1; j < DIM; ++j) cp += G[((long)i * DIM + j) * nc + o] * tP[j];
      const T up = out ? upwind_rec<T, DIM>(m, G, cv.rec_mom ? psi : nullptr, i, i, f, o, uo[i], gv)
                       : bu[i];
      wr(i, (pA * nrm[i] - gA * (bu[i] - uo[i] - cp)) + mdot * up);
    }
    wr(L::P, mdot);
    if (TURB) {
      const T vflux = mdot * irho;
      const bool vout = val(vflux) >= 0.0;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int q = s == 0 ? L::K : L::W;
        const T go = cl[(4L + s) * nc + o];
        const T phio = st((long)q * nc + o);
        T cp = G[((long)q * DIM) * nc + o] * tP[0];
#pragma unroll
        for (int j = 1; j < DIM; ++j) cp += G[((long)q * DIM + j) * nc + o] * tP[j];
        const T bphi = s == 0 ? bscalar(cv.kkind[f], cv.kval[f], phio, cp)
                              : bscalar(cv.wkind[f], cv.wval[f], phio, cp);
        T gface = go;
        if (s == 0 && cv.swall[f]) gface = (1.0 - wall_weight(par.nu, gv.wd(cv, o), phio)) * go;
        const T up = vout ? upwind_rec<T, DIM>(m, G, cv.rec_sca ? psi : nullptr, DIM + s, q, f, o,
                                               phio, gv)
                          : bphi;
        wr(q, vflux * up - gface * (A * gv.inv_dpn(m, f)) * (bphi - phio - cp));
      }
    }
  }
}

template <class T>
struct FluxStore {
  T* FL;
  int nf, f;
  __device__ __forceinline__ void operator()(int q, const T& x) const { FL[(long)q * nf + f] = x; }
};

template <class T, int DIM, bool TURB>
__device__ __forceinline__ void k_flux_at(const int f, MeshView m, CaseView cv, Src<T> st, Par<T> par,
                                              const T* G, const T* cl, const T* dco, const T* me,
                                              const T* psi, bool recompute_me, T* FL, double* aux) {
  if (f >= m.nf) return;
  flux_face<T, DIM, TURB>(m, cv, st, par, G, cl, dco, me, psi, recompute_me, f,
                          FluxStore<T>{FL, m.nf, f}, aux);
}

template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_flux(MeshView m, CaseView cv, Src<T> st, Par<T> par,
                                              const T* G, const T* cl, const T* dco, const T* me,
                                              const T* psi, bool recompute_me, T* FL, double* aux,
                                              int face0 = 0) {
  k_flux_at<T, DIM, TURB>(face0 + blockIdx.x * blockDim.x + threadIdx.x, m, cv, st, par, G, cl, dco, me, psi, recompute_me, FL, aux);
}

// The interior face fluxes of a state-tangent dual-number pass at a held linearisation (first-order
// upwind): the primal face intermediates the double pass kept (mass flux, pressure damping,
// interpolated d, conductances and their partial derivatives in the cell diffusivities, the
// cross-diffusion numerators) stand in for their recomputation, so only the tangent arithmetic of
// flux_face runs -- the forward-mode counterpart of the adjoint's use of the same intermediates.
// The primal fluxes are the kept ones.  Mass-flux estimate, gradients, closure and d arrive as dual
// numbers from the pass's earlier stages.
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_flux_tangent(MeshView m, CaseView cv, Src<Dual> st,
                                                      const Dual* G, const Dual* cl,
                                                      const Dual* dco, const Dual* me,
                                                      const double* aux, const double* flp,
                                                      Dual* FL) {
  using L = Layout<DIM, TURB>;
  using AX = Aux<DIM, TURB>;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nfi) return;
  const long nc = m.nc, nf = m.nf;
  const int o = m.owner[f], n = m.nb[f];
  const double A = m.area[f], g = m.g[f];
  const double rho = cv.rho, irho = 1.0 / cv.rho;
  const double mdot = aux[0L * nf + f], damping = aux[1L * nf + f], dhat = aux[2L * nf + f];
  const double cmo = aux[3L * nf + f], dcdo = aux[4L * nf + f], dcdn = aux[5L * nf + f];
  double gd = 0.0, gs = 0.0;
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    const double gpf = lerp(G[((long)L::P * DIM + j) * nc + o].d, G[((long)L::P * DIM + j) * nc + n].d, g);
    gd += gpf * m.dvec[(long)j * nf + f];
    gs += gpf * m.skew[(long)j * nf + f];
  }
  const double dhat_t = m.nn2[f] * lerp(dco[o].d, dco[n].d, g);
  const Dual po = st((long)L::P * nc + o), pn = st((long)L::P * nc + n);
  const double damp_t = ((pn.d - po.d) - gd) * m.inv_nd[f];
  const double mdot_t = me[f].d - (rho * A) * (dhat_t * damping + dhat * damp_t);
  const double pA_t = (lerp(po.d, pn.d, g) + gs) * A;
  // d(mu + rho nu_t) for a state tangent (the molecular viscosity is a parameter)
  const double mo_t = TURB ? rho * cl[2L * nc + o].d : 0.0;
  const double mn_t = TURB ? rho * cl[2L * nc + n].d : 0.0;
  const double cmo_t = dcdo * mo_t + dcdn * mn_t;
  const bool out = mdot >= 0.0;
  double tP[DIM], tN[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    tP[j] = m.tP[(long)j * nf + f];
    tN[j] = m.tN[(long)j * nf + f];
  }
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    const Dual uo = st((long)i * nc + o), un = st((long)i * nc + n);
    double cpn_t = un.d - uo.d;
#pragma unroll
    for (int j = 0; j < DIM; ++j)
      cpn_t += G[((long)i * DIM + j) * nc + n].d * tN[j] - G[((long)i * DIM + j) * nc + o].d * tP[j];
    const double cpn = aux[(long)(AX::CPN + i) * nf + f];
    const double up = out ? uo.v : un.v, up_t = out ? uo.d : un.d;
    const double ft = (pA_t * m.normal[(long)i * nf + f] - (cmo_t * cpn + cmo * cpn_t)) +
                      (mdot_t * up + mdot * up_t);
    FL[(long)i * nf + f] = Dual{flp[(long)i * nf + f], ft};
  }
  FL[(long)L::P * nf + f] = Dual{flp[(long)L::P * nf + f], mdot_t};
  if (TURB) {
    const double vflux = mdot * irho, vflux_t = mdot_t * irho;
    const bool vout = vflux >= 0.0;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int q = s == 0 ? L::K : L::W;
      const long b0 = AX::S0 + 4 * s;
      const double go_t = cl[(4L + s) * nc + o].d, gn_t = cl[(4L + s) * nc + n].d;
      const Dual phio = st((long)q * nc + o), phin = st((long)q * nc + n);
      double cpn_t = phin.d - phio.d;
#pragma unroll
      for (int j = 0; j < DIM; ++j)
        cpn_t += G[((long)q * DIM + j) * nc + n].d * tN[j] - G[((long)q * DIM + j) * nc + o].d * tP[j];
      const double cs = aux[b0 * nf + f], cpn = aux[(b0 + 3) * nf + f];
      const double cs_t = aux[(b0 + 1) * nf + f] * go_t + aux[(b0 + 2) * nf + f] * gn_t;
      const double up = vout ? phio.v : phin.v, up_t = vout ? phio.d : phin.d;
      const double ft = (vflux_t * up + vflux * up_t) - (cs_t * cpn + cs * cpn_t);
      FL[(long)q * nf + f] = Dual{flp[(long)q * nf + f], ft};
    }
  }
}

// ---------------------------------------------------------------- k_sum
// SST rows of cell c: k and omega source terms added to the face sums rk / rw, and the omega
// wall-cell fixation (aquaflux/turbulence/sources.py:60-412, fixed_value.py:124-158).
template <class T, int DIM, class Acc, class GV = typename GeoOf<T>::type>
__device__ __forceinline__ void sst_rows(const MeshView& m, const CaseView& cv, const Acc& st,
                                         const Par<T>& par, const T* cl, const T* G, const T* Gwi,
                                         int c, T& rk, T& rw, const GV& gv = GV{}) {
  using L = Layout<DIM, true>;
  using GT = decltype(gv.area(m, 0));
  const int nc = m.nc;
  const GT V = gv.vol(m, c);
  const T k = st((long)L::K * nc + c), w = st((long)L::W * nc + c);
  const T S = cl[c], F1 = cl[(long)nc + c], nut = cl[2L * nc + c];
  const T nu = par.nu;
  const GT d = gv.wd(cv, c);
  const bool wall = cv.wcell[c] != 0;
  const T kp = pos(k);
  const T limit = (PROD_RATIO * BETA_STAR) * kp * w;
  T lim = fv_min(nut * (S * S), limit);
  T weff = w;
  if (wall) {
    const T lw = wall_weight(nu, d, k);
    const T pw = (nu + nut_wall(nu, d, k)) * cl[3L * nc + c] * log_shear(d, k);
    lim = (1.0 - lw) * lim + lw * pw;
    weff = omega_wall(nu, d, k);
  }
  rk = rk - lim * V;
  rk = rk + BETA_STAR * V * k * weff;
  if (wall) {
    // DifferenceRow w - omega_wall, or LogRatioRow log(w / omega_wall) for a log-solved omega
    // (aquaflux/discretization/fixed_value.py:80-120)
    rw = cv.log_w ? fv_log(w / omega_wall(nu, d, k)) : w - omega_wall(nu, d, k);
  } else {
    const T alpha = ALPHA_2 + F1 * (ALPHA_1 - ALPHA_2);
    const T cap = limit / fv_max(nut, cst(NUT_FLOOR, nut));
    const T beta = BETA_2 + F1 * (BETA_1 - BETA_2);
    T dkw = G[((long)L::K * DIM) * nc + c] * Gwi[c];
#pragma unroll
    for (int j = 1; j < DIM; ++j) dkw += G[((long)L::K * DIM + j) * nc + c] * Gwi[(long)j * nc + c];
    const T cross = (2.0 * SIGMA_W2) * (1.0 - F1) * dkw / w;
    rw = rw + V * (beta * (w * w) - alpha * fv_min(S * S, cap) - cross);
  }
}

template <class T, int DIM, bool TURB>
__device__ __forceinline__ void k_sum_at(const int c, MeshView m, CaseView cv, Src<T> st, Par<T> par, const T* FL, const T* cl,
                                             const T* G, const T* Gwi, double* R, double* JV) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  T r[NF];
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      T x = FL[(long)q * nf + f];
      if (isnb) x = -x;
      r[q] = i == b ? x : r[q] + x;
    }
  }
  if (c == cv.pin) r[L::P] = st((long)L::P * nc + c) - cv.pin_value;
  if constexpr (TURB) sst_rows<T, DIM>(m, cv, st, par, cl, G, Gwi, c, r[L::K], r[L::W]);
#pragma unroll
  for (int q = 0; q < NF; ++q) put<T>(R, JV, (long)q * nc + c, r[q]);
}

template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_sum(MeshView m, CaseView cv, Src<T> st, Par<T> par, const T* FL, const T* cl,
                                             const T* G, const T* Gwi, double* R, double* JV) {
  k_sum_at<T, DIM, TURB>(stage_cell<T>(m, cv), m, cv, st, par, FL, cl, G, Gwi, R, JV);
}

// ---------------------------------------------------------------- linearised SST closure
// Off the wall, the closure fields and the k / omega source terms of a cell depend on the state
// through four scalars only: k, omega, the strain rate S and grad k . grad omega.  At a held
// linearisation their tangents are therefore linear forms in those four tangents, tabulated once
// per linearisation (k_lin_closure_coef) and applied by every Krylov product (k_closure_lin,
// k_sum_lin) instead of the dual-number closure and source rows.  Wall cells (wall functions,
// omega fixation) keep the dual-number path.

// A value with N tangent directions, under the dual number's rules (max / min split the tangent
// at a tie; safe_sqrt and the k >= 0 clamp give a zero tangent where they clamp).
template <int N>
struct DualV {
  double v, d[N];
};
template <int N>
__device__ __forceinline__ double val(const DualV<N>& x) { return x.v; }
template <int N>
__device__ __forceinline__ DualV<N> cst(double x, const DualV<N>&) {
  DualV<N> r;
  r.v = x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N>
__device__ __forceinline__ DualV<N> lin_comb(double v, double a, const DualV<N>& x, double b,
                                            const DualV<N>& y) {  // value v, tangent a x' + b y'
  DualV<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a * x.d[i] + b * y.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualV<N> scaled(double v, double a, const DualV<N>& x) {
  DualV<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a * x.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ DualV<N> operator+(const DualV<N>& a, const DualV<N>& b) {
  return lin_comb(a.v + b.v, 1.0, a, 1.0, b);
}
template <int N>
__device__ __forceinline__ DualV<N> operator-(const DualV<N>& a, const DualV<N>& b) {
  return lin_comb(a.v - b.v, 1.0, a, -1.0, b);
}
template <int N>
__device__ __forceinline__ DualV<N> operator*(const DualV<N>& a, const DualV<N>& b) {
  return lin_comb(a.v * b.v, b.v, a, a.v, b);
}
template <int N>
__device__ __forceinline__ DualV<N> operator/(const DualV<N>& a, const DualV<N>& b) {
  const double r = 1.0 / b.v, q = a.v * r;
  return lin_comb(q, r, a, -q * r, b);
}
template <int N>
__device__ __forceinline__ DualV<N> operator+(const DualV<N>& a, double b) { return scaled(a.v + b, 1.0, a); }
template <int N>
__device__ __forceinline__ DualV<N> operator+(double a, const DualV<N>& b) { return scaled(a + b.v, 1.0, b); }
template <int N>
__device__ __forceinline__ DualV<N> operator-(const DualV<N>& a, double b) { return scaled(a.v - b, 1.0, a); }
template <int N>
__device__ __forceinline__ DualV<N> operator-(double a, const DualV<N>& b) { return scaled(a - b.v, -1.0, b); }
template <int N>
__device__ __forceinline__ DualV<N> operator*(const DualV<N>& a, double b) { return scaled(a.v * b, b, a); }
template <int N>
__device__ __forceinline__ DualV<N> operator*(double a, const DualV<N>& b) { return scaled(a * b.v, a, b); }
template <int N>
__device__ __forceinline__ DualV<N> operator/(const DualV<N>& a, double b) {
  const double r = 1.0 / b;
  return scaled(a.v * r, r, a);
}
template <int N>
__device__ __forceinline__ DualV<N> operator/(double a, const DualV<N>& b) {
  const double r = 1.0 / b.v, q = a * r;
  return scaled(q, -q * r, b);
}
template <int N>
__device__ __forceinline__ DualV<N> fv_max(const DualV<N>& a, const DualV<N>& b) {
  if (a.v > b.v) return a;
  if (a.v < b.v) return b;
  return lin_comb(a.v, 0.5, a, 0.5, b);
}
template <int N>
__device__ __forceinline__ DualV<N> fv_min(const DualV<N>& a, const DualV<N>& b) {
  if (a.v < b.v) return a;
  if (a.v > b.v) return b;
  return lin_comb(a.v, 0.5, a, 0.5, b);
}
template <int N>
__device__ __forceinline__ DualV<N> fv_sqrt(const DualV<N>& x) {
  const double r = sqrt(x.v);
  return scaled(r, 0.5 / r, x);
}
template <int N>
__device__ __forceinline__ DualV<N> fv_tanh(const DualV<N>& x) {
  const double t = tanh(x.v);
  return scaled(t, 1.0 - t * t, x);
}

// The off-wall SST closure of closure_cell and source rows of sst_rows as functions of (S, k,
// omega, grad k . grad omega), the same formulas: out = (F1, nu_t, k diffusivity, omega
// diffusivity, F2, k source, omega source), the sources as they enter the face sums.
template <class T>
__device__ __forceinline__ void sst_off_wall(T S, T k, T w, T dot_kw, double nu, double id,
                                             double id2, double V, T (&out)[7]) {
  const T kp = pos(k);
  const T iw = 1.0 / w;
  const T cd = fv_max((2.0 * SIGMA_W2) * dot_kw * iw, cst(CROSS_FLOOR, w));
  const T sk = safe_sqrt(kp);
  const T vt = ((500.0 * id2) * nu) * iw;
  const T c1 = sk * iw * (id / BETA_STAR);
  const T arg1 = fv_min(fv_max(c1, vt), (4.0 * SIGMA_W2 * id2) * kp / cd);
  const T a1sq = arg1 * arg1;
  const T F1 = fv_tanh(a1sq * a1sq);
  const T arg2 = fv_max(2.0 * c1, vt);
  const T F2 = fv_tanh(arg2 * arg2);
  const T nut = A1 * kp / fv_max(A1 * w, S * F2);
  out[0] = F1;
  out[1] = nut;
  out[2] = nu + (SIGMA_K2 + F1 * (SIGMA_K1 - SIGMA_K2)) * nut;
  out[3] = nu + (SIGMA_W2 + F1 * (SIGMA_W1 - SIGMA_W2)) * nut;
  out[4] = F2;
  const T limit = (PROD_RATIO * BETA_STAR) * kp * w;
  const T lim = fv_min(nut * (S * S), limit);
  out[5] = BETA_STAR * V * k * w - lim * V;
  const T alpha = ALPHA_2 + F1 * (ALPHA_1 - ALPHA_2);
  const T cap = limit / fv_max(nut, cst(NUT_FLOOR, nut));
  const T beta = BETA_2 + F1 * (BETA_1 - BETA_2);
  const T cross = (2.0 * SIGMA_W2) * (1.0 - F1) * dot_kw / w;
  out[6] = V * (beta * (w * w) - alpha * fv_min(S * S, cap) - cross);
}

// Coefficients per cell (LIN_NCOEF rows of nc): 2 / S (the strain rate's tangent is
// 2 / S sum_ij s_ij (grad u)'_ij, 0 where S = 0), then for each output of sst_off_wall its
// linear form in (k', omega', S', (grad k . grad omega)').
constexpr int LIN_NCOEF = 29;

// At a held linearisation: keep the closure fields (hcl, 7 rows of nc) and tabulate the off-wall
// cells' coefficients from the evaluation's state, gradients and closure fields.
template <int DIM>
__global__ void k_lin_closure_coef(MeshView m, CaseView cv, const double* state, const double* G,
                                   const double* cl, double nu, double* hcl, double* cc) {
  using L = Layout<DIM, true>;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const long nc = m.nc;
#pragma unroll
  for (int q = 0; q < 7; ++q) hcl[q * nc + c] = cl[q * nc + c];
  if (cv.wcell[c]) return;
  const GeoPlain gv{};
  const double S = cl[c];
  cc[c] = S > 0.0 ? 2.0 / S : 0.0;
  double dot = G[((long)L::K * DIM) * nc + c] * G[((long)L::W * DIM) * nc + c];
#pragma unroll
  for (int j = 1; j < DIM; ++j)
    dot += G[((long)L::K * DIM + j) * nc + c] * G[((long)L::W * DIM + j) * nc + c];
  DualV<4> in[4];
  const double v0[4] = {state[(long)L::K * nc + c], state[(long)L::W * nc + c], S, dot};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    in[a].v = v0[a];
#pragma unroll
    for (int i = 0; i < 4; ++i) in[a].d[i] = a == i ? 1.0 : 0.0;
  }
  DualV<4> out[7];
  sst_off_wall<DualV<4>>(in[2], in[0], in[1], in[3], nu, gv.inv_wd(cv, c), gv.inv_wd2(cv, c),
                         gv.vol(m, c), out);
#pragma unroll
  for (int q = 0; q < 7; ++q)
#pragma unroll
    for (int i = 0; i < 4; ++i) cc[(1L + 4 * q + i) * nc + c] = out[q].d[i];
}

// The closure stage of a Krylov product at the held linearisation: off the wall, the held fields
// with tangents from the tabulated forms, the omega gradient passed through, and the k / omega
// source tangents (src, 2 rows of nc) for k_sum_lin; wall cells by the dual-number closure.
template <int DIM>
__global__ void __launch_bounds__(128) k_closure_lin(MeshView m, CaseView cv, Src<Dual> st,
                                                     Par<Dual> par, const Dual* G,
                                                     const double* hcl, const double* cc, Dual* cl,
                                                     Dual* Gwi, double* src) {
  using L = Layout<DIM, true>;
  const int c = stage_cell<Dual>(m, cv);
  if (c >= m.nc) return;
  if (cv.wcell[c]) {
    k_closure_at<Dual, DIM>(c, m, cv, st, par, G, cl, Gwi);
    return;
  }
  const long nc = m.nc;
  double gv[DIM][DIM], gd[DIM][DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const Dual g = G[((long)i * DIM + j) * nc + c];
      gv[i][j] = g.v;
      gd[i][j] = g.d;
    }
  double ss = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) ss += (0.5 * (gv[i][j] + gv[j][i])) * gd[i][j];
  const double t[4] = {st.t ? st.t[(long)L::K * nc + c] : 0.0,
                       st.t ? st.t[(long)L::W * nc + c] : 0.0, cc[c] * ss, 0.0};
  double ddot = 0.0;
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    const Dual gk = G[((long)L::K * DIM + j) * nc + c], gw = G[((long)L::W * DIM + j) * nc + c];
    ddot += gk.d * gw.v + gk.v * gw.d;
    Gwi[(long)j * nc + c] = gw;
  }
  auto form = [&](int q) {
    const double* a = cc + (1L + 4 * q) * nc + c;
    return a[0] * t[0] + a[nc] * t[1] + a[2 * nc] * t[2] + a[3 * nc] * ddot;
  };
  cl[c] = Dual{hcl[c], t[2]};
  cl[nc + c] = Dual{hcl[nc + c], form(0)};
  cl[2 * nc + c] = Dual{hcl[2 * nc + c], form(1)};
  cl[3 * nc + c] = Dual{hcl[3 * nc + c], 0.0};  // the wall shear rate: 0 off the wall
  cl[4 * nc + c] = Dual{hcl[4 * nc + c], form(2)};
  cl[5 * nc + c] = Dual{hcl[5 * nc + c], form(3)};
  cl[6 * nc + c] = Dual{hcl[6 * nc + c], form(4)};
  src[c] = form(5);
  src[nc + c] = form(6);
}

// The face sums of a Krylov product at the held linearisation: tangents only (the product's
// output), the pin row, the k / omega source tangents of k_closure_lin off the wall and the
// dual-number source rows on it.
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_sum_lin(MeshView m, CaseView cv, Src<Dual> st,
                                                 Par<Dual> par, const Dual* FL, const Dual* cl,
                                                 const Dual* G, const Dual* Gwi,
                                                 const double* src, double* JV) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  const int c = stage_cell<Dual>(m, cv);
  if (c >= m.nc) return;
  const long nc = m.nc, nf = m.nf;
  double r[NF];
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      double x = FL[(long)q * nf + f].d;
      if (isnb) x = -x;
      r[q] = i == b ? x : r[q] + x;
    }
  }
  if (c == cv.pin) r[L::P] = st.t ? st.t[(long)L::P * nc + c] : 0.0;
  if constexpr (TURB) {
    if (cv.wcell[c]) {
      Dual rk{0.0, r[L::K]}, rw{0.0, r[L::W]};
      sst_rows<Dual, DIM>(m, cv, st, par, cl, G, Gwi, c, rk, rw);
      r[L::K] = rk.d;
      r[L::W] = rw.d;
    } else {
      r[L::K] += src[c];
      r[L::W] += src[nc + c];
    }
  }
#pragma unroll
  for (int q = 0; q < NF; ++q) JV[(long)q * nc + c] = r[q];
}

// Zero the tangent of n dual values (the "frozen" JVP holds gradients, closure and a_P fixed).
__global__ void k_freeze(long n, Dual* x) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i].d = 0.0;
}
template <class T>
void freeze(T*, long, cudaStream_t) {}
template <>
void freeze<Dual>(Dual* x, long n, cudaStream_t s) {
  k_freeze<<<fv_blocks(n, 256), 256, 0, s>>>(n, x);
}
__global__ void k_freeze_f(long n, DualF* x) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i].d = 0.0f;
}
template <>
void freeze<DualF>(DualF* x, long n, cudaStream_t s) {
  k_freeze_f<<<fv_blocks(n, 256), 256, 0, s>>>(n, x);
}

// Every field's gradient with the case's scheme, into w.G.
template <class T, int DIM, bool TURB>
void gradient_stage(FvCase* cs, Src<T> st, Par<T> par, const Work<T>& w, cudaStream_t s) {
  const MeshView& m = cs->mesh->view;
  const CaseView& cv = cs->view;
  constexpr int NF = Layout<DIM, TURB>::NFLD;
  const int TB = cs->tbs[0];
  const int bc = fv_blocks(m.nc, TB);
  const int sweeps = cs->desc.gradient_sweeps;
  const double rel = sweeps >= 1 ? cs->desc.gradient_relaxation : 1.0;
  if (sweeps <= 1) {
    k_grad<T, DIM, TURB><<<bc, TB, 0, s>>>(m, cv, st, par, w.G, nullptr, rel);
    return;
  }
  T* x0 = ((sweeps - 1) % 2 == 0) ? w.G : w.Galt;
  T* x1 = x0 == w.G ? w.Galt : w.G;
  k_grad<T, DIM, TURB><<<bc, TB, 0, s>>>(m, cv, st, par, x0, w.Bg, rel);
  gg_sweeps<T, DIM, NF>(m, sweeps, rel, w.Bg, x0, x1, w.FL, s);
}

template <class T, int DIM, bool TURB>
int run(FvCase* cs, Src<T> st, Par<T> par, double* R, double* JV, cudaStream_t s,
        bool frozen = false, bool end_profile_run = true, double* aux = nullptr) {
  const MeshView& m = cs->mesh->view;
  const CaseView& cv = cs->view;
  const long nc = m.nc, nf = m.nf;
  cs->fwd_valid = 0;  // the workspace is about to hold this pass
  Work<T> w = work_layout<T, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
  // each stage at its own block size (the index is the stage's profiling mark)
  const int* tb = cs->tbs;
  auto bc = [&](int k) { return fv_blocks(nc, tb[k]); };
  auto bf = [&](int k) { return fv_blocks(nf, tb[k]); };
  // a held linearisation (a state-tangent dual-number pass, first-order upwind): the linear
  // compact gradients and the interior faces' coefficient and flux stages take their primal
  // values from it and compute only tangents
  bool lin = false;
  if constexpr (std::is_same<T, Dual>::value) lin = cs->lin_use && !frozen && !psi_count<DIM, TURB>(cs);
  // ... and the closure and face-sum stages from its tabulated closure forms (the product only:
  // fv_jvp_linearised returns the residual the linearisation held)
  const bool lin_sum = lin && R == nullptr && (!TURB || cs->lin_cc != nullptr);
  fv_prof_mark(cs, 0, s);
  if constexpr (std::is_same<T, Dual>::value) {
    if (lin && cs->desc.gradient_sweeps == 0)  // the compact scheme (no relaxation factor)
      k_grad_tangent<DIM, TURB><<<bc(0), tb[0], 0, s>>>(m, cv, st, par, cs->lin_g, w.G);
    else
      gradient_stage<T, DIM, TURB>(cs, st, par, w, s);
  } else {
    gradient_stage<T, DIM, TURB>(cs, st, par, w, s);
  }
  fv_prof_mark(cs, 1, s);
  if (TURB) {
    bool done = false;
    if constexpr (std::is_same<T, Dual>::value) {
      if (lin_sum) {
        k_closure_lin<DIM><<<bc(1), tb[1], 0, s>>>(m, cv, st, par, w.G, cs->lin_cl, cs->lin_cc,
                                                   w.cl, w.Gwi, cs->lin_src);
        done = true;
      }
    }
    if (!done) k_closure<T, DIM><<<bc(1), tb[1], 0, s>>>(m, cv, st, par, w.G, w.cl, w.Gwi);
  }
  fv_prof_mark(cs, 2, s);
  if constexpr (std::is_same<T, Dual>::value) {
    if (lin) {
      if (m.nfi > 0)
        k_apcoef_tangent<DIM, TURB><<<fv_blocks(m.nfi, tb[2]), tb[2], 0, s>>>(
            m, cv, st, w.G, w.cl, cs->lin_aux, cs->lin_ac, w.acown, w.acnb, w.me);
      if (nf > m.nfi)
        k_apcoef<T, DIM, TURB><<<fv_blocks(nf - m.nfi, tb[2]), tb[2], 0, s>>>(
            m, cv, st, par, w.G, w.cl, w.acown, w.acnb, w.me, m.nfi);
    } else {
      k_apcoef<T, DIM, TURB><<<bf(2), tb[2], 0, s>>>(m, cv, st, par, w.G, w.cl, w.acown, w.acnb,
                                                     w.me);
    }
  } else {
    k_apcoef<T, DIM, TURB><<<bf(2), tb[2], 0, s>>>(m, cv, st, par, w.G, w.cl, w.acown, w.acnb,
                                                   w.me);
  }
  fv_prof_mark(cs, 3, s);
  k_dcoeff<T><<<bc(3), tb[3], 0, s>>>(m, w.acown, w.acnb, w.dco);
  const long npsi = psi_count<DIM, TURB>(cs);
  if (npsi)
    k_limiter<T, DIM, TURB><<<bc(3), tb[3], 0, s>>>(m, st, w.G, cv.lim_km, cv.lim_ks, w.psi);
  // G, closure, Gwi, a_P, d and the slope limiters
  if (frozen) freeze<T>(w.G, (long)(w.psi + npsi - w.G), s);
  fv_prof_mark(cs, 4, s);
  bool flux_done = false;
  if constexpr (std::is_same<T, Dual>::value) {
    if (lin) {
      // a held linearisation: the interior faces' tangent fluxes from its kept intermediates, the
      // boundary faces by the full dual-number flux
      if (m.nfi > 0)
        k_flux_tangent<DIM, TURB><<<fv_blocks(m.nfi, tb[4]), tb[4], 0, s>>>(
            m, cv, st, w.G, w.cl, w.dco, w.me, cs->lin_aux, cs->lin_fl, w.FL);
      if (nf > m.nfi)
        k_flux<T, DIM, TURB><<<fv_blocks(nf - m.nfi, tb[4]), tb[4], 0, s>>>(
            m, cv, st, par, w.G, w.cl, w.dco, w.me, nullptr, false, w.FL, nullptr, m.nfi);
      flux_done = true;
    }
  }
  if (!flux_done)
    k_flux<T, DIM, TURB><<<bf(4), tb[4], 0, s>>>(m, cv, st, par, w.G, w.cl, w.dco, w.me,
                                                 npsi ? w.psi : nullptr, frozen, w.FL, aux);
  fv_prof_mark(cs, 5, s);
  bool summed = false;
  if constexpr (std::is_same<T, Dual>::value) {
    if (lin_sum) {
      k_sum_lin<DIM, TURB><<<bc(5), tb[5], 0, s>>>(m, cv, st, par, w.FL, w.cl, w.G, w.Gwi,
                                                   cs->lin_src, JV);
      summed = true;
    }
  }
  if (!summed)
    k_sum<T, DIM, TURB><<<bc(5), tb[5], 0, s>>>(m, cv, st, par, w.FL, w.cl, w.G, w.Gwi, R, JV);
  fv_prof_mark(cs, 6, s);
  if (end_profile_run) fv_prof_end_run(cs);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

template <int DIM, bool TURB>
int dispatch_t(FvCase* cs, const double* state, const double* tangent, int kind, double* R,
               double* JV, cudaStream_t s) {
  const double irho = 1.0 / cs->desc.rho;
  if (kind == FV_TAN_NONE) {
    return run<double, DIM, TURB>(
        cs, Src<double>{state}, Par<double>{cs->mu, cs->inlet_scale, cs->mu * irho}, R, nullptr, s);
  }
  if (kind == FV_TAN_STATE32 || kind == FV_TAN_FROZEN32) {
    constexpr int NF = Layout<DIM, TURB>::NFLD;
    const long n = (long)NF * cs->mesh->nc;
    int rc = fv_case_ensure_f32(cs, s);
    if (rc == FV_OK) rc = fv_d2f(n, state, cs->f_state, s);
    if (rc == FV_OK && tangent) rc = fv_d2f(n, tangent, cs->f_tangent, s);
    if (rc != FV_OK) return rc;
    Par<DualF> pf{{(float)cs->mu, 0.0f}, {(float)cs->inlet_scale, 0.0f},
                  {(float)(cs->mu * irho), 0.0f}};
    return run<DualF, DIM, TURB>(cs, Src<DualF>{cs->f_state, tangent ? cs->f_tangent : nullptr},
                                 pf, R, JV, s, kind == FV_TAN_FROZEN32);
  }
  const double dmu = kind == FV_TAN_MU ? 1.0 : 0.0;
  Par<Dual> par{{cs->mu, dmu}, {cs->inlet_scale, kind == FV_TAN_INLET ? 1.0 : 0.0},
                {cs->mu * irho, dmu * irho}};
  Src<Dual> st{state, (kind == FV_TAN_STATE || kind == FV_TAN_FROZEN) ? tangent : nullptr};
  return run<Dual, DIM, TURB>(cs, st, par, R, JV, s, kind == FV_TAN_FROZEN);
}

#include "adjoint.inc.cuh"
#include "assemble.inc.cuh"

template <int DIM, bool TURB>
AdjWork adj_layout(FvCase* cs) {
  using L = Layout<DIM, TURB>;
  const long nc = cs->mesh->view.nc;
  AdjWork aw;
  double* p = cs->adj;
  aw.Wt = p; p += L::NFLD * nc;
  aw.sb = p; p += L::NFLD * nc;
  aw.Gb = p; p += L::NFLD * DIM * nc;
  aw.dcob = p; p += nc;
  aw.clb = p; p += 4 * nc;
  aw.Gwib = p; p += DIM * nc;
  aw.Gb2 = p; p += L::NFLD * DIM * nc;  // present when the case is swept
  aw.Bb = p;
  aw.FLx = cs->flx_active ? cs->flx : nullptr;
  p += L::NFLD * DIM * nc;  // Bb
  constexpr int NA = n_advected<DIM, TURB>();
  aw.psi = nullptr;
  aw.psib = p; p += (long)NA * nc;
  aw.lnb = p;
  return aw;
}

// ---------------------------------------------------------------- one persistent launch
// The whole residual + VJP evaluation of a case with compact gradients and first-order upwind
// advection as ONE cooperative launch: the stages of run<double> and of the adjoint in order, each
// over its cells or faces, separated by grid-wide barriers (cooperative_groups grid sync; the
// cooperative launch guarantees every block is resident).  Each thread takes `chunk` consecutive
// cells / faces per step of a grid-stride loop.  Every cell or face is computed by the same body
// as in the stage-per-launch path, so the result is bitwise the same.
struct PersistentVjp {
  Work<double> w;
  AdjWork aw;
  const double* W;
  double* aux;
  double* R;
  double* out;
  double rel;
  int chunk;
};

template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_persistent_vjp(MeshView m, CaseView cv, Src<double> st,
                                                        Par<double> par, PersistentVjp a) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  const long nthr = (long)gridDim.x * blockDim.x;
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int chunk = a.chunk;
  auto each = [&](long n, auto&& fn) {
    for (long base = tid * chunk; base < n; base += nthr * chunk)
      for (int k = 0; k < chunk && base + k < n; ++k) fn((int)(base + k));
  };
  const Work<double>& w = a.w;
  const AdjWork& aw = a.aw;
  each(m.nc, [&](int c) { k_grad_at<double, DIM, TURB>(c, m, cv, st, par, w.G, nullptr, a.rel); });
  grid.sync();
  if constexpr (TURB) {
    each(m.nc, [&](int c) { k_closure_at<double, DIM>(c, m, cv, st, par, w.G, w.cl, w.Gwi); });
    grid.sync();
  }
  each(m.nf, [&](int f) {
    k_apcoef_at<double, DIM, TURB>(f, m, cv, st, par, w.G, w.cl, w.acown, w.acnb, w.me);
  });
  grid.sync();
  each(m.nc, [&](int c) { k_dcoeff_at<double>(c, m, w.acown, w.acnb, w.dco); });
  grid.sync();
  each(m.nf, [&](int f) {
    k_flux_at<double, DIM, TURB>(f, m, cv, st, par, w.G, w.cl, w.dco, w.me, nullptr, false, w.FL,
                                 a.aux);
  });
  grid.sync();
  each(m.nc, [&](int c) {
    k_sum_at<double, DIM, TURB>(c, m, cv, st, par, w.FL, w.cl, w.G, w.Gwi, a.R, nullptr);
  });
  grid.sync();
  each(m.nc, [&](int c) { a_sum_at<DIM, TURB>(c, m, cv, st, par, a.W, w.cl, w.G, w.Gwi, aw); });
  grid.sync();
  each(m.nc, [&](int c) {
    a_flux_at<DIM, TURB>(c, m, cv, st, par, w.G, w.cl, w.dco, w.me, a.aux, aw);
  });
  grid.sync();
  each(m.nc, [&](int c) {
    a_apcoef_at<DIM, TURB>(c, m, cv, st, par, w.G, w.cl, w.dco, w.me, a.aux, aw);
  });
  grid.sync();
  if constexpr (TURB) {
    each(m.nc, [&](int c) { a_closure_at<DIM>(c, m, cv, st, par, w.G, w.cl, aw); });
    grid.sync();
  }
  each(m.nf, [&](int f) { a_grad_face_at<DIM, TURB>(f, m, cv, aw, aw.Gb, nullptr, a.rel, w.FL); });
  grid.sync();
  each(m.nc, [&](int c) { a_grad_at<DIM, TURB>(c, m, cv, aw, w.FL, a.out); });
}

// Whether the case's schemes are those the persistent kernel runs.
bool persistent_supported(const FvCase* cs) {
  return cs->desc.gradient_sweeps <= 1 && !cs->view.rec_mom && !cs->view.rec_sca &&
         !cs->flx_active;
}

template <int DIM, bool TURB>
int run_vjp_persistent(FvCase* cs, const double* state, const double* W, double* R, double* out,
                       cudaStream_t s) {
  const MeshView& m = cs->mesh->view;
  const long nc = m.nc, nf = m.nf;
  PersistentVjp a;
  a.w = work_layout<double, DIM, TURB>(cs->work, nc, nf, 0);
  a.aw = adj_layout<DIM, TURB>(cs);
  a.W = W;
  a.aux = cs->aux;
  a.R = R ? R : cs->tmp;
  a.out = out;
  a.rel = cs->desc.gradient_sweeps >= 1 ? cs->desc.gradient_relaxation : 1.0;
  a.chunk = cs->pchunk;
  Src<double> st{state};
  Par<double> par{cs->mu, cs->inlet_scale, cs->mu / cs->desc.rho};
  const MeshView mv = m;
  const CaseView cv = cs->view;
  auto kern = k_persistent_vjp<DIM, TURB>;
  int dev = 0, sms = 0, per_sm = 0;
  FV_CUDA_TRY(cudaGetDevice(&dev));
  FV_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  FV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, cs->pblock, 0));
  if (per_sm < 1) {
    fv_set_error("persistent residual + VJP: no block of %d threads fits on an SM", cs->pblock);
    return FV_ERR_ARG;
  }
  void* args[] = {(void*)&mv, (void*)&cv, (void*)&st, (void*)&par, (void*)&a};
  FV_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)kern, dim3(per_sm * sms),
                                          dim3(cs->pblock), args, 0, s));
  return FV_OK;
}

// gb_save (optional, (NF, DIM, nc)): receives the gradient cotangent before the corrected
// scheme's backward sweeps overwrite it (the mesh-coordinate adjoint re-runs them).
template <int DIM, bool TURB>
int run_vjp(FvCase* cs, const double* state, const double* W, double* R, double* out,
            cudaStream_t s, double* gb_save = nullptr, bool held = false) {
  if (held) {
    if (!cs->fwd_valid) {
      fv_set_error("fv_vjp_held: no forward pass held; call fv_hold_forward at this state (again "
                   "after any other evaluation or a parameter, viscosity-field, wall-distance or "
                   "geometry change)");
      return FV_ERR_ARG;
    }
  } else if (cs->persistent && !gb_save && persistent_supported(cs)) {
    cs->fwd_valid = 0;
    return run_vjp_persistent<DIM, TURB>(cs, state, W, R, out, s);
  }
  using L = Layout<DIM, TURB>;
  const MeshView& m = cs->mesh->view;
  const CaseView& cv = cs->view;
  const long nc = m.nc, nf = m.nf;
  Src<double> st{state};
  Par<double> par{cs->mu, cs->inlet_scale, cs->mu / cs->desc.rho};
  if (held) {
    // the forward stages' profiling marks at one instant: they took no time in this call
    for (int k = 0; k <= 6; ++k) fv_prof_mark(cs, k, s);
  } else {
    int rc = run<double, DIM, TURB>(cs, st, par, R ? R : cs->tmp, nullptr, s, false, false,
                                    cs->aux);
    if (rc != FV_OK) return rc;
    cs->fwd_valid = 1;  // the adjoint stages below read but do not change it
  }
  // forward workspace (double layout, as written by run<double>)
  Work<double> fw = work_layout<double, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
  double* G = fw.G;
  double* cl = fw.cl;
  double* Gwi = fw.Gwi;
  double* dco = fw.dco;
  AdjWork aw = adj_layout<DIM, TURB>(cs);
  const int* tb = cs->tbs;  // each stage at its own block size (its profiling mark's index)
  auto bc = [&](int k) { return fv_blocks(nc, tb[k]); };
  a_sum<DIM, TURB><<<bc(6), tb[6], 0, s>>>(m, cv, st, par, W, cl, G, Gwi, aw);
  fv_prof_mark(cs, 7, s);
  const bool lim = psi_count<DIM, TURB>(cs) > 0;
  if (lim) aw.psi = fw.psi;
  if (aw.FLx && lim)
    a_flux<DIM, TURB, true, true><<<bc(7), tb[7], 0, s>>>(m, cv, st, par, G, cl, dco, fw.me,
                                                          cs->aux, aw);
  else if (aw.FLx)
    a_flux<DIM, TURB, true><<<bc(7), tb[7], 0, s>>>(m, cv, st, par, G, cl, dco, fw.me, cs->aux,
                                                    aw);
  else if (lim)
    a_flux<DIM, TURB, false, true><<<bc(7), tb[7], 0, s>>>(m, cv, st, par, G, cl, dco, fw.me,
                                                           cs->aux, aw);
  else
    a_flux<DIM, TURB><<<bc(7), tb[7], 0, s>>>(m, cv, st, par, G, cl, dco, fw.me, cs->aux, aw);
  if (lim && (cv.lim_km > 0.0 || cv.lim_ks > 0.0)) {
    a_limiter<DIM, TURB><<<bc(7), tb[7], 0, s>>>(m, st, G, cv.lim_km, cv.lim_ks, aw);
    a_limiter_gather<DIM, TURB><<<bc(7), tb[7], 0, s>>>(m, aw);
  }
  fv_prof_mark(cs, 8, s);
  a_apcoef<DIM, TURB><<<bc(8), tb[8], 0, s>>>(m, cv, st, par, G, cl, dco, fw.me, cs->aux, aw);
  fv_prof_mark(cs, 9, s);
  if (TURB) a_closure<DIM><<<bc(9), tb[9], 0, s>>>(m, cv, st, par, G, cl, aw);
  fv_prof_mark(cs, 10, s);
  const int sweeps = cs->desc.gradient_sweeps;
  const double rel = sweeps >= 1 ? cs->desc.gradient_relaxation : 1.0;
  const double* gb0 = aw.Gb;
  if (gb_save)
    FV_CUDA_TRY(cudaMemcpyAsync(gb_save, aw.Gb, sizeof(double) * L::NFLD * DIM * nc,
                                cudaMemcpyDeviceToDevice, s));
  if (sweeps >= 2) gb0 = gg_sweeps_adjoint<DIM, L::NFLD>(m, sweeps, rel, aw, fw.FL, s);
  a_grad_face<DIM, TURB><<<fv_blocks(nf, tb[10]), tb[10], 0, s>>>(m, cv, aw, gb0,
                                                                 sweeps >= 2 ? aw.Bb : nullptr,
                                                                 rel, fw.FL);
  a_grad<DIM, TURB><<<bc(10), tb[10], 0, s>>>(m, cv, aw, fw.FL, out);
  fv_prof_mark(cs, 11, s);
  fv_prof_end_run(cs);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

bool g_const_ready = false;

}  // namespace

#include "node_adjoint.inc.cuh"

size_t fv_adjoint_work_bytes(int dim, int turb, long nc, long nf, int sweeps, int advection) {
  long nfld = dim + 1 + (turb ? 2 : 0);
  long n = 2 * nfld * nc + nfld * dim * nc + nc + 4 * nc + dim * nc;
  // the sweeps' second iterate cotangent and B phi's (the limiter buffers follow them)
  if (sweeps >= 1 || advection >= 1) n += 2 * nfld * dim * nc;
  if (advection >= 1) n += (long)(dim + (turb ? 2 : 0)) * (nc + 2 * nf);
  return sizeof(double) * (size_t)n;
}

size_t fv_aux_bytes(int dim, int turb, long nf) {
  return sizeof(double) * (size_t)(6 + dim + (turb ? 8 : 0)) * nf;
}

int fv_case_vjp_run(FvCase* cs, const double* state, const double* W, double* R, double* out,
                    cudaStream_t s) {
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2)
    return turb ? run_vjp<2, true>(cs, state, W, R, out, s) : run_vjp<2, false>(cs, state, W, R, out, s);
  return turb ? run_vjp<3, true>(cs, state, W, R, out, s) : run_vjp<3, false>(cs, state, W, R, out, s);
}

namespace {
template <int DIM, bool TURB>
int hold_forward(FvCase* cs, const double* state, double* R, cudaStream_t s) {
  Par<double> par{cs->mu, cs->inlet_scale, cs->mu / cs->desc.rho};
  int rc = run<double, DIM, TURB>(cs, Src<double>{state}, par, R ? R : cs->tmp, nullptr, s, false,
                                  true, cs->aux);
  if (rc == FV_OK) cs->fwd_valid = 1;
  return rc;
}
}  // namespace

int fv_case_hold_forward(FvCase* cs, const double* state, double* R, cudaStream_t s) {
  if (cs->wd_missing) {
    fv_set_error("turbulent case without SST wall faces: set its wall distance first "
                 "(fv_case_set_wall_distance)");
    return FV_ERR_ARG;
  }
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2) return turb ? hold_forward<2, true>(cs, state, R, s) : hold_forward<2, false>(cs, state, R, s);
  return turb ? hold_forward<3, true>(cs, state, R, s) : hold_forward<3, false>(cs, state, R, s);
}

int fv_case_vjp_held(FvCase* cs, const double* state, const double* W, double* out,
                     cudaStream_t s) {
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2)
    return turb ? run_vjp<2, true>(cs, state, W, nullptr, out, s, nullptr, true)
                : run_vjp<2, false>(cs, state, W, nullptr, out, s, nullptr, true);
  return turb ? run_vjp<3, true>(cs, state, W, nullptr, out, s, nullptr, true)
              : run_vjp<3, false>(cs, state, W, nullptr, out, s, nullptr, true);
}

namespace {
template <int DIM, bool TURB>
int linearise(FvCase* cs, const double* state, double* R, cudaStream_t s) {
  const long nc = cs->mesh->nc, nf = cs->mesh->nf;
  constexpr int NF = Layout<DIM, TURB>::NFLD;
  if (psi_count<DIM, TURB>(cs) > 0) {
    fv_set_error("fv_case_linearise: the linearised JVP covers first-order upwind advection only");
    return FV_ERR_ARG;
  }
  if (!cs->lin_aux) FV_CUDA_TRY(cudaMalloc(&cs->lin_aux, fv_aux_bytes(DIM, TURB, nf)));
  if (!cs->lin_fl) FV_CUDA_TRY(cudaMalloc(&cs->lin_fl, sizeof(double) * NF * nf));
  if (!cs->lin_ac) FV_CUDA_TRY(cudaMalloc(&cs->lin_ac, sizeof(double) * 3 * nf));
  if (!cs->lin_g) FV_CUDA_TRY(cudaMalloc(&cs->lin_g, sizeof(double) * NF * DIM * nc));
  cs->lin_valid = 0;
  const double irho = 1.0 / cs->desc.rho;
  int rc = run<double, DIM, TURB>(cs, Src<double>{state},
                                  Par<double>{cs->mu, cs->inlet_scale, cs->mu * irho}, R, nullptr,
                                  s, false, true, cs->lin_aux);
  if (rc != FV_OK) return rc;
  Work<double> w = work_layout<double, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
  FV_CUDA_TRY(cudaMemcpyAsync(cs->lin_fl, w.FL, sizeof(double) * NF * nf,
                              cudaMemcpyDeviceToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(cs->lin_ac, w.acown, sizeof(double) * nf, cudaMemcpyDeviceToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(cs->lin_ac + nf, w.acnb, sizeof(double) * nf,
                              cudaMemcpyDeviceToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(cs->lin_ac + 2 * nf, w.me, sizeof(double) * nf,
                              cudaMemcpyDeviceToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(cs->lin_g, w.G, sizeof(double) * NF * DIM * nc,
                              cudaMemcpyDeviceToDevice, s));
  if (!cs->lin_r) FV_CUDA_TRY(cudaMalloc(&cs->lin_r, sizeof(double) * NF * nc));
  FV_CUDA_TRY(cudaMemcpyAsync(cs->lin_r, R, sizeof(double) * NF * nc, cudaMemcpyDeviceToDevice, s));
  if constexpr (TURB) {
    if (!cs->lin_cl) FV_CUDA_TRY(cudaMalloc(&cs->lin_cl, sizeof(double) * 7 * nc));
    if (!cs->lin_cc) FV_CUDA_TRY(cudaMalloc(&cs->lin_cc, sizeof(double) * LIN_NCOEF * nc));
    if (!cs->lin_src) FV_CUDA_TRY(cudaMalloc(&cs->lin_src, sizeof(double) * 2 * nc));
    k_lin_closure_coef<DIM><<<fv_blocks(nc, 128), 128, 0, s>>>(
        cs->mesh->view, cs->view, state, w.G, w.cl, cs->mu * irho, cs->lin_cl, cs->lin_cc);
    FV_CUDA_TRY(cudaGetLastError());
  }
  cs->lin_valid = 1;
  return FV_OK;
}
}  // namespace

int fv_case_linearise(FvCase* cs, const double* state, double* R, cudaStream_t s) {
  if (cs->wd_missing) {
    fv_set_error("turbulent case without SST wall faces: set its wall distance first "
                 "(fv_case_set_wall_distance)");
    return FV_ERR_ARG;
  }
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2) return turb ? linearise<2, true>(cs, state, R, s) : linearise<2, false>(cs, state, R, s);
  return turb ? linearise<3, true>(cs, state, R, s) : linearise<3, false>(cs, state, R, s);
}

size_t fv_residual_work_bytes(int dim, int turb, long nc, long nf, int sweeps, int advection) {
  long nfld = dim + 1 + (turb ? 2 : 0);
  long n = nfld * dim * nc + 7 * nc + dim * nc + 3 * nf + nc + nfld * nf;
  if (advection >= 1) n += (long)(dim + (turb ? 2 : 0)) * nc;  // slope limiters
  if (sweeps >= 2) n += 2 * nfld * dim * nc;  // B phi and the second sweep iterate
  return (size_t)n * sizeof(Dual);
}

size_t fv_jac_face_bytes(int dim, int turb, long nf) {
  long nfld = dim + 1 + (turb ? 2 : 0);
  return sizeof(double) * (size_t)(2 * nfld * nfld) * nf;
}

int fv_case_assemble_frozen(FvCase* cs, const double* state, const int* indptr,
                            const int* indices, void* values, void* D, int fp32,
                            cudaStream_t s) {
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  auto go = [&](auto t) {
    using T = decltype(t);
    GS<T>* v = (GS<T>*)values;
    GS<T>* d = (GS<T>*)D;
    if (dim == 2)
      return turb ? assemble_frozen<T, 2, true>(cs, state, indptr, indices, v, d, s)
                  : assemble_frozen<T, 2, false>(cs, state, indptr, indices, v, d, s);
    return turb ? assemble_frozen<T, 3, true>(cs, state, indptr, indices, v, d, s)
                : assemble_frozen<T, 3, false>(cs, state, indptr, indices, v, d, s);
  };
  return fp32 ? go(DualF{}) : go(Dual{});
}

int fv_gg_sweeps_scalar(const MeshView& m, int sweeps, double rel, const double* num, double* x0,
                        double* x1, double* wface, cudaStream_t s) {
  if (m.dim == 2)
    gg_sweeps<double, 2, 1>(m, sweeps, rel, num, x0, x1, wface, s);
  else
    gg_sweeps<double, 3, 1>(m, sweeps, rel, num, x0, x1, wface, s);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

int fv_residual_init_constants() {
  if (g_const_ready) return FV_OK;
  SstConst h;
  h.bs4 = pow(BETA_STAR, 0.25);
  double y = 11.0;
  for (int i = 0; i < 10; ++i) y = log(E_WALL * y) / KAPPA;
  h.ylam = y;
  FV_CUDA_TRY(cudaMemcpyToSymbol(c_sst, &h, sizeof(h)));
  g_const_ready = true;
  return FV_OK;
}

int fv_case_ensure_f32(FvCase* c, cudaStream_t s) {
  FvMesh* m = c->mesh;
  int rc = fv_mesh_ensure_f32(m, s);
  if (rc != FV_OK) return rc;
  const long nc = m->nc, dim = m->dim;
  if (!c->f32) {
    // wd (nc), wdg (dim nc), 1/wd and 1/wd^2 (2 nc), per-cell viscosity (nc)
    FV_CUDA_TRY(cudaMalloc(&c->f32, sizeof(float) * (size_t)(nc * (4 + dim))));
    FV_CUDA_TRY(cudaMalloc(&c->f_state, sizeof(float) * (size_t)c->nfld * nc));
    FV_CUDA_TRY(cudaMalloc(&c->f_tangent, sizeof(float) * (size_t)c->nfld * nc));
    float* p = c->f32;
    if ((rc = fv_d2f(nc, c->wd, p, s)) != FV_OK) return rc;
    if ((rc = fv_d2f(dim * nc, c->wdg, p + nc, s)) != FV_OK) return rc;
    if ((rc = fv_d2f(2 * nc, c->inv_wd, p + (1 + dim) * nc, s)) != FV_OK) return rc;
    CaseView& v = c->view;
    v.f_wd = p;
    v.f_wdg = p + nc;
    v.f_inv_wd = p + (1 + dim) * nc;
    v.f_inv_wd2 = p + (2 + dim) * nc;
    v.f_rho = (float)c->desc.rho;
  }
  if (c->mu_cell) {  // the per-cell viscosity can change between calls
    if ((rc = fv_d2f(nc, c->mu_cell, c->f32 + (3 + dim) * nc, s)) != FV_OK) return rc;
    c->view.f_mu_cell = c->f32 + (3 + dim) * nc;
  }
  return FV_OK;
}

// nu_t of a (physical) state: one residual evaluation, then the closure's eddy-viscosity row.
int fv_case_eddy_viscosity(FvCase* cs, const double* state, double* nut, cudaStream_t s) {
  const int dim = cs->mesh->dim;
  const long nc = cs->mesh->nc, nf = cs->mesh->nf;
  int rc = fv_case_run(cs, state, nullptr, FV_TAN_NONE, cs->tmp, nullptr, s);
  if (rc != FV_OK) return rc;
  const double* cl = dim == 2 ? work_layout<double, 2, true>(cs->work, nc, nf, psi_count<2, true>(cs)).cl
                              : work_layout<double, 3, true>(cs->work, nc, nf, psi_count<3, true>(cs)).cl;
  FV_CUDA_TRY(cudaMemcpyAsync(nut, cl + 2 * nc, sizeof(double) * nc, cudaMemcpyDeviceToDevice, s));
  return FV_OK;
}

int fv_case_run(FvCase* cs, const double* state, const double* tangent, int kind, double* R,
                double* JV, cudaStream_t s) {
  if (cs->wd_missing) {
    fv_set_error("turbulent case without SST wall faces: set its wall distance first "
                 "(fv_case_set_wall_distance)");
    return FV_ERR_ARG;
  }
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2) {
    return turb ? dispatch_t<2, true>(cs, state, tangent, kind, R, JV, s)
                : dispatch_t<2, false>(cs, state, tangent, kind, R, JV, s);
  }
  return turb ? dispatch_t<3, true>(cs, state, tangent, kind, R, JV, s)
              : dispatch_t<3, false>(cs, state, tangent, kind, R, JV, s);
}
