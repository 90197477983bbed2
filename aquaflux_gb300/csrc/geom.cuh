// Mesh geometry formulas as templates over the scalar type: T = double is the geometry pipeline
// (mesh.cu), T = Dual differentiates the same arithmetic for the mesh-coordinate adjoint.
//
//   face_geom     2D edge (aquaflux/mesh/face.py:217-230) / 3D centre fan (face.py:292-349):
//                 area, unit normal (unoriented), centroid of one face from its nodes
//   cell_geom     recentred divergence-theorem volume and centroid (aquaflux/mesh/cell.py:124-170)
//                 about the mean of the face centroids (cell.py:84-108)
//   face_factors  the per-face interpolation / distance factors (aquaflux/flow/momentum.py:266-279,
//                 aquaflux/schemes/interpolation.py:27-176, aquaflux/discretization/diffusion.py)
#pragma once

#include "common.cuh"

FV_HD double gsqrt(double x) { return sqrt(x); }
FV_HD Dual gsqrt(Dual x) {
  const double s = sqrt(x.v);
  return {s, 0.5 * x.d / s};
}

// P(i, j): coordinate j of the face's i-th node (perimeter order), k nodes.
template <class T, int DIM, class NodeFn>
__device__ __forceinline__ void face_geom(int k, const NodeFn& P, T& area, T* n, T* xf) {
  if constexpr (DIM == 2) {
    const T dx = P(1, 0) - P(0, 0), dy = P(1, 1) - P(0, 1);
    const T sq = dx * dx + dy * dy;
    const bool pos = val(sq) > 0.0;
    const T a = pos ? gsqrt(sq) : cst(0.0, sq);
    area = a;
    xf[0] = 0.5 * (P(0, 0) + P(1, 0));
    xf[1] = 0.5 * (P(0, 1) + P(1, 1));
    n[0] = pos ? dy / a : cst(0.0, sq);
    n[1] = pos ? -dx / a : cst(0.0, sq);
  } else {
    T pa[3];
    for (int j = 0; j < 3; ++j) pa[j] = cst(0.0, P(0, 0));
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < 3; ++j) pa[j] += P(i, j);
    const double inv = 1.0 / (double)k;
    for (int j = 0; j < 3; ++j) pa[j] = pa[j] * inv;
    T S[3];
    for (int j = 0; j < 3; ++j) S[j] = cst(0.0, pa[0]);
    for (int i = 0; i < k; ++i) {
      const int i1 = (i + 1) % k;
      const T u0 = P(i, 0) - pa[0], u1 = P(i, 1) - pa[1], u2 = P(i, 2) - pa[2];
      const T v0 = P(i1, 0) - pa[0], v1 = P(i1, 1) - pa[1], v2 = P(i1, 2) - pa[2];
      S[0] += 0.5 * (u1 * v2 - u2 * v1);
      S[1] += 0.5 * (u2 * v0 - u0 * v2);
      S[2] += 0.5 * (u0 * v1 - u1 * v0);
    }
    const T sq = S[0] * S[0] + S[1] * S[1] + S[2] * S[2];
    const bool pos = val(sq) > 0.0;
    const T a = pos ? gsqrt(sq) : cst(0.0, sq);
    for (int j = 0; j < 3; ++j) n[j] = pos ? S[j] / a : cst(0.0, sq);
    T c[3];
    for (int j = 0; j < 3; ++j) c[j] = cst(0.0, sq);
    for (int i = 0; i < k; ++i) {
      const int i1 = (i + 1) % k;
      const T u0 = P(i, 0) - pa[0], u1 = P(i, 1) - pa[1], u2 = P(i, 2) - pa[2];
      const T v0 = P(i1, 0) - pa[0], v1 = P(i1, 1) - pa[1], v2 = P(i1, 2) - pa[2];
      const T d0 = 0.5 * (u1 * v2 - u2 * v1);
      const T d1 = 0.5 * (u2 * v0 - u0 * v2);
      const T d2 = 0.5 * (u0 * v1 - u1 * v0);
      const T w = d0 * n[0] + d1 * n[1] + d2 * n[2];
      for (int j = 0; j < 3; ++j) c[j] += w * ((pa[j] + P(i, j) + P(i1, j)) / 3.0);
    }
    const T sa = val(a) > 0.0 ? a : cst(1.0, a);
    area = a;
    for (int j = 0; j < 3; ++j) xf[j] = c[j] / sa;
  }
}

// F(i, A, n, xf, nb): the i-th of the cell's nf faces (ascending), nb = the cell is its neighbour.
template <class T, int DIM, class FaceFn>
__device__ __forceinline__ void cell_geom(int nfaces, const FaceFn& F, T& vol, T* xc) {
  T a[DIM], cs[DIM];
  T A, n[DIM], x[DIM];
  bool isnb;
  F(0, A, n, x, isnb);
  for (int j = 0; j < DIM; ++j) {
    a[j] = cst(0.0, A);
    cs[j] = cst(0.0, A);
  }
  for (int i = 0; i < nfaces; ++i) {
    F(i, A, n, x, isnb);
    for (int j = 0; j < DIM; ++j) a[j] += x[j];
  }
  const double inv_n = 1.0 / (double)nfaces;
  for (int j = 0; j < DIM; ++j) a[j] = a[j] * inv_n;
  T v = cst(0.0, A);
  for (int i = 0; i < nfaces; ++i) {
    F(i, A, n, x, isnb);
    T loc[DIM];
    T dn = cst(0.0, A);
    for (int j = 0; j < DIM; ++j) {
      loc[j] = x[j] - a[j];
      dn += loc[j] * n[j];
    }
    T fl = dn * A;
    if (isnb) fl = -fl;
    v += fl;
    for (int j = 0; j < DIM; ++j) cs[j] += fl * loc[j];
  }
  const T volume = v / (double)DIM;
  vol = volume;
  const T inv = 1.0 / ((double)(DIM + 1) * volume);
  for (int j = 0; j < DIM; ++j) xc[j] = cs[j] * inv + a[j];
}

// Per-face factors from the (oriented) normal, the face centroid and the two cell centroids
// (xn = xo on a boundary face).
template <class T, int DIM>
struct FaceFactors {
  T g, nd, dpn, dnn, nn2, inv_nd, inv_dpn;
  T dvec[DIM], skew[DIM], tP[DIM], tN[DIM], ns[DIM * DIM];
};
template <class T, int DIM>
__device__ __forceinline__ void face_factors(const T* n_, const T* xf, const T* xo, const T* xn,
                                             bool interior, FaceFactors<T, DIM>& F) {
  T d[DIM], dp[DIM], dn[DIM];
  T dd = cst(0.0, n_[0]), fd = dd, vpn = dd, vnn = dd, s2 = dd;
  for (int j = 0; j < DIM; ++j) {
    d[j] = xn[j] - xo[j];
    dp[j] = xf[j] - xo[j];
    dn[j] = xf[j] - xn[j];
    dd += d[j] * d[j];
    fd += dp[j] * d[j];
    vpn += dp[j] * n_[j];
    vnn += dn[j] * n_[j];
    s2 += n_[j] * n_[j];
  }
  const T gg = interior ? fd / dd : cst(0.0, fd);
  T dn_ = cst(0.0, fd);
  for (int j = 0; j < DIM; ++j) dn_ += d[j] * n_[j];
  F.g = gg;
  const T ndv = interior ? dn_ : vpn;
  F.nd = ndv;
  F.dpn = vpn;
  F.dnn = vnn;
  F.nn2 = s2;
  F.inv_nd = 1.0 / ndv;
  F.inv_dpn = 1.0 / vpn;
  for (int j = 0; j < DIM; ++j) {
    F.dvec[j] = d[j];
    F.skew[j] = xf[j] - (xo[j] + d[j] * gg);
    F.tP[j] = dp[j] - n_[j] * vpn;
    F.tN[j] = dn[j] - n_[j] * vnn;
  }
  for (int j = 0; j < DIM; ++j)
    for (int q = 0; q < DIM; ++q) F.ns[j * DIM + q] = n_[j] * F.skew[q];
}
