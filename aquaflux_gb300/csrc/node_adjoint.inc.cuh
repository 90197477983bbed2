// Mesh-coordinate adjoint: dL/dnodes of L = w . R(state, nodes), the node-coordinate part of
// theta_bar = -(dR/dtheta)^T lambda in _implicit_solve_bwd (aquaflux/solve/implicit.py:733-761).
// Included by residual.cu after the state adjoint (it reuses that adjoint's cotangents).
//
// Reverse mode over the stages, each stage's geometry cotangent formed by local forward mode: a
// stage's formula is evaluated once more with a dual number on one geometric input (GeoSeed) and
// the tangent contracted with the stage's output cotangent, which the state adjoint has left:
//   face fluxes           FL_bar = Wt_P - Wt_N                                 (k_nadj_flux)
//   a_P face coefficients a_bar = -d_bar d^2 / V of the owner / neighbour      (k_nadj_apcoef)
//   Green-Gauss gradients G_bar (linear in S_f, g, 1/V: written out)          (k_nadj_grad_*)
//   SST closure           (S, F1, nu_t, shear, imposed omega gradient)_bar     (k_nadj_closure)
//   SST sources           w on the k and omega rows                           (k_nadj_src)
//   d = V / a_P           d_bar d / V                                          (k_nadj_dcoeff)
// then back through the geometry, again by dual numbers on the same formulas as the forward
// pipeline (geom.cuh): the per-face factors (normal, face and cell centroids), the wall distance
// (nearest wall-face centroid) and its Green-Gauss gradient, the cell volumes / centroids (face
// areas, normals, centroids) and the face geometry (node coordinates; the owner-outward flip is a
// constant sign).  Every scatter is a gather over a precomputed incidence list: deterministic.
// Advection: first-order upwind and the limited linear upwind reconstruction (the centroids it
// reads, and the Venkatakrishnan limiters' geometry by seeded dual evaluations, k_nadj_limiter).
// Gradients: the compact scheme (with its relaxation) and the corrected scheme's swept solve
// (aquaflux/schemes/gradient.py:618-705, 1122-1337): the forward iterates X_0 .. X_{S-2} are
// recomputed, the sweeps reversed once more, and each sweep X' = X + rel (B - V X + C(X)) / V
// contributes the cotangents of 1/V, V and of C(X) = sum_f +-S_f ((1 - g) skew . X_P +
// g skew . X_N) (S_f, g, skew) at its own input; the numerator B takes rel X0_bar / V plus the
// sweeps' share (k_nadj_numerator_bar).  The SST wall-distance gradient is reversed the same way.


namespace {

__global__ void k_lift(long n, const double* src, Dual* dst) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = Dual{src[i], 0.0};
}

struct Contract {
  const double* w;
  double* acc;
  __device__ __forceinline__ void operator()(int q, const Dual& x) const { *acc += w[q] * x.d; }
};

// psi (dual, zero tangents; null without a limited reconstruction): the forward's slope limiters,
// with them the centroid seeds too -- x_f into xfb, the owner's and neighbour's x_c into recxc
// ((2, DIM, nf), gathered per cell by k_nadj_centroid_gather).
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_nadj_flux(MeshView m, CaseView cv, const double* state,
                                                   Par<Dual> par, const Dual* G, const Dual* cl,
                                                   const Dual* dco, const double* Wt,
                                                   const double* FLx, const Dual* psi, double* Fb,
                                                   double* wdf, double* xfb, double* recxc) {
  constexpr int NF = Layout<DIM, TURB>::NFLD;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f];
  const bool interior = f < m.nfi;
  double FLb[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q)
    FLb[q] = Wt[(long)q * nc + o] - (interior ? Wt[(long)q * nc + m.nb[f]] : 0.0) +
             (FLx ? FLx[(long)q * nf + f] : 0.0);
  const Src<Dual> st{state, nullptr};
  auto contract = [&](const GeoSeed& gs) {
    double acc = 0.0;
    flux_face<Dual, DIM, TURB>(m, cv, st, par, G, cl, dco, (const Dual*)nullptr, psi, true, f,
                               Contract{FLb, &acc}, nullptr, gs);
    return acc;
  };
#pragma unroll 1
  for (int comp = 0; comp < GF_COUNT; ++comp) Fb[(long)comp * nf + f] += contract(GeoSeed{comp, -1, f, -1});
  wdf[f] = (TURB && !interior) ? contract(GeoSeed{-1, GC_WD, -1, o}) : 0.0;
  if (psi) {
#pragma unroll 1
    for (int j = 0; j < DIM; ++j) {
      xfb[(long)j * nf + f] += contract(GeoSeed{GF_XF + j, -1, f, -1});
      recxc[(long)j * nf + f] = contract(GeoSeed{-1, GC_XC + j, -1, o});
      recxc[(long)(DIM + j) * nf + f] = interior ? contract(GeoSeed{-1, GC_XC + j, -1, m.nb[f]}) : 0.0;
    }
  }
}

// The Venkatakrishnan limiters' geometry (limiter_cell reads x_f, x_c and V): per cell and
// advected field with a limiter, d psi / d(geometry) by seeded dual evaluations contracted with
// psi_bar -- into Vb, limxc (DIM, nc) and limxf (DIM, ncf: per cell-face entry).
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_nadj_limiter(MeshView m, const double* state,
                                                      const double* G, double Km, double Ks,
                                                      const double* psib, double* Vb,
                                                      double* limxc, double* limxf, long ncf) {
  constexpr int NA = DIM + (TURB ? 2 : 0);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
#pragma unroll 1
  for (int a = 0; a < NA; ++a) {
    const double K = a < DIM ? Km : Ks;
    const double pb = psib[(long)a * nc + c];
    if (!(K > 0.0) || pb == 0.0) continue;
    const int q = advected_field<DIM, TURB>(a);
    auto eval = [&](const GeoSeed& gs) {
      auto phi = [&](int cell) { return Dual{state[(long)q * nc + cell], 0.0}; };
      auto grad = [&](int j) { return Dual{G[((long)q * DIM + j) * nc + c], 0.0}; };
      return limiter_cell<Dual, DIM>(m, c, K, phi, grad, gs).d;
    };
    Vb[c] += pb * eval(GeoSeed{-1, GC_VOL, -1, c});
#pragma unroll 1
    for (int j = 0; j < DIM; ++j) limxc[(long)j * nc + c] += pb * eval(GeoSeed{-1, GC_XC + j, -1, c});
#pragma unroll 1
    for (int i = b; i < e; ++i) {
      const int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
      for (int j = 0; j < DIM; ++j) limxf[(long)j * ncf + i] += pb * eval(GeoSeed{GF_XF + j, -1, f, -1});
    }
  }
}

// Cell-centroid cotangents of the reconstruction (recxc, per face and side) and of the limiters
// (limxc), added to xcb.
template <int DIM>
__global__ void k_nadj_centroid_gather(MeshView m, const double* recxc, const double* limxc,
                                       double* xcb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  for (int j = 0; j < DIM; ++j) {
    double acc = limxc[(long)j * nc + c];
    for (int i = m.cf_ptr[c]; i < m.cf_ptr[c + 1]; ++i) {
      const unsigned ent = m.cf_face[i];
      const int f = (int)(ent & ~FV_NB_BIT);
      acc += recxc[((long)((ent & FV_NB_BIT) ? DIM : 0) + j) * nf + f];
    }
    xcb[(long)j * nc + c] += acc;
  }
}

template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_nadj_apcoef(MeshView m, CaseView cv, const double* state,
                                                     Par<Dual> par, const Dual* G, const Dual* cl,
                                                     const double* dco, const double* dcob,
                                                     double* Fb, double* wdf) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nf = m.nf;
  const int o = m.owner[f];
  const bool interior = f < m.nfi;
  const double abo = -dcob[o] * dco[o] * dco[o] * m.inv_vol[o];
  double abn = 0.0;
  if (interior) {
    const int n = m.nb[f];
    abn = -dcob[n] * dco[n] * dco[n] * m.inv_vol[n];
  }
  const Src<Dual> st{state, nullptr};
#pragma unroll 1
  for (int comp = 0; comp < GF_COUNT; ++comp) {
    Dual ao, an, mf;
    apcoef_face<Dual, DIM, TURB>(m, cv, st, par, G, cl, f, GeoSeed{comp, -1, f, -1}, ao, an, mf);
    Fb[(long)comp * nf + f] += abo * ao.d + abn * an.d;
  }
  if (TURB && !interior) {
    Dual ao, an, mf;
    apcoef_face<Dual, DIM, TURB>(m, cv, st, par, G, cl, f, GeoSeed{-1, GC_WD, -1, o}, ao, an, mf);
    wdf[f] += abo * ao.d;
  }
}

// Green-Gauss: G_c = (1/V_c) sum_f +-S_f phi_f, S_f = n_f A_f, phi_f = lerp(phi_P, phi_N, g_f) or
// the leading-order boundary value.
// nbar: the cotangent of the Green-Gauss numerator B phi per cell, (NF, DIM, nc).
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_nadj_grad_face(MeshView m, CaseView cv,
                                                        const double* state, Par<double> par,
                                                        const double* nbar, double* Fb) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f];
  const double A = m.area[f];
  double nrm[DIM], Sb[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    nrm[j] = m.normal[(long)j * nf + f];
    Sb[j] = 0.0;
  }
  if (f < m.nfi) {
    const int n = m.nb[f];
    const double g = m.g[f];
    double gb = 0.0;
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      const double po = state[(long)q * nc + o], pn = state[(long)q * nc + n];
      const double pf = lerp(po, pn, g);
      double pbar = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        const double y = nbar[((long)q * DIM + j) * nc + o] - nbar[((long)q * DIM + j) * nc + n];
        Sb[j] += pf * y;
        pbar += nrm[j] * A * y;
      }
      gb += pbar * (pn - po);
    }
    Fb[(long)GF_G * nf + f] += gb;
  } else {
    const signed char kind = cv.fkind[f];
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      const double po = state[(long)q * nc + o];
      double pb;
      if (q < DIM) pb = bvel(cv, nf, f, q, kind, po, par);
      else if (q == L::P) pb = bpress(cv, f, kind, po);
      else if (q == L::K) pb = bscalar(cv.kkind[f], cv.kval[f], po, 0.0);
      else pb = bscalar(cv.wkind[f], cv.wval[f], po, 0.0);
#pragma unroll
      for (int j = 0; j < DIM; ++j) Sb[j] += pb * nbar[((long)q * DIM + j) * nc + o];
    }
  }
  double ab = 0.0;
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    ab += Sb[j] * nrm[j];
    Fb[(long)(GF_NORMAL + j) * nf + f] += Sb[j] * A;
  }
  Fb[(long)GF_AREA * nf + f] += ab;
}

// The numerator cotangent of NQ Green-Gauss fields: X0 = rel B / V (the gradient itself for the
// compact scheme), so B_bar = rel X0_bar / V, plus the swept sweeps' share Bsw (may be null).
template <int DIM, int NQ>
__global__ void k_nadj_numerator_bar(MeshView m, const double* X0b, const double* Bsw, double rel,
                                     double* nbar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
  const double r = rel * m.inv_vol[c];
  for (int k = 0; k < NQ * DIM; ++k) {
    const long i = (long)k * nc + c;
    nbar[i] = X0b[i] * r + (Bsw ? Bsw[i] : 0.0);
  }
}

// 1/V part of the first gradient iterate X0 = rel B / V: ivb += rel X0_bar . B, with B = X0 V / rel
// for the compact scheme (Bnum null) or the stored numerator.
template <int DIM, int NQ>
__global__ void k_nadj_grad_cell(MeshView m, const double* X0b, const double* X0,
                                 const double* Bnum, double rel, double* ivb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
  double acc = 0.0;
  for (int k = 0; k < NQ * DIM; ++k) acc += X0b[(long)k * nc + c] * (Bnum ? Bnum[(long)k * nc + c] : X0[(long)k * nc + c]);
  ivb[c] += Bnum ? rel * acc : acc * m.vol[c];
}

// d = V / a_P: the volume part.
__global__ void k_nadj_dcoeff(MeshView m, const double* dco, const double* dcob, double* Cb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  Cb[(long)GC_VOL * m.nc + c] += dcob[c] * dco[c] / m.vol[c];
}

// X0 = rel B / V.
template <int DIM, int NQ>
__global__ void k_nadj_x0(MeshView m, const double* B, double rel, double* X0) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
  const double iv = m.inv_vol[c];
  for (int k = 0; k < NQ * DIM; ++k) X0[(long)k * nc + c] = rel * (B[(long)k * nc + c] * iv);
}

// One swept sweep X' = X + rel (B - (V X - C(X))) / V, its geometry cotangents at input X with
// output cotangent Y.  Face part (interior faces): w_f = (1 - g) skew . X_P + g skew . X_N (kept
// in wface for the cell part) and the cotangents of S_f, g, skew from C = sum +-S_f w_f.
template <int DIM, int NQ>
__global__ void __launch_bounds__(128) k_nadj_sweep_face(MeshView m, const double* X,
                                                         const double* Y, double rel, double* Fb,
                                                         double* wface) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nfi) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f], n = m.nb[f];
  const double A = m.area[f], g = m.g[f];
  const double ro = rel * m.inv_vol[o], rn = rel * m.inv_vol[n];
  double nrm[DIM], sk[DIM], Sb[DIM], skb[DIM];
  for (int j = 0; j < DIM; ++j) {
    nrm[j] = m.normal[(long)j * nf + f];
    sk[j] = m.skew[(long)j * nf + f];
    Sb[j] = 0.0;
    skb[j] = 0.0;
  }
  double gb = 0.0;
  for (int q = 0; q < NQ; ++q) {
    double so = 0.0, sn = 0.0;
    for (int j = 0; j < DIM; ++j) {
      so += sk[j] * X[((long)q * DIM + j) * nc + o];
      sn += sk[j] * X[((long)q * DIM + j) * nc + n];
    }
    const double w = (1.0 - g) * so + g * sn;
    wface[(long)q * nf + f] = w;
    double wb = 0.0;
    for (int j = 0; j < DIM; ++j) {
      const double D = Y[((long)q * DIM + j) * nc + o] * ro - Y[((long)q * DIM + j) * nc + n] * rn;
      Sb[j] += D * w;
      wb += D * nrm[j] * A;
    }
    gb += wb * (sn - so);
    for (int j = 0; j < DIM; ++j)
      skb[j] += wb * ((1.0 - g) * X[((long)q * DIM + j) * nc + o] + g * X[((long)q * DIM + j) * nc + n]);
  }
  double ab = 0.0;
  for (int j = 0; j < DIM; ++j) {
    ab += Sb[j] * nrm[j];
    Fb[(long)(GF_NORMAL + j) * nf + f] += Sb[j] * A;
    Fb[(long)(GF_SKEW + j) * nf + f] += skb[j];
  }
  Fb[(long)GF_AREA * nf + f] += ab;
  Fb[(long)GF_G * nf + f] += gb;
}

// ... cell part: C(X) from wface, then the cotangents of 1/V (rel (B - V X + C) . Y) and of V
// (-rel X . Y / V).
template <int DIM, int NQ>
__global__ void __launch_bounds__(128) k_nadj_sweep_cell(MeshView m, const double* X,
                                                         const double* Y, const double* B,
                                                         const double* wface, double rel,
                                                         double* ivb, double* Vb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  double corr[NQ][DIM];
  for (int q = 0; q < NQ; ++q)
    for (int j = 0; j < DIM; ++j) corr[q][j] = 0.0;
  bool any = false;
  for (int i = m.cf_ptr[c]; i < m.cf_ptr[c + 1]; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    if (f >= m.nfi) continue;
    any = true;
    const double A = (ent & FV_NB_BIT) ? -m.area[f] : m.area[f];
    for (int q = 0; q < NQ; ++q)
      for (int j = 0; j < DIM; ++j) corr[q][j] += (m.normal[(long)j * nf + f] * A) * wface[(long)q * nf + f];
  }
  const double V = m.vol[c];
  double aiv = 0.0, av = 0.0;
  for (int q = 0; q < NQ; ++q)
    for (int j = 0; j < DIM; ++j) {
      const long k = ((long)q * DIM + j) * nc + c;
      const double x = X[k], y = Y[k];
      const double ax = any ? x * V - corr[q][j] : x * V;
      aiv += (B[k] - ax) * y;
      av += x * y;
    }
  ivb[c] += rel * aiv;
  Vb[c] += -rel * m.inv_vol[c] * av;
}

// Buffers of the swept reversal for NQ fields: S - 1 forward iterates, two cotangents, a
// numerator-sweep accumulator, and the face values.
struct SweepBufs {
  double* X;     // (S - 1) iterates X_0 .. X_{S-2}, each (NQ, DIM, nc)
  double* Y0;
  double* Y1;
  double* Bsw;   // sum over the sweeps of rel Y / V: the numerator's share
  double* nbar;
  double* wface; // (NQ, nf)
};

SweepBufs sweep_layout(double* p, int sweeps, int nq, int dim, long nc, long nf) {
  const long blk = (long)nq * dim * nc;
  SweepBufs b;
  b.X = p; p += (long)std::max(sweeps - 1, 1) * blk;
  b.Y0 = p; p += blk;
  b.Y1 = p; p += blk;
  b.Bsw = p; p += blk;
  b.nbar = p; p += blk;
  b.wface = p;
  return b;
}

size_t sweep_doubles(int sweeps, int nq, int dim, long nc, long nf) {
  return (size_t)(std::max(sweeps - 1, 1) + 4) * nq * dim * nc + (size_t)nq * nf;
}

// The corrected scheme's reversal for NQ fields with numerator B (stored) and the cotangent Gb of
// the last iterate: contributions of every sweep to Fb / ivb / Vb; on return bf.nbar holds the
// numerator's cotangent and ivb the first iterate's 1/V part.
template <int DIM, int NQ>
int sweeps_geometry(const MeshView& m, int sweeps, double rel, const double* B, const double* Gb,
                    const SweepBufs& bf, double* Fb, double* ivb, double* Vb, cudaStream_t s) {
  constexpr int TB = 128;
  const long blk = (long)NQ * DIM * m.nc;
  const int bc = fv_blocks(m.nc, TB), bfi = fv_blocks(m.nfi > 0 ? m.nfi : 1, TB);
  // forward iterates X_0 .. X_{S-2}
  k_nadj_x0<DIM, NQ><<<bc, TB, 0, s>>>(m, B, rel, bf.X);
  for (int it = 1; it < sweeps - 1; ++it) {
    if (m.nfi > 0) k_gg_skew<double, DIM, NQ><<<bfi, TB, 0, s>>>(m, bf.X + (it - 1) * blk, bf.wface);
    k_gg_sweep<double, DIM, NQ><<<bc, TB, 0, s>>>(m, B, bf.X + (it - 1) * blk, bf.wface, rel,
                                                   bf.X + it * blk);
  }
  // backward: sweep k maps X_{k-1} to X_k; Y holds X_k's cotangent
  FV_CUDA_TRY(cudaMemcpyAsync(bf.Y0, Gb, sizeof(double) * blk, cudaMemcpyDeviceToDevice, s));
  double* Y = bf.Y0;
  double* Yn = bf.Y1;
  MeshView mv = m;
  for (int k = sweeps - 1; k >= 1; --k) {
    const double* Xin = bf.X + (k - 1) * blk;
    if (m.nfi > 0) k_nadj_sweep_face<DIM, NQ><<<bfi, TB, 0, s>>>(mv, Xin, Y, rel, Fb, bf.wface);
    k_nadj_sweep_cell<DIM, NQ><<<bc, TB, 0, s>>>(mv, Xin, Y, B, bf.wface, rel, ivb, Vb);
    if (m.nfi > 0) a_gg_skew<DIM, NQ><<<bfi, TB, 0, s>>>(mv, Y, rel, bf.wface);
    a_gg_sweep<DIM, NQ><<<bc, TB, 0, s>>>(mv, Y, bf.wface, rel, k == sweeps - 1, bf.Bsw, Yn);
    double* t = Y;
    Y = Yn;
    Yn = t;
  }
  // Y = X0_bar
  k_nadj_numerator_bar<DIM, NQ><<<bc, TB, 0, s>>>(mv, Y, bf.Bsw, rel, bf.nbar);
  k_nadj_grad_cell<DIM, NQ><<<bc, TB, 0, s>>>(mv, Y, bf.X, B, rel, ivb);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

// The wall-distance gradient's numerator sum_f +-S_f d_f (d_f the interpolated distance, 0 on SST
// walls, the owner's value on other boundaries), (DIM, nc).
template <int DIM>
__global__ void k_nadj_wd_numerator(MeshView m, CaseView cv, double* num) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  double acc[DIM];
  for (int j = 0; j < DIM; ++j) acc[j] = 0.0;
  const double phic = cv.wd[c];
  for (int i = m.cf_ptr[c]; i < m.cf_ptr[c + 1]; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    double phif;
    if (f < m.nfi) {
      const double g = m.g[f];
      phif = (1.0 - g) * cv.wd[m.owner[f]] + g * cv.wd[m.nb[f]];
    } else {
      phif = cv.swall[f] ? 0.0 : phic;
    }
    const double sgn = (ent & FV_NB_BIT) ? -phif : phif;
    for (int j = 0; j < DIM; ++j) acc[j] += (m.normal[(long)j * nf + f] * m.area[f]) * sgn;
  }
  for (int j = 0; j < DIM; ++j) num[(long)j * nc + c] = acc[j];
}

template <int DIM>
__global__ void __launch_bounds__(128) k_nadj_closure(MeshView m, CaseView cv, const double* state,
                                                      Par<Dual> par, const Dual* G,
                                                      const double* clb, const double* Gwib,
                                                      double* Cb, double* Fb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const Src<Dual> st{state, nullptr};
  auto contract = [&](const GeoSeed& gs) {
    Dual out[7], gw[DIM];
    closure_cell<Dual, DIM>(m, cv, st, par, G, c, gs, out, gw);
    double acc = 0.0;
    for (int i = 0; i < 4; ++i) acc += clb[(long)i * nc + c] * out[i].d;
    for (int j = 0; j < DIM; ++j) acc += Gwib[(long)j * nc + c] * gw[j].d;
    return acc;
  };
#pragma unroll 1
  for (int comp = GC_WD; comp < GC_WDG + DIM; ++comp)
    Cb[(long)comp * nc + c] += contract(GeoSeed{-1, comp, -1, c});
  if (cv.wcell[c]) {
    const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
    for (int i = b; i < e; ++i) {
      const int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
      if (f < m.nfi || !cv.swall[f]) continue;
      Fb[(long)GF_AREA * nf + f] += contract(GeoSeed{GF_AREA, -1, f, -1});
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(128) k_nadj_src(MeshView m, CaseView cv, const double* state,
                                                  Par<Dual> par, const Dual* cl, const Dual* G,
                                                  const Dual* Gwi, const double* W, double* Cb) {
  using L = Layout<DIM, true>;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
  const Src<Dual> st{state, nullptr};
  const double wk = W[(long)L::K * nc + c], ww = W[(long)L::W * nc + c];
  for (int comp = GC_VOL; comp <= GC_WD; ++comp) {
    Dual rk{0.0, 0.0}, rw{0.0, 0.0};
    sst_rows<Dual, DIM>(m, cv, st, par, cl, G, Gwi, c, rk, rw, GeoSeed{-1, comp, -1, c});
    Cb[(long)comp * nc + c] += wk * rk.d + ww * rw.d;
  }
}

// Wall-distance gradient (compact Green-Gauss of d: Dirichlet 0 on SST walls, the owner value on
// other boundaries): face part.
// nb: the cotangent of the gradient's numerator per cell, (DIM, nc).
template <int DIM>
__global__ void k_nadj_wdg_face(MeshView m, CaseView cv, const double* nb, double* Fb,
                                double* dpart) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f];
  const double A = m.area[f];
  double nrm[DIM], Sb[DIM];
  for (int j = 0; j < DIM; ++j) {
    nrm[j] = m.normal[(long)j * nf + f];
    Sb[j] = 0.0;
  }
  double pbar = 0.0, d_o = 0.0, d_n = 0.0, po = 0.0, pn = 0.0;
  if (f < m.nfi) {
    const int n = m.nb[f];
    const double g = m.g[f];
    d_o = cv.wd[o];
    d_n = cv.wd[n];
    const double df = (1.0 - g) * d_o + g * d_n;
    for (int j = 0; j < DIM; ++j) {
      const double y = nb[(long)j * nc + o] - nb[(long)j * nc + n];
      Sb[j] += df * y;
      pbar += nrm[j] * A * y;
    }
    Fb[(long)GF_G * nf + f] += pbar * (d_n - d_o);
    po = (1.0 - g) * pbar;
    pn = g * pbar;
  } else {
    const double df = cv.swall[f] ? 0.0 : cv.wd[o];
    for (int j = 0; j < DIM; ++j) {
      const double y = nb[(long)j * nc + o];
      Sb[j] += df * y;
      pbar += nrm[j] * A * y;
    }
    po = cv.swall[f] ? 0.0 : pbar;
  }
  double ab = 0.0;
  for (int j = 0; j < DIM; ++j) {
    ab += Sb[j] * nrm[j];
    Fb[(long)(GF_NORMAL + j) * nf + f] += Sb[j] * A;
  }
  Fb[(long)GF_AREA * nf + f] += ab;
  dpart[f] = po;
  dpart[(long)nf + f] = pn;
}

// ... cell part: the d cotangent from the faces (the 1/V part goes through ivb).
template <int DIM>
__global__ void k_nadj_wdg_cell(MeshView m, CaseView cv, const double* dpart, double* Cb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  double db = 0.0;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    db += (ent & FV_NB_BIT) ? dpart[(long)nf + f] : dpart[f];
  }
  Cb[(long)GC_WD * nc + c] += db;
}

// Cell scalars: V_bar (with the 1/V cotangent) and the wall-distance cotangent; the nearest wall
// face's centroid and the cell centroid take d_bar (x_c - x_w) / d.
template <int DIM, bool TURB>
__global__ void k_nadj_cell_chain(MeshView m, CaseView cv, const double* Cb, const double* ivb,
                                  const double* wdf, const int* wnear, double* Vb, double* xcb,
                                  double* wcon) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const double iv = m.inv_vol[c];
  Vb[c] += Cb[(long)GC_VOL * nc + c] - ivb[c] * iv * iv;
  for (int j = 0; j < DIM; ++j) xcb[(long)j * nc + c] = 0.0;
  if (!TURB) return;
  double db = Cb[(long)GC_WD * nc + c];
  const double i1 = cv.inv_wd[c], i2 = cv.inv_wd2[c];
  db += -Cb[(long)GC_INV_WD * nc + c] * i1 * i1 - 2.0 * Cb[(long)GC_INV_WD2 * nc + c] * i1 * i2;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
    if (f >= m.nfi && m.owner[f] == c) db += wdf[f];
  }
  const int w = wnear[c];
  const double d = cv.wd[c];
  for (int j = 0; j < DIM; ++j) {
    const double t = d > 0.0 ? db * (m.xc[(long)j * nc + c] - m.xf[(long)j * nf + w]) / d : 0.0;
    xcb[(long)j * nc + c] = t;
    wcon[(long)j * nc + c] = t;
  }
}

template <int DIM>
__global__ void k_nadj_wall_face(MeshView m, const int* wall_ptr, const int* wall_cell,
                                 const double* wcon, double* xfb) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  for (int i = wall_ptr[f]; i < wall_ptr[f + 1]; ++i) {
    const int c = wall_cell[i];
    for (int j = 0; j < DIM; ++j) xfb[(long)j * nf + f] -= wcon[(long)j * nc + c];
  }
}

// Per-face factors -> normal, face centroid and the two cell centroids.
template <int DIM>
__global__ void __launch_bounds__(128) k_nadj_factors(MeshView m, const double* Fb, double* nbt,
                                                      double* xfb, double* xcpart) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f];
  const bool interior = f < m.nfi;
  const int n = interior ? m.nb[f] : o;
  double nv[DIM], xv[DIM], ov[DIM], wv[DIM];
  for (int j = 0; j < DIM; ++j) {
    nv[j] = m.normal[(long)j * nf + f];
    xv[j] = m.xf[(long)j * nf + f];
    ov[j] = m.xc[(long)j * nc + o];
    wv[j] = m.xc[(long)j * nc + n];
  }
  const int groups = interior ? 4 : 3;
#pragma unroll 1
  for (int sdx = 0; sdx < groups * DIM; ++sdx) {
    const int grp = sdx / DIM, sj = sdx % DIM;
    Dual nd[DIM], xd[DIM], od[DIM], wd[DIM];
    for (int j = 0; j < DIM; ++j) {
      nd[j] = {nv[j], (grp == 0 && j == sj) ? 1.0 : 0.0};
      xd[j] = {xv[j], (grp == 1 && j == sj) ? 1.0 : 0.0};
      od[j] = {ov[j], (grp == 2 && j == sj) ? 1.0 : 0.0};
      wd[j] = {wv[j], (grp == 3 && j == sj) ? 1.0 : 0.0};
    }
    FaceFactors<Dual, DIM> F;
    face_factors<Dual, DIM>(nd, xd, od, interior ? wd : od, interior, F);
    auto fb = [&](int comp) { return Fb[(long)comp * nf + f]; };
    double acc = fb(GF_G) * F.g.d + fb(GF_DPN) * F.dpn.d + fb(GF_DNN) * F.dnn.d +
                 fb(GF_NN2) * F.nn2.d + fb(GF_INV_ND) * F.inv_nd.d + fb(GF_INV_DPN) * F.inv_dpn.d;
    for (int j = 0; j < DIM; ++j)
      acc += fb(GF_DVEC + j) * F.dvec[j].d + fb(GF_SKEW + j) * F.skew[j].d +
             fb(GF_TP + j) * F.tP[j].d + fb(GF_TN + j) * F.tN[j].d;
    for (int k = 0; k < DIM * DIM; ++k) acc += fb(GF_NS + k) * F.ns[k].d;
    if (grp == 0) nbt[(long)sj * nf + f] = fb(GF_NORMAL + sj) + acc;
    else if (grp == 1) xfb[(long)sj * nf + f] += acc;
    else if (grp == 2) xcpart[(long)sj * nf + f] = acc;
    else xcpart[(long)(DIM + sj) * nf + f] = acc;
  }
  if (!interior)
    for (int j = 0; j < DIM; ++j) xcpart[(long)(DIM + j) * nf + f] = 0.0;
}

template <int DIM>
__global__ void k_nadj_xc_gather(MeshView m, const double* xcpart, double* xcb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    const long base = (ent & FV_NB_BIT) ? (long)DIM * nf : 0;
    for (int j = 0; j < DIM; ++j) xcb[(long)j * nc + c] += xcpart[base + (long)j * nf + f];
  }
}

// Cell volume and centroid -> the areas, normals and centroids of the cell's faces.
template <int DIM>
__global__ void __launch_bounds__(128) k_nadj_cell_geom(MeshView m, const double* Vb,
                                                        const double* xcb, double* cfA,
                                                        double* cfN, double* cfX, long ncf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  const int k = e - b;
  const double vb = Vb[c];
  double xb[DIM];
  for (int j = 0; j < DIM; ++j) xb[j] = xcb[(long)j * nc + c];
#pragma unroll 1
  for (int sdx = 0; sdx < k * (1 + 2 * DIM); ++sdx) {
    const int slot = sdx / (1 + 2 * DIM), comp = sdx % (1 + 2 * DIM);
    auto F = [&](int i, Dual& A, Dual* n, Dual* x, bool& isnb) {
      const unsigned ent = m.cf_face[b + i];
      const int f = (int)(ent & ~FV_NB_BIT);
      const bool hit = i == slot;
      A = {m.area[f], (hit && comp == 0) ? 1.0 : 0.0};
      for (int j = 0; j < DIM; ++j) {
        n[j] = {m.normal[(long)j * nf + f], (hit && comp == 1 + j) ? 1.0 : 0.0};
        x[j] = {m.xf[(long)j * nf + f], (hit && comp == 1 + DIM + j) ? 1.0 : 0.0};
      }
      isnb = (ent & FV_NB_BIT) != 0;
    };
    Dual vol, xc[DIM];
    cell_geom<Dual, DIM>(k, F, vol, xc);
    double acc = vb * vol.d;
    for (int j = 0; j < DIM; ++j) acc += xb[j] * xc[j].d;
    const long ent = b + slot;
    if (comp == 0) cfA[ent] = acc;
    else if (comp <= DIM) cfN[(long)(comp - 1) * ncf + ent] = acc;
    else cfX[(long)(comp - 1 - DIM) * ncf + ent] = acc;
  }
}

__device__ __forceinline__ int cf_entry(const MeshView& m, int c, int f, bool nb) {
  const unsigned want = (unsigned)f | (nb ? FV_NB_BIT : 0u);
  for (int i = m.cf_ptr[c]; i < m.cf_ptr[c + 1]; ++i)
    if (m.cf_face[i] == want) return i;
  return -1;
}

// Totals of the face primitives' cotangents (residual stages + factors + cell geometry).
template <int DIM>
__global__ void k_nadj_cf_gather(MeshView m, const double* Fb, const double* cfA, const double* cfN,
                                 const double* cfX, const double* limxf, long ncf, double* Ab,
                                 double* nbt, double* xfb) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nf = m.nf;
  const int eo = cf_entry(m, m.owner[f], f, false);
  const int en = f < m.nfi ? cf_entry(m, m.nb[f], f, true) : -1;
  double a = Fb[(long)GF_AREA * nf + f];
  if (eo >= 0) a += cfA[eo];
  if (en >= 0) a += cfA[en];
  Ab[f] = a;
  for (int j = 0; j < DIM; ++j) {
    double nb = 0.0, xb = 0.0;
    if (eo >= 0) {
      nb += cfN[(long)j * ncf + eo];
      xb += cfX[(long)j * ncf + eo];
      if (limxf) xb += limxf[(long)j * ncf + eo];
    }
    if (en >= 0) {
      nb += cfN[(long)j * ncf + en];
      xb += cfX[(long)j * ncf + en];
      if (limxf) xb += limxf[(long)j * ncf + en];
    }
    nbt[(long)j * nf + f] += nb;
    xfb[(long)j * nf + f] += xb;
  }
}

// Face area / normal / centroid -> the face's node coordinates.
template <int DIM>
__global__ void __launch_bounds__(128) k_nadj_face_geom(MeshView m, const double* Ab,
                                                        const double* nbt, const double* xfb,
                                                        double* nodepart) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nf = m.nf;
  const int b = m.fn_ptr[f], e = m.fn_ptr[f + 1];
  const int k = e - b;
  double ns_[DIM], nbf[DIM], xbf[DIM];
  for (int j = 0; j < DIM; ++j) {
    ns_[j] = m.normal[(long)j * nf + f];
    nbf[j] = nbt[(long)j * nf + f];
    xbf[j] = xfb[(long)j * nf + f];
  }
  const double ab = Ab[f];
#pragma unroll 1
  for (int sdx = 0; sdx < k * DIM; ++sdx) {
    const int si = sdx / DIM, sj = sdx % DIM;
    auto P = [&](int i, int j) -> Dual {
      return {m.nodes[(long)DIM * m.fn_idx[b + i] + j], (i == si && j == sj) ? 1.0 : 0.0};
    };
    Dual A, n[DIM], x[DIM];
    face_geom<Dual, DIM>(k, P, A, n, x);
    double dot = 0.0;
    for (int j = 0; j < DIM; ++j) dot += n[j].v * ns_[j];
    const double sgn = dot < 0.0 ? -1.0 : 1.0;  // the owner-outward flip
    double acc = ab * A.d;
    for (int j = 0; j < DIM; ++j) acc += nbf[j] * sgn * n[j].d + xbf[j] * x[j].d;
    nodepart[(long)(b + si) * DIM + sj] = acc;
  }
}

__global__ void k_nadj_nodes(int nn, int dim, const int* node_ptr, const int* node_ent,
                             const double* nodepart, double* dnodes) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nn) return;
  for (int j = 0; j < dim; ++j) {
    double acc = 0.0;
    for (int i = node_ptr[v]; i < node_ptr[v + 1]; ++i)
      acc += nodepart[(long)node_ent[i] * dim + j];
    dnodes[(long)v * dim + j] = acc;
  }
}

// The pressure part sum_i w_i p_f A n_i of a viscous-only functional on boundary faces: its
// geometry cotangents are subtracted (p_f = the owner pressure, or the outlet value).
template <int DIM, bool TURB>
__global__ void k_nadj_pressure_term(MeshView m, CaseView cv, const double* state,
                                     const double* FLx, double* Fb) {
  using L = Layout<DIM, TURB>;
  const int f = m.nfi + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nf = m.nf;
  const int o = m.owner[f];
  const double pf = bpress(cv, f, cv.fkind[f], state[(long)L::P * m.nc + o]);
  const double A = m.area[f];
  double ab = 0.0;
  for (int i = 0; i < DIM; ++i) {
    const double wi = FLx[(long)i * nf + f];
    ab += wi * pf * m.normal[(long)i * nf + f];
    Fb[(long)(GF_NORMAL + i) * nf + f] -= wi * pf * A;
  }
  Fb[(long)GF_AREA * nf + f] -= ab;
}

struct NadjBuffers {
  double *Fb, *Cb, *ivb, *wdf, *dpart, *Vb, *Ab, *nbt, *xfb, *xcpart, *xcb, *wcon, *cfA, *cfN,
      *cfX, *nodepart;
};

NadjBuffers nadj_layout(double* p, int dim, long nc, long nf, long ncf, long nfn) {
  NadjBuffers B;
  B.Fb = p; p += (long)GF_COUNT * nf;
  B.Cb = p; p += (long)GC_COUNT * nc;
  B.ivb = p; p += nc;
  B.wdf = p; p += nf;
  B.dpart = p; p += 2 * nf;
  B.Vb = p; p += nc;
  B.Ab = p; p += nf;
  B.nbt = p; p += (long)dim * nf;
  B.xfb = p; p += (long)dim * nf;
  B.xcpart = p; p += 2L * dim * nf;
  B.xcb = p; p += (long)dim * nc;
  B.wcon = p; p += (long)dim * nc;
  B.cfA = p; p += ncf;
  B.cfN = p; p += (long)dim * ncf;
  B.cfX = p; p += (long)dim * ncf;
  B.nodepart = p;
  return B;
}

size_t nadj_doubles(int dim, long nc, long nf, long ncf, long nfn) {
  return (size_t)GF_COUNT * nf + (size_t)GC_COUNT * nc + 2 * nc + 4 * nf + 2 * dim * nf +
         2 * dim * nf + 2 * dim * nc + ncf * (1 + 2 * dim) + (size_t)dim * nfn;
}

int nadj_setup(FvCase* cs, cudaStream_t s) {
  if (cs->nadj) return FV_OK;
  FvMesh* M = cs->mesh;
  const int dim = M->dim;
  const long nc = M->nc, nf = M->nf;
  const long ncf = M->h_cf_ptr[nc];
  std::vector<int> fp(nf + 1);
  FV_CUDA_TRY(cudaMemcpyAsync(fp.data(), M->fn_ptr, sizeof(int) * (nf + 1), cudaMemcpyDeviceToHost, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  const long nfn = fp[nf];
  std::vector<int> fi(nfn);
  FV_CUDA_TRY(cudaMemcpy(fi.data(), M->fn_idx, sizeof(int) * nfn, cudaMemcpyDeviceToHost));
  // node -> entries of fn_idx (ascending)
  std::vector<int> np(M->nn + 1, 0), ne(nfn);
  for (long i = 0; i < nfn; ++i) np[fi[i] + 1]++;
  for (int v = 0; v < M->nn; ++v) np[v + 1] += np[v];
  std::vector<int> fill(np.begin(), np.end() - 1);
  for (long i = 0; i < nfn; ++i) ne[fill[fi[i]]++] = (int)i;
  // face -> cells whose nearest wall face it is
  std::vector<int> wp(nf + 1, 0), wc;
  if (cs->desc.turbulent) {
    std::vector<int> near(nc);
    FV_CUDA_TRY(cudaMemcpy(near.data(), cs->wnear, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    for (long c = 0; c < nc; ++c) wp[near[c] + 1]++;
    for (long f = 0; f < nf; ++f) wp[f + 1] += wp[f];
    wc.assign(nc, 0);
    std::vector<int> wf(wp.begin(), wp.end() - 1);
    for (long c = 0; c < nc; ++c) wc[wf[near[c]]++] = (int)c;
  }
  NodeAdjoint* na = new NodeAdjoint();
  cs->nadj = na;
  FV_CUDA_TRY(cudaMalloc(&na->dual_work, cs->work_bytes));
  FV_CUDA_TRY(cudaMalloc(&na->buf, sizeof(double) * nadj_doubles(dim, nc, nf, ncf, nfn)));
  {
    // gradient reversal: the saved last-iterate cotangent (nfld, dim, nc), the wall-distance
    // numerator (dim, nc) and the sweep buffers of the flow fields
    const int sweeps = std::max(cs->desc.gradient_sweeps, 1);
    const size_t n = (size_t)cs->nfld * dim * nc + (size_t)dim * nc +
                     sweep_doubles(sweeps, cs->nfld, dim, nc, nf);
    FV_CUDA_TRY(cudaMalloc(&na->sweep, sizeof(double) * n));
  }
  if (cs->view.rec_mom || cs->view.rec_sca)  // recxc (2, dim, nf), limxc (dim, nc), limxf (dim, ncf)
    FV_CUDA_TRY(cudaMalloc(&na->rec, sizeof(double) * ((size_t)2 * dim * nf + (size_t)dim * nc +
                                                       (size_t)dim * ncf)));
  FV_CUDA_TRY(cudaMalloc(&na->node_ptr, sizeof(int) * np.size()));
  FV_CUDA_TRY(cudaMalloc(&na->node_ent, sizeof(int) * std::max<long>(nfn, 1)));
  FV_CUDA_TRY(cudaMalloc(&na->wall_ptr, sizeof(int) * wp.size()));
  FV_CUDA_TRY(cudaMalloc(&na->wall_cell, sizeof(int) * std::max<size_t>(wc.size(), 1)));
  FV_CUDA_TRY(cudaMemcpyAsync(na->node_ptr, np.data(), sizeof(int) * np.size(), cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(na->node_ent, ne.data(), sizeof(int) * nfn, cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaMemcpyAsync(na->wall_ptr, wp.data(), sizeof(int) * wp.size(), cudaMemcpyHostToDevice, s));
  if (!wc.empty())
    FV_CUDA_TRY(cudaMemcpyAsync(na->wall_cell, wc.data(), sizeof(int) * wc.size(), cudaMemcpyHostToDevice, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  return FV_OK;
}

template <int DIM, bool TURB>
int node_vjp(FvCase* cs, const double* state, const double* W, double* dnodes, cudaStream_t s) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  NodeAdjoint* na0 = cs->nadj;
  const int sweeps = cs->desc.gradient_sweeps;
  const double rel = sweeps >= 1 ? cs->desc.gradient_relaxation : 1.0;
  double* gb_last = na0->sweep;                                  // (NF, DIM, nc)
  double* wd_num = gb_last + (long)NF * DIM * cs->mesh->nc;      // (DIM, nc)
  double* sweep_area = wd_num + (long)DIM * cs->mesh->nc;
  // cotangents of every stage (the gradient's saved before the backward sweeps overwrite it)
  int rc = run_vjp<DIM, TURB>(cs, state, W, nullptr, cs->tmp2, s, sweeps >= 2 ? gb_last : nullptr);
  if (rc != FV_OK) return rc;
  FvMesh* M = cs->mesh;
  const MeshView& m = M->view;
  const CaseView& cv = cs->view;
  const long nc = m.nc, nf = m.nf;
  const long ncf = M->h_cf_ptr[nc];
  NodeAdjoint* na = cs->nadj;
  Work<double> fw = work_layout<double, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
  Work<Dual> dw = work_layout<Dual, DIM, TURB>(na->dual_work, nc, nf, psi_count<DIM, TURB>(cs));
  AdjWork aw = adj_layout<DIM, TURB>(cs);
  NadjBuffers B = nadj_layout(na->buf, DIM, nc, nf, ncf, 0);
  constexpr int TB = 128;
  const int bc = fv_blocks(nc, TB), bf = fv_blocks(nf, TB);
  auto lift = [&](const double* src, Dual* dst, long n) {
    k_lift<<<fv_blocks(n, 256), 256, 0, s>>>(n, src, dst);
  };
  lift(fw.G, dw.G, (long)NF * DIM * nc);
  lift(fw.cl, dw.cl, 7 * nc);
  lift(fw.Gwi, dw.Gwi, (long)DIM * nc);
  lift(fw.dco, dw.dco, nc);
  const long npsi = psi_count<DIM, TURB>(cs);
  double* recxc = na->rec;
  double* limxc = recxc ? recxc + 2L * DIM * nf : nullptr;
  double* limxf = recxc ? limxc + (long)DIM * nc : nullptr;
  if (npsi) {
    lift(fw.psi, dw.psi, npsi);
    FV_CUDA_TRY(cudaMemsetAsync(limxc, 0, sizeof(double) * ((size_t)DIM * nc + (size_t)DIM * ncf), s));
  }
  FV_CUDA_TRY(cudaMemsetAsync(B.Fb, 0, sizeof(double) * ((size_t)GF_COUNT * nf + (size_t)GC_COUNT * nc + nc), s));
  FV_CUDA_TRY(cudaMemsetAsync(B.Vb, 0, sizeof(double) * nc, s));
  FV_CUDA_TRY(cudaMemsetAsync(B.xfb, 0, sizeof(double) * DIM * nf, s));
  const double irho = 1.0 / cs->desc.rho;
  const Par<Dual> pd{{cs->mu, 0.0}, {cs->inlet_scale, 0.0}, {cs->mu * irho, 0.0}};
  const Par<double> pdd{cs->mu, cs->inlet_scale, cs->mu * irho};
  k_nadj_flux<DIM, TURB><<<bf, TB, 0, s>>>(m, cv, state, pd, dw.G, dw.cl, dw.dco, aw.Wt, aw.FLx,
                                           npsi ? dw.psi : nullptr, B.Fb, B.wdf, B.xfb, recxc);
  if (aw.FLx && cs->flx_viscous)
    k_nadj_pressure_term<DIM, TURB><<<bf, TB, 0, s>>>(m, cv, state, aw.FLx, B.Fb);
  k_nadj_apcoef<DIM, TURB><<<bf, TB, 0, s>>>(m, cv, state, pd, dw.G, dw.cl, fw.dco, aw.dcob, B.Fb, B.wdf);
  // Green-Gauss gradients of the fields: the swept sweeps' geometry, then the numerator's
  {
    SweepBufs sb = sweep_layout(sweep_area, std::max(sweeps, 1), NF, DIM, nc, nf);
    if (sweeps >= 2) {
      rc = sweeps_geometry<DIM, NF>(m, sweeps, rel, fw.Bg, gb_last, sb, B.Fb, B.ivb, B.Vb, s);
      if (rc != FV_OK) return rc;
    } else {
      k_nadj_numerator_bar<DIM, NF><<<bc, TB, 0, s>>>(m, aw.Gb, nullptr, rel, sb.nbar);
      k_nadj_grad_cell<DIM, NF><<<bc, TB, 0, s>>>(m, aw.Gb, fw.G, nullptr, rel, B.ivb);
    }
    k_nadj_grad_face<DIM, TURB><<<bf, TB, 0, s>>>(m, cv, state, pdd, sb.nbar, B.Fb);
  }
  k_nadj_dcoeff<<<bc, TB, 0, s>>>(m, fw.dco, aw.dcob, B.Cb);
  if constexpr (TURB) {
    k_nadj_closure<DIM><<<bc, TB, 0, s>>>(m, cv, state, pd, dw.G, aw.clb, aw.Gwib, B.Cb, B.Fb);
    k_nadj_src<DIM><<<bc, TB, 0, s>>>(m, cv, state, pd, dw.cl, dw.G, dw.Gwi, W, B.Cb);
    // the wall-distance gradient, the same scheme as the fields'
    SweepBufs sd = sweep_layout(sweep_area, std::max(sweeps, 1), 1, DIM, nc, nf);
    const double* yb = B.Cb + (long)GC_WDG * nc;
    if (sweeps >= 2) {
      k_nadj_wd_numerator<DIM><<<bc, TB, 0, s>>>(m, cv, wd_num);
      rc = sweeps_geometry<DIM, 1>(m, sweeps, rel, wd_num, yb, sd, B.Fb, B.ivb, B.Vb, s);
      if (rc != FV_OK) return rc;
    } else {
      k_nadj_numerator_bar<DIM, 1><<<bc, TB, 0, s>>>(m, yb, nullptr, rel, sd.nbar);
      k_nadj_grad_cell<DIM, 1><<<bc, TB, 0, s>>>(m, yb, cv.wdg, nullptr, rel, B.ivb);
    }
    k_nadj_wdg_face<DIM><<<bf, TB, 0, s>>>(m, cv, sd.nbar, B.Fb, B.dpart);
    k_nadj_wdg_cell<DIM><<<bc, TB, 0, s>>>(m, cv, B.dpart, B.Cb);
  }
  if (npsi && (cv.lim_km > 0.0 || cv.lim_ks > 0.0))
    k_nadj_limiter<DIM, TURB><<<bc, TB, 0, s>>>(m, state, fw.G, cv.lim_km, cv.lim_ks, aw.psib,
                                                B.Vb, limxc, limxf, ncf);
  k_nadj_cell_chain<DIM, TURB><<<bc, TB, 0, s>>>(m, cv, B.Cb, B.ivb, B.wdf, cs->wnear, B.Vb, B.xcb,
                                                 B.wcon);
  if (npsi) k_nadj_centroid_gather<DIM><<<bc, TB, 0, s>>>(m, recxc, limxc, B.xcb);
  if constexpr (TURB)
    k_nadj_wall_face<DIM><<<bf, TB, 0, s>>>(m, na->wall_ptr, na->wall_cell, B.wcon, B.xfb);
  k_nadj_factors<DIM><<<bf, TB, 0, s>>>(m, B.Fb, B.nbt, B.xfb, B.xcpart);
  k_nadj_xc_gather<DIM><<<bc, TB, 0, s>>>(m, B.xcpart, B.xcb);
  k_nadj_cell_geom<DIM><<<bc, TB, 0, s>>>(m, B.Vb, B.xcb, B.cfA, B.cfN, B.cfX, ncf);
  k_nadj_cf_gather<DIM><<<bf, TB, 0, s>>>(m, B.Fb, B.cfA, B.cfN, B.cfX, npsi ? limxf : nullptr, ncf,
                                          B.Ab, B.nbt, B.xfb);
  k_nadj_face_geom<DIM><<<bf, TB, 0, s>>>(m, B.Ab, B.nbt, B.xfb, B.nodepart);
  k_nadj_nodes<<<fv_blocks(M->nn, 256), 256, 0, s>>>(M->nn, DIM, na->node_ptr, na->node_ent,
                                                    B.nodepart, dnodes);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

}  // namespace

int fv_case_node_vjp(FvCase* cs, const double* state, const double* w, double* dnodes,
                     cudaStream_t s) {
  if (cs->wd_external) {
    fv_set_error("fv_node_vjp: the wall distance was set by the caller (fv_case_set_wall_distance), "
                 "so its dependence on the nodes is unknown here");
    return FV_ERR_ARG;
  }
  int rc = nadj_setup(cs, s);
  if (rc != FV_OK) return rc;
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2)
    return turb ? node_vjp<2, true>(cs, state, w, dnodes, s) : node_vjp<2, false>(cs, state, w, dnodes, s);
  return turb ? node_vjp<3, true>(cs, state, w, dnodes, s) : node_vjp<3, false>(cs, state, w, dnodes, s);
}

void fv_node_adjoint_free(FvCase* cs) {
  NodeAdjoint* na = cs->nadj;
  if (!na) return;
  cudaFree(na->dual_work);
  cudaFree(na->buf);
  cudaFree(na->node_ptr);
  cudaFree(na->node_ent);
  cudaFree(na->wall_ptr);
  cudaFree(na->wall_cell);
  cudaFree(na->sweep);
  cudaFree(na->rec);
  delete na;
  cs->nadj = nullptr;
}

// ------------------------------------------------------------------------ face-flux functionals
// J = sum_f sum_q w_qf FL_q(f), optionally less the pressure part sum_i w_if p_f A_f n_if on
// boundary faces (the viscous, "wall shear" force): the outlet mass flux (w = 1 on the
// continuity flux of the outlet faces) and the wall shear force (w = 1 on a momentum component of
// the wall faces) of the 3D channel's adjoint objectives.  Value, dJ/dstate (the state adjoint
// with w as an extra face-flux cotangent), the parameter partials (forward tangents of the face
// fluxes) and dJ/dnodes (the mesh-coordinate adjoint with the same extra cotangent).
namespace {

constexpr int kFnBlocks = 304;

__global__ void k_face_in(int nf, int nfld, const int* face_old, const double* w_ref,
                          double* w_int) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int r = face_old[f];
  for (int q = 0; q < nfld; ++q) w_int[(long)q * nf + f] = w_ref[(long)q * nf + r];
}

template <class T>
__device__ __forceinline__ double part_of(const T& x, bool tangent);
template <>
__device__ __forceinline__ double part_of<double>(const double& x, bool) { return x; }
template <>
__device__ __forceinline__ double part_of<Dual>(const Dual& x, bool tangent) {
  return tangent ? x.d : x.v;
}

template <int DIM, bool TURB, class T>
__global__ void __launch_bounds__(256) k_functional_partial(MeshView m, CaseView cv,
                                                            const double* state, const double* w,
                                                            const T* FL, int viscous, int tangent,
                                                            double* part) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  __shared__ double red[256];
  const int nf = m.nf;
  double acc = 0.0;
  for (long f = (long)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (long)gridDim.x * blockDim.x) {
    double a = 0.0;
    for (int q = 0; q < NF; ++q) {
      const double wq = w[(long)q * nf + f];
      if (wq != 0.0) a += wq * part_of(FL[(long)q * nf + f], tangent != 0);
    }
    if (viscous && !tangent && f >= m.nfi) {
      const int o = m.owner[f];
      const double pf = bpress(cv, (int)f, cv.fkind[f], state[(long)L::P * m.nc + o]);
      for (int i = 0; i < DIM; ++i)
        a -= w[(long)i * nf + f] * pf * m.area[f] * m.normal[(long)i * nf + f];
    }
    acc += a;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_functional_final(int nparts, const double* part, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = 0.0;
  for (int i = 0; i < nparts; ++i) acc += part[i];
  *out = acc;
}

// d(pressure part)/d(owner pressure) on boundary faces whose pressure is the owner's.
template <int DIM, bool TURB>
__global__ void k_functional_pressure_state(MeshView m, CaseView cv, const double* w,
                                            double* dstate) {
  using L = Layout<DIM, TURB>;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nf = m.nf;
  double acc = 0.0;
  for (int i = m.cf_ptr[c]; i < m.cf_ptr[c + 1]; ++i) {
    const int f = (int)(m.cf_face[i] & ~FV_NB_BIT);
    const signed char kind = cv.fkind[f];
    if (f < m.nfi || kind < 0 || kind > 2) continue;
    for (int j = 0; j < DIM; ++j) acc += w[(long)j * nf + f] * m.area[f] * m.normal[(long)j * nf + f];
  }
  dstate[(long)L::P * m.nc + c] -= acc;
}

template <int DIM, bool TURB>
int face_functional(FvCase* cs, const double* state, const double* wref, int viscous,
                    double* value, double* dstate, double* dparams, double* dnodes,
                    cudaStream_t s) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  const MeshView& m = cs->mesh->view;
  const CaseView& cv = cs->view;
  const long nc = m.nc, nf = m.nf, n = (long)NF * nc;
  if (!cs->flx) FV_CUDA_TRY(cudaMalloc(&cs->flx, sizeof(double) * ((size_t)NF * nf + n)));
  if (!cs->red) FV_CUDA_TRY(cudaMalloc(&cs->red, sizeof(double) * kFnBlocks));
  double* zeros = cs->flx + (long)NF * nf;
  FV_CUDA_TRY(cudaMemsetAsync(zeros, 0, sizeof(double) * n, s));
  k_face_in<<<fv_blocks(nf, 256), 256, 0, s>>>((int)nf, NF, cs->mesh->face_old, wref, cs->flx);
  // value
  int rc = fv_case_run(cs, state, nullptr, FV_TAN_NONE, cs->tmp, nullptr, s);
  if (rc != FV_OK) return rc;
  {
    Work<double> fw = work_layout<double, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
    k_functional_partial<DIM, TURB, double><<<kFnBlocks, 256, 0, s>>>(m, cv, state, cs->flx, fw.FL,
                                                                      viscous, 0, cs->red);
    k_functional_final<<<1, 32, 0, s>>>(kFnBlocks, cs->red, value);
  }
  // parameter partials at fixed state
  if (dparams) {
    const int kinds[2] = {FV_TAN_MU, FV_TAN_INLET};
    for (int i = 0; i < 2; ++i) {
      rc = fv_case_run(cs, state, nullptr, kinds[i], nullptr, cs->tmp2, s);
      if (rc != FV_OK) return rc;
      cs->fwd_valid = 0;  // the workspace is about to hold a dual-number pass
      Work<Dual> dw = work_layout<Dual, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
      k_functional_partial<DIM, TURB, Dual><<<kFnBlocks, 256, 0, s>>>(m, cv, state, cs->flx, dw.FL,
                                                                      0, 1, cs->red);
      k_functional_final<<<1, 32, 0, s>>>(kFnBlocks, cs->red, dparams + i);
    }
  }
  // state partial: the adjoint with no residual cotangent and w on the face fluxes
  cs->flx_active = true;
  cs->flx_viscous = viscous != 0;
  rc = run_vjp<DIM, TURB>(cs, state, zeros, nullptr, dstate, s);
  if (rc == FV_OK && viscous)
    k_functional_pressure_state<DIM, TURB><<<fv_blocks(nc, 128), 128, 0, s>>>(m, cv, cs->flx, dstate);
  if (rc == FV_OK && dnodes) rc = fv_case_node_vjp(cs, state, zeros, dnodes, s);
  cs->flx_active = false;
  cs->flx_viscous = false;
  if (rc != FV_OK) return rc;
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

}  // namespace

int fv_case_face_functional(FvCase* cs, const double* state, const double* weights_ref,
                            int viscous_only, double* value, double* dstate, double* dparams,
                            double* dnodes, cudaStream_t s) {
  const int dim = cs->mesh->dim;
  const bool turb = cs->desc.turbulent != 0;
  if (dim == 2)
    return turb ? face_functional<2, true>(cs, state, weights_ref, viscous_only, value, dstate, dparams, dnodes, s)
                : face_functional<2, false>(cs, state, weights_ref, viscous_only, value, dstate, dparams, dnodes, s);
  return turb ? face_functional<3, true>(cs, state, weights_ref, viscous_only, value, dstate, dparams, dnodes, s)
              : face_functional<3, false>(cs, state, weights_ref, viscous_only, value, dstate, dparams, dnodes, s);
}
