// Reverse-mode (vector-Jacobian product) of the residual pipeline, hand-written.
//
// Included inside residual.cu's anonymous namespace: it reuses the forward helpers (SST wall
// functions, boundary closures, Layout) and the forward workspace (G, closure fields, momentum-
// diagonal coefficients, d) that a double-precision forward pass leaves behind.
//
// Given w = dL/dR, the kernels accumulate dL/dstate backwards through the stages
//   a_sum      cell  replaced rows (pressure pin, omega wall fixation) and the SST sources
//                    -> effective flux cotangents Wt, state / closure / gradient adjoints
//   a_flux     cell  adjoint of the face fluxes (Rhie-Chow mass flux, diffusion, pressure,
//                    upwind advection, k / omega transport) for this cell's side of each face
//   a_apcoef   cell  adjoint of a_P through d = V / a_P and the face coefficients
//   a_closure  cell  adjoint of the SST closure (strain, wall blends, F1, F2, nu_t, shear rate)
//   a_grad     cell  adjoint of the compact Green-Gauss gradients; writes dL/dstate
// Every accumulation is a per-cell sum over the cell's faces in ascending order (deterministic,
// no atomics).  Subgradients follow the forward pass: a max / min tie splits the cotangent in
// half (JAX's rule), safe_sqrt and the k >= 0 clamps have zero derivative where clamped.

// d max(x, 0) / dx with the tie rule.
__device__ __forceinline__ double dpos(double x) { return x > 0.0 ? 1.0 : (x == 0.0 ? 0.5 : 0.0); }
// Split the cotangent `bar` of max(a, b) (or min with `is_min`) onto a and b.
__device__ __forceinline__ void split_ext(double a, double b, double bar, bool is_min, double* abar,
                                          double* bbar) {
  bool pick_a = is_min ? a < b : a > b;
  bool pick_b = is_min ? a > b : a < b;
  if (pick_a) {
    *abar += bar;
  } else if (pick_b) {
    *bbar += bar;
  } else {
    *abar += 0.5 * bar;
    *bbar += 0.5 * bar;
  }
}

struct AdjWork {
  double* Wt;    // (NF, nc) effective flux-sum cotangent (0 on replaced rows)
  double* sb;    // (NF, nc) state adjoint (accumulated)
  double* Gb;    // (NF, D, nc) gradient adjoint
  double* dcob;  // (nc) d-coefficient adjoint
  double* clb;   // (4, nc) strain, F1, nu_t, shear-rate adjoints
  double* Gwib;  // (D, nc) imposed omega-gradient adjoint
  double* Gb2;   // (NF, D, nc) second iterate cotangent of the corrected-gradient sweeps
  double* Bb;    // (NF, D, nc) cotangent of the corrected scheme's right-hand side B phi
  const double* FLx;  // (NF, nf) extra face-flux cotangent (a face-flux functional), or null
  const double* psi;  // (NA, nc) forward slope limiters (limited upwind), or null
  double* psib;       // (NA, nc) their cotangents
  double* lnb;        // (2, NA, nf) limiter cotangent to the other cell of each face
};

// Gradient of advected field q at cell cu dotted with (x_f - x_cu): the limited reconstruction's
// increment (the forward pass's upwind_rec without psi).
template <int DIM>
__device__ __forceinline__ double rec_dot(const MeshView& m, const double* G, int q, int f, int cu) {
  const int nc = m.nc, nf = m.nf;
  double d = G[((long)q * DIM) * nc + cu] * (m.xf[f] - m.xc[cu]);
#pragma unroll
  for (int j = 1; j < DIM; ++j)
    d = d + G[((long)q * DIM + j) * nc + cu] * (m.xf[(long)j * nf + f] - m.xc[(long)j * nc + cu]);
  return d;
}

// ---------------------------------------------------------------- a_sum
template <int DIM, bool TURB>
__device__ __forceinline__ void a_sum_at(const int c, MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                             const double* W, const double* cl, const double* G,
                                             const double* Gwi, AdjWork aw) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  if (c >= m.nc) return;
  const int nc = m.nc;
  double wr[NF], sb[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    wr[q] = W[(long)q * nc + c];
    sb[q] = 0.0;
  }
  if (c == cv.pin) {
    sb[L::P] += wr[L::P];
    wr[L::P] = 0.0;
  }
  double Sb = 0.0, F1b = 0.0, ntb = 0.0, shb = 0.0;
  double gkb[DIM], gwib[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) gkb[j] = gwib[j] = 0.0;
  if (TURB) {
    const double V = m.vol[c];
    const double k = st((long)L::K * nc + c), w = st((long)L::W * nc + c);
    const double S = cl[c], F1 = cl[(long)nc + c], nut = cl[2L * nc + c], shear = cl[3L * nc + c];
    const double nu = par.nu;
    const double d = cv.wd[c];
    const bool wall = cv.wcell[c] != 0;
    const Dual kd{k, 1.0};
    const Dual nud{nu, 0.0};
    // ---- omega row
    double Ww = wr[L::W];
    if (wall) {
      // R_w = w - omega_wall(nu, d, k), or log(w / omega_wall) for a log-solved omega: the
      // flux sum and the sources are overwritten
      Dual ow = omega_wall(nud, d, kd);
      if (cv.log_w) {
        sb[L::W] += Ww / w;
        sb[L::K] += -Ww * ow.d / ow.v;
      } else {
        sb[L::W] += Ww;
        sb[L::K] += -Ww * ow.d;
      }
      Ww = 0.0;
      wr[L::W] = 0.0;
    }
    if (Ww != 0.0) {
      const double alpha = F1 * ALPHA_1 + (1.0 - F1) * ALPHA_2;
      const double kp = fmax(k, 0.0);
      const double num = PROD_RATIO * BETA_STAR * kp * w;
      const double den = fmax(nut, NUT_FLOOR);
      const double iden = 1.0 / den;
      const double cap = num * iden;
      const double S2 = S * S;
      const double mn = fmin(S2, cap);
      // R_w -= alpha * min(S^2, cap) * V
      const double mbar = -Ww * alpha * V;
      F1b += -Ww * mn * V * (ALPHA_1 - ALPHA_2);
      double S2b = 0.0, capb = 0.0;
      split_ext(S2, cap, mbar, true, &S2b, &capb);
      Sb += S2b * 2.0 * S;
      double numb = capb * iden, denb = -capb * cap * iden;
      double nutb_f = 0.0, flb = 0.0;
      split_ext(nut, NUT_FLOOR, denb, false, &nutb_f, &flb);
      ntb += nutb_f;
      sb[L::K] += numb * PROD_RATIO * BETA_STAR * w * dpos(k);
      sb[L::W] += numb * PROD_RATIO * BETA_STAR * kp;
      // R_w += beta * w^2 * V
      const double beta = F1 * BETA_1 + (1.0 - F1) * BETA_2;
      F1b += Ww * w * w * V * (BETA_1 - BETA_2);
      sb[L::W] += Ww * beta * 2.0 * w * V;
      // R_w -= cross * V,  cross = 2 (1 - F1) sigma_w2 (gk . gwi) / w
      double dkw = 0.0;
      double gk[DIM], gwi[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        gk[j] = G[((long)L::K * DIM + j) * nc + c];
        gwi[j] = Gwi[(long)j * nc + c];
        dkw += gk[j] * gwi[j];
      }
      const double iw = 1.0 / w;
      const double cross = 2.0 * (1.0 - F1) * SIGMA_W2 * dkw * iw;
      const double crb = -Ww * V;
      F1b += crb * (-2.0 * SIGMA_W2 * dkw * iw);
      const double dotb = crb * 2.0 * (1.0 - F1) * SIGMA_W2 * iw;
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        gkb[j] += dotb * gwi[j];
        gwib[j] += dotb * gk[j];
      }
      sb[L::W] += crb * (-cross * iw);
    }
    // ---- k row: R_k -= lim * V;  R_k += beta* k weff V
    const double Wk = wr[L::K];
    if (Wk != 0.0) {
      const double kp = fmax(k, 0.0);
      const double prod = nut * (S * S);
      const double limit = PROD_RATIO * BETA_STAR * kp * w;
      const double lim0 = fmin(prod, limit);
      double weff = w;
      const double limb = -Wk * V;
      double lim0b = limb;
      if (wall) {
        Dual lw = wall_weight(nud, d, kd);
        Dual ntw = nut_wall(nud, d, kd);
        Dual ls = log_shear(d, kd);
        const double tau = (nu + ntw.v) * shear;
        const double pw = tau * ls.v;
        lim0b = (1.0 - lw.v) * limb;
        const double lwb = (pw - lim0) * limb;
        const double pwb = lw.v * limb;
        const double taub = pwb * ls.v;
        sb[L::K] += lwb * lw.d + pwb * tau * ls.d + taub * shear * ntw.d;
        shb += taub * (nu + ntw.v);
        Dual ow = omega_wall(nud, d, kd);
        weff = ow.v;
        const double weffb = Wk * BETA_STAR * k * V;
        sb[L::K] += weffb * ow.d;
      } else {
        sb[L::W] += Wk * BETA_STAR * k * V;
      }
      sb[L::K] += Wk * BETA_STAR * weff * V;
      double prodb = 0.0, limitb = 0.0;
      split_ext(prod, limit, lim0b, true, &prodb, &limitb);
      ntb += prodb * S * S;
      Sb += prodb * 2.0 * nut * S;
      sb[L::K] += limitb * PROD_RATIO * BETA_STAR * w * dpos(k);
      sb[L::W] += limitb * PROD_RATIO * BETA_STAR * kp;
    }
  }
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    aw.Wt[(long)q * nc + c] = wr[q];
    aw.sb[(long)q * nc + c] = sb[q];
#pragma unroll
    for (int j = 0; j < DIM; ++j) aw.Gb[((long)q * DIM + j) * nc + c] = 0.0;
  }
  if (TURB) {
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      aw.Gb[((long)L::K * DIM + j) * nc + c] = gkb[j];
      aw.Gwib[(long)j * nc + c] = gwib[j];
    }
    aw.clb[c] = Sb;
    aw.clb[(long)nc + c] = F1b;
    aw.clb[2L * nc + c] = ntb;
    aw.clb[3L * nc + c] = shb;
  }
  aw.dcob[c] = 0.0;
}

template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) a_sum(MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                             const double* W, const double* cl, const double* G,
                                             const double* Gwi, AdjWork aw) {
  a_sum_at<DIM, TURB>(stage_cell(m, cv), m, cv, st, par, W, cl, G, Gwi, aw);
}

// momentum-normal flux mn(f) = sum_j n_j ((rho u_j)_f + (rho grad u_j)_f . skew) -- its partial
// derivatives are n_j w rho (u) and n_j w rho skew_q (grad u), w = 1 - g (owner) or g (neighbour).
template <int DIM>
__device__ __forceinline__ void mn_adjoint(const MeshView& m, int f, double wgt, double rho,
                                           double mnb, double* ub, double* Gub /*[DIM][DIM]*/) {
  const int nf = m.nf;
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    const double nj = m.normal[(long)j * nf + f];
    const double t = mnb * nj * wgt * rho;
    ub[j] += t;
#pragma unroll
    for (int q = 0; q < DIM; ++q) Gub[j * DIM + q] += t * m.skew[(long)q * nf + f];
  }
}

// ---------------------------------------------------------------- a_flux
// Forward relations reversed here (interior face, o = owner, n = neighbour, w_o = 1 - g, w_n = g):
//   mdot = me - rho A dhat damping,  dhat = nn2 (w_o d_o + w_n d_n),
//   damping = ((p_n - p_o) - gpf . dvec) / nd,  gpf = w_o gp_o + w_n gp_n,  pf = lerp(p) + gpf . skew
//   F_i = pf n_i A - c (u_n - u_o + G_n . tN - G_o . tP) + mdot upwind(u),  c = m_o m_n A / den,
//   den = dpn m_n - m_o dnn  (m = mu + rho nu_t);  F_p = mdot;
//   F_s = (mdot / rho) upwind(phi) - c_s (phi_n - phi_o + ...), c_s from the cell diffusivities.
template <int DIM, bool TURB, bool FLX = false, bool LIM = false>
__device__ __forceinline__ void a_flux_at(const int c, MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                              const double* G, const double* cl, const double* dco,
                                              const double* me, const double* aux, AdjWork aw) {
  using AX = Aux<DIM, TURB>;
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const double rho = cv.rho, irho = 1.0 / cv.rho;
  const double nu = par.nu;
  double sb[NF], Gb[NF][DIM];
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    sb[q] = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) Gb[q][j] = 0.0;
  }
  double dcb = 0.0, F1b = 0.0, ntb = 0.0;
  constexpr int NA = DIM + (TURB ? 2 : 0);
  double psb[NA];
#pragma unroll
  for (int a = 0; a < NA; ++a) psb[a] = 0.0;
  // this cell's share of a limited reconstruction it is the upwind cell of: t = the cotangent of
  // the reconstructed face value
  auto rec_adj = [&](int a, int q, int f, double t) {
    const double ps = aw.psi[(long)a * nc + c];
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const double dx = m.xf[(long)j * nf + f] - m.xc[(long)j * nc + c];
      Gb[q][j] += t * ps * dx;
    }
    psb[a] += t * rec_dot<DIM>(m, G, q, f, c);
  };
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int it = b; it < e; ++it) {
    const unsigned ent = m.cf_face[it];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
    const int o = m.owner[f];
    const double A = m.area[f];
    double nrm[DIM], tP[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      nrm[j] = m.normal[(long)j * nf + f];
      tP[j] = m.tP[(long)j * nf + f];
    }
    const double mo = TURB ? par.mu + rho * cl[2L * nc + o] : (cv.mu_cell ? cv.mu_cell[o] : par.mu);
    const double po = st((long)L::P * nc + o);
    if (f < m.nfi) {
      const int n = m.nb[f];
      const double g = m.g[f];
      const double wgt = isnb ? g : 1.0 - g;  // this side's interpolation weight
      // this side's correction vector: tP on the owner side, tN on the neighbour side (the two
      // sides run one code path on selected operands, so a warp mixing them does not diverge)
      double tS[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) tS[j] = isnb ? m.tN[(long)j * nf + f] : tP[j];
      double FLb[NF];
#pragma unroll
      for (int q = 0; q < NF; ++q) {
        FLb[q] = aw.Wt[(long)q * nc + o] - aw.Wt[(long)q * nc + n];
        if constexpr (FLX) FLb[q] += aw.FLx[(long)q * nf + f];
      }
      // forward face intermediates kept by k_flux
      const double mdot = aux[0L * nf + f];
      const double damping = aux[1L * nf + f];
      const double dhat = aux[2L * nf + f];
      const double cmo = aux[3L * nf + f];
      const double inv_nd = m.inv_nd[f];
      const bool out = mdot >= 0.0;
      // reverse
      double mdotb = FLb[L::P];
      double pfb = 0.0, cb = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        const double uo = st((long)i * nc + o), un = st((long)i * nc + n);
        const double cpn = aux[(long)(AX::CPN + i) * nf + f];
        const double fb = FLb[i];
        double up = out ? uo : un;
        if constexpr (LIM) {
          if (cv.rec_mom) {
            const int cu = out ? o : n;
            up += aw.psi[(long)i * nc + cu] * rec_dot<DIM>(m, G, i, f, cu);
            if (out != isnb) rec_adj(i, i, f, fb * mdot);
          }
        }
        mdotb += fb * up;
        // F_i = ... - c cpn: +k1 on the owner's state and gradient, -k1 on the neighbour's; the
        // upwind term goes to the upwind side
        const double k1 = isnb ? -(fb * cmo) : fb * cmo;
        cb -= fb * cpn;
        sb[i] += k1 + (out != isnb ? fb * mdot : 0.0);
#pragma unroll
        for (int j = 0; j < DIM; ++j) Gb[i][j] += k1 * tS[j];
        pfb += fb * nrm[i] * A;
      }
      if (TURB) ntb += cb * aux[(isnb ? 5L : 4L) * nf + f] * rho;
      // pf = lerp(p) + gpf . skew
      double gpfb[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) gpfb[j] = pfb * m.skew[(long)j * nf + f];
      sb[L::P] += wgt * pfb;
      if (TURB) {
        const double vflux = mdot * irho;
        const bool vout = vflux >= 0.0;
        const double F1X = cl[(long)nc + (isnb ? n : o)], ntX = cl[2L * nc + (isnb ? n : o)];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int q = s == 0 ? L::K : L::W;
          const double in = s == 0 ? SIGMA_K1 : SIGMA_W1, ou = s == 0 ? SIGMA_K2 : SIGMA_W2;
          const long b0 = AX::S0 + 4 * s;
          const double cs_ = aux[b0 * nf + f];
          const double cpn = aux[(b0 + 3) * nf + f];
          const double phio = st((long)q * nc + o), phin = st((long)q * nc + n);
          const double fb = FLb[q];
          double up = vout ? phio : phin;
          if constexpr (LIM) {
            if (cv.rec_sca) {
              const int cu = vout ? o : n;
              up += aw.psi[(long)(DIM + s) * nc + cu] * rec_dot<DIM>(m, G, q, f, cu);
              if (vout != isnb) rec_adj(DIM + s, q, f, fb * vflux);
            }
          }
          mdotb += fb * up * irho;
          const double k1 = isnb ? -(fb * cs_) : fb * cs_;
          sb[q] += k1 + (vout != isnb ? fb * vflux : 0.0);
#pragma unroll
          for (int j = 0; j < DIM; ++j) Gb[q][j] += k1 * tS[j];
          const double gXb = -fb * cpn * aux[(b0 + (isnb ? 2 : 1)) * nf + f];
          // gamma_X = nu + (sig_out + F1 (sig_in - sig_out)) nu_t
          F1b += gXb * (in - ou) * ntX;
          ntb += gXb * (ou + F1X * (in - ou));
        }
      }
      // mdot = me - rho A dhat damping
      const double dhatb = -mdotb * (rho * A) * damping;
      const double dampb = -mdotb * (rho * A) * dhat;
      sb[L::P] += (isnb ? dampb : -dampb) * inv_nd;
#pragma unroll
      for (int j = 0; j < DIM; ++j) gpfb[j] -= dampb * inv_nd * m.dvec[(long)j * nf + f];
#pragma unroll
      for (int j = 0; j < DIM; ++j) Gb[L::P][j] += wgt * gpfb[j];
      dcb += dhatb * m.nn2[f] * wgt;
      // me = rho A (sum_j n_j lerp(u_j) + sum_jq ns_jq lerp(G_jq))
      const double meb = mdotb * rho * A * wgt;
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        sb[j] += meb * nrm[j];
#pragma unroll
        for (int q = 0; q < DIM; ++q) Gb[j][q] += meb * m.ns[(long)(j * DIM + q) * nf + f];
      }
    } else {
      // boundary face: this cell is the owner
      const signed char kind = cv.fkind[f];
      double FLb[NF];
#pragma unroll
      for (int q = 0; q < NF; ++q) {
        FLb[q] = aw.Wt[(long)q * nc + o];
        if constexpr (FLX) FLb[q] += aw.FLx[(long)q * nf + f];
      }
      double uo[DIM], bu[DIM];
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        uo[j] = st((long)j * nc + o);
        bu[j] = bvel(cv, nf, f, j, kind, uo[j], par);
      }
      double mdot = 0.0, dh = 0.0, compact = 0.0, interp = 0.0;
      if (kind == 2) {
        double un = bu[0] * nrm[0];
#pragma unroll
        for (int j = 1; j < DIM; ++j) un += bu[j] * nrm[j];
        mdot = (rho * A) * un;
      } else if (kind == 3) {
        double un = uo[0] * nrm[0];
        interp = G[((long)L::P * DIM) * nc + o] * nrm[0];
#pragma unroll
        for (int j = 1; j < DIM; ++j) {
          un += uo[j] * nrm[j];
          interp += G[((long)L::P * DIM + j) * nc + o] * nrm[j];
        }
        dh = m.nn2[f] * dco[o];
        compact = (cv.fp[f] - po) * m.inv_nd[f];
        mdot = (rho * A) * (un - dh * (compact - interp));
      }
      double gbv = mo;
      double dgb_dk = 0.0;  // d gamma_b / d k_owner (SST wall faces)
      bool gb_is_mo = true;
      if (TURB && (kind == 0 || kind == 1)) {
        gb_is_mo = false;
        if (cv.swall[f]) {
          Dual nw = nut_wall(Dual{nu, 0.0}, cv.wd[o], Dual{st((long)L::K * nc + o), 1.0});
          gbv = par.mu + rho * nw.v;
          dgb_dk = rho * nw.d;
        } else {
          gbv = cv.mu_cell ? cv.mu_cell[o] : par.mu;
        }
      }
      const double Ad = A * m.inv_dpn[f];
      const bool out = mdot >= 0.0;
      double mdotb = FLb[L::P], pfb = 0.0, gbb = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        double cp = 0.0;
#pragma unroll
        for (int j = 0; j < DIM; ++j) cp += G[((long)i * DIM + j) * nc + o] * tP[j];
        const double num = bu[i] - uo[i] - cp;
        const double fb = FLb[i];
        double up = out ? uo[i] : bu[i];
        if constexpr (LIM) {
          if (out && cv.rec_mom) {
            up += aw.psi[(long)i * nc + o] * rec_dot<DIM>(m, G, i, f, o);
            rec_adj(i, i, f, fb * mdot);
          }
        }
        mdotb += fb * up;
        const double numb = -fb * gbv * Ad;
        gbb -= fb * num * Ad;
        const double bub = numb + (!out ? fb * mdot : 0.0);
        sb[i] += -numb + (out ? fb * mdot : 0.0);
        if (kind == 3) sb[i] += bub;
#pragma unroll
        for (int j = 0; j < DIM; ++j) Gb[i][j] -= numb * tP[j];
        pfb += fb * nrm[i] * A;
      }
      if (kind >= 0 && kind <= 2) sb[L::P] += pfb;
      if (TURB) {
        if (gb_is_mo) ntb += gbb * rho;
        else sb[L::K] += gbb * dgb_dk;
        const double vflux = mdot * irho;
        const bool vout = vflux >= 0.0;
        const double F1o = cl[(long)nc + o], nto = cl[2L * nc + o];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int q = s == 0 ? L::K : L::W;
          const double in = s == 0 ? SIGMA_K1 : SIGMA_W1, ou = s == 0 ? SIGMA_K2 : SIGMA_W2;
          const double go = cl[(4L + s) * nc + o];
          const double phio = st((long)q * nc + o);
          double cp = 0.0;
#pragma unroll
          for (int j = 0; j < DIM; ++j) cp += G[((long)q * DIM + j) * nc + o] * tP[j];
          const signed char sk = s == 0 ? cv.kkind[f] : cv.wkind[f];
          const double sval = s == 0 ? cv.kval[f] : cv.wval[f];
          const double bphi = bscalar(sk, sval, phio, cp);
          double gface = go, wwd = 0.0, wwv = 0.0;
          const bool wallk = s == 0 && cv.swall[f];
          if (wallk) {
            Dual ww = wall_weight(Dual{nu, 0.0}, cv.wd[o], Dual{phio, 1.0});
            wwv = ww.v;
            wwd = ww.d;
            gface = (1.0 - wwv) * go;
          }
          const double num = bphi - phio - cp;
          const double fb = FLb[q];
          double up = vout ? phio : bphi;
          if constexpr (LIM) {
            if (vout && cv.rec_sca) {
              up += aw.psi[(long)(DIM + s) * nc + o] * rec_dot<DIM>(m, G, q, f, o);
              rec_adj(DIM + s, q, f, fb * vflux);
            }
          }
          mdotb += fb * up * irho;
          const double numb = -fb * gface * Ad;
          const double gfb = -fb * num * Ad;
          const double bphib = numb + (!vout ? fb * vflux : 0.0);
          sb[q] += -numb + (vout ? fb * vflux : 0.0);
#pragma unroll
          for (int j = 0; j < DIM; ++j) Gb[q][j] -= numb * tP[j];
          if (sk == 1) {
            sb[q] += bphib;
#pragma unroll
            for (int j = 0; j < DIM; ++j) Gb[q][j] += bphib * tP[j];
          }
          double gob = gfb;
          if (wallk) {
            gob = gfb * (1.0 - wwv);
            sb[L::K] -= gfb * go * wwd;
          }
          F1b += gob * (in - ou) * nto;
          ntb += gob * (ou + F1o * (in - ou));
        }
      }
      if (kind == 3) {
        const double base = mdotb * rho * A;
#pragma unroll
        for (int j = 0; j < DIM; ++j) sb[j] += base * nrm[j];
        dcb -= base * (compact - interp) * m.nn2[f];
        sb[L::P] += base * dh * m.inv_nd[f];
#pragma unroll
        for (int j = 0; j < DIM; ++j) Gb[L::P][j] += base * dh * nrm[j];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    aw.sb[(long)q * nc + c] += sb[q];
#pragma unroll
    for (int j = 0; j < DIM; ++j) aw.Gb[((long)q * DIM + j) * nc + c] += Gb[q][j];
  }
  aw.dcob[c] = dcb;
  if (TURB) {
    aw.clb[(long)nc + c] += F1b;
    aw.clb[2L * nc + c] += ntb;
  }
  if constexpr (LIM) {
#pragma unroll
    for (int a = 0; a < NA; ++a) aw.psib[(long)a * nc + c] = psb[a];
  }
}

template <int DIM, bool TURB, bool FLX = false, bool LIM = false>
__global__ void __launch_bounds__(128) a_flux(MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                              const double* G, const double* cl, const double* dco,
                                              const double* me, const double* aux, AdjWork aw) {
  a_flux_at<DIM, TURB, FLX, LIM>(stage_cell(m, cv), m, cv, st, par, G, cl, dco, me, aux, aw);
}

// ---------------------------------------------------------------- a_limiter
// Adjoint of the Venkatakrishnan limiters: psi of cell c depends on its own value and gradient and
// on its face neighbours' values (the stencil extrema); d psi / d(input) by dual numbers seeded on
// one input at a time (the forward formula, limiter_cell).  Own contributions go to the state and
// gradient cotangents; a neighbour's to lnb (per face and side), gathered by a_limiter_gather.
template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) a_limiter(MeshView m, Src<double> st, const double* G,
                                                 double Km, double Ks, AdjWork aw) {
  constexpr int NA = DIM + (TURB ? 2 : 0);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
#pragma unroll 1
  for (int a = 0; a < NA; ++a) {
    const int q = advected_field<DIM, TURB>(a);
    const double K = a < DIM ? Km : Ks;
    const double pb = aw.psib[(long)a * nc + c];
    if (!(K > 0.0)) {  // psi = 1: no dependence (the neighbour slots still need writing)
      for (int i = b; i < e; ++i) {
        const unsigned ent = m.cf_face[i];
        const int f = (int)(ent & ~FV_NB_BIT);
        if (f < m.nfi) aw.lnb[((long)((ent & FV_NB_BIT) ? NA : 0) + a) * nf + f] = 0.0;
      }
      continue;
    }
    // seeds: -1 = phi_c, 0..DIM-1 = grad_j, then the cell's faces (their other cell's phi)
    auto eval = [&](int seed_grad, int seed_cell) {
      auto phi = [&](int cell) {
        return Dual{st((long)q * nc + cell), cell == seed_cell ? 1.0 : 0.0};
      };
      auto grad = [&](int j) {
        return Dual{G[((long)q * DIM + j) * nc + c], j == seed_grad ? 1.0 : 0.0};
      };
      return limiter_cell<Dual, DIM>(m, c, K, phi, grad).d;
    };
    aw.sb[(long)q * nc + c] += pb * eval(-1, c);
#pragma unroll 1
    for (int j = 0; j < DIM; ++j) aw.Gb[((long)q * DIM + j) * nc + c] += pb * eval(j, -1);
    for (int i = b; i < e; ++i) {
      const unsigned ent = m.cf_face[i];
      const int f = (int)(ent & ~FV_NB_BIT);
      if (f >= m.nfi) continue;
      const bool isnb = (ent & FV_NB_BIT) != 0;
      const int other = isnb ? m.owner[f] : m.nb[f];
      // slot 0: the owner's limiter to the neighbour's value; slot 1: the neighbour's to the owner's
      aw.lnb[((long)(isnb ? NA : 0) + a) * nf + f] = pb * eval(-1, other);
    }
  }
}

template <int DIM, bool TURB>
__global__ void a_limiter_gather(MeshView m, AdjWork aw) {
  constexpr int NA = DIM + (TURB ? 2 : 0);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  double acc[NA];
#pragma unroll
  for (int a = 0; a < NA; ++a) acc[a] = 0.0;
  for (int i = m.cf_ptr[c]; i < m.cf_ptr[c + 1]; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    if (f >= m.nfi) continue;
    // this cell is the neighbour: the owner's limiter wrote slot 0; the owner: slot 1
    const long slot = (ent & FV_NB_BIT) ? 0 : NA;
#pragma unroll
    for (int a = 0; a < NA; ++a) acc[a] += aw.lnb[(slot + a) * nf + f];
  }
#pragma unroll
  for (int a = 0; a < NA; ++a)
    aw.sb[(long)advected_field<DIM, TURB>(a) * nc + c] += acc[a];
}

// ---------------------------------------------------------------- a_apcoef
// a_P(c) = sum of face coefficients; d = V / a_P  =>  abar = -dbar d^2 / V.
template <int DIM, bool TURB>
__device__ __forceinline__ void a_apcoef_at(const int c, MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                                const double* G, const double* cl, const double* dco,
                                                const double* me, const double* aux, AdjWork aw) {
  using L = Layout<DIM, TURB>;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const double rho = cv.rho;
  double ub[DIM], Gub[DIM * DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) ub[j] = 0.0;
#pragma unroll
  for (int j = 0; j < DIM * DIM; ++j) Gub[j] = 0.0;
  double ntb = 0.0, kb = 0.0;
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int it = b; it < e; ++it) {
    const unsigned ent = m.cf_face[it];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
    const int o = m.owner[f];
    const double A = m.area[f];
    const double abo = -aw.dcob[o] * dco[o] * dco[o] * m.inv_vol[o];
    const double mdot = me[f];
    double meb;
    if (f < m.nfi) {
      const int n = m.nb[f];
      const double g = m.g[f];
      const double abn = -aw.dcob[n] * dco[n] * dco[n] * m.inv_vol[n];
      meb = (abo * dpos(mdot) - abn * dpos(-mdot)) * (isnb ? g : 1.0 - g);
      if (TURB) {
        // the viscous conductance is the flux stage's c(m_o, m_n): its derivatives were kept
        ntb += rho * (abo + abn) * aux[(isnb ? 5L : 4L) * nf + f];
      }
    } else {
      const signed char kind = cv.fkind[f];
      const double vob = (kind >= 0 && kind <= 2) ? abo : 0.0;
      const double convb = (kind == 2 || kind == 3) ? abo : 0.0;
      meb = convb * dpos(mdot);
      if (TURB && vob != 0.0) {
        const double Ad = A * m.inv_nd[f];
        if (kind == 0 || kind == 1) {
          if (cv.swall[f]) {
            Dual nw = nut_wall(Dual{par.nu, 0.0}, cv.wd[o], Dual{st((long)L::K * nc + o), 1.0});
            kb += vob * Ad * rho * nw.d;
          }
        } else {
          ntb += vob * Ad * rho;
        }
      }
    }
    // me = rho A (sum_j n_j lerp(u_j) + sum_jq ns_jq lerp(G_jq)); meb already carries the weight
    const double t = meb * rho * A;
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      ub[j] += t * m.normal[(long)j * nf + f];
#pragma unroll
      for (int q = 0; q < DIM; ++q) Gub[j * DIM + q] += t * m.ns[(long)(j * DIM + q) * nf + f];
    }
  }
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    aw.sb[(long)j * nc + c] += ub[j];
#pragma unroll
    for (int q = 0; q < DIM; ++q) aw.Gb[((long)j * DIM + q) * nc + c] += Gub[j * DIM + q];
  }
  if (TURB) {
    aw.clb[2L * nc + c] += ntb;
    aw.sb[(long)L::K * nc + c] += kb;
  }
}

template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) a_apcoef(MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                                const double* G, const double* cl, const double* dco,
                                                const double* me, const double* aux, AdjWork aw) {
  a_apcoef_at<DIM, TURB>(stage_cell(m, cv), m, cv, st, par, G, cl, dco, me, aux, aw);
}

// ---------------------------------------------------------------- a_closure (SST)
template <int DIM>
__device__ __forceinline__ void a_closure_at(const int c, MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                                 const double* G, const double* cl, AdjWork aw) {
  using L = Layout<DIM, true>;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const double k = st((long)L::K * nc + c), w = st((long)L::W * nc + c);
  const double nu = par.nu;
  const double d = cv.wd[c];
  const bool wall = cv.wcell[c] != 0;
  double Sb = aw.clb[c], F1b = aw.clb[(long)nc + c], ntb = aw.clb[2L * nc + c];
  const double shb = aw.clb[3L * nc + c];
  double gu[DIM][DIM], gk[DIM], gw[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) gu[i][j] = G[((long)i * DIM + j) * nc + c];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    gk[j] = G[((long)L::K * DIM + j) * nc + c];
    gw[j] = G[((long)L::W * DIM + j) * nc + c];
  }
  // forward recomputation
  double sum = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      double sij = 0.5 * (gu[i][j] + gu[j][i]);
      sum += sij * sij;
    }
  const double S0 = 2.0 * sum > 0.0 ? sqrt(2.0 * sum) : 0.0;
  double S = S0;
  Dual wgt{0.0, 0.0}, ls{0.0, 0.0}, dwdd{0.0, 0.0}, dwdk{0.0, 0.0};
  if (wall) {
    const Dual kd{k, 1.0}, nud{nu, 0.0};
    wgt = wall_weight(nud, d, kd);
    ls = log_shear(d, kd);
    S = (1.0 - wgt.v) * S0 + wgt.v * ls.v;
    omega_wall_partials(nud, d, kd, &dwdd, &dwdk);
#pragma unroll
    for (int j = 0; j < DIM; ++j) gw[j] = cv.wdg[(long)j * nc + c] * dwdd.v + gk[j] * dwdk.v;
  }
  const double kp = fmax(k, 0.0);
  double dot_kw = gk[0] * gw[0];
#pragma unroll
  for (int j = 1; j < DIM; ++j) dot_kw += gk[j] * gw[j];
  const double iw = 1.0 / w, id = cv.inv_wd[c], id2 = cv.inv_wd2[c];
  const double cd0 = (2.0 * SIGMA_W2) * dot_kw * iw;
  const double cd = fmax(cd0, CROSS_FLOOR);
  const double icd = 1.0 / cd;
  const double sk = kp > 0.0 ? sqrt(kp) : 0.0;
  const double vt = (500.0 * id2) * nu * iw;
  const double c1 = sk * iw * (id / BETA_STAR);
  const double inner = fmax(c1, vt);
  const double c2 = (4.0 * SIGMA_W2 * id2) * kp * icd;
  const double arg1 = fmin(inner, c2);
  const double a1sq = arg1 * arg1;
  const double F1 = cl[(long)nc + c];   // tanh(arg1^4), kept by the forward closure
  const double a2 = 2.0 * c1;
  const double arg2 = fmax(a2, vt);
  const double F2 = cl[6L * nc + c];    // tanh(arg2^2)
  const double Mx = fmax(A1 * w, S * F2);
  const double iMx = 1.0 / Mx;
  // reverse: nut = A1 kp / M
  double kpb = ntb * A1 * iMx;
  const double Mb = -ntb * A1 * kp * iMx * iMx;
  double awb = 0.0, sfb = 0.0;
  split_ext(A1 * w, S * F2, Mb, false, &awb, &sfb);
  double wb = awb * A1;
  Sb += sfb * F2;
  const double F2b = sfb * S;
  const double arg2b = F2b * (1.0 - F2 * F2) * 2.0 * arg2;
  double a2b = 0.0, vtb = 0.0;
  split_ext(a2, vt, arg2b, false, &a2b, &vtb);
  // a2 = 2 c1
  double c1b = 2.0 * a2b;
  // F1 = tanh(arg1^4)
  const double arg1b = F1b * (1.0 - F1 * F1) * 4.0 * a1sq * arg1;
  double innerb = 0.0, c2b = 0.0;
  split_ext(inner, c2, arg1b, true, &innerb, &c2b);
  split_ext(c1, vt, innerb, false, &c1b, &vtb);
  // c1 = sk / (beta* w d), vt = 500 nu / (d^2 w)
  double skb = c1b * iw * (id / BETA_STAR);
  wb -= (c1b * c1 + vtb * vt) * iw;
  kpb += c2b * (4.0 * SIGMA_W2 * id2) * icd;
  const double cdb = -c2b * c2 * icd;
  double cd0b = 0.0, flb = 0.0;
  split_ext(cd0, CROSS_FLOOR, cdb, false, &cd0b, &flb);
  const double dotb = cd0b * (2.0 * SIGMA_W2) * iw;
  wb -= cd0b * cd0 * iw;
  double gkb[DIM], gwb[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    gkb[j] = dotb * gw[j];
    gwb[j] = dotb * gk[j] + aw.Gwib[(long)j * nc + c];
  }
  kpb += kp > 0.0 ? skb * 0.5 / sk : 0.0;
  double kb = kpb * dpos(k);
  double S0b = Sb;
  double ub[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) ub[j] = 0.0;
  if (wall) {
    S0b = Sb * (1.0 - wgt.v);
    const double wgtb = Sb * (ls.v - S0);
    const double lsb = Sb * wgt.v;
    kb += wgtb * wgt.d + lsb * ls.d;
    // imposed omega gradient: gw = wdg * dwdd(k) + gk * dwdk(k)
    double ddb = 0.0, dkb = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      ddb += gwb[j] * cv.wdg[(long)j * nc + c];
      dkb += gwb[j] * gk[j];
      gkb[j] += gwb[j] * dwdk.v;
      gwb[j] = 0.0;  // the reconstructed omega gradient does not reach an imposed cell
    }
    kb += ddb * dwdd.d + dkb * dwdk.d;
    // wall shear rate: sum(rate A) / sum(A), rate = |u - u_b| / d
    if (shb != 0.0) {
      double den = 0.0;
      const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
      for (int it = b; it < e; ++it) {
        const int f = (int)(m.cf_face[it] & ~FV_NB_BIT);
        if (f < m.nfi || !cv.swall[f]) continue;
        den += m.area[f];
      }
      for (int it = b; it < e; ++it) {
        const int f = (int)(m.cf_face[it] & ~FV_NB_BIT);
        if (f < m.nfi || !cv.swall[f]) continue;
        const signed char kind = cv.fkind[f];
        if (kind == 3) continue;  // zero-gradient velocity: slip identically zero
        double sl[DIM], s2 = 0.0;
#pragma unroll
        for (int j = 0; j < DIM; ++j) {
          const double u = st((long)j * nc + c);
          sl[j] = u - bvel(cv, nf, f, j, kind, u, par);
          s2 += sl[j] * sl[j];
        }
        if (s2 > 0.0) {
          const double rb = shb * m.area[f] / den;
          const double s2b = rb * 0.5 / (sqrt(s2) * d);
#pragma unroll
          for (int j = 0; j < DIM; ++j) ub[j] += s2b * 2.0 * sl[j];
        }
      }
    }
  }
  // S0 = safe_sqrt(2 sum s_ij^2)
  if (S0 > 0.0 && S0b != 0.0) {
    const double sumb = S0b / S0;  // d sqrt(2 sum) / d sum = 1 / S0
#pragma unroll
    for (int i = 0; i < DIM; ++i)
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        const double sij = 0.5 * (gu[i][j] + gu[j][i]);
        const double sijb = sumb * 2.0 * sij;
        aw.Gb[((long)i * DIM + j) * nc + c] += 0.5 * sijb;
        aw.Gb[((long)j * DIM + i) * nc + c] += 0.5 * sijb;
      }
  }
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    aw.Gb[((long)L::K * DIM + j) * nc + c] += gkb[j];
    aw.Gb[((long)L::W * DIM + j) * nc + c] += gwb[j];
    aw.sb[(long)j * nc + c] += ub[j];
  }
  aw.sb[(long)L::K * nc + c] += kb;
  aw.sb[(long)L::W * nc + c] += wb;
}

template <int DIM>
__global__ void __launch_bounds__(128) a_closure(MeshView m, CaseView cv, Src<double> st, Par<double> par,
                                                 const double* G, const double* cl, AdjWork aw) {
  a_closure_at<DIM>(stage_cell(m, cv), m, cv, st, par, G, cl, aw);
}

// ---------------------------------------------------------------- a_grad
// G_c = (1/V_c) sum_f (+-) S_f phi_f  =>  phib_f = S_f . (Gb_o / V_o - Gb_n / V_n), then each side
// takes its interpolation weight of phib_f.  The face pass forms phib once per face (into `pb`,
// (NF, nf)); the cell pass gathers it.
// ---------------------------------------------------------------- corrected-gradient sweeps
// Adjoint of the swept corrected Green-Gauss solve (gradient.py:618-705, 1122-1337).  Forward:
// X_0 = rel B phi / V, X_i = X_{i-1} + rel (B phi - V X_{i-1} + C X_{i-1}) / V.  Backward, with
// y = rel Xb / V per cell: Bb += y and Xb <- Xb - V y + C^T y, where
// (C^T y)_P += (1 - g) skew wb_f, (C^T y)_N += g skew wb_f, wb_f = S_f . (y_P - y_N).
template <int DIM, int NQ>
__global__ void __launch_bounds__(128) a_gg_skew(MeshView m, const double* Xb, double rel,
                                                 double* wb) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nfi) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f], n = m.nb[f];
  const double A = m.area[f];
  const double ro = rel * m.inv_vol[o], rn = rel * m.inv_vol[n];
  double S[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) S[j] = m.normal[(long)j * nf + f] * A;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j)
      acc += S[j] * (Xb[((long)q * DIM + j) * nc + o] * ro - Xb[((long)q * DIM + j) * nc + n] * rn);
    wb[(long)q * nf + f] = acc;
  }
}

template <int DIM, int NQ>
__global__ void __launch_bounds__(128) a_gg_sweep(MeshView m, const double* Xb, const double* wb,
                                                  double rel, bool first, double* Bb, double* Xbn) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  const double V = m.vol[c], r = rel * m.inv_vol[c];
  double acc[NQ][DIM];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const long k = ((long)q * DIM + j) * nc + c;
      const double x = Xb[k];
      const double y = x * r;
      Bb[k] = first ? y : Bb[k] + y;
      acc[q][j] = x - V * y;
    }
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    if (f >= m.nfi) continue;
    const double g = m.g[f];
    const double wgt = (ent & FV_NB_BIT) ? g : 1.0 - g;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const double t = wgt * wb[(long)q * nf + f];
#pragma unroll
      for (int j = 0; j < DIM; ++j) acc[q][j] += t * m.skew[(long)j * nf + f];
    }
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int j = 0; j < DIM; ++j) Xbn[((long)q * DIM + j) * nc + c] = acc[q][j];
}

// Runs the backward sweeps from aw.Gb; returns the cotangent of the first iterate (aw.Gb or
// aw.Gb2).  With fewer than two sweeps there is nothing to run and aw.Bb stays unused.
template <int DIM, int NQ>
const double* gg_sweeps_adjoint(const MeshView& m, int sweeps, double rel, const AdjWork& aw,
                                double* wface, cudaStream_t s) {
  constexpr int TB = 128;
  const int bc = fv_blocks(m.nc, TB), bfi = fv_blocks(m.nfi > 0 ? m.nfi : 1, TB);
  double* cur = aw.Gb;
  double* nxt = aw.Gb2;
  for (int it = 1; it < sweeps; ++it) {
    if (m.nfi > 0) a_gg_skew<DIM, NQ><<<bfi, TB, 0, s>>>(m, cur, rel, wface);
    a_gg_sweep<DIM, NQ><<<bc, TB, 0, s>>>(m, cur, wface, rel, it == 1, aw.Bb, nxt);
    double* t = cur;
    cur = nxt;
    nxt = t;
  }
  return cur;
}

// Face cotangents of the Green-Gauss face values: pb_f = S_f . (nb_P - nb_N) with nb the
// cotangent of the Green-Gauss numerator B phi, nb = rel Gb0 / V (+ Bb when swept).  Gb0 is the
// cotangent of the first gradient iterate (the gradient itself for the compact scheme).
template <int DIM, bool TURB>
__device__ __forceinline__ void a_grad_face_at(const int f, MeshView m, CaseView cv, AdjWork aw,
                                                   const double* Gb0, const double* Bb, double rel,
                                                   double* pb) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  const int o = m.owner[f];
  const double A = m.area[f];
  double S[DIM];
#pragma unroll
  for (int j = 0; j < DIM; ++j) S[j] = m.normal[(long)j * nf + f] * A;
  const double ivo = m.inv_vol[o];
  if (Bb || rel != 1.0) {
    const double ro = rel * ivo;
    const int n = f < m.nfi ? m.nb[f] : o;
    const double rn = rel * m.inv_vol[n];
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      double phib = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        const long ko = ((long)q * DIM + j) * nc + o;
        double nbo = Gb0[ko] * ro;
        if (Bb) nbo += Bb[ko];
        if (f < m.nfi) {
          const long kn = ((long)q * DIM + j) * nc + n;
          double nbn = Gb0[kn] * rn;
          if (Bb) nbn += Bb[kn];
          phib += S[j] * (nbo - nbn);
        } else {
          phib += S[j] * nbo;
        }
      }
      pb[(long)q * nf + f] = phib;
    }
    return;
  }
  if (f < m.nfi) {
    const int n = m.nb[f];
    const double ivn = m.inv_vol[n];
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      double phib = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j)
        phib += S[j] * (Gb0[((long)q * DIM + j) * nc + o] * ivo -
                        Gb0[((long)q * DIM + j) * nc + n] * ivn);
      pb[(long)q * nf + f] = phib;
    }
  } else {
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      double phib = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) phib += S[j] * Gb0[((long)q * DIM + j) * nc + o];
      pb[(long)q * nf + f] = phib * ivo;
    }
  }
}

template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) a_grad_face(MeshView m, CaseView cv, AdjWork aw,
                                                   const double* Gb0, const double* Bb, double rel,
                                                   double* pb) {
  a_grad_face_at<DIM, TURB>(blockIdx.x * blockDim.x + threadIdx.x, m, cv, aw, Gb0, Bb, rel, pb);
}

template <int DIM, bool TURB>
__device__ __forceinline__ void a_grad_at(const int c, MeshView m, CaseView cv, AdjWork aw, const double* pb,
                                              double* out) {
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  if (c >= m.nc) return;
  const int nc = m.nc, nf = m.nf;
  double acc[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q) acc[q] = aw.sb[(long)q * nc + c];
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int it = b; it < e; ++it) {
    const unsigned ent = m.cf_face[it];
    const int f = (int)(ent & ~FV_NB_BIT);
    if (f < m.nfi) {
      const double g = m.g[f];
      const double wgt = (ent & FV_NB_BIT) ? g : 1.0 - g;
#pragma unroll
      for (int q = 0; q < NF; ++q) acc[q] += wgt * pb[(long)q * nf + f];
    } else {
      // leading-order boundary values depend on the owner value: outlet velocity,
      // wall / inlet pressure, zero-gradient k and omega
      const signed char kind = cv.fkind[f];
#pragma unroll
      for (int q = 0; q < NF; ++q) {
        bool dep;
        if (q < DIM) dep = kind == 3;
        else if (q == L::P) dep = kind >= 0 && kind <= 2;
        else if (q == L::K) dep = cv.kkind[f] == 1;
        else dep = cv.wkind[f] == 1;
        if (dep) acc[q] += pb[(long)q * nf + f];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NF; ++q) out[(long)q * nc + c] = acc[q];
}

template <int DIM, bool TURB>
__global__ void __launch_bounds__(128) a_grad(MeshView m, CaseView cv, AdjWork aw, const double* pb,
                                              double* out) {
  a_grad_at<DIM, TURB>(stage_cell(m, cv), m, cv, aw, pb, out);
}
