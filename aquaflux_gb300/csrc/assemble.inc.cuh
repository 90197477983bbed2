// Direct assembly of the frozen (reach-1) block Jacobian J_direct, the operator that
// materialize_block_jacobian (aquaflux/solve/sparse_jacobian.py:722-847) recovers by coloured JVP
// probes of the frozen JVP.  Included by residual.cu (shares its device helpers).
//
// With the gradients, the SST closure fields and a_P held at their values for `state`, a face's
// fluxes depend on its owner's and neighbour's unknowns only and a cell's SST sources on its own k
// and omega only, so the Jacobian needs no colouring:
//   k_jac_face  face  forward-mode derivative of every flux of the face with respect to each of the
//                     2 x NF unknowns of its two cells (the flux code of the residual, evaluated with
//                     one seeded tangent per unknown), into D (nf, 2, NF, NF): each face's 2 NF^2
//                     derivatives contiguous, so the cell gather reads whole rows;
//   k_jac_cell  cell  the cell's block row: the face derivatives summed in the cell's face order
//                     with the residual's signs (whole face blocks, contiguous), then the SST
//                     source rows, the omega wall-cell rows and the pressure-pin row.
// Every entry is the tangent the coloured probe computes for it, by the same arithmetic in the
// same order.

// The state with a unit tangent on one unknown (index `seed` of the field-major state); T = Dual,
// or DualF for the fp32 assembly of an fp32 preconditioner.
template <class T>
struct SeedSrc {
  const decltype(T::v)* v;  // the state in the pass's precision
  long seed;
  __device__ __forceinline__ T operator()(long i) const {
    return T{v[i], (decltype(T::v))(i == seed ? 1 : 0)};
  }
};

// Keeps the tangent of flux q as D[((f * 2 + side) * NF + q) * NF + r].
template <class T>
struct DerivStore {
  GS<T>* D;  // fp32 for an fp32 pass
  long base;  // ((f * 2 + side) * NF) * NF + r
  long qstride;  // NF
  __device__ __forceinline__ void operator()(int q, const T& x) const {
    D[base + q * qstride] = x.d;
  }
};

template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_jac_face(MeshView m, CaseView cv,
                                                  const decltype(T::v)* state,
                                                  Par<T> par, const T* G, const T* cl,
                                                  const T* dco, const T* psi, GS<T>* D) {
  constexpr int NF = Layout<DIM, TURB>::NFLD;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int nc = m.nc, nf = m.nf;
  const int nside = f < m.nfi ? 2 : 1;
  for (int side = 0; side < nside; ++side) {
    const int cell = side ? m.nb[f] : m.owner[f];
#pragma unroll 1
    for (int r = 0; r < NF; ++r) {
      const SeedSrc<T> st{state, (long)r * nc + cell};
      const DerivStore<T> wr{D, ((long)f * 2 + side) * NF * NF + r, (long)NF};
      flux_face<T, DIM, TURB>(m, cv, st, par, G, cl, dco, (const T*)nullptr, psi, true, f, wr,
                              nullptr);
    }
  }
}

template <class T, int DIM, bool TURB>
__global__ void __launch_bounds__(128) k_jac_cell(MeshView m, CaseView cv,
                                                  const decltype(T::v)* state,
                                                  Par<T> par, const T* G, const T* cl,
                                                  const T* Gwi, const GS<T>* __restrict__ D,
                                                  const int* indptr, const int* indices,
                                                  GS<T>* __restrict__ values) {
  using V = GS<T>;  // the pass's precision: the sums and the stored blocks
  using L = Layout<DIM, TURB>;
  constexpr int NF = L::NFLD;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nc) return;
  const int nc = m.nc;
  const int bp = indptr[c], be = indptr[c + 1];  // (the block rows were zeroed before the launch)
  // rows without the face sum: the pinned pressure row, the omega wall-cell row
  bool skip[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q) skip[q] = false;
  if (c == cv.pin) skip[L::P] = true;
  if constexpr (TURB) skip[L::W] = cv.wcell[c] != 0;
  V dg[NF][NF];
#pragma unroll
  for (int q = 0; q < NF; ++q)
#pragma unroll
    for (int r = 0; r < NF; ++r) dg[q][r] = V(0);
  const int b = m.cf_ptr[c], e = m.cf_ptr[c + 1];
  for (int i = b; i < e; ++i) {
    const unsigned ent = m.cf_face[i];
    const int f = (int)(ent & ~FV_NB_BIT);
    const bool isnb = (ent & FV_NB_BIT) != 0;
    const V sg = isnb ? V(-1) : V(1);
    const V* self = D + ((long)f * 2 + (isnb ? 1 : 0)) * NF * NF;
#pragma unroll
    for (int q = 0; q < NF; ++q)
#pragma unroll
      for (int r = 0; r < NF; ++r) {
        const V x = sg * self[q * NF + r];
        dg[q][r] = i == b ? x : dg[q][r] + x;
      }
    if (f < m.nfi) {
      const int j = isnb ? m.owner[f] : m.nb[f];
      int slot = -1;
      for (int p = bp; p < be; ++p)
        if (indices[p] == j) {
          slot = p;
          break;
        }
      if (slot >= 0) {
        const V* oth = D + ((long)f * 2 + (isnb ? 0 : 1)) * NF * NF;
        V* blk = values + (long)slot * NF * NF;
#pragma unroll
        for (int q = 0; q < NF; ++q) {
          if (skip[q]) continue;
          V o[NF], b0[NF];
#pragma unroll
          for (int r = 0; r < NF; ++r) {
            o[r] = oth[q * NF + r];
            b0[r] = blk[q * NF + r];
          }
#pragma unroll
          for (int r = 0; r < NF; ++r) blk[q * NF + r] = b0[r] + sg * o[r];
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NF; ++q)
    if (skip[q])
#pragma unroll
      for (int r = 0; r < NF; ++r) dg[q][r] = V(0);
  if (c == cv.pin) {
#pragma unroll
    for (int r = 0; r < NF; ++r) dg[L::P][r] = r == L::P ? V(1) : V(0);
  }
  if constexpr (TURB) {
    // only k and omega of the cell itself enter its source rows: one seeded evaluation per
    // column gives both rows (each row's tangent starts from its own face sum)
#pragma unroll
    for (int r = L::K; r <= L::W; ++r) {
      using S = decltype(T::v);
      const SeedSrc<T> st{state, (long)r * nc + c};
      T rk{S(0), S(dg[L::K][r])}, rw{S(0), S(dg[L::W][r])};
      sst_rows<T, DIM>(m, cv, st, par, cl, G, Gwi, c, rk, rw);
      dg[L::K][r] = rk.d;
      dg[L::W][r] = rw.d;
    }
  }
  for (int p = bp; p < be; ++p)
    if (indices[p] == c) {
      V* blk = values + (long)p * NF * NF;
#pragma unroll
      for (int q = 0; q < NF; ++q)
#pragma unroll
        for (int r = 0; r < NF; ++r) blk[q * NF + r] = dg[q][r];
      break;
    }
}

template <class T, int DIM, bool TURB>
int assemble_frozen(FvCase* cs, const double* state, const int* indptr, const int* indices,
                    GS<T>* values, GS<T>* D, cudaStream_t s) {
  using S = decltype(T::v);
  const MeshView& m = cs->mesh->view;
  const CaseView& cv = cs->view;
  const long nc = m.nc, nf = m.nf;
  constexpr int NF = Layout<DIM, TURB>::NFLD;
  cs->fwd_valid = 0;  // the workspace is about to hold this pass
  Work<T> w = work_layout<T, DIM, TURB>(cs->work, nc, nf, psi_count<DIM, TURB>(cs));
  const S* sv;  // the state in the pass's precision
  if constexpr (std::is_same<S, float>::value) {
    int rc = fv_case_ensure_f32(cs, s);
    if (rc != FV_OK) return rc;
    rc = fv_d2f((long)NF * nc, state, cs->f_state, s);
    if (rc != FV_OK) return rc;
    sv = cs->f_state;
  } else {
    sv = state;
  }
  Src<T> st{sv, nullptr};  // zero tangent: the forward stages give the frozen values
  const double irho = 1.0 / cs->desc.rho;
  Par<T> par{{S(cs->mu), S(0)}, {S(cs->inlet_scale), S(0)}, {S(cs->mu * irho), S(0)}};
  constexpr int TB = 128;
  const int bc = fv_blocks(nc, TB), bf = fv_blocks(nf, TB);
  gradient_stage<T, DIM, TURB>(cs, st, par, w, s);
  if (TURB) k_closure<T, DIM><<<bc, TB, 0, s>>>(m, cv, st, par, w.G, w.cl, w.Gwi);
  k_apcoef<T, DIM, TURB><<<bf, TB, 0, s>>>(m, cv, st, par, w.G, w.cl, w.acown, w.acnb, w.me);
  k_dcoeff<T><<<bc, TB, 0, s>>>(m, w.acown, w.acnb, w.dco);
  const long npsi = psi_count<DIM, TURB>(cs);
  if (npsi)
    k_limiter<T, DIM, TURB><<<bc, TB, 0, s>>>(m, st, w.G, cv.lim_km, cv.lim_ks, w.psi);
  k_jac_face<T, DIM, TURB><<<bf, TB, 0, s>>>(m, cv, sv, par, w.G, w.cl, w.dco,
                                             npsi ? w.psi : nullptr, D);
  if (cs->jac_indptr != indptr) {  // the pattern's block count, read once per pattern
    int nnzb = 0;
    FV_CUDA_TRY(cudaMemcpyAsync(&nnzb, indptr + nc, sizeof(int), cudaMemcpyDeviceToHost, s));
    FV_CUDA_TRY(cudaStreamSynchronize(s));
    cs->jac_indptr = indptr;
    cs->jac_nnzb = nnzb;
  }
  FV_CUDA_TRY(cudaMemsetAsync(values, 0, sizeof(GS<T>) * (size_t)NF * NF * (size_t)cs->jac_nnzb,
                              s));
  k_jac_cell<T, DIM, TURB><<<fv_blocks(nc, TB), TB, 0, s>>>(
      m, cv, sv, par, w.G, w.cl, w.Gwi, D, indptr, indices, values);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}
