/* fvgb.h -- C ABI of the GB300 finite-volume hot path (libfvgb.so).
 *
 * A drop-in for the data-parallel path of the reference solver: the cell-centred finite-volume
 * residual R(state, params) of the coupled Rhie-Chow (u, v[, w], p) system with optional
 * k-omega SST, its Jacobian-vector product, and the block-sparse SpMV / zero-fill ILU(0) the
 * Newton-Krylov driver applies.
 *
 * Conventions
 *  - Every entry point returns an int status (FV_OK = 0); fv_last_error() gives the message.
 *  - Array arguments documented "device" are CUDA device pointers owned by the caller; "host"
 *    arrays are read once during the call.  Index arrays are int32, values float64 unless stated.
 *  - `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).  All device
 *    work is stream-ordered; no entry point synchronizes the host except the *_create calls.
 *  - State vectors are field-major, [u(C), v(C), (w(C)), p(C), (k(C), omega(C))], the layout of
 *    aquaflux/flow/state.py:36-69 and aquaflux/turbulence/coupled.py:239-269.
 *  - Faces are identified by their index in the caller's (reference) face order.
 *  - Handles are not thread-safe across concurrent streams.  Evaluation calls allocate nothing.
 */
#ifndef FVGB_H
#define FVGB_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FV_OK = 0,
  FV_ERR_ARG = 1,        /* bad argument / shape (reference: ValueError) */
  FV_ERR_CUDA = 2,       /* a CUDA runtime call failed */
  FV_ERR_NO_DIAG = 3,    /* ILU(0): a row stores no diagonal entry (reference: ValueError) */
  FV_ERR_ZERO_PIVOT = 4, /* ILU(0): exactly zero pivot (reference: ZeroDivisionError) */
  FV_ERR_NONFINITE = 5,  /* a non-finite value where a finite one is required */
  FV_ERR_NOT_CONVERGED = 6,
  FV_ERR_TIMEOUT = 7
};

/* Last error message of the calling thread ("" if none). */
const char* fv_last_error(void);
/* Row / index associated with the last FV_ERR_NO_DIAG / FV_ERR_ZERO_PIVOT (else -1). */
long fv_last_error_index(void);
/* Library version string. */
const char* fv_version(void);

/* ------------------------------------------------------------------------------------------
 * Mesh.  Replaces Mesh.from_csr + Mesh.geometry (aquaflux/mesh/mesh.py:137-206, 341-387):
 * uploads the connectivity, renumbers faces internally by owner for coalesced gathers, builds the
 * cell->face incidence used for deterministic face-to-cell sums, and computes the geometry on the
 * GPU (edge / centre-fan face geometry, owner-outward normals, recentred divergence-theorem
 * cell volume and centroid).
 * ------------------------------------------------------------------------------------------ */
typedef struct FvMesh FvMesh;

int fv_mesh_create(int dim, int n_cells, int n_faces, int n_nodes,
                   const double* nodes,      /* host (n_nodes, dim) row-major */
                   const int* fn_offsets,    /* host (n_faces + 1) CSR pointers */
                   const int* fn_indices,    /* host (fn_offsets[n_faces]) node indices */
                   const int* owner,         /* host (n_faces) */
                   const int* neighbour,     /* host (n_faces), -1 = boundary face */
                   void* stream, FvMesh** out);
int fv_mesh_destroy(FvMesh* mesh);
/* Replace the node coordinates (device (n_nodes, dim) row-major) and recompute the geometry.
 * Turbulent cases on this mesh then need fv_case_refresh_geometry (their wall distance). */
int fv_mesh_set_nodes(FvMesh* mesh, const double* nodes_device, void* stream);
/* Copy the geometry out in reference face order, device outputs (any may be NULL):
 * area (F), normal (F, dim), face_centroid (F, dim), volume (C), cell_centroid (C, dim). */
int fv_mesh_geometry(const FvMesh* mesh, double* area, double* normal, double* face_centroid,
                     double* volume, double* cell_centroid, void* stream);
int fv_mesh_sizes(const FvMesh* mesh, int* dim, int* n_cells, int* n_faces, int* n_nodes);

/* ------------------------------------------------------------------------------------------
 * Case.  Replaces MomentumContinuity.build (aquaflux/flow/momentum.py:233-293) and, with
 * turbulent = 1, SSTTurbulence.build + CoupledRANS.build (aquaflux/turbulence/transport.py:198-243,
 * coupled.py:311-340).  Schemes: compact or corrected (swept) Green-Gauss gradients, first-order
 * upwind advection.
 * Boundary tables are per face in reference face order (entries of interior faces ignored):
 *   flow_kind: -1 none, 0 NoSlipWall, 1 MovingWall, 2 VelocityInlet, 3 PressureOutlet
 *   flow_vel (F, dim): the MovingWall / VelocityInlet velocity;  flow_p (F): outlet pressure
 *   k_kind / omega_kind: -1 none, 0 Dirichlet (value in *_val), 1 ZeroGradient
 *   sst_wall (F): 1 on faces of the SST wall patches (wall distance, wall functions)
 * ------------------------------------------------------------------------------------------ */
typedef struct FvCase FvCase;

typedef struct FvCaseDesc {
  int turbulent;             /* 0: MomentumContinuity, 1: CoupledRANS (direct k, omega) */
  double mu;                 /* molecular dynamic viscosity (Constant) */
  double rho;                /* density (Constant) */
  int pressure_pin;          /* cell index whose pressure row is fixed, -1 for none */
  double pressure_pin_value;
  /* Gradient scheme: 0 = CompactGreenGauss (aquaflux/schemes/gradient.py:129-153); s >= 1 =
   * CorrectedGreenGauss solved by SweptGradientSolve with s sweeps and the given relaxation in
   * (0, 1] (gradient.py:547-705, 1122-1337; preconditioner InverseCellVolume).  Applies to every
   * reconstructed gradient, the wall-distance gradient included. */
  int gradient_sweeps;
  double gradient_relaxation;
  /* Advection scheme of the momentum (and k, omega) face values: 0 FirstOrderUpwind; 1
   * LimitedUpwind without a limiter; 2 LimitedUpwind with VenkatakrishnanLimiter(k = limiter_k)
   * (aquaflux/discretization/advection.py:99-157, aquaflux/schemes/limiter.py:78-117). */
  int advection;
  double limiter_k;
  /* Solved variable of the turbulence scalars (CoupledRANS k_transform / omega_transform,
   * aquaflux/turbulence/coupled.py:111-207): bit 0 set = k is solved as w_k with k = exp(w_k),
   * bit 1 set = omega as w with omega = exp(w) (LogScalars); clear = the field itself
   * (DirectScalars).  The state vectors of every call hold the solved variables; the residual
   * rows stay the physical transport residuals, except the near-wall omega fixation, which under a
   * log omega is the log ratio log(omega / omega_wall) (LogRatioRow,
   * aquaflux/discretization/fixed_value.py:96-120).  Turbulent cases only. */
  int scalar_transform;
  /* Advection scheme of k and omega when it differs from the momentum's (the reference builds
   * SSTTurbulence with its own scheme, aquaflux/turbulence/transport.py:266-312): 0 = the momentum
   * scheme above; 1 FirstOrderUpwind; 2 LimitedUpwind without a limiter; 3 LimitedUpwind with
   * VenkatakrishnanLimiter(k = scalar_limiter_k).  Turbulent cases only. */
  int scalar_advection;
  double scalar_limiter_k;
} FvCaseDesc;

int fv_case_create(const FvMesh* mesh, const FvCaseDesc* desc,
                   const signed char* flow_kind, const double* flow_vel, const double* flow_p,
                   const signed char* k_kind, const double* k_val,
                   const signed char* omega_kind, const double* omega_val,
                   const unsigned char* sst_wall, void* stream, FvCase** out);
int fv_case_destroy(FvCase* c);
/* Change the differentiable physical parameters: molecular viscosity and a factor applied to
 * every prescribed inlet velocity.  Takes effect for later calls on `stream`. */
int fv_case_set_params(FvCase* c, double mu, double inlet_scale);
/* Per-cell molecular viscosity (host or device, n_cells; NULL restores the constant): the
 * viscosity of independent instances held in one disjoint-union mesh (the batched calibration
 * sweep).  Laminar cases only.  The viscosity tangent (fv_param_jvp / fv_param_vjp) seeds every
 * cell's viscosity with 1; its dot product with an adjoint restricted to one instance's unknowns
 * (fv_segment_dot) is that instance's derivative. */
int fv_case_set_viscosity_field(FvCase* c, const double* mu_cell, void* stream);
/* Threads per block of the residual / JVP / VJP stage kernels (a multiple of 32 in [32, 128];
 * results do not depend on it): fv_case_set_block_size sets every stage.  fv_case_autotune times
 * the residual + VJP step at state / w with every stage at 32, 64, 96 and 128 threads, stage by
 * stage (the profiling marks), keeps each stage's fastest, and returns the fastest uniform size
 * in best (out: n_unknowns scratch; no stage profile may be open).  fv_case_block_sizes copies
 * the per-stage sizes (stages in the order of fv_case_profile_end's). */
int fv_case_set_block_size(FvCase* c, int threads);
int fv_case_block_sizes(const FvCase* c, int* threads, int n);
/* Residual + VJP (fv_vjp) as ONE persistent cooperative launch (all stages in one kernel,
 * grid-wide barriers between them; compact gradients and first-order upwind; bitwise the
 * stage-per-launch result): enable != 0 with `block` threads per block (multiple of 32 in
 * [32, 128]) and `chunk` consecutive cells / faces per thread per stage (1 .. 64).  The batched
 * calibration sweep's instances run side by side in one such launch.  fv_case_autotune_persistent
 * times every (block in {64, 128}) x (chunk in {1, 2, 4, 8}) at state / w, keeps the fastest
 * (without enabling the path) and returns it with its time per evaluation. */
int fv_case_set_persistent(FvCase* c, int enable, int block, int chunk);
/* Order in which the threads of the cell-centric stages (gradients, closure, face sums and their
 * adjoints) take the cells.  coherent != 0 (the default of fv_case_create): cells grouped by the
 * pattern of their face lists -- owner / neighbour / boundary table entry at each position -- so
 * that the lanes of a warp take the same branches; 0: the natural order.  Results are bitwise the
 * same either way.  n_classes (optional) receives the number of distinct patterns.  No reference
 * counterpart: an evaluation-order choice of this implementation. */
int fv_case_set_cell_order(FvCase* c, int coherent, int* n_classes);
int fv_case_autotune_persistent(FvCase* c, const double* state, const double* w, double* out,
                                void* stream, int* best_block, int* best_chunk, float* best_ms);
int fv_case_autotune(FvCase* c, const double* state, const double* w, double* out, void* stream,
                     int* best);
/* After fv_mesh_set_nodes: recompute a turbulent case's SST wall distance (to each cell's nearest
 * wall face found at case creation, held fixed as the mesh-coordinate adjoint differentiates it),
 * its gradient and their fp32 mirrors.  No-op for laminar cases.  The reference recomputes
 * WallDistance from the mesh inside the differentiated residual (aquaflux/mesh/distance.py:52-84,
 * aquaflux/turbulence/transport.py:86-111). */
int fv_case_refresh_geometry(FvCase* c, void* stream);
/* Replace a turbulent case's SST wall distance (device, C) and recompute its gradient: a case on
 * a partition's local mesh takes the global distance, whose nearest wall face may lie outside
 * it.  The mesh-coordinate adjoint and fv_case_refresh_geometry then refuse the case.  A
 * turbulent case created on a mesh without SST wall faces evaluates nothing until this is
 * called. */
int fv_case_set_wall_distance(FvCase* c, const double* distance, void* stream);
/* Device copies (C) and (C, dim) of the SST wall distance and its gradient (turbulent cases). */
int fv_case_wall_distance(const FvCase* c, double* distance, double* gradient, void* stream);
/* Number of unknowns: (dim + 1) * C, or (dim + 3) * C when turbulent. */
long fv_case_n_unknowns(const FvCase* c);

/* R = residual(state).  MomentumContinuity.residual (aquaflux/flow/momentum.py:880) or
 * CoupledRANS.residual (aquaflux/turbulence/coupled.py:437).  Device in/out. */
int fv_residual(FvCase* c, const double* state, double* residual, void* stream);
/* nu_t (C, device) of a turbulent case at state: CoupledRANS.eddy_viscosity
 * (aquaflux/turbulence/coupled.py), the coefficient the staleness measure eddy_viscosity_drift
 * (coupled.py:681-717) watches. */
int fv_eddy_viscosity(FvCase* c, const double* state, double* nut, void* stream);
/* jv = J(state) v, the directional derivative jax.jvp(R, (state,), (v,)) of
 * aquaflux/solve/newton.py:110-111.  `residual` (may be NULL) receives R(state).  Device. */
int fv_jvp(FvCase* c, const double* state, const double* v, double* residual, double* jv,
           void* stream);
/* The linearised Jacobian-vector product (jax.linearize's split of the reference's
 * jax.jvp(residual_fn, (phi,), (v,)), aquaflux/solve/newton.py:110-111): fv_linearise evaluates the
 * residual at `state` (into `residual`, device, may be NULL) and holds that evaluation's face
 * intermediates, primal face fluxes, gradients, residual and (SST) the off-wall cells' closure and
 * source tangents as linear forms in (k', omega', S', (grad k . grad omega)'); fv_jvp_linearised then
 * gives J(state) v (and, when `residual` is not NULL, the held residual) with the interior faces'
 * flux, coefficient and compact-gradient stages, the off-wall closure and the face sums computed as
 * tangents only, every other stage as fv_jvp does.  `state` must be the linearised one.  A change of parameters, of the
 * viscosity field, of the wall distance or of the geometry (fv_case_refresh_geometry) drops the
 * linearisation; fv_jvp_linearised then refuses until fv_linearise runs again.  First-order upwind
 * advection only (a limited reconstruction is refused by fv_linearise). */
int fv_linearise(FvCase* c, const double* state, double* residual, void* stream);
int fv_jvp_linearised(FvCase* c, const double* state, const double* v, double* residual,
                      double* jv, void* stream);
/* jv = J_direct v: the derivative with the gradients, the SST closure fields and the momentum
 * diagonal a_P held at their values for `state` (a reach-1 operator: the "frozen" Jacobian the
 * preconditioner is built from).  No reference counterpart as an entry point; it is the
 * linearisation a Picard / SIMPLE-type preconditioner uses.  Device. */
int fv_jvp_frozen(FvCase* c, const double* state, const double* v, double* jv, void* stream);
/* k directional derivatives at one state: jv[i] = J(state) v[i] for the row-major (k, n) seed
 * block v, the vmapped JVP of aquaflux/turbulence/coupled.py:741-752 (_batched_jacobian_matvec).
 * Device. */
int fv_jvp_batch(FvCase* c, const double* state, const double* v, int k, double* jv, void* stream);
/* Materialise the Jacobian (frozen = 1: J_direct; 0: the full J, exact on the pattern only when
 * the colouring's reach covers J's) into a cell-major BSR matrix with b = number of fields, by
 * coloured JVP probes: materialize_block_jacobian (aquaflux/solve/sparse_jacobian.py:722-847).
 * colour (device, C) and n_colours from fv_saturation_colouring; indptr / indices (device) the
 * block pattern over cells (sorted); values (device, nnzb * b * b) row-major blocks. */
int fv_probe_jacobian(FvCase* c, const double* state, int frozen, const int* colour,
                      int n_colours, const int* indptr, const int* indices, double* values,
                      void* stream);
/* The same frozen Jacobian (J_direct, reach 1) assembled directly: forward-mode derivatives of
 * every face flux with respect to the unknowns of its two cells, summed into the block rows in
 * the residual's face order, then the SST source, omega wall-cell and pressure-pin rows.  Needs
 * no colouring (one face pass instead of n_colours * b probes); the pattern must hold every
 * cell's diagonal block and the blocks of its face neighbours (blocks outside reach 1 are set to
 * 0).  Fast path of materialize_block_jacobian (aquaflux/solve/sparse_jacobian.py:722-847) for
 * the frozen operator.  Allocates a face-derivative buffer of 2 b^2 doubles per face on first
 * use (kept with the case).  Device. */
int fv_assemble_jacobian(FvCase* c, const double* state, const int* indptr, const int* indices,
                         double* values, void* stream);
/* The same assembly, and the same JVP as fv_jvp, evaluated in fp32 arithmetic (single-precision
 * dual numbers on fp32 copies of the geometry and the state; fp64 state in; fp32 block values
 * out, fp64 jv out): the Jacobian of an fp32 preconditioner and the Krylov operator of a
 * mixed-precision Newton, whose defect R stays fp64.  Agree with the fp64 forms to fp32 rounding
 * (~1e-6 relative). */
int fv_assemble_jacobian_f32(FvCase* c, const double* state, const int* indptr, const int* indices,
                             float* values, void* stream);
int fv_jvp_f32(FvCase* c, const double* state, const double* v, double* jv, void* stream);
/* jv = J v + shift * v (the pseudo-transient operator of aquaflux/solve/continuation.py:111-112);
 * `shift` is a device vector of the state's length. */
int fv_jvp_shift(FvCase* c, const double* state, const double* v, const double* shift, double* jv,
                 void* stream);
/* Directional derivative of the residual with respect to the scalar parameters:
 * out_mu = dR/dmu, out_inlet = dR/d(inlet_scale) (either may be NULL).  Device. */
int fv_param_jvp(FvCase* c, const double* state, double* out_mu, double* out_inlet, void* stream);

/* vjp = J(state)^T w, the vector-Jacobian product jax.vjp(R(., theta), state) of
 * aquaflux/solve/implicit.py:753 (hand-written adjoint kernels; geometry is held fixed).
 * `residual` (may be NULL) receives R(state), computed by the same forward pass.  Device. */
int fv_vjp(FvCase* c, const double* state, const double* w, double* residual, double* vjp,
           void* stream);
/* Parameter cotangents w^T dR/dtheta for theta = (mu, inlet_scale): the vjp_theta of
 * aquaflux/solve/implicit.py:759-760.  `out` is a device array of 2 doubles. */
int fv_param_vjp(FvCase* c, const double* state, const double* w, double* out, void* stream);
/* The VJP's forward pass held for repeated products at one state (the adjoint solve's operator
 * w -> J^T w: aquaflux/solve/implicit.py:733-761 applies jax.vjp's pullback, built once, at every
 * Krylov step): fv_hold_forward evaluates the residual at `state` (into `residual`, may be NULL)
 * keeping the forward intermediates the adjoint stages read; fv_vjp_held then runs the adjoint
 * stages only -- bitwise fv_vjp's result.  `state` must be the held one.  Any other evaluation on
 * the case (residual, JVP, Jacobian assembly, node adjoint ...) or a parameter, viscosity-field,
 * wall-distance or geometry change drops the hold; fv_vjp_held then refuses.  fv_vjp itself leaves
 * its forward pass held. */
int fv_hold_forward(FvCase* c, const double* state, double* residual, void* stream);
int fv_vjp_held(FvCase* c, const double* state, const double* w, double* vjp, void* stream);
/* dnodes = d/dnodes (w . R(state, nodes)): the mesh-coordinate adjoint (the node-coordinate part
 * of theta_bar in _implicit_solve_bwd, aquaflux/solve/implicit.py:733-761), through the face
 * areas, normals and centroids, the cell volumes and centroids, every factor derived from them and
 * (turbulent cases) the wall distance to the nearest wall face and its gradient; the owner-outward
 * normal flip is a constant sign.  Device (n_nodes, dim) row-major output in the caller's node
 * order.  Compact gradient scheme only (FV_ERR_ARG otherwise).  Allocates a workspace with the
 * case on first use. */
int fv_node_vjp(FvCase* c, const double* state, const double* w, double* dnodes, void* stream);
/* A face-flux functional J = sum_f sum_q weights[q, f] FL_q(f) of the residual's face fluxes
 * (weights device (nfld, F) field-major, reference face order; FL_q(f) the flux of field q
 * through face f, owner-outward: mass flux for the continuity field, momentum / k / omega fluxes
 * otherwise), with viscous_only != 0 taking the pressure part sum_i w_i p_f A n_i out on boundary
 * faces (the wall shear force).  The outlet mass flux and the wall shear of the adjoint objectives
 * are such functionals.  value: device scalar J; dstate (device, n_unknowns): dJ/dstate; dparams
 * (device (2), may be NULL): the partials dJ/d(mu, inlet_scale) at fixed state; dnodes (device
 * (n_nodes, dim), may be NULL): dJ/dnodes at fixed state (compact gradient scheme).  The total
 * derivative at a converged state is dJ/dtheta - lambda^T dR/dtheta with J^T lambda = dJ/dstate
 * (fv_vjp / fv_param_vjp / fv_node_vjp). */
int fv_face_functional(FvCase* c, const double* state, const double* weights, int viscous_only,
                       double* value, double* dstate, double* dparams, double* dnodes,
                       void* stream);

/* Per-stage CUDA-event timing of the next `max_runs` pipeline runs on this case (diagnostics;
 * no reference counterpart).  profile_end synchronizes, writes the summed milliseconds of each
 * stage (grad, closure, apcoef, dcoeff, flux, sum, and for a VJP a_sum, a_flux, a_apcoef,
 * a_closure, a_grad) and the number of runs recorded. */
int fv_case_profile_begin(FvCase* c, int max_runs);
int fv_case_profile_end(FvCase* c, float* stage_ms, int n_stages, int* n_runs);

/* ------------------------------------------------------------------------------------------
 * Block-sparse (BSR, b x b dense blocks, row-major inside a block) operators.
 * Replaces _CsrOperator.apply (aquaflux/solve/multigrid.py:1302-1390).
 * ------------------------------------------------------------------------------------------ */
/* y = A x (transpose = 0) or y = A^T x (transpose = 1); fp64. Device arrays. */
int fv_bsr_spmv_f64(int n_block_rows, int b, const int* indptr, const int* indices,
                    const double* values, const double* x, double* y, int transpose,
                    void* stream);
/* y = A^T x for a square BSR matrix (fp64) WITHOUT allocating device memory.  No counterpart in
 * the reference: it serves callers that cannot allocate while they run (an FFI custom call inside
 * a framework that owns all device memory, such as an XLA custom call, or an embedded solver that
 * forbids allocation after start-up), where fv_bsr_spmv_f64(transpose = 1) would allocate its
 * transpose map.  The map is built in a fixed 16 MiB static device array that every GPU loading
 * the library holds until exit; patterns needing more than 4,194,304 ints
 * (2 * n_block_rows + 2 + 2 * nnzb) are rejected with FV_ERR_ARG.  nnzb must equal
 * indptr[n_block_rows] and every column index must lie in [0, n_block_rows): otherwise every
 * entry of y is set to NaN (the check runs on the GPU; nothing is read back).  The result is
 * bitwise that of fv_bsr_spmv_f64(transpose = 1).  The first call on each device looks the
 * array's address up (cudaGetSymbolAddress) and must come before any stream capture.  All calls
 * share the one array: calls that overlap on the GPU (different streams, or concurrent host
 * threads) race and give wrong results.  Device arrays. */
int fv_bsr_spmv_t_f64_noalloc(int n_block_rows, long nnzb, int b, const int* indptr,
                              const int* indices, const double* values, const double* x,
                              double* y, void* stream);
/* fp32 values and vectors. */
int fv_bsr_spmv_f32(int n_block_rows, int b, const int* indptr, const int* indices,
                    const float* values, const float* x, float* y, int transpose, void* stream);
/* Transpose map of a square BSR pattern (host): tptr (n + 1) / tidx (nnzb) list, for block row j
 * of A^T, the rows i of A holding a block (i, j); tblk (nnzb) that block's index in A. */
int fv_bsr_transpose_map(int n, const int* indptr, const int* indices, int* tptr, int* tidx,
                         int* tblk);
/* y = A^T x through that map (device; fp64 when f64 != 0, else fp32; allocates nothing): the
 * transposed products of the exact V-cycle transpose (aquaflux/solve/ilu_inverse.py:275-308). */
int fv_bsr_spmv_t_mapped(int n, int b, const int* tptr, const int* tidx, const int* tblk,
                         const void* values, const void* x, void* y, int f64, void* stream);
/* tvalues[q] = values[tblk[q]]^T for the nnzb blocks of a map from fv_bsr_transpose_map (device;
 * fp64 when f64 != 0, else fp32): A^T in BSR with b x b row-major blocks on the pattern (tptr,
 * tidx), so that fv_bsr_spmv_f64 / _f32 with transpose = 0 on it gives A^T x -- the same products
 * in the same order as fv_bsr_spmv_t_mapped, bitwise, with the forward kernel's row-wise vector
 * loads.  No reference counterpart (the reference transposes through jax.linear_transpose). */
int fv_bsr_transpose_blocks(long nnzb, int b, const int* tblk, const void* values, void* tvalues,
                            int f64, void* stream);

/* ------------------------------------------------------------------------------------------
 * Zero-fill ILU(0) over a BSR pattern.  Replaces Ilu0 (aquaflux/solve/ilu0.py:153-255) and the
 * compiled kernel aquaflux/solve/_ilu0.pyx (diagonal_positions :35-65, factor :68-121, solve
 * :124-147, solve_transpose :150-178).  With b = 1 it is the reference's scalar CSR ILU(0); with
 * b > 1 the b x b blocks are dense and the elimination is the same scalar ILU(0) over the
 * block-expanded pattern (cell-major interleaved ordering, aquaflux/solve/ordering.py:195-242).
 * Rows are eliminated in level-set order on the GPU, which reproduces the sequential result.
 * ------------------------------------------------------------------------------------------ */
typedef struct FvIlu0 FvIlu0;

/* Analyse the pattern (host CSR/BSR arrays, sorted column indices); precision: 32 or 64. */
int fv_ilu0_create(int n_block_rows, int b, const int* indptr, const int* indices, int precision,
                   void* stream, FvIlu0** out);
int fv_ilu0_destroy(FvIlu0* f);
/* A factor object on the same pattern as `src` without analysing it again: the level sets and
 * device pattern are copied on the device, the host pattern is shared.  precision 32 or 64 gives
 * a factor ready for fv_ilu0_factor; precision 0 a structure-only template (it cannot factor or
 * solve) to clone later factors from.  No reference counterpart: the reference re-analyses the
 * pattern of every ILU(0) it builds (aquaflux/solve/_ilu0.pyx:35-65). */
int fv_ilu0_clone(const FvIlu0* src, int precision, void* stream, FvIlu0** out);
/* Numeric factorization of new values (device, nnzb * b * b, same dtype as `precision`, or
 * float64 when values_f64 != 0 and precision == 32: converted on the fly). */
int fv_ilu0_factor(FvIlu0* f, const void* values, int values_f64, void* stream);
/* x = (LU)^-1 r, or (LU)^-T r when transpose != 0.  Device vectors of `precision`.  On a stream
 * under capture the level kernels are recorded into the caller's graph (x may alias r, and must be
 * 16-byte aligned: FV_ERR_ARG otherwise); a transposed solve needs one uncaptured transposed solve
 * first. */
int fv_ilu0_apply(FvIlu0* f, const void* r, void* x, int transpose, void* stream);
/* Copy the factor (device, nnzb * b * b, `precision`) -- combined L (unit diagonal) and U. */
int fv_ilu0_factor_values(const FvIlu0* f, void* out, void* stream);

/* ------------------------------------------------------------------------------------------
 * The shifted, equilibrated cell-major operator D (J + diag(shift)) D of
 * ShiftedCellMajorOperator.assemble (aquaflux/solve/amg_preconditioner.py:545-658), with
 * shifted_jacobian (sparse_jacobian.py:893-927) and the equilibration of
 * frozen_operator.py:72-143.  The matrix is cell-major BSR (b x b row-major blocks, the reference's
 * cell-major CSR with every block entry stored).  shift (field-major, n * b) may be NULL; with
 * equilibrate != 0 every entry is scaled by s[row] then s[column], s = 1 / sqrt(|shifted diagonal|)
 * (|0| read as 1), and scale_fm (may be NULL) receives s in field-major order.  work: device scratch
 * of 2 n b + 1 doubles.  out: nnzb b^2 values, fp64 (out_f64 != 0) or fp32.  A block row without a
 * diagonal block returns FV_ERR_NO_DIAG.  Synchronizes the stream (to report that error).
 * ------------------------------------------------------------------------------------------ */
int fv_bsr_shift_equilibrate(int n, int b, const int* indptr, const int* indices,
                             const double* values, const double* shift, int equilibrate,
                             double* scale_fm, double* work, void* out, int out_f64, void* stream);

/* ------------------------------------------------------------------------------------------
 * Graph colouring for compressed Jacobian probing.  Replaces _saturation_colouring
 * (aquaflux/solve/sparse_jacobian.py:409-534): saturation-degree greedy colouring of the conflict
 * graph given as host CSR (the same neighbour order gives the same colours).  Host arrays;
 * `colour` receives n ints, `n_colours` the number of colours.
 * ------------------------------------------------------------------------------------------ */
int fv_saturation_colouring(int n, const int* indptr, const int* indices, int* colour,
                            int* n_colours);
/* First-fit greedy colouring in index order (O(edges); not the reference's): the AMG fine-level
 * ordering of 3D operators, where only a small colour count matters. */
int fv_greedy_colouring(int n, const int* indptr, const int* indices, int* colour, int* n_colours);
/* Reach-1 cell pattern (host): row i = {i} + the cells sharing an interior face with i, sorted
 * and unique (the pattern of the frozen Jacobian; stencil_pattern with reach 1,
 * aquaflux/solve/sparse_jacobian.py).  indptr (n + 1); indices capacity n + 2 * n_pairs. */
int fv_cell_pattern(int n, long n_pairs, const int* owner, const int* neighbour, int* indptr,
                    int* indices);

/* ------------------------------------------------------------------------------------------
 * Aggregation multigrid.  Replaces the aggregation hierarchy of aquaflux/solve/multigrid.py
 * (_build_aggregation_hierarchy :1011, _mis_aggregate :353) as used by the ILU-smoothed V-cycle
 * of aquaflux/solve/ilu_inverse.py:160-308, with unsmoothed (piecewise-constant) prolongation.
 * ------------------------------------------------------------------------------------------ */
/* Aggregate the cells of a symmetric cell graph (host CSR); agg[i] in [0, *n_agg). */
int fv_aggregate(int n, const int* indptr, const int* indices, int* agg, int* n_agg);
/* Saturation-degree colouring (fv_saturation_colouring) of the aggregate graph of `agg`: the
 * sorted coarse pattern, self included, read from the fine pattern without the block lists.  The
 * colour-by-colour numbering of the coarse levels. */
int fv_colour_aggregates(int n, const int* indptr, const int* indices, const int* agg, int na,
                         int* colour, int* n_colours);
/* One coarsening of a (block) pattern by an aggregation agg (host): mptr (na + 1) / mlist (n)
 * the members of every aggregate in ascending order; cip (na + 1) / cix (capacity nnz) the sorted
 * coarse pattern; gptr (capacity nnz + 1) / glist (nnz) for every coarse block the fine blocks
 * summed into it, ascending (both NULL: the pattern only); n_coarse_blocks the coarse pattern's
 * size.  No reference counterpart as an entry point: the Galerkin product of the
 * piecewise-constant aggregation prolongation (aquaflux/solve/multigrid.py:1011-1245) as ordered
 * block lists. */
int fv_coarsen(int n, const int* indptr, const int* indices, const int* agg, int na, int* mptr,
               int* mlist, int* cip, int* cix, long* gptr, long* glist, long* n_coarse_blocks);
/* Galerkin coarse blocks: coarse[Q] = sum of the fine blocks glist[gptr[Q] .. gptr[Q+1]) in list
 * order (device; fine fp64 when fine_f64 != 0, else fp32; coarse fp32; b x b row-major blocks). */
int fv_galerkin_f32(long n_coarse_blocks, int b, const long* gptr, const long* glist,
                    const void* fine, int fine_f64, float* coarse, void* stream);
/* rc[I] = sum of r over the member cells mlist[mptr[I] .. mptr[I+1]) (b values per cell). */
int fv_restrict_f32(int n_coarse, int b, const int* mptr, const int* mlist, const float* r,
                    float* rc, void* stream);
/* x[i] += xc[agg[i]] (b values per cell). */
int fv_prolong_add_f32(int n_fine, int b, const int* agg, const float* xc, float* x, void* stream);
/* Symmetric block permutation of a pattern (host): new row r = old row perm[r], rows sorted;
 * bmap (nnz) the old block index of every new block. */
int fv_permute_pattern(int n, const int* indptr, const int* indices, const int* perm,
                       int* out_indptr, int* out_indices, long* bmap);
/* dst block q = src block bmap[q] (device; b x b entries; fp64 when *_f64 != 0, else fp32). */
int fv_gather_blocks(long nnzb, int b, const long* bmap, const void* src, int src_f64, void* dst,
                     int dst_f64, void* stream);
/* Field-major fp64 state-layout vector <-> cell-major vector in a permuted cell order
 * (perm NULL: identity), each entry multiplied by scale_fm (field-major, may be NULL):
 * out[r * b + a] = in[a * n + perm[r]] * scale_fm[a * n + perm[r]] and its inverse (device). */
int fv_to_cells(int n, int b, const int* perm, const double* scale_fm, const double* in, void* out,
                int out_f64, void* stream);
int fv_from_cells(int n, int b, const int* perm, const double* scale_fm, const void* in,
                  int in_f64, double* out, void* stream);
/* The same three in fp64 (the fp64 V-cycle of the all-fp64 Newton-Krylov solve). */
int fv_galerkin_f64(long n_coarse_blocks, int b, const long* gptr, const long* glist,
                    const void* fine, int fine_f64, double* coarse, void* stream);
int fv_restrict_f64(int n_coarse, int b, const int* mptr, const int* mlist, const double* r,
                    double* rc, void* stream);
int fv_prolong_add_f64(int n_fine, int b, const int* agg, const double* xc, double* x,
                       void* stream);

/* ------------------------------------------------------------------------------------------
 * Deterministic reductions for the Krylov solver (fixed blocking, fixed order: run-to-run
 * bit-identical).  Device arrays; `out` is a device scalar.
 * ------------------------------------------------------------------------------------------ */
int fv_dot_f64(long n, const double* x, const double* y, double* out, void* stream);
/* Per-segment dot products over field-major vectors: out[i] = sum over fields q and cells
 * c in [seg[i], seg[i + 1]) of a[q nc + c] b[q nc + c] (device; fixed order).  The per-instance
 * reductions of the batched calibration sweep (independent instances as cell ranges of one
 * disjoint-union mesh). */
int fv_segment_dot(int n_seg, const int* seg, int nfld, int nc, const double* a, const double* b,
                   double* out, void* stream);

/* ------------------------------------------------------------------------------------------
 * Cell renumbering on the GPU.  Replaces ReverseCuthillMcKee.permutation
 * (aquaflux/mesh/reorder.py:147-159) over cell_adjacency_coo (aquaflux/mesh/graph.py:29-56): the
 * same permutation as scipy.sparse.csgraph.reverse_cuthill_mckee(symmetric_mode=True).
 * ------------------------------------------------------------------------------------------ */
/* Symmetric cell graph of n_pairs interior (owner, neighbour) pairs (device) as sorted,
 * coalesced CSR: indptr (n + 1), indices (up to 2 n_pairs; indptr[n] used).  work: 2 n + 2 +
 * 2 n_pairs ints (device).  Pairs out of range or joining a cell to itself are refused. */
int fv_cell_graph(int n, long n_pairs, const int* owner, const int* neighbour, int* indptr,
                  int* indices, int* work, void* stream);
/* perm[old] = new (device, n) of reverse Cuthill-McKee on a sorted symmetric CSR graph (device),
 * node degrees at most 64.  seed_order (host, n): numpy.argsort of the degrees, the component
 * seeds' order.  work: 3 n + 1 ints (device). */
int fv_rcm_permutation(int n, const int* indptr, const int* indices, const long* seed_order,
                       int* perm, int* work, void* stream);

/* ------------------------------------------------------------------------------------------
 * Flexible GMRES(m) on the device, fp64, bitwise reproducible (fixed blocking and summation order).
 * Replaces the lineax GMRES behind solve_linear / relative_residual_gmres
 * (aquaflux/solve/linear.py:138-298; the inexact forward solve of aquaflux/solve/implicit.py:50).
 * The caller owns the bases: V (m + 1 rows of n) and Z (m rows of n), device, row-major.  A
 * workspace holds the Hessenberg matrix, the Givens rotations, the rotated right-hand side g and
 * the reduction partials; one workspace serves one stream at a time.
 * ------------------------------------------------------------------------------------------ */
typedef struct FvKrylov FvKrylov;
int fv_krylov_create(int m, FvKrylov** out);
int fv_krylov_destroy(FvKrylov* kr);
/* Start a cycle from the residual r: beta = ||r||, V0 = r / beta, g = (beta, 0, ...).  est (may
 * be NULL; device or pinned host) receives (beta, beta). */
int fv_krylov_start(FvKrylov* kr, long n, const double* r, double* V0, double* est, void* stream);
/* Arnoldi step j (0 <= j < m) on w = A M v_j: CGS2 against V[0..j], column j of H, Givens
 * reduction, V[j + 1] = w / ||w|| (w is overwritten).  est (may be NULL; device or pinned host)
 * receives (|g[j + 1]|, h[j + 1, j]): the residual estimate after j + 1 columns and the new
 * basis norm (0 at a breakdown). */
int fv_krylov_arnoldi(FvKrylov* kr, int j, long n, double* V, double* w, double* est,
                      void* stream);
/* End a cycle after k columns: y = H[0..k, 0..k)^-1 g[0..k), x += Z[0..k)^T y. */
int fv_krylov_update(FvKrylov* kr, int k, long n, const double* Z, double* x, void* stream);
/* out (device) = ||x||, deterministic. */
int fv_krylov_norm(FvKrylov* kr, long n, const double* x, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FVGB_H */
