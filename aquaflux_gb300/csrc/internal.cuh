// Library-internal structures shared by the .cu files of libfvgb.
#pragma once

#include <vector>

#include "common.cuh"

// Bit set in a cell->face incidence entry when the cell is the face's neighbour (its sums take
// the face flux with a minus sign, the conservative scatter of aquaflux/mesh/connectivity.py:262).
#define FV_NB_BIT 0x80000000u

// Read-only view of the device mesh passed by value to kernels.  Faces are stored in the
// internal order: interior faces first, sorted by (owner, neighbour), then boundary faces sorted
// by owner.  Vector quantities are struct-of-arrays: component j of face f is at [j * nf + f].
struct MeshView {
  int dim, nc, nf, nfi, nn;
  const int* owner;
  const int* nb;
  const int* cf_ptr;           // (nc + 1) cell -> face incidence, faces ascending
  const unsigned* cf_face;     // face index | FV_NB_BIT when the cell is the neighbour
  const int* fn_ptr;           // (nf + 1) face -> node CSR (internal face order)
  const int* fn_idx;
  const double* nodes;         // (nn, dim) row-major
  // geometry
  const double* area;          // (nf)
  const double* normal;        // (dim, nf) owner-outward unit normal
  const double* xf;            // (dim, nf) face centroid
  const double* vol;           // (nc)
  const double* xc;            // (dim, nc) cell centroid
  // geometry-derived per-face factors (aquaflux/flow/momentum.py:266-279,
  // aquaflux/schemes/interpolation.py:27-176, aquaflux/discretization/diffusion.py:85-199)
  const double* g;             // (nf) projection factor, 0 on boundary faces
  const double* nd;            // (nf) normal distance: d.n (interior), (x_f - x_P).n (boundary)
  const double* dpn;           // (nf) (x_f - x_P).n
  const double* dnn;           // (nf) (x_f - x_N).n (boundary: = dpn)
  const double* dvec;          // (dim, nf) x_N - x_P (0 on boundary faces)
  const double* skew;          // (dim, nf) x_f - (x_P + g d)
  const double* tP;            // (dim, nf) (x_f - x_P) - dpn n
  const double* tN;            // (dim, nf) (x_f - x_N) - dnn n
  const double* nn2;           // (nf) sum_j n_j n_j
  const double* inv_nd;        // (nf) 1 / nd
  const double* inv_dpn;       // (nf) 1 / dpn
  const double* ns;            // (dim * dim, nf) n_j skew_q at [(j * dim + q) * nf + f]
  const double* inv_vol;       // (nc) 1 / V
  // fp32 mirror of the geometry (same layout), for the fp32 dual-number passes; null until
  // fv_mesh_ensure_f32 makes it
  const float *f_area, *f_normal, *f_xf, *f_vol, *f_xc, *f_g, *f_nd, *f_dpn, *f_dnn, *f_dvec,
      *f_skew, *f_tP, *f_tN, *f_nn2, *f_inv_nd, *f_inv_dpn, *f_ns, *f_inv_vol;
};

struct FvMesh {
  int dim = 0, nc = 0, nf = 0, nfi = 0, nn = 0;
  std::vector<int> h_face_old;  // internal face -> reference face
  std::vector<int> h_face_new;  // reference face -> internal face
  std::vector<int> h_owner, h_nb;  // internal order
  std::vector<int> h_cf_ptr;
  std::vector<unsigned> h_cf_face;
  int* owner = nullptr;
  int* nb = nullptr;
  int* cf_ptr = nullptr;
  unsigned* cf_face = nullptr;
  int* fn_ptr = nullptr;
  int* fn_idx = nullptr;
  int* face_old = nullptr;  // device copy of h_face_old
  double* nodes = nullptr;
  double* geo = nullptr;  // one allocation holding every geometry / factor array
  size_t geo_n = 0;
  float* geo_f = nullptr;  // its fp32 mirror (fp32 passes), kept in step with the geometry
  double* approx = nullptr;  // (dim, nc) approximate centroids (work)
  MeshView view;
};

// Geometry pipeline (mesh.cu).
int fv_mesh_compute_geometry(FvMesh* m, cudaStream_t s);

// Device case tables (internal face order) and the residual workspace (residual.cu).
struct CaseView {
  int turb;
  double rho;
  int pin;
  double pin_value;
  const signed char* fkind;   // (nf) flow boundary kind
  const double* fvel;         // (dim, nf)
  const double* fp;           // (nf)
  const signed char* kkind;   // (nf)
  const double* kval;         // (nf)
  const signed char* wkind;   // (nf)
  const double* wval;         // (nf)
  const unsigned char* swall; // (nf) SST wall face
  const unsigned char* wcell; // (nc) SST wall cell
  const double* wd;           // (nc) wall distance
  const double* wdg;          // (dim, nc) wall-distance gradient
  const double* inv_wd;       // (nc) 1 / wall distance
  const double* inv_wd2;      // (nc) 1 / wall distance^2
  const double* mu_cell;      // (nc) per-cell molecular viscosity (laminar), or null
  int log_w;                  // the omega fixation row is the log ratio (log-solved omega)
  // fp32 copies for the fp32 dual-number passes (null until made)
  const float *f_wd, *f_wdg, *f_inv_wd, *f_inv_wd2, *f_mu_cell;
  float f_rho;
  int rec_mom, rec_sca;       // linear-upwind reconstruction of the momentum / the k, omega faces
  double lim_km, lim_ks;      // their Venkatakrishnan constants (0: unlimited, psi = 1)
  const int* sched;           // (nc) the cell each thread of a cell stage evaluates, or null
};

// Workspace of the mesh-coordinate adjoint (residual.cu), allocated on its first use.
struct NodeAdjoint {
  void* dual_work = nullptr;  // forward workspace as dual numbers with zero tangents
  double* buf = nullptr;
  int* node_ptr = nullptr;    // node -> face-node entries (CSR over fn_idx positions)
  int* node_ent = nullptr;
  int* wall_ptr = nullptr;    // face -> cells whose nearest wall face it is
  int* wall_cell = nullptr;
  double* sweep = nullptr;    // corrected gradients: forward iterates, their cotangents, scratch
  double* rec = nullptr;      // limited reconstruction: centroid and limiter partials
};

#define FV_MAX_STAGES 12
struct FvCase {
  FvMesh* mesh = nullptr;
  FvCaseDesc desc{};
  int nfld = 0;            // dim + 1 (+ 2 when turbulent)
  double mu = 0.0;         // current molecular viscosity
  double inlet_scale = 1.0;
  signed char* fkind = nullptr;
  double* fvel = nullptr;
  double* fp = nullptr;
  signed char* kkind = nullptr;
  double* kval = nullptr;
  signed char* wkind = nullptr;
  double* wval = nullptr;
  unsigned char* swall = nullptr;
  unsigned char* wcell = nullptr;
  double* wd = nullptr;
  double* wdg = nullptr;
  double* inv_wd = nullptr;   // (2, nc): 1 / d and 1 / d^2
  void* work = nullptr;     // residual scratch, sized for the Dual pipeline
  size_t work_bytes = 0;
  double* tmp = nullptr;    // (n_unknowns) scratch vector
  double* tmp2 = nullptr;   // (n_unknowns) scratch vector
  double* adj = nullptr;    // adjoint workspace
  double* aux = nullptr;    // face intermediates of the double forward pass (for the adjoint)
  double* dscalar = nullptr; // (4) device scalars
  double* jac_face = nullptr; // (nf, 2, nfld, nfld) face flux derivatives of the Jacobian assembly
  const int* jac_indptr = nullptr;  // the block pattern last assembled into, and its block count
  long jac_nnzb = 0;
  int* wnear = nullptr;       // (nc) nearest SST wall face (internal index), turbulent cases
  bool wd_external = false;   // wd set by fv_case_set_wall_distance (wnear no longer describes it)
  bool wd_missing = false;    // turbulent, no SST wall face, distance not yet set: no evaluation
  NodeAdjoint* nadj = nullptr;  // mesh-coordinate adjoint workspace, allocated on first use
  int tb = 128;                 // threads per block of the residual / JVP / VJP stages (autotuned)
  int tbs[FV_MAX_STAGES] = {128, 128, 128, 128, 128, 128, 128, 128, 128, 128, 128, 128};
                                // ... per stage (the profiling marks' order), tuned one by one
  int persistent = 0;           // residual + VJP as one cooperative launch (compact, upwind cases)
  int pchunk = 1;               // ... consecutive cells / faces per thread per stage
  int pblock = 128;             // ... threads per block
  int* sched = nullptr;         // (nc) warp-coherent cell order of the cell stages
  int n_cell_classes = 0;       // distinct face-list patterns it groups
  double* lin_aux = nullptr;    // face intermediates of the held linearisation (fv_case_linearise)
  double* lin_fl = nullptr;     // ... and its primal face fluxes (nfld, nf)
  double* lin_ac = nullptr;     // ... its face coefficients and mass-flux estimates (3, nf)
  double* lin_g = nullptr;      // ... its gradients (nfld, dim, nc)
  double* lin_r = nullptr;      // ... its residual (nfld, nc)
  double* lin_cl = nullptr;     // ... its SST closure fields (7, nc)
  double* lin_cc = nullptr;     // ... the off-wall closure and source forms (29, nc)
  double* lin_src = nullptr;    // a product's off-wall k / omega source tangents (2, nc)
  int lin_valid = 0;            // a linearisation is held (parameter / geometry changes clear it)
  int lin_use = 0;              // the running dual-number pass takes its flux stage from it
  int fwd_valid = 0;            // work / aux hold the double forward pass of the last VJP's state
  double* mu_cell = nullptr;    // (nc) per-cell viscosity field (laminar batched instances)
  double* flx = nullptr;        // (nfld, nf) weights of a face-flux functional (internal order)
  bool flx_active = false;      // the adjoints add flx to their face-flux cotangents
  bool flx_viscous = false;     // ... with the pressure part p_f A n_i taken out
  double* red = nullptr;        // reduction partials of the functional
  float* f32 = nullptr;         // fp32 copies: wd, wdg, 1/wd, 1/wd^2, per-cell viscosity
  float* f_state = nullptr;     // (n_unknowns) fp32 state of an fp32 pass
  float* f_tangent = nullptr;   // (n_unknowns) fp32 tangent of an fp32 pass
  double* phys = nullptr;       // (n_unknowns) physical state of a log-transformed case
  double* tphys = nullptr;      // (n_unknowns) physical tangent of a log-transformed case
  CaseView view;
  // optional per-stage CUDA-event profiling (fv_case_profile_begin / _end)
  std::vector<cudaEvent_t> prof_events;  // max_runs * (FV_MAX_STAGES + 1)
  int prof_max_runs = 0, prof_runs = 0, prof_stages = 0;
  std::vector<int> prof_run_marks;  // boundaries recorded per run
};
// Record the stage boundary `k` of the current profiled run (no-op when profiling is off);
// fv_prof_end_run closes the run.  Boundaries 0..6 delimit the six forward stages, 7..11 the
// five adjoint stages of a VJP.
void fv_prof_mark(FvCase* c, int k, cudaStream_t s);
void fv_prof_end_run(FvCase* c);

// fp32 mirrors for the fp32 dual-number passes (made on first use)
int fv_d2f(long n, const double* in, float* out, cudaStream_t s);
int fv_mesh_ensure_f32(FvMesh* m, cudaStream_t s);
int fv_case_eddy_viscosity(FvCase* cs, const double* state, double* nut, cudaStream_t s);
int fv_case_ensure_f32(FvCase* c, cudaStream_t s);
int fv_case_run(FvCase* c, const double* state, const double* tangent, int tangent_kind,
                double* residual, double* jv, cudaStream_t s);
int fv_case_vjp_run(FvCase* c, const double* state, const double* w, double* residual, double* out,
                    cudaStream_t s);
// The residual at a (physical) state with its face intermediates and primal face fluxes kept for
// the linearised JVP (residual.cu); refuses limited reconstruction.
int fv_case_linearise(FvCase* c, const double* state, double* residual, cudaStream_t s);
// The VJP's forward pass at a (physical) state, held in the workspace for fv_case_vjp_held, which
// runs only the adjoint stages (residual.cu).  Any other evaluation drops the hold.
int fv_case_hold_forward(FvCase* c, const double* state, double* residual, cudaStream_t s);
int fv_case_vjp_held(FvCase* c, const double* state, const double* w, double* out, cudaStream_t s);
// Frozen reach-1 Jacobian by per-face forward-mode derivatives (residual.cu); D holds
// fv_jac_face_bytes.
// Mesh-coordinate adjoint dL/dnodes of L = w . R(state, nodes) (residual.cu).
int fv_case_node_vjp(FvCase* c, const double* state, const double* w, double* dnodes,
                     cudaStream_t s);
void fv_node_adjoint_free(FvCase* c);
// Face-flux functional J = sum_f sum_q w_qf FL_q(f) (- the pressure part), its value and partial
// derivatives (residual.cu).
int fv_case_face_functional(FvCase* c, const double* state, const double* weights_ref,
                            int viscous_only, double* value, double* dstate, double* dparams,
                            double* dnodes, cudaStream_t s);
int fv_case_assemble_frozen(FvCase* c, const double* state, const int* indptr, const int* indices,
                            void* values, void* D, int fp32, cudaStream_t s);
size_t fv_jac_face_bytes(int dim, int turb, long nf);
enum { FV_TAN_NONE = 0, FV_TAN_STATE = 1, FV_TAN_MU = 2, FV_TAN_INLET = 3, FV_TAN_FROZEN = 4,
       FV_TAN_STATE32 = 5, FV_TAN_FROZEN32 = 6 };  // 32: the tangent pass in fp32 (DualF)

// Wall distance + gradient for a turbulent case (mesh.cu).
int fv_wall_distance_compute(FvMesh* m, const unsigned char* swall_dev, int n_wall_faces,
                             double* wd, double* wdg, int gradient_sweeps,
                             double gradient_relaxation, int* nearest_face, cudaStream_t s);
// The Green-Gauss gradient of a given wall distance (the case's scheme).
int fv_wall_distance_gradient(FvMesh* m, const unsigned char* swall_dev, const double* wd,
                              double* wdg, int sweeps, double rel, cudaStream_t s);
// The same distance to each cell's kept nearest wall face (after the nodes moved) and its gradient.
int fv_wall_distance_refresh(FvMesh* m, const unsigned char* swall_dev, const int* nearest,
                             double* wd, double* wdg, int sweeps, double rel, cudaStream_t s);
// Corrected Green-Gauss sweeps of one scalar field's gradient (residual.cu): on entry x0 holds
// rel * B phi / V and num holds B phi; the last iterate lands in x0 or x1 by the sweep count's
// parity (x0 when sweeps - 1 is even).
int fv_gg_sweeps_scalar(const MeshView& m, int sweeps, double rel, const double* num, double* x0,
                        double* x1, double* wface, cudaStream_t s);
