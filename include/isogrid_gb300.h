/* C ABI of the IsoGridDFT GB300 hot path (libisogrid_gb300.so).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (cudaStream_t passed as void*), enqueues its work on that stream and
 * returns an int status (IGD_OK = 0).  Nothing here allocates device memory:
 * callers pass all inputs, outputs and workspace.  Fields are C-order
 * (nx, ny, nz) arrays with z fastest (the reference's layout,
 * grid/mapping.py:123-135); an orbital block is nb such fields separated by
 * `orbital_stride` elements (ks/eigensolver.py:197-216).
 *
 * dtype: IGD_F32 or IGD_F64 selects the arithmetic type of orbitals,
 * potentials and geometry coefficients; reductions always accumulate in FP64.
 */
#ifndef ISOGRID_GB300_H
#define ISOGRID_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  IGD_OK = 0,
  IGD_ERR_ARG = 1,         /* bad size, pointer or enum value            */
  IGD_ERR_DTYPE = 2,       /* unsupported dtype                          */
  IGD_ERR_CUDA = 3,        /* a CUDA launch or runtime call failed       */
  IGD_ERR_BREAKDOWN = 4,   /* Krylov breakdown (|p.Ap| or |rho| tiny)     */
  IGD_ERR_NOT_CONVERGED = 5, /* informational: iteration limit reached   */
  IGD_ERR_NONFINITE = 6,   /* NaN/Inf detected in an input or iterate     */
  IGD_ERR_TOO_LARGE = 7    /* size exceeds a documented fixed maximum     */
};
enum { IGD_F32 = 0, IGD_F64 = 1 };
enum { IGD_CLOSURE_TRIAL_FIX = 0, IGD_CLOSURE_PRODUCTION = 1 };
enum { IGD_GRID_MONITOR = 0, IGD_GRID_LEGACY = 1 };
enum { IGD_PREC_FP64 = 0, IGD_PREC_MIXED = 1 };

/* Library version / build identification (for loaders and tests). */
int igd_version(void);

/* Read the calling host thread's device error word (bit 0: a bounded
 * mbarrier wait inside a kernel this thread launched gave up, so that
 * launch's output is invalid) into *flags_out, optionally clearing it;
 * synchronises `stream`.  Each host thread has its own word (64 words,
 * assigned in thread order; a 65th thread shares the first thread's word).
 * No reference counterpart: the reference has no device code. */
int igd_error_flags(unsigned int* flags_out, int clear, void* stream);
/* Self-test of that failure path (no reference counterpart): one kernel waits on
 * an mbarrier that nothing arrives at, gives up after `polls` polls (1..65536)
 * and sets bit 0 of the calling thread's error word; no fault, no hang, and the
 * context stays usable. */
int igd_selftest_wait_timeout(int polls, void* stream);

/* ---------------------------------------------------------------- geometry
 * Fold the monitor-grid geometry into the 7 coefficient fields the stencil
 * streams: A~ab = J g^ab / (4 h_a h_b) for ab in (xx, yy, zz, xy, xz, yz) and
 * 1/J, stored as 7 consecutive fields of n = nx*ny*nz elements of `dtype`.
 * jacobian: n doubles; inverse_metric: n*9 doubles ((nx,ny,nz,3,3) as in
 * grid/monitor_model.py:166).  h = logical spacing per axis.
 * Replaces the per-call reads of grid_geometry.jacobian / .inverse_metric_tensor
 * in ops/kinetic.py:212-252. */
int igd_agrid_prepare_geometry(int dtype, int nx, int ny, int nz, double hx, double hy, double hz,
                               const double* jacobian, const double* inverse_metric, void* coeffs, void* stream);

/* -------------------------------------------------------------------- H.Psi
 * out_i = kscale * (1/J) d_a (J g^ab d_b psi_i) + vscale * veff * psi_i for
 * i < nb, on the monitor A-grid.  closure selects the edge rule of both
 * derivative passes: IGD_CLOSURE_PRODUCTION = np.gradient(edge_order=2)
 * (ops/kinetic.py:190-209, 255-276), IGD_CLOSURE_TRIAL_FIX = zero ghost
 * (ops/kinetic.py:165-187).  kscale = -0.5 gives the kinetic operator
 * (ops/kinetic.py:340-358), kscale = 1 the Laplacian (:279-337); veff may be
 * NULL.  Fused replacement of apply_fixed_potential_static_local_operator
 * (ks/eigensolver.py:729-784) for a whole orbital block. */
int igd_hpsi_agrid(int dtype, int closure, int nx, int ny, int nz, const void* coeffs, const void* veff,
                   const void* psi, void* out, int nb, long long orbital_stride, double kscale, double vscale,
                   void* stream);

/* Host-to-host form of igd_hpsi_agrid for callers whose orbital block lives in
 * host memory (the reference's NumPy block apply, ks/eigensolver.py:773-784):
 * host_psi and host_out hold nb contiguous orbitals of nx*ny*nz values of
 * `dtype` (pinned host memory for the copies to overlap; pageable memory works
 * without overlap); dev_in and dev_out are caller-owned device scratch of the
 * same size.  The block streams through in chunks of `chunk` orbitals (0: eight
 * chunks of nb/8 orbitals, rounded up): the copy in of chunk i+1, the stencil on chunk i and the
 * copy out of chunk i-1 overlap on two copy streams of the calling thread.
 * The work is ordered after earlier work on `stream`, later work on `stream`
 * is ordered after it, and the call returns once host_out is complete. */
int igd_hpsi_agrid_host(int dtype, int closure, int nx, int ny, int nz, const void* coeffs, const void* veff,
                        const void* host_psi, void* host_out, int nb, double kscale, double vscale, void* dev_in,
                        void* dev_out, int chunk, void* stream);

/* Kernel selection for igd_hpsi_agrid (a test hook, per host thread): 0 = the
 * fastest applicable kernel (whole-row z-vectorised, then the tiled TMA
 * kernel, then the cp.async kernel), 1 = skip the whole-row kernel, 2 = the
 * cp.async kernel only.  No reference counterpart. */
int igd_hpsi_select(int path);
/* Autotuner of the whole-row H.Psi kernel (process-wide; no reference
 * counterpart): mode 1 (default) times every orbitals-per-CTA choice (4, 2, 1)
 * on the caller's stream the first time a (closure, grid shape, orbital count,
 * v_eff present) key is seen outside a stream capture (fastest of three
 * launches each) and keeps the fixed rule unless another choice is at least
 * 20 % faster; mode 0 uses the fixed rule.  The candidates compute identical
 * values. */
int igd_hpsi_autotune(int mode);
/* The tuner's picks, one text line per key ("closure nx ny nz nb veff -> NB (us)");
 * returns the length written, or the full length when buf is null. */
int igd_hpsi_autotune_report(char* buf, int len);
/* Test hook: Gram kernel for the calling host thread (0 automatic, 1 tensor
 * pipe where it applies, 2 pipelined CUDA-core, 3 register-tiled CUDA-core).
 * No reference counterpart. */
int igd_gram_select(int path);
/* Kernel that ran the calling thread's last igd_block_gram (1, 2, 3 as above). */
int igd_gram_last_path(void);

/* Legacy separable sinh grid, 7-point flux form with zero ghosts
 * (ops/kinetic.py:87-153).  axis_coeffs holds 6 arrays of FP64 in order
 * cxm[nx], cxp[nx], cym[ny], cyp[ny], czm[nz], czp[nz] with
 * out = kscale * sum_axes (cp (psi[i+1]-psi[i]) - cm (psi[i]-psi[i-1]))
 *       + vscale * veff * psi. */
int igd_hpsi_legacy(int dtype, int nx, int ny, int nz, const double* axis_coeffs, const void* veff,
                    const void* psi, void* out, int nb, long long orbital_stride, double kscale, double vscale,
                    void* stream);

/* ------------------------------------------------------------------ Poisson
 * Interior solve of -L u = f with u = 0 on the faces (f is a full field; its
 * face entries are ignored), L the monitor Laplacian with the np.gradient
 * closure (grid_kind IGD_GRID_MONITOR, op_coeffs64/op_coeffs32 = folded
 * coefficients from igd_agrid_prepare_geometry in FP64 / FP32) or the legacy
 * 7-point Laplacian (IGD_GRID_LEGACY, op_coeffs64 = the axis coefficients of
 * igd_hpsi_legacy).  BiCGSTAB from x0 = 0, stopping at ||r||_2 <= rtol ||f||_2
 * (the SciPy rule of poisson/open_boundary.py:1017-1064 and :1229-1276).
 * precision IGD_PREC_FP64: FP64 Krylov; IGD_PREC_MIXED: FP32 BiCGSTAB inside
 * FP64 iterative refinement (FP64 residual recomputed each round).  Host-
 * blocking (convergence checks every 8 iterations).  info (host, 6 doubles):
 * iterations, relative residual, status, refinement rounds, ||f - A u||_2,
 * max |f - A u| (interior).  Returns IGD_ERR_BREAKDOWN on Krylov breakdown;
 * reaching max_iterations is reported through info, not as an error. */
long long igd_poisson_workspace_bytes(int precision, long long n);
/* Test hook for the calling host thread: 0 = the inner FP32 solve of the mixed
 * Poisson path uses the fused iteration (dot products from the stencil
 * epilogue, scalars recomputed in the vector kernels) wherever the whole-row
 * operator applies, 1 = the unfused iteration.  No reference counterpart. */
int igd_poisson_select(int path);
/* The JAX route of the monitor-grid solve (poisson/poisson_jax.py:675-750):
 * preconditioned CG on the interior -L (production closure, FP64) from x = 0,
 * stopping when max |r| < tolerance or after max_iterations, with the route's
 * preconditioners (poisson_jax.py:248-579): IGD_PCG_NONE; IGD_PCG_DIAG
 * (pc_data = 1/diag as a full field, zero faces); IGD_PCG_SEPARABLE (pc_data32 =
 * the three orthonormal sine matrices mx^2, my^2, mz^2 then the inverse separable
 * spectrum mx*my*mz, m = n - 2; applied in FP32); IGD_PCG_LINE (pc_data = lower,
 * c', 1/den of the Thomas factorisation along pc_axis, three full fields).  f is
 * the full right-hand side (faces ignored); x gets the solution with zero faces;
 * info[0] iterations, info[1] max |r|, info[2] converged. */
enum { IGD_PCG_NONE = 0, IGD_PCG_DIAG = 1, IGD_PCG_SEPARABLE = 2, IGD_PCG_LINE = 3 };
long long igd_poisson_pcg_workspace_bytes(int precond, int nx, int ny, int nz);
int igd_poisson_pcg(int nx, int ny, int nz, const double* op_coeffs64, const double* f, double* x, double tolerance,
                    int max_iterations, int precond, const double* pc_data, const float* pc_data32, int pc_axis,
                    void* workspace, long long workspace_bytes, double* info, void* stream);
int igd_poisson_solve(int grid_kind, int precision, int nx, int ny, int nz, const void* op_coeffs64,
                      const void* op_coeffs32, const double* f, double* u, double rtol, int max_iterations,
                      void* workspace, long long workspace_bytes, double* info, void* stream);
/* Same solve starting from the u passed in (interior values; faces are reset
 * to zero): a correction solve to rtol ||f|| / ||f - A u||, so a good starting
 * point (the previous SCF step's solution) needs fewer iterations.  No
 * reference counterpart (the reference always starts from zero). */
int igd_poisson_solve_from(int grid_kind, int precision, int nx, int ny, int nz, const void* op_coeffs64,
                           const void* op_coeffs32, const double* f, double* u, double rtol, int max_iterations,
                           void* workspace, long long workspace_bytes, double* info, void* stream);

/* ------------------------------------------------------- multipole boundary
 * Moments are 10 doubles (q, p_x, p_y, p_z, Q_xx, Q_xy, Q_xz, Q_yy, Q_yz, Q_zz)
 * written to device memory.  Replaces _compute_multipole_boundary_condition
 * and helpers (poisson/open_boundary.py:182-495, :559-719, :794-987). */
/* sum rho W frac (1, d, 3dd - r^2) about c (frac may be NULL) (:816-851, :267-296). */
int igd_multipole_nodal_moments(long long n, const double* rho, const double* cell_volumes, const double* x,
                                const double* y, const double* z, const double* frac, double cx, double cy, double cz,
                                double* out, void* stream);
/* per-cell quadratic least-squares fit over the 4x4x4 nodes + 2x2x2 sub-cell
 * quadrature (:299-464 mode 0; :589-699 modes 1, 2); cells = (i,j,k) int triples. */
int igd_multipole_cell_quadrature(int nx, int ny, int nz, const double* x, const double* y, const double* z,
                                  const double* jacobian, const double* rho, const int* cells, int ncells,
                                  double subcell_volume, int mode, double cx, double cy, double cz, double* out,
                                  int* fail, void* stream);
/* multipole potential on the six faces (:467-495); add = 1 accumulates. */
int igd_multipole_boundary(int nx, int ny, int nz, const double* x, const double* y, const double* z,
                           const double* moments, int order, double cx, double cy, double cz, double* out, int add,
                           void* stream);
/* f = 4 pi rho + L(b) inside, zero on faces (:1143-1146). */
int igd_poisson_rhs(int nx, int ny, int nz, const double* rho, const double* Lb, double* f, void* stream);
/* v = b on faces, u inside (:1173-1174). */
int igd_poisson_compose(int nx, int ny, int nz, const double* b, const double* u, double* v, void* stream);
/* *out = sum a b w in FP64 (b, w may be NULL): integrate_field (ops/kinetic.py:61-66),
 * evaluate_hartree_energy (poisson/hartree.py:117-129). */
int igd_weighted_sum(int dtype, long long n, const void* a, const void* b, const double* w, double* out, void* stream);

/* --------------------------------------------------------- LSDA and density
 * igd_lsda replaces evaluate_lsda_terms / evaluate_lsda_energy (xc/lsda.py:70-174;
 * the reference calls libxc "lda,vwn" through PySCF): Slater + VWN5
 * (functional 0) or Slater + PW92 (1), arithmetic in `math` (IGD_F64 / IGD_F32),
 * I/O in `dtype`, energy sum rho eps W in FP64.  Outputs may be NULL;
 * flags |= 1 (non-finite input), 2 (negative below -1e-14). */
int igd_lsda(int dtype, int math, int functional, long long n, const void* rho_up, const void* rho_down, void* eps,
             void* v_up, void* v_down, void* energy_density, const double* w, double* energy, int* flags,
             void* stream);
/* rho (FP64) [+]= sum_i occ_i psi_i^2; integral = sum rho W
 * (_build_density_from_occupied_orbitals, scf/driver.py:663-676). */
int igd_density(int dtype, long long n, int nb, long long stride, const void* psi, const double* occupations,
                const double* w, double* rho, double* integral, int accumulate, void* stream);
/* rho *= target / *integral on the device (_renormalize_density, scf/driver.py:679-690). */
int igd_density_renormalize(long long n, double* rho, const double* integral, double target, int* flags,
                            void* stream);
/* *out = squared weighted residual of a spin-density pair (_density_residual, scf/driver.py:693-702). */
int igd_density_residual2(long long n, const double* up_in, const double* dn_in, const double* up_out,
                          const double* dn_out, const double* w, double* out, void* stream);

/* ------------------------------------------------- eigensolver linear algebra
 * Orbital blocks are row-major (k, n) with a row stride.  Gram replaces
 * weighted_overlap_matrix (ks/eigensolver.py:246-272) and
 * _weighted_overlap_columns (ks/eigensolver_jax.py:105); rotation replaces the
 * basis @ coeffs products and two-part compressions (eigensolver_jax.py:178-251). */
long long igd_block_gram_workspace_bytes(long long n, int a, int b);
/* out (a x b FP64) [+]= A diag(w) B^T (w may be NULL); FP64 accumulation.
 * FP32 blocks of up to 64 x 64 outputs with 16-byte aligned rows run on the
 * tensor pipe (tcgen05, 3xTF32 split products; FP32 accumulation over 128
 * points, the hi*hi products apart from the cross terms; FP64 beyond) on grids
 * of 2^18 points or more; other shapes on CUDA cores. */
int igd_block_gram(int dtype, long long n, int a, const void* A, long long sa, int b, const void* B, long long sb,
                   const double* w, double* out, int accumulate, void* workspace, long long workspace_bytes,
                   void* stream);
/* out (c x n) [+]= A^T C1 + B^T C2 with FP64 coefficients C1 (a x c), C2 (b x c). */
int igd_block_rotate(int dtype, long long n, int a, const void* A, long long sa, const double* C1, int b,
                     const void* B, long long sb, const double* C2, int c, void* out, long long so, int accumulate,
                     void* stream);

/* Stream-ordered copy of `bytes` from host memory (pinned for an asynchronous
 * copy) to device memory: the eigensolver's per-iteration coefficient upload.
 * No reference counterpart. */
int igd_copy_h2d(void* dst, const void* src, long long bytes, void* stream);

/* Host half of one fused eigensolver iteration (plain C++, no device work):
 * from G0 = [B;R]^T W [HB;HR] and G1 = [B;R]^T W [B;R] ((m+k) x (m+k) FP64,
 * row-major) the W-projection of R against B, its rank-revealing whitening
 * (eigenvalues > cut * max diag(R^T W R)), the trial Rayleigh-Ritz on [B R'],
 * the compression to m columns and its re-whitening.  Writes
 * coeff = [CB (m x m); CR (k x m); V_k (m x k); -V_k diag(lam_k) (m x k)],
 * P (m x m), lam (m, ascending), V (m x m) and the kept rank.  m + k <= 64.
 * The algebra of eigensolver_jax.py:417-524 for one iteration, reordered.
 * IGD_ERR_NONFINITE on a numerical failure (callers fall back). */
int igd_subspace_step_host(int m, int k, const double* G0, const double* G1, double cut, double* coeff, double* P,
                           double* lam, double* V, int* rank_out);

/* Residual preconditioner of the eigensolver (no reference counterpart: the
 * reference expands its subspace with the raw residual): one damped Jacobi
 * sweep for (T + sigma) t = r on k columns of n values, dinv = 1/(diag T + sigma).
 * first != 0: t = dinv r; else t += omega dinv (r - tt - sigma t) with tt = T t
 * from the stencil.  Column strides sr, st, stt in elements. */
int igd_precond_jacobi(int dtype, long long n, int k, const void* r, long long sr, void* t, long long st,
                       const void* tt, long long stt, const void* dinv, double sigma, double omega, int first,
                       void* stream);

/* ---------------------------------------------------------------- GTH terms
 * Local GTH potential summed over atoms (pseudo/local.py:138-357); atoms holds
 * 8 doubles per atom: x, y, z, Z_ion, rloc, C1, C2, C3. */
int igd_gth_local_potential(long long n, const double* x, const double* y, const double* z, int natoms,
                            const double* atoms, double* out, void* stream);

/* Hellmann-Feynman force of the local GTH potential on each atom (no reference
 * counterpart; the reference has no forces): out[3a + c] = sum_i rho_i w_i
 * dV_a/dr (x_i - R_a)_c / r for the atoms table of igd_gth_local_potential
 * (8 doubles per atom).  rho, w: n doubles.  out: 3 * natoms doubles. */
int igd_gth_local_force(long long n, const double* x, const double* y, const double* z, const double* rho,
                        const double* w, int natoms, const double* atoms, double* out, void* stream);

/* Near-core local-GTH patch correction (pseudo/local.py:379-703): for nq patch
 * points (qx, qy, qz), the k <= 16 nearest of the n main-grid points (exhaustive
 * search, replaces the cKDTree query of _interpolate_field_to_patch_points) and
 * their normalised 1/d^2 weights (a point within 1e-12 of a grid point copies it).
 * idx: nq*k int32, w: nq*k doubles.  igd_patch_gather: out[q] = sum_j w[q][j] field[idx[q][j]]. */
int igd_patch_knn(int nq, const double* qx, const double* qy, const double* qz, long long n, const double* x,
                  const double* y, const double* z, int k, int* idx, double* w, void* stream);
int igd_patch_gather(int nq, int k, const int* idx, const double* w, const double* field, double* out,
                     void* stream);
/* out += scale * V_nl psi over compact projector point lists
 * (pseudo/nonlocal.py:209-337); workspace: 2 * nproj * nb doubles. */
int igd_gth_nonlocal_apply(int dtype, int nproj, const long long* offsets, const int* idx, const double* val,
                           int ngroups, const int* groups, const long long* hoff, const double* hmat,
                           const double* w, const void* psi, void* out, int nb, long long stride, double scale,
                           double* workspace, void* stream);
/* Projections <p_j | psi_o>_W (nproj x nb doubles, overwritten): the gather
 * stage of igd_gth_nonlocal_apply.  With tables of the projector gradients in
 * val it gives <d p_j / d x | psi_o>_W for the nonlocal Hellmann-Feynman force
 * (no reference counterpart: the reference computes no forces). */
int igd_gth_projections(int dtype, int nproj, const long long* offsets, const int* idx, const double* val,
                        const double* w, const void* psi, int nb, long long stride, double* out, void* stream);

/* ------------------------------------------------------ monitor A-grid build
 * Device restatement of grid/monitor_geometry.py (FP64).  Coordinates are SoA
 * (X[n], Y[n], Z[n]) of n = nx*ny*nz doubles, contiguous as one 3n buffer.
 * Replaces evaluate_global_monitor_field (:51-113); atoms holds 13 doubles per
 * atom (position, kinetic weight / radius / exponent, local weight / radius /
 * exponent, projector weight / radius / exponent, monitor cap). */
int igd_grid_monitor_field(long long n, const double* X, const double* Y, const double* Z, int natoms,
                           const double* atoms, double* values, double* raw, void* stream);
/* 7-point smoothing and max(., 1) (_smooth_monitor_field, :116-135). */
int igd_grid_smooth(int nx, int ny, int nz, const double* monitor, double* out, double smoothing, void* stream);
/* Up to `sweeps` damped-Jacobi sweeps of _solve_weighted_harmonic_coordinates
 * (:268-321) ping-ponging buf0/buf1 (3n doubles each, buf0 = start); state is
 * a 16-byte workspace whose int at byte offset 12 receives the index of the
 * sweep that met `tol` (-1 if none).  No host synchronisation. */
int igd_grid_harmonic_sweeps(int nx, int ny, int nz, const double* monitor, double* buf0, double* buf1, double hx,
                             double hy, double hz, double relaxation, double tol, int sweeps, void* state,
                             void* stream);
/* Zero-allocation variant of igd_grid_harmonic_sweeps.  No counterpart in the
 * reference.  For hosts that cannot let a library call cudaMalloc (an SCF
 * driver embedded in a larger code that pre-reserves its whole device memory
 * budget and treats later allocations as errors; cudaMalloc may also
 * synchronise the device).  The second coordinate buffer and the sweep state
 * live in a fixed library-owned device array sized for grids of at most
 * IGD_NOALLOC_MAX_POINTS points (6 MiB, held by every GPU that loads the
 * library until exit); larger grids return IGD_ERR_TOO_LARGE.  coords (3n
 * doubles) holds the start (with the fixed faces) and receives the result;
 * *conv_sweep_out (device int, may be NULL) receives the converged sweep index
 * or -1.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * The address is remembered per device ordinal for the rest of the process and
 * belongs to the device's primary context: calling this entry point under
 * another context made current through the driver API, or after
 * cudaDeviceReset, is not supported.
 * All calls share the array and it keeps the last call's contents; the state
 * is cleared at the start of every call.  Calls that overlap on the GPU race:
 * serialise them.  Allocates nothing. */
#define IGD_NOALLOC_MAX_POINTS (64LL * 64LL * 64LL)
int igd_grid_harmonic_sweeps_noalloc(int nx, int ny, int nz, const double* monitor, double* coords, double hx,
                                     double hy, double hz, double relaxation, double tol, int sweeps,
                                     int* conv_sweep_out, void* stream);
/* min det(covariant basis) of X + alpha (S - X) (alpha < 0: of X) into
 * *out_min (device double); scratch = 8 bytes (_backtracking_update, :376-396). */
int igd_grid_min_jacobian(int nx, int ny, int nz, const double* X, const double* S, double alpha, double hx,
                          double hy, double hz, void* scratch, double* out_min, void* stream);
/* X <- X + alpha (S - X) over 3n values, *out_max = max |change| (device). */
int igd_grid_relax_update(long long n3, double* X, const double* S, double alpha, void* scratch, double* out_max,
                          void* stream);
/* Covariant basis, metric, inverse metric ((n,3,3) each), Jacobian, cell
 * volumes and (n,3) point spacings (_basic_geometry_from_coordinates, :353-373). */
int igd_grid_geometry(int nx, int ny, int nz, const double* X, double hx, double hy, double hz, double* basis,
                      double* metric, double* inverse_metric, double* jacobian, double* cell_volumes, double* spacing,
                      void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ISOGRID_GB300_H */
