/* emerge_gb300 — C ABI of the GB300 (sm_103a) frequency-domain FEM hot path.
 *
 * Every entry point returns 0 on success and a nonzero status otherwise;
 * emg_last_error() then describes the failure (thread-local string).  Array
 * arguments are plain pointers with the sizes passed beside them; "device"
 * pointers are CUDA global-memory addresses on the current device, "host"
 * pointers are ordinary (preferably pinned) host memory.  ``stream`` is a
 * cudaStream_t passed as void* (NULL = legacy default stream).  Arrays use the
 * reference's numpy C-order layouts, with int32 indices and complex values
 * stored as interleaved (re, im) doubles.
 */
#ifndef EMERGE_GB300_H
#define EMERGE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMG_OK 0
#define EMG_ERR_ARG 1      /* invalid argument (sizes, null pointers, index out of range) */
#define EMG_ERR_CUDA 2     /* a CUDA runtime call failed */
#define EMG_ERR_MESH 3     /* the mesh violates an assumption (see emg_last_error) */
#define EMG_ERR_LIMIT 4    /* a documented size limit was exceeded */
#define EMG_ERR_NOCONV 5   /* an iterative solve did not reach its tolerance */

/* Thread-local description of the last failing call. */
const char* emg_last_error(void);

/* Library version string. */
const char* emg_version(void);

/* ------------------------------------------------------------ assembly ---
 * Replaces fem/physics/edm/optimized_assembly.py:43-64
 * (tet_mass_stiffness_matrices) and :66-116 (_matrix_builder): integrates the
 * second-order Nedelec curl-curl (E) and mass (B) element matrices of every
 * tetrahedron and sums them into CSR matrices whose pattern equals
 * scipy's coo_matrix(...).tocsr() of the reference COO triplets.
 */
typedef struct emg_plan emg_plan;

/* Builds the per-mesh assembly plan (DOF incidence lists and the CSR
 * pattern).  All arrays are DEVICE pointers, layouts as in Mesh3D/Nedelec2
 * (fem/mesh3d.py:224-355, fem/elements/nedelec2.py:32-62):
 *   nodes (3, n_nodes) f64; tets (4, n_tets); edges (2, n_edges);
 *   tris (3, n_tris); tet_to_field (20, n_tets); tet_to_edge (6, n_tets);
 *   edge_lengths (n_edges) f64.   n_field = 2*n_edges + 2*n_tris.
 * The plan keeps device copies of what it needs; the inputs may be freed
 * afterwards.  Synchronises ``stream``. */
int emg_plan_create(int64_t n_nodes, int64_t n_tets, int64_t n_edges, int64_t n_tris, int64_t n_field,
                    const double* nodes, const int32_t* tets, const int32_t* edges, const int32_t* tris,
                    const int32_t* tet_to_field, const int32_t* tet_to_edge, const double* edge_lengths,
                    void* stream, emg_plan** plan);

/* Number of stored entries of each of E and B. */
int64_t emg_plan_nnz(const emg_plan* plan);

/* Copies the CSR pattern to DEVICE arrays indptr (n_field+1, int64) and
 * indices (nnz, int32): rows sorted, columns sorted ascending within a row,
 * identical to scipy's coo_matrix((d,(rows,cols))).tocsr() pattern. */
int emg_plan_pattern(const emg_plan* plan, int64_t* indptr, int32_t* indices, void* stream);

/* Fills the CSR values of E (curl-curl, weighted by mu^-1) and B (mass,
 * weighted by eps) for one material assignment.  eps and mu_inv are DEVICE
 * arrays of n_tets complex scalars (isotropic materials: er = eps*I,
 * matinv(ur) = mu_inv*I, fem/physics/edm/optimized_assembly.py:98-105).
 * E_data and B_data are DEVICE arrays of nnz complex values.  Asynchronous on
 * ``stream``; deterministic (bitwise repeatable). */
int emg_assemble_tet(emg_plan* plan, const double* eps, const double* mu_inv, double* E_data, double* B_data,
                     void* stream);

/* Same as emg_assemble_tet with HOST arrays (eps, mu_inv: n_tets complex;
 * E_data, B_data: nnz complex): copies the materials in and the values out
 * around the device call and synchronises ``stream``.  This is the call a
 * host-side binding of tet_mass_stiffness_matrices makes.  When E_data and
 * B_data are page-locked (cudaHostAlloc'd or cudaHostRegister'ed), the fill
 * stores the values straight into them, overlapping the element arithmetic with
 * the device-to-host transfer; pageable outputs go through device staging. */
int emg_assemble_tet_host(emg_plan* plan, const double* eps, const double* mu_inv, double* E_data,
                          double* B_data, void* stream);

/* Tensor (anisotropic) materials: the general case of _matrix_builder
 * (fem/physics/edm/optimized_assembly.py:66-116), which passes the (3,3)
 * tensors er[:,:,t] and matinv(ur[:,:,t]) (fem/mth/optimized.py:441-461) to
 * ned2_tet_stiff_mass as Mm and Ms.
 *   eps9, mu_inv9: complex (9, n_tets), element (i, j) of tet t at
 *     (i*3 + j)*n_tets + t, i.e. the reference's (3,3,nT) array in C order;
 *     mu_inv9 already holds matinv(ur) per tet.
 * FP64 on the CUDA cores (warp per DOF entity, as emg_assemble_tet); same
 * pattern, same output layout.  Device arrays; the _host variant takes host
 * arrays, copies them around the call and synchronises ``stream``. */
int emg_assemble_tet_tensor(emg_plan* plan, const double* eps9, const double* mu_inv9, double* E_data,
                            double* B_data, void* stream);
int emg_assemble_tet_tensor_host(emg_plan* plan, const double* eps9, const double* mu_inv9, double* E_data,
                                 double* B_data, void* stream);

/* Releases the plan and its device memory. */
void emg_plan_destroy(emg_plan* plan);

/* matinv (fem/mth/optimized.py:440-461) of every tet's material tensor, on the device:
 * the Ms = matinv(ur) that _matrix_builder passes to ned2_tet_stiff_mass
 * (fem/physics/edm/optimized_assembly.py:98-105).  ncomp 9: s and out are complex
 * (9, n_tets) DEVICE arrays (the reference's (3,3,n_tets) C order); a tensor with all
 * off-diagonal entries zero gets its reciprocal diagonal, any other the reference's
 * adj(s) * det(s).  ncomp 1: complex scalars (isotropic s * I), out = 1 / s. */
int emg_matinv(int64_t n_tets, int ncomp, const double* s, double* out, void* stream);

/* ------------------------------------------------------- surface terms ---
 * Replace the per-triangle Robin kernels behind assemble_robin_bc_excited /
 * assemble_robin_bc (fem/physics/edm/assembler.py:83-144).  One thread per
 * triangle, FP64.  All arrays are DEVICE arrays, complex = interleaved doubles.
 */

/* ned2_tri_stiff_force (fem/mth/tri.py:575-695) for n_tris waveport triangles:
 * lcs_xy (2, 3, n_tris): local x and y of each triangle's three vertices (tri
 * vertex order) = rows 0-1 of local_basis @ (nodes - origin); uinc
 * (3, npts, n_tris) complex: U_inc at the quadrature points of each triangle;
 * dpts (4, npts): weights and barycentrics (gaus_quad_tri(4): npts = 6).
 * Outputs B_out (n_tris, 8, 8) and b_out (n_tris, 8), complex, gamma applied. */
int emg_tri_robin_force(int64_t n_tris, const double* lcs_xy, const double* uinc, const double* dpts, int npts,
                        double gamma_re, double gamma_im, double* B_out, double* b_out, void* stream);

/* ned2_tri_stiff (fem/mth/tri.py:697-797) for n_tris absorbing-boundary
 * triangles: xyz (3, 3, n_tris) = coordinate c of vertex k at [c][k][t];
 * edge_lengths (3, n_tris) of the edges (v0v1, v1v2, v0v2).  B_out (n_tris, 8, 8). */
int emg_tri_robin_abc(int64_t n_tris, const double* xyz, const double* edge_lengths, double gamma_re,
                      double gamma_im, double* B_out, void* stream);

/* pos[i] = position of column cols[i] within CSR row rows[i] of (indptr,
 * indices), -1 if the pair is not in the pattern. */
int emg_csr_positions(int64_t n, const int32_t* rows, const int32_t* cols, const int64_t* indptr,
                      const int32_t* indices, int64_t* pos, void* stream);

/* Deterministic scatter-add: for each segment s,
 * out[dst[s]] += alpha * sum(src[perm[k]] for k in [seg_ptr[s], seg_ptr[s+1])),
 * summed in perm order (complex).  Replaces the duplicate summation of
 * coo_matrix(...).tocsr() and the ``K + B_p`` / ``Bvec[indices] += bvec`` updates. */
int emg_segment_add(int64_t n_seg, const int64_t* seg_ptr, const int64_t* perm, const int64_t* dst,
                    const double* src, double alpha_re, double alpha_im, double* out, void* stream);

/* K = E - k0sq * B on a shared CSR pattern (fem/physics/edm/assembler.py:333). */
int emg_combine(int64_t nnz, const double* E, const double* B, double k0sq, double* K, void* stream);

/* ------------------------------------------------------------- solver ---
 * Replaces the solve of SolveRoutine.solve (fem/solver.py:405-469): restriction
 * to solve_ids (solver.py:434-435), the sparse solve (SuperLU / PARDISO / GMRES,
 * solver.py:220-309) and the scatter back with zeros on PEC DOFs
 * (solver.py:465).  Batched: Bc right-hand-side columns, column c solved with
 * stored matrix cmat[c] of Bm.  Layouts: matrices [nnz_r][Bm], vectors
 * [n_solve][Bc], complex interleaved, DEVICE arrays unless stated.
 */
typedef struct emg_rplan emg_rplan;

/* Restricted pattern A[ix_(solve_ids, solve_ids)] of a full CSR pattern
 * (indptr int64 N+1, indices int32), ILU(0) level schedule and update lists.
 * Synchronises ``stream``. */
int emg_rplan_create(int64_t N, const int64_t* indptr, const int32_t* indices, int64_t nnz_full, int64_t n_solve,
                     const int64_t* solve_ids, void* stream, emg_rplan** plan);
int64_t emg_rplan_n(const emg_rplan* plan);
int64_t emg_rplan_nnz(const emg_rplan* plan);
int64_t emg_rplan_levels(const emg_rplan* plan);
/* HOST copies of the restricted CSR pattern: indptr (n_solve+1), indices (nnz_r). */
int emg_rplan_pattern(const emg_rplan* plan, int64_t* indptr_out, int32_t* indices_out);
void emg_rplan_destroy(emg_rplan* plan);

/* Restricted matrices A_m = E - k2[m] B + sum_p gam[p][m] P_p (m < Bm) from
 * full-pattern values E, B (nnz_full complex), unit port matrices P
 * (n_ports x nnz_full complex), k2 (Bm doubles), gam (n_ports x Bm complex).
 * Forms K(k0) of fem/physics/edm/assembler.py:333,382-383 for Bm frequencies. */
int emg_rplan_form(const emg_rplan* plan, int64_t Bm, const double* E, const double* B, const double* k2,
                   int64_t n_ports, const double* P, const double* gam, double* A, void* stream);

/* In-place ILU(0) of Bm matrices (LU holds a copy of A on entry). */
int emg_ilu0(const emg_rplan* plan, int64_t Bm, double* LU, void* stream);

/* X <- (LU)^-1 X (forward and backward level-scheduled substitution). */
int emg_ilu_apply(const emg_rplan* plan, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* LU, double* X,
                  void* stream);

/* Y = A X, or Y = Bv - A X when Bv is not NULL. */
int emg_spmv(const emg_rplan* plan, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* A, const double* X,
             const double* Bv, double* Y, void* stream);

/* Y = A_c X (or Bv - A_c X) with the column operator formed on the fly from a
 * matrix family: A_c = sum_a coef[c][a] fam[a], fam [nfam][nnz_r], coef [Bc][nfam]
 * (complex, DEVICE), nfam <= 8.  A frequency sweep's A(k) = E - k^2 B +
 * sum_p gamma_p(k) P_p is the family (E, B, P_1, ...) with coefficients
 * (1, -k^2, gamma_1, ...): one copy of the matrices serves every frequency. */
int emg_spmv_family(const emg_rplan* plan, int64_t Bc, int nfam, const double* fam, const double* coef,
                    const double* X, const double* Bv, double* Y, void* stream);

/* out[i][c] = full[c][solve_ids[i]] (full: Bc vectors of N) and the inverse
 * scatter (zeros on removed DOFs). */
int emg_rplan_gather(const emg_rplan* plan, int64_t Bc, const double* full, double* out, void* stream);
int emg_rplan_scatter(const emg_rplan* plan, int64_t Bc, const double* x, double* full, void* stream);

/* Right-preconditioned restarted GMRES(restart <= 256) with CGS2, columns in
 * lockstep; x holds the initial guess on entry.  Stops a column at relative
 * residual tol or after max_iter total iterations; iters_out (Bc int32) and
 * resid_out (Bc doubles, explicit ||b - A x|| / ||b||) are DEVICE arrays.
 * Synchronises ``stream``. */
int emg_gmres(const emg_rplan* plan, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* A, const double* LU,
              const double* rhs, double* x, int restart, int max_iter, double tol, int32_t* iters_out,
              double* resid_out, void* stream);

/* ---------------------------------------------------- field evaluation ---
 * Second-order Nedelec field at arbitrary points, the counterpart of
 * ned2_tet_interp (fem/mth/tet.py:372-497).  points (3, n_points) row-major
 * (x[], y[], z[]); nodes (3, n_nodes); tets (4, n_tets), edges (2, n_edges), tris
 * (3, n_tris), tet_to_field (20, n_tets) int32; solution complex (n_field);
 * tetids (n_tetids) the tets searched, the last containing tet in list order
 * winning as in the reference; E_out (3, n_points) complex (zero where no tet
 * contains the point).  All DEVICE arrays. */
int emg_field_interp(int64_t n_points, const double* points, int64_t n_nodes, const double* nodes, int64_t n_tets,
                     const int32_t* tets, int64_t n_edges, const int32_t* edges, int64_t n_tris, const int32_t* tris,
                     const int32_t* tet_to_field, const double* solution, int64_t n_tetids, const int32_t* tetids,
                     double* E_out, void* stream);

/* Linear functionals of the field along directions: for point i with vector
 * dirs[:, i] (3, n_points), the 20 DOFs of the containing tet (same search as
 * emg_field_interp) in dofs_out[i*20 + k] and weights_out[i*20 + k] =
 * dirs[:, i] . N_k(points[:, i]), so that sum_k weights * solution[dofs] =
 * dirs . E(point) for every solution.  -1 / 0 where no tet contains the point.
 * The voltage of a lumped port (fem/physics/edm/emfreq3d.py:752-757) is the sum
 * of these over its line midpoints with the line steps as dirs.  DEVICE arrays. */
int emg_field_weights(int64_t n_points, const double* points, const double* dirs, int64_t n_nodes,
                      const double* nodes, int64_t n_tets, const int32_t* tets, int64_t n_edges, const int32_t* edges,
                      int64_t n_tris, const int32_t* tris, const int32_t* tet_to_field, int64_t n_tetids,
                      const int32_t* tetids, int32_t* dofs_out, double* weights_out, void* stream);

/* ------------------------------------------------------- slab solver ---
 * Direct block-tridiagonal factorization of the restricted system, the
 * counterpart of the reference's direct solvers (SolverSuperLU / SolverPardiso /
 * SolverUMFPACK, fem/solver.py:220-309) on guided-wave structures.  Breadth-first
 * level sets of the restricted pattern ("slabs") make A block tridiagonal; the
 * factor holds the dense inverses of the slab Schur complements in complex FP32
 * (precision 1) or FP64 (precision 2).  One emg_slab holds F factorizations at
 * once (e.g. anchor frequencies of a sweep), built in the same launches. */
typedef struct emg_slab emg_slab;

/* Slab structure of a restricted plan (host breadth-first search; synchronises
 * ``stream``).  With n_seeds > 0 the search starts from all seeds (HOST int64
 * restricted indices) at once, e.g. the DOFs next to one end face, which makes
 * the slabs planar cross-sections; otherwise from a pseudo-peripheral DOF.
 * order_key (HOST int64 per restricted DOF, may be NULL) orders the DOFs inside a
 * slab; a spatially local order with the two DOFs of an entity adjacent makes the
 * FP32 slab inverses 40-50x more accurate than the DOF-index order.
 * EMG_ERR_LIMIT if a slab is wider than 12288 DOFs. */
int emg_slab_create(const emg_rplan* plan, int64_t n_seeds, const int64_t* seeds, const int64_t* order_key,
                    void* stream, emg_slab** slab);
void emg_slab_destroy(emg_slab* slab);
/* info[8] (host): slabs, widest slab, dense entries per factor, coupling entries,
 * factors held, precision, perturbed pivots and skipped refinements (slabs whose
 * ||I - S X||_F was not below 1/2) of the last factorization. */
int emg_slab_info(const emg_slab* slab, int64_t* info);
/* HOST outputs: slab boundaries off_out (slabs+1) and, if not NULL, perm_out
 * (n_solve): restricted index of each slab position. */
int emg_slab_levels(const emg_slab* slab, int64_t* off_out, int32_t* perm_out);
/* Factor the F matrices A[:, amat[f]] (A: [nnz_r][Bm] complex, DEVICE; amat: F
 * HOST int32).  refine = 1 applies one Newton-Schulz step X <- X (2I - S X) to
 * every slab inverse whose residual ||I - S X||_F is below 1/2 (two extra dense
 * products; recovers most of the accuracy that inverting without pivoting across
 * 64-row tiles loses); 0 = none.
 * Replaces any factorization held.  Synchronises ``stream``. */
int emg_slab_factor(emg_slab* slab, int precision, int64_t F, const int32_t* amat, int64_t Bm, const double* A,
                    int refine, void* stream);
/* X_out = A_f^-1 X_in column by column, f = cfac[c] (HOST int32, Bc); X_in and
 * X_out are distinct DEVICE [n_solve][Bc] complex arrays. */
int emg_slab_apply(emg_slab* slab, int64_t Bc, const int32_t* cfac, const double* X_in, double* X_out, void* stream);
/* on != 0: the dense products of FP32-factor solves over wide column groups (see
 * emg_slab_set_wide_group) run on the tcgen05 tensor cores (TF32 products, FP32 accumulation);
 * the slab solve is a preconditioner, so the TF32 rounding only adds to the FP32
 * factor's own error.  Default off. */
int emg_slab_set_tensor_cores(emg_slab* slab, int on);
/* on != 0 (default): the rank-64 updates of FP32 factorizations (emg_slab_factor,
 * precision 1) run on the tcgen05 tensor cores with split-TF32 products (hi*hi +
 * hi*lo + lo*hi of x = hi + lo) and FP32 accumulation, i.e. FP32-equivalent rounding;
 * off: CUDA-core FP32.  FP64 factorizations always use the FP64 pipes.  A tensor-core
 * tile whose bounded wait runs out makes emg_slab_factor return EMG_ERR_CUDA with the
 * factors released.  (Replaces nothing in the reference: part of the GPU solver
 * behind fem/solver.py's solve slot.) */
int emg_slab_set_factor_tensor_cores(emg_slab* slab, int on);
/* Column groups of at least min_columns use 64 x 64 tiled dense products (with
 * split-K), narrower ones a warp per row.  Default 8: the tiled products are faster
 * even for 8-column groups (measured 80 vs 156 ms per solve on the 2 mm iris). */
int emg_slab_set_wide_group(emg_slab* slab, int min_columns);
/* Cap on the K splits of the tiled products (1..16; default 8).  The splits per
 * slab are chosen for two CTAs per SM with at least 256 K columns each. */
int emg_slab_set_max_splits(emg_slab* slab, int max_splits);

/* Flexible GMRES (FGMRES, restart <= 256) right-preconditioned by the slab
 * factors: column c solves A[:, cmat[c]] x = rhs with factor cfac[c] (HOST).  The
 * residual is FP64 throughout; with FP32 factors this is the mixed-precision
 * solve (FP32 inner, FP64 refinement).  Same outputs as emg_gmres. */
int emg_gmres_slab(const emg_rplan* plan, emg_slab* slab, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* A,
                   const int32_t* cfac, const double* rhs, double* x, int restart, int max_iter, double tol,
                   int32_t* iters_out, double* resid_out, void* stream);

/* Mixed-precision solve with FP32 slab factors: FP64 iterative refinement (true
 * residual b - A x in FP64 each step) around an inner FGMRES on complex FP32
 * vectors with an FP32 copy of A (made inside, nnz_r * Bm * 8 bytes), run to the
 * relative tolerance inner_tol per step (1e-4 gains four digits per step; FP32
 * vectors stall near 1e-6, so tighter values only add iterations).  iters_out:
 * inner iterations summed over the steps; *steps_out (HOST, may be NULL):
 * refinement steps. */
int emg_gmres_slab_mixed(const emg_rplan* plan, emg_slab* slab, int64_t Bc, const int32_t* cmat, int64_t Bm,
                         const double* A, const int32_t* cfac, const double* rhs, double* x, int restart, int max_iter,
                         double tol, double inner_tol, int32_t* iters_out, double* resid_out, int32_t* steps_out,
                         void* stream);

/* emg_gmres_slab with the operators of a matrix family (see emg_spmv_family)
 * instead of stored matrices. */
int emg_gmres_slab_family(const emg_rplan* plan, emg_slab* slab, int64_t Bc, int nfam, const double* fam,
                          const double* coef, const int32_t* cfac, const double* rhs, double* x, int restart,
                          int max_iter, double tol, int32_t* iters_out, double* resid_out, void* stream);

/* D = A B^T on the 5th-generation tensor cores (tcgen05.mma kind::tf32, FP32
 * accumulation in tensor memory): A (M x K, ld lda), B (N x K, ld ldb), D (M x N,
 * ld ldd), row-major FP32 DEVICE arrays; TF32 products (10-bit mantissa).
 * *status (DEVICE int32, set to 0 by the caller) becomes 1 if a tile's bounded
 * wait (10 ms) on its tensor-core work ran out; D is then invalid and the caller
 * discards it rather than relaunching on the same data. */
int emg_tc_gemm_tf32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
                     float* D, int64_t ldd, int32_t* status, void* stream);

/* ------------------------------------------------------ warm-start MLP ---
 * No counterpart in the reference (a sweep acceleration).  A multilayer
 * perceptron in_dim -> hidden_layers x hidden (tanh) -> out_dim with BF16
 * weights and activations, FP32 accumulation on the tcgen05 tensor cores
 * (kind::f16), FP32 master weights and Adam.  Dimensions are padded to
 * multiples of 16 internally; batches up to max_batch rows.  x, y, target are
 * DEVICE float arrays, row-major (batch x dim).  A tensor-core wait that runs out
 * makes emg_mlp_forward (and emg_mlp_train_step with grads_out) return
 * EMG_ERR_CUDA from then on. */
typedef struct emg_mlp emg_mlp;
int emg_mlp_create(int in_dim, int hidden, int hidden_layers, int out_dim, int max_batch, uint64_t seed,
                   emg_mlp** mlp);
int64_t emg_mlp_nparam(const emg_mlp* mlp);
/* HOST copies of the flat FP32 parameters: per layer W (N x K) then b (N). */
int emg_mlp_get_params(const emg_mlp* mlp, float* host_out);
int emg_mlp_set_params(emg_mlp* mlp, const float* host_in);
int emg_mlp_forward(emg_mlp* mlp, int batch, const float* x, float* y, void* stream);
/* Forward, mean-squared-error loss (*loss_out, DEVICE), backward; an Adam step
 * when lr > 0; the gradient is copied to grads_out (DEVICE, nparam) if not NULL. */
int emg_mlp_train_step(emg_mlp* mlp, int batch, const float* x, const float* target, float lr, float* loss_out,
                       float* grads_out, void* stream);
void emg_mlp_destroy(emg_mlp* mlp);

/* CSR pattern without any device allocation.  No counterpart in the reference:
 * an addition for callers that cannot call cudaMalloc, e.g. a host application
 * that must not allocate device memory of its own (its memory is owned by
 * another allocator, or cudaMalloc's implicit device synchronisation cannot be
 * afforded in its loop).  Computes the same indptr/indices as emg_plan_create +
 * emg_plan_pattern for meshes of at most 8192 tets and 65536 DOFs (larger sizes
 * return EMG_ERR_LIMIT).  Inputs and outputs are caller-owned DEVICE arrays:
 * tet_to_field (20, n_tets) int32, indptr (n_field+1) int64, indices
 * (indices_capacity) int32; *nnz_out (host) receives nnz, and EMG_ERR_LIMIT is
 * returned when nnz > indices_capacity.  After that capacity shortfall *nnz_out
 * and indptr are already valid (indices is not written), so the caller can size
 * indices from *nnz_out and call again.  The scratch is one ~4.9 MB device array
 * in the library, held by every GPU that loads it until the process exits; the
 * first call on a device looks up its address.  All calls share that array, so
 * calls that overlap on the GPU (other streams or host threads) race.
 * Synchronises ``stream``. */
int emg_csr_pattern_noalloc(int64_t n_tets, int64_t n_field, const int32_t* tet_to_field, int64_t* indptr,
                            int32_t* indices, int64_t indices_capacity, int64_t* nnz_out, void* stream);

/* ------------------------------------------------------- mesh topology ---
 * Replace the topology loops of Mesh3D.update (fem/mesh3d.py:224-355) and the
 * DOF map of Nedelec2.__init__ (fem/elements/nedelec2.py:32-62): edges and
 * faces of a tetrahedral mesh numbered in ascending vertex-tuple order, the
 * tet -> edge / face maps in the reference's slot order, tri -> edge, tri ->
 * tet and tet_to_field.  tets: DEVICE (4, n_tets) int32.  Synchronises
 * ``stream``; EMG_ERR_MESH for a vertex index out of range or a face shared by
 * more than two tets. */
typedef struct emg_topology emg_topology;
int emg_topology_create(int64_t n_nodes, int64_t n_tets, const int32_t* tets, void* stream, emg_topology** out);
int emg_topology_sizes(const emg_topology* topo, int64_t* n_edges, int64_t* n_tris);
/* Copies into caller-owned DEVICE arrays (int32; any may be NULL to skip it):
 * edges (2, nE), tris (3, nTri), tet_to_edge (6, nT), tet_to_tri (4, nT),
 * tri_to_edge (3, nTri), tri_to_tet (2, nTri; -1 = no second tet),
 * tet_to_field (20, nT). */
int emg_topology_get(const emg_topology* topo, int32_t* edges, int32_t* tris, int32_t* tet_to_edge,
                     int32_t* tet_to_tri, int32_t* tri_to_edge, int32_t* tri_to_tet, int32_t* tet_to_field,
                     void* stream);
void emg_topology_destroy(emg_topology* topo);
/* Edge lengths sqrt(dx^2 + dy^2 + dz^2) (fem/mesh3d.py:351), each step rounded
 * in order (bitwise equal to NumPy's).  nodes (3, n_nodes) f64, edges (2,
 * n_edges) int32, lengths (n_edges) f64: DEVICE arrays. */
int emg_edge_lengths(int64_t n_nodes, const double* nodes, int64_t n_edges, const int32_t* edges, double* lengths,
                     void* stream);

/* ---------------------------------------------------------- port modes ---
 * Element matrices of the 2-D waveguide-port eigenproblem A x = lambda B x
 * (lambda = -beta^2), the counterpart of generalized_matrix_GQ
 * (fem/physics/edm/nedeleclegrange2.py:224-382): second-order Nedelec transverse
 * and Lagrange longitudinal functions, 14 DOFs per triangle.  xy (2, 3, n_tris):
 * local port-plane coordinates of each triangle's vertices; local_edge_map
 * (2, 3, n_tris) int32: local vertex indices of each triangle edge; Ms9 =
 * matinv(ur), Mm9 = er, complex (9, n_tris) as for emg_assemble_tet_tensor.
 * face_block = 0 keeps the reference's zero face-face entries of the transverse
 * B block; 1 integrates them (the consistent discretisation).
 * A_out, B_out: (n_tris, 14, 14) complex.  DEVICE arrays; one block per triangle. */
int emg_port_element_matrices(int64_t n_tris, const double* xy, const int32_t* local_edge_map, const double* Ms9,
                              const double* Mm9, double k0, int face_block, double* A_out, double* B_out,
                              void* stream);

/* Field of a port mode at points of the port plane: ned2_tri_interp_full (which = 0,
 * E) and ned2_tri_interp_curl (which = 1, the curl term of H without its factor
 * j/(omega mu0)) of fem/mth/tri.py:228-401, as interpolate_Ef / interpolate_Hf of
 * fem/elements/nedleg2.py:82-105 call them.  DEVICE arrays: xy (2, npts) local point
 * coordinates; tris (3, n_tris) surface node ids; nodes2 (2, n_nodes) local node
 * coordinates; tri_to_field (14, n_tris); field (n_field) complex; urinv_diag
 * (3, n_tris) complex, the diagonal of matinv(ur) per triangle (which = 1 only); out
 * (3, npts) complex local components.  The last triangle that contains a point gives
 * its value, as in the reference; a point in none gets zero. */
int emg_port_interp(int64_t npts, const double* xy, int64_t n_tris, const int32_t* tris, int64_t n_nodes,
                    const double* nodes2, const int32_t* tri_to_field, const double* field, const double* urinv_diag,
                    double beta, int which, double* out, void* stream);

/* --------------------------------------------------------- far field ---
 * Stratton-Chu transform, the counterpart of stratton_chu_ff
 * (fem/physics/edm/sc.py:26-140).  Sources j < n_src at vis (3, n_src) f32 with
 * weights wns (3, n_src) f32 (n * area / 3 summed over the surface triangles of
 * each edge, sc.py:159-165) and fields E, H (3, n_src) complex64; sources with
 * |E| <= 1e-3 max|E| are dropped as the reference does.  Directions: elevation
 * theta, azimuth phi (n_dir f32), r = (cos th cos ph, cos th sin ph, sin th).
 * Eout, Hout: (3, n_dir) complex128.  All arrays DEVICE; synchronises ``stream``. */
int emg_stratton_chu(int64_t n_src, const float* E, const float* H, const float* vis, const float* wns,
                     int64_t n_dir, const float* theta, const float* phi, float k0, double* Eout, double* Hout,
                     void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EMERGE_GB300_H */
