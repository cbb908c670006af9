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
 * host-side binding of tet_mass_stiffness_matrices makes. */
int emg_assemble_tet_host(emg_plan* plan, const double* eps, const double* mu_inv, double* E_data,
                          double* B_data, void* stream);

/* Releases the plan and its device memory. */
void emg_plan_destroy(emg_plan* plan);

/* CSR pattern without any device allocation.  No counterpart in the reference:
 * an addition for callers that cannot call cudaMalloc, e.g. a host application
 * that must not allocate device memory of its own (its memory is owned by
 * another allocator, or cudaMalloc's implicit device synchronisation cannot be
 * afforded in its loop).  Computes the same indptr/indices as emg_plan_create +
 * emg_plan_pattern for meshes of at most 8192 tets and 65536 DOFs (larger sizes
 * return EMG_ERR_LIMIT).  Inputs and outputs are caller-owned DEVICE arrays:
 * tet_to_field (20, n_tets) int32, indptr (n_field+1) int64, indices
 * (indices_capacity) int32; *nnz_out (host) receives nnz, and EMG_ERR_LIMIT is
 * returned when nnz > indices_capacity.  The scratch is one ~4.9 MB device array
 * in the library, held by every GPU that loads it until the process exits; the
 * first call on a device looks up its address.  All calls share that array, so
 * calls that overlap on the GPU (other streams or host threads) race.
 * Synchronises ``stream``. */
int emg_csr_pattern_noalloc(int64_t n_tets, int64_t n_field, const int32_t* tet_to_field, int64_t* indptr,
                            int32_t* indices, int64_t indices_capacity, int64_t* nnz_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EMERGE_GB300_H */
