/*
 * uhm_gb300 C ABI.
 *
 * Part 1 mirrors the reference's Fortran/C interface one to one
 * (UHM/include/uhm/wrapper/fort.hxx:47-190, implemented in
 * UHM/src/wrapper/fort.cxx:47-321): same names (trailing underscore, the
 * UHM_C2F convention of UHM/include/uhm/util.hxx:39), arguments passed by
 * pointer, mesh / element / node handles as `long` casts of C++ pointers,
 * `void` returns.  Where the reference aborts on bad input, these record an
 * error that uhm_gpu_get_status / uhm_gpu_get_last_error report.
 *
 * Part 2 (uhm_gpu_*) adds what the device path needs and the reference has
 * no call for: explicit tree construction through the Element API, status
 * codes, precision / refinement control, bulk transfers and timings.
 *
 * Constants (UHM/include/uhm/wrapper/fort.f90:33-53):
 *   UHM_REAL = 101, UHM_COMPLEX = 103 (unsupported), UHM_LHS = 1, UHM_RHS = 2,
 *   UHM_PHYSICS_SINGLE = 1, UHM_PHYSICS_MULTI = 2.
 */
#ifndef UHM_GB300_H
#define UHM_GB300_H

/* the constants above, for C callers (the reference defines them for
 * Fortran in fort.f90 and for C++ in UHM/include/uhm/const.hxx; C++ callers
 * of this library have them in uhm_gb300/csrc/mesh.hpp) */
#ifndef __cplusplus
#ifndef UHM_REAL
#define UHM_REAL 101
#endif
#ifndef UHM_COMPLEX
#define UHM_COMPLEX 103
#endif
#ifndef UHM_LHS
#define UHM_LHS 1
#endif
#ifndef UHM_RHS
#define UHM_RHS 2
#endif
#ifndef UHM_PHYSICS_SINGLE
#define UHM_PHYSICS_SINGLE 1
#endif
#ifndef UHM_PHYSICS_MULTI
#define UHM_PHYSICS_MULTI 2
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Part 1: reference interface (fort.hxx) ---------------------------- */
/* fort.hxx:51    */ void uhm_initialize_fla_(void);
/* fort.hxx:52    */ void uhm_finalize_fla_(void);
/* fort.hxx:54    */ void uhm_set_num_threads_(int* n_threads);
/* fort.hxx:55    */ void uhm_get_num_threads_(int* n_threads);
/* fort.hxx:57    */ void uhm_set_hier_block_size_(int* size);
/* fort.hxx:58    */ void uhm_get_hier_block_size_(int* size);
/* fort.hxx:60-65: thresholds of SVD fronts (the reference declares them
 * without defining them); kept and returned, used by nothing here */
/* fort.hxx:60    */ void set_svd_relative_threshold_(double* val);
/* fort.hxx:61    */ void set_svd_absolute_threshold_(double* val);
/* fort.hxx:62    */ void get_svd_relative_threshold_(double* val);
/* fort.hxx:63    */ void get_svd_absolute_threshold_(double* val);
/* fort.hxx:64    */ void set_svd_cutoff_small_(int* flag);
/* fort.hxx:65    */ void get_svd_cutoff_small_(int* flag);
/* fort.hxx:67    */ void uhm_reset_flop_(void);
/* fort.hxx:68    */ void uhm_get_flop_(double* flop);
/* fort.hxx:69    */ void uhm_get_buffer_used_(double* buffer);
/* fort.hxx:70    */ void uhm_get_max_buffer_used_(double* buffer);
/* fort.hxx:72    */ void uhm_is_multithreading_enable_(int* flag);
/* fort.hxx:73    */ void uhm_is_hier_matrix_enable_(int* flag);
/* fort.hxx:75    */ void uhm_timer_(double* t);

/* fort.hxx:79    */ void uhm_mesh_create_(long* mesh);
/* fort.hxx:80    */ void uhm_mesh_delete_(long* mesh);
/* fort.hxx:82-83 */ void uhm_add_element_(long* mesh, long* elt);
/* fort.hxx:85-90 */ void uhm_add_node_(long* mesh, int* id, int* phy, int* n_dof, int* p, long* nod);
/* fort.hxx:92-93 */ void uhm_element_add_node_(long* elt, long* nod);
/* fort.hxx:95-103*/ void uhm_copy_in_(long* mesh, long* elt, int* datatype, int* mm, int* nn,
                                       int* node_disp, int* nods, int* side, double* buffer);
/* fort.hxx:105-113*/ void uhm_copy_out_(long* mesh, long* elt, int* datatype, int* mm, int* nn,
                                        int* node_disp, int* nods, int* side, double* buffer);
/* fort.hxx:115   */ void uhm_mesh_disp_(long* mesh);
/* fort.hxx:117-118*/ void uhm_get_n_dof_(long* mesh, int* n_dof);
/* fort.hxx:120-121*/ void uhm_get_n_nonzero_(long* mesh, int* n_nonzero);
/* fort.hxx:124-131*/ void uhm_estimate_cost_(long* mesh, int* method, int* datatype, int* n_rhs,
                                             double* flop_decompose, double* flop_solve,
                                             unsigned* n_nonzero_factor, double* buffer);
/* fort.hxx:133-134*/ void uhm_mesh_import_(long* mesh, char* filename);
/* fort.hxx:136: the reference partitions with METIS (build_tree.cxx:52-54,
 * build_tree_var4.cxx); here the heavy-edge matching of its
 * build_tree_var1.cxx:53-181 over the elements without a parent (ties by
 * element and node id; one tree per connected part; new elements that would
 * eliminate nothing are left out) */
/* fort.hxx:136   */ void uhm_build_tree_(long* mesh);
/* fort.hxx:138-140*/ void uhm_create_matrix_without_buffer_(long* mesh, int* datatype, int* n_rhs);
/* fort.hxx:142   */ void uhm_create_leaf_matrix_buffer_(long* mesh);
/* fort.hxx:143-144*/ void uhm_create_element_matrix_buffer_(long* mesh, int* is_schur);
/* fort.hxx:146   */ void uhm_set_rhs_(long* mesh);
/* fort.hxx:148-150: pseudo-random leaf matrices and right-hand sides for
 * benchmarks (the reference uses libflame's generator, whose values are not
 * reproduced: see uhm_gb300/csrc/fill.cpp); triangularize is a no-op, every
 * Cholesky kernel here reading lower triangles only */
/* fort.hxx:148   */ void uhm_random_spd_matrix_(long* mesh);
/* fort.hxx:149   */ void uhm_random_matrix_(long* mesh);
/* fort.hxx:150   */ void uhm_triangularize_(long* mesh);
/* fort.hxx:152   */ void uhm_lock_(long* mesh);
/* fort.hxx:153   */ void uhm_unlock_(long* mesh);

/* fort.hxx:158-163 decomposition */
void uhm_chol_with_free_(long* mesh);
void uhm_lu_nopiv_with_free_(long* mesh);
void uhm_lu_piv_with_free_(long* mesh);
/* fort.hxx:168-173 solution */
void uhm_solve_chol_(long* mesh);
void uhm_solve_lu_nopiv_(long* mesh);
void uhm_solve_lu_piv_(long* mesh);
/* fort.hxx:178-183 checking (computes the residual on the element matrices) */
void uhm_check_chol_(long* mesh);
void uhm_check_lu_nopiv_(long* mesh);
void uhm_check_lu_piv_(long* mesh);
/* fort.hxx:161,171,181: lu_incpiv factors the fronts with partial pivoting
 * over their eliminated rows, exactly as lu_piv (the reference pivots within
 * each diagonal block; solutions agree to rounding) and is solved by
 * uhm_solve_lu_piv_ or uhm_solve_lu_incpiv_ (the same call).
 * fort.hxx:162-163,172-173,182-183: QR and SVD fronts are not provided:
 * status 30. */
void uhm_lu_incpiv_with_free_(long* mesh);
void uhm_solve_lu_incpiv_(long* mesh);
void uhm_check_lu_incpiv_(long* mesh);
void uhm_qr_with_free_(long* mesh);
void uhm_solve_qr_(long* mesh);
void uhm_check_qr_(long* mesh);
void uhm_svd_with_free_(long* mesh);
void uhm_solve_svd_(long* mesh);
void uhm_check_svd_(long* mesh);
/* fort.hxx:188-189 residual: ||b - A x||_1 on the unassembled operator */
void uhm_get_residual_(long* mesh, double* res);

/* ---- Part 2: device-path additions (no counterpart in fort.hxx) ------- */
/* Mesh_::add_element(int gen) (UHM/include/uhm/mesh/mesh.hxx:160) */
int uhm_gpu_add_element_with_generation(long* mesh, int* gen, long* elt);
/* Element_::set_parent / add_child (UHM/include/uhm/mesh/element.hxx:104,139) */
int uhm_gpu_element_set_parent(long* elt, long* parent);
int uhm_gpu_element_add_child(long* elt, long* child);

/* Factor reuse.  The reference has these as C++ only (Mesh_::backup and
 * Mesh_::check_reuse, UHM/src/mesh/mesh.cxx:113-225; Element_::set_reuse and
 * is_matrix_reusable, UHM/src/mesh/element.cxx:75,216).  backup copies the
 * connectivity of mesh into the mesh backup (another handle from
 * uhm_mesh_create_); check_reuse flags the elements of mesh whose factor and
 * schur nodes are unchanged since, clearing the flag up the tree from any
 * that changed.  A factorisation then keeps, instead of redoing, every front
 * whose element is flagged, whose factor from the previous factorisation of
 * the same locked mesh is still held, whose element matrix was not copied in
 * since, and whose children are all kept.  uhm_gpu_get_n_refactored gives the
 * number of fronts the last factorisation redid. */
int uhm_gpu_element_set_reuse(long* elt, int flag);
int uhm_gpu_element_get_reuse(long* elt, int* flag);
int uhm_gpu_mesh_backup(long* mesh, long* backup);
int uhm_gpu_mesh_check_reuse(long* mesh, long* backup);
int uhm_gpu_get_n_refactored(long* mesh, int* n);

/* The element tree: every element (id order) with its parent (-1 for a
 * root) and generation; n is set to the element count, and nothing else is
 * written when cap < n.  uhm_gpu_get_children: an element's children in
 * child order. */
int uhm_gpu_get_tree(long* mesh, int cap, int* elt_id, int* parent_id, int* generation, int* n);
int uhm_gpu_get_children(long* mesh, int elt_id, int cap, int* child_id, int* n);

/* The assembled operator as a sparse matrix for external solvers: the
 * reference's DSparse_ (UHM/include/uhm/interf/sparse.hxx:99-129,
 * UHM/src/interf/sparse.cxx:188-460) over every leaf, in leaf order.  Entries
 * are keyed by global (row, col), or (col, row) when cs, with global dofs as
 * the mesh numbers them (uhm_gpu_get_node_offsets); contributions to one
 * entry are added in leaf order (axpy = 1) or the first kept (axpy = 0).
 * compress = 0: triplets in key order, rows in ia, columns in ja
 * (DSparse_::triplet); compress = 1: compressed rows (cs = 0: ia pointers,
 * ja columns) or columns (cs = 1: ja pointers, ia rows) (DSparse_::compress).
 * is_sym keeps the entries whose key has second >= first; fort adds 1 to
 * every index and pointer.  b is the assembled right-hand sides, column-major
 * (n_dof x n_rhs); n_rhs = 0 and no b when some leaf has none copied in.  Call once with ia, ja, a, b NULL for the lengths
 * (len_ia, len_ja, n_nz), then with arrays of those lengths.  n_dof is the
 * number of dofs (the reference's triplet reports its last index instead). */
int uhm_gpu_export_sparse(long* mesh, int is_sym, int fort, int cs, int compress, int axpy, int* n_dof,
                          int* n_rhs, long* len_ia, long* len_ja, long* n_nz, int* ia, int* ja, double* a,
                          double* b);
/* the first global dof of each node (single physics ids) in the locked mesh */
int uhm_gpu_get_node_offsets(long* mesh, int n, const int* ids, int* offsets);

/* 0 = ok; 4 = device allocation failed; 5..9 = API misuse; 11 = front not
 * positive definite; 12 = zero pivot; 13 = NaN; 20 = refinement missed its
 * tolerance (solution redone in FP64); 30 = unsupported call. */
int uhm_gpu_get_status(long* mesh);
int uhm_gpu_get_last_error(long* mesh, char* buf, int len);

/* mode 0: plain FP64 fronts.  mode 1: mixed precision, fronts in
 * default_prec (0 FP64, 1 FP32, 2 BF16-split tensor-core Schur update) with
 * FP64 iterative refinement on the element matrices until the backward error
 * is <= tol or max_iter corrections have been applied; default_prec 3 is the
 * six-term BF16 split and 4 the learned per-front choice (below). */
int uhm_gpu_set_mode(long* mesh, int mode, int default_prec, double tol, int max_iter);
/* per-front precision, indexed by element id (-1 = default) */
int uhm_gpu_set_front_precision(long* mesh, int n, const int* prec_by_element_id);

/* Bulk element transfer for all leaves in element-id order: nods_all holds
 * each leaf's node ids back to back (element's node count each, single
 * physics); buffer holds each leaf's m x m matrix (LHS) or m x n_rhs block
 * (RHS), column-major, back to back.  Same semantics as one uhm_copy_in_ per
 * leaf, with one host-to-device copy. */
int uhm_gpu_copy_in_leaves(long* mesh, int side, const int* nods_all, const double* buffer,
                           long n_values);
/* solution for all leaves, same layout as the RHS of uhm_gpu_copy_in_leaves */
int uhm_gpu_copy_out_leaves(long* mesh, double* buffer, long n_values);
/* solution of listed nodes (single physics ids), each node's dofs in order */
int uhm_gpu_get_node_solution(long* mesh, int n_nodes, const int* node_ids, double* out,
                              long n_values);

/* ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), A the assembled sum of
 * element matrices, evaluated in FP64 on the device */
int uhm_gpu_backward_error(long* mesh, double* berr);
/* out[0..8] = upload ms, factor ms, solve ms, refine ms, total ms,
 * refinement iterations, backward error, kernel launches, backward error of
 * the first (unrefined) solve */
int uhm_gpu_get_timing(long* mesh, double* out);

/* Per-kernel profile: when on, every launch of the factor / solve programs
 * is bracketed by CUDA events (use outside timed regions).  Per op kind
 * (0 assemble, 1 small-front factor, 2 diagonal POTRF, 3 panel TRSM,
 * 4 trailing SYRK, 5 LU panel, 6 LU row solve, 7 LU trailing GEMM,
 * 8..16 solve kernels, 17..25 the step-by-step tensor-core and LU
 * kernels, 26..32 the cooperative-panel Cholesky kernels; n_kinds up to
 * 40): total ms, algorithmic flops, algorithmic bytes, launches since
 * profiling was switched on. */
int uhm_gpu_set_profiling(long* mesh, int on);
int uhm_gpu_get_profile(long* mesh, int n_kinds, double* ms, double* flops, double* bytes,
                        long* launches);
/* every profiled launch in launch order: op kind, items (CTAs of work), ms;
 * *n_out = number recorded (entries beyond cap are not written) */
int uhm_gpu_get_op_log(long* mesh, int cap, int* kind, int* n_items, double* ms, int* n_out);

/* front table after lock + create_matrix_without_buffer: per front (leaf to
 * root order) the element id, generation, fs, ss */
int uhm_gpu_get_n_fronts(long* mesh, int* n);
int uhm_gpu_get_fronts(long* mesh, int n, int* elt_id, int* generation, int* fs, int* ss);
/* node ids of one front, factor nodes then schur nodes, in front order */
int uhm_gpu_get_front_nodes(long* mesh, int elt_id, int cap, int* ids, int* n_factor,
                            int* n_schur);

/* Element matrices generated on the device instead of copied in (no
 * counterpart in the reference, which takes element matrices from its caller
 * through copy_in, UHM/src/mesh/interf.cxx:108-204): uniform quad (dim 2) or
 * hex (dim 3) meshes with integrated-Legendre (Lobatto) modes.  Per element
 * (leaf order, as uhm_gpu_copy_in_leaves): order p_el (1..7), diffusion
 * coefficient kappa, optional reaction react (or NULL) and, for all elements,
 * optional convection velocity beta[dim] (or NULL); its retained tensor modes
 * sel[sel_ptr[e] .. sel_ptr[e+1]) (flat index mi[0] + mi[1] (p+1) + mi[2]
 * (p+1)^2, in the element's row order).  ref holds, from ref_off[p], the
 * (p+1) x (p+1) 1D mass, stiffness and convection matrices (row-major) of
 * order p.  hh = h/2; cmass, cconv: the mass and convection scale factors
 * ((h/2)^dim and (h/2)^(dim-1)).  The element node lists must be known: a
 * uhm_gpu_copy_in_leaves with nods_all (e.g. of the right-hand sides) gives
 * them.  method as for the factorisation.  Afterwards, until the next
 * factorisation, uhm_gpu_get_timing's out[0] is the generation kernel's
 * device time in ms. */
int uhm_gpu_generate_lobatto_elements(long* mesh, int method, int dim, double hh, double cmass, double cconv,
                                      int n_el, const double* ref, const long* ref_off, int n_ref_off,
                                      const int* p_el, const double* kappa, const double* react,
                                      const double* beta, const long* sel_ptr, const int* sel);

/* Kernel-selection thresholds (no counterpart in the reference, whose block
 * size is a compile-time knob, UHM/include/uhm/const.hxx): values[0] whole-front
 * shared-memory factorisation up to n (FP64, at most 160), values[1] the same
 * for FP32 (at most 224), values[2] tensor-core BF16-split fronts from n,
 * values[3] LU panels on many CTAs from this many rows below the diagonal,
 * values[4] k: diagonal block and panel TRSM of a Cholesky step in one launch
 * when that launch has at most k CTAs per SM (0: never), values[5] outer
 * panel width of tensor-core fronts factored step by step (128, 256 or 512:
 * LU fronts, and Cholesky fronts when values[6] is 0), values[6] outer panel
 * width of BF16X3 Cholesky fronts on the cooperative-panel path: 256 (the
 * default) factors each panel's diagonal block and its inverse with a
 * cooperative kernel and solves the rows below on the tensor cores, 512
 * factors whole panels with the cooperative kernel, 0 puts these fronts on
 * the step-by-step path; values[7] rows (columns) per CTA of the
 * flag-driven forward (backward) solves of large Cholesky fronts (64 or
 * 256), values[8] 1: with panels of 256, the next panel's diagonal kernel
 * runs on a second stream beside the current panel's trailing update,
 * values[9] 1: the 64-row solves of FP32 fronts run as chains (one CTA per
 * front solves the diagonal blocks from shared memory, helper CTAs sum the
 * blocks further from the diagonal), 0 (the default): as flag-driven 64-row
 * blocks.
 * uhm_gpu_autotune times candidate values on this mesh (element matrices and
 * right-hand sides copied in; reps factor+solve runs per candidate, the
 * fastest kept) and leaves the mesh factored and solved with the choice;
 * n_timed returns how many candidates were timed. */
int uhm_gpu_set_tunables(long* mesh, const int* values);
int uhm_gpu_get_tunables(long* mesh, int* values);
int uhm_gpu_autotune(long* mesh, int method, int reps, int* n_timed);

/* Learned per-front precision (uhm_gpu_set_mode default_prec = 4): a
 * 12 -> 64 -> 64 -> 3 MLP (classes 0 FP64, 1 FP32, 2 BF16-split) reads per-front
 * features computed from the element matrices and the tree and picks each
 * front's precision before the first factorisation; a solve that misses the
 * refinement tolerance is redone in FP64 (status 20).  Parameters: 5187
 * floats, layout W1[64][12] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]. */
int uhm_gpu_set_selector(long* mesh, const float* params, int n);
/* One block of a front, read back from the device (the C form of
 * uhm::Matrix_::copy_out, UHM/include/uhm/matrix/uhm/matrix.hxx:86-87):
 * mat 1 ATL (fs x fs), 2 ATR (fs x ss), 3 ABL (ss x fs), 4 ABR (ss x ss)
 * after a factorisation; 5 P (fs int pivots, LU) ; 7 XT (fs x n_rhs), 8 XB
 * (ss x n_rhs) after a solve.  out is column-major with leading dimension m;
 * (m, n) must be the block's size.  Cholesky blocks hold L (ATL, lower
 * triangle) and the Schur complement (ABR, lower triangle), zero above. */
int uhm_gpu_get_front_block(long* mesh, int elt_id, int mat, int m, int n, void* out);
/* per-front features (front order of uhm_gpu_get_fronts, 12 floats each),
 * after the element matrices are copied in; method as for the factorisation */
int uhm_gpu_get_front_features(long* mesh, int method, int n_fronts, float* out);
/* per front: precision used by the last plan (0 FP64, 1 FP32, 2 BF16X3,
 * 3 BF16X6) and the selector's class (-1 if it has not run) */
int uhm_gpu_get_front_precision(long* mesh, int n_fronts, int* prec, int* learned_class);
/* the selector network on caller samples X (N x 12, row-major, host memory):
 * class and class probabilities; class-weighted cross-entropy gradient over
 * all N samples (checks the training kernels); Adam training on shuffled
 * minibatches, parameters updated in place, mean loss per epoch */
int uhm_gpu_mlp_n_params(void);
int uhm_gpu_mlp_n_features(void);
int uhm_gpu_mlp_predict(const float* X, int N, const float* params, int* cls, float* prob);
int uhm_gpu_mlp_gradient(const float* X, const int* Y, const float* class_weight, int N, const float* params,
                         float* grad, float* loss);
int uhm_gpu_mlp_train(const float* X, const int* Y, const float* class_weight, int N, float* params, int epochs,
                      int batch, float lr, unsigned long long seed, float* loss_hist);

/* Solves (L L^T) x = b for a dense SPD matrix whose lower Cholesky factor L
 * (n x n, column-major, leading dimension ld >= n, FP64) the caller already
 * holds in device memory; x holds b on entry and the solution on return,
 * also in device memory.  Nothing is allocated: this is for callers that may
 * not call cudaMalloc (an application that owns all device memory through
 * its own pool, a real-time loop that cannot take an allocation's implicit
 * synchronisation).  It has no counterpart in the reference.
 *   - n <= 262144; larger n returns 30, bad arguments return 7, a device
 *     wait that gave up returns 14.  After a return of 14 the contents of x
 *     are undefined (blocks that gave up still write their part): keep a
 *     copy of b if it is needed again.
 *   - Scratch: a fixed 32 KB device array inside this library (ticket, error
 *     word, per-block completion flags), present on every GPU that loads the
 *     library; each call clears the part it uses on `stream` first.  The
 *     first call on a device looks up that array's device address (once per
 *     device).
 *   - Calls share the array: calls that overlap on the GPU (other streams,
 *     other host threads) race and must be serialised by the caller.
 *   - The call reads the error word back into host memory and waits for
 *     `stream`, so it cannot be made while `stream` (or any stream) is being
 *     captured into a CUDA graph.  The work runs on `stream` (NULL = the
 *     legacy default stream). */
int uhm_gpu_dense_chol_solve_noalloc(const double* L, int n, int ld, double* x, void* stream);

/* Iteration limit of every bounded wait inside the device kernels (flag
 * hand-offs of the tree solves, the grid barrier of the cooperative LU panel,
 * the mbarrier waits of the tensor-core update, the allocation-free solve).
 * The default keeps each wait under about a second; a wait that runs out
 * records an error, the call returns status 14 and the device stays usable.
 * iters >= 0 sets the limit (0: a wait not satisfied at its first look gives
 * up, which lets a test make a wait run out); iters < 0 restores the
 * defaults.  Copies in flight are still waited for with a fixed limit before
 * a kernel frees its memory.  It has no counterpart in the reference, which
 * has no device waits.  Returns 0, or 7 when no device is present. */
int uhm_gpu_set_wait_limit(long long iters);

/* pinned host memory for the bulk transfers */
void* uhm_gpu_host_alloc(long bytes);
void uhm_gpu_host_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
