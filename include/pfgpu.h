/*
 * pfgpu.h -- C-ABI of the GB300 element-by-element PCG library (libpfgpu.so).
 *
 * The library replaces the solve section of ParaFEM's p121 driver
 * (src/programs/5th_ed/p121/p121.f90:39-104: storkm formation, Jacobi
 * diagonal, preconditioned CG with checon_par) and, as a second entry
 * layer, the element-product offload of the xx3 experiment
 * (src/programs/dev/xx3/cuda_helpers.cu:183-368).
 *
 * Conventions follow xx3's ISO_C_BINDING layer (xx3.f90:56-148):
 *   - every argument is passed by reference;
 *   - host arrays are caller-owned and Fortran column-major;
 *   - device objects are opaque handles held by the caller (void**);
 *   - every entry point returns int: 0 = EXIT_SUCCESS, 1 = EXIT_FAILURE.
 * Unlike xx3 nothing is printed on failure: the message is kept per thread
 * and returned by pf_last_error.  All entry points are synchronous.
 *
 * Array layouts (Fortran shapes, 1-based ids as p121 holds them):
 *   g_num(20,nels)      node numbers in Smith-Griffiths order
 *   g_g(60,nels)        equation numbers, 0 = restrained (find_g3 output)
 *   g_coord(20,3,nels)  nodal coordinates per element
 *   storkm(60,60,nels)  element stiffness matrices
 *   r, xnew(neq)        load and displacement vectors in equation order
 */
#ifndef PFGPU_H
#define PFGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define PF_SUCCESS 0
#define PF_FAILURE 1

/* pf_solve modes */
#define PF_MODE_P121     0 /* FP64 storkm, checon_par test (p121.f90:88-104)      */
#define PF_MODE_FP64_RES 1 /* FP64 storkm, stop at ||r||2/||f||2 <= tol           */
#define PF_MODE_MIXED    2 /* FP32-storkm PCG with FP64 defect correction by
                              residual replacement (search direction kept),
                              stop at the FP64 true ||f-Ku||2/||f||2 <= tol        */
#define PF_MODE_MIXED_RESTART 3 /* FP32-storkm inner PCG restarted on each FP64
                              defect f-Ku (classic iterative refinement)           */
#define PF_MODE_MIXED16  4 /* as PF_MODE_MIXED with FP16 storkm (scaled per
                              element) in the inner products: half the bytes per
                              iteration, more inner iterations; same FP64 stop    */

/* pf_form_storkm flags */
#define PF_FORM_EXACT_WEIGHTS 1 /* exact 5/9, 8/9 Gauss factors instead of
                                   p121's single-precision literals
                                   (new_library.f90:1493)                        */
#define PF_FORM_NO_FP32       2 /* do not keep the FP32 copy of storkm            */

/* ---------------------------------------------------------------------- */
/* xx3 layer: same names and argument meaning as
 * src/programs/dev/xx3/cuda_helpers.cu, so xx3.f90 links unchanged.       */

/* cuda_helpers.cu:183 set_gpu */
int set_gpu(const int *device_id);
/* cuda_helpers.cu:198 allocate_memory_on_gpu (sizes multiplied in 64 bits) */
int allocate_memory_on_gpu(const int *n_elements, const int *element_size,
                           void **device_pointer);
/* cuda_helpers.cu:216 free_memory_on_gpu */
int free_memory_on_gpu(void **device_pointer);
/* cuda_helpers.cu:232 copy_data_to_gpu */
int copy_data_to_gpu(const int *n_elements, const int *element_size,
                     const void *host_data, void **device_pointer);
/* cuda_helpers.cu:255 copy_data_from_gpu */
int copy_data_from_gpu(const int *n_elements, const int *element_size,
                       void *host_data, void **device_pointer);
/* cuda_helpers.cu:278 matrix_vector_multiplies: for every matrix m,
 * rhs(:,m) = matrix(:,:,m) . lhs(:,m), FP64, column-major matrices. */
int matrix_vector_multiplies(int *n_mat, int *n_row, int *n_col,
                             void **d_lhs_vector, void **d_matrix,
                             void **d_rhs_vector);

/* ---------------------------------------------------------------------- */
/* Solve layer (replaces p121.f90:39-104).                                 */

/* Copies the calling thread's last error message (NUL-terminated). */
int pf_last_error(char *buf, const int *len);

/* Creates a solver context on a device (set_gpu(numpe-1) of xx3.f90:412). */
int pf_ctx_create(const int *device, void **ctx);
int pf_ctx_destroy(void **ctx);

/* Mesh and steering: the arrays p121 holds after find_g3 (p121.f90:33-49).
 * nn: number of nodes (ids in g_num are 1..nn); neq = MAXVAL(g_g). */
int pf_setup(void **ctx, const int *nels, const int *nn, const int *neq,
             const int *g_num, const int *g_g, const double *g_coord);

/* Material: n = 1 (one E, v for every element, p121.f90:54) or n = nels
 * (per element, as rfemsolve.f90:217-221). */
int pf_set_material(void **ctx, const int *n, const double *e, const double *v);

/* storkm integration and Jacobi diagonal on the GPU (p121.f90:54-69):
 * SAMPLE / SHAPE_DER / DEEMAT / BEEMAT / INVERT, K = sum B'DB det w. */
int pf_form_storkm(void **ctx, const int *nip, const int *flags);

/* Host-formed storkm(60,60,nels) instead of pf_form_storkm (FP64; the FP32
 * copy for PF_MODE_MIXED is derived on the device). */
int pf_set_storkm(void **ctx, const double *storkm);

/* Forms the stiffness matrix of element iel (1-based) of the mesh, with
 * its material, on the GPU into km(60,60) on the host: the km a PCG_KM
 * caller integrates once for a uniform mesh. */
int pf_form_km(void **ctx, const int *iel, const int *nip, const int *flags, double *km);

/* One element matrix km(60,60) for every element, replacing PCG_KM
 * (src/modules/mpi/maths.f90:1152-1323; the uniform-mesh case of xx9,
 * src/programs/dev/xx9/mathsgpu.f90).  The Jacobi diagonal is assembled
 * from diag(km) over the mesh, and every later pf_solve / pf_ebe_matvec /
 * pf_bench_iterations uses km: FP64 products on CUDA cores for
 * PF_MODE_P121 and PF_MODE_FP64_RES, tensor-core products (BF16 x3 split,
 * FP32 accumulation) for the inner iterations of PF_MODE_MIXED.  No
 * per-element storkm is held; pf_form_storkm / pf_set_storkm switch back.
 * pf_solve_multi and pf_get_storkm need per-element storkm. */
int pf_set_shared_km(void **ctx, const double *km);

/* Copies elements first..first+count-1 (0-based) of the FP64 storkm back. */
int pf_get_storkm(void **ctx, const int *first, const int *count, double *storkm);

/* Assembled (not inverted) Jacobi diagonal in equation order (neq). */
int pf_get_diag(void **ctx, double *diag);

/* One element-by-element product u = K p in equation order (GATHER,
 * element MATMUL, SCATTER of p121.f90:92-97).  prec 64: FP64 storkm;
 * 32: packed-symmetric FP32 storkm (used by PF_MODE_MIXED); 31: full FP32
 * storkm; 16: packed-symmetric FP16 storkm scaled per element (used by
 * PF_MODE_MIXED16).  The packed products are P K_e P p_e, P removing each
 * element's mean translation (equal to K_e p_e in exact arithmetic). */
int pf_ebe_matvec(void **ctx, const int *prec, const double *p, double *u);

/* The PCG solve (p121.f90:86-104).  r: loads (neq); xnew: result (neq);
 * iters: PCG iterations (inner iterations for PF_MODE_MIXED);
 * relres: final FP64 ||f - K xnew||2 / ||f||2 (computed on the device). */
int pf_solve(void **ctx, const double *r, const double *tol, const int *limit,
             const int *mode, double *xnew, int *iters, double *relres);

/* Statistics of the last pf_solve, written to stats[0..n-1]:
 *  [0] iterations  [1] outer corrections  [2] solve milliseconds (device)
 *  [3] final stopping metric  [4] FP64 matvecs  [5] FP32 matvecs
 *  [6] true relative residual */
int pf_solve_stats(void **ctx, double *stats, const int *n);

/* Times `steps` PCG iterations on the resident state (prec 64, 32, 31 or 16) with
 * CUDA events on the library stream.  ms_total: all steps; ms_elem: summed
 * duration of the element-product kernel launches; ms_scatter: summed
 * duration of the node-scatter kernel launches. */
int pf_bench_iterations(void **ctx, const int *prec, const int *steps,
                        double *ms_total, double *ms_elem, double *ms_scatter);

/* Centroid stresses of one element from a displacement vector
 * (p121.f90:112-123): sigma(6) = D . B(0,0,0) . u_e; iel is 1-based. */
int pf_centroid_stress(void **ctx, const int *iel, const double *xnew, double *sigma);

/* Centroid stresses of elements first..first+count-1 (1-based) for the
 * displacements xnew(neq): sigma(6, count), one thread per element (the
 * post-solve stress recovery of p121.f90:112-123 for the whole mesh). */
int pf_element_stresses(void **ctx, const double *xnew, const int *first, const int *count, double *sigma);

/* The autotuner's choice for the packed-symmetric FP32 element kernel, made
 * at pf_form_storkm / pf_set_storkm by timing every configuration on this
 * mesh: warps per CTA, shared-memory stages per warp, and the measured
 * milliseconds per launch of the configurations (14,2), (12,2), (8,3). */
int pf_tuning(void **ctx, int *warps, int *stages, float *ms);

/* The same for the packed FP16 element kernel (PF_MODE_MIXED16, pf_ebe_matvec
 * prec 16), tuned when the FP16 storkm is packed on its first use:
 * configurations (20,2), (24,2), (28,2).  Fails before that first use. */
int pf_tuning16(void **ctx, int *warps, int *stages, float *ms);

/* Force configuration *config (0: 14x2, 1: 12x2, 2: 8x3) of that kernel, or
 * re-run the autotuner (*config = -1).  Every configuration gives bitwise
 * the same products; only the speed differs. */
int pf_set_tuning(void **ctx, const int *config);

/* PCG iterations are replayed from a CUDA graph of 8 iterations (captured
 * on first use per solve mode) when *on != 0, the default; *on == 0 launches
 * every kernel directly.  Both give bitwise the same iterates. */
int pf_set_graphs(void **ctx, const int *on);

/* The PCG iteration's scatter, update passes and finish (p121.f90:90-104
 * with DOT_PRODUCT_P, maths.f90:168-215, and checon_par, maths.f90:999-1069)
 * run as one persistent cooperative kernel with grid-wide barriers when
 * *on != 0; FP64 solves (PF_MODE_P121, PF_MODE_FP64_RES) on per-element
 * storkm then run whole iterations, element products included, up to 32
 * per launch.  *on == 0, the default, launches the separate scatter, update
 * and finish kernels, replayed from CUDA graphs, which measure faster on
 * GB300.  Both give bitwise the same iterates.  Applies to 20-node
 * contexts; 8-node contexts always use the separate kernels. */
int pf_set_persistent(void **ctx, const int *on);

/* Self-check of the error path of the bulk-copy element kernels (no
 * reference counterpart).  Every mbarrier wait in those kernels is bounded;
 * one that runs out records an error word that the next synchronising call
 * reports as PF_FAILURE.  This runs one such wait, limited to *polls polls,
 * on a barrier that no copy completes (no copy is ever in flight), and
 * reports it the same way: it returns PF_FAILURE with the message "element
 * kernel: a shared-memory bulk-copy wait timed out (code 2)" and clears the
 * word, so the context's next call runs normally.  It returns PF_SUCCESS
 * only if the wait completed, which would mean the check itself is broken. */
int pf_check_wait_timeout(void **ctx, const int *polls);

/* ---- p123: 3-D Laplace with 8-node bricks (src/programs/5th_ed/p123/p123.f90) ----
 * A context set up with pf_setup_scalar8 holds one freedom per node:
 * g_num(8,nels), g_g(8,nels) (0 = restrained), g_coord(8,3,nels).  pf_solve
 * (PF_MODE_P121 or PF_MODE_FP64_RES), pf_ebe_matvec (prec 64),
 * pf_bench_iterations (prec 64), pf_get_diag and pf_solve_stats apply. */
int pf_setup_scalar8(void **ctx, const int *nels, const int *nn, const int *neq,
                     const int *g_num, const int *g_g, const double *g_coord);
/* storkc = sum over the Gauss points of (kx dx dx' + ky dy dy' + kz dz dz')
 * det w (p123.f90:70-85) and the Jacobi diagonal (:87-94). */
int pf_form_storkc(void **ctx, const int *nip, const double *kx, const double *ky, const double *kz);
int pf_get_storkc(void **ctx, const int *first, const int *count, double *storkc);
/* Fixed freedoms by the penalty method (p123.f90:104-131): diag(eq) +=
 * penalty for each listed equation, and every product then returns
 * u(eq) = p(eq) * diag(eq).  The caller sets r(eq) = diag(eq) * value
 * (pf_get_diag gives diag(eq) after this call).  pf_form_storkc clears them. */
int pf_set_fixed(void **ctx, const int *nfix, const int *eqs, const double *penalty);

/* ---- 8-node elasticity bricks (p122's demo deck: nod = 8, three freedoms per node) ----
 * g_num(8,nels), g_g(24,nels) (0 = restrained), g_coord(8,3,nels), the node
 * order of SHAPE_DER's 8-node brick.  pf_set_material, pf_form_storkm (FP64
 * storkm(24,24,e) and the Jacobi diagonal), pf_get_storkm, pf_get_diag,
 * pf_set_fixed, pf_solve (PF_MODE_P121 or PF_MODE_FP64_RES), pf_ebe_matvec
 * (prec 64) and pf_p122_solve_fixed apply.  Inside a PCG run the product at
 * a fixed freedom is p * store (pf_set_fixed); the residual f - K x uses the
 * plain K, as p122 forms r = loads - K x (p122.f90:142-146). */
int pf_setup_solid8(void **ctx, const int *nels, const int *nn, const int *neq,
                    const int *g_num, const int *g_g, const double *g_coord);

/* ---- p122: elastic-plastic (Mohr-Coulomb) solid, viscoplastic strain method ----
 * The solve of src/programs/5th_ed/p122/p122.f90:78-225 for 20-node bricks
 * under load control, on a context with storkm formed (pf_form_storkm with
 * nip and one material E, v).  For each load increment iy (qinc(iy) times
 * the nodal loads ld0(neq)), plastic iterations of a warm-started PCG
 * (tolerance cjtol, at most cjits iterations, checon_par) and a Gauss-point
 * pass (INVAR, MOCOUF, MOCOUQ, FORMM, the viscoplastic strains and body
 * loads) until checon_par of the displacements meets plastol or plasits
 * iterations.  results(6, incs) per increment: totd(1), sigma z, sigma x,
 * sigma y at element 1 Gauss point 1, PCG iterations, plastic iterations.
 * totd(neq, incs) (may be NULL): the total displacements after each increment.
 * phi, c, psi: friction angle, cohesion, dilation angle (degrees). */
int pf_p122_solve(void **ctx, const int *nip, const double *phi, const double *c, const double *psi,
                  const int *incs, const double *qinc, const int *plasits, const int *cjits,
                  const double *plastol, const double *cjtol, const double *ld0, double *results,
                  double *totd, int *incs_done);
/* The same solve on a 20-node or an 8-node context (pf_setup_solid8), with
 * displacement control: nfix fixed freedoms (p122.f90:96-113), equations
 * fix_eqs(nfix) (1-based) with prescribed values fix_vals(nfix).  Their
 * diagonal takes the penalty 1e20 and store = the penalised diagonal; on the
 * first plastic iteration of an increment loads(fix) = store * value *
 * qinc(iy) and the PCG product there is p * store, after it loads(fix) = 0
 * and the product is 0 (p122.f90:122-158).  ld0 may be NULL (no loaded
 * nodes); with both, the first plastic iteration's loads are ld0 * qinc +
 * bdylds everywhere, as p122 computes them.  Fixed freedoms need an 8-node
 * context.  The context's diagonal is restored afterwards. */
int pf_p122_solve_fixed(void **ctx, const int *nip, const double *phi, const double *c, const double *psi,
                        const int *incs, const double *qinc, const int *plasits, const int *cjits,
                        const double *plastol, const double *cjtol, const double *ld0, const int *nfix,
                        const int *fix_eqs, const double *fix_vals, double *results, double *totd,
                        int *incs_done);

/* Number of kernels this library launched since the context was created. */
int pf_kernel_launches(void **ctx, long long *count);

/* ---------------------------------------------------------------------- */
/* Several load cases of one mesh (block PCG).  No counterpart in p121
 * (one load case per run); the shared-matrix products follow the idea of
 * xx9's batched MATMUL (src/programs/dev/xx9/mathsgpu.f90:479).          */

/* k independent solves K x_j = r_j that share every element-matrix read
 * (k a multiple of 8, 8..128): r and xnew are (neq, k) column-major; iters
 * and relres hold k values (relres: FP64 true residual).  prec 16: block
 * products on the tensor cores (tcgen05, K_e and P_e each split into two
 * FP16 terms scaled by powers of two, FP32 accumulation; the cases taken
 * in passes of up to 64, the pass width autotuned on the mesh); 32: the
 * same products on CUDA cores in FP32.  FP64 vectors, dots and alpha/beta;
 * FP64 residual replacement as PF_MODE_MIXED. */
int pf_solve_multi(void **ctx, const int *k, const double *r, const double *tol, const int *limit,
                   const int *prec, double *xnew, int *iters, double *relres);
/* Block product U = K P for k cases (k a multiple of 8, 8..128; equation
 * order, (neq,k) column-major); prec 16 (tensor cores), 32 (FP32 CUDA
 * cores), 64 (FP64). */
int pf_ebe_matvec_multi(void **ctx, const int *k, const int *prec, const double *p, double *u);
/* The tensor-core block product's autotuner: *kb = the pass width (cases
 * per pass) chosen for the context's current k; cand[4] the widths timed
 * (0 = unused) and ms[4] one full product with each (0 when only one width
 * was possible). */
int pf_multi_tuning(void **ctx, int *kb, int *cand, float *ms);
/* Device time (CUDA events, ms per product, averaged over *reps after one
 * warm-up) of the tensor-core block product U = K P for the k columns of p
 * ((neq, k) column-major), with P resident on the device. */
int pf_multi_product_ms(void **ctx, const int *k, const double *p, const int *reps, double *ms);
/* Releases the context's block-solve buffers (allocated by the first
 * pf_solve_multi or pf_ebe_matvec_multi; also released with the mesh and by
 * pf_ctx_destroy). */
int pf_multi_free(void **ctx);

/* ---------------------------------------------------------------------- */
/* Serving layer: continuous batching of many independent solves.  No
 * counterpart in the reference (p121 solves one mesh per run); every solve
 * is p121's Jacobi-PCG to ||r||2/||f||2 <= tol.                           */

#define PF_BUSY 2   /* pf_batch_admit: no room yet; retry after a sync */

/* A batch on one device with a fixed device-memory budget (bytes) for its
 * arenas and at most max_meshes solves resident at once.  prec 64: FP64
 * element products; prec 32: FP32 products with FP64 residual replacement
 * per mesh (the PF_MODE_MIXED scheme); prec 16: FP16 storkm in the products
 * (the PF_MODE_MIXED16 scheme). */
int pf_batch_create(const int *device, const long long *budget_bytes, const int *max_meshes, const int *prec,
                    void **batch);
int pf_batch_destroy(void **batch);
/* Arena capacity in elements and nodes. */
int pf_batch_capacity(void **batch, long long *elements, long long *nodes);
/* Admits one solve (arrays as pf_setup / pf_set_material, r in equation
 * order).  Returns PF_SUCCESS and its id, PF_BUSY when it does not fit yet,
 * or PF_FAILURE.  Its storkm is formed on the GPU behind the running work. */
int pf_batch_admit(void **batch, const int *nels, const int *nn, const int *neq, const int *g_num,
                   const int *g_g, const double *g_coord, const int *nmat, const double *e, const double *v,
                   const int *nip, const double *r, const double *tol, const int *limit, int *id);
/* Enqueues `iters` PCG iterations of every resident solve and returns.  By
 * default the chunk is replayed from a CUDA graph, captured again (or
 * updated in place) only when the set of resident solves changes. */
int pf_batch_launch(void **batch, const int *iters);
/* *on == 0: launch every kernel directly instead of replaying the graph.
 * Both give bitwise the same results. */
int pf_batch_set_graphs(void **batch, const int *on);
/* Waits for the enqueued work and retires converged solves. */
int pf_batch_sync(void **batch, int *n_active, int *n_done);
/* Pops one retired solve: id, iterations, FP64 true relative residual and
 * x (neq values; x_cap = capacity of x). */
int pf_batch_collect(void **batch, int *id, int *iters, double *relres, double *x, const int *x_cap, int *neq);
int pf_batch_launches(void **batch, long long *count);

/* No counterpart in the reference.  u(neq) = K p for callers that cannot
 * allocate device memory while they run (memory reserved up front by a pool
 * or a host framework, cudaMalloc forbidden in the solve phase, or a fixed
 * device budget).  storkm(60,60,nels), g_g(60,nels), p(neq) and u(neq) are
 * the caller's DEVICE buffers on the current device.  The library's own
 * scratch is a fixed array inside libpfgpu.so (about 14.3 MiB, held on every
 * device that loads the library until exit) that limits nels <= 16384 and
 * neq <= 262144; larger sizes are rejected.  The first call on a device looks
 * the array up, which (under CUDA's lazy module loading) is also when its
 * device memory is taken: make that first call during set-up, before the
 * caller reserves the rest of device memory and before any stream capture; a
 * call with *nels = *neq = 0 does only this set-up.  Each call runs on the
 * legacy default stream and waits for the whole device before it returns.
 * If g_g holds an equation number outside 0..neq the call fails and leaves u
 * unchanged.  All calls share the array: calls that overlap on the GPU race
 * and must not be made. */
int pf_ebe_matvec_noalloc(const int *nels, const int *neq, const double *storkm,
                          const int *g_g, const double *p, double *u);

/* ---------------------------------------------------------------------- */
/* Host-side driver layer (C++, no GPU work): deck I/O and generators.     */

/* p12meshgen's p121 and p123 cases (src/tools/preprocessing/p12meshgen/
 * p12meshgen.f90:118-323, 658-801): reads job.mg and writes job.dat, job.d,
 * job.bnd, job.lds (and job.fix for p123 decks with fixed freedoms). */
int pf_p12meshgen(const char *job);

/* Runs the whole p121 job (p121.f90:1-141) on the GPU: reads job.dat/.d/
 * .bnd/.lds, solves, writes job.res and job.ensi.DISPL-000001.
 * mode: PF_MODE_*; iters and central (xnew(1)) are returned. */
int pf_p121_run(const char *job, const int *device, const int *mode,
                int *iters, double *central);

/* load_p121's patch load on the top face of a 20-node cube (loading.f90:
 * 386-480), nle = nxe/5: r(z equation of each patch node) = factor x the
 * pattern multiplier (LOAD + SCATTER_NOADD semantics: assignment).  p122's
 * decks use factor = -aa*bb/12 (p12meshgen.f90:420). */
int pf_patch_loads(const int *nxe, const int *nze, const double *factor, const int *nels, const int *g_num,
                   const int *g_g, const int *neq, double *r);

/* The whole p122 job (p122.f90:1-233) for 20-node bricks under load
 * control: reads job.dat (READ_P122's record and the qinc values), .d,
 * .bnd, .lds; solves every increment on the GPU (pf_p122_solve); writes
 * job.res and job.ensi.DISPL-0000nn per increment. */
int pf_p122_run(const char *job, const int *device, int *incs_done);

/* Host side of p123: an nxe x nye x nze box of 8-node bricks numbered as
 * GEOMETRY_8BXZ (geometry.f90:70-166): g_num(8,nels), g_coord(8,3,nels). */
int pf_mesh_box8(const int *nxe, const int *nye, const int *nze, const double *aa, const double *bb,
                 const double *cc, int *g_num, double *g_coord);
/* box_bc8's restraints (geometry.f90:655-696): node_fix(nn) = 1 free, 0 fixed. */
int pf_box8_restraints(const int *nxe, const int *nye, const int *nze, int *node_fix);
/* One freedom per node: equation = free nodes up to and including the node
 * (rearrange_2 + find_g4, new_library.f90:3118-3271). */
int pf_number_equations1(const int *nels, const int *nn, const int *nod, const int *g_num,
                         const int *node_fix, int *g_g, int *neq);
/* The whole p123 job: reads job.dat/.d/.bnd/.lds/.fix, solves on the GPU,
 * writes job.res and job.ensi.NDPTL-000001; returns the iterations and the
 * four printed potentials (equations nres..nres+3). */
int pf_p123_run(const char *job, const int *device, int *iters, double *potentials);

/* Structured 20-node cube mesh in GEOMETRY_20BXZ numbering
 * (src/modules/shared/geometry.f90:172-290), nxe x nye x nze elements of
 * size aa x bb x cc.  First call with g_num == NULL returns the sizes
 * (nels, nn); the second fills g_num(20,nels) and g_coord(20,3,nels). */
int pf_mesh_cube(const int *nxe, const int *nye, const int *nze, const double *aa,
                 const double *bb, const double *cc, int *nels, int *nn,
                 int *g_num, double *g_coord);

/* Restraints and loads of the synthetic cube problems:
 *   bc 0: cube_bc20 rollers + fixed base (geometry.f90:425-504)
 *   bc 1: every dof fixed on the base face z = -nze*cc, nothing else
 * Fills node_fix(3,nn) with 1 = free, 0 = fixed.  */
int pf_cube_restraints(const int *nxe, const int *nye, const int *nze, const int *bc,
                       int *node_fix);

/* Equation numbering (REARRANGE + find_g3, new_library.f90:3059-3212):
 * node_fix(3,nn) -> g_g(60,nels) and neq. */
int pf_number_equations(const int *nels, const int *nn, const int *g_num,
                        const int *node_fix, int *g_g, int *neq);

/* Consistent nodal loads of a uniform pressure p (force per area, acting
 * in -z) on the top face z = 0 of a GEOMETRY_20BXZ cube mesh, added into r
 * (equation order, neq): per top face, corners +pA/12 and mid-sides -pA/3,
 * the rule behind load_p121's 1:-4 pattern (loading.f90:437-495). */
int pf_cube_top_pressure(const int *nxe, const int *nze, const int *nels,
                         const double *aa, const double *bb, const double *p,
                         const int *g_g, const int *neq, double *r);

/* Per-element material field from a counter-based generator (Philox4x32-10,
 * key = seed, counter = element index): E log-uniform in [e_lo, e_hi],
 * v uniform in [v_lo, v_hi]. */
int pf_random_material(const int *nels, const long long *seed, const double *e_lo,
                       const double *e_hi, const double *v_lo, const double *v_hi,
                       double *e, double *v);

#ifdef __cplusplus
}
#endif

#endif /* PFGPU_H */
