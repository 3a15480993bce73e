/*
 * thc_gb300.h -- C ABI of the GB300 ISDF library (libthc_gb300.so).
 *
 * Plain pointers and sizes only.  Every array argument may be a host pointer or a
 * device pointer of the context's device; the library detects which with
 * cudaPointerGetAttributes, copies host inputs to the device and writes outputs back
 * to wherever the output pointer lives.  Nothing here frees caller memory.  All entry
 * points return a status (THC_OK = 0) and never exit the process.
 *
 * The entry points replace the arithmetic behind thcpp's C++ solver classes:
 *
 *   thc_kmeans_initial_indices  KMeansSolver::guess_initial_centroids
 *                               (src/kmeans.cpp:159-175)
 *   thc_kmeans                  KMeansSolver::kernel (src/kmeans.cpp:187-264) with
 *                               classify_grid_points (:88-106), update_centroids
 *                               (:108-144), normed_difference
 *                               (src/matrix_operations.h:42-57) and map_to_grid (:146-157)
 *   thc_isdf                    IVecs::IVecs + IVecs::kernel
 *                               (src/interpolating_vectors.cpp:17-57, :406-455):
 *                               setup_pseudo_dm/setup_CZt (:59-141), setup_CCt (:163-190),
 *                               least_squares (:416), fft_vectors (:331-404),
 *                               construct_muv (:247-281), dump_thc_data's Cholesky (:283-315)
 *   thc_qrcp                    QRCP::QRCPSolver::kernel (src/qrcp.cpp:100-173): setup_Z_matrix /
 *                               setup_Z_half_matrix (:34-67), pzgeqpf (matrix_operations.h:
 *                               757-790), the first thc_cfac * N_o pivots sorted (:149-160)
 *   thc_qrcp_complex            thc_qrcp for complex aoR
 *   thc_isdf_complex            the same for complex aoR (P = Phi_mu^H Phi, :117; Z = P o conj(P))
 *   thc_isdf_half_complex       the same for complex aoR / aoR_half
 *   thc_isdf_interpolating_vectors  the least-squares solution zeta of the last ISDF call
 *                               (interpolating_vectors.cpp:416)
 *   thc_isdf_half               IVecs with rotate = true (src/interpolating_vectors.cpp:45-49):
 *                               setup_CZt_half (:143-161), the IVMG product of
 *                               construct_muv (:271-273), dump_thc_data's Muv (:317-328)
 *
 * Threading: calls on distinct contexts may run concurrently from different host
 * threads; one context must not be used by two threads at once.
 */
#ifndef THC_GB300_H
#define THC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define THC_OK                0
#define THC_ERR_ARG           1  /* invalid argument (sizes, null pointers, max_it < 1) */
#define THC_ERR_CUDA          2  /* CUDA runtime error (message in thc_ctx_last_error)  */
#define THC_ERR_EMPTY_CLUSTER 3  /* a k-means centroid weight fell below 1e-8
                                    (the reference exits: src/kmeans.cpp:131-143)        */
#define THC_ERR_NOT_PD        4  /* Cholesky of M failed; the info field holds the
                                    1-based leading minor (the reference prints it and
                                    still writes Luv: src/interpolating_vectors.cpp:296-304) */
#define THC_ERR_SHAPE         5  /* mesh product != N_g, or sizes above the limits     */
#define THC_ERR_IO            6  /* file I/O (host tools only)                          */
#define THC_ERR_TIMEOUT       7  /* a bounded device wait gave up                       */
#define THC_ERR_NOMEM         8  /* device allocation failed                            */
#define THC_ERR_CUFFT         9  /* cuFFT plan or execution failed                      */

/* Arithmetic of a context. */
#define THC_PREC_FP64  0  /* all-FP64: the drop-in path                                  */
#define THC_PREC_MIXED 1  /* FP32 k-means assign + FP64 recheck, sliced-BF16 tensor-core
                             GEMMs, FP32 FFT, FP64 Cholesky of C and of M               */

typedef struct thc_ctx thc_ctx;

typedef struct thc_kmeans_stats {
  int iterations;          /* completed k-means iterations                               */
  int converged;           /* 1 if the normed difference fell below the threshold        */
  int zero_filled;         /* 1 if the last difference neither fell below nor rose above
                              the threshold (the reference then leaves the indices 0)    */
  int duplicates;          /* repeated indices after sorting (the reference warns)       */
  double final_diff;       /* last normed difference                                     */
  double pct_changed;      /* % of grid points whose label changed in the last iteration */
  long long rechecked;     /* points resolved by the FP64 recheck (mixed precision)      */
  double device_ms;        /* device time of the call                                    */
} thc_kmeans_stats;

typedef struct thc_isdf_stats {
  int chol_c_info;         /* 0, or 1-based pivot at which Cholesky of C broke down with no
                              shift (before the shift retry)                             */
  int chol_m_info;         /* 0, or 1-based leading minor of M that is not positive      */
  int rank_deficient;      /* 1 if C needed the diagonal shift                           */
  int n_anti;              /* half-spectrum points where v(G) != v(-G)                   */
  double shift_used;       /* absolute diagonal shift added to C                         */
  double c_min_pivot;      /* min / max squared Cholesky pivot of C (cond estimate^-1)   */
  double device_ms;        /* device time of the call                                    */
} thc_isdf_stats;

typedef struct thc_qrcp_stats {
  int numerical_rank;      /* pivots before |R_kk| fell to 1e-7 |R_00| (the residuals of
                              the Gram form are rounding beyond that)                     */
  double device_ms;        /* device time of the call                                    */
} thc_qrcp_stats;

/* Context lifetime.  `precision` is THC_PREC_FP64 or THC_PREC_MIXED. */
int thc_ctx_create(int device, int precision, thc_ctx** out_ctx);
int thc_ctx_destroy(thc_ctx* ctx);
/* Run on a caller stream (a cudaStream_t); NULL restores the context's own stream. */
int thc_ctx_set_stream(thc_ctx* ctx, void* cuda_stream);
/* Named numeric options: "slices_p", "slices_z", "slices_m" (sliced-GEMM depths of the
 * P, zeta and Coulomb products, 2..6); "gemm_tc" (1 = tcgen05 tensor-core kernel, the
 * default; 0 = warp-level mma.sync kernel); "km_prune" (1 = spatially pruned k-means
 * assignment, the default; 0 = exhaustive scan -- both exact); "graphs" (1 = replay the
 * k-means iteration block as a CUDA graph, the default); "tc_bk" (k-step per
 * pipeline stage of the tensor-core kernel: 32, the default, or 16; setting it turns the
 * autotuner off); "tc_bn" (tile width of the tensor-core kernel: 128, the default, or 64
 * with k-step 16 and two CTAs per SM; setting it turns the autotuner off); "tc_persistent"
 * (1 = the persistent tensor-core kernel, one CTA per SM walking 128 x 64 tiles with two TMEM
 * buffers, for every product with K <= 512 and no split of K; setting it turns the
 * autotuner off); "autotune" (1 = choose k-step, tile order and split of K per product shape
 * by timing the candidates once per process, the default); "fft64" (mixed path: 1 = zeta
 * in FP64 through a D2Z FFT, 0 = FP32 and R2C, the default);
 * "profile" (1 = record a CUDA event pair around every launch of the named kernels,
 * 0 = stop and clear); "refine" (steps of iterative refinement of zeta after a shifted
 * solve of C, 0..8, default 0); "equilibrate" (mixed path: solve on C scaled to a unit-range
 * diagonal by powers of two, default 1); "overlap" (mixed path: factor C on a second stream
 * beside the P product, default 0); "spin_limit" (polls before a bounded device wait gives
 * up with THC_ERR_TIMEOUT, default 2^24); "tc_hi" (drain period of the tensor-core kernel's
 * level >= 3 accumulator in 16-k steps, a power of two 1..32, default 8); "qrcp_all_pairs"
 * (half-rotated QRCP: 1 = every (occupied, orbital) pair instead of the reference's
 * overlapping row layout, default 0). */
int thc_ctx_set_option(thc_ctx* ctx, const char* key, double value);
/* Accumulated device time (ms, from the profile events) and launch count of the kernels
 * named `kernel` since profiling was enabled; synchronises the context's stream. */
int thc_ctx_kernel_time(thc_ctx* ctx, const char* kernel, double* ms, long long* launches);
const char* thc_ctx_last_error(const thc_ctx* ctx);
/* The decisions of the tensor-core GEMM's autotuner on the context's device, one line per
 * shape class: k-step, tile order, split of K and the timed duration (context option
 * "autotune", default 1; the text stays valid until the next call on the context). */
const char* thc_ctx_autotune_log(thc_ctx* ctx);
const char* thc_status_string(int status);
/* Number of kernels this context has launched so far (its own kernels only). */
long long thc_ctx_kernel_launches(const thc_ctx* ctx);

/*
 * Initial interpolating-point indices (host only): iota(0..ng-1) shuffled by
 * std::shuffle with std::mt19937(seed), the first nmu kept and sorted ascending.
 */
int thc_kmeans_initial_indices(long long ng, int nmu, unsigned int seed, int* out_idx);

/*
 * Density-weighted k-means at the semantics of one MPI rank of the reference.
 *   grid      ng x 3 doubles, C order (the `real_space_grid` dataset)
 *   rho       ng doubles (the `density` / `density_occ` dataset)
 *   init_idx  nmu initial grid indices (from thc_kmeans_initial_indices)
 *   out_idx   nmu sorted interpolating-point indices (bit-identical to the reference)
 *   stats     optional
 * Returns THC_ERR_EMPTY_CLUSTER where the reference exits.
 */
int thc_kmeans(thc_ctx* ctx, const double* grid, const double* rho, long long ng, int nmu,
               const int* init_idx, int max_it, double threshold, int* out_idx,
               thc_kmeans_stats* stats);

/*
 * Per-iteration history of the last thc_kmeans call on this context: the normed
 * difference and the % of labels changed (the reference prints every 10th,
 * src/kmeans.cpp:238).  n must not exceed the last call's iteration count.
 */
int thc_kmeans_history(thc_ctx* ctx, double* diff, double* pct_changed, int n);

/*
 * Synthetic inputs: periodised Gaussian s/p basis functions on the mesh, as the reference's
 * input generator evaluates them with pyscf (tools/thcpy/thcpy/transform_basis.py:51-148)
 * for the seeded synthetic systems.  out[p * nfunc + f] (device, N_g x nfunc, overwritten)
 * = sum over the image centres c of atom a = f / 4 within rcut of point p of
 * exp(-alphas[f] |d|^2), times d_x, d_y or d_z for f % 4 = 1, 2, 3 (d = r_p - centre).
 *   grid         N_g x 3 doubles (host or device), C order over mesh (n2 fastest)
 *   mesh         3 ints (host)
 *   centres      ncentres x 3 doubles, the atom positions plus lattice translations that
 *                can reach the cell, grouped by atom (centre_atom non-decreasing)
 * Values agree with an FP64 evaluation to ~1e-6 relative (FP32 distances and expf).
 */
int thc_synth_gaussian_basis(thc_ctx* ctx, const double* grid, const int* mesh,
                             const double* centres, const int* centre_atom, int ncentres,
                             const double* alphas, int nfunc, double rcut, double* out);

/*
 * thc_kmeans without any device allocation.  No counterpart in the reference: it exists
 * for callers whose device memory is owned by their own pool allocator and who therefore
 * cannot let a library call cudaMalloc/cudaFree.  Same arguments, results and status codes
 * as thc_kmeans (bit-identical indices), for N_g <= 65,536, N_mu <= 1,024 and
 * max_it <= 1,000 (THC_ERR_SHAPE beyond).  All device scratch comes from one file-scope
 * 12 MiB device array shared by every call in the process; it keeps the last call's
 * contents (the call clears what must start at zero), and calls that overlap on the GPU
 * race on it, so serialise them.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress) and may load the module: make it before any stream capture.
 * thc_kmeans_history reports no history for these calls.
 */
int thc_kmeans_noalloc(thc_ctx* ctx, const double* grid, const double* rho, long long ng,
                       int nmu, const int* init_idx, int max_it, double threshold,
                       int* out_idx, thc_kmeans_stats* stats);

/*
 * ISDF interpolating vectors + FFT Coulomb matrix + its Cholesky factor.
 *   phi           ng x norb doubles, C order: the real part of `aoR` (real orbitals)
 *   idx           nmu grid indices (the k-means output)
 *   mesh          3 ints, n0*n1*n2 == ng (the `fft_grid` dataset)
 *   coulG         ng doubles (the `fft_coulomb` dataset)
 *   shift_rel     < 0: automatic (no shift unless Cholesky of C breaks down, then
 *                 1e-10 * tr(C)/nmu); >= 0: shift = shift_rel * tr(C)/nmu always
 *   out_orbitals  norb x nmu x 2 doubles: `/Hamiltonian/THC/Orbitals` (may be NULL)
 *   out_M         nmu x nmu x 2 doubles: the full Hermitian Coulomb matrix M (may be NULL)
 *   out_L         nmu x nmu x 2 doubles: `/Hamiltonian/THC/Luv`, lower triangle of
 *                 chol(M), upper triangle zero, C order (may be NULL)
 * Returns THC_ERR_NOT_PD (after writing all outputs) when Cholesky of M fails, as the
 * reference prints a warning and still writes Luv.
 */
int thc_isdf(thc_ctx* ctx, const double* phi, long long ng, int norb, const int* idx, int nmu,
             const int* mesh, const double* coulG, double shift_rel, double* out_orbitals,
             double* out_M, double* out_L, thc_isdf_stats* stats);

/*
 * thc_isdf for complex orbitals (k-point data): phi is ng x norb x 2 doubles, the `aoR`
 * dataset as stored ((re, im) pairs, C order); out_orbitals receives the complex values.
 * P = Phi_mu^H Phi is complex, but Z = P o conj(P) = |P|^2 and C = Z[:, idx] are real, so
 * the interpolating vectors, M and its factor follow the real path.  Runs in FP64 in both
 * precisions.
 */
int thc_isdf_complex(thc_ctx* ctx, const double* phi, long long ng, int norb, const int* idx,
                     int nmu, const int* mesh, const double* coulG, double shift_rel,
                     double* out_orbitals, double* out_M, double* out_L, thc_isdf_stats* stats);

/*
 * Half-rotated ISDF (the reference's `half_rotated` input option).  Same inputs as
 * thc_isdf plus the occupied orbitals; the pseudo-density products become
 *   Z = P_occ o P,  P = Phi_mu Phi^T,  P_occ = Phi_occ,mu Phi_occ^T,  C = Z[:, idx],
 * and M is written without a Cholesky factor.
 *   phi_occ            ng x nocc doubles, C order: the real part of `aoR_half`
 *   out_orbitals       norb x nmu x 2: `/Hamiltonian/THC/HalfTransformedFullOrbitals`
 *   out_occ_orbitals   nocc x nmu x 2: `/Hamiltonian/THC/HalfTransformedOccOrbitals`
 *   out_M              nmu x nmu x 2: `/Hamiltonian/THC/HalfTransformedMuv`
 * (each may be NULL).  C is symmetric positive semi-definite (a Schur product of two Gram
 * matrices), so the Cholesky solve and shift policy of thc_isdf apply unchanged.  Runs in
 * FP64 in both precisions.
 */
int thc_isdf_half(thc_ctx* ctx, const double* phi, long long ng, int norb, const double* phi_occ,
                  int nocc, const int* idx, int nmu, const int* mesh, const double* coulG,
                  double shift_rel, double* out_orbitals, double* out_occ_orbitals,
                  double* out_M, thc_isdf_stats* stats);

/*
 * The interpolating vectors of the last thc_isdf / thc_isdf_complex / thc_isdf_half call on
 * this context: out_zeta (nmu x ng doubles, host or device; row mu is zeta_mu on the grid,
 * in grid order) receives the solution of the least-squares problem C zeta^T = Z^T
 * (IVecs::kernel's least_squares, src/interpolating_vectors.cpp:416, whose result the
 * reference keeps in CZt before fft_vectors, :331-404).  The mixed path keeps them in FP32
 * (its FFT input); they are widened to FP64.  ng / nmu must be the last call's sizes
 * (THC_ERR_SHAPE otherwise); THC_ERR_ARG when the context holds no such result (no ISDF call
 * yet, or a later QRCP or failed ISDF call reused the workspace).
 */
int thc_isdf_interpolating_vectors(thc_ctx* ctx, long long ng, int nmu, double* out_zeta);

/*
 * thc_isdf_half for complex orbitals (k-point data): phi (ng x norb x 2) and phi_occ
 * (ng x nocc x 2) are `aoR` and `aoR_half` as stored ((re, im) pairs, C order).  As the
 * reference forms them (src/interpolating_vectors.cpp:143-161, :384-391, :261-273):
 * P = Phi_mu^H Phi, P_occ = Phi_occ,mu^H Phi_occ, Z = P_occ o conj(P), C = Z[:, idx] (complex,
 * not Hermitian), zeta = conj(C^{-1} Z), IVG / IVMG its forward / backward unnormalised FFTs
 * and M = IVMG^T diag(v) IVG (HalfTransformedMuv, no Cholesky factor).  C is inverted by
 * Gauss-Jordan elimination with partial pivoting in place of the reference's QR
 * (thc_isdf_stats.c_min_pivot = min / max |pivot|^2); THC_ERR_NOT_PD if a column has no
 * non-zero pivot.  out_orbitals / out_occ_orbitals receive the complex orbitals at the
 * points (HalfTransformedFullOrbitals / HalfTransformedOccOrbitals).  FP64 in both precisions.
 */
int thc_isdf_half_complex(thc_ctx* ctx, const double* phi, long long ng, int norb,
                          const double* phi_occ, int nocc, const int* idx, int nmu,
                          const int* mesh, const double* coulG, double* out_orbitals,
                          double* out_occ_orbitals, double* out_M, thc_isdf_stats* stats);

/*
 * Interpolating points by QR with column pivoting of Z^T (the reference's "qrcp" point
 * solver): [Z^T]_{(ik)a} = phi_i(r_a) phi_k(r_a) for real orbitals, or with phi_occ the
 * half-rotated rows phi_occ,i(r_a) phi_k(r_a) in the reference's row layout (rows
 * i * nocc + k, later pairs overwriting earlier ones when norb > nocc; the context option
 * "qrcp_all_pairs" = 1 keeps every pair instead).  The pivot sequence is computed as a
 * pivoted Cholesky factorisation of Z Z^T (the same pivots in exact arithmetic; Z^T is
 * never formed).  Ties go to the lowest grid index.
 *   phi         ng x norb doubles (the real part of `aoR`)
 *   phi_occ     ng x nocc doubles (the real part of `aoR_half`) or NULL
 *   npts        number of points (thc_cfac * norb), <= ng
 *   out_idx     npts grid indices, 0-based, sorted ascending
 *   out_order   npts pivots in the order chosen (may be NULL)
 *   out_diag    npts values |R_kk| in pivot order (may be NULL)
 */
int thc_qrcp(thc_ctx* ctx, const double* phi, long long ng, int norb, const double* phi_occ,
             int nocc, int npts, int* out_idx, int* out_order, double* out_diag,
             thc_qrcp_stats* stats);

/*
 * thc_qrcp for complex orbitals: phi is ng x norb x 2 doubles ((re, im) pairs, as `aoR` is
 * stored); the rows of Z^T are conj(phi_i) phi_k and its Gram matrix is |Phi^H Phi|^2.
 */
int thc_qrcp_complex(thc_ctx* ctx, const double* phi, long long ng, int norb, int npts,
                     int* out_idx, int* out_order, double* out_diag, thc_qrcp_stats* stats);

/*
 * One system of a batch: the inputs of thc_kmeans (grid, rho, init_idx, max_it, threshold)
 * and of thc_isdf (phi, norb, mesh, coulG, shift_rel), with nmu shared; outputs as in those
 * calls (out_idx required, the others optional).  status / stats are written back.
 */
typedef struct thc_system {
  const double* grid;
  const double* rho;
  long long ng;
  int nmu;
  const int* init_idx;
  int max_it;
  double threshold;
  const double* phi;
  int norb;
  const int* mesh;
  const double* coulG;
  double shift_rel;
  int* out_idx;
  double* out_orbitals;
  double* out_M;
  double* out_L;
  int status;
  thc_kmeans_stats kmeans_stats;
  thc_isdf_stats isdf_stats;
  char error[192];          /* the worker context's last error message when status != 0 */
} thc_system;

/*
 * Factorise nsys independent systems (k-means points, then ISDF) on one device.  Work is
 * spread over nstreams worker contexts, each with its own CUDA stream, workspace and host
 * thread, so that the kernels of small systems overlap on the GPU; nstreams = 1 runs the
 * systems one after another.  Worker contexts are cached per (device, precision) and
 * reused by later calls.  Returns THC_OK if every system succeeded (each system's own
 * status is in systems[i].status).  The reference factorises one system per run of
 * thcpp.x (src/main.cpp:18-77); this batches that sequence.
 */
int thc_factorize_batched(int device, int precision, thc_system* systems, int nsys, int nstreams);

#ifdef __cplusplus
}
#endif
#endif /* THC_GB300_H */
