/* qcmg.h -- C ABI of the GB300 (sm_103a) engine for pyqcm's exact
 * diagonalization hot path: the factorized Hubbard Hamiltonian-vector product
 * inside Lanczos and band Lanczos, the Lehmann (Q-matrix) Green function, and
 * the CPT/VCA/CDMFT k x omega lattice integrals over it.
 *
 * Plain C types only: pointers, sizes, doubles.  Every function returns 0 on
 * success or a negative QCMG_ERR_* code; qcmg_last_error() then holds a
 * message for the calling thread.  Handles are independent: two threads may
 * use two handles concurrently; one handle must not be used by two threads
 * at once.  All arrays are caller-owned.  Unless a flag says otherwise,
 * vector arguments are HOST pointers and the call copies them to and from the
 * device; with QCMG_DEVICE_PTRS they are device pointers on the handle's GPU.
 *
 * Conventions shared with the reference (pyqcm, src_ed/):
 *  - orbitals 0..L-1 are spin up, L..2L-1 spin down; a one-body element
 *    (r, c, v) is v c^dagger_r c_c and must be given for both (r,c) and (c,r);
 *  - half basis of a spin = increasing L-bit integers with popcount N
 *    (src_ed/ED_basis.cpp:115-135); factorized index
 *    I = i_up + dim_up * i_dn (src_ed/ED_basis.cpp:142-165);
 *  - a hop r <- c carries the sign (-1)^(occupied orbitals strictly between)
 *    (src_ed/binary_state.hpp:42-49).
 */
#ifndef QCMG_H
#define QCMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QCMG_OK 0
#define QCMG_ERR_ARG -1      /* invalid argument (size, index, null pointer) */
#define QCMG_ERR_CUDA -2     /* CUDA runtime or library failure */
#define QCMG_ERR_NOMEM -3    /* device allocation failed */
#define QCMG_ERR_NOCONV -4   /* iteration limit reached before convergence */
#define QCMG_ERR_DEVICE -5   /* no usable GPU */
#define QCMG_ERR_NUMERIC -6  /* non-finite value or breakdown detected */

#define QCMG_DEVICE_PTRS 1u  /* vector arguments are device pointers */
#define QCMG_ACCUMULATE 2u   /* y += H x (otherwise y = H x) */
#define QCMG_ASYNC 4u        /* with QCMG_DEVICE_PTRS: return without waiting for the GPU */

typedef struct qcmg_hamiltonian qcmg_hamiltonian;

/* Version string of the library. */
const char* qcmg_version(void);

/* Copies the calling thread's last error message into buf (NUL-terminated,
 * truncated to n bytes).  Returns the full message length. */
size_t qcmg_last_error(char* buf, size_t n);

/* Selects the GPU used by handles created afterwards on this thread. */
int qcmg_set_device(int device);

/* Half basis of L orbitals with N electrons, built on the GPU by unranking
 * the combinatorial number system.  Writes at most cap states into out and
 * the dimension C(L,N) into *dim.
 * Replaces ED_halfbasis::ED_halfbasis (src_ed/ED_basis.cpp:115-125). */
int qcmg_halfbasis(int L, int N, uint32_t* out, size_t cap, size_t* dim);

/* Ranks of n half-states (popcount N) computed on the GPU; a state that is
 * not in the basis gets rank dim.
 * Replaces ED_halfbasis::index (src_ed/ED_basis.cpp:130-135). */
int qcmg_halfbasis_rank(int L, int N, const uint32_t* states, size_t n, uint32_t* ranks);

/* Factorized Hamiltonian of the sector (N_up, N_dn) on L orbitals:
 *   H = T_dn (x) 1 + 1 (x) T_up + sum_pairs v n_r n_c
 * hop_{up,dn}: n_hop one-body elements (r, c, v) of each spin, with r, c in
 *   0..L-1, the coefficients of the value map already applied and both
 *   triangles given (r == c adds v n_r);
 * pairs: n_pair density-density elements (r, c, v) on spin-orbitals
 *   0..2L-1, adding v n_r n_c.
 * The half-operators are built on the GPU from these elements.
 * Replaces Hamiltonian_Factorized::Hamiltonian_Factorized and its
 * HS_ops_map (src_ed/Hamiltonian/Hamiltonian_Factorized.hpp:31-87), the
 * HS_half_operator construction (src_ed/Operators/HS_half_operator.hpp:21-45)
 * and the HS_interaction_operator table
 * (src_ed/Operators/HS_interaction_operator.hpp:32-54). */
int qcmg_hamiltonian_create(int L, int n_up, int n_dn,
                            int n_hop_up, const int32_t* up_r, const int32_t* up_c,
                            const double* up_v,
                            int n_hop_dn, const int32_t* dn_r, const int32_t* dn_c,
                            const double* dn_v,
                            int n_pair, const int32_t* pair_r, const int32_t* pair_c,
                            const double* pair_v,
                            qcmg_hamiltonian** out);

int qcmg_hamiltonian_destroy(qcmg_hamiltonian* H);

/* Makes the handle launch its work on `stream` (a cudaStream_t of the
 * handle's device; NULL restores the handle's own stream).  No counterpart
 * in the reference, whose products run on the calling CPU thread. */
int qcmg_hamiltonian_set_stream(qcmg_hamiltonian* H, void* stream);

/* Sector dimensions: dim_up, dim_dn and dim = dim_up * dim_dn. */
int qcmg_hamiltonian_dims(const qcmg_hamiltonian* H, size_t* dim_up, size_t* dim_dn,
                          size_t* dim);

/* Exports the half-operator of one spin (0 up, 1 down) as CSR rows indexed
 * by the input state: rowptr[dim_s+1], col[nnz], val[nnz], diag[dim_s].
 * Call with rowptr == NULL to get *nnz only.  For checking against the
 * reference's HS_half_operator tables. */
int qcmg_hamiltonian_halfop(const qcmg_hamiltonian* H, int spin, size_t* nnz, uint32_t* rowptr,
                            uint32_t* col, double* val, double* diag);

/* y = H x, or y += H x with QCMG_ACCUMULATE.  x and y have length dim.
 * Replaces Hamiltonian_Factorized::mult_add
 * (src_ed/Hamiltonian/Hamiltonian_Factorized.hpp:50-58) with
 * HS_factorized_operator::multiply_add (HS_factorized_operator.hpp:57-84)
 * and HS_interaction_operator::multiply_add (HS_interaction_operator.hpp:62-70).
 * Host vectors (no QCMG_DEVICE_PTRS): x is copied to the device; when all of
 * y lies in one page-locked allocation of the handle's device, the result
 * is read-modify-written into y in host memory by the device (zero copy),
 * otherwise y is staged through device memory.  QCMG_VERBOSE in the
 * environment prints the form taken and its phase times on stderr. */
int qcmg_matvec(qcmg_hamiltonian* H, const double* x, double* y, unsigned flags);

/* Chooses the arithmetic of the handle's products and Lanczos runs:
 * path 1 (default) uses the fixed-point fast path whenever the sector's hops
 * have one magnitude per spin (the Hubbard form), path 0 always uses the
 * FP64 kernels.  No counterpart in the reference (FP64 throughout). */
int qcmg_hamiltonian_set_path(qcmg_hamiltonian* H, int path);

/* *available = 1 when the fixed-point fast path applies to this sector. */
int qcmg_hamiltonian_fx_available(qcmg_hamiltonian* H, int* available);

/* Device vectors in the fixed-point format of the fast path:
 * value_i = q_i * 2^E with |q_i| < 2^mb.  Conversions run on `stream`
 * (a cudaStream_t, NULL = default stream); all pointers are device pointers. */
int qcmg_fx_from_f64(size_t n, const double* x, int64_t* q, int* E, int* mb, void* stream);
int qcmg_fx_to_f64(size_t n, const int64_t* q, int E, double* x, void* stream);

/* y = H x on fixed-point device vectors (length dim): x given by (qx, Ex,
 * mbx); the result's exponent is returned in *Ey (|qy| < 2^56).  With
 * QCMG_ACCUMULATE, y = y + H x: *Ey gives the input y's exponent on entry
 * (|qy| < 2^56) and the result's on return.  Launches on the handle's
 * stream; QCMG_ASYNC returns without waiting.  Same product as qcmg_matvec
 * (Hamiltonian_Factorized::mult_add), exact integer arithmetic on the hops
 * and one rounding per diagonal term. */
int qcmg_matvec_fx(qcmg_hamiltonian* H, const int64_t* qx, int Ex, int mbx, int64_t* qy, int* Ey,
                   unsigned flags);

/* out[k] = <V_k, w> for k < m: V is a device array of m device pointers to
 * vectors of length n, w a device vector, out a host array of m doubles.
 * Fixed-order (deterministic) two-level reduction on `stream`; allocates its
 * device scratch for the call.  The projections of classical Gram-Schmidt
 * reorthogonalization and of band Lanczos' inner products
 * (src_ed/Hamiltonian/Lanczos.hpp:255-330 computes them one ddot at a time). */
int qcmg_multidot(int m, const double* const* V, const double* w, size_t n, double* out,
                  void* stream);

/* qcmg_multidot for callers that may not allocate device memory (a host
 * framework owning the GPU through its own pool or a memory cap; code that
 * must not allocate while other work runs).  No counterpart in the
 * reference.  Same arguments and kernels, except that out is a DEVICE array
 * of m doubles, the call returns without waiting, and it runs on the calling
 * thread's current CUDA device (not the one chosen with qcmg_set_device).
 * Allocates nothing: the partial sums live in a fixed 155,648-byte device
 * array of the library, so m is limited to 64 (QCMG_ERR_ARG beyond; m == 0
 * returns QCMG_OK).  The array is reserved when CUDA loads the library's
 * module on the device, which under lazy module loading (the default) is the
 * first call: make that first call before handing the GPU's memory to a
 * pool or a cap, and before any stream capture (it also looks up the
 * array's address, once per device and context).  Calls that overlap in
 * time on one device race on the array: serialize them. */
int qcmg_multidot_noalloc(int m, const double* const* V, const double* w, size_t n, double* out,
                          void* stream);

/* Seeded start vector of the reference: std::default_random_engine(seed)
 * drawing std::normal_distribution(0,1), normalized.
 * Replaces random() (src_util/vector_num.cpp:114-119). */
int qcmg_seeded_vector(size_t dim, unsigned seed, double* out);

/* Lanczos ground state.  x0 (length dim, normalized; NULL = seeded start
 * with `seed`) starts the three-term recurrence of the reference
 * (no reorthogonalization when reorth == 0); iteration stops when the Ritz
 * residual |s_last * beta| < tol or after max_iter steps.  With reorth > 0 the
 * Lanczos basis is kept on the device and every new vector is
 * reorthogonalized (classical Gram-Schmidt, twice) against all previous ones;
 * at most `reorth` vectors are kept: when that many are held and the residual
 * has not converged, the iteration restarts from the current Ritz vector.
 * Outputs: *E0; psi (length dim, may be NULL: then no second pass);
 * *niter (all iterations, restarts included); alpha, beta (capacity `cap`,
 * may be NULL: the coefficients of the last restart cycle).
 * Replaces LanczosEigenvalue + LanczosEigenvector
 * (src_ed/Hamiltonian/Lanczos.hpp:41-143) as called from
 * Hamiltonian::states (src_ed/Hamiltonian/Hamiltonian_base.hpp:114-221). */
int qcmg_lanczos_ground_state(qcmg_hamiltonian* H, const double* x0, unsigned seed, double tol,
                              int max_iter, int reorth, double* E0, double* psi, int* niter,
                              double* alpha, double* beta, int cap);

/* Lanczos ground states of n sectors (handles H[0..n-1], one device, no
 * handle twice) at once: the three-term recurrence of
 * qcmg_lanczos_ground_state (no reorthogonalization, FP64 product, seeded
 * start `seed`) with alpha, beta and the step index kept on the device, each
 * sector's steps captured once as a CUDA graph of `chunk` steps (rounded up
 * to even) on a stream of its own and relaunched until the Ritz residual is
 * below tol (tested after every step, as the reference does) or max_iter
 * steps; sectors of any sizes run side by side.  Outputs per sector: E0[i],
 * niter[i] (may be NULL), status[i] (QCMG_OK, QCMG_ERR_NOCONV or
 * QCMG_ERR_NUMERIC; may be NULL) and, where psi[i] is not NULL (psi itself
 * may be NULL), the ground-state vector (host array of length dim).  The
 * energies, coefficients and vectors equal those of
 * qcmg_lanczos_ground_state on the FP64 path bit for bit.  Replaces the
 * per-sector LanczosEigenvalue + LanczosEigenvector calls
 * (src_ed/Hamiltonian/Lanczos.hpp:41-143) that the reference's
 * low_energy_states makes sector by sector
 * (src_ed/model_instance.hpp:274-292). */
int qcmg_lanczos_batch(int n, qcmg_hamiltonian* const* H, unsigned seed, double tol, int max_iter,
                       int chunk, double* E0, int* niter, double* const* psi, int* status);

/* FP64 FMA rate of the current device in TFLOP/s: one timed launch of
 * eight independent FMA chains per thread over 8 blocks of 256 threads per
 * SM (after one untimed launch).  The roofline denominator of the FP64
 * kernels; not part of the reference's interface. */
int qcmg_fp64_fma_rate(double* tflops);

/* Breakdown of the last reorthogonalized qcmg_lanczos_ground_state on H:
 * device time of the products and of the Gram-Schmidt sweeps (ms), the
 * sweeps' algorithmic bytes (16 per stored vector element per pass, two
 * passes per step), restarts, vectors held at most, and the length of the
 * last restart cycle (the number of alpha/beta coefficients returned).  Any
 * pointer may be NULL.  No counterpart in the reference, whose Lanczos has no
 * reorthogonalization (src_ed/Hamiltonian/Lanczos.hpp:41-95). */
int qcmg_lanczos_last_stats(qcmg_hamiltonian* H, double* product_ms, double* reorth_ms,
                            double* reorth_bytes, int* restarts, int* vectors, int* cycle);

/* Band Lanczos from p start vectors phi (p x dim, row-major: vector k at
 * phi + k*dim).  M_target is the requested number of steps (the reference
 * uses 14 p ln(dim), capped at max_iter); deflation below acc_deflation;
 * stops when the lowest eigenvalue of the projected matrix moves by less
 * than acc_band between checks.
 * Outputs: *M (number of poles), evals[M] and Q (p x M, row-major) =
 * P U restricted to the first p Lanczos vectors; caller capacity `cap` >= M.
 * Replaces bandLanczos + Hamiltonian::build_Q_matrix
 * (src_ed/Hamiltonian/Lanczos.hpp:214-395, Hamiltonian_base.hpp:229-254). */
int qcmg_band_lanczos(qcmg_hamiltonian* H, int p, const double* phi, int M_target, int max_iter,
                      double acc_deflation, double acc_band, int* M, double* evals, double* Q,
                      int cap);

/* Continued-fraction Lanczos from one normalized start vector psi (length
 * dim; a device pointer with QCMG_DEVICE_PTRS): the three-term recurrence
 * with the reference's stopping rule (the product of the b's or the last b
 * at or below accur, or max_iter steps).  Outputs *n steps, a[n] and
 * b[n + 1] with b[0] = 1; capacity cap >= n.  Replaces LanczosGreen
 * (src_ed/Hamiltonian/Lanczos.hpp:156-183), called by
 * model_instance<double>::build_cf (src_ed/model_instance.cpp:35-100). */
int qcmg_lanczos_green(qcmg_hamiltonian* H, const double* psi, unsigned flags, double accur,
                       int max_iter, int* n, double* a, double* b, int cap);

/* Block Lanczos for the matrix continued fraction (GF_method 'M'), with
 * the reference's default polar coupling blocks: p start vectors phi (p x
 * dim, row-major; device pointers with QCMG_DEVICE_PTRS) are factored
 * phi = q W by modified Gram-Schmidt (stopping at the first column of norm
 * below acc_deflation: *p_actual <= p), then the block recurrence
 * H Q_j = Q_{j-1} B_{j-1} + Q_j A_j + Q_{j+1} B_j runs for at most
 * min(M_target, max_iter) steps, stopping when the lowest eigenvalue of the
 * block-tridiagonal projection moves by less than acc_band between checks
 * (every p_actual steps) or a coupling block becomes singular.
 * Outputs: *M blocks A and B (each p_actual x p_actual, row-major, the last B
 * being the truncation residual) and W (p_actual x p, row-major); capacity
 * cap >= *M blocks.  Replaces blockLanczosSVD (src_ed/Hamiltonian/Lanczos.hpp:
 * 603-790) and the start-block factorization of model_instance::build_mcf
 * (src_ed/model_instance.hpp:847-955). */
int qcmg_block_lanczos(qcmg_hamiltonian* H, int p, const double* phi, unsigned flags,
                       int M_target, int max_iter, double acc_deflation, double acc_band, int* M,
                       int* p_actual, double* A, double* B, double* W, int cap);

/* qcmg_band_lanczos with the p host start vectors given as an array of
 * pointers (phi[k] of length dim), as the reference holds them
 * (vector<vector<HF>>& phi of Hamiltonian::build_Q_matrix,
 * src_ed/Hamiltonian/Hamiltonian_base.hpp:229-254): each is copied to the
 * device directly, with no flat host copy. */
int qcmg_band_lanczos_ptrs(qcmg_hamiltonian* H, int p, const double* const* phi, int M_target,
                           int max_iter, double acc_deflation, double acc_band, int* M,
                           double* evals, double* Q, int cap);

/* qcmg_band_lanczos with the start vectors already in the handle's device
 * memory (p x dim, row-major; e.g. written there by qcmg_apply_c with
 * QCMG_DEVICE_PTRS), so they cross no host link.  The call waits for the
 * device before reading them and only reads them.  Same reference
 * interface as qcmg_band_lanczos (Hamiltonian_base.hpp:229-254), whose
 * start vectors the reference builds in host memory. */
int qcmg_band_lanczos_device(qcmg_hamiltonian* H, int p, const double* phi_dev, int M_target,
                             int max_iter, double acc_deflation, double acc_band, int* M,
                             double* evals, double* Q, int cap);

/* c_orb (pm = -1) or c^dagger_orb (pm = +1) applied to x of sector
 * (n_up, n_dn) on L orbitals; orb >= L is a down orbital.  y (target sector,
 * length dim_up' * dim_dn') receives y (+)= z * c x.
 * Replaces model::create_or_destroy, factorized branch
 * (src_ed/model.cpp:155-180) with Destroy (src_ed/ED_basis.cpp:79-110). */
int qcmg_apply_c(int L, int orb, int pm, int n_up, int n_dn, const double* x, double* y,
                 double z, unsigned flags);

/* Lehmann Green function G(z_w) = sum_i v_i v_i^dagger / (z_w - e_i) for nz
 * frequencies, batched on the GPU.  e[M]; v: complex L x M (interleaved
 * re,im, column-major: element (a,i) at 2*(a + L*i)); z: nz complex
 * (interleaved); G: nz blocks of L x L complex, column-major, in the
 * reference's orientation G(b,a) = sum_i v_ai u_i conj(v_bi).
 * Replaces Q_matrix::Green_function + VDVH_naive
 * (src_ed/Q_matrix.hpp:133-151, src_util/VDVH_kernel.cpp:28-48). */
int qcmg_green_function(int L, int M, const double* e, const double* v, int nz, const double* z,
                        double* G);

/* ---------------------------------------------------------------------------
 * Lattice integrals (CPT / VCA / CDMFT) over a cluster Green function.
 *
 * A lattice handle holds one spin block of a lattice model instance:
 *   t(K) - t_c = Hdiff + sum_e v_e exp(2 pi i K.R[n_e]) |r_e><c_e|
 * with K in the reduced (superlattice-dual) basis and R[n] the superlattice
 * translations in the superlattice basis; Hdiff (L x L complex, row-major,
 * interleaved re/im) is the k-independent difference between the lattice and
 * cluster one-body matrices; gpos (L x 3) are the orbital positions in the
 * superlattice basis (for periodization).  This is the data the reference's
 * lattice_model_instance::set_V combines (src_qcm/CPT.cpp:22-64): R =
 * lattice_model::neighbor, elements = lattice_operator::IGF_elem times the
 * parameter values, Hdiff = H - Hc. */
/* Cluster self-energy and hybridization function at nz complex frequencies
 * z (re, im pairs), on the device:
 *   Gamma(z) = tcb (z - diag(eb))^-1 tcb^dagger,
 *   Sigma(z) = z - t_c - Gamma(z) - G(z)^-1,
 * with G(z) from the Q-matrix (e, v as in qcmg_green_function: v
 * column-major, element (a, i) at a + L i), tcb the L x nb cluster-bath block
 * (column-major, (r, i) at r + L i), eb the nb bath energies (bath
 * diagonalized) and t_c the L x L cluster block (row-major complex).
 * sigma and gamma (may be NULL): nz x L x L complex, row-major [w][r][c].
 * Replaces model_instance::self_energy and hybridization_function
 * (src_ed/model_instance.hpp:683-700, 1004-1017), frequency by frequency
 * there. */
int qcmg_self_energy(int L, int M, const double* e, const double* v, int nb, const double* tcb,
                     const double* eb, const double* tc, int nz, const double* z, double* sigma,
                     double* gamma);

typedef struct qcmg_lattice qcmg_lattice;

int qcmg_lattice_create(int L, int nR, const double* R, int nel, const int32_t* el_r,
                        const int32_t* el_c, const int32_t* el_n, const double* el_v,
                        const double* hdiff, const double* gpos, qcmg_lattice** out);
int qcmg_lattice_destroy(qcmg_lattice* lat);

/* Cluster Green function of the block: Q-matrix (e[M], v: L x M complex,
 * column-major interleaved) and bath hybridization tcb (L x nb complex,
 * column-major), eb[nb]: Gamma(z) = sum_i tcb_i tcb_i^+ / (z - eb_i).
 * Replaces cluster_Green_function + hybridization_function
 * (src_qcm/lattice_model_instance.cpp, src_ed/model_instance.hpp:1004-1017). */
int qcmg_lattice_set_green(qcmg_lattice* lat, int M, const double* e, const double* v, int nb,
                           const double* tcb, const double* eb);

/* out = sum_w wt[w] (1/Nk) sum_K log|det(V(K, i w) G(i w) - 1)| on the grid
 * K = (i/nkx, j/nky, l/nkz).  The caller combines spin blocks as the
 * reference does (x2 for normal mixing).  Replaces the fixed-grid branch of
 * lattice_model_instance::Potthoff_functional with SEF_integrand_k and
 * QCM::k_integral_grid (src_qcm/lattice_model_instance.cpp:520-546,624-643,
 * src_util/integrate.cpp:177-239). */
int qcmg_sef_grid(qcmg_lattice* lat, int nw, const double* w, const double* wt, int nkx, int nky,
                  int nkz, double* out);

/* Periodized CPT Green function g(K, z) = (1/L) sum_ab Gcpt_ab(K,z)
 * exp(2 pi i K.(x_b - x_a)) for nz complex frequencies z and nk reduced
 * wavevectors K (nk x 3); g is nz x nk complex (interleaved).  Replaces
 * set_Gcpt + lattice_model::periodize (src_qcm/CPT.cpp:76-86,171-176,
 * src_qcm/lattice_model.cpp:724-740) for one band. */
int qcmg_cpt_periodized(qcmg_lattice* lat, int nz, const double* z, int nk, const double* K,
                        double* g);

/* Mean of the CPT Green function (G(z)^-1 - V(K))^-1 over the K grid
 * ((i + off)/nkx, (j + off)/nky, (l + off)/nkz) for nz complex frequencies z
 * (re, im pairs); out is nz blocks of L x L complex, row-major.  Replaces
 * the K sums of lattice_model_instance::dos on the wavevector grid
 * (src_qcm/average.cpp:294-347, whose diagonal gives the density of states)
 * and of projected_Green_function. */
int qcmg_lattice_kmean(qcmg_lattice* lat, int nz, const double* z, int nkx, int nky, int nkz,
                       double off, double* out);

/* K moments of the CPT Green function on the same grid: for nmom (1..16)
 * translations R_m (nmom x 3, in the basis of qcmg_lattice_create's R),
 *   out[w][m] = mean_K exp(2 pi i K.R_m) (G(z_w)^-1 - V(K))^-1,
 * nz x nmom blocks of L x L complex, row-major.  Every lattice average is a
 * real linear form in these blocks: the K sum of average_integrand_k
 * (src_qcm/average.cpp:157-190), sum_e v_e Gcpt(c_e, r_e) phase_n(e)(K),
 * regrouped by translation, for lattice_model_instance::averages on the
 * frequency and wavevector grids (src_qcm/average.cpp:24-105). */
int qcmg_lattice_kmoments(qcmg_lattice* lat, int nz, const double* z, int nkx, int nky, int nkz,
                          double off, int nmom, const double* R, double* out);

/* Projected (k-averaged) CPT Green function on the midpoint grid of side
 * kside in dimk dimensions, at imaginary frequencies i w: pgf is nw blocks of
 * L x L complex, row-major.  Replaces lattice_model_instance::
 * projected_Green_function (src_qcm/CPT.cpp:283-345), the kernel of
 * CDMFT_host. */
int qcmg_cdmft_projected(qcmg_lattice* lat, int nw, const double* w, int kside, int dimk,
                         double* pgf);

/* CDMFT bath fit of n_inst instances at once on the device (one CTA each):
 * least squares of r_n = sqrt(weights_n) (Gamma(i w_n) + host_n), real and
 * imaginary parts, Gamma(z) = theta (z - E)^-1 theta^T with theta the
 * ns x nb cluster-bath block and E = diag(e) the bath energies.  The npar
 * parameters x enter linearly through nent entries: entry q adds
 * ent_val[q] * x[ent_par[q]] to theta[ent_i[q]][ent_j[q]] (ent_kind 0) or
 * to e[ent_j[q]] (ent_kind 1, with ent_i == ent_j), on top of the fixed
 * parts theta0 (n_inst x ns x nb) and e0 (n_inst x nb).  host: n_inst x nw x
 * ns x ns complex (re, im), row-major.  x (n_inst x npar): start in, fit
 * out.  Levenberg-Marquardt on the exact normal equations; stops when the
 * cost decrease on a well-predicted step is below ftol * cost (status 1),
 * the step below xtol (xtol + |x|) (2), the gradient below gtol (3), or
 * after max_iter iterations (0); -1: the damped normal equations stayed
 * singular.  With ftol = 0 the fit then takes exact Gauss-Newton steps for
 * as long as they lower the gradient (convergence on the gradient).  cost[k] = 1/2 sum r^2 at the fit.  Limits: ns <= 8, nb <= 16,
 * npar <= 32, nent <= 128.  Replaces the bath optimization of the
 * reference's CDMFT step: CDMFT_residuals / CDMFT_distance
 * (src_qcm/CPT.cpp:519-672) minimized by SciPy from pyqcm/cdmft.py:1539-1640. */
int qcmg_bath_fit(int n_inst, int ns, int nb, int nw, const double* w, const double* weights,
                  const double* host, int npar, int nent, const int* ent_par, const int* ent_kind,
                  const int* ent_i, const int* ent_j, const double* ent_val, const double* theta0,
                  const double* e0, double* x, int max_iter, double xtol, double ftol,
                  double gtol, double* cost, int* iters, int* status);

/* ---------------------------------------------------------------------------
 * Multilayer perceptron of the learned CDMFT warm start (no counterpart in
 * the reference).  Layers l < n_layers map width[l] -> width[l+1]; hidden
 * layers use tanh, the last one is linear.  Parameters are FP32 on the host
 * side of the ABI, laid out W_0, b_0, W_1, b_1, ... with W_l row-major
 * [width[l+1] x width[l]]; the device keeps an FP32 master copy and uses a
 * BF16 copy of the weights in every product, accumulating in FP32.  All
 * arrays below are host arrays, row-major [batch x width]. */
typedef struct qcmg_mlp qcmg_mlp;

int qcmg_mlp_create(int n_layers, const int* widths, qcmg_mlp** out);
int qcmg_mlp_destroy(qcmg_mlp* mlp);
int qcmg_mlp_num_params(qcmg_mlp* mlp, size_t* n);
/* Sets the FP32 master parameters (and their BF16 copy); resets Adam. */
int qcmg_mlp_set_params(qcmg_mlp* mlp, const float* params);
int qcmg_mlp_get_params(qcmg_mlp* mlp, float* params);
int qcmg_mlp_forward(qcmg_mlp* mlp, int batch, const float* x, float* y);
/* Mean squared error against t and its gradient with respect to the FP32
 * parameters (grad may be NULL). */
int qcmg_mlp_loss_grad(qcmg_mlp* mlp, int batch, const float* x, const float* t, float* loss,
                       float* grad);
/* Adam (beta1 0.9, beta2 0.999, eps 1e-8) over `epochs` shuffled passes of
 * minibatches of `batch` rows, the learning rate annealed from lr to 0 along
 * half a cosine over the run's steps; *final_loss = mean loss of the last
 * epoch. */
int qcmg_mlp_train(qcmg_mlp* mlp, int n, const float* x, const float* t, int epochs, int batch,
                   float lr, unsigned seed, float* final_loss);

#ifdef __cplusplus
}
#endif
#endif
