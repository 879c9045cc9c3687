/* ctgpu.h - C ABI of the GB300 implementation of chemtensor's two-site DMRG path.
 *
 * Drop-in boundary: dmrg_twosite below has the reference's exact name,
 * signature, argument meaning, ownership rules and return codes, so a C caller
 * of the reference (python/pymodule.c:3317, perf/perf_dmrg.c:94,
 * examples/dmrg/basic_dmrg_fermi_hubbard.c:79) links libctgpu.so in place of
 * the reference's dmrg.c and is otherwise unchanged. All other entry points
 * carry a ctgpu_ prefix so that the library can sit beside the reference's
 * own symbols in one process.
 *
 * Return codes (reference: src/util/krylov.c:220-236, src/algorithm/dmrg.c:310-355):
 *    0  success
 *   -1  Lanczos breakdown before the first eigenvalue, or SVD / RQ failure
 *   -2  tridiagonal eigensolver failure
 *   -5  invalid arguments or a CUDA runtime error (message via ctgpu_last_error);
 *       this code has no counterpart in the reference, where such cases are assert()s
 *
 * Threading: every host thread gets its own CUDA stream and memory pool, so
 * independent calls from several threads run concurrently on the GPU.
 */
#ifndef CTGPU_H
#define CTGPU_H

#include <stddef.h>

#include "ct_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Two-site DMRG ground-state search.
 * Replaces dmrg_twosite, src/algorithm/dmrg.c:262-399 (declared in include/algorithm/dmrg.h:11-12).
 * hamiltonian: read only. psi: in/out; its site tensors are freed with free() and replaced by
 * tensors allocated with aligned_alloc(16, .), as the reference does. en_sweeps[num_sweeps] and
 * entropy[nsites-1] are caller-allocated; entropy[i] is written on the right-to-left pass. */
/* Tensors may be CT_DOUBLE_REAL or CT_DOUBLE_COMPLEX (MPO and MPS of the same type), as in the
 * reference; with complex tensors ctgpu_set_precision(1) is ignored (complex FP64 throughout). */
int dmrg_twosite(const struct mpo* hamiltonian, const int num_sweeps, const int maxiter_lanczos,
	const double tol_split, const ct_long max_vdim, struct mps* psi, double* en_sweeps, double* entropy);

/* Single-site DMRG ground-state search (bond dimensions fixed by the initial psi).
 * Replaces dmrg_singlesite, src/algorithm/dmrg.c:155-254 (declared in include/algorithm/dmrg.h:10).
 * Same ownership rules as dmrg_twosite; en_sweeps[num_sweeps] is caller-allocated. Always FP64. */
int dmrg_singlesite(const struct mpo* hamiltonian, const int num_sweeps, const int maxiter_lanczos,
	struct mps* psi, double* en_sweeps);

/* Arithmetic of the bulk block GEMMs for subsequent calls from this thread, all but 0 on the
 * tcgen05 tensor cores with FP32 accumulation:
 *   0 = FP64 (plain path);
 *   1 = split-BF16: each operand value split into a high and a low BF16 part, three products
 *       hi*hi + hi*lo + lo*hi, about 2^-16 relative error per product;
 *   2 = TF32: operands rounded to TF32, one product, about 2^-11;
 *   3 = three-part split-BF16: hi + mid + lo BF16 parts of the FP32 value, six products (every
 *       term down to 2^-16 relative), about 2^-23, i.e. FP32-like accuracy.
 * With 1-3, dmrg_twosite runs all sweeps but the last in that arithmetic and the last sweep
 * entirely in FP64, so returned energies and tensors are FP64 results; the single-operation entry
 * points below use the setting as given. The reference has no such setting (it always computes
 * in FP64). Returns the previous value, or -5 for an unknown value (the setting is then unchanged). */
int ctgpu_set_precision(int precision);

/* Number of trailing sweeps of dmrg_twosite that run entirely in FP64 when ctgpu_set_precision
 * selects a reduced arithmetic (default 1, at least 1). Per thread; returns the previous value, or -5
 * for n < 1. No counterpart in the reference. */
int ctgpu_set_final_fp64_sweeps(int n);

/* With 1, the environment updates of the split-BF16 sweeps (ctgpu_set_precision(1)) also run in
 * split-BF16; with 0 (default) they stay FP64 in every sweep. The trailing FP64 sweep rebuilds
 * every environment in FP64 either way. Per thread; returns the previous value. No counterpart in
 * the reference. */
int ctgpu_set_reduced_environments(int on);

/* Drop the lowered operations (device work lists) that this thread's context keeps for reuse
 * across calls; the next calls rebuild them as needed. No counterpart in the reference. */
int ctgpu_clear_plan_cache(void);

/* CUDA device used by subsequent calls from this thread. Returns the previous device. */
int ctgpu_set_device(int device);

/* Measurements of the most recent dmrg_twosite call in this thread. */
struct ctgpu_stats
{
	double wall_s;            /* host wall time of the whole call */
	double upload_s;          /* host structs -> HBM */
	double download_s;        /* HBM -> host structs */
	double setup_s;           /* right-normalisation, environments, merged MPO pairs */
	double sweep_s;           /* all sweeps */
	double lanczos_ms;        /* device time in the Lanczos eigensolver */
	double split_ms;          /* time in the SVD split, including the truncation decision */
	double env_ms;            /* device time in the environment updates */
	double matvec_flops;      /* algorithmic GEMM FLOPs of all local-Hamiltonian applications */
	double total_gemm_flops;  /* algorithmic GEMM FLOPs of the whole call */
	long   matvecs;           /* local-Hamiltonian applications */
	long   kernel_launches;   /* kernels launched by the call */
	int    sweeps;
	ct_long max_bond_dim;
	int    svd_max_sweeps;    /* largest Jacobi sweep count of any block SVD */
	double host_plan_s;       /* host time spent lowering operations into device work lists */
	long   plan_hits;         /* lowered operations reused from the per-thread plan cache */
	long   plan_misses;       /* lowered operations built afresh */
	double svd_flops;         /* FP64 flops of the block SVDs: Jacobi inner products and rotations as
	                             executed, QR and output factors estimated at full rank */
	long   near_ties;         /* SVD splits whose max_vdim cut fell between two singular values less
	                             than 1e-12 of the largest apart: rounding alone could then change which
	                             one is kept, and for exactly equal values the order of the sort decides
	                             (the reference sorts with the C library's qsort) */
};
int ctgpu_get_last_stats(struct ctgpu_stats* out);

/* Retained singular values (in the order the truncation keeps them, as split_block_sparse_matrix_svd
 * passes them on, src/algorithm/bond_ops.c:15-138) of the most recent split at bond `bond` (sites
 * bond, bond + 1) in this thread's last dmrg_twosite call; after a completed call these are the
 * values of the final right-to-left pass. Fills up to max entries of out and returns the count, or
 * -1 if that bond was not split. No counterpart in the reference. */
ct_long ctgpu_get_bond_singular_values(int bond, double* out, ct_long max);

/* Message of the most recent failure in this thread ("" if none). */
const char* ctgpu_last_error(void);

/* Measurement hooks (no counterpart in the reference, which only times whole calls). */

/* Time every kernel launch of subsequent calls by kernel class with CUDA events, from sweep
 * skip_sweeps on. Returns the previous setting. */
int ctgpu_set_profiling(int enable, int skip_sweeps);

/* Overwrite a device buffer of this many bytes before every sweep (0 = off), so that each
 * sweep starts with a cold L2. */
void ctgpu_set_l2_flush_bytes(ct_long bytes);

/* Device time (ms, CUDA events on the call's stream) and kernel launches of every sweep of the
 * most recent call; fills up to max entries and returns the number of sweeps. */
int ctgpu_get_sweep_times(double* ms, long* launches, int max);

/* Profile of one kernel class over the profiled sweeps of the most recent call:
 * 0 block GEMM (FP64), 1 permute, 2 row map, 3 axis scaling, 4 block SVD, 5 block RQ,
 * 6 Lanczos vectors, 7 block GEMM (split-BF16 tensor cores).
 * flops = algorithmic FLOPs (GEMM: sum of 2 m n k), bytes = algorithmic bytes moved. */
int ctgpu_get_kernel_profile(int cls, long* launches, double* ms, double* flops, double* bytes);

/* FP64 FMA throughput of the current device in TFLOP/s, measured with register-resident FMA
 * chains (the roofline denominator of the FP64 path); -1 on failure. */
double ctgpu_measure_fp64_tflops(void);

/* Choices of the reduced-precision GEMM autotuner so far in this process, one line per work-list
 * histogram key: "key choice ms64 ms128 ms256 ms_fp64 source", choice = tensor-core tile columns
 * (64, 128, 256) or 0 for the FP64 GEMM (products too small for the tensor cores to pay off), source
 * "timed" or "file" (read back from the tuning file). Writes at most cap - 1 characters and a
 * terminating zero to buf and returns the length of the whole text. No counterpart in the reference. */
int ctgpu_tile_tuning_report(char* buf, int cap);

/* Lowest eigenpair of the k x k symmetric tridiagonal matrix with diagonal alpha[0..k-1] and
 * off-diagonal beta[0..k-2] (1 <= k <= 32), by the device solver that every Lanczos run uses (the
 * reference calls LAPACK dsteqr here, src/util/krylov.c:230): *lambda and y[0..k-1] (unit norm,
 * largest-magnitude component positive). For parity tests of that solver. Returns 0, -2 if the
 * solver failed, or -5. */
int ctgpu_tridiag_lowest(const double* alpha, const double* beta, int k, double* lambda, double* y);

/* Host-side fault injection for tests of the error paths, per thread: which = 1 makes the next
 * `count` block SVDs report non-convergence (dmrg_twosite then returns -1, as the reference does
 * when LAPACK's SVD fails, src/tensor/block_sparse_tensor.c:2843-2847); which = 2 makes the next
 * `count` Lanczos tridiagonal eigensolves report failure (-2, as for a dsteqr failure,
 * src/util/krylov.c:231-236); which = 3 zeroes the start vector of the next `count` local
 * eigenproblems with a host-issued memset, so that the device's own norm check takes the breakdown
 * exit (-1: fewer Lanczos iterations than eigenvalues, src/util/krylov.c:218-223). No kernel is
 * made to fault. Returns 0, or -5 for other values. No counterpart in the reference. */
int ctgpu_inject_failure(int which, int count);

/* Column width of the tensor-core GEMM tiles for products planned from now on, process-wide:
 * 64, 128 or 256, or 0 (default) to let the tile autotuner choose per product. Products already
 * planned (and cached by a thread's context, see ctgpu_clear_plan_cache) keep their width.
 * Returns 0, or -5 for another value. No counterpart in the reference. */
int ctgpu_set_tc_tile_width(int bn);

/* Number of polls after which a bounded mbarrier wait inside the tensor-core GEMM gives up
 * (0 restores the default, 2^26). A wait that runs out makes the kernel record an error flag,
 * let its copies in flight land, free its tensor memory and return; the call that launched it
 * then returns -5. For tests of that error path; process-wide. No counterpart in the reference. */
void ctgpu_set_tc_wait_limit(long long polls);

/* ---- inputs ------------------------------------------------------------------------------ */

/* Seeded random MPS with the reference's generator, bit for bit: seed_rng_state followed by
 * construct_random_mps (src/util/rng.c:15-27, src/state/mps.c:93-175), real double precision.
 * Tensors are allocated with aligned_alloc(16, .). Returns 0, or -5 on invalid arguments. */
int ctgpu_construct_random_mps(int nsites, ct_long d, const qnumber* qsite, qnumber qnum_sector,
	ct_long max_vdim, uint64_t rng_seed, struct mps* mps);

/* First n standard normal draws of a freshly seeded generator (randn, src/util/rng.c:116-125). */
void ctgpu_randn_sequence(uint64_t seed, int n, double* out);

/* Free and total device memory of a CUDA device (cudaMemGetInfo), for admission control of
 * concurrent solves. Returns 0 or -5. No counterpart in the reference. */
int ctgpu_device_memory(int device, size_t* free_bytes, size_t* total_bytes);

/* <chi|psi> (chi complex conjugated) and ||psi||, contracted on the device (site tensors uploaded,
 * the environment kept in HBM). Replace mps_vdot (src/state/mps.c:314-370) and mps_norm
 * (src/state/mps.c:375-424). ctgpu_mps_vdot writes one double for CT_DOUBLE_REAL MPS and two (real,
 * imaginary part) for CT_DOUBLE_COMPLEX ones, as the reference writes one entry of the MPS's numeric
 * type. Leading and trailing virtual bonds must have dimension 1. Return 0, or -5 (message via
 * ctgpu_last_error). */
int ctgpu_mps_vdot(const struct mps* chi, const struct mps* psi, double* ret);
int ctgpu_mps_norm(const struct mps* psi, double* ret);

/* <chi|op|psi> (chi complex conjugated), contracted on the device by right environments with the
 * environment kept in HBM. Replaces mpo_inner_product (src/algorithm/chain_ops.c:274-317, declared in
 * include/algorithm/chain_ops.h:26): one double for CT_DOUBLE_REAL tensors, two (real, imaginary
 * part) for CT_DOUBLE_COMPLEX ones. Leading and trailing virtual bonds must have dimension 1 (the
 * reference asserts this). Returns 0, or -5 (message via ctgpu_last_error). */
int ctgpu_mpo_inner_product(const struct mps* chi, const struct mpo* op, const struct mps* psi, double* ret);

/* Spin-orbital molecular Hamiltonian
 *   H = sum_{ij,s} tkin[i,j] a+_{is} a_{js} + 1/2 sum_{ijkl,s,u} vint[i,j,k,l] a+_{is} a+_{ju} a_{lu} a_{ks}
 * as an MPO with one site per spatial orbital (local basis |0>, |dn>, |up>, |up dn>).
 * Replaces construct_spin_molecular_hamiltonian_mpo_assembly with optimize = false followed by
 * mpo_from_assembly (src/operator/hamiltonian.c:2768-2979, src/operator/mpo.c:59-174): same
 * operator and the same virtual bond dimensions (2 + 4n + 2M^2 - M, M = 2 min(b, n-b)) and bond
 * quantum numbers. tkin: n x n, vint: n x n x n x n, row-major. Host-only; the tensors of out are
 * allocated with aligned_alloc. Returns 0, or -5 for invalid arguments. */
int ctgpu_construct_spin_molecular_mpo(int nsites, const double* tkin, const double* vint, struct mpo* out);

/* ---- single operations, for parity checks of the device kernels ------------------------ */

/* block_sparse_tensor_dot (src/tensor/block_sparse_tensor.c:1826-2001); axrange 0 = leading,
 * 1 = trailing; r is allocated here (aligned_alloc / free contract). */
int ctgpu_block_sparse_tensor_dot(const struct block_sparse_tensor* s, int axrange_s,
	const struct block_sparse_tensor* t, int axrange_t, int ndim_mult, struct block_sparse_tensor* r);

/* block_sparse_tensor_transpose (src/tensor/block_sparse_tensor.c:785-870) */
int ctgpu_block_sparse_tensor_transpose(const int* perm, const struct block_sparse_tensor* t,
	struct block_sparse_tensor* r);

/* apply_local_hamiltonian (src/algorithm/chain_ops.c:353-390): b = H_loc(w, l, r) a */
int ctgpu_apply_local_hamiltonian(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
	const struct block_sparse_tensor* l, const struct block_sparse_tensor* r, struct block_sparse_tensor* b);

/* Measurement hook (no counterpart in the reference): device time *ms (CUDA events) of nmatvec
 * back-to-back applications of the local Hamiltonian of apply_local_hamiltonian to a, with the
 * tensors resident in HBM and the work lists built once, in the arithmetic of ctgpu_set_precision;
 * *flops receives the algorithmic GEMM FLOPs of one application (sum of 2 m n k). */
int ctgpu_time_local_hamiltonian(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
	const struct block_sparse_tensor* l, const struct block_sparse_tensor* r, int nmatvec, double* ms, double* flops);

/* contraction_operator_step_left / _right (src/algorithm/chain_ops.c:196-245 / :116-165), with b = a */
int ctgpu_contraction_operator_step_left(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
	const struct block_sparse_tensor* l, struct block_sparse_tensor* l_next);
int ctgpu_contraction_operator_step_right(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
	const struct block_sparse_tensor* r, struct block_sparse_tensor* r_next);

/* singular values of a block-sparse matrix as block_sparse_tensor_svd orders them
 * (src/tensor/block_sparse_tensor.c:2686-2848); sigma must hold min(dim0, dim1) entries,
 * *ns receives the count */
int ctgpu_block_sparse_tensor_svd_values(const struct block_sparse_tensor* a, double* sigma, ct_long* ns);

/* block_sparse_tensor_qr / block_sparse_tensor_rq (src/tensor/block_sparse_tensor.c:2402-2540 /
 * :2544-2676), mode QR_REDUCED (= 0) only; blocks factored with the conventions of LAPACK
 * dgeqrf + dorgqr and dgerqf + dorgrq (dense_tensor.c:2253-2651 / :2680-2880). Other modes
 * return -5. */
int ctgpu_block_sparse_tensor_qr(const struct block_sparse_tensor* a, int mode, struct block_sparse_tensor* q,
	struct block_sparse_tensor* r);
int ctgpu_block_sparse_tensor_rq(const struct block_sparse_tensor* a, int mode, struct block_sparse_tensor* r,
	struct block_sparse_tensor* q);

/* release a tensor returned by one of the calls above (free() on every array) */
void ctgpu_delete_block_sparse_tensor(struct block_sparse_tensor* t);

/* SVD of one dense row-major m x n FP64 matrix that is already in device memory, for callers
 * that must not allocate device memory while they run (for example a service whose device memory
 * is reserved up front by its own pool, or code whose stream must not be stalled by the implicit
 * device-wide synchronisation of cudaMalloc / cudaFree). It allocates nothing: its workspace is a
 * fixed 4 MiB array inside the library, held on every GPU that loads the library until the
 * process exits, which limits m and n to 1..256.
 * Outputs (device memory, row-major): d_u (m x k), d_s (k), d_vh (k x n), k = min(m, n), singular
 * values in descending order; *d_info (device) becomes 0, or -1 if the Jacobi iteration did not
 * converge. The work is queued on 'stream' (a cudaStream_t, or NULL for the legacy default stream)
 * and the call returns without waiting; it returns 0 once queued, -5 for sizes outside 1..256, a
 * null pointer, a CUDA error of one of its own launches, or a CUDA error already pending from the
 * caller's earlier work (which it reports and leaves in place, queueing nothing). The first call on
 * a device looks up the array's device address (once per device, with that device current); make
 * that first call before any stream capture. With lazy module loading (the CUDA default) that first
 * call, or the first use of the library on a device, also loads the library's kernels and the 4 MiB
 * array onto the device: a caller that reserves the rest of device memory for its own pool makes
 * the first call before reserving it, or runs with CUDA_MODULE_LOADING=EAGER.
 * All calls share the array, so calls whose work overlaps on the GPU race and must be serialised
 * by the caller.
 * No counterpart in the reference, which computes block SVDs with LAPACK on the host. */
int ctgpu_dense_svd_noalloc(const double* d_a, int m, int n, double* d_u, double* d_s, double* d_vh,
	int* d_info, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CTGPU_H */
