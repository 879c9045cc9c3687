/* ct_oracle.h - CPU restatement of chemtensor's DMRG path (two-site and single-site).
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker for the GB300
 * implementation and the timed CPU baseline; nothing in the product links or
 * calls it. It restates, in plain C with OpenMP and BLAS/LAPACK (the OpenBLAS
 * bundled with scipy), the reference algorithms cited beside each function in
 * ct_oracle.c. Parity of this restatement is pinned against the reference
 * itself (compiled from its own sources into oracle/_ref/) and the golden
 * fixtures under tests/golden/.
 *
 * Real double precision (CT_DOUBLE_REAL) only.
 */
#ifndef CT_ORACLE_H
#define CT_ORACLE_H

#include "ct_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* dmrg_twosite (src/algorithm/dmrg.c:262-399); same arguments and return codes */
int oracle_dmrg_twosite(const struct mpo* hamiltonian, int num_sweeps, int maxiter_lanczos, double tol_split,
	ct_long max_vdim, struct mps* psi, double* en_sweeps, double* entropy);

/* dmrg_singlesite (src/algorithm/dmrg.c:155-254); same arguments and return codes */
int oracle_dmrg_singlesite(const struct mpo* hamiltonian, int num_sweeps, int maxiter_lanczos, struct mps* psi,
	double* en_sweeps);

/* apply_local_hamiltonian (src/algorithm/chain_ops.c:353-390): b = H_loc a, b allocated here */
void oracle_apply_local_hamiltonian(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
	const struct block_sparse_tensor* l, const struct block_sparse_tensor* r, struct block_sparse_tensor* b);

/* block_sparse_tensor_dot (src/tensor/block_sparse_tensor.c:1826-2001); axrange 0 = leading, 1 = trailing */
void oracle_block_sparse_tensor_dot(const struct block_sparse_tensor* s, int axrange_s,
	const struct block_sparse_tensor* t, int axrange_t, int ndim_mult, struct block_sparse_tensor* r);

/* block_sparse_tensor_transpose (src/tensor/block_sparse_tensor.c:785-870) */
void oracle_block_sparse_tensor_transpose(const int* perm, const struct block_sparse_tensor* t, struct block_sparse_tensor* r);

/* block_sparse_tensor_svd (src/tensor/block_sparse_tensor.c:2686-2848); s has length returned in *ns,
 * allocated with aligned_alloc; returns 0 or -1 */
int oracle_block_sparse_tensor_svd(const struct block_sparse_tensor* a, struct block_sparse_tensor* u,
	double** s, ct_long* ns, struct block_sparse_tensor* vh);

/* block_sparse_tensor_qr / _rq (src/tensor/block_sparse_tensor.c:2402-2540 / :2544-2676), QR_REDUCED;
 * factors allocated here; return 0 or -1 */
int oracle_block_sparse_tensor_qr(const struct block_sparse_tensor* a, struct block_sparse_tensor* q,
	struct block_sparse_tensor* r);
int oracle_block_sparse_tensor_rq(const struct block_sparse_tensor* a, struct block_sparse_tensor* r,
	struct block_sparse_tensor* q);

/* contraction_operator_step_left / _right (src/algorithm/chain_ops.c:196-245 / :116-165) */
void oracle_contraction_operator_step_left(const struct block_sparse_tensor* a, const struct block_sparse_tensor* b,
	const struct block_sparse_tensor* w, const struct block_sparse_tensor* l, struct block_sparse_tensor* l_next);
void oracle_contraction_operator_step_right(const struct block_sparse_tensor* a, const struct block_sparse_tensor* b,
	const struct block_sparse_tensor* w, const struct block_sparse_tensor* r, struct block_sparse_tensor* r_next);

/* mps_vdot (src/state/mps.c:314), real case: <chi|psi> */
double oracle_mps_vdot(const struct mps* chi, const struct mps* psi);

/* retained_bond_indices (src/algorithm/truncation.c:110-223); ind must hold n entries;
 * returns the number retained and fills norm / entropy / tol_eff */
ct_long oracle_retained_bond_indices(const double* sigma, ct_long n, double tol, int relative_thresh, ct_long max_vdim,
	ct_long* ind, double* norm_sigma, double* entropy, double* tol_eff);

/* eigensystem_krylov_symmetric with an explicit dense symmetric matrix as the linear map
 * (src/util/krylov.c:24-89, :172-251); for pinning the Lanczos restatement */
int oracle_lanczos_dense(ct_long n, const double* h, const double* vstart, int maxiter,
	double* lambda, double* u_ritz);

/* release a tensor allocated by any oracle routine (free() on every array) */
void oracle_delete_block_sparse_tensor(struct block_sparse_tensor* t);

/* wall time in seconds of every sweep of the last oracle_dmrg_twosite call; returns the count */
int oracle_get_sweep_times(double* out, int max);

/* retained singular values (in the order the truncation keeps them) of the most recent split at
 * bond `bond` (sites bond, bond+1) during the last oracle_dmrg_twosite call; fills up to max
 * entries and returns the count, or -1 if that bond was never split */
ct_long oracle_get_bond_sigma(int bond, double* out, ct_long max);

/* construct_random_mps (src/state/mps.c:93-175) after seed_rng_state(rng_seed) (src/util/rng.c:15-27),
 * real double precision; returns 0, or -1 on invalid arguments */
int oracle_construct_random_mps(int nsites, ct_long d, const qnumber* qsite, qnumber qnum_sector, ct_long max_vdim,
	uint64_t rng_seed, struct mps* mps);

/* number of OpenMP threads the oracle runs with (set via OMP_NUM_THREADS or this call) */
int oracle_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
