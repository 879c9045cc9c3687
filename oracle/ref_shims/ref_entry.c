/* Flat entry points around the chemtensor reference, compiled together with
 * the reference sources into oracle/_ref/libct_ref.so (this container only).
 * They let the golden-fixture script build the reference's own inputs
 * (Hamiltonian MPOs from the reference's assembly code, seeded random MPS)
 * and run its dmrg_twosite through ctypes. Test infrastructure only. */
#include <stdlib.h>
#include <string.h>
#include "mps.h"
#include "mpo.h"
#include "hamiltonian.h"
#include "dmrg.h"
#include "chain_ops.h"
#include "rng.h"
#include "aligned_memory.h"

/* construct_heisenberg_xxz_1d_mpo_assembly (src/operator/hamiltonian.c:102) + mpo_from_assembly */
void ref_heisenberg_mpo(int nsites, double J, double D, double h, struct mpo* out)
{
	struct mpo_assembly assembly;
	construct_heisenberg_xxz_1d_mpo_assembly(nsites, J, D, h, &assembly);
	mpo_from_assembly(&assembly, out);
	delete_mpo_assembly(&assembly);
}

/* construct_fermi_hubbard_1d_mpo_assembly (src/operator/hamiltonian.c:240) + mpo_from_assembly */
void ref_hubbard_mpo(int nsites, double t, double u, double mu, struct mpo* out)
{
	struct mpo_assembly assembly;
	construct_fermi_hubbard_1d_mpo_assembly(nsites, t, u, mu, &assembly);
	mpo_from_assembly(&assembly, out);
	delete_mpo_assembly(&assembly);
}

/* construct_spin_molecular_hamiltonian_mpo_assembly (src/operator/hamiltonian.c:2768) + mpo_from_assembly;
 * tkin is n x n and vint n x n x n x n, row-major float64 */
void ref_spin_molecular_mpo(int n, const double* tkin, const double* vint, int optimize, struct mpo* out)
{
	struct dense_tensor tk, vi;
	const ct_long dt[2] = { n, n };
	const ct_long dv[4] = { n, n, n, n };
	allocate_dense_tensor(CT_DOUBLE_REAL, 2, dt, &tk);
	allocate_dense_tensor(CT_DOUBLE_REAL, 4, dv, &vi);
	memcpy(tk.data, tkin, sizeof(double) * n * n);
	memcpy(vi.data, vint, sizeof(double) * n * n * n * n);
	struct mpo_assembly assembly;
	construct_spin_molecular_hamiltonian_mpo_assembly(&tk, &vi, optimize != 0, &assembly);
	mpo_from_assembly(&assembly, out);
	delete_mpo_assembly(&assembly);
	delete_dense_tensor(&vi);
	delete_dense_tensor(&tk);
}

/* seed_rng_state + construct_random_mps (src/state/mps.c:93), as the Python binding does it */
void ref_random_mps(int dtype, int nsites, ct_long d, const qnumber* qsite, qnumber qnum_sector,
	ct_long max_vdim, uint64_t seed, struct mps* out)
{
	struct rng_state rng;
	seed_rng_state(seed, &rng);
	construct_random_mps((enum numeric_type)dtype, nsites, d, qsite, qnum_sector, max_vdim, &rng, out);
}

/* first 'n' standard normal draws of a freshly seeded generator (RNG restatement check) */
void ref_randn_sequence(uint64_t seed, int n, double* out)
{
	struct rng_state rng;
	seed_rng_state(seed, &rng);
	for (int i = 0; i < n; i++) {
		out[i] = randn(&rng);
	}
}

/* <chi|psi> for real MPS (src/state/mps.c:314) */
double ref_mps_vdot_real(const struct mps* chi, const struct mps* psi)
{
	double r = 0;
	mps_vdot(chi, psi, &r);
	return r;
}

/* single application of the local two-site Hamiltonian, with the reference's own
 * environment construction: used to pin the local-H apply on one bond */
void ref_local_hamiltonian_setup(const struct mpo* h, const struct mps* psi, int ibond,
	struct block_sparse_tensor* h2, struct block_sparse_tensor* lenv, struct block_sparse_tensor* renv, struct block_sparse_tensor* a2)
{
	const int nsites = h->nsites;
	struct block_sparse_tensor* lb = ct_malloc(nsites * sizeof(struct block_sparse_tensor));
	struct block_sparse_tensor* rb = ct_malloc(nsites * sizeof(struct block_sparse_tensor));
	compute_right_operator_blocks(psi, psi, h, rb);
	create_dummy_operator_block_left(&psi->a[0], &psi->a[0], &h->a[0], &lb[0]);
	for (int i = 0; i < ibond; i++) {
		contraction_operator_step_left(&psi->a[i], &psi->a[i], &h->a[i], &lb[i], &lb[i + 1]);
	}
	copy_block_sparse_tensor(&lb[ibond], lenv);
	copy_block_sparse_tensor(&rb[ibond + 1], renv);
	for (int i = 0; i <= ibond; i++) {
		delete_block_sparse_tensor(&lb[i]);
	}
	for (int i = 0; i < nsites; i++) {
		delete_block_sparse_tensor(&rb[i]);
	}
	ct_free(lb);
	ct_free(rb);
	mpo_merge_tensor_pair(&h->a[ibond], &h->a[ibond + 1], h2);
	mps_merge_tensor_pair(&psi->a[ibond], &psi->a[ibond + 1], a2);
}
