// ctg_dmrg.h - two-site DMRG on one GB300, MPS / MPO / environments resident in HBM.
#pragma once

#include "ct_structs.h"
#include "ctg_engine.h"

namespace ctg {

struct DmrgOptions {
	int device = 0;
	int precision = GEMM_FP64;   // GemmPrecision of the bulk local-H GEMMs
	int final_fp64_sweeps = 1;   // trailing sweeps forced to FP64 when precision != FP64
	bool reduced_env = false;    // environment updates of the reduced-precision sweeps in that precision too
	int verbose = 0;
	i64 l2_flush_bytes = 0;      // if > 0, overwrite a buffer of this size before every sweep
	int profile = 0;             // time every launch by kernel class (CUDA events)
	int profile_skip_sweeps = 0; // ... starting with this sweep
};

struct DmrgStats {
	double wall_s = 0;           // host wall time of the whole call
	double upload_s = 0;         // host structs -> HBM
	double download_s = 0;       // HBM -> host structs
	double setup_s = 0;          // right-normalisation, environments, merged MPO pairs
	double sweep_s = 0;          // all sweeps
	double lanczos_ms = 0;       // device time in the Lanczos eigensolver (CUDA events)
	double split_ms = 0;         // device+host time in the SVD split
	double env_ms = 0;           // device time in the environment updates (both directions)
	double matvec_flops = 0;     // algorithmic GEMM FLOPs of all local-H applications
	double total_gemm_flops = 0; // algorithmic GEMM FLOPs of everything
	long matvecs = 0;
	long kernel_launches = 0;
	int sweeps = 0;
	i64 max_bond_dim = 0;
	int svd_max_sweeps = 0;             // largest Jacobi sweep count of any block SVD
	double host_plan_s = 0;             // host time lowering operations into device work lists
	long plan_hits = 0, plan_misses = 0;
	double svd_flops = 0;               // FP64 flops of the block SVDs
	std::vector<double> sweep_ms;       // device time of every sweep (CUDA events on the stream)
	std::vector<long> sweep_launches;   // kernels launched by every sweep
	KProf prof[K_NUM_CLASSES];          // per kernel class, over the profiled sweeps
	// retained singular values of the most recent split at every bond (after the last sweep: those of
	// its right-to-left pass), in the order the truncation keeps them
	std::vector<std::vector<double>> bond_sigma;
	// splits whose bond-dimension cut fell between two singular values less than 1e-12 of the largest
	// apart (rounding alone could then change the kept set)
	long near_ties = 0;
};

// Same contract as dmrg_twosite (src/algorithm/dmrg.c:262-399).
int dmrg_twosite_gpu(const struct mpo* hamiltonian, int num_sweeps, int maxiter_lanczos, double tol_split, i64 max_vdim,
                     struct mps* psi, double* en_sweeps, double* entropy, const DmrgOptions& opt, DmrgStats* stats);

// Same contract as dmrg_singlesite (src/algorithm/dmrg.c:155-254): bond dimensions fixed by psi.
int dmrg_singlesite_gpu(const struct mpo* hamiltonian, int num_sweeps, int maxiter_lanczos, struct mps* psi,
                        double* en_sweeps, const DmrgOptions& opt, DmrgStats* stats);

// truncation rule of retained_bond_indices (src/algorithm/truncation.c:110-223)
struct TruncResult {
	std::vector<i64> ind;
	double norm_sigma = 0, entropy = 0, tol_eff = 0;
	// the cut at max_vdim separates two singular values less than 1e-12 of the largest apart
	bool near_tie = false;
};
TruncResult retained_bond_indices(const double* sigma, i64 n, double tol, bool relative_thresh, i64 max_vdim);

// environment updates with b = a (src/algorithm/chain_ops.c:196-245, :116-165)
DTensor contraction_step_left(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& l, int precision = GEMM_FP64);
DTensor contraction_step_right(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& r, int precision = GEMM_FP64);

// one application of the local two-site Hamiltonian (src/algorithm/chain_ops.c:353-390)
DTensor apply_local_hamiltonian_once(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& l, const DTensor& r,
                                     int precision);

// device time (ms, CUDA events) of nmatvec back-to-back applications of the local Hamiltonian
// after three untimed ones; *flops receives the algorithmic GEMM FLOPs of one application
double time_local_hamiltonian(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& l, const DTensor& r,
                              int precision, int nmatvec, double* flops);

// <chi|psi> of two MPS on the device (mps_vdot, src/state/mps.c:314-370); ret receives one double
// (real MPS) or two (complex: real and imaginary part)
void mps_vdot_gpu(const struct mps* chi, const struct mps* psi, int device, double* ret);

// <chi|op|psi> on the device (mpo_inner_product, src/algorithm/chain_ops.c:274-317); ret as above
void mpo_inner_product_gpu(const struct mps* chi, const struct mpo* op, const struct mps* psi, int device, double* ret);

// contraction_operator_step_right (src/algorithm/chain_ops.c:116-165) with ket a and bra b
DTensor contraction_step_right_ab(Ctx& c, const DTensor& a, const DTensor& b, const DTensor& w, const DTensor& r,
                                  int precision = GEMM_FP64);

// spin-orbital molecular Hamiltonian as an MPO (construct_spin_molecular_hamiltonian_mpo_assembly with
// optimize = false + mpo_from_assembly, src/operator/hamiltonian.c:2768-2979); tkin n x n and vint
// n x n x n x n row-major; out receives reference-layout tensors
int build_spin_molecular_mpo(int n, const double* tkin, const double* vint, struct mpo* out);

// host <-> device conversions of reference structs
Meta meta_from_struct(const struct block_sparse_tensor* t);
DTensor tensor_from_struct(Ctx& c, const struct block_sparse_tensor* t);
void tensor_to_struct(Ctx& c, const DTensor& t, struct block_sparse_tensor* out);
// allocate a reference-layout tensor (aligned_alloc) holding host entries in block order
void write_struct_host(const Meta& m, const double* host, struct block_sparse_tensor* out, bool cplx = false);
void free_struct(struct block_sparse_tensor* t);

}  // namespace ctg
