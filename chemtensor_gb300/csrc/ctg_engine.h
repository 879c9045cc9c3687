// ctg_engine.h - device-resident block-sparse tensors and their operations.
//
// A DTensor is a host-side Meta (block structure, integers only) plus one
// contiguous device buffer holding every dense block in row-major block
// order. Operations are lowered on the host into descriptor arrays ("plans")
// that are uploaded once and launched on the engine's stream; the host never
// touches tensor entries except at the C-ABI boundary and when it reads the
// singular values needed for the truncation decision.
#pragma once

#include <memory>

#include "ctg_kernels.h"
#include "ctg_meta.h"

namespace ctg {

class Ctx;

// kernel classes for profiling
enum KClass { K_GEMM = 0, K_PERMUTE, K_ROWMAP, K_SCALE, K_SVD, K_RQ, K_LANCZOS, K_GEMM_TC, K_NUM_CLASSES };
struct KProf {
	long launches = 0;
	double ms = 0;               // summed device time of the launches
	double flops = 0;            // algorithmic FLOPs (GEMM: sum of 2 m n k)
	double bytes = 0;            // algorithmic HBM bytes (copies: read + write of the entries moved)
};

// Counts (and, when profiling, times) the launches issued inside its scope.
struct KScope {
	Ctx& c;
	int cls, launches;
	double flops, bytes;
	KScope(Ctx& ctx, int cls_, int launches_, double flops_ = 0, double bytes_ = 0);
	~KScope();
};

// Stream-ordered device allocation, freed on the owning context's stream.
struct DBuf {
	Ctx* ctx = nullptr;
	void* ptr = nullptr;
	size_t bytes = 0;
	DBuf(Ctx* c, size_t n);
	~DBuf();
	DBuf(const DBuf&) = delete;
	DBuf& operator=(const DBuf&) = delete;
};
using DBufPtr = std::shared_ptr<DBuf>;

struct DTensor {
	std::shared_ptr<const Meta> meta;
	DBufPtr buf;
	bool cplx = false;      // complex128 entries (interleaved real and imaginary parts)
	bool conj = false;      // read as complex conjugate (a view; only dots honour it)
	double* data() const { return buf ? (double*)buf->ptr : nullptr; }
	const Meta& m() const { return *meta; }
	int width() const { return cplx ? 2 : 1; }    // doubles per entry
};

// Execution context: one CUDA stream, a private memory pool and a pinned staging
// arena for descriptor uploads. All work of one DMRG call runs on this stream.
class Ctx {
public:
	explicit Ctx(int device);
	~Ctx();
	cudaStream_t stream() const { return st_; }
	int device() const { return dev_; }
	// auxiliary streams for independent launches: fork(n) makes aux(0..n-1) wait for the work
	// queued so far on stream(); join(n) makes stream() wait for everything queued on them
	static constexpr int NUM_AUX = 8;
	cudaStream_t aux(int i);
	void fork(int n);
	void join(int n);
	void* alloc(size_t bytes);
	void free(void* p);
	// make the private pool hold at least this many bytes, so that later allocations are served
	// without growing it (growing maps new physical memory, which costs milliseconds)
	void reserve(size_t bytes);
	// copy host bytes to a new device buffer (through pinned staging, asynchronous)
	DBufPtr upload(const void* host, size_t bytes);
	// block until the stream is idle; recycles the staging arena
	void sync();
	DTensor empty(const Meta& m, bool cplx = false);
	DTensor empty(const std::shared_ptr<const Meta>& m, bool cplx = false);   // shares the structure, no copy
	DTensor zeros(const Meta& m, bool cplx = false);
	// statistics
	double gemm_flops = 0;       // algorithmic GEMM FLOPs issued
	long kernel_launches = 0;
	int svd_max_sweeps = 0;      // largest Jacobi sweep count of any block SVD
	double svd_flops = 0;        // FP64 flops of the block SVDs (Jacobi executed, QR and outputs estimated)
	int svd_full_reruns = 0;     // SVDs repeated at full resolution for the truncation decision
	double host_plan_s = 0;      // host time spent lowering operations into descriptor lists
	double host_alloc_s = 0, host_upload_s = 0;   // host time in device allocation / descriptor uploads
	double host_plan_cpu_s = 0;                   // thread CPU time of the planning
	long plan_hits = 0, plan_misses = 0;
	// with CTGPU_SVD_PHASES set: summed QR / Jacobi / output / launch time (ms) of the block that
	// finished last in each block SVD
	double svd_phase_ms[4] = {0, 0, 0, 0};
	double svd_qr_cycles[5] = {0, 0, 0, 0, 0};     // distributed QR: candidates, reflectors, exchange, fetch, updates
	double svd_jacobi_cycles[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // FP64 step cycles, FP64 sweeps, FP32 sweeps, exchange / FP32 / hand-over / FP32 exchange / T = R^T V cycles
	// cache of lowered operations, keyed by operation and operand structures (DMRG revisits the
	// same block structures every sweep once the bond dimensions have settled)
	struct PlanCache* plans() { return plans_; }
	void clear_plans();
	// device flag raised by a tensor-core kernel whose bounded wait timed out (checked at sync)
	int* tc_error();
	int num_sms() const { return sms_; }
	// pinned host memory for small device-to-host results read after a synchronisation
	int* svd_status_host() { return (int*)pinned_; }
	LanczosScalars* lanczos_host() { return (LanczosScalars*)((char*)pinned_ + 256); }
	double* svd_flops_host() { return (double*)((char*)pinned_ + 2048); }
	// n doubles of pinned host memory (contents valid until the next call); only call while no
	// asynchronous copy into it is pending
	double* pinned_doubles(size_t n);
	// optional per-kernel-class timing with CUDA events on this stream (resolved at sync points)
	bool profile = false;
	KProf prof[K_NUM_CLASSES];
	void prof_begin();
	void prof_end(int cls, int launches, double flops, double bytes);
	void prof_resolve();
	void prof_reset();

private:
	struct Pending { int cls, launches; cudaEvent_t e0, e1; double flops, bytes; };
	std::vector<Pending> pending_;
	std::vector<cudaEvent_t> event_pool_;
	cudaEvent_t open_ = nullptr;
	cudaEvent_t get_event();
	int dev_;
	int sms_ = 1;
	int* tc_error_ = nullptr;
	bool tc_used_ = false;
	struct PlanCache* plans_ = nullptr;
	cudaStream_t st_ = nullptr;
	cudaStream_t aux_[NUM_AUX] = {};
	cudaEvent_t fork_ev_ = nullptr;
	cudaEvent_t join_ev_[NUM_AUX] = {};
	cudaMemPool_t pool_ = nullptr;
	char* staging_ = nullptr;
	void* pinned_ = nullptr;                 // status words and Lanczos scalars
	double* pinned_d_ = nullptr;
	size_t pinned_d_cap_ = 0;
	size_t staging_cap_ = 0, staging_used_ = 0;
	size_t reserved_ = 0;
};

// Adds the host time of its scope to Ctx::host_plan_s.
struct PlanTimer {
	Ctx& c;
	double t0, cpu0;
	explicit PlanTimer(Ctx& ctx);
	~PlanTimer();
};

// Per-thread execution context for a device, created on first use and kept for the
// life of the thread, so that repeated calls reuse the stream, pool and staging arena.
Ctx& context_for_device(int device);

// ---- plans ------------------------------------------------------------------------

struct DotPlan {
	std::shared_ptr<const Meta> out;
	DBufPtr desc;
	int ntiles[NUM_TILE_CLASSES] = {};
	const GemmTile* tiles[NUM_TILE_CLASSES] = {};
	const GemmOut* outs = nullptr;
	const GemmContrib* cons = nullptr;
	const GemmSplit* splits = nullptr;   // tiles whose sum is split over several CTAs
	int nsplits = 0;
	DBufPtr work;                        // their partial sums
	DBufPtr counters;                    // their completion counters (one int per split tile)
	i64 a_entries = 0, b_entries = 0;    // entries of the two operand tensors
	// tensor-core path: packed operand records (see launch_tc_pack) and per-contribution records
	const TcContrib* tcons = nullptr;
	const TcPack* apacks = nullptr;
	const TcPack* bpacks = nullptr;
	i64 a_recs = 0, b_recs = 0;
	int tc_fmt = TC_BF16X3;              // operand format (TcFormat)
	int tc_bn = 64;                      // tile columns, from the tile autotuner
	double flops = 0;
	double flops_cls[NUM_TILE_CLASSES] = {};
	int precision = GEMM_FP64;
	// complex128 (precision GEMM_Z64): tiles of the complex GEMM
	int nztiles = 0;
	const ZTile* ztiles = nullptr;
	void run(Ctx& c, const double* A, const double* B, double* C) const;
	// complex128 entries, operands optionally read conjugated
	void run_z(Ctx& c, const double* A, const double* B, double* C, bool conj_a, bool conj_b) const;
	// tensor-core path in parts, so that an operand used by many runs is packed once; src_f32: the
	// operand holds FP32 entries (the output of another reduced-precision product)
	i64 a_rec_bytes() const { return a_recs * tc_a_rec_bytes(tc_fmt); }
	i64 b_rec_bytes() const { return b_recs * tc_b_rec_bytes(tc_fmt); }
	void pack_a(Ctx& c, const void* A, void* apack, bool src_f32 = false) const;
	void pack_b(Ctx& c, const void* B, void* bpack, bool src_f32 = false) const;
	// out_f32: C receives FP32 entries
	void run_packed(Ctx& c, const void* apack, const void* bpack, void* C, bool out_f32 = false) const;
};
// out_perm (every precision): the result is written straight in the layout of its transpose by out_perm
// (see lower_dot), and the plan's `out` is that transposed structure
DotPlan make_dot_plan(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision = GEMM_FP64,
                      const int* out_perm = nullptr);

// Tile autotuner of the reduced-precision GEMMs: the column width (64, 128 or 256) of a product's
// tensor-core tiles, or FP64 (0) where the product is too small for the tensor cores to pay for the
// operand packing, keyed by a histogram of its work list (flop shares of the output blocks by column
// extent and by summed contracted extent, the precision and the total work). On first sight of a key
// the three widths and the FP64 GEMM are timed on the product's own work lists (CUDA events, zero
// operands) and the fastest is kept, in memory and appended to a text file (CTGPU_TUNE_FILE, default
// tile_tuning.txt beside the library), which later processes read back. CTGPU_TC_BN=64|128|256
// forces a width.
struct TuneEntry {
	std::string key;
	int bn = 64;                         // 64, 128, 256, or 0 for FP64
	double ms[4] = {0, 0, 0, 0};         // timed widths 64, 128, 256 (B packing + GEMM) and FP64
	bool from_file = false;
};
std::vector<TuneEntry> tile_tuning_entries();
// use this width for every product planned from now on (0: the autotuner decides); plans already in a
// context's cache keep theirs
void force_tc_tile_width(int bn);

struct CopyPlan {
	std::shared_ptr<const Meta> out;
	DBufPtr desc;
	int kind = 0;                // 0 permute, 1 rowmap
	int nchunks = 0;
	const Chunk* chunks = nullptr;
	const void* descs = nullptr;
	const i64* maps = nullptr;
	i64 elements = 0;            // entries moved
	void run(Ctx& c, const double* src, double* dst, bool cplx = false) const;
};
CopyPlan make_transpose_plan(Ctx& c, const Meta& t, const int* perm);
CopyPlan make_flatten_plan(Ctx& c, const Meta& t, int ax, int newdir);
CopyPlan make_split_plan(Ctx& c, const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq);
CopyPlan make_slice_plan(Ctx& c, const Meta& t, int ax, const std::vector<i64>& ind);

// ---- one-shot operations (plan + run) ------------------------------------------------

DTensor op_dot(Ctx& c, const DTensor& s, int axs, const DTensor& t, int axt, int nmult, int precision = GEMM_FP64);
DTensor op_transpose(Ctx& c, const DTensor& t, const int* perm);
DTensor op_flatten(Ctx& c, const DTensor& t, int ax, int newdir);
DTensor op_split(Ctx& c, const DTensor& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq);
DTensor op_slice(Ctx& c, const DTensor& t, int ax, const std::vector<i64>& ind);
// multiply along the leading (axrange 0) or trailing (1) axis by a device vector indexed by logical position
DTensor op_scale_axis(Ctx& c, const DTensor& s, const double* dvec, int axrange);
// same entries, all axis directions reversed (structure cached per context)
DTensor view_reversed(Ctx& c, const DTensor& t);
// cyclic partial trace of one leading with one trailing axis of logical dimension 1 (a relabelling)
DTensor view_trace_unit(const DTensor& t);

// block SVD (block_sparse_tensor_svd, block_sparse_tensor.c:2686-2848); singular values in a
// device buffer indexed like the logical intermediate axis.
struct SvdResult {
	DTensor u, vh;
	DBufPtr s;
	i64 ns = 0;
};
// what op_svd_finish needs to check a launched SVD
struct SvdPending {
	std::vector<SvdDesc> descs;
	size_t launches = 0;
	DTensor a;
	double other_flops = 0;      // QR and output flops (host estimate at full rank)
	DBufPtr zstatus;             // complex128: per-block convergence status
	int zblocks = 0;
};
// enqueue the SVD without waiting for it; its status reaches pinned host memory when the stream
// gets there, so op_svd_finish may run only after a synchronisation of c's stream
// discard_weight: the caller discards singular values from the smallest up while their squares sum
// to at most this (the relative truncation of the two-site split times a lower bound of ||a||_F^2;
// 0: the full SVD is needed). Every value whose square is below discard_weight / (2 k), k the total
// number of singular values, is then certainly discarded, and the block SVD may leave the mutual
// rotations of such columns out.
int op_svd_launch(Ctx& c, const DTensor& a, SvdResult& res, SvdPending& pend, double discard_weight = 0.0);
// 0, or -1 if a block did not converge (diagnostics on stderr)
int op_svd_finish(Ctx& c, const SvdPending& pend);
// launch, synchronise, finish. Returns 0 or -1.
int op_svd(Ctx& c, const DTensor& a, SvdResult& res);
// host-side fault injection for tests of the error paths (per thread): the next n block SVDs report
// non-convergence, the next n Lanczos tridiagonal eigensolves report failure, the next n local
// eigenproblems start from a vector the host has zeroed
extern thread_local int g_inject_svd_failure;
extern thread_local int g_inject_tridiag_failure;
extern thread_local int g_inject_zero_start;

// block RQ (block_sparse_tensor_rq, block_sparse_tensor.c:2544-2676). Returns 0 or -1.
int op_rq(Ctx& c, const DTensor& a, DTensor& r, DTensor& q);
// block QR (block_sparse_tensor_qr, block_sparse_tensor.c:2402-2540). Returns 0 or -1.
int op_qr(Ctx& c, const DTensor& a, DTensor& q, DTensor& r);

// host <-> device entry copies (asynchronous on the context stream; host memory must stay valid)
void copy_to_device(Ctx& c, DTensor& t, const double* host);
void copy_to_host(Ctx& c, const DTensor& t, double* host);

}  // namespace ctg
