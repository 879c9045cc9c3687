// ctg_kernels.h - device work descriptors and launchers for the block-sparse engine.
//
// A block-sparse operation is lowered on the host (integer arithmetic only) into
// flat descriptor arrays; the kernels below consume them. One launch covers all
// dense blocks of one tensor operation.
#pragma once

#include "ctg_common.h"

namespace ctg {

// ---- grouped block GEMM ----------------------------------------------------
// Output block: C[m x n] (row-major, leading dimension n) at c_off in the output
// buffer equals the sum over its contributions of op(A) op(B), where A element
// (i, kk) lives at a_off + i*sAm + kk*sAk and B element (kk, j) at
// b_off + kk*sBk + j*sBn. Outputs with no contribution are written as zeros.
struct GemmOut {
	i64 c_off;
	int m, n;
	int c0, nc;        // contribution range in the contribution array
	// where element (i, j) of the block goes: c_off + (i / r1) sr0 + (i % r1) sr1 + (j / c1) sc0 +
	// (j % c1); the plain row-major block is r1 = m, sr1 = n, c1 = n (sr0, sc0 unused). Other values
	// write the block straight into the layout of a transposed result (two runs of row axes and two
	// of column axes rearranged, the last column run innermost), so that no transpose pass is needed.
	int r1, c1;
	i64 sr0, sr1, sc0;
};

__host__ __device__ inline i64 gemm_out_index(const GemmOut& o, int i, int j)
{
	return o.c_off + (i64)(i / o.r1) * o.sr0 + (i64)(i % o.r1) * o.sr1 + (i64)(j / o.c1) * o.sc0 + (j % o.c1);
}

struct GemmContrib {
	i64 a_off, b_off;
	int k;
	int sAm, sAk, sBk, sBn;
};

// One CTA's share of an output tile: the terms from (contribution c0, k = k0) up to (contribution c1,
// k = k1 exclusive) of the tile's sum over its contributions and their inner index k, in order.
// split < 0: the share is the whole sum and goes to C; otherwise the CTA is share sp of GemmSplit
// entry `split`: it writes its partial sum to work[part + sp * stride + i * ld + j], and the CTA
// that finishes its split last adds the partial sums in order of sp and writes C.
struct GemmTile {
	int out;           // output block
	int m0, n0;        // tile origin inside the output block
	int c0, k0;
	int c1, k1;        // c1 < c0: no terms (the tile is written as zeros)
	int cls;           // tile class (shape), see TILE_*
	int split, sp;
};

// A tile whose sum is split over nsplit CTAs: C = sum over p < nsplit of the partial tile at
// work[part + p * stride] (rows x cols used, leading dimension ld), added in order of p.
struct GemmSplit {
	int out, m0, n0, rows, cols, nsplit, ld, stride;
	i64 part;
};

// tile classes (rows x cols of C per CTA of 256 threads): 256 outputs, one per thread (S 16 x 16,
// R8 8 x 32, R4 4 x 64, C8 32 x 8, C4 64 x 4); 1024 outputs, four per thread (M 32 x 32, W 16 x 64,
// T 64 x 16, W8 8 x 128, T8 128 x 8); L 64 x 64, sixteen per thread. Block-sparse DMRG outputs are
// mostly small and skinny, and FP64 FMAs spent on tile padding cost as much as useful ones.
enum {
	TILE_S = 0, TILE_M, TILE_L, TILE_W, TILE_T, TILE_R8, TILE_R4, TILE_C8, TILE_C4, TILE_W8, TILE_T8,
	NUM_TILE_CLASSES
};
constexpr int TILE_ROWS[NUM_TILE_CLASSES] = {16, 32, 64, 16, 64, 8, 4, 32, 64, 8, 128};
constexpr int TILE_COLS[NUM_TILE_CLASSES] = {16, 32, 64, 64, 16, 32, 64, 8, 4, 128, 8};
int tile_rows(int cls);
int tile_cols(int cls);

// every tile of every class in one launch (256 threads per CTA, the tile's class picks its shape);
// split tiles use `counters` (one per GemmSplit, zero before the launch and again after it)
void launch_gemm_f64(int ntiles, const GemmTile* tiles, const GemmOut* outs, const GemmContrib* cons,
                     const GemmSplit* splits, int* counters, const double* A, const double* B, double* C, double* work,
                     cudaStream_t st, double flops = 0.0);

// Same work lists on the tcgen05 tensor cores with FP32 accumulation, output tiles of
// tc_tile_rows() x BN (BN = 64, 128 or 256, chosen per product). Operand formats (TcFormat):
//   TC_BF16X3  x = hi + lo (BF16 parts), products hi.hi + hi.lo + lo.hi: about 2^-16 relative
//   TC_BF16X6  x = hi + mid + lo (BF16 parts of FP32 x), products hh hm mh hl mm lh: about 2^-23
//   TC_TF32    x rounded to TF32, one product (kind::tf32): about 2^-11
//
// Operands are packed first: every operand block is cut into K-major records of 128 (A) or 64 (B)
// rows by one 64-byte k chunk (32 BF16 or 16 TF32 elements), each record holding its parts back to
// back, each part in the canonical no-swizzle core-matrix layout of the tcgen05 shared-memory
// descriptors; zero outside the block. B blocks get a multiple of BN / 64 row records. A record
// moves into shared memory with bulk copies (cp.async.bulk). *error becomes 1 if a bounded wait
// inside the GEMM ran out (set_tc_wait_limit sets the number of polls; 0 restores the default).
enum TcFormat { TC_BF16X3 = 0, TC_BF16X6 = 1, TC_TF32 = 2 };
int tc_tile_rows();
int tc_parts(int fmt);
int tc_k_chunk(int fmt);            // elements of k per record
constexpr int TC_A_ROWS = 128, TC_B_ROWS = 64, TC_KB = 64;
i64 tc_a_rec_bytes(int fmt);
i64 tc_b_rec_bytes(int fmt);
void set_tc_wait_limit(long long polls);
struct TcPack {
	i64 src;           // element offset of (row 0, k 0) of the block in the operand
	int rows, k;       // block extent
	int s_row, s_k;    // element strides of rows and k
	int row0, k0;      // tile origin
	i64 rec;           // destination record
};
struct TcContrib {
	i64 a_rec, b_rec;  // first record of the A block (tiles mt * kt + j) and of the B block (nt64 * kt + j)
	int kt;            // k chunks
	int pad;
};
// a_side: records of TC_A_ROWS rows (A operand), else TC_B_ROWS (B operand); src_f32: the operand
// holds FP32 entries (an intermediate written by a reduced-precision product), else FP64
void launch_tc_pack(int fmt, int nrec, const TcPack* packs, int a_side, const void* src, bool src_f32, void* dst,
                    cudaStream_t st);
// out_f32: C receives FP32 entries, else FP64
void launch_gemm_tc(int fmt, int bn, int ntiles, const GemmTile* tiles, const GemmOut* outs, const TcContrib* tcons,
                    const void* apack, const void* bpack, void* C, bool out_f32, int* error, cudaStream_t st);

// ---- data movement -----------------------------------------------------------
// Generic per-block permutation: dst block (row-major over dims) gathers
// src[src_off + sum_i idx_i * sstr_i].
struct PermDesc {
	i64 src_off, dst_off, n;
	int ndim;
	int dims[6];
	i64 sstr[6];
};

// Row map: for lead < nlead, j < nrow, t < ntrail:
//   gather  (scatter == 0): dst[(lead*dst_rows + j)*ntrail + t]        = src[(lead*src_rows + map[j])*ntrail + t]
//   scatter (scatter == 1): dst[(lead*dst_rows + map[j])*ntrail + t]   = src[(lead*src_rows + j)*ntrail + t]
struct RowDesc {
	i64 src_off, dst_off;
	i64 nlead, ntrail;
	int nrow, src_rows, dst_rows, scatter;
	i64 map_off;
};

// Chunk of work for the copy kernels: descriptor index and first element.
struct Chunk {
	int desc;
	int pad;
	i64 start;
};

constexpr int COPY_CHUNK = 4096;

// cplx: entries are complex128 (two doubles each); descriptors count entries
void launch_permute(int nchunks, const Chunk* chunks, const PermDesc* descs, const double* src, double* dst, cudaStream_t st,
                    bool cplx = false);
void launch_rowmap(int nchunks, const Chunk* chunks, const RowDesc* descs, const i64* maps, const double* src, double* dst,
                   cudaStream_t st, bool cplx = false);

// Multiply entries along one axis of each block by vec[map[position]]:
// entry (lead, p, trail) of a block of shape (nlead, nax, ntrail) is scaled by vec[map[map_off + p]].
struct ScaleDesc {
	i64 off, nlead, ntrail;
	int nax, pad;
	i64 map_off;
};
void launch_scale_axis(int nchunks, const Chunk* chunks, const ScaleDesc* descs, const i64* maps, const double* vec,
                       const double* src, double* dst, cudaStream_t st, bool cplx = false);

// ---- dense linear algebra per block ---------------------------------------------
// SVD of a row-major m x n block: u (m x k), s (k), vh (k x n), k = min(m, n), singular values
// in descending order; one thread-block cluster per block. Entries of u, s and vh beyond the
// numerical rank are not written (the caller zeroes them). status[0] becomes -1 if a block does
// not converge within SVD_MAX_SWEEPS FP64 Jacobi sweeps, status[1] receives the largest sweep
// count; flops[0] (zeroed by the caller) accumulates the FP64 flops executed by the Jacobi inner
// products and rotations of the shared-memory path.
constexpr int SVD_MAX_SWEEPS = 60;
// per-block diagnostics of the SVD kernel (CTGPU_SVD_PHASES): [0] start, [1] after the QR, [2] after
// the Jacobi sweeps, [3] end (global timer, ns); on the critical CTA: [4] SM cycles of the FP64
// steps (inner products, rotation parameters, rotations), [5] FP64 sweeps, [6] FP32 sweeps, SM
// cycles of [7] exchanges, [8] FP32 sweeps, [9] FP32 to FP64 hand-over (Newton-Schulz steps and
// T = R^T V); SM cycles of the distributed QR's steps in [10] pivot candidates, [11] candidate
// reflectors, [12] candidate exchange and cluster barrier, [13] pivot reflector fetch, [14] updates;
// [15] refinement iterations of the mixed path (plus 100 when it handed over to FP64 sweeps), SM
// cycles of the refinement's [16] Gram matrices, [17] analysis (cosines, tail, clusters, generator),
// [18] updates, [19] cluster rotations. With the refinement, [4] holds its SM cycles and [9] those
// of the Newton-Schulz steps and T = R^T V.
constexpr int SVD_PHASE_SLOTS = 22;
struct SvdDesc {
	i64 a_off, u_off, s_off, v_off, w_off;
	int m, n;
};
i64 svd_scratch_doubles(int m, int n);

// Launch configuration of one block's SVD: cluster size, dynamic shared memory, and whether the
// Jacobi columns live in global memory (blocks too large for the shared-memory path).
struct SvdLaunch {
	int cluster = 1;
	int smem = 0;
	int global = 0;
};
// largest cluster the device schedules for the SVD kernel (16 where non-portable sizes work, else 8)
int svd_max_cluster(int device);
// smallest configuration with at least 'want' CTAs (a power of two) that fits an m x n block
SvdLaunch svd_launch_for(int m, int n, int want, int max_cluster);
// SVDs of descs[first .. first + count), all with configuration g, on stream st. With phase_ts
// non-null (shared-memory path only), the first CTA of each block's cluster writes four
// %globaltimer stamps (start, QR done, Jacobi done, outputs done) to phase_ts[8 block ..] and
// its SM clock cycles spent in the Jacobi inner products, rotation parameters, rotations and
// cluster exchanges to phase_ts[8 block + 4 ..].
// discard2: the caller discards every singular value whose square is below it (0: none); the
// refinement of the mixed path then leaves the mutual rotations of those columns out.
void launch_svd_group(const SvdLaunch& g, int first, int count, const SvdDesc* descs, const double* a, double* u,
                      double* s, double* vh, double* scratch, int* status, double* flops, cudaStream_t st,
                      unsigned long long* phase_ts = nullptr, double discard2 = 0.0);

// Householder RQ of a row-major m x n block: A = R Q with Q (k x n) orthonormal rows, R (m x k), k = min(m, n).
// Scratch holds n*m + n*k + k doubles per block.
struct RqDesc {
	i64 a_off, r_off, q_off, w_off;   // w_off: scratch of m n + max(m, n) min(m, n) + min(m, n) doubles
	int m, n;
	int qr;                           // 1: A = Q R (dgeqrf convention), 0: A = R Q (dgerqf convention)
};
void launch_rq_householder(int nblocks, const RqDesc* descs, const double* a, double* r, double* q, double* scratch,
                           cudaStream_t st);

// ---- complex128 (interleaved real / imaginary parts, element offsets and strides) -------
// Tiles of the complex block GEMM: 32 x 32 of output block `out`, all of its contributions.
struct ZTile {
	int out, m0, n0, pad;
};
// C = sum op(A) op(B) over the same GemmOut / GemmContrib lists as the FP64 GEMM; conj_a / conj_b
// conjugate the operand's entries as they are read.
void launch_gemm_z(int ntiles, const ZTile* tiles, const GemmOut* outs, const GemmContrib* cons, const double* A,
                   const double* B, double* C, int conj_a, int conj_b, cudaStream_t st);
// complex SVD of each block (SvdDesc offsets in complex elements, s_off in doubles, w_off in
// complex elements of scratch); status[b] = 1 if block b did not converge
i64 svd_z_scratch(int m, int n);
void launch_svd_z(int nblocks, const SvdDesc* descs, const double* a, double* u, double* s, double* vh, double* work,
                  int* status, cudaStream_t st);
// complex QR / RQ of each block (RqDesc offsets in complex elements; scratch of
// m n + max(m, n) min(m, n) + min(m, n) complex elements per block)
void launch_qr_z(int nblocks, const RqDesc* descs, const double* a, double* r, double* q, double* scratch, cudaStream_t st);

// ---- Lanczos (krylov.c:24-89) ------------------------------------------------------
// Device-resident scalars of one Lanczos run.
constexpr int LANCZOS_MAX = 32;     // largest maxiter_lanczos accepted

struct LanczosScalars {
	double alpha[LANCZOS_MAX];
	double beta[LANCZOS_MAX];
	double y[LANCZOS_MAX];  // Ritz coefficients of the lowest eigenpair
	double lambda;         // lowest Ritz value
	double nrm0;           // norm of the start vector
	int numiter;
	int stopped;
	int status;            // 0 ok, -1 fewer iterations than eigenvalues, -2 tridiagonal solver failure
	int pad;
};

// fixed grid of the cooperative Lanczos kernels (deterministic reductions): one block of 512 threads
// per SM, so that each grid barrier has 152 participants and each block sums 152 partials
constexpr int RED_BLOCKS = 152;
// shared scratch (doubles) of the one-warp tridiagonal eigensolver
constexpr int TRIDIAG_SCRATCH = 9 * LANCZOS_MAX;
// vectors of up to this many doubles take the cluster form of the Lanczos kernels (one
// thread-block cluster, cluster barriers) instead of the cooperative grid form
constexpr i64 LZ_CLUSTER_MAX_N = (i64)1 << 19;

// one cooperative launch each (partial: 2 RED_BLOCKS doubles): a whole Lanczos step
// (alpha; unless last: orthogonalisation, beta and the early exit, next vector), and the start
// vector's normalisation (a start vector of norm zero sets status -1 and stops the iteration)
// n doubles per vector (a complex128 vector counts twice); the breakdown test beta < 100 nthr eps
// uses nthr, the number of entries (krylov.c:62, :129)
void launch_lz_step(double* w, const double* vj, const double* vjm1, double* vj1, i64 n, i64 nthr, int j, int last,
                    double* partial, LanczosScalars* sc, cudaStream_t st);
void launch_lz_start(const double* v0, double* v, i64 n, double* partial, LanczosScalars* sc, cudaStream_t st);
// the last step (alpha_{maxiter-1}, unless the iteration stopped early), the lowest eigenpair of the
// tridiagonal Lanczos matrix and the Ritz vector out = V y, in one cooperative launch
void launch_lz_finish(const double* w, const double* V, i64 n, int maxiter, double* partial, LanczosScalars* sc,
                      double* out, cudaStream_t st);
// the tridiagonal eigensolver of launch_lz_finish alone (one warp, k <= LANCZOS_MAX): d_out receives
// lambda, the status and y[0..k-1]
void tridiag_lowest_test(const double* d_alpha, const double* d_beta, int k, double* d_out, cudaStream_t st);

// Sustained FP64 FMA rate of the device in TFLOP/s (register-resident FMA chains).
double measure_fp64_fma_tflops(int device);

}  // namespace ctg
