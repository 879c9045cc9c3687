// ctg_svd.cu - block SVD: QR with column pivoting, then one-sided Jacobi on R^T, on
// thread-block clusters.
//
// Replaces LAPACK dgesvd in dense_tensor_svd_fill (dense_tensor.c:3538-3680), which
// block_sparse_tensor_svd (block_sparse_tensor.c:2686-2848) calls once per
// quantum-number block. FP64 results. Singular values agree with dgesvd to rounding
// (dgesvd resolves them to ~eps sigma_max absolute, this method to ~(m + n) eps sigma_max);
// singular vectors up to sign / rotation within degenerate subspaces.
//
// Method (Drmac & Veselic, "New fast and accurate Jacobi SVD algorithm", SIAM J. Matrix
// Anal. Appl. 29 (2008), the scheme behind LAPACK dgejsv), with B the block oriented so
// that it has at least as many rows as columns:
//   1. Householder QR with column pivoting, B P = Q R, stopped at the numerical rank r
//      (largest remaining column norm below eps ||B||_F);
//   2. one-sided Jacobi on R^T (N x r): R^T V = T with orthogonal columns, sigma = ||T_c||;
//      on the pivoted, graded R^T this takes about half the sweeps that Jacobi on B needs
//      for the graded spectra of two-site DMRG matrices;
//   3. B = (Q V) Sigma (P T Sigma^-1)^T.
// On GB300 an SM retires about two FP64 FMAs per clock and every FP64 warp instruction
// occupies its SM sub-partition for 64 cycles whatever the number of active lanes, so each
// dense block gets a cluster of up to 16 CTAs sized to its share of the work: the pivoted QR
// runs on one CTA, the Jacobi sweeps on the whole cluster with the columns in shared memory
// (k_svd_tour), the outputs on the whole cluster. Blocks too large for shared memory keep
// their columns in global memory (k_svd_global: one cluster barrier per round of disjoint
// pairs, L2-coherent loads).
#include <cfloat>
#include <cstdio>
#include <mutex>
#include <stdexcept>

#include <cooperative_groups.h>

#include "ctg_fp64.cuh"
#include "ctg_kernels.h"
#include "ctg_svd_schedule.h"

namespace cg = cooperative_groups;

namespace ctg {

namespace {

constexpr int SVD_THREADS = 256;
constexpr int NWARPS = SVD_THREADS / 32;
constexpr int SVD_STEP_PAIRS = 32;            // most column pairs of one inner step (group size <= 32)
constexpr int SVD_SMEM_LIMIT = 220 * 1024;    // dynamic shared memory per CTA (227 KB less static use)
constexpr int SVD_F32_SWEEPS = 5;             // default: most FP32 preconditioning sweeps
constexpr int SVD_F32_SWEEPS_MAX = 8;         // capacity of the FP32 sweep flags
constexpr float SVD_F32_COS = 0.0f;           // default: FP32 sweeps rotate every pair above N eps_32
constexpr int SVD_F32_MIN_RANK = 32;          // default: smallest rank preconditioned in FP32
constexpr int SVD_F32_CLUSTER = 8;            // default: CTAs of the FP32 sweeps
constexpr int SVD_OUT_RC = 32;                // reflectors staged per round of the output phase

// shared memory (doubles) of the Jacobi tour: two buffers of two column groups (records of 2 N),
// their norms and the per-step pair data
__host__ __device__ inline i64 tour_jac_doubles(int N, int cl)
{
	const i64 nblk = 2 * cl, bsmax = (N + nblk - 1) / nblk;
	return 4 * bsmax * 2 * N + 4 * bsmax + 3 * SVD_STEP_PAIRS + SVD_STEP_PAIRS / 2 + 16;
}

// records of the FP32 tour: 2 N floats rounded up to a multiple of four, so that every column
// starts on a 16-byte boundary (the exchanges between CTAs move float4)
__host__ __device__ inline int f32_record(int N) { return (2 * N + 3) & ~3; }

// shared memory (bytes) of the FP32 tour over 2 cf groups of the r columns
__host__ __device__ inline i64 f32_tour_bytes(int N, int r, int cf)
{
	const i64 bs = (r + 2 * cf - 1) / (2 * cf);
	return 4 * (4 * bs * (i64)f32_record(N) + 4 * bs + 4);
}

// scratch (doubles) of one block's SVD before the refinement's arrays: the larger of the
// shared-memory path's layout (W, T, V, norms, reflector scalars, singular values, misc, flags,
// pivots) and the global-memory path's (W, Q, T, V, ...), rounded up to a multiple of 2
__host__ __device__ inline i64 svd_refine_offset(i64 M, i64 N)
{
	const i64 base = 2 * M * N + 2 * N * N + 3 * N + 4 + 2 * SVD_MAX_SWEEPS + (N + 1) / 2 + 1;
	return (base + 1) & ~(i64)1;
}
// the refinement's arrays: G (N x N doubles), X (N x N floats), (hi, lo) float pairs of T (N x N)
// and V (N x N), per iteration a failure flag, the largest cosine and the number of cluster edges,
// and the cluster-edge list (4 N pairs)
__host__ __device__ inline i64 svd_refine_doubles(i64 N)
{
	return N * N + (N * N + 1) / 2 + 2 * N * N + 12 + 4 * N;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

__device__ double block_sum(double v, double* red)
{
	v = warp_sum(v);
	__syncthreads();
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
	__syncthreads();
	double t = 0;
	for (int w = 0; w < NWARPS; w++) t += red[w];
	return t;
}

// Householder QR with column pivoting of W (M x N, column-major) inside one CTA, stopped at
// the numerical rank; returns r. W keeps R in its upper triangle and the Householder vectors
// below it; tau and perm receive the scalars and the column permutation. The squared norms of
// the trailing column parts are downdated after every step (nrm[j] -= R_kj^2) and recomputed
// when cancellation has eaten more than sqrt(eps) of the last exactly computed value (ref), the
// safeguard of LAPACK's xLAQP2.
__device__ int qr_pivoted_cta(double* W, int M, int N, double* nrm, double* ref, double* tau, int* perm,
                              double rank_thresh2)
{
	__shared__ double red[NWARPS];
	__shared__ double sh_beta, sh_tau, sh_scale;
	__shared__ int sh_piv, sh_stop;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const double tol3z = sqrt(DBL_EPSILON);
	for (int j = warp; j < N; j += NWARPS)
	{
		const double* wj = W + (i64)j * M;
		double acc = 0;
		for (int i = lane; i < M; i += 32) acc = fma(wj[i], wj[i], acc);
		acc = warp_sum(acc);
		if (lane == 0) nrm[j] = ref[j] = acc;
	}
	__syncthreads();
	int r = 0;
	for (int k = 0; k < N; k++)
	{
		if (warp == 0)
		{
			double best = -1;
			int bi = k;
			for (int j = k + lane; j < N; j += 32)
				if (nrm[j] > best) { best = nrm[j]; bi = j; }
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
			{
				const double ob = __shfl_xor_sync(0xffffffffu, best, o);
				const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
				if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
			}
			if (lane == 0)
			{
				sh_piv = bi;
				sh_stop = (best <= rank_thresh2 || best <= 0.0) ? 1 : 0;
			}
		}
		__syncthreads();
		if (sh_stop) break;
		const int p = sh_piv;
		if (p != k)
		{
			double* wk = W + (i64)k * M;
			double* wp = W + (i64)p * M;
			for (int i = tid; i < M; i += SVD_THREADS)
			{
				const double t = wk[i];
				wk[i] = wp[i];
				wp[i] = t;
			}
			if (tid == 0)
			{
				const int t = perm[k];
				perm[k] = perm[p];
				perm[p] = t;
				double x = nrm[k];
				nrm[k] = nrm[p];
				nrm[p] = x;
				x = ref[k];
				ref[k] = ref[p];
				ref[p] = x;
			}
		}
		__syncthreads();
		double* wk = W + (i64)k * M;
		double part = 0;
		for (int i = k + 1 + tid; i < M; i += SVD_THREADS) part = fma(wk[i], wk[i], part);
		const double xnorm2 = block_sum(part, red);
		if (tid == 0)
		{
			const double alpha = wk[k];
			if (xnorm2 == 0.0)
			{
				sh_tau = 0.0;
				sh_beta = alpha;
				sh_scale = 0.0;
			}
			else
			{
				const double beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
				sh_tau = (beta - alpha) / beta;
				sh_beta = beta;
				sh_scale = 1.0 / (alpha - beta);
			}
		}
		__syncthreads();
		const double tk = sh_tau;
		for (int i = k + 1 + tid; i < M; i += SVD_THREADS) wk[i] *= sh_scale;
		__syncthreads();
		if (tid == 0) { wk[k] = sh_beta; tau[k] = tk; }
		__syncthreads();
		for (int j = k + 1 + warp; j < N; j += NWARPS)
		{
			double* wj = W + (i64)j * M;
			if (tk != 0.0)
			{
				double acc = 0;
				for (int i = k + lane; i < M; i += 32) acc = fma(i == k ? 1.0 : wk[i], wj[i], acc);
				acc = warp_sum(acc) * tk;
				for (int i = k + lane; i < M; i += 32) wj[i] -= acc * (i == k ? 1.0 : wk[i]);
			}
			// downdate the trailing norm by R_kj^2 (lane 0 holds row k of this column)
			int recompute = 0;
			if (lane == 0)
			{
				const double rkj = wj[k];
				const double v = fmax(fma(-rkj, rkj, nrm[j]), 0.0);
				nrm[j] = v;
				recompute = v <= tol3z * ref[j];
			}
			if (__shfl_sync(0xffffffffu, recompute, 0))
			{
				double acc = 0;
				for (int i = k + 1 + lane; i < M; i += 32) acc = fma(wj[i], wj[i], acc);
				acc = warp_sum(acc);
				if (lane == 0) nrm[j] = ref[j] = acc;
			}
		}
		__syncthreads();
		r = k + 1;
	}
	return r;
}

// ---- one-sided Jacobi on a thread-block cluster, columns resident in shared memory ----------
//
// The r columns of R^T (with their rows of V) are cut into 2 cl groups of bs consecutive columns.
// Each CTA of the cluster holds two groups (slots 0 and 1) in shared memory. A sweep is a
// round-robin tournament over the groups (circle method, 2 cl - 1 rounds): in each round a CTA
// rotates every column of its slot-0 group against every column of its slot-1 group (bs steps of
// bs disjoint pairs), in round 0 also the pairs inside each group; then it writes both groups into
// the shared memory of the CTAs that hold them in the next round (distributed shared memory,
// double-buffered) and the cluster synchronises once. Each column pair meets once per sweep,
// as in the cyclic one-sided Jacobi method; a round costs one cluster barrier instead of one per
// pair set, and the column data never leaves the SMs.

__device__ __forceinline__ unsigned long long globaltimer()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ float rcp_approx(float x)
{
	float y;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

// FP32 mantissa in [1, 2) (truncated to 23 bits) and unbiased exponent of a finite normal double,
// by integer operations: on GB300 a double -> float conversion costs as much as an FP64 FMA
__device__ __forceinline__ float mant_exp(double x, int& e)
{
	const int hi = __double2hiint(x), lo = __double2loint(x);
	e = ((hi >> 20) & 0x7ff) - 1023;
	return __int_as_float(0x3f800000 | ((hi & 0x000fffff) << 3) | (int)((unsigned)lo >> 29));
}

// the double m * 2^e for a normal float m (exact), by integer operations
__device__ __forceinline__ double make_double(float m, int e)
{
	const int fb = __float_as_int(m);
	if ((fb & 0x7fffffff) == 0) return 0.0;
	const int fe = ((fb >> 23) & 0xff) - 127 + e;
	const int hi = (fb & (int)0x80000000) | ((fe + 1023) << 20) | ((fb & 0x007fffff) >> 3);
	return __hiloint2double(hi, (fb & 0x7) << 29);
}

__device__ __forceinline__ float sqrt_approx(float x)
{
	float y;
	asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

// 2^k as a float for -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k)
{
	return __int_as_float((k + 127) << 23);
}

// Jacobi rotation for the 2 x 2 Gram matrix [al ga; ga be] of a column pair (al, be > 0).
// Returns false if the pair counts as orthogonal (cos^2 = ga^2 / (al be) <= tol2); c2 receives
// the FP32 estimate of cos^2 (1 when it is not small). Otherwise the
// rotation angle theta (tan theta the smaller root of t^2 + 2 zeta t - 1 = 0, zeta = (be - al) /
// (2 ga)) is found in FP32 on mantissas and integer exponents, and the rotation is returned as
// tau = tan(theta / 2) and sn = sin theta = 2 tau / (1 + tau^2) in FP64, for the three-shear form
// x1 = x - tau y, y' = y + sn x1, x' = x1 - tau y' (Paeth), which is a rotation up to FP64
// rounding for any tau; t = tan theta (FP32 accuracy) updates the squared norms. Only the
// difference be - al, the FP64 reciprocal of 1 + tau^2 (FP32 estimate, one cubically convergent
// Newton step d0 (1 + e + e^2), e = 1 - q d0) and the products use the FP64 pipe: an FP64 division
// or square root costs over a thousand cycles on GB300. The angle is accurate to FP32 only: the
// rotation leaves a cosine of about 1e-7 of the previous one, which a later sweep removes.
__device__ __forceinline__ bool rotation_params(double al, double be, double ga, float tol2, double& tau, double& sn,
                                                double& t, float& c2)
{
	c2 = 0.0f;
	// zero and sign tests on the bit patterns: an FP64 compare would take an FP64 pipe slot on the
	// serial chain of every step
	const long long gbits = __double_as_longlong(ga);
	if ((gbits & 0x7fffffffffffffffll) == 0) return false;
	int ea, eb, eg;
	const float ma = mant_exp(al, ea), mb = mant_exp(be, eb), mg = mant_exp(ga, eg);
	const int k2 = 2 * eg - ea - eb;
	if (k2 < -120) return false;
	if (k2 <= 0)
	{
		c2 = __fdividef(mg * mg, ma * mb) * pow2f(k2);
		if (c2 <= tol2) return false;
	}
	else c2 = 1.0f;
	const double dl = be - al;
	const long long dbits = __double_as_longlong(dl);
	const bool neg = (dbits < 0) != (gbits < 0);
	float tm, taum;
	int te = 0;
	if ((dbits & 0x7fffffffffffffffll) == 0)
	{
		tm = 1.0f;
		taum = 0.41421356f;
	}
	else
	{
		int ed;
		const float md = mant_exp(dl, ed);
		const int k = ed - eg - 1;                 // |zeta| = (md / mg) 2^k
		if (k >= 40)
		{
			// tan theta ~ 1 / (2 |zeta|), tan(theta / 2) ~ tan theta / 2
			tm = __fdividef(0.5f * mg, md);
			te = -k;
			taum = 0.5f * tm;
		}
		else if (k <= -40)
		{
			tm = 1.0f;
			taum = 0.41421356f;
		}
		else
		{
			// single-instruction approximations: the angle needs FP32 accuracy only
			const float z = __fdividef(md, mg) * pow2f(k);
			tm = __fdividef(1.0f, z + sqrt_approx(fmaf(z, z, 1.0f)));
			taum = __fdividef(tm, 1.0f + sqrt_approx(fmaf(tm, tm, 1.0f)));
		}
	}
	if (neg)
	{
		tm = -tm;
		taum = -taum;
	}
	tau = make_double(taum, te);
	t = make_double(tm, te);
	const double q = fma(tau, tau, 1.0);
	int eq;
	const double d0 = make_double(rcp_approx(mant_exp(q, eq)), -eq);
	const double e = fma(-q, d0, 1.0);
	const double w = fma(d0, fma(e, e, e), d0);
	sn = make_double(taum + taum, te) * w;
	return (__double_as_longlong(sn) & 0x7fffffffffffffffll) != 0;
}

struct Tour {
	int nblk, nm, bs, bsmax, r, N, ld;
	double* sm;
	__device__ double* col(int buf, int slot, int c) const { return sm + (i64)((buf * 2 + slot) * bsmax + c) * ld; }
	__device__ double* nrm(int buf, int slot) const { return sm + (i64)4 * bsmax * ld + (buf * 2 + slot) * bsmax; }
	__device__ int cnt(int x) const
	{
		const int c = r - x * bs;
		return c < 0 ? 0 : (c > bs ? bs : c);
	}
};

struct StepBuf {
	int* local_rot;              // set when a rotation was applied in the current sweep
	int* max_c2;                 // largest cos^2 of the sweep's pairs (bits of a non-negative float)
};

__device__ __forceinline__ bool step_pair(const Tour& t, int mode, int step, int k, int cA, int cB, int npad, int& sp,
                                          int& cp, int& sq, int& cq)
{
	return step_pair_idx(mode, step, k, t.bs, cA, cB, npad, sp, cp, sq, cq);
}

// One inner step of the FP64 tour. The pairs of a step are disjoint, so each warp takes whole
// pairs: the inner product (every lane gets the sum), the rotation parameters (computed by every
// lane: an FP64 warp instruction costs the same whatever the number of active lanes) and the
// three-shear rotation of the two records (T entries 0 .. N-1, V entries N .. N+r-1). One CTA
// barrier per step, and the warps of different pairs run on different SM sub-partitions.
__device__ void jacobi_step(const Tour& t, int buf, int mode, int step, int cA, int cB, int npad, float tol2, const StepBuf& sb,
                            long long* cyc, long long& flops)
{
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const long long c0 = cyc ? clock64() : 0;
	const int np = mode == 0 ? npad : t.bs;
	const int len = t.N + t.r;
	for (int k = warp; k < np; k += NWARPS)
	{
		int sp, cp, sq, cq;
		if (!step_pair(t, mode, step, k, cA, cB, npad, sp, cp, sq, cq)) continue;
		double* x = t.col(buf, sp, cp);
		double* y = t.col(buf, sq, cq);
		double g = 0;
		for (int i = lane; i < t.N; i += 32) g = fma(x[i], y[i], g);
		g = warp_sum(g);
		double* pa = t.nrm(buf, sp) + cp;
		double* pb = t.nrm(buf, sq) + cq;
		const double al = *pa, be = *pb;
		double tau, sn, tn;
		float c2;
		const bool rot = rotation_params(al, be, g, tol2, tau, sn, tn, c2);
		// executed FP64 flops: an inner product per examined pair, three FMAs per entry of the two
		// column records per rotation (counted on lane 0 of each warp)
		if (lane == 0)
		{
			flops += 2 * t.N;                    // integer: no FP64 slot on the chain
			atomicMax(sb.max_c2, __float_as_int(c2));
		}
		if (rot)
		{
			for (int i = lane; i < len; i += 32)
			{
				const double x1 = fma(-tau, y[i], x[i]);
				const double y1 = fma(sn, x1, y[i]);
				x[i] = fma(-tau, y1, x1);
				y[i] = y1;
			}
			__syncwarp();
			if (lane == 0)
			{
				*pa = fma(-tn, g, al);
				*pb = fma(tn, g, be);
				*sb.local_rot = 1;
				flops += 6 * len;
			}
		}
	}
	__syncthreads();
	if (cyc) cyc[0] += clock64() - c0;
}

// ---- FP32 preconditioning ----------------------------------------------------------------
//
// An SM retires 128 FP32 FMAs per clock against two FP64 FMAs, and the first Jacobi sweeps rotate
// almost every pair. So for larger blocks the tour first runs on FP32 copies of R^T and V (same
// schedule, records of N + r floats) until the cosines fall to about N eps_32. V is then made
// orthogonal to FP64 rounding by two Newton-Schulz steps V <- V - V (V^T V - I) / 2 (the error
// squares each step: 1e-5, 1e-10, below eps) and T = R^T V is formed in FP64. The FP64 sweeps
// that follow start from columns orthogonal to FP32 accuracy and converge quadratically, in
// about two sweeps plus the one that confirms convergence, where six to nine are needed from
// R^T itself. The FP64 sweeps alone decide the result: the FP32 phase only chooses the starting
// basis. (Low-precision Jacobi SVD as preconditioner of a high-precision one-sided Jacobi: W. Gao,
// Y. Ma, M. Shao, "A mixed precision Jacobi SVD algorithm", arXiv:2209.04626.)

struct Tour32 {
	int nblk, nm, bs, bsmax, r, N, ld;
	float* sm;
	__device__ float* col(int buf, int slot, int c) const { return sm + (i64)((buf * 2 + slot) * bsmax + c) * ld; }
	__device__ float* nrm(int buf, int slot) const { return sm + (i64)4 * bsmax * ld + (buf * 2 + slot) * bsmax; }
	__device__ int cnt(int x) const
	{
		const int c = r - x * bs;
		return c < 0 ? 0 : (c > bs ? bs : c);
	}
};

__device__ __forceinline__ float warp_sumf(float v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// One inner step of the FP32 tour. The pairs of a step are disjoint, so each warp takes whole
// pairs: inner product (every lane gets the sum), classical Jacobi rotation (tan theta the
// smaller root of t^2 + 2 zeta t - 1 = 0, computed by every lane), rotation of the two records.
// One CTA barrier per step.
__device__ void jacobi_step32(const Tour32& t, int buf, int mode, int step, int cA, int cB, int npad, float tol2,
                              int* local_rot)
{
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int np = mode == 0 ? npad : t.bs;
	const int len = t.N + t.r;
	for (int k = warp; k < np; k += NWARPS)
	{
		int sp, cp, sq, cq;
		if (!step_pair_idx(mode, step, k, t.bs, cA, cB, npad, sp, cp, sq, cq)) continue;
		float* x = t.col(buf, sp, cp);
		float* y = t.col(buf, sq, cq);
		// the lane's entries loaded eight at a time before they are added (in the same order): the
		// loads of a step are then in flight together instead of one pair per iteration
		float g = 0.0f;
		for (int i0 = 0; i0 < t.N; i0 += 256)
		{
			float xs[8], ys[8];
#pragma unroll
			for (int u = 0; u < 8; u++)
			{
				const int i = i0 + lane + 32 * u;
				xs[u] = i < t.N ? x[i] : 0.0f;
				ys[u] = i < t.N ? y[i] : 0.0f;
			}
#pragma unroll
			for (int u = 0; u < 8; u++)
				if (i0 + 32 * u < t.N) g = fmaf(xs[u], ys[u], g);     // the same in every lane
		}
		g = warp_sumf(g);
		float* pa = t.nrm(buf, sp) + cp;
		float* pb = t.nrm(buf, sq) + cq;
		const float al = *pa, be = *pb;
		if (g != 0.0f && g * g > tol2 * al * be)
		{
			// single-instruction approximations: the FP32 angle needs FP32 accuracy only (the FP64
			// finish removes what is left), and the IEEE division and square root sequences sit on
			// the serial chain of every step
			const float zeta = __fdividef(be - al, 2.0f * g);
			const float az = fabsf(zeta);
			float tn = az > 1e10f ? __fdividef(0.5f, az) : __fdividef(1.0f, az + sqrt_approx(fmaf(az, az, 1.0f)));
			tn = copysignf(tn, zeta);
			const float c = rsqrtf(fmaf(tn, tn, 1.0f));
			const float sn = c * tn;
			for (int i0 = 0; i0 < len; i0 += 128)
			{
				float xv[4], yv[4];
#pragma unroll
				for (int u = 0; u < 4; u++)
				{
					const int i = i0 + lane + 32 * u;
					xv[u] = i < len ? x[i] : 0.0f;
					yv[u] = i < len ? y[i] : 0.0f;
				}
#pragma unroll
				for (int u = 0; u < 4; u++)
				{
					const int i = i0 + lane + 32 * u;
					if (i < len)
					{
						x[i] = fmaf(c, xv[u], -sn * yv[u]);
						y[i] = fmaf(sn, xv[u], c * yv[u]);
					}
				}
			}
			__syncwarp();
			if (lane == 0)
			{
				*pa = fmaf(-tn, g, al);
				*pb = fmaf(tn, g, be);
				*local_rot = 1;
			}
		}
	}
	__syncthreads();
}

struct SvdScratch {
	double *W, *T, *V, *nrm, *tau, *sig, *misc;
	int *flags, *perm, *flags32, *cmax;
	double* G;                   // refinement of the mixed path: G, X, (hi, lo) copies of T and V
};

// workspace of one block: W (M x N, B then R and the reflectors), T (N x r), V (r x r), column
// norms, reflector scalars, singular values, misc [rank, ||B||_F^2, unscale], sweep flags, pivots,
// FP32 sweep flags, largest cos^2 per sweep; after the larger of this layout and the global-memory
// path's, the refinement's arrays (svd_refine_offset)
__device__ __forceinline__ SvdScratch scratch_layout(double* base, int M, int N)
{
	SvdScratch x;
	x.W = base;
	x.T = x.W + (i64)M * N;
	x.V = x.T + (i64)N * N;
	x.nrm = x.V + (i64)N * N;
	x.tau = x.nrm + N;
	x.sig = x.tau + N;
	x.misc = x.sig + N;
	x.flags = (int*)(x.misc + 4);
	x.perm = x.flags + SVD_MAX_SWEEPS;
	x.flags32 = x.perm + N;
	x.cmax = x.flags32 + SVD_F32_SWEEPS_MAX;
	x.G = base + svd_refine_offset(M, N);
	return x;
}

// Warp-wide argmax of 64-bit keys (a non-negative double's bits, or -1 for no candidate): the
// largest key, equal keys to the smallest index, by three warp reductions (redux.sync on the key's
// high and low words, then on the index) instead of a five-round shuffle butterfly on the serial
// chain of every QR step. Every lane returns the winner's key (-1 if none) and index.
__device__ __forceinline__ void warp_argmax_key(long long key, int idx, long long& kbest, int& ibest)
{
	const unsigned long long u = key < 0 ? 0ull : (unsigned long long)key + 1ull;   // 0: no candidate
	const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
	const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
	const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
	const bool win = hi == mhi && lo == mlo;
	ibest = (int)__reduce_min_sync(0xffffffffu, win ? (unsigned)idx : 0xffffffffu);
	const unsigned long long ub = ((unsigned long long)mhi << 32) | mlo;
	kbest = ub == 0ull ? -1 : (long long)(ub - 1ull);
}

// Householder QR with column pivoting of the scaled block over a whole cluster. Column j lives in
// the shared memory of CTA j % cl; columns are not moved. Every step the first warp of each CTA
// picks the CTA's best remaining column and forms its reflector in its own shared memory
// (speculatively: only the pivot's is used); the CTA writes the column's squared norm, index and
// reflector scalars into every CTA's shared memory (distributed shared memory, double-buffered by
// step parity). After one cluster barrier every CTA holds all candidates' scalars, agrees on the
// pivot (largest norm, then smallest index), reads the pivot's reflector from the CTA that formed
// it, and applies it to its own remaining columns, downdating
// the norms (recomputed when cancellation has eaten more than sqrt(eps) of the last exact value,
// as in qr_pivoted_cta).
// Its shared memory (doubles):
__host__ __device__ inline i64 qr_cluster_doubles(int M, int N, int cl)
{
	const i64 nloc = (N + cl - 1) / cl;
	return nloc * M + 2 * nloc + 3 * (i64)M + 16 + 3 * 2 * 16 + (2 * 16 + nloc + 1) / 2 + 8;
}

__device__ int qr_pivoted_cluster(cg::cluster_group& cluster, double* smem, const double* ab, bool tall, int n, int M, int N,
                                  int cl, const SvdScratch& xs, long long* qc)
{
	const int rank = (int)cluster.block_rank();
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int nloc_max = (N + cl - 1) / cl;
	const int nloc = (N - rank + cl - 1) / cl;           // columns j = rank + cl * jl, jl < nloc
	double* qcol = smem;                                 // nloc_max x M
	double* qnrm = qcol + (i64)nloc_max * M;
	double* qref = qnrm + nloc_max;
	double* cand = qref + nloc_max;                      // [2][M] own candidate reflector, by step parity
	double* vloc = cand + 2 * (i64)M;                    // [M] the pivot's reflector, fetched from its CTA
	double* part = vloc + M;                             // [cl] partial Frobenius sums
	double* hnrm = part + 16;                            // [2][16] candidate squared norm per CTA
	double* htau = hnrm + 32;                            // [2][16] candidate tau per CTA
	double* hbeta = htau + 32;                           // [2][16] candidate beta per CTA
	int* hidx = (int*)(hbeta + 32);                      // [2][16] candidate column per CTA
	int* qdone = hidx + 32;                              // [nloc_max] step that took the column, or -1
	__shared__ double red[NWARPS];
	__shared__ double sh_tau, sh_beta, sh_best;
	__shared__ int sh_jl;

	// load the own columns (B oriented tall) and their squared sums
	double psum = 0;
	for (i64 e = tid; e < (i64)nloc * M; e += SVD_THREADS)
	{
		const int jl = (int)(e / M), row = (int)(e % M);
		const int col = rank + cl * jl;
		const double x = tall ? ab[(i64)row * n + col] : ab[(i64)col * n + row];
		qcol[e] = x;
		psum = fma(x, x, psum);
	}
	psum = block_sum(psum, red);
	if (tid < cl) *cluster.map_shared_rank(part + rank, (unsigned)tid) = psum;
	cluster.sync();
	double total = 0;
	for (int i = 0; i < cl; i++) total += part[i];
	// exact power-of-two scaling to a Frobenius norm in [1/2, 1)
	int ex = 0;
	if (total > 0) frexp(sqrt(total), &ex);
	const double sc = ldexp(1.0, -ex);
	for (i64 e = tid; e < (i64)nloc * M; e += SVD_THREADS) qcol[e] *= sc;
	__syncthreads();
	for (int jl = warp; jl < nloc; jl += NWARPS)
	{
		const double* w = qcol + (i64)jl * M;
		double acc = 0;
		for (int i = lane; i < M; i += 32) acc = fma(w[i], w[i], acc);
		acc = warp_sum(acc);
		if (lane == 0)
		{
			qnrm[jl] = qref[jl] = acc;
			qdone[jl] = -1;
		}
	}
	const double thresh = DBL_EPSILON * DBL_EPSILON * total * sc * sc;
	const double tol3z = sqrt(DBL_EPSILON);
	__syncthreads();

	int r = 0;
	for (int k = 0; k < N; k++)
	{
		const int par = k & 1;
		double* cbuf = cand + (i64)par * M;
		long long q0 = qc ? clock64() : 0;
		// a. warp 0: this CTA's best remaining column and its reflector (speculative)
		if (warp == 0)
		{
			// the squared norms are non-negative doubles, which order like their bit patterns as
			// signed integers: the argmax compares integers (an FP64 compare costs an FP64 pipe slot)
			long long bbits = -1;
			int bi = N;
			for (int jl = lane; jl < nloc; jl += 32)
			{
				const long long nb = __double_as_longlong(qnrm[jl]);
				if (qdone[jl] < 0 && nb > bbits) { bbits = nb; bi = rank + cl * jl; }
			}
			warp_argmax_key(bbits, bi, bbits, bi);
			const int bj = bbits >= 0 ? (bi - rank) / cl : -1;
			double best = bbits < 0 ? -1.0 : __longlong_as_double(bbits);
			double tk = 0.0, beta = 0.0;
			if (bj >= 0 && bbits > __double_as_longlong(thresh))
			{
				const double* w = qcol + (i64)bj * M;
				double x2 = 0;
				for (int i = k + 1 + lane; i < M; i += 32) x2 = fma(w[i], w[i], x2);
				x2 = warp_sum(x2);
				const double alpha = w[k];
				double scl = 0.0;
				if (__double_as_longlong(x2) == 0) beta = alpha;    // x2 >= +0: its bits are zero only at zero
				else
				{
					// |beta| = sqrt(alpha^2 + x2) >= the remaining norm, above the rank threshold:
					// normal doubles. tau = (beta - alpha) / beta = (|beta| + |alpha|) / |beta|,
					// scale = 1 / (alpha - beta) = sign(alpha) / (|alpha| + |beta|).
					double sq, rsq;
					sqrt_rsqrt64(fma(alpha, alpha, x2), sq, rsq);
					beta = -copysign(sq, alpha);
					const double sum = sq + fabs(alpha);
					tk = sum * rsq;
					scl = copysign(rcp64(sum), alpha);
				}
				for (int i = k + lane; i < M; i += 32) cbuf[i] = (i == k) ? 1.0 : w[i] * scl;
			}
			else best = -1.0;
			if (lane == 0)
			{
				sh_best = best;
				sh_jl = bj;
				sh_tau = tk;
				sh_beta = beta;
			}
		}
		__syncthreads();
		if (qc)
		{
			const long long q1 = clock64();
			qc[0] += q1 - q0;
			q0 = q1;
		}
		// b. the candidate's norm, column and scalars into every CTA's shared memory; its reflector
		// stays here (cand[par]) and only the winner's is read, after the barrier. cand[par] is
		// written again two steps later, after the next step's barrier, which every CTA reaches
		// only once it has read this step's pivot.
		const double best = sh_best;
		if (tid < cl)
		{
			*cluster.map_shared_rank(hnrm + par * 16 + rank, (unsigned)tid) = best;
			*cluster.map_shared_rank(hidx + par * 16 + rank, (unsigned)tid) = best > 0.0 ? rank + cl * sh_jl : N;
			*cluster.map_shared_rank(htau + par * 16 + rank, (unsigned)tid) = sh_tau;
			*cluster.map_shared_rank(hbeta + par * 16 + rank, (unsigned)tid) = sh_beta;
		}
		if (qc)
		{
			const long long q1 = clock64();
			qc[1] += q1 - q0;
			q0 = q1;
		}
		cluster.sync();
		if (qc)
		{
			const long long q1 = clock64();
			qc[2] += q1 - q0;
			q0 = q1;
		}
		// c. the pivot: every warp reduces the candidates itself (no barrier); a CTA without a
		// candidate posts -1, every other candidate norm is positive: integer compares of the bits
		long long pb = -1;
		if (lane < cl)
		{
			const long long hb = __double_as_longlong(hnrm[par * 16 + lane]);    // -1.0: no candidate
			pb = hb > 0 ? hb : -1;
		}
		int p = lane < cl ? hidx[par * 16 + lane] : N;
		warp_argmax_key(pb, p, pb, p);
		if (pb <= __double_as_longlong(thresh) || pb <= 0 || p >= N) break;
		const int owner = p % cl;                            // column p lives in CTA p mod cl
		const double tk = htau[par * 16 + owner];
		const double* vbuf = cbuf;
		if (owner != rank)                                   // uniform in the CTA
		{
			const double* src = cluster.map_shared_rank(cbuf, (unsigned)owner);
			for (int i = k + tid; i < M; i += SVD_THREADS) vloc[i] = src[i];
			vbuf = vloc;
			__syncthreads();
		}
		// the owner stores R_kk and the reflector in place (the updates below skip that column)
		const int pjl = owner == rank ? p / cl : -1;
		if (pjl >= 0)
		{
			double* w = qcol + (i64)pjl * M;
			for (int i = k + 1 + tid; i < M; i += SVD_THREADS) w[i] = cbuf[i];
			if (tid == 0)
			{
				w[k] = hbeta[par * 16 + owner];
				xs.tau[k] = tk;
				qdone[pjl] = k;
			}
		}
		if (qc)
		{
			const long long q1 = clock64();
			qc[3] += q1 - q0;
			q0 = q1;
		}
		// d. apply the reflector to the own remaining columns, downdate their norms
		for (int jl = warp; jl < nloc; jl += NWARPS)
		{
			if (jl == pjl || qdone[jl] >= 0) continue;
			double* w = qcol + (i64)jl * M;
			if (__double_as_longlong(tk) != 0)               // tk >= +0
			{
				double acc = 0;
				for (int i = k + lane; i < M; i += 32) acc = fma(vbuf[i], w[i], acc);
				acc = warp_sum(acc) * tk;
				for (int i = k + lane; i < M; i += 32) w[i] -= acc * vbuf[i];
			}
			int recompute = 0;
			if (lane == 0)
			{
				const double rkj = w[k];
				const double v = fmax(fma(-rkj, rkj, qnrm[jl]), 0.0);
				qnrm[jl] = v;
				recompute = v <= tol3z * qref[jl];
			}
			if (__shfl_sync(0xffffffffu, recompute, 0))
			{
				double acc = 0;
				for (int i = k + 1 + lane; i < M; i += 32) acc = fma(w[i], w[i], acc);
				acc = warp_sum(acc);
				if (lane == 0) qnrm[jl] = qref[jl] = acc;
			}
		}
		__syncthreads();
		if (qc) qc[4] += clock64() - q0;
		r = k + 1;
	}
	// columns to global memory in pivot order, the remaining ones after them in source order
	int* gdone = (int*)xs.T;                             // scratch until the Jacobi writes T
	for (int jl = tid; jl < nloc; jl += SVD_THREADS) gdone[rank + cl * jl] = qdone[jl];
	cluster.sync();
	for (int jl = warp; jl < nloc; jl += NWARPS)
	{
		const int j = rank + cl * jl;
		int pos = qdone[jl];
		if (pos < 0)
		{
			int cnt = 0;
			for (int j2 = lane; j2 < j; j2 += 32) cnt += __ldcg(gdone + j2) < 0 ? 1 : 0;
			pos = r + (int)__reduce_add_sync(0xffffffffu, (unsigned)cnt);
		}
		const double* w = qcol + (i64)jl * M;
		for (int i = lane; i < M; i += 32) xs.W[(i64)pos * M + i] = w[i];
		if (lane == 0) xs.perm[pos] = j;
	}
	if (rank == 0 && tid == 0)
	{
		xs.misc[0] = (double)r;
		xs.misc[1] = total;
		xs.misc[2] = ldexp(1.0, ex);
	}
	return r;
}

// FP32 preconditioning of the tour (see above). The FP32 sweeps run on the first cf CTAs of the
// cluster (a tour over 2 cf groups; the others only keep the cluster barriers in step): their
// cost is latency and barriers, not arithmetic, and fewer, larger groups need fewer rounds. On
// return, V (r x r, orthogonal to FP32 accuracy, column g at xs.V + g r) is in global memory.
__device__ void precondition_f32(cg::cluster_group& cluster, const Tour& t, double* smem, const SvdScratch& xs, int M,
                                 int cf, int rank, int nsw, float cos_min, long long* cyc)
{
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const long long c0 = cyc ? clock64() : 0;
	const int N = t.N, r = t.r;
	Tour32 f;
	f.nblk = 2 * cf;
	f.nm = f.nblk - 1;
	f.bs = (r + f.nblk - 1) / f.nblk;
	f.bsmax = f.bs;
	f.r = r;
	f.N = N;
	f.ld = f32_record(N);
	f.sm = (float*)smem;
	int* local_rot = (int*)(f.sm + (i64)4 * f.bsmax * f.ld + 4 * f.bsmax);
	int A, B;
	if (rank < cf)
	{
		round_groups(0, rank, f.nm, A, B);
		// column g of T is row g of R (upper triangle of W); column g of V is e_g
		for (int slot = 0; slot < 2; slot++)
		{
			const int x = slot ? B : A;
			float* dst = f.col(0, slot, 0);
			for (i64 e = tid; e < (i64)f.cnt(x) * f.ld; e += SVD_THREADS)
			{
				const int c = (int)(e / f.ld), i = (int)(e % f.ld);
				const int g = x * f.bs + c;
				float v;
				if (i < N) v = (i >= g) ? (float)__ldcg(xs.W + (i64)i * M + g) : 0.0f;
				else v = (i - N == g) ? 1.0f : 0.0f;
				dst[e] = v;
			}
		}
		__syncthreads();
		const float tol2 = fmaxf((float)N * FLT_EPSILON * (float)N * FLT_EPSILON, cos_min * cos_min);
		int buf = 0, done32 = nsw;
		for (int sweep = 0; sweep < nsw; sweep++)
		{
			round_groups(0, rank, f.nm, A, B);
			for (int slot = 0; slot < 2; slot++)
			{
				const int nc = f.cnt(slot ? B : A);
				for (int c = warp; c < nc; c += NWARPS)
				{
					const float* col = f.col(buf, slot, c);
					float acc = 0.0f;
					for (int i0 = 0; i0 < N; i0 += 256)
					{
						float xs[8];
#pragma unroll
						for (int u = 0; u < 8; u++)
						{
							const int i = i0 + lane + 32 * u;
							xs[u] = i < N ? col[i] : 0.0f;
						}
#pragma unroll
						for (int u = 0; u < 8; u++)
							if (i0 + 32 * u < N) acc = fmaf(xs[u], xs[u], acc);
					}
					acc = warp_sumf(acc);
					if (lane == 0) f.nrm(buf, slot)[c] = acc;
				}
			}
			if (tid == 0) *local_rot = 0;
			__syncthreads();
			for (int rho = 0; rho < f.nm; rho++)
			{
				round_groups(rho, rank, f.nm, A, B);
				const int cA = f.cnt(A), cB = f.cnt(B);
				if (rho == 0)
				{
					const int npad = f.bs + (f.bs & 1);
					for (int st = 0; st < npad - 1; st++) jacobi_step32(f, buf, 0, st, cA, cB, npad, tol2, local_rot);
				}
				for (int st = 0; st < f.bs; st++) jacobi_step32(f, buf, 1, st, cA, cB, 0, tol2, local_rot);
				if (cf > 1)
				{
					const long long cx = cyc ? clock64() : 0;
					if (tid == 0 && rho == f.nm - 1 && *local_rot) atomicOr(xs.flags32 + sweep, 1);
					const int rho1 = (rho + 1) % f.nm;
					for (int slot = 0; slot < 2; slot++)
					{
						const int x = slot ? B : A, nc = f.cnt(x);
						int pi2, slot2;
						group_owner(x, rho1, f.nm, pi2, slot2);
						const float4* src = (const float4*)f.col(buf, slot, 0);
						float4* dst = (float4*)cluster.map_shared_rank(f.col(buf ^ 1, slot2, 0), (unsigned)pi2);
						for (i64 e = tid; e < (i64)nc * f.ld / 4; e += SVD_THREADS) dst[e] = src[e];
						const float* nsrc = f.nrm(buf, slot);
						float* ndst = cluster.map_shared_rank(f.nrm(buf ^ 1, slot2), (unsigned)pi2);
						for (int e = tid; e < nc; e += SVD_THREADS) ndst[e] = nsrc[e];
					}
					cluster.sync();
					buf ^= 1;
					if (cyc) cyc[10] += clock64() - cx;
				}
			}
			bool conv;
			if (cf > 1) conv = __ldcg(xs.flags32 + sweep) == 0;
			else
			{
				conv = *local_rot == 0;
				__syncthreads();
			}
			if (conv)
			{
				done32 = sweep + 1;
				break;
			}
		}
		if (cyc) cyc[2] += done32;
		// V (FP32) to global memory, column g at V + g r
		round_groups(0, rank, f.nm, A, B);
		for (int slot = 0; slot < 2; slot++)
		{
			const int x = slot ? B : A, nc = f.cnt(x);
			const float* src = f.col(buf, slot, 0);
			for (i64 e = tid; e < (i64)nc * r; e += SVD_THREADS)
			{
				const int c = (int)(e / r), i = (int)(e % r);
				xs.V[(i64)(x * f.bs + c) * r + i] = (double)src[(i64)c * f.ld + N + i];
			}
		}
	}
	else if (cf > 1)
	{
		// the barriers of the working CTAs' rounds, and their convergence decision
		for (int sweep = 0; sweep < nsw; sweep++)
		{
			for (int rho = 0; rho < f.nm; rho++) cluster.sync();
			if (__ldcg(xs.flags32 + sweep) == 0) break;
		}
	}
	cluster.sync();
	if (cyc) cyc[4] += clock64() - c0;
}

// ---- FP64 finish of the mixed path: Newton-Schulz, T = R^T V, simultaneous refinement -------
//
// After the FP32 sweeps the columns of R^T V are orthogonal to about N eps_32 (cosines ~1e-5)
// and V to FP32 accuracy. FP64 Jacobi sweeps from there cost ~6.5 n^3 FP64 FMAs each (a pair
// rotation after every inner product, one barrier per step) and GB300 retires two FP64 FMAs per
// clock per SM. This finish does its FP64 work as inner products of whole Gram matrices and applies
// the corrections, which are small, with products accumulated in double-float on the FP32 pipe:
//   1. two Newton-Schulz steps V <- V (I - E / 2), E = V^T V - I (E from FP64 inner products);
//   2. T = R^T V (FP64);
//   3. G = T^T T (FP64 inner products, each pair once). For columns i, j whose squared norms lie
//      apart, the first-order generator X_ij = G_ij / (G_jj - G_ii) (antisymmetric) removes the
//      cosine of the pair to second order; T and V are multiplied by I + X + X^2 / 2, which is
//      orthogonal to O(X^4). Columns whose squared norms lie within a relative gap gamma of their
//      neighbours (a cluster, where the first-order angle would not be small) get X = 0 and are
//      rotated afterwards among themselves by exact one-sided Jacobi rotations (one warp per
//      cluster). gamma = c_max / (2 delta) keeps every first-order angle below delta = 3e-4 for
//      the largest cosine c_max. Repeat until every cosine is within the FP64 sweeps' tolerance
//      (the cosines fall quadratically: ~1e-5, ~1e-10, below eps).
// The scheme is the iterative refinement of a symmetric eigendecomposition of Ogita and Aishima
// (Japan J. Indust. Appl. Math. 35, 2018) applied one-sided to the columns of T. A block whose
// clusters are too wide or too large, or that does not converge in RF_MAX_IT iterations, continues
// with the FP64 sweeps from the current columns (V stays orthogonal to FP64 rounding throughout).

constexpr int RF_MAX_IT = 6;              // refinement iterations before the FP64 sweeps take over
constexpr float RF_DELTA = 3e-4f;         // largest first-order angle outside a cluster
constexpr int RF_CLUSTER_MAX = 16;        // most columns of one cluster
constexpr int RF_CLUSTER_SWEEPS = 8;      // most Jacobi sweeps inside one cluster
constexpr int RF_EDGES_PER_COL = 4;       // capacity of the cluster-edge list, per column

// a double as the pair hi + lo of floats (hi: the leading 24 bits, lo: the next 24), by integer
// operations (a double -> float conversion costs an FP64 instruction on GB300); values below 2^-126
// (far below any entry that matters here) give zero, lo below 2^-126 is dropped
__device__ __forceinline__ float dbl_hi(double x, int& e)
{
	const int hi = __double2hiint(x), lo = __double2loint(x);
	e = ((hi >> 20) & 0x7ff) - 1023;
	if (e < -126) return 0.0f;
	return __int_as_float((hi & (int)0x80000000) | ((e + 127) << 23) | ((hi & 0x000fffff) << 3) | (int)((unsigned)lo >> 29));
}
__device__ __forceinline__ float2 split_hilo(double x)
{
	int e;
	const float h = dbl_hi(x, e);
	if (h == 0.0f || e < -74) return make_float2(h, 0.0f);
	const int lo = __double2loint(x);
	float l = __int2float_rn(lo & 0x1fffffff) * pow2f(e - 52);
	if (__double2hiint(x) < 0) l = -l;
	return make_float2(h, l);
}
__device__ __forceinline__ float dbl_to_f32(double x)
{
	int e;
	return dbl_hi(x, e);
}

// |g|^2 / (a b) in FP32 for a, b > 0 (capped at 1), from mantissas and exponents
__device__ __forceinline__ float cos2_f32(double g, double a, double b)
{
	if (g == 0.0) return 0.0f;
	int eg, ea, eb;
	const float mg = mant_exp(g, eg), ma = mant_exp(a, ea), mb = mant_exp(b, eb);
	const int k2 = 2 * eg - ea - eb;
	if (k2 < -120) return 0.0f;
	if (k2 > 0) return 1.0f;
	return fminf(__fdividef(mg * mg, ma * mb) * pow2f(k2), 1.0f);
}

// n / d in FP32 (d != 0), from mantissas and exponents; |result| < 2^-126 gives 0, large
// results are capped at 2 (they mark a pair that should have been in a cluster)
__device__ __forceinline__ float ratio_f32(double n, double d)
{
	if (n == 0.0) return 0.0f;
	int en, ed;
	const float mn = mant_exp(n, en), md = mant_exp(d, ed);
	const int k = en - ed;
	if (k < -125) return 0.0f;
	float v = k > 0 ? 2.0f : __fdividef(mn, md) * pow2f(k);
	if ((__double2hiint(n) < 0) != (__double2hiint(d) < 0)) v = -v;
	return v;
}

struct Refine {
	// global
	double* G;        // r x r Gram matrix (symmetric; column j at G + j r)
	float* X;         // r x r first-order generator (column j at X + j r)
	double* Tr;       // T row-major, entry (k, i) at Tr + k r + i (the scratch T area)
	double* Vr;       // V row-major (the scratch V area)
	float2* Th;       // T column-major as (hi, lo) pairs, entry (k, i) at Th + i N + k
	float2* Vh;       // V column-major as (hi, lo) pairs, entry (k, i) at Vh + i r + k
	int* gfail;       // per iteration: a first-order angle came out too large
	int* gc2;         // per iteration: largest cos^2 (bits of a non-negative float)
	int* gne;         // per iteration: cluster edges found
	int2* gedges;     // the cluster edges of the current iteration
	// shared
	float* F;         // own columns of the update, leading floats (column jj at F + jj r)
	float* Fl;        // ... and the trailing floats: F + Fl is X + X^2 / 2 exactly
	float* Xo;        // own columns of X
	double* D;        // diagonal of G
	float* key;       // D as floats
	int* cid;         // cluster of each column: its smallest column index
	int* cnt;         // columns per cluster (at the cluster's smallest index)
	int* qidx;        // 2 + index of the non-singleton cluster whose smallest index this is, else 0
	unsigned char* tail;   // 1: among the smallest columns whose squared norms fit the discard budget
	int2* edges;      // cluster edges (pairs whose first-order angle would exceed delta)
	int* memb;        // members of the cluster being rotated (RF_CLUSTER_MAX)
	double* cstage;   // that cluster's columns [T; V] (RF_CLUSTER_MAX records of N + r, stride ldc)
	int* misc;        // [0] non-singleton clusters, [1] failure, [2] edges, [3] labels changed, [4] rotated
	float* red;       // [NWARPS] block reduction
	// own columns
	int A, B, own0, nown;
};

// shared memory (doubles) of the mixed path: the FP64 tour's buffers (the records the finish works
// on, and the fallback sweeps), then the refinement's arrays
__host__ __device__ inline i64 refine_doubles(int N, int cl)
{
	const i64 nblk = 2 * cl, bsmax = (N + nblk - 1) / nblk;
	const i64 bytes = 8 * (i64)N                              // D
	                  + 8 * (i64)RF_CLUSTER_MAX * (2 * N + 1) // cstage
	                  + 3 * 4 * (2 * bsmax * N)               // F, Fl, Xo
	                  + 4 * 4 * (i64)N                        // key, cid, cnt, qidx
	                  + 8 * (i64)RF_EDGES_PER_COL * N         // edges
	                  + 4 * (i64)RF_CLUSTER_MAX               // memb
	                  + 4 * 8 + 4 * NWARPS                    // misc, red
	                  + (i64)N + 16;                          // tail
	return tour_jac_doubles(N, cl) + (bytes + 7) / 8 + 2;
}

__device__ __forceinline__ double* rf_rec(const Tour& t, const Refine& rf, int jj)
{
	return jj < rf.own0 ? t.col(0, 0, jj) : t.col(0, 1, jj - rf.own0);
}
__device__ __forceinline__ int rf_col(const Tour& t, const Refine& rf, int jj)
{
	return jj < rf.own0 ? rf.A * t.bs + jj : rf.B * t.bs + (jj - rf.own0);
}

// own columns to the global copies: row-major FP64 and column-major (hi, lo) pairs; T entries
// only when with_t
__device__ void rf_write_own(const Tour& t, const Refine& rf, bool with_t)
{
	const int tid = threadIdx.x, N = t.N, r = t.r;
	if (with_t)
		for (int e = tid; e < rf.nown * N; e += SVD_THREADS)
		{
			const int jj = e / N, k = e % N, g = rf_col(t, rf, jj);
			const double x = rf_rec(t, rf, jj)[k];
			rf.Tr[(i64)k * r + g] = x;
			rf.Th[(i64)g * N + k] = split_hilo(x);
		}
	for (int e = tid; e < rf.nown * r; e += SVD_THREADS)
	{
		const int jj = e / r, k = e % r, g = rf_col(t, rf, jj);
		const double x = rf_rec(t, rf, jj)[N + k];
		rf.Vr[(i64)k * r + g] = x;
		rf.Vh[(i64)g * r + k] = split_hilo(x);
	}
}

// S_ij = sum_k A_ki A_kj (minus 1 on the diagonal when sub_identity) for the own columns j and
// every i <= j, written to S at (i, j) and (j, i): each pair once over the cluster (the CTA
// holding groups p and 2 cl - 1 - p gets the same share of pairs as every other CTA). A is
// row-major (A + k r + i, len rows), column j is read from the own record at offset off. A warp
// takes 32 consecutive i against one own column; two independent FP64 accumulators.
__device__ double rf_gram(const Tour& t, const Refine& rf, const double* Ar, int len, int off, bool sub_identity,
                          double* S)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, r = t.r;
	const int nchunk = (r + 31) / 32;
	double fl = 0;
	for (int task = warp; task < rf.nown * nchunk; task += NWARPS)
	{
		const int jj = task % rf.nown, c = task / rf.nown;
		const int g = rf_col(t, rf, jj);
		if (32 * c > g) continue;
		const int i = 32 * c + lane;
		const bool valid = i < r && i <= g;
		const double* rec = rf_rec(t, rf, jj) + off;
		const double* a = Ar + (valid ? i : 0);
		// sixteen loads in flight per thread (a warp reads 32 consecutive doubles of a row per load):
		// the loop is bound by L2 latency, not by the FP64 pipe
		double acc[4] = {0.0, 0.0, 0.0, 0.0};
		int k = 0;
		for (; k + 15 < len; k += 16)
		{
			double x[16];
#pragma unroll
			for (int u = 0; u < 16; u++) x[u] = __ldcg(a + (i64)(k + u) * r);
#pragma unroll
			for (int u = 0; u < 16; u++) acc[u & 3] = fma(x[u], rec[k + u], acc[u & 3]);
		}
		for (; k + 7 < len; k += 8)
		{
			double x[8];
#pragma unroll
			for (int u = 0; u < 8; u++) x[u] = __ldcg(a + (i64)(k + u) * r);
#pragma unroll
			for (int u = 0; u < 8; u++) acc[u & 3] = fma(x[u], rec[k + u], acc[u & 3]);
		}
		for (; k < len; k++) acc[0] = fma(__ldcg(a + (i64)k * r), rec[k], acc[0]);
		const double v = ((acc[0] + acc[1]) + (acc[2] + acc[3])) - ((sub_identity && i == g) ? 1.0 : 0.0);
		if (valid)
		{
			S[(i64)i * r + g] = v;
			S[(i64)g * r + i] = v;
		}
		if (lane == 0) fl += 2.0 * len * (double)min(32, g + 1 - 32 * c);
	}
	return fl;
}

// own columns += [T; V] (F + Fl) (rows 0..N-1 of T when with_t, then the r rows of V), the sums
// accumulated in double-float: exact products of the leading floats (fma error term), the
// trailing-float cross terms in FP32, two-sum accumulation; the FP64 record gets hi + lo of the sum
__device__ void rf_update(const Tour& t, const Refine& rf, bool with_t)
{
	const int tid = threadIdx.x, N = t.N, r = t.r;
	constexpr int JB = 8;
	const int row0 = with_t ? 0 : N;
	const int nrows = N + r - row0;
	const int nb = (rf.nown + JB - 1) / JB;
	for (int task = tid; task < nrows * nb; task += SVD_THREADS)
	{
		const int kr = row0 + task % nrows, b = task / nrows;
		const float2* h = kr < N ? rf.Th + kr : rf.Vh + (kr - N);
		const i64 ld = kr < N ? N : r;
		float sh[JB], sl[JB];
#pragma unroll
		for (int q = 0; q < JB; q++) sh[q] = sl[q] = 0.0f;
		const int j0 = b * JB;
		const int nj = min(JB, rf.nown - j0);
#pragma unroll 8
		for (int i = 0; i < r; i++)
		{
			const float2 v = __ldcg(h + (i64)i * ld);
#pragma unroll
			for (int q = 0; q < JB; q++)
			{
				if (q >= nj) break;
				const float f = rf.F[(j0 + q) * r + i], fl = rf.Fl[(j0 + q) * r + i];
				const float p = v.x * f;
				float e = fmaf(v.x, f, -p);
				e = fmaf(v.y, f, e);
				e = fmaf(v.x, fl, e);
				const float s = sh[q] + p;
				const float bp = s - sh[q];
				const float err = (sh[q] - (s - bp)) + (p - bp);
				sh[q] = s;
				sl[q] += err + e;
			}
		}
		for (int q = 0; q < nj; q++)
		{
			double* rec = rf_rec(t, rf, j0 + q);
			rec[kr] = rec[kr] + (make_double(sh[q], 0) + make_double(sl[q], 0));
		}
	}
}

// one-sided Jacobi sweeps inside each non-singleton cluster, one CTA per cluster: the cluster's
// columns [T; V] are staged in shared memory, each round rotates disjoint pairs (one warp per pair,
// circle method), one CTA barrier per round; the columns go back to the global row-major copies.
// Returns the FP64 flops (counted on lane 0 of each warp).
__device__ double rf_cluster_jacobi(const Tour& t, const Refine& rf, int cl, int rank, float tol2)
{
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, N = t.N, r = t.r;
	const int len = N + r, ldc = len | 1;
	double fl = 0;
	const int ncl = rf.misc[0];
	for (int q = rank; q < ncl; q += cl)
	{
		if (warp == 0)
		{
			// the cluster's smallest column, then its members in increasing order
			int root = -1;
			for (int i = lane; i < r; i += 32)
				if (rf.qidx[i] == 2 + q) root = i;
			for (int o = 16; o > 0; o >>= 1) root = max(root, __shfl_xor_sync(0xffffffffu, root, o));
			int c = 0;
			for (int base = 0; base < r; base += 32)
			{
				const int i = base + lane;
				const bool in = root >= 0 && i < r && rf.cid[i] == root;
				const unsigned m = __ballot_sync(0xffffffffu, in);
				const int at = c + __popc(m & ((1u << lane) - 1));
				if (in && at < RF_CLUSTER_MAX) rf.memb[at] = i;
				c += __popc(m);
			}
			if (lane == 0) rf.misc[5] = min(c, RF_CLUSTER_MAX);
		}
		__syncthreads();
		const int c = rf.misc[5];
		for (int e = tid; e < c * len; e += SVD_THREADS)
		{
			const int m = e / len, k = e % len, col = rf.memb[m];
			rf.cstage[(i64)m * ldc + k] = k < N ? __ldcg(rf.Tr + (i64)k * r + col) : __ldcg(rf.Vr + (i64)(k - N) * r + col);
		}
		__syncthreads();
		const int cpad = c + (c & 1);
		for (int sweep = 0; sweep < RF_CLUSTER_SWEEPS; sweep++)
		{
			if (tid == 0) rf.misc[4] = 0;
			__syncthreads();
			for (int rnd = 0; rnd < cpad - 1; rnd++)
			{
				int pa, pb;
				if (warp < cpad / 2)
				{
					round_robin_pair(rnd, warp, cpad, pa, pb);
					if (pb < c)
					{
						double* x = rf.cstage + (i64)pa * ldc;
						double* y = rf.cstage + (i64)pb * ldc;
						double al = 0, be = 0, ga = 0;
						for (int k = lane; k < N; k += 32)
						{
							al = fma(x[k], x[k], al);
							be = fma(y[k], y[k], be);
							ga = fma(x[k], y[k], ga);
						}
						al = warp_sum(al);
						be = warp_sum(be);
						ga = warp_sum(ga);
						double tau, sn, tn;
						float c2;
						if (lane == 0) fl += 6.0 * N;
						if (al > 0.0 && be > 0.0 && rotation_params(al, be, ga, tol2, tau, sn, tn, c2))
						{
							for (int k = lane; k < len; k += 32)
							{
								const double x1 = fma(-tau, y[k], x[k]);
								const double y1 = fma(sn, x1, y[k]);
								x[k] = fma(-tau, y1, x1);
								y[k] = y1;
							}
							if (lane == 0)
							{
								rf.misc[4] = 1;
								fl += 6.0 * len;
							}
						}
					}
				}
				__syncthreads();
			}
			const bool any = rf.misc[4] != 0;
			__syncthreads();
			if (!any) break;
		}
		for (int e = tid; e < c * len; e += SVD_THREADS)
		{
			const int m = e / len, k = e % len, col = rf.memb[m];
			const double v = rf.cstage[(i64)m * ldc + k];
			if (k < N) __stcg(rf.Tr + (i64)k * r + col, v);
			else __stcg(rf.Vr + (i64)(k - N) * r + col, v);
		}
		__syncthreads();
	}
	return fl;
}

// Steps 1-3 above on the cluster. On entry the FP32 phase has left V (r x r, column g at
// xs.V + g r) in global memory. tail2: the caller discards every singular value whose square is
// below this (scaled as B here; 0: none), so the mutual rotations of the smallest columns whose
// squared norms sum to at most tail2 are skipped. On return buffer 0 of the FP64 tour holds this
// CTA's round-0 records [T | V]; the return value says whether the refinement converged (the same
// on every CTA of the cluster); if not, the FP64 sweeps continue from those records.
__device__ bool finish_mixed(cg::cluster_group& cluster, const Tour& t, double* smem, const SvdScratch& xs, int M,
                             int cl, int rank, bool refine, float tail2, double& flops, long long* cyc, int& iters)
{
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int N = t.N, r = t.r;
	const long long c0 = cyc ? clock64() : 0;
	Refine rf;
	round_groups(0, rank, t.nm, rf.A, rf.B);
	rf.own0 = t.cnt(rf.A);
	rf.nown = rf.own0 + t.cnt(rf.B);
	rf.G = xs.G;
	rf.X = (float*)(xs.G + (i64)N * N);
	rf.Th = (float2*)(xs.G + (i64)N * N + ((i64)N * N + 1) / 2);
	rf.Vh = rf.Th + (i64)N * N;
	rf.gfail = (int*)(rf.Vh + (i64)N * N);
	rf.gc2 = rf.gfail + 8;
	rf.gne = rf.gfail + 16;
	rf.gedges = (int2*)(rf.gfail + 24);
	rf.Tr = xs.T;
	rf.Vr = xs.V;
	{
		char* p = (char*)(smem + tour_jac_doubles(N, cl));
		rf.D = (double*)p;
		p += 8 * (i64)N;
		rf.cstage = (double*)p;
		p += 8 * (i64)RF_CLUSTER_MAX * (2 * N + 1);
		rf.edges = (int2*)p;
		p += 8 * (i64)RF_EDGES_PER_COL * N;
		rf.F = (float*)p;
		p += 4 * (i64)(2 * t.bsmax) * N;
		rf.Fl = (float*)p;
		p += 4 * (i64)(2 * t.bsmax) * N;
		rf.Xo = (float*)p;
		p += 4 * (i64)(2 * t.bsmax) * N;
		rf.key = (float*)p;
		p += 4 * (i64)N;
		rf.cid = (int*)p;
		p += 4 * (i64)N;
		rf.cnt = (int*)p;
		p += 4 * (i64)N;
		rf.qidx = (int*)p;
		p += 4 * (i64)N;
		rf.memb = (int*)p;
		p += 4 * (i64)RF_CLUSTER_MAX;
		rf.misc = (int*)p;
		p += 4 * 8;
		rf.red = (float*)p;
		p += 4 * NWARPS;
		rf.tail = (unsigned char*)p;
	}
	double fl = 0;

	// ---- 1. Newton-Schulz on V: own columns from the FP32 phase's output ----
	for (int e = tid; e < rf.nown * N; e += SVD_THREADS)
	{
		const int jj = e / N, k = e % N;
		rf_rec(t, rf, jj)[N + k] = k < r ? __ldcg(xs.V + (i64)rf_col(t, rf, jj) * r + k) : 0.0;
	}
	if (rank == 0 && tid < 24) rf.gfail[tid] = 0;        // failure flags, cosines, edge counts
	cluster.sync();                              // xs.V is read before its row-major overwrite
	for (int step = 0; step < 2; step++)
	{
		rf_write_own(t, rf, false);
		cluster.sync();
		fl += rf_gram(t, rf, rf.Vr, r, N, true, rf.G);
		cluster.sync();
		for (int e = tid; e < rf.nown * r; e += SVD_THREADS)
		{
			const int jj = e / r, i = e % r;
			rf.F[jj * r + i] = -0.5f * dbl_to_f32(__ldcg(rf.G + (i64)rf_col(t, rf, jj) * r + i));
			rf.Fl[jj * r + i] = 0.0f;
		}
		__syncthreads();
		rf_update(t, rf, false);
		cluster.sync();                          // every CTA has read the (hi, lo) pairs
	}

	// ---- 2. T = R^T V for the own columns (R_ki = W_ik, k <= i), FP64 ----
	// one task per (32 rows of T, own column): a lane forms one entry, its k loop in order over its
	// row of R (column i of W, read from L2); the tasks go round the warps so that the FP64 work of
	// the long rows (row i takes i + 1 terms) is spread over every sub-partition
	const long long ct = cyc ? clock64() : 0;
	{
		const int ngrp = (N + 31) / 32;
		for (int task = warp; task < ngrp * rf.nown; task += NWARPS)
		{
			const int gi = ngrp - 1 - task / rf.nown, jj = task % rf.nown;
			const int i = 32 * gi + lane;
			double* rec = rf_rec(t, rf, jj);
			const double* v = rec + N;
			if (i < N)
			{
				const int kmax = i < r - 1 ? i : r - 1;
				const double* wi = xs.W + (i64)i * M;
				double acc = 0.0;
#pragma unroll 8
				for (int k = 0; k <= kmax; k++) acc = fma(__ldcg(wi + k), v[k], acc);
				rec[i] = acc;
			}
		}
		if (tid == 0) fl += 2.0 * ((double)N * r - 0.5 * (double)r * r) * rf.nown;
		__syncthreads();
	}
	const long long c1 = cyc ? clock64() : 0;
	if (cyc) cyc[5] += c1 - c0;
	if (cyc) cyc[11] += c1 - ct;
	iters = 0;
	if (!refine)
	{
		if (lane == 0) flops += fl;
		return false;
	}

	// ---- 3. refinement ----
	const float tol2 = (float)((double)N * DBL_EPSILON * (double)N * DBL_EPSILON);
	bool converged = false;
	if (tid == 0) rf.misc[6] = 0;            // largest cluster seen
	__syncthreads();
	int fail = 0;            // why the FP64 sweeps take over: 1 edge list full, 2 labels unsettled,
	                         // 3 cluster too large, 4 first-order angle too large, 5 no convergence
	long long ck = cyc ? clock64() : 0;
	auto lap = [&](int slot) {
		if (cyc)
		{
			const long long now = clock64();
			cyc[slot] += now - ck;
			ck = now;
		}
	};
	for (int it = 0; it < RF_MAX_IT; it++)
	{
		rf_write_own(t, rf, true);
		cluster.sync();
		fl += rf_gram(t, rf, rf.Tr, N, 0, false, rf.G);
		cluster.sync();
		lap(6);
		// diagonal; the discarded tail: the smallest columns whose squared norms sum to at most tail2
		// (every CTA computes the same sets and values from the same global G)
		for (int i = tid; i < r; i += SVD_THREADS)
		{
			const double d = __ldcg(rf.G + (i64)i * r + i);
			rf.D[i] = d;
			rf.key[i] = dbl_to_f32(d);
		}
		__syncthreads();
		for (int i = tid; i < r; i += SVD_THREADS)
		{
			// squared norms up to and including column i in increasing order (ties by index)
			const float ki = rf.key[i];
			float below = 0.0f;
			for (int k = 0; k < r; k++)
			{
				const float kk = rf.key[k];
				if (kk < ki || (kk == ki && k <= i)) below += kk;
			}
			rf.tail[i] = below <= tail2 ? 1 : 0;
		}
		__syncthreads();
		// the pairs (i, g), i < g, of the own columns g (each pair once over the cluster): largest
		// cosine over the pairs not both in the tail, and the cluster edges, pairs (not both in the
		// tail) whose first-order angle |G_ig / (D_g - D_i)| would exceed delta, to global memory
		{
			float c2 = 0.0f;
			for (int e = tid; e < rf.nown * r; e += SVD_THREADS)
			{
				const int jj = e / r, i = e % r, g = rf_col(t, rf, jj);
				if (i >= g || (rf.tail[i] && rf.tail[g])) continue;
				const double gv = __ldcg(rf.G + (i64)g * r + i);
				c2 = fmaxf(c2, cos2_f32(gv, rf.D[i], rf.D[g]));
				if (fabsf(dbl_to_f32(gv)) > RF_DELTA * fabsf(rf.key[g] - rf.key[i]))
				{
					const int at = atomicAdd(rf.gne + it, 1);
					if (at < RF_EDGES_PER_COL * r) rf.gedges[at] = make_int2(i, g);
				}
			}
			for (int o = 16; o > 0; o >>= 1) c2 = fmaxf(c2, __shfl_xor_sync(0xffffffffu, c2, o));
			if (lane == 0 && c2 > 0.0f) atomicMax(rf.gc2 + it, __float_as_int(c2));
		}
		cluster.sync();
		iters = it + 1;
		if (__int_as_float(__ldcg(rf.gc2 + it)) <= tol2)
		{
			converged = true;
			break;
		}
		// clusters: connected components of the edges, labelled by their smallest column
		if (tid == 0) rf.misc[1] = 0;
		for (int i = tid; i < r; i += SVD_THREADS)
		{
			rf.cid[i] = i;
			rf.cnt[i] = 0;
		}
		const int nedge_all = __ldcg(rf.gne + it);
		if (nedge_all > RF_EDGES_PER_COL * r)
		{
			fail = 1;
			break;                                                  // uniform: one global count
		}
		for (int e = tid; e < nedge_all; e += SVD_THREADS) rf.edges[e] = __ldcg(rf.gedges + e);
		__syncthreads();
		const int nedge = nedge_all;
		// minimum-label propagation with pointer jumping (labels are column indices of the same
		// component and only decrease; cid[cid[i]] shortcuts chains, so a component typically
		// settles in a number of rounds logarithmic in its diameter). After k rounds every label is
		// at most the smallest column within k edges, so r + 1 rounds always settle: the outcome is
		// the same on every CTA of the cluster
		bool settled = nedge == 0;
		for (int round = 0; round <= r && !settled; round++)
		{
			if (tid == 0) rf.misc[3] = 0;
			__syncthreads();
			for (int e = tid; e < nedge; e += SVD_THREADS)
			{
				const int2 ed = rf.edges[e];
				const int a = rf.cid[ed.x], b = rf.cid[ed.y];
				if (a != b)
				{
					const int m = min(a, b);
					atomicMin(rf.cid + ed.x, m);
					atomicMin(rf.cid + ed.y, m);
					atomicMin(rf.cid + max(a, b), m);
					rf.misc[3] = 1;
				}
			}
			__syncthreads();
			for (int i = tid; i < r; i += SVD_THREADS)
			{
				const int c = rf.cid[i], cc = rf.cid[c];
				if (cc < c)
				{
					atomicMin(rf.cid + i, cc);
					rf.misc[3] = 1;
				}
			}
			__syncthreads();
			settled = rf.misc[3] == 0;
			__syncthreads();
		}
		if (!settled)
		{
			fail = 2;
			break;
		}
		for (int i = tid; i < r; i += SVD_THREADS) atomicAdd(rf.cnt + rf.cid[i], 1);
		__syncthreads();
		if (warp == 0)
		{
			// index of every non-singleton cluster, in increasing order of its smallest column
			int carry = 0, largest = 0;
			bool big = false;
			for (int base = 0; base < r; base += 32)
			{
				const int i = base + lane;
				const int c = i < r ? rf.cnt[i] : 0;
				const bool multi = c >= 2 && c <= RF_CLUSTER_MAX;
				big = big || c > RF_CLUSTER_MAX;
				largest = max(largest, c);
				const unsigned m = __ballot_sync(0xffffffffu, multi);
				if (i < r) rf.qidx[i] = multi ? 2 + carry + __popc(m & ((1u << lane) - 1)) : 0;
				carry += __popc(m);
			}
			big = __any_sync(0xffffffffu, big);
			for (int o = 16; o > 0; o >>= 1) largest = max(largest, __shfl_xor_sync(0xffffffffu, largest, o));
			if (lane == 0)
			{
				rf.misc[0] = carry;
				rf.misc[1] = big ? 1 : 0;
				rf.misc[6] = max(rf.misc[6], largest);
			}
		}
		__syncthreads();
		// a component larger than RF_CLUSTER_MAX: the FP64 sweeps take over (applying this iteration's
		// first-order step to the other pairs first was measured not to save any of their sweeps)
		if (rf.misc[1])
		{
			fail = 3;
			break;
		}
		// first-order generator, own columns (zero inside a cluster and between tail columns)
		for (int e = tid; e < rf.nown * r; e += SVD_THREADS)
		{
			const int jj = e / r, i = e % r, g = rf_col(t, rf, jj);
			float x = 0.0f;
			if (i != g && rf.cid[i] != rf.cid[g] && !(rf.tail[i] && rf.tail[g]))
			{
				const double den = rf.D[g] - rf.D[i];
				x = den != 0.0 ? ratio_f32(__ldcg(rf.G + (i64)g * r + i), den) : 2.0f;
				// should have been an edge (float rounding of the edge test): the FP64 sweeps take over
				if (fabsf(x) > 4.0f * RF_DELTA) atomicOr(rf.gfail + it, 1);
			}
			rf.Xo[jj * r + i] = x;
			rf.X[(i64)g * r + i] = x;
		}
		cluster.sync();
		lap(7);
		if (__ldcg(rf.gfail + it))
		{
			fail = 4;
			break;
		}
		// F + Fl = X + X^2 / 2 exactly (two-sum) for the own columns ((X^2)_ij = sum_k X_ik X_kj,
		// X_ik at X + k r + i): the antisymmetric X stays exact in F + Fl
		// one thread per row i and up to XB own columns at a time: each entry X_ik is loaded once
		// for all of them (eight loads in flight)
		{
			constexpr int XB = 8;
			const int nb = (rf.nown + XB - 1) / XB;
			for (int e = tid; e < nb * r; e += SVD_THREADS)
			{
				const int b = e / r, i = e % r, j0 = b * XB, nj = min(XB, rf.nown - j0);
				float acc[XB];
#pragma unroll
				for (int q = 0; q < XB; q++) acc[q] = 0.0f;
				int k = 0;
				for (; k + 7 < r; k += 8)
				{
					float xv[8];
#pragma unroll
					for (int u = 0; u < 8; u++) xv[u] = __ldcg(rf.X + (i64)(k + u) * r + i);
#pragma unroll
					for (int q = 0; q < XB; q++)
						if (q < nj)
						{
							const float* xo = rf.Xo + (j0 + q) * r + k;
#pragma unroll
							for (int u = 0; u < 8; u++) acc[q] = fmaf(xv[u], xo[u], acc[q]);
						}
				}
				for (; k < r; k++)
				{
					const float xv = __ldcg(rf.X + (i64)k * r + i);
#pragma unroll
					for (int q = 0; q < XB; q++)
						if (q < nj) acc[q] = fmaf(xv, rf.Xo[(j0 + q) * r + k], acc[q]);
				}
#pragma unroll
				for (int q = 0; q < XB; q++)
					if (q < nj)
					{
						const int jj = j0 + q;
						const float x = rf.Xo[jj * r + i], h = 0.5f * acc[q];
						const float sum = x + h, bp = sum - x;
						rf.F[jj * r + i] = sum;
						rf.Fl[jj * r + i] = (x - (sum - bp)) + (h - bp);
					}
			}
		}
		__syncthreads();
		rf_update(t, rf, true);
		cluster.sync();                          // every CTA has read the global copies
		lap(8);
		if (rf.misc[0] > 0)
		{
			rf_write_own(t, rf, true);
			cluster.sync();
			fl += rf_cluster_jacobi(t, rf, cl, rank, tol2);
			cluster.sync();
			for (int e = tid; e < rf.nown * (N + r); e += SVD_THREADS)
			{
				const int jj = e / (N + r), k = e % (N + r), g = rf_col(t, rf, jj);
				rf_rec(t, rf, jj)[k] = k < N ? __ldcg(rf.Tr + (i64)k * r + g) : __ldcg(rf.Vr + (i64)(k - N) * r + g);
			}
			__syncthreads();
			lap(9);
		}
	}
	if (!converged && fail == 0) fail = 5;
	iters += 10 * fail + 1000 * min(rf.misc[6], 999);
	// every CTA has finished reading the global copies before the columns go back (the write-back
	// after the sweeps reuses the T and V areas)
	cluster.sync();
	if (cyc) cyc[0] += clock64() - c1;
	if (lane == 0) flops += fl;
	return converged;
}

__global__ void __launch_bounds__(SVD_THREADS, 1)
k_svd_tour(const SvdDesc* __restrict__ descs, int first, const double* __restrict__ a, double* __restrict__ u,
           double* __restrict__ s, double* __restrict__ vh, double* __restrict__ scratch, int* __restrict__ status,
           double* __restrict__ flops, int cl, int smem_bytes, unsigned long long* __restrict__ phase_ts, int f32_min,
           int f32_cl, int refine, double tail2, int f32_sweeps, float f32_cos)
{
	extern __shared__ __align__(16) double smem[];
	cg::cluster_group cluster = cg::this_cluster();
	const int rank = (int)cluster.block_rank();
	const int blk = first + blockIdx.x / cl;
	const SvdDesc d = descs[blk];
	const int m = d.m, n = d.n;
	const bool tall = m >= n;
	const int M = tall ? m : n, N = tall ? n : m;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const SvdScratch xs = scratch_layout(scratch + d.w_off, M, N);
	const double* ab = a + d.a_off;

	for (int e = rank * SVD_THREADS + tid; e < SVD_MAX_SWEEPS; e += cl * SVD_THREADS) xs.flags[e] = 0;
	for (int e = rank * SVD_THREADS + tid; e < SVD_F32_SWEEPS_MAX; e += cl * SVD_THREADS) xs.flags32[e] = 0;
	for (int e = rank * SVD_THREADS + tid; e < SVD_MAX_SWEEPS; e += cl * SVD_THREADS) xs.cmax[e] = 0;
	const bool stamp = phase_ts && rank == 0 && tid == 0;
	if (stamp) phase_ts[SVD_PHASE_SLOTS * blk] = globaltimer();

	// ---- 1. pivoted QR of B scaled to a Frobenius norm in [1/2, 1): over the cluster, or on the
	// single CTA of a one-CTA cluster ----
	long long qcyc[5] = {0, 0, 0, 0, 0};
	if (cl > 1) qr_pivoted_cluster(cluster, smem, ab, tall, n, M, N, cl, xs, phase_ts && tid == 0 && rank == 1 ? qcyc : nullptr);
	else
	{
		__shared__ double red[NWARPS];
		double part = 0;
		for (i64 e = tid; e < (i64)M * N; e += SVD_THREADS)
		{
			const i64 col = e / M, row = e % M;
			const double x = tall ? ab[row * n + col] : ab[col * n + row];
			part = fma(x, x, part);
		}
		for (int j = tid; j < N; j += SVD_THREADS) xs.perm[j] = j;
		const double total = block_sum(part, red);
		// exact power-of-two scaling: keeps products of squared column norms far from underflow
		int ex = 0;
		if (total > 0) frexp(sqrt(total), &ex);
		const double sc = ldexp(1.0, -ex);
		// the factorisation runs in shared memory when the block fits, then W goes to global memory
		const bool in_smem = (i64)M * N * 8 <= (i64)smem_bytes;
		double* Wq = in_smem ? smem : xs.W;
		for (i64 e = tid; e < (i64)M * N; e += SVD_THREADS)
		{
			const i64 col = e / M, row = e % M;
			Wq[e] = sc * (tall ? ab[row * n + col] : ab[col * n + row]);
		}
		__syncthreads();
		const int rr = qr_pivoted_cta(Wq, M, N, xs.nrm, xs.sig, xs.tau, xs.perm, DBL_EPSILON * DBL_EPSILON * total * sc * sc);
		if (in_smem)
			for (i64 e = tid; e < (i64)M * N; e += SVD_THREADS) xs.W[e] = Wq[e];
		if (tid == 0)
		{
			xs.misc[0] = (double)rr;
			xs.misc[1] = total;
			xs.misc[2] = ldexp(1.0, ex);
		}
	}
	cluster.sync();
	const int r = (int)__ldcg(xs.misc);
	if (stamp) phase_ts[SVD_PHASE_SLOTS * blk + 1] = globaltimer();

	// ---- 2. one-sided Jacobi on R^T (N x r), block-pair tournament over the cluster ----
	Tour t;
	t.nblk = 2 * cl;
	t.nm = t.nblk - 1;
	t.r = r;
	t.N = N;
	t.ld = 2 * N;
	t.bsmax = (N + t.nblk - 1) / t.nblk;
	t.bs = r > 0 ? (r + t.nblk - 1) / t.nblk : 1;
	t.sm = smem;
	StepBuf sb;
	sb.local_rot = (int*)(smem + (i64)4 * t.bsmax * t.ld + 4 * t.bsmax);
	sb.max_c2 = sb.local_rot + 1;

	int A, B;
	double jflops = 0;                                 // counted on lane 0 of every warp
	long long jsteps = 0;                              // the FP64 sweeps' share, as an integer
	// FP64 steps (or the refinement), FP64 sweeps, FP32 sweeps, exchanges, FP32 cycles, hand-over cycles;
	// refinement cycles: Gram matrices, analysis (cosines, tail, clusters, generator), updates, clusters
	long long cyc_acc[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
	// counted on the second CTA: the first one holds the last column group, often short or empty
	const bool count = phase_ts && tid == 0 && rank == (cl > 1 ? 1 : 0);
	long long* cyc = count ? cyc_acc : nullptr;
	// FP32 sub-cluster: the requested size, or larger until its column groups fit
	int cf = f32_cl < cl ? f32_cl : cl;
	while (cf < cl && f32_tour_bytes(N, r, cf) > (i64)smem_bytes) cf *= 2;
	const bool mixed = f32_min > 0 && r >= f32_min && 8 * refine_doubles(N, cl) <= (i64)smem_bytes &&
	                   f32_tour_bytes(N, r, cf) <= (i64)smem_bytes;
	bool refined = false;
	int rf_iters = 0;
	if (mixed)
	{
		precondition_f32(cluster, t, smem, xs, M, cf, rank, f32_sweeps, f32_cos, cyc);
		const double us = __ldcg(xs.misc + 2);
		refined = finish_mixed(cluster, t, smem, xs, M, cl, rank, refine != 0, (float)(tail2 / (us * us)), jflops, cyc,
		                       rf_iters);
	}
	else
	{
		round_groups(0, rank, t.nm, A, B);
		// column g of T is row g of R (upper triangle of W); column g of V is e_g
		for (int slot = 0; slot < 2; slot++)
		{
			const int x = slot ? B : A;
			double* dst = t.col(0, slot, 0);
			for (i64 e = tid; e < (i64)t.cnt(x) * t.ld; e += SVD_THREADS)
			{
				const int c = (int)(e / t.ld), i = (int)(e % t.ld);
				const int g = x * t.bs + c;
				double v;
				if (i < N) v = (i >= g) ? __ldcg(xs.W + (i64)i * M + g) : 0.0;
				else v = (i - N == g) ? 1.0 : 0.0;
				dst[e] = v;
			}
		}
		__syncthreads();
	}

	const float tol2 = (float)((double)N * DBL_EPSILON * (double)N * DBL_EPSILON);
	int buf = 0, sweep = 0;
	bool converged = r <= 1 || refined;
	for (; sweep < SVD_MAX_SWEEPS && !converged; sweep++)
	{
		round_groups(0, rank, t.nm, A, B);
		// exact squared norms of the columns held here
		for (int slot = 0; slot < 2; slot++)
		{
			const int nc = t.cnt(slot ? B : A);
			for (int c = warp; c < nc; c += NWARPS)
			{
				const double* col = t.col(buf, slot, c);
				double acc = 0;
				for (int i = lane; i < N; i += 32) acc = fma(col[i], col[i], acc);
				acc = warp_sum(acc);
				if (lane == 0) t.nrm(buf, slot)[c] = acc;
			}
		}
		if (tid == 0)
		{
			*sb.local_rot = 0;
			*sb.max_c2 = 0;
		}
		__syncthreads();
		for (int rho = 0; rho < t.nm; rho++)
		{
			round_groups(rho, rank, t.nm, A, B);
			const int cA = t.cnt(A), cB = t.cnt(B);
			if (rho == 0)
			{
				const int npad = t.bs + (t.bs & 1);
				for (int st = 0; st < npad - 1; st++) jacobi_step(t, buf, 0, st, cA, cB, npad, tol2, sb, cyc, jsteps);
			}
			for (int st = 0; st < t.bs; st++) jacobi_step(t, buf, 1, st, cA, cB, 0, tol2, sb, cyc, jsteps);
			if (cl > 1)
			{
				const long long cx = cyc ? clock64() : 0;
				// jacobi_step ended with a CTA barrier: this round's rotations are complete
				// one global flag per sweep, raised after the sweep's last round by any CTA that rotated
				if (tid == 0 && rho == t.nm - 1)
				{
					if (*sb.local_rot) atomicOr(xs.flags + sweep, 1);
					atomicMax(xs.cmax + sweep, *sb.max_c2);
				}
				const int rho1 = (rho + 1) % t.nm;
				for (int slot = 0; slot < 2; slot++)
				{
					const int x = slot ? B : A, nc = t.cnt(x);
					int pi2, slot2;
					group_owner(x, rho1, t.nm, pi2, slot2);
					const double2* src = (const double2*)t.col(buf, slot, 0);
					double2* dst = (double2*)cluster.map_shared_rank(t.col(buf ^ 1, slot2, 0), (unsigned)pi2);
					for (i64 e = tid; e < (i64)nc * t.ld / 2; e += SVD_THREADS) dst[e] = src[e];
					const double* nsrc = t.nrm(buf, slot);
					double* ndst = cluster.map_shared_rank(t.nrm(buf ^ 1, slot2), (unsigned)pi2);
					for (int e = tid; e < nc; e += SVD_THREADS) ndst[e] = nsrc[e];
				}
				cluster.sync();
				buf ^= 1;
				if (cyc) cyc[3] += clock64() - cx;
			}
		}
		// Converged when the sweep rotated nothing, or when every pair of the sweep had cos^2 <=
		// eps / 4: a rotation by an angle of about cos_pq changes the cosine of a pair (p, r) by about
		// cos_pq cos_qr (whatever the column norms), so after such a sweep every cosine is below
		// 2 N (eps / 4) <= N eps / 2, within the tolerance, and the confirming sweep is skipped.
		const int skip_bits = __float_as_int(0.25f * (float)DBL_EPSILON);
		if (cl > 1) converged = __ldcg(xs.flags + sweep) == 0 || __ldcg(xs.cmax + sweep) <= skip_bits;
		else
		{
			converged = *sb.local_rot == 0 || *sb.max_c2 <= skip_bits;
			__syncthreads();
		}
	}
	// columns back in global memory (arrangement of round 0), singular values as column norms
	round_groups(0, rank, t.nm, A, B);
	for (int slot = 0; slot < 2; slot++)
	{
		const int x = slot ? B : A, nc = t.cnt(x);
		const double* src = t.col(buf, slot, 0);
		for (i64 e = tid; e < (i64)nc * t.ld; e += SVD_THREADS)
		{
			const int c = (int)(e / t.ld), i = (int)(e % t.ld);
			const int g = x * t.bs + c;
			if (i < N) xs.T[(i64)g * N + i] = src[e];
			else if (i - N < r) xs.V[(i64)g * r + (i - N)] = src[e];
		}
		for (int c = warp; c < nc; c += NWARPS)
		{
			const double* col = t.col(buf, slot, c);
			double acc = 0;
			for (int i = lane; i < N; i += 32) acc = fma(col[i], col[i], acc);
			acc = warp_sum(acc);
			if (lane == 0) xs.sig[x * t.bs + c] = sqrt(acc);
		}
	}
	jflops += (double)jsteps;
	if (lane == 0 && jflops > 0) atomicAdd(flops, jflops);
	if (rank == 0 && tid == 0)
	{
		atomicMax(status + 1, sweep);
		if (!converged) atomicExch(status, -1);
	}
	cluster.sync();
	if (stamp) phase_ts[SVD_PHASE_SLOTS * blk + 2] = globaltimer();
	if (count)
	{
		cyc_acc[1] = sweep;
		for (int i = 0; i < 6; i++) phase_ts[SVD_PHASE_SLOTS * blk + 4 + i] = (unsigned long long)cyc_acc[i];
		for (int i = 0; i < 5; i++) phase_ts[SVD_PHASE_SLOTS * blk + 10 + i] = (unsigned long long)qcyc[i];
		phase_ts[SVD_PHASE_SLOTS * blk + 15] = (unsigned long long)(rf_iters + (mixed && !refined ? 100 : 0));
		for (int i = 0; i < 4; i++) phase_ts[SVD_PHASE_SLOTS * blk + 16 + i] = (unsigned long long)cyc_acc[6 + i];
		phase_ts[SVD_PHASE_SLOTS * blk + 20] = (unsigned long long)cyc_acc[10];
		phase_ts[SVD_PHASE_SLOTS * blk + 21] = (unsigned long long)cyc_acc[11];
	}

	// ---- 3. outputs: L = Q V (M x r) by the r reflectors applied to [V_c; 0], Rf = P T Sigma^-1 ----
	const double unscale = __ldcg(xs.misc + 2);
	const int kk = N;                                     // min(m, n): width of the factor blocks
	// one warp per column of V; the reflectors are staged in shared memory SVD_OUT_RC at a time (in
	// the order they are applied, last first), so the serial chain of each column reads shared
	// memory instead of L2
	double* ub = smem + (i64)warp * M;
	// as many reflectors per round as the shared memory holds (at least 4, at most SVD_OUT_RC)
	const i64 room = ((i64)smem_bytes / 8 - (i64)NWARPS * M - SVD_OUT_RC) / M;
	const int rc = room < 1 ? 1 : (room > SVD_OUT_RC ? SVD_OUT_RC : (int)room);
	double* ws = smem + (i64)NWARPS * M;                  // staged reflectors, unit leading entry
	double* ts = ws + (i64)rc * M;                        // their scalars
	const int nround = (r + cl * NWARPS - 1) / (cl * NWARPS);
	for (int round = 0; round < nround; round++)
	{
		const int c = rank * NWARPS + warp + round * cl * NWARPS;
		const bool has = c < r;
		if (has)
			for (int i = lane; i < M; i += 32) ub[i] = i < r ? __ldcg(xs.V + (i64)c * r + i) : 0.0;
		for (int k1 = r - 1; k1 >= 0; k1 -= rc)
		{
			const int k0 = k1 - rc + 1 > 0 ? k1 - rc + 1 : 0;
			__syncthreads();
			for (i64 e = tid; e < (i64)(k1 - k0 + 1) * M; e += SVD_THREADS)
			{
				const int k = k0 + (int)(e / M), i = (int)(e % M);
				ws[e] = i > k ? __ldcg(xs.W + (i64)k * M + i) : (i == k ? 1.0 : 0.0);
			}
			for (int e = tid; e <= k1 - k0; e += SVD_THREADS) ts[e] = __ldcg(xs.tau + k0 + e);
			__syncthreads();
			if (!has) continue;
			for (int k = k1; k >= k0; k--)
			{
				const double tk = ts[k - k0];
				if (__double_as_longlong(tk) == 0) continue;     // tk >= +0: bits zero only at zero
				const double* wk = ws + (i64)(k - k0) * M;
				double acc = 0;
				for (int i = k + lane; i < M; i += 32) acc = fma(wk[i], ub[i], acc);
				acc = warp_sum(acc) * tk;
				for (int i = k + lane; i < M; i += 32) ub[i] -= acc * wk[i];
				__syncwarp();
			}
		}
		if (!has) continue;
		const double sc = __ldcg(xs.sig + c);
		int cnt = 0;
		for (int c2 = lane; c2 < r; c2 += 32)
		{
			const double v = __ldcg(xs.sig + c2);
			cnt += (v > sc || (v == sc && c2 < c)) ? 1 : 0;
		}
		const int pos = (int)__reduce_add_sync(0xffffffffu, (unsigned)cnt);
		if (lane == 0) s[d.s_off + pos] = sc * unscale;
		const double inv = sc > 0 ? 1.0 / sc : 0.0;
		for (int i = lane; i < M; i += 32)
		{
			if (tall) u[d.u_off + (i64)i * kk + pos] = ub[i];       // u: m x k, row i
			else vh[d.v_off + (i64)pos * n + i] = ub[i];            // vh: k x n, column i
		}
		const double* tc = xs.T + (i64)c * N;
		for (int j = lane; j < N; j += 32)
		{
			const double x = __ldcg(tc + j) * inv;
			const int pj = __ldcg(xs.perm + j);
			if (tall) vh[d.v_off + (i64)pos * n + pj] = x;         // vh: k x n
			else u[d.u_off + (i64)pj * kk + pos] = x;               // u: m x k
		}
		__syncwarp();
	}
	if (phase_ts)
	{
		cluster.sync();
		if (stamp) phase_ts[SVD_PHASE_SLOTS * blk + 3] = globaltimer();
	}
}

// ---- global-memory variant for blocks too large for shared memory ----
__global__ void __launch_bounds__(SVD_THREADS)
k_svd_global(const SvdDesc* __restrict__ descs, int first, const double* __restrict__ a, double* __restrict__ u,
              double* __restrict__ s, double* __restrict__ vh, double* __restrict__ scratch, int* __restrict__ status,
              double tiny_rel2, double* __restrict__ tail, int cl)
{
	cg::cluster_group cluster = cg::this_cluster();
	const int rank = (int)cluster.block_rank();
	const SvdDesc d = descs[first + blockIdx.x / cl];
	const int m = d.m, n = d.n;
	const bool tall = m >= n;
	const int M = tall ? m : n, N = tall ? n : m;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int gtid = rank * SVD_THREADS + tid, gstride = cl * SVD_THREADS;
	const int gwarp = rank * NWARPS + warp, gwarps = cl * NWARPS;

	double* W = scratch + d.w_off;                        // M x N: B, then R and the Householder vectors
	double* Q = W + (i64)M * N;                           // M x N: explicit Q (first r columns)
	double* T = Q + (i64)M * N;                           // N x N: R^T, orthogonalised by Jacobi
	double* V = T + (i64)N * N;                           // N x N: Jacobi rotations (r x r used)
	double* nrm = V + (i64)N * N;                         // N squared column norms
	double* tau = nrm + N;                                // N Householder scalars
	double* sig = tau + N;                                // N singular values
	double* misc = sig + N;                               // [0] rank, [1] Frobenius norm^2
	volatile int* flags = (volatile int*)(misc + 2);      // one "rotated" flag per sweep
	unsigned long long* amax = (unsigned long long*)(misc + 2) + SVD_MAX_SWEEPS;
	int* perm = (int*)(amax + SVD_MAX_SWEEPS);            // N column permutation
	const double* ab = a + d.a_off;

	for (int e = gtid; e < SVD_MAX_SWEEPS; e += gstride)
	{
		flags[e] = 0;
		amax[e] = 0ull;
	}
	// ---- 1. pivoted QR on the cluster's first CTA ----
	if (rank == 0)
	{
		__shared__ double red[NWARPS];
		double part = 0;
		for (i64 e = tid; e < (i64)M * N; e += SVD_THREADS)
		{
			const i64 col = e / M, row = e % M;
			const double x = tall ? ab[row * n + col] : ab[col * n + row];
			W[e] = x;
			part = fma(x, x, part);
		}
		for (int j = tid; j < N; j += SVD_THREADS) perm[j] = j;
		const double total = block_sum(part, red);
		__syncthreads();
		const int r = qr_pivoted_cta(W, M, N, nrm, sig, tau, perm, DBL_EPSILON * DBL_EPSILON * total);
		if (tid == 0)
		{
			misc[0] = (double)r;
			misc[1] = total;
		}
	}
	cluster.sync();
	const int r = (int)__ldcg(misc);

	// ---- 2. one-sided Jacobi on R^T (N x r) over the cluster ----
	for (i64 e = gtid; e < (i64)N * r; e += gstride)
	{
		const int c = (int)(e / N), j = (int)(e % N);
		T[e] = (j >= c) ? __ldcg(W + (i64)j * M + c) : 0.0;
	}
	for (i64 e = gtid; e < (i64)r * r; e += gstride) V[e] = (e / r == e % r) ? 1.0 : 0.0;
	cluster.sync();
	// rotate while the cosine of a pair exceeds N eps; the rank cut of step 1 has removed the
	// columns at the rounding-noise floor, whose cosines would never settle
	const double tol = (double)N * DBL_EPSILON;
	const int np = r + (r & 1);
	int sweep = 0;
	for (; sweep < SVD_MAX_SWEEPS && r > 1; sweep++)
	{
		for (int c = gwarp; c < r; c += gwarps)
		{
			const double* tc = T + (i64)c * N;
			double acc = 0;
			for (int i = lane; i < N; i += 32) { const double x = __ldcg(tc + i); acc = fma(x, x, acc); }
			acc = warp_sum(acc);
			if (lane == 0)
			{
				nrm[c] = acc;
				// non-negative doubles order like their bit patterns
				atomicMax(amax + sweep, (unsigned long long)__double_as_longlong(acc));
			}
		}
		cluster.sync();
		const double cmax = __longlong_as_double((long long)__ldcg(amax + sweep));
		const double tiny = tiny_rel2 * cmax;
		for (int rnd = 0; rnd < np - 1; rnd++)
		{
			for (int pi = gwarp; pi < np / 2; pi += gwarps)
			{
				int p, q;
				round_robin_pair(rnd, pi, np, p, q);
				if (q >= r) continue;
				double* tp = T + (i64)p * N;
				double* tq = T + (i64)q * N;
				double ga = 0;
				for (int i = lane; i < N; i += 32) ga = fma(__ldcg(tp + i), __ldcg(tq + i), ga);
				ga = warp_sum(ga);
				const double al = __ldcg(nrm + p), be = __ldcg(nrm + q);
				if (ga != 0.0 && fmax(al, be) > tiny && fabs(ga) > tol * sqrt(al * be))
				{
					const double zeta = (be - al) / (2.0 * ga);
					const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
					const double c = 1.0 / sqrt(1.0 + t * t);
					const double sn = c * t;
					for (int i = lane; i < N; i += 32)
					{
						const double x = __ldcg(tp + i), y = __ldcg(tq + i);
						tp[i] = c * x - sn * y;
						tq[i] = sn * x + c * y;
					}
					double* vp = V + (i64)p * r;
					double* vq = V + (i64)q * r;
					for (int i = lane; i < r; i += 32)
					{
						const double x = __ldcg(vp + i), y = __ldcg(vq + i);
						vp[i] = c * x - sn * y;
						vq[i] = sn * x + c * y;
					}
					if (lane == 0)
					{
						nrm[p] = al - t * ga;
						nrm[q] = be + t * ga;
						flags[sweep] = 1;
					}
				}
			}
			cluster.sync();
		}
		if (!__ldcg((const int*)flags + sweep)) break;
	}
	if (rank == 0 && tid == 0)
	{
		atomicMax(status + 1, sweep + 1);
		if (sweep >= SVD_MAX_SWEEPS) atomicExch(status, -1);
	}
	for (int c = gwarp; c < r; c += gwarps)
	{
		const double* tc = T + (i64)c * N;
		double acc = 0;
		for (int i = lane; i < N; i += 32) { const double x = __ldcg(tc + i); acc = fma(x, x, acc); }
		acc = warp_sum(acc);
		if (lane == 0)
		{
			sig[c] = sqrt(acc);
			// weight of the directions left unresolved (both partners below the tiny bound)
			if (tiny_rel2 > 0 && acc <= tiny_rel2 * __longlong_as_double((long long)__ldcg(amax)))
				atomicAdd(tail + first + blockIdx.x / cl, acc);
		}
	}

	// ---- 3. explicit Q (M x r) = H_0 ... H_{r-1} E_r over the cluster ----
	for (i64 e = gtid; e < (i64)M * r; e += gstride) Q[e] = (e / M == e % M) ? 1.0 : 0.0;
	cluster.sync();
	for (int k = r - 1; k >= 0; k--)
	{
		const double tk = __ldcg(tau + k);
		const double* wk = W + (i64)k * M;
		if (tk != 0.0)
		{
			for (int j = gwarp; j < r; j += gwarps)
			{
				double* qj = Q + (i64)j * M;
				double acc = 0;
				for (int i = k + lane; i < M; i += 32) acc = fma(i == k ? 1.0 : __ldcg(wk + i), __ldcg(qj + i), acc);
				acc = warp_sum(acc) * tk;
				for (int i = k + lane; i < M; i += 32) qj[i] = __ldcg(qj + i) - acc * (i == k ? 1.0 : __ldcg(wk + i));
			}
		}
		cluster.sync();
	}

	// ---- outputs: L = Q V (M x r), Rf = P T Sigma^-1 (N x r); descending sigma ----
	const int kk = N;                                     // min(m, n): width of the factor blocks
	for (int c = gwarp; c < r; c += gwarps)
	{
		const double sc = __ldcg(sig + c);
		int cnt = 0;
		for (int c2 = lane; c2 < r; c2 += 32)
		{
			const double v = __ldcg(sig + c2);
			cnt += (v > sc || (v == sc && c2 < c)) ? 1 : 0;
		}
		const int pos = (int)__reduce_add_sync(0xffffffffu, (unsigned)cnt);
		if (lane == 0) s[d.s_off + pos] = sc;
		const double inv = sc > 0 ? 1.0 / sc : 0.0;
		const double* vc = V + (i64)c * r;
		const double* tc = T + (i64)c * N;
		for (int i = lane; i < M; i += 32)
		{
			double acc = 0;
			for (int l = 0; l < r; l++) acc = fma(__ldcg(Q + (i64)l * M + i), __ldcg(vc + l), acc);
			if (tall) u[d.u_off + (i64)i * kk + pos] = acc;       // u: m x k, row i
			else vh[d.v_off + (i64)pos * n + i] = acc;            // vh: k x n, column i
		}
		for (int j = lane; j < N; j += 32)
		{
			const double x = __ldcg(tc + j) * inv;
			const int pj = __ldcg(perm + j);
			if (tall) vh[d.v_off + (i64)pos * n + pj] = x;       // vh: k x n
			else u[d.u_off + (i64)pj * kk + pos] = x;             // u: m x k
		}
	}
}

}  // namespace

// ------------------------------------------------------------------------------------
// SVD of one dense block without any device allocation
// ------------------------------------------------------------------------------------
// Some callers cannot allocate device memory while they run: a service whose device memory is
// fully reserved up front by its own pool, or code whose stream must not be stalled by the
// implicit device-wide synchronisation of cudaMalloc / cudaFree. For them the block SVD has a
// variant whose workspace is this fixed array: every GPU that loads the library keeps it
// (4 MiB) until the process exits, and it bounds the block to NOALLOC_SVD_MAX_DIM rows and
// columns. All calls share the array, so calls whose work overlaps on the GPU (for example on
// two streams) race on it and must be serialised by the caller. With lazy module loading (the
// CUDA default), the array's memory and the library's kernels are loaded onto a device by the
// first call there (or by any first use of the library on that device); a caller that reserves
// the rest of the device for its own pool makes that first call before reserving, or sets
// CUDA_MODULE_LOADING=EAGER.

constexpr int NOALLOC_SVD_MAX_DIM = 256;
constexpr i64 NOALLOC_SCRATCH_DOUBLES = (i64)1 << 19;   // 4 MiB

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

namespace {

// layout of the fixed array: descriptor, status[2] + flop counter (as doubles), then the SVD workspace
constexpr i64 NA_DESC = 0;
constexpr i64 NA_STATUS = (sizeof(SvdDesc) + 7) / 8;
constexpr i64 NA_WORK = NA_STATUS + 2;

__global__ void k_noalloc_prepare(double* base, SvdDesc d, double* u, double* s, double* vh)
{
	// the array keeps the previous call's contents: reset everything that must start at zero
	if (blockIdx.x == 0 && threadIdx.x == 0)
	{
		*(SvdDesc*)(base + NA_DESC) = d;
		int* status = (int*)(base + NA_STATUS);
		status[0] = 0;
		status[1] = 0;
		base[NA_STATUS + 1] = 0.0;                  // flop counter
	}
	// factor entries beyond the numerical rank are not written by the SVD kernel
	const i64 k = d.m < d.n ? d.m : d.n;
	const i64 stride = (i64)gridDim.x * blockDim.x;
	for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < (i64)d.m * k; e += stride) u[e] = 0.0;
	for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < k * (i64)d.n; e += stride) vh[e] = 0.0;
	for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < k; e += stride) s[e] = 0.0;
}

__global__ void k_noalloc_finish(const double* base, int* info)
{
	*info = ((const int*)(base + NA_STATUS))[0];
}

}  // namespace

}  // namespace ctg

extern "C" int ctgpu_dense_svd_noalloc(const double* d_a, int m, int n, double* d_u, double* d_s, double* d_vh,
                                       int* d_info, void* stream)
{
	using namespace ctg;
	if (m < 1 || n < 1 || m > NOALLOC_SVD_MAX_DIM || n > NOALLOC_SVD_MAX_DIM)
	{
		fprintf(stderr, "ctgpu_dense_svd_noalloc: block of %d x %d is outside 1..%d rows and columns\n", m, n,
		        NOALLOC_SVD_MAX_DIM);
		return -5;
	}
	if (NA_WORK + svd_scratch_doubles(m, n) > NOALLOC_SCRATCH_DOUBLES) return -5;
	if (!d_a || !d_u || !d_s || !d_vh || !d_info) return -5;
	// an error left by the caller's earlier work is not this call's to consume: report and leave it
	{
		const cudaError_t pending = cudaPeekAtLastError();
		if (pending != cudaSuccess)
		{
			fprintf(stderr, "ctgpu_dense_svd_noalloc: a CUDA error from earlier work is pending (%s); nothing queued\n",
			        cudaGetErrorString(pending));
			return -5;
		}
	}
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -5;
	// device address of the fixed array, taken once per device with that device current
	static double* addr[64] = {nullptr};
	static std::mutex lock;
	{
		std::lock_guard<std::mutex> g(lock);
		if (!addr[dev])
		{
			void* p = nullptr;
			const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
			if (e != cudaSuccess)
			{
				fprintf(stderr, "ctgpu_dense_svd_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
				return -5;
			}
			addr[dev] = (double*)p;
		}
	}
	double* base = addr[dev];
	cudaStream_t st = (cudaStream_t)stream;
	SvdDesc d = {};
	d.a_off = 0;
	d.u_off = 0;
	d.s_off = 0;
	d.v_off = 0;
	d.w_off = 0;
	d.m = m;
	d.n = n;
	// every launch reports its own status (cudaLaunchKernel / cudaLaunchKernelEx return it), so this
	// call never reads or clears the thread's last-error state on behalf of other work
	{
		void* args[] = {&base, &d, &d_u, &d_s, &d_vh};
		const cudaError_t e = cudaLaunchKernel((const void*)k_noalloc_prepare, dim3(64), dim3(256), args, 0, st);
		if (e != cudaSuccess)
		{
			fprintf(stderr, "ctgpu_dense_svd_noalloc: launch failed: %s\n", cudaGetErrorString(e));
			return -5;
		}
	}
	const SvdDesc* descs = (const SvdDesc*)(base + NA_DESC);
	int* status = (int*)(base + NA_STATUS);
	double* flops = base + NA_STATUS + 1;
	try
	{
		const int maxcl = svd_max_cluster(dev);
		launch_svd_group(svd_launch_for(m, n, maxcl, maxcl), 0, 1, descs, d_a, d_u, d_s, d_vh, base + NA_WORK, status,
		                 flops, st);
		const double* cbase = base;
		void* args[] = {(void*)&cbase, &d_info};
		const cudaError_t e = cudaLaunchKernel((const void*)k_noalloc_finish, dim3(1), dim3(1), args, 0, st);
		if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
	}
	catch (const std::exception& ex)
	{
		fprintf(stderr, "ctgpu_dense_svd_noalloc: launch failed: %s\n", ex.what());
		return -5;
	}
	return 0;
}

namespace ctg {

i64 svd_scratch_doubles(int m, int n)
{
	const i64 M = m >= n ? m : n, N = m >= n ? n : m;
	// the larger of the two layouts: global-memory path (W, Q, T, V, nrm, tau, sig, misc, flags +
	// amax, perm) and shared-memory path (W, T, V, nrm, tau, sig, misc, flags, perm); then the
	// refinement's arrays of the mixed path
	return svd_refine_offset(M, N) + svd_refine_doubles(N);
}

// smallest rank preconditioned in FP32 (CTGPU_SVD_F32_MIN overrides; 0 disables)
static int svd_f32_min()
{
	static const int v = [] {
		const char* e = getenv("CTGPU_SVD_F32_MIN");
		return e ? atoi(e) : SVD_F32_MIN_RANK;
	}();
	return v;
}

// CTAs of the FP32 sweeps (CTGPU_SVD_F32_CLUSTER overrides; a power of two)
static int svd_f32_cluster()
{
	static const int v = [] {
		const char* e = getenv("CTGPU_SVD_F32_CLUSTER");
		int c = e ? atoi(e) : SVD_F32_CLUSTER;
		int p = 1;
		while (p < c && p < 16) p *= 2;
		return p;
	}();
	return v;
}

// most FP32 preconditioning sweeps (CTGPU_SVD_F32_SWEEPS overrides, 1 to SVD_F32_SWEEPS_MAX)
static int svd_f32_sweeps()
{
	static const int v = [] {
		const char* e = getenv("CTGPU_SVD_F32_SWEEPS");
		const int k = e ? atoi(e) : SVD_F32_SWEEPS;
		return k < 1 ? 1 : (k > SVD_F32_SWEEPS_MAX ? SVD_F32_SWEEPS_MAX : k);
	}();
	return v;
}

// cosine below which the FP32 sweeps leave a pair alone, if above N eps_32 (CTGPU_SVD_F32_COS
// overrides; default SVD_F32_COS)
static float svd_f32_cos()
{
	static const float v = [] {
		const char* e = getenv("CTGPU_SVD_F32_COS");
		return e ? (float)atof(e) : SVD_F32_COS;
	}();
	return v;
}

// FP64 finish of the mixed path by simultaneous refinement, the FP64 sweeps taking over where it
// does not converge (CTGPU_SVD_REFINE=0: the FP64 sweeps start right after T = R^T V)
static int svd_refine()
{
	static const int v = [] {
		const char* e = getenv("CTGPU_SVD_REFINE");
		return e ? atoi(e) : 1;
	}();
	return v;
}

static i64 tour_smem_bytes(int M, int N, int cl)
{
	const i64 jac = tour_jac_doubles(N, cl);
	const i64 out = (i64)(NWARPS + 4) * M + SVD_OUT_RC;     // column buffers, at least 4 staged reflectors
	i64 need = jac > out ? jac : out;
	// FP32 preconditioning and the refinement, where the rank may reach the threshold and their
	// arrays fit
	const int f32 = svd_f32_min();
	if (f32 > 0 && N >= f32)
	{
		const i64 f32d = (f32_tour_bytes(N, N, std::min(svd_f32_cluster(), cl)) + 7) / 8;
		const i64 mix = std::max(refine_doubles(N, cl), f32d);
		if (8 * mix <= SVD_SMEM_LIMIT && mix > need) need = mix;
	}
	// distributed QR (clusters of more than one CTA): own columns, norms, reflectors, exchange slots
	const i64 qr = qr_cluster_doubles(M, N, cl);
	if (cl > 1 && qr > need) need = qr;
	// pivoted QR staged in shared memory when the whole block fits
	if ((i64)M * N * 8 <= SVD_SMEM_LIMIT && (i64)M * N > need) need = (i64)M * N;
	return 8 * need;
}

int svd_max_cluster(int device)
{
	static int cache[64] = {0};
	static std::mutex lock;
	std::lock_guard<std::mutex> g(lock);
	if (device < 0 || device >= 64) return 8;
	if (cache[device]) return cache[device];
	int best = 8;
	// 16-CTA clusters are a non-portable size: use them where the device can schedule one
	if (cudaFuncSetAttribute(k_svd_tour, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
	    cudaFuncSetAttribute(k_svd_tour, cudaFuncAttributeMaxDynamicSharedMemorySize, SVD_SMEM_LIMIT) == cudaSuccess)
	{
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(16);
		cfg.blockDim = dim3(SVD_THREADS);
		cfg.dynamicSmemBytes = 64 * 1024;
		cudaLaunchAttribute attr[1];
		attr[0].id = cudaLaunchAttributeClusterDimension;
		attr[0].val.clusterDim.x = 16;
		attr[0].val.clusterDim.y = 1;
		attr[0].val.clusterDim.z = 1;
		cfg.attrs = attr;
		cfg.numAttrs = 1;
		int nclusters = 0;
		if (cudaOccupancyMaxActiveClusters(&nclusters, k_svd_tour, &cfg) == cudaSuccess && nclusters >= 1) best = 16;
	}
	cudaGetLastError();
	cache[device] = best;
	return best;
}

SvdLaunch svd_launch_for(int m, int n, int want, int max_cluster)
{
	const int M = m >= n ? m : n, N = m >= n ? n : m;
	SvdLaunch l;
	for (int cl = want < 1 ? 1 : want; cl <= max_cluster; cl *= 2)
	{
		const int bsmax = (N + 2 * cl - 1) / (2 * cl);
		const i64 bytes = tour_smem_bytes(M, N, cl);
		if (bsmax <= SVD_STEP_PAIRS && bytes <= SVD_SMEM_LIMIT)
		{
			l.cluster = cl;
			l.smem = (int)bytes;
			l.global = 0;
			return l;
		}
	}
	// too large for the shared-memory path: columns stay in global memory
	l.cluster = want < 1 ? 1 : (want > 8 ? 8 : want);
	l.smem = 0;
	l.global = 1;
	return l;
}

void launch_svd_group(const SvdLaunch& g, int first, int count, const SvdDesc* descs, const double* a, double* u,
                      double* s, double* vh, double* scratch, int* status, double* flops, cudaStream_t st,
                      unsigned long long* phase_ts, double discard2)
{
	if (count <= 0) return;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)(count * g.cluster));
	cfg.blockDim = dim3(SVD_THREADS);
	cfg.dynamicSmemBytes = (size_t)g.smem;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = (unsigned)g.cluster;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	if (g.global)
	{
		CTG_CUDA(cudaLaunchKernelEx(&cfg, k_svd_global, descs, first, a, u, s, vh, scratch, status, 0.0, flops, g.cluster));
		return;
	}
	static std::once_flag attr_once[64];
	int dev = 0;
	CTG_CUDA(cudaGetDevice(&dev));
	if (dev >= 0 && dev < 64)
		std::call_once(attr_once[dev], [] {
			CTG_CUDA(cudaFuncSetAttribute(k_svd_tour, cudaFuncAttributeMaxDynamicSharedMemorySize, SVD_SMEM_LIMIT));
			CTG_CUDA(cudaFuncSetAttribute(k_svd_tour, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
		});
	CTG_CUDA(cudaLaunchKernelEx(&cfg, k_svd_tour, descs, first, a, u, s, vh, scratch, status, flops, g.cluster, g.smem,
	                             phase_ts, svd_f32_min(), svd_f32_cluster(), svd_refine(), discard2, svd_f32_sweeps(),
	                             svd_f32_cos()));
}

}  // namespace ctg
