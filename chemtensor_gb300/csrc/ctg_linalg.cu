// ctg_linalg.cu - FP64 dense linear algebra on the device: per-block SVD
// (one-sided Jacobi), per-block RQ (Householder) and the Lanczos vector
// operations with deterministic warp-shuffle reductions.
#include <atomic>
#include <cstdlib>
#include <mutex>
#include <cfloat>

#include <cooperative_groups.h>

#include "ctg_fp64.cuh"
#include "ctg_kernels.h"
#include "ctg_launch.cuh"

namespace cg = cooperative_groups;

namespace ctg {

__device__ __forceinline__ double warp_sum(double v)
{
	// xor butterfly: every lane ends with the bitwise-identical total
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// ------------------------------------------------------------------------------------
// block QR / RQ by Householder reflections, one CTA per block.
// QR (desc.qr = 1) follows LAPACK dgeqrf + dorgqr in dense_tensor_qr_fill (dense_tensor.c:2253-2651):
// A = Q R, R upper triangular with diagonal entries -sign(alpha) * |x| of the reflectors.
// RQ (desc.qr = 0) follows dgerqf + dorgrq in dense_tensor_rq_fill (dense_tensor.c:2680-2880):
// dgerqf eliminates the rows of A from the last one upwards, each towards its trailing column; that
// is the QR above applied to W = J A^T J (J reverses an index), with A = (J R_W^T J) (J Q_W^T J).
// Both run the same column-Householder loop on a column-major work matrix W (p x s).
// ------------------------------------------------------------------------------------

constexpr int RQ_THREADS = 256;

__device__ double block_sum(double v, double* red)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	v = warp_sum(v);
	__syncthreads();
	if (lane == 0) red[warp] = v;
	__syncthreads();
	double t = 0;
	for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
	return t;
}

__global__ void __launch_bounds__(RQ_THREADS)
k_rq_householder(const RqDesc* __restrict__ descs, const double* __restrict__ a, double* __restrict__ r,
                 double* __restrict__ q, double* __restrict__ scratch)
{
	__shared__ double red[RQ_THREADS / 32];
	__shared__ double sh_beta, sh_tau, sh_scale;
	const RqDesc d = descs[blockIdx.x];
	const int m = d.m, n = d.n;
	const bool qr = d.qr != 0;
	const int k = min(m, n);
	const int p = qr ? m : n, s = qr ? n : m;   // W is p x s, column-major
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = RQ_THREADS / 32;
	double* B = scratch + d.w_off;             // W, p x s
	double* Q = B + (i64)p * s;                // Q_W, p x k
	double* tau = Q + (i64)p * k;              // k
	const double* ab = a + d.a_off;
	for (i64 e = tid; e < (i64)p * s; e += RQ_THREADS)
	{
		const i64 i = e % p, j = e / p;
		B[e] = qr ? ab[i * n + j] : ab[(m - 1 - j) * n + (n - 1 - i)];
	}
	__syncthreads();
	for (int c = 0; c < k; c++)
	{
		double* bc = B + (i64)c * p;
		double part = 0;
		for (int i = c + 1 + tid; i < p; i += RQ_THREADS) part = fma(bc[i], bc[i], part);
		const double xnorm2 = block_sum(part, red);
		if (tid == 0)
		{
			const double alpha = bc[c];
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
		const double tc = sh_tau;
		for (int i = c + 1 + tid; i < p; i += RQ_THREADS) bc[i] *= sh_scale;
		__syncthreads();
		if (tid == 0) { bc[c] = sh_beta; tau[c] = tc; }
		__syncthreads();
		// apply H = I - tau v v^T (v = (1, bc[c+1:])) to the remaining columns
		if (tc != 0.0)
		{
			for (int c2 = c + 1 + warp; c2 < s; c2 += nwarps)
			{
				double* b2 = B + (i64)c2 * p;
				double acc = 0;
				for (int i = c + lane; i < p; i += 32) acc = fma(i == c ? 1.0 : bc[i], b2[i], acc);
				acc = warp_sum(acc) * tc;
				for (int i = c + lane; i < p; i += 32) b2[i] -= acc * (i == c ? 1.0 : bc[i]);
			}
		}
		__syncthreads();
	}
	// Q_W = H_0 ... H_{k-1} E (p x k), accumulated backwards, column-major
	for (i64 e = tid; e < (i64)p * k; e += RQ_THREADS) Q[e] = (e / p == e % p) ? 1.0 : 0.0;
	__syncthreads();
	for (int c = k - 1; c >= 0; c--)
	{
		const double tc = tau[c];
		const double* bc = B + (i64)c * p;
		if (tc != 0.0)
		{
			for (int j = warp; j < k; j += nwarps)
			{
				double* qj = Q + (i64)j * p;
				double acc = 0;
				for (int i = c + lane; i < p; i += 32) acc = fma(i == c ? 1.0 : bc[i], qj[i], acc);
				acc = warp_sum(acc) * tc;
				for (int i = c + lane; i < p; i += 32) qj[i] -= acc * (i == c ? 1.0 : bc[i]);
			}
		}
		__syncthreads();
	}
	if (qr)
	{
		// R (k x n) = upper part of W; Q (m x k) = Q_W
		for (i64 e = tid; e < (i64)k * n; e += RQ_THREADS)
		{
			const i64 i = e / n, j = e % n;
			r[d.r_off + e] = (i <= j) ? B[i + (i64)p * j] : 0.0;
		}
		for (i64 e = tid; e < (i64)m * k; e += RQ_THREADS)
		{
			const i64 i = e / k, j = e % k;
			q[d.q_off + e] = Q[i + (i64)p * j];
		}
	}
	else
	{
		// R (m x k): R[i][j] = R_W[k-1-j][m-1-i]; Q (k x n): Q[j][i] = Q_W[n-1-i][k-1-j]
		for (i64 e = tid; e < (i64)m * k; e += RQ_THREADS)
		{
			const i64 i = e / k, j = e % k;
			const i64 a0 = k - 1 - j, b0 = m - 1 - i;
			r[d.r_off + e] = (a0 <= b0) ? B[a0 + (i64)p * b0] : 0.0;
		}
		for (i64 e = tid; e < (i64)k * n; e += RQ_THREADS)
		{
			const i64 j = e / n, i = e % n;
			q[d.q_off + e] = Q[(n - 1 - i) + (i64)p * (k - 1 - j)];
		}
	}
}

void launch_rq_householder(int nblocks, const RqDesc* descs, const double* a, double* r, double* q, double* scratch,
                           cudaStream_t st)
{
	if (nblocks <= 0) return;
	k_rq_householder<<<nblocks, RQ_THREADS, 0, st>>>(descs, a, r, q, scratch);
	CTG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------
// Lanczos (lanczos_iteration_d, krylov.c:24-89; eigensystem_krylov_symmetric, :172-251)
// Reductions: fixed grid, fixed per-thread stride, fixed tree, so results are
// reproducible run to run.
// ------------------------------------------------------------------------------------

constexpr int RED_THREADS = 512;

__device__ void block_partial(double v, double* partial)
{
	__shared__ double red[RED_THREADS / 32];
	v = warp_sum(v);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double t = 0;
		for (int w = 0; w < RED_THREADS / 32; w++) t += red[w];
		partial[blockIdx.x] = t;
	}
}

__device__ double final_sum(const double* partial)
{
	__shared__ double red[RED_THREADS / 32];
	double v = 0;
	for (int i = threadIdx.x; i < RED_BLOCKS; i += RED_THREADS) v += partial[i];
	v = warp_sum(v);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
	__syncthreads();
	double t = 0;
	for (int w = 0; w < RED_THREADS / 32; w++) t += red[w];
	return t;
}

// The vector kernels reduce either over the whole grid (a cooperative launch of RED_BLOCKS blocks,
// one per SM; partial sums in global memory, grid barriers) or over one thread-block cluster of
// LZ_CLUSTER blocks (partial sums in distributed shared memory, cluster barriers), which is chosen
// for vectors of up to LZ_CLUSTER_MAX_N entries: those live in L2 between launches, and a cluster
// barrier costs a fraction of a grid barrier over 152 blocks. Both partition the entries and order
// the sums in a fixed way, so that a given n gives the same bits in every run.
struct GridReduce {
	cg::grid_group g;
	double* partial;                     // [slot][RED_BLOCKS] in global memory
	__device__ explicit GridReduce(double* p) : g(cg::this_grid()), partial(p) {}
	__device__ int blocks() const { return RED_BLOCKS; }
	__device__ int block() const { return (int)blockIdx.x; }
	__device__ double sum(double v, int slot)
	{
		block_partial(v, partial + slot * RED_BLOCKS);
		g.sync();
		return final_sum(partial + slot * RED_BLOCKS);
	}
	__device__ void sync() { g.sync(); }
	__device__ void finish() {}
};

struct ClusterReduce {
	cg::cluster_group c;
	double* part;                        // [3] this block's partial sum per slot (shared memory)
	double* red;                         // [RED_THREADS / 32] per-warp sums (shared memory)
	double* bc;                          // [3] the cluster's sum per slot (shared memory)
	__device__ ClusterReduce(double* p, double* r, double* b) : c(cg::this_cluster()), part(p), red(r), bc(b) {}
	__device__ int blocks() const { return (int)c.num_blocks(); }
	__device__ int block() const { return (int)c.block_rank(); }
	__device__ double sum(double v, int slot)
	{
		v = warp_sum(v);
		if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
		__syncthreads();
		if (threadIdx.x == 0)
		{
			double t = 0;
			for (int w = 0; w < RED_THREADS / 32; w++) t += red[w];
			part[slot] = t;
		}
		c.sync();
		if (threadIdx.x < 32)
		{
			// the blocks' partial sums in rank order, added by the fixed butterfly of one warp
			double t = (int)threadIdx.x < blocks() ? *c.map_shared_rank(part + slot, threadIdx.x) : 0.0;
			t = warp_sum(t);
			if (threadIdx.x == 0) bc[slot] = t;
		}
		__syncthreads();
		return bc[slot];
	}
	__device__ void sync() { c.sync(); }
	// no block leaves while another may still read its partial sums
	__device__ void finish() { c.sync(); }
};

// One whole Lanczos step in one launch: alpha_j = <w, v_j>, then unless it is the last step
// w -= alpha_j v_j + beta_{j-1} v_{j-1}, beta_j = ||w|| with the early-exit test, v_{j+1} = w / beta_j.
// Every block forms the scalar reductions itself from the fixed-order partial sums, so no block
// waits for another except at the two barriers. `partial` holds 2 RED_BLOCKS doubles (grid form).
template <class R>
__device__ void lz_step(R& red, double* __restrict__ w, const double* __restrict__ vj, const double* __restrict__ vjm1,
                        double* __restrict__ vj1, i64 n, i64 nthr, int j, int last, LanczosScalars* sc)
{
	if (sc->stopped) return;               // read before the first barrier: the same in every block
	const i64 stride = (i64)red.blocks() * RED_THREADS;
	const i64 first = (i64)red.block() * RED_THREADS + threadIdx.x;
	double v = 0;
	for (i64 i = first; i < n; i += stride) v = fma(w[i], vj[i], v);
	const double al = red.sum(v, 0);
	if (red.block() == 0 && threadIdx.x == 0) sc->alpha[j] = al;
	if (last)
	{
		red.finish();
		return;
	}
	const double be = j > 0 ? sc->beta[j - 1] : 0.0;
	v = 0;
	for (i64 i = first; i < n; i += stride)
	{
		// w = w' - alpha_j v_j - beta_{j-1} v_{j-1}, evaluated as in krylov.c:44-53
		const double x = (j > 0) ? w[i] - (al * vj[i] + be * vjm1[i]) : w[i] - al * vj[i];
		w[i] = x;
		v = fma(x, x, v);
	}
	const double b = sqrt(red.sum(v, 1));
	const bool stop = b < 100.0 * (double)nthr * DBL_EPSILON;
	if (red.block() == 0 && threadIdx.x == 0)
	{
		sc->beta[j] = b;
		if (stop)
		{
			sc->stopped = 1;
			sc->numiter = j + 1;
		}
	}
	if (!stop)
	{
		const double inv = 1.0 / b;
		for (i64 i = first; i < n; i += stride) vj1[i] = inv * w[i];
	}
	red.finish();
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_step(double* __restrict__ w, const double* __restrict__ vj, const double* __restrict__ vjm1,
          double* __restrict__ vj1, i64 n, i64 nthr, int j, int last, double* __restrict__ partial, LanczosScalars* sc)
{
	GridReduce red(partial);
	lz_step(red, w, vj, vjm1, vj1, n, nthr, j, last, sc);
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lzc_step(double* __restrict__ w, const double* __restrict__ vj, const double* __restrict__ vjm1,
           double* __restrict__ vj1, i64 n, i64 nthr, int j, int last, LanczosScalars* sc)
{
	pdl_wait();
	pdl_trigger();
	__shared__ double part[3], wred[RED_THREADS / 32], bc[3];
	ClusterReduce red(part, wred, bc);
	lz_step(red, w, vj, vjm1, vj1, n, nthr, j, last, sc);
}

// Normalisation of the start vector in one launch.
template <class R>
__device__ void lz_start(R& red, const double* __restrict__ v0, double* __restrict__ v, i64 n, LanczosScalars* sc)
{
	const i64 stride = (i64)red.blocks() * RED_THREADS;
	const i64 first = (i64)red.block() * RED_THREADS + threadIdx.x;
	double x = 0;
	for (i64 i = first; i < n; i += stride) x = fma(v0[i], v0[i], x);
	const double nrm = sqrt(red.sum(x, 0));
	// a start vector of norm zero (or not finite) admits no Lanczos iteration: fewer iterations than
	// the one eigenvalue asked for, status -1 (krylov.c:218-223); the later kernels see `stopped`
	const bool bad = !(nrm > 0.0) || !isfinite(nrm);
	if (red.block() == 0 && threadIdx.x == 0)
	{
		sc->nrm0 = nrm;
		sc->stopped = bad ? 1 : 0;
		sc->numiter = 0;
		sc->status = bad ? -1 : 0;
	}
	if (!bad)
	{
		const double inv = 1.0 / nrm;
		for (i64 i = first; i < n; i += stride) v[i] = inv * v0[i];
	}
	red.finish();
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_start(const double* __restrict__ v0, double* __restrict__ v, i64 n, double* __restrict__ partial, LanczosScalars* sc)
{
	GridReduce red(partial);
	lz_start(red, v0, v, n, sc);
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lzc_start(const double* __restrict__ v0, double* __restrict__ v, i64 n, LanczosScalars* sc)
{
	pdl_wait();
	pdl_trigger();
	__shared__ double part[3], wred[RED_THREADS / 32], bc[3];
	ClusterReduce red(part, wred, bc);
	lz_start(red, v0, v, n, sc);
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_finish(const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter, double* __restrict__ partial,
            LanczosScalars* sc, double* __restrict__ out);
__global__ void __launch_bounds__(RED_THREADS, 1)
k_lzc_finish(const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter, LanczosScalars* sc,
             double* __restrict__ out);

static void check_coop(const void* fn)
{
	static std::atomic<int> ok[3] = {{0}, {0}, {0}};
	const int which = fn == (const void*)k_lz_step ? 0 : fn == (const void*)k_lz_start ? 1 : 2;
	if (ok[which].load()) return;
	int dev = 0, sms = 0, per_sm = 0, coop = 0;
	CTG_CUDA(cudaGetDevice(&dev));
	CTG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	CTG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
	CTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, RED_THREADS, 0));
	CTG_CHECK(coop && per_sm * sms >= RED_BLOCKS, "Lanczos: the cooperative vector kernels do not fit on this device");
	ok[which].store(1);
}

// blocks of the cluster form on this device: 16 (a non-portable cluster size) where every
// cluster-form kernel can be scheduled with it, else 8; per device, decided once
static int lz_cluster(const void* fn)
{
	static std::mutex mu;
	static int cache[64][3] = {};
	int dev = 0;
	CTG_CUDA(cudaGetDevice(&dev));
	const int which = fn == (const void*)k_lzc_step ? 0 : fn == (const void*)k_lzc_start ? 1 : 2;
	std::lock_guard<std::mutex> g(mu);
	int& c = cache[dev & 63][which];
	if (c) return c;
	c = 8;
	bool refused = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess;
	if (!refused)
	{
		cudaLaunchConfig_t cfg = {};
		cudaLaunchAttribute at[1];
		cfg.gridDim = dim3(16);
		cfg.blockDim = dim3(RED_THREADS);
		at[0].id = cudaLaunchAttributeClusterDimension;
		at[0].val.clusterDim.x = 16;
		at[0].val.clusterDim.y = 1;
		at[0].val.clusterDim.z = 1;
		cfg.attrs = at;
		cfg.numAttrs = 1;
		int nclusters = 0;
		refused = cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) != cudaSuccess;
		if (!refused && nclusters >= 1) c = 16;
	}
	if (refused) cudaGetLastError();     // a refused attribute or query leaves no error behind
	return c;
}

// largest vector (doubles) of the cluster form (CTGPU_LZ_CLUSTER_MAX_N overrides; 0 keeps every
// vector on the grid form)
static i64 lz_cluster_max_n()
{
	static const i64 v = [] {
		const char* e = getenv("CTGPU_LZ_CLUSTER_MAX_N");
		return e ? (i64)atoll(e) : LZ_CLUSTER_MAX_N;
	}();
	return v;
}

template <class... Args>
static void launch_cluster_form(void (*fn)(Args...), cudaStream_t st, Args... args)
{
	const int cl = lz_cluster((const void*)fn);
	cudaLaunchConfig_t cfg = {};
	cudaLaunchAttribute at[1];
	cfg.gridDim = dim3(cl);
	cfg.blockDim = dim3(RED_THREADS);
	cfg.stream = st;
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = cl;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	launch_pdl(cfg, fn, args...);
}

void launch_lz_step(double* w, const double* vj, const double* vjm1, double* vj1, i64 n, i64 nthr, int j, int last,
                    double* partial, LanczosScalars* sc, cudaStream_t st)
{
	if (n <= lz_cluster_max_n())
	{
		launch_cluster_form(k_lzc_step, st, w, vj, vjm1, vj1, n, nthr, j, last, sc);
		return;
	}
	check_coop((const void*)k_lz_step);
	void* args[] = {&w, (void*)&vj, (void*)&vjm1, &vj1, &n, &nthr, &j, &last, &partial, &sc};
	CTG_CUDA(cudaLaunchCooperativeKernel((const void*)k_lz_step, dim3(RED_BLOCKS), dim3(RED_THREADS), args, 0, st));
}

void launch_lz_start(const double* v0, double* v, i64 n, double* partial, LanczosScalars* sc, cudaStream_t st)
{
	if (n <= lz_cluster_max_n())
	{
		launch_cluster_form(k_lzc_start, st, v0, v, n, sc);
		return;
	}
	check_coop((const void*)k_lz_start);
	void* args[] = {(void*)&v0, &v, &n, &partial, &sc};
	CTG_CUDA(cudaLaunchCooperativeKernel((const void*)k_lz_start, dim3(RED_BLOCKS), dim3(RED_THREADS), args, 0, st));
}

// Lowest eigenpair of the k x k symmetric tridiagonal Lanczos matrix T (replaces LAPACK dsteqr,
// krylov.c:230, for the lowest eigenpair only). One warp, k <= LANCZOS_MAX = 32. The Lanczos matrix
// is unreduced (every beta above the breakdown threshold), so its eigenvalues are simple and, by
// interlacing, the lowest one lies strictly below those of every leading submatrix T_j: at
// x <= lambda_0 the pivots d_1 .. d_{k-1} of the LDL^T factorisation of T - x I are positive and the
// number of negative pivots (Sturm count) is the number of eigenvalues below x.
//   1. FP32 multisection: the 32 lanes take Sturm counts at 32 points of the Gershgorin interval and
//      keep the sub-interval where the count first reaches one (33x narrower per round), to FP32
//      resolution;
//   2. FP64 Newton on the characteristic polynomial, taken from the left end of the FP32 bracket,
//      where p is positive, decreasing and convex (no overshoot; two or three steps), with p and p'
//      from the three-term recurrence of the leading minors (one FMA of serial chain per step);
//   3. eigenvector of the twisted factorisation (twisted where the eigenvector is largest; robust
//      when converged Lanczos runs leave it concentrated at one end) from the leading and trailing
//      minors, one component per lane, normalised, its largest-magnitude component made positive
//      (deterministic sign).
// Where a minor would leave [2^-600, 2^600] or the Newton steps do not settle, steps 2 and 3 run
// in the pivot form instead (LDL^T pivots, a reciprocal per step, bisection as the last resort).
// Reciprocals are rcp64 (FP32 seed, cubic correction): an FP64 division costs over a thousand
// cycles of GB300's FP64 pipe. Status -2 if the result is not finite.
__device__ __forceinline__ int sturm_count32(const float* a, const float* b2, int k, float x)
{
	int neg = 0;
	float d = a[0] - x;
	for (int i = 0;; i++)
	{
		if (fabsf(d) < 1e-30f) d = -1e-30f;
		neg += d < 0.0f ? 1 : 0;
		if (i + 1 >= k) break;
		d = (a[i + 1] - x) - __fdividef(b2[i], d);
	}
	return neg;
}

// Sturm count of T - x I and S = p'(x) / p(x) for the characteristic polynomial p = prod_i d_i (the
// LDL^T pivots): S = sum_i d_i' / d_i, the derivatives following d_{i+1}' = -1 + b_i^2 d_i' / d_i^2
__device__ __forceinline__ void pivots64(const double* a, const double* b2, int k, double x, int& neg, double& S)
{
	double d = a[0] - x, dd = -1.0;
	if (fabs(d) < 1e-300) d = -1e-300;
	neg = d < 0.0 ? 1 : 0;
	double inv = rcp64(d);
	S = dd * inv;
	for (int i = 0; i + 1 < k; i++)
	{
		const double t = b2[i] * inv;
		dd = fma(t * inv, dd, -1.0);
		d = (a[i + 1] - x) - t;
		if (fabs(d) < 1e-300) d = -1e-300;
		neg += d < 0.0 ? 1 : 0;
		inv = rcp64(d);
		S = fma(dd, inv, S);
	}
}

// Leading principal minors of T - x I by the three-term recurrence p_{i+1} = (a_i - x) p_i -
// b_{i-1}^2 p_{i-1} (p_0 = 1) with their derivative q = dp/dx (q_{i+1} = (a_i - x) q_i -
// b_{i-1}^2 q_{i-1} - p_i): returns p_k, q_k, whether every minor p_1 .. p_k is positive (x lies
// below the smallest eigenvalue: T - x I is positive definite) and whether every nonzero minor
// stayed within [2^-600, 2^600] in magnitude. The chain of a step is one FMA deep (the b^2 p_{i-1}
// term is ready a step early), against a reciprocal per step in the pivot form; the sign and range
// tests read bits (integer instructions, not FP64 compares).
__device__ __forceinline__ void minors64(const double* A, const double* B2, int k, double x, double& p, double& q,
                                         bool& allpos, bool& inrange)
{
	double p0 = 0.0, p1 = 1.0, q0 = 0.0, q1 = 0.0;
	bool notpos = false, out = false;
	for (int i = 0; i < k; i++)
	{
		const double s = A[i] - x;
		const double bb = i > 0 ? B2[i - 1] : 0.0;
		const double pn = fma(s, p1, -bb * p0);
		const double qn = fma(s, q1, fma(-bb, q0, -p1));
		p0 = p1;
		q0 = q1;
		p1 = pn;
		q1 = qn;
		const long long bits = __double_as_longlong(pn);
		const int e = (int)((bits >> 52) & 0x7ff);
		notpos |= bits <= 0;
		out |= e > 1023 + 600 || (e < 1023 - 600 && (bits & 0x7fffffffffffffffll) != 0);
	}
	p = p1;
	q = q1;
	allpos = !notpos;
	inrange = !out;
}

// Lowest eigenpair of the k x k tridiagonal (diagonal al[0..k-1], off-diagonal be[0..k-2]); called
// by all 32 lanes of one warp; lane 0 writes *lambda, y[0..k-1] and *status (0, or -2 if the result
// is not finite). `sh` is shared scratch of 6 LANCZOS_MAX doubles.
__device__ void tridiag_lowest(const double* al, const double* be, int k, double* sh, double* lambda, double* y, int* status)
{
	const int lane = threadIdx.x & 31;
	double* A = sh;
	double* B2 = sh + LANCZOS_MAX;
	double* Bv = sh + 2 * LANCZOS_MAX;
	double* Y = sh + 3 * LANCZOS_MAX;
	float* Af = (float*)(sh + 4 * LANCZOS_MAX);
	float* B2f = Af + LANCZOS_MAX;
	if (lane < k)
	{
		A[lane] = al[lane];
		Af[lane] = (float)A[lane];
		const double b = lane + 1 < k ? be[lane] : 0.0;
		Bv[lane] = b;
		B2[lane] = b * b;
		B2f[lane] = (float)(b * b);
	}
	__syncwarp();
	if (k == 1)
	{
		if (lane == 0)
		{
			*lambda = A[0];
			y[0] = 1.0;
			*status = isfinite(A[0]) ? 0 : -2;
		}
		__syncwarp();
		return;
	}
	// Gershgorin interval of all eigenvalues (FP32, widened by a relative margin)
	float glo = 3.0e38f, ghi = -3.0e38f;
	for (int i = 0; i < k; i++)
	{
		const float r = (i > 0 ? fabsf((float)Bv[i - 1]) : 0.0f) + fabsf((float)Bv[i]);
		glo = fminf(glo, Af[i] - r);
		ghi = fmaxf(ghi, Af[i] + r);
	}
	const float span = fmaxf(ghi - glo, 1e-30f);
	float lo = glo - 1e-3f * span, hi = ghi + 1e-3f * span;
	// 1. FP32 multisection
	for (int round = 0; round < 8; round++)
	{
		const float w = hi - lo;
		if (w <= 4e-7f * fmaxf(fabsf(lo), fabsf(hi))) break;
		const float x = lo + w * (float)(lane + 1) * (1.0f / 33.0f);
		const unsigned mask = __ballot_sync(0xffffffffu, sturm_count32(Af, B2f, k, x) >= 1);
		const int f = mask ? __ffs(mask) - 1 : 32;
		const float xf = lo + w * (float)(f + 1) * (1.0f / 33.0f), xl = lo + w * (float)f * (1.0f / 33.0f);
		if (f < 32) hi = xf;
		lo = f > 0 ? xl : lo;
	}
	// 2. FP64 Newton on the leading minors, from the left end of the FP32 bracket (count 0: every
	// minor positive), where p_k is positive, decreasing and convex below its smallest root: the
	// steps x - p_k / p_k' approach lambda_0 from below without passing it, quadratically once close
	// (two or three steps from the FP32 bracket). A step below the tolerance ends the iteration, and
	// so does one that lands at or past the root (only rounding can do that).
	// 3. The eigenvector from the minors at that x: with p_i the leading and r_i the trailing minors
	// (r_k = 1, r_i = (a_i - x) r_{i+1} - b_i^2 r_{i+2}), 1 / gamma_i = p_i r_{i+1} / p_k is the i-th
	// diagonal entry of (T - x I)^{-1}, so the twist index of the twisted factorisation,
	// argmin |gamma_i|, is argmax |p_i r_{i+1}|, and its solution with y_t = 1 is
	//   y_i = (-1)^{t-i} b_i .. b_{t-1} p_i / p_t (i <= t),  y_i = (-1)^{i-t} b_t .. b_{i-1} r_{i+1} / r_{t+1} (i >= t)
	// (the products of the twisted factorisation's pivot ratios, d+_i = p_{i+1} / p_i and
	// d-_i = r_i / r_{i+1}), every component on its own lane. Where a minor leaves the safe range,
	// or the Newton steps do not settle, the pivot form below takes over.
	{
		double x = 0.0;
		int fast = 0;
		if (lane == 0)
		{
			const double gspan = (double)span;
			x = (double)lo;
			double p, q;
			bool pos, inr;
			minors64(A, B2, k, x, p, q, pos, inr);
			if (!pos)
			{
				x = (double)glo - gspan;
				minors64(A, B2, k, x, p, q, pos, inr);
			}
			bool done = false;
			for (int it = 0; it < 100 && pos && inr && !done; it++)
			{
				const double step = -p * rcp64(q);
				const double tol = 2.0 * DBL_EPSILON * (fabs(x) + gspan);
				// step >= 0 and tol > 0: their bits order like the values (a negative step, from
				// rounding, has the sign bit and compares below)
				if (__double_as_longlong(step) <= __double_as_longlong(tol))
				{
					x += step;
					done = true;
					break;
				}
				const double xn = x + step;
				bool posn;
				minors64(A, B2, k, xn, p, q, posn, inr);
				x = xn;
				if (!posn) done = true;
			}
			fast = done && inr && isfinite(x) ? 1 : 0;
		}
		fast = __shfl_sync(0xffffffffu, fast, 0);
		x = __shfl_sync(0xffffffffu, x, 0);
		if (fast)
		{
			// leading minors P[0..k] on lane 0, trailing minors R[0..k] on lane 1, in one loop
			double* P = sh + 6 * LANCZOS_MAX;
			double* Rm = P + LANCZOS_MAX + 2;
			bool out = false;
			if (lane < 2)
			{
				double m0 = 0.0, m1 = 1.0;
				if (lane == 0) P[0] = 1.0;
				else Rm[k] = 1.0;
				for (int t = 0; t < k; t++)
				{
					const int i = lane == 0 ? t : k - 1 - t;
					const double bb = t == 0 ? 0.0 : (lane == 0 ? B2[t - 1] : B2[i]);
					const double mn = fma(A[i] - x, m1, -bb * m0);
					m0 = m1;
					m1 = mn;
					const long long bits = __double_as_longlong(mn);
					const int e = (int)((bits >> 52) & 0x7ff);
					out |= e > 1023 + 600 || (e < 1023 - 600 && (bits & 0x7fffffffffffffffll) != 0);
					if (lane == 0) P[t + 1] = mn;
					else Rm[i] = mn;
				}
			}
			__syncwarp();
			const bool ok = !__any_sync(0xffffffffu, out);
			long long g = -1;
			int t = lane;
			if (ok)
			{
				// twist index: the largest |p_i r_{i+1}| (magnitude bits as integers; ties to the
				// smallest index)
				if (lane < k) g = __double_as_longlong(fabs(P[lane] * Rm[lane + 1]));
#pragma unroll
				for (int o = 16; o > 0; o >>= 1)
				{
					const long long og = __shfl_xor_sync(0xffffffffu, g, o);
					const int ot = __shfl_xor_sync(0xffffffffu, t, o);
					if (og > g || (og == g && ot < t)) { g = og; t = ot; }
				}
			}
			if (ok && g > 0)                 // g: the same in every lane after the butterfly
			{
				const double invp = rcp64(P[t]), invr = rcp64(Rm[t + 1]);
				double yi = 0.0;
				if (lane < k)
				{
					const int i0 = lane < t ? lane : t, i1 = lane < t ? t : lane;
					double bp = 1.0;
					for (int j = i0; j < i1; j++) bp *= Bv[j];
					if ((i1 - i0) & 1) bp = -bp;
					yi = lane <= t ? bp * (P[lane] * invp) : bp * (Rm[lane + 1] * invr);
				}
				const double nrm2 = warp_sum(yi * yi);
				double sq, rsq;
				sqrt_rsqrt64(nrm2, sq, rsq);
				// sign: the largest-magnitude component positive (ties to the smallest index)
				long long m = lane < k ? __double_as_longlong(fabs(yi)) : -1;
				int im = lane;
#pragma unroll
				for (int o = 16; o > 0; o >>= 1)
				{
					const long long om = __shfl_xor_sync(0xffffffffu, m, o);
					const int oi = __shfl_xor_sync(0xffffffffu, im, o);
					if (om > m || (om == m && oi < im)) { m = om; im = oi; }
				}
				const double ymax = __shfl_sync(0xffffffffu, yi, im);
				const double v = (ymax < 0.0 ? -rsq : rsq) * yi;
				const bool fin = __all_sync(0xffffffffu, isfinite(v)) && isfinite(x);
				if (lane < k) y[lane] = v;
				if (lane == 0)
				{
					*lambda = x;
					*status = fin ? 0 : -2;
				}
				__syncwarp();
				return;
			}
		}
	}
	if (lane == 0)
	{
		// Fallback, the pivot form (a reciprocal per step, no range limit). FP64 Newton on the
		// characteristic polynomial p from the left end of the Sturm bracket
		// [L, R] (count(L) = 0, count(R) >= 1): left of its smallest root a real-rooted polynomial is
		// positive, decreasing and convex, so Newton steps x - p / p' = x - 1 / S approach lambda_0
		// from below without passing it (quadratically once close). A step that lands at or past the
		// root can only be rounding, and a step below the tolerance means convergence: either ends
		// the iteration. Bisection is the fallback (a bracket reset to the Gershgorin bounds).
		const double gspan = (double)span;
		double L = (double)lo, R = (double)hi;
		double SL, S;
		int neg;
		pivots64(A, B2, k, L, neg, SL);
		if (neg != 0)
		{
			L = (double)glo - gspan;
			pivots64(A, B2, k, L, neg, SL);
		}
		pivots64(A, B2, k, R, neg, S);
		if (neg == 0) R = (double)ghi + gspan;
		bool ok = false;
		double x = 0.0;
		for (int it = 0; it < 200; it++)
		{
			const double tol = 2.0 * DBL_EPSILON * (fmax(fabs(L), fabs(R)) + gspan);
			if (R - L <= 2.0 * tol)
			{
				x = 0.5 * (L + R);
				ok = true;
				break;
			}
			const double mid = 0.5 * (L + R);
			bool newton = SL < 0.0;
			const double step = newton ? -rcp64(SL) : 0.0;
			if (newton && step <= tol)
			{
				x = L + step;
				ok = true;
				break;
			}
			double xn = newton ? L + step : mid;
			if (!(xn > L && xn < R))
			{
				xn = mid;
				newton = false;
			}
			const double dx = xn - L;
			pivots64(A, B2, k, xn, neg, S);
			if (neg == 0)
			{
				L = xn;
				SL = S;
				if (newton && dx <= tol)
				{
					x = xn;
					ok = true;
					break;
				}
			}
			else
			{
				R = xn;
				if (newton)
				{
					x = xn;
					ok = true;
					break;
				}
			}
		}
		// eigenvector by the twisted factorisation at x (robust where the eigenvector is small at
		// either end): forward pivots d+ (in Y) and backward pivots d- (Dm), twist index r = argmin
		// |d+_r + d-_r - (a_r - x)|; y_r = 1, y_i = -(b_i / d+_i) y_{i+1} above r, y_i = -(b_{i-1} /
		// d-_i) y_{i-1} below
		double Dm[LANCZOS_MAX];
		{
			double d = A[k - 1] - x;
			for (int i = k - 1; i >= 0; i--)
			{
				if (i < k - 1) d = (A[i] - x) - B2[i] * rcp64(d);
				if (fabs(d) < 1e-300) d = 1e-300;
				Dm[i] = d;
			}
		}
		int r = 0;
		double gbest = 0.0;
		{
			double d = A[0] - x;
			for (int i = 0; i < k; i++)
			{
				if (i > 0) d = (A[i] - x) - B2[i - 1] * rcp64(d);
				if (fabs(d) < 1e-300) d = 1e-300;
				Y[i] = d;
				const double g = fabs(d + Dm[i] - (A[i] - x));
				if (i == 0 || g < gbest)
				{
					gbest = g;
					r = i;
				}
			}
		}
		double nrm2 = 1.0;
		double yn = 1.0;
		for (int i = r - 1; i >= 0; i--)
		{
			yn = -Bv[i] * rcp64(Y[i]) * yn;
			Y[i] = yn;
			nrm2 = fma(yn, yn, nrm2);
		}
		Y[r] = 1.0;
		yn = 1.0;
		for (int i = r + 1; i < k; i++)
		{
			yn = -Bv[i - 1] * rcp64(Dm[i]) * yn;
			Y[i] = yn;
			nrm2 = fma(yn, yn, nrm2);
		}
		double sq, rsq;
		sqrt_rsqrt64(nrm2, sq, rsq);
		int imax = 0;
		for (int i = 1; i < k; i++)
			if (fabs(Y[i]) > fabs(Y[imax])) imax = i;
		const double sgn = Y[imax] < 0 ? -rsq : rsq;
		bool fin = ok && isfinite(x);
		for (int i = 0; i < k; i++)
		{
			const double v = sgn * Y[i];
			fin = fin && isfinite(v);
			y[i] = v;
		}
		*lambda = x;
		*status = fin ? 0 : -2;
	}
	__syncwarp();
}

// the eigensolve alone (test hook): one warp
__global__ void __launch_bounds__(32) k_tridiag_test(const double* al, const double* be, int k, double* out)
{
	__shared__ double sh[TRIDIAG_SCRATCH];
	__shared__ double y[LANCZOS_MAX];
	__shared__ double lam;
	__shared__ int st;
	tridiag_lowest(al, be, k, sh, &lam, y, &st);
	if (threadIdx.x == 0)
	{
		out[0] = lam;
		out[1] = (double)st;
		for (int i = 0; i < k; i++) out[2 + i] = y[i];
	}
}

// The last Lanczos step and the eigenvector in one cooperative launch: unless the iteration stopped
// early, alpha_{k-1} = <w, v_{k-1}> (fixed-order reduction, one grid barrier); then one warp of
// block 0 solves the k x k tridiagonal eigenproblem (k <= 32: microseconds of serial FP64 work, which
// copies in every block would queue on the same SM sub-partitions) and stores lambda, y and the
// status; after a second grid barrier every block writes its share of the Ritz vector out = V y.
// With no iteration at all (a start vector of norm zero) the status is -1 and out is zero.
template <class R>
__device__ void lz_finish(R& red, const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter,
                          LanczosScalars* sc, double* __restrict__ out)
{
	__shared__ double sh[TRIDIAG_SCRATCH];
	__shared__ double al[LANCZOS_MAX], be[LANCZOS_MAX], y[LANCZOS_MAX];
	__shared__ double lam;
	__shared__ int st;
	const bool stopped = sc->stopped != 0;          // read before the barrier: the same in every block
	const i64 stride = (i64)red.blocks() * RED_THREADS;
	const i64 first = (i64)red.block() * RED_THREADS + threadIdx.x;
	const int j = maxiter - 1;
	double alast = 0.0;
	if (!stopped)
	{
		double v = 0;
		const double* vj = V + (i64)j * n;
		for (i64 i = first; i < n; i += stride) v = fma(w[i], vj[i], v);
		alast = red.sum(v, 0);
	}
	const int k = stopped ? sc->numiter : maxiter;
	if (threadIdx.x < LANCZOS_MAX)
	{
		const int t = threadIdx.x;
		al[t] = t < k ? (stopped || t < j ? sc->alpha[t] : alast) : 0.0;
		be[t] = t + 1 < k ? sc->beta[t] : 0.0;
	}
	__syncthreads();
	if (k < 1 || k > LANCZOS_MAX)
	{
		for (i64 i = first; i < n; i += stride) out[i] = 0.0;
		if (red.block() == 0 && threadIdx.x == 0)
		{
			sc->numiter = k < 0 ? 0 : k;
			sc->status = k < 1 ? -1 : -2;
		}
		red.finish();
		return;
	}
	if (red.block() == 0)
	{
		if (threadIdx.x < 32) tridiag_lowest(al, be, k, sh, &lam, y, &st);
		__syncthreads();
		if (threadIdx.x == 0)
		{
			if (!stopped) sc->alpha[j] = alast;
			sc->numiter = k;
			sc->lambda = lam;
			for (int t = 0; t < k; t++) sc->y[t] = y[t];
			sc->status = st;
		}
	}
	red.sync();
	if (threadIdx.x < LANCZOS_MAX) y[threadIdx.x] = threadIdx.x < k ? __ldcg(sc->y + threadIdx.x) : 0.0;
	__syncthreads();
	for (i64 i = first; i < n; i += stride)
	{
		double acc = 0;
		for (int t = 0; t < k; t++) acc = fma(V[(i64)t * n + i], y[t], acc);
		out[i] = acc;
	}
	red.finish();
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_finish(const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter, double* __restrict__ partial,
            LanczosScalars* sc, double* __restrict__ out)
{
	GridReduce red(partial);
	lz_finish(red, w, V, n, maxiter, sc, out);
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lzc_finish(const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter, LanczosScalars* sc,
             double* __restrict__ out)
{
	pdl_wait();
	pdl_trigger();
	__shared__ double part[3], wred[RED_THREADS / 32], bc[3];
	ClusterReduce red(part, wred, bc);
	lz_finish(red, w, V, n, maxiter, sc, out);
}

void launch_lz_finish(const double* w, const double* V, i64 n, int maxiter, double* partial, LanczosScalars* sc,
                      double* out, cudaStream_t st)
{
	if (n <= lz_cluster_max_n())
	{
		launch_cluster_form(k_lzc_finish, st, w, V, n, maxiter, sc, out);
		return;
	}
	check_coop((const void*)k_lz_finish);
	void* args[] = {(void*)&w, (void*)&V, &n, &maxiter, &partial, &sc, &out};
	CTG_CUDA(cudaLaunchCooperativeKernel((const void*)k_lz_finish, dim3(RED_BLOCKS), dim3(RED_THREADS), args, 0, st));
}

void tridiag_lowest_test(const double* d_alpha, const double* d_beta, int k, double* d_out, cudaStream_t st)
{
	k_tridiag_test<<<1, 32, 0, st>>>(d_alpha, d_beta, k, d_out);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
