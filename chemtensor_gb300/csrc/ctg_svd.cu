// ctg_svd.cu - block SVD: QR with column pivoting, then one-sided Jacobi on R^T, on
// thread-block clusters.
//
// Replaces LAPACK dgesvd in dense_tensor_svd_fill (dense_tensor.c:3538-3680), which
// block_sparse_tensor_svd (block_sparse_tensor.c:2686-2848) calls once per
// quantum-number block. FP64 throughout. Singular values agree with dgesvd to rounding
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
// On GB300 an SM retires about two FP64 FMAs per clock, so each dense block gets a cluster
// of up to 8 CTAs: the pivoted QR runs on one CTA, the Jacobi rounds (disjoint column pairs
// shared out over all warps of the cluster), the formation of Q and the outputs run on the
// whole cluster, separated by cluster barriers (release / acquire at cluster scope for the
// global-memory data, which is read with L2-coherent loads).
#include <cfloat>
#include <cstdio>
#include <mutex>

#include <cooperative_groups.h>

#include "ctg_kernels.h"

namespace cg = cooperative_groups;

namespace ctg {

namespace {

constexpr int SVD_THREADS = 256;
constexpr int NWARPS = SVD_THREADS / 32;

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

__device__ __forceinline__ void round_robin_pair(int rnd, int pi, int np, int& p, int& q)
{
	// circle method: index np-1 stays fixed, the others rotate
	if (pi == 0) { p = rnd; q = np - 1; }
	else { p = (rnd + pi) % (np - 1); q = (rnd - pi + (np - 1)) % (np - 1); }
	if (p > q) { const int t = p; p = q; q = t; }
}

// Householder QR with column pivoting of W (M x N, column-major) inside one CTA, stopped at
// the numerical rank; returns r. W keeps R in its upper triangle and the Householder vectors
// below it; tau and perm receive the scalars and the column permutation.
__device__ int qr_pivoted_cta(double* W, int M, int N, double* nrm, double* tau, int* perm, double rank_thresh2)
{
	__shared__ double red[NWARPS];
	__shared__ double sh_beta, sh_tau, sh_scale;
	__shared__ int sh_piv, sh_stop;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	int r = 0;
	for (int k = 0; k < N; k++)
	{
		// squared norms of the trailing parts of the remaining columns
		for (int j = k + warp; j < N; j += NWARPS)
		{
			const double* wj = W + (i64)j * M;
			double acc = 0;
			for (int i = k + lane; i < M; i += 32) acc = fma(wj[i], wj[i], acc);
			acc = warp_sum(acc);
			if (lane == 0) nrm[j] = acc;
		}
		__syncthreads();
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
		if (tk != 0.0)
		{
			for (int j = k + 1 + warp; j < N; j += NWARPS)
			{
				double* wj = W + (i64)j * M;
				double acc = 0;
				for (int i = k + lane; i < M; i += 32) acc = fma(i == k ? 1.0 : wk[i], wj[i], acc);
				acc = warp_sum(acc) * tk;
				for (int i = k + lane; i < M; i += 32) wj[i] -= acc * (i == k ? 1.0 : wk[i]);
			}
		}
		__syncthreads();
		r = k + 1;
	}
	return r;
}

__global__ void __launch_bounds__(SVD_THREADS)
k_svd_cluster(const SvdDesc* __restrict__ descs, const double* __restrict__ a, double* __restrict__ u,
              double* __restrict__ s, double* __restrict__ vh, double* __restrict__ scratch, int* __restrict__ status,
              double tiny_rel2, double* __restrict__ tail, int cl)
{
	cg::cluster_group cluster = cg::this_cluster();
	const int rank = (int)cluster.block_rank();
	const SvdDesc d = descs[blockIdx.x / cl];
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
		const int r = qr_pivoted_cta(W, M, N, nrm, tau, perm, DBL_EPSILON * DBL_EPSILON * total);
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
				atomicAdd(tail + blockIdx.x / cl, acc);
		}
	}
	// rank-deficient part beyond r: its weight is below eps^2 ||B||_F^2 per column
	if (rank == 0 && tid == 0 && r < N)
		atomicAdd(tail + blockIdx.x / cl, (double)(N - r) * DBL_EPSILON * DBL_EPSILON * __ldcg(misc + 1));

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
// two streams) race on it and must be serialised by the caller.

constexpr int NOALLOC_SVD_MAX_DIM = 256;
constexpr i64 NOALLOC_SCRATCH_DOUBLES = (i64)1 << 19;   // 4 MiB

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

namespace {

// layout of the fixed array: descriptor, status[2] + tail (as doubles), then the SVD workspace
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
		base[NA_STATUS + 1] = 0.0;                  // tail weight
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
	k_noalloc_prepare<<<64, 256, 0, st>>>(base, d, d_u, d_s, d_vh);
	const int cl = 8;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)cl);
	cfg.blockDim = dim3(SVD_THREADS);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = (unsigned)cl;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	const SvdDesc* descs = (const SvdDesc*)(base + NA_DESC);
	int* status = (int*)(base + NA_STATUS);
	double* tail = base + NA_STATUS + 1;
	cudaError_t e = cudaLaunchKernelEx(&cfg, k_svd_cluster, descs, d_a, d_u, d_s, d_vh, base + NA_WORK, status, 0.0,
	                                   tail, cl);
	if (e == cudaSuccess)
	{
		k_noalloc_finish<<<1, 1, 0, st>>>(base, d_info);
		e = cudaGetLastError();
	}
	if (e != cudaSuccess)
	{
		fprintf(stderr, "ctgpu_dense_svd_noalloc: launch failed: %s\n", cudaGetErrorString(e));
		return -5;
	}
	return 0;
}

namespace ctg {

i64 svd_scratch_doubles(int m, int n)
{
	const i64 M = m >= n ? m : n, N = m >= n ? n : m;
	// W, Q, T, V, nrm, tau, sig, misc, flags + amax, perm
	return 2 * M * N + 2 * N * N + 3 * N + 2 + 2 * SVD_MAX_SWEEPS + (N + 1) / 2 + 1;
}

void launch_svd_jacobi(int nblocks, int cluster, const SvdDesc* descs, const double* a, double* u, double* s,
                       double* vh, double* scratch, int* status, double tiny_rel2, double* tail, cudaStream_t st)
{
	if (nblocks <= 0) return;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)(nblocks * cluster));
	cfg.blockDim = dim3(SVD_THREADS);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = (unsigned)cluster;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	CTG_CUDA(cudaLaunchKernelEx(&cfg, k_svd_cluster, descs, a, u, s, vh, scratch, status, tiny_rel2, tail, cluster));
}

}  // namespace ctg
