// ctg_linalg.cu - FP64 dense linear algebra on the device: per-block SVD
// (one-sided Jacobi), per-block RQ (Householder) and the Lanczos vector
// operations with deterministic warp-shuffle reductions.
#include <atomic>
#include <cfloat>

#include <cooperative_groups.h>

#include "ctg_fp64.cuh"
#include "ctg_kernels.h"

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

// One whole Lanczos step in one cooperative launch: alpha_j = <w, v_j>, then unless it is the last step
// w -= alpha_j v_j + beta_{j-1} v_{j-1}, beta_j = ||w|| with the early-exit test, v_{j+1} = w / beta_j.
// Every block forms the scalar reductions itself from the fixed-order partial sums, so no block
// waits for another except at the two grid barriers. `partial` holds 2 RED_BLOCKS doubles.
__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_step(double* __restrict__ w, const double* __restrict__ vj, const double* __restrict__ vjm1,
          double* __restrict__ vj1, i64 n, i64 nthr, int j, int last, double* __restrict__ partial, LanczosScalars* sc)
{
	cg::grid_group grid = cg::this_grid();
	if (sc->stopped) return;               // read before the first barrier: the same in every block
	const i64 stride = (i64)RED_BLOCKS * RED_THREADS;
	double v = 0;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) v = fma(w[i], vj[i], v);
	block_partial(v, partial);
	grid.sync();
	const double al = final_sum(partial);
	if (blockIdx.x == 0 && threadIdx.x == 0) sc->alpha[j] = al;
	if (last) return;
	const double be = j > 0 ? sc->beta[j - 1] : 0.0;
	v = 0;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride)
	{
		// w = w' - alpha_j v_j - beta_{j-1} v_{j-1}, evaluated as in krylov.c:44-53
		const double x = (j > 0) ? w[i] - (al * vj[i] + be * vjm1[i]) : w[i] - al * vj[i];
		w[i] = x;
		v = fma(x, x, v);
	}
	block_partial(v, partial + RED_BLOCKS);
	grid.sync();
	const double b = sqrt(final_sum(partial + RED_BLOCKS));
	const bool stop = b < 100.0 * (double)nthr * DBL_EPSILON;
	if (blockIdx.x == 0 && threadIdx.x == 0)
	{
		sc->beta[j] = b;
		if (stop)
		{
			sc->stopped = 1;
			sc->numiter = j + 1;
		}
	}
	if (stop) return;
	const double inv = 1.0 / b;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) vj1[i] = inv * w[i];
}

// Normalisation of the start vector in one cooperative launch.
__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_start(const double* __restrict__ v0, double* __restrict__ v, i64 n, double* __restrict__ partial, LanczosScalars* sc)
{
	cg::grid_group grid = cg::this_grid();
	const i64 stride = (i64)RED_BLOCKS * RED_THREADS;
	double x = 0;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) x = fma(v0[i], v0[i], x);
	block_partial(x, partial);
	grid.sync();
	const double nrm = sqrt(final_sum(partial));
	// a start vector of norm zero (or not finite) admits no Lanczos iteration: fewer iterations than
	// the one eigenvalue asked for, status -1 (krylov.c:218-223); the later kernels see `stopped`
	const bool bad = !(nrm > 0.0) || !isfinite(nrm);
	if (blockIdx.x == 0 && threadIdx.x == 0)
	{
		sc->nrm0 = nrm;
		sc->stopped = bad ? 1 : 0;
		sc->numiter = 0;
		sc->status = bad ? -1 : 0;
	}
	if (bad) return;
	const double inv = 1.0 / nrm;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) v[i] = inv * v0[i];
}

__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_finish(const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter, double* __restrict__ partial,
            LanczosScalars* sc, double* __restrict__ out);

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

void launch_lz_step(double* w, const double* vj, const double* vjm1, double* vj1, i64 n, i64 nthr, int j, int last,
                    double* partial, LanczosScalars* sc, cudaStream_t st)
{
	check_coop((const void*)k_lz_step);
	void* args[] = {&w, (void*)&vj, (void*)&vjm1, &vj1, &n, &nthr, &j, &last, &partial, &sc};
	CTG_CUDA(cudaLaunchCooperativeKernel((const void*)k_lz_step, dim3(RED_BLOCKS), dim3(RED_THREADS), args, 0, st));
}

void launch_lz_start(const double* v0, double* v, i64 n, double* partial, LanczosScalars* sc, cudaStream_t st)
{
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
//   2. FP64 Newton on the characteristic polynomial (p'/p from the same pivot recurrence), taken
//      from the left end of the bracket that the Sturm counts maintain, where p is positive,
//      decreasing and convex (no overshoot; about three steps from the FP32 bracket), with
//      bisection as the fallback;
//   3. eigenvector by a twisted factorisation (forward and backward pivots, twisted where the
//      eigenvector is largest; robust when converged Lanczos runs leave it concentrated at one
//      end), normalised, its largest-magnitude component made positive (deterministic sign).
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
	if (lane == 0)
	{
		// 2. FP64 Newton on the characteristic polynomial p from the left end of the Sturm bracket
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
		// 3. eigenvector by the twisted factorisation at x (robust where the eigenvector is small at
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
	__shared__ double sh[6 * LANCZOS_MAX];
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
__global__ void __launch_bounds__(RED_THREADS, 1)
k_lz_finish(const double* __restrict__ w, const double* __restrict__ V, i64 n, int maxiter, double* __restrict__ partial,
            LanczosScalars* sc, double* __restrict__ out)
{
	cg::grid_group grid = cg::this_grid();
	__shared__ double sh[6 * LANCZOS_MAX];
	__shared__ double al[LANCZOS_MAX], be[LANCZOS_MAX], y[LANCZOS_MAX];
	__shared__ double lam;
	__shared__ int st;
	const bool stopped = sc->stopped != 0;          // read before the barrier: the same in every block
	const i64 stride = (i64)RED_BLOCKS * RED_THREADS;
	const int j = maxiter - 1;
	double alast = 0.0;
	if (!stopped)
	{
		double v = 0;
		const double* vj = V + (i64)j * n;
		for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) v = fma(w[i], vj[i], v);
		block_partial(v, partial);
		grid.sync();
		alast = final_sum(partial);
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
		for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) out[i] = 0.0;
		if (blockIdx.x == 0 && threadIdx.x == 0)
		{
			sc->numiter = k < 0 ? 0 : k;
			sc->status = k < 1 ? -1 : -2;
		}
		return;
	}
	if (blockIdx.x == 0)
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
	grid.sync();
	if (threadIdx.x < LANCZOS_MAX) y[threadIdx.x] = threadIdx.x < k ? __ldcg(sc->y + threadIdx.x) : 0.0;
	__syncthreads();
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride)
	{
		double acc = 0;
		for (int t = 0; t < k; t++) acc = fma(V[(i64)t * n + i], y[t], acc);
		out[i] = acc;
	}
}

void launch_lz_finish(const double* w, const double* V, i64 n, int maxiter, double* partial, LanczosScalars* sc,
                      double* out, cudaStream_t st)
{
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
