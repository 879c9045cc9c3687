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

constexpr int RED_THREADS = 256;

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
__global__ void __launch_bounds__(RED_THREADS, RED_BLOCKS / 152)
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
__global__ void __launch_bounds__(RED_THREADS, RED_BLOCKS / 152)
k_lz_start(const double* __restrict__ v0, double* __restrict__ v, i64 n, double* __restrict__ partial, LanczosScalars* sc)
{
	cg::grid_group grid = cg::this_grid();
	const i64 stride = (i64)RED_BLOCKS * RED_THREADS;
	double x = 0;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) x = fma(v0[i], v0[i], x);
	block_partial(x, partial);
	grid.sync();
	const double nrm = sqrt(final_sum(partial));
	if (blockIdx.x == 0 && threadIdx.x == 0)
	{
		sc->nrm0 = nrm;
		sc->stopped = 0;
		sc->numiter = 0;
		sc->status = 0;
	}
	const double inv = 1.0 / nrm;
	for (i64 i = (i64)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += stride) v[i] = inv * v0[i];
}

static void check_coop(const void* fn)
{
	static std::atomic<int> ok[2] = {{0}, {0}};
	const int which = fn == (const void*)k_lz_step ? 0 : 1;
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

// Lowest eigenpair of the k x k symmetric tridiagonal Lanczos matrix by cyclic Jacobi rotations
// (replaces LAPACK dsteqr, krylov.c:230). One warp; k <= LANCZOS_MAX = 32: the matrix and the
// rotation product live in shared memory, lane r updates row / column r of every rotation.
__global__ void __launch_bounds__(32) k_tridiag(int maxiter, LanczosScalars* sc)
{
	__shared__ double A[LANCZOS_MAX][LANCZOS_MAX + 1], Z[LANCZOS_MAX][LANCZOS_MAX + 1];
	__shared__ double rc[LANCZOS_MAX / 2 + 1], rs[LANCZOS_MAX / 2 + 1];
	__shared__ int rp[LANCZOS_MAX / 2 + 1], rq[LANCZOS_MAX / 2 + 1];
	const int lane = threadIdx.x;
	if (lane == 0 && !sc->stopped) sc->numiter = maxiter;
	__syncwarp();
	const int k = sc->numiter;
	if (k < 1 || k > LANCZOS_MAX)
	{
		if (lane == 0) sc->status = k < 1 ? -1 : -2;
		return;
	}
	if (lane < k)
		for (int j = 0; j < k; j++)
		{
			double v = 0;
			if (lane == j) v = sc->alpha[lane];
			else if (j == lane + 1) v = sc->beta[lane];
			else if (lane == j + 1) v = sc->beta[j];
			A[lane][j] = v;
			Z[lane][j] = (lane == j) ? 1.0 : 0.0;
		}
	__syncwarp();
	// Parallel cyclic Jacobi: each step rotates a set of disjoint pairs (round-robin over k rounded
	// up to even), one lane per pair forming its rotation; A <- J^T A J as all column rotations
	// (lane r updates row r) then all row rotations (lane c updates column c). The angle comes from
	// FP32, the rotation itself is orthogonal to FP64 rounding: t from FP32, c = 1 / sqrt(1 + t^2) and
	// s = t c in FP64. The rotated a_pq (about 1e-7 of its old value) is kept, not set to zero: the
	// transformation stays an orthogonal similarity, and the next sweep removes the residual.
	const int np = k + (k & 1), half = np / 2;
	for (int sweep = 0; sweep < 100; sweep++)
	{
		double off = 0, diag = 0;
		if (lane < k)
		{
			diag = A[lane][lane] * A[lane][lane];
			for (int j = lane + 1; j < k; j++) off = fma(A[lane][j], A[lane][j], off);
		}
		for (int o = 16; o > 0; o >>= 1)
		{
			off += __shfl_xor_sync(0xffffffffu, off, o);
			diag += __shfl_xor_sync(0xffffffffu, diag, o);
		}
		// off-diagonal norm below 1e-15 of the diagonal norm: converged
		if (off <= 1e-30 * diag || off == 0.0) break;
		for (int step = 0; step < np - 1; step++)
		{
			if (lane < half)
			{
				int p, q;
				if (lane == 0) { p = step; q = np - 1; }
				else { p = (step + lane) % (np - 1); q = (step - lane + (np - 1)) % (np - 1); }
				if (p > q) { const int x = p; p = q; q = x; }
				double c = 1.0, sn = 0.0;
				if (q < k)
				{
					const double apq = A[p][q];
					if (apq != 0.0)
					{
						const double app = A[p][p], aqq = A[q][q];
						const double theta = (aqq - app) * rcp64(2.0 * apq);
						double t;
						if (fabs(theta) > 1e15) t = 0.5 * rcp64(theta);
						else
						{
							const float th = (float)theta;
							const float tf = copysignf(1.0f, th) / (fabsf(th) + sqrtf(fmaf(th, th, 1.0f)));
							t = (double)tf;
						}
						double sq, rsq;
						sqrt_rsqrt64(fma(t, t, 1.0), sq, rsq);
						c = rsq;
						sn = t * rsq;
					}
				}
				else q = -1;
				rp[lane] = p;
				rq[lane] = q;
				rc[lane] = c;
				rs[lane] = sn;
			}
			__syncwarp();
			if (lane < k)
				for (int i = 0; i < half; i++)
				{
					const int p = rp[i], q = rq[i];
					if (q < 0) continue;
					const double c = rc[i], sn = rs[i];
					const double arp = A[lane][p], arq = A[lane][q];
					A[lane][p] = c * arp - sn * arq;
					A[lane][q] = sn * arp + c * arq;
					const double zrp = Z[lane][p], zrq = Z[lane][q];
					Z[lane][p] = c * zrp - sn * zrq;
					Z[lane][q] = sn * zrp + c * zrq;
				}
			__syncwarp();
			if (lane < k)
				for (int i = 0; i < half; i++)
				{
					const int p = rp[i], q = rq[i];
					if (q < 0) continue;
					const double c = rc[i], sn = rs[i];
					const double apc = A[p][lane], aqc = A[q][lane];
					A[p][lane] = c * apc - sn * aqc;
					A[q][lane] = sn * apc + c * aqc;
				}
			__syncwarp();
		}
	}
	if (lane == 0)
	{
		int imin = 0;
		for (int i = 1; i < k; i++)
			if (A[i][i] < A[imin][imin]) imin = i;
		sc->lambda = A[imin][imin];
		// deterministic sign: largest-magnitude component positive
		int imax = 0;
		for (int i = 1; i < k; i++)
			if (fabs(Z[i][imin]) > fabs(Z[imax][imin])) imax = i;
		const double sgn = Z[imax][imin] < 0 ? -1.0 : 1.0;
		for (int i = 0; i < k; i++) sc->y[i] = sgn * Z[i][imin];
	}
}

void launch_lz_tridiag(int maxiter, LanczosScalars* sc, cudaStream_t st)
{
	k_tridiag<<<1, 32, 0, st>>>(maxiter, sc);
	CTG_CUDA(cudaGetLastError());
}

__global__ void k_ritz(const double* __restrict__ V, i64 n, const LanczosScalars* sc, double* __restrict__ out)
{
	const int k = sc->numiter;
	for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
	{
		double acc = 0;
		for (int j = 0; j < k; j++) acc = fma(V[(i64)j * n + i], sc->y[j], acc);
		out[i] = acc;
	}
}

void launch_lz_ritz(const double* V, i64 n, int maxiter, const LanczosScalars* sc, double* out, cudaStream_t st)
{
	(void)maxiter;
	k_ritz<<<RED_BLOCKS, 256, 0, st>>>(V, n, sc, out);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
