// ctg_complex.cu - complex128 (CT_DOUBLE_COMPLEX) kernels of the DMRG path.
//
// Complex tensors use the reference's storage (interleaved real and imaginary parts, row-major
// blocks), so the same lowered work lists and copy descriptors serve both element types: offsets,
// strides and counts are in elements, and the kernels here read double2 elements.
//   k_gemm_z   grouped block GEMM over the FP64 work lists (GemmOut / GemmContrib), optionally
//              conjugating either operand (the conjugated bra of the environment updates,
//              chain_ops.c:116-245); one CTA per 32 x 32 tile of an output block
//   k_svd_z    one-sided complex Jacobi SVD of each block (zgesvd in dense_tensor_svd_fill,
//              dense_tensor.c:3538-3680): one CTA per block, columns in global memory, the column
//              pairs of a sweep in round-robin rounds of disjoint pairs, one warp per pair
//   k_qr_z     complex Householder QR / RQ of each block (zgeqrf + zungqr, zgerqf + zungrq in
//              dense_tensor_qr_fill / rq_fill): R has a real diagonal, as LAPACK's
#include <algorithm>
#include <cfloat>

#include "ctg_fp64.cuh"
#include "ctg_kernels.h"

namespace ctg {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
	return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

__device__ __forceinline__ double warp_sum_z(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// sum of 4 values over the CTA (256 threads); every thread gets the totals
__device__ void block_sum4(double v[4], double* red)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int q = 0; q < 4; q++) v[q] = warp_sum_z(v[q]);
	__syncthreads();
	if (lane == 0)
		for (int q = 0; q < 4; q++) red[warp * 4 + q] = v[q];
	__syncthreads();
	for (int q = 0; q < 4; q++)
	{
		double t = 0;
		for (int w = 0; w < nw; w++) t += red[w * 4 + q];
		v[q] = t;
	}
}

// ------------------------------------------------------------------------------------
// grouped complex GEMM
// ------------------------------------------------------------------------------------

constexpr int ZT = 32;   // tile rows and columns
constexpr int ZK = 16;   // k per shared-memory stage

__global__ void __launch_bounds__(256)
k_gemm_z(const ZTile* __restrict__ tiles, const GemmOut* __restrict__ outs, const GemmContrib* __restrict__ cons,
         const double2* __restrict__ A, const double2* __restrict__ B, double2* __restrict__ C, int conj_a, int conj_b)
{
	__shared__ double2 As[ZK][ZT + 1];
	__shared__ double2 Bs[ZK][ZT + 1];
	const ZTile t = tiles[blockIdx.x];
	const GemmOut o = outs[t.out];
	const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
	double2 acc[2][2];
	for (int r = 0; r < 2; r++)
		for (int q = 0; q < 2; q++) acc[r][q] = make_double2(0.0, 0.0);
	for (int c = o.c0; c < o.c0 + o.nc; c++)
	{
		const GemmContrib g = cons[c];
		for (int k0 = 0; k0 < g.k; k0 += ZK)
		{
			for (int e = threadIdx.x; e < ZT * ZK; e += blockDim.x)
			{
				const int i = e % ZT, kk = e / ZT;
				const int gi = t.m0 + i, gk = k0 + kk;
				double2 va = make_double2(0.0, 0.0), vb = make_double2(0.0, 0.0);
				if (gk < g.k)
				{
					if (gi < o.m) va = A[g.a_off + (i64)gi * g.sAm + (i64)gk * g.sAk];
					const int gj = t.n0 + i;
					if (gj < o.n) vb = B[g.b_off + (i64)gk * g.sBk + (i64)gj * g.sBn];
				}
				if (conj_a) va.y = -va.y;
				if (conj_b) vb.y = -vb.y;
				As[kk][i] = va;
				Bs[kk][i] = vb;
			}
			__syncthreads();
#pragma unroll 4
			for (int kk = 0; kk < ZK; kk++)
			{
				const double2 a0 = As[kk][ty * 2], a1 = As[kk][ty * 2 + 1];
				const double2 b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
				const double2 p00 = cmul(a0, b0), p01 = cmul(a0, b1), p10 = cmul(a1, b0), p11 = cmul(a1, b1);
				acc[0][0].x += p00.x; acc[0][0].y += p00.y;
				acc[0][1].x += p01.x; acc[0][1].y += p01.y;
				acc[1][0].x += p10.x; acc[1][0].y += p10.y;
				acc[1][1].x += p11.x; acc[1][1].y += p11.y;
			}
			__syncthreads();
		}
	}
	for (int r = 0; r < 2; r++)
		for (int q = 0; q < 2; q++)
		{
			const int i = t.m0 + ty * 2 + r, j = t.n0 + tx * 2 + q;
			if (i < o.m && j < o.n) C[gemm_out_index(o, i, j)] = acc[r][q];
		}
}

// ------------------------------------------------------------------------------------
// one-sided complex Jacobi SVD, one CTA per block
// ------------------------------------------------------------------------------------

constexpr int SVDZ_MAX_SWEEPS = 60;

// work per block (double2 units from w_off): W (R x K, column-major), V (K x K, column-major),
// K slots for the column permutation, K slots for the sorted singular values
__global__ void __launch_bounds__(256)
k_svd_z(const SvdDesc* __restrict__ descs, const double2* __restrict__ a, double2* __restrict__ u,
        double* __restrict__ s, double2* __restrict__ vh, double2* __restrict__ work, int* __restrict__ status)
{
	__shared__ int sh_rot;
	const SvdDesc d = descs[blockIdx.x];
	const int m = d.m, n = d.n;
	const bool tr = m < n;                   // factor A^H instead (more rows than columns)
	const int R = tr ? n : m, K = tr ? m : n;
	double2* W = work + d.w_off;
	double2* V = W + (i64)R * K;
	int* perm = (int*)(V + (i64)K * K);
	double* sorted = (double*)(V + (i64)K * K + K);
	const double2* ab = a + d.a_off;
	for (i64 e = threadIdx.x; e < (i64)R * K; e += blockDim.x)
	{
		const int r = (int)(e % R), c = (int)(e / R);
		W[e] = tr ? cconj(ab[(i64)c * n + r]) : ab[(i64)r * n + c];
	}
	for (i64 e = threadIdx.x; e < (i64)K * K; e += blockDim.x)
		V[e] = make_double2((e % K) == (e / K) ? 1.0 : 0.0, 0.0);
	__syncthreads();
	// cyclic sweeps in round-robin order: K - 1 rounds of disjoint column pairs (circle method; a
	// phantom column when K is odd), one warp per pair, a CTA barrier between rounds
	const int KP = K + (K & 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
	bool converged = K < 2;
	for (int sweep = 0; sweep < SVDZ_MAX_SWEEPS && !converged; sweep++)
	{
		if (threadIdx.x == 0) sh_rot = 0;
		__syncthreads();
		for (int round = 0; round < KP - 1; round++)
		{
			for (int pk = warp; pk < KP / 2; pk += nwarps)
			{
				int p0, q0;
				if (pk == 0) { p0 = KP - 1; q0 = round; }
				else { p0 = (round + pk) % (KP - 1); q0 = (round - pk + (KP - 1)) % (KP - 1); }
				const int p = min(p0, q0), q = max(p0, q0);
				if (q >= K) continue;                 // pair with the phantom column
				double2* wp = W + (i64)p * R;
				double2* wq = W + (i64)q * R;
				double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
				for (int i = lane; i < R; i += 32)
				{
					const double2 x = wp[i], y = wq[i];
					v0 = fma(x.x, x.x, fma(x.y, x.y, v0));
					v1 = fma(y.x, y.x, fma(y.y, y.y, v1));
					// conj(x) y
					v2 = fma(x.x, y.x, fma(x.y, y.y, v2));
					v3 = fma(x.x, y.y, -fma(x.y, y.x, -v3));
				}
				const double al = warp_sum_z(v0), be = warp_sum_z(v1);
				const double gr = warp_sum_z(v2), gi = warp_sum_z(v3);
				const double gabs = sqrt(gr * gr + gi * gi);
				if (!(gabs > 1e-15 * sqrt(al * be) && gabs > 1e-300)) continue;
				const double zeta = (be - al) / (2.0 * gabs);
				const double tt = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
				const double cc = 1.0 / sqrt(1.0 + tt * tt);
				const double ss = cc * tt;
				// [x, y] <- [x, y] J, J = [[c, s e^{i phi}], [-s e^{-i phi}, c]], e^{i phi} = gamma / |gamma|
				const double2 se = make_double2(ss * gr / gabs, ss * gi / gabs);
				for (int i = lane; i < R; i += 32)
				{
					const double2 x = wp[i], y = wq[i];
					const double2 sy = cmul(cconj(se), y), sx = cmul(se, x);
					wp[i] = make_double2(cc * x.x - sy.x, cc * x.y - sy.y);
					wq[i] = make_double2(sx.x + cc * y.x, sx.y + cc * y.y);
				}
				double2* vp = V + (i64)p * K;
				double2* vq = V + (i64)q * K;
				for (int i = lane; i < K; i += 32)
				{
					const double2 x = vp[i], y = vq[i];
					const double2 sy = cmul(cconj(se), y), sx = cmul(se, x);
					vp[i] = make_double2(cc * x.x - sy.x, cc * x.y - sy.y);
					vq[i] = make_double2(sx.x + cc * y.x, sx.y + cc * y.y);
				}
				if (lane == 0) sh_rot = 1;
			}
			__syncthreads();
		}
		converged = sh_rot == 0;
		__syncthreads();
	}
	if (threadIdx.x == 0) status[blockIdx.x] = converged ? 0 : 1;
	// column norms, ordered descending (ties keep the column order)
	double* sig = s + d.s_off;
	for (int c = threadIdx.x; c < K; c += blockDim.x)
	{
		double t = 0;
		const double2* wc = W + (i64)c * R;
		for (int i = 0; i < R; i++) t = fma(wc[i].x, wc[i].x, fma(wc[i].y, wc[i].y, t));
		sig[c] = sqrt(t);
	}
	__syncthreads();
	if (threadIdx.x == 0)
	{
		for (int c = 0; c < K; c++) perm[c] = c;
		for (int i = 1; i < K; i++)
		{
			const int pi = perm[i];
			int j = i;
			while (j > 0 && sig[perm[j - 1]] < sig[pi])
			{
				perm[j] = perm[j - 1];
				j--;
			}
			perm[j] = pi;
		}
	}
	__syncthreads();
	// singular vectors of W's columns: U_W[:, k] = W[:, perm k] / sigma; written in the original
	// orientation (A = U_W S V^H, or A = V S U_W^H for the transposed case)
	double2* ub = u + d.u_off;
	double2* vb = vh + d.v_off;
	for (i64 e = threadIdx.x; e < (i64)R * K; e += blockDim.x)
	{
		const int r = (int)(e % R), k = (int)(e / R);
		const int c = perm[k];
		const double sg = sig[c];
		const double2 w = W[(i64)c * R + r];
		const double2 x = sg > 0 ? make_double2(w.x / sg, w.y / sg) : make_double2(0.0, 0.0);
		if (!tr) ub[(i64)r * K + k] = x;                 // U: m x K
		else vb[(i64)k * n + r] = cconj(x);               // Vh: K x n, Vh[k][j] = conj(U_W[j][k])
	}
	for (i64 e = threadIdx.x; e < (i64)K * K; e += blockDim.x)
	{
		const int r = (int)(e % K), k = (int)(e / K);
		const double2 x = V[(i64)perm[k] * K + r];
		if (!tr) vb[(i64)k * n + r] = cconj(x);           // Vh[k][j] = conj(V[j][k]), n = K
		else ub[(i64)r * K + k] = x;                      // U = V: m x K, m = K
	}
	__syncthreads();
	// sorted singular values in place
	if (threadIdx.x == 0)
	{
		for (int k = 0; k < K; k++) sorted[k] = sig[perm[k]];
		for (int k = 0; k < K; k++) sig[k] = sorted[k];
	}
}

// ------------------------------------------------------------------------------------
// complex Householder QR / RQ, one CTA per block (same index mappings as the real kernel)
// ------------------------------------------------------------------------------------

__global__ void __launch_bounds__(256)
k_qr_z(const RqDesc* __restrict__ descs, const double2* __restrict__ a, double2* __restrict__ r,
       double2* __restrict__ q, double2* __restrict__ scratch)
{
	__shared__ double red[8 * 4];
	__shared__ double sh_beta;
	__shared__ double2 sh_tau, sh_scale;
	const RqDesc d = descs[blockIdx.x];
	const int m = d.m, n = d.n;
	const bool qr = d.qr != 0;
	const int k = min(m, n);
	const int p = qr ? m : n, s = qr ? n : m;   // W is p x s, column-major
	double2* B = scratch + d.w_off;
	double2* Q = B + (i64)p * s;
	double2* tau = Q + (i64)p * k;
	const double2* ab = a + d.a_off;
	// RQ: W = J A^H J, so that A = (J R_W^H J)(J Q_W^H J)
	for (i64 e = threadIdx.x; e < (i64)p * s; e += blockDim.x)
	{
		const i64 i = e % p, j = e / p;
		B[e] = qr ? ab[i * n + j] : cconj(ab[(m - 1 - j) * n + (n - 1 - i)]);
	}
	__syncthreads();
	for (int c = 0; c < k; c++)
	{
		double2* bc = B + (i64)c * p;
		double v4[4] = {0, 0, 0, 0};
		for (int i = c + 1 + threadIdx.x; i < p; i += blockDim.x) v4[0] = fma(bc[i].x, bc[i].x, fma(bc[i].y, bc[i].y, v4[0]));
		block_sum4(v4, red);
		const double xnorm2 = v4[0];
		if (threadIdx.x == 0)
		{
			const double2 alpha = bc[c];
			if (xnorm2 == 0.0 && alpha.y == 0.0)
			{
				sh_tau = make_double2(0.0, 0.0);
				sh_beta = alpha.x;
				sh_scale = make_double2(0.0, 0.0);
			}
			else
			{
				// zlarfg: beta = -sign(alpha_r) |(alpha, x)|, tau = (beta - alpha) / beta, v = x / (alpha - beta)
				const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
				sh_tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
				sh_beta = beta;
				const double2 den = make_double2(alpha.x - beta, alpha.y);
				const double dd = den.x * den.x + den.y * den.y;
				sh_scale = make_double2(den.x / dd, -den.y / dd);
			}
		}
		__syncthreads();
		const double2 tc = sh_tau;
		for (int i = c + 1 + threadIdx.x; i < p; i += blockDim.x) bc[i] = cmul(bc[i], sh_scale);
		__syncthreads();
		if (threadIdx.x == 0)
		{
			bc[c] = make_double2(sh_beta, 0.0);
			tau[c] = tc;
		}
		__syncthreads();
		// apply H^H = I - conj(tau) v v^H (v = (1, bc[c+1:])) to the remaining columns
		if (tc.x != 0.0 || tc.y != 0.0)
		{
			for (int c2 = c + 1; c2 < s; c2++)
			{
				double2* b2 = B + (i64)c2 * p;
				double w4[4] = {0, 0, 0, 0};
				for (int i = c + threadIdx.x; i < p; i += blockDim.x)
				{
					const double2 vi = i == c ? make_double2(1.0, 0.0) : bc[i];
					const double2 t = cmul(cconj(vi), b2[i]);
					w4[0] += t.x;
					w4[1] += t.y;
				}
				block_sum4(w4, red);
				const double2 f = cmul(cconj(tc), make_double2(w4[0], w4[1]));
				for (int i = c + threadIdx.x; i < p; i += blockDim.x)
				{
					const double2 vi = i == c ? make_double2(1.0, 0.0) : bc[i];
					const double2 t = cmul(f, vi);
					b2[i] = make_double2(b2[i].x - t.x, b2[i].y - t.y);
				}
				__syncthreads();
			}
		}
		__syncthreads();
	}
	// Q_W = H_0 ... H_{k-1} E (p x k), accumulated backwards
	for (i64 e = threadIdx.x; e < (i64)p * k; e += blockDim.x)
		Q[e] = make_double2((e / p == e % p) ? 1.0 : 0.0, 0.0);
	__syncthreads();
	for (int c = k - 1; c >= 0; c--)
	{
		const double2 tc = tau[c];
		const double2* bc = B + (i64)c * p;
		if (tc.x != 0.0 || tc.y != 0.0)
		{
			for (int j = 0; j < k; j++)
			{
				double2* qj = Q + (i64)j * p;
				double w4[4] = {0, 0, 0, 0};
				for (int i = c + threadIdx.x; i < p; i += blockDim.x)
				{
					const double2 vi = i == c ? make_double2(1.0, 0.0) : bc[i];
					const double2 t = cmul(cconj(vi), qj[i]);
					w4[0] += t.x;
					w4[1] += t.y;
				}
				block_sum4(w4, red);
				const double2 f = cmul(tc, make_double2(w4[0], w4[1]));
				for (int i = c + threadIdx.x; i < p; i += blockDim.x)
				{
					const double2 vi = i == c ? make_double2(1.0, 0.0) : bc[i];
					const double2 t = cmul(f, vi);
					qj[i] = make_double2(qj[i].x - t.x, qj[i].y - t.y);
				}
				__syncthreads();
			}
		}
		__syncthreads();
	}
	if (qr)
	{
		for (i64 e = threadIdx.x; e < (i64)k * n; e += blockDim.x)
		{
			const i64 i = e / n, j = e % n;
			r[d.r_off + e] = (i <= j) ? B[i + (i64)p * j] : make_double2(0.0, 0.0);
		}
		for (i64 e = threadIdx.x; e < (i64)m * k; e += blockDim.x)
		{
			const i64 i = e / k, j = e % k;
			q[d.q_off + e] = Q[i + (i64)p * j];
		}
	}
	else
	{
		for (i64 e = threadIdx.x; e < (i64)m * k; e += blockDim.x)
		{
			const i64 i = e / k, j = e % k;
			const i64 a0 = k - 1 - j, b0 = m - 1 - i;
			r[d.r_off + e] = (a0 <= b0) ? cconj(B[a0 + (i64)p * b0]) : make_double2(0.0, 0.0);
		}
		for (i64 e = threadIdx.x; e < (i64)k * n; e += blockDim.x)
		{
			const i64 j = e / n, i = e % n;
			q[d.q_off + e] = cconj(Q[(n - 1 - i) + (i64)p * (k - 1 - j)]);
		}
	}
}

}  // namespace

void launch_gemm_z(int ntiles, const ZTile* tiles, const GemmOut* outs, const GemmContrib* cons, const double* A,
                   const double* B, double* C, int conj_a, int conj_b, cudaStream_t st)
{
	if (ntiles <= 0) return;
	k_gemm_z<<<ntiles, 256, 0, st>>>(tiles, outs, cons, (const double2*)A, (const double2*)B, (double2*)C, conj_a, conj_b);
	CTG_CUDA(cudaGetLastError());
}

i64 svd_z_scratch(int m, int n)
{
	const i64 R = std::max(m, n), K = std::min(m, n);
	return R * K + K * K + 2 * K;
}

void launch_svd_z(int nblocks, const SvdDesc* descs, const double* a, double* u, double* s, double* vh, double* work,
                  int* status, cudaStream_t st)
{
	if (nblocks <= 0) return;
	k_svd_z<<<nblocks, 256, 0, st>>>(descs, (const double2*)a, (double2*)u, s, (double2*)vh, (double2*)work, status);
	CTG_CUDA(cudaGetLastError());
}

void launch_qr_z(int nblocks, const RqDesc* descs, const double* a, double* r, double* q, double* scratch, cudaStream_t st)
{
	if (nblocks <= 0) return;
	k_qr_z<<<nblocks, 256, 0, st>>>(descs, (const double2*)a, (double2*)r, (double2*)q, (double2*)scratch);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
