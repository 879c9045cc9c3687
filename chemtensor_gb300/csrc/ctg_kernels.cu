// ctg_kernels.cu - FP64 grouped block GEMM and the block data-movement kernels.
#include "ctg_kernels.h"
#include "ctg_launch.cuh"

namespace ctg {

// ------------------------------------------------------------------------------------
// grouped FP64 block GEMM (plain path; dense_tensor_dot_update, dense_tensor.c:1761-1837)
// ------------------------------------------------------------------------------------

constexpr int GEMM_THREADS = 256;     // 16 x 16 thread grid for every tile class
constexpr int GEMM_SMEM_DOUBLES = 16 * (128 + 1 + 8 + 1);
constexpr int GEMM_DIRECT_K = 4;      // contributions up to this k skip the shared-memory staging

template <int BM, int BN, int BK, int TM, int TN>
__device__ __forceinline__ void gemm_tile_f64(const GemmTile& tile, const GemmOut* __restrict__ outs,
                                              const GemmContrib* __restrict__ cons, const GemmSplit* __restrict__ splits,
                                              int* __restrict__ counters, const double* __restrict__ A,
                                              const double* __restrict__ B, double* __restrict__ C,
                                              double* __restrict__ work, double* sm)
{
	constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
	static_assert(NT == GEMM_THREADS && BK * (BM + 1 + BN + 1) <= GEMM_SMEM_DOUBLES, "tile class layout");
	double (*As)[BM + 1] = reinterpret_cast<double (*)[BM + 1]>(sm);
	double (*Bs)[BN + 1] = reinterpret_cast<double (*)[BN + 1]>(sm + BK * (BM + 1));
	const GemmOut o = outs[tile.out];
	const int tid = threadIdx.x;
	const int tx = tid % NTX, ty = tid / NTX;
	double acc[TM][TN];
#pragma unroll
	for (int i = 0; i < TM; i++)
#pragma unroll
		for (int j = 0; j < TN; j++) acc[i][j] = 0.0;

	for (int c = tile.c0; c <= tile.c1; c++)
	{
		const GemmContrib g = cons[c];
		const double* a = A + g.a_off;
		const double* b = B + g.b_off;
		const int kb = (c == tile.c0 ? tile.k0 : 0), ke = (c == tile.c1 ? tile.k1 : g.k);
		if (ke - kb <= GEMM_DIRECT_K)
		{
			// short contraction (most contributions of a block-sparse DMRG contraction have k <= 2):
			// operands straight from global memory through L1, no staging and no barrier. Same
			// accumulation order as the staged path.
#pragma unroll 1
			for (int kk = kb; kk < ke; kk++)
			{
				double av[TM], bv[TN];
#pragma unroll
				for (int i = 0; i < TM; i++)
				{
					const int gi = tile.m0 + ty + i * NTY;
					av[i] = gi < o.m ? a[(i64)gi * g.sAm + (i64)kk * g.sAk] : 0.0;
				}
#pragma unroll
				for (int j = 0; j < TN; j++)
				{
					const int gj = tile.n0 + tx + j * NTX;
					bv[j] = gj < o.n ? b[(i64)kk * g.sBk + (i64)gj * g.sBn] : 0.0;
				}
#pragma unroll
				for (int i = 0; i < TM; i++)
#pragma unroll
					for (int j = 0; j < TN; j++) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
			}
			continue;
		}
		for (int k0 = kb; k0 < ke; k0 += BK)
		{
			// A tile: BM x BK; the thread-to-element map follows the unit-stride index
			if (g.sAk == 1)
			{
				for (int e = tid; e < BM * BK; e += NT)
				{
					const int kk = e % BK, i = e / BK;
					const int gi = tile.m0 + i, gk = k0 + kk;
					As[kk][i] = (gi < o.m && gk < ke) ? a[(i64)gi * g.sAm + gk] : 0.0;
				}
			}
			else
			{
				for (int e = tid; e < BM * BK; e += NT)
				{
					const int i = e % BM, kk = e / BM;
					const int gi = tile.m0 + i, gk = k0 + kk;
					As[kk][i] = (gi < o.m && gk < ke) ? a[(i64)gi * g.sAm + (i64)gk * g.sAk] : 0.0;
				}
			}
			// B tile: BK x BN
			if (g.sBn == 1)
			{
				for (int e = tid; e < BK * BN; e += NT)
				{
					const int j = e % BN, kk = e / BN;
					const int gj = tile.n0 + j, gk = k0 + kk;
					Bs[kk][j] = (gj < o.n && gk < ke) ? b[(i64)gk * g.sBk + gj] : 0.0;
				}
			}
			else
			{
				for (int e = tid; e < BK * BN; e += NT)
				{
					const int kk = e % BK, j = e / BK;
					const int gj = tile.n0 + j, gk = k0 + kk;
					Bs[kk][j] = (gj < o.n && gk < ke) ? b[(i64)gk * g.sBk + (i64)gj * g.sBn] : 0.0;
				}
			}
			__syncthreads();
			const int kmax = min(BK, ke - k0);
			for (int kk = 0; kk < kmax; kk++)
			{
				double av[TM], bv[TN];
#pragma unroll
				for (int i = 0; i < TM; i++) av[i] = As[kk][ty + i * NTY];
#pragma unroll
				for (int j = 0; j < TN; j++) bv[j] = Bs[kk][tx + j * NTX];
#pragma unroll
				for (int i = 0; i < TM; i++)
#pragma unroll
					for (int j = 0; j < TN; j++) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
			}
			__syncthreads();
		}
	}
	if (tile.split >= 0)
	{
		// partial sum of a split tile (full BM x BN, leading dimension BN); the CTA that completes
		// the split last adds the partial sums in share order (deterministic) and writes C
		const GemmSplit sp = splits[tile.split];
		double* w = work + sp.part + (i64)tile.sp * sp.stride;
#pragma unroll
		for (int i = 0; i < TM; i++)
#pragma unroll
			for (int j = 0; j < TN; j++) w[(ty + i * NTY) * BN + tx + j * NTX] = acc[i][j];
		__threadfence();
		__syncthreads();
		__shared__ int last;
		if (tid == 0) last = atomicAdd(counters + tile.split, 1) == sp.nsplit - 1;
		__syncthreads();
		if (!last) return;
		__threadfence();
		for (int e = tid; e < sp.rows * sp.cols; e += NT)
		{
			const int i = e / sp.cols, j = e - i * sp.cols;
			const double* pw = work + sp.part + (i64)i * sp.ld + j;
			double sum = 0.0;
			for (int q = 0; q < sp.nsplit; q++) sum += __ldcg(pw + (i64)q * sp.stride);
			C[gemm_out_index(o, sp.m0 + i, sp.n0 + j)] = sum;
		}
		if (tid == 0) counters[tile.split] = 0;
		return;
	}
#pragma unroll
	for (int i = 0; i < TM; i++)
	{
		const int gi = tile.m0 + ty + i * NTY;
		if (gi >= o.m) continue;
#pragma unroll
		for (int j = 0; j < TN; j++)
		{
			const int gj = tile.n0 + tx + j * NTX;
			if (gj < o.n) C[gemm_out_index(o, gi, gj)] = acc[i][j];
		}
	}
}

__global__ void __launch_bounds__(GEMM_THREADS, 3)
k_gemm_f64(const GemmTile* __restrict__ tiles, const GemmOut* __restrict__ outs, const GemmContrib* __restrict__ cons,
           const GemmSplit* __restrict__ splits, int* __restrict__ counters, const double* __restrict__ A,
           const double* __restrict__ B, double* __restrict__ C, double* __restrict__ work)
{
	pdl_wait();
	pdl_trigger();
	__shared__ double sm[GEMM_SMEM_DOUBLES];
	const GemmTile tile = tiles[blockIdx.x];
	switch (tile.cls)
	{
	case TILE_L: gemm_tile_f64<64, 64, 16, 4, 4>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_M: gemm_tile_f64<32, 32, 16, 2, 2>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_W: gemm_tile_f64<16, 64, 16, 1, 4>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_T: gemm_tile_f64<64, 16, 16, 4, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_R8: gemm_tile_f64<8, 32, 16, 1, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_R4: gemm_tile_f64<4, 64, 16, 1, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_C8: gemm_tile_f64<32, 8, 16, 1, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_C4: gemm_tile_f64<64, 4, 16, 1, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_W8: gemm_tile_f64<8, 128, 16, 1, 4>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	case TILE_T8: gemm_tile_f64<128, 8, 16, 4, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	default:     gemm_tile_f64<16, 16, 16, 1, 1>(tile, outs, cons, splits, counters, A, B, C, work, sm); break;
	}
}

int tile_rows(int cls)
{
	return TILE_ROWS[cls];
}

int tile_cols(int cls)
{
	return TILE_COLS[cls];
}

void launch_gemm_f64(int ntiles, const GemmTile* tiles, const GemmOut* outs, const GemmContrib* cons,
                     const GemmSplit* splits, int* counters, const double* A, const double* B, double* C, double* work,
                     cudaStream_t st, double flops)
{
	if (ntiles <= 0) return;
	// programmatic dependent launch for the short products of a sweep (tens of microseconds); a
	// product of milliseconds gains nothing from it and lost 2 % with it (the next kernel's blocks
	// scheduled beside its last waves)
	const cudaLaunchConfig_t cfg = launch_config(dim3(ntiles), dim3(GEMM_THREADS), 0, st);
	if (flops < 2e8) launch_pdl(cfg, k_gemm_f64, tiles, outs, cons, splits, counters, A, B, C, work);
	else CTG_CUDA(cudaLaunchKernelEx(&cfg, k_gemm_f64, tiles, outs, cons, splits, counters, A, B, C, work));
}

// ------------------------------------------------------------------------------------
// block permutation (dense_tensor_transpose, dense_tensor.c:799-932)
// ------------------------------------------------------------------------------------

// T = double, or double2 for complex128 entries (same descriptors, element units)
template <class T>
__global__ void __launch_bounds__(256)
k_permute(const Chunk* __restrict__ chunks, const PermDesc* __restrict__ descs, const T* __restrict__ src,
          T* __restrict__ dst)
{
	pdl_wait();
	pdl_trigger();
	const Chunk ch = chunks[blockIdx.x];
	const PermDesc d = descs[ch.desc];
	const i64 end = min(d.n, ch.start + (i64)COPY_CHUNK);
	if (d.n < ((i64)1 << 31))
	{
		// 32-bit index arithmetic (64-bit integer division is several times slower)
		for (int e = (int)ch.start + threadIdx.x; e < (int)end; e += blockDim.x)
		{
			unsigned r = (unsigned)e;
			i64 so = 0;
			for (int i = d.ndim - 1; i >= 0; i--)
			{
				const unsigned di = (unsigned)d.dims[i];
				const unsigned q = r / di;
				so += (i64)(r - q * di) * d.sstr[i];
				r = q;
			}
			dst[d.dst_off + e] = src[d.src_off + so];
		}
		return;
	}
	for (i64 e = ch.start + threadIdx.x; e < end; e += blockDim.x)
	{
		i64 r = e, so = 0;
		for (int i = d.ndim - 1; i >= 0; i--)
		{
			const i64 q = r / d.dims[i];
			so += (r - q * d.dims[i]) * d.sstr[i];
			r = q;
		}
		dst[d.dst_off + e] = src[d.src_off + so];
	}
}

void launch_permute(int nchunks, const Chunk* chunks, const PermDesc* descs, const double* src, double* dst, cudaStream_t st,
                    bool cplx)
{
	if (nchunks <= 0) return;
	const cudaLaunchConfig_t cfg = launch_config(dim3(nchunks), dim3(256), 0, st);
	if (cplx) launch_pdl(cfg, k_permute<double2>, chunks, descs, (const double2*)src, (double2*)dst);
	else launch_pdl(cfg, k_permute<double>, chunks, descs, src, dst);
	CTG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------
// row maps: flatten / split / slice (block_sparse_tensor.c:950-1553)
// ------------------------------------------------------------------------------------

template <class T>
__global__ void __launch_bounds__(256)
k_rowmap(const Chunk* __restrict__ chunks, const RowDesc* __restrict__ descs, const i64* __restrict__ maps,
         const T* __restrict__ src, T* __restrict__ dst)
{
	pdl_wait();
	pdl_trigger();
	const Chunk ch = chunks[blockIdx.x];
	const RowDesc d = descs[ch.desc];
	const i64 n = d.nlead * d.nrow * d.ntrail;
	const i64 end = min(n, ch.start + (i64)COPY_CHUNK);
	const i64* map = maps + d.map_off;
	if (n < ((i64)1 << 31))
	{
		// 32-bit index arithmetic (64-bit integer division is several times slower)
		const unsigned nt = (unsigned)d.ntrail, nr = (unsigned)d.nrow;
		for (unsigned e = (unsigned)ch.start + threadIdx.x; e < (unsigned)end; e += blockDim.x)
		{
			const unsigned lj = e / nt;
			const unsigned t = e - lj * nt;
			const unsigned lead = lj / nr;
			const unsigned j = lj - lead * nr;
			const i64 mj = map[j];
			const i64 srow = d.scatter ? (i64)j : mj;
			const i64 drow = d.scatter ? mj : (i64)j;
			dst[d.dst_off + ((i64)lead * d.dst_rows + drow) * d.ntrail + t] =
				src[d.src_off + ((i64)lead * d.src_rows + srow) * d.ntrail + t];
		}
		return;
	}
	for (i64 e = ch.start + threadIdx.x; e < end; e += blockDim.x)
	{
		const i64 t = e % d.ntrail;
		const i64 lj = e / d.ntrail;
		const i64 j = lj % d.nrow;
		const i64 lead = lj / d.nrow;
		const i64 mj = map[j];
		const i64 srow = d.scatter ? j : mj;
		const i64 drow = d.scatter ? mj : j;
		dst[d.dst_off + (lead * d.dst_rows + drow) * d.ntrail + t] = src[d.src_off + (lead * d.src_rows + srow) * d.ntrail + t];
	}
}

void launch_rowmap(int nchunks, const Chunk* chunks, const RowDesc* descs, const i64* maps, const double* src, double* dst,
                   cudaStream_t st, bool cplx)
{
	if (nchunks <= 0) return;
	const cudaLaunchConfig_t cfg = launch_config(dim3(nchunks), dim3(256), 0, st);
	if (cplx) launch_pdl(cfg, k_rowmap<double2>, chunks, descs, maps, (const double2*)src, (double2*)dst);
	else launch_pdl(cfg, k_rowmap<double>, chunks, descs, maps, src, dst);
	CTG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------
// pointwise multiplication along an axis (block_sparse_tensor_multiply_pointwise_vector,
// block_sparse_tensor.c:1654-1703)
// ------------------------------------------------------------------------------------

__device__ __forceinline__ double scale_entry(double x, double f) { return x * f; }
__device__ __forceinline__ double2 scale_entry(double2 x, double f) { return make_double2(x.x * f, x.y * f); }

template <class T>
__global__ void __launch_bounds__(256)
k_scale_axis(const Chunk* __restrict__ chunks, const ScaleDesc* __restrict__ descs, const i64* __restrict__ maps,
             const double* __restrict__ vec, const T* __restrict__ src, T* __restrict__ dst)
{
	pdl_wait();
	pdl_trigger();
	const Chunk ch = chunks[blockIdx.x];
	const ScaleDesc d = descs[ch.desc];
	const i64 n = d.nlead * d.nax * d.ntrail;
	const i64 end = min(n, ch.start + (i64)COPY_CHUNK);
	if (n < ((i64)1 << 31))
	{
		const unsigned nt = (unsigned)d.ntrail, na = (unsigned)d.nax;
		for (unsigned e = (unsigned)ch.start + threadIdx.x; e < (unsigned)end; e += blockDim.x)
		{
			const unsigned q = e / nt;
			const unsigned p = q - (q / na) * na;
			dst[d.off + e] = scale_entry(src[d.off + e], vec[maps[d.map_off + p]]);
		}
		return;
	}
	for (i64 e = ch.start + threadIdx.x; e < end; e += blockDim.x)
	{
		const i64 p = (e / d.ntrail) % d.nax;
		dst[d.off + e] = scale_entry(src[d.off + e], vec[maps[d.map_off + p]]);
	}
}

void launch_scale_axis(int nchunks, const Chunk* chunks, const ScaleDesc* descs, const i64* maps, const double* vec,
                       const double* src, double* dst, cudaStream_t st, bool cplx)
{
	if (nchunks <= 0) return;
	const cudaLaunchConfig_t cfg = launch_config(dim3(nchunks), dim3(256), 0, st);
	if (cplx) launch_pdl(cfg, k_scale_axis<double2>, chunks, descs, maps, vec, (const double2*)src, (double2*)dst);
	else launch_pdl(cfg, k_scale_axis<double>, chunks, descs, maps, vec, src, dst);
	CTG_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------
// FP64 FMA throughput probe: the denominator of the plain path's roofline
// ------------------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_fp64_fma(double* out, int iters, double a, double b)
{
	double x[8];
#pragma unroll
	for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-9 + i;
	for (int it = 0; it < iters; it++)
	{
#pragma unroll
		for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
	}
	double s = 0;
#pragma unroll
	for (int i = 0; i < 8; i++) s += x[i];
	if (s == 12345.678) out[0] = s;   // keeps the chains alive
}

double measure_fp64_fma_tflops(int device)
{
	CTG_CUDA(cudaSetDevice(device));
	int sms = 0;
	CTG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
	double* out = nullptr;
	CTG_CUDA(cudaMalloc(&out, sizeof(double)));
	cudaEvent_t e0, e1;
	CTG_CUDA(cudaEventCreate(&e0));
	CTG_CUDA(cudaEventCreate(&e1));
	const int blocks = sms * 8, threads = 256, iters = 4096;
	k_fp64_fma<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);
	CTG_CUDA(cudaEventRecord(e0));
	for (int r = 0; r < 5; r++) k_fp64_fma<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
	CTG_CUDA(cudaEventRecord(e1));
	CTG_CUDA(cudaEventSynchronize(e1));
	float ms = 0;
	CTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	const double flops = 5.0 * blocks * threads * (double)iters * 8 * 2;
	return flops / (ms * 1e-3) / 1e12;
}

}  // namespace ctg
