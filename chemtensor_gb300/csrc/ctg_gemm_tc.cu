// ctg_gemm_tc.cu - grouped block GEMM on the 5th-generation tensor cores (tcgen05), split-BF16.
//
// Same work lists as the FP64 grouped GEMM (GemmOut / GemmContrib / GemmTile): every output block
// C = sum_j op(A_j) op(B_j) with arbitrary element strides for the operands. Each FP64 operand
// value x is split into x_hi = bf16(x) and x_lo = bf16(x - x_hi) once per product by k_split_bf16
// (into two BF16 arrays with the operand's layout), and the product is taken as
// A_hi B_hi + A_hi B_lo + A_lo B_hi (the 3-product split-BF16 form; the dropped A_lo B_lo term and
// the FP32 accumulation give a relative error of about 2^-16). Output in FP64.
//
// Per CTA: one 128 x TC_BN tile of one output block. Four warps stage the BF16 operand tiles into
// shared memory in the canonical no-swizzle K-major layout of the tensor-core shared-memory
// descriptors, double-buffered: while the tensor cores work on one stage the next one is loaded.
// One thread issues the tcgen05.mma instructions into an FP32 accumulator in tensor memory and
// commits each stage to that stage's mbarrier; the epilogue reads the accumulator with tcgen05.ld
// and writes FP64. Every wait on an mbarrier is bounded: on timeout the CTA records an error flag,
// stops issuing work, frees its tensor memory and returns.
#include <algorithm>

#include <cuda_bf16.h>

#include "ctg_kernels.h"

namespace ctg {

namespace {

constexpr int TC_BM = 128;                 // tile rows (MMA M)
constexpr int TC_BN = 64;                  // tile columns (MMA N)
constexpr int TC_BK = 64;                  // K elements per shared-memory stage
constexpr int TC_THREADS = 128;
constexpr int TC_TMEM_COLS = 64;           // FP32 accumulator columns (= TC_BN), power of two >= 32
// canonical no-swizzle K-major layout: 8 x 16-byte core matrices; (row, k) ->
// (row / 8) * SBO + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2
constexpr int TC_LBO = 128;                // bytes between core matrices adjacent in K
constexpr int TC_SBO = (TC_BK / 8) * 128;  // bytes between core matrices adjacent in M / N
constexpr int A_TILE_BYTES = TC_BM * TC_BK * 2;
constexpr int B_TILE_BYTES = TC_BN * TC_BK * 2;
constexpr int STAGE_BYTES = 2 * A_TILE_BYTES + 2 * B_TILE_BYTES;   // hi and lo of A and B
constexpr int TC_STAGES = 2;
constexpr int TC_SMEM_BYTES = TC_STAGES * STAGE_BYTES + 64;
constexpr long long TC_WAIT_LIMIT = 1ll << 26;   // spins before a wait is declared failed

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t canon_offset(int row, int k)
{
	return (uint32_t)((row >> 3) * TC_SBO + (k >> 3) * TC_LBO + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor (no swizzle, K-major)
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr)
{
	uint64_t d = 0;
	d |= (uint64_t)((saddr >> 4) & 0x3FFF);
	d |= (uint64_t)((TC_LBO >> 4) & 0x3FFF) << 16;
	d |= (uint64_t)((TC_SBO >> 4) & 0x3FFF) << 32;
	d |= (uint64_t)1 << 46;                // descriptor version for this architecture
	return d;                              // base offset 0, swizzle none
}

// instruction descriptor: kind::f16 with BF16 A and B, FP32 D, both K-major, M = 128, N = TC_BN
__device__ __forceinline__ uint32_t make_idesc()
{
	uint32_t d = 0;
	d |= 1u << 4;                          // D format FP32
	d |= 1u << 7;                          // A format BF16
	d |= 1u << 10;                         // B format BF16
	d |= (uint32_t)(TC_BN >> 3) << 17;     // N / 8
	d |= (uint32_t)(TC_BM >> 4) << 24;     // M / 16
	return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
		:
		: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, int count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// bounded wait for the given phase parity; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
	for (long long it = 0; it < TC_WAIT_LIMIT; it++)
	{
		uint32_t done = 0;
		asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.b32 %0, 1, 0, p;\n\t}"
			: "=r"(done)
			: "r"(mbar), "r"(parity)
			: "memory");
		if (done) return true;
		if (it > 64) __nanosleep(64);
	}
	return false;
}

__device__ __forceinline__ void fence_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__global__ void __launch_bounds__(256)
k_split_bf16(const double* __restrict__ x, i64 n, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo)
{
	for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
	{
		// FP32 keeps 24 bits of x, more than the 16 that hi + lo carry
		const float f = (float)x[i];
		const __nv_bfloat16 h = __float2bfloat16_rn(f);
		hi[i] = h;
		lo[i] = __float2bfloat16_rn(f - __bfloat162float(h));
	}
}

__global__ void __launch_bounds__(TC_THREADS)
k_gemm_bf16x3(const GemmTile* __restrict__ tiles, const GemmOut* __restrict__ outs, const GemmContrib* __restrict__ cons,
              const unsigned short* __restrict__ Ahi, const unsigned short* __restrict__ Alo,
              const unsigned short* __restrict__ Bhi, const unsigned short* __restrict__ Blo, double* __restrict__ C,
              int* __restrict__ error)
{
	extern __shared__ __align__(1024) unsigned char smem[];
	uint64_t* mbar = (uint64_t*)(smem + TC_STAGES * STAGE_BYTES);     // one per stage
	uint32_t* tmem_slot = (uint32_t*)(mbar + TC_STAGES);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const GemmTile tile = tiles[blockIdx.x];
	const GemmOut o = outs[tile.out];

	if (warp == 0)
	{
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
		             "r"(TC_TMEM_COLS)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0)
		for (int s = 0; s < TC_STAGES; s++) mbar_init(smem_u32(mbar + s), 1);
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;
	const uint32_t idesc = make_idesc();
	bool ok = true;
	int chunk = 0;                                      // k chunks issued so far

	for (int c = o.c0; c < o.c0 + o.nc && ok; c++)
	{
		const GemmContrib g = cons[c];
		for (int k0 = 0; k0 < g.k && ok; k0 += TC_BK, chunk++)
		{
			const int st = chunk % TC_STAGES;
			unsigned char* a_hi = smem + st * STAGE_BYTES;
			unsigned char* a_lo = a_hi + A_TILE_BYTES;
			unsigned char* b_hi = a_lo + A_TILE_BYTES;
			unsigned char* b_lo = b_hi + B_TILE_BYTES;
			if (chunk >= TC_STAGES)
			{
				// the MMAs that read this stage (chunk - TC_STAGES) must be complete
				const bool arrived = mbar_wait(smem_u32(mbar + st), (uint32_t)((chunk / TC_STAGES - 1) & 1));
				ok = __syncthreads_and(arrived ? 1 : 0) != 0;
				if (!ok) break;
				tc_fence_after();
			}
			// A tile: 128 x 64, element (i, kk) -> (m0 + i, k0 + kk); zero outside the block
			for (int e = tid; e < TC_BM * TC_BK; e += TC_THREADS)
			{
				int i, kk;
				if (g.sAk == 1) { kk = e % TC_BK; i = e / TC_BK; }
				else { i = e % TC_BM; kk = e / TC_BM; }
				const int gi = tile.m0 + i, gk = k0 + kk;
				unsigned short h = 0, l = 0;
				if (gi < o.m && gk < g.k)
				{
					const i64 off = g.a_off + (i64)gi * g.sAm + (i64)gk * g.sAk;
					h = Ahi[off];
					l = Alo[off];
				}
				const uint32_t so = canon_offset(i, kk);
				*(unsigned short*)(a_hi + so) = h;
				*(unsigned short*)(a_lo + so) = l;
			}
			// B tile as N x K (K-major): element (j, kk) = op(B)(k0 + kk, n0 + j)
			for (int e = tid; e < TC_BN * TC_BK; e += TC_THREADS)
			{
				int j, kk;
				if (g.sBk == 1) { kk = e % TC_BK; j = e / TC_BK; }
				else { j = e % TC_BN; kk = e / TC_BN; }
				const int gj = tile.n0 + j, gk = k0 + kk;
				unsigned short h = 0, l = 0;
				if (gj < o.n && gk < g.k)
				{
					const i64 off = g.b_off + (i64)gk * g.sBk + (i64)gj * g.sBn;
					h = Bhi[off];
					l = Blo[off];
				}
				const uint32_t so = canon_offset(j, kk);
				*(unsigned short*)(b_hi + so) = h;
				*(unsigned short*)(b_lo + so) = l;
			}
			fence_async_smem();
			tc_fence_before();
			__syncthreads();
			tc_fence_after();
			if (tid == 0)
			{
				const int ksteps = (min(TC_BK, g.k - k0) + 15) / 16;
				for (int s = 0; s < ksteps; s++)
				{
					const uint32_t koff = (uint32_t)s * 2 * TC_LBO;
					const uint64_t dah = make_desc(smem_u32(a_hi) + koff), dal = make_desc(smem_u32(a_lo) + koff);
					const uint64_t dbh = make_desc(smem_u32(b_hi) + koff), dbl = make_desc(smem_u32(b_lo) + koff);
					mma_bf16(tmem, dah, dbh, idesc, chunk > 0 || s > 0);
					mma_bf16(tmem, dah, dbl, idesc, true);
					mma_bf16(tmem, dal, dbh, idesc, true);
				}
				mma_commit(smem_u32(mbar + st));
			}
		}
	}
	if (ok && chunk > 0)
	{
		// the last commit tracks every MMA issued before it
		const int last = chunk - 1;
		const bool arrived = mbar_wait(smem_u32(mbar + last % TC_STAGES), (uint32_t)((last / TC_STAGES) & 1));
		ok = __syncthreads_and(arrived ? 1 : 0) != 0;
	}
	if (!ok && lane == 0) atomicExch(error, 1);
	tc_fence_after();

	// epilogue: each warp owns 32 accumulator rows (tensor-memory lanes 32 w .. 32 w + 31)
	const int row = tile.m0 + warp * 32 + lane;
	double* cblk = C + o.c_off;
	const bool have_acc = ok && chunk > 0;
	for (int cc = 0; cc < TC_BN; cc += 16)
	{
		uint32_t v[16];
		if (have_acc)
		{
			const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
			asm volatile(
				"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
				: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
				  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
				: "r"(taddr));
			asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
		}
		else
		{
			for (int t = 0; t < 16; t++) v[t] = 0u;
		}
		if (row < o.m)
		{
			for (int t = 0; t < 16; t++)
			{
				const int col = tile.n0 + cc + t;
				if (col < o.n) cblk[(i64)row * o.n + col] = (double)__uint_as_float(v[t]);
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0)
	{
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
	}
}

}  // namespace

int tc_tile_rows() { return TC_BM; }
int tc_tile_cols() { return TC_BN; }

void launch_split_bf16(const double* x, i64 n, void* hi, void* lo, cudaStream_t st)
{
	if (n <= 0) return;
	const i64 blocks = std::min<i64>((n + 255) / 256, 4 * 152);
	k_split_bf16<<<(int)blocks, 256, 0, st>>>(x, n, (__nv_bfloat16*)hi, (__nv_bfloat16*)lo);
	CTG_CUDA(cudaGetLastError());
}

void launch_gemm_bf16x3(int ntiles, const GemmTile* tiles, const GemmOut* outs, const GemmContrib* cons,
                        const void* Ahi, const void* Alo, const void* Bhi, const void* Blo, double* C, int* error,
                        cudaStream_t st)
{
	if (ntiles <= 0) return;
	static bool attr_set = false;
	if (!attr_set)
	{
		CTG_CUDA(cudaFuncSetAttribute(k_gemm_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES));
		attr_set = true;
	}
	k_gemm_bf16x3<<<ntiles, TC_THREADS, TC_SMEM_BYTES, st>>>(tiles, outs, cons, (const unsigned short*)Ahi,
	                                                           (const unsigned short*)Alo, (const unsigned short*)Bhi,
	                                                           (const unsigned short*)Blo, C, error);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
