// ctg_gemm_tc.cu - grouped block GEMM on the 5th-generation tensor cores (tcgen05), split-BF16.
//
// Same work lists as the FP64 grouped GEMM (GemmOut / GemmContrib / GemmTile): every output block
// C = sum_j op(A_j) op(B_j) with arbitrary element strides for the operands. Each FP64 operand
// value x is split into x_hi = bf16(x) and x_lo = bf16(x - x_hi), and the product is taken as
// A_hi B_hi + A_hi B_lo + A_lo B_hi (the 3-product split-BF16 form; the dropped A_lo B_lo term and
// the FP32 accumulation give a relative error of about 2^-16). Output in FP64.
//
// Per CTA: one 128 x TC_BN tile of one output block. Four warps load the operand tiles (FP64 ->
// hi / lo BF16 in registers) into shared memory in the canonical no-swizzle K-major layout of the
// tensor-core shared-memory descriptors; one thread issues the tcgen05.mma instructions into an
// FP32 accumulator in tensor memory and commits them to an mbarrier; the epilogue reads the
// accumulator with tcgen05.ld and writes FP64. Every wait on the mbarrier is bounded: on timeout
// the CTA records an error flag, stops issuing work, frees its tensor memory and returns.
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
constexpr int TC_SMEM_BYTES = 2 * A_TILE_BYTES + 2 * B_TILE_BYTES + 64;
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

__device__ __forceinline__ void split_store(unsigned char* hi, unsigned char* lo, uint32_t off, double x)
{
	const __nv_bfloat16 h = __float2bfloat16_rn((float)x);
	const __nv_bfloat16 l = __float2bfloat16_rn((float)(x - (double)__bfloat162float(h)));
	*(__nv_bfloat16*)(hi + off) = h;
	*(__nv_bfloat16*)(lo + off) = l;
}

__global__ void __launch_bounds__(TC_THREADS)
k_gemm_bf16x3(const GemmTile* __restrict__ tiles, const GemmOut* __restrict__ outs, const GemmContrib* __restrict__ cons,
              const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ C, int* __restrict__ error)
{
	extern __shared__ __align__(1024) unsigned char smem[];
	unsigned char* a_hi = smem;
	unsigned char* a_lo = a_hi + A_TILE_BYTES;
	unsigned char* b_hi = a_lo + A_TILE_BYTES;
	unsigned char* b_lo = b_hi + B_TILE_BYTES;
	uint64_t* mbar = (uint64_t*)(b_lo + B_TILE_BYTES);
	uint32_t* tmem_slot = (uint32_t*)(mbar + 1);
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
	if (tid == 0) mbar_init(smem_u32(mbar), 1);
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;
	const uint32_t idesc = make_idesc();
	uint32_t phase = 0;
	bool issued_any = false;
	bool ok = true;

	for (int c = o.c0; c < o.c0 + o.nc && ok; c++)
	{
		const GemmContrib g = cons[c];
		const double* a = A + g.a_off;
		const double* b = B + g.b_off;
		for (int k0 = 0; k0 < g.k && ok; k0 += TC_BK)
		{
			// A tile: 128 x 64, element (i, kk) -> (m0 + i, k0 + kk); zero outside the block
			for (int e = tid; e < TC_BM * TC_BK; e += TC_THREADS)
			{
				int i, kk;
				if (g.sAk == 1) { kk = e % TC_BK; i = e / TC_BK; }
				else { i = e % TC_BM; kk = e / TC_BM; }
				const int gi = tile.m0 + i, gk = k0 + kk;
				const double x = (gi < o.m && gk < g.k) ? a[(i64)gi * g.sAm + (i64)gk * g.sAk] : 0.0;
				split_store(a_hi, a_lo, canon_offset(i, kk), x);
			}
			// B tile as N x K (K-major): element (j, kk) = op(B)(k0 + kk, n0 + j)
			for (int e = tid; e < TC_BN * TC_BK; e += TC_THREADS)
			{
				int j, kk;
				if (g.sBk == 1) { kk = e % TC_BK; j = e / TC_BK; }
				else { j = e % TC_BN; kk = e / TC_BN; }
				const int gj = tile.n0 + j, gk = k0 + kk;
				const double x = (gj < o.n && gk < g.k) ? b[(i64)gk * g.sBk + (i64)gj * g.sBn] : 0.0;
				split_store(b_hi, b_lo, canon_offset(j, kk), x);
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
					mma_bf16(tmem, dah, dbh, idesc, issued_any);
					mma_bf16(tmem, dah, dbl, idesc, true);
					mma_bf16(tmem, dal, dbh, idesc, true);
					issued_any = true;
				}
				mma_commit(smem_u32(mbar));
			}
			// every thread waits until the tensor cores have read this stage; the outcome is made
			// uniform over the CTA so that all threads leave the loop together
			const bool arrived = mbar_wait(smem_u32(mbar), phase);
			phase ^= 1;
			ok = __syncthreads_and(arrived ? 1 : 0) != 0;
			issued_any = true;
		}
	}
	if (!ok && lane == 0) atomicExch(error, 1);
	tc_fence_after();

	// epilogue: each warp owns 32 accumulator rows (tensor-memory lanes 32 w .. 32 w + 31)
	const int row = tile.m0 + warp * 32 + lane;
	double* cblk = C + o.c_off;
	const bool have_acc = ok && o.nc > 0;
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

void launch_gemm_bf16x3(int ntiles, const GemmTile* tiles, const GemmOut* outs, const GemmContrib* cons, const double* A,
                        const double* B, double* C, int* error, cudaStream_t st)
{
	if (ntiles <= 0) return;
	static bool attr_set = false;
	if (!attr_set)
	{
		CTG_CUDA(cudaFuncSetAttribute(k_gemm_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES));
		attr_set = true;
	}
	k_gemm_bf16x3<<<ntiles, TC_THREADS, TC_SMEM_BYTES, st>>>(tiles, outs, cons, A, B, C, error);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
