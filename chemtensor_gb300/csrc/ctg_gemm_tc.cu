// ctg_gemm_tc.cu - grouped block GEMM on the 5th-generation tensor cores (tcgen05), split-BF16.
//
// Same work lists as the FP64 grouped GEMM (GemmOut / GemmTile) with one TcContrib per
// contribution: every output block C = sum_j op(A_j) op(B_j). Each FP64 operand value x is split
// into x_hi = bf16(x) and x_lo = bf16(x - x_hi), and the product is taken as
// A_hi B_hi + A_hi B_lo + A_lo B_hi (the 3-product split-BF16 form; the dropped A_lo B_lo term and
// the FP32 accumulation give a relative error of about 2^-16). Output in FP64.
//
// k_tc_pack writes the operands as records of K-major tiles (hi and lo, canonical no-swizzle
// core-matrix layout of the tensor-core shared-memory descriptors), so that the GEMM moves a tile
// into shared memory with one bulk copy. k_gemm_tc: one CTA per 128 x 64 output tile; one thread
// runs a two-stage pipeline - bulk copies of the A and B records of k chunk t complete on stage
// t's "full" mbarrier (expect-tx), the tcgen05.mma instructions of chunk t - 1 (3 products x 4
// k-steps of 16) accumulate in FP32 in tensor memory and are committed to that stage's "done"
// mbarrier, which frees the stage for chunk t + 1. The epilogue reads the accumulator with
// tcgen05.ld, stages it in shared memory and writes FP64 rows, coalesced, into the output block's
// layout (which may be that of a transposed result, see GemmOut). Every wait is bounded: on timeout the CTA records an error flag,
// stops issuing work, waits (bounded) for its copies in flight, frees its tensor memory and returns.
#include <algorithm>

#include <cuda_bf16.h>

#include <mutex>

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
constexpr int STAGE_BYTES = 2 * A_TILE_BYTES + 2 * B_TILE_BYTES;   // one A record + one B record
constexpr int TC_STAGES = 2;
constexpr int TC_SMEM_BYTES = TC_STAGES * STAGE_BYTES + 128;
static_assert(2 * A_TILE_BYTES == TC_A_REC_BYTES && 2 * B_TILE_BYTES == TC_B_REC_BYTES, "record layout");
static_assert(TC_BM == TC_A_ROWS && TC_BN == TC_B_ROWS && TC_BK == TC_K, "tile shape");
static_assert(TC_BM * (TC_BN + 1) * 4 <= TC_STAGES * STAGE_BYTES, "epilogue tile fits in the stage buffers");
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

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// global -> shared bulk copy completing on an mbarrier (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
	             "l"(src), "r"(bytes), "r"(mbar)
	             : "memory");
}

__device__ __forceinline__ void fence_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

template <int R>
__global__ void __launch_bounds__(128) k_tc_pack(const TcPack* __restrict__ packs, const double* __restrict__ src,
                                                 unsigned char* __restrict__ dst)
{
	const TcPack p = packs[blockIdx.x];
	unsigned char* hi = dst + p.rec * (i64)(2 * R * TC_BK * 2);
	unsigned char* lo = hi + R * TC_BK * 2;
	for (int e = threadIdx.x; e < R * TC_BK; e += blockDim.x)
	{
		// consecutive threads read consecutive addresses along the unit-stride index
		int i, kk;
		if (p.s_k == 1) { kk = e % TC_BK; i = e / TC_BK; }
		else { i = e % R; kk = e / R; }
		const int gi = p.row0 + i, gk = p.k0 + kk;
		// FP32 keeps 24 bits of x, more than the 16 that hi + lo carry
		float f = 0.0f;
		if (gi < p.rows && gk < p.k) f = (float)src[p.src + (i64)gi * p.s_row + (i64)gk * p.s_k];
		const __nv_bfloat16 h = __float2bfloat16_rn(f);
		const uint32_t so = canon_offset(i, kk);
		*(__nv_bfloat16*)(hi + so) = h;
		*(__nv_bfloat16*)(lo + so) = __float2bfloat16_rn(f - __bfloat162float(h));
	}
}

__global__ void __launch_bounds__(TC_THREADS)
k_gemm_tc(const GemmTile* __restrict__ tiles, const GemmOut* __restrict__ outs, const TcContrib* __restrict__ tcons,
          const unsigned char* __restrict__ apack, const unsigned char* __restrict__ bpack, double* __restrict__ C,
          int* __restrict__ error)
{
	extern __shared__ __align__(1024) unsigned char smem[];
	uint64_t* full = (uint64_t*)(smem + TC_STAGES * STAGE_BYTES);     // copies of a stage landed
	uint64_t* done = full + TC_STAGES;                                 // MMAs of a stage finished
	uint32_t* tmem_slot = (uint32_t*)(done + TC_STAGES);
	int* sh_ok = (int*)(tmem_slot + 1);
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
	{
		for (int s = 0; s < TC_STAGES; s++)
		{
			mbar_init(smem_u32(full + s), 1);
			mbar_init(smem_u32(done + s), 1);
		}
		*sh_ok = 1;
	}
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;
	int nchunks = 0;
	for (int c = o.c0; c < o.c0 + o.nc; c++) nchunks += tcons[c].kt;

	if (tid == 0 && nchunks > 0)
	{
		const uint32_t idesc = make_idesc();
		const int mt = tile.m0 / TC_BM, nt = tile.n0 / TC_BN;
		int lc = o.c0, lk = 0;           // load cursor: contribution, k tile
		bool ok = true;
		int issued = 0;                  // chunks whose copies were issued
		for (int t = 0; t <= nchunks && ok; t++)
		{
			if (t < nchunks)
			{
				const int st = t % TC_STAGES;
				if (t >= TC_STAGES && !mbar_wait(smem_u32(done + st), (uint32_t)(((t - TC_STAGES) / TC_STAGES) & 1)))
				{
					ok = false;
					break;
				}
				while (lk >= tcons[lc].kt) { lc++; lk = 0; }
				const TcContrib g = tcons[lc];
				const unsigned char* arec = apack + (g.a_rec + (i64)mt * g.kt + lk) * TC_A_REC_BYTES;
				const unsigned char* brec = bpack + (g.b_rec + (i64)nt * g.kt + lk) * TC_B_REC_BYTES;
				const uint32_t sbase = smem_u32(smem + st * STAGE_BYTES);
				mbar_expect_tx(smem_u32(full + st), (uint32_t)STAGE_BYTES);
				bulk_copy(sbase, arec, (uint32_t)TC_A_REC_BYTES, smem_u32(full + st));
				bulk_copy(sbase + (uint32_t)TC_A_REC_BYTES, brec, (uint32_t)TC_B_REC_BYTES, smem_u32(full + st));
				issued = t + 1;
				lk++;
			}
			if (t >= 1)
			{
				const int u = t - 1, su = u % TC_STAGES;
				if (!mbar_wait(smem_u32(full + su), (uint32_t)((u / TC_STAGES) & 1)))
				{
					ok = false;
					break;
				}
				tc_fence_after();
				const uint32_t a_hi = smem_u32(smem + su * STAGE_BYTES);
				const uint32_t a_lo = a_hi + A_TILE_BYTES;
				const uint32_t b_hi = a_lo + A_TILE_BYTES;
				const uint32_t b_lo = b_hi + B_TILE_BYTES;
				for (int s = 0; s < TC_BK / 16; s++)
				{
					const uint32_t koff = (uint32_t)s * 2 * TC_LBO;
					const uint64_t dah = make_desc(a_hi + koff), dal = make_desc(a_lo + koff);
					const uint64_t dbh = make_desc(b_hi + koff), dbl = make_desc(b_lo + koff);
					mma_bf16(tmem, dah, dbh, idesc, u > 0 || s > 0);
					mma_bf16(tmem, dah, dbl, idesc, true);
					mma_bf16(tmem, dal, dbh, idesc, true);
				}
				mma_commit(smem_u32(done + su));
			}
		}
		if (ok)
		{
			// the last commit tracks every MMA issued before it
			const int last = nchunks - 1;
			ok = mbar_wait(smem_u32(done + last % TC_STAGES), (uint32_t)((last / TC_STAGES) & 1));
		}
		else
		{
			// let the copies in flight land before the CTA's shared memory is released
			for (int u = issued - TC_STAGES; u < issued; u++)
				if (u >= 0) mbar_wait(smem_u32(full + u % TC_STAGES), (uint32_t)((u / TC_STAGES) & 1));
		}
		if (!ok)
		{
			*sh_ok = 0;
			atomicExch(error, 1);
		}
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const bool have_acc = *sh_ok && nchunks > 0;

	// epilogue: each warp reads its 32 accumulator rows (tensor-memory lanes 32 w .. 32 w + 31) into
	// a padded FP32 tile in the (now idle) stage buffers; then the CTA writes the tile row by row,
	// consecutive threads on consecutive columns, into the block's output layout (plain row-major,
	// or the layout of a transposed result: gemm_out_index)
	float* stile = (float*)smem;                                        // TC_BM x (TC_BN + 1)
	if (have_acc)
	{
		for (int cc = 0; cc < TC_BN; cc += 16)
		{
			uint32_t v[16];
			const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
			asm volatile(
				"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
				: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
				  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
				: "r"(taddr));
			asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
			float* srow = stile + (warp * 32 + lane) * (TC_BN + 1) + cc;
			for (int t = 0; t < 16; t++) srow[t] = __uint_as_float(v[t]);
		}
	}
	__syncthreads();
	const int rows = min(TC_BM, o.m - tile.m0), cols = min(TC_BN, o.n - tile.n0);
	for (int e = tid; e < TC_BM * TC_BN; e += TC_THREADS)
	{
		const int r = e / TC_BN, cl = e % TC_BN;
		if (r < rows && cl < cols)
			C[gemm_out_index(o, tile.m0 + r, tile.n0 + cl)] = have_acc ? (double)stile[r * (TC_BN + 1) + cl] : 0.0;
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

void launch_tc_pack(int nrec, const TcPack* packs, int a_side, const double* src, void* dst, cudaStream_t st)
{
	if (nrec <= 0) return;
	if (a_side) k_tc_pack<TC_A_ROWS><<<nrec, 128, 0, st>>>(packs, src, (unsigned char*)dst);
	else k_tc_pack<TC_B_ROWS><<<nrec, 128, 0, st>>>(packs, src, (unsigned char*)dst);
	CTG_CUDA(cudaGetLastError());
}

void launch_gemm_tc(int ntiles, const GemmTile* tiles, const GemmOut* outs, const TcContrib* tcons, const void* apack,
                    const void* bpack, double* C, int* error, cudaStream_t st)
{
	if (ntiles <= 0) return;
	static std::once_flag attr_once;
	std::call_once(attr_once, [] {
		CTG_CUDA(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES));
	});
	k_gemm_tc<<<ntiles, TC_THREADS, TC_SMEM_BYTES, st>>>(tiles, outs, tcons, (const unsigned char*)apack,
	                                                       (const unsigned char*)bpack, C, error);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
