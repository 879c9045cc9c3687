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
// into shared memory with one bulk copy.
//
// k_gemm_tc is persistent and warp-specialised: one CTA per SM walks the output tiles (128 x 64)
// with a stride of the grid size. Warp 0 (one lane) streams the A and B records of every k chunk
// into a ring of shared-memory stages (bulk copies completing on the stage's "full" mbarrier);
// warp 1 (one lane) issues the tcgen05.mma instructions of each chunk (3 products x 4 k-steps of
// 16, FP32 accumulation in tensor memory) and commits them to the stage's "empty" mbarrier, which
// hands the stage back to the copy warp; the accumulator of a tile alternates between two
// tensor-memory buffers, so that warps 2-5 (one per 32-lane quarter of tensor memory) drain tile i
// with tcgen05.ld while the MMAs of tile i + 1 run. The epilogue stages the FP32 tile in shared
// memory and writes FP64 rows, coalesced, into the output block's layout (plain, or that of a
// transposed result, see GemmOut). Every wait is bounded and also ends when another warp has
// recorded a failure: the CTA then records the error flag, lets its copies in flight land, frees
// its tensor memory and returns.
#include <algorithm>

#include <cuda_bf16.h>

#include <mutex>

#include "ctg_kernels.h"

namespace ctg {

namespace {

constexpr int TC_BM = 128;                 // tile rows (MMA M)
constexpr int TC_BN = 64;                  // tile columns (MMA N)
constexpr int TC_BK = 64;                  // K elements per shared-memory stage
constexpr int TC_THREADS = 192;            // copy warp, MMA warp, 4 epilogue warps
constexpr int TC_EPI_THREADS = 128;
constexpr int TC_ACC_BUFS = 2;
constexpr int TC_TMEM_COLS = TC_ACC_BUFS * TC_BN;   // FP32 accumulator columns, power of two >= 32
// canonical no-swizzle K-major layout: 8 x 16-byte core matrices; (row, k) ->
// (row / 8) * SBO + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2
constexpr int TC_LBO = 128;                // bytes between core matrices adjacent in K
constexpr int TC_SBO = (TC_BK / 8) * 128;  // bytes between core matrices adjacent in M / N
constexpr int A_TILE_BYTES = TC_BM * TC_BK * 2;
constexpr int B_TILE_BYTES = TC_BN * TC_BK * 2;
constexpr int STAGE_BYTES = 2 * A_TILE_BYTES + 2 * B_TILE_BYTES;   // one A record + one B record
constexpr int TC_STAGES = 4;
constexpr int TC_EPI_BYTES = TC_BM * (TC_BN + 1) * 4;               // padded FP32 staging tile
constexpr int TC_OFF_BYTES = 8 * (TC_BM + TC_BN);                     // row / column offsets of a tile
constexpr int TC_BAR_BYTES = 8 * (2 * TC_STAGES + 2 * TC_ACC_BUFS) + 16;
constexpr int TC_SMEM_BYTES = TC_STAGES * STAGE_BYTES + TC_EPI_BYTES + TC_OFF_BYTES + TC_BAR_BYTES;
static_assert(2 * A_TILE_BYTES == TC_A_REC_BYTES && 2 * B_TILE_BYTES == TC_B_REC_BYTES, "record layout");
static_assert(TC_BM == TC_A_ROWS && TC_BN == TC_B_ROWS && TC_BK == TC_K, "tile shape");
static_assert(TC_SMEM_BYTES <= 227 * 1024, "shared memory per CTA");
static_assert(TC_EPI_BYTES % 16 == 0, "barrier alignment");
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

// bounded wait for the given phase parity; returns false on timeout, or when *abort is set
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, const volatile int* abort = nullptr)
{
	for (long long it = 0; it < TC_WAIT_LIMIT; it++)
	{
		if (abort && *abort) return false;
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

// One CTA per record. A thread converts one core-matrix row: 8 consecutive k of one row (reads
// 8 FP64 values, strided by s_k) into 16 bytes of hi and 16 bytes of lo; consecutive threads take
// consecutive rows, so that 8 threads fill one 128-byte run of the record.
template <int R>
__global__ void __launch_bounds__(128) k_tc_pack(const TcPack* __restrict__ packs, const double* __restrict__ src,
                                                 unsigned char* __restrict__ dst)
{
	const TcPack p = packs[blockIdx.x];
	unsigned char* hi = dst + p.rec * (i64)(2 * R * TC_BK * 2);
	unsigned char* lo = hi + R * TC_BK * 2;
	constexpr int UNITS = R * (TC_BK / 8);
	for (int u = threadIdx.x; u < UNITS; u += blockDim.x)
	{
		const int i = u % R, kb = u / R;
		const int gi = p.row0 + i;
		const double* rowp = src + p.src + (i64)gi * p.s_row;
		uint32_t h[4], l[4];
#pragma unroll
		for (int t = 0; t < 8; t += 2)
		{
			const int gk = p.k0 + kb * 8 + t;
			// FP32 keeps 24 bits of x, more than the 16 that hi + lo carry
			float f0 = 0.0f, f1 = 0.0f;
			if (gi < p.rows)
			{
				if (gk < p.k) f0 = (float)rowp[(i64)gk * p.s_k];
				if (gk + 1 < p.k) f1 = (float)rowp[(i64)(gk + 1) * p.s_k];
			}
			const __nv_bfloat16 h0 = __float2bfloat16_rn(f0), h1 = __float2bfloat16_rn(f1);
			const __nv_bfloat16 l0 = __float2bfloat16_rn(f0 - __bfloat162float(h0));
			const __nv_bfloat16 l1 = __float2bfloat16_rn(f1 - __bfloat162float(h1));
			h[t / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
			l[t / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
		}
		const uint32_t so = canon_offset(i, kb * 8);
		*(uint4*)(hi + so) = make_uint4(h[0], h[1], h[2], h[3]);
		*(uint4*)(lo + so) = make_uint4(l[0], l[1], l[2], l[3]);
	}
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// named barrier of the four epilogue warps (id 1; id 0 is __syncthreads)
__device__ __forceinline__ void epi_sync()
{
	asm volatile("bar.sync 1, %0;" ::"r"(TC_EPI_THREADS) : "memory");
}

// the same barrier, returning the AND of v over the epilogue threads
__device__ __forceinline__ bool epi_sync_and(bool v)
{
	uint32_t r;
	asm volatile(
		"{\n\t.reg .pred p, q;\n\t"
		"setp.ne.u32 p, %1, 0;\n\t"
		"bar.red.and.pred q, 1, %2, p;\n\t"
		"selp.u32 %0, 1, 0, q;\n\t}"
		: "=r"(r)
		: "r"((uint32_t)v), "r"(TC_EPI_THREADS)
		: "memory");
	return r != 0;
}

__device__ __forceinline__ int tile_chunks(const GemmOut& o, const TcContrib* tcons)
{
	int n = 0;
	for (int c = o.c0; c < o.c0 + o.nc; c++) n += tcons[c].kt;
	return n;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
k_gemm_tc(int ntiles, const GemmTile* __restrict__ tiles, const GemmOut* __restrict__ outs,
          const TcContrib* __restrict__ tcons, const unsigned char* __restrict__ apack,
          const unsigned char* __restrict__ bpack, double* __restrict__ C, int* __restrict__ error)
{
	extern __shared__ __align__(1024) unsigned char smem[];
	float* stile = (float*)(smem + TC_STAGES * STAGE_BYTES);                  // epilogue staging
	i64* rowoff = (i64*)(smem + TC_STAGES * STAGE_BYTES + TC_EPI_BYTES);         // output offsets of
	i64* coloff = rowoff + TC_BM;                                               // the tile's rows, columns
	uint64_t* full = (uint64_t*)(coloff + TC_BN);                               // copies landed
	uint64_t* empty = full + TC_STAGES;                                        // MMAs of a stage done
	uint64_t* acc_full = empty + TC_STAGES;                                    // accumulator ready
	uint64_t* acc_empty = acc_full + TC_ACC_BUFS;                              // accumulator drained
	uint32_t* tmem_slot = (uint32_t*)(acc_empty + TC_ACC_BUFS);
	volatile int* abort = (volatile int*)(tmem_slot + 1);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

	if (warp == 1)
	{
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
		             "r"(TC_TMEM_COLS)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0)
	{
		for (int st = 0; st < TC_STAGES; st++)
		{
			mbar_init(smem_u32(full + st), 1);
			mbar_init(smem_u32(empty + st), 1);
		}
		for (int b = 0; b < TC_ACC_BUFS; b++)
		{
			mbar_init(smem_u32(acc_full + b), 1);
			mbar_init(smem_u32(acc_empty + b), TC_EPI_THREADS / 32);
		}
		*abort = 0;
	}
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;

	if (warp == 0)
	{
		// copy warp: k chunks of every tile of this CTA, in order, into the stage ring
		if (lane == 0)
		{
			long long g = 0;           // chunks issued by this CTA
			bool ok = true;
			for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x)
			{
				const GemmTile tile = tiles[ti];
				const GemmOut o = outs[tile.out];
				const int mt = tile.m0 / TC_BM, nt = tile.n0 / TC_BN;
				for (int c = o.c0; c < o.c0 + o.nc && ok; c++)
				{
					const TcContrib gc = tcons[c];
					for (int lk = 0; lk < gc.kt; lk++, g++)
					{
						const int st = (int)(g % TC_STAGES);
						if (g >= TC_STAGES &&
						    !mbar_wait(smem_u32(empty + st), (uint32_t)(((g / TC_STAGES) - 1) & 1), abort))
						{
							ok = false;
							break;
						}
						const unsigned char* arec = apack + (gc.a_rec + (i64)mt * gc.kt + lk) * TC_A_REC_BYTES;
						const unsigned char* brec = bpack + (gc.b_rec + (i64)nt * gc.kt + lk) * TC_B_REC_BYTES;
						const uint32_t sbase = smem_u32(smem + st * STAGE_BYTES);
						mbar_expect_tx(smem_u32(full + st), (uint32_t)STAGE_BYTES);
						bulk_copy(sbase, arec, (uint32_t)TC_A_REC_BYTES, smem_u32(full + st));
						bulk_copy(sbase + (uint32_t)TC_A_REC_BYTES, brec, (uint32_t)TC_B_REC_BYTES, smem_u32(full + st));
					}
				}
			}
			if (!ok)
			{
				*abort = 1;
				atomicExch(error, 1);
			}
			// the copies of the last chunk of every stage must land before shared memory is released
			for (long long u = g - TC_STAGES; u < g; u++)
				if (u >= 0) mbar_wait(smem_u32(full + (int)(u % TC_STAGES)), (uint32_t)((u / TC_STAGES) & 1));
		}
	}
	else if (warp == 1)
	{
		// MMA warp
		if (lane == 0)
		{
			const uint32_t idesc = make_idesc();
			long long g = 0;           // chunks consumed
			int acc = 0;               // tiles accumulated (tiles with at least one chunk)
			bool ok = true;
			for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x)
			{
				const GemmTile tile = tiles[ti];
				const GemmOut o = outs[tile.out];
				const int nch = tile_chunks(o, tcons);
				if (nch == 0) continue;
				const int b = acc % TC_ACC_BUFS;
				if (acc >= TC_ACC_BUFS &&
				    !mbar_wait(smem_u32(acc_empty + b), (uint32_t)(((acc / TC_ACC_BUFS) - 1) & 1), abort))
				{
					ok = false;
					break;
				}
				tc_fence_after();
				const uint32_t dacc = tmem + (uint32_t)(b * TC_BN);
				for (int u = 0; u < nch; u++, g++)
				{
					const int su = (int)(g % TC_STAGES);
					if (!mbar_wait(smem_u32(full + su), (uint32_t)((g / TC_STAGES) & 1), abort))
					{
						ok = false;
						break;
					}
					tc_fence_after();
					const uint32_t a_hi = smem_u32(smem + su * STAGE_BYTES);
					const uint32_t a_lo = a_hi + A_TILE_BYTES;
					const uint32_t b_hi = a_lo + A_TILE_BYTES;
					const uint32_t b_lo = b_hi + B_TILE_BYTES;
					for (int k = 0; k < TC_BK / 16; k++)
					{
						const uint32_t koff = (uint32_t)k * 2 * TC_LBO;
						const uint64_t dah = make_desc(a_hi + koff), dal = make_desc(a_lo + koff);
						const uint64_t dbh = make_desc(b_hi + koff), dbl = make_desc(b_lo + koff);
						mma_bf16(dacc, dah, dbh, idesc, u > 0 || k > 0);
						mma_bf16(dacc, dah, dbl, idesc, true);
						mma_bf16(dacc, dal, dbh, idesc, true);
					}
					mma_commit(smem_u32(empty + su));
				}
				if (!ok) break;
				mma_commit(smem_u32(acc_full + b));
				acc++;
			}
			if (!ok)
			{
				*abort = 1;
				atomicExch(error, 1);
			}
			// no MMA may still run when tensor memory is freed: the commit after the last chunk
			// consumed tracks every MMA issued before it
			if (g > 0)
				mbar_wait(smem_u32(empty + (int)((g - 1) % TC_STAGES)), (uint32_t)(((g - 1) / TC_STAGES) & 1));
		}
	}
	else
	{
		// epilogue warps: tensor-memory quarter q holds accumulator rows 32 q .. 32 q + 31
		const int q = warp & 3;
		const int et = tid - 64;   // 0 .. 127
		int acc = 0;
		for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
		{
			const GemmTile tile = tiles[ti];
			const GemmOut o = outs[tile.out];
			const int nch = tile_chunks(o, tcons);
			// where the tile's rows and columns go (gemm_out_index split into a row and a column part),
			// while the tile's MMAs may still run
			static_assert(TC_EPI_THREADS == TC_BM && TC_BN <= TC_EPI_THREADS, "one row offset per thread");
			{
				const int i = tile.m0 + et;
				rowoff[et] = i < o.m ? o.c_off + (i64)(i / o.r1) * o.sr0 + (i64)(i % o.r1) * o.sr1 : 0;
				const int j = tile.n0 + et;
				if (et < TC_BN) coloff[et] = j < o.n ? (i64)(j / o.c1) * o.sc0 + (j % o.c1) : -1;
			}
			bool have = false;
			if (nch > 0)
			{
				const int b = acc % TC_ACC_BUFS;
				// warp-uniform outcome: tcgen05.ld is executed by all lanes of a warp or by none
				have = __all_sync(0xffffffffu, mbar_wait(smem_u32(acc_full + b), (uint32_t)((acc / TC_ACC_BUFS) & 1), abort));
				if (have)
				{
					tc_fence_after();
					for (int cc = 0; cc < TC_BN; cc += 16)
					{
						uint32_t v[16];
						const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * TC_BN + cc);
						asm volatile(
							"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
							: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
							  "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
							  "=r"(v[14]), "=r"(v[15])
							: "r"(taddr));
						asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
						float* srow = stile + (q * 32 + lane) * (TC_BN + 1) + cc;
						for (int t = 0; t < 16; t++) srow[t] = __uint_as_float(v[t]);
					}
					tc_fence_before();
					__syncwarp();
					if (lane == 0) mbar_arrive(smem_u32(acc_empty + b));
				}
				acc++;
			}
			// CTA-uniform outcome among the epilogue warps (a failed wait ends all of them together)
			const bool all_have = epi_sync_and(have || nch == 0);
			have = have && all_have;
			const int rows = min(TC_BM, o.m - tile.m0);
			const int cl = et % TC_BN;
			const i64 co = coloff[cl];
			if (co >= 0)
				for (int r = et / TC_BN; r < rows; r += TC_EPI_THREADS / TC_BN)
					C[rowoff[r] + co] = have ? (double)stile[r * (TC_BN + 1) + cl] : 0.0;
			epi_sync();
			if (!all_have)
			{
				*abort = 1;
				atomicExch(error, 1);
				break;
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1)
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
	static int num_sms = 0;
	std::call_once(attr_once, [] {
		CTG_CUDA(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES));
		int dev = 0;
		CTG_CUDA(cudaGetDevice(&dev));
		CTG_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
	});
	// persistent: one CTA per SM (the shared-memory ring admits one), each walking every gridDim-th tile
	const int grid = std::min(ntiles, std::max(num_sms, 1));
	k_gemm_tc<<<grid, TC_THREADS, TC_SMEM_BYTES, st>>>(ntiles, tiles, outs, tcons, (const unsigned char*)apack,
	                                                     (const unsigned char*)bpack, C, error);
	CTG_CUDA(cudaGetLastError());
}

}  // namespace ctg
