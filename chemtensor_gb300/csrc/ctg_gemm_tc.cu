// ctg_gemm_tc.cu - grouped block GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation.
//
// Same work lists as the FP64 grouped GEMM (GemmOut / GemmTile) with one TcContrib per
// contribution: every output block C = sum_j op(A_j) op(B_j). Three operand formats (TcFormat):
//   BF16X3  x = hi + lo, hi = bf16(x), lo = bf16(x - hi); products hi.hi + hi.lo + lo.hi
//           (about 2^-16 relative error per product: the representation keeps 16 bits of x)
//   BF16X6  x = hi + mid + lo, three BF16 parts of the FP32 value of x; products hh, hm, mh, hl,
//           mm, lh (every term down to 2^-16 relative): about 2^-23, FP32-like accuracy
//   TF32    x rounded to TF32 (kind::tf32, one product): about 2^-11
// Output in FP64, or FP32 where the result only feeds another reduced-precision product.
//
// k_tc_pack writes each operand block as records: per 64-byte k chunk (32 BF16 or 16 TF32
// elements) and per part, 128 (A) or 64 (B) rows in the canonical no-swizzle K-major core-matrix
// layout of the tcgen05 shared-memory descriptors, so that the GEMM moves a chunk into shared
// memory with a few bulk copies. Short contracted extents (the quantum-number sectors of a bond)
// waste at most 63 bytes of k per contribution.
//
// k_gemm_tc is persistent and warp-specialised: one CTA per SM walks the output tiles (128 x BN,
// BN = 64, 128 or 256, chosen per product by the tile autotuner) with a stride of the grid size.
// Warp 0 (one lane) streams the A and B records of every k chunk into a ring of shared-memory
// stages (bulk copies completing on the stage's "full" mbarrier); warp 1 (one lane) issues the
// tcgen05.mma instructions of each chunk into FP32 accumulators in tensor memory and commits them
// to the stage's "empty" mbarrier, which hands the stage back to the copy warp; the accumulator of
// a tile alternates between two tensor-memory buffers, so that warps 2-9 (two per 32-lane quarter
// of tensor memory, each half of the columns) drain tile i with tcgen05.ld while the MMAs of tile
// i + 1 run. Each epilogue warp stages 32 rows x 32 columns at a time in its own shared memory and
// writes them row by row,
// coalesced, into the output block's layout (plain, or that of a transposed result, see GemmOut);
// warps whose rows lie outside the block skip the drain. Every wait is bounded and also ends when
// another warp has recorded a failure: the CTA then records the error flag, lets its copies in
// flight land, frees its tensor memory and returns.
#include <algorithm>

#include <cuda_bf16.h>

#include <mutex>

#include "ctg_kernels.h"

namespace ctg {

namespace {

constexpr int TC_BM = 128;                 // tile rows (MMA M)
constexpr int TC_EPI_WARPS = 8;            // two per 32-lane quarter of tensor memory, each half the columns
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;   // copy warp, MMA warp, epilogue warps
constexpr int TC_ACC_BUFS = 2;
// canonical no-swizzle K-major layout of one part: 8-row x 16-byte core matrices;
// (row, byte b of the 64-byte k chunk) -> (row / 8) * SBO + (b / 16) * LBO + (row % 8) * 16 + b % 16
constexpr int TC_LBO = 128;                // bytes between core matrices adjacent in K
constexpr int TC_SBO = (TC_KB / 16) * 128; // bytes between core matrices adjacent in M / N
constexpr int A_PART_BYTES = TC_A_ROWS * TC_KB;      // 8 KiB
constexpr int B_PART_BYTES = TC_B_ROWS * TC_KB;      // 4 KiB
constexpr int TC_EPI_LD = 33;                        // padded FP32 staging row (32 columns)
constexpr int TC_EPI_BYTES = TC_EPI_WARPS * 32 * TC_EPI_LD * 4; // one 32 x 32 staging tile per epilogue warp
constexpr int TC_SMEM_MAX = 227 * 1024;
constexpr int TC_BAR_BYTES = 8 * (2 * 8 + 2 * TC_ACC_BUFS) + 16;
static_assert(TC_A_ROWS == TC_BM, "tile shape");
constexpr long long TC_WAIT_LIMIT_DEFAULT = 1ll << 26;   // spins before a wait is declared failed

template <int FMT>
struct Fmt;
template <>
struct Fmt<TC_BF16X3> {
	static constexpr int PARTS = 2, NPROD = 3, ELEM = 2;
	__device__ static void prod(int i, int& pa, int& pb)
	{
		pa = i == 2 ? 1 : 0;                   // hi.hi, hi.lo, lo.hi
		pb = i == 1 ? 1 : 0;
	}
};
template <>
struct Fmt<TC_BF16X6> {
	static constexpr int PARTS = 3, NPROD = 6, ELEM = 2;
	__device__ static void prod(int i, int& pa, int& pb)
	{
		// hh, hm, mh, hl, mm, lh: every pair with pa + pb <= 2
		const int a[6] = {0, 0, 1, 0, 1, 2}, b[6] = {0, 1, 0, 2, 1, 0};
		pa = a[i];
		pb = b[i];
	}
};
template <>
struct Fmt<TC_TF32> {
	static constexpr int PARTS = 1, NPROD = 1, ELEM = 4;
	__device__ static void prod(int, int& pa, int& pb) { pa = pb = 0; }
};

template <int FMT, int BN>
struct Cfg {
	static constexpr int PARTS = Fmt<FMT>::PARTS;
	static constexpr int A_BYTES = PARTS * A_PART_BYTES;            // one A record
	static constexpr int B_BYTES = PARTS * BN * TC_KB;              // BN / 64 B records
	static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
	static constexpr int FREE = TC_SMEM_MAX - TC_EPI_BYTES - TC_BAR_BYTES - 1024;
	static constexpr int STAGES = FREE / STAGE_BYTES > 8 ? 8 : FREE / STAGE_BYTES;
	static constexpr int SMEM = STAGES * STAGE_BYTES + TC_EPI_BYTES + TC_BAR_BYTES;
	static constexpr int TMEM_COLS = TC_ACC_BUFS * BN;              // FP32 accumulator columns
	static_assert(STAGES >= 2, "shared-memory ring");
	static_assert(SMEM <= TC_SMEM_MAX, "shared memory per CTA");
	static_assert(TMEM_COLS <= 512, "tensor memory");
};

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
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

// instruction descriptor: FP32 D, K-major A and B, M = 128, N = BN; A / B format BF16 (1, kind::f16)
// or TF32 (2, kind::tf32)
template <int FMT, int BN>
__device__ __forceinline__ uint32_t make_idesc()
{
	const uint32_t ab = FMT == TC_TF32 ? 2u : 1u;
	uint32_t d = 0;
	d |= 1u << 4;                          // D format FP32
	d |= ab << 7;                          // A format
	d |= ab << 10;                         // B format
	d |= (uint32_t)(BN >> 3) << 17;        // N / 8
	d |= (uint32_t)(TC_BM >> 4) << 24;     // M / 16
	return d;
}

template <int FMT>
__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
	if constexpr (FMT == TC_TF32)
		asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"setp.ne.b32 p, %4, 0;\n\t"
			"tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
			:
			: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate));
	else
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

// bounded wait for the given phase parity; returns false after `limit` polls, or when *abort is set
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit, const volatile int* abort = nullptr)
{
	for (long long it = 0; it < limit; it++)
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

__device__ __forceinline__ void mbar_arrive(uint32_t mbar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// global -> shared bulk copy completing on an mbarrier (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
	             "l"(src), "r"(bytes), "r"(mbar)
	             : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ uint32_t canon_offset(int row, int kbyte)
{
	return (uint32_t)((row >> 3) * TC_SBO + (kbyte >> 4) * TC_LBO + (row & 7) * 16 + (kbyte & 15));
}

__device__ __forceinline__ uint32_t bf16_bits(float f)
{
	return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(f));
}

__device__ __forceinline__ float bf16_val(uint32_t b)
{
	return __uint_as_float(b << 16);
}

__device__ __forceinline__ uint32_t tf32_bits(float f)
{
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
	return r;
}

// One CTA per record. A thread converts one 16-byte core-matrix row segment of every part: 16 / ELEM
// consecutive k of one row (read from the FP64 or FP32 operand, strided by s_k); consecutive
// threads take consecutive rows, so that 8 threads fill one 128-byte run of a part.
template <int R, int FMT, class SRC>
__global__ void __launch_bounds__(128) k_tc_pack(const TcPack* __restrict__ packs, const SRC* __restrict__ src,
                                                 unsigned char* __restrict__ dst)
{
	using F = Fmt<FMT>;
	constexpr int PART = R * TC_KB;
	constexpr int PER = 16 / F::ELEM;               // elements per 16-byte segment
	constexpr int UNITS = R * (TC_KB / 16);
	const TcPack p = packs[blockIdx.x];
	unsigned char* rec = dst + p.rec * (i64)(F::PARTS * PART);
	for (int u = threadIdx.x; u < UNITS; u += blockDim.x)
	{
		const int i = u % R, seg = u / R;
		const int gi = p.row0 + i;
		const SRC* rowp = src + p.src + (i64)gi * p.s_row;
		float f[PER];
#pragma unroll
		for (int t = 0; t < PER; t++)
		{
			const int gk = p.k0 + seg * PER + t;
			// FP32 keeps 24 bits of x: as many as the three BF16 parts carry
			f[t] = (gi < p.rows && gk < p.k) ? (float)rowp[(i64)gk * p.s_k] : 0.0f;
		}
		const uint32_t so = canon_offset(i, seg * 16);
		if constexpr (FMT == TC_TF32)
		{
			*(uint4*)(rec + so) = make_uint4(tf32_bits(f[0]), tf32_bits(f[1]), tf32_bits(f[2]), tf32_bits(f[3]));
		}
		else
		{
			uint32_t w[F::PARTS][4];
#pragma unroll
			for (int t = 0; t < PER; t += 2)
			{
				float r0 = f[t], r1 = f[t + 1];
#pragma unroll
				for (int q = 0; q < F::PARTS; q++)
				{
					// each part is the BF16 rounding of what the parts before it left over (exact in FP32)
					const uint32_t b0 = bf16_bits(r0), b1 = bf16_bits(r1);
					w[q][t / 2] = b0 | (b1 << 16);
					r0 -= bf16_val(b0);
					r1 -= bf16_val(b1);
				}
			}
#pragma unroll
			for (int q = 0; q < F::PARTS; q++) *(uint4*)(rec + q * PART + so) = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
		}
	}
}

__device__ __forceinline__ int tile_chunks(const GemmOut& o, const TcContrib* tcons)
{
	int n = 0;
	for (int c = o.c0; c < o.c0 + o.nc; c++) n += tcons[c].kt;
	return n;
}

template <int FMT, int BN, class OUT>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_gemm_tc(int ntiles, const GemmTile* __restrict__ tiles, const GemmOut* __restrict__ outs,
          const TcContrib* __restrict__ tcons, const unsigned char* __restrict__ apack,
          const unsigned char* __restrict__ bpack, OUT* __restrict__ C, int* __restrict__ error, long long wait_limit)
{
	using F = Fmt<FMT>;
	using G = Cfg<FMT, BN>;
	constexpr int NST = G::STAGES;
	constexpr int SUB = BN / TC_B_ROWS;             // B records per tile column range
	extern __shared__ __align__(1024) unsigned char smem[];
	float* stile = (float*)(smem + NST * G::STAGE_BYTES);                       // epilogue staging
	uint64_t* full = (uint64_t*)(smem + NST * G::STAGE_BYTES + TC_EPI_BYTES);   // copies landed
	uint64_t* empty = full + 8;                                                 // MMAs of a stage done
	uint64_t* acc_full = empty + 8;                                            // accumulator ready
	uint64_t* acc_empty = acc_full + TC_ACC_BUFS;                              // accumulator drained
	uint32_t* tmem_slot = (uint32_t*)(acc_empty + TC_ACC_BUFS);
	volatile int* abort = (volatile int*)(tmem_slot + 1);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

	if (warp == 1)
	{
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
		             "r"(G::TMEM_COLS)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0)
	{
		for (int st = 0; st < NST; st++)
		{
			mbar_init(smem_u32(full + st), 1);
			mbar_init(smem_u32(empty + st), 1);
		}
		for (int b = 0; b < TC_ACC_BUFS; b++)
		{
			mbar_init(smem_u32(acc_full + b), 1);
			mbar_init(smem_u32(acc_empty + b), TC_EPI_WARPS);      // one arrival per epilogue warp
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
				const int mt = tile.m0 / TC_BM, nt = tile.n0 / BN;
				for (int c = o.c0; c < o.c0 + o.nc && ok; c++)
				{
					const TcContrib gc = tcons[c];
					for (int lk = 0; lk < gc.kt; lk++, g++)
					{
						const int st = (int)(g % NST);
						if (g >= NST && !mbar_wait(smem_u32(empty + st), (uint32_t)(((g / NST) - 1) & 1), wait_limit, abort))
						{
							ok = false;
							break;
						}
						const uint32_t sa = smem_u32(smem + st * G::STAGE_BYTES);
						const uint32_t sb = sa + (uint32_t)G::A_BYTES;
						const uint32_t bar = smem_u32(full + st);
						mbar_expect_tx(bar, (uint32_t)G::STAGE_BYTES);
						// an A record holds its parts back to back, as the stage does
						bulk_copy(sa, apack + (gc.a_rec + (i64)mt * gc.kt + lk) * G::A_BYTES, (uint32_t)G::A_BYTES, bar);
						// B: the SUB consecutive 64-row records of the tile's columns, part by part, so that each
						// part holds BN rows in one canonical layout
#pragma unroll
						for (int s = 0; s < SUB; s++)
						{
							const unsigned char* brec =
							    bpack + (gc.b_rec + (i64)(nt * SUB + s) * gc.kt + lk) * (i64)(F::PARTS * B_PART_BYTES);
#pragma unroll
							for (int q = 0; q < F::PARTS; q++)
								bulk_copy(sb + (uint32_t)(q * BN * TC_KB + s * B_PART_BYTES), brec + q * B_PART_BYTES,
								          (uint32_t)B_PART_BYTES, bar);
						}
					}
				}
			}
			if (!ok)
			{
				*abort = 1;
				atomicExch(error, 1);
			}
			// the copies of the last chunk of every stage must land before shared memory is released
			// (always with the default limit: a lowered limit only shortens the pipeline's waits)
			for (long long u = g - NST; u < g; u++)
				if (u >= 0) mbar_wait(smem_u32(full + (int)(u % NST)), (uint32_t)((u / NST) & 1), TC_WAIT_LIMIT_DEFAULT);
		}
	}
	else if (warp == 1)
	{
		// MMA warp
		if (lane == 0)
		{
			const uint32_t idesc = make_idesc<FMT, BN>();
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
				    !mbar_wait(smem_u32(acc_empty + b), (uint32_t)(((acc / TC_ACC_BUFS) - 1) & 1), wait_limit, abort))
				{
					ok = false;
					break;
				}
				tc_fence_after();
				const uint32_t dacc = tmem + (uint32_t)(b * BN);
				for (int u = 0; u < nch; u++, g++)
				{
					const int su = (int)(g % NST);
					if (!mbar_wait(smem_u32(full + su), (uint32_t)((g / NST) & 1), wait_limit, abort))
					{
						ok = false;
						break;
					}
					tc_fence_after();
					const uint32_t sa = smem_u32(smem + su * G::STAGE_BYTES);
					const uint32_t sb = sa + (uint32_t)G::A_BYTES;
#pragma unroll
					for (int k = 0; k < TC_KB / 32; k++)      // 32 bytes of k per MMA (16 BF16, 8 TF32)
					{
						const uint32_t koff = (uint32_t)k * 2 * TC_LBO;
#pragma unroll
						for (int pr = 0; pr < F::NPROD; pr++)
						{
							int pa, pb;
							F::prod(pr, pa, pb);
							const uint64_t da = make_desc(sa + (uint32_t)(pa * A_PART_BYTES) + koff);
							const uint64_t db = make_desc(sb + (uint32_t)(pb * BN * TC_KB) + koff);
							mma<FMT>(dacc, da, db, idesc, u > 0 || k > 0 || pr > 0);
						}
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
				mbar_wait(smem_u32(empty + (int)((g - 1) % NST)), (uint32_t)(((g - 1) / NST) & 1), TC_WAIT_LIMIT_DEFAULT);
		}
	}
	else
	{
		// epilogue warps: tensor-memory quarter q holds accumulator rows 32 q .. 32 q + 31; lane l of
		// the warp holds row 32 q + l (a warp may only read the lane quarter warp % 4). Two warps per
		// quarter, each draining, staging and writing half of the tile's columns of its rows.
		const int q = warp & 3;
		const int half = (warp - 2) / 4;
		constexpr int HALF = BN / 2;
		float* sw = stile + (warp - 2) * 32 * TC_EPI_LD;
		int acc = 0;
		for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
		{
			const GemmTile tile = tiles[ti];
			const GemmOut o = outs[tile.out];
			const int nch = tile_chunks(o, tcons);
			const int i = tile.m0 + q * 32 + lane;
			const i64 ro = i < o.m ? o.c_off + (i64)(i / o.r1) * o.sr0 + (i64)(i % o.r1) * o.sr1 : -1;
			const int rows = min(32, o.m - tile.m0 - q * 32);      // rows of this warp inside the block
			const int cols = min(BN, o.n - tile.n0);
			const int c_lo = half * HALF, c_hi = min(cols, c_lo + HALF);
			bool ok = true;
			if (nch > 0)
			{
				const int b = acc % TC_ACC_BUFS;
				// warp-uniform outcome: tcgen05.ld is executed by all lanes of a warp or by none
				ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(acc_full + b), (uint32_t)((acc / TC_ACC_BUFS) & 1),
				                                       wait_limit, abort));
				if (ok)
				{
					tc_fence_after();
					for (int cc = c_lo; cc < c_hi && rows > 0; cc += 32)
					{
						uint32_t v[32];
						const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + cc);
						asm volatile(
							"tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
							"%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
							: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
							  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
							  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
							  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
							  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
							: "r"(taddr));
						asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
						for (int t = 0; t < 32; t++) sw[lane * TC_EPI_LD + t] = __uint_as_float(v[t]);
						__syncwarp();
						// row by row: lane = column, coalesced within the output block's rows
						const int j = tile.n0 + cc + lane;
						const i64 co = (cc + lane < c_hi) ? (i64)(j / o.c1) * o.sc0 + (j % o.c1) : -1;
						for (int r = 0; r < rows; r++)
						{
							const i64 rr = __shfl_sync(0xffffffffu, ro, r);
							if (co >= 0) C[rr + co] = (OUT)sw[r * TC_EPI_LD + lane];
						}
						__syncwarp();
					}
					tc_fence_before();
					__syncwarp();
					if (lane == 0) mbar_arrive(smem_u32(acc_empty + b));
				}
				acc++;
			}
			else
			{
				// no contribution: the tile is zero
				for (int cc = c_lo; cc < c_hi && rows > 0; cc += 32)
				{
					const int j = tile.n0 + cc + lane;
					const i64 co = (cc + lane < c_hi) ? (i64)(j / o.c1) * o.sc0 + (j % o.c1) : -1;
					for (int r = 0; r < rows; r++)
					{
						const i64 rr = __shfl_sync(0xffffffffu, ro, r);
						if (co >= 0) C[rr + co] = (OUT)0;
					}
				}
			}
			if (!ok)
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
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G::TMEM_COLS) : "memory");
	}
}

int g_num_sms = 0;
long long g_wait_limit = TC_WAIT_LIMIT_DEFAULT;

template <int FMT, int BN, class OUT>
void launch_gemm_t(int ntiles, const GemmTile* tiles, const GemmOut* outs, const TcContrib* tcons, const void* apack,
                   const void* bpack, OUT* C, int* error, cudaStream_t st)
{
	using G = Cfg<FMT, BN>;
	static std::once_flag attr_once;
	std::call_once(attr_once, [] {
		CTG_CUDA(cudaFuncSetAttribute(k_gemm_tc<FMT, BN, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM));
	});
	// persistent: one CTA per SM (the shared-memory ring admits one), each walking every gridDim-th tile
	const int grid = std::min(ntiles, std::max(g_num_sms, 1));
	k_gemm_tc<FMT, BN, OUT><<<grid, TC_THREADS, G::SMEM, st>>>(ntiles, tiles, outs, tcons, (const unsigned char*)apack,
	                                                          (const unsigned char*)bpack, C, error, g_wait_limit);
	CTG_CUDA(cudaGetLastError());
}

template <int FMT, class OUT>
void launch_gemm_f(int bn, int ntiles, const GemmTile* tiles, const GemmOut* outs, const TcContrib* tcons, const void* apack,
                   const void* bpack, OUT* C, int* error, cudaStream_t st)
{
	switch (bn)
	{
	case 64: launch_gemm_t<FMT, 64, OUT>(ntiles, tiles, outs, tcons, apack, bpack, C, error, st); break;
	case 128: launch_gemm_t<FMT, 128, OUT>(ntiles, tiles, outs, tcons, apack, bpack, C, error, st); break;
	case 256: launch_gemm_t<FMT, 256, OUT>(ntiles, tiles, outs, tcons, apack, bpack, C, error, st); break;
	default: CTG_CHECK(false, "tensor-core GEMM: unsupported tile width");
	}
}

template <int FMT, class SRC>
void launch_pack_f(int nrec, const TcPack* packs, int a_side, const SRC* src, void* dst, cudaStream_t st)
{
	if (a_side) k_tc_pack<TC_A_ROWS, FMT, SRC><<<nrec, 128, 0, st>>>(packs, src, (unsigned char*)dst);
	else k_tc_pack<TC_B_ROWS, FMT, SRC><<<nrec, 128, 0, st>>>(packs, src, (unsigned char*)dst);
}

}  // namespace

int tc_tile_rows() { return TC_BM; }

int tc_parts(int fmt)
{
	return fmt == TC_BF16X6 ? 3 : fmt == TC_TF32 ? 1 : 2;
}

int tc_k_chunk(int fmt)
{
	return fmt == TC_TF32 ? TC_KB / 4 : TC_KB / 2;
}

i64 tc_a_rec_bytes(int fmt) { return (i64)tc_parts(fmt) * A_PART_BYTES; }
i64 tc_b_rec_bytes(int fmt) { return (i64)tc_parts(fmt) * B_PART_BYTES; }

void set_tc_wait_limit(long long polls)
{
	g_wait_limit = polls > 0 ? polls : TC_WAIT_LIMIT_DEFAULT;
}

void launch_tc_pack(int fmt, int nrec, const TcPack* packs, int a_side, const void* src, bool src_f32, void* dst,
                    cudaStream_t st)
{
	if (nrec <= 0) return;
	if (src_f32)
	{
		const float* s = (const float*)src;
		if (fmt == TC_BF16X3) launch_pack_f<TC_BF16X3>(nrec, packs, a_side, s, dst, st);
		else if (fmt == TC_BF16X6) launch_pack_f<TC_BF16X6>(nrec, packs, a_side, s, dst, st);
		else launch_pack_f<TC_TF32>(nrec, packs, a_side, s, dst, st);
	}
	else
	{
		const double* s = (const double*)src;
		if (fmt == TC_BF16X3) launch_pack_f<TC_BF16X3>(nrec, packs, a_side, s, dst, st);
		else if (fmt == TC_BF16X6) launch_pack_f<TC_BF16X6>(nrec, packs, a_side, s, dst, st);
		else launch_pack_f<TC_TF32>(nrec, packs, a_side, s, dst, st);
	}
	CTG_CUDA(cudaGetLastError());
}

void launch_gemm_tc(int fmt, int bn, int ntiles, const GemmTile* tiles, const GemmOut* outs, const TcContrib* tcons,
                    const void* apack, const void* bpack, void* C, bool out_f32, int* error, cudaStream_t st)
{
	if (ntiles <= 0) return;
	static std::once_flag sms_once;
	std::call_once(sms_once, [] {
		int dev = 0;
		CTG_CUDA(cudaGetDevice(&dev));
		CTG_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
	});
	if (out_f32)
	{
		float* c = (float*)C;
		if (fmt == TC_BF16X3) launch_gemm_f<TC_BF16X3>(bn, ntiles, tiles, outs, tcons, apack, bpack, c, error, st);
		else if (fmt == TC_BF16X6) launch_gemm_f<TC_BF16X6>(bn, ntiles, tiles, outs, tcons, apack, bpack, c, error, st);
		else launch_gemm_f<TC_TF32>(bn, ntiles, tiles, outs, tcons, apack, bpack, c, error, st);
	}
	else
	{
		double* c = (double*)C;
		if (fmt == TC_BF16X3) launch_gemm_f<TC_BF16X3>(bn, ntiles, tiles, outs, tcons, apack, bpack, c, error, st);
		else if (fmt == TC_BF16X6) launch_gemm_f<TC_BF16X6>(bn, ntiles, tiles, outs, tcons, apack, bpack, c, error, st);
		else launch_gemm_f<TC_TF32>(bn, ntiles, tiles, outs, tcons, apack, bpack, c, error, st);
	}
}

}  // namespace ctg
