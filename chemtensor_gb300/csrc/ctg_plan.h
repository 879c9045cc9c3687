// ctg_plan.h - lowering of block-sparse operations into descriptor lists (host only).
//
// Every operation on the DMRG path is lowered from the block structures of its operands into
// plain arrays of descriptors that the device kernels walk (block GEMM tiles and contributions,
// block permutations, row maps). This file holds that lowering as pure host code: no CUDA
// call, no device memory. The engine (ctg_engine.cpp) caches the results and uploads them.
#pragma once

#include <memory>

#include "ctg_kernels.h"
#include "ctg_meta.h"

namespace ctg {

// block_sparse_tensor_dot (block_sparse_tensor.c:1826-2001) as GEMM work lists
struct DotLowering {
	std::shared_ptr<Meta> out;
	std::vector<GemmOut> outs;           // one per output block
	std::vector<GemmContrib> cons;       // operand block pairs, grouped by output block
	std::vector<GemmTile> tiles;         // every CTA's tile, all tile classes in one list
	std::vector<GemmSplit> splits;       // tiles whose sum is split over several CTAs
	i64 work_doubles = 0;                // partial-sum scratch of the split tiles
	// tensor-core path: packed operand records and their per-contribution indices
	std::vector<TcContrib> tcons;
	std::vector<TcPack> apacks, bpacks;
	double flops = 0;
	double flops_cls[NUM_TILE_CLASSES] = {};
	i64 a_entries = 0, b_entries = 0;
};
// out_perm (optional, r.ndim entries): write the result in the layout of its transpose by out_perm,
// which must arrange two runs of row axes and two runs of column axes (each run kept in order) with
// the last column run innermost. tc_bn: column width of the tensor-core tiles (64, 128 or 256).
DotLowering lower_dot(const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision, int num_sms,
                      const int* out_perm = nullptr, int tc_bn = 64);

// data movement: kind 0 block permutation (PermDesc), 1 row map (RowDesc + maps), 2 axis scaling
// (ScaleDesc + maps)
struct CopyLowering {
	std::shared_ptr<Meta> out;           // null for the axis scaling (structure unchanged)
	int kind = 0;
	std::vector<PermDesc> perm;
	std::vector<RowDesc> rows;
	std::vector<ScaleDesc> scale;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	i64 elements = 0;
};
CopyLowering lower_transpose(const Meta& t, const int* perm);
CopyLowering lower_flatten(const Meta& t, int ax, int newdir);
CopyLowering lower_split(const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq);
CopyLowering lower_slice(const Meta& t, int ax, const std::vector<i64>& ind);
CopyLowering lower_scale(const Meta& m, int axrange);

// host time of the lowering stages (diagnostics): 0 dot meta, 1 dot enumeration, 2 split-K,
// 3 dot tile lists, 4 transpose meta, 5 transpose loop, 6 flatten meta, 7 flatten loop,
// 8 split meta, 9 split loop, 10 slice, 11 other
extern thread_local double g_plan_stage[12];

}  // namespace ctg
