// ctg_meta.h - host-side block structure of an abelian block-sparse tensor.
//
// The structure rule is the reference's (allocate_block_sparse_tensor,
// src/tensor/block_sparse_tensor.c:37-151): per axis the sorted unique
// quantum numbers and their multiplicities; a dense block exists for every
// combination whose signed quantum numbers sum to zero. Blocks are kept in
// row-major block-index order, which is also the order of their entries in
// the tensor's single contiguous device buffer (the reference's serialized
// entry order, block_sparse_tensor.c:3111-3176). Everything here is integer
// arithmetic, so structures agree with the reference exactly.
#pragma once

#include <unordered_map>

#include "ctg_common.h"

namespace ctg {

struct Meta {
	int ndim = 0;
	std::vector<i64> dim;                     // logical dimensions
	std::vector<int> dir;                     // axis directions (+1 out, -1 in)
	std::vector<std::vector<q32>> ql;         // logical quantum numbers per axis
	std::vector<std::vector<q32>> qb;         // sorted unique quantum numbers per axis
	std::vector<std::vector<i64>> bd;         // multiplicity of each unique quantum number
	std::vector<std::vector<i64>> pos;        // per logical index: position inside its block
	std::vector<std::vector<int>> blk;        // per logical index: its block index on the axis
	std::vector<i64> nb;                      // number of unique quantum numbers per axis

	// nonzero blocks, row-major block order
	int nblocks = 0;
	std::vector<i64> bidx;                    // nblocks x ndim block multi-indices
	std::vector<i64> bdim;                    // nblocks x ndim block dimensions
	std::vector<i64> boff;                    // entry offset of each block
	i64 nnz = 0;

	// block multi-index -> block number (or -1): blocks are enumerated in row-major order, so
	// their linear indices are increasing; a dense table is kept only where it is not much
	// larger than the block list
	std::vector<i64> lin;                     // linear index of every block, increasing
	std::vector<int> lut;                     // dense table over prod(nb), or empty

	const i64* index(int b) const { return &bidx[(size_t)b * ndim]; }
	const i64* dims(int b) const { return &bdim[(size_t)b * ndim]; }
	i64 block_size(int b) const;
	i64 linear(const i64* idx) const;
	int find(const i64* idx) const;
	int find_q(int ax, q32 q) const;          // block index of a quantum number on an axis, or -1
	bool same_structure(const Meta& o) const;
	// hash of (ndim, dim, dir, ql): equal structures hash equally (computed once, on first use)
	uint64_t structure_hash() const;

private:
	mutable uint64_t hash_ = 0;
	mutable bool hashed_ = false;
};

// Build the block structure from logical dims, directions and quantum numbers.
Meta make_meta(int ndim, const i64* dim, const int* dir, const std::vector<std::vector<q32>>& ql);

// Structure of the result of block_sparse_tensor_dot (src/tensor/block_sparse_tensor.c:1826-1900).
Meta dot_result_meta(const Meta& s, int axs, const Meta& t, int axt, int nmult);

// Structure of a transposed tensor (block_sparse_tensor.c:785-870); dst_of_src (optional) receives,
// for every block of t, the index of its permuted block in the result.
Meta transpose_meta(const Meta& t, const int* perm, std::vector<int>* dst_of_src = nullptr);

// Structure after flattening axes ax and ax+1 (block_sparse_tensor.c:950-1000).
Meta flatten_meta(const Meta& t, int ax, int newdir);

// Structure after splitting axis ax (block_sparse_tensor.c:1123-1170).
Meta split_meta(const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq);

// Structure after slicing axis ax with logical indices ind (block_sparse_tensor.c:1446-1475).
Meta slice_meta(const Meta& t, int ax, const std::vector<i64>& ind);

// Same structure with all axis directions reversed (block_sparse_tensor_reverse_axis_directions).
Meta reversed_meta(const Meta& t);

}  // namespace ctg
