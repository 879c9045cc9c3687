/* ct_structs.h - chemtensor's public data structures, laid out byte-for-byte
 * as the reference declares them, so that a caller's struct mpo / struct mps
 * can be handed to the GB300 implementation unchanged.
 *
 * Reference declarations mirrored here:
 *   ct_long                    include/util/util.h:12
 *   qnumber                    include/tensor/qnumber.h:17
 *   enum numeric_type          include/numeric.h:15-22
 *   enum tensor_axis_direction include/tensor/qnumber.h (TENSOR_AXIS_IN = -1, TENSOR_AXIS_OUT = 1)
 *   struct dense_tensor        include/tensor/dense_tensor.h:17-23
 *   struct block_sparse_tensor include/tensor/block_sparse_tensor.h:17-27
 *   struct mps                 include/state/mps.h:14-20
 *   struct mpo                 include/operator/mpo.h:34-40
 *
 * Memory ownership follows the reference: every array hanging off these
 * structs is allocated with aligned_alloc(16, size rounded up to 16) and
 * released with free() (include/aligned_memory.h:17-54). A caller that
 * already includes the reference headers defines CT_USE_REFERENCE_HEADERS
 * and gets its own declarations instead.
 */
#ifndef CT_STRUCTS_H
#define CT_STRUCTS_H

#ifdef CT_USE_REFERENCE_HEADERS
#include "mps.h"
#include "mpo.h"
#else

#include <stdint.h>

typedef int64_t ct_long;
typedef int32_t qnumber;

enum numeric_type
{
	CT_SINGLE_REAL       = 0,
	CT_DOUBLE_REAL       = 1,
	CT_SINGLE_COMPLEX    = 2,
	CT_DOUBLE_COMPLEX    = 3,
	CT_NUM_NUMERIC_TYPES = 4,
};

enum tensor_axis_direction
{
	TENSOR_AXIS_IN  = -1,
	TENSOR_AXIS_OUT =  1,
};

/* row-major dense array */
struct dense_tensor
{
	void* data;
	ct_long* dim;
	enum numeric_type dtype;
	int ndim;
};

/* abelian block-sparse tensor: blocks[] is row-major over dim_blocks and holds
 * NULL for every quantum-number combination that does not sum to zero */
struct block_sparse_tensor
{
	struct dense_tensor** blocks;
	ct_long* dim_blocks;
	ct_long* dim_logical;
	enum tensor_axis_direction* axis_dir;
	qnumber** qnums_blocks;
	qnumber** qnums_logical;
	enum numeric_type dtype;
	int ndim;
};

/* site tensors D_i x d x D_{i+1}, axis directions (OUT, OUT, IN) */
struct mps
{
	struct block_sparse_tensor* a;
	qnumber* qsite;
	ct_long d;
	int nsites;
};

/* site tensors Dw_i x d x d x Dw_{i+1}, axis directions (OUT, OUT, IN, IN) */
struct mpo
{
	struct block_sparse_tensor* a;
	qnumber* qsite;
	ct_long d;
	int nsites;
};

#endif /* CT_USE_REFERENCE_HEADERS */

#endif /* CT_STRUCTS_H */
