// ctg_common.h - shared definitions for the GB300 two-site DMRG engine.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace ctg {

using i64 = int64_t;
using q32 = int32_t;

struct CudaError : std::runtime_error {
	using std::runtime_error::runtime_error;
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line);

#define CTG_CUDA(call)                                                              \
	do {                                                                            \
		cudaError_t ctg_e_ = (call);                                                \
		if (ctg_e_ != cudaSuccess) ::ctg::throw_cuda(ctg_e_, #call, __FILE__, __LINE__); \
	} while (0)

#define CTG_CHECK(cond, msg)                                                        \
	do {                                                                            \
		if (!(cond)) throw std::runtime_error(std::string("ctgpu: ") + (msg));       \
	} while (0)

// Axis range selector of block_sparse_tensor_dot (include/tensor/dense_tensor.h,
// TENSOR_AXIS_RANGE_LEADING = 0, TENSOR_AXIS_RANGE_TRAILING = 1).
enum AxRange { AX_LEADING = 0, AX_TRAILING = 1 };

// Arithmetic used for the bulk block GEMMs.
// The values of the first four are those of ctgpu_set_precision.
enum GemmPrecision {
	GEMM_FP64 = 0,        // plain IEEE double on the FP64 pipe
	GEMM_BF16X3 = 1,      // split-BF16, 3 products, FP32 accumulation on tcgen05
	GEMM_TF32 = 2,        // TF32, one product, FP32 accumulation on tcgen05
	GEMM_BF16X6 = 3,      // three-part split-BF16, 6 products, FP32 accumulation on tcgen05
	GEMM_Z64 = 16,        // complex128 entries (plan kind; the arithmetic is complex FP64)
};

// tensor-core precisions and their operand format (TcFormat in ctg_kernels.h)
inline bool is_tc_precision(int p) { return p == GEMM_BF16X3 || p == GEMM_TF32 || p == GEMM_BF16X6; }
inline int tc_format_of(int p) { return p == GEMM_BF16X6 ? 1 : p == GEMM_TF32 ? 2 : 0; }

}  // namespace ctg
