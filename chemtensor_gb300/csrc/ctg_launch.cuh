// ctg_launch.cuh - programmatic dependent launch for the kernels of a sweep.
//
// A kernel launched with the programmatic-stream-serialisation attribute may be scheduled while
// the kernel before it in the stream is still finishing; it waits at griddepcontrol.wait, before
// its first global-memory access, until that kernel has completed and its writes are visible. A
// kernel that calls pdl_trigger() lets the next one be scheduled once all of its own blocks have
// started. The launch setup of consecutive kernels then overlaps their execution instead of
// following it (a sweep runs a few thousand launches). CTGPU_PDL=0 launches without the attribute.
#pragma once

#include <cstdlib>

#include <cuda_runtime.h>

#include "ctg_common.h"

namespace ctg {

// first statement of every kernel launched by launch_pdl
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

inline bool pdl_enabled()
{
	static const bool v = [] {
		const char* e = getenv("CTGPU_PDL");
		return !e || atoi(e) != 0;
	}();
	return v;
}

// cfg: grid, block, shared memory, stream and up to three caller attributes (cluster size,
// cooperative); the serialisation attribute is added here
template <class... KArgs, class... Args>
void launch_pdl(cudaLaunchConfig_t cfg, void (*fn)(KArgs...), Args... args)
{
	cudaLaunchAttribute at[4];
	for (unsigned i = 0; i < cfg.numAttrs && i < 3; i++) at[i] = cfg.attrs[i];
	unsigned n = cfg.numAttrs < 3 ? cfg.numAttrs : 3;
	if (pdl_enabled())
	{
		at[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
		at[n].val.programmaticStreamSerializationAllowed = 1;
		n++;
	}
	cfg.attrs = at;
	cfg.numAttrs = n;
	CTG_CUDA(cudaLaunchKernelEx(&cfg, fn, args...));
}

inline cudaLaunchConfig_t launch_config(dim3 grid, dim3 block, size_t smem, cudaStream_t st)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = st;
	return cfg;
}

}  // namespace ctg
