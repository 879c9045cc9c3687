// ctg_pool.h - a small pool of host threads for lowering large block-sparse operations.
//
// The lowering of one operation (ctg_plan.cpp) loops over thousands of blocks; for the largest
// operations of a two-site DMRG bond step that loop is split into ranges that run on these
// threads while the calling thread takes its share. The pool is created on first use and lives
// for the rest of the process (its threads sleep between jobs).
#pragma once

#include <functional>

namespace ctg {

// Threads available to parallel_for, including the caller (CTGPU_HOST_THREADS overrides the
// default of min(8, hardware threads); 1 keeps everything on the calling thread).
int host_threads();

// Runs f(i) for every i in [0, n), spread over the pool and the calling thread, and returns when
// all calls are done. An exception thrown by a call is rethrown here (the first one). Calls from
// inside f run serially on the calling thread.
void parallel_for(int n, const std::function<void(int)>& f);

}  // namespace ctg
