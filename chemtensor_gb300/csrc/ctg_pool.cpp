// ctg_pool.cpp - host thread pool for the lowering (see ctg_pool.h).
#include "ctg_pool.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

namespace ctg {

namespace {

thread_local bool t_inside = false;               // set on pool threads and inside a job

void t_inside_worker()
{
	t_inside = true;
}

struct Pool {
	std::mutex mu;
	std::condition_variable wake;
	std::vector<std::thread> workers;
	// current job
	const std::function<void(int)>* fn = nullptr;
	int n = 0;
	std::atomic<int> next{0};
	std::atomic<int> active{0};            // workers still inside the current job
	std::atomic<long> generation{0};
	std::mutex err_mu;
	std::exception_ptr error;

	explicit Pool(int nworkers)
	{
		for (int i = 0; i < nworkers; i++) workers.emplace_back([this] { loop(); });
		for (auto& t : workers) t.detach();
	}

	void run_items()
	{
		for (;;)
		{
			const int i = next.fetch_add(1);
			if (i >= n) return;
			try
			{
				(*fn)(i);
			}
			catch (...)
			{
				std::lock_guard<std::mutex> g(err_mu);
				if (!error) error = std::current_exception();
			}
		}
	}

	void loop()
	{
		t_inside_worker();
		long seen = 0;
		for (;;)
		{
			// jobs of one bond step come tens of microseconds apart: poll for a while before
			// sleeping, so that a new job does not wait for a thread wake-up
			long g = generation.load(std::memory_order_acquire);
			for (int spin = 0; g == seen && spin < (1 << 16); spin++) g = generation.load(std::memory_order_acquire);
			if (g == seen)
			{
				std::unique_lock<std::mutex> lk(mu);
				wake.wait(lk, [&] { return generation.load(std::memory_order_acquire) != seen; });
				g = generation.load(std::memory_order_acquire);
			}
			seen = g;
			run_items();
			active.fetch_sub(1, std::memory_order_acq_rel);
		}
	}
};

Pool* pool_instance()
{
	// created once, never destroyed: its threads sleep until the process ends
	static Pool* p = [] {
		const int nt = host_threads();
		return nt > 1 ? new Pool(nt - 1) : nullptr;
	}();
	return p;
}

}  // namespace

int host_threads()
{
	static const int v = [] {
		if (const char* e = getenv("CTGPU_HOST_THREADS")) return std::max(1, atoi(e));
		const int hw = (int)std::thread::hardware_concurrency();
		return std::max(1, std::min(8, hw));
	}();
	return v;
}

void parallel_for(int n, const std::function<void(int)>& f)
{
	if (n <= 0) return;
	Pool* p = n > 1 && !t_inside ? pool_instance() : nullptr;
	if (!p)
	{
		for (int i = 0; i < n; i++) f(i);
		return;
	}
	static std::mutex one_job;                     // one job at a time (callers from several threads)
	std::lock_guard<std::mutex> job(one_job);
	p->fn = &f;
	p->n = n;
	p->error = nullptr;
	p->next.store(0, std::memory_order_relaxed);
	p->active.store((int)p->workers.size(), std::memory_order_relaxed);
	{
		std::lock_guard<std::mutex> g(p->mu);
		p->generation.fetch_add(1, std::memory_order_release);
	}
	p->wake.notify_all();
	t_inside = true;
	p->run_items();
	t_inside = false;
	while (p->active.load(std::memory_order_acquire) > 0)
	{
	}
	p->fn = nullptr;
	std::exception_ptr err;
	{
		std::lock_guard<std::mutex> g(p->err_mu);
		err = p->error;
	}
	if (err) std::rethrow_exception(err);
}

}  // namespace ctg
