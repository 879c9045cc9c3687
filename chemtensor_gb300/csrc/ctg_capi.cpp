// ctg_capi.cpp - extern "C" boundary (include/ctgpu.h).
#include <algorithm>
#include <cstring>
#include <exception>
#include <cmath>
#include <string>

#include <csignal>
#include <execinfo.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include "ctgpu.h"
#include "ctg_dmrg.h"

namespace {

// opt-in diagnostics: with CTGPU_SEGV_TRACE set, a segmentation fault in the calling process prints
// the native call stack (symbols of the exported functions) to stderr before the default action
void segv_trace(int sig)
{
	void* frames[64];
	const int n = backtrace(frames, 64);
	static const char head[] = "ctgpu: native stack at the fault:\n";
	if (write(2, head, sizeof head - 1) < 0) {}
	backtrace_symbols_fd(frames, n, 2);
	signal(sig, SIG_DFL);
	raise(sig);
}
const bool g_segv_trace_installed = [] {
	if (std::getenv("CTGPU_SEGV_TRACE")) signal(SIGSEGV, segv_trace);
	return true;
}();

thread_local std::string g_last_error;
thread_local ctg::DmrgOptions g_opts = [] {
	ctg::DmrgOptions o;
	if (const char* p = std::getenv("CTGPU_PRECISION"))
		o.precision = ctg::is_tc_precision(std::atoi(p)) ? std::atoi(p) : (int)ctg::GEMM_FP64;
	if (const char* d = std::getenv("CTGPU_DEVICE")) o.device = std::atoi(d);
	return o;
}();
thread_local ctg::DmrgStats g_stats;

constexpr int ERR_RUNTIME = -5;

template <class F>
int guarded(F&& f)
{
	try
	{
		g_last_error.clear();
		return f();
	}
	catch (const std::exception& e)
	{
		g_last_error = e.what();
		fprintf(stderr, "ctgpu: %s\n", e.what());
		return ERR_RUNTIME;
	}
}

}  // namespace

extern "C" {

int dmrg_twosite(const struct mpo* hamiltonian, const int num_sweeps, const int maxiter_lanczos, const double tol_split,
                 const ct_long max_vdim, struct mps* psi, double* en_sweeps, double* entropy)
{
	return guarded([&] {
		CTG_CHECK(hamiltonian && psi && en_sweeps && entropy, "null argument");
		CTG_CHECK(tol_split >= 0, "tol_split must be non-negative");
		CTG_CHECK(max_vdim > 0, "max_vdim must be positive");
		return ctg::dmrg_twosite_gpu(hamiltonian, num_sweeps, maxiter_lanczos, tol_split, max_vdim, psi, en_sweeps, entropy,
		                             g_opts, &g_stats);
	});
}

int dmrg_singlesite(const struct mpo* hamiltonian, const int num_sweeps, const int maxiter_lanczos, struct mps* psi,
                    double* en_sweeps)
{
	return guarded([&] {
		CTG_CHECK(hamiltonian && psi && en_sweeps, "null argument");
		return ctg::dmrg_singlesite_gpu(hamiltonian, num_sweeps, maxiter_lanczos, psi, en_sweeps, g_opts, &g_stats);
	});
}

int ctgpu_set_final_fp64_sweeps(int n)
{
	if (n < 1) return ERR_RUNTIME;
	const int prev = g_opts.final_fp64_sweeps;
	g_opts.final_fp64_sweeps = n;
	return prev;
}

int ctgpu_set_reduced_environments(int on)
{
	const int prev = g_opts.reduced_env ? 1 : 0;
	g_opts.reduced_env = on != 0;
	return prev;
}

int ctgpu_set_precision(int precision)
{
	if (precision != ctg::GEMM_FP64 && !ctg::is_tc_precision(precision)) return ERR_RUNTIME;
	const int old = g_opts.precision;
	g_opts.precision = precision;
	return old;
}

int ctgpu_clear_plan_cache(void)
{
	return guarded([&] {
		ctg::context_for_device(g_opts.device).clear_plans();
		return 0;
	});
}

int ctgpu_set_device(int device)
{
	const int old = g_opts.device;
	g_opts.device = device;
	return old;
}

int ctgpu_get_last_stats(struct ctgpu_stats* out)
{
	if (!out) return -1;
	const ctg::DmrgStats& s = g_stats;
	out->wall_s = s.wall_s;
	out->upload_s = s.upload_s;
	out->download_s = s.download_s;
	out->setup_s = s.setup_s;
	out->sweep_s = s.sweep_s;
	out->lanczos_ms = s.lanczos_ms;
	out->split_ms = s.split_ms;
	out->env_ms = s.env_ms;
	out->matvec_flops = s.matvec_flops;
	out->total_gemm_flops = s.total_gemm_flops;
	out->matvecs = s.matvecs;
	out->kernel_launches = s.kernel_launches;
	out->sweeps = s.sweeps;
	out->max_bond_dim = s.max_bond_dim;
	out->svd_max_sweeps = s.svd_max_sweeps;
	out->host_plan_s = s.host_plan_s;
	out->plan_hits = s.plan_hits;
	out->plan_misses = s.plan_misses;
	out->svd_flops = s.svd_flops;
	out->near_ties = s.near_ties;
	return 0;
}

int ctgpu_tile_tuning_report(char* buf, int cap)
{
	return guarded([&] {
		std::string text;
		for (const ctg::TuneEntry& e : ctg::tile_tuning_entries())
		{
			char line[640];
			snprintf(line, sizeof line, "%s %d %.4f %.4f %.4f %.4f %s\n", e.key.c_str(), e.bn, e.ms[0], e.ms[1], e.ms[2],
			         e.ms[3], e.from_file ? "file" : "timed");
			text += line;
		}
		if (buf && cap > 0)
		{
			const size_t n = std::min(text.size(), (size_t)cap - 1);
			memcpy(buf, text.data(), n);
			buf[n] = 0;
		}
		return (int)text.size();
	});
}

int ctgpu_tridiag_lowest(const double* alpha, const double* beta, int k, double* lambda, double* y)
{
	return guarded([&] {
		CTG_CHECK(alpha && lambda && y && k >= 1 && k <= ctg::LANCZOS_MAX && (k == 1 || beta), "invalid arguments");
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		std::vector<double> in(2 * (size_t)k, 0.0);
		for (int i = 0; i < k; i++) in[(size_t)i] = alpha[i];
		for (int i = 0; i + 1 < k; i++) in[(size_t)k + i] = beta[i];
		ctg::DBufPtr d_in = c.upload(in.data(), in.size() * sizeof(double));
		ctg::DBuf d_out(&c, (2 + (size_t)k) * sizeof(double));
		ctg::tridiag_lowest_test((const double*)d_in->ptr, (const double*)d_in->ptr + k, k, (double*)d_out.ptr, c.stream());
		std::vector<double> out(2 + (size_t)k);
		CTG_CUDA(cudaMemcpyAsync(out.data(), d_out.ptr, out.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream()));
		c.sync();
		*lambda = out[0];
		for (int i = 0; i < k; i++) y[i] = out[2 + (size_t)i];
		return (int)out[1];
	});
}

int ctgpu_inject_failure(int which, int count)
{
	if (count < 0 || which < 1 || which > 3) return ERR_RUNTIME;
	if (which == 1) ctg::g_inject_svd_failure = count;
	else if (which == 2) ctg::g_inject_tridiag_failure = count;
	else ctg::g_inject_zero_start = count;
	return 0;
}

int ctgpu_set_tc_tile_width(int bn)
{
	return guarded([&] {
		ctg::force_tc_tile_width(bn);
		return 0;
	});
}

void ctgpu_set_tc_wait_limit(long long polls)
{
	ctg::set_tc_wait_limit(polls);
}

ct_long ctgpu_get_bond_singular_values(int bond, double* out, ct_long max)
{
	if (bond < 0 || (size_t)bond >= g_stats.bond_sigma.size() || g_stats.bond_sigma[(size_t)bond].empty()) return -1;
	const std::vector<double>& v = g_stats.bond_sigma[(size_t)bond];
	for (ct_long i = 0; i < (ct_long)v.size() && i < max; i++) out[i] = v[(size_t)i];
	return (ct_long)v.size();
}

const char* ctgpu_last_error(void) { return g_last_error.c_str(); }

int ctgpu_set_profiling(int enable, int skip_sweeps)
{
	const int old = g_opts.profile;
	g_opts.profile = enable;
	g_opts.profile_skip_sweeps = skip_sweeps;
	return old;
}

void ctgpu_set_l2_flush_bytes(ct_long bytes) { g_opts.l2_flush_bytes = bytes; }

int ctgpu_get_sweep_times(double* ms, long* launches, int max)
{
	const int n = (int)g_stats.sweep_ms.size();
	for (int i = 0; i < n && i < max; i++)
	{
		if (ms) ms[i] = g_stats.sweep_ms[i];
		if (launches) launches[i] = g_stats.sweep_launches[i];
	}
	return n;
}

int ctgpu_get_kernel_profile(int cls, long* launches, double* ms, double* flops, double* bytes)
{
	if (cls < 0 || cls >= ctg::K_NUM_CLASSES) return -1;
	const ctg::KProf& k = g_stats.prof[cls];
	if (launches) *launches = k.launches;
	if (ms) *ms = k.ms;
	if (flops) *flops = k.flops;
	if (bytes) *bytes = k.bytes;
	return 0;
}

int ctgpu_block_sparse_tensor_dot(const struct block_sparse_tensor* s, int axrange_s, const struct block_sparse_tensor* t,
                                  int axrange_t, int ndim_mult, struct block_sparse_tensor* r)
{
	return guarded([&] {
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor ds = ctg::tensor_from_struct(c, s), dt = ctg::tensor_from_struct(c, t);
		ctg::DTensor dr = ctg::op_dot(c, ds, axrange_s, dt, axrange_t, ndim_mult, g_opts.precision);
		ctg::tensor_to_struct(c, dr, r);
		return 0;
	});
}

int ctgpu_block_sparse_tensor_transpose(const int* perm, const struct block_sparse_tensor* t, struct block_sparse_tensor* r)
{
	return guarded([&] {
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor dt = ctg::tensor_from_struct(c, t);
		ctg::DTensor dr = ctg::op_transpose(c, dt, perm);
		ctg::tensor_to_struct(c, dr, r);
		return 0;
	});
}

int ctgpu_apply_local_hamiltonian(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
                                  const struct block_sparse_tensor* l, const struct block_sparse_tensor* r,
                                  struct block_sparse_tensor* b)
{
	return guarded([&] {
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a), dw = ctg::tensor_from_struct(c, w);
		ctg::DTensor dl = ctg::tensor_from_struct(c, l), dr = ctg::tensor_from_struct(c, r);
		ctg::DTensor out = ctg::apply_local_hamiltonian_once(c, da, dw, dl, dr, g_opts.precision);
		ctg::tensor_to_struct(c, out, b);
		return 0;
	});
}

int ctgpu_time_local_hamiltonian(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
                                 const struct block_sparse_tensor* l, const struct block_sparse_tensor* r, int nmatvec,
                                 double* ms, double* flops)
{
	return guarded([&] {
		CTG_CHECK(nmatvec >= 1 && ms && flops, "invalid arguments");
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a), dw = ctg::tensor_from_struct(c, w);
		ctg::DTensor dl = ctg::tensor_from_struct(c, l), dr = ctg::tensor_from_struct(c, r);
		*ms = ctg::time_local_hamiltonian(c, da, dw, dl, dr, g_opts.precision, nmatvec, flops);
		return 0;
	});
}

int ctgpu_contraction_operator_step_left(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
                                         const struct block_sparse_tensor* l, struct block_sparse_tensor* l_next)
{
	return guarded([&] {
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a), dw = ctg::tensor_from_struct(c, w), dl = ctg::tensor_from_struct(c, l);
		ctg::tensor_to_struct(c, ctg::contraction_step_left(c, da, dw, dl, g_opts.precision), l_next);
		return 0;
	});
}

int ctgpu_contraction_operator_step_right(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
                                          const struct block_sparse_tensor* r, struct block_sparse_tensor* r_next)
{
	return guarded([&] {
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a), dw = ctg::tensor_from_struct(c, w), dr = ctg::tensor_from_struct(c, r);
		ctg::tensor_to_struct(c, ctg::contraction_step_right(c, da, dw, dr, g_opts.precision), r_next);
		return 0;
	});
}

int ctgpu_block_sparse_tensor_svd_values(const struct block_sparse_tensor* a, double* sigma, ct_long* ns)
{
	return guarded([&] {
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a);
		ctg::SvdResult sv;
		const int ret = ctg::op_svd(c, da, sv);
		if (ret < 0) return ret;
		CTG_CUDA(cudaMemcpy(sigma, sv.s->ptr, (size_t)sv.ns * sizeof(double), cudaMemcpyDeviceToHost));
		*ns = sv.ns;
		return 0;
	});
}

int ctgpu_device_memory(int device, size_t* free_bytes, size_t* total_bytes)
{
	return guarded([&] {
		CTG_CHECK(free_bytes && total_bytes, "null argument");
		int prev = 0;
		CTG_CUDA(cudaGetDevice(&prev));
		CTG_CUDA(cudaSetDevice(device));
		CTG_CUDA(cudaMemGetInfo(free_bytes, total_bytes));
		CTG_CUDA(cudaSetDevice(prev));
		return 0;
	});
}

int ctgpu_mpo_inner_product(const struct mps* chi, const struct mpo* op, const struct mps* psi, double* ret)
{
	return guarded([&] {
		CTG_CHECK(ret, "null argument");
		ctg::mpo_inner_product_gpu(chi, op, psi, g_opts.device, ret);
		return 0;
	});
}

int ctgpu_mps_vdot(const struct mps* chi, const struct mps* psi, double* ret)
{
	return guarded([&] {
		CTG_CHECK(ret, "null argument");
		ctg::mps_vdot_gpu(chi, psi, g_opts.device, ret);
		return 0;
	});
}

int ctgpu_mps_norm(const struct mps* psi, double* ret)
{
	return guarded([&] {
		CTG_CHECK(psi && ret, "null argument");
		if (psi->nsites == 0)
		{
			*ret = 0;
			return 0;
		}
		double v[2] = {0.0, 0.0};
		ctg::mps_vdot_gpu(psi, psi, g_opts.device, v);
		const double nrm2 = v[0];
		CTG_CHECK(nrm2 >= -1e-12, "mps_norm: negative squared norm");
		*ret = std::sqrt(std::max(nrm2, 0.0));
		return 0;
	});
}

int ctgpu_construct_spin_molecular_mpo(int nsites, const double* tkin, const double* vint, struct mpo* out)
{
	return guarded([&] { return ctg::build_spin_molecular_mpo(nsites, tkin, vint, out); });
}

int ctgpu_block_sparse_tensor_qr(const struct block_sparse_tensor* a, int mode, struct block_sparse_tensor* q,
                                 struct block_sparse_tensor* r)
{
	return guarded([&] {
		CTG_CHECK(a && q && r, "null argument");
		CTG_CHECK(mode == 0, "block_sparse_tensor_qr: only QR_REDUCED is supported");
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a);
		ctg::DTensor dq, dr;
		const int ret = ctg::op_qr(c, da, dq, dr);
		if (ret < 0) return ret;
		ctg::tensor_to_struct(c, dq, q);
		ctg::tensor_to_struct(c, dr, r);
		return 0;
	});
}

int ctgpu_block_sparse_tensor_rq(const struct block_sparse_tensor* a, int mode, struct block_sparse_tensor* r,
                                 struct block_sparse_tensor* q)
{
	return guarded([&] {
		CTG_CHECK(a && q && r, "null argument");
		CTG_CHECK(mode == 0, "block_sparse_tensor_rq: only QR_REDUCED is supported");
		ctg::Ctx& c = ctg::context_for_device(g_opts.device);
		ctg::DTensor da = ctg::tensor_from_struct(c, a);
		ctg::DTensor dr, dq;
		const int ret = ctg::op_rq(c, da, dr, dq);
		if (ret < 0) return ret;
		ctg::tensor_to_struct(c, dr, r);
		ctg::tensor_to_struct(c, dq, q);
		return 0;
	});
}

double ctgpu_measure_fp64_tflops(void)
{
	double r = -1;
	guarded([&] {
		r = ctg::measure_fp64_fma_tflops(g_opts.device);
		return 0;
	});
	return r;
}

void ctgpu_delete_block_sparse_tensor(struct block_sparse_tensor* t)
{
	if (t) ctg::free_struct(t);
}

}  // extern "C"
