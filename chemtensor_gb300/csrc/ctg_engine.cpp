// ctg_engine.cpp - lowering of block-sparse tensor operations to device work lists.
#include "ctg_engine.h"
#include "ctg_plan.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <functional>
#include <memory>
#include <mutex>
#include <cstring>
#include <ctime>

#include <dlfcn.h>

namespace ctg {

// ------------------------------------------------------------------------------------
// memory and context
// ------------------------------------------------------------------------------------

DBuf::DBuf(Ctx* c, size_t n) : ctx(c), bytes(n) { ptr = c->alloc(n); }
DBuf::~DBuf()
{
	if (ptr && ctx) ctx->free(ptr);
}

// ---- plan cache ------------------------------------------------------------------------
// An entry holds the operand structures it was built for (dims, directions, quantum numbers),
// the operation parameters, and the plan: a lookup is a hash probe plus an exact comparison.
struct StructSig {
	int ndim = 0;
	std::vector<i64> dim;
	std::vector<int> dir;
	std::vector<std::vector<q32>> ql;
	StructSig() = default;
	explicit StructSig(const Meta& m) : ndim(m.ndim), dim(m.dim), dir(m.dir), ql(m.ql) {}
	bool matches(const Meta& m) const { return ndim == m.ndim && dim == m.dim && dir == m.dir && ql == m.ql; }
};

struct PlanEntry {
	int kind = 0;
	std::vector<i64> params;
	StructSig s, t;
	DotPlan dot;
	CopyPlan copy;
};

struct PlanCache {
	std::unordered_multimap<uint64_t, PlanEntry> map;
	size_t bytes = 0;
	static constexpr size_t MAX_ENTRIES = 1 << 14;
	static constexpr size_t MAX_BYTES = (size_t)1 << 30;
};

static uint64_t plan_key(int kind, const std::vector<i64>& params, const Meta& s, const Meta* t)
{
	uint64_t h = s.structure_hash() * 0x9e3779b97f4a7c15ull + (uint64_t)kind;
	if (t) h ^= t->structure_hash() + 0x632be59bd9b4e019ull + (h << 7) + (h >> 3);
	for (i64 v : params) h = (h ^ (uint64_t)v) * 0x100000001b3ull;
	return h;
}

static const PlanEntry* plan_find(Ctx& c, uint64_t key, int kind, const std::vector<i64>& params, const Meta& s,
                                  const Meta* t)
{
	PlanCache* pc = c.plans();
	auto range = pc->map.equal_range(key);
	for (auto it = range.first; it != range.second; ++it)
	{
		const PlanEntry& e = it->second;
		if (e.kind == kind && e.params == params && e.s.matches(s) && (!t || e.t.matches(*t)))
		{
			c.plan_hits++;
			return &e;
		}
	}
	c.plan_misses++;
	return nullptr;
}

void Ctx::clear_plans()
{
	plans_->map.clear();
	plans_->bytes = 0;
}

static void plan_insert(Ctx& c, uint64_t key, PlanEntry&& e, size_t bytes)
{
	PlanCache* pc = c.plans();
	if (pc->map.size() >= PlanCache::MAX_ENTRIES || pc->bytes + bytes > PlanCache::MAX_BYTES)
	{
		pc->map.clear();
		pc->bytes = 0;
	}
	pc->bytes += bytes;
	pc->map.emplace(key, std::move(e));
}

Ctx::Ctx(int device) : dev_(device)
{
	CTG_CUDA(cudaSetDevice(dev_));
	CTG_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev_));
	CTG_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
	cudaMemPoolProps props = {};
	props.allocType = cudaMemAllocationTypePinned;
	props.handleTypes = cudaMemHandleTypeNone;
	props.location.type = cudaMemLocationTypeDevice;
	props.location.id = dev_;
	CTG_CUDA(cudaMemPoolCreate(&pool_, &props));
	uint64_t thr = UINT64_MAX;
	CTG_CUDA(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &thr));
	staging_cap_ = (size_t)64 << 20;
	CTG_CUDA(cudaMallocHost((void**)&staging_, staging_cap_));
	plans_ = new PlanCache();
	CTG_CUDA(cudaMallocHost(&pinned_, 4096));
	memset(pinned_, 0, 4096);
	CTG_CUDA(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
	for (int i = 0; i < NUM_AUX; i++)
	{
		CTG_CUDA(cudaStreamCreateWithFlags(&aux_[i], cudaStreamNonBlocking));
		CTG_CUDA(cudaEventCreateWithFlags(&join_ev_[i], cudaEventDisableTiming));
	}
}

static double host_seconds()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}


static double thread_cpu_seconds()
{
	timespec ts;
	clock_gettime(CLOCK_THREAD_CPUTIME_ID, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

PlanTimer::PlanTimer(Ctx& ctx) : c(ctx), t0(host_seconds()), cpu0(thread_cpu_seconds()) {}

PlanTimer::~PlanTimer()
{
	c.host_plan_s += host_seconds() - t0;
	c.host_plan_cpu_s += thread_cpu_seconds() - cpu0;
}

static_assert(256 + sizeof(LanczosScalars) <= 2048, "pinned result slots overlap");

double* Ctx::pinned_doubles(size_t n)
{
	if (n > pinned_d_cap_)
	{
		if (pinned_d_) CTG_CUDA(cudaFreeHost(pinned_d_));
		pinned_d_ = nullptr;
		pinned_d_cap_ = std::max<size_t>(n, 1 << 16);
		CTG_CUDA(cudaMallocHost((void**)&pinned_d_, pinned_d_cap_ * sizeof(double)));
	}
	return pinned_d_;
}

cudaStream_t Ctx::aux(int i)
{
	return aux_[i % NUM_AUX];
}

void Ctx::fork(int n)
{
	n = std::min(n, (int)NUM_AUX);
	CTG_CUDA(cudaEventRecord(fork_ev_, st_));
	for (int i = 0; i < n; i++) CTG_CUDA(cudaStreamWaitEvent(aux_[i], fork_ev_, 0));
}

void Ctx::join(int n)
{
	n = std::min(n, (int)NUM_AUX);
	for (int i = 0; i < n; i++)
	{
		CTG_CUDA(cudaEventRecord(join_ev_[i], aux_[i]));
		CTG_CUDA(cudaStreamWaitEvent(st_, join_ev_[i], 0));
	}
}

Ctx::~Ctx()
{
	if (st_) cudaStreamSynchronize(st_);
	for (int i = 0; i < NUM_AUX; i++)
	{
		if (aux_[i]) cudaStreamSynchronize(aux_[i]);
		if (aux_[i]) cudaStreamDestroy(aux_[i]);
		if (join_ev_[i]) cudaEventDestroy(join_ev_[i]);
	}
	delete plans_;
	if (pinned_) cudaFreeHost(pinned_);
	if (pinned_d_) cudaFreeHost(pinned_d_);
	if (fork_ev_) cudaEventDestroy(fork_ev_);
	if (staging_) cudaFreeHost(staging_);
	if (pool_) cudaMemPoolDestroy(pool_);
	if (st_) cudaStreamDestroy(st_);
}

Ctx& context_for_device(int device)
{
	// one context per (thread, device); deliberately never destroyed so that no CUDA call
	// runs during process teardown
	thread_local std::vector<Ctx*> ctxs;
	for (Ctx* c : ctxs)
		if (c->device() == device)
		{
			CTG_CUDA(cudaSetDevice(device));
			return *c;
		}
	ctxs.push_back(new Ctx(device));
	return *ctxs.back();
}

void* Ctx::alloc(size_t bytes)
{
	const double t0 = host_seconds();
	void* p = nullptr;
	if (bytes == 0) bytes = 16;
	CTG_CUDA(cudaMallocFromPoolAsync(&p, (bytes + 255) & ~(size_t)255, pool_, st_));
	host_alloc_s += host_seconds() - t0;
	return p;
}

void Ctx::free(void* p)
{
	cudaFreeAsync(p, st_);
}

void Ctx::reserve(size_t bytes)
{
	if (bytes <= reserved_) return;
	void* p = alloc(bytes);
	free(p);
	sync();
	reserved_ = bytes;
}

void Ctx::sync()
{
	CTG_CUDA(cudaStreamSynchronize(st_));
	staging_used_ = 0;
	prof_resolve();
	if (tc_used_)
	{
		int flag = 0;
		CTG_CUDA(cudaMemcpy(&flag, tc_error_, sizeof(int), cudaMemcpyDeviceToHost));
		tc_used_ = false;
		if (flag != 0)
		{
			CTG_CUDA(cudaMemset(tc_error_, 0, sizeof(int)));
			throw std::runtime_error("ctgpu: a tensor-core GEMM timed out waiting for its MMAs");
		}
	}
}

int* Ctx::tc_error()
{
	if (!tc_error_)
	{
		CTG_CUDA(cudaMalloc(&tc_error_, sizeof(int)));
		CTG_CUDA(cudaMemset(tc_error_, 0, sizeof(int)));
	}
	tc_used_ = true;
	return tc_error_;
}

cudaEvent_t Ctx::get_event()
{
	if (event_pool_.empty())
	{
		cudaEvent_t e;
		CTG_CUDA(cudaEventCreate(&e));
		return e;
	}
	cudaEvent_t e = event_pool_.back();
	event_pool_.pop_back();
	return e;
}

void Ctx::prof_begin()
{
	if (!profile) return;
	open_ = get_event();
	CTG_CUDA(cudaEventRecord(open_, st_));
}

void Ctx::prof_end(int cls, int launches, double flops, double bytes)
{
	if (!profile || !open_) return;
	cudaEvent_t e1 = get_event();
	CTG_CUDA(cudaEventRecord(e1, st_));
	pending_.push_back(Pending{cls, launches, open_, e1, flops, bytes});
	open_ = nullptr;
}

void Ctx::prof_resolve()
{
	for (const Pending& p : pending_)
	{
		float ms = 0;
		CTG_CUDA(cudaEventElapsedTime(&ms, p.e0, p.e1));
		KProf& k = prof[p.cls];
		k.launches += p.launches;
		k.ms += ms;
		k.flops += p.flops;
		k.bytes += p.bytes;
		event_pool_.push_back(p.e0);
		event_pool_.push_back(p.e1);
	}
	pending_.clear();
}

void Ctx::prof_reset()
{
	for (auto& k : prof) k = KProf();
}

KScope::KScope(Ctx& ctx, int cls_, int launches_, double flops_, double bytes_)
	: c(ctx), cls(cls_), launches(launches_), flops(flops_), bytes(bytes_)
{
	c.prof_begin();
}

KScope::~KScope()
{
	c.prof_end(cls, launches, flops, bytes);
	c.kernel_launches += launches;
}

DBufPtr Ctx::upload(const void* host, size_t bytes)
{
	CTG_CHECK(host != nullptr || bytes == 0, "upload from a null host pointer");
	struct T { Ctx* c; double t0; ~T() { c->host_upload_s += host_seconds() - t0; } } timer{this, host_seconds()};
	auto b = std::make_shared<DBuf>(this, bytes);
	size_t done = 0;
	while (done < bytes)
	{
		if (staging_used_ >= staging_cap_) sync();
		const size_t chunk = std::min(bytes - done, staging_cap_ - staging_used_);
		char* stage = staging_ + staging_used_;
		memcpy(stage, (const char*)host + done, chunk);
		CTG_CUDA(cudaMemcpyAsync((char*)b->ptr + done, stage, chunk, cudaMemcpyHostToDevice, st_));
		staging_used_ += (chunk + 255) & ~(size_t)255;
		done += chunk;
	}
	return b;
}

DTensor Ctx::empty(const Meta& m, bool cplx)
{
	DTensor t;
	t.meta = std::make_shared<const Meta>(m);
	t.cplx = cplx;
	t.buf = std::make_shared<DBuf>(this, (size_t)std::max<i64>(m.nnz, 1) * t.width() * sizeof(double));
	return t;
}

DTensor Ctx::empty(const std::shared_ptr<const Meta>& m, bool cplx)
{
	DTensor t;
	t.meta = m;
	t.cplx = cplx;
	t.buf = std::make_shared<DBuf>(this, (size_t)std::max<i64>(m->nnz, 1) * t.width() * sizeof(double));
	return t;
}

DTensor Ctx::zeros(const Meta& m, bool cplx)
{
	DTensor t = empty(m, cplx);
	CTG_CUDA(cudaMemsetAsync(t.data(), 0, (size_t)std::max<i64>(m.nnz, 1) * t.width() * sizeof(double), st_));
	return t;
}

void copy_to_device(Ctx& c, DTensor& t, const double* host)
{
	if (t.m().nnz == 0) return;
	DBufPtr b = c.upload(host, (size_t)t.m().nnz * t.width() * sizeof(double));
	t.buf = b;
}

void copy_to_host(Ctx& c, const DTensor& t, double* host)
{
	if (t.m().nnz == 0) return;
	CTG_CUDA(cudaMemcpyAsync(host, t.data(), (size_t)t.m().nnz * t.width() * sizeof(double), cudaMemcpyDeviceToHost,
	                         c.stream()));
	c.sync();
	// a conjugated view is handed out with its conjugation applied
	if (t.conj)
		for (i64 i = 0; i < t.m().nnz; i++) host[2 * i + 1] = -host[2 * i + 1];
}

// ------------------------------------------------------------------------------------
// descriptor packing: several typed arrays in one device buffer
// ------------------------------------------------------------------------------------

namespace {

struct Packer {
	std::vector<char> bytes;
	template <class T>
	size_t add(const std::vector<T>& v)
	{
		const size_t off = (bytes.size() + 15) & ~(size_t)15;
		bytes.resize(off + v.size() * sizeof(T));
		if (!v.empty()) memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
		return off;
	}
};

template <class T>
const T* at(const DBufPtr& b, size_t off)
{
	return (const T*)((const char*)b->ptr + off);
}

}  // namespace

// ------------------------------------------------------------------------------------
// dot (block_sparse_tensor.c:1826-2001; dense_tensor.c:1761-1837)
// ------------------------------------------------------------------------------------

static DotPlan upload_dot_plan(Ctx& c, DotLowering&& l, int precision, int bn);
static int tuned_tile_width(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision,
                            const int* out_perm, const DotLowering& l64);

static DotPlan build_dot_plan(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision,
                              const int* out_perm)
{
	// complex128: the FP64 work lists (outputs, contributions) with tiles of the complex GEMM
	const bool z = precision == GEMM_Z64;
	if (is_tc_precision(precision))
	{
		// the autotuner picks the tile width, or FP64 where the product is too small for the tensor
		// cores to pay for their operand packing (FP64 is then both faster and exact). Its key comes
		// from the output blocks and contributions, which the FP64 lowering has too: a product that
		// stays on FP64 is lowered once, one on the tensor cores twice
		DotLowering l = lower_dot(s, axs, t, axt, nmult, GEMM_FP64, c.num_sms(), out_perm);
		const int bn = tuned_tile_width(c, s, axs, t, axt, nmult, precision, out_perm, l);
		if (bn == 0) return upload_dot_plan(c, std::move(l), GEMM_FP64, 64);
		return upload_dot_plan(c, lower_dot(s, axs, t, axt, nmult, precision, c.num_sms(), out_perm, bn), precision, bn);
	}
	DotLowering l = lower_dot(s, axs, t, axt, nmult, z ? (int)GEMM_FP64 : precision, c.num_sms(), out_perm);
	return upload_dot_plan(c, std::move(l), precision, 64);
}

static DotPlan upload_dot_plan(Ctx& c, DotLowering&& l, int precision, int bn)
{
	const bool z = precision == GEMM_Z64;
	std::vector<ZTile> zt;
	if (z)
	{
		for (size_t b = 0; b < l.outs.size(); b++)
			for (int m0 = 0; m0 < l.outs[b].m; m0 += 32)
				for (int n0 = 0; n0 < l.outs[b].n; n0 += 32) zt.push_back(ZTile{(int)b, m0, n0, 0});
		l.tiles.clear();
		l.splits.clear();
		l.work_doubles = 0;
	}
	DotPlan p;
	p.out = l.out;
	p.precision = precision;
	p.tc_fmt = tc_format_of(precision);
	p.tc_bn = bn;
	Packer pk;
	const size_t o_outs = pk.add(l.outs);
	const size_t o_cons = pk.add(l.cons);
	const size_t o_tiles = pk.add(l.tiles);
	const size_t o_splits = pk.add(l.splits);
	const size_t o_tcons = pk.add(l.tcons), o_apacks = pk.add(l.apacks), o_bpacks = pk.add(l.bpacks);
	const size_t o_zt = pk.add(zt);
	// at least 16 bytes, from the packer's own storage (a product without output blocks packs nothing)
	if (pk.bytes.size() < 16) pk.bytes.resize(16);
	p.desc = c.upload(pk.bytes.data(), pk.bytes.size());
	p.nztiles = (int)zt.size();
	p.ztiles = at<ZTile>(p.desc, o_zt);
	p.tcons = at<TcContrib>(p.desc, o_tcons);
	p.apacks = at<TcPack>(p.desc, o_apacks);
	p.bpacks = at<TcPack>(p.desc, o_bpacks);
	p.a_recs = (i64)l.apacks.size();
	p.b_recs = (i64)l.bpacks.size();
	p.outs = at<GemmOut>(p.desc, o_outs);
	p.cons = at<GemmContrib>(p.desc, o_cons);
	p.splits = at<GemmSplit>(p.desc, o_splits);
	p.nsplits = (int)l.splits.size();
	if (l.work_doubles > 0) p.work = std::make_shared<DBuf>(&c, (size_t)l.work_doubles * sizeof(double));
	if (!l.splits.empty())
	{
		// completion counters of the split tiles: zero now, and reset by the kernel after each use
		p.counters = std::make_shared<DBuf>(&c, l.splits.size() * sizeof(int));
		CTG_CUDA(cudaMemsetAsync(p.counters->ptr, 0, l.splits.size() * sizeof(int), c.stream()));
	}
	p.ntiles[0] = (int)l.tiles.size();
	p.tiles[0] = at<GemmTile>(p.desc, o_tiles);
	p.flops = l.flops;
	for (int k = 0; k < NUM_TILE_CLASSES; k++) p.flops_cls[k] = l.flops_cls[k];
	p.a_entries = l.a_entries;
	p.b_entries = l.b_entries;
	return p;
}

void DotPlan::run(Ctx& c, const double* A, const double* B, double* C) const
{
	if (is_tc_precision(precision))
	{
		if (ntiles[0] > 0)
		{
			DBuf apk(&c, (size_t)std::max<i64>(a_rec_bytes(), 16));
			DBuf bpk(&c, (size_t)std::max<i64>(b_rec_bytes(), 16));
			pack_a(c, A, apk.ptr);
			pack_b(c, B, bpk.ptr);
			run_packed(c, apk.ptr, bpk.ptr, C);
		}
		c.gemm_flops += flops;
		return;
	}
	double* w = work ? (double*)work->ptr : nullptr;
	int* cnt = counters ? (int*)counters->ptr : nullptr;
	if (ntiles[0] > 0)
	{
		KScope ks(c, K_GEMM, 1, flops, 0);
		launch_gemm_f64(ntiles[0], tiles[0], outs, cons, splits, cnt, A, B, C, w, c.stream(), flops);
	}
	c.gemm_flops += flops;
}

void DotPlan::run_z(Ctx& c, const double* A, const double* B, double* C, bool conj_a, bool conj_b) const
{
	CTG_CHECK(precision == GEMM_Z64, "complex GEMM on a real plan");
	KScope ks(c, K_GEMM, 1, 4.0 * flops, 0);
	launch_gemm_z(nztiles, ztiles, outs, cons, A, B, C, conj_a ? 1 : 0, conj_b ? 1 : 0, c.stream());
	c.gemm_flops += 4.0 * flops;
}

void DotPlan::pack_a(Ctx& c, const void* A, void* apack, bool src_f32) const
{
	KScope ks(c, K_GEMM_TC, 1, 0, (src_f32 ? 4.0 : 8.0) * (double)a_entries + (double)a_rec_bytes());
	launch_tc_pack(tc_fmt, (int)a_recs, apacks, 1, A, src_f32, apack, c.stream());
}

void DotPlan::pack_b(Ctx& c, const void* B, void* bpack, bool src_f32) const
{
	KScope ks(c, K_GEMM_TC, 1, 0, (src_f32 ? 4.0 : 8.0) * (double)b_entries + (double)b_rec_bytes());
	launch_tc_pack(tc_fmt, (int)b_recs, bpacks, 0, B, src_f32, bpack, c.stream());
}

void DotPlan::run_packed(Ctx& c, const void* apack, const void* bpack, void* C, bool out_f32) const
{
	if (ntiles[0] > 0)
	{
		KScope ks(c, K_GEMM_TC, 1, flops_cls[0], 0);
		launch_gemm_tc(tc_fmt, tc_bn, ntiles[0], tiles[0], outs, tcons, apack, bpack, C, out_f32, c.tc_error(), c.stream());
	}
}

// ------------------------------------------------------------------------------------
// tile autotuner of the tensor-core GEMM
// ------------------------------------------------------------------------------------

namespace {

struct TuneTable {
	std::mutex mu;
	bool loaded = false;
	std::string path;
	std::vector<TuneEntry> entries;
	const TuneEntry* find(const std::string& k) const
	{
		for (const TuneEntry& e : entries)
			if (e.key == k) return &e;
		return nullptr;
	}
};

TuneTable& tune_table()
{
	static TuneTable t;
	return t;
}

std::string library_dir()
{
	Dl_info info;
	if (dladdr((const void*)&tile_tuning_entries, &info) && info.dli_fname)
	{
		std::string f = info.dli_fname;
		const size_t sl = f.rfind('/');
		if (sl != std::string::npos) return f.substr(0, sl);
	}
	return ".";
}

void tune_load(TuneTable& t)
{
	if (t.loaded) return;
	t.loaded = true;
	const char* env = getenv("CTGPU_TUNE_FILE");
	t.path = env ? env : library_dir() + "/tile_tuning.txt";
	FILE* f = fopen(t.path.c_str(), "r");
	if (!f) return;
	char line[1024], key[512];
	int bn;
	double a, b, d, q;
	while (fgets(line, sizeof line, f))
	{
		if (sscanf(line, "%511s %d %lf %lf %lf %lf", key, &bn, &a, &b, &d, &q) != 6) continue;
		if (bn != 0 && bn != 64 && bn != 128 && bn != 256) continue;
		if (t.find(key)) continue;
		TuneEntry e;
		e.key = key;
		e.bn = bn;
		e.ms[0] = a;
		e.ms[1] = b;
		e.ms[2] = d;
		e.ms[3] = q;
		e.from_file = true;
		t.entries.push_back(e);
	}
	fclose(f);
}

// flop-weighted histogram of a product's output blocks by column extent (<= 64, 128, 256, 512,
// more) and summed contracted extent (<= 64, 256, more), shares rounded to eighths; with the
// precision and the log4 of the total work
std::string tune_key(const DotLowering& l, int precision)
{
	double hn[5] = {0, 0, 0, 0, 0}, hk[3] = {0, 0, 0}, total = 0;
	for (const GemmOut& o : l.outs)
	{
		i64 ks = 0;
		for (int cc = o.c0; cc < o.c0 + o.nc; cc++) ks += l.cons[(size_t)cc].k;
		const double f = 2.0 * (double)o.m * (double)o.n * (double)ks;
		const int bn = o.n <= 64 ? 0 : o.n <= 128 ? 1 : o.n <= 256 ? 2 : o.n <= 512 ? 3 : 4;
		const int bk = ks <= 64 ? 0 : ks <= 256 ? 1 : 2;
		hn[bn] += f;
		hk[bk] += f;
		total += f;
	}
	char buf[160];
	auto q = [&](double x) { return total > 0 ? (int)std::lround(8.0 * x / total) : 0; };
	snprintf(buf, sizeof buf, "p%d_w%d_n%d.%d.%d.%d.%d_k%d.%d.%d", precision,
	         total > 0 ? (int)std::floor(std::log(total) / std::log(4.0)) : 0, q(hn[0]), q(hn[1]), q(hn[2]), q(hn[3]),
	         q(hn[4]), q(hk[0]), q(hk[1]), q(hk[2]));
	return buf;
}

// device time (ms) of one product on zero operands: for the tensor cores, packing the B operand (per
// application one operand is packed afresh) and the GEMM; for FP64 (bn == 0), the FP64 GEMM
double time_tc_variant(Ctx& c, DotLowering&& l, int precision, int bn, const Meta& s, const Meta& t)
{
	DotPlan p = upload_dot_plan(c, std::move(l), bn == 0 ? (int)GEMM_FP64 : precision, bn == 0 ? 64 : bn);
	if (p.ntiles[0] == 0) return 0.0;
	if (bn == 0)
	{
		DBuf A(&c, (size_t)std::max<i64>(s.nnz, 1) * sizeof(double));
		DBuf B(&c, (size_t)std::max<i64>(t.nnz, 1) * sizeof(double));
		DBuf C(&c, (size_t)std::max<i64>(p.out->nnz, 1) * sizeof(double));
		CTG_CUDA(cudaMemsetAsync(A.ptr, 0, A.bytes, c.stream()));
		CTG_CUDA(cudaMemsetAsync(B.ptr, 0, B.bytes, c.stream()));
		cudaEvent_t e[2];
		for (auto& x : e) CTG_CUDA(cudaEventCreate(&x));
		float best = 1e30f;
		for (int rep = 0; rep < 3; rep++)
		{
			CTG_CUDA(cudaEventRecord(e[0], c.stream()));
			launch_gemm_f64(p.ntiles[0], p.tiles[0], p.outs, p.cons, p.splits, p.counters ? (int*)p.counters->ptr : nullptr,
			                (const double*)A.ptr, (const double*)B.ptr, (double*)C.ptr,
			                p.work ? (double*)p.work->ptr : nullptr, c.stream());
			CTG_CUDA(cudaEventRecord(e[1], c.stream()));
			CTG_CUDA(cudaEventSynchronize(e[1]));
			float ms = 0;
			CTG_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
			if (rep > 0) best = std::min(best, ms);
		}
		for (auto& x : e) cudaEventDestroy(x);
		c.sync();
		return best;
	}
	DBuf A(&c, (size_t)std::max<i64>(s.nnz, 1) * sizeof(double));
	DBuf B(&c, (size_t)std::max<i64>(t.nnz, 1) * sizeof(double));
	DBuf C(&c, (size_t)std::max<i64>(p.out->nnz, 1) * sizeof(double));
	DBuf apk(&c, (size_t)std::max<i64>(p.a_rec_bytes(), 16));
	DBuf bpk(&c, (size_t)std::max<i64>(p.b_rec_bytes(), 16));
	CTG_CUDA(cudaMemsetAsync(A.ptr, 0, A.bytes, c.stream()));
	CTG_CUDA(cudaMemsetAsync(B.ptr, 0, B.bytes, c.stream()));
	launch_tc_pack(p.tc_fmt, (int)p.a_recs, p.apacks, 1, A.ptr, false, apk.ptr, c.stream());
	cudaEvent_t e[2];
	for (auto& x : e) CTG_CUDA(cudaEventCreate(&x));
	float best = 1e30f;
	for (int rep = 0; rep < 3; rep++)
	{
		CTG_CUDA(cudaEventRecord(e[0], c.stream()));
		launch_tc_pack(p.tc_fmt, (int)p.b_recs, p.bpacks, 0, B.ptr, false, bpk.ptr, c.stream());
		launch_gemm_tc(p.tc_fmt, bn, p.ntiles[0], p.tiles[0], p.outs, p.tcons, apk.ptr, bpk.ptr, C.ptr, false, c.tc_error(),
		               c.stream());
		CTG_CUDA(cudaEventRecord(e[1], c.stream()));
		CTG_CUDA(cudaEventSynchronize(e[1]));
		float ms = 0;
		CTG_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
		if (rep > 0) best = std::min(best, ms);     // the first run pays for loading the kernel
	}
	for (auto& x : e) cudaEventDestroy(x);
	c.sync();
	return best;
}

}  // namespace

std::atomic<int> g_forced_tc_bn{0};

void force_tc_tile_width(int bn)
{
	CTG_CHECK(bn == 0 || bn == 64 || bn == 128 || bn == 256, "tensor-core tile width must be 0, 64, 128 or 256");
	g_forced_tc_bn.store(bn);
}

std::vector<TuneEntry> tile_tuning_entries()
{
	TuneTable& t = tune_table();
	std::lock_guard<std::mutex> g(t.mu);
	tune_load(t);
	return t.entries;
}

static int tuned_tile_width(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision,
                            const int* out_perm, const DotLowering& l64)
{
	static const int env_forced = [] {
		const char* e = getenv("CTGPU_TC_BN");
		const int v = e ? atoi(e) : 0;
		return (v == 64 || v == 128 || v == 256) ? v : 0;
	}();
	const int forced = g_forced_tc_bn.load();
	if (forced) return forced;
	if (env_forced) return env_forced;
	if (l64.tiles.empty()) return 64;
	const std::string key = tune_key(l64, precision);
	TuneTable& tt = tune_table();
	{
		std::lock_guard<std::mutex> g(tt.mu);
		tune_load(tt);
		if (const TuneEntry* e = tt.find(key)) return e->bn;
	}
	// first sight: time the three widths and the FP64 GEMM (the context's work so far completes first)
	c.sync();
	TuneEntry e;
	e.key = key;
	const int widths[3] = {64, 128, 256};
	double best = 1e300;
	for (int i = 0; i < 3; i++)
	{
		DotLowering l = lower_dot(s, axs, t, axt, nmult, precision, c.num_sms(), out_perm, widths[i]);
		e.ms[i] = time_tc_variant(c, std::move(l), precision, widths[i], s, t);
		if (e.ms[i] < best)
		{
			best = e.ms[i];
			e.bn = widths[i];
		}
	}
	e.ms[3] = time_tc_variant(c, lower_dot(s, axs, t, axt, nmult, GEMM_FP64, c.num_sms(), out_perm), precision, 0, s, t);
	if (e.ms[3] < best) e.bn = 0;
	std::lock_guard<std::mutex> g(tt.mu);
	if (const TuneEntry* prev = tt.find(key)) return prev->bn;    // another thread tuned it meanwhile
	tt.entries.push_back(e);
	if (FILE* f = fopen(tt.path.c_str(), "a"))
	{
		fprintf(f, "%s %d %.6f %.6f %.6f %.6f\n", key.c_str(), e.bn, e.ms[0], e.ms[1], e.ms[2], e.ms[3]);
		fclose(f);
	}
	return e.bn;
}

// ------------------------------------------------------------------------------------
// data movement plans
// ------------------------------------------------------------------------------------

void CopyPlan::run(Ctx& c, const double* src, double* dst, bool cplx) const
{
	if (nchunks == 0) return;
	KScope ks(c, kind == 0 ? K_PERMUTE : K_ROWMAP, 1, 0, (cplx ? 32.0 : 16.0) * (double)elements);
	if (kind == 0) launch_permute(nchunks, chunks, (const PermDesc*)descs, src, dst, c.stream(), cplx);
	else launch_rowmap(nchunks, chunks, (const RowDesc*)descs, maps, src, dst, c.stream(), cplx);
}

static CopyPlan upload_copy(Ctx& c, CopyLowering&& l)
{
	CopyPlan p;
	p.out = std::move(l.out);
	p.kind = l.kind;
	Packer pk;
	size_t od = 0;
	if (l.kind == 0) od = pk.add(l.perm);
	else if (l.kind == 1) od = pk.add(l.rows);
	else od = pk.add(l.scale);
	const size_t oc = pk.add(l.chunks), om = pk.add(l.maps);
	if (pk.bytes.size() < 16) pk.bytes.resize(16);
	p.desc = c.upload(pk.bytes.data(), pk.bytes.size());
	p.descs = (const char*)p.desc->ptr + od;
	p.chunks = at<Chunk>(p.desc, oc);
	p.maps = at<i64>(p.desc, om);
	p.nchunks = (int)l.chunks.size();
	p.elements = l.elements;
	return p;
}

// ---- cached entry points ----------------------------------------------------------------

// opt-in diagnostics: with CTGPU_PLAN_DUMP=path every plan that misses the cache is appended to
// that file as (kind, parameters, operand structures), so that the host lowering can be replayed
// and timed without a device
static void dump_plan_request(int kind, const std::vector<i64>& params, const Meta& s, const Meta* t)
{
	static FILE* f = [] {
		const char* path = getenv("CTGPU_PLAN_DUMP");
		return path ? fopen(path, "wb") : nullptr;
	}();
	if (!f) return;
	static std::mutex mu;
	std::lock_guard<std::mutex> lock(mu);
	auto put_sig = [](const Meta& m) {
		const int32_t nd = m.ndim;
		fwrite(&nd, sizeof(nd), 1, f);
		for (int a = 0; a < m.ndim; a++)
		{
			const int32_t dir = m.dir[(size_t)a];
			fwrite(&m.dim[(size_t)a], sizeof(i64), 1, f);
			fwrite(&dir, sizeof(dir), 1, f);
			fwrite(m.ql[(size_t)a].data(), sizeof(q32), m.ql[(size_t)a].size(), f);
		}
	};
	const int32_t head[2] = {kind, (int32_t)params.size()};
	fwrite(head, sizeof(head), 1, f);
	fwrite(params.data(), sizeof(i64), params.size(), f);
	put_sig(s);
	const int32_t has_t = t ? 1 : 0;
	fwrite(&has_t, sizeof(has_t), 1, f);
	if (t) put_sig(*t);
	fflush(f);
}

DotPlan make_dot_plan(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision,
                      const int* out_perm)
{
	PlanTimer plan_timer(c);
	std::vector<i64> params = {axs, axt, nmult, precision};
	if (out_perm)
		for (int i = 0; i < s.ndim + t.ndim - 2 * nmult; i++) params.push_back(out_perm[i]);
	const uint64_t key = plan_key(0, params, s, &t);
	if (const PlanEntry* e = plan_find(c, key, 0, params, s, &t)) return e->dot;
	dump_plan_request(0, params, s, &t);
	PlanEntry e;
	e.kind = 0;
	e.params = params;
	e.s = StructSig(s);
	e.t = StructSig(t);
	e.dot = build_dot_plan(c, s, axs, t, axt, nmult, precision, out_perm);
	const size_t bytes = e.dot.desc ? e.dot.desc->bytes : 0;
	DotPlan p = e.dot;
	plan_insert(c, key, std::move(e), bytes);
	return p;
}

static CopyPlan cached_copy(Ctx& c, int kind, const std::vector<i64>& params, const Meta& t,
                            const std::function<CopyPlan()>& build)
{
	const uint64_t key = plan_key(kind, params, t, nullptr);
	if (const PlanEntry* e = plan_find(c, key, kind, params, t, nullptr)) return e->copy;
	dump_plan_request(kind, params, t, nullptr);
	PlanEntry e;
	e.kind = kind;
	e.params = params;
	e.s = StructSig(t);
	e.copy = build();
	const size_t bytes = e.copy.desc ? e.copy.desc->bytes : 0;
	CopyPlan p = e.copy;
	plan_insert(c, key, std::move(e), bytes);
	return p;
}

CopyPlan make_transpose_plan(Ctx& c, const Meta& t, const int* perm)
{
	PlanTimer plan_timer(c);
	const std::vector<i64> params(perm, perm + t.ndim);
	return cached_copy(c, 1, params, t, [&] { return upload_copy(c, lower_transpose(t, perm)); });
}

CopyPlan make_flatten_plan(Ctx& c, const Meta& t, int ax, int newdir)
{
	PlanTimer plan_timer(c);
	return cached_copy(c, 2, {ax, newdir}, t, [&] { return upload_copy(c, lower_flatten(t, ax, newdir)); });
}

CopyPlan make_split_plan(Ctx& c, const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq)
{
	PlanTimer plan_timer(c);
	std::vector<i64> params = {ax, nd[0], nd[1], ndir[0], ndir[1], nq ? 1 : 0};
	if (nq)
		for (q32 q : *nq) params.push_back(q);
	return cached_copy(c, 3, params, t, [&] { return upload_copy(c, lower_split(t, ax, nd, ndir, nq)); });
}

CopyPlan make_slice_plan(Ctx& c, const Meta& t, int ax, const std::vector<i64>& ind)
{
	PlanTimer plan_timer(c);
	std::vector<i64> params = {ax};
	params.insert(params.end(), ind.begin(), ind.end());
	return cached_copy(c, 4, params, t, [&] { return upload_copy(c, lower_slice(t, ax, ind)); });
}

// ------------------------------------------------------------------------------------
// one-shot operations
// ------------------------------------------------------------------------------------

DTensor op_dot(Ctx& c, const DTensor& s, int axs, const DTensor& t, int axt, int nmult, int precision)
{
	if (s.cplx || t.cplx)
	{
		CTG_CHECK(s.cplx && t.cplx, "dot: real and complex operands");
		DotPlan p = make_dot_plan(c, s.m(), axs, t.m(), axt, nmult, GEMM_Z64);
		DTensor r = c.empty(p.out, true);
		if (p.out->nnz > 0)
			CTG_CUDA(cudaMemsetAsync(r.data(), 0, (size_t)p.out->nnz * 2 * sizeof(double), c.stream()));
		p.run_z(c, s.data(), t.data(), r.data(), s.conj, t.conj);
		return r;
	}
	DotPlan p = make_dot_plan(c, s.m(), axs, t.m(), axt, nmult, precision);
	DTensor r;
	r.meta = p.out;
	r.buf = std::make_shared<DBuf>(&c, (size_t)std::max<i64>(p.out->nnz, 1) * sizeof(double));
	p.run(c, s.data(), t.data(), r.data());
	return r;
}

static DTensor run_copy(Ctx& c, const CopyPlan& p, const DTensor& src)
{
	CTG_CHECK(!src.conj, "copy of a conjugated view");
	DTensor r;
	r.meta = p.out;
	r.cplx = src.cplx;
	r.buf = std::make_shared<DBuf>(&c, (size_t)std::max<i64>(p.out->nnz, 1) * r.width() * sizeof(double));
	p.run(c, src.data(), r.data(), src.cplx);
	return r;
}

DTensor op_transpose(Ctx& c, const DTensor& t, const int* perm)
{
	return run_copy(c, make_transpose_plan(c, t.m(), perm), t);
}

DTensor op_flatten(Ctx& c, const DTensor& t, int ax, int newdir)
{
	return run_copy(c, make_flatten_plan(c, t.m(), ax, newdir), t);
}

DTensor op_split(Ctx& c, const DTensor& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq)
{
	return run_copy(c, make_split_plan(c, t.m(), ax, nd, ndir, nq), t);
}

DTensor op_slice(Ctx& c, const DTensor& t, int ax, const std::vector<i64>& ind)
{
	return run_copy(c, make_slice_plan(c, t.m(), ax, ind), t);
}

DTensor op_scale_axis(Ctx& c, const DTensor& s, const double* dvec, int axrange)
{
	CopyPlan p;
	{
		PlanTimer plan_timer(c);
		p = cached_copy(c, 5, {axrange}, s.m(), [&] { return upload_copy(c, lower_scale(s.m(), axrange)); });
	}
	CTG_CHECK(!s.conj, "scaling of a conjugated view");
	DTensor r = c.empty(s.meta, s.cplx);
	if (p.nchunks > 0)
	{
		KScope ks(c, K_SCALE, 1, 0, 16.0 * s.width() * (double)s.m().nnz);
		launch_scale_axis(p.nchunks, p.chunks, (const ScaleDesc*)p.descs, p.maps, dvec, s.data(), r.data(), c.stream(),
		                  s.cplx);
	}
	return r;
}

DTensor view_reversed(Ctx& c, const DTensor& t)
{
	CopyPlan p;
	{
		PlanTimer plan_timer(c);
		p = cached_copy(c, 6, {}, t.m(), [&] {
			CopyPlan q;
			q.out = std::make_shared<const Meta>(reversed_meta(t.m()));
			return q;
		});
	}
	DTensor r;
	r.meta = p.out;
	r.buf = t.buf;
	r.cplx = t.cplx;
	r.conj = t.conj;
	return r;
}

// block_sparse_tensor_cyclic_partial_trace with ndim_trace = 1 (block_sparse_tensor.c:1560-1611):
// with unit traced dimensions carrying equal quantum numbers and opposite directions, the
// traced tensor has the same blocks in the same order and the same entries
DTensor view_trace_unit(const DTensor& t)
{
	const Meta& m = t.m();
	CTG_CHECK(m.ndim >= 3 && m.dim[0] == 1 && m.dim[m.ndim - 1] == 1, "trace: unit outer dimensions expected");
	CTG_CHECK(m.dir[0] == -m.dir[m.ndim - 1] && m.ql[0] == m.ql[m.ndim - 1], "trace: outer axes must match");
	std::vector<std::vector<q32>> ql(m.ql.begin() + 1, m.ql.end() - 1);
	Meta r = make_meta(m.ndim - 2, m.dim.data() + 1, m.dir.data() + 1, ql);
	CTG_CHECK(r.nnz == m.nnz && r.nblocks == m.nblocks, "trace: unexpected block structure");
	DTensor o;
	o.meta = std::make_shared<const Meta>(std::move(r));
	o.buf = t.buf;
	o.cplx = t.cplx;
	o.conj = t.conj;
	return o;
}

// ------------------------------------------------------------------------------------
// SVD and RQ of block-sparse matrices
// ------------------------------------------------------------------------------------

int op_svd_launch(Ctx& c, const DTensor& a, SvdResult& res, SvdPending& pend, double discard_weight)
{
	const Meta& am = a.m();
	pend = SvdPending();
	pend.a = a;
	CTG_CHECK(am.ndim == 2, "svd: matrix expected");
	// intermediate axis: column quantum numbers (sorted), min(m, n) copies per block
	std::vector<q32> qi;
	struct Blk { int ab; i64 m, n, k; };
	std::vector<Blk> blks;
	for (i64 j = 0; j < am.nb[1]; j++)
		for (i64 i = 0; i < am.nb[0]; i++)
		{
			const i64 idx[2] = {i, j};
			const int b = am.find(idx);
			if (b < 0) continue;
			const i64 m = am.dims(b)[0], n = am.dims(b)[1], k = std::min(m, n);
			for (i64 l = 0; l < k; l++) qi.push_back(am.qb[1][j]);
			blks.push_back(Blk{b, m, n, k});
		}
	bool dummy = false;
	if (qi.empty())
	{
		dummy = true;
		qi.push_back(-am.dir[0] * am.dir[1] * am.qb[0][0]);
	}
	const i64 ni = (i64)qi.size();
	// squared singular values below which every value is discarded by the caller
	const double discard2 = discard_weight > 0 ? discard_weight / (2.0 * (double)ni) : 0.0;
	const i64 du[2] = {am.dim[0], ni};
	Meta mu = make_meta(2, du, am.dir.data(), {am.ql[0], qi});
	const i64 dv[2] = {ni, am.dim[1]};
	const int dirv[2] = {-am.dir[1], am.dir[1]};
	Meta mv = make_meta(2, dv, dirv, {qi, am.ql[1]});
	CTG_CHECK(!a.conj, "svd of a conjugated view");
	res.u = c.zeros(mu, a.cplx);
	res.vh = c.zeros(mv, a.cplx);
	res.ns = ni;
	res.s = std::make_shared<DBuf>(&c, (size_t)ni * sizeof(double));
	CTG_CUDA(cudaMemsetAsync(res.s->ptr, 0, (size_t)ni * sizeof(double), c.stream()));
	if (dummy)
	{
		const i64 idx[2] = {0, (i64)mu.find_q(1, qi[0])};
		const int b = mu.find(idx);
		CTG_CHECK(b >= 0, "svd: dummy block missing");
		static const double one = 1.0;
		CTG_CUDA(cudaMemcpyAsync(res.u.data() + mu.boff[b] * res.u.width(), &one, sizeof(double), cudaMemcpyHostToDevice,
		                         c.stream()));
		return 0;
	}
	if (a.cplx)
	{
		// complex128: one-sided complex Jacobi per block (offsets in complex elements)
		std::vector<SvdDesc> zd;
		i64 zw = 0;
		for (const Blk& bl : blks)
		{
			const i64* ia = am.index(bl.ab);
			const i64 kb = mu.find_q(1, am.qb[1][ia[1]]);
			const i64 iu[2] = {ia[0], kb}, iv[2] = {kb, ia[1]};
			const int bu = mu.find(iu), bv = mv.find(iv);
			CTG_CHECK(bu >= 0 && bv >= 0, "svd: factor blocks missing");
			i64 first = 0;
			while (mu.ql[1][(size_t)first] != am.qb[1][ia[1]]) first++;
			SvdDesc d = {};
			d.a_off = am.boff[bl.ab];
			d.u_off = mu.boff[bu];
			d.v_off = mv.boff[bv];
			d.s_off = first;
			d.w_off = zw;
			d.m = (int)bl.m;
			d.n = (int)bl.n;
			zw += svd_z_scratch(d.m, d.n);
			zd.push_back(d);
		}
		DBufPtr desc = c.upload(zd.data(), zd.size() * sizeof(SvdDesc));
		DBuf scratch(&c, (size_t)std::max<i64>(zw, 1) * 2 * sizeof(double));
		pend.zstatus = std::make_shared<DBuf>(&c, zd.size() * sizeof(int));
		pend.zblocks = (int)zd.size();
		KScope ks(c, K_SVD, 1);
		launch_svd_z((int)zd.size(), (const SvdDesc*)desc->ptr, a.data(), res.u.data(), (double*)res.s->ptr,
		             res.vh.data(), (double*)scratch.ptr, (int*)pend.zstatus->ptr, c.stream());
		return 0;
	}
	std::vector<SvdDesc> descs;
	i64 woff = 0;
	for (const Blk& bl : blks)
	{
		const i64* ia = am.index(bl.ab);
		const i64 kb = mu.find_q(1, am.qb[1][ia[1]]);
		const i64 iu[2] = {ia[0], kb}, iv[2] = {kb, ia[1]};
		const int bu = mu.find(iu), bv = mv.find(iv);
		CTG_CHECK(bu >= 0 && bv >= 0, "svd: factor blocks missing");
		CTG_CHECK(std::min(bl.m, bl.n) <= 4096, "svd: block with more than 4096 singular values");
		i64 first = 0;
		while (mu.ql[1][(size_t)first] != am.qb[1][ia[1]]) first++;
		SvdDesc d = {};
		d.a_off = am.boff[bl.ab];
		d.u_off = mu.boff[bu];
		d.v_off = mv.boff[bv];
		d.s_off = first;
		d.w_off = woff;
		d.m = (int)bl.m;
		d.n = (int)bl.n;
		woff += svd_scratch_doubles(d.m, d.n);
		descs.push_back(d);
	}
	// One cluster per block, sized to the block's share of the Jacobi work (~N^2 (M + N)): the
	// largest block gets the largest cluster, and every other block the smallest power of two
	// that finishes it within about the largest block's time. One launch per configuration,
	// the launches side by side on auxiliary streams.
	const int maxcl = svd_max_cluster(c.device());
	std::vector<double> work(descs.size());
	double wmax = 0;
	for (size_t b = 0; b < descs.size(); b++)
	{
		const double M = std::max(descs[b].m, descs[b].n), N = std::min(descs[b].m, descs[b].n);
		work[b] = N * N * (M + N);
		wmax = std::max(wmax, work[b]);
	}
	int forced = 0;
	if (const char* e = getenv("CTGPU_SVD_CLUSTER")) forced = std::max(1, std::min(maxcl, atoi(e)));
	std::vector<SvdLaunch> cfg(descs.size());
	static const double slack0 = getenv("CTGPU_SVD_SLACK") ? atof(getenv("CTGPU_SVD_SLACK")) : 0.75;
	for (double slack = slack0;; slack *= 2)
	{
		int total = 0;
		for (size_t b = 0; b < descs.size(); b++)
		{
			// at least two columns per column group (four per CTA): below that the cluster barriers
			// of the Jacobi rounds cost more than the extra CTAs save
			const int ncol = std::min(descs[b].m, descs[b].n);
			int want = 1;
			while (want < maxcl && 2 * (2 * (2 * want)) <= ncol && work[b] > slack * wmax / maxcl * want) want *= 2;
			if (forced) want = forced;
			cfg[b] = svd_launch_for(descs[b].m, descs[b].n, want, maxcl);
			total += cfg[b].cluster;
		}
		if (forced || total <= 2 * c.num_sms() || slack > 1e6) break;
	}
	std::vector<int> order(descs.size());
	for (size_t b = 0; b < order.size(); b++) order[b] = (int)b;
	std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
		if (cfg[x].global != cfg[y].global) return cfg[x].global > cfg[y].global;
		return cfg[x].cluster > cfg[y].cluster;
	});
	{
		std::vector<SvdDesc> sorted(descs.size());
		std::vector<SvdLaunch> scfg(descs.size());
		for (size_t b = 0; b < order.size(); b++)
		{
			sorted[b] = descs[(size_t)order[b]];
			scfg[b] = cfg[(size_t)order[b]];
		}
		descs.swap(sorted);
		cfg.swap(scfg);
	}
	struct Group { SvdLaunch l; int first, count; };
	std::vector<Group> groups;
	for (int b = 0; b < (int)descs.size(); b++)
	{
		if (!groups.empty() && groups.back().l.cluster == cfg[b].cluster && groups.back().l.global == cfg[b].global)
		{
			groups.back().count++;
			groups.back().l.smem = std::max(groups.back().l.smem, cfg[b].smem);
		}
		else groups.push_back(Group{cfg[b], b, 1});
	}
	DBufPtr desc = c.upload(descs.data(), descs.size() * sizeof(SvdDesc));
	DBuf scratch(&c, (size_t)std::max<i64>(woff, 1) * sizeof(double));
	DBuf status(&c, 2 * sizeof(int));
	CTG_CUDA(cudaMemsetAsync(status.ptr, 0, 2 * sizeof(int), c.stream()));
	DBuf tail(&c, descs.size() * sizeof(double));     // [0]: executed Jacobi FP64 flops
	CTG_CUDA(cudaMemsetAsync(tail.ptr, 0, descs.size() * sizeof(double), c.stream()));
	// opt-in diagnostics: per-block phase stamps (QR, Jacobi, outputs) of the shared-memory path
	static const bool phases = getenv("CTGPU_SVD_PHASES") != nullptr;
	std::unique_ptr<DBuf> ts;
	if (phases)
	{
		ts.reset(new DBuf(&c, descs.size() * SVD_PHASE_SLOTS * sizeof(unsigned long long)));
		CTG_CUDA(cudaMemsetAsync(ts->ptr, 0, ts->bytes, c.stream()));
	}
	unsigned long long* tsp = ts ? (unsigned long long*)ts->ptr : nullptr;
	{
		KScope ks(c, K_SVD, (int)groups.size());
		const int ng = (int)std::min<size_t>(groups.size(), Ctx::NUM_AUX);
		if (groups.size() == 1)
			launch_svd_group(groups[0].l, groups[0].first, groups[0].count, (const SvdDesc*)desc->ptr, a.data(),
			                 res.u.data(), (double*)res.s->ptr, res.vh.data(), (double*)scratch.ptr, (int*)status.ptr,
			                 (double*)tail.ptr, c.stream(), tsp, discard2);
		else
		{
			c.fork(ng);
			for (size_t g = 0; g < groups.size(); g++)
				launch_svd_group(groups[g].l, groups[g].first, groups[g].count, (const SvdDesc*)desc->ptr, a.data(),
				                 res.u.data(), (double*)res.s->ptr, res.vh.data(), (double*)scratch.ptr,
				                 (int*)status.ptr, (double*)tail.ptr, c.aux((int)g), tsp, discard2);
			c.join(ng);
		}
	}
	if (ts)
	{
		std::vector<unsigned long long> h(descs.size() * SVD_PHASE_SLOTS);
		CTG_CUDA(cudaMemcpyAsync(h.data(), ts->ptr, ts->bytes, cudaMemcpyDeviceToHost, c.stream()));
		c.sync();
		// the block that finished last sets the launch's duration
		size_t crit = 0;
		unsigned long long t0 = ~0ull, t1 = 0;
		for (size_t b = 0; b < descs.size(); b++)
		{
			if (!h[SVD_PHASE_SLOTS * b]) continue;
			t0 = std::min(t0, h[SVD_PHASE_SLOTS * b]);
			if (h[SVD_PHASE_SLOTS * b + 3] > t1) { t1 = h[SVD_PHASE_SLOTS * b + 3]; crit = b; }
		}
		if (t1 > 0)
		{
			c.svd_phase_ms[0] += 1e-6 * (double)(h[SVD_PHASE_SLOTS * crit + 1] - h[SVD_PHASE_SLOTS * crit]);
			c.svd_phase_ms[1] += 1e-6 * (double)(h[SVD_PHASE_SLOTS * crit + 2] - h[SVD_PHASE_SLOTS * crit + 1]);
			c.svd_phase_ms[2] += 1e-6 * (double)(h[SVD_PHASE_SLOTS * crit + 3] - h[SVD_PHASE_SLOTS * crit + 2]);
			c.svd_phase_ms[3] += 1e-6 * (double)(t1 - t0);
			for (int i = 0; i < 6; i++) c.svd_jacobi_cycles[i] += (double)h[SVD_PHASE_SLOTS * crit + 4 + i];
			c.svd_jacobi_cycles[6] += (double)h[SVD_PHASE_SLOTS * crit + 20];
			c.svd_jacobi_cycles[7] += (double)h[SVD_PHASE_SLOTS * crit + 21];
			for (int i = 0; i < 5; i++) c.svd_qr_cycles[i] += (double)h[SVD_PHASE_SLOTS * crit + 10 + i];
			// CTGPU_SVD_PHASES=2: one line per call for the block that finished last
			static const bool each = atoi(getenv("CTGPU_SVD_PHASES")) >= 2;
			if (each)
				fprintf(stderr, "ctgpu: svd call: %zu blocks, critical %d x %d (cluster %d): QR %.3f Jacobi %.3f outputs %.3f ms, FP32 sweeps %llu, FP64 sweeps %llu, refinement %llu (kcycles: gram %llu analysis %llu update %llu clusters %llu)\n",
				        descs.size(), descs[crit].m, descs[crit].n, cfg[crit].cluster,
				        1e-6 * (double)(h[SVD_PHASE_SLOTS * crit + 1] - h[SVD_PHASE_SLOTS * crit]),
				        1e-6 * (double)(h[SVD_PHASE_SLOTS * crit + 2] - h[SVD_PHASE_SLOTS * crit + 1]),
				        1e-6 * (double)(h[SVD_PHASE_SLOTS * crit + 3] - h[SVD_PHASE_SLOTS * crit + 2]),
				        h[SVD_PHASE_SLOTS * crit + 6], h[SVD_PHASE_SLOTS * crit + 5], h[SVD_PHASE_SLOTS * crit + 15],
				        h[SVD_PHASE_SLOTS * crit + 16] / 1000, h[SVD_PHASE_SLOTS * crit + 17] / 1000,
				        h[SVD_PHASE_SLOTS * crit + 18] / 1000, h[SVD_PHASE_SLOTS * crit + 19] / 1000);
		}
	}
	// the status and the flop count reach pinned host memory once the stream gets there (read by
	// op_svd_finish)
	CTG_CUDA(cudaMemcpyAsync(c.svd_status_host(), status.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream()));
	CTG_CUDA(cudaMemcpyAsync(c.svd_flops_host(), tail.ptr, sizeof(double), cudaMemcpyDeviceToHost, c.stream()));
	// Householder QR (2 M N^2 - 2 N^3 / 3) and the reflectors applied to V (~4 M N^2 - 2 N^3) at
	// full rank, counted on the host
	pend.other_flops = 0;
	for (const SvdDesc& d : descs)
	{
		const double M = std::max(d.m, d.n), N = std::min(d.m, d.n);
		pend.other_flops += 2.0 * M * N * N - 2.0 * N * N * N / 3.0 + 4.0 * M * N * N - 2.0 * N * N * N;
	}
	pend.descs = descs;
	pend.launches = groups.size();
	return 0;
}

thread_local int g_inject_svd_failure = 0;
thread_local int g_inject_tridiag_failure = 0;
thread_local int g_inject_zero_start = 0;

int op_svd_finish(Ctx& c, const SvdPending& pend)
{
	if (g_inject_svd_failure > 0)
	{
		// host-side fault injection (tests of the error path): this SVD reports non-convergence
		g_inject_svd_failure--;
		fprintf(stderr, "ctgpu: block SVD did not converge (injected failure)\n");
		return -1;
	}
	if (pend.zblocks > 0)
	{
		std::vector<int> st((size_t)pend.zblocks);
		CTG_CUDA(cudaMemcpy(st.data(), pend.zstatus->ptr, st.size() * sizeof(int), cudaMemcpyDeviceToHost));
		for (int v : st)
			if (v != 0)
			{
				fprintf(stderr, "ctgpu: complex block SVD did not converge\n");
				return -1;
			}
		return 0;
	}
	if (pend.descs.empty()) return 0;
	c.svd_flops += *c.svd_flops_host() + pend.other_flops;
	const int* hst = c.svd_status_host();
	c.svd_max_sweeps = std::max(c.svd_max_sweeps, hst[1]);
	if (hst[0] == 0) return 0;
	int mmax = 0, nmax = 0;
	for (const SvdDesc& d : pend.descs) { mmax = std::max(mmax, d.m); nmax = std::max(nmax, d.n); }
	fprintf(stderr, "ctgpu: block SVD did not converge within %d Jacobi sweeps (%zu blocks, largest %d x %d, %zu launches)\n",
	        SVD_MAX_SWEEPS, pend.descs.size(), mmax, nmax, pend.launches);
	// opt-in diagnostics: write the input matrix (row-major blocks) for offline analysis
	if (const char* path = getenv("CTGPU_SVD_DUMP"))
	{
		std::vector<double> host((size_t)pend.a.m().nnz);
		copy_to_host(c, pend.a, host.data());
		if (FILE* f = fopen(path, "wb"))
		{
			const i64 nb = (i64)pend.descs.size();
			fwrite(&nb, sizeof(i64), 1, f);
			for (const SvdDesc& d : pend.descs)
			{
				const i64 mn[2] = {d.m, d.n};
				fwrite(mn, sizeof(i64), 2, f);
				fwrite(host.data() + d.a_off, sizeof(double), (size_t)d.m * d.n, f);
			}
			fclose(f);
		}
	}
	return -1;
}

int op_svd(Ctx& c, const DTensor& a, SvdResult& res)
{
	SvdPending pend;
	const int ret = op_svd_launch(c, a, res, pend);
	if (ret < 0) return ret;
	c.sync();
	return op_svd_finish(c, pend);
}

int op_rq(Ctx& c, const DTensor& a, DTensor& r, DTensor& q)
{
	const Meta& am = a.m();
	CTG_CHECK(am.ndim == 2, "rq: matrix expected");
	std::vector<q32> qi;
	struct Blk { int ab; i64 m, n, k; };
	std::vector<Blk> blks;
	for (i64 i = 0; i < am.nb[0]; i++)
		for (i64 j = 0; j < am.nb[1]; j++)
		{
			const i64 idx[2] = {i, j};
			const int b = am.find(idx);
			if (b < 0) continue;
			const i64 m = am.dims(b)[0], n = am.dims(b)[1], k = std::min(m, n);
			for (i64 l = 0; l < k; l++) qi.push_back(am.qb[0][i]);
			blks.push_back(Blk{b, m, n, k});
		}
	bool dummy = false;
	if (qi.empty())
	{
		dummy = true;
		qi.push_back(-am.dir[0] * am.dir[1] * am.qb[1][0]);
	}
	const i64 ni = (i64)qi.size();
	const i64 dr[2] = {am.dim[0], ni};
	const int dirr[2] = {am.dir[0], -am.dir[0]};
	Meta mr = make_meta(2, dr, dirr, {am.ql[0], qi});
	const i64 dq[2] = {ni, am.dim[1]};
	Meta mq = make_meta(2, dq, am.dir.data(), {qi, am.ql[1]});
	CTG_CHECK(!a.conj, "rq of a conjugated view");
	r = c.zeros(mr, a.cplx);
	q = c.zeros(mq, a.cplx);
	if (dummy)
	{
		const i64 idx[2] = {(i64)mq.find_q(0, qi[0]), 0};
		const int b = mq.find(idx);
		CTG_CHECK(b >= 0, "rq: dummy block missing");
		static const double one = 1.0;
		CTG_CUDA(cudaMemcpyAsync(q.data() + mq.boff[b] * q.width(), &one, sizeof(double), cudaMemcpyHostToDevice, c.stream()));
		c.sync();
		return 0;
	}
	std::vector<RqDesc> descs;
	i64 woff = 0;
	for (const Blk& bl : blks)
	{
		const i64* ia = am.index(bl.ab);
		const i64 kb = mq.find_q(0, am.qb[0][ia[0]]);
		const i64 ir[2] = {ia[0], kb}, iq[2] = {kb, ia[1]};
		const int br = mr.find(ir), bq = mq.find(iq);
		CTG_CHECK(br >= 0 && bq >= 0, "rq: factor blocks missing");
		RqDesc d = {};
		d.a_off = am.boff[bl.ab];
		d.r_off = mr.boff[br];
		d.q_off = mq.boff[bq];
		d.w_off = woff;
		d.m = (int)bl.m;
		d.n = (int)bl.n;
		d.qr = 0;
		woff += bl.n * bl.m + bl.n * bl.k + bl.k;
		descs.push_back(d);
	}
	DBufPtr desc = c.upload(descs.data(), descs.size() * sizeof(RqDesc));
	DBuf scratch(&c, (size_t)std::max<i64>(woff, 1) * a.width() * sizeof(double));
	KScope ks(c, K_RQ, 1);
	if (a.cplx)
		launch_qr_z((int)descs.size(), (const RqDesc*)desc->ptr, a.data(), r.data(), q.data(), (double*)scratch.ptr, c.stream());
	else
		launch_rq_householder((int)descs.size(), (const RqDesc*)desc->ptr, a.data(), r.data(), q.data(), (double*)scratch.ptr,
		                      c.stream());
	return 0;
}

int op_qr(Ctx& c, const DTensor& a, DTensor& q, DTensor& r)
{
	const Meta& am = a.m();
	CTG_CHECK(am.ndim == 2, "qr: matrix expected");
	std::vector<q32> qi;
	struct Blk { int ab; i64 m, n, k; };
	std::vector<Blk> blks;
	// column blocks outer: the intermediate quantum numbers come out sorted
	for (i64 j = 0; j < am.nb[1]; j++)
		for (i64 i = 0; i < am.nb[0]; i++)
		{
			const i64 idx[2] = {i, j};
			const int b = am.find(idx);
			if (b < 0) continue;
			const i64 m = am.dims(b)[0], n = am.dims(b)[1], k = std::min(m, n);
			for (i64 l = 0; l < k; l++) qi.push_back(am.qb[1][j]);
			blks.push_back(Blk{b, m, n, k});
		}
	bool dummy = false;
	if (qi.empty())
	{
		dummy = true;
		qi.push_back(-am.dir[0] * am.dir[1] * am.qb[0][0]);
	}
	const i64 ni = (i64)qi.size();
	const i64 dq[2] = {am.dim[0], ni};
	Meta mq = make_meta(2, dq, am.dir.data(), {am.ql[0], qi});
	const i64 dr[2] = {ni, am.dim[1]};
	const int dirr[2] = {-am.dir[1], am.dir[1]};
	Meta mr = make_meta(2, dr, dirr, {qi, am.ql[1]});
	CTG_CHECK(!a.conj, "qr of a conjugated view");
	q = c.zeros(mq, a.cplx);
	r = c.zeros(mr, a.cplx);
	if (dummy)
	{
		const i64 idx[2] = {0, (i64)mq.find_q(1, qi[0])};
		const int b = mq.find(idx);
		CTG_CHECK(b >= 0, "qr: dummy block missing");
		static const double one = 1.0;
		CTG_CUDA(cudaMemcpyAsync(q.data() + mq.boff[b] * q.width(), &one, sizeof(double), cudaMemcpyHostToDevice, c.stream()));
		c.sync();
		return 0;
	}
	std::vector<RqDesc> descs;
	i64 woff = 0;
	for (const Blk& bl : blks)
	{
		const i64* ia = am.index(bl.ab);
		const i64 kb = mq.find_q(1, am.qb[1][ia[1]]);
		const i64 iq[2] = {ia[0], kb}, ir[2] = {kb, ia[1]};
		const int bq = mq.find(iq), br = mr.find(ir);
		CTG_CHECK(br >= 0 && bq >= 0, "qr: factor blocks missing");
		RqDesc d = {};
		d.a_off = am.boff[bl.ab];
		d.r_off = mr.boff[br];
		d.q_off = mq.boff[bq];
		d.w_off = woff;
		d.m = (int)bl.m;
		d.n = (int)bl.n;
		d.qr = 1;
		woff += bl.m * bl.n + bl.m * bl.k + bl.k;
		descs.push_back(d);
	}
	DBufPtr desc = c.upload(descs.data(), descs.size() * sizeof(RqDesc));
	DBuf scratch(&c, (size_t)std::max<i64>(woff, 1) * a.width() * sizeof(double));
	KScope ks(c, K_RQ, 1);
	if (a.cplx)
		launch_qr_z((int)descs.size(), (const RqDesc*)desc->ptr, a.data(), r.data(), q.data(), (double*)scratch.ptr, c.stream());
	else
		launch_rq_householder((int)descs.size(), (const RqDesc*)desc->ptr, a.data(), r.data(), q.data(), (double*)scratch.ptr,
		                      c.stream());
	return 0;
}

}  // namespace ctg
