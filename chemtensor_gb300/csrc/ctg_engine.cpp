// ctg_engine.cpp - lowering of block-sparse tensor operations to device work lists.
#include "ctg_engine.h"

#include <algorithm>
#include <cmath>
#include <chrono>
#include <functional>
#include <memory>
#include <cstring>
#include <ctime>

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

// host time of plan-building stages (diagnostics): 0 dot meta, 1 dot enumeration, 2 split-K,
// 3 dot packing, 4 transpose meta, 5 transpose loop, 6 flatten meta, 7 flatten loop, 8 split meta,
// 9 split loop, 10 slice, 11 other
double g_plan_stage[12];

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

DTensor Ctx::empty(const Meta& m)
{
	DTensor t;
	t.meta = std::make_shared<const Meta>(m);
	t.buf = std::make_shared<DBuf>(this, (size_t)std::max<i64>(m.nnz, 1) * sizeof(double));
	return t;
}

DTensor Ctx::empty(const std::shared_ptr<const Meta>& m)
{
	DTensor t;
	t.meta = m;
	t.buf = std::make_shared<DBuf>(this, (size_t)std::max<i64>(m->nnz, 1) * sizeof(double));
	return t;
}

DTensor Ctx::zeros(const Meta& m)
{
	DTensor t = empty(m);
	CTG_CUDA(cudaMemsetAsync(t.data(), 0, (size_t)std::max<i64>(m.nnz, 1) * sizeof(double), st_));
	return t;
}

void copy_to_device(Ctx& c, DTensor& t, const double* host)
{
	if (t.m().nnz == 0) return;
	DBufPtr b = c.upload(host, (size_t)t.m().nnz * sizeof(double));
	t.buf = b;
}

void copy_to_host(Ctx& c, const DTensor& t, double* host)
{
	if (t.m().nnz == 0) return;
	CTG_CUDA(cudaMemcpyAsync(host, t.data(), (size_t)t.m().nnz * sizeof(double), cudaMemcpyDeviceToHost, c.stream()));
	c.sync();
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

i64 prod(const i64* d, int n)
{
	i64 p = 1;
	for (int i = 0; i < n; i++) p *= d[i];
	return p;
}

void add_chunks(std::vector<Chunk>& chunks, int desc, i64 n)
{
	for (i64 s = 0; s < n; s += COPY_CHUNK) chunks.push_back(Chunk{desc, 0, s});
}

// logical indices carrying quantum number q on an axis, in order
std::vector<i64> fanout(const Meta& t, int ax, q32 q)
{
	std::vector<i64> f;
	for (i64 j = 0; j < t.dim[ax]; j++)
		if (t.ql[ax][(size_t)j] == q) f.push_back(j);
	return f;
}

int tile_class(int m, int n)
{
	// the tile that pads the block least (FP64 FMAs on padding cost as much as useful ones)
	if (m <= 16 && n <= 16) return TILE_S;
	if (m <= 16) return TILE_W;
	if (n <= 16) return TILE_T;
	if (m <= 32 || n <= 32) return TILE_M;
	return TILE_L;
}

}  // namespace

// ------------------------------------------------------------------------------------
// dot (block_sparse_tensor.c:1826-2001; dense_tensor.c:1761-1837)
// ------------------------------------------------------------------------------------

static DotPlan build_dot_plan(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision)
{
	DotPlan p;
	double ts0 = host_seconds();
	auto out = std::make_shared<Meta>(dot_result_meta(s, axs, t, axt, nmult));
	p.out = out;
	g_plan_stage[0] += host_seconds() - ts0;
	ts0 = host_seconds();
	const Meta& r = *out;
	const int shift_s = (axs == AX_LEADING ? 0 : s.ndim - nmult);
	const int shift_t = (axt == AX_LEADING ? 0 : t.ndim - nmult);
	const int off_s = (axs == AX_LEADING ? nmult : 0);
	const int off_t = (axt == AX_LEADING ? nmult : 0);
	const int nfs = s.ndim - nmult, nft = t.ndim - nmult;
	const int nlds = (axs == AX_LEADING ? nmult : s.ndim - nmult);
	const int nldt = (axt == AX_LEADING ? nmult : t.ndim - nmult);

	std::vector<GemmOut> outs(r.nblocks);
	std::vector<GemmContrib> cons;
	std::vector<std::pair<int, int>> con_blocks;   // (s block, t block) of every contribution
	std::vector<GemmTile> tiles[NUM_TILE_CLASSES];
	// contracted block indices: all combinations over the first nmult - 1 contracted axes; the
	// last one is fixed by the conservation law of s
	i64 ncontract = 1;
	for (int i = 0; i < nmult - 1; i++) ncontract *= t.nb[shift_t + i];
	const int lc = shift_s + nmult - 1;          // last contracted axis of s
	std::vector<i64> is(s.ndim), it(t.ndim), ic(nmult);
	double flops = 0;
	for (int b = 0; b < r.nblocks; b++)
	{
		const i64* ir = r.index(b);
		const i64* rd = r.dims(b);
		GemmOut& o = outs[b];
		o.c_off = r.boff[b];
		o.m = (int)prod(rd, nfs);
		o.n = (int)prod(rd + nfs, nft);
		o.c0 = (int)cons.size();
		long long qfree = 0;
		for (int i = 0; i < nfs; i++) qfree += (long long)s.dir[off_s + i] * s.qb[off_s + i][ir[i]];
		for (i64 mm = 0; mm < ncontract; mm++)
		{
			i64 rem = mm;
			long long qsum = qfree;
			for (int i = nmult - 2; i >= 0; i--)
			{
				ic[i] = rem % t.nb[shift_t + i];
				rem /= t.nb[shift_t + i];
				qsum += (long long)s.dir[shift_s + i] * s.qb[shift_s + i][ic[i]];
			}
			const long long qneed = -(long long)s.dir[lc] * qsum;
			if (qneed < INT32_MIN || qneed > INT32_MAX) continue;
			const int jl = s.find_q(lc, (q32)qneed);
			if (jl < 0) continue;
			ic[nmult - 1] = jl;
			for (int i = 0; i < nfs; i++) is[off_s + i] = ir[i];
			for (int i = 0; i < nmult; i++) is[shift_s + i] = ic[i];
			const int bs = s.find(is.data());
			if (bs < 0) continue;
			for (int i = 0; i < nft; i++) it[off_t + i] = ir[nfs + i];
			for (int i = 0; i < nmult; i++) it[shift_t + i] = ic[i];
			const int bt = t.find(it.data());
			CTG_CHECK(bt >= 0, "dot: missing partner block");
			const i64* sd = s.dims(bs);
			const i64* td = t.dims(bt);
			const i64 lds = prod(sd, nlds), tds = prod(sd + nlds, s.ndim - nlds);
			const i64 ldt = prod(td, nldt), tdt = prod(td + nldt, t.ndim - nldt);
			GemmContrib g;
			g.a_off = s.boff[bs];
			g.b_off = t.boff[bt];
			const i64 k = (axs == AX_LEADING ? lds : tds);
			g.k = (int)k;
			if (axs == AX_LEADING) { g.sAm = 1; g.sAk = (int)tds; }
			else { g.sAm = (int)tds; g.sAk = 1; }
			if (axt == AX_LEADING) { g.sBk = (int)tdt; g.sBn = 1; }
			else { g.sBk = 1; g.sBn = (int)tdt; }
			CTG_CHECK(k == (axt == AX_LEADING ? ldt : tdt), "dot: inner dimensions differ");
			// every operand access stays inside its block (checked once per plan, on the host)
			CTG_CHECK(k >= 1 && g.a_off + (i64)(o.m - 1) * g.sAm + (k - 1) * g.sAk < s.boff[bs] + s.block_size(bs),
			          "dot: A operand out of range");
			CTG_CHECK(g.b_off + (k - 1) * g.sBk + (i64)(o.n - 1) * g.sBn < t.boff[bt] + t.block_size(bt),
			          "dot: B operand out of range");
			cons.push_back(g);
			con_blocks.emplace_back(bs, bt);
			flops += 2.0 * (double)o.m * (double)o.n * (double)k;
			p.flops_cls[tile_class(o.m, o.n)] += 2.0 * (double)o.m * (double)o.n * (double)k;
		}
		o.nc = (int)cons.size() - o.c0;
		CTG_CHECK(o.m >= 1 && o.n >= 1 && o.c_off + (i64)o.m * o.n <= r.nnz, "dot: output block out of range");
		// every tile first takes the whole sum over the block's contributions
		GemmTile whole = {};
		whole.out = b;
		whole.c0 = o.c0;
		whole.k0 = 0;
		whole.c1 = o.c0 + o.nc - 1;
		whole.k1 = o.nc > 0 ? cons[(size_t)whole.c1].k : 0;
		whole.part = -1;
		if (precision == GEMM_BF16X3)
		{
			// tensor-core tiles: one tile class
			for (int m0 = 0; m0 < o.m; m0 += tc_tile_rows())
				for (int n0 = 0; n0 < o.n; n0 += tc_tile_cols())
				{
					whole.m0 = m0;
					whole.n0 = n0;
					tiles[0].push_back(whole);
				}
			continue;
		}
		const int cls = tile_class(o.m, o.n);
		const int tr = tile_rows(cls), tc = tile_cols(cls);
		whole.cls = cls;
		for (int m0 = 0; m0 < o.m; m0 += tr)
			for (int n0 = 0; n0 < o.n; n0 += tc)
			{
				whole.m0 = m0;
				whole.n0 = n0;
				tiles[cls].push_back(whole);
			}
	}
	// Split-K: on GB300 one SM retires about two FP64 FMAs per clock, so a block GEMM with fewer
	// tiles than SMs leaves most of the FP64 pipes idle. Tiles whose work exceeds a fair share of
	// the whole product are cut into shares of consecutive 16-wide k chunks, one CTA each; their
	// partial sums are added in a fixed order (deterministic) by k_gemm_reduce.
	g_plan_stage[1] += host_seconds() - ts0;
	ts0 = host_seconds();
	std::vector<GemmSplit> splits;
	i64 wsz = 0;
	if (precision != GEMM_BF16X3)
	{
		constexpr int KCH = 16;                  // k chunk of the FP64 kernels
		auto nchunks = [&](const GemmOut& o) {
			i64 n = 0;
			for (int cc = o.c0; cc < o.c0 + o.nc; cc++) n += (cons[(size_t)cc].k + KCH - 1) / KCH;
			return n;
		};
		double total = 0;
		for (int k = 0; k < NUM_TILE_CLASSES; k++)
			for (const GemmTile& t : tiles[k])
				total += (double)tile_rows(k) * tile_cols(k) * (double)(nchunks(outs[(size_t)t.out]) * KCH);
		const double target = std::max(total / (2.0 * c.num_sms()), 65536.0);
		std::vector<std::pair<int, int>> pos;
		for (int k = 0; k < NUM_TILE_CLASSES; k++)
		{
			std::vector<GemmTile> kept;
			const int tr = tile_rows(k), tc = tile_cols(k);
			for (const GemmTile& t : tiles[k])
			{
				const GemmOut& o = outs[(size_t)t.out];
				const i64 n = nchunks(o);
				const double w = (double)tr * tc * (double)(n * KCH);
				const int S = (int)std::min<double>((double)n, std::ceil(w / target));
				if (S <= 1)
				{
					kept.push_back(t);
					continue;
				}
				pos.clear();
				for (int cc = o.c0; cc < o.c0 + o.nc; cc++)
					for (int kk = 0; kk < cons[(size_t)cc].k; kk += KCH) pos.emplace_back(cc, kk);
				for (int sp = 0; sp < S; sp++)
				{
					const i64 a = sp * n / S, e = (sp + 1) * n / S;
					GemmTile u = t;
					u.c0 = pos[(size_t)a].first;
					u.k0 = pos[(size_t)a].second;
					u.c1 = pos[(size_t)e - 1].first;
					u.k1 = std::min(pos[(size_t)e - 1].second + KCH, cons[(size_t)u.c1].k);
					u.part = wsz + (i64)sp * tr * tc;
					kept.push_back(u);
				}
				GemmSplit g = {};
				g.out = t.out;
				g.m0 = t.m0;
				g.n0 = t.n0;
				g.rows = std::min(tr, o.m - t.m0);
				g.cols = std::min(tc, o.n - t.n0);
				g.nsplit = S;
				g.ld = tc;
				g.stride = tr * tc;
				g.part = wsz;
				splits.push_back(g);
				wsz += (i64)S * tr * tc;
			}
			tiles[k].swap(kept);
		}
	}
	// tensor-core operands: one set of packed tile records per operand block, shared by every
	// contribution that uses the block
	std::vector<TcContrib> tcons;
	std::vector<TcPack> apacks, bpacks;
	if (precision == GEMM_BF16X3)
	{
		std::unordered_map<int, i64> abase, bbase;
		tcons.resize(cons.size());
		for (size_t ci = 0; ci < cons.size(); ci++)
		{
			const GemmContrib& g = cons[ci];
			const int bs = con_blocks[ci].first, bt = con_blocks[ci].second;
			const int kt = (g.k + TC_K - 1) / TC_K;
			// rows of the A view of block bs and of the B view of block bt
			const i64* sd = s.dims(bs);
			const i64* td = t.dims(bt);
			const int am = (int)prod(sd + (axs == AX_LEADING ? nmult : 0), s.ndim - nmult);
			const int bn = (int)prod(td + (axt == AX_LEADING ? nmult : 0), t.ndim - nmult);
			auto ia = abase.find(bs);
			if (ia == abase.end())
			{
				const i64 base = (i64)apacks.size();
				const int mtiles = (am + TC_A_ROWS - 1) / TC_A_ROWS;
				for (int mt = 0; mt < mtiles; mt++)
					for (int j = 0; j < kt; j++)
						apacks.push_back(TcPack{g.a_off, am, g.k, g.sAm, g.sAk, mt * TC_A_ROWS, j * TC_K, base + mt * kt + j});
				ia = abase.emplace(bs, base).first;
			}
			auto ib = bbase.find(bt);
			if (ib == bbase.end())
			{
				const i64 base = (i64)bpacks.size();
				const int ntiles_b = (bn + TC_B_ROWS - 1) / TC_B_ROWS;
				for (int nt = 0; nt < ntiles_b; nt++)
					for (int j = 0; j < kt; j++)
						bpacks.push_back(TcPack{g.b_off, bn, g.k, g.sBn, g.sBk, nt * TC_B_ROWS, j * TC_K, base + nt * kt + j});
				ib = bbase.emplace(bt, base).first;
			}
			tcons[ci] = TcContrib{ia->second, ib->second, kt, 0};
		}
	}
	g_plan_stage[2] += host_seconds() - ts0;
	ts0 = host_seconds();
	p.precision = precision;
	if (precision == GEMM_BF16X3)
	{
		for (int k = 1; k < NUM_TILE_CLASSES; k++) p.flops_cls[0] += p.flops_cls[k], p.flops_cls[k] = 0;
	}
	// one launch covers every class: all tiles in one list
	for (int k = 1; k < NUM_TILE_CLASSES; k++)
	{
		tiles[0].insert(tiles[0].end(), tiles[k].begin(), tiles[k].end());
		tiles[k].clear();
	}
	Packer pk;
	const size_t o_outs = pk.add(outs);
	const size_t o_cons = pk.add(cons);
	size_t o_tiles[NUM_TILE_CLASSES];
	for (int k = 0; k < NUM_TILE_CLASSES; k++) o_tiles[k] = pk.add(tiles[k]);
	const size_t o_splits = pk.add(splits);
	const size_t o_tcons = pk.add(tcons), o_apacks = pk.add(apacks), o_bpacks = pk.add(bpacks);
	p.desc = c.upload(pk.bytes.data(), std::max<size_t>(pk.bytes.size(), 16));
	p.tcons = at<TcContrib>(p.desc, o_tcons);
	p.apacks = at<TcPack>(p.desc, o_apacks);
	p.bpacks = at<TcPack>(p.desc, o_bpacks);
	p.a_recs = (i64)apacks.size();
	p.b_recs = (i64)bpacks.size();
	p.outs = at<GemmOut>(p.desc, o_outs);
	p.cons = at<GemmContrib>(p.desc, o_cons);
	p.splits = at<GemmSplit>(p.desc, o_splits);
	p.nsplits = (int)splits.size();
	if (wsz > 0) p.work = std::make_shared<DBuf>(&c, (size_t)wsz * sizeof(double));
	for (int k = 0; k < NUM_TILE_CLASSES; k++)
	{
		p.ntiles[k] = (int)tiles[k].size();
		p.tiles[k] = at<GemmTile>(p.desc, o_tiles[k]);
	}
	p.flops = flops;
	p.a_entries = s.nnz;
	p.b_entries = t.nnz;
	g_plan_stage[3] += host_seconds() - ts0;
	return p;
}

void DotPlan::run(Ctx& c, const double* A, const double* B, double* C) const
{
	if (precision == GEMM_BF16X3)
	{
		if (ntiles[0] > 0)
		{
			DBuf apk(&c, (size_t)std::max<i64>(a_recs, 1) * TC_A_REC_BYTES);
			DBuf bpk(&c, (size_t)std::max<i64>(b_recs, 1) * TC_B_REC_BYTES);
			pack_a(c, A, apk.ptr);
			pack_b(c, B, bpk.ptr);
			run_packed(c, apk.ptr, bpk.ptr, C);
		}
		c.gemm_flops += flops;
		return;
	}
	double* w = work ? (double*)work->ptr : nullptr;
	if (ntiles[0] > 0)
	{
		KScope ks(c, K_GEMM, 1, flops, 0);
		launch_gemm_f64(ntiles[0], tiles[0], outs, cons, A, B, C, w, c.stream());
	}
	if (nsplits > 0)
	{
		KScope ks(c, K_GEMM, 1, 0, 0);
		launch_gemm_reduce(nsplits, splits, outs, w, C, c.stream());
	}
	c.gemm_flops += flops;
}

void DotPlan::pack_a(Ctx& c, const double* A, void* apack) const
{
	KScope ks(c, K_GEMM_TC, 1, 0, 8.0 * (double)a_entries + (double)a_recs * TC_A_REC_BYTES);
	launch_tc_pack((int)a_recs, apacks, 1, A, apack, c.stream());
}

void DotPlan::pack_b(Ctx& c, const double* B, void* bpack) const
{
	KScope ks(c, K_GEMM_TC, 1, 0, 8.0 * (double)b_entries + (double)b_recs * TC_B_REC_BYTES);
	launch_tc_pack((int)b_recs, bpacks, 0, B, bpack, c.stream());
}

void DotPlan::run_packed(Ctx& c, const void* apack, const void* bpack, double* C) const
{
	if (ntiles[0] > 0)
	{
		KScope ks(c, K_GEMM_TC, 1, flops_cls[0], 0);
		launch_gemm_tc(ntiles[0], tiles[0], outs, tcons, apack, bpack, C, c.tc_error(), c.stream());
	}
}

// ------------------------------------------------------------------------------------
// data movement plans
// ------------------------------------------------------------------------------------

void CopyPlan::run(Ctx& c, const double* src, double* dst) const
{
	if (nchunks == 0) return;
	KScope ks(c, kind == 0 ? K_PERMUTE : K_ROWMAP, 1, 0, 16.0 * (double)elements);
	if (kind == 0) launch_permute(nchunks, chunks, (const PermDesc*)descs, src, dst, c.stream());
	else launch_rowmap(nchunks, chunks, (const RowDesc*)descs, maps, src, dst, c.stream());
}

static CopyPlan finish_perm(Ctx& c, std::shared_ptr<Meta> out, const std::vector<PermDesc>& d, const std::vector<Chunk>& ch)
{
	CopyPlan p;
	p.out = out;
	p.kind = 0;
	Packer pk;
	const size_t od = pk.add(d), oc = pk.add(ch);
	p.desc = c.upload(pk.bytes.data(), std::max<size_t>(pk.bytes.size(), 16));
	p.descs = at<PermDesc>(p.desc, od);
	p.chunks = at<Chunk>(p.desc, oc);
	p.nchunks = (int)ch.size();
	p.elements = out->nnz;
	return p;
}

static void check_rows(const std::vector<RowDesc>& descs, const std::vector<i64>& maps, i64 src_nnz, i64 dst_nnz)
{
	for (const RowDesc& d : descs)
	{
		CTG_CHECK(d.map_off + d.nrow <= (i64)maps.size(), "row map: table out of range");
		const int mrows = d.scatter ? d.dst_rows : d.src_rows;
		for (int j = 0; j < d.nrow; j++)
			CTG_CHECK(maps[(size_t)(d.map_off + j)] >= 0 && maps[(size_t)(d.map_off + j)] < mrows, "row map: entry out of range");
		CTG_CHECK(d.src_off + d.nlead * d.src_rows * d.ntrail <= src_nnz, "row map: source out of range");
		CTG_CHECK(d.dst_off + d.nlead * d.dst_rows * d.ntrail <= dst_nnz, "row map: destination out of range");
		CTG_CHECK(d.scatter ? d.nrow <= d.src_rows : d.nrow <= d.dst_rows, "row map: row count out of range");
	}
}

static CopyPlan finish_rows(Ctx& c, std::shared_ptr<Meta> out, const std::vector<RowDesc>& d, const std::vector<Chunk>& ch,
                            const std::vector<i64>& maps)
{
	CopyPlan p;
	p.out = out;
	p.kind = 1;
	Packer pk;
	const size_t od = pk.add(d), oc = pk.add(ch), om = pk.add(maps);
	p.desc = c.upload(pk.bytes.data(), std::max<size_t>(pk.bytes.size(), 16));
	p.descs = at<RowDesc>(p.desc, od);
	p.chunks = at<Chunk>(p.desc, oc);
	p.maps = at<i64>(p.desc, om);
	p.nchunks = (int)ch.size();
	p.elements = out->nnz;
	return p;
}

// block_sparse_tensor_transpose (block_sparse_tensor.c:785-870)
static CopyPlan build_transpose_plan(Ctx& c, const Meta& t, const int* perm)
{
	double ts0 = host_seconds();
	auto out = std::make_shared<Meta>(transpose_meta(t, perm));
	g_plan_stage[4] += host_seconds() - ts0;
	ts0 = host_seconds();
	const Meta& r = *out;
	CTG_CHECK(t.ndim <= 6, "transpose: at most 6 axes");
	std::vector<PermDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> ir(t.ndim);
	for (int b = 0; b < t.nblocks; b++)
	{
		const i64* it = t.index(b);
		const i64* td = t.dims(b);
		for (int i = 0; i < t.ndim; i++) ir[i] = it[perm[i]];
		const int rb = r.find(ir.data());
		CTG_CHECK(rb >= 0, "transpose: missing block");
		i64 st[8];
		st[t.ndim - 1] = 1;
		for (int i = t.ndim - 2; i >= 0; i--) st[i] = st[i + 1] * td[i + 1];
		PermDesc d = {};
		d.src_off = t.boff[b];
		d.dst_off = r.boff[rb];
		d.n = t.block_size(b);
		d.ndim = t.ndim;
		for (int i = 0; i < t.ndim; i++) { d.dims[i] = (int)td[perm[i]]; d.sstr[i] = st[perm[i]]; }
		i64 smax = 0;
		for (int i = 0; i < t.ndim; i++) smax += (i64)(d.dims[i] - 1) * d.sstr[i];
		CTG_CHECK(d.src_off + smax < t.nnz && d.dst_off + d.n <= r.nnz, "transpose: descriptor out of range");
		add_chunks(chunks, (int)descs.size(), d.n);
		descs.push_back(d);
	}
	g_plan_stage[5] += host_seconds() - ts0;
	return finish_perm(c, out, descs, chunks);
}

// block_sparse_tensor_flatten_axes (block_sparse_tensor.c:950-1112): each source block
// scatters its rows (j0, j1) into the fused rows of one target block
static CopyPlan build_flatten_plan(Ctx& c, const Meta& t, int ax, int newdir)
{
	double ts0 = host_seconds();
	auto out = std::make_shared<Meta>(flatten_meta(t, ax, newdir));
	g_plan_stage[6] += host_seconds() - ts0;
	ts0 = host_seconds();
	const Meta& r = *out;
	const i64 d1 = t.dim[ax + 1];
	std::vector<RowDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	std::vector<i64> ir(r.ndim);
	for (int b = 0; b < t.nblocks; b++)
	{
		const i64* it = t.index(b);
		const i64* td = t.dims(b);
		const q32 q0 = t.qb[ax][it[ax]], q1 = t.qb[ax + 1][it[ax + 1]];
		const q32 qf = newdir * (t.dir[ax] * q0 + t.dir[ax + 1] * q1);
		for (int i = 0; i < ax; i++) ir[i] = it[i];
		ir[ax] = r.find_q(ax, qf);
		for (int i = ax + 2; i < t.ndim; i++) ir[i - 1] = it[i];
		const int rb = r.find(ir.data());
		CTG_CHECK(rb >= 0, "flatten: missing target block");
		const auto f0 = fanout(t, ax, q0), f1 = fanout(t, ax + 1, q1);
		RowDesc d = {};
		d.src_off = t.boff[b];
		d.dst_off = r.boff[rb];
		d.nlead = prod(td, ax);
		d.ntrail = prod(td + ax + 2, t.ndim - ax - 2);
		d.nrow = (int)(td[ax] * td[ax + 1]);
		d.src_rows = d.nrow;
		d.dst_rows = (int)r.dims(rb)[ax];
		d.scatter = 1;
		d.map_off = (i64)maps.size();
		for (size_t j0 = 0; j0 < f0.size(); j0++)
			for (size_t j1 = 0; j1 < f1.size(); j1++) maps.push_back(r.pos[ax][(size_t)(f0[j0] * d1 + f1[j1])]);
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nrow * d.ntrail);
		descs.push_back(d);
	}
	check_rows(descs, maps, t.nnz, r.nnz);
	g_plan_stage[7] += host_seconds() - ts0;
	return finish_rows(c, out, descs, chunks, maps);
}

// block_sparse_tensor_split_axis (block_sparse_tensor.c:1123-1285): each target block
// gathers its rows (j0, j1) from the fused rows of one source block
static CopyPlan build_split_plan(Ctx& c, const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq)
{
	double ts0 = host_seconds();
	auto out = std::make_shared<Meta>(split_meta(t, ax, nd, ndir, nq));
	g_plan_stage[8] += host_seconds() - ts0;
	ts0 = host_seconds();
	const Meta& r = *out;
	std::vector<RowDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	std::vector<i64> it(t.ndim);
	for (int b = 0; b < r.nblocks; b++)
	{
		const i64* ir = r.index(b);
		const i64* rd = r.dims(b);
		const q32 q0 = r.qb[ax][ir[ax]], q1 = r.qb[ax + 1][ir[ax + 1]];
		const q32 qf = t.dir[ax] * (r.dir[ax] * q0 + r.dir[ax + 1] * q1);
		for (int i = 0; i < ax; i++) it[i] = ir[i];
		it[ax] = t.find_q(ax, qf);
		for (int i = ax + 1; i < t.ndim; i++) it[i] = ir[i + 1];
		const int tb = t.find(it.data());
		CTG_CHECK(tb >= 0, "split: missing source block");
		const auto f0 = fanout(r, ax, q0), f1 = fanout(r, ax + 1, q1);
		RowDesc d = {};
		d.src_off = t.boff[tb];
		d.dst_off = r.boff[b];
		d.nlead = prod(rd, ax);
		d.ntrail = prod(rd + ax + 2, r.ndim - ax - 2);
		d.nrow = (int)(rd[ax] * rd[ax + 1]);
		d.dst_rows = d.nrow;
		d.src_rows = (int)t.dims(tb)[ax];
		d.scatter = 0;
		d.map_off = (i64)maps.size();
		for (size_t j0 = 0; j0 < f0.size(); j0++)
			for (size_t j1 = 0; j1 < f1.size(); j1++) maps.push_back(t.pos[ax][(size_t)(f0[j0] * nd[1] + f1[j1])]);
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nrow * d.ntrail);
		descs.push_back(d);
	}
	check_rows(descs, maps, t.nnz, r.nnz);
	g_plan_stage[9] += host_seconds() - ts0;
	return finish_rows(c, out, descs, chunks, maps);
}

// block_sparse_tensor_slice (block_sparse_tensor.c:1446-1553)
static CopyPlan build_slice_plan(Ctx& c, const Meta& t, int ax, const std::vector<i64>& ind)
{
	auto out = std::make_shared<Meta>(slice_meta(t, ax, ind));
	const Meta& r = *out;
	std::vector<RowDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	std::vector<i64> it(t.ndim);
	for (int b = 0; b < r.nblocks; b++)
	{
		const i64* ir = r.index(b);
		const i64* rd = r.dims(b);
		const q32 qn = r.qb[ax][ir[ax]];
		for (int i = 0; i < t.ndim; i++) it[i] = ir[i];
		it[ax] = t.find_q(ax, qn);
		const int tb = t.find(it.data());
		CTG_CHECK(tb >= 0, "slice: missing source block");
		const auto fr = fanout(r, ax, qn);
		RowDesc d = {};
		d.src_off = t.boff[tb];
		d.dst_off = r.boff[b];
		d.nlead = prod(rd, ax);
		d.ntrail = prod(rd + ax + 1, r.ndim - ax - 1);
		d.nrow = (int)rd[ax];
		d.dst_rows = d.nrow;
		d.src_rows = (int)t.dims(tb)[ax];
		d.scatter = 0;
		d.map_off = (i64)maps.size();
		for (size_t j = 0; j < fr.size(); j++) maps.push_back(t.pos[ax][(size_t)ind[(size_t)fr[j]]]);
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nrow * d.ntrail);
		descs.push_back(d);
	}
	check_rows(descs, maps, t.nnz, r.nnz);
	return finish_rows(c, out, descs, chunks, maps);
}


// ---- cached entry points ----------------------------------------------------------------

DotPlan make_dot_plan(Ctx& c, const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision)
{
	PlanTimer plan_timer(c);
	const std::vector<i64> params = {axs, axt, nmult, precision};
	const uint64_t key = plan_key(0, params, s, &t);
	if (const PlanEntry* e = plan_find(c, key, 0, params, s, &t)) return e->dot;
	PlanEntry e;
	e.kind = 0;
	e.params = params;
	e.s = StructSig(s);
	e.t = StructSig(t);
	e.dot = build_dot_plan(c, s, axs, t, axt, nmult, precision);
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
	return cached_copy(c, 1, params, t, [&] { return build_transpose_plan(c, t, perm); });
}

CopyPlan make_flatten_plan(Ctx& c, const Meta& t, int ax, int newdir)
{
	PlanTimer plan_timer(c);
	return cached_copy(c, 2, {ax, newdir}, t, [&] { return build_flatten_plan(c, t, ax, newdir); });
}

CopyPlan make_split_plan(Ctx& c, const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq)
{
	PlanTimer plan_timer(c);
	std::vector<i64> params = {ax, nd[0], nd[1], ndir[0], ndir[1], nq ? 1 : 0};
	if (nq)
		for (q32 q : *nq) params.push_back(q);
	return cached_copy(c, 3, params, t, [&] { return build_split_plan(c, t, ax, nd, ndir, nq); });
}

CopyPlan make_slice_plan(Ctx& c, const Meta& t, int ax, const std::vector<i64>& ind)
{
	PlanTimer plan_timer(c);
	std::vector<i64> params = {ax};
	params.insert(params.end(), ind.begin(), ind.end());
	return cached_copy(c, 4, params, t, [&] { return build_slice_plan(c, t, ax, ind); });
}

// ------------------------------------------------------------------------------------
// one-shot operations
// ------------------------------------------------------------------------------------

DTensor op_dot(Ctx& c, const DTensor& s, int axs, const DTensor& t, int axt, int nmult, int precision)
{
	DotPlan p = make_dot_plan(c, s.m(), axs, t.m(), axt, nmult, precision);
	DTensor r;
	r.meta = p.out;
	r.buf = std::make_shared<DBuf>(&c, (size_t)std::max<i64>(p.out->nnz, 1) * sizeof(double));
	p.run(c, s.data(), t.data(), r.data());
	return r;
}

static DTensor run_copy(Ctx& c, const CopyPlan& p, const DTensor& src)
{
	DTensor r;
	r.meta = p.out;
	r.buf = std::make_shared<DBuf>(&c, (size_t)std::max<i64>(p.out->nnz, 1) * sizeof(double));
	p.run(c, src.data(), r.data());
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

// block_sparse_tensor_multiply_pointwise_vector (block_sparse_tensor.c:1654-1703)
static CopyPlan build_scale_plan(Ctx& c, const Meta& m, int axrange)
{
	const int ax = (axrange == AX_LEADING ? 0 : m.ndim - 1);
	std::vector<ScaleDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	for (int b = 0; b < m.nblocks; b++)
	{
		const i64* ib = m.index(b);
		const i64* bd = m.dims(b);
		const auto f = fanout(m, ax, m.qb[ax][ib[ax]]);
		ScaleDesc d = {};
		d.off = m.boff[b];
		d.nlead = prod(bd, ax);
		d.nax = (int)bd[ax];
		d.ntrail = prod(bd + ax + 1, m.ndim - ax - 1);
		d.map_off = (i64)maps.size();
		maps.insert(maps.end(), f.begin(), f.end());
		CTG_CHECK((i64)f.size() == d.nax && d.off + d.nlead * d.nax * d.ntrail <= m.nnz, "scale: descriptor out of range");
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nax * d.ntrail);
		descs.push_back(d);
	}
	Packer pk;
	const size_t od = pk.add(descs), oc = pk.add(chunks), om = pk.add(maps);
	CopyPlan p;
	p.kind = 2;
	p.desc = c.upload(pk.bytes.data(), std::max<size_t>(pk.bytes.size(), 16));
	p.descs = at<ScaleDesc>(p.desc, od);
	p.chunks = at<Chunk>(p.desc, oc);
	p.maps = at<i64>(p.desc, om);
	p.nchunks = (int)chunks.size();
	p.elements = m.nnz;
	return p;
}

DTensor op_scale_axis(Ctx& c, const DTensor& s, const double* dvec, int axrange)
{
	CopyPlan p;
	{
		PlanTimer plan_timer(c);
		p = cached_copy(c, 5, {axrange}, s.m(), [&] { return build_scale_plan(c, s.m(), axrange); });
	}
	DTensor r = c.empty(s.meta);
	if (p.nchunks > 0)
	{
		KScope ks(c, K_SCALE, 1, 0, 16.0 * (double)s.m().nnz);
		launch_scale_axis(p.nchunks, p.chunks, (const ScaleDesc*)p.descs, p.maps, dvec, s.data(), r.data(), c.stream());
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
	return o;
}

// ------------------------------------------------------------------------------------
// SVD and RQ of block-sparse matrices
// ------------------------------------------------------------------------------------

int op_svd_launch(Ctx& c, const DTensor& a, SvdResult& res, SvdPending& pend)
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
	const i64 du[2] = {am.dim[0], ni};
	Meta mu = make_meta(2, du, am.dir.data(), {am.ql[0], qi});
	const i64 dv[2] = {ni, am.dim[1]};
	const int dirv[2] = {-am.dir[1], am.dir[1]};
	Meta mv = make_meta(2, dv, dirv, {qi, am.ql[1]});
	res.u = c.zeros(mu);
	res.vh = c.zeros(mv);
	res.ns = ni;
	res.s = std::make_shared<DBuf>(&c, (size_t)ni * sizeof(double));
	CTG_CUDA(cudaMemsetAsync(res.s->ptr, 0, (size_t)ni * sizeof(double), c.stream()));
	if (dummy)
	{
		const i64 idx[2] = {0, (i64)mu.find_q(1, qi[0])};
		const int b = mu.find(idx);
		CTG_CHECK(b >= 0, "svd: dummy block missing");
		static const double one = 1.0;
		CTG_CUDA(cudaMemcpyAsync(res.u.data() + mu.boff[b], &one, sizeof(double), cudaMemcpyHostToDevice, c.stream()));
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
	for (double slack = 1.5;; slack *= 2)
	{
		int total = 0;
		for (size_t b = 0; b < descs.size(); b++)
		{
			int want = 1;
			while (want < maxcl && work[b] > slack * wmax / maxcl * want) want *= 2;
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
		ts.reset(new DBuf(&c, descs.size() * 8 * sizeof(unsigned long long)));
		CTG_CUDA(cudaMemsetAsync(ts->ptr, 0, ts->bytes, c.stream()));
	}
	unsigned long long* tsp = ts ? (unsigned long long*)ts->ptr : nullptr;
	{
		KScope ks(c, K_SVD, (int)groups.size());
		const int ng = (int)std::min<size_t>(groups.size(), Ctx::NUM_AUX);
		if (groups.size() == 1)
			launch_svd_group(groups[0].l, groups[0].first, groups[0].count, (const SvdDesc*)desc->ptr, a.data(),
			                 res.u.data(), (double*)res.s->ptr, res.vh.data(), (double*)scratch.ptr, (int*)status.ptr,
			                 (double*)tail.ptr, c.stream(), tsp);
		else
		{
			c.fork(ng);
			for (size_t g = 0; g < groups.size(); g++)
				launch_svd_group(groups[g].l, groups[g].first, groups[g].count, (const SvdDesc*)desc->ptr, a.data(),
				                 res.u.data(), (double*)res.s->ptr, res.vh.data(), (double*)scratch.ptr,
				                 (int*)status.ptr, (double*)tail.ptr, c.aux((int)g), tsp);
			c.join(ng);
		}
	}
	if (ts)
	{
		std::vector<unsigned long long> h(descs.size() * 8);
		CTG_CUDA(cudaMemcpyAsync(h.data(), ts->ptr, ts->bytes, cudaMemcpyDeviceToHost, c.stream()));
		c.sync();
		// the block that finished last sets the launch's duration
		size_t crit = 0;
		unsigned long long t0 = ~0ull, t1 = 0;
		for (size_t b = 0; b < descs.size(); b++)
		{
			if (!h[8 * b]) continue;
			t0 = std::min(t0, h[8 * b]);
			if (h[8 * b + 3] > t1) { t1 = h[8 * b + 3]; crit = b; }
		}
		if (t1 > 0)
		{
			c.svd_phase_ms[0] += 1e-6 * (double)(h[8 * crit + 1] - h[8 * crit]);
			c.svd_phase_ms[1] += 1e-6 * (double)(h[8 * crit + 2] - h[8 * crit + 1]);
			c.svd_phase_ms[2] += 1e-6 * (double)(h[8 * crit + 3] - h[8 * crit + 2]);
			c.svd_phase_ms[3] += 1e-6 * (double)(t1 - t0);
			for (int i = 0; i < 4; i++) c.svd_jacobi_cycles[i] += (double)h[8 * crit + 4 + i];
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

int op_svd_finish(Ctx& c, const SvdPending& pend)
{
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
	r = c.zeros(mr);
	q = c.zeros(mq);
	if (dummy)
	{
		const i64 idx[2] = {(i64)mq.find_q(0, qi[0]), 0};
		const int b = mq.find(idx);
		CTG_CHECK(b >= 0, "rq: dummy block missing");
		static const double one = 1.0;
		CTG_CUDA(cudaMemcpyAsync(q.data() + mq.boff[b], &one, sizeof(double), cudaMemcpyHostToDevice, c.stream()));
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
		woff += bl.n * bl.m + bl.n * bl.k + bl.k;
		descs.push_back(d);
	}
	DBufPtr desc = c.upload(descs.data(), descs.size() * sizeof(RqDesc));
	DBuf scratch(&c, (size_t)std::max<i64>(woff, 1) * sizeof(double));
	KScope ks(c, K_RQ, 1);
	launch_rq_householder((int)descs.size(), (const RqDesc*)desc->ptr, a.data(), r.data(), q.data(), (double*)scratch.ptr,
	                      c.stream());
	return 0;
}

}  // namespace ctg
