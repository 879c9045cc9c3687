// ctg_plan.cpp - lowering of block-sparse operations into descriptor lists (host only).
#include "ctg_plan.h"
#include "ctg_pool.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <unordered_map>

namespace ctg {

thread_local double g_plan_stage[12];

namespace {

double host_seconds()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
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

// logical indices of an axis grouped by block, each group in increasing order (a CSR list over
// the axis' quantum-number blocks, built once per lowering instead of one scan per block)
struct AxisFan {
	std::vector<i64> start, idx;
	AxisFan(const Meta& t, int ax) : start((size_t)t.nb[ax] + 1, 0), idx((size_t)t.dim[ax])
	{
		const std::vector<int>& blk = t.blk[ax];
		const std::vector<i64>& pos = t.pos[ax];
		for (size_t j = 0; j < blk.size(); j++) start[(size_t)blk[j] + 1]++;
		for (size_t b = 1; b < start.size(); b++) start[b] += start[b - 1];
		for (size_t j = 0; j < blk.size(); j++) idx[(size_t)(start[(size_t)blk[j]] + pos[j])] = (i64)j;
	}
	const i64* of(i64 b) const { return idx.data() + start[(size_t)b]; }
	i64 count(i64 b) const { return start[(size_t)b + 1] - start[(size_t)b]; }
};

int tile_class(int m, int n, bool allow_large)
{
	// the tile shape with the fewest padded outputs, counting 128 outputs of fixed cost per tile;
	// 64 x 64 tiles only in products large enough to fill every SM with them (one such tile holds
	// 65536 FMAs per 16-wide k chunk, a long serial share when the whole product is small)
	// tile sides are powers of two: ceilings by shifts
	static const int lr[NUM_TILE_CLASSES] = {4, 5, 6, 4, 6, 3, 2, 5, 6, 3, 7};
	static const int lc[NUM_TILE_CLASSES] = {4, 5, 6, 6, 4, 5, 6, 3, 2, 7, 3};
	int best = TILE_S;
	i64 best_cost = INT64_MAX;
	for (int c = 0; c < NUM_TILE_CLASSES; c++)
	{
		if (c == TILE_L && !allow_large) continue;
		const i64 cost = (i64)(((m - 1) >> lr[c]) + 1) * (((n - 1) >> lc[c]) + 1) * ((1 << (lr[c] + lc[c])) + 128);
		if (cost < best_cost)
		{
			best_cost = cost;
			best = c;
		}
	}
	return best;
}

void check_rows(const std::vector<RowDesc>& descs, const std::vector<i64>& maps, i64 src_nnz, i64 dst_nnz)
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


CopyLowering perm_lowering(std::shared_ptr<Meta> out, std::vector<PermDesc>&& d, std::vector<Chunk>&& ch)
{
	CopyLowering p;
	p.kind = 0;
	p.elements = out->nnz;
	p.out = std::move(out);
	p.perm = std::move(d);
	p.chunks = std::move(ch);
	return p;
}

CopyLowering rows_lowering(std::shared_ptr<Meta> out, std::vector<RowDesc>&& d, std::vector<Chunk>&& ch, std::vector<i64>&& maps)
{
	CopyLowering p;
	p.kind = 1;
	p.elements = out->nnz;
	p.out = std::move(out);
	p.rows = std::move(d);
	p.chunks = std::move(ch);
	p.maps = std::move(maps);
	return p;
}

}  // namespace


// ------------------------------------------------------------------------------------
// dot (block_sparse_tensor.c:1826-2001; dense_tensor.c:1761-1837)
// ------------------------------------------------------------------------------------

DotLowering lower_dot(const Meta& s, int axs, const Meta& t, int axt, int nmult, int precision, int num_sms,
                      const int* out_perm, int tc_bn)
{
	CTG_CHECK(!is_tc_precision(precision) || tc_bn == 64 || tc_bn == 128 || tc_bn == 256,
	          "dot: tensor-core tile width must be 64, 128 or 256");
	DotLowering p;
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
	// Operand blocks keyed by (free part, contracted part), both row-major linear indices over the
	// block grid, and sorted: the blocks with one free index form a run ordered by contracted
	// index. The contracted axes carry the same quantum numbers in both operands, so their block
	// indices agree, and by the conservation law the runs of the two free parts of an output
	// block hold the same contracted indices. Its contributions come from joining the runs, in
	// increasing contracted index (the order of the reference's loop over contracted blocks).
	struct Key { i64 f, c; int b; };
	auto keyed = [nmult](const Meta& m, int shift, int off, int nfree) {
		std::vector<Key> v((size_t)m.nblocks);
		for (int b = 0; b < m.nblocks; b++)
		{
			const i64* ib = m.index(b);
			i64 f = 0, cc = 0;
			for (int i = 0; i < nfree; i++) f = f * m.nb[off + i] + ib[off + i];
			for (int i = 0; i < nmult; i++) cc = cc * m.nb[shift + i] + ib[shift + i];
			v[(size_t)b] = Key{f, cc, b};
		}
		auto less = [](const Key& x, const Key& y) { return x.f < y.f || (x.f == y.f && x.c < y.c); };
		if (!std::is_sorted(v.begin(), v.end(), less))
		{
			// The blocks are in row-major order over all axes, so within one free index the
			// contracted indices already increase: a stable sort by the free index alone gives the
			// (free, contracted) order. LSD radix sort on the free index, 8 bits per pass.
			i64 fmax = 0;
			for (const Key& x : v) fmax = std::max(fmax, x.f);
			std::vector<Key> tmp(v.size());
			for (int shift = 0; shift < 64 && (fmax >> shift) > 0; shift += 8)
			{
				size_t cnt[257] = {0};
				for (const Key& x : v) cnt[((x.f >> shift) & 255) + 1]++;
				for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
				for (const Key& x : v) tmp[cnt[(x.f >> shift) & 255]++] = x;
				v.swap(tmp);
			}
		}
		return v;
	};
	const std::vector<Key> ks = keyed(s, shift_s, off_s, nfs), kt = keyed(t, shift_t, off_t, nft);
	auto run_of = [](const std::vector<Key>& v, i64 f, size_t& lo, size_t& hi) {
		lo = (size_t)(std::lower_bound(v.begin(), v.end(), f, [](const Key& x, i64 y) { return x.f < y; }) - v.begin());
		hi = lo;
		while (hi < v.size() && v[hi].f == f) hi++;
	};
	// operand geometry per block, once: rows of the leading and trailing axis groups, entries
	auto geometry = [](const Meta& m, int nld, std::vector<i64>& lead, std::vector<i64>& trail) {
		lead.resize((size_t)m.nblocks);
		trail.resize((size_t)m.nblocks);
		for (int b = 0; b < m.nblocks; b++)
		{
			const i64* d = m.dims(b);
			lead[(size_t)b] = prod(d, nld);
			trail[(size_t)b] = prod(d + nld, m.ndim - nld);
		}
	};
	std::vector<i64> s_lead, s_trail, t_lead, t_trail;
	geometry(s, nlds, s_lead, s_trail);
	geometry(t, nldt, t_lead, t_trail);
	constexpr int KCH = 16;                      // k chunk of the FP64 kernels
	std::vector<i64> nchunk((size_t)r.nblocks, 0), ksum((size_t)r.nblocks, 0);
	// The output blocks are cut into ranges lowered side by side on the host threads (each range
	// into its own lists, joined in range order afterwards, so the plan does not depend on the
	// number of threads); small products stay on the calling thread.
	const int nrange = r.nblocks >= 4096 ? std::min(4 * host_threads(), std::max(1, r.nblocks / 1024)) : 1;
	struct Range {
		std::vector<GemmContrib> cons;
		std::vector<std::pair<int, int>> con_blocks;
		std::vector<GemmTile> tiles[NUM_TILE_CLASSES];
		double flops = 0, flops_cls[NUM_TILE_CLASSES] = {};
	};
	std::vector<Range> rng((size_t)nrange);
	auto range_of = [&](int q, int& b0, int& b1) {
		b0 = (int)((i64)r.nblocks * q / nrange);
		b1 = (int)((i64)r.nblocks * (q + 1) / nrange);
	};
	parallel_for(nrange, [&](int q) {
		int b0, b1;
		range_of(q, b0, b1);
		Range& R = rng[(size_t)q];
		R.cons.reserve((size_t)(b1 - b0) * 2);
		i64 fs_prev = -1;
		size_t s0 = 0, s1 = 0, tcur = 0;
		for (int b = b0; b < b1; b++)
		{
			const i64* ir = r.index(b);
			const i64* rd = r.dims(b);
			GemmOut& o = outs[b];
			o.c_off = r.boff[b];
			o.m = (int)prod(rd, nfs);
			o.n = (int)prod(rd + nfs, nft);
			o.r1 = o.m;
			o.sr0 = 0;
			o.sr1 = o.n;
			o.c1 = o.n;
			o.sc0 = 0;
			o.c0 = (int)R.cons.size();             // range-local until the join
			i64 fs = 0, ft = 0;
			for (int i = 0; i < nfs; i++) fs = fs * r.nb[i] + ir[i];
			for (int i = 0; i < nft; i++) ft = ft * r.nb[nfs + i] + ir[nfs + i];
			// output blocks come in row-major order: the s run changes only with fs, and within one
			// fs the t free indices increase, so the t runs are found by a forward scan
			if (fs != fs_prev)
			{
				run_of(ks, fs, s0, s1);
				fs_prev = fs;
				tcur = (size_t)(std::lower_bound(kt.begin(), kt.end(), ft, [](const Key& x, i64 y) { return x.f < y; }) -
				                kt.begin());
			}
			while (tcur < kt.size() && kt[tcur].f < ft) tcur++;
			const size_t t0 = tcur;
			size_t t1 = t0;
			while (t1 < kt.size() && kt[t1].f == ft) t1++;
			CTG_CHECK(s1 - s0 == t1 - t0, "dot: operand block runs differ");
			const double mn2 = 2.0 * (double)o.m * (double)o.n;
			i64 nch = 0;
			for (size_t x = s0, y = t0; x < s1; x++, y++)
			{
				CTG_CHECK(ks[x].c == kt[y].c, "dot: missing partner block");
				const int bs = ks[x].b, bt = kt[y].b;
				const i64 lds = s_lead[(size_t)bs], tds = s_trail[(size_t)bs];
				const i64 ldt = t_lead[(size_t)bt], tdt = t_trail[(size_t)bt];
				GemmContrib g = {};
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
				CTG_CHECK(k >= 1 && g.a_off + (i64)(o.m - 1) * g.sAm + (k - 1) * g.sAk < s.boff[bs] + lds * tds,
				          "dot: A operand out of range");
				CTG_CHECK(g.b_off + (k - 1) * g.sBk + (i64)(o.n - 1) * g.sBn < t.boff[bt] + ldt * tdt,
				          "dot: B operand out of range");
				R.cons.push_back(g);
				if (is_tc_precision(precision)) R.con_blocks.emplace_back(bs, bt);
				R.flops += mn2 * (double)k;
				ksum[(size_t)b] += k;
				nch += (k + KCH - 1) / KCH;
			}
			nchunk[(size_t)b] = nch;
			o.nc = (int)R.cons.size() - o.c0;
			CTG_CHECK(o.m >= 1 && o.n >= 1 && o.c_off + (i64)o.m * o.n <= r.nnz, "dot: output block out of range");
		}
	});
	// join the contribution lists; the output blocks' contribution ranges become global
	double flops = 0;
	{
		size_t ncons = 0;
		for (const Range& R : rng) ncons += R.cons.size();
		if (nrange == 1)
		{
			cons.swap(rng[0].cons);
			con_blocks.swap(rng[0].con_blocks);
			flops = rng[0].flops;
		}
		else cons.reserve(ncons);
		for (int q = 0; q < nrange && nrange > 1; q++)
		{
			Range& R = rng[(size_t)q];
			int b0, b1;
			range_of(q, b0, b1);
			const int base = (int)cons.size();
			for (int b = b0; b < b1; b++) outs[(size_t)b].c0 += base;
			cons.insert(cons.end(), R.cons.begin(), R.cons.end());
			con_blocks.insert(con_blocks.end(), R.con_blocks.begin(), R.con_blocks.end());
			flops += R.flops;
			std::vector<GemmContrib>().swap(R.cons);
		}
	}
	// tiles: every tile first takes the whole sum over its output block's contributions; the FP64
	// tile class of every output block first, so that each class list is allocated once
	const bool allow_large = flops / 2 > (double)num_sms * 8 * 65536;
	std::vector<unsigned char> ocls(is_tc_precision(precision) ? 0 : (size_t)r.nblocks);
	parallel_for(nrange, [&](int q) {
		int b0, b1;
		range_of(q, b0, b1);
		Range& R = rng[(size_t)q];
		if (!is_tc_precision(precision))
		{
			size_t cnt[NUM_TILE_CLASSES] = {};
			for (int b = b0; b < b1; b++)
			{
				const GemmOut& o = outs[(size_t)b];
				const int cls = tile_class(o.m, o.n, allow_large);
				ocls[(size_t)b] = (unsigned char)cls;
				cnt[cls] += (size_t)((o.m + TILE_ROWS[cls] - 1) / TILE_ROWS[cls]) * ((o.n + TILE_COLS[cls] - 1) / TILE_COLS[cls]);
			}
			for (int k = 0; k < NUM_TILE_CLASSES; k++) R.tiles[k].reserve(cnt[k]);
		}
		for (int b = b0; b < b1; b++)
		{
			const GemmOut& o = outs[(size_t)b];
			GemmTile whole = {};
			whole.out = b;
			whole.c0 = o.c0;
			whole.k0 = 0;
			whole.c1 = o.c0 + o.nc - 1;
			whole.k1 = o.nc > 0 ? cons[(size_t)whole.c1].k : 0;
			whole.split = -1;
			whole.sp = 0;
			if (is_tc_precision(precision))
			{
				// tensor-core tiles: one tile class, tc_bn columns wide; the row tiles of one column range
				// are consecutive, so that the CTAs running them side by side share its B operand in L2
				R.flops_cls[0] += 2.0 * (double)o.m * (double)o.n * (double)ksum[(size_t)b];
				for (int n0 = 0; n0 < o.n; n0 += tc_bn)
					for (int m0 = 0; m0 < o.m; m0 += tc_tile_rows())
					{
						whole.m0 = m0;
						whole.n0 = n0;
						R.tiles[0].push_back(whole);
					}
				continue;
			}
			const int cls = ocls[(size_t)b];
			R.flops_cls[cls] += 2.0 * (double)o.m * (double)o.n * (double)ksum[(size_t)b];
			const int tr = TILE_ROWS[cls], tc = TILE_COLS[cls];
			whole.cls = cls;
			std::vector<GemmTile>& tl = R.tiles[cls];
			for (int m0 = 0; m0 < o.m; m0 += tr)
				for (int n0 = 0; n0 < o.n; n0 += tc)
				{
					whole.m0 = m0;
					whole.n0 = n0;
					tl.push_back(whole);
				}
		}
	});
	for (int k = 0; k < NUM_TILE_CLASSES; k++)
	{
		if (nrange == 1)
		{
			tiles[k].swap(rng[0].tiles[k]);
			p.flops_cls[k] += rng[0].flops_cls[k];
			continue;
		}
		size_t nt = 0;
		for (const Range& R : rng) nt += R.tiles[k].size();
		tiles[k].reserve(nt);
		for (const Range& R : rng)
		{
			tiles[k].insert(tiles[k].end(), R.tiles[k].begin(), R.tiles[k].end());
			p.flops_cls[k] += R.flops_cls[k];
		}
	}
	// Result written in a transposed layout (see GemmOut). The row axes are cut into two runs
	// [0, x) and [x, nfs), the column axes into [nfs, nfs + y) and [nfs + y, nd); the permutation
	// must arrange these runs (each kept in order) with the last column run innermost. Then every
	// entry's position is i_hi sr0 + i_lo sr1 + j_hi sc0 + j_lo.
	if (out_perm)
	{
		const int nd = r.ndim;
		int cut_x = -1, cut_y = -1;
		int order[4] = {0, 0, 0, 0}, ngroups = 0;       // groups in new order: 0 R_hi, 1 R_lo, 2 C_hi, 3 C_lo
		for (int x = 0; x <= nfs && cut_x < 0; x++)
			for (int y = 0; y <= nft && cut_x < 0; y++)
			{
				const int lo[4] = {0, x, nfs, nfs + y}, hi[4] = {x, nfs, nfs + y, nd};
				int pos = 0, ng = 0, ord[4];
				bool ok = true;
				while (pos < nd && ok)
				{
					int g = -1;
					for (int q = 0; q < 4; q++)
						if (hi[q] > lo[q] && out_perm[pos] == lo[q]) g = q;
					if (g < 0) { ok = false; break; }
					for (int e = lo[g]; e < hi[g] && ok; e++, pos++) ok = pos < nd && out_perm[pos] == e;
					ord[ng++] = g;
				}
				// the last column run, if any, must be innermost
				if (ok && hi[3] > lo[3] && ord[ng - 1] != 3) ok = false;
				if (ok)
				{
					cut_x = x;
					cut_y = y;
					ngroups = ng;
					for (int q = 0; q < ng; q++) order[q] = ord[q];
				}
			}
		CTG_CHECK(cut_x >= 0, "dot: unsupported output permutation");
		std::vector<int> dst_of_src;
		auto outp = std::make_shared<Meta>(transpose_meta(r, out_perm, &dst_of_src));
		for (int b = 0; b < r.nblocks; b++)
		{
			const i64* d = r.dims(b);
			const int bp = dst_of_src[(size_t)b];
			CTG_CHECK(bp >= 0, "dot: missing block of the transposed result");
			const i64 size[4] = {prod(d, cut_x), prod(d + cut_x, nfs - cut_x), prod(d + nfs, cut_y),
			                     prod(d + nfs + cut_y, nft - cut_y)};
			i64 stride[4] = {0, 0, 0, 0}, st = 1;
			for (int q = ngroups - 1; q >= 0; q--)
			{
				stride[order[q]] = st;
				st *= size[order[q]];
			}
			GemmOut& o = outs[(size_t)b];
			o.c_off = outp->boff[bp];
			o.r1 = (int)size[1];
			o.sr0 = stride[0];
			o.sr1 = stride[1];
			o.c1 = (int)size[3];
			o.sc0 = stride[2];
			CTG_CHECK(size[3] == 1 || stride[3] == 1, "dot: output layout");
			CTG_CHECK(o.c_off + (i64)o.m * o.n <= outp->nnz, "dot: transposed output block out of range");
		}
		p.out = outp;
	}
	// Split-K: on GB300 one SM retires about two FP64 FMAs per clock, so a block GEMM with fewer
	// tiles than SMs leaves most of the FP64 pipes idle. Tiles whose work exceeds a fair share of
	// the whole product are cut into shares of consecutive 16-wide k chunks, one CTA each; their
	// partial sums are added in a fixed order (deterministic) by the CTA that completes the split last.
	g_plan_stage[1] += host_seconds() - ts0;
	ts0 = host_seconds();
	std::vector<GemmSplit> splits;
	i64 wsz = 0;
	if (!is_tc_precision(precision))
	{
		double total = 0;
		for (int k = 0; k < NUM_TILE_CLASSES; k++)
			for (const GemmTile& t : tiles[k])
				total += (double)TILE_ROWS[k] * TILE_COLS[k] * (double)(nchunk[(size_t)t.out] * KCH);
		const double target = std::max(total / (2.0 * num_sms), 16384.0);
		std::vector<std::pair<int, int>> pos;
		for (int k = 0; k < NUM_TILE_CLASSES; k++)
		{
			std::vector<GemmTile> kept;
			const int tr = TILE_ROWS[k], tc = TILE_COLS[k];
			for (const GemmTile& t : tiles[k])
			{
				const GemmOut& o = outs[(size_t)t.out];
				const i64 n = nchunk[(size_t)t.out];
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
					u.split = (int)splits.size();
					u.sp = sp;
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
	if (is_tc_precision(precision))
	{
		const int KC = tc_k_chunk(tc_format_of(precision));
		// first record of each operand block's packed tiles (-1: not packed yet)
		std::vector<i64> abase((size_t)s.nblocks, -1), bbase((size_t)t.nblocks, -1);
		tcons.resize(cons.size());
		for (size_t ci = 0; ci < cons.size(); ci++)
		{
			const GemmContrib& g = cons[ci];
			const int bs = con_blocks[ci].first, bt = con_blocks[ci].second;
			const int kt = (g.k + KC - 1) / KC;
			// rows of the A view of block bs and of the B view of block bt
			const i64* sd = s.dims(bs);
			const i64* td = t.dims(bt);
			const int am = (int)prod(sd + (axs == AX_LEADING ? nmult : 0), s.ndim - nmult);
			const int bn = (int)prod(td + (axt == AX_LEADING ? nmult : 0), t.ndim - nmult);
			if (abase[(size_t)bs] < 0)
			{
				const i64 base = (i64)apacks.size();
				const int mtiles = (am + TC_A_ROWS - 1) / TC_A_ROWS;
				for (int mt = 0; mt < mtiles; mt++)
					for (int j = 0; j < kt; j++)
						apacks.push_back(TcPack{g.a_off, am, g.k, g.sAm, g.sAk, mt * TC_A_ROWS, j * KC, base + mt * kt + j});
				abase[(size_t)bs] = base;
			}
			if (bbase[(size_t)bt] < 0)
			{
				const i64 base = (i64)bpacks.size();
				// whole tile widths: a tile's columns are tc_bn / 64 consecutive row records
				const int ntiles_b = (bn + tc_bn - 1) / tc_bn * (tc_bn / TC_B_ROWS);
				for (int nt = 0; nt < ntiles_b; nt++)
					for (int j = 0; j < kt; j++)
						bpacks.push_back(TcPack{g.b_off, bn, g.k, g.sBn, g.sBk, nt * TC_B_ROWS, j * KC, base + nt * kt + j});
				bbase[(size_t)bt] = base;
			}
			tcons[ci] = TcContrib{abase[(size_t)bs], bbase[(size_t)bt], kt, 0};
		}
	}
	g_plan_stage[2] += host_seconds() - ts0;
	ts0 = host_seconds();
	if (is_tc_precision(precision))
	{
		for (int k = 1; k < NUM_TILE_CLASSES; k++) p.flops_cls[0] += p.flops_cls[k], p.flops_cls[k] = 0;
	}
	// one launch covers every class: all tiles in one list
	size_t ntiles = 0;
	for (int k = 0; k < NUM_TILE_CLASSES; k++) ntiles += tiles[k].size();
	p.tiles.reserve(ntiles);
	for (int k = 0; k < NUM_TILE_CLASSES; k++) p.tiles.insert(p.tiles.end(), tiles[k].begin(), tiles[k].end());
	if (is_tc_precision(precision) && !p.tiles.empty())
	{
		// the persistent tensor-core kernel takes tiles in list order, one per CTA at a time: tiles
		// whose outputs start from the same B block and cover the same column range are put next to
		// each other, so that the CTAs running them at the same time read those B records from L2
		// (output blocks of one column sector meet the same B blocks, one per block of A)
		auto first_b = [&](const GemmTile& t) -> i64 {
			const GemmOut& o = outs[(size_t)t.out];
			return o.nc > 0 ? tcons[(size_t)o.c0].b_rec : -1;    // an output without contributions: zero tiles first
		};
		std::stable_sort(p.tiles.begin(), p.tiles.end(), [&](const GemmTile& x, const GemmTile& y) {
			const i64 bx = first_b(x), by = first_b(y);
			if (bx != by) return bx < by;
			return x.n0 < y.n0;
		});
	}
	p.outs = std::move(outs);
	p.cons = std::move(cons);
	p.splits = std::move(splits);
	p.work_doubles = wsz;
	p.tcons = std::move(tcons);
	p.apacks = std::move(apacks);
	p.bpacks = std::move(bpacks);
	p.flops = flops;
	p.a_entries = s.nnz;
	p.b_entries = t.nnz;
	g_plan_stage[3] += host_seconds() - ts0;
	return p;
}

// ------------------------------------------------------------------------------------
// data movement
// ------------------------------------------------------------------------------------

// block_sparse_tensor_transpose (block_sparse_tensor.c:785-870)
CopyLowering lower_transpose(const Meta& t, const int* perm)
{
	double ts0 = host_seconds();
	std::vector<int> dst_of_src;
	auto out = std::make_shared<Meta>(transpose_meta(t, perm, &dst_of_src));
	g_plan_stage[4] += host_seconds() - ts0;
	ts0 = host_seconds();
	const Meta& r = *out;
	CTG_CHECK(t.ndim <= 6, "transpose: at most 6 axes");
	std::vector<PermDesc> descs;
	std::vector<Chunk> chunks;
	descs.reserve((size_t)t.nblocks);
	chunks.reserve((size_t)t.nblocks);
	for (int b = 0; b < t.nblocks; b++)
	{
		const i64* td = t.dims(b);
		const int rb = dst_of_src[(size_t)b];
		CTG_CHECK(rb >= 0 && rb < r.nblocks, "transpose: missing block");
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
	return perm_lowering(out, std::move(descs), std::move(chunks));
}

// block_sparse_tensor_flatten_axes (block_sparse_tensor.c:950-1112): each source block
// scatters its rows (j0, j1) into the fused rows of one target block
CopyLowering lower_flatten(const Meta& t, int ax, int newdir)
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
	const AxisFan fan0(t, ax), fan1(t, ax + 1);
	descs.reserve((size_t)t.nblocks);
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
		const i64 *f0 = fan0.of(it[ax]), *f1 = fan1.of(it[ax + 1]);
		const i64 n0 = fan0.count(it[ax]), n1 = fan1.count(it[ax + 1]);
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
		const i64* rpos = r.pos[ax].data();
		for (i64 j0 = 0; j0 < n0; j0++)
			for (i64 j1 = 0; j1 < n1; j1++) maps.push_back(rpos[f0[j0] * d1 + f1[j1]]);
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nrow * d.ntrail);
		descs.push_back(d);
	}
	check_rows(descs, maps, t.nnz, r.nnz);
	g_plan_stage[7] += host_seconds() - ts0;
	return rows_lowering(out, std::move(descs), std::move(chunks), std::move(maps));
}

// block_sparse_tensor_split_axis (block_sparse_tensor.c:1123-1285): each target block
// gathers its rows (j0, j1) from the fused rows of one source block
CopyLowering lower_split(const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq)
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
	const AxisFan fan0(r, ax), fan1(r, ax + 1);
	descs.reserve((size_t)r.nblocks);
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
		const i64 *f0 = fan0.of(ir[ax]), *f1 = fan1.of(ir[ax + 1]);
		const i64 n0 = fan0.count(ir[ax]), n1 = fan1.count(ir[ax + 1]);
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
		const i64* tpos = t.pos[ax].data();
		for (i64 j0 = 0; j0 < n0; j0++)
			for (i64 j1 = 0; j1 < n1; j1++) maps.push_back(tpos[f0[j0] * nd[1] + f1[j1]]);
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nrow * d.ntrail);
		descs.push_back(d);
	}
	check_rows(descs, maps, t.nnz, r.nnz);
	g_plan_stage[9] += host_seconds() - ts0;
	return rows_lowering(out, std::move(descs), std::move(chunks), std::move(maps));
}

// block_sparse_tensor_slice (block_sparse_tensor.c:1446-1553)
CopyLowering lower_slice(const Meta& t, int ax, const std::vector<i64>& ind)
{
	auto out = std::make_shared<Meta>(slice_meta(t, ax, ind));
	const Meta& r = *out;
	std::vector<RowDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	std::vector<i64> it(t.ndim);
	const AxisFan fan(r, ax);
	descs.reserve((size_t)r.nblocks);
	for (int b = 0; b < r.nblocks; b++)
	{
		const i64* ir = r.index(b);
		const i64* rd = r.dims(b);
		const q32 qn = r.qb[ax][ir[ax]];
		for (int i = 0; i < t.ndim; i++) it[i] = ir[i];
		it[ax] = t.find_q(ax, qn);
		const int tb = t.find(it.data());
		CTG_CHECK(tb >= 0, "slice: missing source block");
		const i64* fr = fan.of(ir[ax]);
		const i64 nr = fan.count(ir[ax]);
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
		for (i64 j = 0; j < nr; j++) maps.push_back(t.pos[ax][(size_t)ind[(size_t)fr[j]]]);
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nrow * d.ntrail);
		descs.push_back(d);
	}
	check_rows(descs, maps, t.nnz, r.nnz);
	return rows_lowering(out, std::move(descs), std::move(chunks), std::move(maps));
}


// block_sparse_tensor_multiply_pointwise_vector (block_sparse_tensor.c:1654-1703)
CopyLowering lower_scale(const Meta& m, int axrange)
{
	const int ax = (axrange == AX_LEADING ? 0 : m.ndim - 1);
	std::vector<ScaleDesc> descs;
	std::vector<Chunk> chunks;
	std::vector<i64> maps;
	const AxisFan fan(m, ax);
	descs.reserve((size_t)m.nblocks);
	for (int b = 0; b < m.nblocks; b++)
	{
		const i64* ib = m.index(b);
		const i64* bd = m.dims(b);
		const i64* f = fan.of(ib[ax]);
		const i64 nf = fan.count(ib[ax]);
		ScaleDesc d = {};
		d.off = m.boff[b];
		d.nlead = prod(bd, ax);
		d.nax = (int)bd[ax];
		d.ntrail = prod(bd + ax + 1, m.ndim - ax - 1);
		d.map_off = (i64)maps.size();
		maps.insert(maps.end(), f, f + nf);
		CTG_CHECK(nf == d.nax && d.off + d.nlead * d.nax * d.ntrail <= m.nnz, "scale: descriptor out of range");
		add_chunks(chunks, (int)descs.size(), d.nlead * d.nax * d.ntrail);
		descs.push_back(d);
	}
	CopyLowering p;
	p.kind = 2;
	p.scale = std::move(descs);
	p.chunks = std::move(chunks);
	p.maps = std::move(maps);
	p.elements = m.nnz;
	return p;
}

}  // namespace ctg
