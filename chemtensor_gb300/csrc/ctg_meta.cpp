// ctg_meta.cpp - block structure rules (integer arithmetic only).
#include "ctg_meta.h"

#include <algorithm>
#include <numeric>

namespace ctg {

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line)
{
	char buf[512];
	snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file, line);
	throw CudaError(buf);
}

i64 Meta::block_size(int b) const
{
	i64 p = 1;
	for (int i = 0; i < ndim; i++) p *= bdim[(size_t)b * ndim + i];
	return p;
}

i64 Meta::linear(const i64* idx) const
{
	i64 k = 0;
	for (int i = 0; i < ndim; i++) k = k * nb[i] + idx[i];
	return k;
}

int Meta::find(const i64* idx) const
{
	for (int i = 0; i < ndim; i++)
		if (idx[i] < 0 || idx[i] >= nb[i]) return -1;
	const i64 k = linear(idx);
	if (!lut.empty()) return lut[(size_t)k];
	auto it = std::lower_bound(lin.begin(), lin.end(), k);
	return (it == lin.end() || *it != k) ? -1 : (int)(it - lin.begin());
}

int Meta::find_q(int ax, q32 q) const
{
	const auto& v = qb[ax];
	auto it = std::lower_bound(v.begin(), v.end(), q);
	if (it == v.end() || *it != q) return -1;
	return (int)(it - v.begin());
}

bool Meta::same_structure(const Meta& o) const
{
	return ndim == o.ndim && dim == o.dim && dir == o.dir && ql == o.ql;
}

static inline uint64_t mix64(uint64_t h, uint64_t v)
{
	// splitmix64 finaliser applied to the running state combined with the next word
	uint64_t z = h ^ (v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2));
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

uint64_t Meta::structure_hash() const
{
	if (!hashed_)
	{
		uint64_t h = mix64(0, (uint64_t)ndim);
		for (int i = 0; i < ndim; i++)
		{
			h = mix64(h, (uint64_t)dim[(size_t)i]);
			h = mix64(h, (uint64_t)(int64_t)dir[(size_t)i]);
			for (q32 q : ql[(size_t)i]) h = mix64(h, (uint64_t)(uint32_t)q);
		}
		hash_ = h;
		hashed_ = true;
	}
	return hash_;
}

namespace {

// Axes of a new structure that are axes of an existing one (same logical quantum numbers): their
// sorted unique quantum numbers, multiplicities and index maps are copied instead of recomputed.
struct AxisSource {
	const Meta* m[8] = {};
	int ax[8] = {};
};

Meta build_meta(int ndim, const i64* dim, const int* dir, std::vector<std::vector<q32>> ql, const AxisSource* src);

}  // namespace

Meta make_meta(int ndim, const i64* dim, const int* dir, const std::vector<std::vector<q32>>& ql)
{
	return build_meta(ndim, dim, dir, ql, nullptr);
}

namespace {

Meta build_meta(int ndim, const i64* dim, const int* dir, std::vector<std::vector<q32>> ql, const AxisSource* src)
{
	CTG_CHECK(ndim >= 1 && ndim <= 8, "tensor degree out of range");
	Meta m;
	m.ndim = ndim;
	m.dim.assign(dim, dim + ndim);
	m.dir.assign(dir, dir + ndim);
	m.ql = std::move(ql);
	m.qb.resize(ndim);
	m.bd.resize(ndim);
	m.pos.resize(ndim);
	m.blk.resize(ndim);
	m.nb.resize(ndim);
	for (int a = 0; a < ndim; a++)
	{
		CTG_CHECK(dim[a] > 0 && (i64)m.ql[a].size() == dim[a], "logical quantum numbers do not match the dimension");
		if (src && src->m[a])
		{
			const Meta& o = *src->m[a];
			const int b = src->ax[a];
			m.qb[a] = o.qb[b];
			m.nb[a] = o.nb[b];
			m.bd[a] = o.bd[b];
			m.pos[a] = o.pos[b];
			m.blk[a] = o.blk[b];
			continue;
		}
		std::vector<q32> u(m.ql[a]);
		std::sort(u.begin(), u.end());
		u.erase(std::unique(u.begin(), u.end()), u.end());
		m.qb[a] = u;
		m.nb[a] = (i64)u.size();
		m.bd[a].assign(u.size(), 0);
		m.pos[a].resize(dim[a]);
		m.blk[a].resize(dim[a]);
		for (i64 j = 0; j < dim[a]; j++)
		{
			const int b = (int)(std::lower_bound(u.begin(), u.end(), m.ql[a][j]) - u.begin());
			m.blk[a][j] = b;
			m.pos[a][j] = m.bd[a][b]++;
		}
	}
	// Enumerate the allowed blocks in row-major order by meeting in the middle: the axes are cut
	// into a prefix [0, k) and a suffix [k, ndim). Every suffix index tuple is listed once with its
	// signed quantum-number sum, grouped by sum (row-major order inside a group); then every
	// prefix tuple, in row-major order, looks up the group whose sum cancels its own and emits
	// one block per member. Cost ~ prefixes + suffixes + blocks instead of the product of all
	// but one axis, which matters for pair-encoded quantum numbers (many sectors per bond,
	// few allowed combinations). The cut minimises prefixes + 2 x suffixes.
	int k = ndim - 1;
	{
		double best = 1e300;
		for (int kk = 0; kk < ndim; kk++)
		{
			double pcount = 1, scount = 1;
			for (int a = 0; a < kk; a++) pcount *= (double)m.nb[a];
			for (int a = kk; a < ndim; a++) scount *= (double)m.nb[a];
			const double cost = pcount + 2 * scount;
			if (cost < best) { best = cost; k = kk; }
		}
	}
	const int ns = ndim - k;
	i64 nsuf = 1, npre = 1;
	for (int a = k; a < ndim; a++) nsuf *= m.nb[a];
	for (int a = 0; a < k; a++) npre *= m.nb[a];
	CTG_CHECK(nsuf <= ((i64)1 << 26) && npre <= ((i64)1 << 40), "block structure too large to enumerate");
	// suffix tuples: (sum, suffix linear index), sorted by sum then index
	std::vector<std::pair<long long, i64>> suf((size_t)nsuf);
	{
		i64 sidx[8] = {0};
		long long part[9] = {0};
		for (int a = k; a < ndim; a++) part[a - k + 1] = part[a - k] + (long long)dir[a] * m.qb[a][0];
		for (i64 s = 0; s < nsuf; s++)
		{
			if (s > 0)
			{
				int a = ns - 1;
				while (++sidx[a] == m.nb[k + a])
				{
					sidx[a] = 0;
					a--;
				}
				for (int i = a; i < ns; i++) part[i + 1] = part[i] + (long long)dir[k + i] * m.qb[k + i][sidx[i]];
			}
			suf[(size_t)s] = {part[ns], s};
		}
	}
	std::sort(suf.begin(), suf.end());
	std::vector<long long> keys;
	std::vector<i64> gstart;
	for (size_t s = 0; s < suf.size(); s++)
		if (s == 0 || suf[s].first != suf[s - 1].first)
		{
			keys.push_back(suf[s].first);
			gstart.push_back((i64)s);
		}
	gstart.push_back((i64)suf.size());
	// suffix index tuples of the sorted list, decoded once
	std::vector<int> stup((size_t)nsuf * ns);
	for (size_t s = 0; s < suf.size(); s++)
	{
		i64 r = suf[s].second;
		for (int a = ns - 1; a >= 0; a--)
		{
			stup[s * ns + (size_t)a] = (int)(r % m.nb[k + a]);
			r /= m.nb[k + a];
		}
	}
	// prefix tuples in row-major order: the group of each (pass 1 counts, pass 2 fills)
	std::vector<int> grp((size_t)npre, -1);
	i64 nblk = 0;
	{
		i64 pidx[8] = {0};
		long long part[9] = {0};
		for (int a = 0; a < k; a++) part[a + 1] = part[a] + (long long)dir[a] * m.qb[a][0];
		for (i64 p = 0; p < npre; p++)
		{
			if (p > 0)
			{
				int a = k - 1;
				while (++pidx[a] == m.nb[a])
				{
					pidx[a] = 0;
					a--;
				}
				for (int i = a; i < k; i++) part[i + 1] = part[i] + (long long)dir[i] * m.qb[i][pidx[i]];
			}
			const long long need = -part[k];
			auto it = std::lower_bound(keys.begin(), keys.end(), need);
			if (it == keys.end() || *it != need) continue;
			const int g = (int)(it - keys.begin());
			grp[(size_t)p] = g;
			nblk += gstart[(size_t)g + 1] - gstart[(size_t)g];
		}
	}
	CTG_CHECK(nblk <= INT32_MAX, "too many blocks");
	m.nblocks = (int)nblk;
	m.bidx.resize((size_t)nblk * ndim);
	m.bdim.resize((size_t)nblk * ndim);
	m.boff.resize((size_t)nblk);
	m.lin.resize((size_t)nblk);
	i64 off = 0;
	{
		const i64* bdp[8];
		for (int a = 0; a < ndim; a++) bdp[a] = m.bd[a].data();
		i64 pidx[8] = {0};
		i64 pdim = 1;
		size_t b = 0;
		for (i64 p = 0; p < npre; p++)
		{
			if (p > 0)
			{
				int a = k - 1;
				while (++pidx[a] == m.nb[a])
				{
					pidx[a] = 0;
					a--;
				}
			}
			const int g = grp[(size_t)p];
			if (g < 0) continue;
			pdim = 1;
			for (int a = 0; a < k; a++) pdim *= bdp[a][pidx[a]];
			for (i64 s = gstart[(size_t)g]; s < gstart[(size_t)g + 1]; s++)
			{
				i64* bi = &m.bidx[b * ndim];
				i64* bdm = &m.bdim[b * ndim];
				i64 size = pdim;
				for (int a = 0; a < k; a++)
				{
					bi[a] = pidx[a];
					bdm[a] = bdp[a][pidx[a]];
				}
				const int* st = &stup[(size_t)s * ns];
				for (int a = 0; a < ns; a++)
				{
					bi[k + a] = st[a];
					bdm[k + a] = bdp[k + a][st[a]];
					size *= bdm[k + a];
				}
				m.boff[b] = off;
				m.lin[b] = p * nsuf + suf[(size_t)s].second;
				off += size;
				b++;
			}
		}
	}
	m.nnz = off;
	i64 total = 1;
	bool dense = true;
	for (int a = 0; a < ndim; a++)
	{
		total *= m.nb[a];
		if (total > 4 * (i64)m.nblocks + 4096) { dense = false; break; }
	}
	if (dense)
	{
		m.lut.assign((size_t)total, -1);
		for (int b = 0; b < m.nblocks; b++) m.lut[(size_t)m.lin[(size_t)b]] = b;
	}
	return m;
}

}  // namespace

Meta dot_result_meta(const Meta& s, int axs, const Meta& t, int axt, int nmult)
{
	const int shift_s = (axs == AX_LEADING ? 0 : s.ndim - nmult);
	const int shift_t = (axt == AX_LEADING ? 0 : t.ndim - nmult);
	for (int i = 0; i < nmult; i++)
	{
		CTG_CHECK(s.dim[shift_s + i] == t.dim[shift_t + i], "dot: contracted dimensions differ");
		CTG_CHECK(s.dir[shift_s + i] == -t.dir[shift_t + i], "dot: contracted axis directions must be reversed");
		CTG_CHECK(s.ql[shift_s + i] == t.ql[shift_t + i], "dot: contracted quantum numbers differ");
	}
	const int off_s = (axs == AX_LEADING ? nmult : 0);
	const int off_t = (axt == AX_LEADING ? nmult : 0);
	const int nfs = s.ndim - nmult, nft = t.ndim - nmult;
	std::vector<i64> dim;
	std::vector<int> dir;
	std::vector<std::vector<q32>> ql;
	AxisSource src;
	for (int i = 0; i < nfs; i++)
	{
		dim.push_back(s.dim[off_s + i]);
		dir.push_back(s.dir[off_s + i]);
		ql.push_back(s.ql[off_s + i]);
		src.m[i] = &s;
		src.ax[i] = off_s + i;
	}
	for (int i = 0; i < nft; i++)
	{
		dim.push_back(t.dim[off_t + i]);
		dir.push_back(t.dir[off_t + i]);
		ql.push_back(t.ql[off_t + i]);
		src.m[nfs + i] = &t;
		src.ax[nfs + i] = off_t + i;
	}
	CTG_CHECK(!dim.empty(), "dot: scalar results are not on the DMRG path");
	CTG_CHECK(dim.size() <= 8, "tensor degree out of range");
	return build_meta((int)dim.size(), dim.data(), dir.data(), std::move(ql), &src);
}

Meta transpose_meta(const Meta& t, const int* perm, std::vector<int>* dst_of_src)
{
	// The allowed blocks of a transposed tensor are the permuted allowed blocks (the rule is a sum
	// over axes), so the structure follows from t's without a new enumeration: permute the axis
	// data and the block multi-indices, then order the blocks row-major under the new axis order.
	const int nd = t.ndim;
	Meta m;
	m.ndim = nd;
	m.dim.resize(nd);
	m.dir.resize(nd);
	m.ql.resize(nd);
	m.qb.resize(nd);
	m.bd.resize(nd);
	m.pos.resize(nd);
	m.blk.resize(nd);
	m.nb.resize(nd);
	for (int a = 0; a < nd; a++)
	{
		const int p = perm[a];
		CTG_CHECK(p >= 0 && p < nd, "transpose: invalid permutation");
		m.dim[a] = t.dim[p];
		m.dir[a] = t.dir[p];
		m.ql[a] = t.ql[p];
		m.qb[a] = t.qb[p];
		m.bd[a] = t.bd[p];
		m.pos[a] = t.pos[p];
		m.blk[a] = t.blk[p];
		m.nb[a] = t.nb[p];
	}
	const int nb = t.nblocks;
	std::vector<std::pair<i64, int>> order((size_t)nb);
	for (int b = 0; b < nb; b++)
	{
		const i64* ib = t.index(b);
		i64 k = 0;
		for (int a = 0; a < nd; a++) k = k * m.nb[a] + ib[perm[a]];
		order[(size_t)b] = {k, b};
	}
	std::sort(order.begin(), order.end());
	m.nblocks = nb;
	m.bidx.resize((size_t)nb * nd);
	m.bdim.resize((size_t)nb * nd);
	m.boff.resize((size_t)nb);
	m.lin.resize((size_t)nb);
	i64 off = 0;
	if (dst_of_src) dst_of_src->assign((size_t)nb, -1);
	for (int b = 0; b < nb; b++)
	{
		const int src = order[(size_t)b].second;
		if (dst_of_src) (*dst_of_src)[(size_t)src] = b;
		const i64* ib = t.index(src);
		const i64* db = t.dims(src);
		i64 size = 1;
		for (int a = 0; a < nd; a++)
		{
			m.bidx[(size_t)b * nd + a] = ib[perm[a]];
			m.bdim[(size_t)b * nd + a] = db[perm[a]];
			size *= db[perm[a]];
		}
		m.boff[(size_t)b] = off;
		m.lin[(size_t)b] = order[(size_t)b].first;
		off += size;
	}
	m.nnz = off;
	i64 total = 1;
	bool dense = true;
	for (int a = 0; a < nd; a++)
	{
		total *= m.nb[a];
		if (total > 4 * (i64)m.nblocks + 4096) { dense = false; break; }
	}
	if (dense)
	{
		m.lut.assign((size_t)total, -1);
		for (int b = 0; b < m.nblocks; b++) m.lut[(size_t)m.lin[(size_t)b]] = b;
	}
	return m;
}

Meta flatten_meta(const Meta& t, int ax, int newdir)
{
	CTG_CHECK(ax >= 0 && ax + 1 < t.ndim, "flatten: axis out of range");
	std::vector<i64> dim;
	std::vector<int> dir;
	std::vector<std::vector<q32>> ql;
	AxisSource src;
	for (int i = 0; i < ax; i++)
	{
		dim.push_back(t.dim[i]);
		dir.push_back(t.dir[i]);
		ql.push_back(t.ql[i]);
		src.m[i] = &t;
		src.ax[i] = i;
	}
	const i64 d0 = t.dim[ax], d1 = t.dim[ax + 1];
	std::vector<q32> qf((size_t)(d0 * d1));
	for (i64 j = 0; j < d0; j++)
		for (i64 k = 0; k < d1; k++)
			qf[(size_t)(j * d1 + k)] = newdir * (t.dir[ax] * t.ql[ax][j] + t.dir[ax + 1] * t.ql[ax + 1][k]);
	dim.push_back(d0 * d1);
	dir.push_back(newdir);
	ql.push_back(qf);
	for (int i = ax + 2; i < t.ndim; i++)
	{
		src.m[dim.size()] = &t;
		src.ax[dim.size()] = i;
		dim.push_back(t.dim[i]);
		dir.push_back(t.dir[i]);
		ql.push_back(t.ql[i]);
	}
	return build_meta((int)dim.size(), dim.data(), dir.data(), std::move(ql), &src);
}

Meta split_meta(const Meta& t, int ax, const i64 nd[2], const int ndir[2], const std::vector<q32>* nq)
{
	CTG_CHECK(nd[0] * nd[1] == t.dim[ax], "split: dimensions do not multiply to the original");
	for (i64 j = 0; j < nd[0]; j++)
		for (i64 k = 0; k < nd[1]; k++)
			CTG_CHECK(t.dir[ax] * t.ql[ax][(size_t)(j * nd[1] + k)] == ndir[0] * nq[0][j] + ndir[1] * nq[1][k],
			          "split: quantum numbers inconsistent with the original axis");
	std::vector<i64> dim;
	std::vector<int> dir;
	std::vector<std::vector<q32>> ql;
	AxisSource src;
	for (int i = 0; i < ax; i++)
	{
		src.m[dim.size()] = &t;
		src.ax[dim.size()] = i;
		dim.push_back(t.dim[i]);
		dir.push_back(t.dir[i]);
		ql.push_back(t.ql[i]);
	}
	for (int h = 0; h < 2; h++) { dim.push_back(nd[h]); dir.push_back(ndir[h]); ql.push_back(nq[h]); }
	for (int i = ax + 1; i < t.ndim; i++)
	{
		CTG_CHECK(dim.size() < 8, "tensor degree out of range");
		src.m[dim.size()] = &t;
		src.ax[dim.size()] = i;
		dim.push_back(t.dim[i]);
		dir.push_back(t.dir[i]);
		ql.push_back(t.ql[i]);
	}
	return build_meta((int)dim.size(), dim.data(), dir.data(), std::move(ql), &src);
}

Meta slice_meta(const Meta& t, int ax, const std::vector<i64>& ind)
{
	CTG_CHECK(!ind.empty(), "slice: empty index list");
	std::vector<std::vector<q32>> ql = t.ql;
	std::vector<i64> dim = t.dim;
	ql[ax].resize(ind.size());
	for (size_t j = 0; j < ind.size(); j++)
	{
		CTG_CHECK(ind[j] >= 0 && ind[j] < t.dim[ax], "slice: index out of range");
		ql[ax][j] = t.ql[ax][(size_t)ind[j]];
	}
	dim[ax] = (i64)ind.size();
	AxisSource src;
	for (int i = 0; i < t.ndim; i++)
		if (i != ax)
		{
			src.m[i] = &t;
			src.ax[i] = i;
		}
	return build_meta(t.ndim, dim.data(), t.dir.data(), std::move(ql), &src);
}

Meta reversed_meta(const Meta& t)
{
	Meta r = t;
	for (auto& d : r.dir) d = -d;
	return r;
}

}  // namespace ctg
