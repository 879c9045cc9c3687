// Block enumeration of make_meta (ctg_meta.cpp) against a brute-force scan over all block
// multi-indices: allowed blocks (quantum numbers summing to zero with the axis directions, the
// rule of block_sparse_tensor.c:78-140), row-major order, offsets, dimensions and find().
// Small quantum numbers, and pairs packed as (a << 16) + b as the Fermi-Hubbard model encodes
// particle number and spin (wide value ranges, many sectors, few allowed combinations).
// Also: transpose_meta (permutes an existing structure), and the result structures of dot,
// flatten and slice (which copy the per-axis data of unchanged axes) against make_meta of the
// same axes, every field.
// Built and run by tests/test_host_logic.py on the host; no GPU involved.
#include <algorithm>
#include <cstdio>
#include <random>
#include "ctg_meta.h"
using namespace ctg;
int main()
{
	std::mt19937 rng(7);
	int bad = 0;
	for (int trial = 0; trial < 6000; trial++)
	{
		const bool pairs = trial >= 3000;
		const int nd = 1 + rng() % 6;
		std::vector<i64> dim(nd);
		std::vector<int> dir(nd);
		std::vector<std::vector<q32>> ql(nd);
		for (int a = 0; a < nd; a++)
		{
			dim[a] = 1 + rng() % (pairs ? 14 : 9);
			dir[a] = (rng() & 1) ? 1 : -1;
			for (int j = 0; j < dim[a]; j++)
			{
				if (pairs) ql[a].push_back((int)(rng() % 5) * 65536 + (int)(rng() % 5) - 2);
				else ql[a].push_back((int)(rng() % 7) - 3);
			}
		}
		Meta m = make_meta(nd, dim.data(), dir.data(), ql);
		// brute force over all block multi-indices in row-major order
		i64 total = 1;
		for (int a = 0; a < nd; a++) total *= m.nb[a];
		std::vector<i64> idx(nd);
		int b = 0;
		i64 off = 0;
		for (i64 p = 0; p < total; p++)
		{
			i64 r = p;
			for (int a = nd - 1; a >= 0; a--) { idx[a] = r % m.nb[a]; r /= m.nb[a]; }
			long long q = 0;
			for (int a = 0; a < nd; a++) q += (long long)dir[a] * m.qb[a][idx[a]];
			const int f = m.find(idx.data());
			if (q != 0) { if (f != -1) bad++; continue; }
			if (f != b) bad++;
			for (int a = 0; a < nd; a++) if (m.index(b)[a] != idx[a] || m.dims(b)[a] != m.bd[a][idx[a]]) bad++;
			if (m.boff[b] != off) bad++;
			off += m.block_size(b);
			b++;
		}
		if (b != m.nblocks || off != m.nnz) bad++;
	}
	for (int trial = 0; trial < 2000; trial++)
	{
		const int nd = 2 + (int)(rng() % 5);
		std::vector<i64> dim(nd);
		std::vector<int> dir(nd);
		std::vector<std::vector<q32>> ql(nd);
		for (int a = 0; a < nd; a++)
		{
			dim[a] = 1 + (i64)(rng() % 9);
			dir[a] = (rng() & 1) ? 1 : -1;
			ql[a].resize((size_t)dim[a]);
			for (auto& q : ql[a]) q = (q32)(rng() % 5) - 2;
		}
		const Meta t = make_meta(nd, dim.data(), dir.data(), ql);
		std::vector<int> perm(nd);
		for (int a = 0; a < nd; a++) perm[a] = a;
		std::shuffle(perm.begin(), perm.end(), rng);
		const Meta x = transpose_meta(t, perm.data());
		std::vector<i64> d2(nd);
		std::vector<int> r2(nd);
		std::vector<std::vector<q32>> q2(nd);
		for (int i = 0; i < nd; i++) { d2[i] = dim[perm[i]]; r2[i] = dir[perm[i]]; q2[i] = ql[perm[i]]; }
		const Meta y = make_meta(nd, d2.data(), r2.data(), q2);
		const bool same = x.nblocks == y.nblocks && x.nnz == y.nnz && x.bidx == y.bidx && x.bdim == y.bdim &&
		                  x.boff == y.boff && x.lin == y.lin && x.lut == y.lut && x.qb == y.qb && x.bd == y.bd &&
		                  x.pos == y.pos && x.blk == y.blk && x.nb == y.nb && x.dim == y.dim && x.dir == y.dir &&
		                  x.ql == y.ql;
		if (!same) bad++;
	}
	auto same_meta = [](const Meta& x, const Meta& y) {
		return x.nblocks == y.nblocks && x.nnz == y.nnz && x.bidx == y.bidx && x.bdim == y.bdim && x.boff == y.boff &&
		       x.lin == y.lin && x.lut == y.lut && x.qb == y.qb && x.bd == y.bd && x.pos == y.pos && x.blk == y.blk &&
		       x.nb == y.nb && x.dim == y.dim && x.dir == y.dir && x.ql == y.ql;
	};
	for (int trial = 0; trial < 1000; trial++)
	{
		// s (a, b, k) . t (k', c): dot over one axis; flatten of s's (a, b); slice of s's axis b
		auto rq = [&](i64 d) { std::vector<q32> q((size_t)d); for (auto& x : q) x = (q32)(rng() % 5) - 2; return q; };
		const i64 da = 1 + rng() % 7, db = 1 + rng() % 7, dk = 1 + rng() % 7, dc = 1 + rng() % 7;
		const std::vector<q32> qa = rq(da), qbv = rq(db), qk = rq(dk), qc = rq(dc);
		const int sa = (rng() & 1) ? 1 : -1, sb = (rng() & 1) ? 1 : -1, sk = (rng() & 1) ? 1 : -1, sc = (rng() & 1) ? 1 : -1;
		const i64 ds[3] = {da, db, dk}, dt[2] = {dk, dc};
		const int rs[3] = {sa, sb, sk}, rt[2] = {-sk, sc};
		const Meta ms = make_meta(3, ds, rs, {qa, qbv, qk});
		const Meta mt = make_meta(2, dt, rt, {qk, qc});
		const i64 dr[3] = {da, db, dc};
		const int rr[3] = {sa, sb, sc};
		if (!same_meta(dot_result_meta(ms, AX_TRAILING, mt, AX_LEADING, 1), make_meta(3, dr, rr, {qa, qbv, qc}))) bad++;
		std::vector<q32> qf((size_t)(da * db));
		for (i64 j = 0; j < da; j++)
			for (i64 k = 0; k < db; k++) qf[(size_t)(j * db + k)] = -1 * (sa * qa[(size_t)j] + sb * qbv[(size_t)k]);
		const i64 dfl[2] = {da * db, dk};
		const int rfl[2] = {-1, sk};
		if (!same_meta(flatten_meta(ms, 0, -1), make_meta(2, dfl, rfl, {qf, qk}))) bad++;
		std::vector<i64> ind;
		for (i64 j = 0; j < db; j += 2) ind.push_back(j);
		std::vector<q32> qsl;
		for (i64 j : ind) qsl.push_back(qbv[(size_t)j]);
		const i64 dsl[3] = {da, (i64)ind.size(), dk};
		if (!same_meta(slice_meta(ms, 1, ind), make_meta(3, dsl, rs, {qa, qsl, qk}))) bad++;
	}
	printf("mismatches: %d\n", bad);
	return bad != 0;
}
