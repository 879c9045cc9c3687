// Block enumeration of make_meta (ctg_meta.cpp) against a brute-force scan over all block
// multi-indices: allowed blocks (quantum numbers summing to zero with the axis directions, the
// rule of block_sparse_tensor.c:78-140), row-major order, offsets, dimensions and find().
// Small quantum numbers, and pairs packed as (a << 16) + b as the Fermi-Hubbard model encodes
// particle number and spin (wide value ranges, many sectors, few allowed combinations).
// Built and run by tests/test_host_logic.py on the host; no GPU involved.
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
	printf("mismatches: %d\n", bad);
	return bad != 0;
}
