// ctg_svd_schedule.h - index arithmetic of the cluster Jacobi schedule in ctg_svd.cu, shared with
// the host test that checks it (every column pair once per sweep, no column twice in a step,
// exchanges consistent with the next round's ownership).
#pragma once

#include <cuda_runtime.h>

namespace ctg {

// Pair pi (0 <= pi < np / 2) of round rnd (0 <= rnd < np - 1) of the circle method over np (even)
// indices: index np - 1 stays fixed, the others rotate; p < q on return. The residues mod np - 1
// by one conditional subtraction (both sums lie below 2 (np - 1)): an integer division sits on
// the serial chain of every Jacobi step.
__host__ __device__ inline void round_robin_pair(int rnd, int pi, int np, int& p, int& q)
{
	const int m = np - 1;
	if (pi == 0) { p = rnd; q = m; }
	else
	{
		p = rnd + pi;
		if (p >= m) p -= m;
		q = rnd - pi + m;
		if (q >= m) q -= m;
	}
	if (p > q) { const int t = p; p = q; q = t; }
}

// Column groups held by CTA pi in round rho (circle method over nm + 1 groups; group nm stays
// with CTA 0): a in slot 0, b in slot 1.
__host__ __device__ inline void round_groups(int rho, int pi, int nm, int& a, int& b)
{
	if (pi == 0) { a = rho; b = nm; }
	else { a = (rho + pi) % nm; b = (rho - pi + nm) % nm; }
}

// CTA and slot that hold group x in round rho (the inverse of round_groups).
__host__ __device__ inline void group_owner(int x, int rho, int nm, int& pi, int& slot)
{
	if (x == nm) { pi = 0; slot = 1; return; }
	const int dd = ((x - rho) % nm + nm) % nm;
	const int half = (nm + 1) / 2;
	if (dd == 0) { pi = 0; slot = 0; }
	else if (dd <= half - 1) { pi = dd; slot = 0; }
	else { pi = nm - dd; slot = 1; }
}

// Pair k of inner step `step` of a CTA holding groups of cA and cB columns (group size bs):
// mode 0 pairs columns inside each slot (circle method over npad = bs rounded up to even
// columns; pairs k < npad / 2 in slot 0, the others in slot 1), mode 1 pairs slot-0 column k with
// slot-1 column (k + step) mod bs. Returns false for a pair that involves a missing column.
__host__ __device__ inline bool step_pair_idx(int mode, int step, int k, int bs, int cA, int cB, int npad, int& sp,
                                              int& cp, int& sq, int& cq)
{
	if (mode == 0)
	{
		const int half = npad >> 1;
		const int sl = k < half ? 0 : 1;
		int p, q;
		round_robin_pair(step, k < half ? k : k - half, npad, p, q);
		sp = sl;
		sq = sl;
		cp = p;
		cq = q;
		return q < (sl == 0 ? cA : cB);
	}
	sp = 0;
	sq = 1;
	cp = k;
	cq = k + step;                 // (k + step) mod bs, with k, step < bs
	if (cq >= bs) cq -= bs;
	return k < cA && cq < cB;
}

}  // namespace ctg
