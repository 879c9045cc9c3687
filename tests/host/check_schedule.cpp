// The cluster Jacobi schedule of ctg_svd.cu (ctg_svd_schedule.h) for every cluster size 1..16 and
// many block sizes: each sweep pairs every two columns exactly once, no column takes part in two
// pairs of one inner step, the exchange after every round delivers each group to the CTA and slot
// that hold it in the next round (no target twice), and a sweep ends in the round-0 arrangement.
// Built and run by tests/test_host_logic.py on the host; no GPU involved.
#include <cstdio>
#include <map>
#include <set>
#include <utility>
#include <vector>

#include "ctg_svd_schedule.h"

using namespace ctg;

int main()
{
	int bad = 0, cases = 0;
	for (int cl = 1; cl <= 16; cl *= 2)
		for (int N = 1; N <= 300; N += 7)
			for (int r : {0, 1, 2, N / 2, N - 1, N})
			{
				if (r < 0 || r > N) continue;
				const int nblk = 2 * cl, nm = nblk - 1;
				const int bsmax = (N + nblk - 1) / nblk;
				const int bs = r > 0 ? (r + nblk - 1) / nblk : 1;
				if (bsmax > 32) continue;
				cases++;
				auto cnt = [&](int x) { const int c = r - x * bs; return c < 0 ? 0 : (c > bs ? bs : c); };
				std::vector<std::pair<int, int>> hold(cl);
				for (int pi = 0; pi < cl; pi++) round_groups(0, pi, nm, hold[pi].first, hold[pi].second);
				std::map<std::pair<int, int>, int> seen;
				for (int rho = 0; rho < nm; rho++)
				{
					for (int pi = 0; pi < cl; pi++)
					{
						int A, B;
						round_groups(rho, pi, nm, A, B);
						if (A != hold[pi].first || B != hold[pi].second) bad++;
						const int cA = cnt(A), cB = cnt(B);
						const int grp[2] = {A, B};
						auto run_step = [&](int mode, int st, int np, int npad) {
							std::set<std::pair<int, int>> used;
							for (int k = 0; k < np; k++)
							{
								int sp, cp, sq, cq;
								if (!step_pair_idx(mode, st, k, bs, cA, cB, npad, sp, cp, sq, cq)) continue;
								if (!used.insert({sp, cp}).second || !used.insert({sq, cq}).second) bad++;
								int g0 = grp[sp] * bs + cp, g1 = grp[sq] * bs + cq;
								if (g0 > g1) std::swap(g0, g1);
								if (g0 == g1 || g1 >= r) bad++;
								seen[{g0, g1}]++;
							}
						};
						if (rho == 0)
						{
							const int npad = bs + (bs & 1);
							if (npad > 32) bad++;
							for (int st = 0; st < npad - 1; st++) run_step(0, st, npad, npad);
						}
						for (int st = 0; st < bs; st++) run_step(1, st, bs, 0);
					}
					if (cl > 1)
					{
						const int rho1 = (rho + 1) % nm;
						std::map<std::pair<int, int>, int> next;
						for (int pi = 0; pi < cl; pi++)
							for (int slot = 0; slot < 2; slot++)
							{
								const int x = slot ? hold[pi].second : hold[pi].first;
								int pi2, s2;
								group_owner(x, rho1, nm, pi2, s2);
								if (pi2 < 0 || pi2 >= cl || next.count({pi2, s2})) bad++;
								next[{pi2, s2}] = x;
							}
						for (int pi = 0; pi < cl; pi++) hold[pi] = {next[{pi, 0}], next[{pi, 1}]};
					}
				}
				for (int pi = 0; pi < cl; pi++)
				{
					int A, B;
					round_groups(0, pi, nm, A, B);
					if (A != hold[pi].first || B != hold[pi].second) bad++;
				}
				if ((long)seen.size() != (long)r * (r - 1) / 2) bad++;
				for (const auto& kv : seen)
					if (kv.second != 1) bad++;
			}
	printf("cases: %d, mismatches: %d\n", cases, bad);
	return bad != 0;
}
