// ctg_random.cpp - seeded random MPS, reproducing the reference's generator bit for bit.
//
// Restates, for input generation on the host:
//   PCG32 and the 2x32-bit combination (M. E. O'Neill, "PCG: A family of simple fast
//     space-efficient statistically good algorithms for random number generation",
//     2014; as used in src/util/pcg_basic.c),
//   seed_rng_state, rand_interval, rand_choice (Floyd), randu, randn (Box-Muller)
//     (src/util/rng.c:15-125),
//   construct_random_mps (src/state/mps.c:93-175).
// Host code only; the GPU path takes the resulting MPS as its input.
#include <cmath>
#include <cstring>

#include "ctgpu.h"
#include "ctg_dmrg.h"

namespace {

struct Pcg32 {
	uint64_t state = 0, inc = 0;
	uint32_t next()
	{
		const uint64_t old = state;
		state = old * 6364136223846793005ULL + inc;
		const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
		const uint32_t rot = (uint32_t)(old >> 59u);
		return (xs >> rot) | (xs << ((-rot) & 31));
	}
	void seed(uint64_t initstate, uint64_t initseq)
	{
		state = 0;
		inc = (initseq << 1u) | 1u;
		next();
		state += initstate;
		next();
	}
};

struct Rng {
	Pcg32 g[2];
	uint64_t u64() { return ((uint64_t)g[0].next() << 32) | g[1].next(); }
	uint64_t bounded(uint64_t bound)
	{
		const uint64_t threshold = (0 - bound) % bound;
		for (;;)
		{
			const uint64_t r = u64();
			if (r >= threshold) return r % bound;
		}
	}
	double uniform() { return std::ldexp((double)u64(), -64); }
	double normal()
	{
		const double two_pi = 6.2831853071795864769;
		double u1 = uniform();
		const double u2 = uniform();
		if (u1 == 0) u1 = 1;
		return std::sqrt(-2 * std::log(u1)) * std::sin(two_pi * u2);
	}
	// seed_rng_state: a temporary generator derives both seeds and stream selectors
	explicit Rng(uint64_t seed)
	{
		Pcg32 t;
		t.seed(seed, 6364136223846793005ULL * seed + 1442695040888963407ULL);
		auto draw64 = [&] { const uint64_t hi = t.next(); return (hi << 32) | t.next(); };
		const uint64_t s1 = draw64(), s2 = draw64(), q1 = draw64();
		uint64_t q2 = draw64();
		const uint64_t mask = ~0ull >> 1;
		if ((q1 & mask) == (q2 & mask)) q2 = ~q2;
		g[0].seed(s1, q1);
		g[1].seed(s2, q2);
	}
	// Floyd's sampling of num distinct values from [0, bound)
	void choice(uint64_t bound, uint64_t num, std::vector<uint64_t>& out)
	{
		out.assign(num, 0);
		for (uint64_t i = 0; i < num; i++)
		{
			const uint64_t j = bound - num + 1 + i;
			const uint64_t t = bounded(j);
			bool drawn = false;
			for (uint64_t k = 0; k < i; k++)
				if (out[k] == t) { drawn = true; break; }
			out[i] = drawn ? j - 1 : t;
		}
	}
};

}  // namespace

extern "C" {

void ctgpu_randn_sequence(uint64_t seed, int n, double* out)
{
	Rng r(seed);
	for (int i = 0; i < n; i++) out[i] = r.normal();
}

int ctgpu_construct_random_mps(int nsites, ct_long d, const qnumber* qsite, qnumber qnum_sector, ct_long max_vdim,
                               uint64_t rng_seed, struct mps* mps)
{
	if (nsites < 1 || d < 1 || max_vdim < 1 || !qsite || !mps) return -5;
	using ctg::i64;
	using ctg::q32;
	Rng rng(rng_seed);
	std::vector<std::vector<q32>> qb(nsites + 1);
	qb[0] = {0};
	qb[nsites] = {qnum_sector};
	auto bond = [&](const std::vector<q32>& prev, int sign) {
		std::vector<q32> full;
		for (q32 a : prev)
			for (i64 j = 0; j < d; j++) full.push_back(a + sign * qsite[j]);
		if ((i64)full.size() <= max_vdim) return full;
		std::vector<uint64_t> idx;
		rng.choice(full.size(), (uint64_t)max_vdim, idx);
		std::vector<q32> sel;
		for (uint64_t k : idx) sel.push_back(full[(size_t)k]);
		return sel;
	};
	for (int l = 1; l < (nsites + 1) / 2; l++) qb[l] = bond(qb[l - 1], +1);
	for (int l = nsites - 1; l >= (nsites + 1) / 2; l--) qb[l] = bond(qb[l + 1], -1);

	mps->nsites = nsites;
	mps->d = d;
	mps->qsite = (qnumber*)aligned_alloc(16, ((size_t)d * sizeof(qnumber) + 15) & ~(size_t)15);
	memcpy(mps->qsite, qsite, (size_t)d * sizeof(qnumber));
	mps->a = (struct block_sparse_tensor*)aligned_alloc(16, ((size_t)nsites * sizeof(struct block_sparse_tensor) + 15) & ~(size_t)15);
	memset(mps->a, 0, (size_t)nsites * sizeof(struct block_sparse_tensor));
	const std::vector<q32> qs(qsite, qsite + d);
	for (int l = 0; l < nsites; l++)
	{
		const i64 dim[3] = {(i64)qb[l].size(), d, (i64)qb[l + 1].size()};
		const int dir[3] = {TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN};
		ctg::Meta m = ctg::make_meta(3, dim, dir, {qb[l], qs, qb[l + 1]});
		std::vector<double> v((size_t)m.nnz);
		const double alpha = 1.0 / std::sqrt((double)(dim[0] * dim[1] * dim[2]));
		for (auto& x : v) x = alpha * rng.normal() + 0.0;
		ctg::write_struct_host(m, v.data(), &mps->a[l]);
	}
	return 0;
}

}  // extern "C"
