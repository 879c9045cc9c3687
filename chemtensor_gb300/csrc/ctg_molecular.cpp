// ctg_molecular.cpp - MPO of the spin-orbital molecular Hamiltonian (host).
//
// Replaces construct_spin_molecular_hamiltonian_mpo_assembly with optimize = false, followed by
// mpo_from_assembly (src/operator/hamiltonian.c:2768-2979, src/operator/mpo.c:59-174):
//
//   H = sum_{i,j,s} t_ij a+_{i,s} a_{j,s} + 1/2 sum_{i,j,k,l,s,u} v_ijkl a+_{i,s} a+_{j,u} a_{l,u} a_{k,s}
//
// Sites are spatial orbitals with the local basis |0>, |dn>, |up>, |up dn> (index 2 n_up + n_dn,
// quantum numbers (N, 2 Sz) = (0,0), (1,-1), (1,1), (2,0)); the Jordan-Wigner order of the spin
// orbitals is (0 up, 0 dn, 1 up, 1 dn, ...), as in the reference's dense test Hamiltonian
// (test/operator/hamiltonian.py:260-290, :335-360).
//
// Construction (a state machine over the bonds). Every term is brought into Jordan-Wigner order
// (a sign per exchange of two different spin orbitals); the operator of a term then factorises
// into site-local matrices: the product of its operators at that site, times the local parity
// F = Z x Z when an odd number of the term's operators sits on this site or to its left. At bond b
// (between sites b-1 and b) a term is in one of these states, by how many of its operators lie
// left of the bond:
//   I       none yet                        D        all of them
//   L1[x]   only x (two-body terms)         R1[y]    all but y (y the last operator)
//   L2[x,x'] the first two, for b <= n/2    R2[y,y'] all but the last two, for b > n/2
// L-states are named by the operators already placed, R-states by the operators still to come,
// so every state is one fixed operator on its side of the bond and is shared by all terms that
// pass through it; transitions between two L-states or two R-states carry weight 1. Each term
// has exactly one transition from an L-state into an R-state (into R1 directly for one-body
// terms), and that transition carries the term's coefficient. Pair states are kept on the side
// with fewer spin orbitals, giving the bond dimension 2 + 4n + 2M^2 - M with M = 2 min(b, n-b),
// at most 2n^2 + 3n + 2. Bond quantum numbers are the (N, 2 Sz) change of the operator left of
// the bond: that of the placed operators for L-states, minus that of the pending ones for
// R-states.
#include <cmath>
#include <cstring>
#include <vector>

#include "ct_structs.h"
#include "ctg_dmrg.h"
#include "ctg_meta.h"

namespace {

using ctg::i64;
using ctg::q32;

typedef double Mat4[4][4];

// operator id x = 4 site + 2 spin + type; spin 0 up, 1 down; type 0 creation, 1 annihilation
inline int op_site(int x) { return x >> 2; }
inline int op_spin(int x) { return (x >> 1) & 1; }
inline int op_type(int x) { return x & 1; }

inline q32 encode_pair(int n, int s2) { return (q32)(n * 65536 + s2); }

q32 op_qnum(int x)
{
	const int dn = op_type(x) == 0 ? 1 : -1;
	const int ds = (op_spin(x) == 0 ? 1 : -1) * dn;
	return encode_pair(dn, ds);
}

void mat_identity(Mat4 m)
{
	memset(m, 0, sizeof(Mat4));
	for (int i = 0; i < 4; i++) m[i][i] = 1;
}

// local matrix of an operator (row = out state): basis index 2 n_up + n_dn
void mat_op(int x, Mat4 m)
{
	memset(m, 0, sizeof(Mat4));
	for (int s = 0; s < 4; s++)
	{
		const int nup = s >> 1, ndn = s & 1;
		const int occ = op_spin(x) == 0 ? nup : ndn;
		const bool create = op_type(x) == 0;
		if (create == (occ == 1)) continue;
		const int t = op_spin(x) == 0 ? (s ^ 2) : (s ^ 1);
		// the down orbital follows the up orbital of the same site in the string
		const double sign = (op_spin(x) == 1 && nup == 1) ? -1.0 : 1.0;
		m[t][s] = sign;
	}
}

void mat_parity(Mat4 m)
{
	memset(m, 0, sizeof(Mat4));
	for (int s = 0; s < 4; s++) m[s][s] = (__builtin_popcount((unsigned)s) & 1) ? -1.0 : 1.0;
}

void mat_mul(const Mat4 a, const Mat4 b, Mat4 c)
{
	Mat4 t;
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++)
		{
			double s = 0;
			for (int k = 0; k < 4; k++) s += a[i][k] * b[k][j];
			t[i][j] = s;
		}
	memcpy(c, t, sizeof(Mat4));
}

struct Bond {
	int b = 0;
	bool has_i = false, has_d = false, left_pairs = true;
	int n_l1 = 0, n_r1 = 0, x_lo = 0, x_hi = 0;      // pair operators drawn from [x_lo, x_hi)
	int off_l1 = 0, off_p = 0, off_r1 = 0, off_d = 0, dim = 0;
	std::vector<int> pidx;                          // (x1 - x_lo) * K + (x2 - x_lo) -> pair index
	std::vector<q32> q;

	int l1(int x) const { return off_l1 + x; }
	int r1(int y) const { return off_r1 + (y - 4 * b); }
	int pair(int x1, int x2) const
	{
		const int K = x_hi - x_lo;
		return off_p + pidx[(size_t)(x1 - x_lo) * K + (x2 - x_lo)];
	}
};

Bond make_bond(int b, int n, int bstar)
{
	Bond s;
	s.b = b;
	const bool inner = b >= 1 && b <= n - 1;
	s.has_i = b <= n - 1;
	s.has_d = b >= 1;
	s.n_l1 = inner ? 4 * b : 0;
	s.n_r1 = inner ? 4 * (n - b) : 0;
	s.left_pairs = b <= bstar;
	if (inner)
	{
		s.x_lo = s.left_pairs ? 0 : 4 * b;
		s.x_hi = s.left_pairs ? 4 * b : 4 * n;
	}
	const int K = s.x_hi - s.x_lo;
	s.pidx.assign((size_t)K * K, -1);
	int np = 0;
	for (int i = 0; i < K; i++)
		for (int j = i + 1; j < K; j++) s.pidx[(size_t)i * K + j] = np++;
	int off = 0;
	if (s.has_i) off++;
	s.off_l1 = off;
	off += s.n_l1;
	s.off_p = off;
	off += np;
	s.off_r1 = off;
	off += s.n_r1;
	s.off_d = off;
	if (s.has_d) off++;
	s.dim = off;
	s.q.assign((size_t)s.dim, 0);
	for (int x = 0; x < s.n_l1; x++) s.q[(size_t)s.l1(x)] = op_qnum(x);
	for (int i = 0; i < K; i++)
		for (int j = i + 1; j < K; j++)
		{
			const q32 qq = op_qnum(s.x_lo + i) + op_qnum(s.x_lo + j);
			s.q[(size_t)s.pair(s.x_lo + i, s.x_lo + j)] = s.left_pairs ? qq : -qq;
		}
	for (int y = 4 * b; y < 4 * b + s.n_r1; y++) s.q[(size_t)s.r1(y)] = -op_qnum(y);
	return s;
}

// one site tensor, host entries in block order
struct SiteTensor {
	ctg::Meta m;
	std::vector<double> v;

	void add(int sin, int sout, double coef, const Mat4 op)
	{
		for (int a = 0; a < 4; a++)
			for (int c = 0; c < 4; c++)
			{
				if (op[a][c] == 0) continue;
				const i64 li[4] = {sin, a, c, sout};
				i64 idx[4], pos[4];
				for (int ax = 0; ax < 4; ax++)
				{
					idx[ax] = m.blk[(size_t)ax][(size_t)li[ax]];
					pos[ax] = m.pos[(size_t)ax][(size_t)li[ax]];
				}
				const int blk = m.find(idx);
				CTG_CHECK(blk >= 0, "molecular MPO: entry outside the allowed blocks");
				const i64* bd = m.dims(blk);
				const i64 off = ((pos[0] * bd[1] + pos[1]) * bd[2] + pos[2]) * bd[3] + pos[3];
				v[(size_t)(m.boff[(size_t)blk] + off)] += coef * op[a][c];
			}
	}
};

// product of the operators ops[0..k) (as written) times F^parity
void local_product(const int* ops, int k, int parity, Mat4 out)
{
	mat_identity(out);
	Mat4 t;
	for (int i = 0; i < k; i++)
	{
		mat_op(ops[i], t);
		mat_mul(out, t, out);
	}
	if (parity & 1)
	{
		mat_parity(t);
		mat_mul(out, t, out);
	}
}

}  // namespace

namespace ctg {

int build_spin_molecular_mpo(int n, const double* tkin, const double* vint, struct mpo* out)
{
	CTG_CHECK(n >= 1 && tkin && vint && out, "construct_spin_molecular_mpo: invalid arguments");
	const int bstar = n / 2;
	std::vector<Bond> bonds;
	for (int b = 0; b <= n; b++) bonds.push_back(make_bond(b, n, bstar));
	const std::vector<q32> qsite = {encode_pair(0, 0), encode_pair(1, -1), encode_pair(1, 1), encode_pair(2, 0)};
	std::vector<SiteTensor> W((size_t)n);
	for (int p = 0; p < n; p++)
	{
		const i64 dim[4] = {bonds[(size_t)p].dim, 4, 4, bonds[(size_t)p + 1].dim};
		const int dir[4] = {TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN, TENSOR_AXIS_IN};
		W[(size_t)p].m = make_meta(4, dim, dir, {bonds[(size_t)p].q, qsite, qsite, bonds[(size_t)p + 1].q});
		W[(size_t)p].v.assign((size_t)W[(size_t)p].m.nnz, 0.0);
	}

	Mat4 id, fpar, t, u;
	mat_identity(id);
	mat_parity(fpar);

	// transitions of weight 1 between L-states and between R-states
	for (int p = 0; p < n; p++)
	{
		const Bond& l = bonds[(size_t)p];
		const Bond& r = bonds[(size_t)p + 1];
		SiteTensor& w = W[(size_t)p];
		if (l.has_i && r.has_i) w.add(0, 0, 1.0, id);
		if (l.has_d && r.has_d) w.add(l.off_d, r.off_d, 1.0, id);
		// L1: pass with F; created here with x F
		if (l.n_l1 > 0 && r.n_l1 > 0)
			for (int x = 0; x < 4 * p; x++) w.add(l.l1(x), r.l1(x), 1.0, fpar);
		if (r.n_l1 > 0)
			for (int x = 4 * p; x < 4 * p + 4; x++)
			{
				local_product(&x, 1, 1, t);
				w.add(0, r.l1(x), 1.0, t);
			}
		// L2 (bond p + 1 keeps left pairs)
		if (r.n_l1 > 0 && r.left_pairs)
		{
			for (int x1 = 0; x1 < 4 * p; x1++)
				for (int x2 = x1 + 1; x2 < 4 * p; x2++)
					if (l.left_pairs && l.n_l1 > 0) w.add(l.pair(x1, x2), r.pair(x1, x2), 1.0, id);
			for (int x2 = 4 * p; x2 < 4 * p + 4; x2++)
			{
				local_product(&x2, 1, 0, t);
				if (l.n_l1 > 0)
					for (int x1 = 0; x1 < 4 * p; x1++) w.add(l.l1(x1), r.pair(x1, x2), 1.0, t);
				for (int x1 = 4 * p; x1 < x2; x1++)
				{
					const int ops[2] = {x1, x2};
					local_product(ops, 2, 0, u);
					w.add(0, r.pair(x1, x2), 1.0, u);
				}
			}
		}
		// R2 (bond p holds right pairs): pass, or place the first pending operator here
		if (l.n_r1 > 0 && !l.left_pairs)
		{
			for (int y1 = 4 * p; y1 < 4 * p + 4; y1++)
			{
				for (int y2 = y1 + 1; y2 < 4 * p + 4; y2++)
				{
					const int ops[2] = {y1, y2};
					local_product(ops, 2, 0, u);
					w.add(l.pair(y1, y2), r.off_d, 1.0, u);
				}
				if (r.n_r1 > 0)
				{
					local_product(&y1, 1, 1, t);
					for (int y2 = 4 * p + 4; y2 < 4 * n; y2++) w.add(l.pair(y1, y2), r.r1(y2), 1.0, t);
				}
			}
			if (r.n_r1 > 0)
				for (int y1 = 4 * p + 4; y1 < 4 * n; y1++)
					for (int y2 = y1 + 1; y2 < 4 * n; y2++) w.add(l.pair(y1, y2), r.pair(y1, y2), 1.0, id);
		}
		// R1: pass with F, or place the last operator here
		if (l.n_r1 > 0)
		{
			if (r.n_r1 > 0)
				for (int y = 4 * p + 4; y < 4 * n; y++) w.add(l.r1(y), r.r1(y), 1.0, fpar);
			for (int y = 4 * p; y < 4 * p + 4; y++)
			{
				local_product(&y, 1, 0, t);
				w.add(l.r1(y), r.off_d, 1.0, t);
			}
		}
	}

	// the coefficient transition of every term
	auto add_term = [&](double coef, int* x, int r) {
		if (coef == 0) return;
		// Jordan-Wigner order; creation precedes annihilation in every term, so no exchange of two
		// operators of the same spin orbital occurs
		double sign = 1;
		for (int i = 1; i < r; i++)
			for (int j = i; j > 0 && x[j - 1] > x[j]; j--)
			{
				std::swap(x[j - 1], x[j]);
				sign = -sign;
			}
		for (int i = 1; i < r; i++)
			if (x[i] == x[i - 1]) return;   // a+ a+ or a a of one spin orbital
		int s[4];
		for (int i = 0; i < r; i++) s[i] = op_site(x[i]);
		int B;
		if (r == 2) B = s[0];
		else B = bstar <= s[1] ? s[1] : std::min(s[2], bstar);
		int jin = 0, jout = 0;
		for (int i = 0; i < r; i++)
		{
			jin += s[i] < B;
			jout += s[i] <= B;
		}
		const Bond& l = bonds[(size_t)B];
		const Bond& rb = bonds[(size_t)B + 1];
		int sin, sout;
		if (jin == 0) sin = 0;
		else if (jin == 1) sin = l.l1(x[0]);
		else sin = l.pair(x[0], x[1]);
		if (jout == r) sout = rb.off_d;
		else if (jout == r - 1) sout = rb.r1(x[r - 1]);
		else sout = rb.pair(x[2], x[3]);
		Mat4 op;
		local_product(x + jin, jout - jin, jout, op);
		W[(size_t)B].add(sin, sout, sign * coef, op);
	};
	for (int i = 0; i < n; i++)
		for (int j = 0; j < n; j++)
			for (int sp = 0; sp < 2; sp++)
			{
				int x[2] = {4 * i + 2 * sp, 4 * j + 2 * sp + 1};
				add_term(tkin[(size_t)i * n + j], x, 2);
			}
	for (int i = 0; i < n; i++)
		for (int j = 0; j < n; j++)
			for (int k = 0; k < n; k++)
				for (int l = 0; l < n; l++)
				{
					const double v = vint[(((size_t)i * n + j) * n + k) * n + l];
					if (v == 0) continue;
					for (int sp = 0; sp < 2; sp++)
						for (int tp = 0; tp < 2; tp++)
						{
							int x[4] = {4 * i + 2 * sp, 4 * j + 2 * tp, 4 * l + 2 * tp + 1, 4 * k + 2 * sp + 1};
							add_term(0.5 * v, x, 4);
						}
				}

	out->nsites = n;
	out->d = 4;
	out->qsite = (qnumber*)aligned_alloc(16, 16);
	for (int i = 0; i < 4; i++) out->qsite[i] = qsite[(size_t)i];
	out->a = (struct block_sparse_tensor*)aligned_alloc(16, ((size_t)n * sizeof(struct block_sparse_tensor) + 15) & ~(size_t)15);
	memset(out->a, 0, (size_t)n * sizeof(struct block_sparse_tensor));
	for (int p = 0; p < n; p++) write_struct_host(W[(size_t)p].m, W[(size_t)p].v.data(), &out->a[p]);
	return 0;
}

}  // namespace ctg
