// ctg_dmrg.cpp - two-site DMRG driver on the device engine.
//
// Control flow follows dmrg_twosite (src/algorithm/dmrg.c:262-399): right
// normalisation, right environments, merged MPO pairs, then sweeps of
// merge -> Lanczos -> SVD split -> environment update. All tensors stay in
// HBM for the whole call; the host only handles block structure (integers)
// and, once per bond, the singular values that decide the truncation.
#include "ctg_dmrg.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace ctg {

extern thread_local double g_plan_stage[12];

namespace {

double now_s()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void* ct_alloc(size_t n)
{
	// the reference's ct_malloc contract (include/aligned_memory.h:17-29)
	void* p = aligned_alloc(16, std::max<size_t>(16, (n + 15) & ~(size_t)15));
	if (!p) throw std::bad_alloc();
	return p;
}

template <class T>
T* ct_copy(const T* src, size_t n)
{
	T* p = (T*)ct_alloc(n * sizeof(T));
	if (n) memcpy(p, src, n * sizeof(T));
	return p;
}

}  // namespace

// ------------------------------------------------------------------------------------
// boundary conversions
// ------------------------------------------------------------------------------------

Meta meta_from_struct(const struct block_sparse_tensor* t)
{
	CTG_CHECK(t->ndim >= 1, "tensor of degree 0 at the boundary");
	CTG_CHECK(t->dtype == CT_DOUBLE_REAL || t->dtype == CT_DOUBLE_COMPLEX,
	          "only double precision tensors (real or complex) are supported");
	std::vector<i64> dim(t->dim_logical, t->dim_logical + t->ndim);
	std::vector<int> dir(t->ndim);
	std::vector<std::vector<q32>> ql(t->ndim);
	for (int i = 0; i < t->ndim; i++)
	{
		dir[i] = (int)t->axis_dir[i];
		ql[i].assign(t->qnums_logical[i], t->qnums_logical[i] + dim[i]);
	}
	Meta m = make_meta(t->ndim, dim.data(), dir.data(), ql);
	for (int i = 0; i < t->ndim; i++)
	{
		CTG_CHECK(t->dim_blocks[i] == m.nb[i], "block dimensions differ from the structure rule");
		for (i64 j = 0; j < m.nb[i]; j++)
			CTG_CHECK(t->qnums_blocks[i][j] == m.qb[i][(size_t)j], "block quantum numbers differ from the structure rule");
	}
	return m;
}

DTensor tensor_from_struct(Ctx& c, const struct block_sparse_tensor* t)
{
	Meta m = meta_from_struct(t);
	const int w = t->dtype == CT_DOUBLE_COMPLEX ? 2 : 1;
	std::vector<double> host((size_t)std::max<i64>(m.nnz, 1) * w);
	for (int b = 0; b < m.nblocks; b++)
	{
		const struct dense_tensor* bl = t->blocks[m.linear(m.index(b))];
		CTG_CHECK(bl != nullptr, "missing dense block in the input tensor");
		CTG_CHECK(bl->dtype == t->dtype, "dense block of another numeric type");
		for (int i = 0; i < m.ndim; i++) CTG_CHECK(bl->dim[i] == m.dims(b)[i], "dense block shape mismatch");
		memcpy(host.data() + m.boff[b] * w, bl->data, (size_t)m.block_size(b) * w * sizeof(double));
	}
	DTensor d;
	d.meta = std::make_shared<const Meta>(std::move(m));
	d.cplx = w == 2;
	d.buf = c.upload(host.data(), host.size() * sizeof(double));
	return d;
}

void tensor_to_struct(Ctx& c, const DTensor& t, struct block_sparse_tensor* out)
{
	std::vector<double> host((size_t)std::max<i64>(t.m().nnz, 1) * t.width());
	copy_to_host(c, t, host.data());
	write_struct_host(t.m(), host.data(), out, t.cplx);
}

void write_struct_host(const Meta& m, const double* host, struct block_sparse_tensor* out, bool cplx)
{
	const int w = cplx ? 2 : 1;
	out->dtype = cplx ? CT_DOUBLE_COMPLEX : CT_DOUBLE_REAL;
	out->ndim = m.ndim;
	out->dim_logical = ct_copy(m.dim.data(), (size_t)m.ndim);
	out->dim_blocks = ct_copy(m.nb.data(), (size_t)m.ndim);
	out->axis_dir = (enum tensor_axis_direction*)ct_alloc(m.ndim * sizeof(enum tensor_axis_direction));
	for (int i = 0; i < m.ndim; i++) out->axis_dir[i] = (enum tensor_axis_direction)m.dir[i];
	out->qnums_logical = (qnumber**)ct_alloc(m.ndim * sizeof(qnumber*));
	out->qnums_blocks = (qnumber**)ct_alloc(m.ndim * sizeof(qnumber*));
	for (int i = 0; i < m.ndim; i++)
	{
		out->qnums_logical[i] = ct_copy(m.ql[i].data(), m.ql[i].size());
		out->qnums_blocks[i] = ct_copy(m.qb[i].data(), m.qb[i].size());
	}
	i64 total = 1;
	for (int i = 0; i < m.ndim; i++) total *= m.nb[i];
	out->blocks = (struct dense_tensor**)ct_alloc((size_t)total * sizeof(struct dense_tensor*));
	memset(out->blocks, 0, (size_t)total * sizeof(struct dense_tensor*));
	for (int b = 0; b < m.nblocks; b++)
	{
		struct dense_tensor* d = (struct dense_tensor*)ct_alloc(sizeof(struct dense_tensor));
		d->dtype = out->dtype;
		d->ndim = m.ndim;
		d->dim = ct_copy(m.dims(b), (size_t)m.ndim);
		d->data = ct_copy(host + m.boff[b] * w, (size_t)m.block_size(b) * w);
		out->blocks[m.linear(m.index(b))] = d;
	}
}

void free_struct(struct block_sparse_tensor* t)
{
	// delete_block_sparse_tensor (src/tensor/block_sparse_tensor.c:168-205)
	if (!t->blocks) return;
	i64 total = 1;
	for (int i = 0; i < t->ndim; i++) total *= t->dim_blocks[i];
	for (i64 k = 0; k < total; k++)
	{
		if (!t->blocks[k]) continue;
		free(t->blocks[k]->data);
		free(t->blocks[k]->dim);
		free(t->blocks[k]);
	}
	free(t->blocks);
	for (int i = 0; i < t->ndim; i++)
	{
		free(t->qnums_blocks[i]);
		free(t->qnums_logical[i]);
	}
	free(t->qnums_blocks);
	free(t->qnums_logical);
	free(t->axis_dir);
	free(t->dim_blocks);
	free(t->dim_logical);
	t->blocks = nullptr;
}

// ------------------------------------------------------------------------------------
// truncation (src/algorithm/truncation.c:110-223, von_neumann_entropy :13-31)
// ------------------------------------------------------------------------------------

TruncResult retained_bond_indices(const double* sigma, i64 n, double tol, bool relative_thresh, i64 max_vdim)
{
	TruncResult res;
	res.tol_eff = tol;
	// ascending by value; equal values in index order
	std::vector<std::pair<double, i64>> ss((size_t)n);
	for (i64 i = 0; i < n; i++) ss[(size_t)i] = {sigma[i], i};
	std::stable_sort(ss.begin(), ss.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
	double sqsum = 0;
	for (auto& p : ss) { p.first = p.first * p.first; sqsum += p.first; }
	if (sqsum == 0) return res;
	// near-tie at the bond-dimension cut: the last discarded and the first kept value (ascending order)
	// closer than the resolution of the singular values themselves (1e-12 of the largest), so that
	// rounding alone could swap them
	if (max_vdim < n && max_vdim > 0)
	{
		const double a = sigma[ss[(size_t)(n - max_vdim - 1)].second], b = sigma[ss[(size_t)(n - max_vdim)].second];
		const double smax = sigma[ss[(size_t)(n - 1)].second];
		res.near_tie = b - a <= 1e-12 * smax;
	}
	if (relative_thresh)
		for (auto& p : ss) p.first /= sqsum;
	for (size_t i = 1; i < ss.size(); i++) ss[i].first += ss[i - 1].first;
	if (max_vdim < n)
	{
		res.tol_eff = std::fmax(tol, ss[(size_t)(n - max_vdim - 1)].first);
		for (i64 i = 0; i < n - max_vdim; i++) ss[(size_t)i].first = 0;
	}
	std::vector<double> accum((size_t)n);
	for (const auto& p : ss) accum[(size_t)p.second] = p.first;
	for (i64 i = 0; i < n; i++)
		if (accum[(size_t)i] > tol) res.ind.push_back(i);
	if (res.ind.empty()) return res;
	double nrm2 = 0;
	for (i64 i : res.ind) nrm2 += sigma[i] * sigma[i];
	res.norm_sigma = std::sqrt(nrm2);
	double s = 0;
	for (i64 i : res.ind)
	{
		const double x = sigma[i] / res.norm_sigma;
		if (x > 0) s -= x * x * std::log(x * x);
	}
	res.entropy = s;
	return res;
}

// ------------------------------------------------------------------------------------
// chain operations on device tensors
// ------------------------------------------------------------------------------------

namespace {

// mps_merge_tensor_pair (src/state/mps.c:1166-1178)
DTensor merge_mps_pair(Ctx& c, const DTensor& a0, const DTensor& a1)
{
	DTensor t = op_dot(c, a0, AX_TRAILING, a1, AX_LEADING, 1);
	return op_flatten(c, t, 1, TENSOR_AXIS_OUT);
}

// mpo_merge_tensor_pair (src/operator/mpo.c:255-279)
DTensor merge_mpo_pair(Ctx& c, const DTensor& w0, const DTensor& w1)
{
	DTensor t = op_dot(c, w0, AX_TRAILING, w1, AX_LEADING, 1);
	const int perm[6] = {0, 1, 3, 2, 4, 5};
	DTensor p = op_transpose(c, t, perm);
	DTensor f = op_flatten(c, p, 1, TENSOR_AXIS_OUT);
	return op_flatten(c, f, 2, TENSOR_AXIS_IN);
}

}  // namespace

// contraction_operator_step_left (src/algorithm/chain_ops.c:196-245), with b = a
DTensor contraction_step_left(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& l, int precision)
{
	// the bra: a with reversed axis directions, complex conjugated (chain_ops.c:204-215)
	DTensor br = view_reversed(c, a);
	br.conj = a.cplx;
	DTensor s = op_dot(c, l, AX_TRAILING, br, AX_LEADING, 1, precision);
	const int p0[5] = {0, 1, 4, 2, 3};
	DTensor t = op_transpose(c, s, p0);
	s = op_dot(c, t, AX_TRAILING, w, AX_LEADING, 2, precision);
	const int p1[5] = {1, 3, 4, 2, 0};
	t = op_transpose(c, s, p1);
	s = op_dot(c, a, AX_LEADING, t, AX_LEADING, 2, precision);
	const int p2[4] = {3, 0, 1, 2};
	return op_transpose(c, s, p2);
}

// contraction_operator_step_right (src/algorithm/chain_ops.c:116-165) with ket a and bra b
DTensor contraction_step_right_ab(Ctx& c, const DTensor& a, const DTensor& b, const DTensor& w, const DTensor& r,
                                  int precision)
{
	DTensor s = op_dot(c, a, AX_TRAILING, r, AX_LEADING, 1, precision);
	const int p0[5] = {1, 2, 0, 3, 4};
	DTensor t = op_transpose(c, s, p0);
	s = op_dot(c, w, AX_TRAILING, t, AX_LEADING, 2, precision);
	const int p1[5] = {4, 2, 0, 1, 3};
	t = op_transpose(c, s, p1);
	// the bra: b with reversed axis directions, complex conjugated (chain_ops.c:138-149)
	DTensor br = view_reversed(c, b);
	br.conj = b.cplx;
	s = op_dot(c, t, AX_TRAILING, br, AX_TRAILING, 2, precision);
	const int p2[4] = {1, 2, 3, 0};
	return op_transpose(c, s, p2);
}

// contraction_operator_step_right with b = a
DTensor contraction_step_right(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& r, int precision)
{
	return contraction_step_right_ab(c, a, a, w, r, precision);
}

namespace {

// create_dummy_operator_block_right / _left (src/algorithm/chain_ops.c:14-85)
DTensor dummy_block(Ctx& c, const std::vector<q32>& qa, const std::vector<q32>& qw, const std::vector<q32>& qb, bool right,
                    bool cplx = false)
{
	const i64 dim[6] = {1, 1, 1, 1, 1, 1};
	const int dir[6] = {TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN, TENSOR_AXIS_IN, TENSOR_AXIS_IN, TENSOR_AXIS_OUT};
	Meta m = make_meta(6, dim, dir, {qa, qw, qb, qa, qw, qb});
	CTG_CHECK(m.nblocks == 1, "dummy operator block: unexpected structure");
	const double one[2] = {1.0, 0.0};
	DTensor s;
	s.meta = std::make_shared<const Meta>(std::move(m));
	s.cplx = cplx;
	s.buf = c.upload(one, (size_t)s.width() * sizeof(double));
	if (right)
	{
		DTensor t = op_flatten(c, s, 4, TENSOR_AXIS_IN);
		return op_flatten(c, t, 3, TENSOR_AXIS_IN);
	}
	DTensor t = op_flatten(c, s, 0, TENSOR_AXIS_OUT);
	return op_flatten(c, t, 0, TENSOR_AXIS_OUT);
}

// mps_local_orthonormalize_rq (src/state/mps.c:560-600)
int local_orthonormalize_rq(Ctx& c, DTensor& a, DTensor& a_prev)
{
	const Meta& am = a.m();
	const i64 dr[2] = {am.dim[1], am.dim[2]};
	const std::vector<q32> qr[2] = {am.ql[1], am.ql[2]};
	const int adr[2] = {TENSOR_AXIS_OUT, TENSOR_AXIS_IN};
	DTensor mat = op_flatten(c, a, 1, TENSOR_AXIS_IN);
	DTensor r, q;
	const int ret = op_rq(c, mat, r, q);
	a = op_split(c, q, 1, dr, adr, qr);
	a_prev = op_dot(c, a_prev, AX_TRAILING, r, AX_LEADING, 1);
	return ret;
}

// mps_local_orthonormalize_qr (src/state/mps.c:513-553)
int local_orthonormalize_qr(Ctx& c, DTensor& a, DTensor& a_next)
{
	const Meta& am = a.m();
	CTG_CHECK(am.ndim == 3 && am.dir[0] == TENSOR_AXIS_OUT && am.dir[1] == TENSOR_AXIS_OUT,
	          "mps_local_orthonormalize_qr: unexpected tensor layout");
	const i64 dl[2] = {am.dim[0], am.dim[1]};
	const std::vector<q32> ql[2] = {am.ql[0], am.ql[1]};
	const int adl[2] = {TENSOR_AXIS_OUT, TENSOR_AXIS_OUT};
	DTensor mat = op_flatten(c, a, 0, TENSOR_AXIS_OUT);
	DTensor q, r;
	const int ret = op_qr(c, mat, q, r);
	a = op_split(c, q, 0, dl, adl, ql);
	a_next = op_dot(c, r, AX_TRAILING, a_next, AX_LEADING, 1);
	return ret;
}

DTensor head_tensor(Ctx& c, const DTensor& a0, double value)
{
	const i64 dim[3] = {a0.m().dim[0], 1, a0.m().dim[0]};
	const int dir[3] = {TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN};
	Meta m = make_meta(3, dim, dir, {a0.m().ql[0], std::vector<q32>{0}, a0.m().ql[0]});
	DTensor h = c.zeros(m, a0.cplx);
	if (value != 0 && m.nblocks > 0)
	{
		std::vector<double> v((size_t)m.nnz * h.width(), 0.0);
		v[0] = value;
		h.buf = c.upload(v.data(), v.size() * sizeof(double));
	}
	return h;
}

// mps_split_tensor_svd (src/state/mps.c:1119-1159) -> split_block_sparse_matrix_svd (bond_ops.c:15-138)
int split_mps_svd(Ctx& c, const DTensor& a, i64 d, const std::vector<q32>& qsite, double tol, i64 max_vdim, bool distr_left,
                  DTensor& a0, DTensor& a1, double* entropy, std::vector<double>* kept = nullptr, long* near_ties = nullptr)
{
	const i64 dd[2] = {d, d};
	const int od[2] = {TENSOR_AXIS_OUT, TENSOR_AXIS_OUT};
	const std::vector<q32> qq[2] = {qsite, qsite};
	DTensor a4 = op_split(c, a, 1, dd, od, qq);
	DTensor tmp = op_flatten(c, a4, 0, TENSOR_AXIS_OUT);
	DTensor am = op_flatten(c, tmp, 1, TENSOR_AXIS_IN);
	SvdResult sv;
	SvdPending pend;
	// relative truncation: the discarded squares sum to at most tol ||a||_F^2; a is the normalised
	// Lanczos solution, so tol / 2 is a safe lower bound of that budget
	int ret = op_svd_launch(c, am, sv, pend, tol > 0 ? 0.5 * tol : 0.0);
	if (ret < 0) return ret;
	// the one host synchronisation of a bond step: the truncation needs the singular values
	double* sigma = c.pinned_doubles((size_t)sv.ns);
	CTG_CUDA(cudaMemcpyAsync(sigma, sv.s->ptr, (size_t)sv.ns * sizeof(double), cudaMemcpyDeviceToHost, c.stream()));
	c.sync();
	ret = op_svd_finish(c, pend);
	if (ret < 0) return ret;
	TruncResult tr = retained_bond_indices(sigma, sv.ns, tol, true, max_vdim);
	if (tr.near_tie && near_ties) (*near_ties)++;
	std::vector<double> sret;
	if (tr.ind.empty())
	{
		tr.ind = {0};
		sret = {0.0};
		tr.entropy = 0;
	}
	else
	{
		for (i64 i : tr.ind) sret.push_back(sigma[(size_t)i]);
	}
	*entropy = tr.entropy;
	if (kept) *kept = sret;
	DTensor m0 = op_slice(c, sv.u, 1, tr.ind);
	DTensor m1 = op_slice(c, sv.vh, 0, tr.ind);
	DBufPtr dsv = c.upload(sret.data(), sret.size() * sizeof(double));
	if (distr_left) m0 = op_scale_axis(c, m0, (const double*)dsv->ptr, AX_TRAILING);
	else m1 = op_scale_axis(c, m1, (const double*)dsv->ptr, AX_LEADING);
	const Meta& m4 = a4.m();
	const i64 d01[2] = {m4.dim[0], m4.dim[1]};
	const int r01[2] = {m4.dir[0], m4.dir[1]};
	const std::vector<q32> q01[2] = {m4.ql[0], m4.ql[1]};
	const i64 d23[2] = {m4.dim[2], m4.dim[3]};
	const int r23[2] = {m4.dir[2], m4.dir[3]};
	const std::vector<q32> q23[2] = {m4.ql[2], m4.ql[3]};
	a0 = op_split(c, m0, 0, d01, r01, q01);
	a1 = op_split(c, m1, 1, d23, r23, q23);
	return 0;
}

// ------------------------------------------------------------------------------------
// local Hamiltonian (apply_local_hamiltonian, src/algorithm/chain_ops.c:353-390) as a
// reusable plan: the block structure is fixed for all Lanczos iterations of one bond
// ------------------------------------------------------------------------------------

struct LocalH {
	DotPlan d1, d2, d3;
	DTensor k;                       // transpose(l, {0,3,1,2}), computed once per bond
	DTensor w, r;
	DBufPtr tt1, tt2;                // the two intermediates, in their transposed layouts
	DBufPtr pk_r, pk_w, pk_k, pk_x, pk_t1, pk_t2;   // packed tensor-core operands
	bool tc1 = false, tc2 = false, tc3 = false;     // product on the tensor cores (else FP64)
	bool f1 = false, f2 = false;     // intermediate in FP32 (written and read by tensor-core products only)
	bool z = false;                  // complex128 entries
	double flops = 0;

	LocalH(Ctx& c, const Meta& a, const DTensor& w_, const DTensor& l, const DTensor& r_, int precision) : w(w_), r(r_)
	{
		z = w.cplx || l.cplx || r.cplx;
		if (z)
		{
			CTG_CHECK(w.cplx && l.cplx && r.cplx, "local Hamiltonian: real and complex operands");
			precision = GEMM_Z64;
		}
		// the reference's transposes {1,2,0,3,4} and {2,0,1,3,4} of the first two products are written
		// by the GEMM epilogues (the results land in the transposed layouts), in FP64 and on the tensor
		// cores alike; no separate transpose pass
		const int p0[5] = {1, 2, 0, 3, 4};
		const int p1[5] = {2, 0, 1, 3, 4};
		const int p2[4] = {0, 3, 1, 2};
		d1 = make_dot_plan(c, a, AX_TRAILING, r.m(), AX_LEADING, 1, precision, p0);
		d2 = make_dot_plan(c, w.m(), AX_TRAILING, *d1.out, AX_LEADING, 2, precision, p1);
		k = op_transpose(c, l, p2);
		d3 = make_dot_plan(c, k.m(), AX_TRAILING, *d2.out, AX_LEADING, 2, precision);
		// the cyclic partial trace of the unit outer bonds keeps blocks and entries (view_trace_unit):
		// with outer axes of dimension 1, equal quantum numbers and opposite directions, the inner
		// axes obey the conservation law of a, so equal inner axes mean an equal block structure
		const Meta& o = *d3.out;
		bool same = o.ndim == a.ndim + 2 && o.dim[0] == 1 && o.dim[(size_t)o.ndim - 1] == 1 &&
		            o.dir[0] == -o.dir[(size_t)o.ndim - 1] && o.ql[0] == o.ql[(size_t)o.ndim - 1] && o.nnz == a.nnz &&
		            o.nblocks == a.nblocks;
		for (int i = 0; same && i < a.ndim; i++)
			same = o.dim[(size_t)i + 1] == a.dim[(size_t)i] && o.dir[(size_t)i + 1] == a.dir[(size_t)i] &&
			       o.ql[(size_t)i + 1] == a.ql[(size_t)i];
		CTG_CHECK(same, "local Hamiltonian output structure differs from the input");
		const size_t wz = z ? 2 : 1;
		// each product runs where its plan says: the autotuner keeps small products on FP64
		tc1 = is_tc_precision(d1.precision);
		tc2 = is_tc_precision(d2.precision);
		tc3 = is_tc_precision(d3.precision);
		// an intermediate that only feeds a tensor-core product from a tensor-core product is FP32
		// (which keeps all the bits the operand formats use): half the traffic
		f1 = tc1 && tc2;
		f2 = tc2 && tc3;
		tt1 = std::make_shared<DBuf>(&c, (size_t)std::max<i64>(d1.out->nnz, 1) * wz * (f1 ? sizeof(float) : sizeof(double)));
		tt2 = std::make_shared<DBuf>(&c, (size_t)std::max<i64>(d2.out->nnz, 1) * wz * (f2 ? sizeof(float) : sizeof(double)));
		flops = (z ? 4.0 : 1.0) * (d1.flops + d2.flops + d3.flops);
		// operands fixed for the bond (r, w, k) are packed once; x and the intermediates per apply
		auto rec = [&](i64 bytes) { return std::make_shared<DBuf>(&c, (size_t)std::max<i64>(bytes, 16)); };
		if (tc1)
		{
			pk_r = rec(d1.b_rec_bytes());
			pk_x = rec(d1.a_rec_bytes());
			d1.pack_b(c, r.data(), pk_r->ptr);
		}
		if (tc2)
		{
			pk_w = rec(d2.a_rec_bytes());
			pk_t1 = rec(d2.b_rec_bytes());
			d2.pack_a(c, w.data(), pk_w->ptr);
		}
		if (tc3)
		{
			pk_k = rec(d3.a_rec_bytes());
			pk_t2 = rec(d3.b_rec_bytes());
			d3.pack_a(c, k.data(), pk_k->ptr);
		}
	}

	void apply(Ctx& c, const double* x, double* y) const
	{
		double* t1 = (double*)tt1->ptr;
		double* t2 = (double*)tt2->ptr;
		if (z)
		{
			d1.run_z(c, x, r.data(), t1, false, false);
			d2.run_z(c, w.data(), t1, t2, false, false);
			d3.run_z(c, k.data(), t2, y, false, false);
			return;
		}
		if (tc1)
		{
			d1.pack_a(c, x, pk_x->ptr);
			d1.run_packed(c, pk_x->ptr, pk_r->ptr, t1, f1);
			c.gemm_flops += d1.flops;
		}
		else d1.run(c, x, r.data(), t1);
		if (tc2)
		{
			d2.pack_b(c, t1, pk_t1->ptr, f1);
			d2.run_packed(c, pk_w->ptr, pk_t1->ptr, t2, f2);
			c.gemm_flops += d2.flops;
		}
		else d2.run(c, w.data(), t1, t2);
		if (tc3)
		{
			d3.pack_b(c, t2, pk_t2->ptr, f2);
			d3.run_packed(c, pk_k->ptr, pk_t2->ptr, y);
			c.gemm_flops += d3.flops;
		}
		else d3.run(c, k.data(), t2, y);
	}
};

// minimize_local_energy (src/algorithm/dmrg.c:86-147) with lanczos_iteration_d and
// eigensystem_krylov_symmetric (src/util/krylov.c:24-89, :172-251) on the device
thread_local double g_host_detail[4];       // host time: local-H setup, matvecs, vector kernels, teardown

int minimize_local_energy(Ctx& c, const DTensor& w, const DTensor& l, const DTensor& r, const DTensor& a_start, int maxiter,
                          LanczosScalars* d_sc, DTensor& a_opt, DmrgStats* st, int precision)
{
	double hz = now_s();
	LocalH h(c, a_start.m(), w, l, r, precision);
	g_host_detail[0] += now_s() - hz;
	CTG_CHECK(a_start.cplx == h.z, "local eigenproblem: start vector and operator of different numeric types");
	// the vector as doubles (a complex128 vector is its real and imaginary parts: the Lanczos
	// scalars alpha = Re <v, w> and beta = ||w|| of lanczos_iteration_z are the real ones of
	// that vector, krylov.c:96-165); the breakdown test counts entries
	const i64 nent = a_start.m().nnz;
	const i64 n = nent * a_start.width();
	DBuf V(&c, (size_t)maxiter * n * sizeof(double));
	DBuf wv(&c, (size_t)n * sizeof(double));
	DBuf partial(&c, 2 * RED_BLOCKS * sizeof(double));
	double* Vp = (double*)V.ptr;
	double* wp = (double*)wv.ptr;
	double* pp = (double*)partial.ptr;
	cudaStream_t s = c.stream();
	const double dn = (double)n;
	if (g_inject_zero_start > 0)
	{
		// host-side fault injection (tests of the error path): the start vector is zeroed, so that the
		// device's own check of its norm takes the breakdown exit (status -1)
		g_inject_zero_start--;
		CTG_CUDA(cudaMemsetAsync(a_start.data(), 0, (size_t)n * sizeof(double), s));
	}
	{
		KScope ks(c, K_LANCZOS, 1, 3.0 * dn, 24.0 * dn);
		launch_lz_start(a_start.data(), Vp, n, pp, d_sc, s);
	}
	a_opt = c.empty(a_start.meta, a_start.cplx);
	for (int j = 0; j < maxiter; j++)
	{
		hz = now_s();
		h.apply(c, Vp + (i64)j * n, wp);
		g_host_detail[1] += now_s() - hz;
		hz = now_s();
		if (j < maxiter - 1)
		{
			KScope ks(c, K_LANCZOS, 1, 9.0 * dn, 72.0 * dn);
			launch_lz_step(wp, Vp + (i64)j * n, j > 0 ? Vp + (i64)(j - 1) * n : Vp, Vp + (i64)(j + 1) * n, n, nent, j, 0, pp,
			               d_sc, s);
		}
		else
		{
			// alpha of the last step, the tridiagonal eigensolve and the Ritz vector in one launch
			KScope ks(c, K_LANCZOS, 1, 2.0 * (maxiter + 1) * dn, 8.0 * (maxiter + 3) * dn);
			launch_lz_finish(wp, Vp, n, maxiter, pp, d_sc, a_opt.data(), s);
		}
		g_host_detail[2] += now_s() - hz;
	}
	if (st)
	{
		st->matvecs += maxiter;
		st->matvec_flops += h.flops * maxiter;
	}
	return 0;
}

}  // namespace

DTensor apply_local_hamiltonian_once(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& l, const DTensor& r,
                                     int precision)
{
	LocalH h(c, a.m(), w, l, r, precision);
	DTensor out = c.empty(a.meta);
	h.apply(c, a.data(), out.data());
	return out;
}

double time_local_hamiltonian(Ctx& c, const DTensor& a, const DTensor& w, const DTensor& l, const DTensor& r,
                              int precision, int nmatvec, double* flops)
{
	LocalH h(c, a.m(), w, l, r, precision);
	DTensor out = c.empty(a.meta);
	for (int i = 0; i < 3; i++) h.apply(c, a.data(), out.data());
	cudaEvent_t e[2];
	for (auto& x : e) CTG_CUDA(cudaEventCreate(&x));
	c.sync();
	CTG_CUDA(cudaEventRecord(e[0], c.stream()));
	for (int i = 0; i < nmatvec; i++) h.apply(c, a.data(), out.data());
	CTG_CUDA(cudaEventRecord(e[1], c.stream()));
	c.sync();
	float ms = 0;
	CTG_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
	for (auto& x : e) cudaEventDestroy(x);
	if (flops) *flops = h.flops;
	return ms;
}

// ------------------------------------------------------------------------------------
// dmrg_twosite
// ------------------------------------------------------------------------------------

int dmrg_twosite_gpu(const struct mpo* H, int num_sweeps, int maxiter, double tol_split, i64 max_vdim, struct mps* psi,
                     double* en_sweeps, double* entropy, const DmrgOptions& opt, DmrgStats* stats)
{
	const double t_start = now_s();
	DmrgStats local;
	DmrgStats* st = stats ? stats : &local;
	*st = DmrgStats();
	const int L = H->nsites;
	CTG_CHECK(L >= 2 && psi->nsites == L, "dmrg_twosite: need nsites >= 2 and matching MPO / MPS lengths");
	CTG_CHECK(psi->d == H->d, "dmrg_twosite: physical dimensions of MPO and MPS differ");
	CTG_CHECK(maxiter >= 1 && maxiter <= LANCZOS_MAX, "dmrg_twosite: maxiter_lanczos out of the supported range");
	CTG_CHECK(num_sweeps >= 0, "dmrg_twosite: negative number of sweeps");
	const std::vector<q32> qsite(psi->qsite, psi->qsite + psi->d);

	Ctx& c = context_for_device(opt.device);
	{
		// working set of a sweep: a few hundred times the largest two-site tensor at max_vdim
		// (MPS, environments, Lanczos basis, local-Hamiltonian intermediates, SVD workspace);
		// reserved up front so that the memory pool does not grow during the sweeps
		size_t free_b = 0, total_b = 0;
		CTG_CUDA(cudaMemGetInfo(&free_b, &total_b));
		const double two_site = 8.0 * (double)max_vdim * (double)max_vdim * (double)psi->d * (double)psi->d;
		const double want = std::min(0.25 * (double)free_b, std::max(256.0 * 1048576.0, 400.0 * two_site));
		c.reserve((size_t)want);
	}
	c.gemm_flops = 0;
	c.kernel_launches = 0;
	c.profile = false;
	c.prof_reset();
	c.svd_max_sweeps = 0;
	c.svd_flops = 0;
	c.host_plan_s = 0;
	c.host_alloc_s = 0;
	c.host_upload_s = 0;
	c.host_plan_cpu_s = 0;
	for (double& x : g_plan_stage) x = 0;
	c.plan_hits = 0;
	c.plan_misses = 0;
	for (double& x : c.svd_phase_ms) x = 0;
	for (double& x : c.svd_jacobi_cycles) x = 0;
	for (double& x : c.svd_qr_cycles) x = 0;
	for (double& x : g_host_detail) x = 0;
	DBuf sc_buf(&c, sizeof(LanczosScalars));
	LanczosScalars* d_sc = (LanczosScalars*)sc_buf.ptr;

	// upload
	std::vector<DTensor> W(L), A(L);
	for (int i = 0; i < L; i++) W[i] = tensor_from_struct(c, &H->a[i]);
	for (int i = 0; i < L; i++) A[i] = tensor_from_struct(c, &psi->a[i]);
	c.sync();
	const double t_up = now_s();
	st->upload_s = t_up - t_start;

	int ret = 0;
	// right-normalise (mps_orthonormalize_qr, src/state/mps.c:609-757)
	for (int i = L - 1; i > 0 && ret == 0; i--) ret = local_orthonormalize_rq(c, A[i], A[i - 1]);
	{
		DTensor head = head_tensor(c, A[0], 1.0);
		if (ret == 0) ret = local_orthonormalize_rq(c, A[0], head);
		std::vector<double> hv((size_t)std::max<i64>(head.m().nnz, 1) * head.width(), 0.0);
		if (head.m().nnz > 0) copy_to_host(c, head, hv.data());
		double nrm = head.m().nblocks > 0 ? hv[0] : 0.0;
		if (nrm < 0)
		{
			// flip the sign of site 0 so that the normalisation factor is non-negative
			std::vector<double> vec((size_t)A[0].m().dim[0], -1.0);
			DBufPtr mv = c.upload(vec.data(), vec.size() * sizeof(double));
			A[0] = op_scale_axis(c, A[0], (const double*)mv->ptr, AX_LEADING);
			nrm = -nrm;
		}
		if (nrm == 0) printf("Warning: in 'dmrg_twosite': initial MPS has norm zero (possibly due to mismatching quantum numbers)\n");
	}
	if (ret < 0) return ret;

	// environments and merged MPO pairs
	std::vector<DTensor> lb(L), rb(L), h2(L - 1);
	rb[L - 1] = dummy_block(c, A[L - 1].m().ql[2], W[L - 1].m().ql[3], A[L - 1].m().ql[2], true, A[L - 1].cplx);
	for (int i = L - 1; i > 0; i--) rb[i - 1] = contraction_step_right(c, A[i], W[i], rb[i]);
	lb[0] = dummy_block(c, A[0].m().ql[0], W[0].m().ql[0], A[0].m().ql[0], false, A[0].cplx);
	for (int i = 1; i < L; i++) lb[i] = lb[0];
	for (int i = 0; i < L - 1; i++) h2[i] = merge_mpo_pair(c, W[i], W[i + 1]);
	c.sync();
	const double t_setup = now_s();
	st->setup_s = t_setup - t_up;

	st->bond_sigma.assign((size_t)(L - 1), std::vector<double>());
	// four events per bond step (start, Lanczos done, split done, environment done), read at the
	// end of each sweep so that timing adds no host synchronisation
	const int nbond = 2 * (L - 1);
	std::vector<cudaEvent_t> bev((size_t)4 * nbond);
	for (auto& e : bev) CTG_CUDA(cudaEventCreate(&e));
	LanczosScalars* h_sc = c.lanczos_host();
	double host_t[3] = {0, 0, 0};             // host time enqueueing Lanczos, in the split, enqueueing environments
	auto bond_step = [&](int i, bool left_to_right, int prec, int slot) -> int {
		cudaEvent_t* ev = &bev[(size_t)4 * slot];
		const double h0 = now_s();
		CTG_CUDA(cudaEventRecord(ev[0], c.stream()));
		DTensor cur = merge_mps_pair(c, A[i], A[i + 1]);
		DTensor aopt;
		int r = minimize_local_energy(c, h2[i], lb[i], rb[i + 1], cur, maxiter, d_sc, aopt, st, prec);
		if (r < 0) return r;
		CTG_CUDA(cudaMemcpyAsync(h_sc, d_sc, sizeof(LanczosScalars), cudaMemcpyDeviceToHost, c.stream()));
		CTG_CUDA(cudaEventRecord(ev[1], c.stream()));
		const double h1 = now_s();
		double ent = 0;
		// synchronises once (for the singular values); the Lanczos scalars have arrived by then
		r = split_mps_svd(c, aopt, psi->d, qsite, tol_split, max_vdim, !left_to_right, A[i], A[i + 1], &ent,
		                  &st->bond_sigma[(size_t)i], &st->near_ties);
		if (g_inject_tridiag_failure > 0)
		{
			// host-side fault injection (tests of the error path): this eigensolve reports failure
			g_inject_tridiag_failure--;
			h_sc->status = -2;
		}
		// the Lanczos status first: the reference returns before it splits (dmrg.c:312-323)
		if (h_sc->status != 0) return h_sc->status;
		if (r < 0) return r;
		CTG_CUDA(cudaEventRecord(ev[2], c.stream()));
		const double h2 = now_s();
		// environments stay FP64 unless reduced_env is set: each one is built from its neighbour, so
		// rounding errors of a reduced-precision product accumulate along the chain (the trailing
		// FP64 sweeps rebuild them)
		const int eprec = opt.reduced_env ? prec : (int)GEMM_FP64;
		if (left_to_right) lb[i + 1] = contraction_step_left(c, A[i], W[i], lb[i], eprec);
		else
		{
			entropy[i] = ent;
			rb[i] = contraction_step_right(c, A[i + 1], W[i + 1], rb[i + 1], eprec);
		}
		CTG_CUDA(cudaEventRecord(ev[3], c.stream()));
		const double h3 = now_s();
		host_t[0] += h1 - h0;
		host_t[1] += h2 - h1;
		host_t[2] += h3 - h2;
		return 0;
	};

	std::unique_ptr<DBuf> flush;
	if (opt.l2_flush_bytes > 0) flush.reset(new DBuf(&c, (size_t)opt.l2_flush_bytes));
	cudaEvent_t sw_ev[2];
	for (auto& e : sw_ev) CTG_CUDA(cudaEventCreate(&e));
	double en = 0;
	for (int sw = 0; sw < num_sweeps && ret == 0; sw++)
	{
		// each sweep starts from an idle device (and, if requested, a flushed L2)
		if (flush) CTG_CUDA(cudaMemsetAsync(flush->ptr, sw & 0xff, flush->bytes, c.stream()));
		c.sync();
		c.profile = opt.profile && sw >= opt.profile_skip_sweeps;
		const long launches0 = c.kernel_launches;
		// reduced-precision local eigenproblems first; the trailing final_fp64_sweeps solve every
		// local eigenproblem in FP64, so the returned state and energies are FP64 results
		const int prec = sw < num_sweeps - std::max(opt.final_fp64_sweeps, 0) ? opt.precision : (int)GEMM_FP64;
		CTG_CUDA(cudaEventRecord(sw_ev[0], c.stream()));
		int slot = 0;
		for (int i = 0; i < L - 2 && ret == 0; i++) ret = bond_step(i, true, prec, slot++);
		for (int i = L - 2; i >= 0 && ret == 0; i--) ret = bond_step(i, false, prec, slot++);
		if (ret < 0) break;
		en = h_sc->lambda;
		// right-normalise the leftmost tensor (dmrg.c:366-378)
		DTensor t = head_tensor(c, A[0], 0.0);
		ret = local_orthonormalize_rq(c, A[0], t);
		en_sweeps[sw] = en;
		CTG_CUDA(cudaEventRecord(sw_ev[1], c.stream()));
		c.sync();
		float sms = 0;
		CTG_CUDA(cudaEventElapsedTime(&sms, sw_ev[0], sw_ev[1]));
		st->sweep_ms.push_back(sms);
		st->sweep_launches.push_back(c.kernel_launches - launches0);
		for (int k = 0; k < slot; k++)
		{
			const cudaEvent_t* ev = &bev[(size_t)4 * k];
			float ms = 0;
			CTG_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
			st->lanczos_ms += ms;
			CTG_CUDA(cudaEventElapsedTime(&ms, ev[1], ev[2]));
			st->split_ms += ms;
			CTG_CUDA(cudaEventElapsedTime(&ms, ev[2], ev[3]));
			st->env_ms += ms;
		}
		c.profile = false;
		st->sweeps++;
	}
	c.sync();
	c.profile = false;
	for (int k = 0; k < K_NUM_CLASSES; k++) st->prof[k] = c.prof[k];
	for (auto& e : bev) cudaEventDestroy(e);
	for (auto& e : sw_ev) cudaEventDestroy(e);
	if (getenv("CTGPU_HOST_TIMES") && st->sweeps > 0)
	{
		fprintf(stderr, "ctgpu: host ms per sweep: Lanczos enqueue %.1f, split (incl. wait) %.1f, environment enqueue %.1f\n",
		        1e3 * host_t[0] / st->sweeps, 1e3 * host_t[1] / st->sweeps, 1e3 * host_t[2] / st->sweeps);
		fprintf(stderr, "ctgpu: host ms per sweep: planning %.1f (thread CPU %.1f; device allocation %.1f, descriptor upload %.1f)\n",
		        1e3 * c.host_plan_s / st->sweeps, 1e3 * c.host_plan_cpu_s / st->sweeps, 1e3 * c.host_alloc_s / st->sweeps,
		        1e3 * c.host_upload_s / st->sweeps);
		fprintf(stderr, "ctgpu: plan stages ms per sweep:");
		for (int k = 0; k < 12; k++) fprintf(stderr, " %.1f", 1e3 * g_plan_stage[k] / st->sweeps);
		fprintf(stderr, "\n");
		fprintf(stderr, "ctgpu: host ms per sweep in Lanczos: local-H setup %.1f, matvec enqueue %.1f, vector kernels %.1f\n",
		        1e3 * g_host_detail[0] / st->sweeps, 1e3 * g_host_detail[1] / st->sweeps, 1e3 * g_host_detail[2] / st->sweeps);
	}
	const double t_sweeps = now_s();
	st->sweep_s = t_sweeps - t_setup;
	if (ret < 0) return ret;

	// hand the optimised MPS back in the reference's layout (the caller's tensors are replaced)
	for (int i = 0; i < L; i++)
	{
		free_struct(&psi->a[i]);
		tensor_to_struct(c, A[i], &psi->a[i]);
		st->max_bond_dim = std::max(st->max_bond_dim, A[i].m().dim[2]);
	}
	c.sync();
	st->download_s = now_s() - t_sweeps;
	st->kernel_launches = c.kernel_launches;
	st->total_gemm_flops = c.gemm_flops;
	st->svd_max_sweeps = c.svd_max_sweeps;
	st->host_plan_s = c.host_plan_s;
	st->plan_hits = c.plan_hits;
	st->svd_flops = c.svd_flops;
	st->plan_misses = c.plan_misses;
	if (getenv("CTGPU_SVD_PHASES") && st->sweeps > 0)
		fprintf(stderr, "ctgpu: block SVD, last-finishing block per call, ms per sweep: QR %.2f Jacobi %.2f outputs %.2f launch %.2f\n",
		        c.svd_phase_ms[0] / st->sweeps, c.svd_phase_ms[1] / st->sweeps, c.svd_phase_ms[2] / st->sweeps,
		        c.svd_phase_ms[3] / st->sweeps);
	if (getenv("CTGPU_SVD_PHASES") && st->sweeps > 0)
		fprintf(stderr, "ctgpu: Jacobi of that block, SM cycles per sweep: FP64 steps %.3g exchanges %.3g FP32 sweeps %.3g (exchanges %.3g) FP32-to-FP64 %.3g (T = R^T V %.3g); Jacobi sweeps per sweep: FP64 %.0f FP32 %.0f\n",
		        c.svd_jacobi_cycles[0] / st->sweeps, c.svd_jacobi_cycles[3] / st->sweeps, c.svd_jacobi_cycles[4] / st->sweeps,
		        c.svd_jacobi_cycles[6] / st->sweeps,
		        c.svd_jacobi_cycles[5] / st->sweeps, c.svd_jacobi_cycles[7] / st->sweeps, c.svd_jacobi_cycles[1] / st->sweeps,
		        c.svd_jacobi_cycles[2] / st->sweeps);
	if (getenv("CTGPU_SVD_PHASES") && st->sweeps > 0)
		fprintf(stderr, "ctgpu: distributed QR of that block, SM cycles per sweep: candidates %.3g reflectors %.3g exchange %.3g fetch %.3g updates %.3g\n",
		        c.svd_qr_cycles[0] / st->sweeps, c.svd_qr_cycles[1] / st->sweeps, c.svd_qr_cycles[2] / st->sweeps,
		        c.svd_qr_cycles[3] / st->sweeps, c.svd_qr_cycles[4] / st->sweeps);
	st->wall_s = now_s() - t_start;
	return 0;
}

// ------------------------------------------------------------------------------------
// mps_vdot (src/state/mps.c:314-370): <chi|psi> by contraction from the right (chi conjugated)
// ------------------------------------------------------------------------------------

void mps_vdot_gpu(const struct mps* chi, const struct mps* psi, int device, double* ret)
{
	CTG_CHECK(chi && psi && chi->nsites == psi->nsites && psi->nsites >= 1, "mps_vdot: invalid arguments");
	const int L = psi->nsites;
	CTG_CHECK(chi->a[0].dim_logical[0] == 1 && psi->a[0].dim_logical[0] == 1 &&
	              chi->a[L - 1].dim_logical[2] == 1 && psi->a[L - 1].dim_logical[2] == 1,
	          "mps_vdot: leading and trailing virtual bonds must have dimension 1");
	Ctx& c = context_for_device(device);
	// r: 1 x 1 x 1 x 1 with (OUT, IN, IN, OUT) on (psi, chi, psi, chi) trailing bonds, entry 1,
	// axes 2 and 3 flattened
	const std::vector<q32> qp(psi->a[L - 1].qnums_logical[2], psi->a[L - 1].qnums_logical[2] + 1);
	const std::vector<q32> qc(chi->a[L - 1].qnums_logical[2], chi->a[L - 1].qnums_logical[2] + 1);
	const i64 dim[4] = {1, 1, 1, 1};
	const int dir[4] = {TENSOR_AXIS_OUT, TENSOR_AXIS_IN, TENSOR_AXIS_IN, TENSOR_AXIS_OUT};
	Meta m = make_meta(4, dim, dir, {qp, qc, qp, qc});
	const bool cplx = psi->a[0].dtype == CT_DOUBLE_COMPLEX;
	CTG_CHECK(chi->a[0].dtype == psi->a[0].dtype, "mps_vdot: MPS of different numeric types");
	DTensor r;
	if (m.nblocks == 1)
	{
		const double one[2] = {1.0, 0.0};
		r.meta = std::make_shared<const Meta>(std::move(m));
		r.cplx = cplx;
		r.buf = c.upload(one, (size_t)r.width() * sizeof(double));
	}
	else r = c.zeros(m, cplx);
	r = op_flatten(c, r, 2, TENSOR_AXIS_IN);
	for (int i = L - 1; i >= 0; i--)
	{
		// mps_contraction_step_right (src/state/mps.c:279-306)
		DTensor a = tensor_from_struct(c, &psi->a[i]);
		DTensor b = tensor_from_struct(c, &chi->a[i]);
		DTensor s1 = op_dot(c, a, AX_TRAILING, r, AX_LEADING, 1);
		DTensor bc = view_reversed(c, b);
		bc.conj = b.cplx;                 // <chi| is complex conjugated
		const int perm0[4] = {3, 0, 1, 2};
		DTensor t = op_transpose(c, s1, perm0);
		DTensor s2 = op_dot(c, t, AX_TRAILING, bc, AX_TRAILING, 2);
		const int perm1[3] = {1, 2, 0};
		r = op_transpose(c, s2, perm1);
	}
	DTensor rf = op_flatten(c, r, 0, TENSOR_AXIS_OUT);
	CTG_CHECK(rf.m().ndim == 2 && rf.m().dim[0] == 1 && rf.m().dim[1] == 1, "mps_vdot: unexpected result shape");
	double v[2] = {0.0, 0.0};
	if (rf.m().nnz > 0) copy_to_host(c, rf, v);
	c.sync();
	ret[0] = v[0];
	if (cplx) ret[1] = v[1];
}

// ------------------------------------------------------------------------------------
// mpo_inner_product (src/algorithm/chain_ops.c:274-317): <chi|op|psi> by right environments
// ------------------------------------------------------------------------------------

void mpo_inner_product_gpu(const struct mps* chi, const struct mpo* op, const struct mps* psi, int device, double* ret)
{
	CTG_CHECK(chi && op && psi && op->nsites >= 1 && chi->nsites == op->nsites && psi->nsites == op->nsites,
	          "mpo_inner_product: invalid arguments");
	const int L = op->nsites;
	CTG_CHECK(chi->a[0].dim_logical[0] == 1 && op->a[0].dim_logical[0] == 1 && psi->a[0].dim_logical[0] == 1 &&
	              chi->a[L - 1].dim_logical[2] == 1 && op->a[L - 1].dim_logical[3] == 1 &&
	              psi->a[L - 1].dim_logical[2] == 1,
	          "mpo_inner_product: leading and trailing virtual bonds must have dimension 1");
	const bool cplx = psi->a[0].dtype == CT_DOUBLE_COMPLEX;
	CTG_CHECK(chi->a[0].dtype == psi->a[0].dtype && op->a[0].dtype == psi->a[0].dtype,
	          "mpo_inner_product: MPS and MPO of different numeric types");
	Ctx& c = context_for_device(device);
	const std::vector<q32> qa(psi->a[L - 1].qnums_logical[2], psi->a[L - 1].qnums_logical[2] + 1);
	const std::vector<q32> qw(op->a[L - 1].qnums_logical[3], op->a[L - 1].qnums_logical[3] + 1);
	const std::vector<q32> qb(chi->a[L - 1].qnums_logical[2], chi->a[L - 1].qnums_logical[2] + 1);
	DTensor r = dummy_block(c, qa, qw, qb, true, cplx);
	for (int i = L - 1; i >= 0; i--)
	{
		DTensor a = tensor_from_struct(c, &psi->a[i]);
		DTensor b = tensor_from_struct(c, &chi->a[i]);
		DTensor w = tensor_from_struct(c, &op->a[i]);
		r = contraction_step_right_ab(c, a, b, w, r);
	}
	// flatten the left virtual bonds: a 1 x 1 tensor remains
	DTensor t = op_flatten(c, r, 0, TENSOR_AXIS_OUT);
	t = op_flatten(c, t, 0, TENSOR_AXIS_OUT);
	CTG_CHECK(t.m().ndim == 2 && t.m().dim[0] == 1 && t.m().dim[1] == 1, "mpo_inner_product: unexpected result shape");
	double v[2] = {0.0, 0.0};
	if (t.m().nnz > 0) copy_to_host(c, t, v);
	c.sync();
	ret[0] = v[0];
	if (cplx) ret[1] = v[1];
}

// ------------------------------------------------------------------------------------
// dmrg_singlesite (src/algorithm/dmrg.c:155-254)
// ------------------------------------------------------------------------------------

int dmrg_singlesite_gpu(const struct mpo* H, int num_sweeps, int maxiter, struct mps* psi, double* en_sweeps,
                        const DmrgOptions& opt, DmrgStats* stats)
{
	const double t_start = now_s();
	DmrgStats local;
	DmrgStats* st = stats ? stats : &local;
	*st = DmrgStats();
	const int L = H->nsites;
	CTG_CHECK(L >= 1 && psi->nsites == L, "dmrg_singlesite: need nsites >= 1 and matching MPO / MPS lengths");
	CTG_CHECK(psi->d == H->d, "dmrg_singlesite: physical dimensions of MPO and MPS differ");
	CTG_CHECK(maxiter >= 1 && maxiter <= LANCZOS_MAX, "dmrg_singlesite: maxiter_lanczos out of the supported range");
	CTG_CHECK(num_sweeps >= 0, "dmrg_singlesite: negative number of sweeps");

	Ctx& c = context_for_device(opt.device);
	c.gemm_flops = 0;
	c.kernel_launches = 0;
	c.profile = false;
	std::vector<DTensor> W(L), A(L);
	for (int i = 0; i < L; i++) W[i] = tensor_from_struct(c, &H->a[i]);
	for (int i = 0; i < L; i++) A[i] = tensor_from_struct(c, &psi->a[i]);
	c.sync();
	const double t_up = now_s();
	st->upload_s = t_up - t_start;

	int ret = 0;
	// right-normalise (mps_orthonormalize_qr, src/state/mps.c:609-757)
	for (int i = L - 1; i > 0 && ret == 0; i--) ret = local_orthonormalize_rq(c, A[i], A[i - 1]);
	{
		DTensor head = head_tensor(c, A[0], 1.0);
		if (ret == 0) ret = local_orthonormalize_rq(c, A[0], head);
		std::vector<double> hv((size_t)std::max<i64>(head.m().nnz, 1) * head.width(), 0.0);
		if (head.m().nnz > 0) copy_to_host(c, head, hv.data());
		double nrm = head.m().nblocks > 0 ? hv[0] : 0.0;
		if (nrm < 0)
		{
			std::vector<double> vec((size_t)A[0].m().dim[0], -1.0);
			DBufPtr mv = c.upload(vec.data(), vec.size() * sizeof(double));
			A[0] = op_scale_axis(c, A[0], (const double*)mv->ptr, AX_LEADING);
			nrm = -nrm;
		}
		if (nrm == 0) printf("Warning: in 'dmrg_singlesite': initial MPS has norm zero (possibly due to mismatching quantum numbers)\n");
	}
	if (ret < 0) return ret;

	// environments (dmrg.c:175-182)
	std::vector<DTensor> lb(L), rb(L);
	rb[L - 1] = dummy_block(c, A[L - 1].m().ql[2], W[L - 1].m().ql[3], A[L - 1].m().ql[2], true, A[L - 1].cplx);
	for (int i = L - 1; i > 0; i--) rb[i - 1] = contraction_step_right(c, A[i], W[i], rb[i]);
	lb[0] = dummy_block(c, A[0].m().ql[0], W[0].m().ql[0], A[0].m().ql[0], false, A[0].cplx);
	for (int i = 1; i < L; i++) lb[i] = lb[0];
	c.sync();
	const double t_setup = now_s();
	st->setup_s = t_setup - t_up;

	// local optimisation of site i; the Lanczos status is checked per site as in the reference
	// every local problem of a sweep writes its Lanczos scalars to its own slot; the host reads them
	// once per sweep (no synchronisation per site: nothing on the host waits for a site's result),
	// and reports the first failing site's status as the reference would have returned it
	const int nsteps = 2 * std::max(L - 1, 0);
	DBuf steps_buf(&c, (size_t)std::max(nsteps, 1) * sizeof(LanczosScalars));
	LanczosScalars* d_steps = (LanczosScalars*)steps_buf.ptr;
	std::vector<LanczosScalars> h_steps((size_t)std::max(nsteps, 1));
	int step = 0;
	auto site_step = [&](int i) -> int {
		DTensor aopt;
		int r = minimize_local_energy(c, W[i], lb[i], rb[i], A[i], maxiter, d_steps + step, aopt, st, GEMM_FP64);
		step++;
		if (r < 0) return r;
		A[i] = aopt;
		return 0;
	};
	cudaEvent_t sw_ev[2];
	for (auto& e : sw_ev) CTG_CUDA(cudaEventCreate(&e));
	for (int sw = 0; sw < num_sweeps && ret == 0; sw++)
	{
		c.sync();
		const long launches0 = c.kernel_launches;
		CTG_CUDA(cudaEventRecord(sw_ev[0], c.stream()));
		step = 0;
		// sweep from left to right
		for (int i = 0; i < L - 1 && ret == 0; i++)
		{
			ret = site_step(i);
			if (ret < 0) break;
			ret = local_orthonormalize_qr(c, A[i], A[i + 1]);
			lb[i + 1] = contraction_step_left(c, A[i], W[i], lb[i]);
		}
		// sweep from right to left
		for (int i = L - 1; i > 0 && ret == 0; i--)
		{
			ret = site_step(i);
			if (ret < 0) break;
			ret = local_orthonormalize_rq(c, A[i], A[i - 1]);
			rb[i - 1] = contraction_step_right(c, A[i], W[i], rb[i]);
		}
		if (ret < 0) break;
		// right-normalise the leftmost tensor so that psi is normalised (dmrg.c:230-243)
		DTensor t = head_tensor(c, A[0], 0.0);
		ret = local_orthonormalize_rq(c, A[0], t);
		CTG_CUDA(cudaEventRecord(sw_ev[1], c.stream()));
		if (step > 0)
			CTG_CUDA(cudaMemcpyAsync(h_steps.data(), d_steps, (size_t)step * sizeof(LanczosScalars), cudaMemcpyDeviceToHost,
			                         c.stream()));
		c.sync();
		for (int k = 0; k < step; k++)
			if (h_steps[(size_t)k].status != 0) return h_steps[(size_t)k].status;
		en_sweeps[sw] = step > 0 ? h_steps[(size_t)step - 1].lambda : 0.0;
		float sms = 0;
		CTG_CUDA(cudaEventElapsedTime(&sms, sw_ev[0], sw_ev[1]));
		st->sweep_ms.push_back(sms);
		st->sweep_launches.push_back(c.kernel_launches - launches0);
		st->sweeps++;
	}
	for (auto& e : sw_ev) cudaEventDestroy(e);
	c.sync();
	const double t_sweeps = now_s();
	st->sweep_s = t_sweeps - t_setup;
	if (ret < 0) return ret;
	for (int i = 0; i < L; i++)
	{
		free_struct(&psi->a[i]);
		tensor_to_struct(c, A[i], &psi->a[i]);
		st->max_bond_dim = std::max(st->max_bond_dim, A[i].m().dim[2]);
	}
	c.sync();
	st->download_s = now_s() - t_sweeps;
	st->kernel_launches = c.kernel_launches;
	st->total_gemm_flops = c.gemm_flops;
	st->wall_s = now_s() - t_start;
	return 0;
}

}  // namespace ctg
