/* ct_oracle.c - CPU restatement of chemtensor's two-site DMRG path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and timed CPU baseline for the
 * GB300 implementation. The product never links, loads or calls this file.
 *
 * Each routine states which reference routine (file:line in the chemtensor
 * sources) it follows. Block-sparse tensors use the reference's own struct
 * layout (include/ct_structs.h), including its allocation contract
 * (aligned_alloc + free). Arithmetic is IEEE double; BLAS/LAPACK calls use
 * the same routines and arguments as the reference (dgemm, dgesvd,
 * dgerqf/dorgrq, dsteqr), so on the same BLAS build the results agree with
 * the reference to rounding of the OpenMP/BLAS reduction order.
 */
#include <assert.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include <time.h>
#include "ct_oracle.h"

/* ---- BLAS / LAPACK (OpenBLAS bundled with scipy: LP64, "scipy_" prefix) ---- */

enum { ROW_MAJOR = 101, NO_TRANS = 111, TRANS = 112 };
void   scipy_cblas_dgemm(int order, int ta, int tb, int m, int n, int k, double alpha, const double* a, int lda,
                         const double* b, int ldb, double beta, double* c, int ldc);
double scipy_cblas_ddot(int n, const double* x, int incx, const double* y, int incy);
double scipy_cblas_dnrm2(int n, const double* x, int incx);
void   scipy_dgesvd_(const char* jobu, const char* jobvt, const int* m, const int* n, double* a, const int* lda,
                     double* s, double* u, const int* ldu, double* vt, const int* ldvt, double* work, const int* lwork,
                     int* info, size_t, size_t);
void   scipy_dgerqf_(const int* m, const int* n, double* a, const int* lda, double* tau, double* work,
                     const int* lwork, int* info);
void   scipy_dorgrq_(const int* m, const int* n, const int* k, double* a, const int* lda, const double* tau,
                     double* work, const int* lwork, int* info);
void   scipy_dgeqrf_(const int* m, const int* n, double* a, const int* lda, double* tau, double* work,
                     const int* lwork, int* info);
void   scipy_dorgqr_(const int* m, const int* n, const int* k, double* a, const int* lda, const double* tau,
                     double* work, const int* lwork, int* info);
void   scipy_dsteqr_(const char* compz, const int* n, double* d, double* e, double* z, const int* ldz, double* work,
                     int* info, size_t);
void   scipy_openblas_set_num_threads(int);

#define AXR_LEADING  0
#define AXR_TRAILING 1

/* ---- memory: the reference's ct_malloc / ct_free (include/aligned_memory.h:17-54) ---- */

static void* xmalloc(size_t n)
{
	if (n == 0) n = 1;
	void* p = aligned_alloc(16, (n + 15) & ~(size_t)15);
	if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
	return p;
}

static void* xcalloc(size_t num, size_t size)
{
	void* p = xmalloc(num * size);
	memset(p, 0, num * size);
	return p;
}

static ct_long iprod(const ct_long* d, int n)
{
	ct_long p = 1;
	for (int i = 0; i < n; i++) p *= d[i];
	return p;
}

static void unravel(int ndim, const ct_long* dims, ct_long k, ct_long* idx)
{
	for (int i = ndim - 1; i >= 0; i--) { idx[i] = k % dims[i]; k /= dims[i]; }
}

static ct_long ravel(int ndim, const ct_long* dims, const ct_long* idx)
{
	ct_long k = 0;
	for (int i = 0; i < ndim; i++) k = k * dims[i] + idx[i];
	return k;
}

/* ---- dense blocks ---- */

static struct dense_tensor* dense_new(int ndim, const ct_long* dim)
{
	struct dense_tensor* b = xcalloc(1, sizeof(*b));
	b->dtype = CT_DOUBLE_REAL;
	b->ndim = ndim;
	b->dim = xmalloc(ndim * sizeof(ct_long));
	memcpy(b->dim, dim, ndim * sizeof(ct_long));
	b->data = xcalloc(iprod(dim, ndim) > 0 ? iprod(dim, ndim) : 1, sizeof(double));
	return b;
}

static void dense_free(struct dense_tensor* b)
{
	if (!b) return;
	free(b->data);
	free(b->dim);
	free(b);
}

/* ---- block-sparse allocation: allocate_block_sparse_tensor (block_sparse_tensor.c:37-151) ---- */

static int cmp_q(const void* a, const void* b)
{
	const qnumber x = *(const qnumber*)a, y = *(const qnumber*)b;
	return (x > y) - (x < y);
}

static void bst_alloc(int ndim, const ct_long* dim, const enum tensor_axis_direction* dir, const qnumber* const* qnums,
                      struct block_sparse_tensor* t)
{
	assert(ndim >= 1);
	t->dtype = CT_DOUBLE_REAL;
	t->ndim = ndim;
	t->dim_logical = xmalloc(ndim * sizeof(ct_long));
	memcpy(t->dim_logical, dim, ndim * sizeof(ct_long));
	t->dim_blocks = xcalloc(ndim, sizeof(ct_long));
	t->axis_dir = xmalloc(ndim * sizeof(enum tensor_axis_direction));
	memcpy(t->axis_dir, dir, ndim * sizeof(enum tensor_axis_direction));
	t->qnums_logical = xcalloc(ndim, sizeof(qnumber*));
	t->qnums_blocks = xcalloc(ndim, sizeof(qnumber*));
	ct_long** counts = xcalloc(ndim, sizeof(ct_long*));
	for (int i = 0; i < ndim; i++)
	{
		assert(dim[i] > 0);
		t->qnums_logical[i] = xmalloc(dim[i] * sizeof(qnumber));
		memcpy(t->qnums_logical[i], qnums[i], dim[i] * sizeof(qnumber));
		/* sorted unique quantum numbers */
		qnumber* u = xmalloc(dim[i] * sizeof(qnumber));
		memcpy(u, qnums[i], dim[i] * sizeof(qnumber));
		qsort(u, dim[i], sizeof(qnumber), cmp_q);
		ct_long nu = 0;
		for (ct_long j = 0; j < dim[i]; j++) {
			if (nu == 0 || u[nu - 1] != u[j]) u[nu++] = u[j];
		}
		t->dim_blocks[i] = nu;
		t->qnums_blocks[i] = xmalloc(nu * sizeof(qnumber));
		memcpy(t->qnums_blocks[i], u, nu * sizeof(qnumber));
		free(u);
		/* multiplicities */
		counts[i] = xcalloc(nu, sizeof(ct_long));
		for (ct_long j = 0; j < dim[i]; j++) {
			const qnumber* f = bsearch(&qnums[i][j], t->qnums_blocks[i], nu, sizeof(qnumber), cmp_q);
			counts[i][f - t->qnums_blocks[i]]++;
		}
	}
	const ct_long nblocks = iprod(t->dim_blocks, ndim);
	t->blocks = xcalloc(nblocks, sizeof(struct dense_tensor*));
	ct_long idx[16], bdim[16];
	for (ct_long k = 0; k < nblocks; k++)
	{
		unravel(ndim, t->dim_blocks, k, idx);
		qnumber qsum = 0;
		for (int i = 0; i < ndim; i++) qsum += dir[i] * t->qnums_blocks[i][idx[i]];
		if (qsum != 0) continue;
		for (int i = 0; i < ndim; i++) bdim[i] = counts[i][idx[i]];
		t->blocks[k] = dense_new(ndim, bdim);
	}
	for (int i = 0; i < ndim; i++) free(counts[i]);
	free(counts);
}

void oracle_delete_block_sparse_tensor(struct block_sparse_tensor* t)
{
	if (!t->blocks) return;
	const ct_long nblocks = iprod(t->dim_blocks, t->ndim);
	for (ct_long k = 0; k < nblocks; k++) dense_free(t->blocks[k]);
	free(t->blocks);
	for (int i = 0; i < t->ndim; i++) { free(t->qnums_blocks[i]); free(t->qnums_logical[i]); }
	free(t->qnums_blocks);
	free(t->qnums_logical);
	free(t->axis_dir);
	free(t->dim_blocks);
	free(t->dim_logical);
	memset(t, 0, sizeof(*t));
}

static void bst_copy(const struct block_sparse_tensor* s, struct block_sparse_tensor* t)
{
	bst_alloc(s->ndim, s->dim_logical, s->axis_dir, (const qnumber* const*)s->qnums_logical, t);
	const ct_long nblocks = iprod(s->dim_blocks, s->ndim);
	for (ct_long k = 0; k < nblocks; k++) {
		if (s->blocks[k]) {
			memcpy(t->blocks[k]->data, s->blocks[k]->data, iprod(s->blocks[k]->dim, s->ndim) * sizeof(double));
		}
	}
}

static ct_long block_index_of(const struct block_sparse_tensor* t, int ax, qnumber q)
{
	for (ct_long j = 0; j < t->dim_blocks[ax]; j++) {
		if (t->qnums_blocks[ax][j] == q) return j;
	}
	return -1;
}

/* positions of the logical indices with quantum number q along axis ax, in order */
static ct_long fanout(const struct block_sparse_tensor* t, int ax, qnumber q, ct_long* out)
{
	ct_long c = 0;
	for (ct_long j = 0; j < t->dim_logical[ax]; j++) {
		if (t->qnums_logical[ax][j] == q) out[c++] = j;
	}
	return c;
}

/* for every logical index: its position inside its quantum-number block
 * (construct_logical_to_block_index_maps, block_sparse_tensor.c:891-915) */
static ct_long* fanin(const struct block_sparse_tensor* t, int ax)
{
	ct_long* pos = xmalloc(t->dim_logical[ax] * sizeof(ct_long));
	ct_long* cnt = xcalloc(t->dim_blocks[ax], sizeof(ct_long));
	for (ct_long j = 0; j < t->dim_logical[ax]; j++) {
		const ct_long b = block_index_of(t, ax, t->qnums_logical[ax][j]);
		pos[j] = cnt[b]++;
	}
	free(cnt);
	return pos;
}

/* ---- dot: block_sparse_tensor_dot (block_sparse_tensor.c:1826-2001) with
 *      dense_tensor_dot_update (dense_tensor.c:1761-1837) ---- */

static void dense_dot_update(const struct dense_tensor* s, int axs, const struct dense_tensor* t, int axt, int nmult,
                             struct dense_tensor* r)
{
	const int nlds = (axs == AXR_LEADING ? nmult : s->ndim - nmult);
	const int nldt = (axt == AXR_LEADING ? nmult : t->ndim - nmult);
	const ct_long lds = iprod(s->dim, nlds), tds = iprod(s->dim + nlds, s->ndim - nlds);
	const ct_long ldt = iprod(t->dim, nldt), tdt = iprod(t->dim + nldt, t->ndim - nldt);
	const int ta = (axs == AXR_LEADING ? TRANS : NO_TRANS);
	const int tb = (axt == AXR_LEADING ? NO_TRANS : TRANS);
	const ct_long m = (axs == AXR_LEADING ? tds : lds);
	const ct_long n = (axt == AXR_LEADING ? tdt : ldt);
	const ct_long k = (axs == AXR_LEADING ? lds : tds);
	assert(k == (axt == AXR_LEADING ? ldt : tdt));
	scipy_cblas_dgemm(ROW_MAJOR, ta, tb, (int)m, (int)n, (int)k, 1.0, s->data, (int)tds, t->data, (int)tdt, 1.0,
	                  r->data, (int)n);
}

void oracle_block_sparse_tensor_dot(const struct block_sparse_tensor* s, int axs, const struct block_sparse_tensor* t,
                                    int axt, int nmult, struct block_sparse_tensor* r)
{
	const int shift_s = (axs == AXR_LEADING ? 0 : s->ndim - nmult);
	const int shift_t = (axt == AXR_LEADING ? 0 : t->ndim - nmult);
	const int off_s = (axs == AXR_LEADING ? nmult : 0);
	const int off_t = (axt == AXR_LEADING ? nmult : 0);
	const int nfs = s->ndim - nmult, nft = t->ndim - nmult;
	const int ndr = nfs + nft;
	assert(ndr >= 1);
	for (int i = 0; i < nmult; i++) {
		assert(s->dim_logical[shift_s + i] == t->dim_logical[shift_t + i]);
		assert(s->axis_dir[shift_s + i] == -t->axis_dir[shift_t + i]);
	}
	ct_long dim[16];
	enum tensor_axis_direction dir[16];
	const qnumber* q[16];
	for (int i = 0; i < nfs; i++) {
		dim[i] = s->dim_logical[off_s + i]; dir[i] = s->axis_dir[off_s + i]; q[i] = s->qnums_logical[off_s + i];
	}
	for (int i = 0; i < nft; i++) {
		dim[nfs + i] = t->dim_logical[off_t + i]; dir[nfs + i] = t->axis_dir[off_t + i];
		q[nfs + i] = t->qnums_logical[off_t + i];
	}
	bst_alloc(ndr, dim, dir, q, r);

	const ct_long nblocks = iprod(r->dim_blocks, ndr);
	const ct_long ncontract = iprod(t->dim_blocks + shift_t, nmult);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks; k++)
	{
		struct dense_tensor* br = r->blocks[k];
		if (!br) continue;
		ct_long ir[16], is[16], it[16], ic[16];
		unravel(ndr, r->dim_blocks, k, ir);
		for (ct_long m = 0; m < ncontract; m++)
		{
			unravel(nmult, t->dim_blocks + shift_t, m, ic);
			for (int i = 0; i < nfs; i++) is[off_s + i] = ir[i];
			for (int i = 0; i < nmult; i++) is[shift_s + i] = ic[i];
			qnumber qsum = 0;
			for (int i = 0; i < s->ndim; i++) qsum += s->axis_dir[i] * s->qnums_blocks[i][is[i]];
			if (qsum != 0) continue;
			for (int i = 0; i < nft; i++) it[off_t + i] = ir[nfs + i];
			for (int i = 0; i < nmult; i++) it[shift_t + i] = ic[i];
			const struct dense_tensor* bs = s->blocks[ravel(s->ndim, s->dim_blocks, is)];
			const struct dense_tensor* bt = t->blocks[ravel(t->ndim, t->dim_blocks, it)];
			assert(bs && bt);
			dense_dot_update(bs, axs, bt, axt, nmult, br);
		}
	}
}

/* ---- transpose: block_sparse_tensor_transpose (block_sparse_tensor.c:785-870),
 *      dense_tensor_transpose (dense_tensor.c:799-932) ---- */

static void dense_transpose(const int* perm, const struct dense_tensor* t, struct dense_tensor* r)
{
	const int nd = t->ndim;
	ct_long tstride[16], rs[16], idx[16];
	tstride[nd - 1] = 1;
	for (int i = nd - 2; i >= 0; i--) tstride[i] = tstride[i + 1] * t->dim[i + 1];
	for (int i = 0; i < nd; i++) rs[i] = tstride[perm[i]];
	const ct_long n = iprod(r->dim, nd);
	memset(idx, 0, sizeof(idx));
	const double* td = t->data;
	double* rd = r->data;
	ct_long off = 0;
	for (ct_long j = 0; j < n; j++)
	{
		rd[j] = td[off];
		for (int i = nd - 1; i >= 0; i--) {
			idx[i]++; off += rs[i];
			if (idx[i] < r->dim[i]) break;
			off -= rs[i] * idx[i]; idx[i] = 0;
		}
	}
}

void oracle_block_sparse_tensor_transpose(const int* perm, const struct block_sparse_tensor* t, struct block_sparse_tensor* r)
{
	const int nd = t->ndim;
	ct_long dim[16];
	enum tensor_axis_direction dir[16];
	const qnumber* q[16];
	for (int i = 0; i < nd; i++) {
		dim[i] = t->dim_logical[perm[i]]; dir[i] = t->axis_dir[perm[i]]; q[i] = t->qnums_logical[perm[i]];
	}
	bst_alloc(nd, dim, dir, q, r);
	const ct_long nblocks = iprod(t->dim_blocks, nd);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks; k++)
	{
		const struct dense_tensor* bt = t->blocks[k];
		if (!bt) continue;
		ct_long it[16], ir[16];
		unravel(nd, t->dim_blocks, k, it);
		for (int i = 0; i < nd; i++) ir[i] = it[perm[i]];
		struct dense_tensor* br = r->blocks[ravel(nd, r->dim_blocks, ir)];
		assert(br);
		dense_transpose(perm, bt, br);
	}
}

/* ---- flatten two neighbouring axes (block_sparse_tensor.c:950-1112) ---- */

static void bst_flatten(const struct block_sparse_tensor* t, int ax, enum tensor_axis_direction newdir,
                        struct block_sparse_tensor* r)
{
	const int nd = t->ndim;
	ct_long dim[16];
	enum tensor_axis_direction dir[16];
	const qnumber* q[16];
	const ct_long d0 = t->dim_logical[ax], d1 = t->dim_logical[ax + 1];
	qnumber* qf = xmalloc(d0 * d1 * sizeof(qnumber));
	for (ct_long j = 0; j < d0; j++)
		for (ct_long k = 0; k < d1; k++)
			qf[j * d1 + k] = newdir * (t->axis_dir[ax] * t->qnums_logical[ax][j] + t->axis_dir[ax + 1] * t->qnums_logical[ax + 1][k]);
	for (int i = 0; i < ax; i++) { dim[i] = t->dim_logical[i]; dir[i] = t->axis_dir[i]; q[i] = t->qnums_logical[i]; }
	dim[ax] = d0 * d1; dir[ax] = newdir; q[ax] = qf;
	for (int i = ax + 2; i < nd; i++) { dim[i - 1] = t->dim_logical[i]; dir[i - 1] = t->axis_dir[i]; q[i - 1] = t->qnums_logical[i]; }
	bst_alloc(nd - 1, dim, dir, q, r);
	free(qf);

	ct_long* pos_r = fanin(r, ax);
	const ct_long nblocks = iprod(t->dim_blocks, nd);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks; k++)
	{
		const struct dense_tensor* bt = t->blocks[k];
		if (!bt) continue;
		ct_long it[16], ir[16];
		unravel(nd, t->dim_blocks, k, it);
		const qnumber q0 = t->qnums_blocks[ax][it[ax]], q1 = t->qnums_blocks[ax + 1][it[ax + 1]];
		const qnumber qflat = newdir * (t->axis_dir[ax] * q0 + t->axis_dir[ax + 1] * q1);
		for (int i = 0; i < ax; i++) ir[i] = it[i];
		ir[ax] = block_index_of(r, ax, qflat);
		assert(ir[ax] >= 0);
		for (int i = ax + 2; i < nd; i++) ir[i - 1] = it[i];
		struct dense_tensor* br = r->blocks[ravel(nd - 1, r->dim_blocks, ir)];
		assert(br);
		ct_long* f0 = xmalloc(bt->dim[ax] * sizeof(ct_long));
		ct_long* f1 = xmalloc(bt->dim[ax + 1] * sizeof(ct_long));
		fanout(t, ax, q0, f0);
		fanout(t, ax + 1, q1, f1);
		const ct_long stride = iprod(bt->dim + ax + 2, nd - ax - 2);
		const ct_long nlead = iprod(bt->dim, ax);
		const ct_long b0 = bt->dim[ax], b1 = bt->dim[ax + 1];
		const ct_long rdim_ax = br->dim[ax];
		for (ct_long p = 0; p < nlead; p++)
			for (ct_long j0 = 0; j0 < b0; j0++)
				for (ct_long j1 = 0; j1 < b1; j1++)
				{
					const ct_long dst = pos_r[f0[j0] * d1 + f1[j1]];
					memcpy((double*)br->data + ((p * rdim_ax + dst) * stride),
					       (const double*)bt->data + (((p * b0 + j0) * b1 + j1) * stride), stride * sizeof(double));
				}
		free(f0);
		free(f1);
	}
	free(pos_r);
}

/* ---- split an axis in two (block_sparse_tensor.c:1123-1285) ---- */

static void bst_split(const struct block_sparse_tensor* t, int ax, const ct_long nd2[2], const enum tensor_axis_direction nd2dir[2],
                      const qnumber* const nq[2], struct block_sparse_tensor* r)
{
	const int nd = t->ndim;
	assert(nd2[0] * nd2[1] == t->dim_logical[ax]);
	ct_long dim[16];
	enum tensor_axis_direction dir[16];
	const qnumber* q[16];
	for (int i = 0; i < ax; i++) { dim[i] = t->dim_logical[i]; dir[i] = t->axis_dir[i]; q[i] = t->qnums_logical[i]; }
	dim[ax] = nd2[0]; dir[ax] = nd2dir[0]; q[ax] = nq[0];
	dim[ax + 1] = nd2[1]; dir[ax + 1] = nd2dir[1]; q[ax + 1] = nq[1];
	for (int i = ax + 1; i < nd; i++) { dim[i + 1] = t->dim_logical[i]; dir[i + 1] = t->axis_dir[i]; q[i + 1] = t->qnums_logical[i]; }
	bst_alloc(nd + 1, dim, dir, q, r);

	ct_long* pos_t = fanin(t, ax);
	const ct_long nblocks = iprod(r->dim_blocks, nd + 1);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks; k++)
	{
		struct dense_tensor* br = r->blocks[k];
		if (!br) continue;
		ct_long ir[16], it[16];
		unravel(nd + 1, r->dim_blocks, k, ir);
		const qnumber q0 = r->qnums_blocks[ax][ir[ax]], q1 = r->qnums_blocks[ax + 1][ir[ax + 1]];
		const qnumber qflat = t->axis_dir[ax] * (r->axis_dir[ax] * q0 + r->axis_dir[ax + 1] * q1);
		for (int i = 0; i < ax; i++) it[i] = ir[i];
		it[ax] = block_index_of(t, ax, qflat);
		assert(it[ax] >= 0);
		for (int i = ax + 1; i < nd; i++) it[i] = ir[i + 1];
		const struct dense_tensor* bt = t->blocks[ravel(nd, t->dim_blocks, it)];
		assert(bt);
		ct_long* f0 = xmalloc(br->dim[ax] * sizeof(ct_long));
		ct_long* f1 = xmalloc(br->dim[ax + 1] * sizeof(ct_long));
		fanout(r, ax, q0, f0);
		fanout(r, ax + 1, q1, f1);
		const ct_long stride = iprod(br->dim + ax + 2, nd - ax - 1);
		const ct_long nlead = iprod(br->dim, ax);
		const ct_long b0 = br->dim[ax], b1 = br->dim[ax + 1];
		const ct_long tdim_ax = bt->dim[ax];
		for (ct_long p = 0; p < nlead; p++)
			for (ct_long j0 = 0; j0 < b0; j0++)
				for (ct_long j1 = 0; j1 < b1; j1++)
				{
					const ct_long src = pos_t[f0[j0] * nd2[1] + f1[j1]];
					memcpy((double*)br->data + (((p * b0 + j0) * b1 + j1) * stride),
					       (const double*)bt->data + ((p * tdim_ax + src) * stride), stride * sizeof(double));
				}
		free(f0);
		free(f1);
	}
	free(pos_t);
}

/* ---- slice along an axis (block_sparse_tensor.c:1446-1553) ---- */

static void bst_slice(const struct block_sparse_tensor* t, int ax, const ct_long* ind, ct_long nind, struct block_sparse_tensor* r)
{
	const int nd = t->ndim;
	ct_long dim[16];
	const qnumber* q[16];
	qnumber* qs = xmalloc(nind * sizeof(qnumber));
	for (ct_long j = 0; j < nind; j++) qs[j] = t->qnums_logical[ax][ind[j]];
	for (int i = 0; i < nd; i++) { dim[i] = t->dim_logical[i]; q[i] = t->qnums_logical[i]; }
	dim[ax] = nind; q[ax] = qs;
	bst_alloc(nd, dim, t->axis_dir, q, r);
	free(qs);
	ct_long* pos_t = fanin(t, ax);
	const ct_long nblocks = iprod(r->dim_blocks, nd);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks; k++)
	{
		struct dense_tensor* br = r->blocks[k];
		if (!br) continue;
		ct_long ir[16], it[16];
		unravel(nd, r->dim_blocks, k, ir);
		const qnumber qn = r->qnums_blocks[ax][ir[ax]];
		memcpy(it, ir, nd * sizeof(ct_long));
		it[ax] = block_index_of(t, ax, qn);
		const struct dense_tensor* bt = t->blocks[ravel(nd, t->dim_blocks, it)];
		assert(bt);
		ct_long* fr = xmalloc(br->dim[ax] * sizeof(ct_long));
		fanout(r, ax, qn, fr);
		const ct_long stride = iprod(br->dim + ax + 1, nd - ax - 1);
		const ct_long nlead = iprod(br->dim, ax);
		for (ct_long p = 0; p < nlead; p++)
			for (ct_long j = 0; j < br->dim[ax]; j++)
			{
				const ct_long src = pos_t[ind[fr[j]]];
				memcpy((double*)br->data + ((p * br->dim[ax] + j) * stride),
				       (const double*)bt->data + ((p * bt->dim[ax] + src) * stride), stride * sizeof(double));
			}
		free(fr);
	}
	free(pos_t);
}

/* ---- cyclic partial trace (block_sparse_tensor.c:1560-1611; dense_tensor.c:269-344) ---- */

static void bst_cyclic_partial_trace(const struct block_sparse_tensor* t, int ntr, struct block_sparse_tensor* r)
{
	const int ndr = t->ndim - 2 * ntr;
	bst_alloc(ndr, t->dim_logical + ntr, t->axis_dir + ntr, (const qnumber* const*)(t->qnums_logical + ntr), r);
	const ct_long nblocks_r = iprod(r->dim_blocks, ndr);
	const ct_long nblocks_p = iprod(t->dim_blocks, ntr);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks_r; k++)
	{
		struct dense_tensor* br = r->blocks[k];
		if (!br) continue;
		ct_long it[16], ip[16];
		unravel(ndr, r->dim_blocks, k, it + ntr);
		for (ct_long j = 0; j < nblocks_p; j++)
		{
			unravel(ntr, t->dim_blocks, j, ip);
			for (int i = 0; i < ntr; i++) { it[i] = ip[i]; it[ntr + ndr + i] = ip[i]; }
			const struct dense_tensor* bt = t->blocks[ravel(t->ndim, t->dim_blocks, it)];
			assert(bt);
			const ct_long stride = iprod(bt->dim, ntr);
			const ct_long nr = iprod(br->dim, ndr);
			const double* td = bt->data;
			double* rd = br->data;
			for (ct_long p = 0; p < stride; p++)
				for (ct_long jj = 0; jj < nr; jj++)
					rd[jj] += td[(p * nr + jj) * stride + p];
		}
	}
}

/* ---- pointwise multiply along leading / trailing axis (block_sparse_tensor.c:1654-1703) ---- */

static void bst_scale_axis(const struct block_sparse_tensor* s, const double* vec, int axrange, struct block_sparse_tensor* r)
{
	const int nd = s->ndim;
	const int ax = (axrange == AXR_LEADING ? 0 : nd - 1);
	bst_alloc(nd, s->dim_logical, s->axis_dir, (const qnumber* const*)s->qnums_logical, r);
	const ct_long nblocks = iprod(r->dim_blocks, nd);
	#pragma omp parallel for schedule(dynamic)
	for (ct_long k = 0; k < nblocks; k++)
	{
		struct dense_tensor* br = r->blocks[k];
		if (!br) continue;
		const struct dense_tensor* bs = s->blocks[k];
		ct_long ir[16];
		unravel(nd, r->dim_blocks, k, ir);
		ct_long* f = xmalloc(br->dim[ax] * sizeof(ct_long));
		fanout(r, ax, r->qnums_blocks[ax][ir[ax]], f);
		const ct_long n = iprod(br->dim, nd);
		const ct_long inner = iprod(br->dim + ax + 1, nd - ax - 1);
		const double* sd = bs->data;
		double* rd = br->data;
		for (ct_long j = 0; j < n; j++) {
			const ct_long a = (j / inner) % br->dim[ax];
			rd[j] = sd[j] * vec[f[a]];
		}
		free(f);
	}
}

/* ---- dense SVD and RQ with the reference's LAPACK calls ---- */

/* dense_tensor_svd_fill (dense_tensor.c:3538-3680), real double case */
static int dense_svd(const struct dense_tensor* a, struct dense_tensor* u, double* s, struct dense_tensor* vh)
{
	const int m = (int)a->dim[0], n = (int)a->dim[1];
	const int k = m < n ? m : n;
	int info, lwork = -1;
	double wsz;
	if (m >= n)
	{
		memcpy(u->data, a->data, (size_t)m * n * sizeof(double));
		scipy_dgesvd_("S", "O", &n, &m, NULL, &k, NULL, NULL, &n, NULL, &k, &wsz, &lwork, &info, 1, 1);
		if (info != 0) return -1;
		lwork = (int)wsz;
		double* work = xmalloc((size_t)lwork * sizeof(double));
		scipy_dgesvd_("S", "O", &n, &m, u->data, &n, s, vh->data, &n, NULL, &k, work, &lwork, &info, 1, 1);
		free(work);
	}
	else
	{
		memcpy(vh->data, a->data, (size_t)m * n * sizeof(double));
		scipy_dgesvd_("O", "S", &n, &m, NULL, &n, NULL, NULL, &n, NULL, &k, &wsz, &lwork, &info, 1, 1);
		if (info != 0) return -1;
		lwork = (int)wsz;
		double* work = xmalloc((size_t)lwork * sizeof(double));
		scipy_dgesvd_("O", "S", &n, &m, vh->data, &n, s, NULL, &n, u->data, &k, work, &lwork, &info, 1, 1);
		free(work);
	}
	return info == 0 ? 0 : -1;
}

/* dense_tensor_rq_fill (dense_tensor.c:2680-2880), QR_REDUCED, real double case */
static int dense_rq(const struct dense_tensor* a, struct dense_tensor* r, struct dense_tensor* q)
{
	const int m = (int)a->dim[0], n = (int)a->dim[1];
	const int k = m < n ? m : n;
	const int l = k;
	const int ldt = m;
	const int tshift_col = n > m ? n - m : 0;
	double* tau = xmalloc(k * sizeof(double));
	double* t = xcalloc((size_t)ldt * n, sizeof(double));
	const double* ad = a->data;
	for (int i = 0; i < m; i++)
		for (int j = 0; j < n; j++) t[i + (size_t)ldt * j] = ad[(size_t)i * n + j];
	int info, lwork = -1;
	double wsz;
	scipy_dgerqf_(&m, &n, NULL, &ldt, NULL, &wsz, &lwork, &info);
	if (info != 0) { free(t); free(tau); return -1; }
	lwork = (int)wsz;
	double* work = xmalloc((size_t)lwork * sizeof(double));
	scipy_dgerqf_(&m, &n, t, &ldt, tau, work, &lwork, &info);
	free(work);
	if (info != 0) { free(t); free(tau); return -1; }
	double* rd = r->data;
	const int rshift_row = m > l ? m - l : 0;
	const int rshift_col = l > m ? l - m : 0;
	for (int i = 0; i < m; i++)
	{
		int numzero = rshift_col + (i - rshift_row > 0 ? i - rshift_row : 0);
		for (int j = 0; j < numzero; j++) rd[(size_t)i * l + j] = 0;
		for (int j = numzero; j < l; j++) rd[(size_t)i * l + j] = t[i + (size_t)ldt * (tshift_col + j)];
	}
	lwork = -1;
	scipy_dorgrq_(&l, &n, &k, NULL, &ldt, NULL, &wsz, &lwork, &info);
	if (info != 0) { free(t); free(tau); return -2; }
	lwork = (int)wsz;
	work = xmalloc((size_t)lwork * sizeof(double));
	scipy_dorgrq_(&l, &n, &k, t + rshift_row, &ldt, tau, work, &lwork, &info);
	free(work);
	if (info != 0) { free(t); free(tau); return -2; }
	double* qd = q->data;
	for (int i = 0; i < l; i++)
		for (int j = 0; j < n; j++) qd[(size_t)i * n + j] = t[rshift_row + i + (size_t)ldt * j];
	free(t);
	free(tau);
	return 0;
}

/* dense_tensor_qr_fill (dense_tensor.c:2253-2651), QR_REDUCED, real double case */
static int dense_qr(const struct dense_tensor* a, struct dense_tensor* q, struct dense_tensor* r)
{
	const int m = (int)a->dim[0], n = (int)a->dim[1];
	const int k = m < n ? m : n;
	const int l = k;
	double* tau = xmalloc(k * sizeof(double));
	double* t = xcalloc((size_t)m * n, sizeof(double));
	const double* ad = a->data;
	for (int i = 0; i < m; i++)
		for (int j = 0; j < n; j++) t[i + (size_t)m * j] = ad[(size_t)i * n + j];
	int info, lwork = -1;
	double wsz;
	scipy_dgeqrf_(&m, &n, NULL, &m, NULL, &wsz, &lwork, &info);
	if (info != 0) { free(t); free(tau); return -1; }
	lwork = (int)wsz;
	double* work = xmalloc((size_t)lwork * sizeof(double));
	scipy_dgeqrf_(&m, &n, t, &m, tau, work, &lwork, &info);
	free(work);
	if (info != 0) { free(t); free(tau); return -1; }
	double* rd = r->data;
	for (int i = 0; i < l; i++)
	{
		const int numzero = i < n ? i : n;
		for (int j = 0; j < numzero; j++) rd[(size_t)i * n + j] = 0;
		for (int j = numzero; j < n; j++) rd[(size_t)i * n + j] = t[i + (size_t)m * j];
	}
	lwork = -1;
	scipy_dorgqr_(&m, &l, &k, NULL, &m, NULL, &wsz, &lwork, &info);
	if (info != 0) { free(t); free(tau); return -2; }
	lwork = (int)wsz;
	work = xmalloc((size_t)lwork * sizeof(double));
	scipy_dorgqr_(&m, &l, &k, t, &m, tau, work, &lwork, &info);
	free(work);
	if (info != 0) { free(t); free(tau); return -2; }
	double* qd = q->data;
	for (int i = 0; i < m; i++)
		for (int j = 0; j < l; j++) qd[(size_t)i * l + j] = t[i + (size_t)m * j];
	free(t);
	free(tau);
	return 0;
}

/* block_sparse_tensor_svd (block_sparse_tensor.c:2686-2848) */
int oracle_block_sparse_tensor_svd(const struct block_sparse_tensor* a, struct block_sparse_tensor* u, double** s_out,
                                   ct_long* ns, struct block_sparse_tensor* vh)
{
	assert(a->ndim == 2);
	ct_long dim_interm = 0;
	qnumber* qi = xcalloc(a->dim_logical[1] + 1, sizeof(qnumber));
	for (ct_long j = 0; j < a->dim_blocks[1]; j++)
		for (ct_long i = 0; i < a->dim_blocks[0]; i++)
		{
			if (a->axis_dir[0] * a->qnums_blocks[0][i] + a->axis_dir[1] * a->qnums_blocks[1][j] != 0) continue;
			const struct dense_tensor* b = a->blocks[i * a->dim_blocks[1] + j];
			const ct_long k = b->dim[0] < b->dim[1] ? b->dim[0] : b->dim[1];
			for (ct_long l = 0; l < k; l++) qi[dim_interm + l] = a->qnums_blocks[1][j];
			dim_interm += k;
		}
	int dummy = 0;
	if (dim_interm == 0)
	{
		dummy = 1;
		dim_interm = 1;
		qi[0] = -a->axis_dir[0] * a->axis_dir[1] * a->qnums_blocks[0][0];
	}
	const ct_long dim_u[2] = { a->dim_logical[0], dim_interm };
	const qnumber* qu[2] = { a->qnums_logical[0], qi };
	bst_alloc(2, dim_u, a->axis_dir, qu, u);
	double* s = xcalloc(dim_interm, sizeof(double));
	const ct_long dim_vh[2] = { dim_interm, a->dim_logical[1] };
	const enum tensor_axis_direction dvh[2] = { -a->axis_dir[1], a->axis_dir[1] };
	const qnumber* qv[2] = { qi, a->qnums_logical[1] };
	bst_alloc(2, dim_vh, dvh, qv, vh);
	free(qi);
	*s_out = s;
	*ns = dim_interm;
	if (dummy)
	{
		const qnumber q0 = a->qnums_blocks[0][0];
		const qnumber q1 = -a->axis_dir[0] * a->axis_dir[1] * q0;
		const ct_long j = block_index_of(u, 1, q1);
		((double*)u->blocks[0 * u->dim_blocks[1] + j]->data)[0] = 1.0;
		return 0;
	}
	int failed = 0;
	#pragma omp parallel for schedule(dynamic) collapse(2)
	for (ct_long i = 0; i < a->dim_blocks[0]; i++)
		for (ct_long j = 0; j < a->dim_blocks[1]; j++)
		{
			const struct dense_tensor* ba = a->blocks[i * a->dim_blocks[1] + j];
			if (!ba) continue;
			const ct_long kb = block_index_of(u, 1, a->qnums_blocks[1][j]);
			struct dense_tensor* bu = u->blocks[i * u->dim_blocks[1] + kb];
			struct dense_tensor* bv = vh->blocks[kb * vh->dim_blocks[1] + j];
			ct_long first;
			for (first = 0; first < u->dim_logical[1]; first++)
				if (u->qnums_logical[1][first] == a->qnums_blocks[1][j]) break;
			if (dense_svd(ba, bu, s + first, bv) != 0) failed = 1;
		}
	return failed ? -1 : 0;
}

/* block_sparse_tensor_rq (block_sparse_tensor.c:2544-2676), QR_REDUCED */
static int bst_rq(const struct block_sparse_tensor* a, struct block_sparse_tensor* r, struct block_sparse_tensor* q)
{
	assert(a->ndim == 2);
	ct_long dim_interm = 0;
	qnumber* qi = xcalloc(a->dim_logical[1] + 1, sizeof(qnumber));
	for (ct_long i = 0; i < a->dim_blocks[0]; i++)
		for (ct_long j = 0; j < a->dim_blocks[1]; j++)
		{
			if (a->axis_dir[0] * a->qnums_blocks[0][i] + a->axis_dir[1] * a->qnums_blocks[1][j] != 0) continue;
			const struct dense_tensor* b = a->blocks[i * a->dim_blocks[1] + j];
			const ct_long k = b->dim[0] < b->dim[1] ? b->dim[0] : b->dim[1];
			for (ct_long l = 0; l < k; l++) qi[dim_interm + l] = a->qnums_blocks[0][i];
			dim_interm += k;
		}
	int dummy = 0;
	if (dim_interm == 0)
	{
		dummy = 1;
		dim_interm = 1;
		qi[0] = -a->axis_dir[0] * a->axis_dir[1] * a->qnums_blocks[1][0];
	}
	const ct_long dim_r[2] = { a->dim_logical[0], dim_interm };
	const enum tensor_axis_direction dr[2] = { a->axis_dir[0], -a->axis_dir[0] };
	const qnumber* qr_[2] = { a->qnums_logical[0], qi };
	bst_alloc(2, dim_r, dr, qr_, r);
	const ct_long dim_q[2] = { dim_interm, a->dim_logical[1] };
	const qnumber* qq[2] = { qi, a->qnums_logical[1] };
	bst_alloc(2, dim_q, a->axis_dir, qq, q);
	free(qi);
	if (dummy)
	{
		const qnumber q1 = a->qnums_blocks[1][0];
		const qnumber q0 = -a->axis_dir[0] * a->axis_dir[1] * q1;
		const ct_long i0 = block_index_of(q, 0, q0);
		((double*)q->blocks[i0 * q->dim_blocks[1] + 0]->data)[0] = 1.0;
		return 0;
	}
	int failed = 0;
	#pragma omp parallel for schedule(dynamic) collapse(2)
	for (ct_long i = 0; i < a->dim_blocks[0]; i++)
		for (ct_long j = 0; j < a->dim_blocks[1]; j++)
		{
			const struct dense_tensor* ba = a->blocks[i * a->dim_blocks[1] + j];
			if (!ba) continue;
			const ct_long kb = block_index_of(q, 0, a->qnums_blocks[0][i]);
			struct dense_tensor* br = r->blocks[i * r->dim_blocks[1] + kb];
			struct dense_tensor* bq = q->blocks[kb * q->dim_blocks[1] + j];
			if (dense_rq(ba, br, bq) != 0) failed = 1;
		}
	return failed ? -1 : 0;
}

/* block_sparse_tensor_qr (block_sparse_tensor.c:2402-2540), QR_REDUCED */
static int bst_qr(const struct block_sparse_tensor* a, struct block_sparse_tensor* q, struct block_sparse_tensor* r)
{
	assert(a->ndim == 2);
	ct_long dim_interm = 0;
	qnumber* qi = xcalloc(a->dim_logical[0] + 1, sizeof(qnumber));
	for (ct_long j = 0; j < a->dim_blocks[1]; j++)
		for (ct_long i = 0; i < a->dim_blocks[0]; i++)
		{
			if (a->axis_dir[0] * a->qnums_blocks[0][i] + a->axis_dir[1] * a->qnums_blocks[1][j] != 0) continue;
			const struct dense_tensor* b = a->blocks[i * a->dim_blocks[1] + j];
			const ct_long k = b->dim[0] < b->dim[1] ? b->dim[0] : b->dim[1];
			for (ct_long l = 0; l < k; l++) qi[dim_interm + l] = a->qnums_blocks[1][j];
			dim_interm += k;
		}
	int dummy = 0;
	if (dim_interm == 0)
	{
		dummy = 1;
		dim_interm = 1;
		qi[0] = -a->axis_dir[0] * a->axis_dir[1] * a->qnums_blocks[0][0];
	}
	const ct_long dim_q[2] = { a->dim_logical[0], dim_interm };
	const qnumber* qq[2] = { a->qnums_logical[0], qi };
	bst_alloc(2, dim_q, a->axis_dir, qq, q);
	const ct_long dim_r[2] = { dim_interm, a->dim_logical[1] };
	const enum tensor_axis_direction dr[2] = { -a->axis_dir[1], a->axis_dir[1] };
	const qnumber* qr_[2] = { qi, a->qnums_logical[1] };
	bst_alloc(2, dim_r, dr, qr_, r);
	free(qi);
	if (dummy)
	{
		const qnumber q0 = a->qnums_blocks[0][0];
		const qnumber q1 = -a->axis_dir[0] * a->axis_dir[1] * q0;
		const ct_long j1 = block_index_of(q, 1, q1);
		((double*)q->blocks[0 * q->dim_blocks[1] + j1]->data)[0] = 1.0;
		return 0;
	}
	int failed = 0;
	#pragma omp parallel for schedule(dynamic) collapse(2)
	for (ct_long i = 0; i < a->dim_blocks[0]; i++)
		for (ct_long j = 0; j < a->dim_blocks[1]; j++)
		{
			const struct dense_tensor* ba = a->blocks[i * a->dim_blocks[1] + j];
			if (!ba) continue;
			const ct_long kb = block_index_of(q, 1, a->qnums_blocks[1][j]);
			struct dense_tensor* bq = q->blocks[i * q->dim_blocks[1] + kb];
			struct dense_tensor* br = r->blocks[kb * r->dim_blocks[1] + j];
			if (dense_qr(ba, bq, br) != 0) failed = 1;
		}
	return failed ? -1 : 0;
}

int oracle_block_sparse_tensor_qr(const struct block_sparse_tensor* a, struct block_sparse_tensor* q,
                                  struct block_sparse_tensor* r)
{
	return bst_qr(a, q, r);
}

int oracle_block_sparse_tensor_rq(const struct block_sparse_tensor* a, struct block_sparse_tensor* r,
                                  struct block_sparse_tensor* q)
{
	return bst_rq(a, r, q);
}

/* ---- truncation: retained_bond_indices (truncation.c:110-223), von_neumann_entropy (:13-31) ---- */

struct vi { double v; ct_long i; };

static int cmp_vi(const void* a, const void* b)
{
	const struct vi* x = a;
	const struct vi* y = b;
	if (x->v < y->v) return -1;
	if (y->v < x->v) return 1;
	/* equal values keep their original order (the reference's glibc qsort is a stable merge sort) */
	return (x->i > y->i) - (x->i < y->i);
}

ct_long oracle_retained_bond_indices(const double* sigma, ct_long n, double tol, int relative_thresh, ct_long max_vdim,
                                     ct_long* ind, double* norm_sigma, double* entropy, double* tol_eff)
{
	*tol_eff = tol;
	struct vi* ss = xmalloc(n * sizeof(struct vi));
	for (ct_long i = 0; i < n; i++) { ss[i].v = sigma[i]; ss[i].i = i; }
	qsort(ss, n, sizeof(struct vi), cmp_vi);
	double sqsum = 0;
	for (ct_long i = 0; i < n; i++) { ss[i].v = ss[i].v * ss[i].v; sqsum += ss[i].v; }
	if (sqsum == 0) { free(ss); *norm_sigma = 0; *entropy = 0; return 0; }
	if (relative_thresh) for (ct_long i = 0; i < n; i++) ss[i].v /= sqsum;
	for (ct_long i = 1; i < n; i++) ss[i].v += ss[i - 1].v;
	if (max_vdim < n)
	{
		*tol_eff = fmax(tol, ss[n - max_vdim - 1].v);
		for (ct_long i = 0; i < n - max_vdim; i++) ss[i].v = 0;
	}
	double* accum = xmalloc(n * sizeof(double));
	for (ct_long i = 0; i < n; i++) accum[ss[i].i] = ss[i].v;
	free(ss);
	ct_long num = 0;
	for (ct_long i = 0; i < n; i++) if (accum[i] > tol) ind[num++] = i;
	free(accum);
	if (num == 0) { *norm_sigma = 0; *entropy = 0; return 0; }
	double* ret = xmalloc(num * sizeof(double));
	for (ct_long i = 0; i < num; i++) ret[i] = sigma[ind[i]];
	*norm_sigma = scipy_cblas_dnrm2((int)num, ret, 1);
	double s = 0;
	for (ct_long i = 0; i < num; i++)
	{
		const double x = ret[i] / *norm_sigma;
		if (x > 0) { const double sq = x * x; s -= sq * log(sq); }
	}
	*entropy = s;
	free(ret);
	return num;
}

/* retained singular values of the most recent split at every bond of the last oracle_dmrg_twosite
 * call (after the final sweep: those of its right-to-left pass) */
#define MAX_BONDS 4096
static double* g_bond_sigma[MAX_BONDS];
static ct_long g_bond_nsigma[MAX_BONDS];
static double* g_split_sigma = NULL;     /* written by split_matrix_svd */
static ct_long g_split_nsigma = 0;

ct_long oracle_get_bond_sigma(int bond, double* out, ct_long max)
{
	if (bond < 0 || bond >= MAX_BONDS || !g_bond_sigma[bond]) return -1;
	for (ct_long i = 0; i < g_bond_nsigma[bond] && i < max; i++) out[i] = g_bond_sigma[bond][i];
	return g_bond_nsigma[bond];
}

static void record_bond_sigma(int bond)
{
	if (bond < 0 || bond >= MAX_BONDS) return;
	free(g_bond_sigma[bond]);
	g_bond_sigma[bond] = g_split_sigma;
	g_bond_nsigma[bond] = g_split_nsigma;
	g_split_sigma = NULL;
	g_split_nsigma = 0;
}

/* ---- split_block_sparse_matrix_svd (bond_ops.c:15-138), renormalize = false ---- */

static int split_matrix_svd(const struct block_sparse_tensor* a, double tol, ct_long max_vdim, int distr_left,
                            struct block_sparse_tensor* a0, struct block_sparse_tensor* a1, double* entropy)
{
	struct block_sparse_tensor u, vh;
	double* s;
	ct_long ns;
	int ret = oracle_block_sparse_tensor_svd(a, &u, &s, &ns, &vh);
	if (ret < 0) return ret;
	ct_long* ind = xmalloc(ns * sizeof(ct_long));
	double norm_sigma, tol_eff;
	ct_long num = oracle_retained_bond_indices(s, ns, tol, 1, max_vdim, ind, &norm_sigma, entropy, &tol_eff);
	double* sret;
	if (num == 0)
	{
		num = 1;
		ind[0] = 0;
		sret = xcalloc(1, sizeof(double));
	}
	else
	{
		sret = xmalloc(num * sizeof(double));
		for (ct_long i = 0; i < num; i++) sret[i] = s[ind[i]];
	}
	free(g_split_sigma);
	g_split_sigma = xmalloc(num * sizeof(double));
	memcpy(g_split_sigma, sret, num * sizeof(double));
	g_split_nsigma = num;
	struct block_sparse_tensor m0, m1;
	bst_slice(&u, 1, ind, num, &m0);
	bst_slice(&vh, 0, ind, num, &m1);
	oracle_delete_block_sparse_tensor(&u);
	oracle_delete_block_sparse_tensor(&vh);
	if (distr_left)
	{
		bst_scale_axis(&m0, sret, AXR_TRAILING, a0);
		oracle_delete_block_sparse_tensor(&m0);
		*a1 = m1;
	}
	else
	{
		bst_scale_axis(&m1, sret, AXR_LEADING, a1);
		oracle_delete_block_sparse_tensor(&m1);
		*a0 = m0;
	}
	free(sret);
	free(ind);
	free(s);
	return 0;
}

/* ---- MPS / MPO two-site helpers ---- */

/* mps_merge_tensor_pair (mps.c:1166-1178) */
static void merge_mps_pair(const struct block_sparse_tensor* a0, const struct block_sparse_tensor* a1, struct block_sparse_tensor* a)
{
	struct block_sparse_tensor t;
	oracle_block_sparse_tensor_dot(a0, AXR_TRAILING, a1, AXR_LEADING, 1, &t);
	bst_flatten(&t, 1, TENSOR_AXIS_OUT, a);
	oracle_delete_block_sparse_tensor(&t);
}

/* mpo_merge_tensor_pair (mpo.c:255-279) */
static void merge_mpo_pair(const struct block_sparse_tensor* a0, const struct block_sparse_tensor* a1, struct block_sparse_tensor* a)
{
	struct block_sparse_tensor t, p, f;
	oracle_block_sparse_tensor_dot(a0, AXR_TRAILING, a1, AXR_LEADING, 1, &t);
	const int perm[6] = { 0, 1, 3, 2, 4, 5 };
	oracle_block_sparse_tensor_transpose(perm, &t, &p);
	oracle_delete_block_sparse_tensor(&t);
	bst_flatten(&p, 1, TENSOR_AXIS_OUT, &f);
	oracle_delete_block_sparse_tensor(&p);
	bst_flatten(&f, 2, TENSOR_AXIS_IN, a);
	oracle_delete_block_sparse_tensor(&f);
}

/* mps_split_tensor_svd (mps.c:1119-1159) */
static int split_mps_tensor_svd(const struct block_sparse_tensor* a, ct_long d, const qnumber* qsite, double tol,
                                ct_long max_vdim, int distr_left, struct block_sparse_tensor* a0,
                                struct block_sparse_tensor* a1, double* entropy)
{
	const ct_long dd[2] = { d, d };
	const enum tensor_axis_direction od[2] = { TENSOR_AXIS_OUT, TENSOR_AXIS_OUT };
	const qnumber* qq[2] = { qsite, qsite };
	struct block_sparse_tensor a4, tmp, am;
	bst_split(a, 1, dd, od, qq, &a4);
	bst_flatten(&a4, 0, TENSOR_AXIS_OUT, &tmp);
	bst_flatten(&tmp, 1, TENSOR_AXIS_IN, &am);
	oracle_delete_block_sparse_tensor(&tmp);
	struct block_sparse_tensor m0, m1;
	int ret = split_matrix_svd(&am, tol, max_vdim, distr_left, &m0, &m1, entropy);
	oracle_delete_block_sparse_tensor(&am);
	if (ret < 0) { oracle_delete_block_sparse_tensor(&a4); return ret; }
	bst_split(&m0, 0, a4.dim_logical, a4.axis_dir, (const qnumber* const*)a4.qnums_logical, a0);
	bst_split(&m1, 1, a4.dim_logical + 2, a4.axis_dir + 2, (const qnumber* const*)(a4.qnums_logical + 2), a1);
	oracle_delete_block_sparse_tensor(&m0);
	oracle_delete_block_sparse_tensor(&m1);
	oracle_delete_block_sparse_tensor(&a4);
	return 0;
}

/* mps_local_orthonormalize_rq (mps.c:560-600) */
static int local_orthonormalize_rq(struct block_sparse_tensor* a, struct block_sparse_tensor* a_prev)
{
	const ct_long dr[2] = { a->dim_logical[1], a->dim_logical[2] };
	qnumber* qr_[2];
	for (int i = 0; i < 2; i++) {
		qr_[i] = xmalloc(dr[i] * sizeof(qnumber));
		memcpy(qr_[i], a->qnums_logical[1 + i], dr[i] * sizeof(qnumber));
	}
	const enum tensor_axis_direction adr[2] = { TENSOR_AXIS_OUT, TENSOR_AXIS_IN };
	struct block_sparse_tensor am, r, q, upd;
	bst_flatten(a, 1, TENSOR_AXIS_IN, &am);
	oracle_delete_block_sparse_tensor(a);
	int ret = bst_rq(&am, &r, &q);
	oracle_delete_block_sparse_tensor(&am);
	bst_split(&q, 1, dr, adr, (const qnumber* const*)qr_, a);
	oracle_delete_block_sparse_tensor(&q);
	free(qr_[0]);
	free(qr_[1]);
	oracle_block_sparse_tensor_dot(a_prev, AXR_TRAILING, &r, AXR_LEADING, 1, &upd);
	oracle_delete_block_sparse_tensor(a_prev);
	*a_prev = upd;
	oracle_delete_block_sparse_tensor(&r);
	return ret;
}

/* mps_local_orthonormalize_qr (mps.c:513-553) */
static int local_orthonormalize_qr(struct block_sparse_tensor* a, struct block_sparse_tensor* a_next)
{
	const ct_long dl[2] = { a->dim_logical[0], a->dim_logical[1] };
	qnumber* ql[2];
	for (int i = 0; i < 2; i++) {
		ql[i] = xmalloc(dl[i] * sizeof(qnumber));
		memcpy(ql[i], a->qnums_logical[i], dl[i] * sizeof(qnumber));
	}
	const enum tensor_axis_direction adl[2] = { TENSOR_AXIS_OUT, TENSOR_AXIS_OUT };
	struct block_sparse_tensor am, q, r, upd;
	bst_flatten(a, 0, TENSOR_AXIS_OUT, &am);
	oracle_delete_block_sparse_tensor(a);
	int ret = bst_qr(&am, &q, &r);
	oracle_delete_block_sparse_tensor(&am);
	bst_split(&q, 0, dl, adl, (const qnumber* const*)ql, a);
	oracle_delete_block_sparse_tensor(&q);
	free(ql[0]);
	free(ql[1]);
	oracle_block_sparse_tensor_dot(&r, AXR_TRAILING, a_next, AXR_LEADING, 1, &upd);
	oracle_delete_block_sparse_tensor(a_next);
	*a_next = upd;
	oracle_delete_block_sparse_tensor(&r);
	return ret;
}

static void scale_tensor(struct block_sparse_tensor* t, double alpha)
{
	const ct_long nblocks = iprod(t->dim_blocks, t->ndim);
	for (ct_long k = 0; k < nblocks; k++) {
		if (!t->blocks[k]) continue;
		double* d = t->blocks[k]->data;
		const ct_long n = iprod(t->blocks[k]->dim, t->ndim);
		for (ct_long j = 0; j < n; j++) d[j] *= alpha;
	}
}

/* dummy 1 x 1 x 1 head tensor carrying the left bond's quantum number
 * (mps.c:719-731, dmrg.c:366-378) */
static void make_head(const struct block_sparse_tensor* a0, struct block_sparse_tensor* h)
{
	const ct_long dim[3] = { a0->dim_logical[0], 1, a0->dim_logical[0] };
	const enum tensor_axis_direction dir[3] = { TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN };
	const qnumber qz[1] = { 0 };
	const qnumber* q[3] = { a0->qnums_logical[0], qz, a0->qnums_logical[0] };
	bst_alloc(3, dim, dir, q, h);
}

/* mps_orthonormalize_qr(..., MPS_ORTHONORMAL_RIGHT) (mps.c:609-757) */
static double orthonormalize_right(struct mps* psi, int* err)
{
	*err = 0;
	for (int i = psi->nsites - 1; i > 0; i--)
		if (local_orthonormalize_rq(&psi->a[i], &psi->a[i - 1]) < 0) *err = -1;
	struct block_sparse_tensor h;
	make_head(&psi->a[0], &h);
	((double*)h.blocks[0]->data)[0] = 1.0;
	if (local_orthonormalize_rq(&psi->a[0], &h) < 0) *err = -1;
	double norm = 0;
	if (h.blocks[0])
	{
		norm = ((double*)h.blocks[0]->data)[0];
		if (norm < 0) { scale_tensor(&psi->a[0], -1.0); norm = -norm; }
	}
	oracle_delete_block_sparse_tensor(&h);
	return norm;
}

/* ---- environment blocks (chain_ops.c:14-85, :116-267) ---- */

static void reversed_view(const struct block_sparse_tensor* b, struct block_sparse_tensor* br, enum tensor_axis_direction* dirbuf)
{
	*br = *b;
	for (int i = 0; i < b->ndim; i++) dirbuf[i] = -b->axis_dir[i];
	br->axis_dir = dirbuf;
}

static void dummy_block(const qnumber* qa, const qnumber* qw, const qnumber* qb, int right, struct block_sparse_tensor* out)
{
	const ct_long dim[6] = { 1, 1, 1, 1, 1, 1 };
	const enum tensor_axis_direction dir[6] = { TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN,
	                                            TENSOR_AXIS_IN, TENSOR_AXIS_IN, TENSOR_AXIS_OUT };
	const qnumber* q[6] = { qa, qw, qb, qa, qw, qb };
	struct block_sparse_tensor s, t;
	bst_alloc(6, dim, dir, q, &s);
	((double*)s.blocks[0]->data)[0] = 1.0;
	if (right)
	{
		bst_flatten(&s, 4, TENSOR_AXIS_IN, &t);
		oracle_delete_block_sparse_tensor(&s);
		bst_flatten(&t, 3, TENSOR_AXIS_IN, out);
	}
	else
	{
		bst_flatten(&s, 0, TENSOR_AXIS_OUT, &t);
		oracle_delete_block_sparse_tensor(&s);
		bst_flatten(&t, 0, TENSOR_AXIS_OUT, out);
	}
	oracle_delete_block_sparse_tensor(&t);
}

void oracle_contraction_operator_step_right(const struct block_sparse_tensor* a, const struct block_sparse_tensor* b,
                                            const struct block_sparse_tensor* w, const struct block_sparse_tensor* r,
                                            struct block_sparse_tensor* r_next)
{
	struct block_sparse_tensor s, t, br;
	enum tensor_axis_direction dirbuf[3];
	oracle_block_sparse_tensor_dot(a, AXR_TRAILING, r, AXR_LEADING, 1, &s);
	const int perm0[5] = { 1, 2, 0, 3, 4 };
	oracle_block_sparse_tensor_transpose(perm0, &s, &t);
	oracle_delete_block_sparse_tensor(&s);
	oracle_block_sparse_tensor_dot(w, AXR_TRAILING, &t, AXR_LEADING, 2, &s);
	oracle_delete_block_sparse_tensor(&t);
	const int perm1[5] = { 4, 2, 0, 1, 3 };
	oracle_block_sparse_tensor_transpose(perm1, &s, &t);
	oracle_delete_block_sparse_tensor(&s);
	reversed_view(b, &br, dirbuf);
	oracle_block_sparse_tensor_dot(&t, AXR_TRAILING, &br, AXR_TRAILING, 2, &s);
	oracle_delete_block_sparse_tensor(&t);
	const int perm2[4] = { 1, 2, 3, 0 };
	oracle_block_sparse_tensor_transpose(perm2, &s, r_next);
	oracle_delete_block_sparse_tensor(&s);
}

void oracle_contraction_operator_step_left(const struct block_sparse_tensor* a, const struct block_sparse_tensor* b,
                                           const struct block_sparse_tensor* w, const struct block_sparse_tensor* l,
                                           struct block_sparse_tensor* l_next)
{
	struct block_sparse_tensor s, t, br;
	enum tensor_axis_direction dirbuf[3];
	reversed_view(b, &br, dirbuf);
	oracle_block_sparse_tensor_dot(l, AXR_TRAILING, &br, AXR_LEADING, 1, &s);
	const int perm0[5] = { 0, 1, 4, 2, 3 };
	oracle_block_sparse_tensor_transpose(perm0, &s, &t);
	oracle_delete_block_sparse_tensor(&s);
	oracle_block_sparse_tensor_dot(&t, AXR_TRAILING, w, AXR_LEADING, 2, &s);
	oracle_delete_block_sparse_tensor(&t);
	const int perm1[5] = { 1, 3, 4, 2, 0 };
	oracle_block_sparse_tensor_transpose(perm1, &s, &t);
	oracle_delete_block_sparse_tensor(&s);
	oracle_block_sparse_tensor_dot(a, AXR_LEADING, &t, AXR_LEADING, 2, &s);
	oracle_delete_block_sparse_tensor(&t);
	const int perm2[4] = { 3, 0, 1, 2 };
	oracle_block_sparse_tensor_transpose(perm2, &s, l_next);
	oracle_delete_block_sparse_tensor(&s);
}

void oracle_apply_local_hamiltonian(const struct block_sparse_tensor* a, const struct block_sparse_tensor* w,
                                    const struct block_sparse_tensor* l, const struct block_sparse_tensor* r,
                                    struct block_sparse_tensor* b)
{
	struct block_sparse_tensor s, t, k;
	oracle_block_sparse_tensor_dot(a, AXR_TRAILING, r, AXR_LEADING, 1, &s);
	const int perm0[5] = { 1, 2, 0, 3, 4 };
	oracle_block_sparse_tensor_transpose(perm0, &s, &t);
	oracle_delete_block_sparse_tensor(&s);
	oracle_block_sparse_tensor_dot(w, AXR_TRAILING, &t, AXR_LEADING, 2, &s);
	oracle_delete_block_sparse_tensor(&t);
	const int perm1[5] = { 2, 0, 1, 3, 4 };
	oracle_block_sparse_tensor_transpose(perm1, &s, &t);
	oracle_delete_block_sparse_tensor(&s);
	const int perm2[4] = { 0, 3, 1, 2 };
	oracle_block_sparse_tensor_transpose(perm2, l, &k);
	oracle_block_sparse_tensor_dot(&k, AXR_TRAILING, &t, AXR_LEADING, 2, &s);
	oracle_delete_block_sparse_tensor(&k);
	oracle_delete_block_sparse_tensor(&t);
	bst_cyclic_partial_trace(&s, 1, b);
	oracle_delete_block_sparse_tensor(&s);
}

/* ---- Lanczos (krylov.c:24-89) and Ritz vector (krylov.c:172-251) ---- */

typedef void (*linmap)(ct_long n, const void* data, const double* v, double* ret);

static int eigensystem_krylov(ct_long n, linmap f, const void* data, const double* vstart, int maxiter,
                              double* lambda, double* u_ritz)
{
	double* alpha = xmalloc(maxiter * sizeof(double));
	double* beta = xmalloc((maxiter > 1 ? maxiter - 1 : 1) * sizeof(double));
	double* v = xmalloc((size_t)maxiter * n * sizeof(double));
	double* w = xmalloc(n * sizeof(double));
	int numiter = maxiter;
	memcpy(v, vstart, n * sizeof(double));
	const double nrm0 = scipy_cblas_dnrm2((int)n, v, 1);
	for (ct_long i = 0; i < n; i++) v[i] *= 1 / nrm0;
	for (int j = 0; j < maxiter - 1; j++)
	{
		f(n, data, &v[(size_t)j * n], w);
		alpha[j] = scipy_cblas_ddot((int)n, w, 1, &v[(size_t)j * n], 1);
		if (j > 0) {
			for (ct_long i = 0; i < n; i++) w[i] -= alpha[j] * v[(size_t)j * n + i] + beta[j - 1] * v[(size_t)(j - 1) * n + i];
		} else {
			for (ct_long i = 0; i < n; i++) w[i] -= alpha[j] * v[(size_t)j * n + i];
		}
		beta[j] = scipy_cblas_dnrm2((int)n, w, 1);
		if (beta[j] < 100 * n * 2.2204460492503131e-16) { numiter = j + 1; break; }
		const double ib = 1 / beta[j];
		for (ct_long i = 0; i < n; i++) v[(size_t)(j + 1) * n + i] = ib * w[i];
	}
	if (numiter == maxiter)
	{
		const int j = maxiter - 1;
		f(n, data, &v[(size_t)j * n], w);
		alpha[j] = scipy_cblas_ddot((int)n, w, 1, &v[(size_t)j * n], 1);
	}
	free(w);
	int ret = 0;
	double* u = xmalloc((size_t)numiter * numiter * sizeof(double));
	double* work = xmalloc((2 * numiter > 2 ? 2 * numiter - 2 : 1) * sizeof(double));
	int info;
	scipy_dsteqr_("I", &numiter, alpha, beta, u, &numiter, work, &info, 1);
	if (info != 0) ret = -2;
	else
	{
		lambda[0] = alpha[0];
		scipy_cblas_dgemm(ROW_MAJOR, TRANS, TRANS, (int)n, 1, numiter, 1.0, v, (int)n, u, numiter, 0.0, u_ritz, 1);
	}
	free(work);
	free(u);
	free(v);
	free(beta);
	free(alpha);
	return ret;
}

struct dense_map { const double* h; };

static void dense_apply(ct_long n, const void* data, const double* v, double* ret)
{
	const struct dense_map* m = data;
	scipy_cblas_dgemm(ROW_MAJOR, NO_TRANS, NO_TRANS, (int)n, 1, (int)n, 1.0, m->h, (int)n, v, 1, 0.0, ret, 1);
}

int oracle_lanczos_dense(ct_long n, const double* h, const double* vstart, int maxiter, double* lambda, double* u_ritz)
{
	struct dense_map m = { h };
	return eigensystem_krylov(n, dense_apply, &m, vstart, maxiter, lambda, u_ritz);
}

/* block_sparse_tensor_serialize_entries / deserialize (block_sparse_tensor.c:3111-3176) */
static ct_long num_entries(const struct block_sparse_tensor* t)
{
	ct_long n = 0;
	const ct_long nb = iprod(t->dim_blocks, t->ndim);
	for (ct_long k = 0; k < nb; k++) if (t->blocks[k]) n += iprod(t->blocks[k]->dim, t->ndim);
	return n;
}

static void serialize(const struct block_sparse_tensor* t, double* v)
{
	const ct_long nb = iprod(t->dim_blocks, t->ndim);
	for (ct_long k = 0; k < nb; k++) {
		if (!t->blocks[k]) continue;
		const ct_long n = iprod(t->blocks[k]->dim, t->ndim);
		memcpy(v, t->blocks[k]->data, n * sizeof(double));
		v += n;
	}
}

static void deserialize(struct block_sparse_tensor* t, const double* v)
{
	const ct_long nb = iprod(t->dim_blocks, t->ndim);
	for (ct_long k = 0; k < nb; k++) {
		if (!t->blocks[k]) continue;
		const ct_long n = iprod(t->blocks[k]->dim, t->ndim);
		memcpy(t->blocks[k]->data, v, n * sizeof(double));
		v += n;
	}
}

/* local_hamiltonian_data and its wrapper (dmrg.c:15-50) */
struct hdata {
	const struct block_sparse_tensor *w, *l, *r;
	struct block_sparse_tensor* a;
};

static void apply_wrapper(ct_long n, const void* data, const double* v, double* ret)
{
	(void)n;
	const struct hdata* h = data;
	deserialize(h->a, v);
	struct block_sparse_tensor ha;
	oracle_apply_local_hamiltonian(h->a, h->w, h->l, h->r, &ha);
	serialize(&ha, ret);
	oracle_delete_block_sparse_tensor(&ha);
}

/* minimize_local_energy (dmrg.c:86-147) */
static int minimize_local_energy(const struct block_sparse_tensor* w, const struct block_sparse_tensor* l,
                                 const struct block_sparse_tensor* r, const struct block_sparse_tensor* a_start,
                                 int maxiter, double* en, struct block_sparse_tensor* a_opt)
{
	const ct_long n = num_entries(a_start);
	double* vstart = xmalloc(n * sizeof(double));
	serialize(a_start, vstart);
	bst_alloc(a_start->ndim, a_start->dim_logical, a_start->axis_dir, (const qnumber* const*)a_start->qnums_logical, a_opt);
	struct hdata h = { w, l, r, a_opt };
	double* u = xmalloc(n * sizeof(double));
	int ret = eigensystem_krylov(n, apply_wrapper, &h, vstart, maxiter, en, u);
	if (ret == 0) deserialize(a_opt, u);
	free(u);
	free(vstart);
	return ret;
}

/* ---- per-sweep wall time of the last call (CLOCK_MONOTONIC, as src/util/timing.c:26-41) ---- */

#define MAX_SWEEP_TIMES 1024
static double g_sweep_times[MAX_SWEEP_TIMES];
static int g_num_sweep_times = 0;

static double wall_seconds(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int oracle_get_sweep_times(double* out, int max)
{
	for (int i = 0; i < g_num_sweep_times && i < max; i++) out[i] = g_sweep_times[i];
	return g_num_sweep_times;
}

/* ---- dmrg_twosite (dmrg.c:262-399) ---- */

int oracle_dmrg_twosite(const struct mpo* ham, int num_sweeps, int maxiter, double tol_split, ct_long max_vdim,
                        struct mps* psi, double* en_sweeps, double* entropy)
{
	const int L = ham->nsites;
	assert(L == psi->nsites && L >= 2);
	scipy_openblas_set_num_threads(1);
	int err = 0;
	double nrm = orthonormalize_right(psi, &err);
	if (err < 0) return err;
	if (nrm == 0) printf("Warning: in 'dmrg_twosite': initial MPS has norm zero (possibly due to mismatching quantum numbers)\n");

	struct block_sparse_tensor* lb = xcalloc(L, sizeof(*lb));
	struct block_sparse_tensor* rb = xcalloc(L, sizeof(*rb));
	dummy_block(psi->a[L - 1].qnums_logical[2], ham->a[L - 1].qnums_logical[3], psi->a[L - 1].qnums_logical[2], 1, &rb[L - 1]);
	for (int i = L - 1; i > 0; i--)
		oracle_contraction_operator_step_right(&psi->a[i], &psi->a[i], &ham->a[i], &rb[i], &rb[i - 1]);
	dummy_block(psi->a[0].qnums_logical[0], ham->a[0].qnums_logical[0], psi->a[0].qnums_logical[0], 0, &lb[0]);
	for (int i = 1; i < L; i++) bst_copy(&lb[0], &lb[i]);
	struct block_sparse_tensor* h2 = xcalloc(L - 1, sizeof(*h2));
	for (int i = 0; i < L - 1; i++) merge_mpo_pair(&ham->a[i], &ham->a[i + 1], &h2[i]);

	int ret = 0;
	g_num_sweep_times = 0;
	for (int n = 0; n < num_sweeps && ret == 0; n++)
	{
		const double t_sweep = wall_seconds();
		double en = 0;
		for (int i = 0; i < L - 2 && ret == 0; i++)
		{
			struct block_sparse_tensor cur, opt;
			merge_mps_pair(&psi->a[i], &psi->a[i + 1], &cur);
			oracle_delete_block_sparse_tensor(&psi->a[i]);
			oracle_delete_block_sparse_tensor(&psi->a[i + 1]);
			ret = minimize_local_energy(&h2[i], &lb[i], &rb[i + 1], &cur, maxiter, &en, &opt);
			oracle_delete_block_sparse_tensor(&cur);
			if (ret < 0) break;
			double ent;
			ret = split_mps_tensor_svd(&opt, psi->d, psi->qsite, tol_split, max_vdim, 0, &psi->a[i], &psi->a[i + 1], &ent);
			oracle_delete_block_sparse_tensor(&opt);
			if (ret < 0) break;
			record_bond_sigma(i);
			oracle_delete_block_sparse_tensor(&lb[i + 1]);
			oracle_contraction_operator_step_left(&psi->a[i], &psi->a[i], &ham->a[i], &lb[i], &lb[i + 1]);
		}
		for (int i = L - 2; i >= 0 && ret == 0; i--)
		{
			struct block_sparse_tensor cur, opt;
			merge_mps_pair(&psi->a[i], &psi->a[i + 1], &cur);
			oracle_delete_block_sparse_tensor(&psi->a[i]);
			oracle_delete_block_sparse_tensor(&psi->a[i + 1]);
			ret = minimize_local_energy(&h2[i], &lb[i], &rb[i + 1], &cur, maxiter, &en, &opt);
			oracle_delete_block_sparse_tensor(&cur);
			if (ret < 0) break;
			double ent;
			ret = split_mps_tensor_svd(&opt, psi->d, psi->qsite, tol_split, max_vdim, 1, &psi->a[i], &psi->a[i + 1], &ent);
			oracle_delete_block_sparse_tensor(&opt);
			if (ret < 0) break;
			record_bond_sigma(i);
			entropy[i] = ent;
			oracle_delete_block_sparse_tensor(&rb[i]);
			oracle_contraction_operator_step_right(&psi->a[i + 1], &psi->a[i + 1], &ham->a[i + 1], &rb[i + 1], &rb[i]);
		}
		if (ret < 0) break;
		struct block_sparse_tensor t;
		make_head(&psi->a[0], &t);
		if (local_orthonormalize_rq(&psi->a[0], &t) < 0) ret = -1;
		oracle_delete_block_sparse_tensor(&t);
		en_sweeps[n] = en;
		if (g_num_sweep_times < MAX_SWEEP_TIMES) g_sweep_times[g_num_sweep_times++] = wall_seconds() - t_sweep;
	}

	for (int i = 0; i < L - 1; i++) oracle_delete_block_sparse_tensor(&h2[i]);
	free(h2);
	for (int i = 0; i < L; i++) { oracle_delete_block_sparse_tensor(&rb[i]); oracle_delete_block_sparse_tensor(&lb[i]); }
	free(rb);
	free(lb);
	return ret;
}

/* ---- dmrg_singlesite (dmrg.c:155-254) ---- */

int oracle_dmrg_singlesite(const struct mpo* ham, int num_sweeps, int maxiter, struct mps* psi, double* en_sweeps)
{
	const int L = ham->nsites;
	assert(L == psi->nsites && L >= 1);
	scipy_openblas_set_num_threads(1);
	int err = 0;
	double nrm = orthonormalize_right(psi, &err);
	if (err < 0) return err;
	if (nrm == 0) printf("Warning: in 'dmrg_singlesite': initial MPS has norm zero (possibly due to mismatching quantum numbers)\n");

	struct block_sparse_tensor* lb = xcalloc(L, sizeof(*lb));
	struct block_sparse_tensor* rb = xcalloc(L, sizeof(*rb));
	dummy_block(psi->a[L - 1].qnums_logical[2], ham->a[L - 1].qnums_logical[3], psi->a[L - 1].qnums_logical[2], 1, &rb[L - 1]);
	for (int i = L - 1; i > 0; i--)
		oracle_contraction_operator_step_right(&psi->a[i], &psi->a[i], &ham->a[i], &rb[i], &rb[i - 1]);
	dummy_block(psi->a[0].qnums_logical[0], ham->a[0].qnums_logical[0], psi->a[0].qnums_logical[0], 0, &lb[0]);
	for (int i = 1; i < L; i++) bst_copy(&lb[0], &lb[i]);

	int ret = 0;
	g_num_sweep_times = 0;
	for (int n = 0; n < num_sweeps && ret == 0; n++)
	{
		const double t_sweep = wall_seconds();
		double en = 0;
		for (int i = 0; i < L - 1 && ret == 0; i++)
		{
			struct block_sparse_tensor opt;
			ret = minimize_local_energy(&ham->a[i], &lb[i], &rb[i], &psi->a[i], maxiter, &en, &opt);
			if (ret < 0) break;
			oracle_delete_block_sparse_tensor(&psi->a[i]);
			psi->a[i] = opt;
			if (local_orthonormalize_qr(&psi->a[i], &psi->a[i + 1]) < 0) ret = -1;
			oracle_delete_block_sparse_tensor(&lb[i + 1]);
			oracle_contraction_operator_step_left(&psi->a[i], &psi->a[i], &ham->a[i], &lb[i], &lb[i + 1]);
		}
		for (int i = L - 1; i > 0 && ret == 0; i--)
		{
			struct block_sparse_tensor opt;
			ret = minimize_local_energy(&ham->a[i], &lb[i], &rb[i], &psi->a[i], maxiter, &en, &opt);
			if (ret < 0) break;
			oracle_delete_block_sparse_tensor(&psi->a[i]);
			psi->a[i] = opt;
			if (local_orthonormalize_rq(&psi->a[i], &psi->a[i - 1]) < 0) ret = -1;
			oracle_delete_block_sparse_tensor(&rb[i - 1]);
			oracle_contraction_operator_step_right(&psi->a[i], &psi->a[i], &ham->a[i], &rb[i], &rb[i - 1]);
		}
		if (ret < 0) break;
		struct block_sparse_tensor t;
		make_head(&psi->a[0], &t);
		if (local_orthonormalize_rq(&psi->a[0], &t) < 0) ret = -1;
		oracle_delete_block_sparse_tensor(&t);
		en_sweeps[n] = en;
		if (g_num_sweep_times < MAX_SWEEP_TIMES) g_sweep_times[g_num_sweep_times++] = wall_seconds() - t_sweep;
	}
	for (int i = 0; i < L; i++) { oracle_delete_block_sparse_tensor(&rb[i]); oracle_delete_block_sparse_tensor(&lb[i]); }
	free(rb);
	free(lb);
	return ret;
}

/* ---- mps_vdot (mps.c:314-370), real case ---- */

double oracle_mps_vdot(const struct mps* chi, const struct mps* psi)
{
	const int L = psi->nsites;
	/* contract from the left: t = chi[0]^* . psi[0] over the physical and left dummy legs */
	struct block_sparse_tensor t, u, c0;
	enum tensor_axis_direction dirbuf[3];
	/* leading dummy bond and physical leg of chi reversed, contracted with psi's */
	reversed_view(&chi->a[0], &c0, dirbuf);
	oracle_block_sparse_tensor_dot(&c0, AXR_LEADING, &psi->a[0], AXR_LEADING, 2, &t);
	for (int i = 1; i < L; i++)
	{
		struct block_sparse_tensor ci;
		enum tensor_axis_direction db[3];
		reversed_view(&chi->a[i], &ci, db);
		/* t (Dc, Dp) . psi (Dp, d, D') -> (Dc, d, D') */
		oracle_block_sparse_tensor_dot(&t, AXR_TRAILING, &psi->a[i], AXR_LEADING, 1, &u);
		oracle_delete_block_sparse_tensor(&t);
		/* chi^ (Dc, d, Dc') leading 2 with u leading 2 -> (Dc', D') */
		oracle_block_sparse_tensor_dot(&ci, AXR_LEADING, &u, AXR_LEADING, 2, &t);
		oracle_delete_block_sparse_tensor(&u);
	}
	double r = 0;
	const ct_long nb = iprod(t.dim_blocks, t.ndim);
	for (ct_long k = 0; k < nb; k++) if (t.blocks[k]) r += ((double*)t.blocks[k]->data)[0];
	oracle_delete_block_sparse_tensor(&t);
	return r;
}

int oracle_set_num_threads(int n)
{
	if (n > 0) omp_set_num_threads(n);
	scipy_openblas_set_num_threads(1);
	return omp_get_max_threads();
}

/* ---- seeded random MPS: seed_rng_state, rand_interval, rand_choice, randu, randn (rng.c:15-125),
 *      the PCG32 generators they use (pcg_basic.c:33-54, :115-151), and construct_random_mps
 *      (mps.c:93-175), real double precision ---- */

struct pcg32 { uint64_t state, inc; };

static uint32_t pcg32_next(struct pcg32* g)
{
	const uint64_t old = g->state;
	g->state = old * 6364136223846793005ULL + g->inc;
	const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
	const uint32_t rot = (uint32_t)(old >> 59u);
	return (xs >> rot) | (xs << ((-rot) & 31));
}

static void pcg32_seed(struct pcg32* g, uint64_t initstate, uint64_t initseq)
{
	g->state = 0;
	g->inc = (initseq << 1u) | 1u;
	pcg32_next(g);
	g->state += initstate;
	pcg32_next(g);
}

struct orng { struct pcg32 g[2]; };

static uint64_t orng_u64(struct orng* r)
{
	const uint64_t hi = pcg32_next(&r->g[0]);
	return (hi << 32) | pcg32_next(&r->g[1]);
}

static void orng_seed(struct orng* r, uint64_t seed)
{
	struct pcg32 t;
	pcg32_seed(&t, seed, 6364136223846793005ULL * seed + 1442695040888963407ULL);
	uint64_t v[4];
	for (int i = 0; i < 4; i++) { const uint64_t hi = pcg32_next(&t); v[i] = (hi << 32) | pcg32_next(&t); }
	const uint64_t mask = ~0ull >> 1;
	if ((v[2] & mask) == (v[3] & mask)) v[3] = ~v[3];
	pcg32_seed(&r->g[0], v[0], v[2]);
	pcg32_seed(&r->g[1], v[1], v[3]);
}

static uint64_t orng_bounded(struct orng* r, uint64_t bound)
{
	const uint64_t threshold = (0 - bound) % bound;
	for (;;) { const uint64_t x = orng_u64(r); if (x >= threshold) return x % bound; }
}

static double orng_normal(struct orng* r)
{
	double u1 = ldexp((double)orng_u64(r), -64);
	const double u2 = ldexp((double)orng_u64(r), -64);
	if (u1 == 0) u1 = 1;
	return sqrt(-2 * log(u1)) * sin(6.2831853071795864769 * u2);
}

/* bond quantum numbers of one virtual bond: all outer sums, or a Floyd sample of max_vdim of them */
static qnumber* random_bond(struct orng* r, const qnumber* prev, ct_long nprev, int sign, const qnumber* qsite, ct_long d,
                            ct_long max_vdim, ct_long* nout)
{
	const ct_long nfull = nprev * d;
	qnumber* full = xmalloc(nfull * sizeof(qnumber));
	for (ct_long i = 0; i < nprev; i++)
		for (ct_long j = 0; j < d; j++) full[i * d + j] = prev[i] + sign * qsite[j];
	if (nfull <= max_vdim) { *nout = nfull; return full; }
	uint64_t* idx = xmalloc(max_vdim * sizeof(uint64_t));
	for (uint64_t i = 0; i < (uint64_t)max_vdim; i++)
	{
		const uint64_t j = (uint64_t)nfull - (uint64_t)max_vdim + 1 + i;
		const uint64_t t = orng_bounded(r, j);
		int drawn = 0;
		for (uint64_t k = 0; k < i; k++) if (idx[k] == t) { drawn = 1; break; }
		idx[i] = drawn ? j - 1 : t;
	}
	qnumber* sel = xmalloc(max_vdim * sizeof(qnumber));
	for (ct_long i = 0; i < max_vdim; i++) sel[i] = full[idx[i]];
	free(idx);
	free(full);
	*nout = max_vdim;
	return sel;
}

int oracle_construct_random_mps(int nsites, ct_long d, const qnumber* qsite, qnumber qnum_sector, ct_long max_vdim,
                                uint64_t rng_seed, struct mps* mps)
{
	if (nsites < 1 || d < 1 || max_vdim < 1) return -1;
	struct orng r;
	orng_seed(&r, rng_seed);
	ct_long* nb = xcalloc(nsites + 1, sizeof(ct_long));
	qnumber** qb = xcalloc(nsites + 1, sizeof(qnumber*));
	nb[0] = 1; qb[0] = xcalloc(1, sizeof(qnumber));
	nb[nsites] = 1; qb[nsites] = xmalloc(sizeof(qnumber)); qb[nsites][0] = qnum_sector;
	for (int l = 1; l < (nsites + 1) / 2; l++) qb[l] = random_bond(&r, qb[l - 1], nb[l - 1], 1, qsite, d, max_vdim, &nb[l]);
	for (int l = nsites - 1; l >= (nsites + 1) / 2; l--) qb[l] = random_bond(&r, qb[l + 1], nb[l + 1], -1, qsite, d, max_vdim, &nb[l]);
	mps->nsites = nsites;
	mps->d = d;
	mps->qsite = xmalloc(d * sizeof(qnumber));
	memcpy(mps->qsite, qsite, d * sizeof(qnumber));
	mps->a = xcalloc(nsites, sizeof(struct block_sparse_tensor));
	const enum tensor_axis_direction dir[3] = { TENSOR_AXIS_OUT, TENSOR_AXIS_OUT, TENSOR_AXIS_IN };
	for (int l = 0; l < nsites; l++)
	{
		const ct_long dim[3] = { nb[l], d, nb[l + 1] };
		const qnumber* qn[3] = { qb[l], qsite, qb[l + 1] };
		bst_alloc(3, dim, dir, qn, &mps->a[l]);
		/* block_sparse_tensor_fill_random_normal: blocks in index order, entries alpha * randn + 0 */
		const double alpha = 1.0 / sqrt((double)(dim[0] * dim[1] * dim[2]));
		const ct_long nblk = iprod(mps->a[l].dim_blocks, 3);
		for (ct_long k = 0; k < nblk; k++)
		{
			struct dense_tensor* b = mps->a[l].blocks[k];
			if (!b) continue;
			double* v = b->data;
			const ct_long ne = iprod(b->dim, b->ndim);
			for (ct_long j = 0; j < ne; j++) v[j] = alpha * orng_normal(&r) + 0.0;
		}
	}
	for (int l = 0; l <= nsites; l++) free(qb[l]);
	free(qb);
	free(nb);
	return 0;
}
