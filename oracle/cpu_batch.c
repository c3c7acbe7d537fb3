/*
 * cpu_batch.c -- multi-threaded CPU batch runner (TEST AND CPU-BASELINE INFRASTRUCTURE).
 *
 * Compiled twice by oracle/Makefile:
 *   - into liboracle.so against the scalar restatement (ksw2_oracle.c), and
 *   - with -DBATCH_REF into oracle/_ref/libksw2ref.so against the reference's
 *     own SSE sources (ksw2_extz2_sse.c, ksw2_extd2_sse.c, ksw2_ll_sse.c),
 *     compiled from where they lie in the reference tree.
 * In the reference build the jobs are spread over the threads by the
 * reference's own kt_for (kthread.c:54), compiled from its kthread.c; the
 * restatement uses a pthread pool whose workers pull job indices from an
 * atomic counter.  Either way each worker keeps one ksw_extz_t that it reuses
 * across calls, as align.c:908 does.
 */
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include "ksw2_oracle.h"

#ifdef BATCH_REF
#include "ksw2.h"
#include "kthread.h"
#define EZ_T ksw_extz_t
#define LLRST_T ksw_llrst_t
#define RUN_EXTZ2(ql, qs, tl, ts, m, mat, q, e, w, zd, eb, fl, ez) ksw_extz2_sse(0, ql, qs, tl, ts, m, mat, q, e, w, zd, eb, fl, ez)
#define RUN_EXTD2(ql, qs, tl, ts, m, mat, q, e, q2, e2, w, zd, eb, fl, ez) ksw_extd2_sse(0, ql, qs, tl, ts, m, mat, q, e, q2, e2, w, zd, eb, fl, ez)
#define RUN_QINIT(sz, ql, qs, m, mat) ksw_ll_qinit(0, sz, ql, qs, m, mat)
#define RUN_U8(qp, tl, ts, go, ge, x) ksw_ll_u8_core(qp, tl, ts, go, ge, x)
#define RUN_I16(qp, tl, ts, go, ge, x) ksw_ll_i16_core(qp, tl, ts, go, ge, x)
#define EXT_BATCH ref_ext_batch
#define LL_BATCH ref_ll_batch
#else
#define EZ_T orc_extz_t
#define LLRST_T orc_llrst_t
#define RUN_EXTZ2(ql, qs, tl, ts, m, mat, q, e, w, zd, eb, fl, ez) orc_extz2(ql, qs, tl, ts, m, mat, q, e, w, zd, eb, fl, ez, 0)
#define RUN_EXTD2(ql, qs, tl, ts, m, mat, q, e, q2, e2, w, zd, eb, fl, ez) orc_extd2(ql, qs, tl, ts, m, mat, q, e, q2, e2, w, zd, eb, fl, ez, 0)
#define RUN_QINIT(sz, ql, qs, m, mat) orc_ll_qinit(sz, ql, qs, m, mat)
#define RUN_U8(qp, tl, ts, go, ge, x) orc_ll_u8_core(qp, tl, ts, go, ge, x)
#define RUN_I16(qp, tl, ts, go, ge, x) orc_ll_i16_core(qp, tl, ts, go, ge, x)
#define EXT_BATCH orc_ext_batch
#define LL_BATCH orc_ll_batch
#endif

typedef struct {
	int kind, n_jobs, size;
	const orc_job_t *jobs;
	const uint8_t *qbuf, *tbuf;
	int8_t m;
	const int8_t *mat;
	int8_t q, e, q2, e2;
	int gapo, gape, xtra;
	orc_res_t *res;
	orc_llrst_t *llres;
	uint32_t *cigar_out;
	const int64_t *cig_off;
	volatile int next, slot;
	EZ_T *ez;  /* one per worker thread, reused across its calls */
} batch_ctx_t;

static void ext_one(batch_ctx_t *c, long i, int tid)
{
	const orc_job_t *j = &c->jobs[i];
	EZ_T *ez = &c->ez[tid];
	orc_res_t *o;
	if (c->kind == 0)
		RUN_EXTZ2(j->qlen, c->qbuf + j->qoff, j->tlen, c->tbuf + j->toff, c->m, c->mat, c->q, c->e, j->w, j->zdrop, j->end_bonus, j->flag, ez);
	else
		RUN_EXTD2(j->qlen, c->qbuf + j->qoff, j->tlen, c->tbuf + j->toff, c->m, c->mat, c->q, c->e, c->q2, c->e2, j->w, j->zdrop, j->end_bonus, j->flag, ez);
	o = &c->res[i];
	o->score = ez->score, o->max = (int32_t)ez->max, o->max_q = ez->max_q, o->max_t = ez->max_t;
	o->mqe = ez->mqe, o->mqe_t = ez->mqe_t, o->mte = ez->mte, o->mte_q = ez->mte_q;
	o->zdropped = ez->zdropped, o->reach_end = ez->reach_end, o->n_cigar = ez->n_cigar, o->n_diag = 0;
	o->cigar_off = c->cig_off[i];
	if (ez->n_cigar > 0) memcpy(c->cigar_out + c->cig_off[i], ez->cigar, (size_t)ez->n_cigar * 4);
}

static void ll_one(batch_ctx_t *c, long i)
{
	const orc_job_t *j = &c->jobs[i];
	void *qp;
	LLRST_T r;
	qp = RUN_QINIT(c->size, j->qlen, c->qbuf + j->qoff, c->m, c->mat);
	if (c->size == 1) r = RUN_U8(qp, j->tlen, c->tbuf + j->toff, c->gapo, c->gape, c->xtra);
	else r = RUN_I16(qp, j->tlen, c->tbuf + j->toff, c->gapo, c->gape, c->xtra);
	free(qp);
	c->llres[i].score = r.score, c->llres[i].te = r.te, c->llres[i].qe = r.qe;
	c->llres[i].score2 = r.score2, c->llres[i].te2 = r.te2;
}

#ifdef BATCH_REF
static void ext_kt(void *data, long i, int tid) { ext_one((batch_ctx_t *)data, i, tid); }
static void ll_kt(void *data, long i, int tid) { (void)tid; ll_one((batch_ctx_t *)data, i); }
#else
static void *ext_worker(void *arg)
{
	batch_ctx_t *c = (batch_ctx_t *)arg;
	int tid = __atomic_fetch_add(&c->slot, 1, __ATOMIC_RELAXED); /* this worker's ksw_extz_t */
	for (;;) {
		int i = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED);
		if (i >= c->n_jobs) break;
		ext_one(c, i, tid);
	}
	return 0;
}

static void *ll_worker(void *arg)
{
	batch_ctx_t *c = (batch_ctx_t *)arg;
	for (;;) {
		int i = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED);
		if (i >= c->n_jobs) break;
		ll_one(c, i);
	}
	return 0;
}

static void run_pool(void *(*fn)(void *), batch_ctx_t *c, int nthreads)
{
	pthread_t *tid;
	int i;
	if (nthreads <= 1) {
		fn(c);
		return;
	}
	tid = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
	for (i = 0; i < nthreads; ++i) pthread_create(&tid[i], 0, fn, c);
	for (i = 0; i < nthreads; ++i) pthread_join(tid[i], 0);
	free(tid);
}
#endif

int64_t EXT_BATCH(int kind, int n_jobs, const orc_job_t *jobs, const uint8_t *qbuf, const uint8_t *tbuf,
				  int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
				  orc_res_t *res, uint32_t *cigar_out, int64_t cigar_cap, int nthreads, int64_t *cells)
{
	batch_ctx_t c;
	int64_t *off, tot = 0;
	int i;
	off = (int64_t *)malloc(sizeof(int64_t) * (n_jobs + 1));
	for (i = 0; i < n_jobs; ++i) off[i] = tot, tot += jobs[i].qlen + jobs[i].tlen + 1;
	if (tot > cigar_cap) {
		free(off);
		return -1;
	}
	memset(&c, 0, sizeof(c));
	c.kind = kind, c.n_jobs = n_jobs, c.jobs = jobs, c.qbuf = qbuf, c.tbuf = tbuf;
	c.m = m, c.mat = mat, c.q = q, c.e = e, c.q2 = q2, c.e2 = e2;
	c.res = res, c.cigar_out = cigar_out, c.cig_off = off, c.next = 0;
	if (nthreads < 1) nthreads = 1;
	c.ez = (EZ_T *)calloc(nthreads, sizeof(EZ_T));
#ifdef BATCH_REF
	kt_for(nthreads, ext_kt, &c, n_jobs);
#else
	run_pool(ext_worker, &c, nthreads);
#endif
	for (i = 0; i < nthreads; ++i) free(c.ez[i].cigar);
	free(c.ez);
	free(off);
	if (cells) *cells = 0;
	return tot;
}

void LL_BATCH(int size, int n_jobs, const orc_job_t *jobs, const uint8_t *qbuf, const uint8_t *tbuf,
			  int m, const int8_t *mat, int gapo, int gape, int xtra, orc_llrst_t *res, int nthreads,
			  int64_t *cells)
{
	batch_ctx_t c;
	memset(&c, 0, sizeof(c));
	c.size = size, c.n_jobs = n_jobs, c.jobs = jobs, c.qbuf = qbuf, c.tbuf = tbuf;
	c.m = (int8_t)m, c.mat = mat, c.gapo = gapo, c.gape = gape, c.xtra = xtra;
	c.llres = res, c.next = 0;
#ifdef BATCH_REF
	kt_for(nthreads < 1 ? 1 : nthreads, ll_kt, &c, n_jobs);
#else
	run_pool(ll_worker, &c, nthreads);
#endif
	if (cells) *cells = 0;
}
