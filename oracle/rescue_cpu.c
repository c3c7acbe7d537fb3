/*
 * rescue_cpu.c -- mate rescue on the CPU (TEST AND CPU-BASELINE INFRASTRUCTURE ONLY).
 *
 * A scalar C restatement of pe.c's rescue of one candidate window
 * (mb_matesw_core's body, pe.c:340-368, and mb_matesw_align, pe.c:249-300)
 * composed from the oracle's l2b_getseq, mb_ungap, ksw_ll and extz2
 * restatements, plus a multi-threaded batch over candidates with the work
 * counter of the reference's kt_for (kthread.c:54-72).  The job, option and
 * result layouts are those of ksw2g_rescue_job_t, ksw2g_rescue_opt_t and
 * ksw2g_rescue_result_t.  The tests check it against oracle.rescue() and the
 * reference's own mb_matesw_core; bench.py times it as the CPU baseline.
 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "ksw2_oracle.h"

static void rescue_one(const orc_rescue_opt_t *o, const orc_rescue_job_t *J, const uint8_t *q,
					   const uint64_t *pac, const uint64_t *ctg_off, int64_t n_ambi, const uint64_t *ambi,
					   orc_rescue_res_t *R, uint32_t *cigar, int64_t cigar_off, orc_extz_t *ez)
{
	const int64_t tl = J->te - J->ts;
	int64_t ts2 = J->ts, te2 = J->te, max_sc;
	int max_i, n_good, n_kmer, max_ug, b_mm, size, qe, te;
	uint8_t *t, *rq, *rt;
	int8_t mat[25];
	void *qp;
	orc_llrst_t r;

	memset(R, 0, sizeof(*R));
	R->ext.cigar_off = -1;
	t = (uint8_t *)malloc(tl > 0 ? tl : 1);
	orc_l2b_getseq(pac, ctg_off, n_ambi, ambi, J->tid, J->ts, tl, 0, t);
	max_ug = orc_ungap(J->qlen, q, (int)tl, t, 7, J->meth, &max_i, &n_good, &n_kmer);
	R->max_ug = max_ug, R->max_i = max_i, R->n_good = n_good, R->n_kmer = n_kmer;
	if (max_ug >= 10 && max_ug >= J->qlen >> 1 && n_good == 1) { /* pe.c:347-352 */
		ts2 = J->ts + max_i - J->qlen / 2;
		te2 = ts2 + (int64_t)J->qlen * 2;
		if (ts2 < J->ts) ts2 = J->ts;
		if (te2 > J->te) te2 = J->te;
	}
	R->ts2 = ts2, R->te2 = te2;
	if (!(max_ug >= 10 || max_ug >= n_kmer * 0.33)) goto done;
	max_sc = J->qlen < te2 - ts2 ? J->qlen : te2 - ts2;
	if (max_sc >= 32767) goto done;
	b_mm = (o->b + o->a - 1) / o->a;
	orc_gen_nt4_mat(mat, 1, (int8_t)b_mm, (int8_t)((o->b_ts + o->a - 1) / o->a), (int8_t)((o->b_ambi + o->a - 1) / o->a),
					J->meth);
	size = max_sc < 255 - b_mm ? 1 : 2;
	qp = orc_ll_qinit(size, J->qlen, q, 5, mat);
	if (size == 1)
		r = orc_ll_u8_core(qp, (int)(te2 - ts2), t + (ts2 - J->ts), (o->q + o->a - 1) / o->a, (o->e + o->a - 1) / o->a,
						   0x40000 | o->min_len);
	else
		r = orc_ll_i16_core(qp, (int)(te2 - ts2), t + (ts2 - J->ts), (o->q + o->a - 1) / o->a, (o->e + o->a - 1) / o->a,
							0x40000 | o->min_len);
	free(qp);
	R->ll_done = 1, R->ll_score = r.score, R->ll_te = r.te, R->ll_qe = r.qe, R->ll_score2 = r.score2, R->ll_te2 = r.te2;
	if (!(r.score >= o->min_dp_max && r.score >= J->min_sc)) goto done;
	qe = r.qe + 1, te = r.te + 1;
	rq = (uint8_t *)malloc(qe + te + 2);
	rt = rq + qe + 1;
	for (int i = 0; i < qe; ++i) rq[i] = q[qe - 1 - i];                   /* mb_seq_rev(qe, qseq) */
	for (int i = 0; i < te; ++i) rt[i] = t[ts2 - J->ts + te - 1 - i];     /* mb_seq_rev(te, tseq) */
	orc_gen_nt4_mat(mat, (int8_t)o->a, (int8_t)o->b, (int8_t)o->b_ts, (int8_t)o->b_ambi, J->meth);
	orc_extz2(qe, rq, te, rt, 5, mat, (int8_t)o->q, (int8_t)o->e, o->bw, o->zdrop, o->end_bonus,
			  0x40 | 0x02 | 0x80 | (J->meth ? 0x04 : 0), ez, 0);
	free(rq);
	R->ext_done = 1;
	R->ext.score = ez->score, R->ext.max = (int32_t)ez->max, R->ext.max_q = ez->max_q, R->ext.max_t = ez->max_t;
	R->ext.mqe = ez->mqe, R->ext.mqe_t = ez->mqe_t, R->ext.mte = ez->mte, R->ext.mte_q = ez->mte_q;
	R->ext.zdropped = ez->zdropped, R->ext.reach_end = ez->reach_end, R->ext.n_cigar = ez->n_cigar;
	if (ez->n_cigar > 0) {
		memcpy(cigar + cigar_off, ez->cigar, (size_t)ez->n_cigar * 4);
		R->ext.cigar_off = cigar_off;
	}
	if (ez->n_cigar > 0 && (int)ez->max >= o->min_dp_max * o->a) { /* pe.c:291-304, 361-368 */
		int qs = qe - (ez->reach_end ? qe : ez->max_q + 1), qe2 = qe;
		int32_t d2 = (int32_t)((double)ez->max / r.score * r.score2 + .499);
		R->rescued = 1;
		R->ts = ts2 + te - (ez->reach_end ? ez->mqe_t + 1 : ez->max_t + 1);
		R->te = ts2 + te;
		R->dp_max2 = d2 < 0 ? 0 : d2;
		if (J->rev) {
			int tmp = qs;
			qs = J->qlen - qe2, qe2 = J->qlen - tmp;
		}
		R->qs = qs, R->qe = qe2;
	}
done:
	free(t);
}

typedef struct {
	const orc_rescue_opt_t *o;
	const orc_rescue_job_t *jobs;
	const uint8_t *qbuf;
	const uint64_t *pac, *ctg_off, *ambi;
	int64_t n_ambi;
	orc_rescue_res_t *res;
	uint32_t *cigar;
	const int64_t *cig_off;
	int n;
	volatile int next;
} rescue_ctx_t;

static void *rescue_worker(void *arg)
{
	rescue_ctx_t *c = (rescue_ctx_t *)arg;
	orc_extz_t ez;
	memset(&ez, 0, sizeof(ez));
	for (;;) {
		int i = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED);
		if (i >= c->n) break;
		rescue_one(c->o, &c->jobs[i], c->qbuf + c->jobs[i].qoff, c->pac, c->ctg_off, c->n_ambi, c->ambi, &c->res[i],
				   c->cigar, c->cig_off[i], &ez);
	}
	free(ez.cigar);
	return 0;
}

int64_t orc_rescue_batch(const orc_rescue_opt_t *o, int n, const orc_rescue_job_t *jobs, const uint8_t *qbuf,
						 const uint64_t *pac, const uint64_t *ctg_off, int64_t n_ambi, const uint64_t *ambi,
						 orc_rescue_res_t *res, uint32_t *cigar, int64_t cigar_cap, int nthreads)
{
	rescue_ctx_t c;
	int64_t *off, tot = 0;
	int i;
	off = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
	for (i = 0; i < n; ++i) off[i] = tot, tot += jobs[i].qlen + (jobs[i].te - jobs[i].ts) + 1;
	if (tot > cigar_cap) {
		free(off);
		return -1;
	}
	memset(&c, 0, sizeof(c));
	c.o = o, c.jobs = jobs, c.qbuf = qbuf, c.pac = pac, c.ctg_off = ctg_off, c.ambi = ambi, c.n_ambi = n_ambi;
	c.res = res, c.cigar = cigar, c.cig_off = off, c.n = n, c.next = 0;
	if (nthreads <= 1) {
		rescue_worker(&c);
	} else {
		pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
		for (i = 0; i < nthreads; ++i) pthread_create(&tid[i], 0, rescue_worker, &c);
		for (i = 0; i < nthreads; ++i) pthread_join(tid[i], 0);
		free(tid);
	}
	free(off);
	return tot;
}
