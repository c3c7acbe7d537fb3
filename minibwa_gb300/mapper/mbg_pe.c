/* mbg_pe.c -- minibwa's pairing step (pe.c) with the mate rescue of a whole mini-batch on the GPU.
 *
 * mb_pair (pe.c:461-582) rescues mates one candidate window after another: mb_matesw
 * (pe.c:380-459) walks the candidates of the pair, mb_matesw_core (pe.c:319-378) computes each
 * permitted orientation's window from the hit and the insert-size statistics, runs mb_ungap and
 * the narrowing, and mb_matesw_align (pe.c:249-312) runs ksw_ll and the reverse extz2.  Which
 * candidates run depends on the rescues before them (skip[r], pe.c:447), but no window and no
 * DP result does.  So:
 *   1. for every pair, the candidates mb_matesw would collect and the windows mb_matesw_core
 *      would try for each of them (pe.c:389-413, 326-343), on a copy of the pair's hits;
 *   2. every window of the mini-batch through one ksw2g_rescue_batch on the device (mb_ungap,
 *      the narrowing, ksw_ll and extz2, pe.c:344-358 and 262-291);
 *   3. mb_pair itself per pair on the kt_for workers, its call of mb_matesw_align replaced
 *      (one line of pe.c, substituted at build time) by mbg_matesw_align, which takes the
 *      window's device result and leaves in the hit what mb_matesw_align leaves (pe.c:261-311).
 * Pairs whose rescue stops early leave some device results unused. */
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "kalloc.h"
#include "kthread.h"
#include "ksw2.h"
#include "ksw2_gb300.h"
#include "mbg.h"

static void mbg_matesw_align(void *km, const mb_opt_t *opt, int32_t qlen, uint8_t *qseq, int32_t tlen, uint8_t *tseq,
                             mb_hit_t *h, int32_t min_sc, l2b_meth_t mt, ksw_extz_t *ez, int64_t tid, int64_t ts,
                             int64_t te, int is_rev);

#include "pe_batched.c"  // the reference's pe.c, its call of mb_matesw_align (pe.c:359) routed to mbg_matesw_align

ksw2g_ctx_t *mbg_ctx(const mb_idx_t *idx);  // mbg_map.c
ksw2g_ref_t *mbg_ref(void);

typedef struct {
	int64_t tid, ts, te;  // the window before mb_ungap's narrowing
	int32_t is_rev, len;  // orientation and length of the rescued read
	int32_t rr, mt;       // the rescued read (0 or 1) and the window's methylation mode
	int32_t min_sc, job;  // min_sc already divided by a; the job's index in the batch
} mbg_rwin_t;

typedef struct {
	int32_t n_win;
	mbg_rwin_t *win;
	uint8_t *qs;        // both reads in both orientations, as mb_matesw lays them out (pe.c:416-427)
	int32_t qlen[2];
	int64_t q_base;     // of qs in the batch's read buffer
} mbg_pair_t;

typedef struct {
	const mb_opt_t *opt;
	const mb_idx_t *idx;
	const int32_t *seg_off, *seg_cnt;
	const mb_bseq1_t *seq;
	int32_t *n_hit;
	mb_hit_t **hit;
	const mb_pestat_t *pes;
	mb_tbuf_t **tbuf;
	mbg_pair_t *pr;
	const ksw2g_rescue_result_t *res;
	const uint32_t *cig;
} mbg_pe_shared_t;

#define MBG_MS(a, b) (((b).tv_sec - (a).tv_sec) * 1e3 + ((b).tv_usec - (a).tv_usec) * 1e-3)

static __thread const mbg_pair_t *tl_pair;
static __thread const mbg_pe_shared_t *tl_pe;

static void mbg_pe_collect(void *data, long i, int tid)
{ // the windows mb_matesw_core would try for every candidate of mb_matesw (speculatively: no skip)
	const mbg_pe_shared_t *s = (const mbg_pe_shared_t*)data;
	const mb_opt_t *opt = s->opt;
	const l2b_t *l2b = s->idx->l2b;
	mbg_pair_t *P = &s->pr[i];
	void *km = mb_tbuf_km(s->tbuf[tid]);
	int32_t off, r, k, n_hit[2], is_meth = !!(opt->flag & MB_F_METH), min_sc[2], dir, skip[4], m_win = 0;
	mb_hit_t *hit[2];
	mb_pairaux_t paux;
	if (s->seg_cnt[i] != 2) return;
	off = s->seg_off[i];
	n_hit[0] = s->n_hit[off], n_hit[1] = s->n_hit[off + 1];
	if ((n_hit[0] == 0 && n_hit[1] == 0) || opt->max_rescue == 0) return;
	for (r = 0; r < 2; ++r) { // mb_pair_hits sets proper_pair: work on copies
		hit[r] = (mb_hit_t*)malloc((n_hit[r] + 1) * sizeof(mb_hit_t));
		if (n_hit[r]) memcpy(hit[r], s->hit[off + r], n_hit[r] * sizeof(mb_hit_t));
	}
	mb_pair_hits(km, opt, l2b, n_hit, hit, s->pes, &paux);
	for (dir = 0; dir < 4; ++dir) skip[dir] = !!s->pes[dir].failed;
	if ((paux.n_pp > 0 && paux.score == paux.sub_sc) || skip[0] + skip[1] + skip[2] + skip[3] == 4) goto end_collect;
	for (r = 0; r < 2; ++r) {
		const mb_bseq1_t *t = &s->seq[off + r];
		P->qlen[r] = t->l_seq;
	}
	P->qs = (uint8_t*)malloc(2 * ((int64_t)P->qlen[0] + P->qlen[1]) + 1);
	for (r = 0; r < 2; ++r) {
		uint8_t *f = P->qs + (r? 2 * P->qlen[0] : 0), *b = f + P->qlen[r];
		const char *q = s->seq[off + r].seq;
		for (k = 0; k < P->qlen[r]; ++k) {
			int32_t c = kom_nt4_table[(uint8_t)q[k]];
			f[k] = c, b[P->qlen[r] - 1 - k] = c < 4? 3 - c : 4;
		}
	}
	min_sc[0] = mb_hit_sum_score(km, n_hit[0], hit[0]) / opt->a - opt->pen_unpair;
	min_sc[1] = mb_hit_sum_score(km, n_hit[1], hit[1]) / opt->a - opt->pen_unpair;
	for (r = 0; r < 2; ++r) {
		int32_t m, j, len = P->qlen[!r];
		const mb_hit_t *h0s = hit[r];
		for (j = 0, m = 0; j < n_hit[r] && m < opt->max_rescue; ++j) {
			const mb_hit_t *h0 = &h0s[j];
			l2b_meth_t mt0 = !is_meth? L2B_METH_NONE : r == 0? L2B_METH_G2A : L2B_METH_C2T; // pe.c:442
			int64_t pos5;
			if (!(h0->proper_pair == 0 && h0->p->dp_max >= h0s[0].p->dp_max - opt->pen_unpair * opt->a)) continue;
			++m;
			pos5 = h0->rev? h0->te : h0->ts;
			for (dir = 0; dir < 4; ++dir) { // pe.c:326-343
				int is_rev, is_larger;
				int64_t ts, te;
				if (skip[dir]) continue;
				is_rev = (dir>>1 != (dir&1)) ^ h0->rev;
				if (dir>>1 != (dir&1)) is_larger = dir>>1 ^ is_rev;
				else is_larger = dir>>1 ^ r ^ h0->rev;
				ts = (is_larger? pos5 + s->pes[dir].lo : pos5 - s->pes[dir].hi) - (!is_rev? 0 : len);
				te = (is_larger? pos5 + s->pes[dir].hi : pos5 - s->pes[dir].lo) + (!is_rev? len : 0);
				if (ts < 0) ts = 0;
				if (te > (int64_t)l2b->ctg[h0->tid].len) te = l2b->ctg[h0->tid].len;
				if (te - ts <= len) continue;
				if (P->n_win == m_win) P->win = (mbg_rwin_t*)realloc(P->win, (m_win = m_win? m_win << 1 : 4) * sizeof(mbg_rwin_t));
				{
					mbg_rwin_t *w = &P->win[P->n_win++];
					w->tid = h0->tid, w->ts = ts, w->te = te, w->is_rev = is_rev, w->len = len;
					w->rr = !r, w->mt = (int32_t)(is_rev? l2b_meth_rev(mt0) : mt0), w->min_sc = min_sc[!r], w->job = -1;
				}
			}
		}
	}
end_collect:
	free(hit[0]), free(hit[1]);
}

static void mbg_pe_worker(void *data, long i, int tid)
{ // worker_for_pe (map-main.c:96-110) with this pair's device results in reach of mbg_matesw_align
	const mbg_pe_shared_t *s = (const mbg_pe_shared_t*)data;
	int32_t off, r, len[2];
	char *seq[2];
	if (s->seg_cnt[i] != 2) return;
	off = s->seg_off[i];
	for (r = 0; r < 2; ++r)
		seq[r] = s->seq[off + r].seq, len[r] = s->seq[off + r].l_seq;
	tl_pair = &s->pr[i], tl_pe = s;
	mb_pair(mb_tbuf_km(s->tbuf[tid]), s->opt, s->idx->l2b, &s->n_hit[off], &s->hit[off], s->pes, len, seq);
	tl_pair = 0, tl_pe = 0;
}

static void mbg_matesw_align(void *km, const mb_opt_t *opt, int32_t qlen, uint8_t *qseq, int32_t tlen, uint8_t *tseq,
                             mb_hit_t *h, int32_t min_sc, l2b_meth_t mt, ksw_extz_t *ez, int64_t tid, int64_t ts,
                             int64_t te, int is_rev)
{ // mb_matesw_align (pe.c:249-312) from the window's device result
	const mbg_pair_t *P = tl_pair;
	const ksw2g_rescue_result_t *R = 0;
	int8_t mat[25];
	int32_t k, max_sc = qlen < tlen? qlen : tlen;
	(void)ez;
	memset(h, 0, sizeof(*h));
	for (k = 0; P && k < P->n_win; ++k)
		if (P->win[k].tid == tid && P->win[k].ts == ts && P->win[k].te == te && P->win[k].is_rev == is_rev &&
			P->win[k].len == qlen) {
			R = &tl_pe->res[P->win[k].job];
			break;
		}
	if (!R || R->te2 - R->ts2 != tlen) {
		fprintf(stderr, "[E::%s] no device result for the rescue window [%ld,%ld) of contig %ld\n", __func__, (long)ts,
				(long)te, (long)tid);
		exit(1);
	}
	if (max_sc >= 32767 || !R->ll_done) return;
	if (R->ll_score >= opt->min_dp_max && R->ll_score >= min_sc && R->ext_done && R->ext.n_cigar > 0 &&
		R->ext.max >= opt->min_dp_max * opt->a) {
		const ksw2g_ext_result_t *E = &R->ext;
		int32_t qe = R->ll_qe + 1, te1 = R->ll_te + 1;
		mb_append_cigar(h, E->n_cigar, tl_pe->cig + E->cigar_off);
		h->rescued = 1;
		h->qe = qe, h->te = te1;
		h->ts = te1 - (E->reach_end? E->mqe_t + 1 : E->max_t + 1);
		h->qs = qe - (E->reach_end? qe : E->max_q + 1);
		h->p->dp_max = h->p->dp_score = E->max;
		h->p->dp_max2 = (int32_t)((double)E->max / R->ll_score * R->ll_score2 + .499);
		if (h->p->dp_max2 < 0) h->p->dp_max2 = 0;
		h->score = h->score0 = R->ll_score;
		h->subsc = R->ll_score2;
		h->cnt = 0, h->as = -1;
		h->parent = MB_PARENT_UNSET;
		ksw_gen_nt4_mat(mat, opt->a, opt->b, opt->b_ts, opt->b_ambi, (int)mt);
		mb_update_extra(km, h, &qseq[h->qs], &tseq[h->ts], mat, opt->q, opt->e, opt->flag, 0);
	}
}

void mbg_pair_step(const mb_opt_t *opt, const mb_idx_t *idx, int n_thread, mb_tbuf_t **tbuf, int64_t n_frag,
                   const int32_t *seg_off, const int32_t *seg_cnt, const mb_bseq1_t *seq, int32_t *n_hit,
                   mb_hit_t **hit, const mb_pestat_t *pes)
{
	mbg_pe_shared_t s;
	int64_t i, n_job = 0, n_q = 0, cap = 16, used = 0;
	int32_t k;
	ksw2g_rescue_job_t *jobs;
	ksw2g_rescue_result_t *res = 0;
	ksw2g_rescue_opt_t ro;
	uint32_t *cig = 0;
	uint8_t *qbuf;
	struct timeval t0, t1, t2, t3;
	gettimeofday(&t0, 0);
	memset(&s, 0, sizeof(s));
	s.opt = opt, s.idx = idx, s.seg_off = seg_off, s.seg_cnt = seg_cnt, s.seq = seq, s.n_hit = n_hit, s.hit = hit;
	s.pes = pes, s.tbuf = tbuf;
	s.pr = (mbg_pair_t*)calloc(n_frag + 1, sizeof(mbg_pair_t));
	kt_for(n_thread, mbg_pe_collect, &s, n_frag);
	gettimeofday(&t1, 0);
	for (i = 0; i < n_frag; ++i) {
		mbg_pair_t *P = &s.pr[i];
		if (P->n_win == 0) continue;
		P->q_base = n_q, n_q += 2 * ((int64_t)P->qlen[0] + P->qlen[1]);
		n_job += P->n_win;
	}
	if (n_job > 0) { // every window of the mini-batch in one device batch
		jobs = (ksw2g_rescue_job_t*)calloc(n_job, sizeof(ksw2g_rescue_job_t));
		qbuf = (uint8_t*)malloc(n_q + 1);
		for (i = 0, n_job = 0; i < n_frag; ++i) {
			mbg_pair_t *P = &s.pr[i];
			if (P->n_win == 0) continue;
			memcpy(qbuf + P->q_base, P->qs, 2 * ((size_t)P->qlen[0] + P->qlen[1]));
			for (k = 0; k < P->n_win; ++k) {
				mbg_rwin_t *w = &P->win[k];
				ksw2g_rescue_job_t *J = &jobs[n_job];
				J->qoff = P->q_base + (w->rr? 2 * (int64_t)P->qlen[0] : 0) + (w->is_rev? P->qlen[w->rr] : 0);
				J->ts = w->ts, J->te = w->te, J->qlen = w->len, J->tid = (int32_t)w->tid;
				J->meth = w->mt, J->min_sc = w->min_sc, J->rev = w->is_rev;
				w->job = (int32_t)n_job++;
				cap += w->len + (w->te - w->ts) + 1;
			}
		}
		ro.a = opt->a, ro.b = opt->b, ro.b_ts = opt->b_ts, ro.b_ambi = opt->b_ambi, ro.q = opt->q, ro.e = opt->e;
		ro.bw = opt->bw, ro.zdrop = opt->zdrop, ro.end_bonus = opt->end_bonus, ro.min_len = opt->min_len;
		ro.min_dp_max = opt->min_dp_max;
		res = (ksw2g_rescue_result_t*)calloc(n_job, sizeof(ksw2g_rescue_result_t));
		cig = (uint32_t*)malloc(cap * sizeof(uint32_t));
		if (ksw2g_rescue_batch(mbg_ctx(idx), mbg_ref(), &ro, (int)n_job, jobs, qbuf, n_q + 1, res, cig, cap, &used)) {
			fprintf(stderr, "[E::%s] ksw2g_rescue_batch: %s\n", __func__, ksw2g_last_error());
			exit(1);
		}
		s.res = res, s.cig = cig;
		free(jobs), free(qbuf);
	}
	gettimeofday(&t2, 0);
	kt_for(n_thread, mbg_pe_worker, &s, n_frag);
	gettimeofday(&t3, 0);
	if (getenv("MBG_TIMING"))
		fprintf(stderr, "[M::mbg] pairing: %ld fragments, %ld rescue windows; windows %.1f ms, device rescue %.1f ms, "
				"mb_pair %.1f ms\n", (long)n_frag, (long)n_job, MBG_MS(t0, t1), MBG_MS(t1, t2), MBG_MS(t2, t3));
	for (i = 0; i < n_frag; ++i) free(s.pr[i].win), free(s.pr[i].qs);
	free(s.pr), free(res), free(cig);
}
