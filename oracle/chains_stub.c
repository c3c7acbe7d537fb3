/* chains_stub.c -- ksw2g_align_chains computed by the reference's own mb_align1 on the CPU
 * (TEST INFRASTRUCTURE ONLY).
 *
 * The batched minibwa (minibwa_gb300/mapper) calls nine functions of libksw2gpu.so:
 * ksw2g_ctx_create, ksw2g_ref_create, ksw2g_ref_destroy, ksw2g_align_chains (and its stats),
 * ksw2g_ll_batch, ksw2g_align_pairs, ksw2g_rescue_batch and ksw2g_last_error.  This file
 * provides them over the reference's own code -- mate rescue over the oracle's restatement of
 * it (rescue_cpu.c), which is pinned to the reference's mb_matesw_core -- and the
 * reference's align.c (included as
 * _ref/align_noextra.c, mb_update_extra at the end of mb_align1 left out, as the device entry
 * point leaves it to its caller): each hit goes through mb_align1 as mb_align_skeleton would
 * call it.  Linked with the reference's ksw2 sources in place of libksw2gpu.so (make
 * mbgstub), the batched mapper then runs without a GPU, so the host side of the batched
 * pipeline -- deferral, rounds of split-off hits, the finishing pass -- can be checked for
 * byte-identical SAM on any machine that has the reference tree.  The device entry point
 * itself is pinned to mb_align1 separately (tests/test_gpu_chains.py). */
#include <stdlib.h>
#include <string.h>

#include "align_noextra.c"
#include "ksw2_gb300.h"
#include "ksw2_oracle.h"

struct ksw2g_ctx { int device; };
struct ksw2g_ref { l2b_t l2b; uint64_t *off; };

const char *ksw2g_last_error(void) { return "chains stub"; }

int ksw2g_align_chains_last_stats(const ksw2g_ctx_t *ctx, double *ms, int64_t *counts)
{
	int k;
	(void)ctx;
	for (k = 0; k < 6; ++k) if (ms) ms[k] = 0;
	for (k = 0; k < 4; ++k) if (counts) counts[k] = 0;
	return 0;
}

int ksw2g_ctx_create(int device, ksw2g_ctx_t **ctx)
{
	*ctx = (ksw2g_ctx_t*)calloc(1, sizeof(ksw2g_ctx_t));
	(*ctx)->device = device;
	return 0;
}

int ksw2g_ref_create(ksw2g_ctx_t *ctx, int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len,
                     const uint64_t *pac, int64_t n_pac, int64_t n_ambi, const uint64_t *ambi, ksw2g_ref_t **ref)
{
	ksw2g_ref_t *r = (ksw2g_ref_t*)calloc(1, sizeof(ksw2g_ref_t));
	int64_t k;
	(void)ctx;
	r->l2b.n_ctg = r->l2b.m_ctg = n_ctg;
	r->l2b.ctg = (l2b_ctg_t*)calloc(n_ctg + 1, sizeof(l2b_ctg_t));
	r->off = (uint64_t*)calloc(n_ctg + 1, sizeof(uint64_t));
	for (k = 0; k < n_ctg; ++k)
		r->l2b.ctg[k].off = r->off[k] = ctg_off[k], r->l2b.ctg[k].len = ctg_len[k], r->l2b.tot_len += ctg_len[k];
	r->l2b.pac = (uint64_t*)pac, r->l2b.n_pac = r->l2b.m_pac = n_pac;
	r->l2b.n_ambi = r->l2b.m_ambi = n_ambi, r->l2b.ambi = (l2b_intv_t*)ambi;
	*ref = r;
	return 0;
}

void ksw2g_ref_destroy(ksw2g_ref_t *ref)
{
	if (ref) free(ref->l2b.ctg), free(ref->off), free(ref);
}

static void stub_opt(const ksw2g_chain_opt_t *c, mb_opt_t *o)
{
	memset(o, 0, sizeof(*o));
	o->a = c->a, o->b = c->b, o->b_ts = c->b_ts, o->b_ambi = c->b_ambi;
	o->q = c->q, o->e = c->e, o->q2 = c->q2, o->e2 = c->e2;
	o->bw = c->bw, o->bw_long = c->bw_long, o->max_gap = c->max_gap, o->end_bonus = c->end_bonus;
	o->zdrop = c->zdrop, o->zdrop_inv = c->zdrop_inv, o->min_ksw_len = c->min_ksw_len, o->min_len = c->min_len;
	o->min_chain_score = c->min_chain_score, o->min_dp_max = c->min_dp_max;
	if (c->long_reads) o->flag |= MB_F_LONG;
	if (c->adaptive) o->flag |= MB_F_ADAP;
	o->max_sr_len = c->max_sr_len;
	if (c->meth) o->flag |= MB_F_METH;
	o->max_sw_mat = c->max_sw_mat;
}

int ksw2g_align_chains(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, int n_opts, const ksw2g_chain_opt_t *opts,
                       int n_chains, const ksw2g_chain_t *chains, ksw2g_anchor_t *anchors, int64_t n_anchors,
                       const uint8_t *qbuf, int64_t qbuf_len, ksw2g_chain_result_t *res, uint32_t *cigar,
                       int64_t cigar_cap, int64_t *cigar_used)
{
	mb_idx_t mi;
	mb_anchor_t *a;
	ksw_extz_t ez;
	int64_t k, used = 0;
	int i;
	(void)ctx, (void)qbuf_len;
	memset(&mi, 0, sizeof mi);
	mi.l2b = (l2b_t*)&ref->l2b;
	a = (mb_anchor_t*)calloc(n_anchors + 1, sizeof(mb_anchor_t));
	for (k = 0; k < n_anchors; ++k) {
		a[k].sid = anchors[k].sid, a[k].len = anchors[k].len, a[k].qpos = anchors[k].qpos;
		a[k].flag = anchors[k].flag & 0x7fffffffu, a[k].flt = anchors[k].flag >> 31, a[k].tpos = anchors[k].tpos;
	}
	memset(&ez, 0, sizeof ez);
	for (i = 0; i < n_chains; ++i) {
		const ksw2g_chain_t *h = &chains[i];
		ksw2g_chain_result_t *R = &res[i];
		mb_opt_t opt;
		mb_hit_t r, r2;
		uint8_t *qseq0[2];
		int rev;
		if (h->opt < 0 || h->opt >= n_opts) return KSW2G_E_ARG;
		stub_opt(&opts[h->opt], &opt);
		memset(&r, 0, sizeof r), memset(&r2, 0, sizeof r2), memset(R, 0, sizeof(*R));
		R->cigar_off = -1, R->cnt = h->cnt, R->score = h->score;
		if (h->cnt <= 0) continue;
		rev = a[h->as].sid & 1;
		qseq0[rev] = (uint8_t*)qbuf + h->qoff; // the other orientation is not read with mb_update_extra left out
		qseq0[!rev] = (uint8_t*)qbuf + h->qoff;
		r.as = (int32_t)h->as, r.cnt = h->cnt, r.mlen = h->mlen, r.score = h->score, r.split_inv = h->split_inv;
		r.tid = a[h->as].sid >> 1, r.rev = rev;
		mb_align1(0, &opt, &mi, h->qlen, qseq0, (l2b_meth_t)h->meth, &r, &r2, (int)n_anchors, a, &ez);
		R->ts = r.ts, R->te = r.te, R->qs = r.qs, R->qe = r.qe, R->cnt = r.cnt, R->score = r.score;
		if (r2.cnt > 0) R->split_n = r2.as - (int32_t)h->as, R->split_inv2 = r2.split_inv;
		if (r.p) {
			R->dp_score = r.p->dp_score, R->n_cigar = r.p->n_cigar;
			if (cigar) {
				if (used + r.p->n_cigar > cigar_cap) { free(r.p), free(a), free(ez.cigar); return KSW2G_E_CAPACITY; }
				memcpy(cigar + used, r.p->cigar, (size_t)r.p->n_cigar * 4);
				R->cigar_off = used;
			}
			used += r.p->n_cigar;
			free(r.p);
		}
	}
	for (k = 0; k < n_anchors; ++k) anchors[k].flag = a[k].flag | (uint32_t)a[k].flt << 31;
	free(a), free(ez.cigar);
	if (cigar_used) *cigar_used = used;
	return 0;
}

/* ksw_ll_i16 (ksw2_ll_sse.c:335-341) per job, or its u8 core for size 1 */
int ksw2g_ll_batch(ksw2g_ctx_t *ctx, int size, int m, const int8_t *mat, int gapo, int gape, int n_jobs,
                   const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                   int64_t tbuf_len, ksw2g_ll_result_t *res)
{
	int i;
	(void)ctx, (void)qbuf_len, (void)tbuf_len;
	for (i = 0; i < n_jobs; ++i) {
		const ksw2g_ll_job_t *J = &jobs[i];
		void *qp = ksw_ll_qinit(0, size, J->qlen, qbuf + J->qoff, m, mat);
		ksw_llrst_t r = size == 1? ksw_ll_u8_core(qp, J->tlen, tbuf + J->toff, gapo, gape, J->xtra)
		                          : ksw_ll_i16_core(qp, J->tlen, tbuf + J->toff, gapo, gape, J->xtra);
		free(qp);
		res[i].score = r.score, res[i].te = r.te, res[i].qe = r.qe, res[i].score2 = r.score2, res[i].te2 = r.te2;
		res[i].rows = 0;
	}
	return 0;
}

/* mb_align_pair (align.c:329-390) per job */
int ksw2g_align_pairs(ksw2g_ctx_t *ctx, const ksw2g_align_opt_t *ao, const int8_t *mat, int n_jobs,
                      const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                      int64_t tbuf_len, ksw2g_ext_result_t *res, uint32_t *cigar, int64_t cigar_cap,
                      int64_t *cigar_used)
{
	mb_opt_t opt;
	ksw_extz_t ez;
	int64_t used = 0;
	int i;
	(void)ctx, (void)qbuf_len, (void)tbuf_len;
	memset(&opt, 0, sizeof opt);
	opt.a = ao->a, opt.b = ao->b, opt.b_ts = ao->b_ts, opt.b_ambi = ao->b_ambi;
	opt.q = ao->q, opt.e = ao->e, opt.q2 = ao->q2, opt.e2 = ao->e2;
	if (ao->meth) opt.flag |= MB_F_METH;
	opt.max_sw_mat = ao->max_sw_mat;
	memset(&ez, 0, sizeof ez);
	for (i = 0; i < n_jobs; ++i) {
		const ksw2g_job_t *J = &jobs[i];
		ksw2g_ext_result_t *R = &res[i];
		mb_align_pair(0, &opt, J->qlen, qbuf + J->qoff, J->tlen, tbuf + J->toff, mat, J->w, J->end_bonus, J->zdrop,
		              J->flag, &ez);
		memset(R, 0, sizeof(*R));
		R->score = ez.score, R->max = (int32_t)ez.max, R->max_q = ez.max_q, R->max_t = ez.max_t, R->mqe = ez.mqe;
		R->mqe_t = ez.mqe_t, R->mte = ez.mte, R->mte_q = ez.mte_q, R->zdropped = ez.zdropped;
		R->reach_end = ez.reach_end, R->n_cigar = ez.n_cigar;
		if (ez.n_cigar > 0 && cigar) {
			if (used + ez.n_cigar > cigar_cap) { free(ez.cigar); return KSW2G_E_CAPACITY; }
			memcpy(cigar + used, ez.cigar, (size_t)ez.n_cigar * 4);
			R->cigar_off = used;
			used += ez.n_cigar;
		}
	}
	free(ez.cigar);
	if (cigar_used) *cigar_used = used;
	return 0;
}

/* mate rescue of candidate windows (pe.c:340-368, 249-300) by the oracle's restatement */
int ksw2g_rescue_batch(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, const ksw2g_rescue_opt_t *opt, int n_jobs,
                       const ksw2g_rescue_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, ksw2g_rescue_result_t *res,
                       uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_used)
{
	int64_t r;
	(void)ctx, (void)qbuf_len;
	r = orc_rescue_batch((const orc_rescue_opt_t*)opt, n_jobs, (const orc_rescue_job_t*)jobs, qbuf, ref->l2b.pac,
	                     ref->off, (int64_t)ref->l2b.n_ambi, (const uint64_t*)ref->l2b.ambi, (orc_rescue_res_t*)res,
	                     cigar, cigar_cap, 8);
	if (r < 0) return KSW2G_E_CAPACITY;
	if (cigar_used) *cigar_used = r;
	return 0;
}
