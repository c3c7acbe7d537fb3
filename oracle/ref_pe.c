/* ref_pe.c -- harness around the reference's own mate rescue (TEST INFRASTRUCTURE ONLY).
 *
 * Built by `make ref` into _ref/libmbpe.so together with the reference's
 * library sources, compiled where they lie in the reference tree.  It includes
 * the reference's pe.c so that its static mb_ungap and mb_matesw_core can be
 * called on synthetic inputs: the rescue restatement in oracle.py (and through
 * it the device pipeline) is pinned against these calls.
 *
 * mb_update_extra (align.c:219), which runs after a rescued extension to fix
 * leading indels and recount the score for mapQ, is outside the rescue's
 * kernels; it is replaced by a no-op here so that the harness returns the hit
 * exactly as the extension left it (pe.c:291-304, 361-368).
 */
#include <stdlib.h>
#include <string.h>

#include "mbpriv.h"
#define mb_update_extra(km, r, qseq, tseq, mat, q, e, flag, lg) ((void)0)
#include "pe.c"

int refpe_ungap(int qlen, const uint8_t *q, int tlen, const uint8_t *t, int kmer, int mt, int *max_i, int *n_good,
                int *n_kmer)
{
	return mb_ungap(0, qlen, q, tlen, t, kmer, (l2b_meth_t)mt, max_i, n_good, n_kmer);
}

static void refpe_l2b(l2b_t *l2b, int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len, const uint64_t *pac,
                      int64_t n_pac, int64_t n_ambi, const uint64_t *ambi)
{
	int64_t k;
	memset(l2b, 0, sizeof *l2b);
	l2b->n_ctg = l2b->m_ctg = n_ctg;
	l2b->ctg = (l2b_ctg_t *)calloc(n_ctg, sizeof(l2b_ctg_t));
	for (k = 0; k < n_ctg; ++k) l2b->ctg[k].off = ctg_off[k], l2b->ctg[k].len = ctg_len[k], l2b->tot_len += ctg_len[k];
	l2b->pac = (uint64_t *)pac, l2b->n_pac = l2b->m_pac = n_pac;
	l2b->n_ambi = l2b->m_ambi = n_ambi, l2b->ambi = (l2b_intv_t *)ambi;
}

/* The reference's l2b_getseq on [st, en) of contig tid; returns its return value. */
int64_t refpe_getseq(int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len, const uint64_t *pac,
                     int64_t n_pac, int64_t n_ambi, const uint64_t *ambi, int64_t tid, int64_t st, int64_t en,
                     uint8_t *seq)
{
	l2b_t l2b;
	int64_t r;
	refpe_l2b(&l2b, n_ctg, ctg_off, ctg_len, pac, n_pac, n_ambi, ambi);
	r = l2b_getseq(&l2b, tid, st, en, seq);
	free(l2b.ctg);
	return r;
}

/* One mb_matesw_core call with a single permitted orientation dir (the other
 * three marked failed).  sc: a, b, b_ts, b_ambi, q, e, bw, zdrop, end_bonus,
 * min_len, min_dp_max.  out: rescued, ts, te, qs, qe, rev, dp_max, dp_max2,
 * score, subsc, n_cigar.  Returns 0, or -1 when the CIGAR does not fit. */
int refpe_matesw(int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len, const uint64_t *pac, int64_t n_pac,
                 int64_t n_ambi, const uint64_t *ambi, const int32_t *sc, int dir, int lo, int hi, int64_t tid,
                 int64_t h_ts, int64_t h_te, int h_rev, int r0, int len, uint8_t *seq_fwd, uint8_t *seq_rc, int mt0,
                 int min_sc, int64_t *out, uint32_t *cigar, int cigar_cap)
{
	l2b_t l2b;
	mb_opt_t opt;
	mb_pestat_t pes[4];
	mb_hit_t h0;
	mb_hit_v h1 = {0, 0, 0};
	ksw_extz_t ez;
	uint8_t *seq[2];
	const mb_hit_t *ret;
	int64_t k;
	int rc = 0;
	refpe_l2b(&l2b, n_ctg, ctg_off, ctg_len, pac, n_pac, n_ambi, ambi);
	memset(&opt, 0, sizeof opt);
	opt.a = sc[0], opt.b = sc[1], opt.b_ts = sc[2], opt.b_ambi = sc[3], opt.q = sc[4], opt.e = sc[5];
	opt.bw = sc[6], opt.zdrop = sc[7], opt.end_bonus = sc[8], opt.min_len = sc[9], opt.min_dp_max = sc[10];
	memset(pes, 0, sizeof pes);
	for (k = 0; k < 4; ++k) pes[k].failed = k != dir, pes[k].lo = lo, pes[k].hi = hi;
	memset(&h0, 0, sizeof h0);
	h0.tid = tid, h0.ts = h_ts, h0.te = h_te, h0.rev = h_rev;
	seq[0] = seq_fwd, seq[1] = seq_rc;
	memset(&ez, 0, sizeof ez);
	ret = mb_matesw_core(0, &opt, &l2b, pes, &h0, r0, len, seq, (l2b_meth_t)mt0, &h1, min_sc, &ez);
	memset(out, 0, 11 * sizeof(int64_t));
	if (ret) {
		out[0] = ret->rescued, out[1] = ret->ts, out[2] = ret->te, out[3] = ret->qs, out[4] = ret->qe;
		out[5] = ret->rev, out[6] = ret->p->dp_max, out[7] = ret->p->dp_max2, out[8] = ret->score;
		out[9] = ret->subsc, out[10] = ret->p->n_cigar;
		if (ret->p->n_cigar <= cigar_cap) memcpy(cigar, ret->p->cigar, ret->p->n_cigar * 4);
		else rc = -1;
	}
	for (k = 0; k < h1.n; ++k) free(h1.a[k].p);
	free(h1.a);
	free(ez.cigar);
	free(l2b.ctg);
	return rc;
}
