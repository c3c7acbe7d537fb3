/* ref_align.c -- harness around the reference's mb_align_pair and mb_align1 (TEST
 * INFRASTRUCTURE ONLY).
 *
 * Built by `make ref` into _ref/libmbpe.so with ref_pe.c and the reference's
 * library sources, compiled where they lie in the reference tree.  It includes
 * the reference's align.c -- as _ref/align_noextra.c, the same file with the
 * one call of mb_update_extra at the end of mb_align1 (align.c:753) replaced by
 * a no-op, a change the Makefile makes at build time -- so that its static
 * mb_align_pair (align.c:329-390: the ungapped shortcuts, the band shrink, the
 * memory cap and the choice of extz2 or extd2 in front of every DP call of
 * mb_align1) and mb_align1 (align.c:548-757) can be called on synthetic inputs;
 * the batched restatements on the device are pinned against them.
 * mb_update_extra fixes leading indels and recounts the scores for mapQ after
 * the alignment; the device entry point leaves it to the caller.
 */
#include <stdlib.h>
#include <string.h>

#include "align_noextra.c"

/* sc: a, b, b_ts, b_ambi, q, e, q2, e2, meth (nonzero: MB_F_METH); max_sw_mat separate.
 * out: max zdropped max_q max_t mqe mqe_t mte mte_q score n_cigar reach_end.
 * Returns 0, or -1 when the CIGAR does not fit. */
int refal_align_pair(const int32_t *sc, int64_t max_sw_mat, int qlen, const uint8_t *qseq, int tlen,
                     const uint8_t *tseq, const int8_t *mat, int w, int end_bonus, int zdrop, int ksw_flag,
                     int32_t *out, uint32_t *cigar, int cigar_cap)
{
	mb_opt_t opt;
	ksw_extz_t ez;
	int rc = 0;
	memset(&opt, 0, sizeof opt);
	opt.a = sc[0], opt.b = sc[1], opt.b_ts = sc[2], opt.b_ambi = sc[3];
	opt.q = sc[4], opt.e = sc[5], opt.q2 = sc[6], opt.e2 = sc[7];
	if (sc[8]) opt.flag |= MB_F_METH;
	opt.max_sw_mat = max_sw_mat;
	memset(&ez, 0, sizeof ez);
	mb_align_pair(0, &opt, qlen, qseq, tlen, tseq, mat, w, end_bonus, zdrop, ksw_flag, &ez);
	out[0] = (int32_t)ez.max, out[1] = ez.zdropped, out[2] = ez.max_q, out[3] = ez.max_t, out[4] = ez.mqe;
	out[5] = ez.mqe_t, out[6] = ez.mte, out[7] = ez.mte_q, out[8] = ez.score, out[9] = ez.n_cigar;
	out[10] = ez.reach_end;
	if (ez.n_cigar <= cigar_cap) memcpy(cigar, ez.cigar, (size_t)ez.n_cigar * 4);
	else rc = -1;
	free(ez.cigar);
	return rc;
}

/* mb_align1 on one hit over a reference built from l2b arrays.  optv: a, b, b_ts, b_ambi, q, e,
 * q2, e2, bw, bw_long, max_gap, end_bonus, zdrop, zdrop_inv, min_ksw_len, min_len,
 * min_chain_score, min_dp_max, long_reads, adaptive, max_sr_len, meth, max_sw_mat.
 * anchors: n_a records of (sid, len, qpos, flag) in ai and tpos in at; the hit is
 * anchors[as .. as+cnt).  out: ts, te, qs, qe, dp_score, n_cigar, cnt, score, r2 cnt (0: no
 * split), r2 as, r2 split_inv, r2 score.  Returns 0, or -1 when the CIGAR does not fit. */
int refal_align1(int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len, const uint64_t *pac, int64_t n_pac,
                 int64_t n_ambi, const uint64_t *ambi, const int64_t *optv, int qlen, uint8_t *seq_fwd,
                 uint8_t *seq_rc, int mt, int n_a, const int32_t *ai, const int64_t *at, int as, int cnt, int mlen,
                 int score, int split_inv, int64_t *out, uint32_t *cigar, int cigar_cap)
{
	l2b_t l2b;
	mb_idx_t mi;
	mb_opt_t opt;
	mb_hit_t r, r2;
	ksw_extz_t ez;
	mb_anchor_t *a;
	uint8_t *qseq0[2];
	int64_t k;
	int rc = 0;
	memset(&l2b, 0, sizeof l2b);
	l2b.n_ctg = l2b.m_ctg = n_ctg;
	l2b.ctg = (l2b_ctg_t *)calloc(n_ctg, sizeof(l2b_ctg_t));
	for (k = 0; k < n_ctg; ++k) l2b.ctg[k].off = ctg_off[k], l2b.ctg[k].len = ctg_len[k], l2b.tot_len += ctg_len[k];
	l2b.pac = (uint64_t *)pac, l2b.n_pac = l2b.m_pac = n_pac;
	l2b.n_ambi = l2b.m_ambi = n_ambi, l2b.ambi = (l2b_intv_t *)ambi;
	memset(&mi, 0, sizeof mi);
	mi.l2b = &l2b;
	memset(&opt, 0, sizeof opt);
	opt.a = optv[0], opt.b = optv[1], opt.b_ts = optv[2], opt.b_ambi = optv[3];
	opt.q = optv[4], opt.e = optv[5], opt.q2 = optv[6], opt.e2 = optv[7];
	opt.bw = optv[8], opt.bw_long = optv[9], opt.max_gap = optv[10], opt.end_bonus = optv[11];
	opt.zdrop = optv[12], opt.zdrop_inv = optv[13], opt.min_ksw_len = optv[14], opt.min_len = optv[15];
	opt.min_chain_score = optv[16], opt.min_dp_max = optv[17];
	if (optv[18]) opt.flag |= MB_F_LONG;
	if (optv[19]) opt.flag |= MB_F_ADAP;
	opt.max_sr_len = optv[20];
	if (optv[21]) opt.flag |= MB_F_METH;
	opt.max_sw_mat = optv[22];
	a = (mb_anchor_t *)calloc(n_a, sizeof(mb_anchor_t));
	for (k = 0; k < n_a; ++k) {
		a[k].sid = ai[4 * k], a[k].len = ai[4 * k + 1], a[k].qpos = ai[4 * k + 2], a[k].flag = ai[4 * k + 3];
		a[k].tpos = at[k];
	}
	memset(&r, 0, sizeof r);
	memset(&r2, 0, sizeof r2);
	r.as = as, r.cnt = cnt, r.mlen = mlen, r.score = score, r.split_inv = split_inv;
	r.tid = a[as].sid >> 1, r.rev = a[as].sid & 1;
	r.id = 0, r.parent = 0;
	qseq0[0] = seq_fwd, qseq0[1] = seq_rc;
	memset(&ez, 0, sizeof ez);
	mb_align1(0, &opt, &mi, qlen, qseq0, (l2b_meth_t)mt, &r, &r2, n_a, a, &ez);
	out[0] = r.ts, out[1] = r.te, out[2] = r.qs, out[3] = r.qe;
	out[4] = r.p ? r.p->dp_score : 0, out[5] = r.p ? r.p->n_cigar : 0;
	out[6] = r.cnt, out[7] = r.score;
	out[8] = r2.cnt, out[9] = r2.as, out[10] = r2.split_inv, out[11] = r2.score;
	if (r.p) {
		if (r.p->n_cigar <= cigar_cap) memcpy(cigar, r.p->cigar, (size_t)r.p->n_cigar * 4);
		else rc = -1;
		free(r.p);
	}
	free(ez.cigar);
	free(a);
	free(l2b.ctg);
	return rc;
}
