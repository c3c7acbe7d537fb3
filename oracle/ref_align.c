/* ref_align.c -- harness around the reference's mb_align_pair (TEST INFRASTRUCTURE ONLY).
 *
 * Built by `make ref` into _ref/libmbpe.so with ref_pe.c and the reference's
 * library sources, compiled where they lie in the reference tree.  It includes
 * the reference's align.c so that its static mb_align_pair (align.c:329-390:
 * the ungapped shortcuts, the band shrink, the memory cap and the choice of
 * extz2 or extd2 in front of every DP call of mb_align1) can be called on
 * synthetic inputs; the batched restatement on the device is pinned against it.
 */
#include <stdlib.h>
#include <string.h>

#include "align.c"

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
