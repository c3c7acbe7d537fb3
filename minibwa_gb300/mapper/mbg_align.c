/* The reference's align.c, compiled here in place of align.o, with its static mb_align1_inv
 * (align.c:759-815) exported for the batched pipeline of mbg_map.c. */
#include "align.c"
#include "mbg.h"

int mbg_align1_inv(void *km, const mb_opt_t *opt, const mb_idx_t *mi, int qlen, uint8_t *qseq0[2], l2b_meth_t mt,
                   const mb_hit_t *r1, const mb_hit_t *r2, mb_hit_t *r_inv)
{
	ksw_extz_t ez;
	int ret;
	memset(&ez, 0, sizeof(ksw_extz_t));
	ret = mb_align1_inv(km, opt, mi, qlen, qseq0, mt, r1, r2, r_inv, &ez);
	kfree(km, ez.cigar);
	return ret;
}
