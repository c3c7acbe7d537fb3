/* Batched mb_align1 for minibwa's mapping pipeline.
 *
 * minibwa maps a mini-batch of reads in map-main.c's worker_pipeline step 1: kt_for runs
 * worker_for_se_batch over sub-batches of 24 fragments, and every read goes through
 * mb_map_sai (map-algo.c:578-664), whose mb_align_skeleton (align.c:894-930) calls mb_align1
 * hit after hit, each gap fill and end extension one synchronous ksw2 call.
 *
 * The build of the batched minibwa changes two lines of map-main.c (Makefile beside this
 * file): the worker's call of mb_map_sai becomes mbg_map_sai_defer, and step 1 brackets its
 * kt_for with mbg_step_begin / mbg_step_end.  The read is seeded, chained and its hits ordered
 * on the worker thread as before; its alignment is deferred.  mbg_step_end then aligns the
 * hits of every read of the mini-batch at once through ksw2g_align_chains on the GPU (hits split
 * off by a z-drop in later rounds, as mb_align_skeleton reaches them), and finishes every read
 * on kt_for workers: mb_update_extra, the inversion check between split hits (mb_align1_inv,
 * its ksw_ll and mb_align_pair batched on the GPU for all reads), hit filtering and sorting,
 * and the rest of mb_map_sai.  A third line replaces step 1's pairing loop by mbg_pair_step,
 * which hands the mate-rescue windows of all pairs to the GPU at once and then runs mb_pair per
 * pair as before.  Output is byte-identical to the stock minibwa. */
#ifndef MBG_H
#define MBG_H

#include "mbpriv.h"
#include "bseq.h"

#ifdef __cplusplus
extern "C" {
#endif

void mbg_step_begin(const mb_idx_t *idx, int64_t n_seq);
void mbg_map_sai_defer(const mb_opt_t *opt, const mb_idx_t *idx, int64_t qlen, const char *seq0, l2b_meth_t mt,
                       mb_sai_v *u, int64_t rid, mb_tbuf_t *b, const char *qname);
void mbg_step_end(const mb_opt_t *opt, const mb_idx_t *idx, int n_thread, mb_tbuf_t **tbuf, int64_t n_seq,
                  mb_hit_t **hit, int32_t *n_hit);
/* step 1's pairing loop (kt_for over worker_for_pe) with the mate rescue of all pairs batched (mbg_pe.c) */
void mbg_pair_step(const mb_opt_t *opt, const mb_idx_t *idx, int n_thread, mb_tbuf_t **tbuf, int64_t n_frag,
                   const int32_t *seg_off, const int32_t *seg_cnt, const mb_bseq1_t *seq, int32_t *n_hit,
                   mb_hit_t **hit, const mb_pestat_t *pes);

#ifdef __cplusplus
}
#endif
#endif
