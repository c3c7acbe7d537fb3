/*
 * ksw2_oracle.h -- CPU restatement of minibwa's ksw2 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its
 * C ABI, the Python host layer) may link, call or load this code; only the
 * tests, the smoke check and the CPU-baseline leg of bench.py use it, and
 * only as the checker.
 *
 * The functions restate, in plain scalar C, the exact lane semantics of
 *   ksw2_extz2_sse.c  (ksw_extz2_sse, affine extension)
 *   ksw2_extd2_sse.c  (ksw_extd2_sse, dual-affine extension)
 *   ksw2_ll_sse.c     (ksw_ll_qinit / ksw_ll_u8_core / ksw_ll_i16_core / ksw_ll_i16)
 *   ksw2.h:124-197    (ksw_push_cigar, ksw_backtrack, ksw_reset_extz, ksw_apply_zdrop)
 * Parity is pinned by tests that compare every field and the CIGAR with the
 * reference SSE code compiled from its own sources (oracle/build_ref.sh) and
 * with golden vectors recorded from it (tests/golden/).
 */
#ifndef KSW2_ORACLE_H
#define KSW2_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as ksw_extz_t (ksw2.h:36-45). */
typedef struct {
	uint32_t max:31, zdropped:1;
	int max_q, max_t;
	int mqe, mqe_t;
	int mte, mte_q;
	int score;
	int m_cigar, n_cigar;
	int reach_end;
	uint32_t *cigar;
} orc_extz_t;

/* Same layout as ksw_llrst_t (ksw2.h:47-51). */
typedef struct {
	int score;
	int te, qe;
	int score2, te2;
} orc_llrst_t;

/* Work counters for GCUPS accounting: nominal band cells (en0-st0+1 summed over
 * the anti-diagonals actually processed) and padded cells (16-byte blocks). */
typedef struct {
	int64_t cells;
	int64_t padded_cells;
	int32_t n_diag;
} orc_stats_t;

void orc_extz2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m, const int8_t *mat,
			   int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, orc_extz_t *ez, orc_stats_t *st);

void orc_extd2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m, const int8_t *mat,
			   int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus, int flag,
			   orc_extz_t *ez, orc_stats_t *st);

void *orc_ll_qinit(int size, int qlen, const uint8_t *query, int m, const int8_t *mat);
orc_llrst_t orc_ll_u8_core(void *qp, int tlen, const uint8_t *target, int gapo, int gape, int xtra);
orc_llrst_t orc_ll_i16_core(void *qp, int tlen, const uint8_t *target, int gapo, int gape, int xtra);
int orc_ll_i16(void *qp, int tlen, const uint8_t *target, int gapo, int gape, int *qe, int *te);
/* rows of the target actually processed by the last core call on this profile */
int orc_ll_rows(const void *qp);

/* ksw_gen_nt4_mat (ksw2.h:199-219) */
void orc_gen_nt4_mat(int8_t *mat, int8_t a, int8_t b, int8_t b_ts, int8_t b_ambi, int32_t mt);

/* Batch helpers used by the CPU baseline: run a flat job list over nthreads
 * host threads (atomic work counter).  Layout of the job arrays matches the
 * GPU batch API (include/ksw2_gb300.h). */
typedef struct {
	int64_t qoff, toff;
	int32_t qlen, tlen;
	int32_t w, zdrop, end_bonus, flag;
} orc_job_t;

typedef struct {
	int32_t score, max, max_q, max_t, mqe, mqe_t, mte, mte_q;
	int32_t zdropped, reach_end, n_cigar, n_diag;
	int64_t cigar_off;
} orc_res_t;

/* kind: 0 = extz2, 1 = extd2.  cigar_out receives the CIGARs back to back
 * (cigar_off per job); cigar_cap bounds it.  Returns total CIGAR words, or -1
 * if the capacity was too small. */
int64_t orc_ext_batch(int kind, int n_jobs, const orc_job_t *jobs, const uint8_t *qbuf, const uint8_t *tbuf,
					  int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
					  orc_res_t *res, uint32_t *cigar_out, int64_t cigar_cap, int nthreads, int64_t *cells);

/* ll batch: size 1 = u8 core, 2 = i16 core. */
void orc_ll_batch(int size, int n_jobs, const orc_job_t *jobs, const uint8_t *qbuf, const uint8_t *tbuf,
				  int m, const int8_t *mat, int gapo, int gape, int xtra, orc_llrst_t *res, int nthreads,
				  int64_t *cells);

void orc_l2b_getseq(const uint64_t *pac, const uint64_t *ctg_off, int64_t n_ambi, const uint64_t *ambi, int64_t tid,
					int64_t st, int64_t len, int flags, uint8_t *seq);

int orc_ungap(int qlen, const uint8_t *qseq, int tlen, const uint8_t *tseq, int kmer, int mt, int *max_i,
			  int *n_good, int *n_kmer);

/* Mate rescue (rescue_cpu.c); layouts of ksw2g_rescue_opt_t / _job_t / _result_t. */
typedef struct {
	int32_t a, b, b_ts, b_ambi, q, e;
	int32_t bw, zdrop, end_bonus, min_len, min_dp_max;
} orc_rescue_opt_t;
typedef struct {
	int64_t qoff, ts, te;
	int32_t qlen, tid, meth, min_sc, rev, pad;
} orc_rescue_job_t;
typedef struct {
	int32_t max_ug, max_i, n_good, n_kmer;
	int64_t ts2, te2;
	int32_t ll_done, ll_score, ll_te, ll_qe, ll_score2, ll_te2;
	int32_t ext_done, rescued;
	int32_t qs, qe, dp_max2, pad;
	int64_t ts, te;
	struct {
		int32_t score, max, max_q, max_t, mqe, mqe_t, mte, mte_q;
		int32_t zdropped, reach_end, n_cigar, n_diag;
		int64_t cigar_off, cells;
	} ext;
} orc_rescue_res_t;
/* Rescue of n candidates over nthreads threads; CIGARs at res[i].ext.cigar_off in
 * cigar (qlen + te - ts + 1 words reserved per candidate).  Returns the words
 * reserved, or -1 if cigar_cap is too small. */
int64_t orc_rescue_batch(const orc_rescue_opt_t *o, int n, const orc_rescue_job_t *jobs, const uint8_t *qbuf,
						 const uint64_t *pac, const uint64_t *ctg_off, int64_t n_ambi, const uint64_t *ambi,
						 orc_rescue_res_t *res, uint32_t *cigar, int64_t cigar_cap, int nthreads);
#ifdef __cplusplus
}
#endif
#endif
