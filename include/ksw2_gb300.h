/*
 * ksw2_gb300.h -- batched and served entry points of the GB300 ksw2 library
 * (libksw2gpu.so).  These have no one-to-one counterpart in the reference:
 * they let a caller that has many independent DP jobs (the gap fills and end
 * extensions of align.c:mb_align1, the rescue jobs of pe.c:mb_matesw_core)
 * hand them over in one call instead of one synchronous call per job.
 * Every job's result is bit-identical to the per-call ksw_extz2_sse /
 * ksw_extd2_sse / ksw_ll_* result on the same inputs.
 *
 * Conventions: plain pointers and sizes; host buffers unless a name says
 * "dev"; return value 0 on success or a negative KSW2G_E* code, with a
 * thread-local message from ksw2g_last_error().
 */
#ifndef KSW2_GB300_H_
#define KSW2_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KSW2G_OK           0
#define KSW2G_E_CUDA      -1  /* a CUDA call failed */
#define KSW2G_E_ARG       -2  /* invalid argument */
#define KSW2G_E_BAND      -3  /* band or query too long for the kernels (no-alloc path, very long ll queries) */
#define KSW2G_E_NOMEM     -4  /* device or pinned allocation failed */
#define KSW2G_E_CAPACITY  -5  /* caller's output buffer too small */
#define KSW2G_E_UNSUPPORTED -6 /* e.g. GENERIC_SC with m > 16 */

typedef struct ksw2g_ctx ksw2g_ctx_t;
typedef struct ksw2g_batch ksw2g_batch_t;

/* One extension job.  qoff/toff index qbuf/tbuf (codes 0..m-1, one byte per
 * base); w, zdrop, end_bonus and flag mean what they mean for ksw_extz2_sse. */
typedef struct {
	int64_t qoff, toff;
	int32_t qlen, tlen;
	int32_t w, zdrop, end_bonus, flag;
} ksw2g_job_t;

/* Result of one extension job: the ksw_extz_t fields plus counters.
 * The CIGAR (n_cigar words, len<<4|op) is at cigar[cigar_off].
 * n_diag: anti-diagonals computed; cells: nominal band cells computed. */
typedef struct {
	int32_t score, max, max_q, max_t, mqe, mqe_t, mte, mte_q;
	int32_t zdropped, reach_end, n_cigar, n_diag;
	int64_t cigar_off;
	int64_t cells;
} ksw2g_ext_result_t;

/* One local-alignment (ksw_ll) job; xtra as for ksw_ll_u8_core. */
typedef struct {
	int64_t qoff, toff;
	int32_t qlen, tlen;
	int32_t xtra, pad;
} ksw2g_ll_job_t;

/* ksw_llrst_t plus the number of target rows processed. */
typedef struct {
	int32_t score, te, qe, score2, te2, rows;
} ksw2g_ll_result_t;

/* ---- context: one CUDA stream and its memory pools on one device ---- */
int ksw2g_ctx_create(int device, ksw2g_ctx_t **ctx);
void ksw2g_ctx_destroy(ksw2g_ctx_t *ctx);
void *ksw2g_ctx_stream(ksw2g_ctx_t *ctx);          /* the cudaStream_t all work of ctx runs on */
int ksw2g_ctx_sync(ksw2g_ctx_t *ctx);
/* Device bytes a batch may hold for traceback at once (jobs run in waves
 * under this budget, longest jobs first).  Default 16 GiB.  Batches of many
 * long pairs with CIGAR gain from more: 200k pairs of median 2 kb at w=500
 * (about 420 GB of rows) ran 11% faster with 48 GiB, in a third as many
 * waves.  The one-shot calls' chunk pipeline holds up to 2.5 times the
 * budget (three sub-contexts of half of it each). */
int ksw2g_ctx_set_tb_budget(ksw2g_ctx_t *ctx, int64_t bytes);
const char *ksw2g_last_error(void);

/* ---- one-shot batch: host buffers in, host results out ---- */
int ksw2g_ext_batch(ksw2g_ctx_t *ctx, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
					int n_jobs, const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
					const uint8_t *tbuf, int64_t tbuf_len,
					ksw2g_ext_result_t *res, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_used);

int ksw2g_ll_batch(ksw2g_ctx_t *ctx, int size, int m, const int8_t *mat, int gapo, int gape,
				   int n_jobs, const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
				   const uint8_t *tbuf, int64_t tbuf_len, ksw2g_ll_result_t *res);

/* ---- resident batch: upload once, run many times (async), fetch ---- */
int ksw2g_ext_prepare(ksw2g_ctx_t *ctx, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
					  int n_jobs, const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
					  const uint8_t *tbuf, int64_t tbuf_len, ksw2g_batch_t **batch);
int ksw2g_ll_prepare(ksw2g_ctx_t *ctx, int size, int m, const int8_t *mat, int gapo, int gape,
					 int n_jobs, const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
					 const uint8_t *tbuf, int64_t tbuf_len, ksw2g_batch_t **batch);
/* Enqueue DP (+ backtrack) of every job on the context stream; returns at once. */
int ksw2g_batch_run(ksw2g_ctx_t *ctx, ksw2g_batch_t *batch);
/* Wait for the batch and copy results (and for extension batches the CIGARs). */
int ksw2g_ext_fetch(ksw2g_ctx_t *ctx, ksw2g_batch_t *batch, ksw2g_ext_result_t *res, uint32_t *cigar,
					int64_t cigar_cap, int64_t *cigar_used);
int ksw2g_ll_fetch(ksw2g_ctx_t *ctx, ksw2g_batch_t *batch, ksw2g_ll_result_t *res);
/* Kernel launches the last run of this batch enqueued. */
int ksw2g_batch_launches(const ksw2g_batch_t *batch);
void ksw2g_batch_free(ksw2g_batch_t *batch);
/* Per-kernel timing of a batch's runs: with timing on, every kernel of a run is
 * bracketed by CUDA events on the launching stream.  ksw2g_batch_kernel_ms
 * waits for the runs and returns, for the DP kernels and the backtrack kernels
 * of all runs since timing was last switched on, the time covered by their
 * launches (launches on the two streams of a run may overlap; overlapping time
 * counts once) and the launch counts.  Off by default; not for batches captured
 * in a graph. */
int ksw2g_batch_set_timing(ksw2g_batch_t *batch, int on);
int ksw2g_batch_kernel_ms(ksw2g_batch_t *batch, double *dp_ms, double *bt_ms, int *n_dp, int *n_bt);

/* ---- a 2-bit reference resident on the device ----
 * minibwa's l2b layout (l2bit.h:18-32): base i of the concatenated contigs is
 * the 2-bit field at bits 2*(i%32) of pac[i/32]; contig k spans
 * [ctg_off[k], ctg_off[k]+ctg_len[k]); ambi holds n_ambi sorted, disjoint
 * [st, en) pairs (same coordinate) that read as N.  Extension and ksw_ll
 * batches can then name their targets as windows (contig tid[k], start
 * jobs[k].toff, length jobs[k].tlen) decoded on the device as l2b_getseq does
 * (l2bit.c:52-77), with per-job flags: */
#define KSW2G_REF_REVERSE 1  /* reversed in place (mb_seq_rev, align.c:643-644) */
#define KSW2G_REF_C2T     2  /* l2b_meth_convert(L2B_METH_C2T) (l2bit.c:79-90) */
#define KSW2G_REF_G2A     4  /* l2b_meth_convert(L2B_METH_G2A) */
typedef struct ksw2g_ref ksw2g_ref_t;
int ksw2g_ref_create(ksw2g_ctx_t *ctx, int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len,
					 const uint64_t *pac, int64_t n_pac, int64_t n_ambi, const uint64_t *ambi, ksw2g_ref_t **ref);
void ksw2g_ref_destroy(ksw2g_ref_t *ref);
/* One window decoded on the device into host bytes (windows must lie inside their contig). */
int ksw2g_ref_getseq(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, int64_t tid, int64_t st, int64_t len, int flags,
					 uint8_t *seq);
/* ksw2g_ext_batch / ksw2g_ext_prepare / ksw2g_ll_batch with reference targets:
 * only the queries travel from the host; tflags may be NULL. */
int ksw2g_ext_batch_ref(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, int dual, int8_t m, const int8_t *mat, int8_t q,
						int8_t e, int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs, const int32_t *tid,
						const int32_t *tflags, const uint8_t *qbuf, int64_t qbuf_len, ksw2g_ext_result_t *res,
						uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_used);
int ksw2g_ext_prepare_ref(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, int dual, int8_t m, const int8_t *mat, int8_t q,
						  int8_t e, int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs, const int32_t *tid,
						  const int32_t *tflags, const uint8_t *qbuf, int64_t qbuf_len, ksw2g_batch_t **batch);
int ksw2g_ll_batch_ref(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, int size, int m, const int8_t *mat, int gapo,
					   int gape, int n_jobs, const ksw2g_ll_job_t *jobs, const int32_t *tid, const int32_t *tflags,
					   const uint8_t *qbuf, int64_t qbuf_len, ksw2g_ll_result_t *res);

/* ---- align.c's pair alignment (mb_align_pair, align.c:329-390) over a batch ----
 * Every left extension, chain gap fill and right extension mb_align1 issues goes
 * through mb_align_pair: the ungapped shortcuts, the band shrink of short pairs,
 * the DP memory cap, then ksw_extz2_sse (q == q2 and e == e2) or ksw_extd2_sse.
 * ksw2g_align_pairs applies the shortcuts on the host and runs the pairs that need
 * DP as one batch; each result equals mb_align_pair's ksw_extz_t (n_diag and cells
 * are 0 for pairs settled without DP).  jobs[k].zdrop is mb_align_pair's zdrop
 * argument (scaled by a here, as there) and jobs[k].flag its ksw_flag; mat is
 * ksw_gen_nt4_mat's 5x5 matrix. */
typedef struct {
	int32_t a, b, b_ts, b_ambi, q, e, q2, e2;  /* mb_opt_t scores */
	int32_t meth, pad;                         /* opt->flag & MB_F_METH */
	int64_t max_sw_mat;                        /* opt->max_sw_mat (0: no cap) */
} ksw2g_align_opt_t;

int ksw2g_align_pairs(ksw2g_ctx_t *ctx, const ksw2g_align_opt_t *opt, const int8_t *mat, int n_jobs,
					  const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
					  int64_t tbuf_len, ksw2g_ext_result_t *res, uint32_t *cigar, int64_t cigar_cap,
					  int64_t *cigar_used);

/* ---- whole chains of mb_align1 (align.c:548-757), gap fills issued speculatively ----
 * For every hit (chain of anchors) the call derives the DP jobs mb_align1 runs: the left
 * extension, the gap fill between consecutive anchors (align.c:668-740) and the right
 * extension, with the anchor trimming of short-read mode (mb_max_stretch, align.c:522-546)
 * or long-read mode (mm_fix_bad_ends, mm_filter_bad_seeds(_alt), align.c:392-520).  Every
 * job of every chain goes to the device at once, the gap fills in their first, approximate
 * z-drop pass; the reference's z-drop test on their CIGARs (mm_test_zdrop, align.c:26-68,
 * with its inversion check on the device) selects the second, exact pass; then each chain is
 * assembled in order as mb_align1 does: the first gap fill that z-drops ends the chain and
 * cancels the jobs behind it (align.c:698-720), splitting the hit when the anchors behind
 * carry enough matches.  Results are mb_align1's, up to the call of mb_update_extra
 * (align.c:753), which stays with the caller. */
typedef struct {          /* mb_anchor_t (mbpriv.h:26-32) */
	int32_t sid;          /* tid << 1 | rev */
	int32_t len;          /* anchor length */
	int32_t qpos;         /* query coordinate of the anchor's last base */
	uint32_t flag;        /* MB_SEED_LONG_JOIN 0x1, MB_SEED_IGNORE 0x2 */
	int64_t tpos;         /* contig coordinate of the anchor's last base */
} ksw2g_anchor_t;
typedef struct {          /* one hit: the fields of mb_hit_t that mb_align1 reads */
	int64_t as;           /* anchors[as .. as+cnt) of the anchor array */
	int64_t qoff;         /* the read in qbuf, in the orientation aligned (seq[rev]) */
	int32_t cnt;
	int32_t mlen, score;  /* r->mlen, r->score */
	int32_t qlen;
	int32_t meth;         /* the read's methylation mode as mb_align1 receives it (flipped for rev strands) */
	int32_t split_inv;    /* r->split_inv */
	int32_t opt;          /* index of the hit's option set (mb_opt_adap varies them with the read length) */
	int32_t pad;
} ksw2g_chain_t;
typedef struct {          /* the mb_opt_t fields mb_align1 reads */
	int32_t a, b, b_ts, b_ambi, q, e, q2, e2;
	int32_t bw, bw_long, max_gap, end_bonus, zdrop, zdrop_inv;
	int32_t min_ksw_len, min_len, min_chain_score, min_dp_max;
	int32_t long_reads;   /* MB_F_LONG */
	int32_t adaptive;     /* MB_F_ADAP: reads longer than max_sr_len align as long reads */
	int32_t max_sr_len;
	int32_t meth;         /* MB_F_METH */
	int64_t max_sw_mat;
} ksw2g_chain_opt_t;
typedef struct {
	int64_t ts, te;       /* r->ts, r->te */
	int32_t qs, qe;       /* r->qs, r->qe (on the read's forward strand, as mb_align1 sets them) */
	int32_t dp_score;     /* r->p->dp_score */
	int32_t n_cigar;      /* r->p->n_cigar; the CIGAR is at cigar + cigar_off */
	int64_t cigar_off;
	int32_t cnt, score;   /* r->cnt, r->score after a split */
	int32_t split_n;      /* > 0: the hit was split by mb_split_hit(r, r2, split_n, ...) */
	int32_t split_inv2;   /* r2->split_inv of that split */
	int32_t n_dp;         /* DP jobs whose results the chain used */
	int32_t n_dp_issued;  /* DP jobs issued for it (the speculative ones included) */
} ksw2g_chain_result_t;
/* opts: n_opts option sets that agree in their scores (a, b, b_ts, b_ambi, q, e, q2, e2, meth,
 * max_sw_mat).  As mb_align1 does, the call sets MB_SEED_IGNORE / MB_SEED_LONG_JOIN in the
 * flags of the anchors of long-read hits; a hit split off by a z-drop is aligned by a later
 * call over the anchors so flagged.  CIGARs go to cigar[cigar_off ..] in hit order. */
int ksw2g_align_chains(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, int n_opts, const ksw2g_chain_opt_t *opts,
					   int n_chains, const ksw2g_chain_t *chains, ksw2g_anchor_t *anchors, int64_t n_anchors,
					   const uint8_t *qbuf, int64_t qbuf_len, ksw2g_chain_result_t *res, uint32_t *cigar,
					   int64_t cigar_cap, int64_t *cigar_used);
/* The context's last ksw2g_align_chains call: host wall time of its stages in ms[6] (deriving
 * the jobs, gathering the windows, the first pass, the z-drop tests with the inversion checks,
 * the second pass, assembly) and counts[4] (hits, first-pass jobs, second-pass jobs, inversion
 * checks). */
int ksw2g_align_chains_last_stats(const ksw2g_ctx_t *ctx, double *ms, int64_t *counts);

/* ---- mate rescue over the resident reference (pe.c:209-372) ----
 * One candidate is one (read, window) pair of mb_matesw_core: the window
 * [ts, te) on contig tid computed from the insert-size statistics and clamped
 * to the contig (pe.c:336-339), the read in the orientation aligned
 * (seq[is_rev]), the window's methylation mode (l2b_meth_rev applied when
 * is_rev: 0 none, 1 C2T, 2 G2A) and min_sc already divided by a.  Per
 * candidate the call runs mb_ungap (7-mer Hough votes along diagonals), the
 * narrowing and thresholds of pe.c:347-353, ksw_ll with the matrix scaled by a
 * (u8 or i16 by pe.c:263's rule) and, when ksw_ll's score passes, ksw_extz2 on
 * the reversed prefixes ending at ksw_ll's end (pe.c:283-290).  The windows are
 * decoded on the device; only the reads travel from the host. */
typedef struct {
	int32_t a, b, b_ts, b_ambi, q, e;      /* mb_opt_t scores, unscaled */
	int32_t bw, zdrop, end_bonus, min_len, min_dp_max;
} ksw2g_rescue_opt_t;

typedef struct {
	int64_t qoff;                        /* read in qbuf */
	int64_t ts, te;                      /* candidate window on contig tid */
	int32_t qlen, tid, meth, min_sc, rev, pad;
} ksw2g_rescue_job_t;

typedef struct {
	int32_t max_ug, max_i, n_good, n_kmer; /* mb_ungap's return value and outputs */
	int64_t ts2, te2;                      /* the window ksw_ll ran on */
	int32_t ll_done, ll_score, ll_te, ll_qe, ll_score2, ll_te2;
	int32_t ext_done, rescued;             /* extz2 ran; the hit passed pe.c:291 */
	int32_t qs, qe, dp_max2, pad;          /* hit on the read, flipped when rev (pe.c:364-368) */
	int64_t ts, te;                        /* hit on the contig */
	ksw2g_ext_result_t ext;                /* extz2 result; CIGAR at cigar[ext.cigar_off] */
} ksw2g_rescue_result_t;

int ksw2g_rescue_batch(ksw2g_ctx_t *ctx, const ksw2g_ref_t *ref, const ksw2g_rescue_opt_t *opt, int n_jobs,
					   const ksw2g_rescue_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
					   ksw2g_rescue_result_t *res, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_used);
/* The last rescue call of ctx: kernels launched, and the wall time (ms) of its three
 * stages (window gather + prefilter, ksw_ll, extz2), each including its copies. */
int ksw2g_rescue_last_stats(const ksw2g_ctx_t *ctx, int *launches, double *ms3);
/* Its ksw_ll and extz2 (DP and backtrack) kernels' device time in ms[0], ms[1], from CUDA events
 * around the launches; the rest of a stage's wall time is host work and copies. */
int ksw2g_rescue_last_device_ms(const ksw2g_ctx_t *ctx, double *ms2);

/* ---- CUDA graphs: one launch runs several prepared batches concurrently ----
 * Captures the kernels of n prepared batches (extension or ll) into one CUDA
 * graph.  Each batch is a branch of the graph, so the batches run
 * concurrently; each extension batch gets its own traceback region, sized for
 * its largest wave.  ksw2g_graph_launch enqueues the whole graph on ctx's
 * stream; the results are read with ksw2g_ext_fetch / ksw2g_ll_fetch, as after
 * ksw2g_batch_run.  The batches must stay alive, and must not be prepared
 * again, while the graph exists. */
typedef struct ksw2g_graph ksw2g_graph_t;
int ksw2g_graph_create(ksw2g_ctx_t *ctx, int n_batches, ksw2g_batch_t *const *batches, ksw2g_graph_t **graph);
int ksw2g_graph_launch(ksw2g_ctx_t *ctx, ksw2g_graph_t *graph);
int ksw2g_graph_launches(const ksw2g_graph_t *graph);  /* kernel launches in one graph launch */
void ksw2g_graph_destroy(ksw2g_graph_t *graph);

/* Select the thread-group shape used for extension jobs whose reference
 * n_col_ (16-byte blocks per anti-diagonal) lies in [ncol_lo, ncol_hi]:
 * shape s < ksw2g_ext_num_shapes() runs the DP on four byte lanes per 32-bit
 * register, shape ksw2g_ext_num_shapes() + s the same thread-group shape on two
 * 16-bit lanes with DPX min/max instructions (used where the scoring allows
 * it: gap costs non-negative, q+e and q2+e2 at most 128).  Both are bit-exact
 * with the reference.  Used by the autotuner. */
int ksw2g_ext_num_shapes(void);
int ksw2g_ext_shape_info(int shape, int *group_threads, int *words_per_thread);
int ksw2g_ext_set_shape(int dual, int mode, int ncol_lo, int ncol_hi, int shape);
/* Force the lane width of extension batches prepared after the call: 0 bytes,
 * 1 16-bit halves (where the scoring allows it), -1 (default) whatever the
 * shape preferences select.  Process-wide.  Returns 0 or KSW2G_E_ARG. */
int ksw2g_ext_set_family(int family);
int ksw2g_ext_get_family(void);
/* Use of the block-split kernel for extension batches prepared after the call: -1 (default)
 * the batch decides (a block per pair for the jobs of a band class that are few and wide),
 * 0 never, 1 for every job whose band a block holds.  Process-wide; the environment variable
 * KSW2G_SPLIT (-1, 0 or 1) sets the value a process starts with.  Returns 0 or KSW2G_E_ARG. */
int ksw2g_ext_set_split(int mode);
int ksw2g_ext_get_split(void);

/*
 * Extension batch that allocates nothing (no counterpart in the reference).
 *
 * For callers that cannot let a library call cudaMalloc: a framework that owns
 * all device memory through its own caching allocator, or a serving loop that
 * cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  It runs
 * the same DP and backtrack kernels as ksw2g_ext_batch; all scratch (job table
 * copy, traceback offsets and rows, work counters) lives in one fixed static
 * device array of KSW2G_NOALLOC_SCRATCH_BYTES that every GPU loading this part
 * of the library keeps until the process exits.
 *
 *  jobs     host array; qoff/toff index d_arena, which must use the padded
 *           layout: every sequence starts 16-byte aligned with at least 32 zero
 *           bytes before it and zeros after it up to the next 16-byte boundary
 *           plus 32 bytes.  All jobs of one call use the same gap mode
 *           (score-only, left-aligned or right-aligned CIGAR).  The host copies
 *           the array on the stream, so it must stay unchanged until the stream
 *           has passed the call.  Under stream capture the copy is recorded with
 *           the pointer and every replay reads the array again, without the
 *           checks of the captured call: it must then hold the same jobs for as
 *           long as the graph is replayed.
 *  arena_len bytes of d_arena; a job whose sequence plus its padding ends past
 *           it is rejected (KSW2G_E_ARG) before any device work.
 *  d_res    device array of n_jobs results (as ksw2g_ext_batch fills them).
 *  d_cigar  device array of cigar_cap words; cigar_cap must be at least the sum
 *           of qlen+tlen+1 over the jobs when CIGARs are requested.
 *  stream   cudaStream_t the work is enqueued on; the call returns before it ends.
 *
 * Rejects (KSW2G_E_CAPACITY, message in ksw2g_last_error()) any call whose
 * scratch (traceback rows, plus 64 bytes per job and at most 1 KiB) exceeds
 * KSW2G_NOALLOC_SCRATCH_BYTES, and (KSW2G_E_BAND) bands wider than 512 blocks of
 * 16 cells; bands wider than 64 blocks run one pair per block.  The first call on each device looks up the
 * array's device address; make that first call before any stream capture.
 * The address is kept for the life of the process, so calls after a
 * cudaDeviceReset of that device are not supported.
 * Every call reuses the same array and clears its counters at the start:
 * calls whose work overlaps on the GPU (different streams, or another host
 * thread) race on it and must be serialised by the caller.
 */
#define KSW2G_NOALLOC_SCRATCH_BYTES (64ll << 20)
int ksw2g_ext_noalloc(int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
					  int n_jobs, const ksw2g_job_t *jobs, const uint8_t *d_arena, int64_t arena_len,
					  ksw2g_ext_result_t *d_res, uint32_t *d_cigar, int64_t cigar_cap, void *stream);

/* ---- serving engine: continuous batching over a fixed traceback budget ----
 * Requests are admitted in arrival order as soon as one of n_slots slots is
 * free and the request's traceback rows (the reference's footprint,
 * ksw2_extz2_sse.c:84, summed over its jobs) fit in the tb_budget bytes of
 * device memory the engine owns; queued requests of the same kind and
 * scoring scheme join the admitted request's launch.  Admitted requests run
 * concurrently on the slots' streams.  The caller's buffers (jobs, sequences, results, CIGAR) must
 * stay valid until ksw2g_server_wait returns for that request. */
typedef struct ksw2g_server ksw2g_server_t;
int ksw2g_server_create(int device, int n_slots, int64_t tb_budget, ksw2g_server_t **server);
void ksw2g_server_destroy(ksw2g_server_t *server);          /* drains queued requests first */
/* Returns a request id (> 0) or a negative error code. */
int64_t ksw2g_server_submit_ext(ksw2g_server_t *server, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
								int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs, const uint8_t *qbuf,
								int64_t qbuf_len, const uint8_t *tbuf, int64_t tbuf_len, ksw2g_ext_result_t *res,
								uint32_t *cigar, int64_t cigar_cap);
int64_t ksw2g_server_submit_ll(ksw2g_server_t *server, int size, int m, const int8_t *mat, int gapo, int gape,
							   int n_jobs, const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
							   const uint8_t *tbuf, int64_t tbuf_len, ksw2g_ll_result_t *res);
/* Blocks until the request is done; returns its status (0 or an error code) and
 * its latency (submit to results in the caller's buffers) and queueing time. */
int ksw2g_server_wait(ksw2g_server_t *server, int64_t id, double *latency_ms, double *queue_ms, int64_t *cigar_used);
int ksw2g_server_stats(ksw2g_server_t *server, int64_t *admitted, int64_t *done, int64_t *peak_inflight,
					   int64_t *peak_pool_bytes);
/* Launches issued and the most requests merged into one launch.  Queued
 * requests of the head request's kind and scoring scheme are merged into its
 * launch while they fit the pool and the merge limit. */
int ksw2g_server_launch_stats(ksw2g_server_t *server, int64_t *launches, int64_t *max_merged);
/* Most jobs one merged launch may hold (default 8,192; 1 turns merging off).
 * Smaller launches finish sooner, larger ones fill the GPU: a latency /
 * throughput knob. */
int ksw2g_server_set_merge(ksw2g_server_t *server, int max_jobs);

/* Failure injection for host-side tests (no counterpart in the reference): the nth device
 * buffer growth after this call fails as if the device had no memory left, so the call that
 * needed it returns KSW2G_E_NOMEM; 0 turns the injection off.  Nothing runs on the GPU for it. */
void ksw2g_debug_fail_device_alloc(int nth);

/* Measured 32-bit integer instruction throughput of the device (lane-ops per
 * second), the denominator of the DP kernels' integer-pipe roofline. */
int ksw2g_probe_int32_peak(int device, double *ops_per_s);

#ifdef __cplusplus
}
#endif
#endif
