/* mbg_map.c -- minibwa's per-read mapping (map-algo.c:578-664) with the alignment of all reads
 * of a mini-batch on the GPU.
 *
 * mb_map_sai is cut in three:
 *   1. mbg_map_sai_defer, on the worker thread that seeded the read: anchors, chaining,
 *      re-chaining, hit generation and the first mb_set_parent / mb_select_sub
 *      (map-algo.c:594-637).  What the read keeps for later is allocated with libc, because
 *      the worker's kalloc pool is reset when the worker returns (map-main.c:93).
 *   2. mbg_step_end, once per mini-batch: mb_squeeze_a and the query in both orientations as
 *      mb_align_skeleton prepares them (align.c:900-907), then mb_align1 of every hit of every
 *      read through ksw2g_align_chains, one call per round: the first round aligns the hits
 *      mb_gen_hit made, each later round the hits the previous one split off at a z-drop, which
 *      mb_align_skeleton inserts after their parent and reaches next (align.c:911-912).
 *   3. per read on kt_for workers: mb_update_extra of every aligned hit (align.c:750-755) and
 *      the tests mb_align1_inv makes on each split hit and its predecessor (align.c:765-776);
 *      the ksw_ll and mb_align_pair of the pairs that pass, for all reads in two device
 *      batches (align.c:779-792); then per read again the INV hits inserted where
 *      mb_align_skeleton inserts them (align.c:913-918), the rest of mb_align_skeleton
 *      (align.c:921-927) and of mb_map_sai (map-algo.c:640-657).
 * The hits each step leaves are those the stock code leaves, so the SAM output is the same.
 * mb_map_sai's debug prints (kom_dbg_flag) are not emitted on this path. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <pthread.h>

#include "kalloc.h"
#include "kthread.h"
#include "ksw2.h"
#include "ksw2_gb300.h"
#include "mbg.h"

void mb_update_dp_max(int qlen, int n_regs, mb_hit_t *regs, double frac, int a, int b);  // align.c:867
int32_t mb_cal_high_cov(void *km, int32_t n, const mb_sai_t *sai, int32_t max_occ);     // map-algo.c:175

typedef struct {
	int32_t state;        // 0: no read, 1: hits final, 2: alignment deferred
	int32_t qlen, is_sr, hi_cov, sub_diff, n_a, n_hit;
	l2b_meth_t mt;
	uint32_t hash;
	double seed_ratio;
	mb_opt_t opt;         // the read's options (mb_opt_adap)
	const char *qname;
	uint8_t *seq;         // nt4 codes
	uint8_t *qseq0;       // forward, then reverse complement
	mb_anchor_t *a;
	mb_hit_t *hit;
	uint8_t *aligned;     // per hit: mb_align1 left r->p
	int64_t a_base, q_base;
	int32_t n_inv;
	struct mbg_inv_s *inv; // inversion checks between a split hit and its predecessor
} mbg_read_t;

// One pair (regs[i-1], regs[i]) that passes mb_align1_inv's tests before its ksw_ll
// (align.c:766-776), with the sequences that ksw_ll and mb_align_pair take
typedef struct mbg_inv_s {
	const mb_opt_t *opt;    // the read's options
	int32_t i, ql, tl, mt;  // mt: the matrix's methylation mode (align.c:777)
	uint8_t *q, *t;         // the query and target between the two hits, forward
	int32_t score, q_off, t_off;
	ksw2g_ext_result_t ez;
	uint32_t *cigar;
} mbg_inv_t;

static mbg_read_t *g_rd;
static int64_t g_n_rd;
static ksw2g_ctx_t *g_ctx;
static ksw2g_ref_t *g_ref;
static const l2b_t *g_l2b;
static int g_n_thread = 1;
static double g_t_begin;
static int g_timing = -1;  // MBG_TIMING set: stage times of every mini-batch on stderr

static double mbg_ms(void)
{
	struct timeval tv;
	gettimeofday(&tv, 0);
	return tv.tv_sec * 1e3 + tv.tv_usec * 1e-3;
}

static void mbg_fail(const char *what)
{
	fprintf(stderr, "[E::%s] %s: %s\n", __func__, what, ksw2g_last_error());
	exit(1);
}

static void mbg_gpu_init(const mb_idx_t *idx);
static pthread_t g_init_tid;
static int g_init_running;

// Bringing up the CUDA context takes about 0.1 s.  A map run starts it when the program starts,
// on a thread of its own, so that it overlaps the loading of the index and of the first reads;
// mbg_gpu_init waits for it and reports its failure.
static pthread_t g_ctx_tid;
static int g_ctx_running, g_ctx_rc;
static char g_ctx_err[512];
static double g_t_start, g_t_ctx;  // program start; the context's creation time

static void *mbg_ctx_thread(void *unused)
{
	const char *dev = getenv("MBG_DEVICE");
	double t0 = mbg_ms();
	(void)unused;
	if ((g_ctx_rc = ksw2g_ctx_create(dev? atoi(dev) : 0, &g_ctx)) != 0)
		snprintf(g_ctx_err, sizeof(g_ctx_err), "%s", ksw2g_last_error());
	g_t_ctx = mbg_ms() - t0;
	return 0;
}

__attribute__((constructor)) static void mbg_ctx_early(int argc, char **argv)
{ // glibc passes the program's arguments to constructors
	g_t_start = mbg_ms();
	if (argc > 1 && argv && argv[1] && strcmp(argv[1], "map") == 0)
		g_ctx_running = pthread_create(&g_ctx_tid, 0, mbg_ctx_thread, 0) == 0;
}

static void mbg_exit_timing(void)
{ // registered after the CUDA runtime's own exit handler, so it runs before the runtime's teardown
	fprintf(stderr, "[M::mbg] exit begins %.1f ms after the program started\n", mbg_ms() - g_t_start);
}

static void *mbg_gpu_init_thread(void *idx)
{
	mbg_gpu_init((const mb_idx_t*)idx);
	return 0;
}

void mbg_step_begin(const mb_idx_t *idx, int64_t n_seq)
{
	g_rd = (mbg_read_t*)calloc(n_seq > 0? n_seq : 1, sizeof(mbg_read_t));
	g_n_rd = n_seq;
	if (g_timing < 0) g_timing = getenv("MBG_TIMING") != 0;
	g_t_begin = mbg_ms();
	if (!g_ctx && !g_init_running) // the CUDA context and the reference upload overlap the seeding
		g_init_running = pthread_create(&g_init_tid, 0, mbg_gpu_init_thread, (void*)idx) == 0;
}

void mbg_map_sai_defer(const mb_opt_t *opt, const mb_idx_t *idx, int64_t qlen, const char *seq0, l2b_meth_t mt,
                       mb_sai_v *u, int64_t rid, mb_tbuf_t *b, const char *qname)
{
	const int32_t min_rechain_len = 1000;
	const double min_rechain_ratio = 0.1;
	mbg_read_t *r = &g_rd[rid];
	void *km = mb_tbuf_km(b);
	int32_t i, n_hit;
	uint64_t *w;
	double chn_pen_gap;
	mb_anchor_v v = {0,0,0};
	mb_anchor_t *a;

	r->qlen = (int32_t)qlen, r->mt = mt, r->opt = *opt, r->qname = qname;
	if (opt->flag & MB_F_NO_ALN) { // nothing is aligned: the stock function as it stands
		r->hit = mb_map_sai(opt, idx, qlen, seq0, mt, u, &r->n_hit, b, qname);
		r->state = 1;
		return;
	}
	if (u->n == 0) {
		kfree(km, u->a);
		r->hit = 0, r->n_hit = 0, r->state = 1;
		return;
	}
	r->hash  = qname? mb_hash_str(qname) : 0;
	r->hash ^= mb_hash64(qlen) + mb_hash64(opt->seed);
	r->hash  = mb_hash64(r->hash);
	r->seq = (uint8_t*)malloc(qlen > 0? qlen : 1);
	for (i = 0; i < qlen; ++i) r->seq[i] = kom_nt4_table[(uint8_t)seq0[i]];
	r->hi_cov = mb_cal_high_cov(km, u->n, u->a, opt->max_occ);
	r->is_sr = mb_is_sr_mode(opt, qlen);
	r->sub_diff = opt->a + opt->b > opt->q + opt->e? opt->a + opt->b : opt->q + opt->e;

	chn_pen_gap = opt->chain_gap_scale * .01 * opt->min_len;
	r->seed_ratio = mb_anchor(0, idx, u, opt->min_len, qlen, r->seq, mt, opt->max_occ, &v);
	kfree(km, u->a);
	u->n = 0, u->a = 0;
	a = mb_lchain_dp(0, idx->l2b, opt->max_gap, opt->max_gap, opt->bw, opt->max_chain_skip, opt->max_chain_iter,
					 opt->min_chain_score, chn_pen_gap, v.n, v.a, &n_hit, &w);
	if (opt->bw_long > opt->bw * 2 && !r->is_sr && n_hit > 0) { // re-chaining around the best chain
		int64_t n_a, as, st, en;
		int32_t best;
		for (i = 1, best = 0; i < n_hit; ++i)
			if ((w[i] >> 32) > (w[best] >> 32)) best = i;
		for (i = 0, as = 0; i < best; ++i) as += (int32_t)w[i];
		st = a[as].qpos + 1 - a[as].len;
		en = a[as + (int32_t)w[best] - 1].qpos + 1;
		if (qlen - (en - st) > min_rechain_len && en - st > qlen * min_rechain_ratio) {
			for (i = 0, n_a = 0; i < n_hit; ++i) n_a += (int32_t)w[i];
			kfree(0, w);
			mb_anchor_sort(idx->l2b, n_a, a);
			a = mb_lchain_dp(0, idx->l2b, opt->max_gap, opt->max_gap, opt->bw_long, opt->max_chain_skip,
							 opt->max_chain_iter, opt->min_chain_score, chn_pen_gap, n_a, a, &n_hit, &w);
		}
	}
	r->hit = mb_gen_hit(km, r->hash, qlen, idx->l2b, n_hit, w, a);
	kfree(0, w);
	mb_set_parent(km, opt->mask_level, opt->mask_len, n_hit, r->hit, r->sub_diff, 0);
	mb_select_sub(km, opt->pri_ratio, opt->min_len * 2, opt->best_n, &n_hit, r->hit);
	r->a = a, r->n_hit = n_hit, r->state = 2;
}

// ---- stage 2: the GPU rounds

static void mbg_gpu_init(const mb_idx_t *idx)
{
	const l2b_t *l = idx->l2b;
	uint64_t *off, *len, k;
	const char *dev = getenv("MBG_DEVICE");
	if (g_ctx_running) pthread_join(g_ctx_tid, 0), g_ctx_running = 0;
	if (g_ctx_rc) {
		fprintf(stderr, "[E::%s] ksw2g_ctx_create: %s\n", __func__, g_ctx_err);
		exit(1);
	}
	if (g_ctx && g_l2b == l) return;
	if (!g_ctx && ksw2g_ctx_create(dev? atoi(dev) : 0, &g_ctx)) mbg_fail("ksw2g_ctx_create");
	if (g_ref) ksw2g_ref_destroy(g_ref);
	off = (uint64_t*)malloc(l->n_ctg * 8 + 8), len = (uint64_t*)malloc(l->n_ctg * 8 + 8);
	for (k = 0; k < l->n_ctg; ++k) off[k] = l->ctg[k].off, len[k] = l->ctg[k].len;
	if (ksw2g_ref_create(g_ctx, l->n_ctg, off, len, l->pac, l->n_pac, l->n_ambi, (const uint64_t*)l->ambi, &g_ref))
		mbg_fail("ksw2g_ref_create");
	free(off), free(len);
	if (!g_l2b && getenv("MBG_TIMING")) {
		fprintf(stderr, "[M::mbg] CUDA context created in %.1f ms; reference resident %.1f ms after the program started\n",
				g_t_ctx, mbg_ms() - g_t_start);
		atexit(mbg_exit_timing);
	}
	g_l2b = l;
}

ksw2g_ctx_t *mbg_ctx(const mb_idx_t *idx)
{ // the process's context and resident reference, for mbg_pe.c
	if (g_init_running) pthread_join(g_init_tid, 0), g_init_running = 0;
	mbg_gpu_init(idx);
	return g_ctx;
}

ksw2g_ref_t *mbg_ref(void) { return g_ref; }

static void mbg_chain_opt(const mb_opt_t *o, ksw2g_chain_opt_t *c)
{
	memset(c, 0, sizeof(*c));
	c->a = o->a, c->b = o->b, c->b_ts = o->b_ts, c->b_ambi = o->b_ambi;
	c->q = o->q, c->e = o->e, c->q2 = o->q2, c->e2 = o->e2;
	c->bw = o->bw, c->bw_long = o->bw_long, c->max_gap = o->max_gap, c->end_bonus = o->end_bonus;
	c->zdrop = o->zdrop, c->zdrop_inv = o->zdrop_inv, c->min_ksw_len = o->min_ksw_len, c->min_len = o->min_len;
	c->min_chain_score = o->min_chain_score, c->min_dp_max = o->min_dp_max;
	c->long_reads = !!(o->flag & MB_F_LONG), c->adaptive = !!(o->flag & MB_F_ADAP);
	c->max_sr_len = o->max_sr_len, c->meth = !!(o->flag & MB_F_METH), c->max_sw_mat = o->max_sw_mat;
}

typedef struct { int64_t rid; int32_t hi, opt; } mbg_work_t;

typedef struct {
	const mb_opt_t *opt;
	const mb_idx_t *idx;
	mb_tbuf_t **tbuf;
} mbg_shared_t;

static void mbg_prepare_worker(void *data, long rid, int tid)
{ // mb_align_skeleton's query in both orientations and mb_squeeze_a (align.c:900-909)
	mbg_read_t *r = &g_rd[rid];
	int32_t i, ql = r->qlen;
	(void)data, (void)tid;
	if (r->state != 2) return;
	r->qseq0 = (uint8_t*)malloc(ql * 2 + 1);
	for (i = 0; i < ql; ++i)
		r->qseq0[i] = r->seq[i], r->qseq0[ql + ql - 1 - i] = r->seq[i] < 4? 3 - r->seq[i] : 4;
	r->n_a = mb_squeeze_a(0, r->n_hit, r->hit, r->a);
	r->aligned = (uint8_t*)calloc(r->n_hit + 1, 1);
}

typedef struct { int64_t k0, k1; int32_t n_next, *next_hi; } mbg_group_t;  // one read's work items
typedef struct {
	const mbg_work_t *work;
	const ksw2g_chain_result_t *res;
	const uint32_t *cig;
	mbg_group_t *grp;
} mbg_apply_t;

static void mbg_apply_worker(void *data, long gi, int tid)
{ // one read's results; a split-off hit goes right after its parent, as mb_insert_reg puts it
	mbg_apply_t *ap = (mbg_apply_t*)data;
	mbg_group_t *g = &ap->grp[gi];
	const mbg_work_t *work = ap->work;
	mbg_read_t *r = &g_rd[work[g->k0].rid];
	int64_t n_split = 0, j, o, k;
	mb_hit_t *nh;
	uint8_t *na;
	(void)tid;
	for (k = g->k0; k < g->k1; ++k) n_split += ap->res[k].split_n > 0;
	nh = (mb_hit_t*)malloc((r->n_hit + n_split) * sizeof(mb_hit_t));
	na = (uint8_t*)calloc(r->n_hit + n_split + 1, 1);
	g->next_hi = (int32_t*)malloc((n_split + 1) * sizeof(int32_t));
	for (j = 0, o = 0, k = g->k0; j < r->n_hit; ++j) {
		mb_hit_t r2, *h;
		const ksw2g_chain_result_t *R;
		nh[o] = r->hit[j], na[o] = r->aligned[j];
		if (k == g->k1 || work[k].hi != j) { ++o; continue; } // not aligned in this round
		h = &nh[o], R = &ap->res[k++];
		r2.cnt = 0;
		if (h->cnt == 0) { ++o; continue; } // mb_align1 returns at once (align.c:560)
		if (R->split_n > 0) { // align.c:716-719
			mb_split_hit(h, &r2, R->split_n, r->qlen, r->a, g_l2b);
			if (R->split_inv2) r2.split_inv = 1;
		}
		if (h->cnt != R->cnt || h->score != R->score) {
			fprintf(stderr, "[E::%s] split of hit %ld of read %s disagrees\n", __func__, (long)j, r->qname? r->qname : "*");
			exit(1);
		}
		if (R->n_cigar > 0) {
			mb_append_cigar(h, R->n_cigar, ap->cig + R->cigar_off);
		} else { // as align.c:700-705 allocates it
			uint32_t c = sizeof(mb_extra_t) / 4;
			kom_roundup32(c);
			h->p = (mb_extra_t*)calloc(c, 4);
			h->p->cap = c;
		}
		h->p->dp_score = R->dp_score;
		h->ts = R->ts, h->te = R->te, h->qs = R->qs, h->qe = R->qe;
		na[o++] = 1;
		if (r2.cnt > 0) nh[o] = r2, na[o] = 0, g->next_hi[g->n_next++] = (int32_t)o++;
	}
	free(r->hit), free(r->aligned);
	r->hit = nh, r->aligned = na, r->n_hit = (int32_t)o;
}

static void mbg_align_rounds(const mb_idx_t *idx)
{
	int64_t i, k, n_work = 0, m_work = 0, n_anc = 0, n_q = 0;
	int32_t n_opts = 0, m_opts = 16;
	mbg_work_t *work = 0;
	ksw2g_chain_opt_t *opts = (ksw2g_chain_opt_t*)malloc(m_opts * sizeof(ksw2g_chain_opt_t));
	ksw2g_anchor_t *anc;
	uint8_t *qbuf;
	int32_t *read_opt = (int32_t*)calloc(g_n_rd + 1, sizeof(int32_t));

	// one anchor array, one query buffer and the distinct option sets of the mini-batch
	for (i = 0; i < g_n_rd; ++i) {
		mbg_read_t *r = &g_rd[i];
		ksw2g_chain_opt_t c;
		if (r->state != 2) continue;
		r->a_base = n_anc, n_anc += r->n_a;
		r->q_base = n_q, n_q += 2 * (int64_t)r->qlen;
		mbg_chain_opt(&r->opt, &c);
		for (k = 0; k < n_opts; ++k)
			if (memcmp(&opts[k], &c, sizeof(c)) == 0) break;
		if (k == n_opts) {
			if (n_opts == m_opts) opts = (ksw2g_chain_opt_t*)realloc(opts, (m_opts <<= 1) * sizeof(ksw2g_chain_opt_t));
			opts[n_opts++] = c;
		}
		read_opt[i] = (int32_t)k;
		for (k = 0; k < r->n_hit; ++k) {
			if (n_work == m_work) work = (mbg_work_t*)realloc(work, (m_work = m_work? m_work << 1 : 1024) * sizeof(mbg_work_t));
			work[n_work].rid = i, work[n_work].hi = (int32_t)k, work[n_work++].opt = read_opt[i];
		}
	}
	anc = (ksw2g_anchor_t*)malloc((n_anc + 1) * sizeof(ksw2g_anchor_t));
	qbuf = (uint8_t*)malloc(n_q + 1);
	for (i = 0; i < g_n_rd; ++i) {
		mbg_read_t *r = &g_rd[i];
		if (r->state != 2) continue;
		for (k = 0; k < r->n_a; ++k) {
			ksw2g_anchor_t *d = &anc[r->a_base + k];
			const mb_anchor_t *s = &r->a[k];
			d->sid = s->sid, d->len = s->len, d->qpos = s->qpos, d->flag = s->flag, d->tpos = s->tpos;
		}
		memcpy(qbuf + r->q_base, r->qseq0, 2 * (size_t)r->qlen);
	}

	while (n_work > 0) {
		ksw2g_chain_t *ch = (ksw2g_chain_t*)calloc(n_work, sizeof(ksw2g_chain_t));
		ksw2g_chain_result_t *res = (ksw2g_chain_result_t*)calloc(n_work, sizeof(ksw2g_chain_result_t));
		int64_t cap = 64, used = 0, n_next = 0;
		uint32_t *cig;
		mbg_work_t *next = 0;
		int rc;
		for (k = 0; k < n_work; ++k) {
			const mbg_read_t *r = &g_rd[work[k].rid];
			const mb_hit_t *h = &r->hit[work[k].hi];
			ch[k].as = r->a_base + h->as, ch[k].cnt = h->cnt, ch[k].mlen = h->mlen, ch[k].score = h->score;
			ch[k].qoff = r->q_base + (h->cnt > 0 && (r->a[h->as].sid & 1)? r->qlen : 0), ch[k].qlen = r->qlen;
			ch[k].meth = (int32_t)r->mt, ch[k].split_inv = h->split_inv, ch[k].opt = work[k].opt;
			cap += 3 * (int64_t)r->qlen + 4 * (int64_t)h->cnt;
		}
		double t_call = mbg_ms();
		for (;;) { // the CIGAR bound is a guess: long deletions can exceed it
			cig = (uint32_t*)malloc(cap * sizeof(uint32_t));
			rc = ksw2g_align_chains(g_ctx, g_ref, n_opts, opts, (int)n_work, ch, anc, n_anc, qbuf, n_q, res, cig, cap, &used);
			if (rc != KSW2G_E_CAPACITY) break;
			free(cig);
			cap <<= 1;
		}
		if (rc) mbg_fail("ksw2g_align_chains");
		if (g_timing) {
			double ms[6];
			int64_t cnt[4];
			ksw2g_align_chains_last_stats(g_ctx, ms, cnt);
			fprintf(stderr, "[M::mbg] round: %ld hits, %ld+%ld DP jobs, %ld inversion checks; %.1f ms "
					"(derive %.1f, windows %.1f, pass 1 %.1f, z-drop %.1f, pass 2 %.1f, assemble %.1f)\n",
					(long)cnt[0], (long)cnt[1], (long)cnt[2], (long)cnt[3], mbg_ms() - t_call,
					ms[0], ms[1], ms[2], ms[3], ms[4], ms[5]);
		}
		{ // apply the results read by read on the kt_for workers
			mbg_apply_t ap;
			int64_t n_grp = 0;
			ap.work = work, ap.res = res, ap.cig = cig;
			ap.grp = (mbg_group_t*)calloc(n_work, sizeof(mbg_group_t));
			for (k = 0; k < n_work; ++k) {
				if (k == 0 || work[k].rid != work[k-1].rid) ap.grp[n_grp++].k0 = k;
				ap.grp[n_grp - 1].k1 = k + 1;
			}
			kt_for(g_n_thread, mbg_apply_worker, &ap, n_grp);
			for (k = 0; k < n_grp; ++k) {
				const mbg_group_t *g = &ap.grp[k];
				int32_t l;
				for (l = 0; l < g->n_next; ++l) {
					if ((n_next & (n_next - 1)) == 0) next = (mbg_work_t*)realloc(next, (n_next ? n_next << 1 : 1) * sizeof(mbg_work_t));
					next[n_next].rid = work[g->k0].rid, next[n_next].hi = g->next_hi[l], next[n_next++].opt = work[g->k0].opt;
				}
				free(g->next_hi);
			}
			free(ap.grp);
		}
		free(ch), free(res), free(cig), free(work);
		work = next, n_work = n_next;
	}
	free(work), free(anc), free(qbuf), free(opts), free(read_opt);
}

// ---- stage 3: the rest of mb_align_skeleton and mb_map_sai, per read

static void mbg_extra_worker(void *data, long rid, int tid)
{ // mb_update_extra of every aligned hit (align.c:750-755), then the inversion candidates
	const mbg_shared_t *s = (const mbg_shared_t*)data;
	mbg_read_t *r = &g_rd[rid];
	const mb_opt_t *opt = &r->opt;
	void *km = mb_tbuf_km(s->tbuf[tid]);
	int32_t i, n_regs = r->n_hit, ql = r->qlen;
	mb_hit_t *regs = r->hit;
	uint8_t *qseq0[2];
	if (r->state != 2) return;
	qseq0[0] = r->qseq0, qseq0[1] = r->qseq0 + ql;
	for (i = 0; i < n_regs; ++i) {
		mb_hit_t *h = &regs[i];
		int8_t mat[25];
		int32_t qs1 = h->rev? ql - h->qe : h->qs;
		uint8_t *tseq;
		if (!r->aligned[i] || h->p == 0) continue;
		{ // the CIGAR must span the hit, as mb_update_extra asserts (align.c:264)
			int64_t qn = 0, tn = 0;
			int32_t k;
			for (k = 0; k < h->p->n_cigar; ++k) {
				uint32_t op = h->p->cigar[k] & 0xf, len = h->p->cigar[k] >> 4;
				if (op == MB_CIGAR_MATCH || op == MB_CIGAR_INS) qn += len;
				if (op == MB_CIGAR_MATCH || op == MB_CIGAR_DEL || op == MB_CIGAR_N_SKIP) tn += len;
			}
			if (qn != h->qe - h->qs || tn != h->te - h->ts) {
				fprintf(stderr, "[E::%s] read %s hit %d: CIGAR spans %ld/%ld, coordinates [%d,%d) [%ld,%ld); %d ops\n",
						__func__, r->qname? r->qname : "*", i, (long)qn, (long)tn, h->qs, h->qe, (long)h->ts,
						(long)h->te, h->p->n_cigar);
				abort();
			}
		}
		ksw_gen_nt4_mat(mat, opt->a, opt->b, opt->b_ts, opt->b_ambi, (int)(h->rev? l2b_meth_rev(r->mt) : r->mt));
		tseq = (uint8_t*)kmalloc(km, h->te - h->ts + 1);
		l2b_getseq(s->idx->l2b, h->tid, h->ts, h->te, tseq);
		mb_update_extra(km, h, &qseq0[h->rev][qs1], tseq, mat, opt->q, opt->e, opt->flag, !r->is_sr);
		kfree(km, tseq);
	}
	for (i = 1; i < n_regs; ++i) { // mb_align1_inv's tests (align.c:765-776) on the pairs align.c:913-914 tries
		const mb_hit_t *r1 = &regs[i-1], *r2 = &regs[i];
		int32_t ql2, tl2;
		mbg_inv_t *v;
		if (!r2->split_inv) continue;
		if (!(r1->split&1) || !(r2->split&2)) continue;
		if (r1->id != r1->parent && r1->parent != MB_PARENT_TMP_PRI) continue;
		if (r2->id != r2->parent && r2->parent != MB_PARENT_TMP_PRI) continue;
		if (r1->tid != r2->tid || r1->rev != r2->rev) continue;
		ql2 = r1->rev? r1->qs - r2->qe : r2->qs - r1->qe;
		tl2 = (int32_t)(r2->ts - r1->te);
		if (ql2 < opt->min_chain_score || ql2 > opt->max_gap) continue;
		if (tl2 < opt->min_chain_score || tl2 > opt->max_gap) continue;
		r->inv = (mbg_inv_t*)realloc(r->inv, (r->n_inv + 1) * sizeof(mbg_inv_t));
		v = &r->inv[r->n_inv++];
		memset(v, 0, sizeof(*v));
		v->opt = opt, v->i = i, v->ql = ql2, v->tl = tl2;
		v->mt = (int32_t)(!r1->rev? l2b_meth_rev(r->mt) : r->mt);
		v->q = (uint8_t*)malloc(ql2 + 1), v->t = (uint8_t*)malloc(tl2 + 1);
		memcpy(v->q, r1->rev? &qseq0[0][r2->qe] : &qseq0[1][ql - r2->qs], ql2);
		l2b_getseq(s->idx->l2b, r1->tid, r1->te, r2->ts, v->t);
	}
}

static int64_t g_n_inv_cand, g_n_inv_dp;  // this mini-batch's inversion candidates and their DP

static void mbg_inversions(void)
{ // the ksw_ll and mb_align_pair of every candidate (align.c:779-792), batched on the device
	int64_t i, k, n = 0;
	int mt;
	mbg_inv_t **all;
	for (i = 0; i < g_n_rd; ++i) n += g_rd[i].n_inv;
	g_n_inv_cand = n, g_n_inv_dp = 0;
	if (n == 0) return;
	all = (mbg_inv_t**)malloc(n * sizeof(mbg_inv_t*));
	for (i = 0, n = 0; i < g_n_rd; ++i)
		for (k = 0; k < g_rd[i].n_inv; ++k) all[n++] = &g_rd[i].inv[k];
	for (mt = 0; mt < 3; ++mt) {
		const mb_opt_t *o = 0;
		ksw2g_ll_job_t *lj;
		ksw2g_ll_result_t *lr;
		ksw2g_job_t *aj;
		ksw2g_ext_result_t *ar;
		ksw2g_align_opt_t ao;
		uint8_t *qb, *tb;
		uint32_t *cig;
		int8_t mat[25];
		int64_t nq = 0, nt = 0, m = 0, na = 0, used = 0, cap = 16;
		for (i = k = 0; i < g_n_rd; ++i)
			for (k = 0; k < g_rd[i].n_inv; ++k)
				if (g_rd[i].inv[k].mt == mt) o = &g_rd[i].opt, nq += g_rd[i].inv[k].ql, nt += g_rd[i].inv[k].tl, ++m;
		if (m == 0) continue;
		ksw_gen_nt4_mat(mat, o->a, o->b, o->b_ts, o->b_ambi, mt);
		lj = (ksw2g_ll_job_t*)calloc(m, sizeof(ksw2g_ll_job_t)), lr = (ksw2g_ll_result_t*)calloc(m, sizeof(ksw2g_ll_result_t));
		qb = (uint8_t*)malloc(nq + 1), tb = (uint8_t*)malloc(nt + 1);
		for (i = 0, nq = nt = 0, m = 0; i < n; ++i) { // ksw_ll on the reversed sequences (align.c:781-786)
			mbg_inv_t *v = all[i];
			int32_t x;
			if (v->mt != mt) continue;
			lj[m].qoff = nq, lj[m].toff = nt, lj[m].qlen = v->ql, lj[m].tlen = v->tl;
			for (x = 0; x < v->ql; ++x) qb[nq + x] = v->q[v->ql - 1 - x];
			for (x = 0; x < v->tl; ++x) tb[nt + x] = v->t[v->tl - 1 - x];
			nq += v->ql, nt += v->tl, ++m;
		}
		if (ksw2g_ll_batch(g_ctx, 2, 5, mat, o->q, o->e, (int)m, lj, qb, nq + 1, tb, nt + 1, lr)) mbg_fail("ksw2g_ll_batch");
		aj = (ksw2g_job_t*)calloc(m, sizeof(ksw2g_job_t)), ar = (ksw2g_ext_result_t*)calloc(m, sizeof(ksw2g_ext_result_t));
		for (i = 0, m = 0, nq = nt = 0; i < n; ++i) { // mb_align_pair from ksw_ll's end (align.c:790-792)
			mbg_inv_t *v = all[i];
			if (v->mt != mt) continue;
			v->score = lr[m].score;
			v->q_off = v->ql - (lr[m].qe + 1), v->t_off = v->tl - (lr[m].te + 1);
			++m;
			if (v->score < v->opt->min_dp_max * v->opt->a) { v->score = -1; continue; }
			aj[na].qoff = nq, aj[na].toff = nt, aj[na].qlen = v->ql - v->q_off, aj[na].tlen = v->tl - v->t_off;
			aj[na].w = (int)(v->opt->bw * 1.5), aj[na].zdrop = v->opt->zdrop, aj[na].end_bonus = -1;
			aj[na].flag = KSW_EZ_EXTZ_ONLY;
			memcpy(qb + nq, v->q + v->q_off, aj[na].qlen), memcpy(tb + nt, v->t + v->t_off, aj[na].tlen);
			nq += aj[na].qlen, nt += aj[na].tlen, cap += aj[na].qlen + aj[na].tlen + 1, ++na;
		}
		g_n_inv_dp += na;
		if (na > 0) {
			ao.a = o->a, ao.b = o->b, ao.b_ts = o->b_ts, ao.b_ambi = o->b_ambi, ao.q = o->q, ao.e = o->e;
			ao.q2 = o->q2, ao.e2 = o->e2, ao.meth = !!(o->flag & MB_F_METH), ao.pad = 0, ao.max_sw_mat = o->max_sw_mat;
			cig = (uint32_t*)malloc(cap * sizeof(uint32_t));
			if (ksw2g_align_pairs(g_ctx, &ao, mat, (int)na, aj, qb, nq + 1, tb, nt + 1, ar, cig, cap, &used))
				mbg_fail("ksw2g_align_pairs");
			for (i = 0, na = 0; i < n; ++i) {
				mbg_inv_t *v = all[i];
				if (v->mt != mt || v->score < 0) continue;
				v->ez = ar[na++];
				if (v->ez.n_cigar > 0) {
					v->cigar = (uint32_t*)malloc(v->ez.n_cigar * sizeof(uint32_t));
					memcpy(v->cigar, cig + v->ez.cigar_off, v->ez.n_cigar * sizeof(uint32_t));
				}
			}
			free(cig);
		}
		free(lj), free(lr), free(qb), free(tb), free(aj), free(ar);
	}
	free(all);
}

static void mbg_finish_worker(void *data, long rid, int tid)
{
	const mbg_shared_t *s = (const mbg_shared_t*)data;
	mbg_read_t *r = &g_rd[rid];
	const mb_opt_t *opt = &r->opt;
	void *km = mb_tbuf_km(s->tbuf[tid]);
	int32_t i, k, n_regs = r->n_hit, ql = r->qlen;
	mb_hit_t *regs = r->hit;
	if (r->state != 2) return;
	if (r->n_inv > 0) { // align.c:913-918: an INV hit goes after the split hit; the next pair then starts at it
		mb_hit_t *nr = (mb_hit_t*)malloc((n_regs + r->n_inv) * sizeof(mb_hit_t));
		int32_t o = 0, prev_inv = 0;
		for (i = 0, k = 0; i < n_regs; ++i) {
			mbg_inv_t *v = k < r->n_inv && r->inv[k].i == i? &r->inv[k++] : 0;
			nr[o++] = regs[i];
			if (v && !prev_inv && v->score >= 0 && v->ez.n_cigar > 0) { // align.c:793-810
				const mb_hit_t *r1 = &regs[i-1], *r2 = &regs[i];
				mb_hit_t *ri = &nr[o++];
				int8_t mat[25];
				memset(ri, 0, sizeof(mb_hit_t));
				mb_append_cigar(ri, v->ez.n_cigar, v->cigar);
				ri->p->dp_score = v->ez.max;
				ri->id = -1;
				ri->parent = MB_PARENT_UNSET;
				ri->inv = 1;
				ri->rev = !r1->rev;
				ri->tid = r1->tid;
				if (ri->rev == 0) {
					ri->qs = r2->qe + v->q_off;
					ri->qe = ri->qs + v->ez.max_q + 1;
				} else {
					ri->qe = r2->qs - v->q_off;
					ri->qs = ri->qe - (v->ez.max_q + 1);
				}
				ri->ts = r1->te + v->t_off;
				ri->te = ri->ts + v->ez.max_t + 1;
				ksw_gen_nt4_mat(mat, opt->a, opt->b, opt->b_ts, opt->b_ambi, v->mt);
				mb_update_extra(km, ri, v->q + v->q_off, v->t + v->t_off, mat, opt->q, opt->e, opt->flag,
								mb_is_sr_mode(opt, ql));
				prev_inv = 1;
			} else prev_inv = 0;
		}
		for (k = 0; k < r->n_inv; ++k) free(r->inv[k].q), free(r->inv[k].t), free(r->inv[k].cigar);
		free(r->inv), free(regs);
		r->inv = 0, r->n_inv = 0;
		regs = nr, n_regs = o;
	}
	mb_filter_hits(opt, ql, &n_regs, regs); // align.c:921-927
	if (!mb_is_sr_mode(opt, ql)) {
		mb_update_dp_max(ql, n_regs, regs, 0.9, opt->a, opt->b);
		mb_filter_hits(opt, ql, &n_regs, regs);
	}
	mb_hit_sort(km, &n_regs, regs);
	mb_set_parent(km, opt->mask_level, opt->mask_len, n_regs, regs, r->sub_diff, 0); // map-algo.c:640-657
	mb_select_sub(km, opt->pri_ratio, opt->min_len * 2, opt->best_n, &n_regs, regs);
	mb_set_sam_pri(n_regs, regs, !!(opt->flag & MB_F_PRIMARY5));
	for (i = 0; i < n_regs; ++i) {
		regs[i].frac_high = (int32_t)(255. * r->hi_cov / ql);
		regs[i].seed_ratio = (int32_t)(255. * r->seed_ratio + .499);
		if (regs[i].seed_ratio == 0) regs[i].seed_ratio = 1;
	}
	mb_set_mapq(km, ql, n_regs, regs, opt->min_chain_score, opt->a, r->is_sr, opt->max_sr_len);
	free(r->a), free(r->seq), free(r->qseq0), free(r->aligned);
	r->a = 0, r->seq = r->qseq0 = r->aligned = 0;
	r->hit = regs, r->n_hit = n_regs;
}

void mbg_step_end(const mb_opt_t *opt, const mb_idx_t *idx, int n_thread, mb_tbuf_t **tbuf, int64_t n_seq,
                  mb_hit_t **hit, int32_t *n_hit)
{
	mbg_shared_t s;
	int64_t i, n_def = 0;
	s.opt = opt, s.idx = idx, s.tbuf = tbuf;
	g_n_thread = n_thread;
	for (i = 0; i < n_seq; ++i) n_def += g_rd[i].state == 2;
	if (n_def > 0) {
		double t0 = mbg_ms(), t1, t2, t3, t4;
		if (g_init_running) pthread_join(g_init_tid, 0), g_init_running = 0;
		mbg_gpu_init(idx);
		t1 = mbg_ms();
		kt_for(n_thread, mbg_prepare_worker, &s, n_seq);
		t2 = mbg_ms();
		mbg_align_rounds(idx);
		t3 = mbg_ms();
		kt_for(n_thread, mbg_extra_worker, &s, n_seq);
		mbg_inversions();
		kt_for(n_thread, mbg_finish_worker, &s, n_seq);
		t4 = mbg_ms();
		if (g_timing)
			fprintf(stderr, "[M::mbg] %ld reads (%ld deferred): seeding and chaining %.1f ms, GPU setup %.1f, "
					"prepare %.1f, alignment rounds %.1f, finishing %.1f (%ld inversion candidates, %ld aligned)\n",
					(long)n_seq, (long)n_def, t0 - g_t_begin, t1 - t0, t2 - t1, t3 - t2, t4 - t3,
					(long)g_n_inv_cand, (long)g_n_inv_dp);
	}
	for (i = 0; i < n_seq; ++i)
		if (g_rd[i].state != 0) hit[i] = g_rd[i].hit, n_hit[i] = g_rd[i].n_hit;
	for (i = 0; i < n_thread; ++i) mb_tbuf_reset(tbuf[i], opt->cap_kalloc);
	free(g_rd);
	g_rd = 0, g_n_rd = 0;
}
