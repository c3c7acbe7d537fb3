/*
 * synth.c -- seeded synthetic DP jobs with the shapes of the benchmark
 * configurations (extension pairs: query + mutated copy + random flank;
 * rescue jobs: query vs a window that may hold a planted copy).
 * RNG: splitmix64, the convention of the reference's kom_splitmix64
 * (kommon.h:66).  Bases are codes 0..3, N is 4.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct {
	int qlen_lo, qlen_hi;         /* uniform query length (used when lognorm_median <= 0) */
	double lognorm_median, lognorm_sigma;
	int clip_lo, clip_hi;
	double n_rate, sub_rate, indel_rate, indel_p; /* indel length: geometric(indel_p) capped at indel_max */
	int indel_max, flank;
	double junk_frac;             /* fraction of pairs whose query gets a random suffix */
	int junk_len;
} synth_ext_spec_t;

typedef struct {
	int qlen, tlen_lo, tlen_hi;
	double plant_frac, sub_rate, indel_rate, indel_p;
	int indel_max;
} synth_ll_spec_t;

static inline uint64_t sm64(uint64_t *s)
{
	uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
	return z ^ (z >> 31);
}
static inline double unif(uint64_t *s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }
static inline int ri(uint64_t *s, int lo, int hi) { return lo + (int)(sm64(s) % (uint64_t)(hi - lo + 1)); }
static inline uint8_t base(uint64_t *s) { return (uint8_t)(sm64(s) & 3); }
static int geom(uint64_t *s, double p, int cap)
{
	int l = 1;
	while (l < cap && unif(s) >= p) ++l;
	return l;
}

/* copy src[0..n) into dst with substitutions and indels; returns bases written (<= cap) */
static int64_t mutate(uint64_t *s, const uint8_t *src, int n, uint8_t *dst, int64_t cap, double sub, double ind,
					  double ip, int imax)
{
	int64_t o = 0;
	int i, k;
	for (i = 0; i < n && o < cap; ++i) {
		double u = unif(s);
		if (u < ind * 0.5) { /* deletion from the copy */
			i += geom(s, ip, imax) - 1;
			continue;
		} else if (u < ind) { /* insertion into the copy */
			int l = geom(s, ip, imax);
			for (k = 0; k < l && o < cap; ++k) dst[o++] = base(s);
		}
		if (o >= cap) break;
		{
			uint8_t c = src[i] > 3 ? base(s) : src[i];
			if (unif(s) < sub) c = (uint8_t)((c + 1 + (sm64(s) % 3)) & 3);
			dst[o++] = c;
		}
	}
	return o;
}

/* Returns 0, or -1 when qcap/tcap is too small. */
int synth_ext(const synth_ext_spec_t *sp, uint64_t seed, int n, int64_t *qoff, int32_t *qlen, int64_t *toff,
			  int32_t *tlen, uint8_t *qbuf, int64_t qcap, uint8_t *tbuf, int64_t tcap, int64_t *qused, int64_t *tused)
{
	uint64_t s = seed;
	int64_t qo = 0, to = 0;
	int i, k;
	for (i = 0; i < n; ++i) {
		int L, J = 0;
		int64_t t0;
		if (sp->lognorm_median > 0) {
			double u1 = unif(&s), u2 = unif(&s), z;
			if (u1 < 1e-300) u1 = 1e-300;
			z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
			L = (int)(sp->lognorm_median * exp(sp->lognorm_sigma * z) + 0.5);
			if (L < sp->clip_lo) L = sp->clip_lo;
			if (L > sp->clip_hi) L = sp->clip_hi;
		} else L = ri(&s, sp->qlen_lo, sp->qlen_hi);
		if (sp->junk_frac > 0 && unif(&s) < sp->junk_frac) J = sp->junk_len;
		if (qo + L + J > qcap) return -1;
		for (k = 0; k < L; ++k) qbuf[qo + k] = (sp->n_rate > 0 && unif(&s) < sp->n_rate) ? 4 : base(&s);
		t0 = to;
		to += mutate(&s, qbuf + qo, L, tbuf + to, tcap - to - sp->flank, sp->sub_rate, sp->indel_rate, sp->indel_p,
					 sp->indel_max);
		if (to + sp->flank > tcap) return -1;
		for (k = 0; k < sp->flank; ++k) tbuf[to++] = base(&s);
		for (k = 0; k < J; ++k) qbuf[qo + L + k] = base(&s);
		qoff[i] = qo, qlen[i] = L + J, toff[i] = t0, tlen[i] = (int32_t)(to - t0);
		qo += L + J;
	}
	*qused = qo, *tused = to;
	return 0;
}

int synth_ll(const synth_ll_spec_t *sp, uint64_t seed, int n, int64_t *qoff, int32_t *qlen, int64_t *toff,
			 int32_t *tlen, uint8_t *qbuf, int64_t qcap, uint8_t *tbuf, int64_t tcap, int64_t *qused, int64_t *tused)
{
	uint64_t s = seed;
	int64_t qo = 0, to = 0;
	uint8_t tmp[65536];
	int i, k;
	for (i = 0; i < n; ++i) {
		int T = ri(&s, sp->tlen_lo, sp->tlen_hi), L = sp->qlen;
		if (qo + L > qcap || to + T > tcap || L > 32768) return -1;
		for (k = 0; k < L; ++k) qbuf[qo + k] = base(&s);
		for (k = 0; k < T; ++k) tbuf[to + k] = base(&s);
		if (unif(&s) < sp->plant_frac) {
			int64_t m = mutate(&s, qbuf + qo, L, tmp, sizeof tmp, sp->sub_rate, sp->indel_rate, sp->indel_p, sp->indel_max);
			if (m <= T) {
				int off = ri(&s, 0, T - (int)m);
				memcpy(tbuf + to + off, tmp, (size_t)m);
			}
		}
		qoff[i] = qo, qlen[i] = L, toff[i] = to, tlen[i] = T;
		qo += L, to += T;
	}
	*qused = qo, *tused = to;
	return 0;
}

/* Mate-rescue candidates over a decoded genome (codes 0..4, contigs back to
 * back): an anchor hit, one orientation dir with insert bounds [lo, hi], the
 * candidate window and read orientation as pe.c:330-339 computes them, and the
 * mate read in the orientation pe.c aligns (a mutated copy of a stretch of the
 * window, or random bases), methylation-converted for methylation modes. */
typedef struct {
	int qlen_lo, qlen_hi, lo, hi;
	double p_random, p_meth, sub_rate, indel_rate;
	int min_sc_hi;
} synth_rescue_spec_t;

typedef struct {
	int64_t qoff, ts, te;
	int32_t qlen, tid, meth, min_sc, rev, pad;
} synth_rescue_job_t;

int synth_rescue(const synth_rescue_spec_t *sp, uint64_t seed, const uint8_t *genome, int n_ctg,
				 const uint64_t *ctg_off, const uint64_t *ctg_len, int n, synth_rescue_job_t *jobs, uint8_t *qbuf,
				 int64_t qcap, int64_t *qused)
{
	uint64_t s = seed;
	int64_t qo = 0;
	uint8_t tmp[65536];
	int i, k, tries = 0;
	for (i = 0; i < n;) {
		int t = ri(&s, 0, n_ctg - 1), l0 = ri(&s, sp->qlen_lo, sp->qlen_hi), L = ri(&s, sp->qlen_lo, sp->qlen_hi);
		int h_rev = ri(&s, 0, 1), r0 = ri(&s, 0, 1), dir = ri(&s, 0, 3), is_rev, is_larger, mt0 = 0, mt;
		int64_t clen = (int64_t)ctg_len[t], h_ts, pos5, ts, te;
		if (++tries > 100 * (n + 16)) return -2;
		if (clen < 3 * ((int64_t)sp->hi + 2 * sp->qlen_hi) || L > 32768) continue;
		if (unif(&s) < sp->p_meth) mt0 = ri(&s, 1, 2);
		h_ts = (int64_t)(sm64(&s) % (uint64_t)(clen - l0));
		pos5 = h_rev ? h_ts + l0 : h_ts;
		is_rev = ((dir >> 1) != (dir & 1)) ^ h_rev;
		is_larger = (dir >> 1) != (dir & 1) ? (dir >> 1) ^ is_rev : (dir >> 1) ^ r0 ^ h_rev;
		ts = (is_larger ? pos5 + sp->lo : pos5 - sp->hi) - (!is_rev ? 0 : L);
		te = (is_larger ? pos5 + sp->hi : pos5 - sp->lo) + (!is_rev ? L : 0);
		if (ts < 0) ts = 0;
		if (te > clen) te = clen;
		if (te - ts <= L) continue;
		mt = mt0 == 0 ? 0 : is_rev ? 3 - mt0 : mt0;  /* l2b_meth_rev */
		if (unif(&s) < sp->p_random) {
			for (k = 0; k < L; ++k) tmp[k] = base(&s);
		} else {
			int64_t ms = ts + (int64_t)(sm64(&s) % (uint64_t)(te - ts - L + 1));
			L = (int)mutate(&s, genome + ctg_off[t] + ms, L, tmp, sizeof tmp, sp->sub_rate, sp->indel_rate, 0.5, 3);
			if (mt)
				for (k = 0; k < L; ++k)
					if (tmp[k] == (mt == 1 ? 1 : 2) && unif(&s) < 0.9) tmp[k] = mt == 1 ? 3 : 0;
		}
		/* the window follows the read's final length, as pe.c computes it from len */
		ts = (is_larger ? pos5 + sp->lo : pos5 - sp->hi) - (!is_rev ? 0 : L);
		te = (is_larger ? pos5 + sp->hi : pos5 - sp->lo) + (!is_rev ? L : 0);
		if (ts < 0) ts = 0;
		if (te > clen) te = clen;
		if (te - ts <= L || L <= 0) continue;
		if (qo + L > qcap) return -1;
		memcpy(qbuf + qo, tmp, (size_t)L);
		jobs[i].qoff = qo, jobs[i].ts = ts, jobs[i].te = te, jobs[i].qlen = L, jobs[i].tid = t;
		jobs[i].meth = mt, jobs[i].min_sc = ri(&s, 0, sp->min_sc_hi), jobs[i].rev = is_rev, jobs[i].pad = 0;
		qo += L, ++i;
	}
	*qused = qo;
	return 0;
}
