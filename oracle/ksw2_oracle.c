/*
 * ksw2_oracle.c -- scalar CPU restatement of minibwa's ksw2 kernels.
 *
 * TEST INFRASTRUCTURE ONLY (see ksw2_oracle.h).  This file is the checker for
 * the CUDA implementation; it is never linked into the product library.
 *
 * Every SSE lane operation of the reference is restated as a byte (or 16-bit)
 * operation with the same wrap / saturate / signed / unsigned semantics
 * (the per-intrinsic table in s2n-lite.h:8-53 is the reference for those).
 * The banded extension kernels keep the reference's flat working-memory layout
 * (u, v, x, y, [x2, y2], s, sf, qr packed back to back in 16-byte blocks,
 * ksw2_extz2_sse.c:76-78, ksw2_extd2_sse.c:99-102), because values outside the
 * nominal band -- the 16-byte padding of every anti-diagonal
 * (ksw2_extz2_sse.c:108) and the 16-byte score stores that run past en0
 * (ksw2_extz2_sse.c:118-132) -- are read back as neighbours and therefore
 * decide the result.
 */
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include "ksw2_oracle.h"

#define ORC_NEG_INF (-0x40000000)

/* flag bits, ksw2.h:8-22 */
#define F_SCORE_ONLY  0x01
#define F_RIGHT       0x02
#define F_GENERIC_SC  0x04
#define F_APPROX_MAX  0x08
#define F_APPROX_DROP 0x10
#define F_EXTZ_ONLY   0x40
#define F_REV_CIGAR   0x80
#define F_LL_STOP     0x20000
#define F_LL_SUBO     0x40000

typedef uint8_t u8;

/* ---- byte-lane primitives (one lane of the SSE ops) ---- */
static inline u8 bw_add(u8 a, u8 b) { return (u8)(a + b); }            /* _mm_add_epi8 (wraps) */
static inline u8 bw_sub(u8 a, u8 b) { return (u8)(a - b); }            /* _mm_sub_epi8 (wraps) */
static inline int bs_gt(u8 a, u8 b) { return (int8_t)a > (int8_t)b; }  /* _mm_cmpgt_epi8 */
static inline u8 bs_max(u8 a, u8 b) { return bs_gt(a, b) ? a : b; }     /* _mm_max_epi8 */
static inline u8 bs_min(u8 a, u8 b) { return bs_gt(a, b) ? b : a; }     /* _mm_min_epi8 */
static inline u8 bu_max(u8 a, u8 b) { return a > b ? a : b; }           /* _mm_max_epu8 */
static inline u8 bu_min(u8 a, u8 b) { return a < b ? a : b; }           /* _mm_min_epu8 */
static inline u8 bu_adds(u8 a, u8 b) { int s = a + b; return (u8)(s > 255 ? 255 : s); } /* _mm_adds_epu8 */
static inline u8 bu_subs(u8 a, u8 b) { return a > b ? (u8)(a - b) : 0; }                /* _mm_subs_epu8 */

/* ---- CIGAR push with the reference's growth policy (ksw2.h:124-134) ---- */
static uint32_t *cig_push(int *n_cigar, int *m_cigar, uint32_t *cigar, uint32_t op, int len)
{
	if (*n_cigar == 0 || op != (cigar[*n_cigar - 1] & 0xf)) {
		if (*n_cigar == *m_cigar) {
			*m_cigar = *m_cigar ? (*m_cigar) << 1 : 4;
			cigar = (uint32_t *)realloc(cigar, (size_t)(*m_cigar) << 2);
		}
		cigar[(*n_cigar)++] = (uint32_t)len << 4 | op;
	} else cigar[*n_cigar - 1] += (uint32_t)len << 4;
	return cigar;
}

/* Walk of ksw2.h:140-172 for the rotated (anti-diagonal) layout, without the
 * splice branch (min_intron_len is always 0 on this path). */
static void backtrack_rot(int is_rev, const u8 *p, const int *off, const int *off_end, int n_col, int i0, int j0,
						  int *m_cigar_, int *n_cigar_, uint32_t **cigar_)
{
	int n_cigar = 0, m_cigar = *m_cigar_, i = i0, j = j0, state = 0;
	uint32_t *cigar = *cigar_;
	while (i >= 0 && j >= 0) {
		int r = i + j, force = -1;
		unsigned tb;
		if (i < off[r]) force = 2;
		if (i > off_end[r]) force = 1;
		tb = force < 0 ? p[(size_t)r * n_col + i - off[r]] : 0;
		if (state == 0) state = tb & 7;
		else if (!(tb >> (state + 2) & 1)) state = 0;
		if (state == 0) state = tb & 7;
		if (force >= 0) state = force;
		if (state == 0) cigar = cig_push(&n_cigar, &m_cigar, cigar, 0, 1), --i, --j;
		else if (state == 1 || state == 3) cigar = cig_push(&n_cigar, &m_cigar, cigar, 2, 1), --i;
		else cigar = cig_push(&n_cigar, &m_cigar, cigar, 1, 1), --j;
	}
	if (i >= 0) cigar = cig_push(&n_cigar, &m_cigar, cigar, 2, i + 1);
	if (j >= 0) cigar = cig_push(&n_cigar, &m_cigar, cigar, 1, j + 1);
	if (!is_rev) {
		int k;
		for (k = 0; k < n_cigar >> 1; ++k) {
			uint32_t t = cigar[k];
			cigar[k] = cigar[n_cigar - 1 - k];
			cigar[n_cigar - 1 - k] = t;
		}
	}
	*m_cigar_ = m_cigar, *n_cigar_ = n_cigar, *cigar_ = cigar;
}

static void reset_extz(orc_extz_t *ez) /* ksw2.h:174-179 */
{
	ez->max_q = ez->max_t = ez->mqe_t = ez->mte_q = -1;
	ez->max = 0, ez->score = ez->mqe = ez->mte = ORC_NEG_INF;
	ez->n_cigar = 0, ez->zdropped = 0, ez->reach_end = 0;
}

/* ksw2.h:181-197, rotated coordinates: a = anti-diagonal r, b = target t */
static int apply_zdrop(orc_extz_t *ez, int32_t H, int r, int t, int zdrop, int8_t e)
{
	if (H > (int32_t)ez->max) {
		ez->max = (uint32_t)H, ez->max_t = t, ez->max_q = r - t;
	} else if (t >= ez->max_t && r - t >= ez->max_q) {
		int tl = t - ez->max_t, ql = (r - t) - ez->max_q, l;
		l = tl > ql ? tl - ql : ql - tl;
		if (zdrop >= 0 && (int)ez->max - H > zdrop + l * e) {
			ez->zdropped = 1;
			return 1;
		}
	}
	return 0;
}

/*
 * Shared restatement of ksw_extz2_sse (ksw2_extz2_sse.c:16-296, dual == 0) and
 * ksw_extd2_sse (ksw2_extd2_sse.c:27-403, dual == 1).
 */
static void ext_core(int dual, int qlen, const u8 *query, int tlen, const u8 *target, int8_t m, const int8_t *mat,
					 int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus, int flag,
					 orc_extz_t *ez, orc_stats_t *stt)
{
	int r, t, qe, n_col_, tlen_, qlen_, T, last_st, last_en, max_sc, min_sc, long_thres = 0, long_diff = 0;
	int with_cigar = !(flag & F_SCORE_ONLY), approx_max = !!(flag & F_APPROX_MAX);
	int32_t *H = 0, H0 = 0, last_H0_t = 0, last_max_H = 0;
	int *off = 0, *off_end = 0;
	u8 *mem, *U, *V, *X, *Y, *X2 = 0, *Y2 = 0, *S, *SF, *QR, *P = 0;
	u8 c_q, c_q2 = 0, c_qe, c_qe2, c_mch, c_mis, c_N, c_m1, c_maxsc = 0;
	size_t nblk;

	if (stt) stt->cells = stt->padded_cells = 0, stt->n_diag = 0;
	reset_extz(ez);
	if (m <= dual || qlen <= 0 || tlen <= 0) return; /* extz2:49, extd2:68 */
	qe = q + e; /* extd2:60 takes q+e before the swap below; only H at r == 0 uses it */
	if (dual && q2 + e2 < q + e) { /* extd2:70 */
		int8_t tmp;
		tmp = q, q = q2, q2 = tmp;
		tmp = e, e = e2, e2 = tmp;
	}
	c_q = (u8)q, c_qe = (u8)(q + e);
	c_mch = (u8)mat[0], c_mis = (u8)mat[1], c_m1 = (u8)(m - 1);
	if (!dual) {
		c_qe2 = (u8)((q + e) * 2);                 /* extz2:53 */
		c_N = mat[m * m - 1] == 0 ? (u8)(-e) : (u8)mat[m * m - 1];
		c_maxsc = (u8)(mat[0] + (q + e) * 2);      /* extz2:62 */
	} else {
		c_q2 = (u8)q2, c_qe2 = (u8)(q2 + e2);      /* extd2:74-76 */
		c_N = mat[m * m - 1] == 0 ? (u8)(-e2) : (u8)mat[m * m - 1];
	}
	if (w < 0) w = tlen > qlen ? tlen : qlen;
	tlen_ = (tlen + 15) / 16;
	n_col_ = qlen < tlen ? qlen : tlen;
	n_col_ = ((n_col_ < w + 1 ? n_col_ : w + 1) + 15) / 16 + 1;
	qlen_ = (qlen + 15) / 16;
	for (t = 1, max_sc = mat[0], min_sc = mat[1]; t < m * m; ++t) {
		max_sc = max_sc > mat[t] ? max_sc : mat[t];
		min_sc = min_sc < mat[t] ? min_sc : mat[t];
	}
	if (-min_sc > 2 * (q + e)) return; /* extz2:74, extd2:92 */
	if (dual) { /* extd2:94-97 */
		long_thres = e != e2 ? (q2 - q) / (e - e2) - 1 : 0;
		if (q2 + e2 + long_thres * e2 > q + e + long_thres * e) ++long_thres;
		long_diff = long_thres * (e - e2) - (q2 - q) - e2;
	}

	/* working memory: same block layout as the reference, zero filled */
	T = tlen_ * 16;
	nblk = (size_t)tlen_ * (dual ? 8 : 6) + qlen_ + 1;
	mem = (u8 *)calloc(nblk * 16 + 64, 1);
	U = mem, V = U + T, X = V + T, Y = X + T;
	if (dual) {
		X2 = Y + T, Y2 = X2 + T, S = Y2 + T;
		memset(U, (u8)(-q - e), T); memset(V, (u8)(-q - e), T);
		memset(X, (u8)(-q - e), T); memset(Y, (u8)(-q - e), T);
		memset(X2, (u8)(-q2 - e2), T); memset(Y2, (u8)(-q2 - e2), T);
	} else S = Y + T;
	SF = S + T, QR = SF + T;
	if (!approx_max) {
		H = (int32_t *)malloc((size_t)T * 4);
		for (t = 0; t < T; ++t) H[t] = ORC_NEG_INF;
	}
	if (with_cigar) {
		P = (u8 *)malloc(((size_t)(qlen + tlen - 1) * n_col_ + 1) * 16);
		off = (int *)malloc((size_t)(qlen + tlen - 1) * sizeof(int) * 2);
		off_end = off + qlen + tlen - 1;
	}
	for (t = 0; t < qlen; ++t) QR[t] = query[qlen - 1 - t];
	memcpy(SF, target, tlen);

	for (r = 0, last_st = last_en = -1; r < qlen + tlen - 1; ++r) {
		int st = 0, en = tlen - 1, st0, en0;
		u8 x1, v1, x21 = 0, extx = 0, extv = 0, ox, ov, ox2 = 0;
		const u8 *qrr = QR + (qlen - 1 - r);
		/* band of anti-diagonal r (extz2:99-106) */
		if (st < r - qlen + 1) st = r - qlen + 1;
		if (en > r) en = r;
		if (st < (r - w + 1) >> 1) st = (r - w + 1) >> 1;
		if (en > (r + w) >> 1) en = (r + w) >> 1;
		if (st > en) {
			ez->zdropped = 1;
			break;
		}
		st0 = st, en0 = en;
		st = st / 16 * 16, en = (en + 16) / 16 * 16 - 1; /* extz2:108 */
		if (stt) stt->cells += en0 - st0 + 1, stt->padded_cells += en - st + 1, stt->n_diag++;
		/* boundary values (extz2:110-115, extd2:141-155) */
		if (!dual) {
			if (st > 0) {
				if (st - 1 >= last_st && st - 1 <= last_en) x1 = X[st - 1], v1 = V[st - 1];
				else x1 = v1 = 0;
			} else x1 = 0, v1 = r ? c_q : 0;
			if (en >= r) Y[r] = 0, U[r] = r ? c_q : 0;
			/* _mm_cvtsi32_si128 of an int8_t sign-extends into lanes 1..3 (extz2:138-139) */
			extx = (x1 & 0x80) ? 0xff : 0;
			extv = (v1 & 0x80) ? 0xff : 0;
		} else {
			u8 vb = r == 0 ? (u8)(-q - e) : r < long_thres ? (u8)(-e) : r == long_thres ? (u8)long_diff : (u8)(-e2);
			if (st > 0) {
				if (st - 1 >= last_st && st - 1 <= last_en) x1 = X[st - 1], x21 = X2[st - 1], v1 = V[st - 1];
				else x1 = (u8)(-q - e), x21 = (u8)(-q2 - e2), v1 = (u8)(-q - e);
			} else x1 = (u8)(-q - e), x21 = (u8)(-q2 - e2), v1 = vb;
			if (en >= r) Y[r] = (u8)(-q - e), Y2[r] = (u8)(-q2 - e2), U[r] = vb;
		}
		/* substitution scores ("loop fission", extz2:117-136): 16-byte stores from st0 */
		if (!(flag & F_GENERIC_SC)) {
			for (t = st0; t <= en0; t += 16) {
				u8 tmp[16];
				int k;
				for (k = 0; k < 16; ++k) {
					u8 sq = SF[t + k], sr = qrr[t + k];
					u8 sc = sq == sr ? c_mch : c_mis;
					tmp[k] = (sq == c_m1 || sr == c_m1) ? c_N : sc;
				}
				memcpy(S + t, tmp, 16); /* may run past the s block into sf, as the reference does */
			}
		} else {
			for (t = st0; t <= en0; ++t) S[t] = (u8)mat[SF[t] * m + qrr[t]];
		}
		if (with_cigar) off[r] = st, off_end[r] = en;
		/* core: cells st..en in ascending order; ox/ov/ox2 carry the previous
		 * anti-diagonal's byte at t-1 (extz2:18-39, extd2:30-58) */
		ox = x1, ov = v1, ox2 = x21;
		for (t = st; t <= en; ++t) {
			u8 xp = ox, vp = ov, x2p = ox2, up = U[t], z, a, b, a2 = 0, b2 = 0, d = 0;
			if (!dual && t > st && t <= st + 3) xp |= extx, vp |= extv;
			ox = X[t], ov = V[t];
			if (dual) ox2 = X2[t];
			if (!dual) {
				z = bw_add(S[t], c_qe2);
				a = bw_add(xp, vp);
				b = bw_add(Y[t], up);
				if (!with_cigar) { /* extz2:146-161 */
					z = bs_max(z, a);
					z = bu_max(z, b);
					z = bu_min(z, c_maxsc);
				} else if (!(flag & F_RIGHT)) { /* extz2:169-179 */
					d = bs_gt(a, z) ? 1 : 0;
					z = bs_max(z, a);
					if (bs_gt(b, z)) d = 2;
					z = bu_max(z, b);
					z = bu_min(z, c_maxsc);
				} else { /* extz2:195-205 */
					d = bs_gt(z, a) ? 0 : 1;
					z = bs_max(z, a);
					if (!bs_gt(z, b)) d = 2;
					z = bu_max(z, b);
					z = bu_min(z, c_maxsc);
				}
				U[t] = bw_sub(z, vp);
				V[t] = bw_sub(z, up);
				z = bw_sub(z, c_q);
				a = bw_sub(a, z);
				b = bw_sub(b, z);
				if (!with_cigar) {
					X[t] = bs_max(a, 0), Y[t] = bs_max(b, 0);
				} else if (!(flag & F_RIGHT)) { /* extz2:181-187 */
					if (bs_gt(a, 0)) X[t] = a, d |= 0x08; else X[t] = 0;
					if (bs_gt(b, 0)) Y[t] = b, d |= 0x10; else Y[t] = 0;
				} else { /* extz2:207-213 */
					if (bs_gt(0, a)) X[t] = 0; else X[t] = a, d |= 0x08;
					if (bs_gt(0, b)) Y[t] = 0; else Y[t] = b, d |= 0x10;
				}
			} else {
				u8 tmp;
				z = S[t];
				a = bw_add(xp, vp);
				b = bw_add(Y[t], up);
				a2 = bw_add(x2p, vp);
				b2 = bw_add(Y2[t], up);
				if (!with_cigar) { /* extd2:188-192 */
					z = bs_max(z, a); z = bs_max(z, b); z = bs_max(z, a2); z = bs_max(z, b2);
					z = bs_min(z, c_mch);
				} else if (!(flag & F_RIGHT)) { /* extd2:227-235 */
					d = bs_gt(a, z) ? 1 : 0;
					z = bs_max(z, a);
					if (bs_gt(b, z)) d = 2;
					z = bs_max(z, b);
					if (bs_gt(a2, z)) d = 3;
					z = bs_max(z, a2);
					if (bs_gt(b2, z)) d = 4;
					z = bs_max(z, b2);
					z = bs_min(z, c_mch);
				} else { /* extd2:274-282 */
					d = bs_gt(z, a) ? 0 : 1;
					z = bs_max(z, a);
					if (!bs_gt(z, b)) d = 2;
					z = bs_max(z, b);
					if (!bs_gt(z, a2)) d = 3;
					z = bs_max(z, a2);
					if (!bs_gt(z, b2)) d = 4;
					z = bs_max(z, b2);
					z = bs_min(z, c_mch);
				}
				U[t] = bw_sub(z, vp);
				V[t] = bw_sub(z, up);
				tmp = bw_sub(z, c_q);
				a = bw_sub(a, tmp), b = bw_sub(b, tmp);
				tmp = bw_sub(z, c_q2);
				a2 = bw_sub(a2, tmp), b2 = bw_sub(b2, tmp);
				if (!with_cigar) { /* extd2:194-197 */
					X[t] = bw_sub(bs_max(a, 0), c_qe);
					Y[t] = bw_sub(bs_max(b, 0), c_qe);
					X2[t] = bw_sub(bs_max(a2, 0), c_qe2);
					Y2[t] = bw_sub(bs_max(b2, 0), c_qe2);
				} else if (!(flag & F_RIGHT)) { /* extd2:253-264 */
					if (bs_gt(a, 0)) X[t] = bw_sub(a, c_qe), d |= 0x08; else X[t] = bw_sub(0, c_qe);
					if (bs_gt(b, 0)) Y[t] = bw_sub(b, c_qe), d |= 0x10; else Y[t] = bw_sub(0, c_qe);
					if (bs_gt(a2, 0)) X2[t] = bw_sub(a2, c_qe2), d |= 0x20; else X2[t] = bw_sub(0, c_qe2);
					if (bs_gt(b2, 0)) Y2[t] = bw_sub(b2, c_qe2), d |= 0x40; else Y2[t] = bw_sub(0, c_qe2);
				} else { /* extd2:300-311 */
					if (bs_gt(0, a)) X[t] = bw_sub(0, c_qe); else X[t] = bw_sub(a, c_qe), d |= 0x08;
					if (bs_gt(0, b)) Y[t] = bw_sub(0, c_qe); else Y[t] = bw_sub(b, c_qe), d |= 0x10;
					if (bs_gt(0, a2)) X2[t] = bw_sub(0, c_qe2); else X2[t] = bw_sub(a2, c_qe2), d |= 0x20;
					if (bs_gt(0, b2)) Y2[t] = bw_sub(0, c_qe2); else Y2[t] = bw_sub(b2, c_qe2), d |= 0x40;
				}
			}
			if (with_cigar) P[(size_t)r * n_col_ * 16 + (t - st)] = d;
		}
		/* extz2 reads u/v through uint8_t pointers and subtracts q+e; extd2 through int8_t */
#define VV(i) (dual ? (int32_t)(int8_t)V[i] : (int32_t)V[i] - qe)
#define UU(i) (dual ? (int32_t)(int8_t)U[i] : (int32_t)U[i] - qe)
		if (!approx_max) { /* exact max (extz2:216-261, extd2:315-368) */
			int32_t max_H, max_t;
			if (r > 0) {
				int32_t lH[4], lt[4], en1 = st0 + (en0 - st0) / 4 * 4, i;
				max_H = H[en0] = en0 > 0 ? H[en0 - 1] + UU(en0) : H[en0] + VV(en0);
				max_t = en0;
				for (i = 0; i < 4; ++i) lH[i] = max_H, lt[i] = max_t;
				for (t = st0; t < en1; t += 4) /* four int32 lanes, strictly-greater update */
					for (i = 0; i < 4; ++i) {
						H[t + i] += VV(t + i);
						if (H[t + i] > lH[i]) lH[i] = H[t + i], lt[i] = t;
					}
				for (i = 0; i < 4; ++i)
					if (max_H < lH[i]) max_H = lH[i], max_t = lt[i] + i;
				for (; t < en0; ++t) {
					H[t] += VV(t);
					if (H[t] > max_H) max_H = H[t], max_t = t;
				}
			} else H[0] = VV(0) - qe, max_H = H[0], max_t = 0;
			if (en0 == tlen - 1 && H[en0] > ez->mte) ez->mte = H[en0], ez->mte_q = r - en0;
			if (r - st0 == qlen - 1 && H[st0] > ez->mqe) ez->mqe = H[st0], ez->mqe_t = st0;
			if (apply_zdrop(ez, max_H, r, max_t, zdrop, dual ? e2 : e)) break;
			if (r == qlen + tlen - 2 && en0 == tlen - 1) ez->score = H[tlen - 1];
			if (dual) {
				if (flag & F_EXTZ_ONLY) { /* early stop, extd2:361-367 */
					int32_t rH = last_max_H > max_H ? last_max_H : max_H;
					int32_t rq = qlen - (r - st0), rt = tlen - en0;
					int32_t rm = rq >= tlen - st0 ? tlen - st0 : rt >= qlen - (r - en0) ? qlen - (r - en0) : tlen + qlen - 1 - r;
					if (rH + rm * max_sc + end_bonus < (int)ez->max) break;
				}
				last_max_H = max_H;
			}
		} else { /* approximate max (extz2:262-278, extd2:369-385) */
			if (r > 0) {
				if (last_H0_t >= st0 && last_H0_t <= en0 && last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0) {
					int32_t d0 = VV(last_H0_t), d1 = UU(last_H0_t + 1);
					if (d0 > d1) H0 += d0;
					else H0 += d1, ++last_H0_t;
				} else if (last_H0_t >= st0 && last_H0_t <= en0) {
					H0 += VV(last_H0_t);
				} else {
					++last_H0_t, H0 += UU(last_H0_t);
				}
				if (!dual && (flag & F_APPROX_DROP) && apply_zdrop(ez, H0, r, last_H0_t, zdrop, e)) break;
			} else H0 = VV(0) - qe, last_H0_t = 0;
			if (dual && (flag & F_APPROX_DROP) && apply_zdrop(ez, H0, r, last_H0_t, zdrop, e2)) break;
			if (r == qlen + tlen - 2 && en0 == tlen - 1) ez->score = H0;
		}
#undef VV
#undef UU
		last_st = st, last_en = en;
	}
	free(mem);
	free(H);
	if (with_cigar) { /* backtrack selection, extz2:284-295 */
		int rev = !!(flag & F_REV_CIGAR);
		if (!ez->zdropped && !(flag & F_EXTZ_ONLY)) {
			backtrack_rot(rev, P, off, off_end, n_col_ * 16, tlen - 1, qlen - 1, &ez->m_cigar, &ez->n_cigar, &ez->cigar);
		} else if ((flag & F_EXTZ_ONLY) && ez->mqe + end_bonus > (int)ez->max) {
			ez->reach_end = 1;
			backtrack_rot(rev, P, off, off_end, n_col_ * 16, ez->mqe_t, qlen - 1, &ez->m_cigar, &ez->n_cigar, &ez->cigar);
		} else if (ez->max_t >= 0 && ez->max_q >= 0) {
			backtrack_rot(rev, P, off, off_end, n_col_ * 16, ez->max_t, ez->max_q, &ez->m_cigar, &ez->n_cigar, &ez->cigar);
		}
		free(P);
		free(off);
	}
}

void orc_extz2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m, const int8_t *mat,
			   int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, orc_extz_t *ez, orc_stats_t *st)
{
	ext_core(0, qlen, query, tlen, target, m, mat, q, e, q, e, w, zdrop, end_bonus, flag, ez, st);
}

void orc_extd2(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m, const int8_t *mat,
			   int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus, int flag,
			   orc_extz_t *ez, orc_stats_t *st)
{
	ext_core(1, qlen, query, tlen, target, m, mat, q, e, q2, e2, w, zdrop, end_bonus, flag, ez, st);
}

/* ================= local Smith-Waterman, ksw2_ll_sse.c ================= */

typedef struct {
	int qlen, slen, rows;
	uint8_t shift, mdiff, max, size;
	u8 *qp, *H0, *H1, *E, *Hmax; /* each segment is 16 bytes (16 u8 lanes or 8 i16 lanes) */
} orc_kswq_t;

/* ksw_ll_qinit, ksw2_ll_sse.c:50-97.  One malloc block, released with free(). */
void *orc_ll_qinit(int size, int qlen, const uint8_t *query, int m, const int8_t *mat)
{
	orc_kswq_t *q;
	int slen, a, p;
	size = size > 1 ? 2 : 1;
	p = 8 * (3 - size);
	slen = (qlen + p - 1) / p;
	q = (orc_kswq_t *)malloc(sizeof(orc_kswq_t) + 16 * (size_t)slen * (m + 4) + 16);
	q->qp = (u8 *)(q + 1);
	q->H0 = q->qp + (size_t)slen * m * 16;
	q->H1 = q->H0 + slen * 16;
	q->E = q->H1 + slen * 16;
	q->Hmax = q->E + slen * 16;
	q->slen = slen, q->qlen = qlen, q->size = (uint8_t)size, q->rows = 0;
	q->shift = 127, q->mdiff = 0;
	for (a = 0; a < m * m; ++a) {
		if (mat[a] < (int8_t)q->shift) q->shift = (uint8_t)mat[a];
		if (mat[a] > (int8_t)q->mdiff) q->mdiff = (uint8_t)mat[a];
	}
	q->max = q->mdiff;
	q->shift = (uint8_t)(256 - q->shift);
	q->mdiff = (uint8_t)(q->mdiff + q->shift);
	for (a = 0; a < m; ++a) { /* striped profile: lane l of segment i holds query position i + l*slen */
		int i, l;
		const int8_t *ma = mat + a * m;
		for (i = 0; i < slen; ++i)
			for (l = 0; l < p; ++l) {
				int k = i + l * slen, v = k >= qlen ? -1 : ma[query[k]];
				if (size == 1) q->qp[((size_t)a * slen + i) * 16 + l] = (u8)(v + q->shift);
				else ((int16_t *)q->qp)[((size_t)a * slen + i) * 8 + l] = (int16_t)v;
			}
	}
	return q;
}

int orc_ll_rows(const void *qp) { return ((const orc_kswq_t *)qp)->rows; }

/* second-best bookkeeping of ksw2_ll_sse.c:188-193 / 300-305 */
typedef struct { int n, m; uint64_t *a; } blist_t;
static void blist_add(blist_t *b, int imax, int i)
{
	if (b->n == 0 || (int32_t)b->a[b->n - 1] + 1 != i) {
		if (b->n == b->m) {
			b->m = b->n + 1;
			b->m += (b->m >> 1) + 16;
			b->a = (uint64_t *)realloc(b->a, (size_t)b->m * sizeof(uint64_t));
		}
		b->a[b->n++] = (uint64_t)imax << 32 | (uint32_t)i;
	} else if ((int)(b->a[b->n - 1] >> 32) < imax) b->a[b->n - 1] = (uint64_t)imax << 32 | (uint32_t)i;
}

static void blist_score2(const blist_t *b, int score, int maxsc, int te, orc_llrst_t *r)
{
	int i, c, low, high;
	if (!b->a) return;
	c = maxsc > 0 ? (score + maxsc - 1) / maxsc : 0; /* the reference divides by q->max unguarded */
	low = te - c, high = te + c;
	for (i = 0; i < b->n; ++i) {
		int e = (int32_t)b->a[i];
		if ((e < low || e > high) && (int)(b->a[i] >> 32) > r->score2) r->score2 = (int)(b->a[i] >> 32), r->te2 = e;
	}
}

/* ksw_ll_u8_core, ksw2_ll_sse.c:121-222: 16 unsigned saturating byte lanes */
orc_llrst_t orc_ll_u8_core(void *q_, int tlen, const uint8_t *target, int gapo, int gape, int xtra)
{
	orc_kswq_t *q = (orc_kswq_t *)q_;
	int slen = q->slen, i, j, l, te = -1, gmax = 0, minsc, endsc;
	u8 goe = (u8)(gapo + gape), ge = (u8)gape, sh = q->shift;
	u8 *H0 = q->H0, *H1 = q->H1, *E = q->E, *Hmax = q->Hmax;
	blist_t b = {0, 0, 0};
	orc_llrst_t r = {0, -1, -1, -1, -1};
	minsc = (xtra & F_LL_SUBO) ? xtra & 0xffff : 0x10000;
	endsc = (xtra & F_LL_STOP) ? xtra & 0xffff : 0x10000;
	memset(E, 0, slen * 16), memset(H0, 0, slen * 16), memset(Hmax, 0, slen * 16);
	q->rows = 0;
	for (i = 0; i < tlen; ++i) {
		u8 f[16], mx[16], h[16];
		const u8 *S = q->qp + (size_t)target[i] * slen * 16;
		int imax, k;
		q->rows = i + 1;
		for (l = 0; l < 16; ++l) f[l] = mx[l] = 0;
		h[0] = 0; /* lane shift of the last segment of the previous row */
		for (l = 1; l < 16; ++l) h[l] = H0[(slen - 1) * 16 + l - 1];
		for (j = 0; j < slen; ++j) {
			for (l = 0; l < 16; ++l) {
				u8 hv = bu_subs(bu_adds(h[l], S[j * 16 + l]), sh), ev = E[j * 16 + l];
				hv = bu_max(hv, ev);
				hv = bu_max(hv, f[l]);
				mx[l] = bu_max(mx[l], hv);
				H1[j * 16 + l] = hv;
				E[j * 16 + l] = bu_max(bu_subs(ev, ge), bu_subs(hv, goe));
				f[l] = bu_max(bu_subs(f[l], ge), bu_subs(hv, goe));
				h[l] = H0[j * 16 + l];
			}
		}
		for (k = 0; k < 16; ++k) { /* lazy-F, ksw2_ll_sse.c:175-185 */
			for (l = 15; l > 0; --l) f[l] = f[l - 1];
			f[0] = 0;
			for (j = 0; j < slen; ++j) {
				int all_le = 1;
				for (l = 0; l < 16; ++l) {
					u8 hv = bu_max(H1[j * 16 + l], f[l]);
					H1[j * 16 + l] = hv;
					hv = bu_subs(hv, goe);
					f[l] = bu_subs(f[l], ge);
					if (bu_subs(f[l], hv) != 0) all_le = 0;
				}
				if (all_le) goto end_lazy;
			}
		}
end_lazy:
		for (l = 0, imax = 0; l < 16; ++l) imax = imax > mx[l] ? imax : mx[l];
		if (imax >= minsc) blist_add(&b, imax, i);
		if (imax > gmax) {
			gmax = imax, te = i;
			memcpy(Hmax, H1, slen * 16);
			if (gmax + sh >= 255 || gmax >= endsc) break;
		}
		{ u8 *tmp = H1; H1 = H0; H0 = tmp; }
	}
	r.score = gmax + sh < 255 ? gmax : 255;
	r.te = te;
	if (r.score != 255) { /* query end and second best, ksw2_ll_sse.c:204-218 */
		int mx = -1, tmp, n = slen * 16;
		for (i = 0; i < n; ++i) {
			if ((int)Hmax[i] > mx) mx = Hmax[i], r.qe = i / 16 + i % 16 * slen;
			else if ((int)Hmax[i] == mx && (tmp = i / 16 + i % 16 * slen) < r.qe) r.qe = tmp;
		}
		blist_score2(&b, r.score, q->max, te, &r);
	}
	free(b.a);
	return r;
}

static inline int16_t s16_adds(int16_t a, int16_t b)
{
	int s = (int)a + b;
	return (int16_t)(s > 32767 ? 32767 : s < -32768 ? -32768 : s);
}
static inline int16_t u16_subs(int16_t a, int16_t b)
{
	uint16_t x = (uint16_t)a, y = (uint16_t)b;
	return (int16_t)(x > y ? (uint16_t)(x - y) : 0);
}
static inline int16_t s16_max(int16_t a, int16_t b) { return a > b ? a : b; }

/* ksw_ll_i16_core, ksw2_ll_sse.c:245-333: 8 signed 16-bit lanes */
orc_llrst_t orc_ll_i16_core(void *q_, int tlen, const uint8_t *target, int gapo, int gape, int xtra)
{
	orc_kswq_t *q = (orc_kswq_t *)q_;
	int slen = q->slen, i, j, l, te = -1, gmax = 0, minsc, endsc;
	int16_t goe = (int16_t)(gapo + gape), ge = (int16_t)gape;
	int16_t *H0 = (int16_t *)q->H0, *H1 = (int16_t *)q->H1, *E = (int16_t *)q->E, *Hmax = (int16_t *)q->Hmax;
	const int16_t *qp = (const int16_t *)q->qp;
	blist_t b = {0, 0, 0};
	orc_llrst_t r = {0, -1, -1, -1, -1};
	minsc = (xtra & F_LL_SUBO) ? xtra & 0xffff : 0x10000;
	endsc = (xtra & F_LL_STOP) ? xtra & 0xffff : 0x10000;
	memset(E, 0, slen * 16), memset(H0, 0, slen * 16), memset(Hmax, 0, slen * 16);
	q->rows = 0;
	for (i = 0; i < tlen; ++i) {
		int16_t f[8], mx[8], h[8];
		const int16_t *S = qp + (size_t)target[i] * slen * 8;
		int imax, k;
		q->rows = i + 1;
		for (l = 0; l < 8; ++l) f[l] = mx[l] = 0;
		h[0] = 0;
		for (l = 1; l < 8; ++l) h[l] = H0[(slen - 1) * 8 + l - 1];
		for (j = 0; j < slen; ++j) {
			for (l = 0; l < 8; ++l) {
				int16_t hv = s16_adds(h[l], S[j * 8 + l]), ev = E[j * 8 + l];
				hv = s16_max(hv, ev);
				hv = s16_max(hv, f[l]);
				mx[l] = s16_max(mx[l], hv);
				H1[j * 8 + l] = hv;
				E[j * 8 + l] = s16_max(u16_subs(ev, ge), u16_subs(hv, goe));
				f[l] = s16_max(u16_subs(f[l], ge), u16_subs(hv, goe));
				h[l] = H0[j * 8 + l];
			}
		}
		for (k = 0; k < 16; ++k) { /* lazy-F, ksw2_ll_sse.c:287-297 */
			for (l = 7; l > 0; --l) f[l] = f[l - 1];
			f[0] = 0;
			for (j = 0; j < slen; ++j) {
				int any_gt = 0;
				for (l = 0; l < 8; ++l) {
					int16_t hv = s16_max(H1[j * 8 + l], f[l]);
					H1[j * 8 + l] = hv;
					hv = u16_subs(hv, goe);
					f[l] = u16_subs(f[l], ge);
					if (f[l] > hv) any_gt = 1;
				}
				if (!any_gt) goto end_lazy;
			}
		}
end_lazy:
		for (l = 0, imax = -32768; l < 8; ++l) imax = imax > mx[l] ? imax : mx[l];
		if (imax >= minsc) blist_add(&b, imax, i);
		if (imax > gmax) {
			gmax = imax, te = i;
			memcpy(Hmax, H1, slen * 16);
			if (gmax >= endsc) break;
		}
		{ int16_t *tmp = H1; H1 = H0; H0 = tmp; }
	}
	r.score = gmax, r.te = te;
	{
		int mx = -1, tmp, n = slen * 8;
		const uint16_t *hm = (const uint16_t *)Hmax;
		for (i = 0, r.qe = -1; i < n; ++i) {
			if ((int)hm[i] > mx) mx = hm[i], r.qe = i / 8 + i % 8 * slen;
			else if ((int)hm[i] == mx && (tmp = i / 8 + i % 8 * slen) < r.qe) r.qe = tmp;
		}
		blist_score2(&b, r.score, q->max, te, &r);
	}
	free(b.a);
	return r;
}

int orc_ll_i16(void *qp, int tlen, const uint8_t *target, int gapo, int gape, int *qe, int *te)
{
	orc_llrst_t r = orc_ll_i16_core(qp, tlen, target, gapo, gape, 0);
	*qe = r.qe, *te = r.te;
	return r.score;
}

/* ksw_gen_nt4_mat, ksw2.h:199-219 */
void orc_gen_nt4_mat(int8_t *mat, int8_t a, int8_t b, int8_t b_ts, int8_t b_ambi, int32_t mt)
{
	const int m = 5;
	int i, j;
	a = a < 0 ? -a : a;
	b = b > 0 ? -b : b;
	b_ambi = b_ambi > 0 ? -b_ambi : b_ambi;
	for (i = 0; i < m - 1; ++i) {
		for (j = 0; j < m - 1; ++j) mat[i * m + j] = i == j ? a : b;
		mat[i * m + m - 1] = b_ambi;
	}
	for (j = 0; j < m; ++j) mat[(m - 1) * m + j] = b_ambi;
	if (b_ts != 0 && b_ts != b) {
		b_ts = b_ts > 0 ? -b_ts : b_ts;
		mat[0 * m + 2] = mat[1 * m + 3] = mat[2 * m + 0] = mat[3 * m + 1] = b_ts;
	}
	if (mt == 1) mat[1 * m + 3] = a;
	else if (mt == 2) mat[2 * m + 0] = a;
}

/* l2b_getseq (l2bit.c:52-77) on the l2b arrays, then l2b_meth_convert (l2bit.c:79-90) and
 * the callers' in-place reversal (mb_seq_rev); flags: 1 reverse, 2 C2T, 4 G2A.  The window
 * [st, st+len) must lie inside contig tid. */
void orc_l2b_getseq(const uint64_t *pac, const uint64_t *ctg_off, int64_t n_ambi, const uint64_t *ambi, int64_t tid,
					int64_t st, int64_t len, int flags, uint8_t *seq)
{
	uint64_t g0 = ctg_off[tid] + (uint64_t)st, i;
	int64_t a, p;
	for (i = 0; i < (uint64_t)len; ++i) {
		uint64_t g = g0 + i;
		seq[i] = (uint8_t)(pac[g >> 5] >> ((g & 31) << 1) & 3);
	}
	for (a = 0; a < n_ambi; ++a) { /* N runs overlapping the window */
		uint64_t s = ambi[2 * a] > g0 ? ambi[2 * a] : g0;
		uint64_t e = ambi[2 * a + 1] < g0 + (uint64_t)len ? ambi[2 * a + 1] : g0 + (uint64_t)len;
		for (i = s; i < e; ++i) seq[i - g0] = 4;
	}
	if (flags & 2) { for (p = 0; p < len; ++p) if (seq[p] == 1) seq[p] = 3; }
	else if (flags & 4) { for (p = 0; p < len; ++p) if (seq[p] == 2) seq[p] = 0; }
	if (flags & 1) {
		for (p = 0; p < len / 2; ++p) {
			uint8_t t = seq[p];
			seq[p] = seq[len - 1 - p], seq[len - 1 - p] = t;
		}
	}
}

/* mb_ungap (pe.c:209-247): the 7-mer Hough transform that pe.c's mate rescue runs before
 * ksw_ll.  Every k-mer of the query (bases after the methylation table of mt: 0 none, 1 C2T,
 * 2 G2A) records the last query position where it ends; every k-mer of the target that the
 * query holds votes for the diagonal i - h[x].  Returns the top vote count; *max_i is its
 * first diagonal, *n_good the diagonals with more than half of it, *n_kmer the distinct
 * query k-mers. */
int orc_ungap(int qlen, const uint8_t *qseq, int tlen, const uint8_t *tseq, int kmer, int mt, int *max_i,
			  int *n_good, int *n_kmer)
{
	static const uint8_t c2t[4] = {0, 3, 2, 3}, g2a[4] = {0, 1, 0, 3};
	int i, l, cap = 1 << kmer * 2, mask = cap - 1, max;
	int32_t *a;
	uint16_t *h, x;
	*max_i = -1, *n_good = *n_kmer = 0;
	if (qlen >= 65535) return 0;
	a = (int32_t *)calloc(tlen > 0 ? tlen : 1, sizeof(int32_t));
	h = (uint16_t *)calloc(cap, sizeof(uint16_t));
	for (i = l = 0, x = 0; i < qlen; ++i) {
		if (qseq[i] < 4) {
			uint8_t c = mt == 1 ? c2t[qseq[i]] : mt == 2 ? g2a[qseq[i]] : qseq[i];
			x = (uint16_t)((x << 2 | c) & mask);
			if (++l >= kmer) {
				if (h[x] == 0) ++*n_kmer;
				h[x] = (uint16_t)i;
			}
		} else x = 0, l = 0;
	}
	for (i = l = 0, x = 0; i < tlen; ++i) {
		if (tseq[i] < 4) {
			uint8_t c = mt == 1 ? c2t[tseq[i]] : mt == 2 ? g2a[tseq[i]] : tseq[i];
			x = (uint16_t)((x << 2 | c) & mask);
			if (++l >= kmer && h[x] > 0 && i >= h[x]) ++a[i - h[x]];
		} else x = 0, l = 0;
	}
	for (i = 0, max = 0; i < tlen; ++i)
		if (max < a[i]) max = a[i], *max_i = i;
	for (i = 0, *n_good = 0; i < tlen; ++i)
		if (a[i] > max >> 1) ++*n_good;
	free(h);
	free(a);
	return max;
}
