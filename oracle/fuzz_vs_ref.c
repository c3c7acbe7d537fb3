/*
 * fuzz_vs_ref.c -- differential fuzzer: scalar restatement vs the reference
 * SSE code (TEST INFRASTRUCTURE ONLY; built by `make fuzz` where the reference
 * tree is present).
 *
 * usage: fuzz_vs_ref <n_cases> <seed> [kind]    kind: all|ext|ll
 * Prints the first mismatch and exits 1, or prints a summary and exits 0.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "ksw2.h"
#include "ksw2_oracle.h"

static uint64_t rng_s;
static uint64_t sm64(void) /* splitmix64 */
{
	uint64_t z = (rng_s += 0x9e3779b97f4a7c15ULL);
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
	return z ^ (z >> 31);
}
static int rint_(int lo, int hi) { return lo + (int)(sm64() % (uint64_t)(hi - lo + 1)); }
static double runif(void) { return (sm64() >> 11) * (1.0 / 9007199254740992.0); }

static void gen_pair(int *qlen, uint8_t *q, int *tlen, uint8_t *t, int maxlen, int m)
{
	int i, k, mode = rint_(0, 3), ql, tl = 0;
	double sub = runif() * 0.15, ind = runif() * 0.08, pn = runif() < 0.3 ? runif() * 0.05 : 0;
	ql = rint_(1, maxlen);
	for (i = 0; i < ql; ++i) q[i] = runif() < pn ? (uint8_t)(m - 1) : (uint8_t)rint_(0, m - 2);
	if (mode == 0) { /* unrelated */
		tl = rint_(1, maxlen);
		for (i = 0; i < tl; ++i) t[i] = runif() < pn ? (uint8_t)(m - 1) : (uint8_t)rint_(0, m - 2);
	} else { /* mutated copy + flank */
		for (i = 0; i < ql && tl < 2 * maxlen; ++i) {
			double u = runif();
			if (u < ind / 2) { /* deletion from target */
				i += rint_(0, 4);
			} else if (u < ind) { /* insertion into target */
				int l = rint_(1, 5);
				for (k = 0; k < l && tl < 2 * maxlen; ++k) t[tl++] = (uint8_t)rint_(0, m - 2);
				t[tl++] = q[i];
			} else if (runif() < sub) t[tl++] = (uint8_t)rint_(0, m - 1);
			else t[tl++] = q[i];
		}
		if (mode >= 2) {
			int fl = rint_(0, 40);
			for (k = 0; k < fl && tl < 2 * maxlen + 40; ++k) t[tl++] = (uint8_t)rint_(0, m - 2);
		}
		if (tl == 0) t[tl++] = 0;
	}
	*qlen = ql, *tlen = tl;
}

static int cmp_ez(const ksw_extz_t *a, const orc_extz_t *b)
{
	if (a->max != b->max || a->zdropped != b->zdropped || a->max_q != b->max_q || a->max_t != b->max_t) return 1;
	if (a->mqe != b->mqe || a->mqe_t != b->mqe_t || a->mte != b->mte || a->mte_q != b->mte_q) return 2;
	if (a->score != b->score || a->reach_end != b->reach_end || a->n_cigar != b->n_cigar) return 3;
	if (a->m_cigar != b->m_cigar) return 4;
	if (a->n_cigar > 0 && memcmp(a->cigar, b->cigar, a->n_cigar * 4) != 0) return 5;
	return 0;
}

int main(int argc, char *argv[])
{
	long n = argc > 1 ? atol(argv[1]) : 10000, it, n_ext = 0, n_ll = 0, n_cig = 0;
	const char *kind = argc > 3 ? argv[3] : "all";
	uint8_t *q = malloc(8192), *t = malloc(8192);
	int8_t mat[25 * 25];
	rng_s = argc > 2 ? strtoull(argv[2], 0, 10) : 11;
	for (it = 0; it < n; ++it) {
		int ql, tl, m = 5, i, do_ll;
		int maxlen = runif() < 0.7 ? rint_(1, 40) : rint_(41, 600);
		do_ll = strcmp(kind, "ll") == 0 ? 1 : strcmp(kind, "ext") == 0 ? 0 : (runif() < 0.3);
		if (runif() < 0.1) m = rint_(2, 8);
		gen_pair(&ql, q, &tl, t, maxlen, m);
		if (!do_ll) {
			ksw_extz_t ez1;
			orc_extz_t ez2;
			int8_t a = (int8_t)rint_(1, 6), b = (int8_t)rint_(1, 12), qo = (int8_t)rint_(0, 30), ge = (int8_t)rint_(1, 6);
			int8_t qo2 = (int8_t)rint_(0, 50), ge2 = (int8_t)rint_(1, 6);
			int w = runif() < 0.15 ? -1 : rint_(0, 200), zdrop = runif() < 0.2 ? -1 : rint_(0, 300);
			int end_bonus = runif() < 0.3 ? -1 : rint_(0, 30), flag = 0, dual = runif() < 0.5, rc;
			if (m == 5) orc_gen_nt4_mat(mat, a, b, (int8_t)(runif() < 0.2 ? rint_(1, 12) : 0), (int8_t)rint_(0, 3), runif() < 0.1 ? rint_(1, 2) : 0);
			else for (i = 0; i < m * m; ++i) mat[i] = (i / m == i % m) ? a : -b;
			if (runif() < 0.05) mat[m * m - 1] = 0;
			if (runif() < 0.3) flag |= KSW_EZ_SCORE_ONLY;
			if (runif() < 0.4) flag |= KSW_EZ_RIGHT;
			if (runif() < 0.2) flag |= KSW_EZ_GENERIC_SC;
			if (runif() < 0.2) flag |= KSW_EZ_APPROX_MAX;
			if (runif() < 0.2) flag |= KSW_EZ_APPROX_DROP;
			if (runif() < 0.6) flag |= KSW_EZ_EXTZ_ONLY;
			if (runif() < 0.3) flag |= KSW_EZ_REV_CIGAR;
			memset(&ez1, 0, sizeof(ez1));
			memset(&ez2, 0, sizeof(ez2));
			if (runif() < 0.3) { /* caller-provided CIGAR buffer, as pe.c:435-437 does */
				ez1.m_cigar = ez2.m_cigar = 16;
				ez1.cigar = malloc(64), ez2.cigar = malloc(64);
			}
			if (!dual) {
				ksw_extz2_sse(0, ql, q, tl, t, (int8_t)m, mat, qo, ge, w, zdrop, end_bonus, flag, &ez1);
				orc_extz2(ql, q, tl, t, (int8_t)m, mat, qo, ge, w, zdrop, end_bonus, flag, &ez2, 0);
			} else {
				ksw_extd2_sse(0, ql, q, tl, t, (int8_t)m, mat, qo, ge, qo2, ge2, w, zdrop, end_bonus, flag, &ez1);
				orc_extd2(ql, q, tl, t, (int8_t)m, mat, qo, ge, qo2, ge2, w, zdrop, end_bonus, flag, &ez2, 0);
			}
			rc = cmp_ez(&ez1, &ez2);
			if (rc) {
				printf("MISMATCH(ext,%d) it=%ld dual=%d qlen=%d tlen=%d m=%d q=%d e=%d q2=%d e2=%d w=%d zdrop=%d eb=%d flag=0x%x\n",
					   rc, it, dual, ql, tl, m, qo, ge, qo2, ge2, w, zdrop, end_bonus, flag);
				printf(" ref: max=%u zd=%u mq=%d mt=%d mqe=%d/%d mte=%d/%d score=%d re=%d n=%d\n", ez1.max, ez1.zdropped, ez1.max_q, ez1.max_t, ez1.mqe, ez1.mqe_t, ez1.mte, ez1.mte_q, ez1.score, ez1.reach_end, ez1.n_cigar);
				printf(" orc: max=%u zd=%u mq=%d mt=%d mqe=%d/%d mte=%d/%d score=%d re=%d n=%d\n", ez2.max, ez2.zdropped, ez2.max_q, ez2.max_t, ez2.mqe, ez2.mqe_t, ez2.mte, ez2.mte_q, ez2.score, ez2.reach_end, ez2.n_cigar);
				return 1;
			}
			n_ext++;
			n_cig += ez1.n_cigar > 0;
			free(ez1.cigar);
			free(ez2.cigar);
		} else {
			int sz = runif() < 0.5 ? 1 : 2, xtra = 0, go = rint_(0, 12), ge = rint_(1, 4), qe1, te1, s1, qe2, te2, s2;
			void *qp1, *qp2;
			ksw_llrst_t r1;
			orc_llrst_t r2;
			int8_t a = (int8_t)rint_(1, 4), b = (int8_t)rint_(1, 10);
			if (m == 5) orc_gen_nt4_mat(mat, a, b, 0, (int8_t)rint_(0, 3), 0);
			else for (i = 0; i < m * m; ++i) mat[i] = (i / m == i % m) ? a : -b;
			if (runif() < 0.5) xtra |= KSW_LL_SUBO | rint_(0, 40);
			if (runif() < 0.2) xtra |= KSW_LL_STOP | rint_(1, 200);
			qp1 = ksw_ll_qinit(0, sz, ql, q, m, mat);
			qp2 = orc_ll_qinit(sz, ql, q, m, mat);
			if (runif() < 0.2 && sz == 2) {
				s1 = ksw_ll_i16(qp1, tl, t, go, ge, &qe1, &te1);
				s2 = orc_ll_i16(qp2, tl, t, go, ge, &qe2, &te2);
				if (s1 != s2 || qe1 != qe2 || te1 != te2) {
					printf("MISMATCH(ll_i16) it=%ld qlen=%d tlen=%d go=%d ge=%d: ref %d/%d/%d orc %d/%d/%d\n", it, ql, tl, go, ge, s1, qe1, te1, s2, qe2, te2);
					return 1;
				}
			} else {
				if (sz == 1) r1 = ksw_ll_u8_core(qp1, tl, t, go, ge, xtra), r2 = orc_ll_u8_core(qp2, tl, t, go, ge, xtra);
				else r1 = ksw_ll_i16_core(qp1, tl, t, go, ge, xtra), r2 = orc_ll_i16_core(qp2, tl, t, go, ge, xtra);
				if (r1.score != r2.score || r1.te != r2.te || r1.qe != r2.qe || r1.score2 != r2.score2 || r1.te2 != r2.te2) {
					printf("MISMATCH(ll sz=%d) it=%ld qlen=%d tlen=%d go=%d ge=%d xtra=0x%x: ref %d/%d/%d/%d/%d orc %d/%d/%d/%d/%d\n", sz, it, ql, tl, go, ge, xtra,
						   r1.score, r1.te, r1.qe, r1.score2, r1.te2, r2.score, r2.te, r2.qe, r2.score2, r2.te2);
					return 1;
				}
			}
			free(qp1);
			free(qp2);
			n_ll++;
		}
	}
	printf("OK ext=%ld (with cigar %ld) ll=%ld\n", n_ext, n_cig, n_ll);
	return 0;
}
