/* trace_shim.c -- records every ksw2 call of a minibwa run (TEST INFRASTRUCTURE ONLY).
 *
 * `make trace` links the reference's own minibwa, compiled from its sources
 * where they lie, against this file in place of the ksw2 entry points: the
 * reference's ksw2 objects are compiled with their functions renamed real_*,
 * and the functions here call them and append the call's inputs and outputs to
 * the file named by $KSW2_TRACE.  The recorded calls are the DP jobs that
 * align.c and pe.c really issue (gap fills, end extensions, rescue, the
 * inversion test), replayed through the GPU library by the tests.
 *
 * Record layout (little-endian int32 words unless noted):
 *   extension (kind 1 extz2, 2 extd2):
 *     kind qlen tlen m q e q2 e2 w zdrop end_bonus flag m_cigar_in
 *     mat[m*m] (bytes) query[qlen] target[tlen] (bytes, each padded to 4)
 *     max zdropped max_q max_t mqe mqe_t mte mte_q score m_cigar n_cigar reach_end cigar[n_cigar]
 *   ksw_ll (kind 3 u8 core, 4 i16 core, 5 ksw_ll_i16):
 *     kind size qlen m tlen gapo gape xtra mat[m*m] query[qlen] target[tlen] (padded bytes)
 *     score te qe score2 te2
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ksw2.h"

void real_ksw_extz2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
						const int8_t *mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, ksw_extz_t *ez);
void real_ksw_extd2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
						const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus,
						int flag, ksw_extz_t *ez);
void *real_ksw_ll_qinit(void *km, int size, int qlen, const uint8_t *query, int m, const int8_t *mat);
ksw_llrst_t real_ksw_ll_u8_core(void *q, int tlen, const uint8_t *target, int _gapo, int _gape, int xtra);
ksw_llrst_t real_ksw_ll_i16_core(void *q, int tlen, const uint8_t *target, int _gapo, int _gape, int xtra);
int real_ksw_ll_i16(void *q, int tlen, const uint8_t *target, int _gapo, int _gape, int *qe, int *te);

static pthread_mutex_t tr_mu = PTHREAD_MUTEX_INITIALIZER;
static FILE *tr_fp;
static int tr_init;

static FILE *trace_file(void)
{
	if (!tr_init) {
		const char *fn = getenv("KSW2_TRACE");
		tr_fp = fn ? fopen(fn, "ab") : 0;
		tr_init = 1;
	}
	return tr_fp;
}

static void put_i(FILE *fp, int v) { fwrite(&v, 4, 1, fp); }
static void put_b(FILE *fp, const void *p, int n)
{
	static const char zero[4] = {0, 0, 0, 0};
	if (n > 0) fwrite(p, 1, n, fp);
	if (n & 3) fwrite(zero, 1, 4 - (n & 3), fp);
}

/* the profile a ksw_ll core call runs on: the last qinit of this thread */
static __thread struct {
	void *qp;
	int size, qlen, m;
	uint8_t *query;
	int8_t mat[256];
} ll_last;

static void put_ext(int kind, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
					const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus, int flag,
					int m_cigar_in, const ksw_extz_t *ez)
{
	FILE *fp;
	int i;
	pthread_mutex_lock(&tr_mu);
	if ((fp = trace_file()) != 0) {
		int hdr[13] = {kind, qlen, tlen, m, q, e, q2, e2, w, zdrop, end_bonus, flag, m_cigar_in};
		int out[12] = {(int)ez->max, (int)ez->zdropped, ez->max_q, ez->max_t, ez->mqe, ez->mqe_t, ez->mte, ez->mte_q,
					   ez->score, ez->m_cigar, ez->n_cigar, ez->reach_end};
		for (i = 0; i < 13; ++i) put_i(fp, hdr[i]);
		put_b(fp, mat, m * m);
		put_b(fp, query, qlen);
		put_b(fp, target, tlen);
		for (i = 0; i < 12; ++i) put_i(fp, out[i]);
		if (ez->n_cigar > 0) fwrite(ez->cigar, 4, ez->n_cigar, fp);
	}
	pthread_mutex_unlock(&tr_mu);
}

void ksw_extz2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
				   const int8_t *mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, ksw_extz_t *ez)
{
	int m0 = ez->m_cigar;
	real_ksw_extz2_sse(km, qlen, query, tlen, target, m, mat, q, e, w, zdrop, end_bonus, flag, ez);
	put_ext(1, qlen, query, tlen, target, m, mat, q, e, q, e, w, zdrop, end_bonus, flag, m0, ez);
}

void ksw_extd2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
				   const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus,
				   int flag, ksw_extz_t *ez)
{
	int m0 = ez->m_cigar;
	real_ksw_extd2_sse(km, qlen, query, tlen, target, m, mat, q, e, q2, e2, w, zdrop, end_bonus, flag, ez);
	put_ext(2, qlen, query, tlen, target, m, mat, q, e, q2, e2, w, zdrop, end_bonus, flag, m0, ez);
}

void *ksw_ll_qinit(void *km, int size, int qlen, const uint8_t *query, int m, const int8_t *mat)
{
	void *qp = real_ksw_ll_qinit(km, size, qlen, query, m, mat);
	free(ll_last.query);
	ll_last.qp = qp, ll_last.size = size, ll_last.qlen = qlen, ll_last.m = m;
	ll_last.query = (uint8_t *)malloc(qlen > 0 ? qlen : 1);
	memcpy(ll_last.query, query, qlen > 0 ? qlen : 0);
	memcpy(ll_last.mat, mat, m * m <= 256 ? m * m : 256);
	return qp;
}

static void put_ll(int kind, void *qp, int tlen, const uint8_t *target, int gapo, int gape, int xtra, ksw_llrst_t r)
{
	FILE *fp;
	int i;
	if (qp != ll_last.qp || ll_last.m * ll_last.m > 256) return;
	pthread_mutex_lock(&tr_mu);
	if ((fp = trace_file()) != 0) {
		int hdr[8] = {kind, ll_last.size, ll_last.qlen, ll_last.m, tlen, gapo, gape, xtra};
		int out[5] = {r.score, r.te, r.qe, r.score2, r.te2};
		for (i = 0; i < 8; ++i) put_i(fp, hdr[i]);
		put_b(fp, ll_last.mat, ll_last.m * ll_last.m);
		put_b(fp, ll_last.query, ll_last.qlen);
		put_b(fp, target, tlen);
		for (i = 0; i < 5; ++i) put_i(fp, out[i]);
	}
	pthread_mutex_unlock(&tr_mu);
}

ksw_llrst_t ksw_ll_u8_core(void *q, int tlen, const uint8_t *target, int _gapo, int _gape, int xtra)
{
	ksw_llrst_t r = real_ksw_ll_u8_core(q, tlen, target, _gapo, _gape, xtra);
	put_ll(3, q, tlen, target, _gapo, _gape, xtra, r);
	return r;
}

ksw_llrst_t ksw_ll_i16_core(void *q, int tlen, const uint8_t *target, int _gapo, int _gape, int xtra)
{
	ksw_llrst_t r = real_ksw_ll_i16_core(q, tlen, target, _gapo, _gape, xtra);
	put_ll(4, q, tlen, target, _gapo, _gape, xtra, r);
	return r;
}

int ksw_ll_i16(void *q, int tlen, const uint8_t *target, int _gapo, int _gape, int *qe, int *te)
{
	ksw_llrst_t r;
	r.score = real_ksw_ll_i16(q, tlen, target, _gapo, _gape, qe, te);
	r.qe = *qe, r.te = *te, r.score2 = -1, r.te2 = -1;
	put_ll(5, q, tlen, target, _gapo, _gape, 0, r);
	return r.score;
}
