/*
 * ksw2.h -- drop-in C interface of the GB300 implementation of minibwa's ksw2
 * hot path.  Link libksw2gpu.so in place of ksw2_extz2_sse.o,
 * ksw2_extd2_sse.o and ksw2_ll_sse.o.
 *
 * This header declares only the six entry points the library replaces and
 * the types and flags they take.  It is not a substitute for minibwa's own
 * ksw2.h: callers (align.c, pe.c) keep compiling against that file, whose
 * static inline helpers (ksw_push_cigar, ksw_backtrack, ksw_reset_extz,
 * ksw_apply_zdrop, ksw_gen_nt4_mat) and further flags (KSW_CIGAR_N_SKIP,
 * KSW_EZ_SPLICE_*, KSW_SPSC_OFFSET) stay compiled into them.
 *
 * Every declaration below has the signature, argument meaning and result
 * layout of the reference declaration it replaces (reference file ksw2.h).
 * Each call runs on the calling thread's CUDA stream on the current device
 * and returns when its result is in host memory.  CUDA errors on this
 * per-call path are fatal (message on stderr, then abort()), matching the
 * reference's panic-on-failure convention.  There is no CPU code path.
 */
#ifndef KSW2_H_
#define KSW2_H_

#include <stdint.h>

#define KSW_NEG_INF -0x40000000

#define KSW_EZ_SCORE_ONLY  0x01 /* ksw2.h:8 */
#define KSW_EZ_RIGHT       0x02
#define KSW_EZ_GENERIC_SC  0x04
#define KSW_EZ_APPROX_MAX  0x08
#define KSW_EZ_APPROX_DROP 0x10
#define KSW_EZ_EXTZ_ONLY   0x40
#define KSW_EZ_REV_CIGAR   0x80

#define KSW_LL_STOP  0x20000 /* ksw2.h:21 */
#define KSW_LL_SUBO  0x40000

#define KSW_CIGAR_MATCH  0
#define KSW_CIGAR_INS    1
#define KSW_CIGAR_DEL    2

#ifdef __cplusplus
extern "C" {
#endif

/* ksw2.h:36-45 */
typedef struct {
	uint32_t max:31, zdropped:1;
	int max_q, max_t;
	int mqe, mqe_t;
	int mte, mte_q;
	int score;
	int m_cigar, n_cigar;
	int reach_end;
	uint32_t *cigar;
} ksw_extz_t;

/* ksw2.h:47-51 */
typedef struct {
	int score;
	int te, qe;
	int score2, te2;
} ksw_llrst_t;

/*
 * Replaces ksw_extz2_sse (ksw2.h:73-74, ksw2_extz2_sse.c:16).  ez->cigar is
 * grown with realloc() (the reference's kmalloc family maps to libc when
 * HAVE_KALLOC is undefined, ksw2.h:117-121); km is accepted and ignored.
 */
void ksw_extz2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m, const int8_t *mat,
				   int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag, ksw_extz_t *ez);

/* Replaces ksw_extd2_sse (ksw2.h:79-80, ksw2_extd2_sse.c:27). */
void ksw_extd2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m, const int8_t *mat,
				   int8_t gapo, int8_t gape, int8_t gapo2, int8_t gape2, int w, int zdrop, int end_bonus, int flag, ksw_extz_t *ez);

/*
 * Replaces ksw_ll_qinit (ksw2.h:101, ksw2_ll_sse.c:50).  Returns one malloc()
 * block holding the query and scoring matrix; the caller releases it with
 * free() (kfree(km, qp) in the reference callers, pe.c:280, align.c:63,787).
 */
void *ksw_ll_qinit(void *km, int size, int qlen, const uint8_t *query, int m, const int8_t *mat);
/* Replaces ksw_ll_u8_core (ksw2.h:102, ksw2_ll_sse.c:121). */
ksw_llrst_t ksw_ll_u8_core(void *q, int tlen, const uint8_t *target, int gapo, int gape, int xtra);
/* Replaces ksw_ll_i16_core (ksw2.h:103, ksw2_ll_sse.c:245). */
ksw_llrst_t ksw_ll_i16_core(void *q, int tlen, const uint8_t *target, int gapo, int gape, int xtra);
/* Replaces ksw_ll_i16 (ksw2.h:104, ksw2_ll_sse.c:335). */
int ksw_ll_i16(void *q, int tlen, const uint8_t *target, int gapo, int gape, int *qe, int *te);

#ifdef __cplusplus
}
#endif
#endif
