// ksw2g.h -- device-side job / result layouts shared by the CUDA kernels and
// the host library.  The public C ABI lives in include/ksw2_gb300.h; these
// structs are the same bytes.
#pragma once
#include <stdint.h>

#define KSW2G_NEG_INF (-0x40000000)

// ksw2.h:8-22
#define KSW2G_SCORE_ONLY  0x01
#define KSW2G_RIGHT       0x02
#define KSW2G_GENERIC_SC  0x04
#define KSW2G_APPROX_MAX  0x08
#define KSW2G_APPROX_DROP 0x10
#define KSW2G_EXTZ_ONLY   0x40
#define KSW2G_REV_CIGAR   0x80
#define KSW2G_LL_STOP     0x20000
#define KSW2G_LL_SUBO     0x40000

// One extension job.  qoff/toff index the device sequence arena, where every
// sequence starts 16-byte aligned with at least 32 zero bytes on each side.
struct ksw2g_job {
  int64_t qoff, toff;
  int32_t qlen, tlen;
  int32_t w, zdrop, end_bonus, flag;
};

// Result of one extension job: the ksw_extz_t fields (ksw2.h:36-45) plus
// work counters and the CIGAR location in the output arena.
struct ksw2g_ext_result {
  int32_t score, max, max_q, max_t, mqe, mqe_t, mte, mte_q;
  int32_t zdropped, reach_end, n_cigar, n_diag;
  int64_t cigar_off;
  int64_t cells;
};

// Per-job hand-off from the DP kernel to the backtrack kernel.
struct ksw2g_bt {
  int32_t i0, j0;     // backtrack start (target, query); i0 < 0: none
  int32_t n_rows;     // anti-diagonals whose traceback rows were written
  int32_t pad;
};

// Scoring constants of one batch, derived on the host exactly as the
// reference derives them at the top of ksw_extz2_sse / ksw_extd2_sse.
struct ksw2g_ext_params {
  int32_t dual;                 // 0: extz2, 1: extd2
  int32_t m;
  int32_t q, e, q2, e2;         // after the extd2 swap (ksw2_extd2_sse.c:70)
  int32_t qe_scalar;            // q+e as declared before the swap (only H at r == 0)
  int32_t max_sc, min_sc;
  int32_t skip_all;             // -min_sc > 2(q+e): every job returns right after reset
  int32_t long_thres, long_diff;
  uint32_t c_q, c_q2, c_qe, c_qe2, c_mch, c_mis, c_N, c_m1, c_maxsc;  // byte constants
  int8_t mat[256];              // m*m scores (m <= 16 for GENERIC_SC on device)
};

// The device table may list jobs in any order: `slot` is the job's index in the
// results and the second-best lists (the host orders the table by query length).
struct ksw2g_ll_job {
  int64_t qoff, toff;
  int32_t qlen, tlen;
  int32_t xtra, slot;
};

struct ksw2g_ll_result {
  int32_t score, te, qe, score2, te2, rows;
};
