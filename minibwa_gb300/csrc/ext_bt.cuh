// ext_bt.cuh -- traceback walk (ksw_backtrack, ksw2.h:140-172, rotated layout)
// and the packing of raw sequences into the padded device arena.
#pragma once
#include "ksw2g.h"

namespace ksw2g {

// padded first/last target position of anti-diagonal r (ksw2_extz2_sse.c:99-108)
__device__ __forceinline__ void band_pad(int r, int qlen, int tlen, int w, int &off, int &off_end) {
  int st = r - qlen + 1 > 0 ? r - qlen + 1 : 0;
  int en = r < tlen - 1 ? r : tlen - 1;
  const int a = (r - w + 1) >> 1, b = (r + w) >> 1;
  if (st < a) st = a;
  if (en > b) en = b;
  off = st & ~15;
  off_end = (en & ~15) + 15;
}

// One walk over the traceback from (i0, j0).  The CIGAR runs are produced last
// op first; run k (counting from the walk's start) is stored at scratch[-1-k].
// scratch is the end of the job's own traceback region: the walk reads every
// row at most once, in decreasing order, and after k runs it has left at least
// k rows of n_col_*16 >= 32 bytes behind it, so the runs only overwrite rows it
// has already passed.  Returns the number of runs.
__device__ int bt_walk(const uint8_t *tb, int ncol16, int qlen, int tlen, int w, int i0, int j0,
                       uint32_t *scratch) {
  int i = i0, j = j0, state = 0, n = 0, last_op = -1;
  uint32_t run = 0;
  auto push = [&](int op, int len) {
    if (n == 0 || op != last_op) {
      if (n > 0) scratch[-n] = run << 4 | (uint32_t)last_op;
      ++n, last_op = op, run = (uint32_t)len;
    } else run += (uint32_t)len;
  };
  while (i >= 0 && j >= 0) {
    const int r = i + j;
    int off, off_end, force = -1;
    band_pad(r, qlen, tlen, w, off, off_end);
    if (i < off) force = 2;
    if (i > off_end) force = 1;
    // a plain load: rows behind the walk are overwritten by its output
    const unsigned t = force < 0 ? tb[(size_t)r * ncol16 + (i - off)] : 0u;
    if (state == 0) state = t & 7;
    else if (!(t >> (state + 2) & 1)) state = 0;
    if (state == 0) state = t & 7;
    if (force >= 0) state = force;
    if (state == 0) push(0, 1), --i, --j;
    else if (state == 1 || state == 3) push(2, 1), --i;
    else push(1, 1), --j;
  }
  if (i >= 0) push(2, i + 1);
  if (j >= 0) push(1, j + 1);
  if (n > 0) scratch[-n] = run << 4 | (uint32_t)last_op;
  return n;
}

// One thread per job; jobs order[0..n_jobs) (all jobs when order is null).  The
// walk runs once; its runs are then copied to an exactly sized range of the
// CIGAR arena, reversed into final order unless KSW_EZ_REV_CIGAR (ksw2.h:168-170).
__global__ void ext_bt_kernel(const ksw2g_job *__restrict__ jobs, const int32_t *__restrict__ order, int n_jobs,
                              const ksw2g_bt *__restrict__ bts, uint8_t *tb_pool,
                              const int64_t *__restrict__ tb_off, ksw2g_ext_result *__restrict__ res,
                              uint32_t *__restrict__ cigar_out, unsigned long long *__restrict__ cursor,
                              long long cigar_cap, int *__restrict__ err) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= n_jobs) return;
  const int jid = order ? order[ix] : ix;
  const ksw2g_bt b = bts[jid];
  if (b.i0 < 0) {
    res[jid].n_cigar = 0;
    return;
  }
  const ksw2g_job J = jobs[jid];
  int w = J.w;
  if (w < 0) w = J.tlen > J.qlen ? J.tlen : J.qlen;
  int nc = J.qlen < J.tlen ? J.qlen : J.tlen;
  nc = ((nc < w + 1 ? nc : w + 1) + 15) / 16 + 1;
  const int rev = (J.flag & KSW2G_REV_CIGAR) ? 1 : 0;
  uint8_t *tb = tb_pool + tb_off[jid];
  // the end of row i0+j0: 16-byte aligned (rows are n_col_*16 bytes, regions 16-byte aligned)
  uint32_t *scratch = (uint32_t *)(tb + (size_t)(b.i0 + b.j0 + 1) * (nc * 16));
  const int n = bt_walk(tb, nc * 16, J.qlen, J.tlen, w, b.i0, b.j0, scratch);
  const unsigned long long o = atomicAdd(cursor, (unsigned long long)n);
  if ((long long)(o + n) > cigar_cap) {  // arena too small: report, write nothing
    atomicOr(err, 1);
    res[jid].n_cigar = -n;
    res[jid].cigar_off = -1;
    return;
  }
  uint32_t *out = cigar_out + o;
  // scratch[-1] is the last op of the final CIGAR; scratch[-n] the first
  if (rev)
    for (int k = 0; k < n; ++k) out[k] = scratch[-1 - k];
  else
    for (int k = 0; k < n; ++k) out[k] = scratch[k - n];
  res[jid].n_cigar = n;
  res[jid].cigar_off = (int64_t)o;
}

// Copy raw (unpadded, back-to-back) sequences into the padded arena:
// dst[off-32 .. off+len+32) receives 32 zero bytes, the sequence, then zeros up
// to the next 16-byte boundary plus 32.  One warp per sequence.
__global__ void pack_seqs_kernel(int n, const uint8_t *__restrict__ raw, const int64_t *__restrict__ raw_off,
                                 const int32_t *__restrict__ len, uint8_t *__restrict__ arena,
                                 const int64_t *__restrict__ dst_off) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = warp; s < n; s += nw) {
    const int L = len[s];
    const int64_t so = raw_off[s];
    uint8_t *d = arena + dst_off[s] - 32;
    const int tot = 32 + ((L + 15) & ~15) + 32;
    for (int i = lane; i < tot; i += 32) {
      const int p = i - 32;
      d[i] = (p >= 0 && p < L) ? raw[so + p] : (uint8_t)0;
    }
  }
}

}  // namespace ksw2g
