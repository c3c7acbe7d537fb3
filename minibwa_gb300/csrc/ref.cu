// ref.cu -- a 2-bit reference resident on the device, and the gather of target
// windows from it into a batch's sequence arena.
//
// The layout is minibwa's l2b (l2bit.h:18-32): base i of the concatenated
// contigs is the 2-bit field at bits 2*(i%32) of pac[i/32]; contig k spans
// [ctg_off[k], ctg_off[k] + ctg_len[k]); ambiguous bases are sorted, disjoint
// half-open intervals [st, en) of the same coordinate that read as N (code 4).
// A window (contig, st, len) decodes as l2b_getseq does (l2bit.c:52-77), then
// optionally as l2b_meth_convert (l2bit.c:79-90) and reversed in place, as the
// aligner's callers do around left extensions (mb_seq_rev).  Decoding on the
// device removes the per-job target upload: a batch then carries only its
// queries and a (contig, start, length, flags) record per job.
#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "../../include/ksw2_gb300.h"
#include "batch.h"
#include "host_common.h"

using namespace ksw2g;

struct ksw2g_ref {
  int device = 0;
  int64_t n_ctg = 0, n_pac = 0, n_ambi = 0;
  std::vector<uint64_t> h_off, h_len;  // for argument checks on the host
  DevBuf pac, off, ambi;
};

namespace ksw2g {

// One warp per window: bases, then the N runs that overlap it, then the
// methylation conversion, written (reversed if asked) into the arena slot
// around dst (32 zero bytes before, zeros to the next 16-byte boundary and 32
// more after, like the packed host sequences).
__global__ void ref_gather_kernel(int n, const int32_t *__restrict__ tid, const int64_t *__restrict__ st,
                                  const int32_t *__restrict__ len, const int32_t *__restrict__ flags,
                                  const int64_t *__restrict__ dst_off, uint8_t *__restrict__ arena,
                                  const uint64_t *__restrict__ pac, const uint64_t *__restrict__ ctg_off,
                                  const uint64_t *__restrict__ ambi, int64_t n_ambi) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int j = warp; j < n; j += nw) {
    const int L = len[j], fl = flags ? flags[j] : 0;
    const bool rev = fl & KSW2G_REF_REVERSE;
    const int meth = (fl >> 1) & 3;
    const uint64_t g0 = ctg_off[tid[j]] + (uint64_t)st[j];
    uint8_t *d = arena + dst_off[j];
    const int tot = 32 + ((L + 15) & ~15) + 32;
    auto put = [&](int p, uint8_t c) {  // window position p -> slot byte
      d[rev ? L - 1 - p : p] = c;
    };
    for (int i = lane; i < tot; i += 32) {
      const int p = i - 32;
      if (p < 0 || p >= L) d[p] = 0;
    }
    for (int p = lane; p < L; p += 32) {
      const uint64_t g = g0 + p;
      put(p, (uint8_t)(pac[g >> 5] >> ((g & 31) << 1) & 3));
    }
    __syncwarp();
    // first N interval ending after the window's start (l2bit.c l2b_getambi)
    int64_t lo = 0, hi = n_ambi;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (ambi[2 * mid + 1] > g0) hi = mid;
      else lo = mid + 1;
    }
    for (int64_t a = lo; a < n_ambi && ambi[2 * a] < g0 + (uint64_t)L; ++a) {
      const uint64_t s = ambi[2 * a] > g0 ? ambi[2 * a] : g0;
      const uint64_t e = ambi[2 * a + 1] < g0 + (uint64_t)L ? ambi[2 * a + 1] : g0 + (uint64_t)L;
      for (uint64_t g = s + lane; g < e; g += 32) put((int)(g - g0), 4);
    }
    __syncwarp();
    if (meth) {  // l2b_meth_convert: C2T turns C (1) into T (3), G2A turns G (2) into A (0)
      for (int p = lane; p < L; p += 32) {
        uint8_t &c = d[p];
        if (meth == 1 && c == 1) c = 3;
        else if (meth == 2 && c == 2) c = 0;
      }
    }
    __syncwarp();
  }
}

cudaError_t launch_ref_gather(int n, const int32_t *tid, const int64_t *st, const int32_t *len,
                              const int32_t *flags, const int64_t *dst_off, uint8_t *arena, const ksw2g_ref *R,
                              cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int bs = 256;
  int blocks = (int)(((int64_t)n * 32 + bs - 1) / bs);
  if (blocks > 65535 * 8) blocks = 65535 * 8;
  ref_gather_kernel<<<blocks, bs, 0, stream>>>(n, tid, st, len, flags, dst_off, arena, R->pac.as<uint64_t>(),
                                               R->off.as<uint64_t>(), R->ambi.as<uint64_t>(), R->n_ambi);
  return cudaGetLastError();
}

int64_t ref_ctg_len(const ksw2g_ref *R, int64_t tid) {
  return tid >= 0 && tid < R->n_ctg ? (int64_t)R->h_len[tid] : -1;
}

int ref_check_window(const ksw2g_ref *R, int64_t tid, int64_t st, int64_t len) {
  if (tid < 0 || tid >= R->n_ctg) return report_error(KSW2G_E_ARG, "reference window: contig id out of range");
  if (st < 0 || len < 0 || (uint64_t)(st + len) > R->h_len[tid])
    return report_error(KSW2G_E_ARG, "reference window: outside its contig");
  return 0;
}

}  // namespace ksw2g

extern "C" int ksw2g_ref_create(ksw2g_ctx_t *c, int64_t n_ctg, const uint64_t *ctg_off, const uint64_t *ctg_len,
                                const uint64_t *pac, int64_t n_pac, int64_t n_ambi, const uint64_t *ambi,
                                ksw2g_ref_t **out) {
  if (!c || !out || n_ctg < 1 || !ctg_off || !ctg_len || n_pac < 1 || !pac || n_ambi < 0 || (n_ambi && !ambi))
    return report_error(KSW2G_E_ARG, "reference: bad arguments");
  for (int64_t k = 0; k < n_ctg; ++k)
    if ((ctg_off[k] + ctg_len[k] + 31) / 32 > (uint64_t)n_pac)
      return report_error(KSW2G_E_ARG, "reference: a contig runs past the packed sequence");
  for (int64_t a = 0; a < n_ambi; ++a)
    if (ambi[2 * a] >= ambi[2 * a + 1] || (a && ambi[2 * a] < ambi[2 * a - 1]))
      return report_error(KSW2G_E_ARG, "reference: N intervals must be sorted, disjoint and non-empty");
  if (cudaSetDevice(c->device) != cudaSuccess) return report_error(KSW2G_E_CUDA, "reference: bad device");
  ksw2g_ref *R = new ksw2g_ref;
  R->device = c->device, R->n_ctg = n_ctg, R->n_pac = n_pac, R->n_ambi = n_ambi;
  R->h_off.assign(ctg_off, ctg_off + n_ctg);
  R->h_len.assign(ctg_len, ctg_len + n_ctg);
  int rc;
  if ((rc = R->pac.ensure(8 * (size_t)n_pac)) || (rc = R->off.ensure(8 * (size_t)n_ctg)) ||
      (rc = R->ambi.ensure(16 * (size_t)(n_ambi ? n_ambi : 1)))) {
    ksw2g_ref_destroy(R);
    return rc;
  }
  if (cudaMemcpyAsync(R->pac.p, pac, 8 * (size_t)n_pac, cudaMemcpyHostToDevice, c->st) != cudaSuccess ||
      cudaMemcpyAsync(R->off.p, ctg_off, 8 * (size_t)n_ctg, cudaMemcpyHostToDevice, c->st) != cudaSuccess ||
      (n_ambi && cudaMemcpyAsync(R->ambi.p, ambi, 16 * (size_t)n_ambi, cudaMemcpyHostToDevice, c->st) != cudaSuccess) ||
      cudaStreamSynchronize(c->st) != cudaSuccess) {
    ksw2g_ref_destroy(R);
    return report_error(KSW2G_E_CUDA, "reference: upload failed");
  }
  *out = R;
  return 0;
}

extern "C" void ksw2g_ref_destroy(ksw2g_ref_t *R) {
  if (!R) return;
  cudaSetDevice(R->device);
  R->pac.release(), R->off.release(), R->ambi.release();
  delete R;
}

extern "C" int ksw2g_ref_getseq(ksw2g_ctx_t *c, const ksw2g_ref_t *R, int64_t tid, int64_t st, int64_t len, int flags,
                                uint8_t *seq) {
  if (!c || !R || (len > 0 && !seq)) return report_error(KSW2G_E_ARG, "reference: bad arguments");
  int rc;
  if ((rc = ref_check_window(R, tid, st, len))) return rc;
  if (len == 0) return 0;
  if (cudaSetDevice(c->device) != cudaSuccess) return report_error(KSW2G_E_CUDA, "reference: bad device");
  const size_t slot = (size_t)slot_bytes((int)len);
  if ((rc = c->one.ensure(slot + 64))) return rc;
  uint8_t *d = (uint8_t *)c->one.p;
  struct {
    int64_t st, dst;
    int32_t tid, len, flags, pad;
  } rec = {st, 32, (int32_t)tid, (int32_t)len, flags, 0};
  uint8_t *meta = d + ((slot + 15) & ~(size_t)15);
  if (cudaMemcpyAsync(meta, &rec, sizeof rec, cudaMemcpyHostToDevice, c->st) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "reference: copy failed");
  cudaError_t e = launch_ref_gather(1, (const int32_t *)(meta + 16), (const int64_t *)meta, (const int32_t *)(meta + 20),
                                    (const int32_t *)(meta + 24), (const int64_t *)(meta + 8), d, R, c->st);
  if (e != cudaSuccess || cudaMemcpyAsync(seq, d + 32, (size_t)len, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "reference: gather failed");
  return 0;
}
