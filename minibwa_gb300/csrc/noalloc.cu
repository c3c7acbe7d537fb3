// noalloc.cu -- extension batch that allocates no memory of its own.
//
// Some callers cannot let a library call cudaMalloc: a framework that owns
// all device memory through its own caching allocator (a library-side
// cudaMalloc would bypass its budget and fragment its pool), or a serving loop
// that cannot afford the device-wide synchronisation cudaMalloc/cudaFree
// imply.  For them, ksw2g_ext_noalloc runs the same DP and backtrack kernels
// as ksw2g_ext_batch, but every piece of scratch memory -- the device copy of
// the job table, the per-job traceback offsets, the DP -> backtrack hand-off,
// the work counters and the traceback rows -- lives in one file-scope
// static __device__ array of KSW2G_NOALLOC_SCRATCH_BYTES.  Every GPU that
// loads this part of the library keeps that array until the process exits.
// The caller passes the sequence arena, the results and the CIGAR buffer in
// its own device memory.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/ksw2_gb300.h"
#include "host_common.h"
#include "ksw2g.h"
#include "launch.h"

namespace ksw2g {
int report_error(int code, const char *msg);  // sets ksw2g_last_error() (capi.cu)
}

// The whole scratch of ksw2g_ext_noalloc.  In host code this name is only a
// stand-in for the symbol; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) uint8_t g_noalloc_scratch[KSW2G_NOALLOC_SCRATCH_BYTES];

namespace {

// Scratch layout: [0,256) counters | tb_off[n] | bt[n] | jobs[n] | traceback rows
constexpr size_t kCounters = 256;
inline size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

// Exclusive prefix sum of the jobs' traceback footprints into tb_off; one block.
__global__ void __launch_bounds__(1024) tb_offsets_kernel(const ksw2g_job *__restrict__ jobs, int n, int with_cigar,
                                                          int64_t *__restrict__ tb_off) {
  __shared__ int64_t part[1024];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    int64_t f = 0;
    if (i < n && with_cigar) {
      const ksw2g_job J = jobs[i];
      if (J.qlen > 0 && J.tlen > 0) {
        int w = J.w < 0 ? (J.tlen > J.qlen ? J.tlen : J.qlen) : J.w;
        int nc = J.qlen < J.tlen ? J.qlen : J.tlen;
        nc = ((nc < w + 1 ? nc : w + 1) + 15) / 16 + 1;
        f = (((int64_t)(J.qlen + J.tlen - 1) * nc * 16) + 15) & ~(int64_t)15;
      }
    }
    part[threadIdx.x] = f;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan
      const int64_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
      __syncthreads();
      part[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < n) tb_off[i] = carry + part[threadIdx.x] - f;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
}

std::mutex g_mu;
void *g_scratch_addr[256];  // per device, filled once with that device current

int fail(int code, const char *fmt, ...) {
  char msg[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof msg, fmt, ap);
  va_end(ap);
  return ksw2g::report_error(code, msg);
}

}  // namespace

extern "C" int ksw2g_ext_noalloc(int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
                                 int n_jobs, const ksw2g_job_t *jobs, const uint8_t *d_arena, int64_t arena_len,
                                 ksw2g_ext_result_t *d_res, uint32_t *d_cigar, int64_t cigar_cap, void *stream) {
  using namespace ksw2g;
  if (n_jobs < 0 || (n_jobs > 0 && (!jobs || !d_arena || !d_res)) || !mat || arena_len < 0)
    return fail(KSW2G_E_ARG, "ksw2g_ext_noalloc: null or negative argument");
  if (n_jobs == 0) return 0;
  ksw2g_ext_params P;
  derive_ext_params(dual ? 1 : 0, m, mat, q, e, q2, e2, P);
  const int mode = ext_mode(jobs[0].flag);
  int max_nc = 1;
  int64_t foot = 0, cig = 0;
  for (int i = 0; i < n_jobs; ++i) {
    const ksw2g_job_t &J = jobs[i];
    if (ext_mode(J.flag) != mode)
      return fail(KSW2G_E_ARG, "ksw2g_ext_noalloc: job %d mixes score-only/left/right modes in one call", i);
    if ((J.flag & KSW2G_GENERIC_SC) && m > 16) return fail(KSW2G_E_UNSUPPORTED, "GENERIC_SC needs m <= 16");
    if (J.qlen < 0 || J.tlen < 0 || J.qoff < 32 || J.toff < 32 || (J.qoff & 15) || (J.toff & 15))
      return fail(KSW2G_E_ARG, "ksw2g_ext_noalloc: job %d: offsets must be 16-aligned and >= 32 (padded arena)", i);
    // the kernels read whole 16-byte blocks up to 32 bytes past a sequence's rounded end
    if (J.qoff + (((int64_t)J.qlen + 15) & ~(int64_t)15) + 32 > arena_len ||
        J.toff + (((int64_t)J.tlen + 15) & ~(int64_t)15) + 32 > arena_len)
      return fail(KSW2G_E_ARG, "ksw2g_ext_noalloc: job %d: sequence plus its 32-byte padding ends past the arena", i);
    if (J.qlen > 0 && J.tlen > 0 && !P.skip_all) {
      const int nc = ext_ncol(J.qlen, J.tlen, J.w);
      max_nc = nc > max_nc ? nc : max_nc;
      if (mode) foot += (((int64_t)(J.qlen + J.tlen - 1) * nc * 16) + 15) & ~(int64_t)15;
    }
    if (mode) cig += (int64_t)J.qlen + J.tlen + 1;
  }
  int shape = ext_shape_for(max_nc);
  if (shape < 0) {  // wider than every thread group: one pair per block, which needs no scratch of its own
    const int sp = ext_split_for(max_nc);
    if (sp < 0) return fail(KSW2G_E_BAND, "ksw2g_ext_noalloc: band of %d blocks exceeds the widest kernel", max_nc);
    shape = kSplitBase + sp;
  }
  const size_t o_tbo = kCounters, o_bt = up256(o_tbo + (size_t)n_jobs * 8);
  const size_t o_jobs = up256(o_bt + (size_t)n_jobs * sizeof(ksw2g_bt));
  const size_t o_tb = up256(o_jobs + (size_t)n_jobs * sizeof(ksw2g_job));
  if ((long long)(o_tb + foot) > KSW2G_NOALLOC_SCRATCH_BYTES)
    return fail(KSW2G_E_CAPACITY,
                "ksw2g_ext_noalloc: %d jobs need %lld scratch bytes (traceback %lld); the fixed scratch holds %lld",
                n_jobs, (long long)(o_tb + foot), (long long)foot, (long long)KSW2G_NOALLOC_SCRATCH_BYTES);
  if (mode && (!d_cigar || cigar_cap < cig))
    return fail(KSW2G_E_CAPACITY, "ksw2g_ext_noalloc: CIGAR buffer holds %lld words, %lld may be needed",
                (long long)cigar_cap, (long long)cig);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return fail(KSW2G_E_CUDA, "cudaGetDevice failed");
  uint8_t *S;
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch_addr[dev]) {  // once per device, with that device current
      void *p = nullptr;
      cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (err != cudaSuccess) return fail(KSW2G_E_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(err));
      g_scratch_addr[dev] = p;
    }
    S = (uint8_t *)g_scratch_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t err;
  if ((err = cudaMemsetAsync(S, 0, kCounters, st)) != cudaSuccess ||
      (err = cudaMemcpyAsync(S + o_jobs, jobs, (size_t)n_jobs * sizeof(ksw2g_job), cudaMemcpyHostToDevice, st)) !=
          cudaSuccess)
    return fail(KSW2G_E_CUDA, "ksw2g_ext_noalloc: %s", cudaGetErrorString(err));
  const ksw2g_job *dj = (const ksw2g_job *)(S + o_jobs);
  int64_t *tbo = (int64_t *)(S + o_tbo);
  tb_offsets_kernel<<<1, 1024, 0, st>>>(dj, n_jobs, mode != 0, tbo);
  ExtLaunch L{dj, nullptr, n_jobs, d_arena, (ksw2g_ext_result *)d_res, (ksw2g_bt *)(S + o_bt), S + o_tb, tbo,
              (int *)(S + 16)};
  if ((err = cudaGetLastError()) != cudaSuccess || (err = launch_ext_dp(dual ? 1 : 0, mode, shape, P, L, 0, st)) !=
                                                       cudaSuccess)
    return fail(KSW2G_E_CUDA, "ksw2g_ext_noalloc: %s", cudaGetErrorString(err));
  if (mode && (err = launch_ext_bt(dj, nullptr, n_jobs, (const ksw2g_bt *)(S + o_bt), S + o_tb, tbo,
                                   (ksw2g_ext_result *)d_res, d_cigar, (unsigned long long *)S, (long long)cigar_cap,
                                   (int *)(S + 8), st)) != cudaSuccess)
    return fail(KSW2G_E_CUDA, "ksw2g_ext_noalloc: %s", cudaGetErrorString(err));
  return 0;
}
