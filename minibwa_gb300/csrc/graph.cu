// graph.cu -- CUDA graphs over prepared batches.
//
// The kernels of several prepared batches (each a set of persistent per-bin
// launches fed by its device job queue, plus the backtrack launches of its
// traceback waves) are captured once into one graph.  Every batch is a branch
// forked from the context's stream, so a mixed workload (long extd2 pairs and
// short extz2 pairs, say) fills the GPU with both at once from a single
// launch, and repeated runs cost one cudaGraphLaunch instead of one API call
// per kernel.  Each extension branch owns a disjoint slice of the graph's
// traceback region, sized for its largest wave; a batch of several waves owns
// two and alternates its waves between two streams, so that a wave's tail
// overlaps the next wave.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/ksw2_gb300.h"
#include "batch.h"

using namespace ksw2g;

struct ksw2g_graph {
  int device = 0;
  std::vector<ksw2g_batch *> batches;
  std::vector<cudaStream_t> branch, branch2;  // branch2: second stream of a batch's alternating waves
  std::vector<cudaEvent_t> ev;  // ev[0] forks, ev[1 + i] joins branch i
  DevBuf tb;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t x = nullptr;
  int launches = 0;
};

static void graph_release(ksw2g_graph *G) {
  if (G->x) cudaGraphExecDestroy(G->x);
  if (G->g) cudaGraphDestroy(G->g);
  for (cudaStream_t s : G->branch) cudaStreamDestroy(s);
  for (cudaStream_t s : G->branch2)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : G->ev) cudaEventDestroy(e);
  G->tb.release();
  delete G;
}

extern "C" void ksw2g_graph_destroy(ksw2g_graph_t *G) {
  if (!G) return;
  cudaSetDevice(G->device);
  graph_release(G);
}

extern "C" int ksw2g_graph_create(ksw2g_ctx_t *c, int n, ksw2g_batch_t *const *batches, ksw2g_graph_t **out) {
  if (!c || !out || n < 1 || !batches) return report_error(KSW2G_E_ARG, "graph: need a context and >= 1 batch");
  for (int i = 0; i < n; ++i)
    if (!batches[i]) return report_error(KSW2G_E_ARG, "graph: null batch");
  if (cudaSetDevice(c->device) != cudaSuccess) return report_error(KSW2G_E_CUDA, "graph: bad device");
  ksw2g_graph *G = new ksw2g_graph;
  G->device = c->device;
  G->batches.assign(batches, batches + n);
  // disjoint traceback slices, 256-byte aligned; a batch of two or more waves gets
  // two slices and runs its waves alternately on two streams
  std::vector<int64_t> off(n, 0), off2(n, -1), cap(n, 0);
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    const ksw2g_batch *b = batches[i];
    if (b->kind > 1) continue;
    const int64_t m = ext_max_wave(b), al = (m + 255) & ~(int64_t)255;
    off[i] = total, cap[i] = m;
    total += al;
    if (b->waves.size() >= 2) off2[i] = total, total += al;
  }
  int rc;
  if (total > 0 && (rc = G->tb.ensure((size_t)total))) {
    graph_release(G);
    return rc;
  }
  G->ev.resize(n + 1, nullptr);
  G->branch.resize(n, nullptr);
  G->branch2.resize(n, nullptr);
  for (int i = 0; i <= n; ++i)
    if (cudaEventCreateWithFlags(&G->ev[i], cudaEventDisableTiming) != cudaSuccess) {
      graph_release(G);
      return report_error(KSW2G_E_CUDA, "graph: cudaEventCreate failed");
    }
  for (int i = 0; i < n; ++i) {
    ksw2g_batch *b = batches[i];
    bool ok = cudaStreamCreateWithFlags(&G->branch[i], cudaStreamNonBlocking) == cudaSuccess;
    if (ok && off2[i] >= 0) {
      ok = cudaStreamCreateWithFlags(&G->branch2[i], cudaStreamNonBlocking) == cudaSuccess;
      if (ok && !b->ev_fork)
        ok = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) == cudaSuccess;
    }
    if (!ok) {
      graph_release(G);
      return report_error(KSW2G_E_CUDA, "graph: stream or event creation failed");
    }
  }
  // Relaxed capture: the launchers query occupancy and set kernel attributes,
  // which are not stream operations.
  if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    graph_release(G);
    return report_error(KSW2G_E_CUDA, "graph: cudaStreamBeginCapture failed");
  }
  rc = 0;
  if (cudaEventRecord(G->ev[0], c->st) != cudaSuccess) rc = report_error(KSW2G_E_CUDA, "graph: fork record failed");
  for (int i = 0; i < n && !rc; ++i) {
    ksw2g_batch *b = batches[i];
    if (cudaStreamWaitEvent(G->branch[i], G->ev[0], 0) != cudaSuccess) {
      rc = report_error(KSW2G_E_CUDA, "graph: fork wait failed");
      break;
    }
    if (b->kind > 1)
      rc = ll_run_on(b, G->branch[i]);
    else if (off2[i] >= 0)
      rc = ext_run_on2(b, G->branch[i], G->branch2[i], G->tb.as<uint8_t>() + off[i], G->tb.as<uint8_t>() + off2[i],
                       cap[i]);
    else
      rc = ext_run_on(b, G->branch[i], G->tb.as<uint8_t>() + off[i], cap[i]);
    if (rc) break;
    G->launches += b->launches;
    if (cudaEventRecord(G->ev[1 + i], G->branch[i]) != cudaSuccess ||
        cudaStreamWaitEvent(c->st, G->ev[1 + i], 0) != cudaSuccess)
      rc = report_error(KSW2G_E_CUDA, "graph: join failed");
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(c->st, &g);
  if (!rc && ec != cudaSuccess) rc = report_error(KSW2G_E_CUDA, "graph: cudaStreamEndCapture failed");
  G->g = g;
  if (!rc && cudaGraphInstantiate(&G->x, G->g, 0) != cudaSuccess)
    rc = report_error(KSW2G_E_CUDA, "graph: cudaGraphInstantiate failed");
  if (rc) {
    cudaGetLastError();
    graph_release(G);
    return rc;
  }
  *out = G;
  return 0;
}

extern "C" int ksw2g_graph_launch(ksw2g_ctx_t *c, ksw2g_graph_t *G) {
  if (!c || !G) return report_error(KSW2G_E_ARG, "graph: null");
  if (c->device != G->device) return report_error(KSW2G_E_ARG, "graph: context is on another device");
  if (cudaSetDevice(c->device) != cudaSuccess || cudaGraphLaunch(G->x, c->st) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "graph: cudaGraphLaunch failed");
  return 0;
}

extern "C" int ksw2g_graph_launches(const ksw2g_graph_t *G) { return G ? G->launches : 0; }
