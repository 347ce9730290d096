// Heterogeneous batched sweeps: many contexts (any mix of grids, chiN, f,
// boxes, contour steps) advanced together.  No reference counterpart -- the
// reference's batch is one grid and one parameter set (init.cpp:86-94), split
// over GPUs with no exchange.
//
// One SCF iteration of the whole group is one CUDA-graph launch: the graph
// forks onto every member's stream, runs the member's average_value x2 and
// getConc (Boltzmann factors, the four marches, Q, phi) there, and joins.
// Small grids leave most of the GPU idle when solved one after the other;
// inside the graph their kernels run concurrently.  The field updates
// (simple or Anderson mixing) follow as ordinary launches on the members'
// streams, because Anderson's ring position changes every iteration.
#include <vector>

#include "ctx.h"

// capi.cu
int scft_internal_pre_mix(scft_ctx *ctx);
int scft_internal_mix(scft_ctx *ctx);

struct scft_group {
  std::vector<scft_ctx *> members;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> joined;   // per member
  cudaGraphExec_t exec = nullptr;
  long long nodes = 0;
  long long launches = 0;
  std::string err = "no error";
};

namespace {

int gfail(scft_group *g, int st, const std::string &m) {
  g->err = m;
  return st;
}

#define GCK(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) return gfail(g, SCFT_ERR_CUDA, std::string(#call) + ": " + \
                                                           cudaGetErrorString(e_));  \
  } while (0)

void release(scft_group *g) {
  if (g->exec) cudaGraphExecDestroy(g->exec);
  for (cudaEvent_t e : g->joined) cudaEventDestroy(e);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->done) cudaEventDestroy(g->done);
  if (g->st) cudaStreamDestroy(g->st);
}

int build_graph(scft_group *g) {
  long long l0 = 0;
  for (scft_ctx *c : g->members) l0 += c->launches;
  GCK(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
  int rc = SCFT_OK;
  cudaError_t e = cudaEventRecord(g->fork, g->st);
  for (size_t i = 0; e == cudaSuccess && rc == SCFT_OK && i < g->members.size(); ++i) {
    scft_ctx *c = g->members[i];
    e = cudaStreamWaitEvent(c->st, g->fork, 0);
    if (e != cudaSuccess) break;
    c->capturing = true;
    rc = scft_internal_pre_mix(c);
    c->capturing = false;
    if (rc == SCFT_OK) e = cudaEventRecord(g->joined[i], c->st);
    if (e == cudaSuccess && rc == SCFT_OK) e = cudaStreamWaitEvent(g->st, g->joined[i], 0);
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(g->st, &graph);
  if (rc != SCFT_OK) {
    if (graph) cudaGraphDestroy(graph);
    return gfail(g, rc, "capturing a member failed");
  }
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return gfail(g, SCFT_ERR_CUDA, std::string("group capture: ") +
                                       cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  e = cudaGraphInstantiate(&g->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    g->exec = nullptr;
    return gfail(g, SCFT_ERR_CUDA, std::string("group instantiate: ") + cudaGetErrorString(e));
  }
  long long l1 = 0;
  for (scft_ctx *c : g->members) l1 += c->launches;
  g->nodes = l1 - l0;   // kernel nodes per replay (counted while capturing)
  return SCFT_OK;
}

int iterate_once(scft_group *g) {
  GCK(cudaGraphLaunch(g->exec, g->st));
  g->launches += g->nodes;
  GCK(cudaEventRecord(g->done, g->st));
  for (size_t i = 0; i < g->members.size(); ++i) {
    scft_ctx *c = g->members[i];
    GCK(cudaStreamWaitEvent(c->st, g->done, 0));
    int rc = scft_internal_mix(c);
    if (rc) return gfail(g, rc, std::string("member update: ") + scft_last_error(c));
    GCK(cudaEventRecord(g->joined[i], c->st));
    GCK(cudaStreamWaitEvent(g->st, g->joined[i], 0));
  }
  return SCFT_OK;
}

}  // namespace

extern "C" {

int scft_group_create(scft_ctx *const *ctxs, int n, scft_group **out) {
  if (!ctxs || n < 1 || !out) return SCFT_ERR_INVALID_ARG;
  *out = nullptr;
  const int dev = ctxs[0] ? ctxs[0]->p.device : 0;
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i]) return SCFT_ERR_INVALID_ARG;
    if (ctxs[i]->p.device != dev) return SCFT_ERR_UNSUPPORTED;
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == ctxs[i]) return SCFT_ERR_INVALID_ARG;
  }
  scft_group *g = new scft_group();
  g->members.assign(ctxs, ctxs + n);
  cudaSetDevice(dev);
  bool ok = cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming) == cudaSuccess;
  g->joined.assign(n, nullptr);
  for (int i = 0; ok && i < n; ++i)
    ok = cudaEventCreateWithFlags(&g->joined[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    release(g);
    delete g;
    return SCFT_ERR_CUDA;
  }
  for (scft_ctx *c : g->members) cudaStreamSynchronize(c->st);
  int rc = build_graph(g);
  if (rc) {
    scft_fail(nullptr, rc, g->err);
    release(g);
    delete g;
    return rc;
  }
  *out = g;
  return SCFT_OK;
}

void scft_group_destroy(scft_group *g) {
  if (!g) return;
  if (g->st) cudaStreamSynchronize(g->st);
  release(g);
  delete g;
}

const char *scft_group_last_error(const scft_group *g) { return g ? g->err.c_str() : "null group"; }

int scft_group_iterate(scft_group *g, int n_iter) {
  if (!g || n_iter < 0) return SCFT_ERR_INVALID_ARG;
  for (int it = 0; it < n_iter; ++it) {
    int rc = iterate_once(g);
    if (rc) return rc;
  }
  GCK(cudaStreamSynchronize(g->st));
  return SCFT_OK;
}

int scft_group_time_iterations(scft_group *g, int n_iter, double *ms) {
  if (!g || !ms || n_iter < 0) return SCFT_ERR_INVALID_ARG;
  cudaEvent_t a, b;
  GCK(cudaEventCreate(&a));
  GCK(cudaEventCreate(&b));
  GCK(cudaEventRecord(a, g->st));
  int rc = SCFT_OK;
  for (int it = 0; it < n_iter && rc == SCFT_OK; ++it) rc = iterate_once(g);
  cudaEventRecord(b, g->st);
  cudaEventSynchronize(b);
  float f = 0.f;
  cudaEventElapsedTime(&f, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = f;
  return rc;
}

// Graph-replayed kernel launches so far (the members' own counters hold
// their field-update launches).
long long scft_group_launch_count(const scft_group *g) { return g ? g->launches : -1; }

}  // extern "C"
