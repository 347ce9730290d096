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
//
// Batched march.  Members that share a grid (FP32, one instance each) form a
// bucket whose marches run as one lockstep march, the way the reference
// batches its instances through one cuFFT plan (init_cuda.cu:349-375): at
// contour step t every pass is ONE launch over every member and both chains
// still marching at t, each line set reading its own slices, Boltzmann
// factor and gain table from a per-step descriptor table (PassDesc).  Members
// differ in chiN, f, box and Ns, so their step counts differ and the sets
// drop out as their chains end.  A bucket of n members makes ~2-3 launches
// per step instead of n x ~2.
#include <map>
#include <tuple>
#include <vector>

#include "ctx.h"

// capi.cu
int scft_internal_pre_mix(scft_ctx *ctx);
int scft_internal_mix(scft_ctx *ctx);
int scft_internal_pre_march(scft_ctx *ctx);
int scft_internal_post_march(scft_ctx *ctx);
int scft_internal_chain_step(const scft_ctx *ctx, int chain, int t, int *active,
                             const float **src, float **dst, const float **W, int *seg_start);
int scft_internal_seg_boundary(scft_ctx *ctx, int chain, int seg, cudaStream_t st);

// One march chain of a bucket (chain 0: qA then qB, chain 1: q+B then q+A,
// for every member), marched on its own stream.
struct BucketChain {
  scft::PassDesc *desc = nullptr;   // device: [t][pass][set]
  std::vector<long long> off;       // per step t (1..T): index of its first descriptor
  std::vector<int> nset;            // per step: members whose chain still marches
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
};
struct GroupBucket {
  std::vector<int> mem;             // member indices (same grid)
  bool xy = false;                  // first pass: the x+y plane kernel
  int npass = 0;                    // launches per step
  int T = 0;                        // steps of the longest chain
  BucketChain ch[2];
};

struct scft_group {
  std::vector<scft_ctx *> members;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> joined;   // per member
  std::vector<cudaEvent_t> pre;      // per member: ready for its bucket's march
  std::vector<int> bucket_of;        // per member: bucket index or -1
  std::vector<GroupBucket> buckets;
  long long bucket_launches = 0;     // batched-march launches per replay
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
  for (GroupBucket &b : g->buckets)
    for (BucketChain &c : b.ch) {
      cudaFree(c.desc);
      if (c.ev) cudaEventDestroy(c.ev);
      if (c.st) cudaStreamDestroy(c.st);
    }
  for (cudaEvent_t e : g->pre) cudaEventDestroy(e);
  for (cudaEvent_t e : g->joined) cudaEventDestroy(e);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->done) cudaEventDestroy(g->done);
  if (g->st) cudaStreamDestroy(g->st);
}

// Members that share a lockstep march: FP32, one instance, both contour
// blocks non-empty, grouped by grid; buckets of two or more.  A member with
// fused step pairs (one launch per contour step and chain) keeps its own
// march from 2^16 points up: measured with 21 members per grid, the batched
// (unfused) march wins at 32^3 (81.6 against 64.5 Gpt*step/s) and loses at
// 48^3 (142.3 against 169.4) and 64^3 (172.1 against 196.0).
constexpr long long kBatchFusedBelow = 1LL << 16;
int make_buckets(scft_group *g) {
  std::map<std::tuple<int, int, int>, std::vector<int>> by_grid;
  for (size_t i = 0; i < g->members.size(); ++i) {
    const scft_ctx *c = g->members[i];
    if (c->rkind != kRealF32 || c->batch != 1 || c->NsA < 1 || c->dNsB < 1) continue;
    if (c->fuse_steps && c->M >= kBatchFusedBelow) continue;
    by_grid[std::make_tuple(c->p.nx, c->p.ny, c->p.nz)].push_back((int)i);
  }
  g->bucket_of.assign(g->members.size(), -1);
  for (auto &kv : by_grid) {
    if (kv.second.size() < 2) continue;
    GroupBucket b;
    b.mem = kv.second;
    const scft_ctx *c0 = g->members[b.mem[0]];
    b.xy = c0->passes.size() >= 2 && c0->pass_axis[0] == 0 && c0->pass_axis[1] == 1 &&
           scft::xy_fusable(c0->passes[0], c0->passes[1]);
    b.npass = (int)c0->passes.size() - (b.xy ? 1 : 0);
    for (int m : b.mem) {
      const scft_ctx *c = g->members[m];
      if (c->NsA + c->dNsB > b.T) b.T = c->NsA + c->dNsB;
    }
    g->buckets.push_back(b);   // owned by the group from here (release frees it)
    GroupBucket &bb = g->buckets.back();
    for (int m : bb.mem) g->bucket_of[m] = (int)g->buckets.size() - 1;
    // descriptors per chain: [t][pass][set], sets = members still marching
    for (int ch = 0; ch < 2; ++ch) {
      BucketChain &bc = bb.ch[ch];
      std::vector<scft::PassDesc> host;
      bc.off.assign(bb.T + 1, 0);
      bc.nset.assign(bb.T + 1, 0);
      for (int t = 1; t <= bb.T; ++t) {
        bc.off[t] = (long long)host.size();
        std::vector<scft::PassDesc> step[3];
        for (int m : bb.mem) {
          scft_ctx *c = g->members[m];
          int active = 0, seg = -1;
          const float *src = nullptr, *W = nullptr;
          float *dst = nullptr;
          scft_internal_chain_step(c, ch, t, &active, &src, &dst, &W, &seg);
          if (!active) continue;
          float *tmp0 = static_cast<float *>(c->tmp[2 * ch]);
          float *tmp1 = static_cast<float *>(c->tmp[2 * ch + 1]);
          for (int pi = 0; pi < bb.npass; ++pi) {
            scft::PassDesc d;
            d.in = pi == 0 ? src : ((pi - 1) & 1 ? tmp1 : tmp0);
            d.out = pi == bb.npass - 1 ? dst : (pi & 1 ? tmp1 : tmp0);
            d.pre = pi == 0 ? W : nullptr;
            d.post = pi == bb.npass - 1 ? W : nullptr;
            const int ai = bb.xy ? (pi == 0 ? 0 : pi + 1) : pi;   // the member's axis pass
            d.gain = static_cast<const float *>(c->passes[ai].gain);
            d.gain_y = bb.xy && pi == 0 ? static_cast<const float *>(c->passes[1].gain) : nullptr;
            step[pi].push_back(d);
          }
        }
        bc.nset[t] = (int)step[0].size();
        if (bc.nset[t] > 65535) return gfail(g, SCFT_ERR_UNSUPPORTED, "bucket too large");
        for (int pi = 0; pi < bb.npass; ++pi)
          host.insert(host.end(), step[pi].begin(), step[pi].end());
      }
      if (cudaMalloc(&bc.desc, sizeof(scft::PassDesc) * host.size()) != cudaSuccess) {
        cudaGetLastError();
        return gfail(g, SCFT_ERR_NO_MEMORY, "batched-march descriptor allocation failed");
      }
      GCK(cudaMemcpy(bc.desc, host.data(), sizeof(scft::PassDesc) * host.size(),
                     cudaMemcpyHostToDevice));
      GCK(cudaStreamCreateWithFlags(&bc.st, cudaStreamNonBlocking));
      GCK(cudaEventCreateWithFlags(&bc.ev, cudaEventDisableTiming));
    }
  }
  return SCFT_OK;
}

// The lockstep march of one chain of a bucket on the chain's stream: per
// step, the boundary slices of the segments starting there, then one launch
// per pass.
int bucket_march(scft_group *g, GroupBucket &b, int ch, long long *launches) {
  const scft_ctx *c0 = g->members[b.mem[0]];
  BucketChain &bc = b.ch[ch];
  for (int t = 1; t <= b.T; ++t) {
    const int n = bc.nset[t];
    if (n == 0) break;
    for (int m : b.mem) {
      scft_ctx *c = g->members[m];
      int active = 0, seg = -1;
      const float *src = nullptr, *W = nullptr;
      float *dst = nullptr;
      scft_internal_chain_step(c, ch, t, &active, &src, &dst, &W, &seg);
      if (!active || seg < 0) continue;
      // (counted by the member's own launch counter)
      if (int rc = scft_internal_seg_boundary(c, ch, seg, bc.st))
        return gfail(g, rc, std::string("segment boundary: ") + scft_last_error(c));
    }
    for (int pi = 0; pi < b.npass; ++pi) {
      const scft::PassDesc *d = bc.desc + bc.off[t] + (long long)pi * n;
      scft::PassSet<float> ps;
      memset(&ps, 0, sizeof(ps));
      ps.nset = 1;
      ps.batch = n;
      ps.w_bs = 0;
      ps.desc = d;
      cudaError_t e;
      const int ai = b.xy ? (pi == 0 ? 0 : pi + 1) : pi;
      const scft::AxisPlan &ap = c0->passes[ai];
      if (b.xy && pi == 0) e = scft::launch_xy(c0->passes[0], c0->passes[1], ps, bc.st);
      else if (ap.use_fast) e = scft::launch_fast_line(ap, ps, bc.st);
      else e = scft::launch_line_filter_desc(ap, d, n, bc.st);
      if (e != cudaSuccess)
        return gfail(g, SCFT_ERR_CUDA, std::string("batched pass: ") + cudaGetErrorString(e));
      ++*launches;
    }
  }
  return SCFT_OK;
}

int build_graph(scft_group *g) {
  long long l0 = 0;
  for (scft_ctx *c : g->members) l0 += c->launches;
  GCK(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
  int rc = SCFT_OK;
  long long bl = 0;
  cudaError_t e = cudaEventRecord(g->fork, g->st);
  // members: their own iteration body, or for bucket members the part before
  // the march
  for (size_t i = 0; e == cudaSuccess && rc == SCFT_OK && i < g->members.size(); ++i) {
    scft_ctx *c = g->members[i];
    e = cudaStreamWaitEvent(c->st, g->fork, 0);
    if (e != cudaSuccess) break;
    c->capturing = true;
    const bool bucketed = g->bucket_of[i] >= 0;
    rc = bucketed ? scft_internal_pre_march(c) : scft_internal_pre_mix(c);
    c->capturing = false;
    if (rc != SCFT_OK) break;
    if (bucketed) {
      e = cudaEventRecord(g->pre[i], c->st);
    } else {
      e = cudaEventRecord(g->joined[i], c->st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(g->st, g->joined[i], 0);
    }
  }
  // buckets: the batched march once all members are ready, then each
  // member's Q and phi
  for (size_t k = 0; e == cudaSuccess && rc == SCFT_OK && k < g->buckets.size(); ++k) {
    GroupBucket &b = g->buckets[k];
    for (int ch = 0; ch < 2 && e == cudaSuccess && rc == SCFT_OK; ++ch) {
      for (int m : b.mem)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b.ch[ch].st, g->pre[m], 0);
      if (e != cudaSuccess) break;
      if ((rc = bucket_march(g, b, ch, &bl))) break;
      e = cudaEventRecord(b.ch[ch].ev, b.ch[ch].st);
    }
    for (int m : b.mem) {
      if (e != cudaSuccess || rc != SCFT_OK) break;
      scft_ctx *c = g->members[m];
      e = cudaStreamWaitEvent(c->st, b.ch[0].ev, 0);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c->st, b.ch[1].ev, 0);
      if (e != cudaSuccess) break;
      c->capturing = true;
      rc = scft_internal_post_march(c);
      c->capturing = false;
      if (rc == SCFT_OK) e = cudaEventRecord(g->joined[m], c->st);
      if (e == cudaSuccess && rc == SCFT_OK) e = cudaStreamWaitEvent(g->st, g->joined[m], 0);
    }
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
  g->bucket_launches = bl;
  g->nodes = l1 - l0 + bl;   // kernel nodes per replay (counted while capturing)
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
  g->pre.assign(n, nullptr);
  for (int i = 0; ok && i < n; ++i)
    ok = cudaEventCreateWithFlags(&g->joined[i], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&g->pre[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    release(g);
    delete g;
    return SCFT_ERR_CUDA;
  }
  for (scft_ctx *c : g->members) cudaStreamSynchronize(c->st);
  int rc = make_buckets(g);
  if (rc == SCFT_OK) rc = build_graph(g);
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
