// msf_batch.cu -- many systems of uneven size and grid shape in one CUDA graph.
//
// The reference processes one trajectory per call (dens.compute_sf,
// dens.py:166); a batch holds one plan per system (each with its own grid
// shape and tuning), lays all their workspaces out in one caller buffer,
// and captures every system's histogram chain (msf_hist_sf_f32) into a
// single CUDA graph: the systems are spread over several capture streams
// (largest first, each to the least-loaded stream) forked from and joined
// back to the launch stream, so independent systems run concurrently.
// msf_batch_run replays the graph: one launch for the whole batch.  The
// graph bakes in the device pointers given at creation; callers refresh the
// positions in place and accumulate into the same sf arrays.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "msf_internal.cuh"

struct msf_batch {
  std::vector<msf_batch_system> sys;
  std::vector<msf_plan> plans;
  std::vector<size_t> ws_off;
  std::vector<int> stream_of;
  int n_streams;
  size_t ws_bytes;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  int ready;
};

namespace msf {

static size_t align_ws(size_t x) { return (x + 255) & ~(size_t)255; }

static void release(msf_batch* b) {
  for (msf_plan& p : b->plans) plan_release(&p);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaEvent_t e : b->events) cudaEventDestroy(e);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  b->exec = nullptr;
  b->graph = nullptr;
  b->events.clear();
  b->streams.clear();
  b->ready = 0;
}

}  // namespace msf

using namespace msf;

extern "C" {

int msf_batch_create(msf_batch** out, const msf_batch_system* systems, int32_t n_systems,
                     int32_t n_streams) {
  if (!out || !systems || n_systems < 1 || n_streams < 1 || n_streams > 64) return MSF_E_INVALID;
  *out = nullptr;
  msf_batch* b = new (std::nothrow) msf_batch();
  if (!b) return MSF_E_INVALID;
  b->sys.assign(systems, systems + n_systems);
  b->plans.resize(n_systems);
  b->ws_off.resize(n_systems);
  b->stream_of.resize(n_systems);
  b->n_streams = n_streams < n_systems ? n_streams : n_systems;
  b->graph = nullptr;
  b->exec = nullptr;
  b->ready = 0;
  size_t o = 0;
  std::vector<double> cost(n_systems);
  for (int i = 0; i < n_systems; ++i) {
    const msf_batch_system& s = systems[i];
    if (!s.pos_w || !s.sf || s.n_atoms < 0 || s.n_frames < 0 || (s.flags & ~MSF_WRAP)) {
      delete b;
      return MSF_E_INVALID;
    }
    msf_plan_desc d;
    memset(&d, 0, sizeof(d));
    d.n0 = s.n0; d.n1 = s.n1; d.n2 = s.n2;
    d.box[0] = s.box[0]; d.box[1] = s.box[1]; d.box[2] = s.box[2];
    d.batch = s.batch;
    d.variant = s.variant;
    d.tile_w = s.tile_w;
    d.max_atoms = s.n_atoms;
    const int st = plan_init(&b->plans[i], &d);
    if (st) { delete b; return st; }
    b->ws_off[i] = o;
    o = align_ws(o + b->plans[i].ws_bytes);
    cost[i] = (double)s.n_frames * ((double)s.n0 * s.n1 * s.n2 + 4.0 * s.n_atoms);
  }
  b->ws_bytes = o;
  // longest-processing-time assignment of systems to capture streams
  std::vector<int> order(n_systems);
  for (int i = 0; i < n_systems; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  std::vector<double> load(b->n_streams, 0.0);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    b->stream_of[i] = k;
    load[k] += cost[i];
  }
  *out = b;
  return MSF_OK;
}

size_t msf_batch_workspace_bytes(const msf_batch* b) { return b ? b->ws_bytes : 0; }

int msf_batch_bind(msf_batch* b, void* ws, size_t bytes, msf_stream_t stream) {
  if (!b || !ws) return MSF_E_INVALID;
  if (bytes < b->ws_bytes) return MSF_E_WORKSPACE;
  if (reinterpret_cast<uintptr_t>(ws) % 256) return MSF_E_INVALID;
  release(b);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  const int n = (int)b->sys.size();
  for (int i = 0; i < n; ++i) {
    const int s = msf_plan_bind(&b->plans[i], base + b->ws_off[i], b->plans[i].ws_bytes, stream);
    if (s) return s;
  }
  // capture streams and fork/join events
  b->streams.resize(b->n_streams, nullptr);
  b->events.resize(b->n_streams + 1, nullptr);
  for (int k = 0; k < b->n_streams; ++k)
    if (cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking) != cudaSuccess) { release(b); return MSF_E_CUDA; }
  for (auto& e : b->events)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { release(b); return MSF_E_CUDA; }
  // the plans' tables must be ready before the captured work reads them
  if (cudaStreamSynchronize(st) != cudaSuccess) { release(b); return MSF_E_CUDA; }
  cudaStream_t origin = b->streams[0];
  if (cudaStreamBeginCapture(origin, cudaStreamCaptureModeRelaxed) != cudaSuccess) { release(b); return MSF_E_CUDA; }
  int s = MSF_OK;
  cudaEventRecord(b->events[0], origin);
  for (int k = 1; k < b->n_streams; ++k) cudaStreamWaitEvent(b->streams[k], b->events[0], 0);
  for (int i = 0; i < n && !s; ++i) {
    const msf_batch_system& y = b->sys[i];
    s = hist_sf_chain(&b->plans[i], y.pos_w, nullptr, kLayoutF32x4, y.n_atoms, y.n_frames, y.scale, y.flags,
                      y.sf, b->streams[b->stream_of[i]]);
  }
  for (int k = 1; k < b->n_streams; ++k) {
    cudaEventRecord(b->events[k], b->streams[k]);
    cudaStreamWaitEvent(origin, b->events[k], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(origin, &g);
  if (s || e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    release(b);
    return s ? s : MSF_E_CUDA;
  }
  b->graph = g;
  if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) { release(b); return MSF_E_CUDA; }
  b->ready = 1;
  return MSF_OK;
}

int msf_batch_run(msf_batch* b, msf_stream_t stream) {
  if (!b) return MSF_E_INVALID;
  if (!b->ready) return MSF_E_NOT_BOUND;
  return cuda_status(cudaGraphLaunch(b->exec, reinterpret_cast<cudaStream_t>(stream)));
}

int msf_batch_query(const msf_batch* b, int32_t index, int32_t out[8]) {
  if (!b || !out || index < 0 || index >= (int)b->sys.size()) return MSF_E_INVALID;
  return msf_plan_query(&b->plans[index], out);
}

int msf_batch_destroy(msf_batch* b) {
  if (!b) return MSF_OK;
  release(b);
  delete b;
  return MSF_OK;
}

}  // extern "C"
