// Batches of independent correlation jobs of uneven size, launched as one CUDA graph.
//
// Each job gets its own handle (geometry, F-stage, X-stage, finalisation for its
// FFT length, input format and antenna count).  Creating the batch runs every
// job once eagerly (module loading, kernel attributes, validation), then
// captures all jobs' launch sequences as parallel branches of one graph: a
// launch of the batch is a single cudaGraphLaunch, and the GPU overlaps the
// jobs' kernels.  Jobs on pinned host inputs copy them one job after another
// (each job's copies wait for the previous job's), so that the first jobs
// correlate while the later ones load, instead of every job sharing the host
// link until all copies end together.  Inputs and delay models are fixed at creation (their upload
// copies read pinned staging that the graph replays); build a new batch to
// change them.
#include <stdio.h>

#include <string>
#include <vector>

#include "gxc_internal.h"

struct gxc_batch {
  std::vector<gxc_handle *> handles;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  std::vector<cudaEvent_t> copied;  // per job: its input copies are done
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
  std::string err;
};

namespace {

void destroy_batch(gxc_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaEvent_t e : b->events) cudaEventDestroy(e);
  for (cudaEvent_t e : b->copied) cudaEventDestroy(e);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->origin) cudaStreamDestroy(b->origin);
  for (gxc_handle *h : b->handles) gxc_destroy(h);
  delete b;
}

gxc_status batch_fail(gxc_batch *b, gxc_status st, const std::string &msg) {
  fprintf(stderr, "gxc_batch_create: %s\n", msg.c_str());
  destroy_batch(b);
  return st;
}

}  // namespace

extern "C" {

gxc_status gxc_batch_create(const gxc_job *jobs, int njobs, gxc_batch **out) {
  if (!out || !jobs || njobs < 1) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gxc_batch *b = new gxc_batch();
  cudaGetDevice(&b->device);
  for (int i = 0; i < njobs; i++) {
    const gxc_job &j = jobs[i];
    if (!j.inputs || !j.poly || !j.fso)
      return batch_fail(b, GXC_ERR_INVALID_ARGUMENT, "job " + std::to_string(i) + ": null input or delays");
    gxc_handle *h = nullptr;
    gxc_status st = gxc_create(&j.cfg, &h);
    if (st != GXC_OK) return batch_fail(b, st, "job " + std::to_string(i) + ": " + gxc_status_string(st));
    b->handles.push_back(h);
    st = gxc_set_input(h, j.inputs, gxc_input_bytes_per_antenna(&j.cfg));
    if (st == GXC_OK) st = gxc_set_delays(h, j.poly, j.fso);
    // one eager run: loads modules and sets kernel attributes outside the capture
    if (st == GXC_OK) st = gxc_process(h, nullptr);
    if (st == GXC_OK) st = gxc_sync(h);
    if (st != GXC_OK) return batch_fail(b, st, "job " + std::to_string(i) + ": " + gxc_last_error(h));
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (int i = 0; e == cudaSuccess && i < njobs; i++) {
    cudaStream_t s;
    cudaEvent_t ev;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) b->streams.push_back(s);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) b->events.push_back(ev);
    cudaEvent_t cp;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&cp, cudaEventDisableTiming);
    if (e == cudaSuccess) b->copied.push_back(cp);
  }
  if (e != cudaSuccess) return batch_fail(b, GXC_ERR_CUDA, cudaGetErrorString(e));
  // capture: fork every job onto its own stream, join back to the origin
  e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) e = cudaEventRecord(b->fork, b->origin);
  for (int i = 0; e == cudaSuccess && i < njobs; i++) {
    e = cudaStreamWaitEvent(b->streams[i], b->fork, 0);
    if (e != cudaSuccess) break;
    gxc_status st = gxc::process_chained(b->handles[i], b->streams[i], i > 0 ? b->copied[i - 1] : nullptr,
                                         b->copied[i]);
    if (st != GXC_OK) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(b->origin, &g);
      if (g) cudaGraphDestroy(g);
      return batch_fail(b, st, "capturing job " + std::to_string(i) + ": " + gxc_last_error(b->handles[i]));
    }
    e = cudaEventRecord(b->events[i], b->streams[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->origin, b->events[i], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->origin, &b->graph);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess) return batch_fail(b, GXC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  *out = b;
  return GXC_OK;
}

gxc_status gxc_batch_launch(gxc_batch *b, void *stream) {
  if (!b) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    b->err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(e);
    return GXC_ERR_CUDA;
  }
  return GXC_OK;
}

int gxc_batch_size(const gxc_batch *b) { return b ? (int)b->handles.size() : 0; }

gxc_handle *gxc_batch_job(gxc_batch *b, int i) {
  if (!b || i < 0 || i >= (int)b->handles.size()) return nullptr;
  return b->handles[i];
}

int gxc_batch_launch_count(const gxc_batch *b) {
  if (!b) return 0;
  int n = 0;
  for (const gxc_handle *h : b->handles) n += gxc_last_launch_count(h);
  return n;
}

gxc_status gxc_batch_destroy(gxc_batch *b) {
  if (!b) return GXC_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  destroy_batch(b);
  return GXC_OK;
}

}  // extern "C"
