// gb2d_batch: many independent simulations of uneven grid sizes advanced together on
// one GPU.  Each instance is a full gb2d context with its own stream.
//
// gb2d_batch_run_graph runs the whole batch as one graph launch: each instance is an
// independent branch of one CUDA graph, a WHILE node over its frames whose body is the
// instance's frame captured for the device (frame_capture: the CFL step formed on the
// GPU, every CG solve a nested WHILE node that iterates until it converges), so the
// instances' kernels overlap on the 152 SMs with no host involvement until the run ends.
// gb2d_batch_advance drives the same frames from host worker threads (one per in-flight
// instance, each CG solve one graph launch), placed longest-first by measured cost.
// Each grid size gets the V-cycle smoothing count and tile plan an autotuning pass
// measured fastest.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <utility>
#include <vector>

#include "gb2d_internal.cuh"

using namespace gb2d;

// The captured batch run (gb2d_batch_run_graph) and what it was captured for.
struct BatchGraph {
  cudaGraphExec_t exec = nullptr;
  int frames = -1;
  double cfl = 0;
  gb2d_solve_opts opts = {};
  std::vector<int> smooth, tile;                 // the schedules captured
  std::vector<unsigned long long> frame_nodes;   // kernels of one frame outside the CG loop bodies
  std::vector<unsigned long long> body_nodes;    // kernels of one CG iteration
  double* dev_io = nullptr;  // per instance: [0] dt in / out, [1] CG iterations, [2] max rel. residual^2, [3] capped, [4] flags
  double* host_io = nullptr; // pinned copy
  cudaStream_t stream = nullptr;
};

struct gb2d_batch {
  std::vector<gb2d_ctx*> ctx;
  std::vector<int> smooth;     // V-cycle red-black sweeps per instance
  std::vector<int> tile;       // tile plan per instance (-1: the per-level rule; 0-3: one shape)
  std::vector<double> cost;    // seconds (or cells, before tuning) per frame
  std::vector<int> worker_of;  // worker that drives each instance
  int workers = 1;
  BatchGraph graph;
  char err[512] = {0};
};

namespace {

constexpr int kIo = 5;  // doubles per instance in BatchGraph::dev_io

// Start of an instance's branch: the run's first time step, cleared totals and
// detections, and the frame loop's condition.
__global__ void k_frames_begin(cudaGraphConditionalHandle h, Scalars* fs, const double* io, int frames) {
  fs->dt_frame = io[0];
  fs->g_frames = 0;
  fs->g_iters = 0;
  fs->g_rel2_max = 0.0;
  fs->g_capped = 0;
  fs->flag = 0;
  cudaGraphSetConditional(h, frames > 0 ? 1u : 0u);
}

// Last node of a frame: counts it and continues while frames remain.
__global__ void k_frame_cond(cudaGraphConditionalHandle h, Scalars* fs, int frames) {
  const int n = ++fs->g_frames;
  cudaGraphSetConditional(h, n < frames ? 1u : 0u);
}

// End of an instance's branch: its last time step and totals for the host.
__global__ void k_frames_end(const Scalars* fs, double* io) {
  io[0] = fs->dt_frame;
  io[1] = (double)fs->g_iters;
  io[2] = fs->g_rel2_max;
  io[3] = (double)fs->g_capped;
  io[4] = (double)fs->flag;
}

void drop_graph(BatchGraph& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  g.exec = nullptr;
  g.frames = -1;
}

// Capture instance k's branch into graph g: k_frames_begin, a WHILE node over the frame
// (its body captured on the instance's stream), k_frames_end.
int capture_instance(gb2d_batch* b, int k, cudaGraph_t g, int frames, double cfl, const gb2d_solve_opts* o) {
  gb2d_ctx* c = b->ctx[k];
  cudaStream_t s = c->stream;
  double* io = b->graph.dev_io + (size_t)kIo * k;
  cudaGraphConditionalHandle h;
  if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) return GB2D_ERR_CUDA;
  unsigned long long nodes = 0;
  t_capture_count = &nodes;
  int rc = GB2D_ERR_CUDA;
  if (cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    k_frames_begin<<<1, 1, 0, s>>>(h, c->sc, io, frames);
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    bool ok = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &deps, nullptr, &nd) == cudaSuccess &&
              st == cudaStreamCaptureStatusActive && cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp) == cudaSuccess &&
              cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
    if (ok) k_frames_end<<<1, 1, 0, s>>>(c->sc, io);
    cudaGraph_t out = nullptr;
    ok = cudaStreamEndCapture(s, &out) == cudaSuccess && ok;
    if (ok && cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                  cudaSuccess) {
      nodes = 0;
      rc = frame_capture(c, cfl, o);
      k_frame_cond<<<1, 1, 0, s>>>(h, c->sc, frames);
      ok = cudaStreamEndCapture(s, &out) == cudaSuccess;
      if (rc == GB2D_OK && !ok) rc = GB2D_ERR_CUDA;
    }
  }
  t_capture_count = nullptr;
  b->graph.frame_nodes[k] = nodes + 1;  // + k_frame_cond
  b->graph.body_nodes[k] = solver_body_nodes(c);
  if (rc != GB2D_OK) {
    cudaGetLastError();
    snprintf(b->err, sizeof(b->err), "graph capture, instance %d: %s", k, c->err[0] ? c->err : "capture refused");
  }
  return rc;
}

int build_graph(gb2d_batch* b, int frames, double cfl, const gb2d_solve_opts* opts) {
  BatchGraph& G = b->graph;
  drop_graph(G);
  const int n = (int)b->ctx.size();
  if (!G.dev_io) {
    if (cudaMalloc(&G.dev_io, sizeof(double) * kIo * n) != cudaSuccess ||
        cudaMallocHost(&G.host_io, sizeof(double) * kIo * n) != cudaSuccess ||
        cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking) != cudaSuccess) {
      snprintf(b->err, sizeof(b->err), "graph run: allocation failed");
      return GB2D_ERR_CUDA;
    }
  }
  G.frame_nodes.assign(n, 0);
  G.body_nodes.assign(n, 0);
  for (gb2d_ctx* c : b->ctx)  // capture reads each context's state as its host code left it
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return GB2D_ERR_CUDA;
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return GB2D_ERR_CUDA;
  int rc = GB2D_OK;
  for (int k = 0; k < n && rc == GB2D_OK; ++k) {
    gb2d_solve_opts o = *opts;
    o.mg_smooth = b->smooth[k];
    solver_set_tile_plan(b->ctx[k], b->tile[k]);
    rc = capture_instance(b, k, g, frames, cfl, &o);
  }
  if (rc == GB2D_OK && cudaGraphInstantiate(&G.exec, g, 0) != cudaSuccess) {
    cudaGetLastError();
    G.exec = nullptr;
    snprintf(b->err, sizeof(b->err), "graph run: instantiation refused");
    rc = GB2D_ERR_CUDA;
  }
  cudaGraphDestroy(g);
  if (rc != GB2D_OK) return rc;
  G.frames = frames;
  G.cfl = cfl;
  G.opts = *opts;
  G.smooth = b->smooth;
  G.tile = b->tile;
  return GB2D_OK;
}

void place(gb2d_batch* b) {
  const int n = (int)b->ctx.size();
  std::vector<int> order(n);
  for (int k = 0; k < n; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->cost[a] > b->cost[c]; });
  std::vector<double> load(b->workers, 0.0);
  b->worker_of.assign(n, 0);
  for (int k : order) {
    int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    b->worker_of[k] = w;
    load[w] += b->cost[k];
  }
}

double frame_seconds(gb2d_ctx* c, double cfl, double dt, const gb2d_solve_opts* o, int* rc) {
  auto t0 = std::chrono::steady_clock::now();
  double d = dt;
  gb2d_solve_stats st;
  *rc = gb2d_advance_frame(c, cfl, &d, o, &st);
  if (*rc == GB2D_ERR_MAX_ITERS) *rc = GB2D_OK;
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

int gb2d_batch_create(int n, const gb2d_grid* grids, const gb2d_params* params, const gb2d_flow_params* flows, int workers,
                      gb2d_batch** out) {
  if (n <= 0 || !grids || !params || !out) return GB2D_ERR_ARG;
  *out = nullptr;
  gb2d_batch* b = new (std::nothrow) gb2d_batch();
  if (!b) return GB2D_ERR_ARG;
  for (int k = 0; k < n; ++k) {
    gb2d_ctx* c = nullptr;
    int rc = gb2d_create(&grids[k], &params[k], &c);
    if (rc == GB2D_OK) c->device_loop = 1;  // each CG solve one graph launch (fewer host calls per thread)
    if (rc == GB2D_OK && flows) rc = gb2d_set_flow_params(c, &flows[k]);
    if (rc != GB2D_OK) {
      if (c) gb2d_destroy(c);
      gb2d_batch_destroy(b);
      return rc;
    }
    b->ctx.push_back(c);
    b->smooth.push_back(2);
    b->tile.push_back(-1);
    b->cost.push_back((double)grids[k].ni * grids[k].nj);
  }
  int hw = (int)std::thread::hardware_concurrency();
  if (workers <= 0) workers = std::max(1, std::min(hw > 0 ? hw : 8, 16));
  b->workers = std::max(1, std::min(workers, n));
  place(b);
  *out = b;
  return GB2D_OK;
}

int gb2d_batch_destroy(gb2d_batch* b) {
  if (!b) return GB2D_ERR_ARG;
  drop_graph(b->graph);
  if (b->graph.dev_io) cudaFree(b->graph.dev_io);
  if (b->graph.host_io) cudaFreeHost(b->graph.host_io);
  if (b->graph.stream) cudaStreamDestroy(b->graph.stream);
  for (gb2d_ctx* c : b->ctx)
    if (c) gb2d_destroy(c);
  delete b;
  return GB2D_OK;
}

const char* gb2d_batch_last_error(const gb2d_batch* b) { return b ? b->err : "null batch"; }

int gb2d_batch_size(const gb2d_batch* b, int* n, int* workers) {
  if (!b || !n) return GB2D_ERR_ARG;
  *n = (int)b->ctx.size();
  if (workers) *workers = b->workers;
  return GB2D_OK;
}

int gb2d_batch_context(gb2d_batch* b, int k, gb2d_ctx** ctx) {
  if (!b || !ctx || k < 0 || k >= (int)b->ctx.size()) return GB2D_ERR_ARG;
  *ctx = b->ctx[k];
  return GB2D_OK;
}

int gb2d_batch_autotune(gb2d_batch* b, double cfl, const gb2d_solve_opts* base, int* smooth_out) {
  if (!b || !base) return GB2D_ERR_ARG;
  struct Pick {
    int sweeps, tile;
    double seconds;
  };
  // The schedules tried per grid size: red-black sweeps per V-cycle side x tile plan (the
  // per-level rule, or one shape for every tiled level: 32x16, 32x8, 64x16).
  static const int kPlans[] = {-1, 1, 2, 0};
  std::map<std::pair<int, int>, Pick> best;
  for (size_t k = 0; k < b->ctx.size(); ++k) {
    gb2d_ctx* c = b->ctx[k];
    const std::pair<int, int> key(c->grid.ni, c->grid.nj);
    if (best.count(key)) continue;
    int rc = gb2d_checkpoint_save(c);
    if (rc) return rc;
    double dt0 = 0;
    Pick pick{2, -1, 1e300};
    for (int plan : kPlans) {
      solver_set_tile_plan(c, plan);
      for (int nu = 1; nu <= 3; ++nu) {
        gb2d_solve_opts o = *base;
        o.mg_smooth = nu;
        double t = 1e300;
        for (int rep = 0; rep < 2; ++rep) {  // the first pass also builds the solver's graphs
          if ((rc = gb2d_checkpoint_restore(c))) return rc;
          double s = frame_seconds(c, cfl, dt0, &o, &rc);
          if (rc) {
            snprintf(b->err, sizeof(b->err), "autotune, instance %zu: %s", k, gb2d_last_error(c));
            return rc;
          }
          t = std::min(t, s);
        }
        if (t < pick.seconds) pick = Pick{nu, plan, t};
      }
    }
    solver_set_tile_plan(c, -1);
    if ((rc = gb2d_checkpoint_restore(c))) return rc;
    if ((rc = gb2d_synchronize(c))) return rc;
    best[key] = pick;
  }
  for (size_t k = 0; k < b->ctx.size(); ++k) {
    const Pick& p = best[std::make_pair(b->ctx[k]->grid.ni, b->ctx[k]->grid.nj)];
    b->smooth[k] = p.sweeps;
    b->tile[k] = p.tile;
    b->cost[k] = p.seconds;
    solver_set_tile_plan(b->ctx[k], p.tile);
    if (smooth_out) smooth_out[k] = p.sweeps;
  }
  place(b);
  return GB2D_OK;
}

int gb2d_batch_schedule(const gb2d_batch* b, int k, int* sweeps, int* tile_plan) {
  if (!b || k < 0 || k >= (int)b->ctx.size()) return GB2D_ERR_ARG;
  if (sweeps) *sweeps = b->smooth[k];
  if (tile_plan) *tile_plan = b->tile[k];
  return GB2D_OK;
}

int gb2d_batch_run_graph(gb2d_batch* b, int frames, double cfl, double* dts, const gb2d_solve_opts* opts, gb2d_batch_stats* stats) {
  if (!b || !dts || !opts || frames < 0 || !std::isfinite(cfl)) return GB2D_ERR_ARG;
  const int n = (int)b->ctx.size();
  for (int k = 0; k < n; ++k)
    if (!std::isfinite(dts[k])) return GB2D_ERR_ARG;
  BatchGraph& G = b->graph;
  const bool same = G.exec && G.frames == frames && G.cfl == cfl && memcmp(&G.opts, opts, sizeof *opts) == 0 && G.smooth == b->smooth &&
                    G.tile == b->tile;
  if (!same) {
    int rc = build_graph(b, frames, cfl, opts);
    if (rc) return rc;
  }
  auto t1 = std::chrono::steady_clock::now();
  for (int k = 0; k < n; ++k) G.host_io[(size_t)kIo * k] = dts[k];
  cudaError_t e = cudaSuccess;
  for (gb2d_ctx* c : b->ctx)  // work the host queued on the instances' streams comes first
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(G.dev_io, G.host_io, sizeof(double) * kIo * n, cudaMemcpyHostToDevice, G.stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(G.exec, G.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(G.host_io, G.dev_io, sizeof(double) * kIo * n, cudaMemcpyDeviceToHost, G.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(G.stream);
  auto t2 = std::chrono::steady_clock::now();
  if (e != cudaSuccess) {
    snprintf(b->err, sizeof(b->err), "graph run: %s", cudaGetErrorString(e));
    return GB2D_ERR_CUDA;
  }
  long long iterations = 0;
  double worst = 0;
  int status = GB2D_OK, capped = 0;
  unsigned long long launches = 0;
  for (int k = 0; k < n; ++k) {
    const double* io = G.host_io + (size_t)kIo * k;
    dts[k] = io[0];
    iterations += (long long)io[1];
    worst = std::max(worst, std::sqrt(io[2]));
    capped |= io[3] != 0.0;
    const int flags = (int)io[4];
    launches += 2 + (unsigned long long)frames * G.frame_nodes[k] + (unsigned long long)io[1] * G.body_nodes[k];
    if (status == GB2D_OK && (flags & 2)) {
      status = GB2D_ERR_ZERO_GRADIENT;
      snprintf(b->err, sizeof(b->err), "instance %d: |grad phi| is zero at a node (the reference exits here)", k);
    } else if (status == GB2D_OK && (flags & 4)) {
      status = GB2D_ERR_NONFINITE;
      snprintf(b->err, sizeof(b->err), "instance %d: non-finite residual in a pressure solve", k);
    }
  }
  g_launches += launches;
  if (stats) {
    double cells = 0;
    for (gb2d_ctx* c : b->ctx) cells += (double)c->grid.ni * c->grid.nj;
    const double secs = std::chrono::duration<double>(t2 - t1).count();
    stats->frames = frames;
    stats->instances = n;
    stats->cg_iterations = iterations;
    stats->max_rel_residual = worst;
    stats->wall_ms = secs * 1e3;
    stats->cell_frames_per_s = secs > 0 ? cells * frames / secs : 0;
  }
  if (status != GB2D_OK) return status;
  return capped ? GB2D_ERR_MAX_ITERS : GB2D_OK;
}

int gb2d_batch_advance(gb2d_batch* b, int frames, double cfl, double* dts, const gb2d_solve_opts* opts, gb2d_batch_stats* stats) {
  if (!b || !dts || !opts || frames < 0) return GB2D_ERR_ARG;
  const int n = (int)b->ctx.size();
  std::mutex m;
  int status = GB2D_OK, capped = 0;
  long long iterations = 0;
  double worst = 0;
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](int w) {
    std::vector<int> mine;
    for (int k = 0; k < n; ++k)
      if (b->worker_of[k] == w) mine.push_back(k);
    long long its = 0;
    double res = 0;
    int cap = 0;
    for (int f = 0; f < frames; ++f) {
      for (int k : mine) {
        gb2d_solve_opts o = *opts;
        o.mg_smooth = b->smooth[k];
        gb2d_solve_stats st;
        memset(&st, 0, sizeof st);
        int rc = gb2d_advance_frame(b->ctx[k], cfl, &dts[k], &o, &st);
        if (rc == GB2D_ERR_MAX_ITERS) {
          cap = 1;
        } else if (rc != GB2D_OK) {
          std::lock_guard<std::mutex> hold(m);
          if (status == GB2D_OK) {
            status = rc;
            snprintf(b->err, sizeof(b->err), "instance %d, frame %d: %s", k, f, gb2d_last_error(b->ctx[k]));
          }
          return;
        }
        its += st.iterations;
        res = std::max(res, st.rel_residual);
      }
      {
        std::lock_guard<std::mutex> hold(m);
        if (status != GB2D_OK) return;
      }
    }
    std::lock_guard<std::mutex> hold(m);
    iterations += its;
    worst = std::max(worst, res);
    capped |= cap;
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < b->workers; ++w) pool.emplace_back(work, w);
  work(0);
  for (auto& t : pool) t.join();
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) {
    double cells = 0;
    for (gb2d_ctx* c : b->ctx) cells += (double)c->grid.ni * c->grid.nj;
    stats->frames = frames;
    stats->instances = n;
    stats->cg_iterations = iterations;
    stats->max_rel_residual = worst;
    stats->wall_ms = secs * 1e3;
    stats->cell_frames_per_s = secs > 0 ? cells * frames / secs : 0;
  }
  if (status != GB2D_OK) return status;
  return capped ? GB2D_ERR_MAX_ITERS : GB2D_OK;
}

}  // extern "C"
