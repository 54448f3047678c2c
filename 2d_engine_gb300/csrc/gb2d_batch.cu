// gb2d_batch: many independent simulations of uneven grid sizes advanced together on
// one GPU.  Each instance is a full gb2d context with its own stream; host worker
// threads (one per in-flight instance) drive disjoint sets of instances frame by frame,
// so that the small grids' kernels from different instances overlap on the 152 SMs
// while each instance's solver keeps its own convergence test, on the device: every CG
// solve of an instance is one graph launch whose WHILE node iterates until it
// converges.  Instances are placed on workers longest-first by their measured cost per
// frame, and each grid size gets the V-cycle smoothing count an autotuning pass
// measured fastest.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <utility>
#include <vector>

#include "gb2d_internal.cuh"

struct gb2d_batch {
  std::vector<gb2d_ctx*> ctx;
  std::vector<int> smooth;     // V-cycle red-black sweeps per instance
  std::vector<double> cost;    // seconds (or cells, before tuning) per frame
  std::vector<int> worker_of;  // worker that drives each instance
  int workers = 1;
  char err[512] = {0};
};

namespace {

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
  std::map<std::pair<int, int>, std::pair<int, double>> best;  // size -> (sweeps, seconds per frame)
  for (size_t k = 0; k < b->ctx.size(); ++k) {
    gb2d_ctx* c = b->ctx[k];
    const std::pair<int, int> key(c->grid.ni, c->grid.nj);
    if (best.count(key)) continue;
    int rc = gb2d_checkpoint_save(c);
    if (rc) return rc;
    double dt0 = 0;
    std::pair<int, double> pick(2, 1e300);
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
      if (t < pick.second) pick = std::make_pair(nu, t);
    }
    if ((rc = gb2d_checkpoint_restore(c))) return rc;
    if ((rc = gb2d_synchronize(c))) return rc;
    best[key] = pick;
  }
  for (size_t k = 0; k < b->ctx.size(); ++k) {
    const auto& p = best[std::make_pair(b->ctx[k]->grid.ni, b->ctx[k]->grid.nj)];
    b->smooth[k] = p.first;
    b->cost[k] = p.second;
    if (smooth_out) smooth_out[k] = p.first;
  }
  place(b);
  return GB2D_OK;
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
