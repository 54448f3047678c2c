// C ABI of gb2d: context, state transfer and the step entry points.  The
// orchestration mirrors EULERIAN_FLUID_SOLVER_2D's calls (see include/gb2d.h).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "gb2d_internal.cuh"

namespace gb2d {

std::atomic<unsigned long long> g_launches{0};
thread_local unsigned long long* t_capture_count = nullptr;

Space make_space(int ires, int jres, double x_min, double y_min, double x_max, double y_max) {
  Space s;
  double diff_x = x_max - x_min, diff_y = y_max - y_min;
  s.dx = diff_x / (ires - 1);
  s.dy = diff_y / (jres - 1);
  double two_dx = 2 * s.dx, two_dy = 2 * s.dy;
  double dx2 = s.dx * s.dx, dy2 = s.dy * s.dy;
  s.odx = 1.0 / s.dx;
  s.ody = 1.0 / s.dy;
  s.o2dx = 1.0 / two_dx;
  s.o2dy = 1.0 / two_dy;
  s.odx2 = 1.0 / dx2;
  s.ody2 = 1.0 / dy2;
  return s;
}

}  // namespace gb2d

using namespace gb2d;

namespace {

struct FieldDesc {
  int g, nI, nJ;
};

bool field_desc(const gb2d_grid* g, int field, FieldDesc* d) {
  int ni = g->ni, nj = g->nj;
  switch (field) {
    case GB2D_FIELD_PHI: *d = {2, ni, nj}; return true;
    case GB2D_FIELD_U: *d = {2, ni + 1, nj}; return true;
    case GB2D_FIELD_V: *d = {2, ni, nj + 1}; return true;
    case GB2D_FIELD_UA: *d = {3, ni + 1, nj}; return true;
    case GB2D_FIELD_VA: *d = {3, ni, nj + 1}; return true;
    case GB2D_FIELD_P: *d = {1, ni, nj}; return true;
    case GB2D_FIELD_KAPPA: *d = {0, ni, nj}; return true;
    case GB2D_FIELD_DENSITY: *d = {2, ni, nj}; return true;
    default: return false;
  }
}

size_t field_count(const FieldDesc& d) { return (size_t)(d.nI + 2 * d.g) * (d.nJ + 2 * d.g); }

double* field_ptr(gb2d_ctx* c, int field) {
  switch (field) {
    case GB2D_FIELD_PHI: return c->phi_buf[c->phi_cur];
    case GB2D_FIELD_U: return c->u;
    case GB2D_FIELD_V: return c->v;
    case GB2D_FIELD_UA: return c->ua;
    case GB2D_FIELD_VA: return c->va;
    case GB2D_FIELD_P: return c->p;
    case GB2D_FIELD_KAPPA: return c->kappa;
    case GB2D_FIELD_DENSITY: return c->density;
    default: return nullptr;
  }
}

int check_launch(gb2d_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(c->err, sizeof(c->err), "%s: %s", what, cudaGetErrorString(e));
    return GB2D_ERR_CUDA;
  }
  return GB2D_OK;
}

int sync_check(gb2d_ctx* c, const char* what) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(c->err, sizeof(c->err), "%s: %s", what, cudaGetErrorString(e));
    return GB2D_ERR_CUDA;
  }
  return GB2D_OK;
}

int spare(const gb2d_ctx* c, int a, int b = -1, int d = -1) {
  for (int k = 0; k < 4; ++k)
    if (k != a && k != b && k != d) return k;
  return -1;
  (void)c;
}

// One Levelset_Advection from buffer src into dst: WENO5 sweep, then phi's ghost extrapolation.
void levelset_advection_into(gb2d_ctx* c, int src, int dst, double dt) {
  int mixed = c->prm.advection_precision == GB2D_PRECISION_MIXED;
  launch_weno5_advect(c->stream, c, c->phi_buf[src], c->phi_buf[dst], dt, mixed);
  launch_extrapolate_ghosts(c->stream, c->phi_buf[dst], 2, c->grid.ni, c->grid.nj);
}

// One Reinitialization reading src (never written); sweeps alternate between a and b.
int reinit_run(gb2d_ctx* c, int src, int a, int b) {
  int mixed = c->prm.advection_precision == GB2D_PRECISION_MIXED;
  double dtau = c->base.dx / (double)c->prm.reinit_scaling;
  launch_reinit_sign(c->stream, c, c->phi_buf[src], c->sign);
  int cur = src, nxt = a;
  for (int it = 0; it < c->prm.reinit_iterations; ++it) {
    launch_reinit_sweep(c->stream, c, c->phi_buf[cur], c->phi_buf[nxt], c->sign, dtau, mixed);
    int prev = cur;
    cur = nxt;
    nxt = (prev == src) ? b : prev;
  }
  return cur;
}

void free_ctx(gb2d_ctx* c) {
  if (!c) return;
  if (c->solver) solver_destroy(c->solver);
  double* bufs[] = {c->phi_buf[0], c->phi_buf[1], c->phi_buf[2], c->phi_buf[3], c->u, c->v, c->ua, c->va, c->p,
                    c->kappa, c->sign, c->bx, c->by, c->diag, c->rhs, c->tmp_a, c->tmp_b, c->xw, c->u_alt, c->v_alt,
                    c->u_keep, c->v_keep, c->density, c->adj_coef, c->adj_gvel, c->adj_lam_phi, c->adj_mu_phi,
                    c->adj_lam_u, c->adj_lam_v, c->adj_mu_u, c->adj_mu_v, c->adj_lam_p, c->adj_eno, c->jmp_dens, c->jmp_div,
                    c->jmp_js, c->jmp_jd, c->jmp_nx, c->jmp_ny, c->jmp_phi};
  for (auto b : bufs)
    if (b) cudaFree(b);
  for (auto b : c->ckpt)
    if (b) cudaFree(b);
  if (c->jmp_bc) cudaFree(c->jmp_bc);
  if (c->sc) cudaFree(c->sc);
  if (c->host_stage) cudaFreeHost(c->host_stage);
  if (c->probe.ev) {
    for (int k = 0; k < 2 * c->probe.cap; ++k) cudaEventDestroy(c->probe.ev[k]);
    delete[] c->probe.ev;
    delete[] c->probe.bytes_each;
  }
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->side2) cudaStreamDestroy(c->side2);
  if (c->ev_fork2) cudaEventDestroy(c->ev_fork2);
  if (c->ev_join2) cudaEventDestroy(c->ev_join2);
  if (c->ev_pre0) cudaEventDestroy(c->ev_pre0);
  if (c->xfer) cudaStreamDestroy(c->xfer);
  if (c->body_stream) cudaStreamDestroy(c->body_stream);
  if (c->ev_xfer0) cudaEventDestroy(c->ev_xfer0);
  if (c->ev_xfer) cudaEventDestroy(c->ev_xfer);
  delete c;
}

}  // namespace

extern "C" {

int gb2d_field_extent(const gb2d_grid* grid, int field, int* ires, int* jres) {
  FieldDesc d;
  if (!grid || !ires || !jres || !field_desc(grid, field, &d)) return GB2D_ERR_ARG;
  *ires = d.nI + 2 * d.g;
  *jres = d.nJ + 2 * d.g;
  return GB2D_OK;
}

int gb2d_create(const gb2d_grid* grid, const gb2d_params* params, gb2d_ctx** out) {
  if (!grid || !params || !out) return GB2D_ERR_ARG;
  *out = nullptr;
  if (grid->ni < 4 || grid->nj < 4 || !(grid->x_max > grid->x_min) || !(grid->y_max > grid->y_min)) return GB2D_ERR_ARG;
  if ((long long)grid->ni * grid->nj > (1LL << 30)) return GB2D_ERR_ARG;
  if (params->reinit_scaling <= 0 || params->reinit_iterations < 0 || !(params->water_density > 0) || !(params->air_density > 0))
    return GB2D_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GB2D_ERR_NO_DEVICE;
  }
  gb2d_ctx* c = new (std::nothrow) gb2d_ctx();
  if (!c) return GB2D_ERR_ARG;
  c->grid = *grid;
  c->prm = *params;
  c->flow.water_viscosity = 1.0;  // script defaults (EULERIAN_FLUID_SOLVER_2D.h:183-194)
  c->flow.air_viscosity = 0.0;
  c->flow.gravity_x = 0.0;
  c->flow.gravity_y = -9.8;
  c->flow.cfl_number = 0.5;
  c->flow.viscosity = 0;
  int ni = grid->ni, nj = grid->nj;
  c->base = make_space(ni, nj, grid->x_min, grid->y_min, grid->x_max, grid->y_max);
  c->xs = make_space(ni + 1, nj, grid->x_min - 0.5 * c->base.dx, grid->y_min, grid->x_max + 0.5 * c->base.dx, grid->y_max);
  c->ys = make_space(ni, nj + 1, grid->x_min, grid->y_min - 0.5 * c->base.dy, grid->x_max, grid->y_max + 0.5 * c->base.dy);
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  c->stream = c->own_stream;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_pre0, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->body_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_xfer0, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_xfer, cudaEventDisableTiming);
  struct A {
    double** p;
    size_t n;
  } allocs[] = {
      {&c->phi_buf[0], (size_t)(ni + 4) * (nj + 4)}, {&c->phi_buf[1], (size_t)(ni + 4) * (nj + 4)},
      {&c->phi_buf[2], (size_t)(ni + 4) * (nj + 4)}, {&c->phi_buf[3], (size_t)(ni + 4) * (nj + 4)},
      {&c->u, (size_t)(ni + 5) * (nj + 4)},          {&c->v, (size_t)(ni + 4) * (nj + 5)},
      {&c->ua, (size_t)(ni + 7) * (nj + 6)},         {&c->va, (size_t)(ni + 6) * (nj + 7)},
      {&c->p, (size_t)(ni + 2) * (nj + 2)},          {&c->kappa, (size_t)ni * nj},
      {&c->sign, (size_t)ni * nj},                   {&c->bx, (size_t)(ni + 1) * nj},
      {&c->by, (size_t)ni * (nj + 1)},               {&c->diag, (size_t)ni * nj},
      {&c->rhs, (size_t)ni * nj},                    {&c->tmp_a, (size_t)ni * nj},
      {&c->tmp_b, (size_t)ni * nj},                  {&c->xw, (size_t)(ni + 2) * (nj + 2)},
      {&c->u_alt, (size_t)(ni + 5) * (nj + 4)},      {&c->v_alt, (size_t)(ni + 4) * (nj + 5)},
      {&c->u_keep, (size_t)(ni + 5) * (nj + 4)},     {&c->v_keep, (size_t)(ni + 4) * (nj + 5)},
      {&c->density, (size_t)(ni + 4) * (nj + 4)},
  };
  for (auto& a : allocs) {
    if (e != cudaSuccess) break;
    e = cudaMalloc(a.p, a.n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(*a.p, 0, a.n * sizeof(double));
  }
  if (e == cudaSuccess) e = cudaMalloc(&c->sc, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMemset(c->sc, 0, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMallocHost(&c->host_stage, 64 * sizeof(double));
  if (e != cudaSuccess) {
    free_ctx(c);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? GB2D_ERR_ARG : GB2D_ERR_CUDA;
  }
  c->phi_cur = 0;
  char err[256];
  c->solver = solver_create(ni, nj, err, sizeof err);
  if (!c->solver) {
    free_ctx(c);
    cudaGetLastError();
    return GB2D_ERR_CUDA;
  }
  *out = c;
  return GB2D_OK;
}

int gb2d_destroy(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  free_ctx(c);
  return GB2D_OK;
}

const char* gb2d_last_error(const gb2d_ctx* c) { return c ? c->err : "null context"; }

int gb2d_set_field(gb2d_ctx* c, int field, const double* host) {
  FieldDesc d;
  if (!c || !host || !field_desc(&c->grid, field, &d)) return GB2D_ERR_ARG;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(field_ptr(c, field), host, field_count(d) * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return sync_check(c, "set_field");
}

int gb2d_get_field(gb2d_ctx* c, int field, double* host) {
  FieldDesc d;
  if (!c || !host || !field_desc(&c->grid, field, &d)) return GB2D_ERR_ARG;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(host, field_ptr(c, field), field_count(d) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "get_field");
}

int gb2d_field_device_ptr(gb2d_ctx* c, int field, double** dptr) {
  FieldDesc d;
  if (!c || !dptr || !field_desc(&c->grid, field, &d)) return GB2D_ERR_ARG;
  *dptr = field_ptr(c, field);
  return GB2D_OK;
}

int gb2d_synchronize(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  return sync_check(c, "synchronize");
}

int gb2d_set_stream(gb2d_ctx* c, void* stream) {
  if (!c) return GB2D_ERR_ARG;
  int rc = sync_check(c, "set_stream");
  if (rc) return rc;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return GB2D_OK;
}

int gb2d_set_tile_plan(gb2d_ctx* c, int plan) {
  if (!c || plan > 3) return GB2D_ERR_ARG;
  int rc = sync_check(c, "set_tile_plan");
  if (rc) return rc;
  solver_set_tile_plan(c, plan);
  return GB2D_OK;
}

int gb2d_probe_enable(gb2d_ctx* c, int enable) {
  if (!c) return GB2D_ERR_ARG;
  int rc = sync_check(c, "probe_enable");
  if (rc) return rc;
  if (enable && !c->probe.ev) {
    c->probe.cap = 4096;
    c->probe.ev = new (std::nothrow) cudaEvent_t[2 * c->probe.cap];
    c->probe.bytes_each = new (std::nothrow) double[c->probe.cap];
    if (!c->probe.ev || !c->probe.bytes_each) return GB2D_ERR_ARG;
    for (int k = 0; k < 2 * c->probe.cap; ++k) GB2D_CUDA_TRY(c, cudaEventCreate(&c->probe.ev[k]));
  }
  c->probe.on = enable ? 1 : 0;
  c->probe.n = 0;
  return GB2D_OK;
}

// Launches queued after convergence return at entry; they are excluded as the
// ones shorter than half the median duration.
int gb2d_probe_read(gb2d_ctx* c, int* launches, double* total_ms, double* bytes_per_launch) {
  if (!c || !launches || !total_ms || !bytes_per_launch) return GB2D_ERR_ARG;
  int rc = sync_check(c, "probe_read");
  if (rc) return rc;
  int n = c->probe.n;
  float* ms = new (std::nothrow) float[n > 0 ? n : 1];
  float* srt = new (std::nothrow) float[n > 0 ? n : 1];
  if (!ms || !srt) {
    delete[] ms;
    delete[] srt;
    return GB2D_ERR_ARG;
  }
  for (int k = 0; k < n; ++k) {
    cudaError_t e = cudaEventElapsedTime(&ms[k], c->probe.ev[2 * k], c->probe.ev[2 * k + 1]);
    if (e != cudaSuccess) {
      delete[] ms;
      delete[] srt;
      snprintf(c->err, sizeof(c->err), "probe_read: %s", cudaGetErrorString(e));
      return GB2D_ERR_CUDA;
    }
    srt[k] = ms[k];
  }
  // insertion sort is fine for a few thousand launches
  for (int a = 1; a < n; ++a)
    for (int b = a; b > 0 && srt[b - 1] > srt[b]; --b) {
      float t = srt[b];
      srt[b] = srt[b - 1];
      srt[b - 1] = t;
    }
  double med = n > 0 ? srt[n / 2] : 0.0, tot = 0, bytes = 0;
  int used = 0;
  for (int k = 0; k < n; ++k)
    if (ms[k] >= 0.5 * med) {
      tot += ms[k];
      bytes += c->probe.bytes_each[k];
      used++;
    }
  delete[] ms;
  delete[] srt;
  *launches = used;
  *total_ms = tot;
  *bytes_per_launch = used ? bytes / used : 0.0;
  c->probe.n = 0;
  return GB2D_OK;
}

int gb2d_solver_layout(gb2d_ctx* c, int precision, int* levels, int* cluster_top, int* cluster_ctas) {
  if (!c || !levels || !cluster_top || !cluster_ctas) return GB2D_ERR_ARG;
  if (precision != GB2D_PRECISION_FP64 && precision != GB2D_PRECISION_MIXED) return GB2D_ERR_ARG;
  gb2d::solver_layout(c->solver, precision == GB2D_PRECISION_MIXED, levels, cluster_top, cluster_ctas);
  return GB2D_OK;
}

int gb2d_preconditioner_apply(gb2d_ctx* c, int precision, int mg_smooth, const double* r, double* z) {
  if (!c || !r || !z) return GB2D_ERR_ARG;
  if (precision != GB2D_PRECISION_FP64 && precision != GB2D_PRECISION_MIXED) return GB2D_ERR_ARG;
  const size_t n = (size_t)c->grid.ni * c->grid.nj;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->tmp_a, r, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  // z lands in xw (tmp_b may hold a jump system's diagonal shift)
  int rc = gb2d::solver_precondition(c, precision == GB2D_PRECISION_MIXED, mg_smooth, c->tmp_a, c->xw);
  if (rc) {
    snprintf(c->err, sizeof(c->err), "preconditioner_apply: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
  }
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(z, c->xw, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "preconditioner_apply");
}

int gb2d_check_exact_division(unsigned long long n, unsigned long long seed, unsigned long long* mismatches) {
  if (!mismatches) return GB2D_ERR_ARG;
  int err = 0;
  *mismatches = gb2d::check_div_by(n, seed, &err);
  return err ? GB2D_ERR_CUDA : GB2D_OK;
}

int gb2d_kernel_launches(unsigned long long* count) {
  if (!count) return GB2D_ERR_ARG;
  *count = gb2d::g_launches.load();
  return GB2D_OK;
}

static double* ckpt_field(gb2d_ctx* c, int k) {
  switch (k) {
    case 0: return c->phi_buf[c->phi_cur];
    case 1: return c->u;
    case 2: return c->v;
    case 3: return c->ua;
    case 4: return c->va;
    default: return c->p;
  }
}
static const int kCkptFields[6] = {GB2D_FIELD_PHI, GB2D_FIELD_U, GB2D_FIELD_V, GB2D_FIELD_UA, GB2D_FIELD_VA, GB2D_FIELD_P};

int gb2d_checkpoint_save(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  for (int k = 0; k < 6; ++k) {
    FieldDesc d;
    field_desc(&c->grid, kCkptFields[k], &d);
    size_t bytes = field_count(d) * sizeof(double);
    if (!c->ckpt[k]) GB2D_CUDA_TRY(c, cudaMalloc(&c->ckpt[k], bytes));
    GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->ckpt[k], ckpt_field(c, k), bytes, cudaMemcpyDeviceToDevice, c->stream));
  }
  c->ckpt_phi_cur = c->phi_cur;
  return check_launch(c, "checkpoint_save");
}

int gb2d_checkpoint_restore(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  if (!c->ckpt[0]) {
    snprintf(c->err, sizeof(c->err), "checkpoint_restore: no checkpoint saved");
    return GB2D_ERR_ARG;
  }
  c->phi_cur = c->ckpt_phi_cur;
  for (int k = 0; k < 6; ++k) {
    FieldDesc d;
    field_desc(&c->grid, kCkptFields[k], &d);
    GB2D_CUDA_TRY(c, cudaMemcpyAsync(ckpt_field(c, k), c->ckpt[k], field_count(d) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  }
  return check_launch(c, "checkpoint_restore");
}

int gb2d_levelset_advection(gb2d_ctx* c, double dt) {
  if (!c || !std::isfinite(dt)) return GB2D_ERR_ARG;
  int dst = spare(c, c->phi_cur);
  levelset_advection_into(c, c->phi_cur, dst, dt);
  c->phi_cur = dst;
  return check_launch(c, "levelset_advection");
}

int gb2d_reinitialization(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  int a = spare(c, c->phi_cur), b = spare(c, c->phi_cur, a);
  c->phi_cur = reinit_run(c, c->phi_cur, a, b);
  return check_launch(c, "reinitialization");
}

int gb2d_fast_sweeping(gb2d_ctx* c, int sweeps) {
  if (!c || sweeps < 0) return GB2D_ERR_ARG;
  launch_fast_sweeping(c->stream, c, sweeps);
  return check_launch(c, "fast_sweeping");
}

int gb2d_levelset_rk3(gb2d_ctx* c, double dt) {
  if (!c || !std::isfinite(dt)) return GB2D_ERR_ARG;
  cudaStream_t s = c->stream;
  int A = c->phi_cur, B = spare(c, A), C = spare(c, A, B), D = spare(c, A, B, C);
  // Level-set TVD-RK3 (EULERIAN_FLUID_SOLVER_2D.h:1694-1717); A keeps phi^0.
  levelset_advection_into(c, A, B, dt);
  levelset_advection_into(c, B, C, dt);
  launch_blend(s, c, c->phi_buf[A], c->phi_buf[C], 0.75, 0.25);
  levelset_advection_into(c, C, B, dt);
  launch_blend(s, c, c->phi_buf[A], c->phi_buf[B], 1 / 3.0, 2 / 3.0);
  // Reinitialisation TVD-RK3 (:1719-1741); B keeps the stage-0 level set.
  int R1 = reinit_run(c, B, C, D);
  int o1 = R1 == C ? D : C;
  int R2 = reinit_run(c, R1, o1, A);
  launch_blend(s, c, c->phi_buf[B], c->phi_buf[R2], 0.75, 0.25);
  int o2 = spare(c, B, R2);
  int o3 = spare(c, B, R2, o2);
  int R3 = reinit_run(c, R2, o2, o3);
  launch_blend(s, c, c->phi_buf[B], c->phi_buf[R3], 1 / 3.0, 2 / 3.0);
  c->phi_cur = R3;
  return check_launch(c, "levelset_rk3");
}

int gb2d_velocity_advection(gb2d_ctx* c, double dt) {
  if (!c || !std::isfinite(dt)) return GB2D_ERR_ARG;
  int ni = c->grid.ni, nj = c->grid.nj;
  launch_fill_ghost_copy(c->stream, c->ua, 3, c->u, 2, ni + 1, nj, 3);
  launch_fill_ghost_copy(c->stream, c->va, 3, c->v, 2, ni, nj + 1, 3);
  launch_eno3(c->stream, c, dt);
  return check_launch(c, "velocity_advection");
}

// Detections (c->sc->flag) clear at every host-driven call; a device-driven run keeps
// them for the whole run, which reads them at its end.
static int curvature_impl(gb2d_ctx* c) {
  double* phi = c->phi_buf[c->phi_cur];
  if (!c->graph_mode) GB2D_CUDA_TRY(c, cudaMemsetAsync(&c->sc->flag, 0, sizeof(int), c->stream));
  launch_extrapolate_ghosts(c->stream, phi, 2, c->grid.ni, c->grid.nj);
  launch_curvature(c->stream, c, phi, c->kappa, &c->sc->flag);
  return check_launch(c, "curvature");
}

static int read_flag(gb2d_ctx* c) {
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->host_stage, c->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
  int rc = sync_check(c, "read flags");
  if (rc) return rc;
  const Scalars* h = (const Scalars*)c->host_stage;
  if (h->flag & 2) {
    snprintf(c->err, sizeof(c->err), "curvature: |grad phi| is zero at a node (the reference exits here)");
    return GB2D_ERR_ZERO_GRADIENT;
  }
  return GB2D_OK;
}

int gb2d_curvature(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  int rc = curvature_impl(c);
  if (rc) return rc;
  return read_flag(c);
}

// Curvature and the jump-system assembly: the curvature runs on the side stream
// while the face weights and the diagonal (which do not need it) run on the context
// stream; with solve options, the solver's FP32 hierarchy then starts building from
// them on a third stream, and the right-hand side follows the curvature.
static int curvature_and_assemble(gb2d_ctx* c, double dt, const gb2d_solve_opts* prebuild, cudaEvent_t inputs = nullptr) {
  double* phi = c->phi_buf[c->phi_cur];
  if (!c->graph_mode) GB2D_CUDA_TRY(c, cudaMemsetAsync(&c->sc->flag, 0, sizeof(int), c->stream));
  launch_extrapolate_ghosts(c->stream, phi, 2, c->grid.ni, c->grid.nj);
  GB2D_CUDA_TRY(c, cudaEventRecord(c->ev_fork, c->stream));
  GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0));
  launch_curvature(c->side, c, phi, c->kappa, &c->sc->flag);
  GB2D_CUDA_TRY(c, cudaEventRecord(c->ev_join, c->side));
  launch_faces(c->stream, c, phi, dt);
  launch_diag(c->stream, c, dt);
  if (prebuild) solver_prebuild(c, prebuild);
  GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_join, 0));
  if (inputs) GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->stream, inputs, 0));  // U, V (and p) copied in
  launch_rhs(c->stream, c, phi, dt);
  return check_launch(c, "assemble");
}

// Host buffers of gb2d_projection_host (null: the context's field as it is / not copied out).
struct HostIO {
  const double *phi, *u, *v, *p;
  double *p_out, *u_out, *v_out;
};

static size_t field_bytes(const gb2d_ctx* c, int field) {
  FieldDesc d;
  return field_desc(&c->grid, field, &d) ? field_count(d) * sizeof(double) : 0;
}

static int projection_run(gb2d_ctx* c, double dt, const gb2d_solve_opts* o, gb2d_solve_stats* st, const HostIO* io) {
  double* phi = c->phi_buf[c->phi_cur];
  cudaEvent_t inputs = nullptr;
  if (io && io->phi)
    GB2D_CUDA_TRY(c, cudaMemcpyAsync(phi, io->phi, field_bytes(c, GB2D_FIELD_PHI), cudaMemcpyHostToDevice, c->stream));
  if (io && (io->u || io->v || io->p)) {
    // U, V and the warm-start p stream in beside the curvature, face weights and
    // diagonal, which need phi only; the right-hand side waits for them.
    GB2D_CUDA_TRY(c, cudaEventRecord(c->ev_xfer0, c->stream));
    GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->xfer, c->ev_xfer0, 0));
    if (io->u) GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->u, io->u, field_bytes(c, GB2D_FIELD_U), cudaMemcpyHostToDevice, c->xfer));
    if (io->v) GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->v, io->v, field_bytes(c, GB2D_FIELD_V), cudaMemcpyHostToDevice, c->xfer));
    if (io->p) GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->p, io->p, field_bytes(c, GB2D_FIELD_P), cudaMemcpyHostToDevice, c->xfer));
    GB2D_CUDA_TRY(c, cudaEventRecord(c->ev_xfer, c->xfer));
    inputs = c->ev_xfer;
  }
  int rc;
  if (c->asm_reuse) {
    // The level set's interior has not changed since the previous projection of this
    // time step: its curvature, face weights, diagonal and the solver's levels stand;
    // only the right-hand side follows the new velocity.  phi's ghosts are extrapolated
    // again as every projection does: the extrapolation is not idempotent (its outer
    // layer reads the previous inner layer), and the ghosts are part of the state.
    launch_extrapolate_ghosts(c->stream, phi, 2, c->grid.ni, c->grid.nj);
    if (inputs) GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->stream, inputs, 0));
    launch_rhs(c->stream, c, phi, dt);
    if ((rc = check_launch(c, "assemble"))) return rc;
    solver_keep_levels(c);
  } else if ((rc = curvature_and_assemble(c, dt, o, inputs))) {
    solver_drop_prebuild(c);
    return rc;
  }
  gb2d_solve_stats local;
  memset(&local, 0, sizeof local);
  int src = solver_solve(c, c->rhs, c->p, o, &local);
  if (src != GB2D_OK && src != GB2D_ERR_MAX_ITERS) return src;
  const bool p_out = io && io->p_out;
  if (p_out) {  // p is final: it streams out while the velocity update runs
    GB2D_CUDA_TRY(c, cudaEventRecord(c->ev_xfer0, c->stream));
    GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->xfer, c->ev_xfer0, 0));
    GB2D_CUDA_TRY(c, cudaMemcpyAsync(io->p_out, c->p, field_bytes(c, GB2D_FIELD_P), cudaMemcpyDeviceToHost, c->xfer));
    GB2D_CUDA_TRY(c, cudaEventRecord(c->ev_xfer, c->xfer));
  }
  GB2D_CUDA_TRY(c, cudaMemsetAsync(&c->sc->maxu_bits, 0, 2 * sizeof(unsigned long long), c->stream));
  launch_velocity_update(c->stream, c, phi, dt, c->sc);
  if (io && io->u_out)
    GB2D_CUDA_TRY(c, cudaMemcpyAsync(io->u_out, c->u, field_bytes(c, GB2D_FIELD_U), cudaMemcpyDeviceToHost, c->stream));
  if (io && io->v_out)
    GB2D_CUDA_TRY(c, cudaMemcpyAsync(io->v_out, c->v, field_bytes(c, GB2D_FIELD_V), cudaMemcpyDeviceToHost, c->stream));
  if (p_out) GB2D_CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_xfer, 0));
  if (c->graph_mode) return check_launch(c, "projection");
  if ((rc = read_flag(c))) return rc;
  const Scalars* h = (const Scalars*)c->host_stage;
  double mu, mv;
  memcpy(&mu, &h->maxu_bits, sizeof mu);
  memcpy(&mv, &h->maxv_bits, sizeof mv);
  local.max_velocity_x = mu;
  local.max_velocity_y = mv;
  if (st) *st = local;
  return src;
}

int gb2d_projection(gb2d_ctx* c, double dt, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !o || !std::isfinite(dt) || dt == 0.0) return GB2D_ERR_ARG;
  return projection_run(c, dt, o, st, nullptr);
}

int gb2d_projection_host(gb2d_ctx* c, double dt, const gb2d_solve_opts* o, const double* phi, const double* u, const double* v,
                         const double* p, double* p_out, double* u_out, double* v_out, gb2d_solve_stats* st) {
  if (!c || !o || !std::isfinite(dt) || dt == 0.0) return GB2D_ERR_ARG;
  const HostIO io{phi, u, v, p, p_out, u_out, v_out};
  const int rc = projection_run(c, dt, o, st, &io);
  // On every return, error paths included, no copy still reads or writes the caller's buffers.
  cudaStreamSynchronize(c->stream);
  cudaStreamSynchronize(c->xfer);
  return rc;
}

int gb2d_set_flow_params(gb2d_ctx* c, const gb2d_flow_params* f) {
  if (!c || !f || !std::isfinite(f->water_viscosity) || !std::isfinite(f->air_viscosity) || !std::isfinite(f->gravity_x) ||
      !std::isfinite(f->gravity_y) || !std::isfinite(f->cfl_number))
    return GB2D_ERR_ARG;
  c->flow = *f;
  return GB2D_OK;
}

int gb2d_apply_gravity(gb2d_ctx* c, double dt) {
  if (!c || !std::isfinite(dt)) return GB2D_ERR_ARG;
  launch_flow(c->stream, c, dt, 1, 0, 0, nullptr);
  return check_launch(c, "apply_gravity");
}

int gb2d_sourcing(gb2d_ctx* c, double dt) {
  if (!c || !std::isfinite(dt)) return GB2D_ERR_ARG;
  launch_flow(c->stream, c, dt, 0, c->flow.viscosity, 0, c->density);
  return check_launch(c, "sourcing");
}

int gb2d_velocity_boundary(gb2d_ctx* c) {
  if (!c) return GB2D_ERR_ARG;
  launch_flow(c->stream, c, 0.0, 0, 0, 1, nullptr);
  return check_launch(c, "velocity_boundary");
}

int gb2d_solve_for_rk(gb2d_ctx* c, double dt, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !o || !std::isfinite(dt) || dt == 0.0) return GB2D_ERR_ARG;
  int rc = gb2d_velocity_advection(c, dt);
  if (rc) return rc;
  launch_flow(c->stream, c, dt, 1, c->flow.viscosity, 1, c->density);
  if ((rc = check_launch(c, "solve_for_rk"))) return rc;
  return gb2d_projection(c, dt, o, st);
}

int gb2d_advance_time_step(gb2d_ctx* c, double dt, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !o || !std::isfinite(dt) || dt == 0.0) return GB2D_ERR_ARG;
  int rc = gb2d_levelset_rk3(c, dt);
  if (rc) return rc;
  const int ni = c->grid.ni, nj = c->grid.nj;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->u_keep, c->u, (size_t)(ni + 5) * (nj + 4) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->v_keep, c->v, (size_t)(ni + 4) * (nj + 5) * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  gb2d_solve_stats sum, one;
  memset(&sum, 0, sizeof sum);
  int capped = 0;
  // The level set is fixed through the velocity stages (SolveForRK advects, forces and
  // projects the velocity only): stages 2 and 3 keep the first projection's curvature,
  // face weights, diagonal and solver levels and rebuild only the right-hand side
  // (GB2D_ASM_REUSE=0 rebuilds everything, for comparison).
  static const bool reuse = [] {
    const char* e = getenv("GB2D_ASM_REUSE");
    return !(e && e[0] == '0');
  }();
  for (int stage = 0; stage < 3; ++stage) {
    memset(&one, 0, sizeof one);
    c->asm_reuse = reuse && stage > 0 ? 1 : 0;
    rc = gb2d_solve_for_rk(c, dt, o, &one);
    c->asm_reuse = 0;
    if (rc == GB2D_ERR_MAX_ITERS)
      capped = 1;
    else if (rc)
      return rc;
    sum.iterations += one.iterations;
    sum.outer_iterations += one.outer_iterations;
    if (one.rel_residual > sum.rel_residual) sum.rel_residual = one.rel_residual;
    sum.max_velocity_x = one.max_velocity_x;
    sum.max_velocity_y = one.max_velocity_y;
    if (stage == 1) launch_face_blend(c->stream, c, 0.75, 0.25);
    if (stage == 2) launch_face_blend(c->stream, c, 1 / 3.0, 2 / 3.0);
  }
  if ((rc = check_launch(c, "advance_time_step"))) return rc;
  if (st) *st = sum;
  return capped ? GB2D_ERR_MAX_ITERS : GB2D_OK;
}

int gb2d_cfl_time_step(gb2d_ctx* c, double* dt, double* rates) {
  if (!c || !dt) return GB2D_ERR_ARG;
  launch_cfl(c->stream, c);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->host_stage, c->sc->cfl, sizeof(c->sc->cfl), cudaMemcpyDeviceToHost, c->stream));
  int rc = sync_check(c, "cfl_time_step");
  if (rc) return rc;
  *dt = c->host_stage[0];
  if (rates)
    for (int k = 0; k < 4; ++k) rates[k] = c->host_stage[1 + k];
  return GB2D_OK;
}

int gb2d_advance_frame(gb2d_ctx* c, double cfl, double* dt, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !dt || !o || !std::isfinite(cfl) || !std::isfinite(*dt)) return GB2D_ERR_ARG;
  int rc = gb2d_curvature(c);
  if (rc) return rc;
  double d = 0;
  if ((rc = gb2d_cfl_time_step(c, &d, nullptr))) return rc;
  if (d == 0) d = *dt;  // DetermineTimeStep keeps the previous step (SIMULATION_WORLD.h:1201-1204)
  d = d * cfl;
  *dt = d;
  return gb2d_advance_time_step(c, d, o, st);
}

}  // extern "C"

namespace gb2d {

// One gb2d_advance_frame captured on c->stream for the device (gb2d_batch_run_graph):
// the curvature, the CFL time step formed on the device (launch_frame_dt), and the order-3
// time step with every kernel reading that step (c->dt_dev) and every solve looping on the
// device (c->graph_mode); nothing is read back.  The buffers a frame rotates (the four
// level-set buffers, U/V and their alternates) are copied back to where the frame found
// them, so that the captured frame can run again.
int frame_capture(gb2d_ctx* c, double cfl, const gb2d_solve_opts* o) {
  const int phi0 = c->phi_cur;
  double *u0 = c->u, *v0 = c->v, *ua0 = c->u_alt, *va0 = c->v_alt;
  c->graph_mode = 1;
  c->dt_dev = &c->sc->dt_frame;
  int rc = curvature_impl(c);
  if (rc == GB2D_OK) {
    launch_cfl(c->stream, c);
    launch_frame_dt(c->stream, c, cfl);
    rc = check_launch(c, "frame time step");
  }
  if (rc == GB2D_OK) rc = gb2d_advance_time_step(c, 1.0 /* read on the device */, o, nullptr);
  if (rc == GB2D_OK) {
    const size_t ni = c->grid.ni, nj = c->grid.nj;
    const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaSuccess;
    if (c->phi_cur != phi0) {
      e = cudaMemcpyAsync(c->phi_buf[phi0], c->phi_buf[c->phi_cur], (ni + 4) * (nj + 4) * sizeof(double), d2d, c->stream);
      c->phi_cur = phi0;
    }
    if (c->u != u0) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(u0, c->u, (ni + 5) * (nj + 4) * sizeof(double), d2d, c->stream);
      c->u_alt = c->u;
      c->u = u0;
    }
    if (c->v != v0) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(v0, c->v, (ni + 4) * (nj + 5) * sizeof(double), d2d, c->stream);
      c->v_alt = c->v;
      c->v = v0;
    }
    if (e != cudaSuccess) {
      snprintf(c->err, sizeof(c->err), "frame capture: %s", cudaGetErrorString(e));
      rc = GB2D_ERR_CUDA;
    } else {
      rc = check_launch(c, "frame");
    }
  }
  if (rc != GB2D_OK) {  // nothing captured runs: the buffers keep their roles
    c->phi_cur = phi0;
    c->u = u0;
    c->v = v0;
    c->u_alt = ua0;
    c->v_alt = va0;
  }
  c->graph_mode = 0;
  c->dt_dev = nullptr;
  return rc;
}

}  // namespace gb2d

extern "C" {

int gb2d_weno5_adjoint(gb2d_ctx* c, double dt, const double* lam_phi, double* mu_phi, double* mu_ua, double* mu_va) {
  if (!c || !lam_phi || !mu_phi || !std::isfinite(dt)) return GB2D_ERR_ARG;
  int rc = adjoint_buffers(c);
  if (rc) return rc;
  const size_t ni = c->grid.ni, nj = c->grid.nj;
  const size_t nphi = (ni + 4) * (nj + 4), nua = (ni + 7) * (nj + 6), nva = (ni + 6) * (nj + 7);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_phi, lam_phi, nphi * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (mu_ua) GB2D_CUDA_TRY(c, cudaMemsetAsync(c->adj_mu_u, 0, nua * sizeof(double), c->stream));
  if (mu_va) GB2D_CUDA_TRY(c, cudaMemsetAsync(c->adj_mu_v, 0, nva * sizeof(double), c->stream));
  launch_weno5_adjoint(c->stream, c, dt, mu_ua ? c->adj_mu_u : nullptr, mu_va ? c->adj_mu_v : nullptr);
  if ((rc = check_launch(c, "weno5_adjoint"))) return rc;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_phi, c->adj_mu_phi, nphi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (mu_ua) GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_ua, c->adj_mu_u, nua * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (mu_va) GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_va, c->adj_mu_v, nva * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "weno5_adjoint");
}

int gb2d_projection_adjoint(gb2d_ctx* c, double dt, const double* lam_u, const double* lam_v, const double* lam_p, double* mu_u,
                            double* mu_v, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !lam_u || !lam_v || !mu_u || !mu_v || !o || !std::isfinite(dt) || dt == 0.0) return GB2D_ERR_ARG;
  int rc = adjoint_buffers(c);
  if (rc) return rc;
  const size_t ni = c->grid.ni, nj = c->grid.nj;
  const size_t nu = (ni + 5) * (nj + 4), nv = (ni + 4) * (nj + 5), np = (ni + 2) * (nj + 2);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_u, lam_u, nu * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_v, lam_v, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (lam_p) GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_p, lam_p, np * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_projection_adjoint_rhs(c->stream, c, dt, lam_p != nullptr);
  GB2D_CUDA_TRY(c, cudaMemsetAsync(c->xw, 0, np * sizeof(double), c->stream));
  gb2d_solve_stats local;
  memset(&local, 0, sizeof local);
  int src = solver_solve(c, c->rhs, c->xw, o, &local);
  if (src != GB2D_OK && src != GB2D_ERR_MAX_ITERS) return src;
  launch_projection_adjoint_vel(c->stream, c, dt, c->xw);
  if ((rc = check_launch(c, "projection_adjoint"))) return rc;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_u, c->adj_mu_u, nu * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_v, c->adj_mu_v, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_check(c, "projection_adjoint"))) return rc;
  if (st) *st = local;
  return src;
}

int gb2d_jump_poisson_solve(gb2d_ctx* c, const double* density, const int* bc, const double* div, const double* levelset,
                            const double* jc_solution, const double* jc_derivative, double* pressure, double* normal_x,
                            double* normal_y, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !density || !bc || !div || !levelset || !jc_solution || !jc_derivative || !pressure || !o) return GB2D_ERR_ARG;
  int rc = jump_buffers(c);
  if (rc) {
    snprintf(c->err, sizeof(c->err), "jump_poisson_solve: device allocation failed");
    return rc;
  }
  const size_t ni = c->grid.ni, nj = c->grid.nj, np = (ni + 2) * (nj + 2), nphi = (ni + 4) * (nj + 4);
  const cudaMemcpyKind h2d = cudaMemcpyHostToDevice;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->jmp_dens, density, np * sizeof(double), h2d, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->jmp_bc, bc, np * sizeof(int), h2d, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->jmp_div, div, np * sizeof(double), h2d, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->jmp_phi, levelset, nphi * sizeof(double), h2d, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->jmp_js, jc_solution, np * sizeof(double), h2d, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->jmp_jd, jc_derivative, np * sizeof(double), h2d, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->xw, pressure, np * sizeof(double), h2d, c->stream));
  launch_jump_assemble(c->stream, c);
  if ((rc = check_launch(c, "jump_poisson_assemble"))) return rc;
  gb2d_solve_stats local;
  memset(&local, 0, sizeof local);
  c->sys_shift = c->tmp_b;  // the solver's levels take this system's diagonal shift
  int src = solver_solve(c, c->rhs, c->xw, o, &local);
  c->sys_shift = nullptr;
  if (src != GB2D_OK && src != GB2D_ERR_MAX_ITERS) return src;
  // The solver writes the interior; the ghost ring keeps the caller's values.
  launch_copy_interior(c->stream, c->xw, 1, c->tmp_a, 0, (int)ni, (int)nj);
  std::vector<double> host(ni * nj);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(host.data(), c->tmp_a, ni * nj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (normal_x) GB2D_CUDA_TRY(c, cudaMemcpyAsync(normal_x, c->jmp_nx, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (normal_y) GB2D_CUDA_TRY(c, cudaMemcpyAsync(normal_y, c->jmp_ny, np * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_check(c, "jump_poisson_solve"))) return rc;
  // VectorToGrid (POISSON_SOLVER.cpp:1593-1603): only the unknowns take the solution.
  for (size_t j = 0; j < nj; ++j)
    for (size_t i = 0; i < ni; ++i) {
      const size_t k = (i + 1) + (j + 1) * (ni + 2);
      if (bc[k] >= 0) pressure[k] = host[i + j * ni];
    }
  if (st) *st = local;
  return src;
}

int gb2d_projection_density_gradient(gb2d_ctx* c, double dt, double* d_water_density, double* d_air_density) {
  if (!c || !std::isfinite(dt) || dt == 0.0 || !c->adj_coef) return GB2D_ERR_ARG;
  return density_gradient(c, dt, d_water_density, d_air_density);
}

int gb2d_velocity_advection_adjoint(gb2d_ctx* c, double dt, const double* lam_u, const double* lam_v, double* mu_ua, double* mu_va) {
  if (!c || !lam_u || !lam_v || !mu_ua || !mu_va || !std::isfinite(dt)) return GB2D_ERR_ARG;
  int rc = adjoint_buffers(c);
  if (rc) return rc;
  const size_t ni = c->grid.ni, nj = c->grid.nj;
  const size_t nu = (ni + 5) * (nj + 4), nv = (ni + 4) * (nj + 5), nua = (ni + 7) * (nj + 6), nva = (ni + 6) * (nj + 7);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_u, lam_u, nu * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_v, lam_v, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  eno3_adjoint(c, dt);
  if ((rc = check_launch(c, "velocity_advection_adjoint"))) return rc;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_ua, c->adj_mu_u, nua * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_va, c->adj_mu_v, nva * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "velocity_advection_adjoint");
}

int gb2d_reinit_sweep_apply(gb2d_ctx* c, const double* phi_in, const double* sign, double* phi_out) {
  if (!c || !phi_in || !sign || !phi_out) return GB2D_ERR_ARG;
  const size_t ni = c->grid.ni, nj = c->grid.nj, nphi = (ni + 4) * (nj + 4);
  const int A = spare(c, c->phi_cur), B = spare(c, c->phi_cur, A);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->phi_buf[A], phi_in, nphi * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->sign, sign, ni * nj * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_reinit_sweep(c->stream, c, c->phi_buf[A], c->phi_buf[B], c->sign, c->base.dx / (double)c->prm.reinit_scaling,
                      c->prm.advection_precision == GB2D_PRECISION_MIXED);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(phi_out, c->phi_buf[B], nphi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "reinit_sweep_apply");
}

int gb2d_reinit_sweep_adjoint(gb2d_ctx* c, const double* phi_in, const double* sign, const double* lam, double* mu_phi, double* mu_sign) {
  if (!c || !phi_in || !sign || !lam || !mu_phi || !mu_sign) return GB2D_ERR_ARG;
  int rc = adjoint_buffers(c);
  if (rc) return rc;
  const size_t ni = c->grid.ni, nj = c->grid.nj, nphi = (ni + 4) * (nj + 4);
  const int A = spare(c, c->phi_cur);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->phi_buf[A], phi_in, nphi * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->sign, sign, ni * nj * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_phi, lam, nphi * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  reinit_sweep_vjp(c, c->phi_buf[A], c->sign, c->adj_lam_phi, c->adj_mu_phi, c->adj_gvel);
  if ((rc = check_launch(c, "reinit_sweep_adjoint"))) return rc;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_phi, c->adj_mu_phi, nphi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_sign, c->adj_gvel, ni * nj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "reinit_sweep_adjoint");
}

int gb2d_viscosity_adjoint(gb2d_ctx* c, double dt, const double* lam_u, const double* lam_v, double* mu_u, double* mu_v,
                           double* mu_phi, double* d_density) {
  if (!c || !lam_u || !lam_v || !mu_u || !mu_v || !mu_phi || !std::isfinite(dt)) return GB2D_ERR_ARG;
  int rc = adjoint_buffers(c);
  if (rc) return rc;
  const size_t ni = c->grid.ni, nj = c->grid.nj;
  const size_t nu = (ni + 5) * (nj + 4), nv = (ni + 4) * (nj + 5), nphi = (ni + 4) * (nj + 4);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_u, lam_u, nu * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->adj_lam_v, lam_v, nv * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if ((rc = viscosity_vjp(c, dt, c->adj_lam_u, c->adj_lam_v, c->adj_mu_u, c->adj_mu_v, c->adj_mu_phi, d_density))) return rc;
  if ((rc = check_launch(c, "viscosity_adjoint"))) return rc;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_u, c->adj_mu_u, nu * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_v, c->adj_mu_v, nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(mu_phi, c->adj_mu_phi, nphi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "viscosity_adjoint");
}

int gb2d_projection_phi_gradient(gb2d_ctx* c, double dt, double* d_phi) {
  if (!c || !d_phi || !std::isfinite(dt) || dt == 0.0 || !c->adj_coef) return GB2D_ERR_ARG;
  return phi_gradient(c, dt, d_phi);
}

int gb2d_poisson_assemble(gb2d_ctx* c, double dt, double* bx, double* by, double* diag, double* rhs) {
  if (!c || !std::isfinite(dt) || dt == 0.0) return GB2D_ERR_ARG;
  int rc = curvature_and_assemble(c, dt, nullptr);
  if (rc) return rc;
  size_t ni = c->grid.ni, nj = c->grid.nj;
  if (bx) GB2D_CUDA_TRY(c, cudaMemcpyAsync(bx, c->bx, (ni + 1) * nj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (by) GB2D_CUDA_TRY(c, cudaMemcpyAsync(by, c->by, ni * (nj + 1) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (diag) GB2D_CUDA_TRY(c, cudaMemcpyAsync(diag, c->diag, ni * nj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (rhs) GB2D_CUDA_TRY(c, cudaMemcpyAsync(rhs, c->rhs, ni * nj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = sync_check(c, "poisson_assemble"))) return rc;
  return read_flag(c);
}

int gb2d_poisson_apply(gb2d_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return GB2D_ERR_ARG;
  size_t n = (size_t)c->grid.ni * c->grid.nj;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->tmp_a, x, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  launch_poisson_apply_exact(c->stream, c, c->tmp_a, c->tmp_b);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(y, c->tmp_b, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  return sync_check(c, "poisson_apply");
}

int gb2d_poisson_solve(gb2d_ctx* c, const double* rhs, double* x, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  if (!c || !rhs || !x || !o) return GB2D_ERR_ARG;
  int ni = c->grid.ni, nj = c->grid.nj;
  size_t n = (size_t)ni * nj;
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->rhs, rhs, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(c->tmp_a, x, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GB2D_CUDA_TRY(c, cudaMemsetAsync(c->xw, 0, (size_t)(ni + 2) * (nj + 2) * sizeof(double), c->stream));
  launch_copy_interior(c->stream, c->tmp_a, 0, c->xw, 1, ni, nj);
  gb2d_solve_stats local;
  memset(&local, 0, sizeof local);
  int src = solver_solve(c, c->rhs, c->xw, o, &local);
  if (src != GB2D_OK && src != GB2D_ERR_MAX_ITERS) return src;
  launch_copy_interior(c->stream, c->xw, 1, c->tmp_a, 0, ni, nj);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(x, c->tmp_a, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  int rc = sync_check(c, "poisson_solve");
  if (rc) return rc;
  if (st) *st = local;
  return src;
}

}  // extern "C"
