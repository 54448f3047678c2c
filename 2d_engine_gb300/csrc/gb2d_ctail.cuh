// gb2d_ctail.cuh — the coarse end of the V-cycle as ONE thread-block cluster.
//
// Included by gb2d_solver.cu inside its anonymous namespace (uses Level, Scalars,
// block_sum, publish_rz, kMaxLevels, kCoarseMax).
//
// Every level from the cluster's top level (at most 128^2 cells) down to the dense
// coarse solve runs inside one launch of a cluster of P CTAs (16 where the part
// allows it, else 8), each CTA one SM with 1024 threads:
//
//   * distributed levels: the rows of a level are split into P contiguous
//     stripes, one per CTA, nested from level to level (the fine rows of a CTA's
//     coarse rows are its own fine rows), so restriction and prolongation stay
//     inside a CTA.  A half sweep reads the neighbouring stripe's boundary row
//     straight from that CTA's shared memory (distributed shared memory), and one
//     cluster barrier separates consecutive half sweeps;
//   * local levels (fewer than P * kCtMinRows rows): every CTA gathers the
//     restricted right-hand side from the stripes and runs these levels and the
//     dense coarse solve redundantly in its own shared memory, with block
//     barriers only; every CTA computes identical values (same inputs, same
//     order), and each prolongs from its own copy.
//
// Coefficients, x and b of all levels stay in shared memory for the whole
// V-cycle tail; global memory is read once (coefficients, the top level's b)
// and written once (the top level's x).  <cooperative_groups.h> is included at
// global scope by the including file.

namespace cgx = cooperative_groups;

constexpr int kClusterMax = 16;
constexpr int kCtThreads = 1024;
constexpr int kCtMaxLevels = 10;
constexpr int kCtMinRows = 4;           // rows per CTA on the coarsest distributed level
constexpr int kCtOwnerRows = 256;       // rows of the bottom distributed level (owner table)
constexpr size_t kCtSmemCap = 220 * 1024;
// Largest top level: a 256^2 FP32 level fits in the cluster's shared memory, but
// measured at 1024^2 the projection is faster with 256^2 in the tiled kernels
// (one launch per smoothing side, no cluster barriers) and the cluster from 128^2.
constexpr int kCtMaxTopCells = 128 * 128;

template <typename T>
struct CtLevel {
  int nI, nJ, ld;  // ld = nI + 2 (the padded global layout and the shared copy share it)
  int rows_cap;    // rows held in shared memory: max stripe (distributed) or nJ (local)
  int off;         // shared-memory offset (elements of T) of the six arrays
  int half_log2;   // threads per row in a half sweep = 1 << half_log2
  int full_log2;   // threads per row over whole rows
  const T *cx, *cy, *idg, *dg, *b;
  T* x;
};

template <typename T>
struct CtArgs {
  int nlev;   // levels held; level 0 here is hierarchy level 'ctail'
  int ndist;  // levels [0, ndist) are distributed, the rest local
  int res_off;   // residual of the bottom distributed level (elements of T)
  int ainv_off;  // dense inverse of the coarsest level (elements of T)
  int bc_off;    // the coarsest level's right-hand side in cell order (elements of T)
  CtLevel<T> L[kCtMaxLevels];
  short J0[kCtMaxLevels][kClusterMax + 1];  // CTA c owns rows [J0[l][c], J0[l][c+1])
  Scalars* sc;  // set when the top level is the finest: publish r.z and beta
};

// Asynchronous global -> shared copy of one element (no register staging: every
// copy of the staging loop is in flight at once).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <typename T>
struct CtView {
  T *x, *b, *cx, *cy, *idg, *dg;
};

template <typename T>
__device__ __forceinline__ CtView<T> ct_view(T* sm, const CtLevel<T>& L) {
  const size_t n = (size_t)(L.rows_cap + 2) * L.ld;
  T* p = sm + L.off;
  return CtView<T>{p, p + n, p + 2 * n, p + 3 * n, p + 4 * n, p + 5 * n};
}

// One colour of a red-black Gauss-Seidel sweep over local rows 1..rows (global
// rows J0..J0+rows-1).  xdn / xup: the x row below the first and above the last
// local row (a neighbour's shared memory, or the local zero ghost row).
template <typename T>
__device__ __forceinline__ void ct_half(const CtView<T>& v, int nI, int ld, int J0, int rows, const T* xdn, const T* xup, int lg,
                                        int color) {
  const int tpr = 1 << lg, groups = kCtThreads >> lg;
  const int g = threadIdx.x >> lg, s = threadIdx.x & (tpr - 1);
  const int hw = (nI + 1) >> 1;
  auto row = [&](int lr, const T* xm, const T* xp) {
    const int par = (color + J0 + lr - 1) & 1;  // colour of cell (i, J) is (i + J) & 1
    const int rb = lr * ld;
    for (int m = s; m < hw; m += tpr) {
      const int k = 2 * m + par + 1;
      if (k > nI) continue;
      const int q = rb + k;
      v.x[q] = (v.b[q] + v.cx[q] * v.x[q - 1] + v.cx[q + 1] * v.x[q + 1] + v.cy[q] * xm[k] + v.cy[q + ld] * xp[k]) * v.idg[q];
    }
  };
  for (int lr = 1 + g; lr <= rows; lr += groups) {
    if (lr == 1 || lr == rows)  // a neighbour's row (distributed shared memory) or the wall
      row(lr, lr == 1 ? xdn : v.x + (lr - 1) * ld, lr == rows ? xup : v.x + (lr + 1) * ld);
    else  // both rows in this CTA's shared memory
      row(lr, v.x + (lr - 1) * ld, v.x + (lr + 1) * ld);
  }
}

// b - A x at local row lr, padded column k.
template <typename T>
__device__ __forceinline__ T ct_residual(const CtView<T>& v, int ld, int lr, int rows, int k, const T* xdn, const T* xup) {
  const T* xm = lr == 1 ? xdn : v.x + (size_t)(lr - 1) * ld;
  const T* xp = lr == rows ? xup : v.x + (size_t)(lr + 1) * ld;
  const size_t q = (size_t)lr * ld + k;
  T ax = v.dg[q] * v.x[q] - v.cx[q] * v.x[q - 1] - v.cx[q + 1] * v.x[q + 1] - v.cy[q] * xm[k] - v.cy[q + ld] * xp[k];
  return v.b[q] - ax;
}

// Restriction between two levels whose rows [fJ0, fJ0+frows) and [cJ0, cJ0+crows)
// are held by this CTA, with fJ0 = 2 cJ0: coarse b = average of the fine residuals.
// The pre-smoothing ends with a black half sweep, after which the residual of
// every black cell is zero: only the red cell of each fine row is evaluated.
template <typename T>
__device__ __forceinline__ void ct_restrict(const CtView<T>& f, const CtLevel<T>& F, int fJ0, int frows, const T* xdn, const T* xup,
                                            const CtView<T>& c, const CtLevel<T>& C, int cJ0, int crows) {
  const int lg = C.full_log2, tpr = 1 << lg, groups = kCtThreads >> lg;
  const int g = threadIdx.x >> lg, s = threadIdx.x & (tpr - 1);
  for (int lrc = 1 + g; lrc <= crows; lrc += groups) {
    const int Jc = cJ0 + lrc - 1;
    for (int I = s; I < C.nI; I += tpr) {
      T acc = 0;
#pragma unroll
      for (int bb = 0; bb < 2; ++bb) {
        const int J = 2 * Jc + bb;
        const int i = 2 * I + (J & 1);  // the red cell of this fine row within the coarse cell
        if (J >= F.nJ || i >= F.nI) continue;
        acc += ct_residual(f, F.ld, J - fJ0 + 1, frows, i + 1, xdn, xup);
      }
      c.b[(size_t)lrc * C.ld + I + 1] = (T)0.25 * acc;
    }
  }
}

// x_fine += x_coarse(i/2, j/2) over this CTA's fine rows.
template <typename T>
__device__ __forceinline__ void ct_prolong(const CtView<T>& f, const CtLevel<T>& F, int fJ0, int frows, const CtView<T>& c, const CtLevel<T>& C,
                                           int cJ0) {
  const int lg = F.full_log2, tpr = 1 << lg, groups = kCtThreads >> lg;
  const int g = threadIdx.x >> lg, s = threadIdx.x & (tpr - 1);
  for (int lr = 1 + g; lr <= frows; lr += groups) {
    const int J = fJ0 + lr - 1;
    const size_t cr = (size_t)(J / 2 - cJ0 + 1) * C.ld;
    for (int i = s; i < F.nI; i += tpr) f.x[(size_t)lr * F.ld + i + 1] += c.x[cr + i / 2 + 1];
  }
}

template <typename T>
__global__ void __launch_bounds__(kCtThreads, 1) k_ctail(CtArgs<T> a, const double* __restrict__ ainv, int nu, const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;  // uniform over the cluster: no CTA reaches a cluster barrier
  cgx::cluster_group cl = cgx::this_cluster();
  const int P = (int)cl.num_blocks();
  const int c = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  __shared__ unsigned char owner[kCtOwnerRows];
  __shared__ double rz_part;
  const int nl = a.nlev, nd = a.ndist;

  // ---- stage: coefficients (padded rows, so ghost columns come along as zero),
  // the top level's b, x = 0.
  for (int l = 0; l < nl; ++l) {
    const CtLevel<T>& L = a.L[l];
    const CtView<T> v = ct_view(sm, L);
    const bool dist = l < nd;
    const int J0 = dist ? a.J0[l][c] : 0;
    const int rows = dist ? a.J0[l][c + 1] - J0 : L.nJ;
    const int n = (L.rows_cap + 2) * L.ld;
    // Local row lr is padded global row J0 + lr, so local element u is global
    // element u + J0 ld: the stripe is one contiguous range of each array.
    const T *gcx = L.cx + (size_t)J0 * L.ld, *gcy = L.cy + (size_t)J0 * L.ld, *gid = L.idg + (size_t)J0 * L.ld,
            *gdg = L.dg + (size_t)J0 * L.ld, *gb = L.b + (size_t)J0 * L.ld;
    const int own_lo = L.ld, own_hi = (rows + 1) * L.ld;                              // local rows 1..rows
    const int cy_hi = (rows + 2 < L.nJ + 2 - J0 ? rows + 2 : L.nJ + 2 - J0) * L.ld;  // + the face above the stripe
    for (int u = threadIdx.x; u < n; u += kCtThreads) {
      v.x[u] = (T)0;
      if (u >= own_lo && u < own_hi) {
        cp_async_elem(v.cx + u, gcx + u);
        cp_async_elem(v.idg + u, gid + u);
        cp_async_elem(v.dg + u, gdg + u);
        if (l == 0)
          cp_async_elem(v.b + u, gb + u);
        else
          v.b[u] = (T)0;
      } else {
        v.cx[u] = v.idg[u] = v.dg[u] = v.b[u] = (T)0;
      }
      if (u >= own_lo && u < cy_hi)
        cp_async_elem(v.cy + u, gcy + u);
      else
        v.cy[u] = (T)0;
    }
  }
  {
    const CtLevel<T>& C = a.L[nl - 1];
    const int n = C.nI * C.nJ;
    T* ai = sm + a.ainv_off;
    for (int u = threadIdx.x; u < n * n; u += kCtThreads) ai[u] = (T)ainv[u];
    if (nd > 0) {
      const CtLevel<T>& B = a.L[nd - 1];
      for (int r = threadIdx.x; r < B.nJ && r < kCtOwnerRows; r += kCtThreads) {
        int o = 0;
        while (o + 1 < P && a.J0[nd - 1][o + 1] <= r) ++o;
        owner[r] = (unsigned char)o;
      }
    }
  }
  cp_async_wait_all();
  cl.sync();  // every CTA's shared memory is initialised before any remote read

  // Neighbour rows of a distributed level: the last row of CTA c-1 and the first
  // of CTA c+1, or the local zero ghost rows at the domain's walls.
  auto xdn_of = [&](int l, const CtView<T>& v) -> const T* {
    if (c == 0) return v.x;
    const int rprev = a.J0[l][c] - a.J0[l][c - 1];
    return cl.map_shared_rank(v.x + (size_t)rprev * a.L[l].ld, c - 1);
  };
  auto xup_of = [&](int l, const CtView<T>& v, int rows) -> const T* {
    if (c == P - 1) return v.x + (size_t)(rows + 1) * a.L[l].ld;
    return cl.map_shared_rank(v.x + (size_t)a.L[l].ld, c + 1);
  };

  // ---- down: distributed levels
  for (int l = 0; l < nd; ++l) {
    const CtLevel<T>& L = a.L[l];
    const CtView<T> v = ct_view(sm, L);
    const int J0 = a.J0[l][c], rows = a.J0[l][c + 1] - J0;
    const T* xdn = xdn_of(l, v);
    const T* xup = xup_of(l, v, rows);
    for (int s = 0; s < nu; ++s) {
      ct_half(v, L.nI, L.ld, J0, rows, xdn, xup, L.half_log2, 0);
      cl.sync();
      ct_half(v, L.nI, L.ld, J0, rows, xdn, xup, L.half_log2, 1);
      cl.sync();
    }
    if (l + 1 < nd) {
      const CtLevel<T>& C = a.L[l + 1];
      ct_restrict(v, L, J0, rows, xdn, xup, ct_view(sm, C), C, a.J0[l + 1][c], a.J0[l + 1][c + 1] - a.J0[l + 1][c]);
      __syncthreads();
    } else {
      // Bottom distributed level: residual of the own rows, then every CTA
      // averages the whole next level's right-hand side from all stripes.
      T* res = sm + a.res_off;
      const int lg = L.full_log2, tpr = 1 << lg, groups = kCtThreads >> lg;
      const int g = threadIdx.x >> lg, sl = threadIdx.x & (tpr - 1);
      for (int lr = 1 + g; lr <= rows; lr += groups)
        for (int i = sl; i < L.nI; i += tpr)  // black residuals are zero after the black half sweep
          res[(size_t)lr * L.ld + i + 1] = ((i + J0 + lr - 1) & 1) ? (T)0 : ct_residual(v, L.ld, lr, rows, i + 1, xdn, xup);
      cl.sync();
      const CtLevel<T>& C = a.L[l + 1];
      const CtView<T> cv = ct_view(sm, C);
      for (int u = threadIdx.x; u < C.nI * C.nJ; u += kCtThreads) {
        const int Jc = u / C.nI, I = u - Jc * C.nI;
        T acc = 0;
        for (int bb = 0; bb < 2; ++bb) {
          const int J = 2 * Jc + bb;
          if (J >= L.nJ) continue;
          const int o = owner[J];
          const T* rrow = cl.map_shared_rank(res + (size_t)(J - a.J0[l][o] + 1) * L.ld, o);
          for (int aa = 0; aa < 2; ++aa) {
            const int i = 2 * I + aa;
            if (i < L.nI) acc += rrow[i + 1];
          }
        }
        cv.b[(size_t)(Jc + 1) * C.ld + I + 1] = (T)0.25 * acc;
      }
      __syncthreads();
    }
  }

  // ---- local levels, identical in every CTA
  for (int l = nd; l < nl - 1; ++l) {
    const CtLevel<T>& L = a.L[l];
    const CtView<T> v = ct_view(sm, L);
    const T* z0 = v.x;
    const T* z1 = v.x + (size_t)(L.nJ + 1) * L.ld;
    for (int s = 0; s < nu; ++s) {
      ct_half(v, L.nI, L.ld, 0, L.nJ, z0, z1, L.half_log2, 0);
      __syncthreads();
      ct_half(v, L.nI, L.ld, 0, L.nJ, z0, z1, L.half_log2, 1);
      __syncthreads();
    }
    const CtLevel<T>& C = a.L[l + 1];
    ct_restrict(v, L, 0, L.nJ, z0, z1, ct_view(sm, C), C, 0, C.nJ);
    __syncthreads();
  }
  {
    // Dense coarse solve: b gathered into cell order (bc), then 16 threads per
    // row, 4 terms each, fixed-order tree sum.  (Not the residual buffer: other
    // CTAs may still be reading it.)
    const CtLevel<T>& C = a.L[nl - 1];
    const CtView<T> v = ct_view(sm, C);
    const int n = C.nI * C.nJ;
    const T* ai = sm + a.ainv_off;
    T* bc = sm + a.bc_off;
    const int r = threadIdx.x >> 4, part = threadIdx.x & 15;
    int cr = 0, cc = 0;  // cell of row r
    if (r < n) {
      cr = r / C.nI;
      cc = r - cr * C.nI;
    }
    if (threadIdx.x < (unsigned)n) {
      const int jj = threadIdx.x / C.nI, ii = threadIdx.x - jj * C.nI;
      bc[threadIdx.x] = v.b[(size_t)(jj + 1) * C.ld + ii + 1];
    }
    __syncthreads();
    T acc = 0;
    if (r < n)
      for (int m = part; m < n; m += 16) acc += ai[(size_t)r * n + m] * bc[m];
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (r < n && part == 0) v.x[(size_t)(cr + 1) * C.ld + cc + 1] = acc;
    __syncthreads();
  }
  for (int l = nl - 2; l >= nd; --l) {
    const CtLevel<T>& L = a.L[l];
    const CtView<T> v = ct_view(sm, L);
    const T* z0 = v.x;
    const T* z1 = v.x + (size_t)(L.nJ + 1) * L.ld;
    ct_prolong(v, L, 0, L.nJ, ct_view(sm, a.L[l + 1]), a.L[l + 1], 0);
    __syncthreads();
    for (int s = 0; s < nu; ++s) {
      ct_half(v, L.nI, L.ld, 0, L.nJ, z0, z1, L.half_log2, 1);
      __syncthreads();
      ct_half(v, L.nI, L.ld, 0, L.nJ, z0, z1, L.half_log2, 0);
      __syncthreads();
    }
  }

  // ---- up: distributed levels
  for (int l = nd - 1; l >= 0; --l) {
    const CtLevel<T>& L = a.L[l];
    const CtView<T> v = ct_view(sm, L);
    const int J0 = a.J0[l][c], rows = a.J0[l][c + 1] - J0;
    const CtLevel<T>& C = a.L[l + 1];
    const int cJ0 = l + 1 < nd ? a.J0[l + 1][c] : 0;
    ct_prolong(v, L, J0, rows, ct_view(sm, C), C, cJ0);
    cl.sync();  // neighbours read the corrected boundary rows
    const T* xdn = xdn_of(l, v);
    const T* xup = xup_of(l, v, rows);
    for (int s = 0; s < nu; ++s) {
      ct_half(v, L.nI, L.ld, J0, rows, xdn, xup, L.half_log2, 1);
      cl.sync();
      ct_half(v, L.nI, L.ld, J0, rows, xdn, xup, L.half_log2, 0);
      if (s + 1 < nu) cl.sync();
      else __syncthreads();
    }
  }

  // ---- write the top level's own rows; r.z when the top level is the finest
  {
    const CtLevel<T>& L = a.L[0];
    const CtView<T> v = ct_view(sm, L);
    const int J0 = nd > 0 ? a.J0[0][c] : 0;
    const int rows = nd > 0 ? a.J0[0][c + 1] - J0 : (c == 0 ? L.nJ : 0);
    double acc = 0.0;
    for (int u = threadIdx.x; u < rows * L.nI; u += kCtThreads) {
      const int lr = u / L.nI + 1, i = u - (lr - 1) * L.nI;
      const size_t q = (size_t)lr * L.ld + i + 1;
      L.x[(size_t)(J0 + lr) * L.ld + i + 1] = v.x[q];
      if (a.sc) acc += (double)v.b[q] * (double)v.x[q];
    }
    if (a.sc) {
      acc = block_sum(acc);
      if (threadIdx.x == 0) rz_part = acc;
      cl.sync();
      if (c == 0 && threadIdx.x == 0) {
        double rz = 0.0;
        for (int o = 0; o < P; ++o) rz += *cl.map_shared_rank(&rz_part, o);
        publish_rz(a.sc, rz);
      }
    }
  }
  cl.sync();  // no CTA leaves while a neighbour may still read its shared memory
}
