// Streaming red-black smoother: one thread block marches up a strip of 64 columns,
// row by row, with the 2*NS half sweeps of one V-cycle side pipelined over its warps.
//
// Included by gb2d_solver.cu inside its anonymous namespace (uses Level, Acc,
// diag_of, last_block_sum, publish_rz, pdl_enter from there).
//
// Why: the tiled smoother stages a window with a 2NS-cell halo on every side and
// re-sweeps shrinking windows between block barriers, about 7 instructions per cell
// and half sweep.  Here the vertical halo is paid once per segment of S rows instead
// of once per tile, the horizontal halo is 2NS columns per 64, and every update is
// one cell's five multiply-adds with its operands in shared memory.
//
// Pipeline.  Lane k owns the columns cs + 2k and cs + 2k + 1 of the strip
// [cs, cs + 64); in every half sweep exactly one of them has the sweep's colour.
// Warp w (w = 0 .. 2NS-1) performs half sweep w + 1, and at step t it updates row
// t - 2(w + 1).  Half sweep s of row r reads half sweep s - 1 of rows r - 1, r and
// r + 1 (the other colour); those ran at steps r + 2s - 3 .. r + 2s - 1, before the
// block barrier that ends every step.  Rows written in one step (t - 2, t - 4, ...)
// are never the neighbour rows read in that step (odd offsets), so the warps of a
// step are independent.  The update is the tiled kernel's expression on the same
// operands, so the results are bit-identical.  x of the rows in flight lives in a
// 16-row shared-memory ring; the coefficients b, 1/dg, cx, cy (and after the
// coarse correction x and the coarse x) in a 32-row ring filled by cp.async AHEAD
// rows before they are needed, each warp copying one array.  Cells outside the
// domain are staged as zero, the value of every wall-face conductance.
//
// Pre-smoothing starts from x = 0; one more warp forms the residual of the red
// cells from the final x (the black residuals are zero after the last black half
// sweep) and averages each coarse cell's fine cells into the coarse right-hand
// side.  Post-smoothing starts from x plus the prolonged coarse correction; on the
// finest level it also reduces r.z.
//
// Validity: after 2NS half sweeps a cell is exact when its 2NS neighbours on each
// side were loaded, so a strip outputs its middle 64 - 4NS columns (pre-smoothing,
// whose residual needs one more, its middle 62 - 4NS, starting on an even column
// so that each coarse cell's fine cells are complete), and a segment of S output
// rows processes S + 4NS (+2 for the residual) rows.  Strips and segments overlap
// in their halos; each output cell is written by one block.

namespace st {

constexpr int W = 64;       // columns of one strip
constexpr int XRING = 16;   // rows of x in flight (shared memory)
constexpr int CRING = 32;   // rows of coefficients in flight (shared memory)
constexpr int AHEAD = 12;   // rows staged ahead of the one entering the pipeline

template <bool POST>
struct Arr {
  static constexpr int N = POST ? 6 : 4;  // b, 1/dg, cx, cy [, x, coarse x]
};
constexpr int kB = 0, kId = 1, kCx = 2, kCy = 3, kXa = 4, kXc = 5;

template <int NS, bool POST>
struct Geo {
  static constexpr int WARPS = POST ? 2 * NS : 2 * NS + 1;  // half-sweep warps [+ the residual warp]
  static constexpr int LEFT = POST ? 2 * NS : 2 * NS + 1;   // halo columns left of the first output column
  static constexpr int OUT = POST ? W - 4 * NS : W - 2 - 4 * NS;  // output columns per strip
  static constexpr int BELOW = LEFT;                          // rows processed below the first output row
  static constexpr int EXTRA = POST ? 4 * NS : 4 * NS + 2;    // rows processed beyond the S output rows
  static constexpr int DRAIN = POST ? 4 * NS : 4 * NS + 2;    // steps after the last row enters
};

template <typename T, int NS, bool POST>
constexpr size_t smem_bytes() {
  return sizeof(T) * ((size_t)CRING * Arr<POST>::N * W + (size_t)XRING * W);
}

template <int BYTES>
__device__ __forceinline__ void cp_async_n(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Staging of one array for one lane: its two columns ca, ca + 1 of row r, zero
// outside the domain.  ain / bin: the columns are inside [0, nI).  VEC: the two
// columns are one aligned copy (the level's row length is even).
template <typename T, bool VEC>
__device__ __forceinline__ void stage_pair(T* d, const T* g, bool rin, bool ain, bool bin) {
  if (VEC && rin && ain && bin) {
    cp_async_n<2 * sizeof(T)>(d, g);
  } else {
    if (rin && ain)
      cp_async_n<sizeof(T)>(d, g);
    else
      d[0] = T(0);
    if (rin && bin)
      cp_async_n<sizeof(T)>(d + 1, g + 1);
    else
      d[1] = T(0);
  }
}

// Everything a warp role needs, computed once per block.
template <typename T>
struct StCtx {
  Level<T> L, C;
  T* xout;
  T* cring;
  T* xring;
  int lane, ca, cb, rs, r0, r1, nrows, nsteps;
  bool ain, bin, out_a, out_b;
};

// The step loop, one body for every warp (a warp's role is a runtime value, so
// the code stays small enough for the instruction cache).  role < 2NS: half sweep
// role + 1 (the last one also writes the finished rows); role == 2NS
// (pre-smoothing): residual and restriction.  Row rs + k lives in coefficient slot
// k mod CRING and x slot k mod XRING.  The loop is unrolled by two so that every
// row parity is a compile-time value; each warp passes the block barrier once per
// step.
template <typename T, int NS, bool POST, bool VEC>
__device__ __forceinline__ void stream_loop(const StCtx<T>& c, int role, Acc<T>& acc, bool rz) {
  using G = Geo<NS, POST>;
  constexpr int NA = Arr<POST>::N, ROW = NA * W;
  constexpr int RS_ODD = POST ? 0 : 1;  // rs = r0 - BELOW with r0 even
  constexpr int MAXA = (NA + G::WARPS - 1) / G::WARPS;
  const int lane = c.lane;
  // This warp's staged arrays: their source at column ca of row rs + AHEAD, advanced
  // by one row per step (the coarse correction is addressed per row instead).
  const T* gsrc[MAXA];
  int aoff[MAXA];
#pragma unroll
  for (int m = 0; m < MAXA; ++m) {
    const int a = role + m * G::WARPS;
    aoff[m] = a < NA ? a * W + 2 * lane : -1;
    const T* src = a == kB ? c.L.b : a == kId ? c.L.idg : a == kCx ? c.L.cx : a == kCy ? c.L.cy : c.L.x;
    gsrc[m] = src + (long long)(c.ca + 1) + (long long)(c.rs + AHEAD + 1) * c.L.ld;
  }
  const int s = role + 1;  // half sweep of a sweeping role
  const int color = POST ? (s & 1) : ((s - 1) & 1);  // red first from zero, black first after the correction
  T qacc = T(0);
  for (int i0 = 0; i0 < c.nsteps; i0 += 2) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = i0 + h;  // step: row rs + i enters the pipeline
      cp_wait<AHEAD - 1>();
      asm volatile("bar.sync 0;" ::: "memory");  // row rs + i staged everywhere; the previous step done everywhere
      {
        const int k = i + AHEAD, r = c.rs + k;
        if (k <= c.nrows) {  // one row beyond the last: its cy is the last row's top face
          T* row = c.cring + (size_t)(k & (CRING - 1)) * ROW;
          const bool rin = r >= 0 && r < c.L.nJ;
#pragma unroll
          for (int m = 0; m < MAXA; ++m) {
            if (aoff[m] < 0) continue;
            T* d = row + aoff[m];
            if (POST && aoff[m] - 2 * lane == kXc * W) {  // the coarse correction (piecewise-constant prolongation)
              const T* g = c.C.x + (long long)((r >> 1) + 1) * c.C.ld + 1;
              if (rin && c.ain)
                cp_async_n<sizeof(T)>(d, g + (c.ca >> 1));
              else
                d[0] = T(0);
              if (rin && c.bin)
                cp_async_n<sizeof(T)>(d + 1, g + (c.cb >> 1));
              else
                d[1] = T(0);
            } else {
              stage_pair<T, VEC>(d, gsrc[m], rin, c.ain, c.bin);
            }
            gsrc[m] += c.L.ld;
          }
        }
        cp_commit();
      }
      if (role == 0 && i < c.nrows) {  // x of row rs + i before the sweeps
        const T* R = c.cring + (size_t)(i & (CRING - 1)) * ROW + 2 * lane;
        T* X = c.xring + (size_t)(i & (XRING - 1)) * W + 2 * lane;
        if (POST) {
          X[0] = R[kXa * W] + R[kXc * W];
          X[1] = R[kXa * W + 1] + R[kXc * W + 1];
        } else {
          X[0] = X[1] = T(0);
        }
      }
      if (role < 2 * NS) {
        const int k = i - 2 * s;  // row rs + k: its parity is that of rs + h
        if (k >= 0 && k < c.nrows) {
          // Cell (col, r) has colour (col + r) & 1; ca is odd, cb = ca + 1 even.
          const int col = 2 * lane + (((RS_ODD + h) & 1) == color ? 1 : 0);
          T* X0 = c.xring + (size_t)(k & (XRING - 1)) * W;
          const T* Xm = c.xring + (size_t)((k - 1) & (XRING - 1)) * W;
          const T* Xp = c.xring + (size_t)((k + 1) & (XRING - 1)) * W;
          const T* C0 = c.cring + (size_t)(k & (CRING - 1)) * ROW;
          const T* C1 = c.cring + (size_t)((k + 1) & (CRING - 1)) * ROW;
          const int cl = col > 0 ? col - 1 : 0, cr = col < W - 1 ? col + 1 : W - 1;  // strip edges: halo, any value
          X0[col] = gs_update(C0[kB * W + col], C0[kCx * W + col], X0[cl], C0[kCx * W + cr], X0[cr], C0[kCy * W + col], Xm[col],
                              C1[kCy * W + col], Xp[col], C0[kId * W + col]);
          if (s == 2 * NS) {  // row rs + k is final: write it (and, after the correction, add its r.z)
            const int r = c.rs + k;
            if (r >= c.r0 && r < c.r1 && r < c.L.nJ) {
              __syncwarp();
              T* dst = c.xout + (size_t)(r + 1) * c.L.ld + 1;
              const T xa = X0[2 * lane], xb = X0[2 * lane + 1];
              if (c.out_a) dst[c.ca] = xa;
              if (c.out_b) dst[c.cb] = xb;
              if (POST && rz) {
                if (c.out_a) acc.add(C0[kB * W + 2 * lane] * xa);
                if (c.out_b) acc.add(C0[kB * W + 2 * lane + 1] * xb);
              }
            }
          }
        }
      } else if (!POST) {
        // Residual of row q = rs + k (its final x: rows q - 1 .. q + 1), restricted by row
        // pairs: coarse cell (I, J) averages the red cells (2I, 2J) and (2I + 1, 2J + 1),
        // in that order.
        const int k = i - 4 * NS - 2;  // q has the parity of rs + h
        if (k >= 0 && k < c.nrows - 1) {
          const int q = c.rs + k;
          const bool even = ((RS_ODD + h) & 1) == 0;
          const int col = even ? 2 * lane + 1 : 2 * lane;  // red: cb on even rows, ca on odd rows
          const bool inside = q >= 0 && q < c.L.nJ && (even ? c.bin : c.ain);
          const T* X0 = c.xring + (size_t)(k & (XRING - 1)) * W;
          const T* Xm = c.xring + (size_t)((k - 1) & (XRING - 1)) * W;
          const T* Xp = c.xring + (size_t)((k + 1) & (XRING - 1)) * W;
          const T* C0 = c.cring + (size_t)(k & (CRING - 1)) * ROW;
          const T* C1 = c.cring + (size_t)((k + 1) & (CRING - 1)) * ROW;
          const int cl = col > 0 ? col - 1 : 0, cr = col < W - 1 ? col + 1 : W - 1;
          const T res = gs_residual(C0[kB * W + col], diag_of(C0[kId * W + col]), X0[col], C0[kCx * W + col], X0[cl], C0[kCx * W + cr],
                                    X0[cr], C0[kCy * W + col], Xm[col], C1[kCy * W + col], Xp[col]);
          const T rv = inside ? res : T(0);
          if (even) {
            qacc = T(0);
            qacc += rv;
          } else {
            qacc += __shfl_down_sync(0xffffffffu, rv, 1);  // the next lane's ca is this lane's cb + 1
            const int I = c.cb >> 1, J = q >> 1;
            if (c.out_b && q > c.r0 && q < c.r1 && I < c.C.nI && J < c.C.nJ)
              c.C.b[(size_t)(I + 1) + (size_t)(J + 1) * c.C.ld] = T(0.25) * qacc;
          }
        }
      }
    }
  }
}

}  // namespace st

// One V-cycle side on one level (see the comment at the top of this file).  One
// block per (strip, segment).  POST = false: NS sweeps red first from x = 0, x to
// xout, the coarse right-hand side to C.b.  POST = true: x = L.x + prolonged C.x,
// NS sweeps black first, x to xout; with part_rz (the finest level) r.z is reduced
// and beta published.  S: output rows per segment (even); nsteps: steps per block,
// even, at least S + 2 EXTRA.
template <typename T, int NS, bool POST, bool VEC>
__global__ void __launch_bounds__(32 * st::Geo<NS, POST>::WARPS)
    k_stream(Level<T> L, Level<T> C, T* __restrict__ xout, int S, int nsteps, double* __restrict__ part_rz,
             unsigned* __restrict__ counter, Scalars* sc, const int* __restrict__ done) {
  using namespace st;
  using G = Geo<NS, POST>;
  constexpr int NA = Arr<POST>::N;
  pdl_enter();
  if (*done) return;
  extern __shared__ unsigned char smem_raw[];
  StCtx<T> c;
  c.L = L;
  c.C = C;
  c.xout = xout;
  c.cring = reinterpret_cast<T*>(smem_raw);
  c.xring = c.cring + (size_t)CRING * NA * W;
  const int warp = threadIdx.x >> 5;
  c.lane = threadIdx.x & 31;
  // Output columns [out0 + k OUT, out0 + (k+1) OUT) for strip k: pre from 0, post from -1.
  const int out0 = POST ? -1 : 0;
  const int nstrips = (L.nI - out0 + G::OUT - 1) / G::OUT;
  const int strip = blockIdx.x % nstrips, seg = blockIdx.x / nstrips;
  const int olo = out0 + strip * G::OUT, ohi = olo + G::OUT;  // output columns
  const int cs = olo - G::LEFT;                                // first column of the strip (odd)
  c.ca = cs + 2 * c.lane;
  c.cb = c.ca + 1;
  c.r0 = seg * S;
  c.r1 = c.r0 + S;
  c.rs = c.r0 - G::BELOW;
  c.nrows = S + G::EXTRA;
  c.nsteps = nsteps;
  c.ain = c.ca >= 0 && c.ca < L.nI;
  c.bin = c.cb >= 0 && c.cb < L.nI;
  c.out_a = c.ain && c.ca >= olo && c.ca < ohi;
  c.out_b = c.bin && c.cb >= olo && c.cb < ohi;

  for (int q = threadIdx.x; q < XRING * W; q += blockDim.x) c.xring[q] = T(0);
  // Prologue: rows rs .. rs + AHEAD - 1 (AHEAD < S + EXTRA for every admissible S),
  // warp w copying arrays w, w + WARPS, ...
  for (int k = 0; k < AHEAD; ++k) {
    const int r = c.rs + k;
    const bool rin = r >= 0 && r < L.nJ;
    for (int a = warp; a < NA; a += G::WARPS) {
      T* d = c.cring + (size_t)k * NA * W + a * W + 2 * c.lane;
      if (POST && a == kXc) {
        const T* g = C.x + (long long)((r >> 1) + 1) * C.ld + 1;
        if (rin && c.ain)
          cp_async_n<sizeof(T)>(d, g + (c.ca >> 1));
        else
          d[0] = T(0);
        if (rin && c.bin)
          cp_async_n<sizeof(T)>(d + 1, g + (c.cb >> 1));
        else
          d[1] = T(0);
      } else {
        const T* src = a == kB ? L.b : a == kId ? L.idg : a == kCx ? L.cx : a == kCy ? L.cy : L.x;
        stage_pair<T, VEC>(d, src + (long long)(c.ca + 1) + (long long)(r + 1) * L.ld, rin, c.ain, c.bin);
      }
    }
    cp_commit();
  }
  Acc<T> acc;
  stream_loop<T, NS, POST, VEC>(c, warp, acc, part_rz != nullptr);
  cp_wait<0>();
  if (POST && part_rz) {
    double rz;
    if (last_block_sum(acc, part_rz, gridDim.x, counter, &rz)) publish_rz(sc, rz);
  }
}
