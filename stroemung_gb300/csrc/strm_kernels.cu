// sm_103a kernels of the NaSt2D timestep and the CUDA graph that chains them.
//
// Step graph (red-black solve):
//   bc_kernel        cluster of 8 CTAs: step bookkeeping + compiled boundary program
//   fg_rhs_kernel    tiled F, G (+ their boundary restore) and RHS, one pass
//   fg_rhs32_kernel  the same with the stencil in FP32 (mixed precision)
//   WHILE(solve not done), exact arithmetic:
//     pcopy_kernel     boundary pressure copy
//     sor_color_kernel red cells, then black cells
//     residual_kernel  residual norm, stop test, sets the WHILE condition
//   fast arithmetic: pcopy_kernel, sor_red_res_kernel (first red pass), then
//   WHILE(solve not done):
//     sor_black_res_kernel  the previous iteration's norm and stop test
//                           (every block, from the red pass's partials),
//                           then the black pass + the residual of the black
//                           cells; saves the boundary values, copies the
//                           black-coloured ones for the next iteration
//     sor_red_res_kernel    red pass of the next iteration + this one's
//                           residual of the red cells (partial sums);
//                           copies the red-coloured boundary cells
//   sor_unred_kernel, sor_rollback_kernel  undo the next iteration's red
//                        pass and copy
//   mixed precision: FP32 sweeps with FP64 refinement (see the mixed solve)
//   prange_kernel    pressure range when the solve ran out of iterations
//   velocity_kernel  velocity update + restore + max|u|,|v| + speed range + time
//
// Every kernel that follows a reference formula uses the reference's operation
// order; the translation unit is compiled with --fmad=false so no multiply-add
// is fused behind our back, and divisions by step constants use xdiv (correctly
// rounded), so results are bit-identical to the reference's FP64 arithmetic.
#include <cooperative_groups.h>
#include <float.h>
#include <stddef.h>

#include <algorithm>
#include <atomic>
#include <initializer_list>

#include "strm_kernels.cuh"

namespace cg = cooperative_groups;

namespace strm {

#define OFF(x, y) ((size_t)(x) * (size_t)g.pitch + (size_t)(y))

// Tiles of the grid-stride reduction kernels: 8 rows x 64 columns, 256
// threads, two neighbouring columns per thread.
constexpr int RT_X = 8;
constexpr int RT_Y = 64;

__device__ __forceinline__ double sqd(double x) { return x * x; }

// Programmatic dependent launch (PTX griddepcontrol, sm_90 and later).  A
// colour pass of the FAST solve's loop body starts with both: the trigger
// lets the next pass's blocks be placed on the SMs as this pass's blocks
// finish, instead of after the whole grid has completed and the next launch
// has been processed; the wait holds each block until the previous pass has
// completed and its writes are visible.  Launched without a programmatic
// edge (eager launches, graphs built without them) both do nothing.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Load of a buffer that other CTAs of the same launch may have written
// earlier (the persistent batch solve): COH reads it at L2 (ld.global.cg),
// never through the read-only path; otherwise a plain load.
template <bool COH, typename T>
__device__ __forceinline__ T ldv(const T *p) {
  if constexpr (COH) return __ldcg(p);
  else return *p;
}

// Thread coordinates of a work group of (32 x 8)-style tile kernels: the
// whole CTA of a graph kernel (bar 0: __syncthreads), or one 256-thread half
// of a 512-thread persistent CTA (its own named barrier 1 + half).
struct Thr {
  int tx, ty;      // within the group
  int dx, dy;      // the group's extent (blockDim of a graph kernel)
  int tid;         // tx + dx * ty
  int half;        // 0 or 1
  int bar;         // 0: __syncthreads; 1, 2: named barrier of 256 threads
};
__device__ __forceinline__ Thr thr_cta() {
  Thr t;
  t.tx = threadIdx.x;
  t.ty = threadIdx.y;
  t.dx = blockDim.x;
  t.dy = blockDim.y;
  t.tid = threadIdx.x + blockDim.x * threadIdx.y;
  t.half = 0;
  t.bar = 0;
  return t;
}
__device__ __forceinline__ void gsync(const Thr &t) {
  if (t.bar == 0) __syncthreads();
  else asm volatile("bar.sync %0, 256;" ::"r"(t.bar) : "memory");
}

// ------------------------------------------------------------------------
// reductions
// ------------------------------------------------------------------------

struct OpMax { __device__ double operator()(double a, double b) const { return fmax(a, b); } };
struct OpMin { __device__ double operator()(double a, double b) const { return fmin(a, b); } };
struct OpAdd { __device__ double operator()(double a, double b) const { return a + b; } };

// Deterministic block reduction (fixed shuffle tree, then warp 0).
template <typename Op>
__device__ double block_reduce(double v, Op op, double identity) {
  __shared__ double sm[32];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nthreads = blockDim.x * blockDim.y;
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = tid & 31, w = tid >> 5, nw = (nthreads + 31) >> 5;
  __syncthreads();
  if (lane == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < nw ? sm[lane] : identity;
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;  // valid in thread 0
}

// Returns true in the block that finished last; its reads of the other
// blocks' partials are then ordered after their writes.  Every caller has
// its partials written by thread 0, so thread 0 alone fences: before its
// ticket (release of this block's partials) and, in the last block, after
// it (acquire of the others'); the barrier then orders the block's reads.
// The other threads' stores (field updates) need no fence here: nothing
// reads them before the kernel ends.
__device__ __forceinline__ bool last_block_done(unsigned int *counter) {
  __shared__ bool am_last;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    const bool last = atomicAdd(counter, 1u) == gridDim.x * gridDim.y - 1;
    if (last) __threadfence();
    am_last = last;
  }
  __syncthreads();
  return am_last;
}

// Sums a partials array in a fixed order (deterministic).
template <typename Op>
__device__ double reduce_partials(const double *part, int n, int stride, int idx, Op op,
                                  double identity) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nthreads = blockDim.x * blockDim.y;
  double v = identity;
  for (int k = tid; k < n; k += nthreads) v = op(v, __ldcg(part + (size_t)k * stride + idx));
  return block_reduce(v, op, identity);
}

// ------------------------------------------------------------------------
// K0: classification (src/grid/mod.rs:202-235, 270-332)
// ------------------------------------------------------------------------

__global__ void classify_kernel(uint8_t *flags, Geom g, unsigned long long *fluid_count,
                                long long *first_bad) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y * blockDim.y + threadIdx.y;
  double fluid = 0.0;
  if (x < g.nx && y < g.ny) {
    const size_t o = OFF(x, y);
    const uint8_t k = kind_of(flags[o]);
    if (k == K_FLUID) {
      fluid = 1.0;
      flags[o] = 0;
    } else {
      // Only kind bits of the neighbours are read; edge bits are written
      // concurrently by their own threads.
      const int left = x > 0 && kind_of(flags[OFF(x - 1, y)]) == K_FLUID;
      const int right = x < g.nx - 1 && kind_of(flags[OFF(x + 1, y)]) == K_FLUID;
      const int up = y > 0 && kind_of(flags[OFF(x, y - 1)]) == K_FLUID;
      const int down = y < g.ny - 1 && kind_of(flags[OFF(x, y + 1)]) == K_FLUID;
      const int code = (left << 3) | (right << 2) | (up << 1) | down;
      int e = -1;
      switch (code) {
        case 0x0: e = E_NONE; break;
        case 0x8: e = E_W; break;
        case 0xA: e = E_NW; break;
        case 0x2: e = E_N; break;
        case 0x6: e = E_NE; break;
        case 0x4: e = E_E; break;
        case 0x5: e = E_SE; break;
        case 0x1: e = E_S; break;
        case 0x9: e = E_SW; break;
        default: break;
      }
      if (e < 0) {
        atomicMin(first_bad, (long long)x * g.ny + y);
        e = E_NONE;
      }
      flags[o] = (uint8_t)(k | (e << 3));
    }
  }
  double s = block_reduce(fluid, OpAdd(), 0.0);
  if (threadIdx.x == 0 && threadIdx.y == 0 && s > 0.0)
    atomicAdd(fluid_count, (unsigned long long)s);
}

// ------------------------------------------------------------------------
// K1: step bookkeeping + boundary program (src/grid/mod.rs:414-651)
// ------------------------------------------------------------------------

// The boundary pass is sequential in the reference, and later cells read
// values earlier cells wrote.  The host compiles it into independent
// (target <- expression of pre-pass values) entries; here every entry is
// first evaluated against the pre-pass fields, then a cluster-wide barrier
// orders all those reads before any write.
constexpr int BC_CLUSTER = 8;
constexpr int BC_THREADS = 1024;

__device__ __forceinline__ void step_begin(StepState *st, const Consts &c, double tau,
                                           double delt, unsigned int itermax) {
  double dt = delt;
  if (tau > 0.0) {
    // tau * min(Re/2 / (1/dx^2 + 1/dy^2), dx/max|u|, dy/max|v|)
    const double dt_re = (0.5 * c.re) / ((1.0 / (c.dx * c.dx)) + (1.0 / (c.dy * c.dy)));
    const double dt_u = c.dx / st->umax;
    const double dt_v = c.dy / st->vmax;
    dt = tau * fmin(dt_re, fmin(dt_u, dt_v));
  }
  st->dt = dt;
  st->sor_iters = 0;
  st->converged = 0;
  st->exhausted = (itermax == 0) ? 1u : 0u;
  st->ns = 0.0;
  st->body_count = 0;
  st->overrun = 0;
  st->hist_n = 0;
  st->replay = 0;
}

__global__ void __cluster_dims__(BC_CLUSTER, 1, 1) __launch_bounds__(BC_THREADS)
    bc_kernel(double *u, double *v, double *ru, double *rv, const BcEntry *e, double *val,
              int n, StepState *st, Consts c, double tau, double delt, unsigned int itermax,
              int begin_step) {
  if (begin_step && blockIdx.x == 0 && threadIdx.x == 0) step_begin(st, c, tau, delt, itermax);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = gridDim.x * blockDim.x;
  for (int k = tid; k < n; k += nt) {
    const BcEntry en = e[k];
    const int field = (int)(en.target >> 56);
    const double *srcf = (field & 1) ? v : u;
    const double s = (en.op == 0) ? 0.0 : srcf[en.src];
    double r;
    switch (en.op) {
      case 0: r = en.c; break;
      case 1: r = s; break;
      case 2: r = -s; break;
      default: r = en.c - s; break;
    }
    val[k] = r;
  }
  cg::this_cluster().sync();
  for (int k = tid; k < n; k += nt) {
    const long long t = e[k].target;
    const int field = (int)(t >> 56);
    const long long off = t & ((1LL << 56) - 1);
    double *dst = field == 0 ? u : field == 1 ? v : field == 2 ? ru : rv;
    dst[off] = val[k];
  }
}

// ------------------------------------------------------------------------
// K2: F, G, their restore, RHS (src/simulation.rs:122-214, src/math.rs)
// ------------------------------------------------------------------------

__device__ __forceinline__ double d_du2dx(double u_im1, double u_i, double u_ip1, const Consts &c) {
  const double inner_left1 = sqd(u_i + u_ip1);
  const double inner_right1 = sqd(u_im1 + u_i);
  const double left_side = inner_left1 - inner_right1;
  const double inner_left2 = fabs(u_i + u_ip1) * (u_i - u_ip1);
  const double inner_right2 = fabs(u_im1 + u_i) * (u_im1 - u_i);
  return xdiv(left_side + (c.gamma * (inner_left2 - inner_right2)), c.four_dx, c.r_four_dx);
}

__device__ __forceinline__ double d_duvdx(double u_i_j, double u_i_j_p1, double u_i_m1_j,
                                          double u_i_m1_j_p1, double v_i_j, double v_i_p1_j,
                                          double v_i_m1_j, const Consts &c) {
  const double inner_left1 = (u_i_j + u_i_j_p1) * (v_i_j + v_i_p1_j);
  const double inner_right1 = (u_i_m1_j + u_i_m1_j_p1) * (v_i_m1_j + v_i_j);
  const double left_side = inner_left1 - inner_right1;
  const double inner_left2 = fabs(u_i_j + u_i_j_p1) * (v_i_j - v_i_p1_j);
  const double inner_right2 = fabs(u_i_m1_j + u_i_m1_j_p1) * (v_i_m1_j - v_i_j);
  return xdiv(left_side + (c.gamma * (inner_left2 - inner_right2)), c.four_dx, c.r_four_dx);
}

__device__ __forceinline__ double d_duvdy(double u_i_j, double u_i_j_m1, double u_i_j_p1,
                                          double v_i_j, double v_i_j_m1, double v_i_p1_j,
                                          double v_i_p1_j_m1, const Consts &c) {
  const double inner_left1 = (v_i_j + v_i_p1_j) * (u_i_j + u_i_j_p1);
  const double inner_right1 = (v_i_j_m1 + v_i_p1_j_m1) * (u_i_j_m1 + u_i_j);
  const double left_side = inner_left1 - inner_right1;
  const double inner_left2 = fabs(v_i_j + v_i_p1_j) * (u_i_j - u_i_j_p1);
  const double inner_right2 = fabs(v_i_j_m1 + v_i_p1_j_m1) * (u_i_j_m1 - u_i_j);
  return xdiv(left_side + (c.gamma * (inner_left2 - inner_right2)), c.four_dy, c.r_four_dy);
}

__device__ __forceinline__ double d_dv2dy(double v_i_j_m1, double v_i_j, double v_i_j_p1,
                                          const Consts &c) {
  const double inner_left1 = sqd(v_i_j + v_i_j_p1);
  const double inner_right1 = sqd(v_i_j_m1 + v_i_j);
  const double left_side = inner_left1 - inner_right1;
  const double inner_left2 = fabs(v_i_j + v_i_j_p1) * (v_i_j - v_i_j_p1);
  const double inner_right2 = fabs(v_i_j_m1 + v_i_j) * (v_i_j_m1 - v_i_j);
  return xdiv(left_side + (c.gamma * (inner_left2 - inner_right2)), c.four_dy, c.r_four_dy);
}

__device__ __forceinline__ double d_laplacian(double e_i_j, double e_i_j_m1, double e_i_j_p1,
                                              double e_i_m1_j, double e_i_p1_j, const Consts &c) {
  const double d2edx2 = xdiv(e_i_p1_j - (2. * e_i_j) + e_i_m1_j, c.dx2, c.r_dx2);
  const double d2edy2 = xdiv(e_i_j_p1 - (2. * e_i_j) + e_i_j_m1, c.dy2, c.r_dy2);
  return d2edx2 + d2edy2;
}

constexpr int FG_TX = 16;  // output rows per tile
constexpr int FG_TY = 64;  // output columns per tile
constexpr int FG_THREADS = 256;

// One tile of F/G/RHS.  Shared tiles:
//   su, sv  rows x0-2 .. x0+TX,   cols y0-2 .. y0+TY     (u, v)
//   sfl     rows x0-1 .. x0+TX,   cols y0-1 .. y0+TY     (flags)
//   sF, sG  rows x0-1 .. x0+TX-1, cols y0-1 .. y0+TY-1   (F, G)
__global__ void __launch_bounds__(FG_THREADS)
    fg_rhs_kernel(const double *__restrict__ u, const double *__restrict__ v, double *f,
                  double *gg, double *__restrict__ rhs, const uint8_t *__restrict__ flags, Geom g,
                  Consts c, const StepState *st) {
  __shared__ double su[FG_TX + 3][FG_TY + 3];
  __shared__ double sv[FG_TX + 3][FG_TY + 3];
  __shared__ double sF[FG_TX + 1][FG_TY + 1];
  __shared__ double sG[FG_TX + 1][FG_TY + 1];
  __shared__ uint8_t sfl[FG_TX + 2][FG_TY + 2];
  __shared__ double s_dt, s_rdt;

  const int tid = threadIdx.x;
  const int y0 = blockIdx.x * FG_TY;
  const int x0 = blockIdx.y * FG_TX;
  if (tid == 0) {
    s_dt = st->dt;
    s_rdt = 1.0 / s_dt;
  }
  for (int k = tid; k < (FG_TX + 3) * (FG_TY + 3); k += FG_THREADS) {
    const int i = k / (FG_TY + 3), j = k % (FG_TY + 3);
    const int x = x0 - 2 + i, y = y0 - 2 + j;
    const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
    su[i][j] = in ? u[OFF(x, y)] : 0.0;
    sv[i][j] = in ? v[OFF(x, y)] : 0.0;
  }
  for (int k = tid; k < (FG_TX + 2) * (FG_TY + 2); k += FG_THREADS) {
    const int i = k / (FG_TY + 2), j = k % (FG_TY + 2);
    const int x = x0 - 1 + i, y = y0 - 1 + j;
    const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
    sfl[i][j] = in ? flags[OFF(x, y)] : (uint8_t)0;
  }
  __syncthreads();
  const double dt = s_dt;

  for (int k = tid; k < (FG_TX + 1) * (FG_TY + 1); k += FG_THREADS) {
    const int i = k / (FG_TY + 1), j = k % (FG_TY + 1);
    const int x = x0 - 1 + i, y = y0 - 1 + j;
    double Fv = 0.0, Gv = 0.0;
    if (x >= 0 && y >= 0 && x < g.nx && y < g.ny) {
      const uint8_t fc = sfl[i][j];
      const bool bc = is_bnd(fc);
      const bool keepF = bc || (x + 1 < g.nx && is_bnd(sfl[i + 1][j]));
      const bool keepG = bc || (y + 1 < g.ny && is_bnd(sfl[i][j + 1]));
      const bool interior = x >= 1 && y >= 1 && x <= g.nx - 2 && y <= g.ny - 2;
      // window: w(a, b) = field(x + a, y + b) = s[i + 1 + a][j + 1 + b]
      const int si = i + 1, sj = j + 1;
      if (keepF) {
        Fv = su[si][sj];
      } else if (interior) {
        const double u01 = su[si - 1][sj], u10 = su[si][sj - 1], u11 = su[si][sj];
        const double u12 = su[si][sj + 1], u21 = su[si + 1][sj];
        const double v10 = sv[si][sj - 1], v11 = sv[si][sj], v20 = sv[si + 1][sj - 1];
        const double v21 = sv[si + 1][sj];
        const double lap = d_laplacian(u11, u10, u12, u01, u21, c);
        const double a = d_du2dx(u01, u11, u21, c);
        const double b = d_duvdy(u11, u10, u12, v11, v10, v21, v20, c);
        Fv = u11 + (dt * (xdiv(lap, c.re, c.r_re) - a - b));
      } else {
        Fv = f[OFF(x, y)];
      }
      if (keepG) {
        Gv = sv[si][sj];
      } else if (interior) {
        const double u01 = su[si - 1][sj], u02 = su[si - 1][sj + 1], u11 = su[si][sj];
        const double u12 = su[si][sj + 1];
        const double v01 = sv[si - 1][sj], v10 = sv[si][sj - 1], v11 = sv[si][sj];
        const double v12 = sv[si][sj + 1], v21 = sv[si + 1][sj];
        const double lap = d_laplacian(v11, v10, v12, v01, v21, c);
        const double a = d_duvdx(u11, u12, u01, u02, v11, v21, v01, c);
        const double b = d_dv2dy(v10, v11, v12, c);
        Gv = v11 + (dt * (xdiv(lap, c.re, c.r_re) - a - b));
      } else {
        Gv = gg[OFF(x, y)];
      }
      if (i >= 1 && j >= 1) {
        if (keepF || interior) f[OFF(x, y)] = Fv;
        if (keepG || interior) gg[OFF(x, y)] = Gv;
      }
    }
    sF[i][j] = Fv;
    sG[i][j] = Gv;
  }
  __syncthreads();

  for (int k = tid; k < FG_TX * FG_TY; k += FG_THREADS) {
    const int i = k / FG_TY, j = k % FG_TY;
    const int x = x0 + i, y = y0 + j;
    if (x >= 1 && y >= 1 && x < g.nx && y < g.ny) {
      const double a = xdiv(sF[i + 1][j + 1] - sF[i][j + 1], c.dx, c.r_dx);
      const double b = xdiv(sG[i + 1][j + 1] - sG[i + 1][j], c.dy, c.r_dy);
      rhs[OFF(x, y)] = xdiv(a + b, dt, s_rdt);
    }
  }
}

// F/G/RHS of the mixed-precision step: the tiles, boundary rules and
// restore of fg_rhs_kernel with the advection-diffusion stencil in FP32.
// Each u, v value of the tile is held as a pair of floats (hi = u rounded,
// lo = u - hi rounded), about 48 significant bits.  The stencil takes first
// and second differences of the hi parts first (exact for neighbouring
// values) and adds those of the lo parts, and forms the convective
// differences of products as (A - B) C + B (C - D), so that no FP32
// operation cancels a large value: the FP32 rounding is relative to the
// terms of the increment dt (lap/Re - d(u^2)/dx - d(uv)/dy), not to u.
// F = u + increment is formed in FP64; boundary values (F = u, G = v) are
// exact copies; the RHS takes FP64 differences of F and G (reciprocal
// multiplications).  The terms are the reference's (src/math.rs:19-174),
// rearranged.
struct Consts32F {
  float gamma, r_dx2, r_dy2, r_four_dx, r_four_dy, r_re;
};

struct HL {
  float h, l;
};

__device__ __forceinline__ HL hl_of(double x) {
  HL r;
  r.h = narrow(x);
  r.l = narrow(x - widen(r.h));
  return r;
}
// a - b
__device__ __forceinline__ float hl_dif(HL a, HL b) { return (a.h - b.h) + (a.l - b.l); }
// a + b
__device__ __forceinline__ float hl_sum(HL a, HL b) { return (a.h + b.h) + (a.l + b.l); }
// e - 2c + w
__device__ __forceinline__ float hl_d2(HL e, HL c, HL w) {
  return ((e.h - c.h) - (c.h - w.h)) + ((e.l - c.l) - (c.l - w.l));
}

// d(u^2)/dx (src/math.rs:19-33): a^2 - b^2 as (a - b)(a + b), a - b = u(i+1) - u(i-1)
__device__ __forceinline__ float f_du2dx(HL um1, HL u, HL up1, const Consts32F &k) {
  const float a = hl_sum(u, up1), b = hl_sum(um1, u);
  return (hl_dif(up1, um1) * (a + b) +
          k.gamma * (fabsf(a) * hl_dif(u, up1) - fabsf(b) * hl_dif(um1, u))) *
         k.r_four_dx;
}

// d(v^2)/dy (src/math.rs:136-150)
__device__ __forceinline__ float f_dv2dy(HL vm1, HL v, HL vp1, const Consts32F &k) {
  const float a = hl_sum(v, vp1), b = hl_sum(vm1, v);
  return (hl_dif(vp1, vm1) * (a + b) +
          k.gamma * (fabsf(a) * hl_dif(v, vp1) - fabsf(b) * hl_dif(vm1, v))) *
         k.r_four_dy;
}

// d(uv)/dy (src/math.rs:97-120): A C - B D as (A - B) C + B (C - D)
__device__ __forceinline__ float f_duvdy(HL u_ij, HL u_ijm1, HL u_ijp1, HL v_ij, HL v_ijm1,
                                         HL v_ip1j, HL v_ip1jm1, const Consts32F &k) {
  const float A = hl_sum(v_ij, v_ip1j), B = hl_sum(v_ijm1, v_ip1jm1);
  const float C = hl_sum(u_ij, u_ijp1);
  const float AmB = hl_dif(v_ij, v_ijm1) + hl_dif(v_ip1j, v_ip1jm1);
  const float CmD = hl_dif(u_ijp1, u_ijm1);
  return (AmB * C + B * CmD +
          k.gamma * (fabsf(A) * hl_dif(u_ij, u_ijp1) - fabsf(B) * hl_dif(u_ijm1, u_ij))) *
         k.r_four_dy;
}

// d(uv)/dx (src/math.rs:53-77)
__device__ __forceinline__ float f_duvdx(HL u_ij, HL u_ijp1, HL u_im1j, HL u_im1jp1, HL v_ij,
                                         HL v_ip1j, HL v_im1j, const Consts32F &k) {
  const float A = hl_sum(u_ij, u_ijp1), B = hl_sum(u_im1j, u_im1jp1);
  const float C = hl_sum(v_ij, v_ip1j);
  const float AmB = hl_dif(u_ij, u_im1j) + hl_dif(u_ijp1, u_im1jp1);
  const float CmD = hl_dif(v_ip1j, v_im1j);
  return (AmB * C + B * CmD +
          k.gamma * (fabsf(A) * hl_dif(v_ij, v_ip1j) - fabsf(B) * hl_dif(v_im1j, v_ij))) *
         k.r_four_dx;
}

// laplacian (src/math.rs:162-174)
__device__ __forceinline__ float f_laplacian(HL e, HL e_jm1, HL e_jp1, HL e_im1, HL e_ip1,
                                             const Consts32F &k) {
  return hl_d2(e_ip1, e, e_im1) * k.r_dx2 + hl_d2(e_jp1, e, e_jm1) * k.r_dy2;
}

__global__ void __launch_bounds__(FG_THREADS)
    fg_rhs32_kernel(const double *__restrict__ u, const double *__restrict__ v, double *f,
                    double *gg, double *__restrict__ rhs, const uint8_t *__restrict__ flags,
                    Geom g, Consts c, Consts32F k, const StepState *st) {
  __shared__ HL su[FG_TX + 3][FG_TY + 3];
  __shared__ HL sv[FG_TX + 3][FG_TY + 3];
  __shared__ double sF[FG_TX + 1][FG_TY + 1];
  __shared__ double sG[FG_TX + 1][FG_TY + 1];
  __shared__ uint8_t sfl[FG_TX + 2][FG_TY + 2];

  const int tid = threadIdx.x;
  const int y0 = blockIdx.x * FG_TY;
  const int x0 = blockIdx.y * FG_TX;
  const double dt = st->dt;
  const double rdt = 1.0 / dt;
  const float dt32 = (float)dt;
  const HL zero = {0.f, 0.f};
  for (int q = tid; q < (FG_TX + 3) * (FG_TY + 3); q += FG_THREADS) {
    const int i = q / (FG_TY + 3), j = q % (FG_TY + 3);
    const int x = x0 - 2 + i, y = y0 - 2 + j;
    const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
    su[i][j] = in ? hl_of(u[OFF(x, y)]) : zero;
    sv[i][j] = in ? hl_of(v[OFF(x, y)]) : zero;
  }
  for (int q = tid; q < (FG_TX + 2) * (FG_TY + 2); q += FG_THREADS) {
    const int i = q / (FG_TY + 2), j = q % (FG_TY + 2);
    const int x = x0 - 1 + i, y = y0 - 1 + j;
    const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
    sfl[i][j] = in ? flags[OFF(x, y)] : (uint8_t)0;
  }
  __syncthreads();

  for (int q = tid; q < (FG_TX + 1) * (FG_TY + 1); q += FG_THREADS) {
    const int i = q / (FG_TY + 1), j = q % (FG_TY + 1);
    const int x = x0 - 1 + i, y = y0 - 1 + j;
    double Fv = 0.0, Gv = 0.0;
    if (x >= 0 && y >= 0 && x < g.nx && y < g.ny) {
      const size_t o = OFF(x, y);
      const uint8_t fc = sfl[i][j];
      const bool bc = is_bnd(fc);
      const bool keepF = bc || (x + 1 < g.nx && is_bnd(sfl[i + 1][j]));
      const bool keepG = bc || (y + 1 < g.ny && is_bnd(sfl[i][j + 1]));
      const bool interior = x >= 1 && y >= 1 && x <= g.nx - 2 && y <= g.ny - 2;
      const int si = i + 1, sj = j + 1;
      if (keepF) {
        Fv = u[o];
      } else if (interior) {
        const HL u01 = su[si - 1][sj], u10 = su[si][sj - 1], u11 = su[si][sj];
        const HL u12 = su[si][sj + 1], u21 = su[si + 1][sj];
        const HL v10 = sv[si][sj - 1], v11 = sv[si][sj], v20 = sv[si + 1][sj - 1];
        const HL v21 = sv[si + 1][sj];
        const float inc = dt32 * (f_laplacian(u11, u10, u12, u01, u21, k) * k.r_re -
                                  f_du2dx(u01, u11, u21, k) -
                                  f_duvdy(u11, u10, u12, v11, v10, v21, v20, k));
        Fv = u[o] + widen(inc);
      } else {
        Fv = f[o];
      }
      if (keepG) {
        Gv = v[o];
      } else if (interior) {
        const HL u01 = su[si - 1][sj], u02 = su[si - 1][sj + 1], u11 = su[si][sj];
        const HL u12 = su[si][sj + 1];
        const HL v01 = sv[si - 1][sj], v10 = sv[si][sj - 1], v11 = sv[si][sj];
        const HL v12 = sv[si][sj + 1], v21 = sv[si + 1][sj];
        const float inc = dt32 * (f_laplacian(v11, v10, v12, v01, v21, k) * k.r_re -
                                  f_duvdx(u11, u12, u01, u02, v11, v21, v01, k) -
                                  f_dv2dy(v10, v11, v12, k));
        Gv = v[o] + widen(inc);
      } else {
        Gv = gg[o];
      }
      if (i >= 1 && j >= 1) {
        if (keepF || interior) f[o] = Fv;
        if (keepG || interior) gg[o] = Gv;
      }
    }
    sF[i][j] = Fv;
    sG[i][j] = Gv;
  }
  __syncthreads();

  for (int q = tid; q < FG_TX * FG_TY; q += FG_THREADS) {
    const int i = q / FG_TY, j = q % FG_TY;
    const int x = x0 + i, y = y0 + j;
    if (x >= 1 && y >= 1 && x < g.nx && y < g.ny) {
      const double a = sF[i + 1][j + 1] - sF[i][j + 1];
      const double b = sG[i + 1][j + 1] - sG[i + 1][j];
      rhs[OFF(x, y)] = fma(a, c.r_dx, b * c.r_dy) * rdt;
    }
  }
}

static Consts32F consts32f_of(const Consts &c) {
  Consts32F k;
  k.gamma = (float)c.gamma;
  k.r_dx2 = (float)c.r_dx2;
  k.r_dy2 = (float)c.r_dy2;
  k.r_four_dx = (float)c.r_four_dx;
  k.r_four_dy = (float)c.r_four_dy;
  k.r_re = (float)c.r_re;
  return k;
}

// F/G/RHS of the FAST arithmetic (fused multiply-adds, reciprocal
// multiplies): the reference's terms (src/simulation.rs:122-214,
// src/math.rs:19-174) regrouped as face fluxes, each computed once per face
// instead of once per neighbouring cell.  With k1 = dt/(Re dx^2),
// k2 = dt/(Re dy^2), k3 = dt/(4 dx), k4 = dt/(4 dy):
//
//   PX(x,y) = k1 DX + k3 (SX^2 + gamma |SX| DX),  SX = u(x)+u(x+1), DX = u(x)-u(x+1)
//   PY(x,y) = k2 C + k4 (A B + gamma |A| C),       A = v(x,y)+v(x+1,y),
//                                                  B = u(x,y)+u(x,y+1), C = u(x,y)-u(x,y+1)
//   QX(x,y) = k1 C' + k3 (A B + gamma |B| C'),     C' = v(x,y)-v(x+1,y)
//   QY(x,y) = k2 DY + k3' (SY^2 + gamma |SY| DY),  SY = v(y)+v(y+1), DY = v(y)-v(y+1)
//   F = u + (PX(x-1,y) - PX(x,y)) + (PY(x,y-1) - PY(x,y))
//   G = v + (QX(x-1,y) - QX(x,y)) + (QY(x,y-1) - QY(x,y))
//   RHS = (F(x,y) - F(x-1,y)) / (dx dt) + (G(x,y) - G(x,y-1)) / (dy dt)
//
// In real arithmetic this is the reference's F (u + dt (lap/Re - du2dx -
// duvdy)), G and RHS term for term; only the rounding differs.  About 37
// FP64 operations per cell instead of ~140: the FP64 pipe, about 1.75
// operations per clock per SM on this part, bounds the kernel.  Boundary
// copies (F = u, G = v), the cells left unchanged and the RHS region are
// those of fg_rhs_kernel.  Tiles of 32 x 32 cells; the fluxes of a tile and
// its one-face halo live in dynamic shared memory.
constexpr int FF_T = 32;
constexpr int FF_THREADS = 256;
struct FastFgSmem {
  double u[FF_T + 3][FF_T + 3];  // rows x0-2 .. x0+32, cols y0-2 .. y0+32
  double v[FF_T + 3][FF_T + 3];
  double px[FF_T + 2][FF_T];     // rows x0-2 .. x0+31, cols y0 .. y0+31
  double py[FF_T + 1][FF_T + 1]; // rows x0-1 .. x0+31, cols y0-1 .. y0+31
  double qx[FF_T + 1][FF_T + 1]; // rows x0-1 .. x0+31, cols y0-1 .. y0+31
  double qy[FF_T][FF_T + 2];     // rows x0 .. x0+31,   cols y0-2 .. y0+31
  double f[FF_T + 1][FF_T];      // rows x0-1 .. x0+31, cols y0 .. y0+31
  double g[FF_T][FF_T + 1];      // rows x0 .. x0+31,   cols y0-1 .. y0+31
  uint8_t fl[FF_T + 2][FF_T + 2];  // rows x0-1 .. x0+32, cols y0-1 .. y0+32
  double k[8];                   // k1 k2 k3 k4 k3*gamma k4*gamma c1 c2
};

__global__ void __launch_bounds__(FF_THREADS, 3)
    fg_rhs_fast_kernel(const double *__restrict__ u, const double *__restrict__ v, double *f,
                       double *gg, double *__restrict__ rhs, const uint8_t *__restrict__ flags,
                       Geom g, Consts c, const StepState *st) {
  extern __shared__ __align__(16) unsigned char ff_raw[];
  FastFgSmem &S = *reinterpret_cast<FastFgSmem *>(ff_raw);
  const int tid = threadIdx.x;
  const int y0 = blockIdx.x * FF_T;
  const int x0 = blockIdx.y * FF_T;
  if (tid == 0) {
    const double dt = st->dt;
    const double rdt = 1.0 / dt;
    S.k[0] = dt * (c.r_re * c.r_dx2);
    S.k[1] = dt * (c.r_re * c.r_dy2);
    S.k[2] = dt * c.r_four_dx;
    S.k[3] = dt * c.r_four_dy;
    S.k[4] = S.k[2] * c.gamma;
    S.k[5] = S.k[3] * c.gamma;
    S.k[6] = c.r_dx * rdt;
    S.k[7] = c.r_dy * rdt;
  }
  constexpr int W = FF_T + 3;
  for (int q = tid; q < W * W; q += FF_THREADS) {
    const int i = q / W, j = q % W;
    const int x = x0 - 2 + i, y = y0 - 2 + j;
    const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
    S.u[i][j] = in ? u[OFF(x, y)] : 0.0;
    S.v[i][j] = in ? v[OFF(x, y)] : 0.0;
  }
  constexpr int WF = FF_T + 2;
  for (int q = tid; q < WF * WF; q += FF_THREADS) {
    const int i = q / WF, j = q % WF;
    const int x = x0 - 1 + i, y = y0 - 1 + j;
    const bool in = x >= 0 && x < g.nx && y >= 0 && y < g.ny;
    S.fl[i][j] = in ? flags[OFF(x, y)] : (uint8_t)0;
  }
  __syncthreads();
  const double k1 = S.k[0], k2 = S.k[1], k3 = S.k[2], k4 = S.k[3];
  const double k3g = S.k[4], k4g = S.k[5];

  // x faces of u: PX at rows x0-2 .. x0+31 (u row index i = row - x0 + 2)
  for (int q = tid; q < (FF_T + 2) * FF_T; q += FF_THREADS) {
    const int i = q / FF_T, j = q % FF_T;
    const double a = S.u[i][j + 2], b = S.u[i + 1][j + 2];
    const double sx = a + b, dx_ = a - b;
    S.px[i][j] = fma(dx_, fma(k3g, fabs(sx), k1), (k3 * sx) * sx);
  }
  // y faces of u and x faces of v (they share A B): rows x0-1 .. x0+31,
  // cols y0-1 .. y0+31
  for (int q = tid; q < (FF_T + 1) * (FF_T + 1); q += FF_THREADS) {
    const int i = q / (FF_T + 1), j = q % (FF_T + 1);
    const double u0 = S.u[i + 1][j + 1], uS = S.u[i + 1][j + 2];
    const double v0 = S.v[i + 1][j + 1], vE = S.v[i + 2][j + 1];
    const double A = v0 + vE, B = u0 + uS, C = u0 - uS, Cp = v0 - vE;
    const double AB = A * B;
    S.py[i][j] = fma(C, fma(k4g, fabs(A), k2), k4 * AB);
    S.qx[i][j] = fma(Cp, fma(k3g, fabs(B), k1), k3 * AB);
  }
  // y faces of v: rows x0 .. x0+31, cols y0-2 .. y0+31
  for (int q = tid; q < FF_T * (FF_T + 2); q += FF_THREADS) {
    const int i = q / (FF_T + 2), j = q % (FF_T + 2);
    const double a = S.v[i + 2][j], b = S.v[i + 2][j + 1];
    const double sy = a + b, dy_ = a - b;
    S.qy[i][j] = fma(dy_, fma(k4g, fabs(sy), k2), (k4 * sy) * sy);
  }
  __syncthreads();

  // F at rows x0-1 .. x0+31, cols y0 .. y0+31
  for (int q = tid; q < (FF_T + 1) * FF_T; q += FF_THREADS) {
    const int i = q / FF_T, j = q % FF_T;
    const int x = x0 - 1 + i, y = y0 + j;
    double Fv = 0.0;
    if (x >= 0 && x < g.nx && y < g.ny) {
      const bool keep = is_bnd(S.fl[i][j + 1]) || (x + 1 < g.nx && is_bnd(S.fl[i + 1][j + 1]));
      const bool interior = x >= 1 && y >= 1 && x <= g.nx - 2 && y <= g.ny - 2;
      const double u0 = S.u[i + 1][j + 2];
      if (keep) {
        Fv = u0;
      } else if (interior) {
        Fv = u0 + ((S.px[i][j] - S.px[i + 1][j]) + (S.py[i][j] - S.py[i][j + 1]));
      } else {
        Fv = f[OFF(x, y)];
      }
      if (i >= 1 && (keep || interior)) f[OFF(x, y)] = Fv;
    }
    S.f[i][j] = Fv;
  }
  // G at rows x0 .. x0+31, cols y0-1 .. y0+31
  for (int q = tid; q < FF_T * (FF_T + 1); q += FF_THREADS) {
    const int i = q / (FF_T + 1), j = q % (FF_T + 1);
    const int x = x0 + i, y = y0 - 1 + j;
    double Gv = 0.0;
    if (x < g.nx && y >= 0 && y < g.ny) {
      const bool keep = is_bnd(S.fl[i + 1][j]) || (y + 1 < g.ny && is_bnd(S.fl[i + 1][j + 1]));
      const bool interior = x >= 1 && y >= 1 && x <= g.nx - 2 && y <= g.ny - 2;
      const double v0 = S.v[i + 2][j + 1];
      if (keep) {
        Gv = v0;
      } else if (interior) {
        Gv = v0 + ((S.qx[i][j] - S.qx[i + 1][j]) + (S.qy[i][j] - S.qy[i][j + 1]));
      } else {
        Gv = gg[OFF(x, y)];
      }
      if (j >= 1 && (keep || interior)) gg[OFF(x, y)] = Gv;
    }
    S.g[i][j] = Gv;
  }
  __syncthreads();
  const double c1 = S.k[6], c2 = S.k[7];
  for (int q = tid; q < FF_T * FF_T; q += FF_THREADS) {
    const int i = q / FF_T, j = q % FF_T;
    const int x = x0 + i, y = y0 + j;
    if (x >= 1 && y >= 1 && x < g.nx && y < g.ny)
      rhs[OFF(x, y)] = fma(S.g[i][j + 1] - S.g[i][j], c2, (S.f[i + 1][j] - S.f[i][j]) * c1);
  }
}

// ------------------------------------------------------------------------
// K3: pressure solve (src/simulation.rs:239-285, src/grid/mod.rs:343-412)
// ------------------------------------------------------------------------

__device__ __forceinline__ void pcopy_one(double *p, const PCopy &pc, int pitch) {
  const long long o = pc.off;
  switch (pc.edge) {
    case E_N: p[o] = p[o - 1]; break;
    case E_NE: p[o] = (p[o - 1] + p[o + pitch]) * 0.5; break;
    case E_E: p[o] = p[o + pitch]; break;
    case E_SE: p[o] = (p[o + 1] + p[o + pitch]) * 0.5; break;
    case E_S: p[o] = p[o + 1]; break;
    case E_SW: p[o] = (p[o + 1] + p[o - pitch]) * 0.5; break;
    case E_W: p[o] = p[o - pitch]; break;
    case E_NW: p[o] = (p[o - 1] + p[o - pitch]) * 0.5; break;
    default: break;
  }
}

__global__ void pcopy_kernel(double *p, const PCopy *pc, int n, int pitch) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) pcopy_one(p, pc[k], pitch);
}

// SOR update of one fluid cell in the reference's operation order
// (src/simulation.rs:260-271).  The fast-arithmetic passes form it from the
// residual instead (sor_red_res_kernel, sor_black_res_kernel).
__device__ __forceinline__ double sor_update(double p, double pw, double pe, double pn, double ps,
                                             double r, const Consts &c) {
  return (c.one_minus_w * p) +
         c.middle * (xdiv(pe + pw, c.dx2, c.r_dx2) + xdiv(ps + pn, c.dy2, c.r_dy2) - r);
}

// Residual of one interior cell (src/math.rs:176-186).
template <bool EXACT>
__device__ __forceinline__ double residual_of(double p, double pw, double pe, double pn, double ps,
                                              double r, const Consts &c) {
  if (EXACT) {
    const double part1 = xdiv((pe - p) - (p - pw), c.dx2, c.r_dx2);
    const double part2 = xdiv((ps - p) - (p - pn), c.dy2, c.r_dy2);
    return part1 + part2 - r;
  } else {
    // (pe + pw)/dx^2 + (ps + pn)/dy^2 - 2 (1/dx^2 + 1/dy^2) p - rhs: 5 FP64 operations
    return fma(pe + pw, c.r_dx2, fma(ps + pn, c.r_dy2, fma(-c.two_r_sum, p, -r)));
  }
}

// One colour of an exact-arithmetic red-black sweep: cells with
// (x + y) % 2 == color.  Thread (tx, ty) owns the cell pair y = 2*(y-pair),
// x = row; it updates the member of the pair that has the colour.
__global__ void __launch_bounds__(256)
    sor_color_kernel(double *__restrict__ p, const double *__restrict__ rhs,
                     const uint8_t *__restrict__ flags, Geom g, Consts c, int color) {
  const int x = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int y = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + ((x + color) & 1);
  if (x > g.nx - 2 || y < 1 || y > g.ny - 2) return;
  const size_t o = OFF(x, y);
  if (flags[o] != 0) return;
  const double pc = p[o], pw = p[o - g.pitch], pe = p[o + g.pitch];
  const double pn = p[o - 1], ps = p[o + 1];
  p[o] = sor_update(pc, pw, pe, pn, ps, rhs[o], c);
}

// The colour passes of the FAST red-black solve stride over the virtual
// blocks of the colour-pass layout (gx x gy blocks of kRedBlock threads, a
// thread per cell pair, as sor_color_kernel) with a fixed number of resident
// blocks, each reducing once.  A thread takes kPassUnroll virtual blocks at
// a time and issues every load of those cells (class byte, the five
// pressures, rhs) before it uses one: the pressure loads do not wait for the
// class byte, and several cells' loads are in flight.  The FP64 pipe is the
// bound; memory latency is what keeps it idle.  The passes run two blocks
// of 256 threads per SM (kPassBlocksPerSm; up to 128 registers a thread)
// with five cells per batch.  Measured per 2000-iteration step against
// that: four blocks per SM (64 registers) with three cells 1.7 % slower and
// with four 11 % slower (spilling), three blocks with four cells even,
// three with five 3.6 % slower, two with six 0.9 % slower.
constexpr int kPassUnroll = 5;
constexpr int kPassBlocksPerSm = 2;

struct PassCells {
  size_t o[kPassUnroll];
  bool ok[kPassUnroll];
};

// The cells of colour `color` a thread owns in virtual blocks vb0,
// vb0 + stride, ...; cells outside the interior get a harmless address (an
// interior cell) and ok = false.
__device__ __forceinline__ PassCells pass_cells(int vb0, int stride, int nvb, int gx, int color,
                                                const Geom &g) {
  PassCells pc;
#pragma unroll
  for (int u = 0; u < kPassUnroll; ++u) {
    const int vb = vb0 + u * stride;
    const int x = 1 + (vb / gx) * blockDim.y + threadIdx.y;
    const int y = 2 * ((vb % gx) * blockDim.x + threadIdx.x) + ((x + color) & 1);
    pc.ok[u] = vb < nvb && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2;
    pc.o[u] = pc.ok[u] ? OFF(x, y) : OFF(1, 1);
  }
  return pc;
}

// Block sums of the FAST solve passes: the threads' values go to shared
// memory and warp 0 adds them (nt/32 - 1 additions per lane, then the
// shuffle tree).  That is 12 FP64 additions by one warp per block of 256
// threads, where block_reduce's shuffle tree costs 5 in every warp: the
// passes are bound by the FP64 pipe.  Fixed order (deterministic); at most
// 256 threads, a multiple of 32; the sums are valid in thread 0.
template <bool TWO>
__device__ __forceinline__ void block_sum_pass(double &a, double &b) {
  __shared__ double sa[256];
  __shared__ double sb[TWO ? 256 : 1];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int nt = blockDim.x * blockDim.y;
  sa[tid] = a;
  if (TWO) sb[tid] = b;
  __syncthreads();
  if (tid < 32) {
    double s = sa[tid], s1 = TWO ? sb[tid] : 0.0;
    for (int k = tid + 32; k < nt; k += 32) {
      s += sa[k];
      if (TWO) s1 += sb[k];
    }
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      if (TWO) s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    a = s;
    b = s1;
  }
}

// Boundary pressure copy of one listed cell (src/grid/mod.rs:343-412).
__device__ __forceinline__ void pcopy_cell(double *p, size_t o, int edge, int pitch) {
  PCopy e;
  e.off = (long long)o;
  e.edge = edge;
  pcopy_one(p, e, pitch);
}

// The black pass of a FAST red-black iteration fused with the residual of the
// black fluid cells.  With t = (pe+pw)/dx^2 + (ps+pn)/dy^2 - rhs from the red
// values and r0 = t - 2(1/dx^2+1/dy^2) p the residual before the update, the
// update is p_new = p + omega r0 / (2(1/dx^2+1/dy^2)) (the reference update,
// src/simulation.rs:260-271, rearranged), and since the four (red) neighbours
// are final the cell's residual afterwards is r = (1-omega) r0.  The pass
// sums r0^2 (and r0 when MEAN_FREE) and scales the sums by (1-omega)^2 (and
// 1-omega): 7 FP64 operations per cell.
//
// In the solve (nbl > 0) the pass also works through the boundary-cell list
// bl (black-coloured cells, (x + y) odd, in bl[0..nbl_b), then red-coloured
// ones):
//   * the residual of iteration k of every black-coloured non-fluid interior
//     cell (when ALL: the norm over every interior cell).  Its stencil is
//     the cell and four red-coloured cells, none of which this pass changes;
//   * the boundary copy of iteration k+1 (src/grid/mod.rs:343-412; only
//     when k < itermax, as the copy runs only before another iteration):
//     every copied cell's value of iteration k is saved into pw (read by the
//     red pass for the stale residual, restored by the rollback), and the
//     black-coloured ones get their new values here.  A copied cell's
//     sources are its fluid neighbours, of the other colour: red cells,
//     final since the red pass; and no black cell's stencil holds a
//     black-coloured cell, so nothing in this pass reads what the copy
//     writes.  The cell's own residual is read before the copy, by the
//     same thread.
// The sums of the black fluid cells and of the list go to partials_b.
//
// The stop test of iteration k happens here, at the start of the black pass
// of iteration k+1, not in a last block of the red pass that the whole grid
// would wait for: the red pass of iteration k+1 (which summed iteration k's
// red residuals, the black pass's partials folded into its own) has
// completed, so every block adds its nred partials in the same order, gets
// the same norm and the same decision, and returns at once when the solve
// stops; block 0 records the iteration (sor_iters, ns, the history, the
// stop flags, the WHILE condition).  it = st->pass_iter (written by the red
// pass, 0 before the solve's first black pass: nothing to decide).
template <bool MEAN_FREE>
__device__ __forceinline__ void sum_partials_passes(const double *pr, int n, double &s2,
                                                    double &s1);
__device__ __forceinline__ bool stop_rule_of(double ns, const Consts &c, double ns0,
                                             double ns_start, int strict);

template <bool IN_GRAPH, bool MEAN_FREE, bool ALL>
__global__ void __launch_bounds__(256, kPassBlocksPerSm)
    sor_black_res_kernel(double *__restrict__ p, double *__restrict__ pw,
                         const double *__restrict__ rhs, const uint8_t *__restrict__ flags,
                         Geom g, Consts c, double *__restrict__ partials_b, int gx, int nvb,
                         const BCell *__restrict__ bl, int nbl_b, int nbl, StepState *st,
                         unsigned int itermax, const double *partials_r, int nred, int strict,
                         cudaGraphConditionalHandle h) {
  pdl_trigger();
  pdl_wait();
  // a later iteration of a WHILE body whose solve has stopped: nothing to do
  // (block 0 of this pass may set the flags while another block reads them:
  // either way that block ends as its own decision below would end it)
  if (st->converged | st->exhausted) return;
  const unsigned int it = st->pass_iter;
  // The first batch's loads go out before the stop test and the boundary
  // list, so that their latency overlaps the test's sums: they depend on
  // neither (the list's copy writes black-coloured boundary cells, and no
  // black fluid cell's stencil holds one).
  const int stride = kPassUnroll * gridDim.x;
  int vb0 = blockIdx.x;
  PassCells cells;
  unsigned int f[kPassUnroll];
  double pc[kPassUnroll], pe[kPassUnroll], pwv[kPassUnroll], pn[kPassUnroll],
      ps[kPassUnroll], rh[kPassUnroll];
  auto load_batch = [&]() {
    cells = pass_cells(vb0, gridDim.x, nvb, gx, 1, g);
#pragma unroll
    for (int u = 0; u < kPassUnroll; ++u) {
      const size_t o = cells.o[u];
      f[u] = flags[o];
      pc[u] = p[o];
      pe[u] = p[o + g.pitch];
      pwv[u] = p[o - g.pitch];
      ps[u] = p[o + 1];
      pn[u] = p[o - 1];
      rh[u] = rhs[o];
    }
  };
  load_batch();
  if (it > 0) {
    double s2, s1;
    sum_partials_passes<MEAN_FREE>(partials_r, nred, s2, s1);
    __shared__ int stop;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      const double q = st->pass_inv_cells;
      const double ns = MEAN_FREE ? (s2 - s1 * (s1 * q)) * q : s2 * q;
      const bool done = stop_rule_of(ns, c, st->ns0, st->ns_start, strict);
      stop = done || it >= itermax;
      if (blockIdx.x == 0) {
        st->sor_iters = it;
        st->ns = ns;
        hist_push(st, it, ns);
        st->nonfinite = !isfinite(ns);
        if (done) st->converged = 1;
        else if (it >= itermax) st->exhausted = 1;
        if (IN_GRAPH && stop) cudaGraphSetConditional(h, 0);
      }
    }
    __syncthreads();
    if (stop) return;
  }
  double accl = 0.0;  // residuals of the listed cells (ALL only, never MEAN_FREE)
  {
    const int nt = blockDim.x * blockDim.y;
    int i = blockIdx.x * nt + threadIdx.y * blockDim.x + threadIdx.x;
    if (i < nbl) {
      // this pass is iteration it+1; the copy of iteration it+2 runs only
      // when there is one
      const bool copy = it + 1 < itermax;
      for (; i < nbl; i += gridDim.x * nt) {
        const BCell e = bl[i];
        const size_t o = e.off;
        if (i < nbl_b) {
          if (ALL && (e.flags & BC_RES)) {
            const double r = residual_of<false>(p[o], p[o - g.pitch], p[o + g.pitch], p[o - 1],
                                                p[o + 1], rhs[o], c);
            accl = fma(r, r, accl);
          }
          if (e.flags & BC_COPY) {
            pw[o] = p[o];
            if (copy) pcopy_cell(p, o, e.edge, g.pitch);
          }
        } else if (e.flags & BC_COPY) {
          pw[o] = p[o];
        }
      }
    }
  }
  double acc = 0.0, acc1 = 0.0;
  for (;;) {
#pragma unroll
    for (int u = 0; u < kPassUnroll; ++u) {
      if (!cells.ok[u] || f[u] != 0) continue;
      const double t = fma(pe[u] + pwv[u], c.r_dx2, fma(ps[u] + pn[u], c.r_dy2, -rh[u]));
      const double r0 = fma(-c.two_r_sum, pc[u], t);
      p[cells.o[u]] = fma(c.middle, r0, pc[u]);
      acc = fma(r0, r0, acc);
      if (MEAN_FREE) acc1 += r0;
    }
    vb0 += stride;
    if (vb0 >= nvb) break;
    load_batch();
  }
  const double q = c.one_minus_w;
  double a = fma(acc, q * q, accl), a1 = acc1 * q;
  block_sum_pass<MEAN_FREE>(a, a1);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (MEAN_FREE) {
      partials_b[2 * blockIdx.x] = a;
      partials_b[2 * blockIdx.x + 1] = a1;
    } else {
      partials_b[blockIdx.x] = a;
    }
  }
}

// What a residual launch does once the norm is known.
enum : int { RES_SOLVE = 0, RES_NORM = 1, RES_NS0 = 2, RES_START = 3 };
// bits of the `strict` argument of the residual kernels
enum : int {
  STOP_STRICT = 1,      // stop only at ns < eps^2 (not at ns < the initial norm)
  STOP_FLUID_NORM = 2,  // sum the residual over fluid cells only (not every interior cell)
  STOP_MEAN_FREE = 4,   // with STOP_FLUID_NORM: remove the residual's mean over fluid cells
  STOP_RELATIVE = 8,    // stop at ns < eps^2 * (the norm the solve started from)
};

__device__ __forceinline__ bool stop_rule_of(double ns, const Consts &c, double ns0,
                                             double ns_start, int strict) {
  if (strict & STOP_RELATIVE) return ns < c.eps2 * ns_start;
  if (strict & STOP_STRICT) return ns < c.eps2;
  return (ns < ns0) || (ns < c.eps2);
}

__device__ __forceinline__ bool stop_rule(double ns, const Consts &c, const StepState *st,
                                          int strict) {
  return stop_rule_of(ns, c, st->ns0, st->ns_start, strict);
}

// The norm from the block sums: sum r^2 (and sum r when mean_free, stored
// interleaved), divided by fluid_cells; mean-free: (sum r^2 - (sum r)^2 / n) / n.
__device__ __forceinline__ double finish_norm(const double *partials, int nblocks,
                                              bool mean_free, double fluid_cells) {
  if (!mean_free) return reduce_partials(partials, nblocks, 1, 0, OpAdd(), 0.0) / fluid_cells;
  const double s2 = reduce_partials(partials, nblocks, 2, 0, OpAdd(), 0.0);
  const double s1 = reduce_partials(partials, nblocks, 2, 1, OpAdd(), 0.0);
  return (s2 - s1 * (s1 / fluid_cells)) / fluid_cells;
}

// The same over two partial arrays (the residual pass and the fused black pass).
__device__ __forceinline__ double finish_norm2(const double *pa, int na, const double *pb, int nb,
                                               bool mean_free, double fluid_cells) {
  const int st = mean_free ? 2 : 1;
  const double s2 = reduce_partials(pa, na, st, 0, OpAdd(), 0.0) +
                    reduce_partials(pb, nb, st, 0, OpAdd(), 0.0);
  if (!mean_free) return s2 / fluid_cells;
  const double s1 = reduce_partials(pa, na, 2, 1, OpAdd(), 0.0) +
                    reduce_partials(pb, nb, 2, 1, OpAdd(), 0.0);
  return (s2 - s1 * (s1 / fluid_cells)) / fluid_cells;
}

// Bookkeeping of one pressure iteration once its norm is known
// (src/simulation.rs:272-281): counts it, records the norm, applies the stop
// rule and ends the graph's WHILE loop at the stop or at itermax.
template <bool IN_GRAPH>
__device__ __forceinline__ void solve_iteration_done(StepState *st, double ns, const Consts &c,
                                                     int strict, unsigned int itermax,
                                                     cudaGraphConditionalHandle h) {
  const unsigned int it = st->sor_iters + 1;
  st->sor_iters = it;
  st->ns = ns;
  hist_push(st, it, ns);
  st->nonfinite = !isfinite(ns);
  const bool done = stop_rule(ns, c, st, strict);
  if (done) st->converged = 1;
  else if (it >= itermax) st->exhausted = 1;
  if (IN_GRAPH && (done || it >= itermax)) cudaGraphSetConditional(h, 0);
}

// Independent bound on a WHILE loop: the stop test ends it at iteration
// itermax at the latest; should that bookkeeping ever fail, this ends it two
// launches later and flags the step.
template <bool IN_GRAPH>
__device__ __forceinline__ void loop_guard(StepState *st, unsigned int itermax,
                                           cudaGraphConditionalHandle h) {
  if (IN_GRAPH && blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    const unsigned int launches = atomicAdd(&st->body_count, 1u) + 1;
    if (launches >= itermax + 2) {
      st->overrun = 1;
      cudaGraphSetConditional(h, 0);
    }
  }
}

// This thread's share of the residual sums over the block's tiles: sum r^2
// (and sum r when MEAN_FREE) over interior cells, fluid cells only when FLUID.
template <bool EXACT, bool FLUID, bool MEAN_FREE, bool SKIPB = false>
__device__ __forceinline__ void residual_sum(const double *__restrict__ p,
                                             const double *__restrict__ rhs,
                                             const uint8_t *__restrict__ flags, const Geom &g,
                                             const Consts &c, int tiles_y, int ntiles,
                                             double *acc_out, double *acc1_out) {
  double acc = 0.0, acc1 = 0.0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tx = t / tiles_y, ty = t % tiles_y;
    const int x = 1 + tx * RT_X + threadIdx.y;
    if (x > g.nx - 2) continue;
    const int yb = 1 + ty * RT_Y + 2 * threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int y = yb + q;
      if (y <= g.ny - 2) {
        const size_t o = OFF(x, y);
        if (FLUID && flags[o] != 0) continue;
        // black fluid cells: summed by the fused black pass
        if (SKIPB && flags[o] == 0 && ((x + y) & 1) == 1) continue;
        const double r = residual_of<EXACT>(p[o], p[o - g.pitch], p[o + g.pitch], p[o - 1],
                                            p[o + 1], rhs[o], c);
        acc = EXACT ? acc + sqd(r) : fma(r, r, acc);
        if (MEAN_FREE) acc1 += r;
      }
    }
  }
  *acc_out = acc;
  *acc1_out = acc1;
}

// Residual norm over every interior cell (src/simulation.rs:216-227), in
// grid-stride tiles; the last block to finish sums the per-block partials in
// a fixed order, divides by fluid_cells and applies the stop rule of
// src/simulation.rs:276-281 (mode RES_SOLVE), optionally ending the graph's
// WHILE loop.
template <bool EXACT, bool IN_GRAPH>
__global__ void __launch_bounds__(256)
    residual_kernel(const double *__restrict__ p, const double *__restrict__ rhs,
                    const uint8_t *__restrict__ flags, Geom g, Consts c, StepState *st,
                    double *partials, int tiles_y, int ntiles, cudaGraphConditionalHandle h,
                    unsigned int itermax, int strict, int mode, const double *partials_b,
                    int nbb) {
  const bool fluid_only = (strict & STOP_FLUID_NORM) != 0;
  const bool mean_free = fluid_only && (strict & STOP_MEAN_FREE) != 0;
  double acc = 0.0, acc1 = 0.0;
  // the reference's sum (every interior cell) keeps its own loop: the solve is
  // FP64-bound and pays for every extra operation.  With partials_b the black
  // fluid cells were summed by the fused black pass (sor_black_res_kernel).
  if (partials_b) {
    if (!fluid_only)
      residual_sum<EXACT, false, false, true>(p, rhs, flags, g, c, tiles_y, ntiles, &acc, &acc1);
    else if (!mean_free)
      residual_sum<EXACT, true, false, true>(p, rhs, flags, g, c, tiles_y, ntiles, &acc, &acc1);
    else
      residual_sum<EXACT, true, true, true>(p, rhs, flags, g, c, tiles_y, ntiles, &acc, &acc1);
  } else if (!fluid_only) {
    residual_sum<EXACT, false, false>(p, rhs, flags, g, c, tiles_y, ntiles, &acc, &acc1);
  } else if (!mean_free) {
    residual_sum<EXACT, true, false>(p, rhs, flags, g, c, tiles_y, ntiles, &acc, &acc1);
  } else {
    residual_sum<EXACT, true, true>(p, rhs, flags, g, c, tiles_y, ntiles, &acc, &acc1);
  }
  const double bsum = block_reduce(acc, OpAdd(), 0.0);
  if (mean_free) {
    const double bsum1 = block_reduce(acc1, OpAdd(), 0.0);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      partials[2 * blockIdx.x] = bsum;
      partials[2 * blockIdx.x + 1] = bsum1;
    }
  } else if (threadIdx.x == 0 && threadIdx.y == 0) {
    partials[blockIdx.x] = bsum;
  }
  loop_guard<IN_GRAPH>(st, itermax, h);
  if (!last_block_done(&st->counter)) return;
  const double ns = partials_b ? finish_norm2(partials, gridDim.x, partials_b, nbb, mean_free,
                                              st->fluid_cells)
                               : finish_norm(partials, gridDim.x, mean_free, st->fluid_cells);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    st->counter = 0;
    if (mode == RES_NS0) {
      st->ns0 = ns;
    } else if (mode == RES_START) {
      st->ns_start = ns;
      hist_push(st, 0u, ns);
    } else if (mode == RES_NORM) {
      st->aux = ns;
    } else {
      solve_iteration_done<IN_GRAPH>(st, ns, c, strict, itermax, h);
    }
  }
}

// ------------------------------------------------------------------------
// FAST red-black solve with the red residual taken from the next red pass.
//
// Iteration k ends with the norm of the residual after its black pass.  For
// a red fluid cell whose four neighbours are fluid, that residual is
// t - 2(1/dx^2+1/dy^2) p with t = (pe+pw)/dx^2 + (ps+pn)/dy^2 - rhs, read
// from the black values of iteration k and the red value p of iteration k:
// exactly what the red pass of iteration k+1 reads before it updates p to
// p + omega r / (2(1/dx^2+1/dy^2)) (the reference update, src/simulation.rs:
// 260-271, rearranged).  So the red pass of iteration k+1 sums iteration k's
// red residual and applies the stop test of k; the separate residual pass
// over the red cells disappears (its FP64 operations and its reads of p and
// rhs).  The boundary copy before iteration k+1 (src/grid/mod.rs:343-412)
// needs no launch of its own either.  A copied cell's sources are its fluid
// neighbours, all of the other colour, and a cell's stencil holds only
// cells of the other colour besides itself.  So the black pass of k copies
// the black-coloured boundary cells (red sources, final), which no black
// cell reads, and the red pass of k+1 the red-coloured ones (black sources,
// final), which no red cell reads; the black pass first saves every copied
// cell's value of k into pw.  The norm of iteration k reads the stale
// boundary values of k (the reference copies before each sweep): the black
// pass sums the black-coloured non-fluid interior cells before it copies
// them, and the red pass reads the copied cells in the stencils of the red
// fluid cells next to them (class 1) and of the red-coloured non-fluid
// interior cells from pw.  The stop itself: when iteration k stops the
// solve, the red pass and the copy of k+1 have run; the copy saved what it
// overwrote (in pw), and so did the red pass when omega is near 1; for
// other omega sor_unred_kernel inverts the red pass instead, and
// sor_rollback_kernel puts the saved values back, so the solve ends on
// iteration k's pressure, boundary values included.  Iteration
// k+1's red pass and copy run only when k < itermax.
// Per iteration: black pass (+ its residual, the save and half the copy)
// and red pass (+ the other half, the red residual and the stop test),
// instead of copy, red, black, residual.
// ------------------------------------------------------------------------

// The sum of the red pass's partials (each already holding the black
// pass's partial of the same block index), taken by every block of the
// next black pass before its cells: on the critical path of every
// iteration.  Each thread loads up to three entries at once and adds them
// as a tree, then a tree over the block (one shared-memory level, then one
// warp's additions and shuffles): 8 dependent additions.  Fixed order, so
// every block gets the same bits; blocks of 256 threads; entries past 768
// (grids above 3 blocks per thread) are added to the first slot.  s2 = sum
// r^2, s1 = sum r (when MEAN_FREE); valid in thread 0.
template <bool MEAN_FREE>
__device__ __forceinline__ void sum_partials_passes(const double *pr, int n, double &s2,
                                                    double &s1) {
  constexpr int kNt = 256;
  constexpr int W = MEAN_FREE ? 2 : 1;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  double v[3], w[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const int k = tid + j * kNt;
    v[j] = k < n ? __ldcg(pr + W * k) : 0.0;
    if (MEAN_FREE) w[j] = k < n ? __ldcg(pr + W * k + 1) : 0.0;
  }
  for (int k = tid + 3 * kNt; k < n; k += kNt) {
    v[0] += __ldcg(pr + W * k);
    if (MEAN_FREE) w[0] += __ldcg(pr + W * k + 1);
  }
  __shared__ double sa[kNt];
  __shared__ double sb[MEAN_FREE ? kNt : 1];
  sa[tid] = (v[0] + v[1]) + v[2];
  if (MEAN_FREE) sb[tid] = (w[0] + w[1]) + w[2];
  __syncthreads();
  if (tid < 128) {
    sa[tid] += sa[tid + 128];
    if (MEAN_FREE) sb[tid] += sb[tid + 128];
  }
  __syncthreads();
  s2 = 0.0;
  s1 = 0.0;
  if (tid < 32) {
    double x = (sa[tid] + sa[tid + 64]) + (sa[tid + 32] + sa[tid + 96]);
    double y = MEAN_FREE ? (sb[tid] + sb[tid + 64]) + (sb[tid + 32] + sb[tid + 96]) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      if (MEAN_FREE) y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    s2 = x;
    s1 = y;
  }
}

// Red pass.  mode 0: update only (the first red pass of a solve, and the
// phase entry points).  mode 1 (the solve's loop): the red pass of iteration
// k+1, which updates (saving the old value into pw) only when k < itermax
// and sums the residual of iteration k of
//   * the red fluid cells: class 0 from the values it reads for its update
//     (the four black neighbours are fluid and final); class 1 with the
//     copied neighbours' stale values of iteration k from pw (the black
//     pass wrote their new values into p; the cls byte's bits 2-5 say which
//     of west, east, north, south are copied cells);
//   * the red-coloured non-fluid interior cells bl[nbl_b..nbl) (when ALL),
//     reading the copied cells of their stencil (BCell::mask) from pw;
// and writes the boundary copy of iteration k+1 of the red-coloured listed
// cells (their sources are black cells, final; red cells' stencils hold no
// red-coloured cell, and the residuals here read copied cells from pw).  Each
// block stores its sum with the black pass's partial of its index added;
// the next black pass adds them up and applies the stop test of iteration k
// (sor_black_res_kernel).  Block 0 sets st->pass_iter to k (0 in mode 0)
// and, in mode 0, st->pass_inv_cells.
// SAVE: the red cells' values before the update go to pw for the rollback;
// without it the rollback inverts the update instead (sor_unred_kernel),
// saving the pass 8 bytes of writes per red cell.
template <bool IN_GRAPH, bool MEAN_FREE, bool ALL, bool SAVE = true>
__global__ void __launch_bounds__(256, kPassBlocksPerSm)
    sor_red_res_kernel(double *__restrict__ p, double *__restrict__ pw,
                       const double *__restrict__ rhs, const uint8_t *__restrict__ cls, Geom g,
                       Consts c, StepState *st, double *__restrict__ partials_r,
                       const double *partials_b, int nbb, const BCell *__restrict__ bl,
                       int nbl_b, int nbl, int gx, int nvb, unsigned int itermax,
                       int /* stop rule: applied by the next black pass */,
                       int mode, cudaGraphConditionalHandle h) {
  pdl_trigger();
  pdl_wait();
  // a later iteration of a WHILE body whose solve has stopped: nothing to do
  if (mode == 1 && (st->converged | st->exhausted)) return;
  const bool sum = mode == 1;
  const unsigned int done_iters = st->sor_iters;  // k - 1: iteration k is not decided yet
  const bool write = !sum || done_iters + 1 < itermax;
  if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    st->pass_iter = sum ? done_iters + 1 : 0;
    // the decisions' norms are the sums times this reciprocal (within an
    // ulp of the quotient); the division runs once per solve
    if (!sum) st->pass_inv_cells = 1.0 / st->fluid_cells;
  }
  double acc = 0.0, acc1 = 0.0;
  if (sum) {
    const int nt = blockDim.x * blockDim.y;
    for (int i = nbl_b + blockIdx.x * nt + threadIdx.y * blockDim.x + threadIdx.x; i < nbl;
         i += gridDim.x * nt) {
      const BCell e = bl[i];
      const size_t o = e.off;
      if (ALL && (e.flags & BC_RES)) {
        const unsigned int m = e.mask;
        const double *s0 = (m & 1u) ? pw : p, *sw = (m & 2u) ? pw : p, *se = (m & 4u) ? pw : p;
        const double *sn = (m & 8u) ? pw : p, *ss = (m & 16u) ? pw : p;
        const double r = residual_of<false>(s0[o], sw[o - g.pitch], se[o + g.pitch], sn[o - 1],
                                            ss[o + 1], rhs[o], c);
        acc = fma(r, r, acc);
      }
      if (write && (e.flags & BC_COPY)) pcopy_cell(p, o, e.edge, g.pitch);
    }
  }
  for (int vb0 = blockIdx.x; vb0 < nvb; vb0 += kPassUnroll * gridDim.x) {
    const PassCells cells = pass_cells(vb0, gridDim.x, nvb, gx, 0, g);
    unsigned int k[kPassUnroll];
    double pc[kPassUnroll], pe[kPassUnroll], pwv[kPassUnroll], pn[kPassUnroll],
        ps[kPassUnroll], rh[kPassUnroll];
#pragma unroll
    for (int u = 0; u < kPassUnroll; ++u) {
      const size_t o = cells.o[u];
      k[u] = cls[o];
      pc[u] = p[o];
      pe[u] = p[o + g.pitch];
      pwv[u] = p[o - g.pitch];
      ps[u] = p[o + 1];
      pn[u] = p[o - 1];
      rh[u] = rhs[o];
    }
#pragma unroll
    for (int u = 0; u < kPassUnroll; ++u) {
      const unsigned int kc = k[u] & 3u;
      if (!cells.ok[u] || kc >= CLS_OTHER) continue;
      const double t = fma(pe[u] + pwv[u], c.r_dx2, fma(ps[u] + pn[u], c.r_dy2, -rh[u]));
      const double r = fma(-c.two_r_sum, pc[u], t);
      if (sum) {
        double rk = r;
        if (kc == CLS_FLUID_EDGE) {
          const size_t o = cells.o[u];
          const unsigned int m = k[u] >> 2;
          const double w0 = (m & 1u) ? pw[o - g.pitch] : pwv[u];
          const double e0 = (m & 2u) ? pw[o + g.pitch] : pe[u];
          const double n0 = (m & 4u) ? pw[o - 1] : pn[u];
          const double s0 = (m & 8u) ? pw[o + 1] : ps[u];
          rk = residual_of<false>(pc[u], w0, e0, n0, s0, rh[u], c);
        }
        acc = fma(rk, rk, acc);
        if (MEAN_FREE) acc1 += rk;
      }
      if (write) {
        if (sum && SAVE) pw[cells.o[u]] = pc[u];
        p[cells.o[u]] = fma(c.middle, r, pc[u]);
      }
    }
  }
  if (!sum) return;
  // the black pass has completed: its partial of this block index joins
  // this block's, so that the next black pass sums one array (the two grids
  // are the same size; a larger black grid's rest would go to the blocks of
  // the same index modulo this grid).  Thread 0 loads it before the block
  // sum, which hides the load.
  double pb2 = 0.0, pb1 = 0.0;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int k = blockIdx.x; k < nbb; k += gridDim.x) {
      pb2 += __ldcg(partials_b + (MEAN_FREE ? 2 : 1) * k);
      if (MEAN_FREE) pb1 += __ldcg(partials_b + 2 * k + 1);
    }
  }
  block_sum_pass<MEAN_FREE>(acc, acc1);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (MEAN_FREE) {
      partials_r[2 * blockIdx.x] = acc + pb2;
      partials_r[2 * blockIdx.x + 1] = acc1 + pb1;
    } else {
      partials_r[blockIdx.x] = acc + pb2;
    }
  }
  loop_guard<IN_GRAPH>(st, itermax, h);
}

// After the solve: when it stopped at iteration k < itermax, undo the red
// pass and the boundary copy of iteration k+1.
__global__ void __launch_bounds__(256)
    sor_rollback_kernel(double *__restrict__ p, const double *__restrict__ pw,
                        const uint8_t *__restrict__ cls, const PCopy *__restrict__ pc, int npc,
                        Geom g, const StepState *st, unsigned int itermax, int gx, int nvb,
                        int red_saved) {
  if (!(st->converged && st->sor_iters < itermax)) return;
  for (int vb = blockIdx.x; red_saved && vb < nvb; vb += gridDim.x) {
    const int x = 1 + (vb / gx) * blockDim.y + threadIdx.y;
    const int y = 2 * ((vb % gx) * blockDim.x + threadIdx.x) + (x & 1);
    if (x > g.nx - 2 || y < 1 || y > g.ny - 2) continue;
    const size_t o = OFF(x, y);
    if ((cls[o] & 3u) < CLS_OTHER) p[o] = pw[o];
  }
  const int nt = blockDim.x * blockDim.y;
  for (int k = blockIdx.x * nt + threadIdx.x + threadIdx.y * blockDim.x; k < npc;
       k += gridDim.x * nt)
    p[pc[k].off] = pw[pc[k].off];
}

// The rollback of a red pass that did not save (sor_red_res_kernel, SAVE
// false): every red cell it updated (classes 0 and 1) gets its old value
// back from the update itself.  The pass computed
//   t = (pe + pw)/dx^2 + (ps + pn)/dy^2 - rhs,  r = t - 2(1/dx^2+1/dy^2) p,
//   p' = p + omega / (2(1/dx^2+1/dy^2)) r = (1 - omega) p + middle t,
// from black neighbours (and copied cells) that nothing has changed since,
// so t is recomputed bit for bit and p = (p' - middle t) / (1 - omega),
// within a few units in the last place of p' and middle t, amplified by at
// most 1 / |1 - omega| (the graph builder keeps the saving pass for
// |1 - omega| < 0.5).  It runs before the copied cells are restored (their
// restored values are not the ones the red pass read).
__global__ void __launch_bounds__(256)
    sor_unred_kernel(double *__restrict__ p, const double *__restrict__ rhs,
                     const uint8_t *__restrict__ cls, Geom g, Consts c, const StepState *st,
                     unsigned int itermax, int gx, int nvb) {
  if (!(st->converged && st->sor_iters < itermax)) return;
  const double inv = 1.0 / c.one_minus_w;
  for (int vb0 = blockIdx.x; vb0 < nvb; vb0 += kPassUnroll * gridDim.x) {
    const PassCells cells = pass_cells(vb0, gridDim.x, nvb, gx, 0, g);
#pragma unroll
    for (int u = 0; u < kPassUnroll; ++u) {
      const size_t o = cells.o[u];
      if (!cells.ok[u] || (cls[o] & 3u) >= CLS_OTHER) continue;
      const double t = fma(p[o + g.pitch] + p[o - g.pitch], c.r_dx2,
                           fma(p[o + 1] + p[o - 1], c.r_dy2, -rhs[o]));
      p[o] = fma(-c.middle, t, p[o]) * inv;
    }
  }
}

// Lexicographic Gauss-Seidel SOR in one CTA, bit-identical to the reference
// (src/simulation.rs:239-285): the sweep runs as anti-diagonal wavefronts
// d = x + y (a cell reads its west/north neighbours from wavefront d-1, new,
// and east/south from d+1, old — exactly the x-major order), and the residual
// squares are summed by one thread in x-major order.
__global__ void __launch_bounds__(1024)
    sor_lex_kernel(double *p, const double *__restrict__ rhs, const uint8_t *__restrict__ flags,
                   const PCopy *pc, int npc, Geom g, Consts c, StepState *st, double *r2,
                   unsigned int itermax, int strict) {
  __shared__ int s_done;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int NI = g.nx - 2, NJ = g.ny - 2;
  double ns = 0.0;
  unsigned int iters = 0;
  int conv = 0;
  for (unsigned int it = 0; it < itermax; ++it) {
    for (int k = tid; k < npc; k += nt) pcopy_one(p, pc[k], g.pitch);
    __syncthreads();
    for (int d = 2; d <= NI + NJ; ++d) {
      const int xlo = max(1, d - NJ), xhi = min(NI, d - 1);
      for (int x = xlo + tid; x <= xhi; x += nt) {
        const int y = d - x;
        const size_t o = OFF(x, y);
        if (flags[o] == 0)
          p[o] = sor_update(p[o], p[o - g.pitch], p[o + g.pitch], p[o - 1], p[o + 1],
                                  rhs[o], c);
      }
      __syncthreads();
    }
    for (int k = tid; k < NI * NJ; k += nt) {
      const int x = 1 + k / NJ, y = 1 + k % NJ;
      const size_t o = OFF(x, y);
      r2[k] = sqd(residual_of<true>(p[o], p[o - g.pitch], p[o + g.pitch], p[o - 1], p[o + 1],
                                    rhs[o], c));
    }
    __syncthreads();
    if (tid == 0) {
      double acc = 0.0;
      for (int k = 0; k < NI * NJ; ++k) acc = acc + r2[k];
      ns = acc / st->fluid_cells;
      iters = it + 1;
      conv = stop_rule(ns, c, st, strict);
      s_done = conv;
    }
    __syncthreads();
    if (s_done) break;
  }
  if (tid == 0) {
    st->ns = ns;
    st->sor_iters = conv ? iters : itermax;
    st->converged = conv;
    st->exhausted = conv ? 0u : 1u;
    st->nonfinite = !isfinite(ns);
  }
}

// Pressure range over fluid cells (src/grid/mod.rs:237-251), only when the
// solve ran out of iterations (src/simulation.rs:283) or when forced.
__global__ void __launch_bounds__(256)
    prange_kernel(const double *__restrict__ p, const uint8_t *__restrict__ flags, Geom g,
                  StepState *st, double *partials, int tiles_y, int ntiles, int force) {
  if (!force && !st->exhausted) return;
  double mn = DBL_MAX, mx = 0.0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x = (t / tiles_y) * RT_X + threadIdx.y;
    if (x >= g.nx) continue;
    const int yb = (t % tiles_y) * RT_Y + 2 * threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int y = yb + q;
      if (y < g.ny) {
        const size_t o = OFF(x, y);
        if (flags[o] == 0) {
          mn = fmin(mn, p[o]);
          mx = fmax(mx, p[o]);
        }
      }
    }
  }
  const double bmn = block_reduce(mn, OpMin(), DBL_MAX);
  const double bmx = block_reduce(mx, OpMax(), 0.0);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    partials[2 * blockIdx.x] = bmn;
    partials[2 * blockIdx.x + 1] = bmx;
  }
  if (!last_block_done(&st->counter)) return;
  const double rmn = reduce_partials(partials, gridDim.x, 2, 0, OpMin(), DBL_MAX);
  const double rmx = reduce_partials(partials, gridDim.x, 2, 1, OpMax(), 0.0);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    st->counter = 0;
    st->p_min = ord_enc(rmn);
    st->p_max = ord_enc(rmx);
  }
}

// ------------------------------------------------------------------------
// K4: velocity update (src/simulation.rs:287-322) + statistics
// ------------------------------------------------------------------------

// Fluid cells in [0, nx-1) x [0, ny-1) get u = F - (dt/dx)(p[x+1]-p[x]),
// v = G - (dt/dy)(p[y+1]-p[y]); boundary cells with an edge get the restore
// values the boundary pass recorded (their final value in the reference's
// u_v_restore replay); the rest keep their value.  Then max|u|, max|v| over
// every cell, the fluid speed range and, for a step, time += delt.
//
// FAST (fused multiply-adds) forms u = fma(-dt/dx, dp, F) and
// u^2 + v^2 = fma(u, u, v^2); the exact form keeps the reference's order.
// The maxima and minima are taken on the bit patterns (non-negative doubles
// order like their bits), skipping NaNs as fmax / fmin do, so they are
// exact and cost no FP64-pipe operation: 6 (FAST) or 9 FP64 operations per
// cell instead of 13.
template <bool FASTA>
__global__ void __launch_bounds__(256)
    velocity_kernel(double *u, double *v, const double *__restrict__ f,
                    const double *__restrict__ gg, const double *__restrict__ p,
                    const double *__restrict__ ru, const double *__restrict__ rv,
                    const uint8_t *__restrict__ flags, Geom g, Consts c, StepState *st,
                    double *partials, StepLog *log, int tiles_y, int ntiles, int update,
                    int commit_speed, int advance) {
  constexpr uint64_t kAbs = 0x7FFFFFFFFFFFFFFFull, kInf = 0x7FF0000000000000ull;
  __shared__ double s_cu, s_cv;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    s_cu = st->dt / c.dx;
    s_cv = st->dt / c.dy;
  }
  __syncthreads();
  const double cu = s_cu, cv = s_cv;
  uint64_t umax = f64_bits(1.0e-10), vmax = umax, smin = f64_bits(DBL_MAX), smax = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x = (t / tiles_y) * RT_X + threadIdx.y;
    if (x >= g.nx) continue;
    const int yb = (t % tiles_y) * RT_Y + 2 * threadIdx.x;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int y = yb + q;
      if (y < g.ny) {
        const size_t o = OFF(x, y);
        const uint8_t fl = flags[o];
        double un, vn;
        if (update && is_bnd(fl) && edge_of(fl) != E_NONE) {
          un = ru[o];
          vn = rv[o];
          u[o] = un;
          v[o] = vn;
        } else if (update && !is_bnd(fl) && x < g.nx - 1 && y < g.ny - 1) {
          const double pc = p[o];
          if (FASTA) {
            un = fma(-cu, p[o + g.pitch] - pc, f[o]);
            vn = fma(-cv, p[o + 1] - pc, gg[o]);
          } else {
            un = f[o] - cu * (p[o + g.pitch] - pc);
            vn = gg[o] - cv * (p[o + 1] - pc);
          }
          u[o] = un;
          v[o] = vn;
        } else {
          un = u[o];
          vn = v[o];
        }
        const uint64_t au = f64_bits(un) & kAbs, av = f64_bits(vn) & kAbs;
        if (au <= kInf) umax = au > umax ? au : umax;
        if (av <= kInf) vmax = av > vmax ? av : vmax;
        if (!is_bnd(fl)) {
          const uint64_t s2 = f64_bits(FASTA ? fma(un, un, vn * vn) : sqd(un) + sqd(vn));
          if (s2 <= kInf) {
            smin = s2 < smin ? s2 : smin;
            smax = s2 > smax ? s2 : smax;
          }
        }
      }
    }
  }
  const double b0 = block_reduce(f64_of(umax), OpMax(), 1.0e-10);
  const double b1 = block_reduce(f64_of(vmax), OpMax(), 1.0e-10);
  const double b2 = block_reduce(f64_of(smin), OpMin(), DBL_MAX);
  const double b3 = block_reduce(f64_of(smax), OpMax(), 0.0);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double *pp = partials + 4 * (size_t)blockIdx.x;
    pp[0] = b0;
    pp[1] = b1;
    pp[2] = b2;
    pp[3] = b3;
  }
  if (!last_block_done(&st->counter)) return;
  const double r0 = reduce_partials(partials, gridDim.x, 4, 0, OpMax(), 1.0e-10);
  const double r1 = reduce_partials(partials, gridDim.x, 4, 1, OpMax(), 1.0e-10);
  const double r2 = reduce_partials(partials, gridDim.x, 4, 2, OpMin(), DBL_MAX);
  const double r3 = reduce_partials(partials, gridDim.x, 4, 3, OpMax(), 0.0);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    st->counter = 0;
    st->umax = r0;
    st->vmax = r1;
    if (commit_speed) {
      st->s2_min = ord_enc(sqrt(r2));
      st->s2_max = ord_enc(sqrt(r3));
    }
    if (advance) {
      st->time = st->time + st->dt;
      st->iterations += 1;
      if (log && st->log_pos < st->log_cap) {
        StepLog &l = log[st->log_pos];
        l.ns = st->ns;
        l.dt = st->dt;
        l.sor_iters = st->sor_iters;
        l.converged = st->converged;
        st->log_pos += 1;
      }
    }
  }
}

// ------------------------------------------------------------------------
// Mixed-precision pressure solve: FP32 red-black sweeps on the FP64 defect,
// FP64 norm and FP64 accumulation of the correction (iterative refinement).
//
//   start:  e = 0 on fluid cells; on boundary cells e = delta = copy(p) - p
//   repeat: m x [red sweep, black sweep] on the correction e in FP32;
//           p += e (fluid and boundary cells), e = 0; delta, e_b = delta;
//           FP64 norm of residual(p) -> stop rule; s = (float)(middle * r)
//
// Boundary values follow the reference exactly.  Before every sweep the
// reference copies the fluid pressure to the boundary cells, so a boundary
// value is one sweep stale when the norm is taken and when the solve ends
// (quirk Q2).  Here p = p0 + e, and the copy rule for p becomes
// e_b = delta_b + copy(e) with delta_b = copy(p0) - p0_b fixed for the outer
// iteration (stored in s at boundary cells).  The copy is folded into the
// sweeps: a red boundary cell takes black fluid values, which the red sweep
// does not change; a black boundary cell takes red values, final once the red
// sweep is done.  The last black sweep of an outer iteration skips its copy,
// so after p += e every boundary value is the one copied before the last
// sweep — the reference's stale value — and the norm is the reference's.
// ------------------------------------------------------------------------

struct Consts32 {
  float omw;      // 1 - omega
  float a, b;     // middle / dx^2, middle / dy^2
};

__device__ __forceinline__ float copy32(const float *e, size_t o, int pitch, int edge) {
  switch (edge) {
    case E_N: return e[o - 1];
    case E_NE: return (e[o - 1] + e[o + pitch]) * 0.5f;
    case E_E: return e[o + pitch];
    case E_SE: return (e[o + 1] + e[o + pitch]) * 0.5f;
    case E_S: return e[o + 1];
    case E_SW: return (e[o + 1] + e[o - pitch]) * 0.5f;
    case E_W: return e[o - pitch];
    default: return (e[o - 1] + e[o - pitch]) * 0.5f;  // E_NW
  }
}

// One colour over the whole grid: fluid interior cells of the colour get the
// SOR update, boundary cells of the colour with an edge get the copy (when
// copy_boundary is set).
template <bool COH = false>
__device__ __forceinline__ void sor32_color_cells(float *__restrict__ e,
                                                  const float *__restrict__ s,
                                                  const uint8_t *__restrict__ flags,
                                                  const Geom &g, const Consts32 &k, int color,
                                                  int copy_boundary, int bx, int by,
                                                  const Thr t = thr_cta()) {
  const int x = by * t.dy + t.ty;
  const int y = 2 * (bx * t.dx + t.tx) + ((x + color) & 1);
  if (x >= g.nx || y >= g.ny) return;
  const size_t o = OFF(x, y);
  const uint8_t fl = flags[o];
  if (fl == 0) {
    if (x < 1 || y < 1 || x > g.nx - 2 || y > g.ny - 2) return;
    const float sum_x = ldv<COH>(e + o - g.pitch) + ldv<COH>(e + o + g.pitch);
    const float sum_y = ldv<COH>(e + o - 1) + ldv<COH>(e + o + 1);
    e[o] = fmaf(k.omw, ldv<COH>(e + o), fmaf(k.a, sum_x, fmaf(k.b, sum_y, ldv<COH>(s + o))));
  } else if (copy_boundary && edge_of(fl) != E_NONE) {
    e[o] = ldv<COH>(s + o) + copy32(e, o, g.pitch, edge_of(fl));
  }
}

__global__ void __launch_bounds__(256)
    sor32_color_kernel(float *__restrict__ e, const float *__restrict__ s,
                       const uint8_t *__restrict__ flags, Geom g, Consts32 k, int color,
                       int copy_boundary) {
  sor32_color_cells(e, s, flags, g, k, color, copy_boundary, blockIdx.x, blockIdx.y);
}

// Temporal blocking of the same sweeps: one CTA loads a TX x TY tile of the
// correction with an H-cell halo (and the defect and cell codes) into shared
// memory, runs `n` red-black sweeps there (2n colour passes, n <= H/2; the
// region that is still exact shrinks by one cell per pass) and writes the
// tile back.  Reads come from `ein`, writes go to `eout` (another buffer:
// neighbouring CTAs read this tile's cells as their halo).
//
// Shared memory holds each colour compacted: row lx of colour c keeps the
// cells y = 2j + ((lx + c) & 1), j = 0 .. EY/2-1 (tile origins are even, so
// local and global colours agree).  A colour-c cell (lx, j) then finds its
// four neighbours in the other colour at (lx-1, j), (lx+1, j), (lx, j-1+p)
// and (lx, j+p), p = (lx + c) & 1: consecutive lanes touch consecutive
// words, no bank conflicts, every lane busy.  Each cell sees exactly the
// arithmetic of sor32_color_kernel in the same colour order, so the result
// is bit-identical to n x (red, black) of that kernel.  The last black pass
// skips its boundary copy when skip_last_copy is set.
constexpr uint8_t kFrozen = 0xFF;  // cell code: never written (outside, edge-less boundary)

__device__ __forceinline__ float copy_rb(int code, float up, float dn, float lf, float rt) {
  switch (code) {
    case E_N: return lf;
    case E_NE: return (lf + dn) * 0.5f;
    case E_E: return dn;
    case E_SE: return (rt + dn) * 0.5f;
    case E_S: return rt;
    case E_SW: return (rt + up) * 0.5f;
    case E_W: return up;
    default: return (lf + up) * 0.5f;  // E_NW
  }
}

// Cell code of one flag byte for the blocked sweeps.
__device__ __forceinline__ uint8_t tb_code(uint8_t fl, int x, int y, const Geom &g) {
  if (fl == 0) return (x >= 1 && y >= 1 && x <= g.nx - 2 && y <= g.ny - 2) ? 0 : kFrozen;
  return edge_of(fl) != E_NONE ? edge_of(fl) : kFrozen;
}

// One row of a colour pass in the blocked sweeps: the lane's two compacted
// cells at index i of colour row `ec`, with the other colour's rows above
// (up), at (mid) and below (loaded here) rolling through registers.  P is
// the row's parity (lx + c) & 1: a cell's neighbours along y in the other
// colour are (j-1+P, j+P).
template <int P, int W>
__device__ __forceinline__ void tb_row(float *__restrict__ ec, const float *__restrict__ eo,
                                       const float *__restrict__ svc,
                                       const uint8_t *__restrict__ cc, int i, float2 &up,
                                       float2 &mid, const Consts32 &k, bool copy) {
  const float2 dn = *reinterpret_cast<const float2 *>(eo + i + W);
  const unsigned int cd2 = *reinterpret_cast<const uint16_t *>(cc + i);  // both cells' codes
  const float2 cur = *reinterpret_cast<const float2 *>(ec + i);
  const float2 sv2 = *reinterpret_cast<const float2 *>(svc + i);
  float lf0, rt0, lf1, rt1;
  if (P) {
    lf0 = mid.x;
    rt0 = mid.y;
    lf1 = mid.y;
    rt1 = eo[i + 2];
  } else {
    lf0 = eo[i - 1];
    rt0 = mid.x;
    lf1 = mid.x;
    rt1 = mid.y;
  }
  const float s0 = fmaf(k.omw, cur.x, fmaf(k.a, up.x + dn.x, fmaf(k.b, lf0 + rt0, sv2.x)));
  const float s1 = fmaf(k.omw, cur.y, fmaf(k.a, up.y + dn.y, fmaf(k.b, lf1 + rt1, sv2.y)));
  float2 res = make_float2(s0, s1);
  if (cd2 != 0) {  // a boundary or frozen cell in the pair (rare)
    const unsigned int cx = cd2 & 0xFFu, cy = cd2 >> 8;
    res.x = cx == 0 ? s0 : (copy && cx != kFrozen ? sv2.x + copy_rb(cx, up.x, dn.x, lf0, rt0)
                                                  : cur.x);
    res.y = cy == 0 ? s1 : (copy && cy != kFrozen ? sv2.y + copy_rb(cy, up.y, dn.y, lf1, rt1)
                                                  : cur.y);
  }
  *reinterpret_cast<float2 *>(ec + i) = res;
  up = mid;
  mid = dn;
}

// A warp's strip of up to S consecutive rows (nrows of them inside the
// pass's region), starting with parity P0.
template <int P0, int S, int W>
__device__ __forceinline__ void tb_strip(float *ec, const float *eo, const float *svc,
                                         const uint8_t *cc, int i0, int nrows, float2 &up,
                                         float2 &mid, const Consts32 &k, bool copy) {
  tb_row<P0, W>(ec, eo, svc, cc, i0, up, mid, k, copy);
  if constexpr (S > 1) {
    if (nrows > 1) tb_strip<P0 ^ 1, S - 1, W>(ec, eo, svc, cc, i0 + W, nrows - 1, up, mid, k, copy);
  }
}

// One tile.  Extended rows are EY = 128 cells wide, so each colour row is 64
// words and every lane owns two neighbouring compacted cells (j, j+1): the
// four cells y = 4*lane .. 4*lane+3 of a row land as one pair per colour.
template <int H, int TX, int TY, int WARPS = 16, bool COH = false>
__device__ __forceinline__ void sor32_tb_tile(const float *__restrict__ ein,
                                              float *__restrict__ eout,
                                              const float *__restrict__ s,
                                              const uint8_t *__restrict__ flags, const Geom &g,
                                              const Consts32 &k, int tile, int tiles_y, int n,
                                              int skip_last_copy, unsigned char *smem_raw,
                                              double *__restrict__ pf = nullptr,
                                              double *__restrict__ pw = nullptr) {
  static_assert(H % 4 == 0 && TX % 2 == 0 && TY % 4 == 0, "tile origins must be multiples of 4");
  static_assert(TY + 2 * H == 128, "extended rows are 128 cells");
  constexpr int EX = TX + 2 * H, EY = 128, W = EY / 2, NC = EX * W;
  float *se = reinterpret_cast<float *>(smem_raw);         // [2][EX][W]
  float *ss = se + 2 * NC;                                   // [2][EX][W]
  uint8_t *sc = reinterpret_cast<uint8_t *>(ss + 2 * NC);  // [2][EX][W]: 0 SOR, 1..8 copy, kFrozen
  const int gx0 = (tile / tiles_y) * TX - H;
  const int gy0 = (tile % tiles_y) * TY - H;
  // WARPS warps of 32 threads, in a 1-D block or a (32, WARPS) block
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int j0 = 2 * lane;  // this lane's compacted pair in every row
  // load: lane takes cells y0 .. y0+3 of each row (16-byte aligned: the tile
  // origin and the pitch are multiples of 4 cells)
  static_assert(EX % WARPS == 0, "rows per warp");
#pragma unroll
  for (int lx = warp; lx < EX; lx += WARPS) {
    const int x = gx0 + lx;
    const int y0 = gy0 + 4 * lane;
    float ev[4] = {0.0f, 0.0f, 0.0f, 0.0f}, sv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint8_t cv[4] = {kFrozen, kFrozen, kFrozen, kFrozen};
    if (x >= 0 && x < g.nx) {
      if (y0 >= 0 && y0 + 3 < g.ny) {
        const size_t o = OFF(x, y0);
        const float4 e4 = ldv<COH>(reinterpret_cast<const float4 *>(ein + o));
        const float4 s4 = ldv<COH>(reinterpret_cast<const float4 *>(s + o));
        const uchar4 f4 = *reinterpret_cast<const uchar4 *>(flags + o);
        ev[0] = e4.x; ev[1] = e4.y; ev[2] = e4.z; ev[3] = e4.w;
        sv[0] = s4.x; sv[1] = s4.y; sv[2] = s4.z; sv[3] = s4.w;
        cv[0] = tb_code(f4.x, x, y0, g);
        cv[1] = tb_code(f4.y, x, y0 + 1, g);
        cv[2] = tb_code(f4.z, x, y0 + 2, g);
        cv[3] = tb_code(f4.w, x, y0 + 3, g);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int y = y0 + q;
          if (y >= 0 && y < g.ny) {
            const size_t o = OFF(x, y);
            ev[q] = ldv<COH>(ein + o);
            sv[q] = ldv<COH>(s + o);
            cv[q] = tb_code(flags[o], x, y, g);
          }
        }
      }
    }
    // cells 0, 2 have colour c0 = (lx + 4 lane) & 1 = lx & 1 (local = global colour)
    const int c0 = lx & 1;
    const int i0 = c0 * NC + lx * W + j0, i1 = (1 - c0) * NC + lx * W + j0;
    *reinterpret_cast<float2 *>(se + i0) = make_float2(ev[0], ev[2]);
    *reinterpret_cast<float2 *>(se + i1) = make_float2(ev[1], ev[3]);
    *reinterpret_cast<float2 *>(ss + i0) = make_float2(sv[0], sv[2]);
    *reinterpret_cast<float2 *>(ss + i1) = make_float2(sv[1], sv[3]);
    *reinterpret_cast<uchar2 *>(sc + i0) = make_uchar2(cv[0], cv[2]);
    *reinterpret_cast<uchar2 *>(sc + i1) = make_uchar2(cv[1], cv[3]);
  }
  __syncthreads();
  // Each pass updates the colour on rows lo..hix, every column: a cell outside
  // the region that is still exact gets a value from inexact neighbours, but
  // no cell inside it ever reads such a value (the regions shrink by one cell
  // per pass), and columns 0 / W-1 read the neighbouring row's edge word,
  // which stays inside the tile.  Frozen cells keep their value; boundary
  // cells take the copy.
  // Each warp takes a strip of consecutive rows so that the other colour's
  // rows x-1, x, x+1 roll through registers: one new row per row.
  constexpr int STRIP = (EX - 2 + WARPS - 1) / WARPS;
  for (int pass = 0; pass < 2 * n; ++pass) {
    const int c = pass & 1;
    const bool copy = !(skip_last_copy && pass == 2 * n - 1);
    const int lo = pass + 1, hix = EX - 2 - pass;
    float *ec = se + c * NC;
    const float *eo = se + (1 - c) * NC;
    const float *svc = ss + c * NC;
    const uint8_t *cc = sc + c * NC;
    const int first = lo + warp * STRIP;
    if (first <= hix) {
      float2 up = *reinterpret_cast<const float2 *>(eo + (first - 1) * W + j0);
      float2 mid = *reinterpret_cast<const float2 *>(eo + first * W + j0);
      // row parity alternates along the strip: one warp-uniform branch picks
      // the variant whose rows know their parity at compile time
      const int i0 = first * W + j0, nrows = hix - first + 1;
      if ((first + c) & 1)
        tb_strip<1, STRIP, W>(ec, eo, svc, cc, i0, nrows, up, mid, k, copy);
      else
        tb_strip<0, STRIP, W>(ec, eo, svc, cc, i0, nrows, up, mid, k, copy);
    }
    __syncthreads();
  }
  // write the interior back: lane takes cells 4*lane .. 4*lane+3 of a row
  const int ly0 = 4 * lane;
  if (pf && ly0 >= H && ly0 < H + TY) {
    // the outer iteration's last launch ends it here (as refine_cells):
    // p += e on the cells the sweeps update (fluid interior, boundary cells
    // with an edge), the previous p saved in pw, and eout cleared for the
    // next outer iteration's sweeps
    for (int lx = H + warp; lx < H + TX; lx += WARPS) {
      const int x = gx0 + lx;
      if (x >= g.nx) break;
      const int c0 = lx & 1;
      const int ia = c0 * NC + lx * W + j0, ib = (1 - c0) * NC + lx * W + j0;
      const float2 a = *reinterpret_cast<const float2 *>(se + ia);
      const float2 b = *reinterpret_cast<const float2 *>(se + ib);
      const uchar2 ca = *reinterpret_cast<const uchar2 *>(sc + ia);
      const uchar2 cb = *reinterpret_cast<const uchar2 *>(sc + ib);
      const float ev[4] = {a.x, b.x, a.y, b.y};
      const uint8_t cv[4] = {ca.x, cb.x, ca.y, cb.y};
      const int y0 = gy0 + ly0;
      const size_t o = OFF(x, y0);
      if (y0 + 3 < g.ny) {
        // four consecutive cells: 32-byte aligned (y0 and the pitch are
        // multiples of 4), two 16-byte accesses per FP64 field
        double2 *p2 = reinterpret_cast<double2 *>(pf + o);
        const double2 lo = ldv<COH>(p2), hi = ldv<COH>(p2 + 1);
        if (pw) {
          double2 *w2 = reinterpret_cast<double2 *>(pw + o);
          w2[0] = lo;
          w2[1] = hi;
        }
        const double pv[4] = {lo.x, lo.y, hi.x, hi.y};
        double nv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) nv[q] = cv[q] != kFrozen ? pv[q] + widen(ev[q]) : pv[q];
        p2[0] = make_double2(nv[0], nv[1]);
        p2[1] = make_double2(nv[2], nv[3]);
        *reinterpret_cast<float4 *>(eout + o) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (y0 + q >= g.ny) break;
          const double p0 = ldv<COH>(pf + o + q);
          if (pw) pw[o + q] = p0;
          if (cv[q] != kFrozen) pf[o + q] = p0 + widen(ev[q]);
          eout[o + q] = 0.0f;
        }
      }
    }
  } else if (ly0 >= H && ly0 < H + TY) {
    for (int lx = H + warp; lx < H + TX; lx += WARPS) {
      const int x = gx0 + lx;
      if (x >= g.nx) break;
      const int c0 = lx & 1;
      const float2 a = *reinterpret_cast<const float2 *>(se + c0 * NC + lx * W + j0);
      const float2 b = *reinterpret_cast<const float2 *>(se + (1 - c0) * NC + lx * W + j0);
      const int y0 = gy0 + ly0;
      if (y0 + 3 < g.ny) {
        *reinterpret_cast<float4 *>(eout + OFF(x, y0)) = make_float4(a.x, b.x, a.y, b.y);
      } else {
        const float v[4] = {a.x, b.x, a.y, b.y};
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (y0 + q < g.ny) eout[OFF(x, y0 + q)] = v[q];
      }
    }
  }
}

template <int H, int TX, int TY>
__global__ void __launch_bounds__(512)
    sor32_tb_kernel(const float *__restrict__ ein, float *__restrict__ eout,
                    const float *__restrict__ s, const uint8_t *__restrict__ flags, Geom g,
                    Consts32 k, int tiles_y, int n, int skip_last_copy, double *pf,
                    double *pw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  sor32_tb_tile<H, TX, TY>(ein, eout, s, flags, g, k, (int)blockIdx.x, tiles_y, n,
                           skip_last_copy, smem_raw, pf, pw);
}

// p += e on fluid interior cells and boundary cells with an edge (apply != 0),
// then ez = 0 everywhere (the buffer the next sweeps start from; e itself
// when the sweeps ended where they started).
// save (may be NULL): receives p before the update on every cell (the state
// a sweep-by-sweep redo of this outer iteration starts from).
__device__ __forceinline__ void refine_cells(double *__restrict__ p, const float *e, float *ez,
                                             const uint8_t *__restrict__ flags, const Geom &g,
                                             int apply, int bx, int by,
                                             double *__restrict__ save,
                                             const Thr t = thr_cta()) {
  const int x = by * t.dy + t.ty;
  const int y0 = 2 * (bx * t.dx + t.tx);
  if (x >= g.nx) return;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int y = y0 + q;
    if (y >= g.ny) break;
    const size_t o = OFF(x, y);
    const uint8_t fl = flags[o];
    const bool fluid_in = fl == 0 && x >= 1 && y >= 1 && x <= g.nx - 2 && y <= g.ny - 2;
    if (save) save[o] = p[o];
    if (apply && (fluid_in || (is_bnd(fl) && edge_of(fl) != E_NONE)))
      p[o] = p[o] + widen(e[o]);
    ez[o] = 0.0f;
  }
}

__global__ void __launch_bounds__(256)
    refine_kernel(double *__restrict__ p, const float *e, float *ez,
                  const uint8_t *__restrict__ flags, Geom g, int apply, double *save) {
  refine_cells(p, e, ez, flags, g, apply, blockIdx.x, blockIdx.y, save);
}

// delta_b = copy(p) - p_b on boundary cells with an edge (FP64, stored FP32
// in s and as the starting correction e_b).
template <bool COH = false>
__device__ __forceinline__ void delta_entry(const double *__restrict__ p, float *__restrict__ s,
                                            float *__restrict__ e, const PCopy &pc, int pitch) {
  const long long o = pc.off;
  const double pN = ldv<COH>(p + o - 1), pS = ldv<COH>(p + o + 1);
  const double pW = ldv<COH>(p + o - pitch), pE = ldv<COH>(p + o + pitch);
  double c;
  switch (pc.edge) {
    case E_N: c = pN; break;
    case E_NE: c = (pN + pE) * 0.5; break;
    case E_E: c = pE; break;
    case E_SE: c = (pS + pE) * 0.5; break;
    case E_S: c = pS; break;
    case E_SW: c = (pS + pW) * 0.5; break;
    case E_W: c = pW; break;
    default: c = (pN + pW) * 0.5; break;
  }
  const float d = (float)(c - ldv<COH>(p + o));
  s[o] = d;
  e[o] = d;
}


template <bool FLUID, bool MEAN_FREE, bool COH = false>
__device__ __forceinline__ void mixed_residual_sum(
    const double *__restrict__ p, const double *__restrict__ rhs,
    const uint8_t *__restrict__ flags, float *__restrict__ s, const Geom &g, const Consts &c,
    int tiles_y, int ntiles, int bid, int nblocks, double *acc_out, double *acc1_out,
    const Thr th = thr_cta()) {
  double acc = 0.0, acc1 = 0.0;
  // the defect is rounded to FP32 before the scaling (integer conversion,
  // FP32 multiply): no FP64 operation beyond the residual and its sums
  const float mid32 = narrow(c.middle);
  for (int t = bid; t < ntiles; t += nblocks) {
    const int x = 1 + (t / tiles_y) * RT_X + th.ty;
    if (x > g.nx - 2) continue;
    const int yb = 1 + (t % tiles_y) * RT_Y + 2 * th.tx;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int y = yb + q;
      if (y <= g.ny - 2) {
        const size_t o = OFF(x, y);
        const double r = residual_of<false>(ldv<COH>(p + o), ldv<COH>(p + o - g.pitch),
                                            ldv<COH>(p + o + g.pitch), ldv<COH>(p + o - 1),
                                            ldv<COH>(p + o + 1), rhs[o], c);
        const bool fluid = flags[o] == 0;
        if (fluid || !FLUID) {
          acc = fma(r, r, acc);
          if (MEAN_FREE) acc1 += r;
        }
        if (fluid) s[o] = narrow(r) * mid32;
      }
    }
  }
  *acc_out = acc;
  *acc1_out = acc1;
}

// Group versions of the block sums for 256-thread groups (a graph kernel's
// CTA or half of a persistent CTA), with the same summation trees as
// block_sum_pass / block_reduce / reduce_partials on 256 threads, so the
// results are bit-identical.  Their scratch is passed in (the persistent
// kernel lends the dynamic shared memory its sweep tiles use between
// phases): 2 x 512 + 2 x 32 doubles.
template <bool TWO>
__device__ __forceinline__ void block_sum_pass_g(double &a, double &b, const Thr &t,
                                                 double *scratch) {
  double *sa = scratch + t.half * 512, *sb = sa + 256;
  sa[t.tid] = a;
  if (TWO) sb[t.tid] = b;
  gsync(t);
  if (t.tid < 32) {
    double s0 = sa[t.tid], s1 = TWO ? sb[t.tid] : 0.0;
    for (int k = t.tid + 32; k < 256; k += 32) {
      s0 += sa[k];
      if (TWO) s1 += sb[k];
    }
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      if (TWO) s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    a = s0;
    b = s1;
  }
}

template <typename Op>
__device__ double block_reduce_g(double v, Op op, double identity, const Thr &t,
                                 double *scratch) {
  double *sm = scratch + 1024 + t.half * 32;
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = t.tid & 31, w = t.tid >> 5;
  gsync(t);
  if (lane == 0) sm[w] = v;
  gsync(t);
  if (w == 0) {
    v = lane < 8 ? sm[lane] : identity;
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;  // valid in thread 0 of the group
}

template <typename Op>
__device__ double reduce_partials_g(const double *part, int n, int stride, int idx, Op op,
                                    double identity, const Thr &t, double *scratch) {
  double v = identity;
  for (int k = t.tid; k < n; k += 256) v = op(v, __ldcg(part + (size_t)k * stride + idx));
  return block_reduce_g(v, op, identity, t, scratch);
}

// mixed_residual_sum for a 256-thread group of the persistent batch solve:
// p changes within that launch, so it is read through L2; each 8 x 64 tile
// of p and its one-cell halo is first staged in shared memory (one L2 load
// per cell instead of five), then every thread takes exactly the cells, in
// exactly the order, of mixed_residual_sum: the sums are bit-identical.
// tile: 10 x 66 doubles of the group's shared memory.
template <bool FLUID, bool MEAN_FREE>
__device__ __forceinline__ void mixed_residual_sum_staged(
    const double *__restrict__ p, const double *__restrict__ rhs,
    const uint8_t *__restrict__ flags, float *__restrict__ s, const Geom &g, const Consts &c,
    int tiles_y, int ntiles, int bid, int nblocks, double *acc_out, double *acc1_out,
    const Thr &th, double *tile) {
  constexpr int TW = RT_Y + 2;
  double acc = 0.0, acc1 = 0.0;
  const float mid32 = narrow(c.middle);
  for (int t = bid; t < ntiles; t += nblocks) {
    const int x0 = 1 + (t / tiles_y) * RT_X, y0 = 1 + (t % tiles_y) * RT_Y;
    gsync(th);  // the previous tile's readers are done
    for (int k = th.tid; k < (RT_X + 2) * TW; k += 256) {
      const int i = k / TW, j = k % TW;
      const int x = x0 - 1 + i, y = y0 - 1 + j;
      tile[k] = (x < g.nx && y < g.ny) ? __ldcg(p + OFF(x, y)) : 0.0;
    }
    gsync(th);
    const int x = x0 + th.ty;
    if (x > g.nx - 2) continue;
    const int lx = th.ty + 1;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int ly = 2 * th.tx + q + 1, y = y0 + ly - 1;
      if (y <= g.ny - 2) {
        const size_t o = OFF(x, y);
        const double *tc = tile + lx * TW + ly;
        const double r = residual_of<false>(tc[0], tc[-TW], tc[TW], tc[-1], tc[1], rhs[o], c);
        const bool fluid = flags[o] == 0;
        if (fluid || !FLUID) {
          acc = fma(r, r, acc);
          if (MEAN_FREE) acc1 += r;
        }
        if (fluid) s[o] = narrow(r) * mid32;
      }
    }
  }
  *acc_out = acc;
  *acc1_out = acc1;
}

// FP64 norm of the residual on every interior cell (the reference's norm),
// the scaled FP32 defect s = middle * r on fluid cells for the next sweeps,
// and the stop rule every m sweeps.  Block `bid` of `nblocks` sums its tiles
// into partials[bid] (interleaved with the residual sum when mean-free).
// GRP, th, scratch: a 256-thread group and its reduction scratch (the
// persistent batch solve); by default the CTA and block_sum_pass.
template <bool COH = false, bool GRP = false>
__device__ __forceinline__ void mixed_residual_partial(
    const double *__restrict__ p, const double *__restrict__ rhs,
    const uint8_t *__restrict__ flags, float *__restrict__ s, const Geom &g, const Consts &c,
    double *partials, int tiles_y, int ntiles, int strict, int bid, int nblocks,
    const Thr th = thr_cta(), double *scratch = nullptr) {
  const bool fluid_only = (strict & STOP_FLUID_NORM) != 0;
  const bool mean_free = fluid_only && (strict & STOP_MEAN_FREE) != 0;
  double acc = 0.0, acc1 = 0.0;
  if constexpr (GRP) {
    // the group's p tile follows the reduction scratch (2 x 512 + 2 x 32
    // doubles) in the persistent kernel's shared memory
    double *tile = scratch + 2 * 512 + 2 * 32 + th.half * (RT_X + 2) * (RT_Y + 2);
    if (!fluid_only)
      mixed_residual_sum_staged<false, false>(p, rhs, flags, s, g, c, tiles_y, ntiles, bid,
                                              nblocks, &acc, &acc1, th, tile);
    else if (!mean_free)
      mixed_residual_sum_staged<true, false>(p, rhs, flags, s, g, c, tiles_y, ntiles, bid,
                                             nblocks, &acc, &acc1, th, tile);
    else
      mixed_residual_sum_staged<true, true>(p, rhs, flags, s, g, c, tiles_y, ntiles, bid,
                                            nblocks, &acc, &acc1, th, tile);
  } else {
    if (!fluid_only)
      mixed_residual_sum<false, false, COH>(p, rhs, flags, s, g, c, tiles_y, ntiles, bid,
                                            nblocks, &acc, &acc1, th);
    else if (!mean_free)
      mixed_residual_sum<true, false, COH>(p, rhs, flags, s, g, c, tiles_y, ntiles, bid,
                                           nblocks, &acc, &acc1, th);
    else
      mixed_residual_sum<true, true, COH>(p, rhs, flags, s, g, c, tiles_y, ntiles, bid,
                                          nblocks, &acc, &acc1, th);
  }
  if (mean_free) {
    if constexpr (GRP) block_sum_pass_g<true>(acc, acc1, th, scratch);
    else block_sum_pass<true>(acc, acc1);
    if (th.tid == 0) {
      partials[2 * bid] = acc;
      partials[2 * bid + 1] = acc1;
    }
  } else {
    if constexpr (GRP) block_sum_pass_g<false>(acc, acc1, th, scratch);
    else block_sum_pass<false>(acc, acc1);
    if (th.tid == 0) partials[bid] = acc;
  }
}

// The norm from the partials and the stop rule (every thread of one block
// calls it; thread 0 updates the state).  Returns, in thread 0, SOLVE_GO_ON,
// SOLVE_DONE (the stop rule fired) or SOLVE_NO_ROOM (another `sweeps` would
// pass max_iterations).
enum : int { SOLVE_GO_ON = 0, SOLVE_DONE = 1, SOLVE_NO_ROOM = 2 };

__device__ __forceinline__ int mixed_residual_stop(const double *partials, int nblocks,
                                                   StepState *st, const Consts &c,
                                                   unsigned int itermax, int strict, int sweeps,
                                                   int check) {
  const bool mean_free = (strict & STOP_FLUID_NORM) && (strict & STOP_MEAN_FREE);
  const double ns = finish_norm(partials, nblocks, mean_free, st->fluid_cells);
  int status = SOLVE_GO_ON;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    st->ns = ns;
    hist_push(st, check ? st->sor_iters + sweeps : 0u, ns);
    if (!check) st->ns_start = ns;
    if (check) {
      const unsigned int it = st->sor_iters + sweeps;
      st->sor_iters = it;
      st->nonfinite = !isfinite(ns);
      const bool done = stop_rule(ns, c, st, strict);
      const bool room = it + sweeps <= itermax;
      if (done) st->converged = 1;
      else if (!room) st->exhausted = 1;
      status = done ? SOLVE_DONE : (room ? SOLVE_GO_ON : SOLVE_NO_ROOM);
    }
  }
  return status;
}

// mixed_residual_stop for a 256-thread group with its reduction scratch.
__device__ __forceinline__ int mixed_residual_stop_g(const double *partials, int nblocks,
                                                     StepState *st, const Consts &c,
                                                     unsigned int itermax, int strict,
                                                     int sweeps, int check, const Thr &t,
                                                     double *scratch) {
  const bool mean_free = (strict & STOP_FLUID_NORM) && (strict & STOP_MEAN_FREE);
  double ns;
  if (!mean_free) {
    ns = reduce_partials_g(partials, nblocks, 1, 0, OpAdd(), 0.0, t, scratch) / st->fluid_cells;
  } else {
    const double s2 = reduce_partials_g(partials, nblocks, 2, 0, OpAdd(), 0.0, t, scratch);
    const double s1 = reduce_partials_g(partials, nblocks, 2, 1, OpAdd(), 0.0, t, scratch);
    ns = (s2 - s1 * (s1 / st->fluid_cells)) / st->fluid_cells;
  }
  int status = SOLVE_GO_ON;
  if (t.tid == 0) {
    st->ns = ns;
    hist_push(st, check ? st->sor_iters + sweeps : 0u, ns);
    if (!check) st->ns_start = ns;
    if (check) {
      const unsigned int it = st->sor_iters + sweeps;
      st->sor_iters = it;
      st->nonfinite = !isfinite(ns);
      const bool done = stop_rule(ns, c, st, strict);
      const bool room = it + sweeps <= itermax;
      if (done) st->converged = 1;
      else if (!room) st->exhausted = 1;
      status = done ? SOLVE_DONE : (room ? SOLVE_GO_ON : SOLVE_NO_ROOM);
    }
  }
  return status;
}

// After a coarse (m sweeps per check) loop stopped: which finishing pass the
// solve needs so that it ends at the sweep the per-sweep rule would.
__device__ __forceinline__ unsigned int replay_of(int status, const StepState *st,
                                                  unsigned int itermax) {
  if (status == SOLVE_DONE) return 1u;                                 // redo sweep by sweep
  if (status == SOLVE_NO_ROOM && st->sor_iters < itermax) return 2u;  // the remainder
  return 0u;
}

// check: 0 the solve's starting norm, 1 a stop test after `sweeps` sweeps,
// 2 the defect only (no norm, no state change).  coarse: the loop checks
// every `sweeps` > 1 sweeps; when it stops, st->replay says how the solve
// finishes (and, in a graph, h_replay opens the finishing pass).
// The kernel also writes the boundary entries the next sweeps start from
// (delta_entry for the npc listed boundary cells: s and e there, disjoint
// from the fluid cells' defect).
template <bool IN_GRAPH>
__global__ void __launch_bounds__(256)
    mixed_residual_kernel(const double *__restrict__ p, const double *__restrict__ rhs,
                          const uint8_t *__restrict__ flags, float *__restrict__ s, Geom g,
                          Consts c, StepState *st, double *partials, int tiles_y, int ntiles,
                          cudaGraphConditionalHandle h, unsigned int itermax, int strict,
                          int sweeps, int check, cudaGraphConditionalHandle h_replay,
                          int coarse, const PCopy *__restrict__ pc, int npc,
                          float *__restrict__ e) {
  {
    const int nt = blockDim.x * blockDim.y;
    for (int k = blockIdx.x * nt + threadIdx.y * blockDim.x + threadIdx.x; k < npc;
         k += gridDim.x * nt)
      delta_entry(p, s, e, pc[k], g.pitch);
  }
  mixed_residual_partial(p, rhs, flags, s, g, c, partials, tiles_y, ntiles, strict, blockIdx.x,
                         gridDim.x);
  if (check == 2) return;
  if (IN_GRAPH && check && blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    // independent bound on the WHILE loop, as in residual_kernel
    const unsigned int launches = atomicAdd(&st->body_count, 1u) + 1;
    if ((unsigned long long)launches * (unsigned long long)sweeps >= itermax + 2ull * sweeps) {
      st->overrun = 1;
      cudaGraphSetConditional(h, 0);
    }
  }
  if (!last_block_done(&st->counter)) return;
  const int status = mixed_residual_stop(partials, gridDim.x, st, c, itermax, strict, sweeps,
                                         check);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    st->counter = 0;
    if (check && status != SOLVE_GO_ON) {
      if (coarse) {
        st->replay = replay_of(status, st, itermax);
        if (IN_GRAPH && st->replay) cudaGraphSetConditional(h_replay, 1);
      }
      if (IN_GRAPH) cudaGraphSetConditional(h, 0);
    }
  }
}

// Start of a sweep-by-sweep finishing pass: with replay 1, p returns to its
// value before the last outer iteration (saved in pw) and the iteration
// count and residual history drop that iteration.
__global__ void __launch_bounds__(256)
    restore_kernel(double *__restrict__ p, const double *__restrict__ pw, Geom g, StepState *st,
                   int sweeps) {
  const unsigned int replay = st->replay;
  if (replay == 2u && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    st->exhausted = 0;  // the remaining sweeps follow one by one
  if (replay != 1u) return;
  const int x = blockIdx.y * blockDim.y + threadIdx.y;
  const int y0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (x < g.nx) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int y = y0 + q;
      if (y < g.ny) p[OFF(x, y)] = pw[OFF(x, y)];
    }
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    st->sor_iters -= (unsigned int)sweeps;
    if (st->hist_n > 0) st->hist_n -= 1;
    st->converged = 0;
  }
}

// ------------------------------------------------------------------------
// Headless colour map (src/visualization.rs:7-105): pressure or speed of
// every cell to RGBA8, image rows = y, as the reference's macroquad Image
// (width nx).  Same f32 arithmetic as the reference; channel bytes are
// (c * 255) converted like Rust's `as u8` (NaN -> 0, saturating, truncating).
// ------------------------------------------------------------------------

__device__ __forceinline__ unsigned char channel_u8(float c) {
  const float v = c * 255.0f;
  if (!(v > 0.0f)) return 0;
  if (v >= 255.0f) return 255;
  return (unsigned char)v;
}

__global__ void render_kernel(const double *__restrict__ u, const double *__restrict__ v,
                              const double *__restrict__ p, const uint8_t *__restrict__ flags,
                              Geom g, const StepState *st, int color_type, uchar4 *rgba) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= g.nx || y >= g.ny) return;
  const size_t o = OFF(x, y);
  float r, gg, b;
  if (is_bnd(flags[o])) {
    r = 0.5f;
    gg = color_type == 1 ? 0.5f : 0.0f;
    b = color_type == 1 ? 0.5f : 0.0f;
  } else {
    double hue_d;
    if (color_type == 1) {
      const double r0 = ord_dec(st->s2_min), r1 = ord_dec(st->s2_max);
      const double speed = sqrt(sqd(u[o]) + sqd(v[o]));
      hue_d = 240.0 - (speed - r0) * 240.0 / (r1 - r0);
    } else {
      const double r0 = ord_dec(st->p_min), r1 = ord_dec(st->p_max);
      const double offset = 240.0;
      hue_d = offset - (p[o] - r0) * offset / (r1 - r0);
    }
    const float hue = (float)hue_d;
    // hsl_to_rgb(hue, 1, 0.5), src/visualization.rs:7-27
    const float sat = 1.0f, light = 0.5f;
    const float c = (1.0f - fabsf(2.0f * light - 1.0f)) * sat;
    const float xx = c * (1.0f - fabsf(fmodf(hue / 60.0f, 2.0f) - 1.0f));
    const float m = light - c / 2.0f;
    float rr, g2, bb;
    if (hue < 60.0f) { rr = c; g2 = xx; bb = 0.0f; }
    else if (hue < 120.0f) { rr = xx; g2 = c; bb = 0.0f; }
    else if (hue < 180.0f) { rr = 0.0f; g2 = c; bb = xx; }
    else if (hue < 240.0f) { rr = 0.0f; g2 = xx; bb = c; }
    else if (hue < 300.0f) { rr = xx; g2 = 0.0f; bb = c; }
    else { rr = c; g2 = 0.0f; bb = xx; }
    r = rr + m;
    gg = g2 + m;
    b = bb + m;
  }
  rgba[(size_t)y * g.nx + x] = make_uchar4(channel_u8(r), channel_u8(gg), channel_u8(b),
                                           channel_u8(1.0f));
}

cudaError_t launch_render(const DevFields &d, const Geom &g, int color_type, void *rgba,
                          cudaStream_t s) {
  dim3 blk(32, 8), grd((g.nx + 31) / 32, (g.ny + 7) / 8);
  render_kernel<<<grd, blk, 0, s>>>(d.u, d.v, d.p, d.flags, g, d.st, color_type, (uchar4 *)rgba);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// Warm-start plumbing: dense FP32 copies of RHS / pressure and the flags for
// a predictor, and the application of a predicted FP32 correction to the
// FP64 pressure on fluid interior cells.
// ------------------------------------------------------------------------

__global__ void export_kernel(const double *__restrict__ rhs, const double *__restrict__ p,
                              const uint8_t *__restrict__ flags, Geom g, float *rhs32,
                              float *p32, uint8_t *fl8) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y;
  if (y >= g.ny) return;
  const size_t o = OFF(x, y), dn = (size_t)x * g.ny + y;
  if (rhs32) rhs32[dn] = (float)rhs[o];
  if (p32) p32[dn] = (float)p[o];
  if (fl8) fl8[dn] = flags[o];
}

// p += scale * q on fluid cells.  With jd (device [scale, norm without,
// norm with the correction]) the scale is jd[0], and when cond is set the
// correction is applied only if jd[2] < jd[1] (the judge's choice).
__global__ void apply_correction_kernel(double *__restrict__ p, const uint8_t *__restrict__ flags,
                                        Geom g, const float *__restrict__ q, double scale,
                                        const double *__restrict__ jd, int cond) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int x = blockIdx.y + 1;
  if (y < 1 || y > g.ny - 2 || x > g.nx - 2) return;
  if (jd) {
    if (cond && !(jd[2] < jd[1])) return;
    scale = jd[0];
  }
  const size_t o = OFF(x, y);
  if (flags[o] != 0) return;
  p[o] = p[o] + scale * (double)q[(size_t)(x - 1) * (g.ny - 2) + (y - 1)];
}

cudaError_t launch_export(const DevFields &d, const Geom &g, float *rhs32, float *p32,
                          uint8_t *fl8, cudaStream_t s) {
  export_kernel<<<dim3((g.ny + 127) / 128, g.nx), 128, 0, s>>>(d.rhs, d.p, d.flags, g, rhs32,
                                                               p32, fl8);
  return cudaGetLastError();
}

cudaError_t launch_apply_correction(const DevFields &d, const Geom &g, const float *q,
                                    double scale, cudaStream_t s, const double *jd, int cond) {
  if (g.nx < 3 || g.ny < 3) return cudaSuccess;
  apply_correction_kernel<<<dim3((g.ny + 127) / 128, g.nx - 2), 128, 0, s>>>(d.p, d.flags, g, q,
                                                                             scale, jd, cond);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------

static int g_num_sms = 0;
static int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
  }
  return g_num_sms;
}

static void tiles_of(const Geom &g, int interior, int *tiles_y, int *ntiles) {
  const int nx = interior ? g.nx - 2 : g.nx;
  const int ny = interior ? g.ny - 2 : g.ny;
  *tiles_y = (ny + RT_Y - 1) / RT_Y;
  const int tiles_x = (nx + RT_X - 1) / RT_X;
  *ntiles = (nx > 0 && ny > 0) ? (*tiles_y) * tiles_x : 0;
}

int residual_blocks(const Geom &g) {
  int ty, nt;
  tiles_of(g, 0, &ty, &nt);
  int b = 4 * num_sms();
  if (nt < b) b = nt;
  return b < 1 ? 1 : b;
}

static const dim3 kRedBlock(RT_Y / 2, RT_X);

// Blocks of the fused black pass: enough resident warps to keep the FP64
// pipe busy, each block reducing once.
int black_pass_blocks(const Geom &g) {
  const long long gx = (g.ny / 2 + 1 + (int)kRedBlock.x - 1) / (int)kRedBlock.x;
  const long long gy = (g.nx - 2 + (int)kRedBlock.y - 1) / (int)kRedBlock.y;
  long long n = gx * (gy > 0 ? gy : 0);
  const long long cap = (long long)kPassBlocksPerSm * num_sms();  // one wave
  if (n > cap) n = cap;
  return n < 1 ? 1 : (int)n;
}

// Iterations of the FAST red-black solve per body of its WHILE node: each
// evaluation of the condition costs a few microseconds between the body's
// kernels (measured per step at 2000 iterations: 2 per body -1.5 %, 4
// -3.8 %, 8 -4.6 %); a body that stops early runs the remaining passes as
// launches that return at once.
constexpr int kFastBodyIters = 8;

// Kernel choices of the FAST red-black solve for a stop-rule setting and
// relaxation factor: the red pass saves the values it overwrites only when
// omega is near 1 (|1 - omega| < 0.5); otherwise the rollback inverts it.
struct FastSolveKernels {
  const void *red_graph, *red_eager, *black_graph, *black_eager;
  bool save;
};

template <bool SAVE>
static void fast_red_kernels(FastSolveKernels &k, bool mf, bool fluid) {
  if (mf) {
    k.red_graph = (const void *)sor_red_res_kernel<true, true, false, SAVE>;
    k.red_eager = (const void *)sor_red_res_kernel<false, true, false, SAVE>;
  } else if (fluid) {
    k.red_graph = (const void *)sor_red_res_kernel<true, false, false, SAVE>;
    k.red_eager = (const void *)sor_red_res_kernel<false, false, false, SAVE>;
  } else {
    k.red_graph = (const void *)sor_red_res_kernel<true, false, true, SAVE>;
    k.red_eager = (const void *)sor_red_res_kernel<false, false, true, SAVE>;
  }
}

static FastSolveKernels fast_solve_kernels(int strict, double one_minus_w) {
  const bool fluid = (strict & STOP_FLUID_NORM) != 0;
  const bool mf = fluid && (strict & STOP_MEAN_FREE) != 0;
  FastSolveKernels k;
  k.black_graph = mf      ? (const void *)sor_black_res_kernel<true, true, false>
                  : fluid ? (const void *)sor_black_res_kernel<true, false, false>
                          : (const void *)sor_black_res_kernel<true, false, true>;
  k.black_eager = mf      ? (const void *)sor_black_res_kernel<false, true, false>
                  : fluid ? (const void *)sor_black_res_kernel<false, false, false>
                          : (const void *)sor_black_res_kernel<false, false, true>;
  k.save = fabs(one_minus_w) < 0.5;
  if (k.save)
    fast_red_kernels<true>(k, mf, fluid);
  else
    fast_red_kernels<false>(k, mf, fluid);
  return k;
}

// The sweep schedules: 0 is one launch per colour pass; the others are
// temporal-blocking tile shapes, `sweeps` red-black sweeps per launch.
struct TbShape {
  int halo, tx, ty, sweeps;
  const void *fn;
};

static const TbShape kTbShapes[] = {
    {0, 0, 0, 1, nullptr},
    {4, 56, 120, 2, (const void *)sor32_tb_kernel<4, 56, 120>},
    {8, 48, 112, 4, (const void *)sor32_tb_kernel<8, 48, 112>},
    {16, 32, 96, 8, (const void *)sor32_tb_kernel<16, 32, 96>},
    {8, 80, 112, 4, (const void *)sor32_tb_kernel<8, 80, 112>},
    {8, 112, 112, 4, (const void *)sor32_tb_kernel<8, 112, 112>},
    {16, 64, 96, 8, (const void *)sor32_tb_kernel<16, 64, 96>},
};
constexpr int kNumSchedules = (int)(sizeof(kTbShapes) / sizeof(kTbShapes[0]));

int num_sweep_schedules() { return kNumSchedules; }

static size_t tb_smem(const TbShape &t) {
  const size_t nc = (size_t)(t.tx + 2 * t.halo) * (t.ty + 2 * t.halo);
  return nc * (4 + 4 + 1);
}

// One launch of a sweep schedule: what it reads, writes and how.
struct SweepLaunch {
  const void *fn;
  dim3 grid, block;
  size_t smem;
  const float *ein;
  float *eout;
  int tiles_y, n, skip_last_copy;
  int color, copy;  // schedule 0
  double *pf, *pw;  // blocked: the launch also applies the correction to p
};

// The launches of m inner sweeps (colour passes or blocked tiles) starting
// from correction buffer e32; *final receives the buffer holding the result.
// refine (blocked schedules with an even number of launches): the last
// launch also does the refinement (p += e, p saved in `save` when not NULL,
// its output buffer, e32, cleared) and *final is NULL.
static std::vector<SweepLaunch> sweep_plan(const DevFields &d, const Geom &g, int m, int sched,
                                           float **final, bool refine = false,
                                           double *save = nullptr) {
  std::vector<SweepLaunch> v;
  if (sched <= 0 || sched >= kNumSchedules) {
    dim3 pgrid((g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x,
               (g.nx + kRedBlock.y - 1) / kRedBlock.y);
    for (int i = 0; i < m; ++i)
      for (int color = 0; color < 2; ++color) {
        SweepLaunch l{};
        l.fn = (const void *)sor32_color_kernel;
        l.grid = pgrid;
        l.block = kRedBlock;
        l.ein = d.e32;
        l.eout = d.e32;
        l.color = color;
        l.copy = (color == 0 || i < m - 1) ? 1 : 0;
        v.push_back(l);
      }
    *final = d.e32;
    return v;
  }
  const TbShape &t = kTbShapes[sched];
  const int tiles_x = (g.nx + t.tx - 1) / t.tx, tiles_y = (g.ny + t.ty - 1) / t.ty;
  float *bufs[2] = {d.e32, d.e32b};
  int cur = 0;
  for (int done = 0; done < m; done += t.sweeps) {
    SweepLaunch l{};
    l.fn = t.fn;
    l.grid = dim3(tiles_x * tiles_y);
    l.block = dim3(512);
    l.smem = tb_smem(t);
    l.ein = bufs[cur];
    l.eout = bufs[cur ^ 1];
    l.tiles_y = tiles_y;
    l.n = m - done < t.sweeps ? m - done : t.sweeps;
    l.skip_last_copy = done + l.n >= m ? 1 : 0;
    v.push_back(l);
    cur ^= 1;
  }
  *final = bufs[cur];
  if (refine && cur == 0) {
    v.back().pf = d.p;
    v.back().pw = save;
    *final = nullptr;
  }
  return v;
}

// Opts the blocked kernels into their shared-memory size, once per device.
static cudaError_t tb_prepare() {
  static std::atomic<bool> done_on[64] = {};
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return e0;
  std::atomic<bool> &done = done_on[dev & 63];
  if (done.load()) return cudaSuccess;
  for (int i = 1; i < kNumSchedules; ++i) {
    cudaError_t e = cudaFuncSetAttribute(kTbShapes[i].fn,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tb_smem(kTbShapes[i]));
    if (e != cudaSuccess) return e;
  }
  done = true;
  return cudaSuccess;
}

static cudaError_t issue_sweep(const SweepLaunch &l, const float *s, const uint8_t *flags,
                               const Geom &g, const Consts32 &k32, cudaStream_t st) {
  if (l.smem == 0) {
    sor32_color_kernel<<<l.grid, l.block, 0, st>>>(l.eout, s, flags, g, k32, l.color, l.copy);
  } else {
    void *args[] = {(void *)&l.ein, (void *)&l.eout, (void *)&s, (void *)&flags,
                    (void *)&g, (void *)&k32, (void *)&l.tiles_y, (void *)&l.n,
                    (void *)&l.skip_last_copy, (void *)&l.pf, (void *)&l.pw};
    return cudaLaunchKernel(l.fn, l.grid, l.block, args, l.smem, st);
  }
  return cudaGetLastError();
}


cudaError_t launch_classify(const DevFields &d, const Geom &g, cudaStream_t s) {
  dim3 blk(64, 4), grd((g.ny + 63) / 64, (g.nx + 3) / 4);
  classify_kernel<<<grd, blk, 0, s>>>(d.flags, g, d.fluid_count, d.first_bad);
  return cudaGetLastError();
}

cudaError_t launch_step_begin(const DevFields &d, const RunCfg &r, cudaStream_t s) {
  bc_kernel<<<BC_CLUSTER, BC_THREADS, 0, s>>>(d.u, d.v, d.ru, d.rv, d.bc, d.bc_val, 0, d.st,
                                              r.c, r.tau, r.delt, r.itermax, 1);
  return cudaGetLastError();
}

cudaError_t launch_bc(const DevFields &d, cudaStream_t s) {
  Consts c{};
  bc_kernel<<<BC_CLUSTER, BC_THREADS, 0, s>>>(d.u, d.v, d.ru, d.rv, d.bc, d.bc_val, d.n_bc, d.st,
                                              c, 0.0, 0.0, 0u, 0);
  return cudaGetLastError();
}

// Opts fg_rhs_fast_kernel into its dynamic shared memory (once per device).
static cudaError_t ff_prepare() {
  static std::atomic<bool> done_on[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::atomic<bool> &done = done_on[dev & 63];
  if (done.load()) return cudaSuccess;
  e = cudaFuncSetAttribute(fg_rhs_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(FastFgSmem));
  if (e == cudaSuccess) done = true;
  return e;
}

static dim3 ff_grid(const Geom &g) {
  return dim3((g.ny + FF_T - 1) / FF_T, (g.nx + FF_T - 1) / FF_T);
}

cudaError_t launch_fg_rhs(const DevFields &d, const RunCfg &r, cudaStream_t s) {
  dim3 grd((r.g.ny + FG_TY - 1) / FG_TY, (r.g.nx + FG_TX - 1) / FG_TX);
  if (r.precision == 1) {
    fg_rhs32_kernel<<<grd, FG_THREADS, 0, s>>>(d.u, d.v, d.f, d.g, d.rhs, d.flags, r.g, r.c,
                                               consts32f_of(r.c), d.st);
  } else if (r.arith) {
    cudaError_t e = ff_prepare();
    if (e != cudaSuccess) return e;
    fg_rhs_fast_kernel<<<ff_grid(r.g), FF_THREADS, sizeof(FastFgSmem), s>>>(
        d.u, d.v, d.f, d.g, d.rhs, d.flags, r.g, r.c, d.st);
  } else {
    fg_rhs_kernel<<<grd, FG_THREADS, 0, s>>>(d.u, d.v, d.f, d.g, d.rhs, d.flags, r.g, r.c, d.st);
  }
  return cudaGetLastError();
}

cudaError_t launch_pcopy(const DevFields &d, const Geom &g, cudaStream_t s) {
  if (d.n_pcopy == 0) return cudaSuccess;
  pcopy_kernel<<<(d.n_pcopy + 255) / 256, 256, 0, s>>>(d.p, d.pcopy, d.n_pcopy, g.pitch);
  return cudaGetLastError();
}

cudaError_t launch_norm(const DevFields &d, const RunCfg &r, cudaStream_t s, int set_ns0) {
  int ty, nt;
  tiles_of(r.g, 1, &ty, &nt);
  if (nt == 0) {
    // no interior: the sum is 0.0
    return cudaSuccess;
  }
  int nb = residual_blocks(r.g);
  residual_kernel<true, false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, r.g, r.c, d.st, d.partials,
                                                        ty, nt, 0, r.itermax, r.strict_eps,
                                                        set_ns0 ? RES_NS0 : RES_NORM, nullptr, 0);
  return cudaGetLastError();
}

int interior_tiles(const Geom &g) {
  int ty, nt;
  tiles_of(g, 1, &ty, &nt);
  return nt;
}

cudaError_t launch_norm_one_block_per_tile(const double *p, const double *rhs, const Geom &g,
                                           const Consts &c, StepState *st, double *partials,
                                           cudaStream_t s) {
  int ty, nt;
  tiles_of(g, 1, &ty, &nt);
  if (nt == 0) return cudaSuccess;
  residual_kernel<true, false><<<nt, kRedBlock, 0, s>>>(p, rhs, nullptr, g, c, st, partials, ty, nt, 0,
                                                        0u, 0, RES_NORM, nullptr, 0);
  return cudaGetLastError();
}

cudaError_t launch_velocity(const DevFields &d, const RunCfg &r, cudaStream_t s, int update,
                            int commit_speed, int advance) {
  int ty, nt;
  tiles_of(r.g, 0, &ty, &nt);
  int nb = residual_blocks(r.g);
  auto k = r.arith ? velocity_kernel<true> : velocity_kernel<false>;
  k<<<nb, kRedBlock, 0, s>>>(d.u, d.v, d.f, d.g, d.p, d.ru, d.rv, d.flags, r.g, r.c, d.st,
                             d.partials, d.log, ty, nt, update, commit_speed, advance);
  return cudaGetLastError();
}

cudaError_t launch_prange(const DevFields &d, const RunCfg &r, cudaStream_t s, int force) {
  int ty, nt;
  tiles_of(r.g, 0, &ty, &nt);
  int nb = residual_blocks(r.g);
  prange_kernel<<<nb, kRedBlock, 0, s>>>(d.p, d.flags, r.g, d.st, d.partials, ty, nt, force);
  return cudaGetLastError();
}

static Consts32 consts32_of(const Consts &c) {
  Consts32 k32;
  k32.omw = (float)c.one_minus_w;
  k32.a = (float)(c.middle * c.r_dx2);
  k32.b = (float)(c.middle * c.r_dy2);
  return k32;
}

cudaError_t launch_mixed_sweeps(const DevFields &d, const RunCfg &r, cudaStream_t s, int n) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = tb_prepare();
  if (e != cudaSuccess) return e;
  float *final = nullptr;
  const Consts32 k32 = consts32_of(r.c);
  for (const SweepLaunch &l : sweep_plan(d, r.g, n, r.sweep_schedule, &final))
    if ((e = issue_sweep(l, d.r32, d.flags, r.g, k32, s)) != cudaSuccess) return e;
  if (final != d.e32)
    e = cudaMemcpyAsync(d.e32, final, sizeof(float) * (size_t)r.g.nx * r.g.pitch,
                        cudaMemcpyDeviceToDevice, s);
  return e;
}

cudaError_t launch_sor_iteration(const DevFields &d, const RunCfg &r, cudaStream_t s, int norm) {
  int ty, nt;
  tiles_of(r.g, 1, &ty, &nt);
  if (nt == 0) return cudaSuccess;
  if (r.precision == 1) return launch_mixed_sweeps(d, r, s, 1);
  cudaError_t e = launch_pcopy(d, r.g, s);
  if (e != cudaSuccess) return e;
  dim3 sgrid((r.g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x,
             (r.g.nx - 2 + kRedBlock.y - 1) / kRedBlock.y);
  const int nb = residual_blocks(r.g);
  if (r.arith) {
    // as in the solve: the black pass also sums the black fluid cells' residual
    const int mean_free = (r.strict_eps & STOP_FLUID_NORM) && (r.strict_eps & STOP_MEAN_FREE);
    // the red pass of the solve (its update formula), without its sums
    const int bb = black_pass_blocks(r.g);
    const int nvb = (int)(sgrid.x * sgrid.y);
    sor_red_res_kernel<false, false, true><<<bb, kRedBlock, 0, s>>>(
        d.p, d.pw, d.rhs, d.cls, r.g, r.c, d.st, d.partials_r, d.partials_b, bb, nullptr, 0, 0,
        (int)sgrid.x, nvb, r.itermax, r.strict_eps, 0, 0);
    // (an empty boundary-cell list: the pass makes no boundary copy here)
    // (the red pass in mode 0 leaves no iteration for the black pass to decide)
    if (mean_free)
      sor_black_res_kernel<false, true, false><<<bb, kRedBlock, 0, s>>>(
          d.p, d.pw, d.rhs, d.flags, r.g, r.c, d.partials_b, (int)sgrid.x, nvb, nullptr, 0, 0,
          d.st, r.itermax, d.partials_r, bb, r.strict_eps, 0);
    else
      sor_black_res_kernel<false, false, false><<<bb, kRedBlock, 0, s>>>(
          d.p, d.pw, d.rhs, d.flags, r.g, r.c, d.partials_b, (int)sgrid.x, nvb, nullptr, 0, 0,
          d.st, r.itermax, d.partials_r, bb, r.strict_eps, 0);
    if (norm)
      residual_kernel<false, false><<<nb, kRedBlock, 0, s>>>(
          d.p, d.rhs, d.flags, r.g, r.c, d.st, d.partials, ty, nt, 0, r.itermax, r.strict_eps,
          RES_NORM, d.partials_b, bb);
  } else {
    for (int color = 0; color < 2; ++color)
      sor_color_kernel<<<sgrid, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, r.g, r.c, color);
    if (norm)
      residual_kernel<true, false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, r.g, r.c, d.st,
                                                            d.partials, ty, nt, 0, r.itermax,
                                                            r.strict_eps, RES_NORM, nullptr, 0);
  }
  return cudaGetLastError();
}


cudaError_t launch_sor_lex(const DevFields &d, const RunCfg &r, cudaStream_t s) {
  sor_lex_kernel<<<1, 1024, 0, s>>>(d.p, d.rhs, d.flags, d.pcopy, d.n_pcopy, r.g, r.c, d.st,
                                    d.pw, r.itermax, r.strict_eps);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// eager step: the graph's kernels launched one by one, the pressure loop
// driven from the host (one 12-byte read per iteration).  Same kernels in the
// same order, so results equal the graph's bit for bit; meant for profilers
// that cannot see into conditional graph nodes, and for debugging.
// ------------------------------------------------------------------------

static cudaError_t poll_done(const DevFields &d, cudaStream_t s, StepState *h, bool *done) {
  cudaError_t e = cudaMemcpyAsync(&h->sor_iters, &d.st->sor_iters, 4 * sizeof(unsigned int),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  *done = h->converged || h->exhausted;
  return e;
}

cudaError_t run_step_eager(const DevFields &d, const RunCfg &r, cudaStream_t s, StepState *h) {
  const Geom g = r.g;
  const Consts c = r.c;
  int ty_all, nt_all, ty_int, nt_int;
  tiles_of(g, 0, &ty_all, &nt_all);
  tiles_of(g, 1, &ty_int, &nt_int);
  const int nb = residual_blocks(g);
  cudaError_t e;
  bc_kernel<<<BC_CLUSTER, BC_THREADS, 0, s>>>(d.u, d.v, d.ru, d.rv, d.bc, d.bc_val, d.n_bc, d.st,
                                              c, r.tau, r.delt, r.itermax, 1);
  if ((e = launch_fg_rhs(d, r, s)) != cudaSuccess) return e;
  bool done = false;
  if (r.sor_order == 1) {
    if ((e = launch_sor_lex(d, r, s)) != cudaSuccess) return e;
  } else if (r.precision == 1 && nt_int > 0 && r.itermax > 0) {
    const int m = (int)((unsigned)r.inner_sweeps < r.itermax ? (unsigned)r.inner_sweeps : r.itermax);
    const Consts32 k32 = consts32_of(c);
    dim3 pgrid((g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x,
               (g.nx + kRedBlock.y - 1) / kRedBlock.y);
    if ((e = tb_prepare()) != cudaSuccess) return e;
    float *final = nullptr;
    const int coarse = m > 1 ? 1 : 0;
    const std::vector<SweepLaunch> plan =
        sweep_plan(d, g, m, r.sweep_schedule, &final, true, coarse ? d.pw : nullptr);
    refine_kernel<<<pgrid, kRedBlock, 0, s>>>(d.p, d.e32, d.e32, d.flags, g, 0, nullptr);
    mixed_residual_kernel<false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, d.r32, g, c, d.st,
                                                          d.partials, ty_int, nt_int, 0,
                                                          r.itermax, r.strict_eps, m, 0, 0, coarse,
                                                          d.pcopy, d.n_pcopy, d.e32);
    while (!done) {
      for (const SweepLaunch &l : plan)
        if ((e = issue_sweep(l, d.r32, d.flags, g, k32, s)) != cudaSuccess) return e;
      if (final)  // else the last blocked launch refined
        refine_kernel<<<pgrid, kRedBlock, 0, s>>>(d.p, final, d.e32, d.flags, g, 1,
                                                  coarse ? d.pw : nullptr);
      mixed_residual_kernel<false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, d.r32, g, c,
                                                            d.st, d.partials, ty_int, nt_int, 0,
                                                            r.itermax, r.strict_eps, m, 1, 0,
                                                            coarse, d.pcopy, d.n_pcopy, d.e32);
      if ((e = poll_done(d, s, h, &done)) != cudaSuccess) return e;
    }
    unsigned int replay = 0;
    if (coarse) {
      if ((e = cudaMemcpyAsync(&h->replay, &d.st->replay, sizeof(unsigned int),
                               cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return e;
      replay = h->replay;
    }
    if (replay) {
      // finish sweep by sweep so that the solve stops where a per-sweep test would
      restore_kernel<<<pgrid, kRedBlock, 0, s>>>(d.p, d.pw, g, d.st, m);
      refine_kernel<<<pgrid, kRedBlock, 0, s>>>(d.p, d.e32, d.e32, d.flags, g, 0, nullptr);
      mixed_residual_kernel<false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, d.r32, g, c,
                                                            d.st, d.partials, ty_int, nt_int, 0,
                                                            r.itermax, r.strict_eps, 1, 2, 0, 0,
                                                            d.pcopy, d.n_pcopy, d.e32);
      done = false;
      while (!done) {
        for (int color = 0; color < 2; ++color)
          sor32_color_kernel<<<pgrid, kRedBlock, 0, s>>>(d.e32, d.r32, d.flags, g, k32, color,
                                                         color == 0 ? 1 : 0);
        refine_kernel<<<pgrid, kRedBlock, 0, s>>>(d.p, d.e32, d.e32, d.flags, g, 1, nullptr);
        mixed_residual_kernel<false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, d.r32, g, c,
                                                              d.st, d.partials, ty_int, nt_int,
                                                              0, r.itermax, r.strict_eps, 1, 1, 0,
                                                              0, d.pcopy, d.n_pcopy, d.e32);
        if ((e = poll_done(d, s, h, &done)) != cudaSuccess) return e;
      }
    }
  } else if (nt_int > 0 && r.itermax > 0) {
    dim3 sgrid((g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x,
               (g.nx - 2 + kRedBlock.y - 1) / kRedBlock.y);
    const int nbb = (int)(sgrid.x * sgrid.y);
    if (r.strict_eps & STOP_RELATIVE) {
      // the norm the solve starts from (relative stop rule)
      if (r.arith)
        residual_kernel<false, false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, g, c, d.st,
                                                               d.partials, ty_int, nt_int, 0,
                                                               r.itermax, r.strict_eps, RES_START,
                                                               nullptr, 0);
      else
        residual_kernel<true, false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, g, c, d.st,
                                                              d.partials, ty_int, nt_int, 0,
                                                              r.itermax, r.strict_eps, RES_START,
                                                              nullptr, 0);
    }
    if (r.arith) {
      // fast arithmetic: the red pass of iteration k+1 sums iteration k's
      // red residuals and the black pass of k+1 applies k's stop test (see
      // sor_black_res_kernel); the same launches as the graph
      const FastSolveKernels fk = fast_solve_kernels(r.strict_eps, c.one_minus_w);
      const int bb = black_pass_blocks(g);
      int gx = (int)sgrid.x;
      unsigned int itermax = r.itermax;
      int strict = r.strict_eps, mode = 0;
      cudaGraphConditionalHandle h0 = 0;
      double *p = d.p, *pw = d.pw, *prt_r = d.partials_r, *prt_bw = d.partials_b;
      const double *rhs = d.rhs, *prt_b = d.partials_b;
      const uint8_t *cls = d.cls, *flags = d.flags;
      const BCell *bl = d.blist;
      StepState *st = d.st;
      Geom gg = g;
      Consts cc = c;
      int nbb_b = bb, nvb = nbb, nbl_b = d.n_blist_b, nbl = d.n_blist;
      void *red_args[] = {&p,   &pw,  &rhs,   &cls, &gg,      &cc,     &st,   &prt_r, &prt_b, &nbb_b,
                          &bl, &nbl_b, &nbl, &gx,  &nvb, &itermax, &strict, &mode, &h0};
      const double *prt_rc = d.partials_r;
      int nred = bb;
      void *black_args[] = {&p,   &pw,  &rhs,   &flags, &gg, &cc,      &prt_bw,
                            &gx,  &nvb, &bl,    &nbl_b, &nbl, &st,     &itermax,
                            &prt_rc, &nred, &strict, &h0};
      if ((e = launch_pcopy(d, g, s)) != cudaSuccess) return e;
      if ((e = cudaLaunchKernel(fk.red_eager, dim3(bb), kRedBlock, red_args, 0, s)) !=
          cudaSuccess)
        return e;
      mode = 1;
      while (!done) {
        if ((e = cudaLaunchKernel(fk.black_eager, dim3(bb), kRedBlock, black_args, 0, s)) !=
            cudaSuccess)
          return e;
        if ((e = cudaLaunchKernel(fk.red_eager, dim3(bb), kRedBlock, red_args, 0, s)) !=
            cudaSuccess)
          return e;
        if ((e = poll_done(d, s, h, &done)) != cudaSuccess) return e;
      }
      if (!fk.save)
        sor_unred_kernel<<<bb, kRedBlock, 0, s>>>(d.p, d.rhs, d.cls, g, c, d.st, r.itermax, gx,
                                                  nbb);
      sor_rollback_kernel<<<bb, kRedBlock, 0, s>>>(d.p, d.pw, d.cls, d.pcopy, d.n_pcopy, g, d.st,
                                                   r.itermax, gx, nbb, fk.save ? 1 : 0);
    }
    while (!done) {
      if ((e = launch_pcopy(d, g, s)) != cudaSuccess) return e;
      {
        for (int color = 0; color < 2; ++color)
          sor_color_kernel<<<sgrid, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, g, c, color);
        residual_kernel<true, false><<<nb, kRedBlock, 0, s>>>(d.p, d.rhs, d.flags, g, c, d.st, d.partials,
                                                              ty_int, nt_int, 0, r.itermax,
                                                              r.strict_eps, RES_SOLVE, nullptr, 0);
      }
      if ((e = poll_done(d, s, h, &done)) != cudaSuccess) return e;
    }
  }
  prange_kernel<<<nb, kRedBlock, 0, s>>>(d.p, d.flags, g, d.st, d.partials, ty_all, nt_all, 0);
  auto vk = r.arith ? velocity_kernel<true> : velocity_kernel<false>;
  vk<<<nb, kRedBlock, 0, s>>>(d.u, d.v, d.f, d.g, d.p, d.ru, d.rv, d.flags, g, c, d.st,
                              d.partials, d.log, ty_all, nt_all, 1, 1, 1);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------
// step graph
// ------------------------------------------------------------------------

namespace {

struct GraphBuilder {
  cudaGraph_t graph;
  cudaError_t err = cudaSuccess;
  // kernel parameter storage must outlive cudaGraphAddKernelNode
  std::vector<std::vector<unsigned char>> store;

  template <typename... Args>
  cudaGraphNode_t kernel(cudaGraph_t gr, cudaGraphNode_t dep, const void *fn, dim3 grid,
                         dim3 block, Args... args) {
    if (err != cudaSuccess) return nullptr;
    void *ptrs[sizeof...(Args) + 1];
    size_t i = 0;
    (void)std::initializer_list<int>{(ptrs[i++] = keep(args), 0)...};
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void *>(fn);
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.sharedMemBytes = 0;
    kp.kernelParams = ptrs;
    kp.extra = nullptr;
    cudaGraphNode_t node = nullptr;
    err = cudaGraphAddKernelNode(&node, gr, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
    return node;
  }

  template <typename... Args>
  cudaGraphNode_t kernel_smem(cudaGraph_t gr, cudaGraphNode_t dep, const void *fn, dim3 grid,
                              dim3 block, size_t smem, Args... args) {
    if (err != cudaSuccess) return nullptr;
    void *ptrs[sizeof...(Args) + 1];
    size_t i = 0;
    (void)std::initializer_list<int>{(ptrs[i++] = keep(args), 0)...};
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void *>(fn);
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.sharedMemBytes = (unsigned int)smem;
    kp.kernelParams = ptrs;
    kp.extra = nullptr;
    cudaGraphNode_t node = nullptr;
    err = cudaGraphAddKernelNode(&node, gr, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
    return node;
  }

  // the same as kernel(), the edge from dep programmatic: the node's blocks
  // may start once every block of dep has triggered (pdl_trigger) or ended,
  // and wait (pdl_wait) for dep's completion themselves
  template <typename... Args>
  cudaGraphNode_t kernel_pdl(cudaGraph_t gr, cudaGraphNode_t dep, const void *fn, dim3 grid,
                             dim3 block, Args... args) {
    if (!dep) return kernel(gr, dep, fn, grid, block, args...);
    cudaGraphNode_t node = kernel(gr, nullptr, fn, grid, block, args...);
    if (err != cudaSuccess) return nullptr;
    cudaGraphEdgeData ed{};
    ed.from_port = cudaGraphKernelNodePortProgrammatic;
    ed.type = cudaGraphDependencyTypeProgrammatic;
    err = cudaGraphAddDependencies(gr, &dep, &node, &ed, 1);
    return node;
  }

  template <typename T>
  void *keep(const T &v) {
    store.emplace_back(sizeof(T));
    memcpy(store.back().data(), &v, sizeof(T));
    return store.back().data();
  }
};

std::atomic<int> g_fast_pdl{1};

}  // namespace

int set_fast_pdl(int on) { return g_fast_pdl.exchange(on ? 1 : 0); }
int fast_pdl() { return g_fast_pdl.load(); }

cudaError_t build_step_graph(const DevFields &d, const RunCfg &r, cudaGraph_t *out, int part) {
  GraphBuilder b;
  cudaError_t e = cudaGraphCreate(&b.graph, 0);
  if (e != cudaSuccess) return e;
  b.store.reserve(256);
  const Geom g = r.g;
  const Consts c = r.c;
  int ty_all, nt_all, ty_int, nt_int;
  tiles_of(g, 0, &ty_all, &nt_all);
  tiles_of(g, 1, &ty_int, &nt_int);
  const int nb = residual_blocks(g);

  cudaGraphNode_t n = nullptr;
  if (part != 2 && part != 3) {
    n = b.kernel(b.graph, nullptr, (const void *)bc_kernel, dim3(BC_CLUSTER), dim3(BC_THREADS),
                 d.u, d.v, d.ru, d.rv, (const BcEntry *)d.bc, d.bc_val, d.n_bc, d.st, c, r.tau,
                 r.delt, r.itermax, 1);
    dim3 fg_grid((g.ny + FG_TY - 1) / FG_TY, (g.nx + FG_TX - 1) / FG_TX);
    if (r.precision == 1) {
      n = b.kernel(b.graph, n, (const void *)fg_rhs32_kernel, fg_grid, dim3(FG_THREADS),
                   (const double *)d.u, (const double *)d.v, d.f, d.g, d.rhs,
                   (const uint8_t *)d.flags, g, c, consts32f_of(c), (const StepState *)d.st);
    } else if (r.arith) {
      if (b.err == cudaSuccess) b.err = ff_prepare();
      n = b.kernel_smem(b.graph, n, (const void *)fg_rhs_fast_kernel, ff_grid(g),
                        dim3(FF_THREADS), sizeof(FastFgSmem), (const double *)d.u,
                        (const double *)d.v, d.f, d.g, d.rhs, (const uint8_t *)d.flags, g, c,
                        (const StepState *)d.st);
    } else {
      n = b.kernel(b.graph, n, (const void *)fg_rhs_kernel, fg_grid, dim3(FG_THREADS),
                   (const double *)d.u, (const double *)d.v, d.f, d.g, d.rhs,
                   (const uint8_t *)d.flags, g, c, (const StepState *)d.st);
    }
  }
  if (part == 1 || part == 3) {
    // the first half of a step ends after the RHS; part 3 is the second
    // half without the pressure solve (run by a batch)
  } else if (r.sor_order == 1) {
    n = b.kernel(b.graph, n, (const void *)sor_lex_kernel, dim3(1), dim3(1024), d.p,
                 (const double *)d.rhs, (const uint8_t *)d.flags, (const PCopy *)d.pcopy,
                 d.n_pcopy, g, c, d.st, d.pw, r.itermax, r.strict_eps);
  } else if (r.precision == 1 && nt_int > 0 && r.itermax > 0) {
    const int m = (int)((unsigned)r.inner_sweeps < r.itermax ? (unsigned)r.inner_sweeps : r.itermax);
    const Consts32 k32 = consts32_of(c);
    dim3 pgrid((g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x,
               (g.nx + kRedBlock.y - 1) / kRedBlock.y);
    if (b.err == cudaSuccess) b.err = tb_prepare();
    float *final = nullptr;
    const int coarse_g = m > 1 ? 1 : 0;
    const std::vector<SweepLaunch> plan =
        sweep_plan(d, g, m, r.sweep_schedule, &final, true, coarse_g ? d.pw : nullptr);
    cudaGraphConditionalHandle h;
    if (b.err == cudaSuccess)
      b.err = cudaGraphConditionalHandleCreate(&h, b.graph, 1, cudaGraphCondAssignDefault);
    n = b.kernel(b.graph, n, (const void *)refine_kernel, pgrid, kRedBlock, d.p,
                 (const float *)d.e32, d.e32, (const uint8_t *)d.flags, g, 0, (double *)nullptr);
    const int coarse = m > 1 ? 1 : 0;
    cudaGraphConditionalHandle h_rep{};
    if (b.err == cudaSuccess)
      b.err = cudaGraphConditionalHandleCreate(&h_rep, b.graph, 0, cudaGraphCondAssignDefault);
    n = b.kernel(b.graph, n, (const void *)mixed_residual_kernel<true>, dim3(nb), kRedBlock,
                 (const double *)d.p, (const double *)d.rhs, (const uint8_t *)d.flags, d.r32, g,
                 c, d.st, d.partials, ty_int, nt_int, h, r.itermax, r.strict_eps, m, 0, h_rep,
                 coarse, (const PCopy *)d.pcopy, d.n_pcopy, d.e32);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (b.err == cudaSuccess)
      b.err = cudaGraphAddNode(&wnode, b.graph, n ? &n : nullptr, nullptr, n ? 1 : 0, &cp);
    if (b.err == cudaSuccess) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      cudaGraphNode_t bn = nullptr;
      for (const SweepLaunch &l : plan) {
        if (l.smem == 0)
          bn = b.kernel(body, bn, l.fn, l.grid, l.block, l.eout, (const float *)d.r32,
                        (const uint8_t *)d.flags, g, k32, l.color, l.copy);
        else
          bn = b.kernel_smem(body, bn, l.fn, l.grid, l.block, l.smem, l.ein, l.eout,
                             (const float *)d.r32, (const uint8_t *)d.flags, g, k32, l.tiles_y,
                             l.n, l.skip_last_copy, l.pf, l.pw);
      }
      // the refinement also keeps p before this outer iteration (for a redo);
      // the last blocked launch did it when final is NULL
      if (final)
        bn = b.kernel(body, bn, (const void *)refine_kernel, pgrid, kRedBlock, d.p,
                      (const float *)final, d.e32, (const uint8_t *)d.flags, g, 1,
                      coarse ? d.pw : (double *)nullptr);
      bn = b.kernel(body, bn, (const void *)mixed_residual_kernel<true>, dim3(nb), kRedBlock,
                    (const double *)d.p, (const double *)d.rhs, (const uint8_t *)d.flags, d.r32,
                    g, c, d.st, d.partials, ty_int, nt_int, h, r.itermax, r.strict_eps, m, 1,
                    h_rep, coarse, (const PCopy *)d.pcopy, d.n_pcopy, d.e32);
    }
    n = wnode;
    if (coarse) {
      // IF the coarse loop stopped between checks: redo / finish sweep by sweep
      cudaGraphNodeParams ip = {};
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = h_rep;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      cudaGraphNode_t inode = nullptr;
      if (b.err == cudaSuccess)
        b.err = cudaGraphAddNode(&inode, b.graph, &n, nullptr, 1, &ip);
      if (b.err == cudaSuccess) {
        cudaGraph_t ib = ip.conditional.phGraph_out[0];
        cudaGraphNode_t fn = nullptr;
        fn = b.kernel(ib, fn, (const void *)restore_kernel, pgrid, kRedBlock, d.p,
                      (const double *)d.pw, g, d.st, m);
        fn = b.kernel(ib, fn, (const void *)refine_kernel, pgrid, kRedBlock, d.p,
                      (const float *)d.e32, d.e32, (const uint8_t *)d.flags, g, 0,
                      (double *)nullptr);
        cudaGraphConditionalHandle h_fine{};
        if (b.err == cudaSuccess)
          b.err = cudaGraphConditionalHandleCreate(&h_fine, ib, 1, cudaGraphCondAssignDefault);
        fn = b.kernel(ib, fn, (const void *)mixed_residual_kernel<true>, dim3(nb), kRedBlock,
                      (const double *)d.p, (const double *)d.rhs, (const uint8_t *)d.flags,
                      d.r32, g, c, d.st, d.partials, ty_int, nt_int, h_fine, r.itermax,
                      r.strict_eps, 1, 2, h_fine, 0, (const PCopy *)d.pcopy, d.n_pcopy,
                      d.e32);
        cudaGraphNodeParams fp = {};
        fp.type = cudaGraphNodeTypeConditional;
        fp.conditional.handle = h_fine;
        fp.conditional.type = cudaGraphCondTypeWhile;
        fp.conditional.size = 1;
        cudaGraphNode_t fw = nullptr;
        if (b.err == cudaSuccess) b.err = cudaGraphAddNode(&fw, ib, &fn, nullptr, 1, &fp);
        if (b.err == cudaSuccess) {
          cudaGraph_t fb = fp.conditional.phGraph_out[0];
          cudaGraphNode_t x = nullptr;
          for (int color = 0; color < 2; ++color)
            x = b.kernel(fb, x, (const void *)sor32_color_kernel, pgrid, kRedBlock, d.e32,
                         (const float *)d.r32, (const uint8_t *)d.flags, g, k32, color,
                         color == 0 ? 1 : 0);
          x = b.kernel(fb, x, (const void *)refine_kernel, pgrid, kRedBlock, d.p,
                       (const float *)d.e32, d.e32, (const uint8_t *)d.flags, g, 1,
                       (double *)nullptr);
          x = b.kernel(fb, x, (const void *)mixed_residual_kernel<true>, dim3(nb), kRedBlock,
                       (const double *)d.p, (const double *)d.rhs, (const uint8_t *)d.flags,
                       d.r32, g, c, d.st, d.partials, ty_int, nt_int, h_fine, r.itermax,
                       r.strict_eps, 1, 1, h_fine, 0, (const PCopy *)d.pcopy, d.n_pcopy,
                       d.e32);
        }
      }
      n = inode;
    }
  } else if (nt_int > 0 && r.itermax > 0) {
    cudaGraphConditionalHandle h;
    if (b.err == cudaSuccess)
      b.err = cudaGraphConditionalHandleCreate(&h, b.graph, 1, cudaGraphCondAssignDefault);
    if (r.strict_eps & STOP_RELATIVE) {
      // the norm the solve starts from (relative stop rule)
      const void *k0 = r.arith ? (const void *)residual_kernel<false, false>
                               : (const void *)residual_kernel<true, false>;
      n = b.kernel(b.graph, n, k0, dim3(nb), kRedBlock, (const double *)d.p,
                   (const double *)d.rhs, (const uint8_t *)d.flags, g, c, d.st, d.partials,
                   ty_int, nt_int, h, r.itermax, r.strict_eps, (int)RES_START,
                   (const double *)nullptr, 0);
    }
    dim3 sgrid((g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x,
               (g.nx - 2 + kRedBlock.y - 1) / kRedBlock.y);
    const int nbb = (int)(sgrid.x * sgrid.y);
    const int bb = black_pass_blocks(g);
    const FastSolveKernels fk = fast_solve_kernels(r.strict_eps, c.one_minus_w);
    if (r.arith) {
      // fast arithmetic: first copy and red pass outside the loop; the red
      // pass of iteration k+1 sums iteration k's red residuals, the black
      // pass of k+1 applies k's stop test (sor_black_res_kernel)
      if (d.n_pcopy > 0)
        n = b.kernel(b.graph, n, (const void *)pcopy_kernel, dim3((d.n_pcopy + 255) / 256),
                     dim3(256), d.p, (const PCopy *)d.pcopy, d.n_pcopy, g.pitch);
      n = b.kernel(b.graph, n, fk.red_graph, dim3(bb), kRedBlock, d.p, d.pw,
                   (const double *)d.rhs, (const uint8_t *)d.cls, g, c, d.st, d.partials_r,
                   (const double *)d.partials_b, bb, (const BCell *)d.blist, d.n_blist_b,
                   d.n_blist, (int)sgrid.x, nbb, r.itermax, r.strict_eps, 0, h);
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (b.err == cudaSuccess)
      b.err = cudaGraphAddNode(&wnode, b.graph, n ? &n : nullptr, nullptr, n ? 1 : 0, &cp);
    if (b.err == cudaSuccess) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      cudaGraphNode_t bn = nullptr;
      if (r.arith) {
        // kFastBodyIters iterations per evaluation of the WHILE condition;
        // the passes after the one that stopped the solve return at once.
        // Within the body each pass follows the previous one by a
        // programmatic edge unless switched off (set_fast_pdl)
        const bool pdl = g_fast_pdl.load() != 0;
        auto pass = [&](const void *fn, auto... args) {
          bn = pdl ? b.kernel_pdl(body, bn, fn, dim3(bb), kRedBlock, args...)
                   : b.kernel(body, bn, fn, dim3(bb), kRedBlock, args...);
        };
        for (int i = 0; i < kFastBodyIters; ++i) {
          pass(fk.black_graph, d.p, d.pw, (const double *)d.rhs, (const uint8_t *)d.flags, g,
               c, d.partials_b, (int)sgrid.x, nbb, (const BCell *)d.blist, d.n_blist_b,
               d.n_blist, d.st, r.itermax, (const double *)d.partials_r, bb, r.strict_eps, h);
          pass(fk.red_graph, d.p, d.pw, (const double *)d.rhs, (const uint8_t *)d.cls, g, c,
               d.st, d.partials_r, (const double *)d.partials_b, bb, (const BCell *)d.blist,
               d.n_blist_b, d.n_blist, (int)sgrid.x, nbb, r.itermax, r.strict_eps, 1, h);
        }
      } else {
        if (d.n_pcopy > 0)
          bn = b.kernel(body, nullptr, (const void *)pcopy_kernel, dim3((d.n_pcopy + 255) / 256),
                        dim3(256), d.p, (const PCopy *)d.pcopy, d.n_pcopy, g.pitch);
        const void *kc = (const void *)sor_color_kernel;
        const void *kr = (const void *)residual_kernel<true, true>;
        for (int color = 0; color < 2; ++color)
          bn = b.kernel(body, bn, kc, sgrid, kRedBlock, d.p, (const double *)d.rhs,
                        (const uint8_t *)d.flags, g, c, color);
        bn = b.kernel(body, bn, kr, dim3(nb), kRedBlock, (const double *)d.p,
                      (const double *)d.rhs, (const uint8_t *)d.flags, g, c, d.st, d.partials,
                      ty_int, nt_int, h, r.itermax, r.strict_eps, (int)RES_SOLVE,
                      (const double *)nullptr, 0);
      }
    }
    n = wnode;
    if (r.arith && !fk.save)
      n = b.kernel(b.graph, n, (const void *)sor_unred_kernel, dim3(bb), kRedBlock, d.p,
                   (const double *)d.rhs, (const uint8_t *)d.cls, g, c, (const StepState *)d.st,
                   r.itermax, (int)sgrid.x, nbb);
    if (r.arith)
      n = b.kernel(b.graph, n, (const void *)sor_rollback_kernel, dim3(bb), kRedBlock, d.p,
                   (const double *)d.pw, (const uint8_t *)d.cls, (const PCopy *)d.pcopy,
                   d.n_pcopy, g, (const StepState *)d.st, r.itermax, (int)sgrid.x, nbb,
                   fk.save ? 1 : 0);
  }
  if (part != 1) {
    n = b.kernel(b.graph, n, (const void *)prange_kernel, dim3(nb), kRedBlock,
                 (const double *)d.p, (const uint8_t *)d.flags, g, d.st, d.partials, ty_all,
                 nt_all, 0);
    n = b.kernel(b.graph, n,
                 r.arith ? (const void *)velocity_kernel<true> : (const void *)velocity_kernel<false>,
                 dim3(nb), kRedBlock, d.u, d.v,
                 (const double *)d.f, (const double *)d.g, (const double *)d.p,
                 (const double *)d.ru, (const double *)d.rv, (const uint8_t *)d.flags, g, c,
                 d.st, d.partials, d.log, ty_all, nt_all, 1, 1, 1);
  }
  if (b.err != cudaSuccess) {
    cudaGraphDestroy(b.graph);
    return b.err;
  }
  *out = b.graph;
  return cudaSuccess;
}


// ------------------------------------------------------------------------
// Batches: many independent simulations stepped by one graph.  Each
// instance's boundary pass, F/G/RHS, pressure range and velocity update are
// its own kernels (parallel branches of the graph); the mixed-precision
// pressure solve of all instances is one WHILE loop whose kernels cover
// every instance through tables of (instance, block / tile / entry) pairs,
// skip instances whose solve has stopped, and run each instance's work with
// exactly its single-instance block shapes and reduction order, so every
// instance ends bit-identical to a run of its own.
// ------------------------------------------------------------------------

struct BInst {
  double *p, *rhs;
  double *pw;            // p before the current coarse outer iteration
  const uint8_t *flags;
  float *e32, *e32b, *r32;
  StepState *st;
  double *partials;
  const PCopy *pcopy;
  int npc;               // boundary cells of the copy (pcopy entries)
  Geom g;
  Consts c;
  Consts32 k32;
  unsigned int itermax;
  int strict;
  int solve;             // 0: no pressure solve (no interior or max_iterations 0)
  int nb, ty_int, nt_int;
  int pgx;               // refine grid width (blocks)
  int tb_tiles_y;
};

struct BatchState {
  unsigned int counter;
  unsigned int active;
  unsigned int body_count;
  unsigned int launches;  // independent count of loop bodies (block 0)
  unsigned int replays;   // members that finish sweep by sweep
  // persistent solve: grid barrier, the loop decision of each body (by
  // parity) and of the finishing pass
  unsigned int bar_count;
  unsigned int bar_gen;
  unsigned int go[2];
  unsigned int open_replay;
  unsigned int work[2];   // next table entry of the current phase (by parity)
  // the fields above are zeroed before every persistent solve (a solve cut
  // short by a barrier timeout can leave them anywhere); these two collect
  // over the steps of one call and are reset by the host before it
  unsigned int overrun;   // a loop passed its bound
  unsigned int timeout;   // a CTA of the persistent solve gave up waiting
};

__device__ __forceinline__ bool inst_stopped(const StepState *st) {
  return st->converged || st->exhausted;
}

// Phase of the batched solve a kernel serves: the coarse loop (m sweeps per
// check; every solving member until it stops) or the sweep-by-sweep
// finishing pass (members whose coarse loop stopped between checks).
__device__ __forceinline__ bool in_phase(const BInst &b, int fine) {
  return b.solve && (!fine || b.st->replay != 0u);
}

// The batch kernels' work for one (instance, block) table entry, shared by
// the graph's kernels (one entry per CTA) and the persistent solve (each CTA
// walks the table).
__device__ __forceinline__ void batch_refine_body(const BInst *__restrict__ I, int2 e, int apply,
                                                  int final_b, int fine, int save,
                                                  const Thr t = thr_cta()) {
  const BInst &b = I[e.x];
  if (!in_phase(b, fine) || (apply && inst_stopped(b.st))) return;
  refine_cells(b.p, final_b ? b.e32b : b.e32, b.e32, b.flags, b.g, apply, e.y % b.pgx,
               e.y / b.pgx, (apply && !fine && save) ? b.pw : nullptr, t);
}

template <int H, int TX, int TY, int WARPS, bool COH>
__device__ __forceinline__ void batch_tb_body(const BInst *__restrict__ I, int2 e, int n,
                                              int skip_last_copy, int src_b, int finish,
                                              int save, unsigned char *smem_raw) {
  const BInst &b = I[e.x];
  if (!b.solve || inst_stopped(b.st)) return;
  // finish: the outer iteration's last launch also refines (as for one
  // simulation, see sweep_plan)
  sor32_tb_tile<H, TX, TY, WARPS, COH>(src_b ? b.e32b : b.e32, src_b ? b.e32 : b.e32b, b.r32,
                                  b.flags, b.g, b.k32, e.y, b.tb_tiles_y, n, skip_last_copy,
                                  smem_raw, finish ? b.p : nullptr,
                                  (finish && save) ? b.pw : nullptr);
}

__device__ __forceinline__ void batch_restore_body(const BInst *__restrict__ I, int2 e, int m,
                                                   const Thr t = thr_cta()) {
  const BInst &b = I[e.x];
  if (!b.solve) return;
  StepState *st = b.st;
  const unsigned int replay = st->replay;
  const bool lead = e.y == 0 && t.tid == 0;
  if (replay == 2u && lead) st->exhausted = 0;
  if (replay != 1u) return;
  const Geom &g = b.g;
  const int x = (e.y / b.pgx) * t.dy + t.ty;
  const int y0 = 2 * ((e.y % b.pgx) * t.dx + t.tx);
  if (x < g.nx) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
      if (y0 + q < g.ny) b.p[OFF(x, y0 + q)] = b.pw[OFF(x, y0 + q)];
  }
  if (lead) {
    st->sor_iters -= (unsigned int)m;
    if (st->hist_n > 0) st->hist_n -= 1;
    st->converged = 0;
  }
}

template <bool COH>
__device__ __forceinline__ void batch_color_body(const BInst *__restrict__ I, int2 e, int color,
                                                 int copy, const Thr t = thr_cta()) {
  const BInst &b = I[e.x];
  if (!in_phase(b, 1) || inst_stopped(b.st)) return;
  sor32_color_cells<COH>(b.e32, b.r32, b.flags, b.g, b.k32, color, copy, e.y % b.pgx,
                         e.y / b.pgx, t);
}

template <bool COH, bool GRP = false>
__device__ __forceinline__ void batch_residual_body(const BInst *__restrict__ I, int2 e,
                                                    int check, int fine,
                                                    const Thr t = thr_cta(),
                                                    double *scratch = nullptr) {
  const BInst &b = I[e.x];
  if (!in_phase(b, fine) || (check == 1 && inst_stopped(b.st))) return;
  // the member's boundary deltas, block-strided over its nb blocks (as
  // mixed_residual_kernel does for one simulation)
  const int nt = t.dx * t.dy;
  for (int k = e.y * nt + t.tid; k < b.npc; k += b.nb * nt)
    delta_entry<COH>(b.p, b.r32, b.e32, b.pcopy[k], b.g.pitch);
  mixed_residual_partial<COH, GRP>(b.p, b.rhs, b.flags, b.r32, b.g, b.c, b.partials,
                                   b.ty_int, b.nt_int, b.strict, e.y, b.nb, t, scratch);
}

__global__ void __launch_bounds__(256)
    batch_refine_kernel(const BInst *__restrict__ I, const int2 *__restrict__ tab, int apply,
                        int final_b, int fine, int save) {
  batch_refine_body(I, tab[blockIdx.x], apply, final_b, fine, save);
}

template <int H, int TX, int TY>
__global__ void __launch_bounds__(512)
    batch_tb_kernel(const BInst *__restrict__ I, const int2 *__restrict__ tab, int n,
                    int skip_last_copy, int src_b, int finish, int save) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  batch_tb_body<H, TX, TY, 16, false>(I, tab[blockIdx.x], n, skip_last_copy, src_b, finish,
                                      save, smem_raw);
}

__global__ void __launch_bounds__(256)
    batch_restore_kernel(const BInst *__restrict__ I, const int2 *__restrict__ tab, int m) {
  batch_restore_body(I, tab[blockIdx.x], m);
}

// One colour pass of the finishing members
__global__ void __launch_bounds__(256)
    batch_color_kernel(const BInst *__restrict__ I, const int2 *__restrict__ tab, int color,
                       int copy) {
  batch_color_body<false>(I, tab[blockIdx.x], color, copy);
}

__global__ void __launch_bounds__(256)
    batch_residual_kernel(const BInst *__restrict__ I, const int2 *__restrict__ tab, int check,
                          int fine) {
  batch_residual_body<false>(I, tab[blockIdx.x], check, fine);
}

// One block per instance: its norm and stop rule; the last block to finish
// ends the WHILE loop once no instance goes on, or when the loop passes its
// bound (max max_iterations / sweeps + 2 launches).
__global__ void __launch_bounds__(256)
    batch_finish_kernel(const BInst *__restrict__ I, int n, BatchState *bs,
                        cudaGraphConditionalHandle h, int sweeps, int check,
                        unsigned int itermax_all, int fine, cudaGraphConditionalHandle h_rep) {
  const BInst &b = I[blockIdx.x];
  const bool active = in_phase(b, fine) && !(check && inst_stopped(b.st));
  if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    // Independent bound on the WHILE loop: the normal stop below ends it
    // after max max_iterations / sweeps bodies at the latest; should that
    // bookkeeping ever fail, this ends it two bodies later.
    if (!check) {
      if (!fine) bs->launches = 0;
    } else {
      const unsigned int l = atomicAdd(&bs->launches, 1u) + 1;
      if ((unsigned long long)l * sweeps >= itermax_all + 2ull * sweeps) {
        bs->overrun = 1;
        cudaGraphSetConditional(h, 0);
      }
    }
  }
  __syncthreads();
  int status = SOLVE_GO_ON;
  if (active)
    status = mixed_residual_stop(b.partials, b.nb, b.st, b.c, b.itermax, b.strict, sweeps, check);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (active && status == SOLVE_GO_ON) atomicAdd(&bs->active, 1u);
    if (active && check && status != SOLVE_GO_ON && !fine && sweeps > 1) {
      const unsigned int rp = replay_of(status, b.st, b.itermax);
      b.st->replay = rp;
      if (rp) atomicAdd(&bs->replays, 1u);
    }
    __threadfence();
    const unsigned int t = atomicAdd(&bs->counter, 1u);
    if (t == (unsigned int)n - 1) {
      __threadfence();
      const unsigned int act = atomicAdd(&bs->active, 0u);
      if (check) {
        const unsigned int body = bs->body_count + 1;
        bs->body_count = body;
        if (act == 0) {
          cudaGraphSetConditional(h, 0);
          if (!fine && atomicAdd(&bs->replays, 0u) > 0) cudaGraphSetConditional(h_rep, 1);
        } else if ((unsigned long long)body * sweeps >= itermax_all + 2ull * sweeps) {
          bs->overrun = 1;
          cudaGraphSetConditional(h, 0);
        }
      } else if (!fine) {
        bs->body_count = 0;
        bs->replays = 0;
      }
      bs->active = 0;
      bs->counter = 0;
    }
  }
}

// ------------------------------------------------------------------------
// Persistent batch solve: the whole WHILE loop above (coarse loop, stop
// tests, the sweep-by-sweep finishing pass) as one cooperative kernel.  Its
// CTAs (all resident: cooperative launch) walk the same (instance, block)
// tables phase by phase, calling the graph kernels' bodies, so every member
// ends bit-identical to the graph loop and to stepping it alone.  Phases are
// separated by a grid barrier whose wait is bounded: after `limit` polls a
// CTA sets BatchState::timeout and returns, and every other CTA returns at
// its next wait; the host then reports STRM_ERR_TIMEOUT.  No CTA spins
// without a bound and none traps.
// ------------------------------------------------------------------------

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier (generation counter).  Returns false in every thread of
// a CTA whose wait ran out or that found another CTA's wait run out.
__device__ __forceinline__ bool grid_barrier(BatchState *bs, unsigned long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    int ok = 1;
    const unsigned int gen = ld_acquire_u32(&bs->bar_gen);
    __threadfence();
    const unsigned int arrived = atomicAdd(&bs->bar_count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&bs->bar_count, 0u);
      __threadfence();
      atomicAdd(&bs->bar_gen, 1u);
    } else {
      unsigned long long polls = 0;
      while (ld_acquire_u32(&bs->bar_gen) == gen) {
        if (ld_acquire_u32(&bs->timeout) != 0u || ++polls > limit) {
          atomicExch(&bs->timeout, 1u);
          break;
        }
        __nanosleep(64);
      }
    }
    if (ld_acquire_u32(&bs->timeout) != 0u) ok = 0;
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// batch_finish_kernel's work for member `mi`, the loop decisions written to
// bs->go[par] (another body) and bs->open_replay instead of graph
// conditionals.
__device__ __forceinline__ void batch_finish_body(const BInst *__restrict__ I, int mi, int n,
                                                  BatchState *bs, int sweeps, int check,
                                                  unsigned int itermax_all, int fine, int par,
                                                  const Thr &t, double *scratch) {
  const BInst &b = I[mi];
  const bool active = in_phase(b, fine) && !(check && inst_stopped(b.st));
  if (mi == 0 && t.tid == 0) {
    if (!check) {
      if (!fine) bs->launches = 0;
    } else {
      const unsigned int l = atomicAdd(&bs->launches, 1u) + 1;
      if ((unsigned long long)l * sweeps >= itermax_all + 2ull * sweeps) {
        bs->overrun = 1;
        atomicExch(&bs->go[par], 0u);
      }
    }
  }
  gsync(t);
  int status = SOLVE_GO_ON;
  if (active)
    status = mixed_residual_stop_g(b.partials, b.nb, b.st, b.c, b.itermax, b.strict, sweeps,
                                   check, t, scratch);
  if (t.tid == 0) {
    if (active && status == SOLVE_GO_ON) atomicAdd(&bs->active, 1u);
    if (active && check && status != SOLVE_GO_ON && !fine && sweeps > 1) {
      const unsigned int rp = replay_of(status, b.st, b.itermax);
      b.st->replay = rp;
      if (rp) atomicAdd(&bs->replays, 1u);
    }
    __threadfence();
    const unsigned int ticket = atomicAdd(&bs->counter, 1u);
    if (ticket == (unsigned int)n - 1) {
      __threadfence();
      const unsigned int act = atomicAdd(&bs->active, 0u);
      if (check) {
        const unsigned int body = bs->body_count + 1;
        bs->body_count = body;
        if (act == 0) {
          atomicExch(&bs->go[par], 0u);
          if (!fine && atomicAdd(&bs->replays, 0u) > 0) atomicExch(&bs->open_replay, 1u);
        } else if ((unsigned long long)body * sweeps >= itermax_all + 2ull * sweeps) {
          bs->overrun = 1;
          atomicExch(&bs->go[par], 0u);
        }
      } else if (!fine) {
        bs->body_count = 0;
        bs->replays = 0;
      }
      bs->active = 0;
      bs->counter = 0;
    }
  }
}

struct PersistArgs {
  const BInst *inst;
  const int2 *t_res, *t_ref, *t_tb;
  int nres, nref, ntb, n;
  BatchState *bs;
  int m;             // sweeps per stop test
  int sweeps;        // sweeps per blocked tile pass
  int fused;         // the last blocked pass of an outer iteration refines
  unsigned int itermax_all;
  unsigned long long limit;  // polls a barrier wait may take
};

constexpr int kPersistWarps = 16;  // CTA of (32, 16) threads: two (32, 8) groups
// Members whose state bits each CTA keeps in shared memory (larger batches
// read each member's state from global memory in every phase).
constexpr int kPersistMaxMembers = 1024;
enum : uint8_t { ACT_SOLVE = 1, ACT_STOPPED = 2, ACT_REPLAY = 4 };

template <int H, int TX, int TY>
__global__ void __launch_bounds__(32 * kPersistWarps, 3)
    batch_persistent_kernel(PersistArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const BInst *I = a.inst;
  BatchState *bs = a.bs;
  // the two 256-thread groups of the CTA: each takes its own table entry in
  // the (32 x 8)-block phases; their reduction scratch is the start of the
  // sweep tiles' dynamic shared memory (free between tile phases)
  Thr t;
  t.tx = threadIdx.x;
  t.ty = threadIdx.y & 7;
  t.dx = 32;
  t.dy = 8;
  t.tid = t.tx + 32 * t.ty;
  t.half = threadIdx.y >> 3;
  t.bar = 1 + t.half;
  double *scratch = reinterpret_cast<double *>(smem_raw);
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0;
  const int gstart = 2 * blockIdx.x + t.half, gstride = 2 * gridDim.x;
  // every member's state bits, refreshed after each phase that changes them
  // (the stop tests, the finishing pass's restore), so that entries of
  // members a phase does not touch are skipped without a global load; the
  // bodies still apply their own tests to the entries they get
  __shared__ uint8_t s_act[kPersistMaxMembers];
  __shared__ int s_next[3];  // next entry: the CTA's, then each group's
  const int ctid = threadIdx.y * 32 + threadIdx.x;
  unsigned int phase = 0;    // dynamically scheduled phases so far
  const bool masked = a.n <= kPersistMaxMembers;
  auto refresh = [&]() {
    if (masked) {
      const int tid = threadIdx.y * 32 + threadIdx.x;
      for (int i = tid; i < a.n; i += 32 * kPersistWarps) {
        const BInst &b = I[i];
        uint8_t v = b.solve ? ACT_SOLVE : 0;
        if (b.solve) {
          const StepState *st = b.st;
          if (__ldcg(&st->converged) || __ldcg(&st->exhausted)) v |= ACT_STOPPED;
          if (__ldcg(&st->replay) != 0u) v |= ACT_REPLAY;
        }
        s_act[i] = v;
      }
    }
    __syncthreads();
  };
  // skip tests: no solve; stopped or no solve; not finishing; not finishing
  // or stopped
  auto no_solve = [&](int mi) { return masked && !(s_act[mi] & ACT_SOLVE); };
  auto idle = [&](int mi) {
    return masked && (s_act[mi] & (ACT_SOLVE | ACT_STOPPED)) != ACT_SOLVE;
  };
  auto no_fine = [&](int mi) {
    return masked && (s_act[mi] & (ACT_SOLVE | ACT_REPLAY)) != (ACT_SOLVE | ACT_REPLAY);
  };
  auto idle_fine = [&](int mi) {
    return masked && (s_act[mi] & (ACT_SOLVE | ACT_REPLAY | ACT_STOPPED)) !=
                         (ACT_SOLVE | ACT_REPLAY);
  };
  refresh();
// Entries are handed out dynamically: a CTA (or a group) takes the next
// entry of the phase from an atomic counter, asked for one entry ahead so
// that the atomic's latency overlaps the work; which CTA does an entry does
// not change its result.  The counters alternate by phase parity: the one
// of the previous phase is cleared during this one (every CTA has passed
// the barrier that ended it).
// a phase over the sweep tiles: one entry per CTA at a time
#define TILE_PHASE(N, TAB, SKIP, BODY)                                       \
  {                                                                          \
    unsigned int *ctr = &bs->work[phase & 1];                                \
    if (lead) atomicExch(&bs->work[(phase & 1) ^ 1], 0u);                    \
    if (ctid == 0) s_next[0] = (int)atomicAdd(ctr, 1u);                      \
    __syncthreads();                                                         \
    int vb = s_next[0];                                                      \
    while (vb < (N)) {                                                       \
      __syncthreads();                                                       \
      int nxt = 0;                                                           \
      if (ctid == 0) nxt = (int)atomicAdd(ctr, 1u);                          \
      if (!SKIP((TAB)[vb].x)) {                                              \
        BODY;                                                                \
      }                                                                      \
      if (ctid == 0) s_next[0] = nxt;                                        \
      __syncthreads();                                                       \
      vb = s_next[0];                                                        \
    }                                                                        \
    ++phase;                                                                 \
  }                                                                          \
  if (!grid_barrier(bs, a.limit)) return;
// a phase over (32 x 8)-block entries: one entry per group at a time
#define GROUP_PHASE(N, TAB, SKIP, BODY)                                      \
  {                                                                          \
    unsigned int *ctr = &bs->work[phase & 1];                                \
    if (lead) atomicExch(&bs->work[(phase & 1) ^ 1], 0u);                    \
    if (t.tid == 0) s_next[1 + t.half] = (int)atomicAdd(ctr, 1u);            \
    gsync(t);                                                                \
    int vb = s_next[1 + t.half];                                             \
    while (vb < (N)) {                                                       \
      gsync(t);                                                              \
      int nxt = 0;                                                           \
      if (t.tid == 0) nxt = (int)atomicAdd(ctr, 1u);                         \
      if (!SKIP((TAB)[vb].x)) {                                              \
        BODY;                                                                \
      }                                                                      \
      if (t.tid == 0) s_next[1 + t.half] = nxt;                              \
      gsync(t);                                                              \
      vb = s_next[1 + t.half];                                               \
    }                                                                        \
    ++phase;                                                                 \
  }                                                                          \
  if (!grid_barrier(bs, a.limit)) return;
// the stop tests: every member, then the state bits are refreshed
#define FINISH_PHASE(BODY)                                       \
  for (int vb = gstart; vb < a.n; vb += gstride) {               \
    BODY;                                                        \
    gsync(t);                                                    \
  }                                                              \
  if (!grid_barrier(bs, a.limit)) return;                        \
  refresh();

  // before the loop: clear the corrections, the starting norms
  GROUP_PHASE(a.nref, a.t_ref, no_solve, batch_refine_body(I, a.t_ref[vb], 0, 0, 0, 0, t));
  GROUP_PHASE(a.nres, a.t_res, no_solve,
              (batch_residual_body<true, true>(I, a.t_res[vb], 0, 0, t, scratch)));
  FINISH_PHASE(batch_finish_body(I, vb, a.n, bs, a.m, 0, a.itermax_all, 0, 0, t, scratch));
  // the coarse loop: m sweeps, then the stop test
  for (unsigned int body = 0;; ++body) {
    const int par = body & 1;
    if (lead) atomicExch(&bs->go[par], 1u);
    int launches = 0;
    for (int done = 0; done < a.m; done += a.sweeps, ++launches) {
      const int cnt = a.m - done < a.sweeps ? a.m - done : a.sweeps;
      const int last = done + cnt >= a.m ? 1 : 0;
      TILE_PHASE(a.ntb, a.t_tb, idle,
                 (batch_tb_body<H, TX, TY, kPersistWarps, true>(
                     I, a.t_tb[vb], cnt, last, launches & 1, (last && a.fused) ? 1 : 0,
                     a.m > 1 ? 1 : 0, smem_raw)));
    }
    if (!a.fused) {
      GROUP_PHASE(a.nref, a.t_ref, idle,
                  batch_refine_body(I, a.t_ref[vb], 1, launches & 1, 0, a.m > 1 ? 1 : 0, t));
    }
    GROUP_PHASE(a.nres, a.t_res, idle,
                (batch_residual_body<true, true>(I, a.t_res[vb], 1, 0, t, scratch)));
    FINISH_PHASE(
        batch_finish_body(I, vb, a.n, bs, a.m, 1, a.itermax_all, 0, par, t, scratch));
    if (ld_acquire_u32(&bs->go[par]) == 0u) break;
  }
  if (a.m <= 1 || ld_acquire_u32(&bs->open_replay) == 0u) return;
  // members whose coarse loop stopped between checks finish sweep by sweep
  // (the restore re-opens the members that ran out of room)
  GROUP_PHASE(a.nref, a.t_ref, no_fine, batch_restore_body(I, a.t_ref[vb], a.m, t));
  refresh();
  GROUP_PHASE(a.nref, a.t_ref, no_fine, batch_refine_body(I, a.t_ref[vb], 0, 0, 1, 0, t));
  GROUP_PHASE(a.nres, a.t_res, no_fine,
              (batch_residual_body<true, true>(I, a.t_res[vb], 2, 1, t, scratch)));
  for (unsigned int body = 0;; ++body) {
    const int par = body & 1;
    if (lead) atomicExch(&bs->go[par], 1u);
    GROUP_PHASE(a.nref, a.t_ref, idle_fine, batch_color_body<true>(I, a.t_ref[vb], 0, 1, t));
    GROUP_PHASE(a.nref, a.t_ref, idle_fine, batch_color_body<true>(I, a.t_ref[vb], 1, 0, t));
    GROUP_PHASE(a.nref, a.t_ref, idle_fine, batch_refine_body(I, a.t_ref[vb], 1, 0, 1, 0, t));
    GROUP_PHASE(a.nres, a.t_res, idle_fine,
                (batch_residual_body<true, true>(I, a.t_res[vb], 1, 1, t, scratch)));
    FINISH_PHASE(
        batch_finish_body(I, vb, a.n, bs, 1, 1, a.itermax_all, 1, par, t, scratch));
    if (ld_acquire_u32(&bs->go[par]) == 0u) break;
  }
#undef TILE_PHASE
#undef GROUP_PHASE
#undef FINISH_PHASE
}

static const void *batch_persistent_fn(int sched) {
  switch (sched) {
    case 1: return (const void *)batch_persistent_kernel<4, 56, 120>;
    case 2: return (const void *)batch_persistent_kernel<8, 48, 112>;
    case 3: return (const void *)batch_persistent_kernel<16, 32, 96>;
    case 4: return (const void *)batch_persistent_kernel<8, 80, 112>;
    case 5: return (const void *)batch_persistent_kernel<8, 112, 112>;
    case 6: return (const void *)batch_persistent_kernel<16, 64, 96>;
    default: return nullptr;
  }
}

static const void *batch_tb_fn(int sched) {
  switch (sched) {
    case 1: return (const void *)batch_tb_kernel<4, 56, 120>;
    case 2: return (const void *)batch_tb_kernel<8, 48, 112>;
    case 3: return (const void *)batch_tb_kernel<16, 32, 96>;
    case 4: return (const void *)batch_tb_kernel<8, 80, 112>;
    case 5: return (const void *)batch_tb_kernel<8, 112, 112>;
    case 6: return (const void *)batch_tb_kernel<16, 64, 96>;
    default: return nullptr;
  }
}

void free_batch(BatchPlan *bp) {
  if (bp->graph) cudaGraphDestroy(bp->graph);
  if (bp->graph_pre) cudaGraphDestroy(bp->graph_pre);
  if (bp->graph_solve) cudaGraphDestroy(bp->graph_solve);
  if (bp->dev) cudaFree(bp->dev);
  bp->graph = nullptr;
  bp->graph_pre = nullptr;
  bp->graph_solve = nullptr;
  bp->dev = nullptr;
  bp->state = nullptr;
}

// Dynamic shared memory of the persistent solve: the sweep tiles', which
// also hold the groups' reduction scratch and residual tiles between tile
// phases.
static size_t persist_smem(const TbShape &t) {
  const size_t scratch = (2 * 512 + 2 * 32 + 2 * (RT_X + 2) * (RT_Y + 2)) * sizeof(double);
  const size_t tiles = tb_smem(t);
  return tiles > scratch ? tiles : scratch;
}

static_assert(offsetof(BatchState, overrun) == kBatchOverrunOffset, "overrun offset");
static_assert(offsetof(BatchState, timeout) == kBatchTimeoutOffset, "timeout offset");

cudaError_t build_batch(const std::vector<BatchMember> &mem, int sched, int m, BatchPlan *bp,
                        int persistent, unsigned long long wait_limit) {
  *bp = BatchPlan{};
  const int n = (int)mem.size();
  if (n < 1 || m < 1 || sched < 1 || sched >= kNumSchedules) return cudaErrorInvalidValue;
  cudaError_t e = tb_prepare();
  if (e != cudaSuccess) return e;
  for (int s2 = 1; s2 < kNumSchedules; ++s2) {
    e = cudaFuncSetAttribute(batch_tb_fn(s2), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tb_smem(kTbShapes[s2]));
    if (e != cudaSuccess) return e;
  }
  const TbShape &shape = kTbShapes[sched];
  std::vector<BInst> inst(n);
  std::vector<int2> t_res, t_ref, t_tb;
  unsigned int itermax_all = 0;
  for (int i = 0; i < n; ++i) {
    const DevFields &d = mem[i].d;
    const RunCfg &r = mem[i].r;
    BInst &b = inst[i];
    b.p = d.p;
    b.rhs = d.rhs;
    b.pw = d.pw;
    b.flags = d.flags;
    b.e32 = d.e32;
    b.e32b = d.e32b;
    b.r32 = d.r32;
    b.st = d.st;
    b.partials = d.partials;
    b.pcopy = d.pcopy;
    b.npc = d.n_pcopy;
    b.g = r.g;
    b.c = r.c;
    b.k32 = consts32_of(r.c);
    b.itermax = r.itermax;
    b.strict = r.strict_eps;
    int ty_int, nt_int;
    tiles_of(r.g, 1, &ty_int, &nt_int);
    b.solve = (nt_int > 0 && r.itermax > 0) ? 1 : 0;
    b.nb = residual_blocks(r.g);
    b.ty_int = ty_int;
    b.nt_int = nt_int;
    b.pgx = (r.g.ny / 2 + 1 + kRedBlock.x - 1) / kRedBlock.x;
    const int pgy = (r.g.nx + kRedBlock.y - 1) / kRedBlock.y;
    b.tb_tiles_y = (r.g.ny + shape.ty - 1) / shape.ty;
    const int tb_tiles_x = (r.g.nx + shape.tx - 1) / shape.tx;
    if (!b.solve) continue;
    if (r.itermax < (unsigned int)m) return cudaErrorInvalidValue;
    if (r.itermax > itermax_all) itermax_all = r.itermax;
    for (int k = 0; k < b.nb; ++k) t_res.push_back(make_int2(i, k));
    for (int k = 0; k < b.pgx * pgy; ++k) t_ref.push_back(make_int2(i, k));
    for (int k = 0; k < b.tb_tiles_y * tb_tiles_x; ++k) t_tb.push_back(make_int2(i, k));
  }
  // device tables: instances, the three block tables, the batch state
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_inst = 0, o_res = o_inst + al(sizeof(BInst) * n);
  const size_t o_ref = o_res + al(sizeof(int2) * (t_res.size() + 1));
  const size_t o_tb = o_ref + al(sizeof(int2) * (t_ref.size() + 1));
  const size_t o_bs = o_tb + al(sizeof(int2) * (t_tb.size() + 1));
  const size_t total = o_bs + al(sizeof(BatchState));
  char *dev = nullptr;
  if ((e = cudaMalloc(&dev, total)) != cudaSuccess) return e;
  bp->dev = dev;
  const BInst *d_inst = (const BInst *)(dev + o_inst);
  const int2 *d_res = (const int2 *)(dev + o_res), *d_ref = (const int2 *)(dev + o_ref);
  const int2 *d_tb = (const int2 *)(dev + o_tb);
  BatchState *d_bs = (BatchState *)(dev + o_bs);
  bp->state = d_bs;
  e = cudaMemset(dev, 0, total);
  if (e == cudaSuccess) e = cudaMemcpy(dev + o_inst, inst.data(), sizeof(BInst) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !t_res.empty())
    e = cudaMemcpy(dev + o_res, t_res.data(), sizeof(int2) * t_res.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !t_ref.empty())
    e = cudaMemcpy(dev + o_ref, t_ref.data(), sizeof(int2) * t_ref.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !t_tb.empty())
    e = cudaMemcpy(dev + o_tb, t_tb.data(), sizeof(int2) * t_tb.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_batch(bp);
    return e;
  }

  // the persistent solve: as many CTAs as can be resident at once
  int persist_grid = 0;
  if (persistent) {
    const void *fn = batch_persistent_fn(sched);
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)persist_smem(shape));
    int per_sm = 0;
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * kPersistWarps,
                                                        persist_smem(shape));
    if (e == cudaSuccess && per_sm < 1) e = cudaErrorInvalidConfiguration;
    if (e != cudaSuccess) {
      free_batch(bp);
      return e;
    }
    persist_grid = per_sm * num_sms();
    bp->persist_grid = persist_grid;
  }

  // part 0: the whole step; 1: the members' first halves (boundary pass,
  // F/G, RHS); 2: the pressure solves and the second halves
  auto assemble = [&](int part, cudaGraph_t *out) -> cudaError_t {
  GraphBuilder b;
  cudaError_t e2 = cudaGraphCreate(&b.graph, 0);
  if (e2 != cudaSuccess) return e2;
  b.store.reserve(64);
  // per-instance first halves, in parallel
  std::vector<cudaGraphNode_t> pre(n, nullptr);
  for (int i = 0; i < n && b.err == cudaSuccess && part != 2; ++i) {
    cudaGraph_t child = nullptr;
    b.err = build_step_graph(mem[i].d, mem[i].r, &child, 1);
    if (b.err == cudaSuccess) {
      b.err = cudaGraphAddChildGraphNode(&pre[i], b.graph, nullptr, 0, child);
      cudaGraphDestroy(child);
    }
  }
  if (part == 1) {
    if (b.err != cudaSuccess) {
      cudaGraphDestroy(b.graph);
      return b.err;
    }
    *out = b.graph;
    return cudaSuccess;
  }
  cudaGraphNode_t nd = nullptr;
  if (b.err == cudaSuccess)
    b.err = cudaGraphAddEmptyNode(&nd, b.graph, part == 2 ? nullptr : pre.data(),
                                  part == 2 ? 0 : (size_t)n);
  const int nres = (int)t_res.size(), nref = (int)t_ref.size();
  const int ntb = (int)t_tb.size();
  cudaGraphConditionalHandle h{};
  if (b.err == cudaSuccess && !persistent)
    b.err = cudaGraphConditionalHandleCreate(&h, b.graph, 1, cudaGraphCondAssignDefault);
  if (nres > 0 && persistent) {
    // the whole solve as one cooperative kernel: its barrier state zeroed
    // first, then one CTA per resident slot walking the tables
    cudaMemsetParams ms{};
    ms.dst = (char *)d_bs;
    ms.value = 0;
    ms.elementSize = 4;
    ms.width = offsetof(BatchState, overrun) / 4;
    ms.height = 1;
    cudaGraphNode_t mnode = nullptr;
    if (b.err == cudaSuccess)
      b.err = cudaGraphAddMemsetNode(&mnode, b.graph, nd ? &nd : nullptr, nd ? 1 : 0, &ms);
    PersistArgs pa{};
    pa.inst = d_inst;
    pa.t_res = d_res;
    pa.t_ref = d_ref;
    pa.t_tb = d_tb;
    pa.nres = nres;
    pa.nref = nref;
    pa.ntb = ntb;
    pa.n = n;
    pa.bs = d_bs;
    pa.m = m;
    pa.sweeps = shape.sweeps;
    pa.fused = ((m + shape.sweeps - 1) / shape.sweeps) % 2 == 0 ? 1 : 0;
    pa.itermax_all = itermax_all;
    pa.limit = wait_limit;
    nd = b.kernel_smem(b.graph, mnode, batch_persistent_fn(sched), dim3(persist_grid),
                       dim3(32, kPersistWarps), persist_smem(shape), pa);
    if (b.err == cudaSuccess) {
      cudaLaunchAttributeValue v{};
      v.cooperative = 1;
      b.err = cudaGraphKernelNodeSetAttribute(nd, cudaLaunchAttributeCooperative, &v);
    }
  } else if (nres > 0) {
    cudaGraphConditionalHandle h_rep{};
    if (b.err == cudaSuccess)
      b.err = cudaGraphConditionalHandleCreate(&h_rep, b.graph, 0, cudaGraphCondAssignDefault);
    nd = b.kernel(b.graph, nd, (const void *)batch_refine_kernel, dim3(nref), kRedBlock, d_inst,
                  d_ref, 0, 0, 0, 0);
    nd = b.kernel(b.graph, nd, (const void *)batch_residual_kernel, dim3(nres), kRedBlock,
                  d_inst, d_res, 0, 0);
    nd = b.kernel(b.graph, nd, (const void *)batch_finish_kernel, dim3(n), kRedBlock, d_inst, n,
                  d_bs, h, m, 0, itermax_all, 0, h_rep);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (b.err == cudaSuccess) b.err = cudaGraphAddNode(&wnode, b.graph, &nd, nullptr, 1, &cp);
    if (b.err == cudaSuccess) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      cudaGraphNode_t bn = nullptr;
      int launches = 0;
      // an even number of launches ends in the start buffer: the last one
      // refines (as sweep_plan for one simulation)
      const bool fused = ((m + shape.sweeps - 1) / shape.sweeps) % 2 == 0;
      for (int done = 0; done < m; done += shape.sweeps, ++launches) {
        const int cnt = m - done < shape.sweeps ? m - done : shape.sweeps;
        const int last = done + cnt >= m ? 1 : 0;
        bn = b.kernel_smem(body, bn, batch_tb_fn(sched), dim3(ntb), dim3(512), tb_smem(shape),
                           d_inst, d_tb, cnt, last, launches & 1, (last && fused) ? 1 : 0,
                           m > 1 ? 1 : 0);
      }
      if (!fused)
        bn = b.kernel(body, bn, (const void *)batch_refine_kernel, dim3(nref), kRedBlock,
                      d_inst, d_ref, 1, launches & 1, 0, m > 1 ? 1 : 0);
      bn = b.kernel(body, bn, (const void *)batch_residual_kernel, dim3(nres), kRedBlock,
                    d_inst, d_res, 1, 0);
      bn = b.kernel(body, bn, (const void *)batch_finish_kernel, dim3(n), kRedBlock, d_inst, n,
                    d_bs, h, m, 1, itermax_all, 0, h_rep);
    }
    nd = wnode;
    if (m > 1) {
      // members whose coarse loop stopped between checks finish sweep by sweep
      cudaGraphNodeParams ip = {};
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = h_rep;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      cudaGraphNode_t inode = nullptr;
      if (b.err == cudaSuccess) b.err = cudaGraphAddNode(&inode, b.graph, &nd, nullptr, 1, &ip);
      if (b.err == cudaSuccess) {
        cudaGraph_t ib = ip.conditional.phGraph_out[0];
        cudaGraphNode_t fn = nullptr;
        fn = b.kernel(ib, fn, (const void *)batch_restore_kernel, dim3(nref), kRedBlock, d_inst,
                      d_ref, m);
        fn = b.kernel(ib, fn, (const void *)batch_refine_kernel, dim3(nref), kRedBlock, d_inst,
                      d_ref, 0, 0, 1, 0);
        fn = b.kernel(ib, fn, (const void *)batch_residual_kernel, dim3(nres), kRedBlock,
                      d_inst, d_res, 2, 1);
        cudaGraphConditionalHandle h_fine{};
        if (b.err == cudaSuccess)
          b.err = cudaGraphConditionalHandleCreate(&h_fine, ib, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams fp = {};
        fp.type = cudaGraphNodeTypeConditional;
        fp.conditional.handle = h_fine;
        fp.conditional.type = cudaGraphCondTypeWhile;
        fp.conditional.size = 1;
        cudaGraphNode_t fw = nullptr;
        if (b.err == cudaSuccess) b.err = cudaGraphAddNode(&fw, ib, &fn, nullptr, 1, &fp);
        if (b.err == cudaSuccess) {
          cudaGraph_t fb = fp.conditional.phGraph_out[0];
          cudaGraphNode_t x = nullptr;
          for (int color = 0; color < 2; ++color)
            x = b.kernel(fb, x, (const void *)batch_color_kernel, dim3(nref), kRedBlock, d_inst,
                         d_ref, color, color == 0 ? 1 : 0);
          x = b.kernel(fb, x, (const void *)batch_refine_kernel, dim3(nref), kRedBlock, d_inst,
                       d_ref, 1, 0, 1, 0);
          x = b.kernel(fb, x, (const void *)batch_residual_kernel, dim3(nres), kRedBlock,
                       d_inst, d_res, 1, 1);
          x = b.kernel(fb, x, (const void *)batch_finish_kernel, dim3(n), kRedBlock, d_inst, n,
                       d_bs, h_fine, 1, 1, itermax_all, 1, h_fine);
        }
      }
      nd = inode;
    }
  }
  // per-instance second halves, in parallel
  for (int i = 0; i < n && b.err == cudaSuccess; ++i) {
    cudaGraph_t child = nullptr;
    b.err = build_step_graph(mem[i].d, mem[i].r, &child, 3);
    if (b.err == cudaSuccess) {
      cudaGraphNode_t post = nullptr;
      b.err = cudaGraphAddChildGraphNode(&post, b.graph, nd ? &nd : nullptr, nd ? 1 : 0, child);
      cudaGraphDestroy(child);
    }
  }
  if (b.err != cudaSuccess) {
    cudaGraphDestroy(b.graph);
    return b.err;
  }
  *out = b.graph;
  return cudaSuccess;
  };
  e = assemble(0, &bp->graph);
  if (e == cudaSuccess) e = assemble(1, &bp->graph_pre);
  if (e == cudaSuccess) e = assemble(2, &bp->graph_solve);
  if (e != cudaSuccess) free_batch(bp);
  return e;
}

cudaError_t batch_sweeps(const std::vector<BatchMember> &mem, int sched, int m,
                         cudaStream_t s) {
  // standalone timing helper of the autotuner: m sweeps of every instance
  // with schedule `sched`, one launch per instance per blocked launch
  cudaError_t e = tb_prepare();
  for (const BatchMember &bm : mem) {
    if (e != cudaSuccess) break;
    RunCfg r = bm.r;
    r.sweep_schedule = sched;
    e = launch_mixed_sweeps(bm.d, r, s, m);
  }
  return e;
}
}  // namespace strm
