// Internal device-side definitions shared by the stroemung GB300 kernels.
//
// Data layout in HBM (one arena per simulation):
//   every field is [nx][pitch] with y the contiguous axis, row x at x*pitch,
//   pitch = ny rounded up to 16 elements (128 B for FP64), rows 128-B aligned.
//   flags: one byte per cell, same [nx][pitch] indexing:
//     bits 0-2  cell kind   (0 fluid, 1 no-slip, 2 outflow, 3 inflow, 4 moving wall)
//     bits 3-6  edge code   (0 none, 1 N, 2 NE, 3 E, 4 SE, 5 S, 6 SW, 7 W, 8 NW)
//   The edge code is the reference's EdgeType (src/grid/mod.rs:19-49), in its
//   declaration order; "north" is y-1 (src/grid/mod.rs:168-170).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

namespace strm {

enum : uint8_t { K_FLUID = 0, K_NO_SLIP = 1, K_OUTFLOW = 2, K_INFLOW = 3, K_MOVING = 4 };
enum : uint8_t {
  E_NONE = 0, E_N = 1, E_NE = 2, E_E = 3, E_SE = 4, E_S = 5, E_SW = 6, E_W = 7, E_NW = 8
};

__host__ __device__ __forceinline__ uint8_t kind_of(uint8_t f) { return f & 7u; }
__host__ __device__ __forceinline__ uint8_t edge_of(uint8_t f) { return (f >> 3) & 15u; }
__host__ __device__ __forceinline__ bool is_bnd(uint8_t f) { return (f & 7u) != 0; }

// Geometry of one simulation's device fields.
struct Geom {
  int nx, ny;
  int pitch;  // elements per row
};

// Constants of the stencils, with the exact reciprocals the correctly
// rounded division needs (see xdiv).
struct Consts {
  double dx, dy, gamma, re;
  double dx2, dy2;      // dx*dx, dy*dy   (reference: delx.powi(2))
  double four_dx, four_dy;
  double r_dx, r_dy, r_dx2, r_dy2, r_four_dx, r_four_dy, r_re;
  // pressure solve
  double one_minus_w, middle;  // 1-omega, omega/((2/dx2)+(2/dy2))
  double two_r_sum;            // 2 (1/dx^2 + 1/dy^2) (fast residual)
  double eps2;
};

// Per-simulation device state.  Written by kernels, read by the host after
// each step (one small D2H copy).
struct StepState {
  double dt;           // delt of the current step
  double time;
  double ns0;          // initial_norm_squared
  double ns;           // norm_squared of the last pressure iteration
  double fluid_cells;
  double umax, vmax;   // max |u|, |v| over every cell (adaptive dt input)
  double aux;          // result of a standalone norm
  double ns_start;     // norm the current pressure solve started from
  unsigned long long iterations;
  unsigned int sor_iters;
  unsigned int converged;   // pressure solve met its stop rule
  unsigned int exhausted;   // pressure solve ran max_iterations
  unsigned int nonfinite;   // last norm was NaN/Inf
  unsigned int body_count;  // launches of the pressure-loop body this step
  unsigned int overrun;     // the loop passed its bound without the normal stop
  unsigned int replay;      // mixed solve: 1 redo the last outer iteration sweep by
                            // sweep, 2 finish the remaining sweeps one by one
  // ordered-bit encodings of the ranges (see ord_enc); speeds are squared
  unsigned long long p_min, p_max, s2_min, s2_max;
  unsigned long long umax_bits, vmax_bits;
  unsigned int counter;     // last-block-done ticket for grid reductions
  unsigned int log_pos;     // next slot of the per-step log
  unsigned int log_cap;
  // residual history of the current step's solve: (sweeps, norm) pairs
  double *hist;
  unsigned int hist_n, hist_cap;
  // FAST red-black solve, written by the red pass for the next black pass:
  // 1 / fluid_cells (from the solve's first red pass) and the iteration
  // whose norm the black pass decides (0: none)
  double pass_inv_cells;
  unsigned int pass_iter;
};

// Appends (sweeps, norm) to the solve's residual history (one thread).
__device__ __forceinline__ void hist_push(StepState *st, unsigned int sweeps, double ns) {
  const unsigned int n = st->hist_n;
  if (st->hist && n < st->hist_cap) {
    st->hist[2 * (size_t)n] = (double)sweeps;
    st->hist[2 * (size_t)n + 1] = ns;
    st->hist_n = n + 1;
  }
}

// One record per completed step.
struct StepLog {
  double ns;
  double dt;
  unsigned int sor_iters;
  unsigned int converged;
};

// Correctly rounded a / b for a divisor b known in advance, from its
// correctly rounded reciprocal rb = RN(1/b) (computed with an IEEE division).
// q0 = RN(a*rb) lies within 1.5 ulp of a/b; one remainder correction
// (Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. R&D 34(1), 1990) makes it faithful; a second one, whose
// remainder is then exact, gives RN(a/b).  A zero quotient takes the sign of
// a^b.  Valid for finite a and b with a/b in the normal range; a non-finite
// numerator yields NaN rather than Inf.  Five FP64 pipe operations instead of
// a full division, which matters on a part with a narrow FP64 pipe.
__host__ __device__ __forceinline__ double xdiv(double a, double b, double rb) {
  double q0 = a * rb;
  double r0 = fma(-b, q0, a);
  double q1 = fma(r0, rb, q0);
  double r1 = fma(-b, q1, a);
  double q2 = fma(r1, rb, q1);
#ifdef __CUDA_ARCH__
  long long qb = __double_as_longlong(q2);
  if ((qb << 1) == 0)
    qb = (__double_as_longlong(a) ^ __double_as_longlong(b)) & (long long)0x8000000000000000ULL;
  return __longlong_as_double(qb);
#else
  if (q2 == 0.0) return (signbit(a) != signbit(b)) ? -0.0 : 0.0;
  return q2;
#endif
}

// Conversions between FP32 and FP64 in integer arithmetic.  On this part
// the conversion instructions run on the narrow FP64 pipe; the mixed-precision
// kernels convert every cell, so they use these instead (bit manipulation on
// the integer pipe).  Both flush magnitudes below 2^-126 (the FP32 normal
// range) to zero of the same sign; infinities and NaNs map to themselves.
__host__ __device__ __forceinline__ uint64_t f64_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}
__host__ __device__ __forceinline__ double f64_of(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  memcpy(&b, &x, 4);
  return b;
#endif
}
__host__ __device__ __forceinline__ float f32_of(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  memcpy(&x, &b, 4);
  return x;
#endif
}

// float -> double, exact (FP32 denormals flushed).
__host__ __device__ __forceinline__ double widen(float f) {
  const uint32_t u = f32_bits(f);
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  if (e == 0) return f64_of(sign);
  if (e == 0xFF) return f64_of(sign | 0x7FF0000000000000ull | ((uint64_t)m << 29));
  return f64_of(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29));
}

// double -> float, rounded to nearest (ties to even).
__host__ __device__ __forceinline__ float narrow(double x) {
  const uint64_t b = f64_bits(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int E = (int)((b >> 52) & 0x7FFu);
  const uint64_t M = b & 0xFFFFFFFFFFFFFull;
  if (E == 0x7FF) return f32_of(sign | 0x7F800000u | (M ? 0x400000u : 0u));
  const int e = E - 896;  // FP32 biased exponent
  if (e >= 255) return f32_of(sign | 0x7F800000u);
  if (e <= 0) return f32_of(sign);
  const uint32_t m = (uint32_t)(M >> 29);
  const uint32_t rem = (uint32_t)(M & 0x1FFFFFFFu), half = 0x10000000u;
  uint32_t r = ((uint32_t)e << 23) | m;
  if (rem > half || (rem == half && (m & 1u))) ++r;  // a carry moves into the exponent
  return f32_of(sign | r);
}

// Order-preserving map of a double onto uint64 (for atomicMin/atomicMax).
__host__ __device__ __forceinline__ unsigned long long ord_enc(double d) {
#ifdef __CUDA_ARCH__
  unsigned long long b = (unsigned long long)__double_as_longlong(d);
#else
  unsigned long long b;
  memcpy(&b, &d, 8);
#endif
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__host__ __device__ __forceinline__ double ord_dec(unsigned long long e) {
  unsigned long long b = (e >> 63) ? (e & 0x7fffffffffffffffULL) : ~e;
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}

// One entry of the compiled boundary-condition program: on a given step the
// target (field, cell) receives   c            (op 0)
//                                 +src         (op 1)
//                                 -src         (op 2)
//                                 c - src      (op 3)
// where src is the value the same field held at `src` before the step's
// boundary pass.  Fields: 0 u, 1 v, 2 restore-u, 3 restore-v (src reads u for
// fields 0/2 and v for fields 1/3).
struct BcEntry {
  long long target;  // (field << 56) | offset
  long long src;     // offset
  double c;
  int op;
  int pad_;
};

// A boundary cell whose pressure is copied from its fluid neighbours before
// each pressure iteration (src/grid/mod.rs:343-412).
struct PCopy {
  long long off;
  int edge;
  int pad_;
};

}  // namespace strm
