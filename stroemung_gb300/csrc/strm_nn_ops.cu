// Memory-bound kernels of the learned warm start: input assembly from the
// solver's fields, pooling / upsampling and their adjoints, ReLU masks, bias
// gradients, the 1x1 output head, the relative-residual loss and its
// gradient, the weight re-layout for the data gradient, and Adam.
//
// Activation tensors are BF16 NHWC with an explicit pixel stride (channel
// slices of one buffer form a concatenation); per-sample planes (RHS, fluid
// mask, pressures, flags) are FP32 / u8 [batch][h][w] over the interior cells
// of each sample (ring excluded): cell (x, y) of the solver grid is pixel
// (row x-1, column y-1), rows along the slow axis as in the fields.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/stroemung_nn.h"
#include "strm_internal.cuh"

namespace strm_nn {

using strm::edge_of;
using strm::is_bnd;

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

#define GRID_STRIDE(i, n) \
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
       i += (long long)gridDim.x * blockDim.x)

// 2x2 average pooling: out (B, H/2, W/2) from in (B, H, W), C channels.
__global__ void avgpool_fwd(const __nv_bfloat16 *in, int cs_in, __nv_bfloat16 *out, int cs_out,
                            int batch, int h, int w, int c) {
  const int ho = h / 2, wo = w / 2;
  const long long n = (long long)batch * ho * wo * c;
  GRID_STRIDE(i, n) {
    const int ch = (int)(i % c);
    const long long q = i / c;
    const int xo = (int)(q % wo);
    const long long t = q / wo;
    const int yo = (int)(t % ho);
    const long long b = t / ho;
    const long long q00 = (b * h + 2 * yo) * w + 2 * xo;
    const float s = bf(in[q00 * cs_in + ch]) + bf(in[(q00 + 1) * cs_in + ch]) +
                    bf(in[(q00 + w) * cs_in + ch]) + bf(in[(q00 + w + 1) * cs_in + ch]);
    out[q * cs_out + ch] = __float2bfloat16_rn(0.25f * s);
  }
}

// Adjoint: each input pixel receives a quarter of its pooled gradient,
// added to (accumulate=1) or replacing its gradient.
__global__ void avgpool_bwd(const __nv_bfloat16 *gout, int cs_out, __nv_bfloat16 *gin, int cs_in,
                            int batch, int h, int w, int c, int accumulate) {
  const long long n = (long long)batch * h * w * c;
  GRID_STRIDE(i, n) {
    const int ch = (int)(i % c);
    const long long q = i / c;
    const int xx = (int)(q % w);
    const long long t = q / w;
    const int yy = (int)(t % h);
    const long long b = t / h;
    const long long qo = (b * (h / 2) + yy / 2) * (w / 2) + xx / 2;
    float g = 0.25f * bf(gout[qo * cs_out + ch]);
    if (accumulate) g += bf(gin[q * cs_in + ch]);
    gin[q * cs_in + ch] = __float2bfloat16_rn(g);
  }
}

// Nearest 2x upsampling into a channel slice of the concatenation buffer.
__global__ void upsample_fwd(const __nv_bfloat16 *in, int cs_in, __nv_bfloat16 *out, int cs_out,
                             int batch, int h, int w, int c) {
  const long long n = (long long)batch * h * w * c;  // output pixels (h, w = output size)
  GRID_STRIDE(i, n) {
    const int ch = (int)(i % c);
    const long long q = i / c;
    const int xx = (int)(q % w);
    const long long t = q / w;
    const int yy = (int)(t % h);
    const long long b = t / h;
    const long long qi = (b * (h / 2) + yy / 2) * (w / 2) + xx / 2;
    out[q * cs_out + ch] = in[qi * cs_in + ch];
  }
}

// Adjoint: sum of the four output gradients.
__global__ void upsample_bwd(const __nv_bfloat16 *gout, int cs_out, __nv_bfloat16 *gin, int cs_in,
                             int batch, int h, int w, int c) {
  const int hi = h / 2, wi = w / 2;
  const long long n = (long long)batch * hi * wi * c;
  GRID_STRIDE(i, n) {
    const int ch = (int)(i % c);
    const long long q = i / c;
    const int xi = (int)(q % wi);
    const long long t = q / wi;
    const int yi = (int)(t % hi);
    const long long b = t / hi;
    const long long q00 = (b * h + 2 * yi) * w + 2 * xi;
    const float s = bf(gout[q00 * cs_out + ch]) + bf(gout[(q00 + 1) * cs_out + ch]) +
                    bf(gout[(q00 + w) * cs_out + ch]) + bf(gout[(q00 + w + 1) * cs_out + ch]);
    gin[q * cs_in + ch] = __float2bfloat16_rn(s);
  }
}

// ---- 8-channel (16-byte) versions of the kernels above: same arithmetic per
// element; used when channel counts, strides and addresses allow ----
union V8 {
  uint4 u;
  __nv_bfloat16 h[8];
};

__device__ __forceinline__ V8 ld8(const __nv_bfloat16 *p) {
  V8 v;
  v.u = *reinterpret_cast<const uint4 *>(p);
  return v;
}
__device__ __forceinline__ void st8(__nv_bfloat16 *p, const V8 &v) {
  *reinterpret_cast<uint4 *>(p) = v.u;
}

__global__ void avgpool_rows8(const __nv_bfloat16 *__restrict__ in, int cs_in,
                              __nv_bfloat16 *__restrict__ out, int cs_out, int rows, int h, int w,
                              int c8) {
  const int wo = w / 2, ho = h / 2, n = wo * c8;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int xo = k / c8, ch = 8 * (k - xo * c8);
  for (int r = blockIdx.y; r < rows; r += gridDim.y) {
    const int b = r / ho, yo = r - b * ho;
    const long long q00 = ((long long)b * h + 2 * yo) * w + 2 * xo;
    const V8 a = ld8(in + q00 * cs_in + ch), bb = ld8(in + (q00 + 1) * cs_in + ch);
    const V8 cc = ld8(in + (q00 + w) * cs_in + ch), d = ld8(in + (q00 + w + 1) * cs_in + ch);
    V8 o;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      o.h[j] = __float2bfloat16_rn(0.25f * (bf(a.h[j]) + bf(bb.h[j]) + bf(cc.h[j]) + bf(d.h[j])));
    st8(out + ((long long)r * wo + xo) * cs_out + ch, o);
  }
}

__global__ void upsample_rows8(const __nv_bfloat16 *__restrict__ in, int cs_in,
                               __nv_bfloat16 *__restrict__ out, int cs_out, int rows, int h, int w,
                               int c8) {
  const int wi = w / 2, hi = h / 2, n = wi * c8;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int xi = k / c8, ch = 8 * (k - xi * c8);
  for (int r = blockIdx.y; r < rows; r += gridDim.y) {
    const int b = r / hi, yi = r - b * hi;
    const V8 v = ld8(in + ((long long)r * wi + xi) * cs_in + ch);
    const long long q00 = ((long long)b * h + 2 * yi) * w + 2 * xi;
    st8(out + q00 * cs_out + ch, v);
    st8(out + (q00 + 1) * cs_out + ch, v);
    st8(out + (q00 + w) * cs_out + ch, v);
    st8(out + (q00 + w + 1) * cs_out + ch, v);
  }
}

__global__ void avgpool_bwd8(const __nv_bfloat16 *gout, int cs_out, __nv_bfloat16 *gin,
                             int cs_in, int batch, int h, int w, int c, int accumulate) {
  const int c8 = c / 8;
  const long long n = (long long)batch * h * w * c8;
  GRID_STRIDE(i, n) {
    const int ch = 8 * (int)(i % c8);
    const long long q = i / c8;
    const int xx = (int)(q % w);
    const long long t = q / w;
    const int yy = (int)(t % h);
    const long long b = t / h;
    const long long qo = (b * (h / 2) + yy / 2) * (w / 2) + xx / 2;
    const V8 g = ld8(gout + qo * cs_out + ch);
    V8 prev;
    if (accumulate) prev = ld8(gin + q * cs_in + ch);
    V8 o;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float v = 0.25f * bf(g.h[k]);
      if (accumulate) v += bf(prev.h[k]);
      o.h[k] = __float2bfloat16_rn(v);
    }
    st8(gin + q * cs_in + ch, o);
  }
}

__global__ void upsample_bwd8(const __nv_bfloat16 *gout, int cs_out, __nv_bfloat16 *gin,
                              int cs_in, int batch, int h, int w, int c) {
  const int hi = h / 2, wi = w / 2, c8 = c / 8;
  const long long n = (long long)batch * hi * wi * c8;
  GRID_STRIDE(i, n) {
    const int ch = 8 * (int)(i % c8);
    const long long q = i / c8;
    const int xi = (int)(q % wi);
    const long long t = q / wi;
    const int yi = (int)(t % hi);
    const long long b = t / hi;
    const long long q00 = (b * h + 2 * yi) * w + 2 * xi;
    const V8 a = ld8(gout + q00 * cs_out + ch), bb = ld8(gout + (q00 + 1) * cs_out + ch);
    const V8 cc = ld8(gout + (q00 + w) * cs_out + ch), d = ld8(gout + (q00 + w + 1) * cs_out + ch);
    V8 o;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      o.h[k] = __float2bfloat16_rn(bf(a.h[k]) + bf(bb.h[k]) + bf(cc.h[k]) + bf(d.h[k]));
    st8(gin + q * cs_in + ch, o);
  }
}

__global__ void relu_mask8(const __nv_bfloat16 *g, int cs_g, const __nv_bfloat16 *y, int cs_y,
                           __nv_bfloat16 *out, int cs_out, long long npix, int c) {
  const int c8 = c / 8;
  GRID_STRIDE(i, npix * c8) {
    const int ch = 8 * (int)(i % c8);
    const long long q = i / c8;
    const V8 gv = ld8(g + q * cs_g + ch), yv = ld8(y + q * cs_y + ch);
    V8 o;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      o.h[k] = __float2bfloat16_rn(bf(yv.h[k]) > 0.0f ? bf(gv.h[k]) : 0.0f);
    st8(out + q * cs_out + ch, o);
  }
}

// g <- g * (y > 0) (ReLU adjoint), written to out (may alias g).
__global__ void relu_mask(const __nv_bfloat16 *g, int cs_g, const __nv_bfloat16 *y, int cs_y,
                          __nv_bfloat16 *out, int cs_out, long long npix, int c) {
  GRID_STRIDE(i, npix * c) {
    const int ch = (int)(i % c);
    const long long q = i / c;
    const float v = bf(y[q * cs_y + ch]) > 0.0f ? bf(g[q * cs_g + ch]) : 0.0f;
    out[q * cs_out + ch] = __float2bfloat16_rn(v);
  }
}

// db[c] += sum_q g[q][c] * (y[q][c] > 0 when y given); one block column per
// channel group, partial sums in shared memory then one atomic per channel.
__global__ void bias_grad(const __nv_bfloat16 *g, int cs_g, const __nv_bfloat16 *y, int cs_y,
                          float *db, long long npix, int c) {
  extern __shared__ float acc[];
  for (int i = threadIdx.x; i < c; i += blockDim.x) acc[i] = 0.0f;
  __syncthreads();
  const long long n = npix * c;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % c);
    const long long q = i / c;
    float v = bf(g[q * cs_g + ch]);
    if (y && !(bf(y[q * cs_y + ch]) > 0.0f)) v = 0.0f;
    atomicAdd(&acc[ch], v);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < c; i += blockDim.x) atomicAdd(&db[i], acc[i]);
}

// Data-gradient weights: wt[ci][t][co] = w[co][8 - t][ci] (K padded).
__global__ void flip_weights(const __nv_bfloat16 *w, int cout, int cin_p, int kp,
                             __nv_bfloat16 *wt, int cout_p, int kp_t) {
  // wt has cin_p rows (output channels of the data gradient) and K = 9*cout_p
  const long long n = (long long)cin_p * kp_t;
  GRID_STRIDE(i, n) {
    const int ci = (int)(i / kp_t);
    const int k = (int)(i % kp_t);
    const int t = k / cout_p, co = k % cout_p;
    __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
    if (t < 9 && co < cout) v = w[(size_t)co * kp + (8 - t) * cin_p + ci];
    wt[i] = v;
  }
}

// 1x1 head, FP32: out[q] = sum_c wh[c] * act[q][c] + bh (bh a device scalar).
__global__ void head_fwd(const __nv_bfloat16 *act, int cs, int c, const float *wh,
                         const float *bh, float *out, long long npix) {
  const bool vec = (c % 8 == 0) && (cs % 8 == 0) &&
                   ((reinterpret_cast<uintptr_t>(act) & 15u) == 0);
  GRID_STRIDE(q, npix) {
    float s = *bh;
    if (vec) {
      for (int ch = 0; ch < c; ch += 8) {
        const V8 a = ld8(act + q * cs + ch);
#pragma unroll
        for (int k = 0; k < 8; ++k) s = fmaf(wh[ch + k], bf(a.h[k]), s);
      }
    } else {
      for (int ch = 0; ch < c; ++ch) s = fmaf(wh[ch], bf(act[q * cs + ch]), s);
    }
    out[q] = s;
  }
}

// Head adjoint: gact[q][c] = gout[q] * wh[c]; dwh[c] += sum_q gout[q] act[q][c];
// dbh += sum_q gout[q].  dwh/dbh partial sums per block in shared memory.
__global__ void head_bwd(const __nv_bfloat16 *act, int cs, int c, const float *wh,
                         const float *gout, __nv_bfloat16 *gact, int cs_g, float *dwh, float *dbh,
                         long long npix) {
  extern __shared__ float acc[];  // c + 1
  for (int i = threadIdx.x; i <= c; i += blockDim.x) acc[i] = 0.0f;
  __syncthreads();
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < npix;
       q += (long long)gridDim.x * blockDim.x) {
    const float g = gout[q];
    for (int ch = 0; ch < c; ++ch) {
      gact[q * cs_g + ch] = __float2bfloat16_rn(g * wh[ch]);
      atomicAdd(&acc[ch], g * bf(act[q * cs + ch]));
    }
    atomicAdd(&acc[c], g);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < c; i += blockDim.x) atomicAdd(&dwh[i], acc[i]);
  if (threadIdx.x == 0) atomicAdd(dbh, acc[c]);
}

// Per-sample max |rhs| over fluid cells (the input scale).
__global__ void sample_absmax(const float *rhs, const uint8_t *flags, float *smax, int plane) {
  const int b = blockIdx.y;
  float m = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x)
    if (!is_bnd(flags[(size_t)b * plane + i])) m = fmaxf(m, fabsf(rhs[(size_t)b * plane + i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int *>(smax + b), __float_as_int(m));
}

// Network input, 8 channels, on the interior cells of each sample:
// rhs/s, fluid mask, (p_prev - mean)/(s dx^2), 0...  Full planes are
// [batch][nx][ny] (ring included); the input is [batch][nx-2][ny-2][8].
__global__ void assemble_input(const float *rhs, const uint8_t *flags, const float *pprev,
                               const float *smax, const float *pmean, float dx2,
                               __nv_bfloat16 *xin, int batch, int nx, int ny) {
  const int h = nx - 2, w = ny - 2;
  const long long n = (long long)batch * h * w;
  GRID_STRIDE(i, n) {
    const int b = (int)(i / ((long long)h * w));
    const int rem = (int)(i - (long long)b * h * w);
    const int x = rem / w + 1, y = rem % w + 1;
    const long long f = (long long)b * nx * ny + (long long)x * ny + y;
    const float s = smax[b] > 0.0f ? smax[b] : 1.0f;
    const bool fluid = !is_bnd(flags[f]);
    __align__(16) __nv_bfloat16 v[8];
    v[0] = __float2bfloat16_rn(fluid ? rhs[f] / s : 0.0f);
    v[1] = __float2bfloat16_rn(fluid ? 1.0f : 0.0f);
    v[2] = __float2bfloat16_rn(fluid ? (pprev[f] - pmean[b]) / (s * dx2) : 0.0f);
#pragma unroll
    for (int k = 3; k < 8; ++k) v[k] = __float2bfloat16_rn(0.0f);
    *reinterpret_cast<uint4 *>(xin + i * 8) = *reinterpret_cast<const uint4 *>(v);
  }
}

// Per-sample mean of p_prev over fluid cells (sum and count by atomics).
// Sum and count of p over each sample's non-boundary cells in a fixed order,
// so the network input (and with it the prediction) is the same bits run
// after run: kMeanBlocks blocks per sample reduce strided shares with a fixed
// shuffle tree into partials (sum, count) [batch][kMeanBlocks][2], then one
// warp per sample adds those in order.
constexpr int kMeanBlocks = 64;

__device__ __forceinline__ void block_sum2(float &s, float &c) {
  __shared__ float ss[32], sc[32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    ss[w] = s;
    sc[w] = c;
  }
  __syncthreads();
  if (w == 0) {
    s = lane < nw ? ss[lane] : 0.0f;
    c = lane < nw ? sc[lane] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
  }
}

__global__ void __launch_bounds__(256)
    sample_mean_partial(const float *p, const uint8_t *flags, float *part, int plane) {
  const int b = blockIdx.y;
  float s = 0.0f, c = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x)
    if (!is_bnd(flags[(size_t)b * plane + i])) {
      s += p[(size_t)b * plane + i];
      c += 1.0f;
    }
  block_sum2(s, c);
  if (threadIdx.x == 0) {
    part[((size_t)b * gridDim.x + blockIdx.x) * 2] = s;
    part[((size_t)b * gridDim.x + blockIdx.x) * 2 + 1] = c;
  }
}

__global__ void sample_mean_final(const float *part, int nblocks, float *sum, float *cnt) {
  const int b = blockIdx.x, lane = threadIdx.x;
  float s = 0.0f, c = 0.0f;
  for (int k = lane; k < nblocks; k += 32) {
    s += part[((size_t)b * nblocks + k) * 2];
    c += part[((size_t)b * nblocks + k) * 2 + 1];
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if (lane == 0) {
    sum[b] = s;
    cnt[b] = c;
  }
}

// Predicted pressure on every cell of each sample: p = p_prev + s*dx2*q on
// fluid cells, then the boundary copy (the solver's copy rule) for cells
// with an edge; other cells keep p_prev.
__device__ __forceinline__ float copy_at(const float *p, int i, int w, int edge) {
  switch (edge) {
    case strm::E_N: return p[i - 1];
    case strm::E_NE: return (p[i - 1] + p[i + w]) * 0.5f;
    case strm::E_E: return p[i + w];
    case strm::E_SE: return (p[i + 1] + p[i + w]) * 0.5f;
    case strm::E_S: return p[i + 1];
    case strm::E_SW: return (p[i + 1] + p[i - w]) * 0.5f;
    case strm::E_W: return p[i - w];
    default: return (p[i - 1] + p[i - w]) * 0.5f;
  }
}

// Relative Poisson residual loss over fluid interior cells of each sample:
// r = Lap(p) - rhs (5-point, the solver's stencil, cells outside a sample's
// plane count as its boundary copies), loss_b = sum r^2 / sum rhs^2.
// Planes here are the full sample grids [nx][ny] (ring included) so that
// the boundary copy has its neighbours; `pfull` holds p with the copy
// applied (written by predict_full).
__global__ void predict_full(const float *pprev, const float *q, const uint8_t *flags,
                             const float *smax, float dx2, float *pfull, int batch, int nx,
                             int ny) {
  const long long plane = (long long)nx * ny;
  GRID_STRIDE(i, (long long)batch * plane) {
    const int b = (int)(i / plane);
    const int j = (int)(i - (long long)b * plane);
    const int x = j / ny, y = j % ny;
    const float s = smax[b] > 0.0f ? smax[b] : 1.0f;
    float v = pprev[i];
    if (!is_bnd(flags[i]) && x > 0 && y > 0 && x < nx - 1 && y < ny - 1)
      v += s * dx2 * q[(long long)b * (nx - 2) * (ny - 2) + (long long)(x - 1) * (ny - 2) + (y - 1)];
    pfull[i] = v;
  }
}

__global__ void apply_copy(float *pfull, const uint8_t *flags, int batch, int nx, int ny) {
  const long long plane = (long long)nx * ny;
  GRID_STRIDE(i, (long long)batch * plane) {
    const uint8_t f = flags[i];
    if (is_bnd(f) && edge_of(f) != strm::E_NONE) {
      const long long b = i / plane;
      const int j = (int)(i - b * plane);
      pfull[i] = copy_at(pfull + b * plane, j, ny, edge_of(f));
    }
  }
}

// Residual at fluid interior cells -> r (0 elsewhere), sum r^2 and sum rhs^2 per sample.
__global__ void residual_loss(const float *pfull, const float *rhs, const uint8_t *flags,
                              float rdx2, float rdy2, float *r, float *sum_r2, float *sum_b2,
                              int batch, int nx, int ny) {
  const long long plane = (long long)nx * ny;
  float a = 0.0f, bb = 0.0f;
  int bcur = -1;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < batch * plane;
       i += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(i / plane);
    const int j = (int)(i - (long long)b * plane);
    const int x = j / ny, y = j % ny;
    float rv = 0.0f;
    if (!is_bnd(flags[i]) && x > 0 && y > 0 && x < nx - 1 && y < ny - 1) {
      const float *p = pfull + (long long)b * plane;
      rv = (p[j + ny] + p[j - ny] - 2.0f * p[j]) * rdx2 + (p[j + 1] + p[j - 1] - 2.0f * p[j]) * rdy2 -
           rhs[i];
      if (b != bcur) {
        if (bcur >= 0) {
          atomicAdd(sum_r2 + bcur, a);
          atomicAdd(sum_b2 + bcur, bb);
        }
        bcur = b;
        a = bb = 0.0f;
      }
      a += rv * rv;
      bb += rhs[i] * rhs[i];
    }
    r[i] = rv;
  }
  if (bcur >= 0) {
    atomicAdd(sum_r2 + bcur, a);
    atomicAdd(sum_b2 + bcur, bb);
  }
}

// Gradient of mean_b(sum r^2 / sum rhs^2) with respect to q (fluid cells):
// gp = L^T (2 r / (B sum_b2)) on every cell, then the adjoint of the
// boundary copy moves each boundary cell's share onto the fluid cells it
// copies, then gq = s dx2 gp on fluid cells.
__global__ void residual_grad_p(const float *r, const uint8_t *flags, const float *sum_b2,
                                float rdx2, float rdy2, float *gp, int batch, int nx, int ny) {
  const long long plane = (long long)nx * ny;
  GRID_STRIDE(i, (long long)batch * plane) {
    const int b = (int)(i / plane);
    const int j = (int)(i - (long long)b * plane);
    const int x = j / ny, y = j % ny;
    const float c = 2.0f / ((float)batch * (sum_b2[b] > 0.0f ? sum_b2[b] : 1.0f));
    const float *rb = r + (long long)b * plane;
    float g = -2.0f * (rdx2 + rdy2) * rb[j];
    if (x > 0) g += rdx2 * rb[j - ny];
    if (x < nx - 1) g += rdx2 * rb[j + ny];
    if (y > 0) g += rdy2 * rb[j - 1];
    if (y < ny - 1) g += rdy2 * rb[j + 1];
    gp[i] = c * g;
  }
}

__global__ void copy_adjoint_to_q(const float *gp, const uint8_t *flags, const float *smax,
                                  float dx2, float *gq, int batch, int nx, int ny) {
  const int h = nx - 2, w = ny - 2;
  const long long plane = (long long)nx * ny;
  GRID_STRIDE(i, (long long)batch * h * w) {
    const int b = (int)(i / ((long long)h * w));
    const int rem = (int)(i - (long long)b * h * w);
    const int x = rem / w + 1, y = rem % w + 1;
    const int j = x * ny + y;
    const float *g = gp + (long long)b * plane;
    const uint8_t *f = flags + (long long)b * plane;
    if (is_bnd(f[j])) {
      gq[i] = 0.0f;
      continue;
    }
    float acc = g[j];
    // boundary neighbours whose copy reads this cell
    const int nb[4] = {j - ny, j + ny, j - 1, j + 1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint8_t fb = f[nb[k]];
      if (!is_bnd(fb)) continue;
      const int e = edge_of(fb);
      if (e == strm::E_NONE) continue;
      const bool corner = e == strm::E_NE || e == strm::E_SE || e == strm::E_SW || e == strm::E_NW;
      acc += (corner ? 0.5f : 1.0f) * g[nb[k]];
    }
    const float s = smax[b] > 0.0f ? smax[b] : 1.0f;
    gq[i] = s * dx2 * acc;
  }
}

// Error loss against a target pressure (the converged solution): on fluid
// interior cells e = p_prev + s dx^2 q - p_target and d = p_target - p_prev,
// both with their fluid mean removed (the pressure is defined up to a
// constant); loss_b = sum e^2 / sum d^2.  Pass 1 sums e, d and the cell count
// per sample, pass 2 the squares, pass 3 the gradient with respect to q.
__device__ __forceinline__ bool interior_fluid(const uint8_t *flags, long long i, int x, int y,
                                               int nx, int ny) {
  return flags[i] == 0 && x > 0 && y > 0 && x < nx - 1 && y < ny - 1;
}

__device__ __forceinline__ float err_raw(const float *pprev, const float *q, const float *pt,
                                         const float *smax, float dx2, long long i, int b, int x,
                                         int y, int nx, int ny) {
  const float s = smax[b] > 0.0f ? smax[b] : 1.0f;
  const float qv = q[(long long)b * (nx - 2) * (ny - 2) + (long long)(x - 1) * (ny - 2) + (y - 1)];
  return pprev[i] + s * dx2 * qv - pt[i];
}

__global__ void error_sums(const float *pprev, const float *q, const float *pt,
                           const uint8_t *flags, const float *smax, float dx2, float *work,
                           int batch, int nx, int ny, int pass) {
  // work: [0,B) sum e, [B,2B) sum d, [2B,3B) count, [3B,4B) sum e^2, [4B,5B) sum d^2
  const long long plane = (long long)nx * ny;
  GRID_STRIDE(i, (long long)batch * plane) {
    const int b = (int)(i / plane);
    const int j = (int)(i - (long long)b * plane);
    const int x = j / ny, y = j % ny;
    if (!interior_fluid(flags, i, x, y, nx, ny)) continue;
    const float e = err_raw(pprev, q, pt, smax, dx2, i, b, x, y, nx, ny);
    const float d = pt[i] - pprev[i];
    if (pass == 0) {
      atomicAdd(work + b, e);
      atomicAdd(work + batch + b, d);
      atomicAdd(work + 2 * batch + b, 1.0f);
    } else {
      const float c = work[2 * batch + b];
      const float em = e - work[b] / c, dm = d - work[batch + b] / c;
      atomicAdd(work + 3 * batch + b, em * em);
      atomicAdd(work + 4 * batch + b, dm * dm);
    }
  }
}

__global__ void error_grad(const float *pprev, const float *q, const float *pt,
                           const uint8_t *flags, const float *smax, float dx2, const float *work,
                           float *loss, float *gq, int batch, int nx, int ny) {
  const int h = nx - 2, w = ny - 2;
  GRID_STRIDE(k, (long long)batch * h * w) {
    const int b = (int)(k / ((long long)h * w));
    const int rem = (int)(k - (long long)b * h * w);
    const int x = rem / w + 1, y = rem % w + 1;
    const long long i = (long long)b * nx * ny + (long long)x * ny + y;
    const float d2 = work[4 * batch + b] > 0.0f ? work[4 * batch + b] : 1.0f;
    if (rem == 0 && loss) loss[b] = work[3 * batch + b] / d2;
    if (!gq) continue;
    float g = 0.0f;
    if (flags[i] == 0) {
      const float s = smax[b] > 0.0f ? smax[b] : 1.0f;
      const float em =
          err_raw(pprev, q, pt, smax, dx2, i, b, x, y, nx, ny) - work[b] / work[2 * batch + b];
      g = (2.0f / (float)batch) * em / d2 * s * dx2;
    }
    gq[k] = g;
  }
}

__global__ void mean_div(const float *sum, const float *cnt, float *out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cnt[i] > 0.0f ? sum[i] / cnt[i] : 0.0f;
}

// Adam on FP32 master weights (optionally a padded BF16 copy written as well:
// rows of `row` valid entries in a stride of `ld`).
__global__ void adam_step(float *w, const float *g, float *m, float *v, long long n, float lr,
                          float b1, float b2, float eps, float c1, float c2,
                          __nv_bfloat16 *wbf) {
  GRID_STRIDE(i, n) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wbf) wbf[i] = __float2bfloat16_rn(wi);
  }
}

}  // namespace strm_nn

// ------------------------------------------------------------------------
// C ABI (include/stroemung_nn.h)
// ------------------------------------------------------------------------

namespace {
inline int grid_for(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  if (g > 152 * 16) g = 152 * 16;
  return g < 1 ? 1 : (int)g;
}
inline int done() { return cudaGetLastError() == cudaSuccess ? STRM_NN_OK : STRM_NN_ERR_CUDA; }
// 16-byte vector kernels apply: channel count and strides multiples of 8,
// both base addresses 16-byte aligned
inline bool vec8(const void *a, const void *b, int c, int cs_a, int cs_b) {
  return c % 8 == 0 && cs_a % 8 == 0 && cs_b % 8 == 0 &&
         ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15u) == 0;
}
typedef __nv_bfloat16 bf16;
}  // namespace

using namespace strm_nn;

extern "C" {

int strm_nn_avgpool(const void *in, int cs_in, void *out, int cs_out, int batch, int h, int w,
                    int c, void *stream) {
  if (!in || !out || h % 2 || w % 2) return STRM_NN_ERR_INVALID;
  if (vec8(in, out, c, cs_in, cs_out)) {
    const int rows = batch * (h / 2), n = (w / 2) * (c / 8);
    const dim3 grid((n + 127) / 128, rows < 65535 ? rows : 65535);
    avgpool_rows8<<<grid, 128, 0, (cudaStream_t)stream>>>((const bf16 *)in, cs_in, (bf16 *)out,
                                                          cs_out, rows, h, w, c / 8);
    return done();
  }
  avgpool_fwd<<<grid_for((long long)batch * h * w * c / 4), 256, 0, (cudaStream_t)stream>>>(
      (const bf16 *)in, cs_in, (bf16 *)out, cs_out, batch, h, w, c);
  return done();
}

int strm_nn_avgpool_bwd(const void *gout, int cs_out, void *gin, int cs_in, int batch, int h,
                        int w, int c, int accumulate, void *stream) {
  if (!gout || !gin || h % 2 || w % 2) return STRM_NN_ERR_INVALID;
  if (vec8(gout, gin, c, cs_out, cs_in)) {
    avgpool_bwd8<<<grid_for((long long)batch * h * w * c / 8), 256, 0, (cudaStream_t)stream>>>(
        (const bf16 *)gout, cs_out, (bf16 *)gin, cs_in, batch, h, w, c, accumulate);
    return done();
  }
  avgpool_bwd<<<grid_for((long long)batch * h * w * c), 256, 0, (cudaStream_t)stream>>>(
      (const bf16 *)gout, cs_out, (bf16 *)gin, cs_in, batch, h, w, c, accumulate);
  return done();
}

int strm_nn_upsample(const void *in, int cs_in, void *out, int cs_out, int batch, int h, int w,
                     int c, void *stream) {
  if (!in || !out || h % 2 || w % 2) return STRM_NN_ERR_INVALID;
  if (vec8(in, out, c, cs_in, cs_out)) {
    const int rows = batch * (h / 2), n = (w / 2) * (c / 8);
    const dim3 grid((n + 127) / 128, rows < 65535 ? rows : 65535);
    upsample_rows8<<<grid, 128, 0, (cudaStream_t)stream>>>((const bf16 *)in, cs_in, (bf16 *)out,
                                                           cs_out, rows, h, w, c / 8);
    return done();
  }
  upsample_fwd<<<grid_for((long long)batch * h * w * c), 256, 0, (cudaStream_t)stream>>>(
      (const bf16 *)in, cs_in, (bf16 *)out, cs_out, batch, h, w, c);
  return done();
}

int strm_nn_upsample_bwd(const void *gout, int cs_out, void *gin, int cs_in, int batch, int h,
                         int w, int c, void *stream) {
  if (!gout || !gin || h % 2 || w % 2) return STRM_NN_ERR_INVALID;
  if (vec8(gout, gin, c, cs_out, cs_in)) {
    upsample_bwd8<<<grid_for((long long)batch * h * w * c / 32), 256, 0, (cudaStream_t)stream>>>(
        (const bf16 *)gout, cs_out, (bf16 *)gin, cs_in, batch, h, w, c);
    return done();
  }
  upsample_bwd<<<grid_for((long long)batch * h * w * c / 4), 256, 0, (cudaStream_t)stream>>>(
      (const bf16 *)gout, cs_out, (bf16 *)gin, cs_in, batch, h, w, c);
  return done();
}

int strm_nn_relu_mask(const void *g, int cs_g, const void *y, int cs_y, void *out, int cs_out,
                      long long npix, int c, void *stream) {
  if (!g || !y || !out) return STRM_NN_ERR_INVALID;
  if (vec8(g, out, c, cs_g, cs_out) && vec8(y, y, c, cs_y, cs_y)) {
    relu_mask8<<<grid_for(npix * c / 8), 256, 0, (cudaStream_t)stream>>>(
        (const bf16 *)g, cs_g, (const bf16 *)y, cs_y, (bf16 *)out, cs_out, npix, c);
    return done();
  }
  relu_mask<<<grid_for(npix * c), 256, 0, (cudaStream_t)stream>>>(
      (const bf16 *)g, cs_g, (const bf16 *)y, cs_y, (bf16 *)out, cs_out, npix, c);
  return done();
}

int strm_nn_bias_grad(const void *g, int cs_g, const void *y, int cs_y, float *db,
                      long long npix, int c, void *stream) {
  if (!g || !db || c <= 0 || c > 4096) return STRM_NN_ERR_INVALID;
  bias_grad<<<grid_for(npix * c), 256, c * sizeof(float), (cudaStream_t)stream>>>(
      (const bf16 *)g, cs_g, (const bf16 *)y, cs_y, db, npix, c);
  return done();
}

int strm_nn_flip_weights(const void *w, int cout, int cin_p, int kp, void *wt, int cout_p,
                         int kp_t, void *stream) {
  if (!w || !wt) return STRM_NN_ERR_INVALID;
  flip_weights<<<grid_for((long long)cin_p * kp_t), 256, 0, (cudaStream_t)stream>>>(
      (const bf16 *)w, cout, cin_p, kp, (bf16 *)wt, cout_p, kp_t);
  return done();
}

int strm_nn_head(const void *act, int cs, int c, const float *wh, const float *bh, float *out,
                 long long npix, void *stream) {
  if (!act || !wh || !bh || !out) return STRM_NN_ERR_INVALID;
  head_fwd<<<grid_for(npix), 256, 0, (cudaStream_t)stream>>>((const bf16 *)act, cs, c, wh, bh,
                                                              out, npix);
  return done();
}

int strm_nn_head_bwd(const void *act, int cs, int c, const float *wh, const float *gout,
                     void *gact, int cs_g, float *dwh, float *dbh, long long npix, void *stream) {
  if (!act || !wh || !gout || !gact || !dwh || !dbh || c > 4096) return STRM_NN_ERR_INVALID;
  head_bwd<<<grid_for(npix), 256, (c + 1) * sizeof(float), (cudaStream_t)stream>>>(
      (const bf16 *)act, cs, c, wh, gout, (bf16 *)gact, cs_g, dwh, dbh, npix);
  return done();
}

int strm_nn_prepare_input(const float *rhs, const uint8_t *flags, const float *pprev,
                          float *smax, float *pmean, float *work2, float dx2, void *xin,
                          int batch, int nx, int ny, void *stream) {
  if (!rhs || !flags || !pprev || !smax || !pmean || !work2 || !xin || nx < 3 || ny < 3)
    return STRM_NN_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int plane = nx * ny;
  if (cudaMemsetAsync(smax, 0, sizeof(float) * batch, s) != cudaSuccess ||
      cudaMemsetAsync(work2, 0, sizeof(float) * 2 * batch, s) != cudaSuccess)
    return STRM_NN_ERR_CUDA;
  dim3 g2((plane + 255) / 256 < 64 ? (plane + 255) / 256 : 64, batch);
  sample_absmax<<<g2, 256, 0, s>>>(rhs, flags, smax, plane);
  // the per-block partial sums borrow the start of xin, which
  // assemble_input then overwrites (16 bytes per interior cell; at most
  // 2 partials of 8 bytes per interior cell are used)
  float *part = static_cast<float *>(xin);
  const long long room = (long long)(nx - 2) * (ny - 2) * 2;  // 8-byte partials per sample
  const int nmb = room < kMeanBlocks ? (int)room : kMeanBlocks;
  sample_mean_partial<<<dim3(nmb, batch), 256, 0, s>>>(pprev, flags, part, plane);
  sample_mean_final<<<batch, 32, 0, s>>>(part, nmb, work2, work2 + batch);
  mean_div<<<(batch + 255) / 256, 256, 0, s>>>(work2, work2 + batch, pmean, batch);
  assemble_input<<<grid_for((long long)batch * (nx - 2) * (ny - 2)), 256, 0, s>>>(
      rhs, flags, pprev, smax, pmean, dx2, (bf16 *)xin, batch, nx, ny);
  return done();
}

int strm_nn_residual_loss(const float *pprev, const float *q, const uint8_t *flags,
                          const float *rhs, const float *smax, float dx2, float rdx2, float rdy2,
                          float *pfull, float *r, float *sum_r2, float *sum_b2, int batch, int nx,
                          int ny, void *stream) {
  if (!pprev || !q || !flags || !rhs || !smax || !pfull || !r || !sum_r2 || !sum_b2)
    return STRM_NN_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = (long long)batch * nx * ny;
  if (cudaMemsetAsync(sum_r2, 0, sizeof(float) * batch, s) != cudaSuccess ||
      cudaMemsetAsync(sum_b2, 0, sizeof(float) * batch, s) != cudaSuccess)
    return STRM_NN_ERR_CUDA;
  predict_full<<<grid_for(n), 256, 0, s>>>(pprev, q, flags, smax, dx2, pfull, batch, nx, ny);
  apply_copy<<<grid_for(n), 256, 0, s>>>(pfull, flags, batch, nx, ny);
  residual_loss<<<grid_for(n), 256, 0, s>>>(pfull, rhs, flags, rdx2, rdy2, r, sum_r2, sum_b2,
                                            batch, nx, ny);
  return done();
}

int strm_nn_residual_loss_grad(const float *r, const uint8_t *flags, const float *sum_b2,
                               const float *smax, float dx2, float rdx2, float rdy2, float *gp,
                               float *gq, int batch, int nx, int ny, void *stream) {
  if (!r || !flags || !sum_b2 || !smax || !gp || !gq) return STRM_NN_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const long long n = (long long)batch * nx * ny;
  residual_grad_p<<<grid_for(n), 256, 0, s>>>(r, flags, sum_b2, rdx2, rdy2, gp, batch, nx, ny);
  copy_adjoint_to_q<<<grid_for((long long)batch * (nx - 2) * (ny - 2)), 256, 0, s>>>(
      gp, flags, smax, dx2, gq, batch, nx, ny);
  return done();
}

int strm_nn_error_loss(const float *pprev, const float *q, const float *ptarget,
                       const uint8_t *flags, const float *smax, float dx2, float *work,
                       float *loss, float *gq, int batch, int nx, int ny, void *stream) {
  if (!pprev || !q || !ptarget || !flags || !smax || !work || nx < 3 || ny < 3 || batch < 1)
    return STRM_NN_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(work, 0, sizeof(float) * 5 * batch, s) != cudaSuccess)
    return STRM_NN_ERR_CUDA;
  const long long n = (long long)batch * nx * ny;
  error_sums<<<grid_for(n), 256, 0, s>>>(pprev, q, ptarget, flags, smax, dx2, work, batch, nx,
                                         ny, 0);
  error_sums<<<grid_for(n), 256, 0, s>>>(pprev, q, ptarget, flags, smax, dx2, work, batch, nx,
                                         ny, 1);
  error_grad<<<grid_for((long long)batch * (nx - 2) * (ny - 2)), 256, 0, s>>>(
      pprev, q, ptarget, flags, smax, dx2, work, loss, gq, batch, nx, ny);
  return done();
}

int strm_nn_zero(void *p, long long bytes, void *stream) {
  if (!p || bytes < 0) return STRM_NN_ERR_INVALID;
  return cudaMemsetAsync(p, 0, (size_t)bytes, (cudaStream_t)stream) == cudaSuccess
             ? STRM_NN_OK
             : STRM_NN_ERR_CUDA;
}

int strm_nn_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1,
                 float b2, float eps, int step, void *wbf, void *stream) {
  if (!w || !g || !m || !v || step < 1) return STRM_NN_ERR_INVALID;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  adam_step<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1,
                                                            c2, (bf16 *)wbf);
  return done();
}

}  // extern "C"
