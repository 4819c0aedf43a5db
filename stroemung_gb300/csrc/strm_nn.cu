// Dense contractions of the learned pressure warm start on the tcgen05 tensor
// cores: BF16 operands staged in 128B-swizzled shared memory, FP32
// accumulators in TMEM, one elected thread issuing tcgen05.mma.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <climits>
#include <mutex>

#include "../../include/stroemung_nn.h"
#include "strm_umma.cuh"

namespace strm_nn {

constexpr int GM = 128;  // rows per CTA tile (TMEM lanes)
constexpr int GN = 128;  // columns per CTA tile (TMEM columns)
constexpr int GK = 64;   // K per shared-memory stage (one 128-byte swizzle row)
constexpr uint32_t kWaitLimit = 1u << 26;

// D[M x N] (FP32, row-major) = A[M x K] * B[N x K]^T, A and B BF16 row-major
// (K contiguous).  M, N multiples of 128, K a multiple of 64.
__global__ void __launch_bounds__(128)
    gemm_bf16_kernel(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B,
                     float *__restrict__ D, int M, int N, int K, unsigned int *err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *sA = smem_raw + pad;
  uint8_t *sB = sA + GM * 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * GM, n0 = blockIdx.x * GN;

  if (warp == 0) tmem_alloc(&tmem_slot, GN);
  if (tid == 0) mbar_init(&mbar, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_bf16_f32(GM, GN);

  uint32_t phase = 0;
  int ok = 1;
  for (int k0 = 0; k0 < K && ok; k0 += GK) {
    for (int c = tid; c < GM * 8; c += 128) {
      const int r = c >> 3, j = c & 7;
      const uint4 val = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * K + k0 + j * 8);
      *reinterpret_cast<uint4 *>(sA + sw128_offset(r, j)) = val;
    }
    for (int c = tid; c < GN * 8; c += 128) {
      const int r = c >> 3, j = c & 7;
      const uint4 val = *reinterpret_cast<const uint4 *>(B + (size_t)(n0 + r) * K + k0 + j * 8);
      *reinterpret_cast<uint4 *>(sB + sw128_offset(r, j)) = val;
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint64_t da = desc_kmajor_sw128(smem_u32(sA));
      const uint64_t db = desc_kmajor_sw128(smem_u32(sB));
#pragma unroll
      for (int kk = 0; kk < GK / 16; ++kk)
        umma_bf16(tmem, da + 2 * kk, db + 2 * kk, idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
      umma_commit(&mbar);
    }
    ok = __syncthreads_and(mbar_wait_bounded(&mbar, phase, kWaitLimit) ? 1 : 0);
    phase ^= 1u;
  }
  tc_fence_after();
  if (ok) {
    float *row = D + (size_t)(m0 + warp * 32 + lane) * N + n0;
#pragma unroll 1
    for (int c = 0; c < GN; c += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; i += 4)
        *reinterpret_cast<float4 *>(row + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
  } else if (tid == 0) {
    atomicExch(err, 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, GN);
}

// ------------------------------------------------------------------------
// 3x3 "same" convolution as an implicit GEMM.
//
// Activations are BF16 NHWC: pixel q = (b*H + y)*W + x at x_ptr + q*cs,
// channels contiguous (cs >= channels; a concatenation is two channel slices
// of one buffer).  Input channels are padded to cin_p (a multiple of 8).  The
// GEMM: M = pixels (128 per CTA), N = output channels (the whole Cout, <=
// 256, a multiple of 16), K = 9*cin_p in tap-major order (tap t = (dy+1)*3 +
// (dx+1), then channel), padded to a multiple of 64.  Weights w[co][k] use
// the same K order, zero-padded.  Each 64-wide K chunk is 8 groups of 8
// channels of one tap, i.e. eight 16-byte loads per pixel, zero outside the
// image.  Epilogue: + bias, optional ReLU, BF16 NHWC store.
// ------------------------------------------------------------------------

// The 1x1 FP32 head fused into a convolution's epilogue (q != nullptr):
// q[p] = bh + sum_c wh[c] * y[p][c] over the BF16-rounded outputs, with the
// operations of head_fwd in its order; y may then be left unstored.
struct Head {
  const float *wh = nullptr;
  const float *bh = nullptr;
  float *q = nullptr;
};

struct ConvShape {
  int batch, h, w;
  int cin_p;      // padded input channels (multiple of 8)
  int cs_in;      // input pixel stride (elements)
  int cout;       // output channels (multiple of 16, <= 256)
  int cs_out;     // output pixel stride (elements)
  int kp;         // padded K = roundup(9*cin_p, 64)
  Head hd{};
};

// Epilogue of one 16-channel group of a pixel: bias, ReLU, the store (FP32,
// BF16 or none) and the fused head's share.
// Called by all 32 lanes of a warp together, lane l holding pixel q = (a
// multiple of 32) + l; pixels q >= npix are computed but not stored.
// PAIRED: BF16 stores of whole 32-byte sectors by lane pairs (below);
// otherwise each lane stores its own pixel's two 16-byte halves (fewer
// registers: the 8-channel layer, whose short CTAs gain more from
// occupancy, measured faster that way).
template <bool PAIRED = true>
__device__ __forceinline__ void conv_epilogue16(float *v, int c, const float *bias, int relu,
                                                __nv_bfloat16 *y, float *y32, long long q,
                                                long long npix, const ConvShape &s, float &hs) {
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    v[i] += bias ? bias[c + i] : 0.0f;
    if (relu) v[i] = fmaxf(v[i], 0.0f);
  }
  if (y32) {
    if (q < npix) {
      float *dst = y32 + q * s.cs_out + c;
#pragma unroll
      for (int i = 0; i < 16; ++i) dst[i] = v[i];
    }
    return;
  }
  // BF16 bits of the 16 outputs, two per word (channel 2i in the low half)
  uint32_t pk[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    pk[i] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * i])) |
            ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * i + 1])) << 16);
  if (y && !PAIRED) {
    if (q < npix) {
      uint4 *dst = reinterpret_cast<uint4 *>(y + q * s.cs_out + c);
      dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
  } else if (y) {
    // The two lanes of a pair store one pixel's 32 bytes (16 channels) with
    // one instruction, whole 32-byte sectors: first the even pixel (its
    // low half from the even lane, its high half handed to the odd lane),
    // then the odd pixel (its low half handed to the even lane).
    const uint4 lo = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    const uint4 hi = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    const bool odd = (threadIdx.x & 1) != 0;
    const uint4 snd = odd ? lo : hi;
    uint4 got;
    got.x = __shfl_xor_sync(0xffffffffu, snd.x, 1);
    got.y = __shfl_xor_sync(0xffffffffu, snd.y, 1);
    got.z = __shfl_xor_sync(0xffffffffu, snd.z, 1);
    got.w = __shfl_xor_sync(0xffffffffu, snd.w, 1);
    const long long pe = odd ? q - 1 : q, po = pe + 1;
    const int half = odd ? 8 : 0;  // elements
    if (pe < npix) *reinterpret_cast<uint4 *>(y + pe * s.cs_out + c + half) = odd ? got : lo;
    if (po < npix) *reinterpret_cast<uint4 *>(y + po * s.cs_out + c + half) = odd ? hi : got;
  }
  if (s.hd.q) {
    // the BF16 value as FP32: its bits in the high half
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      hs = fmaf(s.hd.wh[c + 2 * i], __uint_as_float(pk[i] << 16), hs);
      hs = fmaf(s.hd.wh[c + 2 * i + 1], __uint_as_float(pk[i] & 0xFFFF0000u), hs);
    }
  }
}

// Pipelined and warp-specialised: warps 0-3 gather the im2col rows (A) and
// the weights (B) of each 64-wide K chunk into a ring of S shared-memory
// stages with cp.async (16-byte copies, zero-filled outside the image),
// keeping LAG stages in flight; warp 4 (one lane) waits for a stage, issues
// its four MMAs (K = 16 each) and commits them to the stage's "empty"
// barrier, so the gather of later chunks overlaps the tensor-core work.
// Warps 0-3 then read the accumulator out of TMEM (warp w owns lanes
// 32w..32w+31) for the epilogue.  Every wait is bounded; a timeout sets
// *err and the CTA still releases its TMEM.
template <int BN>
struct ConvPipe {
  // stages: the gather is the bound, so fewer stages (more CTAs, more
  // gathering warps per SM) win except at 64 channels; measured on the
  // U-Net forward at 4096 x 1024 (2/3/2: 4.33 ms, 2/3/3: 4.63, 2/3/4: 4.89,
  // 2/2/2-3: 4.75-4.78, 3-4/3-4/4: 5.4-6.2)
  static constexpr int S = BN <= 32 ? 2 : (BN <= 64 ? 3 : 2);
  static constexpr int LAG = S - 1 < 2 ? S - 1 : 2;            // gathers in flight per thread
  static constexpr int A_BYTES = GM * 128;          // 128 rows x 64 BF16
  static constexpr int B_BYTES = BN * 128;
  static constexpr int STAGE = A_BYTES + B_BYTES;   // multiple of 1024
  static constexpr int SMEM = S * STAGE + 1024;
};

template <int BN>
__global__ void __launch_bounds__(160)
    conv3x3_fwd_kernel(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ w,
                       const float *__restrict__ bias, __nv_bfloat16 *__restrict__ y,
                       float *__restrict__ y32, ConvShape s, int relu, unsigned int *err) {
  using P = ConvPipe<BN>;
  constexpr int S = P::S, LAG = P::LAG;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[S], empty[S], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;
  constexpr int TM_COLS = BN < 32 ? 32 : BN;
  const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *stage0 = smem_raw + pad;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long npix = (long long)s.batch * s.h * s.w;
  const long long q0 = (long long)blockIdx.x * GM;
  const int nk = s.kp / GK;

  if (warp == 4) tmem_alloc(&tmem_slot, TM_COLS);
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&full[i], 128);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&done, 1);
    fail = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp < 4) {
    // ---- producers: thread t owns chunk column j = t % 8 of rows t/8 + 16 i ----
    // (pixel indices fit in 32 bits: the launcher checks npix < 2^31)
    const int j = tid & 7, rbase = tid >> 3;
    int px[8], py[8];
    const __nv_bfloat16 *prow[8];  // this row's pixel, channel 0 (NULL past the end)
    {
      int q = (int)q0 + rbase;
      int xx = q % s.w, yy = (q / s.w) % s.h;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        px[i] = xx;
        py[i] = yy;
        prow[i] = q < npix ? x + (size_t)q * s.cs_in : nullptr;
        q += 16;
        xx += 16;
        while (xx >= s.w) {
          xx -= s.w;
          if (++yy == s.h) yy = 0;
        }
      }
    }
    bool ok = true;
    for (int kc = 0; kc < nk; ++kc) {
      const int st = kc % S;
      if (kc >= S && ok) ok = mbar_wait_bounded(&empty[st], ((kc / S) - 1) & 1, kWaitLimit);
      if (ok) {
        uint8_t *sA = stage0 + st * P::STAGE;
        uint8_t *sB = sA + P::A_BYTES;
        const int k = kc * GK + 8 * j;
        const int tap = k / s.cin_p, ch = k - tap * s.cin_p;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        // the same element offset from every row's pixel
        const long long off = ((long long)dy * s.w + dx) * s.cs_in + ch;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int r = rbase + 16 * i;
          const int sy = py[i] + dy, sx = px[i] + dx;
          const bool in = prow[i] && tap < 9 && sy >= 0 && sy < s.h && sx >= 0 && sx < s.w;
          cp_async16(smem_u32(sA + sw128_offset(r, j)), in ? prow[i] + off : x, in ? 16u : 0u);
        }
        for (int c = tid; c < BN * 8; c += 128) {
          const int r = c >> 3, jj = c & 7;
          cp_async16(smem_u32(sB + sw128_offset(r, jj)), w + (size_t)r * s.kp + kc * GK + jj * 8,
                     16u);
        }
      }
      cp_async_commit();
      if (kc >= LAG) {
        cp_async_wait<LAG>();
        fence_async_smem();
        mbar_arrive(&full[(kc - LAG) % S]);
      }
    }
    cp_async_wait<0>();
    fence_async_smem();
    for (int kc = nk - LAG < 0 ? 0 : nk - LAG; kc < nk; ++kc) mbar_arrive(&full[kc % S]);
    if (!ok) atomicExch(&fail, 1);
  } else if (lane == 0) {
    // ---- MMA issuer ----
    const uint32_t idesc = idesc_bf16_f32(GM, BN);
    bool ok = true;
    for (int kc = 0; kc < nk && ok; ++kc) {
      const int st = kc % S;
      ok = mbar_wait_bounded(&full[st], (kc / S) & 1, kWaitLimit);
      if (!ok) break;
      tc_fence_after();
      uint8_t *sA = stage0 + st * P::STAGE;
      const uint64_t da = desc_kmajor_sw128(smem_u32(sA));
      const uint64_t db = desc_kmajor_sw128(smem_u32(sA + P::A_BYTES));
#pragma unroll
      for (int kk = 0; kk < GK / 16; ++kk)
        umma_bf16(tmem, da + 2 * kk, db + 2 * kk, idesc, (kc > 0 || kk > 0) ? 1u : 0u);
      umma_commit(&empty[st]);
    }
    if (ok) umma_commit(&done);
    else atomicExch(&fail, 1);
  }
  if (warp < 4) {
    // ---- epilogue ----
    const bool ok = mbar_wait_bounded(&done, 0, kWaitLimit);
    tc_fence_after();
    const long long q = q0 + warp * 32 + lane;
    if (ok) {
      float hs = s.hd.q ? *s.hd.bh : 0.0f;
#pragma unroll 1
      for (int c = 0; c < BN; c += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
        conv_epilogue16(v, c, bias, relu, y, y32, q, npix, s, hs);
      }
      if (s.hd.q && q < npix) s.hd.q[q] = hs;
    } else {
      atomicExch(&fail, 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && fail) atomicExch(err, 1u);
  if (warp == 4) tmem_dealloc(tmem, TM_COLS);
}

// ------------------------------------------------------------------------
// The same convolution with its operands staged by TMA (layers whose input
// channels are a multiple of 32, or 8, and whose image width is a multiple
// of 128), warp-specialised.  A tile is 128 consecutive pixels of one image
// row; CTA b takes tiles b, b + gridDim.x, ... (the launcher picks how many
// per CTA).  The K loop of a tile runs over taps (or kernel rows, below) and
// CH-channel slices (CH = 64: 128-byte swizzled rows; CH = 32: 64-byte
// swizzled rows; CH = 8: unswizzled 16-byte rows).
//   producer (warp 4, one thread): per K chunk a 4-D TMA load of the input
//     box {CH channels, 128 pixels at x0 + dx, row y + dy, image b} — the
//     border falls outside the tensor and is filled with zeros — and a 2-D
//     TMA load of the weight slice {CH, BN}, into the next stage of an
//     S-stage ring, across tile boundaries;
//   MMA issuer (warp 5, one thread): the chunk's CH/16 MMAs into one of
//     NACC accumulators in TMEM, committed to the stage's "empty" barrier,
//     and the tile's last commit to its accumulator's "full" barrier;
//   epilogue (warps 0-3): reads a finished accumulator, adds the bias,
//     applies the ReLU, stores BF16 (lane pairs writing whole 32-byte
//     sectors; or FP32) and, for the last layer, the 1x1 head, and hands
//     the accumulator back, so that it overlaps the next tile's loads and
//     MMAs.
// Every wait is bounded; a role whose wait runs out flags the CTA and stops,
// the producer still waits (bounded) for the copies it issued, and the CTA
// releases its TMEM.
// ------------------------------------------------------------------------

constexpr int kTmaMaxStages = 32;

// The ring's stage count is a launch parameter (up to kTmaMaxStages): the
// launcher fills the shared memory left by the CTAs it places on an SM.
// ROWS: a chunk is one kernel row dy and channel slice: the input box is the
// tile's 128 pixels with one more on each side (130 operand rows), and the
// three taps dx = -1, 0, +1 read it through descriptors that start 0, 1, 2
// rows in (the swizzle pattern follows the shared-memory address bits, so a
// start one 64- or 128-byte row into the box reads the rows as the copy
// swizzled them), against three weight slices.  Otherwise a chunk is one
// tap and slice (one 128-row box).  Row boxes move a third of the input
// bytes; the launcher takes them (with 32-channel slices) for tiles of up to
// 128 output channels.
//
// CH = 8 (layers with 8 input channels, always with row boxes): 16-byte
// operand rows without swizzle, so that 8 consecutive pixels of a box are
// one 8 x 16-byte core matrix wherever they start.  A K = 16 MMA pairs two
// taps of a row: its A descriptor starts at the first tap's pixel row and
// steps 16 bytes (one pixel) to the second tap's core matrix; the row's
// third tap pairs with a zero weight block (the box holds 131 pixels so
// that this pairing reads inside it).  The weights, 12 K blocks of
// BN x 8 (three rows x [three taps, zeros]), are staged once per CTA.
template <int BN, int CH, bool ROWS>
struct TmaConvPipe {
  static_assert(CH != 8 || ROWS, "8-channel slices take row boxes");
  static constexpr int ROWB = CH * 2;              // bytes per operand row
  static constexpr int A_ROWS = CH == 8 ? GM + 3 : ROWS ? GM + 2 : GM;
  static constexpr int ALIGN = CH == 8 ? 128 : 1024;
  static constexpr int A_BYTES = (A_ROWS * ROWB + ALIGN - 1) / ALIGN * ALIGN;
  static constexpr int TAPS = ROWS ? 3 : 1;        // taps per chunk
  static constexpr int B_TAP = CH == 8 ? 0 : BN * ROWB;
  static constexpr int B_BYTES = TAPS * B_TAP;
  static constexpr int STAGE = A_BYTES + B_BYTES;  // multiple of ALIGN
  static constexpr int TX = A_ROWS * ROWB + B_BYTES;  // bytes the copies write
  static constexpr int B_KBLOCK = BN * 16;           // CH = 8: one K block of the weights
  static constexpr int B_CONST = CH == 8 ? 12 * B_KBLOCK : 0;  // staged once per CTA
  static constexpr int NACC = 2 * BN <= 256 ? 2 : 1;  // accumulators in TMEM
  static constexpr int TM_COLS = NACC * BN < 32 ? 32 : NACC * BN;
  static constexpr int TM_ONE = BN < 32 ? 32 : BN;  // one accumulator
};

template <int BN, int CH, bool ROWS>
__global__ void __launch_bounds__(192)
    conv3x3_fwd_tma_kernel(const __grid_constant__ CUtensorMap tx,
                           const __grid_constant__ CUtensorMap tw, const float *__restrict__ bias,
                           __nv_bfloat16 *__restrict__ y, float *__restrict__ y32, ConvShape s,
                           int relu, int S, const __nv_bfloat16 *__restrict__ w,
                           unsigned int *err) {
  using P = TmaConvPipe<BN, CH, ROWS>;
  constexpr int NACC = P::NACC;
  static_assert(P::STAGE % P::ALIGN == 0, "stage alignment");
  static_assert(CH == 8 || P::B_TAP % (CH == 64 ? 1024 : 512) == 0, "weight slice alignment");
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kTmaMaxStages], empty[kTmaMaxStages], tfull[NACC], tempty[NACC];
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;
  const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *stage0 = smem_raw + pad;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = (int)((long long)s.batch * s.h * s.w / GM);
  const int cpt = s.cin_p / CH;  // chunks per tap
  const int nk = (ROWS ? 3 : 9) * cpt;

  // a CTA with one tile needs one accumulator
  const uint32_t tm_cols = (int)gridDim.x >= ntiles ? (uint32_t)P::TM_ONE : (uint32_t)P::TM_COLS;
  if (warp == 5) tmem_alloc(&tmem_slot, tm_cols);
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < NACC; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 4);  // one arrival per epilogue warp
    }
    fail = 0;
  }
  // CH = 8: the weights, staged once: K block i = 4 ky + t holds taps
  // (ky, t) for t < 3 and zeros for t = 3, n-block j's core matrix at
  // i * B_KBLOCK + 128 j, row n % 8 at +16 (n % 8)
  uint8_t *sB = stage0 + S * P::STAGE;
  if (CH == 8) {
    for (int e = tid; e < 12 * BN; e += blockDim.x) {
      const int i = e / BN, n = e - i * BN, ky = i >> 2, t3 = i & 3;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (t3 < 3) v = *reinterpret_cast<const uint4 *>(w + (size_t)n * s.kp + (ky * 3 + t3) * 8);
      *reinterpret_cast<uint4 *>(sB + i * P::B_KBLOCK + (n >> 3) * 128 + (n & 7) * 16) = v;
    }
    fence_async_smem();  // visible to the tensor core's reads
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 4 && lane == 0) {
    // ---- producer ----
    // stage st of the ring, its use parity ph, and whether every stage has
    // been used once (from then on a stage is refilled only after the MMAs
    // that read it have completed)
    bool ok = true, wrapped = false;
    int st = 0;
    uint32_t ph = 0;
    int issued = 0;  // chunks issued so far (all tiles)
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const long long q0 = (long long)t * GM;
      const int x0 = (int)(q0 % s.w);
      const long long row = q0 / s.w;
      const int yy = (int)(row % s.h), bb = (int)(row / s.h);
      for (int kc = 0; kc < nk; ++kc) {
        if (wrapped) {
          ok = mbar_wait_bounded(&empty[st], ph ^ 1u, kWaitLimit);
          if (!ok) break;
        }
        uint8_t *sA = stage0 + st * P::STAGE;
        mbar_arrive_expect_tx(&full[st], (uint32_t)P::TX);
        if (ROWS) {
          const int ky = kc / cpt, j = kc - ky * cpt;
          tma_load_4d(smem_u32(sA), &tx, j * CH, x0 - 1, yy + ky - 1, bb, &full[st]);
          if (CH != 8)
            for (int kx = 0; kx < 3; ++kx)
              tma_load_2d(smem_u32(sA + P::A_BYTES + kx * P::B_TAP), &tw,
                          (ky * 3 + kx) * s.cin_p + j * CH, 0, &full[st]);
        } else {
          const int tap = kc / cpt, j = kc - tap * cpt;
          const int dy = tap / 3 - 1, dx = tap % 3 - 1;
          tma_load_4d(smem_u32(sA), &tx, j * CH, x0 + dx, yy + dy, bb, &full[st]);
          tma_load_2d(smem_u32(sA + P::A_BYTES), &tw, tap * s.cin_p + j * CH, 0, &full[st]);
        }
        ++issued;
        if (++st == S) {
          st = 0;
          ph ^= 1u;
          wrapped = true;
        }
      }
    }
    if (!ok) atomicExch(&fail, 1);
    // every copy issued has landed before the CTA may leave (bounded): the
    // last min(issued, S) chunks, one per stage
    for (int g = issued - S < 0 ? 0 : issued - S; g < issued; ++g)
      if (!mbar_wait_bounded(&full[g % S], (uint32_t)(g / S) & 1u, kWaitLimit))
        atomicExch(&fail, 1);
  } else if (warp == 5 && lane == 0) {
    // ---- MMA issuer ----
    const uint32_t idesc = idesc_bf16_f32(GM, BN);
    bool ok = true;
    int st = 0;
    uint32_t ph = 0;
    int it = 0;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
      const int acc = it % NACC;
      if (it >= NACC) {
        ok = mbar_wait_bounded(&tempty[acc], (uint32_t)((it / NACC) - 1) & 1u, kWaitLimit);
        if (!ok) break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(acc * BN);
      for (int kc = 0; kc < nk; ++kc) {
        ok = mbar_wait_bounded(&full[st], ph, kWaitLimit);
        if (!ok) break;
        tc_fence_after();
        uint8_t *sA = stage0 + st * P::STAGE;
        if (CH == 8) {
          // taps (kc, 0) + (kc, 1), then (kc, 2) + the zero block
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const uint64_t da = desc_kmajor_noswz(smem_u32(sA + 32 * half), 16, 128);
            const uint64_t db = desc_kmajor_noswz(
                smem_u32(sB + (4 * kc + 2 * half) * P::B_KBLOCK), P::B_KBLOCK, 128);
            umma_bf16(d, da, db, idesc, (kc > 0 || half > 0) ? 1u : 0u);
          }
        } else {
#pragma unroll
        for (int kx = 0; kx < P::TAPS; ++kx) {
          // tap dx = kx - 1 of a row box: the 128 rows from row kx
          const uint32_t a = smem_u32(sA + kx * P::ROWB);
          const uint32_t b = smem_u32(sA + P::A_BYTES + kx * P::B_TAP);
          const uint64_t da = CH == 64 ? desc_kmajor_sw128(a) : desc_kmajor_sw64(a);
          const uint64_t db = CH == 64 ? desc_kmajor_sw128(b) : desc_kmajor_sw64(b);
#pragma unroll
          for (int kk = 0; kk < CH / 16; ++kk)
            umma_bf16(d, da + 2 * kk, db + 2 * kk, idesc,
                      (kc > 0 || kx > 0 || kk > 0) ? 1u : 0u);
        }
        }
        umma_commit(&empty[st]);
        if (++st == S) {
          st = 0;
          ph ^= 1u;
        }
      }
      if (ok) umma_commit(&tfull[acc]);
    }
    if (!ok) atomicExch(&fail, 1);
  } else if (warp < 4) {
    // ---- epilogue ----
    int it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
      const int acc = it % NACC;
      ok = mbar_wait_bounded(&tfull[acc], (uint32_t)(it / NACC) & 1u, kWaitLimit);
      if (!ok) break;
      tc_fence_after();
      const long long q = (long long)t * GM + warp * 32 + lane;
      float hs = s.hd.q ? *s.hd.bh : 0.0f;
#pragma unroll 1
      for (int c = 0; c < BN; c += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc * BN + c), v);
        conv_epilogue16<CH != 8>(v, c, bias, relu, y, y32, q, LLONG_MAX, s, hs);
      }
      if (s.hd.q) s.hd.q[q] = hs;
      // the accumulator may be overwritten once all four warps have read it
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
    }
    if (!ok) atomicExch(&fail, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && fail) atomicExch(err, 1u);
  if (warp == 5) tmem_dealloc(tmem, tm_cols);
}

// ------------------------------------------------------------------------
// Weight gradient of the 3x3 convolution: dW[co][k] += sum over pixels q of
// g[q][co] * im2col(x)[q][k], with g = dY masked by the ReLU (y > 0) when y
// is given.  GEMM with M = K rows (128 per CTA), N = Cout, reduction over
// pixels (64 per stage, `qchunk` pixels per CTA, partial sums added
// atomically in FP32).  Both operands are gathered transposed into the
// K-major swizzled tiles (the reduction index, pixels, along the 128-byte rows).
// ------------------------------------------------------------------------

template <int BN>
__global__ void __launch_bounds__(128)
    conv3x3_wgrad_kernel(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ dy,
                         const __nv_bfloat16 *__restrict__ yact, float *__restrict__ dw,
                         ConvShape s, int cs_dy, int qchunk, unsigned int *err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  constexpr int TM_COLS = BN < 32 ? 32 : BN;
  const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *sA = smem_raw + pad;
  uint8_t *sB = sA + GM * 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long npix = (long long)s.batch * s.h * s.w;
  const int k_base = blockIdx.x * GM;               // rows of dW^T
  const long long q_begin = (long long)blockIdx.y * qchunk;
  const long long q_end = q_begin + qchunk < npix ? q_begin + qchunk : npix;

  if (warp == 0) tmem_alloc(&tmem_slot, TM_COLS);
  if (tid == 0) mbar_init(&mbar, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_bf16_f32(GM, BN);
  __nv_bfloat16 *tA = reinterpret_cast<__nv_bfloat16 *>(sA);
  __nv_bfloat16 *tB = reinterpret_cast<__nv_bfloat16 *>(sB);
  const __nv_bfloat16 bzero = __float2bfloat16_rn(0.0f);

  uint32_t phase = 0;
  int ok = 1;
  bool first = true;
  for (long long qs = q_begin; qs < q_end && ok; qs += GK) {
    // A: 128 K-rows (tap, channel groups of 8) x 64 pixels
    for (int c = tid; c < (GM / 8) * GK; c += 128) {
      const int kg = c / GK, qi = c % GK;  // channel group within the tile, pixel
      const int k = k_base + 8 * kg;
      const long long q = qs + qi;
      const int tap = k / s.cin_p, ch = k - tap * s.cin_p;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (q < q_end && tap < 9 && k < s.kp) {
        const int xx = (int)(q % s.w);
        const int yy = (int)((q / s.w) % s.h);
        const int ddy = tap / 3 - 1, ddx = tap % 3 - 1;
        if (yy + ddy >= 0 && yy + ddy < s.h && xx + ddx >= 0 && xx + ddx < s.w)
          val = *reinterpret_cast<const uint4 *>(x + (q + (long long)ddy * s.w + ddx) * s.cs_in + ch);
      }
      const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&val);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int r = 8 * kg + i;
        tA[(sw128_offset(r, qi >> 3) >> 1) + (qi & 7)] = e[i];
      }
    }
    // B: Cout rows x 64 pixels of the (masked) output gradient
    for (int c = tid; c < (BN / 8) * GK; c += 128) {
      const int cg = c / GK, qi = c % GK;
      const long long q = qs + qi;
      __align__(16) __nv_bfloat16 e[8];
      if (q < q_end) {
        *reinterpret_cast<uint4 *>(e) = *reinterpret_cast<const uint4 *>(dy + q * cs_dy + 8 * cg);
        if (yact) {
          __align__(16) __nv_bfloat16 a[8];
          *reinterpret_cast<uint4 *>(a) =
              *reinterpret_cast<const uint4 *>(yact + q * s.cs_out + 8 * cg);
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!(__bfloat162float(a[i]) > 0.0f)) e[i] = bzero;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) e[i] = bzero;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int r = 8 * cg + i;
        tB[(sw128_offset(r, qi >> 3) >> 1) + (qi & 7)] = e[i];
      }
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint64_t da = desc_kmajor_sw128(smem_u32(sA));
      const uint64_t db = desc_kmajor_sw128(smem_u32(sB));
#pragma unroll
      for (int kk = 0; kk < GK / 16; ++kk)
        umma_bf16(tmem, da + 2 * kk, db + 2 * kk, idesc, (!first || kk > 0) ? 1u : 0u);
      umma_commit(&mbar);
    }
    first = false;
    ok = __syncthreads_and(mbar_wait_bounded(&mbar, phase, kWaitLimit) ? 1 : 0);
    phase ^= 1u;
  }
  tc_fence_after();
  if (ok && !first) {
    const int k = k_base + warp * 32 + lane;
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      if (k < s.kp) {
#pragma unroll
        for (int i = 0; i < 16; ++i) atomicAdd(dw + (size_t)(c + i) * s.kp + k, v[i]);
      }
    }
  } else if (!ok && tid == 0) {
    atomicExch(err, 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, TM_COLS);
}

namespace {
std::mutex g_mu;
unsigned int *g_err[64] = {};

cudaError_t error_flag(unsigned int **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_err[dev]) {
    e = cudaMalloc(&g_err[dev], sizeof(unsigned int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(g_err[dev], 0, sizeof(unsigned int));
    if (e != cudaSuccess) return e;
  }
  *out = g_err[dev];
  return cudaSuccess;
}

// 1: the contractions wait for their kernel and report its timeout flag
std::atomic<int> g_sync{1};

int read_flag(unsigned int *err, cudaStream_t s) {
  unsigned int h = 0;
  if (cudaMemcpyAsync(&h, err, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return STRM_NN_ERR_CUDA;
  return h ? STRM_NN_ERR_TIMEOUT : STRM_NN_OK;
}
}  // namespace

}  // namespace strm_nn

using namespace strm_nn;

extern "C" int strm_nn_gemm_bf16(const void *a, const void *b, float *d, int m, int n, int k,
                                 void *stream) {
  if (!a || !b || !d || m <= 0 || n <= 0 || k <= 0 || m % GM || n % GN || k % GK)
    return STRM_NN_ERR_INVALID;
  unsigned int *err = nullptr;
  if (error_flag(&err) != cudaSuccess) return STRM_NN_ERR_CUDA;
  const int smem = 2 * GM * 128 + 1024;
  cudaStream_t s = (cudaStream_t)stream;
  gemm_bf16_kernel<<<dim3(n / GN, m / GM), 128, smem, s>>>(
      (const __nv_bfloat16 *)a, (const __nv_bfloat16 *)b, d, m, n, k, err);
  if (cudaGetLastError() != cudaSuccess) return STRM_NN_ERR_CUDA;
  return g_sync.load() ? read_flag(err, s) : STRM_NN_OK;
}

namespace {

template <int BN>
int launch_conv(const void *x, int cs_in, int cin_p, const void *w, int kp, const float *bias,
                void *y, float *y32, int cs_out, int batch, int h, int width, int relu,
                cudaStream_t s, unsigned int *err, Head hd = Head{}) {
  ConvShape sh{batch, h, width, cin_p, cs_in, BN, cs_out, kp, hd};
  const int smem = ConvPipe<BN>::SMEM;
  // once per instantiation (thread-safe static initialisation)
  static const bool configured =
      cudaFuncSetAttribute(conv3x3_fwd_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem) == cudaSuccess;
  if (!configured) return STRM_NN_ERR_CUDA;
  const long long npix = (long long)batch * h * width;
  if (npix + GM >= (1LL << 31)) return STRM_NN_ERR_INVALID;
  const unsigned int grid = (unsigned int)((npix + GM - 1) / GM);
  conv3x3_fwd_kernel<BN><<<grid, 160, smem, s>>>((const __nv_bfloat16 *)x,
                                                 (const __nv_bfloat16 *)w, bias,
                                                 (__nv_bfloat16 *)y, y32, sh, relu, err);
  return cudaGetLastError() == cudaSuccess ? STRM_NN_OK : STRM_NN_ERR_CUDA;
}

// 1: layers that qualify use the TMA-fed forward (the default); 0: every
// layer uses the gathering kernel
std::atomic<int> g_conv_tma{1};
// Launch shape of the TMA-fed convolution: CTAs per SM (0: as many as hold a
// two-stage ring each), ring stages (0: the deepest that fits), tiles per
// CTA (0: four while the layer still fills every CTA slot of the GPU once,
// else two, else one — measured at 4096 x 1024: many short CTAs per SM hide
// the TMA latency, and a few tiles per CTA spread its set-up; CTAs walking
// all tiles persistently were slower on every layer), and row boxes of
// 32-channel slices for tiles of up to 128 output channels.
std::atomic<int> g_tma_ctas{0}, g_tma_stages{0}, g_tma_tiles{0}, g_tma_rows{1};

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); NULL when the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, []() {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// The TMA path takes layers whose input channels come in slices of 32 or 64
// and whose image rows hold whole 128-pixel tiles.
bool tma_conv_applies(int cin_p, int width, int cs_in, const void *x) {
  return g_conv_tma.load() && (cin_p % 32 == 0 || cin_p == 8) && width % GM == 0 &&
         cs_in % 8 == 0 && (reinterpret_cast<uintptr_t>(x) & 15u) == 0;
}

// Device limits of a TMA-fed instantiation, queried once (thread-safe
// static initialisation; the kernel's shared-memory attributes are set
// there too): SMs, shared memory per SM, per CTA (opt-in) and reserved per
// CTA, the kernel's static shared memory.
struct TmaLimits {
  int ok, nsm, smem_sm, smem_blk, reserved, stat;
};

template <int BN, int CH, bool ROWS>
TmaLimits tma_limits() {
  static const TmaLimits lim = [] {
    TmaLimits l{0, 0, 0, 0, 0, 0};
    int dev = 0;
    cudaFuncAttributes fa{};
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&l.smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&l.smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&l.reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&l.nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, conv3x3_fwd_tma_kernel<BN, CH, ROWS>) != cudaSuccess)
      return l;
    l.stat = (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(conv3x3_fwd_tma_kernel<BN, CH, ROWS>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             l.smem_blk - l.stat) != cudaSuccess ||
        cudaFuncSetAttribute(conv3x3_fwd_tma_kernel<BN, CH, ROWS>,
                             cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      return l;
    l.ok = 1;
    return l;
  }();
  return lim;
}

template <int BN, int CH, bool ROWS>
int launch_conv_tma(const void *x, int cs_in, int cin_p, const void *w, int kp,
                    const float *bias, void *y, float *y32, int cs_out, int batch, int h,
                    int width, int relu, cudaStream_t s, unsigned int *err, Head hd) {
  using P = TmaConvPipe<BN, CH, ROWS>;
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return -1;
  CUtensorMap tx{}, tw{};
  const CUtensorMapSwizzle sw = CH == 64   ? CU_TENSOR_MAP_SWIZZLE_128B
                                : CH == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                           : CU_TENSOR_MAP_SWIZZLE_NONE;
  // input: {channels (cin_p of a pixel's cs_in), x, y, image}, 2-byte elements
  const cuuint64_t xdim[4] = {(cuuint64_t)cin_p, (cuuint64_t)width, (cuuint64_t)h,
                              (cuuint64_t)batch};
  const cuuint64_t xstr[3] = {(cuuint64_t)cs_in * 2, (cuuint64_t)cs_in * 2 * width,
                              (cuuint64_t)cs_in * 2 * width * h};
  const cuuint32_t xbox[4] = {(cuuint32_t)CH, (cuuint32_t)P::A_ROWS, 1, 1};
  const cuuint32_t one[4] = {1, 1, 1, 1};
  if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(x), xdim, xstr, xbox, one,
          CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return -1;
  // weights: {K, output channels} (CH = 8 stages them without TMA)
  const cuuint64_t wdim[2] = {(cuuint64_t)kp, (cuuint64_t)BN};
  const cuuint64_t wstr[1] = {(cuuint64_t)kp * 2};
  const cuuint32_t wbox[2] = {(cuuint32_t)CH, (cuuint32_t)BN};
  if (CH != 8 &&
      enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(w), wdim, wstr, wbox, one,
          CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return -1;
  if (CH == 8 && (reinterpret_cast<uintptr_t>(w) & 15u) != 0) return -1;
  ConvShape sh{batch, h, width, cin_p, cs_in, BN, cs_out, kp, hd};
  const TmaLimits lim = tma_limits<BN, CH, ROWS>();
  if (!lim.ok) return STRM_NN_ERR_CUDA;
  const int nsm = lim.nsm, smem_sm = lim.smem_sm, smem_blk = lim.smem_blk,
            reserved = lim.reserved, stat = lim.stat;
  // CTAs per SM: the tuned count (TMEM holds 512 columns per SM), and the
  // ring that fills each CTA's share of the SM's shared memory
  const int tiles = g_tma_tiles.load();  // tiles per CTA, 0: by the layer's size
  const int tm_cap = 512 / (tiles != 1 ? P::TM_COLS : P::TM_ONE);
  int ctas = g_tma_ctas.load();
  if (ctas < 1) ctas = smem_sm / (2 * P::STAGE + P::B_CONST + 1024 + reserved + stat);
  if (ctas > 8) ctas = 8;
  if (ctas > tm_cap) ctas = tm_cap;
  // fewer CTAs until each holds a two-stage ring (the mode a layer takes
  // does not depend on the launch shape asked for)
  const int fixed = reserved + stat + 1024 + P::B_CONST;  // per CTA, besides the ring
  while (ctas > 1 && (smem_sm / ctas - fixed) / P::STAGE < 2) --ctas;
  if (ctas < 1) ctas = 1;
  int stages = (smem_sm / ctas - fixed) / P::STAGE;
  const int cap_blk = (smem_blk - stat - 1024 - P::B_CONST) / P::STAGE;
  if (stages > cap_blk) stages = cap_blk;
  if (stages > kTmaMaxStages) stages = kTmaMaxStages;
  const int tuned = g_tma_stages.load();
  if (tuned > 0 && tuned < stages) stages = tuned;
  if (stages < 2) return -1;
  const int dyn = stages * P::STAGE + P::B_CONST + 1024;
  // CTAs per SM at the last ring size asked: (dyn << 32) | fit, one atomic
  // word (concurrent callers store the same value for the same size)
  static std::atomic<unsigned long long> fit_cache{0};
  unsigned long long fc = fit_cache.load(std::memory_order_relaxed);
  int fit = (int)(fc & 0xFFFFFFFFu);
  if ((int)(fc >> 32) != dyn || fit < 1) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, conv3x3_fwd_tma_kernel<BN, CH, ROWS>,
                                                      192, dyn) != cudaSuccess ||
        fit < 1)
      return STRM_NN_ERR_CUDA;
    fit_cache.store(((unsigned long long)dyn << 32) | (unsigned int)fit,
                    std::memory_order_relaxed);
  }
  if (fit < ctas) ctas = fit;
  const long long npix = (long long)batch * h * width;
  if (npix >= (1LL << 31)) return STRM_NN_ERR_INVALID;
  const long long ntiles = npix / GM;
  // `per` tiles per CTA, CTA b taking tiles b, b + grid, ...
  const long long slots = (long long)ctas * nsm;
  const int per = tiles > 0 ? tiles : ntiles >= 4 * slots ? 4 : ntiles >= 2 * slots ? 2 : 1;
  const unsigned int grid = (unsigned int)((ntiles + per - 1) / per);
  conv3x3_fwd_tma_kernel<BN, CH, ROWS><<<grid, 192, dyn, s>>>(
      tx, tw, bias, (__nv_bfloat16 *)y, y32, sh, relu, stages, (const __nv_bfloat16 *)w, err);
  return cudaGetLastError() == cudaSuccess ? STRM_NN_OK : STRM_NN_ERR_CUDA;
}

// The TMA-fed forward when it applies (and its tensor maps encode), else the
// gathering kernel.
template <int BN>
int launch_conv_any(const void *x, int cs_in, int cin_p, const void *w, int kp, const float *bias,
                    void *y, float *y32, int cs_out, int batch, int h, int width, int relu,
                    cudaStream_t s, unsigned int *err, Head hd = Head{}) {
  if (tma_conv_applies(cin_p, width, cs_in, x)) {
    const bool c64 = cin_p % 64 == 0;
    int rc = -1;
    if (cin_p == 8) {
      // 8-channel input (the first layer): row boxes of 16-byte pixels
      if (g_tma_rows.load())
        rc = launch_conv_tma<BN, 8, true>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h,
                                          width, relu, s, err, hd);
      if (rc >= 0) return rc;
      return launch_conv<BN>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width,
                             relu, s, err, hd);
    }
    // row boxes of 32-channel slices (also for channel counts that are
    // multiples of 64) up to 128 output channels; 256-channel tiles keep one
    // box of 64-channel slices per tap (their row stages, with three weight
    // slices, leave too few CTAs per SM: measured slower), and so do
    // 64-channel slices in row boxes of 128-byte rows
    if (g_tma_rows.load() && BN <= 128)
      rc = launch_conv_tma<BN, 32, true>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h,
                                         width, relu, s, err, hd);
    if (rc < 0)
      rc = c64 ? launch_conv_tma<BN, 64, false>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out,
                                                batch, h, width, relu, s, err, hd)
               : launch_conv_tma<BN, 32, false>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out,
                                                batch, h, width, relu, s, err, hd);
    if (rc >= 0) return rc;
  }
  return launch_conv<BN>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width, relu, s,
                         err, hd);
}

template <int BN>
int launch_wgrad(const void *x, int cs_in, int cin_p, int kp, const void *dy, int cs_dy,
                 const void *yact, int cs_out, float *dw, int batch, int h, int width,
                 cudaStream_t s, unsigned int *err) {
  ConvShape sh{batch, h, width, cin_p, cs_in, BN, cs_out, kp};
  const int smem = GM * 128 + BN * 128 + 1024;
  static const bool configured =
      cudaFuncSetAttribute(conv3x3_wgrad_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem) == cudaSuccess;
  if (!configured) return STRM_NN_ERR_CUDA;
  const long long npix = (long long)batch * h * width;
  // split the pixel reduction so that the grid fills the GPU
  const int mtiles = (kp + GM - 1) / GM;
  long long want = (152LL * 4 + mtiles - 1) / mtiles;
  long long qchunk = (npix + want - 1) / want;
  qchunk = (qchunk + GK - 1) / GK * GK;
  if (qchunk < GK) qchunk = GK;
  const unsigned int ysplit = (unsigned int)((npix + qchunk - 1) / qchunk);
  conv3x3_wgrad_kernel<BN><<<dim3(mtiles, ysplit), 128, smem, s>>>(
      (const __nv_bfloat16 *)x, (const __nv_bfloat16 *)dy, (const __nv_bfloat16 *)yact, dw, sh,
      cs_dy, (int)qchunk, err);
  return cudaGetLastError() == cudaSuccess ? STRM_NN_OK : STRM_NN_ERR_CUDA;
}

int finish(unsigned int *err, cudaStream_t s, int rc) {
  if (rc != STRM_NN_OK || !g_sync.load()) return rc;
  return read_flag(err, s);
}

bool conv_args_ok(int cs_in, int cin_p, int kp, int cs_out, int cout) {
  return cin_p > 0 && cin_p % 8 == 0 && cs_in % 8 == 0 && cs_in >= cin_p &&
         kp % GK == 0 && kp >= 9 * cin_p && cs_out % 8 == 0 && cs_out >= cout &&
         (cout == 16 || cout == 32 || cout == 64 || cout == 128 || cout == 256);
}

}  // namespace

extern "C" int strm_nn_set_conv_tma(int use) {
  g_conv_tma.store(use ? 1 : 0);
  return STRM_NN_OK;
}

extern "C" int strm_nn_tune_conv_tma(int ctas_per_sm, int stages, int tiles_per_cta, int rows) {
  if (ctas_per_sm < 0 || ctas_per_sm > 8 || stages < 0 || stages == 1 ||
      stages > kTmaMaxStages || tiles_per_cta < 0 || tiles_per_cta > 64 || rows < 0 ||
      rows > 1)
    return STRM_NN_ERR_INVALID;
  g_tma_ctas.store(ctas_per_sm);
  g_tma_stages.store(stages);
  g_tma_tiles.store(tiles_per_cta);
  g_tma_rows.store(rows);
  return STRM_NN_OK;
}

extern "C" int strm_nn_set_sync(int sync) {
  g_sync.store(sync ? 1 : 0);
  return STRM_NN_OK;
}

extern "C" int strm_nn_status(void *stream) {
  unsigned int *err = nullptr;
  if (error_flag(&err) != cudaSuccess) return STRM_NN_ERR_CUDA;
  return read_flag(err, (cudaStream_t)stream);
}

extern "C" int strm_nn_conv3x3(const void *x, int cs_in, int cin_p, const void *w, int kp,
                               const float *bias, void *y, float *y32, int cs_out, int cout,
                               int batch, int h, int width, int relu, void *stream) {
  if (!x || !w || (!y && !y32) || batch < 1 || h < 1 || width < 1 ||
      !conv_args_ok(cs_in, cin_p, kp, cs_out, cout))
    return STRM_NN_ERR_INVALID;
  unsigned int *err = nullptr;
  if (error_flag(&err) != cudaSuccess) return STRM_NN_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  switch (cout) {
    case 16: rc = launch_conv_any<16>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width, relu, s, err); break;
    case 32: rc = launch_conv_any<32>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width, relu, s, err); break;
    case 64: rc = launch_conv_any<64>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width, relu, s, err); break;
    case 128: rc = launch_conv_any<128>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width, relu, s, err); break;
    default: rc = launch_conv_any<256>(x, cs_in, cin_p, w, kp, bias, y, y32, cs_out, batch, h, width, relu, s, err); break;
  }
  return finish(err, s, rc);
}

extern "C" int strm_nn_conv3x3_head(const void *x, int cs_in, int cin_p, const void *w, int kp,
                                    const float *bias, void *y, int cs_out, int cout, int batch,
                                    int h, int width, const float *wh, const float *bh, float *q,
                                    void *stream) {
  if (!x || !w || !wh || !bh || !q || batch < 1 || h < 1 || width < 1 ||
      !conv_args_ok(cs_in, cin_p, kp, y ? cs_out : cout, cout))
    return STRM_NN_ERR_INVALID;
  unsigned int *err = nullptr;
  if (error_flag(&err) != cudaSuccess) return STRM_NN_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  Head hd;
  hd.wh = wh;
  hd.bh = bh;
  hd.q = q;
  int rc;
  switch (cout) {
    case 16: rc = launch_conv_any<16>(x, cs_in, cin_p, w, kp, bias, y, nullptr, cs_out, batch, h, width, 1, s, err, hd); break;
    case 32: rc = launch_conv_any<32>(x, cs_in, cin_p, w, kp, bias, y, nullptr, cs_out, batch, h, width, 1, s, err, hd); break;
    case 64: rc = launch_conv_any<64>(x, cs_in, cin_p, w, kp, bias, y, nullptr, cs_out, batch, h, width, 1, s, err, hd); break;
    case 128: rc = launch_conv_any<128>(x, cs_in, cin_p, w, kp, bias, y, nullptr, cs_out, batch, h, width, 1, s, err, hd); break;
    default: rc = launch_conv_any<256>(x, cs_in, cin_p, w, kp, bias, y, nullptr, cs_out, batch, h, width, 1, s, err, hd); break;
  }
  return finish(err, s, rc);
}

extern "C" int strm_nn_conv3x3_wgrad(const void *x, int cs_in, int cin_p, int kp, const void *dy,
                                     int cs_dy, const void *yact, int cs_out, float *dw,
                                     int cout, int batch, int h, int width, void *stream) {
  if (!x || !dy || !dw || batch < 1 || h < 1 || width < 1 || cs_dy % 8 ||
      !conv_args_ok(cs_in, cin_p, kp, cs_out, cout))
    return STRM_NN_ERR_INVALID;
  unsigned int *err = nullptr;
  if (error_flag(&err) != cudaSuccess) return STRM_NN_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  switch (cout) {
    case 16: rc = launch_wgrad<16>(x, cs_in, cin_p, kp, dy, cs_dy, yact, cs_out, dw, batch, h, width, s, err); break;
    case 32: rc = launch_wgrad<32>(x, cs_in, cin_p, kp, dy, cs_dy, yact, cs_out, dw, batch, h, width, s, err); break;
    case 64: rc = launch_wgrad<64>(x, cs_in, cin_p, kp, dy, cs_dy, yact, cs_out, dw, batch, h, width, s, err); break;
    case 128: rc = launch_wgrad<128>(x, cs_in, cin_p, kp, dy, cs_dy, yact, cs_out, dw, batch, h, width, s, err); break;
    default: rc = launch_wgrad<256>(x, cs_in, cin_p, kp, dy, cs_dy, yact, cs_out, dw, batch, h, width, s, err); break;
  }
  return finish(err, s, rc);
}
