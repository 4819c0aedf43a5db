// Allocation-free residual norm (strm_norm_squared_noalloc).
//
// For callers that must not allocate device memory once they are running:
// host frameworks whose caching allocator already owns the device budget (a
// cudaMalloc beside that pool can fail or fragment it), and fixed-footprint
// loops that reserve all of their memory at start-up because cudaMalloc may
// synchronise the device and has no latency bound.  They pass their own
// pressure and RHS fields and an 8-byte device output; the reduction scratch
// this needs (one partial sum per 8 x 64 tile of the interior, plus a
// completion ticket) lives in a file-scope __device__ array of fixed size
// that every GPU loading the library keeps until the process exits.
//
// Limit: at most STRM_NORM_NOALLOC_MAX_TILES tiles, i.e. interior grids with
// ceil((nx-2)/8) * ceil((ny-2)/64) <= 16384 (for example 4096 x 2048 interior
// cells); larger grids are rejected with STRM_ERR_INVALID before any GPU work.
//
// All calls share that one array and it keeps the last call's contents, so
// calls whose GPU work overlaps (two streams, or two host threads) race on it
// and give wrong results; serialise them.  Each call clears the fields that
// must start at zero before its reduction runs.
//
// The array's device address is looked up once per device, on the first
// call made with that device current, and kept for the life of the process;
// a cudaDeviceReset while the library is in use invalidates it and is not
// supported.
#include <float.h>

#include <mutex>

#include "../../include/stroemung_gpu.h"
#include "strm_kernels.cuh"

using namespace strm;

namespace {

constexpr size_t kStateDoubles = (sizeof(StepState) + sizeof(double) - 1) / sizeof(double);
constexpr size_t kScratchDoubles = kStateDoubles + STRM_NORM_NOALLOC_MAX_TILES;

// The scratch.  In host code this name is only a stand-in for the symbol, not
// a device address; the address is looked up per device below.
static __device__ __align__(256) double g_norm_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device with that device current.
cudaError_t scratch_address(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_norm_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = (double *)p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

__global__ void noalloc_begin(StepState *st, double fluid_cells) {
  st->counter = 0;
  st->fluid_cells = fluid_cells;
  st->aux = 0.0;
}

__global__ void noalloc_end(const StepState *st, double *out) { *out = st->aux; }

}  // namespace

extern "C" int strm_norm_squared_noalloc(const double *p, const double *rhs, int nx, int ny,
                                         int pitch, double dx, double dy, double fluid_cells,
                                         double *norm_squared, void *stream) {
  // fluid_cells divides the sum (the reference's BoundaryList::fluid_cells):
  // zero, negative or non-finite counts are rejected like the other
  // entry points' bad arguments
  if (!p || !rhs || !norm_squared || nx < 1 || ny < 1 || pitch < ny || !(dx > 0.0) ||
      !(dy > 0.0) || !(fluid_cells > 0.0) || !(fluid_cells <= DBL_MAX))
    return STRM_ERR_INVALID;
  Geom g{nx, ny, pitch};
  const int tiles = interior_tiles(g);
  if (tiles > STRM_NORM_NOALLOC_MAX_TILES) return STRM_ERR_INVALID;
  double *scratch = nullptr;
  if (scratch_address(&scratch) != cudaSuccess) return STRM_ERR_CUDA;
  StepState *st = (StepState *)scratch;
  double *partials = scratch + kStateDoubles;
  Consts c{};
  c.dx = dx;
  c.dy = dy;
  c.dx2 = dx * dx;
  c.dy2 = dy * dy;
  c.r_dx2 = 1.0 / c.dx2;
  c.r_dy2 = 1.0 / c.dy2;
  c.two_r_sum = 2.0 * (c.r_dx2 + c.r_dy2);
  cudaStream_t s = (cudaStream_t)stream;
  noalloc_begin<<<1, 1, 0, s>>>(st, fluid_cells);
  if (cudaGetLastError() != cudaSuccess) return STRM_ERR_CUDA;
  if (launch_norm_one_block_per_tile(p, rhs, g, c, st, partials, s) != cudaSuccess)
    return STRM_ERR_CUDA;
  noalloc_end<<<1, 1, 0, s>>>(st, norm_squared);
  if (cudaGetLastError() != cudaSuccess) return STRM_ERR_CUDA;
  return STRM_OK;
}
