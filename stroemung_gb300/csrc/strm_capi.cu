// C ABI of the GB300 NaSt2D timestep (include/stroemung_gpu.h).
//
// Owns the device arena of one simulation, the compiled boundary program and
// the step graph; every compute call is a kernel or graph launch on the
// simulation's own stream.  There is no host fallback: without a usable
// sm_103 device strm_create fails with STRM_ERR_NO_DEVICE.
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "../../include/stroemung_gpu.h"
#include "strm_bcprog.h"
#include "strm_kernels.cuh"

using namespace strm;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(STRM_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                \
  } while (0)

constexpr int kLogCap = 4096;
// Polls a grid-barrier wait of the persistent batch solve may take before it
// gives up (each poll sleeps ~64 ns and reads L2: about a second or two).
constexpr unsigned long long kDefaultWaitPolls = 1ull << 22;
constexpr int kHistCap = 65536;  // residual history entries of one solve
constexpr int kAbiVersion = 1;

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct strm_sim {
  int dev = 0;
  cudaStream_t stream = nullptr;
  Geom g{};
  RunCfg cfg{};
  strm_params prm{};
  strm_mode mode{};
  DevFields d{};
  void *arena = nullptr;
  std::vector<uint8_t> kind;   // dense host copy of the cell kinds
  std::vector<double> wall;    // dense [nx][ny][2]
  std::vector<uint8_t> edge;   // dense edge codes (from the device classification)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph_pre = nullptr, graph_post = nullptr;
  cudaGraphExec_t exec_pre = nullptr, exec_post = nullptr;
  StepState *h_st = nullptr;   // pinned
  StepLog *h_log = nullptr;    // pinned
  int bc_cap = 0, pcopy_cap = 0, blist_cap = 0;
  void *rgba = nullptr;        // colour-map image, allocated on first use
  // strm_judge_correction's launches as one graph, for this q buffer and
  // sweep count; jd: device [scale, norm without, norm with the correction]
  cudaGraphExec_t judge_exec = nullptr;
  const float *judge_q = nullptr;
  int judge_sweeps = -1;
  double *jd = nullptr;
};

namespace {

double *field_ptr(strm_sim *s, int field) {
  switch (field) {
    case STRM_FIELD_U: return s->d.u;
    case STRM_FIELD_V: return s->d.v;
    case STRM_FIELD_P: return s->d.p;
    case STRM_FIELD_F: return s->d.f;
    case STRM_FIELD_G: return s->d.g;
    case STRM_FIELD_RHS: return s->d.rhs;
    default: return nullptr;
  }
}

Consts make_consts(const strm_params &p) {
  Consts c{};
  c.dx = p.dx;
  c.dy = p.dy;
  c.gamma = p.gamma;
  c.re = p.reynolds;
  c.dx2 = p.dx * p.dx;
  c.dy2 = p.dy * p.dy;
  c.four_dx = 4.0 * p.dx;
  c.four_dy = 4.0 * p.dy;
  c.r_dx = 1.0 / c.dx;
  c.r_dy = 1.0 / c.dy;
  c.r_dx2 = 1.0 / c.dx2;
  c.r_dy2 = 1.0 / c.dy2;
  c.r_four_dx = 1.0 / c.four_dx;
  c.r_four_dy = 1.0 / c.four_dy;
  c.r_re = 1.0 / c.re;
  // src/simulation.rs:240-246
  c.one_minus_w = 1.0 - p.omega;
  c.middle = p.omega / ((2.0 / c.dx2) + (2.0 / c.dy2));
  c.two_r_sum = 2.0 * (c.r_dx2 + c.r_dy2);
  c.eps2 = p.eps * p.eps;
  return c;
}

void update_cfg(strm_sim *s) {
  RunCfg &r = s->cfg;
  r.g = s->g;
  r.c = make_consts(s->prm);
  r.tau = s->prm.tau;
  r.delt = s->prm.delt;
  r.itermax = s->prm.max_iterations;
  r.strict_eps = (s->mode.strict_eps == 1 ? 1 : 0) | (s->mode.strict_eps == 2 ? 8 : 0) |
                 (s->mode.norm_cells != STRM_NORM_ALL_INTERIOR ? 2 : 0) |
                 (s->mode.norm_cells == STRM_NORM_FLUID_MEAN_FREE ? 4 : 0);
  r.sor_order = s->mode.sor_order == STRM_SOR_LEXICOGRAPHIC ? 1 : 0;
  // grids without interior cells run the single-CTA solve, which handles them
  if (s->g.nx < 3 || s->g.ny < 3) r.sor_order = 1;
  r.arith = s->mode.arithmetic == STRM_ARITH_FAST ? 1 : 0;
  r.precision = s->mode.precision;
  r.inner_sweeps = s->mode.inner_sweeps > 0 ? s->mode.inner_sweeps : 16;
  // public schedule numbers: 0 default (48 x 112 tiles, 4 sweeps per launch),
  // 1 one launch per colour pass, 2.. the blocked tile shapes
  r.sweep_schedule = s->mode.sweep_schedule == 0 ? 2 : s->mode.sweep_schedule - 1;
  r.eager = s->mode.execution == STRM_EXEC_EAGER ? 1 : 0;
}

void destroy_graphs(strm_sim *s) {
  if (s->judge_exec) cudaGraphExecDestroy(s->judge_exec);
  s->judge_exec = nullptr;
  s->judge_q = nullptr;
  cudaGraphExec_t *ex[3] = {&s->exec, &s->exec_pre, &s->exec_post};
  cudaGraph_t *gr[3] = {&s->graph, &s->graph_pre, &s->graph_post};
  for (int i = 0; i < 3; ++i) {
    if (*ex[i]) cudaGraphExecDestroy(*ex[i]);
    if (*gr[i]) cudaGraphDestroy(*gr[i]);
    *ex[i] = nullptr;
    *gr[i] = nullptr;
  }
}

static cudaError_t build_graphs(strm_sim *s) {
  cudaGraphExec_t *ex[3] = {&s->exec, &s->exec_pre, &s->exec_post};
  cudaGraph_t *gr[3] = {&s->graph, &s->graph_pre, &s->graph_post};
  for (int part = 0; part < 3; ++part) {
    cudaError_t e = build_step_graph(s->d, s->cfg, gr[part], part);
    if (e == cudaSuccess) e = cudaGraphInstantiate(ex[part], *gr[part], 0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int rebuild_graph(strm_sim *s) {
  destroy_graphs(s);
  update_cfg(s);
  cudaError_t e = build_graphs(s);
  if (e != cudaSuccess && fast_pdl()) {
    // a driver that refuses programmatic edges inside the solve's loop body:
    // build without them, and keep them off if that is what made it work
    destroy_graphs(s);
    (void)cudaGetLastError();
    set_fast_pdl(0);
    e = build_graphs(s);
    if (e != cudaSuccess) set_fast_pdl(1);
  }
  CK(e);
  return STRM_OK;
}

int sync_state(strm_sim *s) {
  CK(cudaMemcpyAsync(s->h_st, s->d.st, sizeof(StepState), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

// Device classification + host compile of the boundary program.
int classify_and_compile(strm_sim *s, long long *bad_out) {
  const Geom &g = s->g;
  const long long none = 0x7fffffffffffffffLL;
  CK(cudaMemcpyAsync(s->d.first_bad, &none, sizeof none, cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemsetAsync(s->d.fluid_count, 0, sizeof(unsigned long long), s->stream));
  CK(launch_classify(s->d, g, s->stream));
  long long bad = none;
  unsigned long long fluid = 0;
  CK(cudaMemcpyAsync(&bad, s->d.first_bad, sizeof bad, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaMemcpyAsync(&fluid, s->d.fluid_count, sizeof fluid, cudaMemcpyDeviceToHost,
                     s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (bad != none) {
    if (bad_out) *bad_out = bad;
    return fail(STRM_ERR_THIN_WALL, "cell (%lld, %lld) has fluid on opposing sides",
                bad / g.ny, bad % g.ny);
  }
  std::vector<uint8_t> flags((size_t)g.nx * g.ny);
  CK(cudaMemcpy2DAsync(flags.data(), g.ny, s->d.flags, g.pitch, g.ny, g.nx,
                       cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->edge.resize(flags.size());
  for (size_t i = 0; i < flags.size(); ++i) s->edge[i] = edge_of(flags[i]);
  std::vector<BcEntry> prog;
  std::vector<PCopy> pc;
  compile_boundary_program(g.nx, g.ny, g.pitch, s->kind.data(), s->edge.data(), s->wall.data(),
                           prog, pc);
  if ((int)prog.size() > s->bc_cap) {
    if (s->d.bc) cudaFree(s->d.bc);
    if (s->d.bc_val) cudaFree(s->d.bc_val);
    s->d.bc = nullptr;
    s->d.bc_val = nullptr;
    s->bc_cap = (int)prog.size() + 1024;
    CK(cudaMalloc(&s->d.bc, sizeof(BcEntry) * s->bc_cap));
    CK(cudaMalloc(&s->d.bc_val, sizeof(double) * s->bc_cap));
  }
  if ((int)pc.size() > s->pcopy_cap) {
    if (s->d.pcopy) cudaFree(s->d.pcopy);
    s->d.pcopy = nullptr;
    s->pcopy_cap = (int)pc.size() + 1024;
    CK(cudaMalloc(&s->d.pcopy, sizeof(PCopy) * s->pcopy_cap));
  }
  // the FAST red-black solve: solver classes (with, for fluid cells next
  // to a non-fluid cell, which neighbours are copied boundary cells) and the
  // boundary-cell list, black-coloured cells ((x + y) odd) first, x-major
  // within a colour
  std::vector<uint8_t> copy_edge((size_t)g.nx * g.pitch, 0);
  for (const PCopy &c : pc) copy_edge[(size_t)c.off] = (uint8_t)c.edge;
  const auto copied = [&](size_t o) { return copy_edge[o] != 0 ? 1u : 0u; };
  std::vector<uint8_t> cls(flags.size(), CLS_OTHER);
  for (int x = 1; x + 1 < g.nx; ++x)
    for (int y = 1; y + 1 < g.ny; ++y) {
      const size_t i = (size_t)x * g.ny + y;
      const size_t o = (size_t)x * g.pitch + y;
      if (flags[i] != 0) continue;
      const bool edge = flags[i - g.ny] || flags[i + g.ny] || flags[i - 1] || flags[i + 1];
      const unsigned int m = copied(o - g.pitch) | copied(o + g.pitch) << 1 |
                             copied(o - 1) << 2 | copied(o + 1) << 3;
      cls[i] = edge ? (uint8_t)(CLS_FLUID_EDGE | m << 2) : (uint8_t)CLS_FLUID;
    }
  std::vector<BCell> blist;
  int n_blist_b = 0;
  for (int colour = 1; colour >= 0; --colour) {
    for (int x = 0; x < g.nx; ++x)
      for (int y = 0; y < g.ny; ++y) {
        const size_t i = (size_t)x * g.ny + y;
        const size_t o = (size_t)x * g.pitch + y;
        if (((x + y) & 1) != colour || flags[i] == 0) continue;
        const bool interior = x >= 1 && x + 1 < g.nx && y >= 1 && y + 1 < g.ny;
        BCell e{};
        e.off = (unsigned int)o;
        e.edge = copy_edge[o];
        e.flags = (uint8_t)((interior ? BC_RES : 0) | (copied(o) ? BC_COPY : 0));
        if (!e.flags) continue;
        if (interior)
          e.mask = (uint8_t)(copied(o) | copied(o - g.pitch) << 1 | copied(o + g.pitch) << 2 |
                             copied(o - 1) << 3 | copied(o + 1) << 4);
        blist.push_back(e);
      }
    if (colour == 1) n_blist_b = (int)blist.size();
  }
  if ((int)blist.size() > s->blist_cap) {
    if (s->d.blist) cudaFree(s->d.blist);
    s->d.blist = nullptr;
    s->blist_cap = (int)blist.size() + 1024;
    CK(cudaMalloc(&s->d.blist, sizeof(BCell) * s->blist_cap));
  }
  s->d.n_blist = (int)blist.size();
  s->d.n_blist_b = n_blist_b;
  if (!blist.empty())
    CK(cudaMemcpyAsync(s->d.blist, blist.data(), sizeof(BCell) * blist.size(),
                       cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpy2DAsync(s->d.cls, g.pitch, cls.data(), g.ny, g.ny, g.nx, cudaMemcpyHostToDevice,
                       s->stream));
  s->d.n_bc = (int)prog.size();
  s->d.n_pcopy = (int)pc.size();
  if (!prog.empty())
    CK(cudaMemcpyAsync(s->d.bc, prog.data(), sizeof(BcEntry) * prog.size(),
                       cudaMemcpyHostToDevice, s->stream));
  if (!pc.empty())
    CK(cudaMemcpyAsync(s->d.pcopy, pc.data(), sizeof(PCopy) * pc.size(), cudaMemcpyHostToDevice,
                       s->stream));
  const double fc = (double)fluid;
  CK(cudaMemcpyAsync(&s->d.st->fluid_cells, &fc, sizeof fc, cudaMemcpyHostToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

void free_sim(strm_sim *s) {
  if (!s) return;
  destroy_graphs(s);
  if (s->arena) cudaFree(s->arena);
  if (s->d.bc) cudaFree(s->d.bc);
  if (s->d.bc_val) cudaFree(s->d.bc_val);
  if (s->d.pcopy) cudaFree(s->d.pcopy);
  if (s->d.blist) cudaFree(s->d.blist);
  if (s->rgba) cudaFree(s->rgba);
  if (s->jd) cudaFree(s->jd);
  if (s->h_st) cudaFreeHost(s->h_st);
  if (s->h_log) cudaFreeHost(s->h_log);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

int check_device(int *dev_out) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(STRM_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  int dev = 0;
  CK(cudaGetDevice(&dev));
  int major = 0, minor = 0;
  CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (major != 10 || minor != 3)
    return fail(STRM_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a",
                dev, major, minor);
  *dev_out = dev;
  return STRM_OK;
}

}  // namespace

namespace {

// The judge's launches on s->stream: both candidates' norms after `sweeps`
// FP64 red-black iterations (fast arithmetic, the sim's norm; 0: the
// initial norm after the boundary copy) into jd[2] (with the correction)
// and jd[1] (without), then the choice, made on the device.
cudaError_t record_judge(strm_sim *s, const float *q, int sweeps) {
  const size_t bytes = sizeof(double) * (size_t)s->g.nx * s->g.pitch;
  DevFields &d = s->d;
  RunCfg rj = s->cfg;
  rj.precision = 0;
  rj.arith = 1;
  cudaError_t e;
  auto norm_into = [&](double *dst) -> cudaError_t {
    cudaError_t err;
    if (sweeps == 0) {
      if ((err = launch_pcopy(d, s->g, s->stream)) != cudaSuccess) return err;
      if ((err = launch_norm(d, s->cfg, s->stream, 0)) != cudaSuccess) return err;
    } else {
      for (int k = 0; k < sweeps; ++k)  // the norm after the last iteration only
        if ((err = launch_sor_iteration(d, rj, s->stream, k + 1 == sweeps)) != cudaSuccess)
          return err;
    }
    return cudaMemcpyAsync(dst, &d.st->aux, sizeof(double), cudaMemcpyDeviceToDevice, s->stream);
  };
  if ((e = cudaMemcpyAsync(d.pw, d.p, bytes, cudaMemcpyDeviceToDevice, s->stream)) != cudaSuccess)
    return e;
  if ((e = launch_apply_correction(d, s->g, q, 0.0, s->stream, s->jd, 0)) != cudaSuccess) return e;
  if ((e = norm_into(s->jd + 2)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(d.p, d.pw, bytes, cudaMemcpyDeviceToDevice, s->stream)) != cudaSuccess)
    return e;
  if ((e = norm_into(s->jd + 1)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(d.p, d.pw, bytes, cudaMemcpyDeviceToDevice, s->stream)) != cudaSuccess)
    return e;
  if ((e = launch_apply_correction(d, s->g, q, 0.0, s->stream, s->jd, 1)) != cudaSuccess) return e;
  return launch_pcopy(d, s->g, s->stream);
}

}  // namespace

extern "C" {

int strm_abi_version(void) { return kAbiVersion; }

int strm_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return STRM_ERR_INVALID;
  snprintf(buf, len, "%s", g_last_error.c_str());
  return STRM_OK;
}

int strm_create(const strm_params *params, int nx, int ny, const uint8_t *kinds,
                const double *wall_uv, const double *u, const double *v, const double *p,
                strm_sim **out, int64_t *bad_index) {
  if (!out) return fail(STRM_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!params || !kinds || !u || !v || !p || nx < 1 || ny < 1)
    return fail(STRM_ERR_INVALID, "invalid arguments");
  // cell offsets of the solver's lists are 32-bit (a grid this large would
  // not fit in device memory anyway)
  if ((unsigned long long)nx * align_up((size_t)ny, 16) >= (1ULL << 32))
    return fail(STRM_ERR_INVALID, "grid of %d x %d cells is too large", nx, ny);
  const size_t ncell = (size_t)nx * ny;
  for (size_t i = 0; i < ncell; ++i)
    if (kinds[i] > STRM_MOVING_WALL)
      return fail(STRM_ERR_BAD_BOUNDARY, "cell %zu has unknown kind %u", i, (unsigned)kinds[i]);
  if (!(params->dx > 0.0) || !(params->dy > 0.0) || !(params->reynolds != 0.0))
    return fail(STRM_ERR_INVALID, "cell sizes must be positive and reynolds non-zero");
  int dev = 0;
  int rc = check_device(&dev);
  if (rc) return rc;

  strm_sim *s = new (std::nothrow) strm_sim();
  if (!s) return fail(STRM_ERR_INVALID, "out of host memory");
  s->dev = dev;
  s->prm = *params;
  s->mode = strm_mode{STRM_SOR_RED_BLACK, STRM_ARITH_EXACT, STRM_PREC_FP64, 0, 0,
                      STRM_EXEC_GRAPH};
  s->g.nx = nx;
  s->g.ny = ny;
  s->g.pitch = (int)align_up((size_t)ny, 16);
  s->kind.assign(kinds, kinds + ncell);
  s->wall.assign(2 * ncell, 0.0);
  if (wall_uv) s->wall.assign(wall_uv, wall_uv + 2 * ncell);

#define CKS(call)              \
  do {                         \
    int rc_ = (call);          \
    if (rc_) {                 \
      free_sim(s);             \
      return rc_;              \
    }                          \
  } while (0)
#define CKC(call) CKS([&]() -> int { CK(call); return STRM_OK; }())

  CKC(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  const size_t nfield = (size_t)nx * s->g.pitch;
  const int nb = residual_blocks(s->g);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  const size_t o_u = take(nfield * 8), o_v = take(nfield * 8), o_p = take(nfield * 8);
  const size_t o_f = take(nfield * 8), o_g = take(nfield * 8), o_rhs = take(nfield * 8);
  const size_t o_ru = take(nfield * 8), o_rv = take(nfield * 8), o_pw = take(nfield * 8);
  const size_t o_e32 = take(nfield * 4), o_r32 = take(nfield * 4), o_e32b = take(nfield * 4);
  const size_t o_fl = take(nfield);
  const size_t o_st = take(sizeof(StepState));
  const size_t o_part = take(sizeof(double) * 4 * (size_t)nb);
  const size_t o_partb = take(sizeof(double) * 2 * (size_t)black_pass_blocks(s->g));
  const size_t o_partr = take(sizeof(double) * 2 * (size_t)black_pass_blocks(s->g));
  const size_t o_cls = take(nfield);
  const size_t o_log = take(sizeof(StepLog) * kLogCap);
  const size_t o_bad = take(8), o_fc = take(8);
  const size_t o_hist = take(sizeof(double) * 2 * kHistCap);
  CKC(cudaMalloc(&s->arena, off));
  char *base = (char *)s->arena;
  DevFields &d = s->d;
  d.u = (double *)(base + o_u);
  d.v = (double *)(base + o_v);
  d.p = (double *)(base + o_p);
  d.f = (double *)(base + o_f);
  d.g = (double *)(base + o_g);
  d.rhs = (double *)(base + o_rhs);
  d.ru = (double *)(base + o_ru);
  d.rv = (double *)(base + o_rv);
  d.pw = (double *)(base + o_pw);
  d.e32 = (float *)(base + o_e32);
  d.r32 = (float *)(base + o_r32);
  d.e32b = (float *)(base + o_e32b);
  d.flags = (uint8_t *)(base + o_fl);
  d.st = (StepState *)(base + o_st);
  d.partials = (double *)(base + o_part);
  d.n_partials = 4 * nb;
  d.partials_b = (double *)(base + o_partb);
  d.partials_r = (double *)(base + o_partr);
  d.cls = (uint8_t *)(base + o_cls);
  d.log = (StepLog *)(base + o_log);
  d.first_bad = (long long *)(base + o_bad);
  d.fluid_count = (unsigned long long *)(base + o_fc);
  CKC(cudaMemsetAsync(s->arena, 0, off, s->stream));
  CKC(cudaMallocHost(&s->h_st, sizeof(StepState)));
  CKC(cudaMallocHost(&s->h_log, sizeof(StepLog) * kLogCap));

  const Geom &g = s->g;
  const size_t pb = (size_t)g.pitch * 8;
  CKC(cudaMemcpy2DAsync(d.u, pb, u, (size_t)ny * 8, (size_t)ny * 8, nx, cudaMemcpyHostToDevice,
                        s->stream));
  CKC(cudaMemcpy2DAsync(d.v, pb, v, (size_t)ny * 8, (size_t)ny * 8, nx, cudaMemcpyHostToDevice,
                        s->stream));
  CKC(cudaMemcpy2DAsync(d.p, pb, p, (size_t)ny * 8, (size_t)ny * 8, nx, cudaMemcpyHostToDevice,
                        s->stream));
  CKC(cudaMemcpy2DAsync(d.flags, g.pitch, kinds, ny, ny, nx, cudaMemcpyHostToDevice, s->stream));

  StepState st{};
  st.dt = params->delt;
  st.time = params->time;
  st.iterations = params->iterations;
  st.ns0 = isnan(params->initial_norm_squared) ? 0.0 : params->initial_norm_squared;
  st.umax = st.vmax = 1.0e-10;
  st.p_min = st.s2_min = ord_enc(DBL_MAX);
  st.p_max = st.s2_max = ord_enc(0.0);
  st.log_cap = kLogCap;
  st.hist = (double *)(base + o_hist);
  st.hist_cap = kHistCap;
  CKC(cudaMemcpyAsync(d.st, &st, sizeof st, cudaMemcpyHostToDevice, s->stream));

  long long bad = -1;
  rc = classify_and_compile(s, &bad);
  if (rc) {
    if (bad_index) *bad_index = bad;
    free_sim(s);
    return rc;
  }
  update_cfg(s);
  // construction passes of SimulationGrid::try_from and Simulation::try_from
  CKC(launch_prange(d, s->cfg, s->stream, 1));
  CKC(launch_velocity(d, s->cfg, s->stream, 0, 1, 0));
  CKC(launch_fg_rhs(d, s->cfg, s->stream));
  if (isnan(params->initial_norm_squared)) CKC(launch_norm(d, s->cfg, s->stream, 1));
  CKS(rebuild_graph(s));
  CKS(sync_state(s));
#undef CKC
#undef CKS
  *out = s;
  return STRM_OK;
}

int strm_destroy(strm_sim *sim) {
  if (!sim) return STRM_ERR_INVALID;
  cudaSetDevice(sim->dev);
  cudaStreamSynchronize(sim->stream);
  free_sim(sim);
  return STRM_OK;
}

int strm_set_mode(strm_sim *s, const strm_mode *mode) {
  if (!s || !mode) return fail(STRM_ERR_INVALID, "invalid arguments");
  if (mode->sor_order < 0 || mode->sor_order > 1 || mode->arithmetic < 0 ||
      mode->arithmetic > 1 || mode->precision < 0 || mode->precision > 1 ||
      mode->execution < 0 || mode->execution > 1 || mode->inner_sweeps < 0 ||
      mode->norm_cells < 0 || mode->norm_cells > 2 || mode->sweep_schedule < 0 ||
      mode->sweep_schedule > num_sweep_schedules())
    return fail(STRM_ERR_INVALID, "unknown mode value");
  if (mode->strict_eps < 0 || mode->strict_eps > 2)
    return fail(STRM_ERR_INVALID, "unknown stop rule %d", mode->strict_eps);
  if (mode->strict_eps == 2 && mode->sor_order == STRM_SOR_LEXICOGRAPHIC)
    return fail(STRM_ERR_INVALID, "the relative stop rule is available with red-black orders");
  if (mode->norm_cells != STRM_NORM_ALL_INTERIOR && mode->sor_order == STRM_SOR_LEXICOGRAPHIC)
    return fail(STRM_ERR_INVALID, "the fluid-cell norms are available with red-black orders");
  CK(cudaSetDevice(s->dev));
  s->mode = *mode;
  return rebuild_graph(s);
}

int strm_tick(strm_sim *s, uint32_t *sor_iterations, double *norm_squared) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  if (s->cfg.eager)
    CK(run_step_eager(s->d, s->cfg, s->stream, s->h_st));
  else
    CK(cudaGraphLaunch(s->exec, s->stream));
  int rc = sync_state(s);
  if (rc) return rc;
  if (sor_iterations) *sor_iterations = s->h_st->sor_iters;
  if (norm_squared) *norm_squared = s->h_st->ns;
  if (s->h_st->overrun) return fail(STRM_ERR_TIMEOUT, "pressure loop passed its bound");
  if (s->h_st->nonfinite) return fail(STRM_ERR_NONFINITE, "norm_squared is not finite");
  return STRM_OK;
}

int strm_step_n(strm_sim *s, int n, strm_step_stats *stats) {
  if (!s || n < 0) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  int done = 0;
  while (done < n) {
    const int chunk = (n - done) < kLogCap ? (n - done) : kLogCap;
    const unsigned int zero = 0;
    CK(cudaMemcpyAsync(&s->d.st->log_pos, &zero, sizeof zero, cudaMemcpyHostToDevice,
                       s->stream));
    for (int i = 0; i < chunk; ++i) {
      if (s->cfg.eager)
        CK(run_step_eager(s->d, s->cfg, s->stream, s->h_st));
      else
        CK(cudaGraphLaunch(s->exec, s->stream));
    }
    if (stats)
      CK(cudaMemcpyAsync(s->h_log, s->d.log, sizeof(StepLog) * chunk, cudaMemcpyDeviceToHost,
                         s->stream));
    int rc = sync_state(s);
    if (rc) return rc;
    if (stats)
      for (int i = 0; i < chunk; ++i) {
        stats[done + i].sor_iterations = s->h_log[i].sor_iters;
        stats[done + i].converged = s->h_log[i].converged;
        stats[done + i].norm_squared = s->h_log[i].ns;
        stats[done + i].delt = s->h_log[i].dt;
      }
    done += chunk;
    if (s->h_st->overrun) return fail(STRM_ERR_TIMEOUT, "pressure loop passed its bound");
  }
  if (s->h_st->nonfinite) return fail(STRM_ERR_NONFINITE, "norm_squared is not finite");
  return STRM_OK;
}

int strm_download(strm_sim *s, int field, double *host) {
  if (!s || !host) return fail(STRM_ERR_INVALID, "invalid arguments");
  double *src = field_ptr(s, field);
  if (!src) return fail(STRM_ERR_INVALID, "unknown field %d", field);
  CK(cudaSetDevice(s->dev));
  const Geom &g = s->g;
  CK(cudaMemcpy2DAsync(host, (size_t)g.ny * 8, src, (size_t)g.pitch * 8, (size_t)g.ny * 8, g.nx,
                       cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_upload(strm_sim *s, int field, const double *host) {
  if (!s || !host) return fail(STRM_ERR_INVALID, "invalid arguments");
  double *dst = field_ptr(s, field);
  if (!dst) return fail(STRM_ERR_INVALID, "unknown field %d", field);
  CK(cudaSetDevice(s->dev));
  const Geom &g = s->g;
  CK(cudaMemcpy2DAsync(dst, (size_t)g.pitch * 8, host, (size_t)g.ny * 8, (size_t)g.ny * 8, g.nx,
                       cudaMemcpyHostToDevice, s->stream));
  if (field == STRM_FIELD_U || field == STRM_FIELD_V)
    CK(launch_velocity(s->d, s->cfg, s->stream, 0, 0, 0));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_download_cells(strm_sim *s, uint8_t *kinds, uint8_t *edges) {
  if (!s) return fail(STRM_ERR_INVALID, "invalid arguments");
  const Geom &g = s->g;
  std::vector<uint8_t> flags((size_t)g.nx * g.ny);
  CK(cudaSetDevice(s->dev));
  CK(cudaMemcpy2DAsync(flags.data(), g.ny, s->d.flags, g.pitch, g.ny, g.nx,
                       cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (size_t i = 0; i < flags.size(); ++i) {
    if (kinds) kinds[i] = kind_of(flags[i]);
    if (edges) edges[i] = edge_of(flags[i]);
  }
  return STRM_OK;
}

int strm_edit_cells(strm_sim *s, int n, const int32_t *xs, const int32_t *ys,
                    const uint8_t *kinds, const double *wall_uv, int64_t *bad_index) {
  if (!s || n < 0 || (n > 0 && (!xs || !ys || !kinds)))
    return fail(STRM_ERR_INVALID, "invalid arguments");
  const Geom &g = s->g;
  for (int i = 0; i < n; ++i) {
    if (xs[i] < 0 || xs[i] >= g.nx || ys[i] < 0 || ys[i] >= g.ny)
      return fail(STRM_ERR_INVALID, "cell (%d, %d) outside the grid", xs[i], ys[i]);
    if (kinds[i] > STRM_MOVING_WALL)
      return fail(STRM_ERR_BAD_BOUNDARY, "unknown kind %u", (unsigned)kinds[i]);
  }
  CK(cudaSetDevice(s->dev));
  struct Backup {
    size_t dense, off;
    double u, v, p, wu, wv;
    uint8_t kind;
  };
  std::vector<Backup> backup;
  const double zero = 0.0;
  for (int i = 0; i < n; ++i) {
    const size_t dense = (size_t)xs[i] * g.ny + ys[i];
    const size_t off = (size_t)xs[i] * g.pitch + ys[i];
    const double wu = wall_uv ? wall_uv[2 * i] : 0.0, wv = wall_uv ? wall_uv[2 * i + 1] : 0.0;
    if (s->kind[dense] == kinds[i] && s->wall[2 * dense] == wu && s->wall[2 * dense + 1] == wv)
      continue;
    Backup b{dense, off, 0, 0, 0, s->wall[2 * dense], s->wall[2 * dense + 1], s->kind[dense]};
    CK(cudaMemcpyAsync(&b.u, s->d.u + off, 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&b.v, s->d.v + off, 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&b.p, s->d.p + off, 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    backup.push_back(b);
    if (s->kind[dense] != kinds[i]) {
      CK(cudaMemcpyAsync(s->d.u + off, &zero, 8, cudaMemcpyHostToDevice, s->stream));
      CK(cudaMemcpyAsync(s->d.v + off, &zero, 8, cudaMemcpyHostToDevice, s->stream));
      CK(cudaMemcpyAsync(s->d.p + off, &zero, 8, cudaMemcpyHostToDevice, s->stream));
    }
    s->kind[dense] = kinds[i];
    s->wall[2 * dense] = wu;
    s->wall[2 * dense + 1] = wv;
    CK(cudaMemcpyAsync(s->d.flags + off, &s->kind[dense], 1, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  }
  if (backup.empty()) return STRM_OK;
  long long bad = -1;
  int rc = classify_and_compile(s, &bad);
  if (rc == STRM_ERR_THIN_WALL) {
    for (auto it = backup.rbegin(); it != backup.rend(); ++it) {
      s->kind[it->dense] = it->kind;
      s->wall[2 * it->dense] = it->wu;
      s->wall[2 * it->dense + 1] = it->wv;
      CK(cudaMemcpyAsync(s->d.u + it->off, &it->u, 8, cudaMemcpyHostToDevice, s->stream));
      CK(cudaMemcpyAsync(s->d.v + it->off, &it->v, 8, cudaMemcpyHostToDevice, s->stream));
      CK(cudaMemcpyAsync(s->d.p + it->off, &it->p, 8, cudaMemcpyHostToDevice, s->stream));
      CK(cudaMemcpyAsync(s->d.flags + it->off, &s->kind[it->dense], 1, cudaMemcpyHostToDevice,
                         s->stream));
      CK(cudaStreamSynchronize(s->stream));
    }
    int rc2 = classify_and_compile(s, nullptr);
    if (rc2) return rc2;
    if (bad_index) *bad_index = bad;
    rebuild_graph(s);
    return fail(STRM_ERR_THIN_WALL, "cell (%lld, %lld) has fluid on opposing sides; edit rolled back",
                bad / g.ny, bad % g.ny);
  }
  if (rc) return rc;
  CK(launch_velocity(s->d, s->cfg, s->stream, 0, 0, 0));
  return rebuild_graph(s);
}

int strm_get_state(strm_sim *s, strm_state *out) {
  if (!s || !out) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  int rc = sync_state(s);
  if (rc) return rc;
  const StepState &st = *s->h_st;
  out->time = st.time;
  out->iterations = st.iterations;
  out->delt = st.dt;
  out->initial_norm_squared = st.ns0;
  out->fluid_cells = st.fluid_cells;
  out->pressure_range[0] = ord_dec(st.p_min);
  out->pressure_range[1] = ord_dec(st.p_max);
  out->speed_range[0] = ord_dec(st.s2_min);
  out->speed_range[1] = ord_dec(st.s2_max);
  out->last_sor_iterations = st.sor_iters;
  out->last_norm_squared = st.ns;
  out->last_converged = st.converged;
  return STRM_OK;
}

int strm_set_boundary_u_and_v(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_bc(s->d, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_calculate_f_g_rhs(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_fg_rhs(s->d, s->cfg, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_copy_pressure_to_boundaries(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_pcopy(s->d, s->g, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_calculate_norm_squared(strm_sim *s, double *norm_squared) {
  if (!s || !norm_squared) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  const double zero = 0.0;
  CK(cudaMemcpyAsync(&s->d.st->aux, &zero, 8, cudaMemcpyHostToDevice, s->stream));
  CK(launch_norm(s->d, s->cfg, s->stream, 0));
  int rc = sync_state(s);
  if (rc) return rc;
  *norm_squared = s->h_st->aux;
  return STRM_OK;
}

int strm_tick_prepare(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(cudaGraphLaunch(s->exec_pre, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_tick_solve(strm_sim *s, uint32_t *sor_iterations, double *norm_squared) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(cudaGraphLaunch(s->exec_post, s->stream));
  int rc = sync_state(s);
  if (rc) return rc;
  if (sor_iterations) *sor_iterations = s->h_st->sor_iters;
  if (norm_squared) *norm_squared = s->h_st->ns;
  if (s->h_st->overrun) return fail(STRM_ERR_TIMEOUT, "pressure loop passed its bound");
  if (s->h_st->nonfinite) return fail(STRM_ERR_NONFINITE, "norm_squared is not finite");
  return STRM_OK;
}

int strm_export_planes(strm_sim *s, float *rhs, float *p, uint8_t *flags) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_export(s->d, s->g, rhs, p, flags, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_apply_correction(strm_sim *s, const float *q, double scale) {
  if (!s || !q) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  CK(launch_apply_correction(s->d, s->g, q, scale, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_judge_correction(strm_sim *s, const float *q, double scale, int sweeps,
                          double *ns_prev, double *ns_pred, int *accepted) {
  if (!s || !q || sweeps < 0 || sweeps > 4096) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  if (!s->jd) CK(cudaMalloc(&s->jd, 4 * sizeof(double)));
  // the launches (~8 per sweep) as one graph, captured once for this q
  // buffer and sweep count (and again after the step graphs are rebuilt)
  if (!s->judge_exec || s->judge_q != q || s->judge_sweeps != sweeps) {
    if (s->judge_exec) cudaGraphExecDestroy(s->judge_exec);
    s->judge_exec = nullptr;
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t er = record_judge(s, q, sweeps);
    const cudaError_t ec = cudaStreamEndCapture(s->stream, &gr);
    cudaError_t ei = cudaSuccess;
    if (er == cudaSuccess && ec == cudaSuccess) ei = cudaGraphInstantiate(&s->judge_exec, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    CK(er);
    CK(ec);
    CK(ei);
    s->judge_q = q;
    s->judge_sweeps = sweeps;
  }
  CK(cudaMemcpyAsync(s->jd, &scale, sizeof scale, cudaMemcpyHostToDevice, s->stream));
  CK(cudaGraphLaunch(s->judge_exec, s->stream));
  double hv[3] = {0.0, 0.0, 0.0};
  CK(cudaMemcpyAsync(hv, s->jd, sizeof hv, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (ns_prev) *ns_prev = hv[1];
  if (ns_pred) *ns_pred = hv[2];
  if (accepted) *accepted = hv[2] < hv[1] ? 1 : 0;
  return STRM_OK;
}

int strm_copy_field_device(strm_sim *s, int field, double *dense, int to_sim) {
  if (!s || !dense) return fail(STRM_ERR_INVALID, "invalid arguments");
  double *f = field_ptr(s, field);
  if (!f) return fail(STRM_ERR_INVALID, "unknown field %d", field);
  CK(cudaSetDevice(s->dev));
  const Geom &g = s->g;
  if (to_sim) {
    CK(cudaMemcpy2DAsync(f, (size_t)g.pitch * 8, dense, (size_t)g.ny * 8, (size_t)g.ny * 8, g.nx,
                         cudaMemcpyDeviceToDevice, s->stream));
    // as strm_upload: new velocities refresh max|u|, max|v| for the adaptive step
    if (field == STRM_FIELD_U || field == STRM_FIELD_V)
      CK(launch_velocity(s->d, s->cfg, s->stream, 0, 0, 0));
  } else
    CK(cudaMemcpy2DAsync(dense, (size_t)g.ny * 8, f, (size_t)g.pitch * 8, (size_t)g.ny * 8, g.nx,
                         cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

// ------------------------------------------------------------------------
// Batches
// ------------------------------------------------------------------------

struct strm_batch {
  int dev = 0;
  cudaStream_t stream = nullptr;
  std::vector<strm_sim *> sims;
  int schedule = 0;     // public sweep schedule number (2..)
  int inner = 16;
  int solver = STRM_BATCH_GRAPH_LOOP;
  unsigned long long wait_limit = kDefaultWaitPolls;
  BatchPlan plan{};
  cudaGraphExec_t exec = nullptr;
  cudaGraphExec_t exec_pre = nullptr, exec_solve = nullptr;
};

namespace {

void batch_destroy_execs(strm_batch *b) {
  cudaGraphExec_t *ex[3] = {&b->exec, &b->exec_pre, &b->exec_solve};
  for (cudaGraphExec_t *e : ex) {
    if (*e) cudaGraphExecDestroy(*e);
    *e = nullptr;
  }
}

int batch_rebuild(strm_batch *b) {
  batch_destroy_execs(b);
  free_batch(&b->plan);
  std::vector<BatchMember> mem;
  for (strm_sim *s : b->sims) mem.push_back(BatchMember{s->d, s->cfg});
  cudaError_t e = build_batch(mem, b->schedule - 1, b->inner, &b->plan,
                              b->solver == STRM_BATCH_PERSISTENT, b->wait_limit);
  if (e == cudaErrorInvalidValue)
    return fail(STRM_ERR_INVALID, "a batch member has max_iterations below the inner sweeps");
  CK(e);
  CK(cudaGraphInstantiate(&b->exec, b->plan.graph, 0));
  CK(cudaGraphInstantiate(&b->exec_pre, b->plan.graph_pre, 0));
  CK(cudaGraphInstantiate(&b->exec_solve, b->plan.graph_solve, 0));
  return STRM_OK;
}

// Copies each member's state and the last n log entries to the host and
// fills stats[member * n + i].
int batch_collect(strm_batch *b, int n, strm_step_stats *stats) {
  unsigned int overrun = 0, timeout = 0;
  CK(cudaMemcpyAsync(&overrun, (char *)b->plan.state + kBatchOverrunOffset, sizeof overrun,
                     cudaMemcpyDeviceToHost, b->stream));
  CK(cudaMemcpyAsync(&timeout, (char *)b->plan.state + kBatchTimeoutOffset, sizeof timeout,
                     cudaMemcpyDeviceToHost, b->stream));
  const int ns = (int)b->sims.size();
  for (int k = 0; k < ns; ++k) {
    strm_sim *s = b->sims[k];
    CK(cudaMemcpyAsync(s->h_st, s->d.st, sizeof(StepState), cudaMemcpyDeviceToHost, b->stream));
    if (stats && n > 0)
      CK(cudaMemcpyAsync(s->h_log, s->d.log, sizeof(StepLog) * n, cudaMemcpyDeviceToHost,
                         b->stream));
    CK(cudaStreamSynchronize(b->stream));
    if (stats)
      for (int i = 0; i < n; ++i) {
        strm_step_stats &o = stats[(size_t)k * n + i];
        o.sor_iterations = s->h_log[i].sor_iters;
        o.converged = s->h_log[i].converged;
        o.norm_squared = s->h_log[i].ns;
        o.delt = s->h_log[i].dt;
      }
  }
  if (timeout)
    return fail(STRM_ERR_TIMEOUT, "a grid barrier of the persistent batch solve gave up "
                                  "waiting");
  if (overrun) return fail(STRM_ERR_TIMEOUT, "batch pressure loop passed its bound");
  for (strm_sim *s : b->sims)
    if (s->h_st->nonfinite) return fail(STRM_ERR_NONFINITE, "norm_squared is not finite");
  return STRM_OK;
}

// Orders the batch stream after the members' own streams and resets their
// step logs and the loop-overrun flag.
int batch_begin(strm_batch *b) {
  const unsigned int zero = 0;
  for (strm_sim *s : b->sims) {
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpyAsync(&s->d.st->log_pos, &zero, sizeof zero, cudaMemcpyHostToDevice, b->stream));
  }
  CK(cudaMemsetAsync((char *)b->plan.state + kBatchOverrunOffset, 0, 2 * sizeof(unsigned int),
                     b->stream));
  return STRM_OK;
}

}  // namespace

int strm_batch_create(strm_sim *const *sims, int n, int inner_sweeps, strm_batch **out) {
  if (!sims || n < 1 || !out || inner_sweeps < 0) return fail(STRM_ERR_INVALID, "invalid arguments");
  *out = nullptr;
  const int dev = sims[0] ? sims[0]->dev : 0;
  for (int i = 0; i < n; ++i) {
    strm_sim *s = sims[i];
    if (!s) return fail(STRM_ERR_INVALID, "sims[%d] is NULL", i);
    for (int j = 0; j < i; ++j)
      if (sims[j] == s) return fail(STRM_ERR_INVALID, "sims[%d] repeats sims[%d]", i, j);
    if (s->dev != dev) return fail(STRM_ERR_INVALID, "batch members must share a device");
    if (s->cfg.precision != 1 || s->cfg.sor_order != 0 || s->cfg.eager)
      return fail(STRM_ERR_INVALID, "batch members need mixed precision, red-black order and "
                                    "graph execution (sims[%d])", i);
  }
  CK(cudaSetDevice(dev));
  strm_batch *b = new strm_batch();
  b->dev = dev;
  b->sims.assign(sims, sims + n);
  b->inner = inner_sweeps > 0 ? inner_sweeps : 16;
  b->schedule = 3;  // 48 x 112 tiles, 4 sweeps per launch
  int rc = STRM_OK;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(STRM_ERR_CUDA, "cudaStreamCreate failed");
  if (rc == STRM_OK) rc = batch_rebuild(b);
  if (rc != STRM_OK) {
    strm_batch_destroy(b);
    return rc;
  }
  *out = b;
  return STRM_OK;
}

int strm_batch_destroy(strm_batch *b) {
  if (!b) return STRM_OK;
  cudaSetDevice(b->dev);
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_destroy_execs(b);
  free_batch(&b->plan);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return STRM_OK;
}

int strm_batch_set_schedule(strm_batch *b, int schedule) {
  if (!b || schedule < 2 || schedule > num_sweep_schedules())
    return fail(STRM_ERR_INVALID, "batches take the blocked schedules 2..%d",
                num_sweep_schedules());
  CK(cudaSetDevice(b->dev));
  CK(cudaStreamSynchronize(b->stream));
  b->schedule = schedule;
  return batch_rebuild(b);
}

int strm_batch_set_solver(strm_batch *b, int solver, uint64_t wait_limit) {
  if (!b || (solver != STRM_BATCH_GRAPH_LOOP && solver != STRM_BATCH_PERSISTENT))
    return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(b->dev));
  CK(cudaStreamSynchronize(b->stream));
  b->solver = solver;
  b->wait_limit = wait_limit ? (unsigned long long)wait_limit : kDefaultWaitPolls;
  return batch_rebuild(b);
}

int strm_batch_step(strm_batch *b, int n, strm_step_stats *stats) {
  if (!b || n < 0) return fail(STRM_ERR_INVALID, "invalid arguments");
  if (n > kLogCap) return fail(STRM_ERR_INVALID, "at most %d steps per call", kLogCap);
  CK(cudaSetDevice(b->dev));
  // the members' own streams may hold work (uploads, edits): order after it
  int rc = batch_begin(b);
  if (rc) return rc;
  for (int i = 0; i < n; ++i) CK(cudaGraphLaunch(b->exec, b->stream));
  return batch_collect(b, n, stats);
}

int strm_batch_prepare(strm_batch *b) {
  if (!b) return fail(STRM_ERR_INVALID, "batch is NULL");
  CK(cudaSetDevice(b->dev));
  int rc = batch_begin(b);
  if (rc) return rc;
  CK(cudaGraphLaunch(b->exec_pre, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return STRM_OK;
}

int strm_batch_solve(strm_batch *b, strm_step_stats *stats) {
  if (!b) return fail(STRM_ERR_INVALID, "batch is NULL");
  CK(cudaSetDevice(b->dev));
  // work queued on the members' streams between the halves (corrections)
  for (strm_sim *s : b->sims) CK(cudaStreamSynchronize(s->stream));
  CK(cudaGraphLaunch(b->exec_solve, b->stream));
  return batch_collect(b, 1, stats);
}

int strm_batch_autotune(strm_batch *b, int reps, int *best, double *ms_per_step) {
  if (!b || reps < 1) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(b->dev));
  // times whole batch steps under every blocked schedule on copies of the
  // members' state, then restores it: the members end where they started
  std::vector<std::vector<char>> saved(b->sims.size());
  std::vector<void *> dsave(b->sims.size(), nullptr);
  size_t k = 0;
  for (strm_sim *s : b->sims) {
    size_t bytes = 0;
    CK(cudaStreamSynchronize(s->stream));
    const size_t nfield = (size_t)s->g.nx * s->g.pitch;
    bytes = nfield * 8 * 3 + sizeof(StepState);
    CK(cudaMalloc(&dsave[k], bytes));
    char *d = (char *)dsave[k];
    CK(cudaMemcpy(d, s->d.u, nfield * 8, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(d + nfield * 8, s->d.v, nfield * 8, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(d + 2 * nfield * 8, s->d.p, nfield * 8, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(d + 3 * nfield * 8, s->d.st, sizeof(StepState), cudaMemcpyDeviceToDevice));
    ++k;
  }
  auto restore = [&]() -> cudaError_t {
    cudaError_t e = cudaSuccess;
    size_t i = 0;
    for (strm_sim *s : b->sims) {
      const size_t nfield = (size_t)s->g.nx * s->g.pitch;
      const char *d = (const char *)dsave[i++];
      if (e == cudaSuccess) e = cudaMemcpy(s->d.u, d, nfield * 8, cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(s->d.v, d + nfield * 8, nfield * 8, cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(s->d.p, d + 2 * nfield * 8, nfield * 8, cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(s->d.st, d + 3 * nfield * 8, sizeof(StepState), cudaMemcpyDeviceToDevice);
    }
    return e;
  };
  cudaEvent_t ev[2];
  cudaEventCreate(&ev[0]);
  cudaEventCreate(&ev[1]);
  int best_v = b->schedule;
  double best_t = -1.0;
  int rc = STRM_OK;
  for (int v = 2; v <= num_sweep_schedules() && rc == STRM_OK; ++v) {
    b->schedule = v;
    rc = batch_rebuild(b);
    if (rc != STRM_OK) break;
    cudaError_t e = cudaGraphLaunch(b->exec, b->stream);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], b->stream);
    for (int i = 0; i < reps && e == cudaSuccess; ++i) e = cudaGraphLaunch(b->exec, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    if (e == cudaSuccess) e = restore();
    if (e != cudaSuccess) {
      rc = fail(STRM_ERR_CUDA, "CUDA error %s", cudaGetErrorString(e));
      break;
    }
    const double per = (double)ms / reps;
    if (ms_per_step) ms_per_step[v] = per;
    if (best_t < 0.0 || per < best_t) {
      best_t = per;
      best_v = v;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  for (void *d : dsave) cudaFree(d);
  if (rc != STRM_OK) return rc;
  if (ms_per_step) ms_per_step[0] = best_t;
  if (best) *best = best_v;
  b->schedule = best_v;
  return batch_rebuild(b);
}

int strm_residual_history(strm_sim *s, double *out, int cap, int *n) {
  if (!s || !n || cap < 0 || (cap > 0 && !out)) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  int rc = sync_state(s);
  if (rc) return rc;
  const int have = (int)s->h_st->hist_n;
  *n = have;
  const int k = have < cap ? have : cap;
  if (k > 0) {
    CK(cudaMemcpyAsync(out, s->h_st->hist, sizeof(double) * 2 * (size_t)k,
                       cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  }
  return STRM_OK;
}

int strm_set_programmatic_launch(int on) { return set_fast_pdl(on); }

int strm_autotune_sweeps(strm_sim *s, int reps, int *best, double *ms_per_sweep) {
  if (!s || reps < 1) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  const int m = s->cfg.inner_sweeps;
  cudaEvent_t ev[2];
  CK(cudaEventCreate(&ev[0]));
  if (cudaEventCreate(&ev[1]) != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return fail(STRM_ERR_CUDA, "cudaEventCreate failed");
  }
  RunCfg r = s->cfg;
  int best_v = 1;
  double best_t = 0.0;
  cudaError_t e = cudaSuccess;
  for (int v = 1; v < STRM_SWEEPS_COUNT && e == cudaSuccess; ++v) {
    r.sweep_schedule = v - 1;
    e = launch_mixed_sweeps(s->d, r, s->stream, m);  // warm-up (and smem opt-in)
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], s->stream);
    for (int i = 0; i < reps && e == cudaSuccess; ++i)
      e = launch_mixed_sweeps(s->d, r, s->stream, m);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], s->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    const double per = (double)ms / ((double)reps * m);
    if (ms_per_sweep) ms_per_sweep[v] = per;
    if (e == cudaSuccess && (v == 1 || per < best_t)) {
      best_t = per;
      best_v = v;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  CK(e);
  if (ms_per_sweep) ms_per_sweep[0] = best_t;
  if (best) *best = best_v;
  s->mode.sweep_schedule = best_v;
  return rebuild_graph(s);
}

int strm_sor_sweeps(strm_sim *s, int n, double *norm_squared) {
  if (!s || n < 0) return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  if (s->cfg.precision == 1)
    CK(launch_mixed_sweeps(s->d, s->cfg, s->stream, n));
  else
    for (int i = 0; i < n; ++i) CK(launch_sor_iteration(s->d, s->cfg, s->stream));
  if (!norm_squared) return STRM_OK;
  int rc = sync_state(s);
  if (rc) return rc;
  *norm_squared = s->h_st->aux;
  return STRM_OK;
}

int strm_synchronize(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_set_u_and_v(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_velocity(s->d, s->cfg, s->stream, 1, 1, 0));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_calculate_pressure_range(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_prange(s->d, s->cfg, s->stream, 1));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_calculate_speed_range(strm_sim *s) {
  if (!s) return fail(STRM_ERR_INVALID, "sim is NULL");
  CK(cudaSetDevice(s->dev));
  CK(launch_velocity(s->d, s->cfg, s->stream, 0, 1, 0));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_render_rgba(strm_sim *s, int color_type, uint8_t *rgba) {
  if (!s || !rgba || color_type < 0 || color_type > 1)
    return fail(STRM_ERR_INVALID, "invalid arguments");
  CK(cudaSetDevice(s->dev));
  const size_t bytes = (size_t)s->g.nx * s->g.ny * 4;
  if (!s->rgba) CK(cudaMalloc(&s->rgba, bytes));
  CK(launch_render(s->d, s->g, color_type, s->rgba, s->stream));
  CK(cudaMemcpyAsync(rgba, s->rgba, bytes, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return STRM_OK;
}

int strm_device_view_get(strm_sim *s, strm_device_view *out) {
  if (!s || !out) return fail(STRM_ERR_INVALID, "invalid arguments");
  out->u = s->d.u;
  out->v = s->d.v;
  out->p = s->d.p;
  out->f = s->d.f;
  out->g = s->d.g;
  out->rhs = s->d.rhs;
  out->flags = s->d.flags;
  out->nx = s->g.nx;
  out->ny = s->g.ny;
  out->pitch = s->g.pitch;
  out->stream = (void *)s->stream;
  return STRM_OK;
}

int strm_host_classify(int nx, int ny, const uint8_t *kinds, uint8_t *edges,
                       double *fluid_cells, int64_t *bad_index) {
  if (nx < 1 || ny < 1 || !kinds || !edges) return fail(STRM_ERR_INVALID, "invalid arguments");
  for (size_t i = 0; i < (size_t)nx * ny; ++i)
    if (kinds[i] > STRM_MOVING_WALL) return fail(STRM_ERR_BAD_BOUNDARY, "unknown kind");
  long long bad = -1;
  if (!classify_host(nx, ny, kinds, edges, fluid_cells, &bad)) {
    if (bad_index) *bad_index = bad;
    return fail(STRM_ERR_THIN_WALL, "cell (%lld, %lld) has fluid on opposing sides", bad / ny,
                bad % ny);
  }
  return STRM_OK;
}

int strm_host_boundary_pass(int nx, int ny, const uint8_t *kinds, const double *wall_uv,
                            double *u, double *v, double *restore_u, double *restore_v) {
  if (nx < 1 || ny < 1 || !kinds || !u || !v || !restore_u || !restore_v)
    return fail(STRM_ERR_INVALID, "invalid arguments");
  std::vector<uint8_t> edge((size_t)nx * ny);
  long long bad = -1;
  int rc = strm_host_classify(nx, ny, kinds, edge.data(), nullptr, (int64_t *)&bad);
  if (rc) return rc;
  std::vector<double> wall(2 * (size_t)nx * ny, 0.0);
  if (wall_uv) wall.assign(wall_uv, wall_uv + 2 * (size_t)nx * ny);
  std::vector<BcEntry> prog;
  std::vector<PCopy> pc;
  compile_boundary_program(nx, ny, ny, kinds, edge.data(), wall.data(), prog, pc);
  apply_boundary_program_host(prog, u, v, restore_u, restore_v);
  return STRM_OK;
}

}  // extern "C"
