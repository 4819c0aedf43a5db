// Host-side interface between the C ABI (strm_capi.cu) and the kernels
// (strm_kernels.cu).  Nothing here is part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "strm_internal.cuh"

namespace strm {

// Solver class of an interior cell for the FAST red-black solve (cls byte,
// pitch layout): bits 0-1 the class (0 fluid with four fluid neighbours, 1
// fluid next to a non-fluid cell, 2 anything else); for class 1, bits 2-5
// say which of the west, east, north, south neighbours are copied boundary
// cells.
enum : uint8_t { CLS_FLUID = 0, CLS_FLUID_EDGE = 1, CLS_OTHER = 2 };

// A listed boundary cell of the FAST red-black solve: every non-fluid
// interior cell (its residual) and every cell of the boundary pressure copy.
enum : uint8_t { BC_RES = 1, BC_COPY = 2 };
struct BCell {
  unsigned int off;     // pitched offset
  unsigned char edge;   // the copy's EdgeType (BC_COPY)
  unsigned char flags;  // BC_RES: a non-fluid interior cell; BC_COPY: copied
  unsigned char mask;   // copied stencil points: bit 0 the cell, 1 west, 2 east,
                        // 3 north, 4 south
  unsigned char pad;
};

// Device buffers of one simulation.
struct DevFields {
  double *u, *v, *p, *f, *g, *rhs;
  double *ru, *rv;        // restore values of boundary cells (per cell)
  uint8_t *flags;
  // mixed-precision pressure solve
  float *e32, *r32;       // FP32 correction and defect
  float *e32b;            // second correction buffer (temporal-blocked sweeps)
  double *pw;             // FP64 work field
  StepState *st;
  double *partials;       // per-CTA residual partial sums
  int n_partials;
  double *partials_b;     // per-CTA sums of the fused black pass (2 per block)
  StepLog *log;
  BcEntry *bc;            // compiled boundary program
  double *bc_val;         // its gathered values
  int n_bc;
  PCopy *pcopy;
  int n_pcopy;
  // FAST red-black solve: solver class per cell (CLS_*), the boundary-cell
  // list (black-coloured cells first), the red pass's partial sums
  uint8_t *cls;
  BCell *blist;
  int n_blist;
  int n_blist_b;
  double *partials_r;
  long long *first_bad;   // classification: first thin-wall cell (x*ny+y)
  unsigned long long *fluid_count;
};

struct RunCfg {
  Geom g;
  Consts c;
  double tau;             // > 0: adaptive time step
  double delt;            // fixed time step when tau <= 0
  unsigned int itermax;
  int strict_eps;
  int sor_order;          // 0 red-black, 1 lexicographic
  int arith;              // 0 exact, 1 fast
  int precision;          // 0 fp64, 1 mixed
  int inner_sweeps;
  int sweep_schedule;     // FP32 sweep schedule (0 per-colour launches, 1.. blocked tiles)
  int eager;              // 1: launch kernels one by one instead of the graph
};

// Standalone launches (phase entry points, creation).
cudaError_t launch_classify(const DevFields &d, const Geom &g, cudaStream_t s);
cudaError_t launch_step_begin(const DevFields &d, const RunCfg &r, cudaStream_t s);
cudaError_t launch_bc(const DevFields &d, cudaStream_t s);
cudaError_t launch_fg_rhs(const DevFields &d, const RunCfg &r, cudaStream_t s);
cudaError_t launch_pcopy(const DevFields &d, const Geom &g, cudaStream_t s);
cudaError_t launch_norm(const DevFields &d, const RunCfg &r, cudaStream_t s, int set_ns0);
cudaError_t launch_velocity(const DevFields &d, const RunCfg &r, cudaStream_t s, int update,
                            int commit_speed, int advance);
cudaError_t launch_prange(const DevFields &d, const RunCfg &r, cudaStream_t s, int force);
cudaError_t launch_sor_lex(const DevFields &d, const RunCfg &r, cudaStream_t s);
// One red-black pressure iteration (copy, red, black, residual) without a
// stop test; norm = 0 leaves the residual norm out.
cudaError_t launch_sor_iteration(const DevFields &d, const RunCfg &r, cudaStream_t s,
                                 int norm = 1);
// n FP32 red-black sweeps of the correction equation on the current defect
// (the inner iteration of the mixed solve), by the configured schedule.
cudaError_t launch_mixed_sweeps(const DevFields &d, const RunCfg &r, cudaStream_t s, int n);
int num_sweep_schedules();

// Colour map into a device RGBA8 image [ny][nx] (0 pressure, 1 speed).
cudaError_t launch_render(const DevFields &d, const Geom &g, int color_type, void *rgba,
                          cudaStream_t s);

// One step with every kernel launched eagerly and the pressure loop driven
// from the host; h is pinned host memory for the polled flags.
cudaError_t run_step_eager(const DevFields &d, const RunCfg &r, cudaStream_t s, StepState *h);

// Builds the whole step as one CUDA graph (the pressure loop as a
// conditional WHILE node for the red-black solve).
// part 0: the whole step; 1: up to the RHS; 2: from the pressure solve on.
cudaError_t build_step_graph(const DevFields &d, const RunCfg &r, cudaGraph_t *out, int part);
// programmatic edges between the FAST loop body's colour passes in the
// graphs built from now on; returns the previous setting
int set_fast_pdl(int on);
int fast_pdl();

// Dense FP32 copies ([nx][ny]) of RHS and pressure and the flag bytes (any
// output may be NULL); p += scale*q on fluid interior cells, q [nx-2][ny-2]
// (with jd, device [scale, norm without, norm with]: the scale from jd[0],
// and when cond only if jd[2] < jd[1]).
cudaError_t launch_export(const DevFields &d, const Geom &g, float *rhs32, float *p32,
                          uint8_t *fl8, cudaStream_t s);
cudaError_t launch_apply_correction(const DevFields &d, const Geom &g, const float *q,
                                    double scale, cudaStream_t s, const double *jd = nullptr,
                                    int cond = 0);

int residual_blocks(const Geom &g);
// Blocks of the fused black pass of the FAST FP64 solve (2 partials each).
int black_pass_blocks(const Geom &g);

// Residual norm of raw pitched fields with one block per 8x64 tile of the
// interior: partials[] must hold interior_tiles(g) doubles; st->fluid_cells
// must be set and st->counter zero; the norm lands in st->aux.
int interior_tiles(const Geom &g);
cudaError_t launch_norm_one_block_per_tile(const double *p, const double *rhs, const Geom &g,
                                           const Consts &c, StepState *st, double *partials,
                                           cudaStream_t s);


// Batches (strm_batch_*): one graph steps many simulations; their pressure
// solves share one WHILE loop of table-driven kernels.
struct BatchMember {
  DevFields d;
  RunCfg r;
};
struct BatchState;
struct BatchPlan {
  void *dev = nullptr;          // device tables (one allocation)
  BatchState *state = nullptr;  // in dev: loop counters and the overrun flag
  int persist_grid = 0;         // CTAs of the persistent solve (0: graph loop)
  cudaGraph_t graph = nullptr;        // the whole step
  cudaGraph_t graph_pre = nullptr;    // the members' boundary pass, F/G, RHS
  cudaGraph_t graph_solve = nullptr;  // the pressure solves and the second halves
};
// sched: internal blocked schedule (1..num_sweep_schedules()-1); m: sweeps
// per refinement (every member needs max_iterations >= m).  persistent: the
// pressure solves run as one cooperative kernel whose grid barriers give up
// after wait_limit polls (otherwise as a WHILE loop of graph kernels).
cudaError_t build_batch(const std::vector<BatchMember> &mem, int sched, int m, BatchPlan *bp,
                        int persistent = 0, unsigned long long wait_limit = 0);
void free_batch(BatchPlan *bp);
// Offsets in bytes of BatchState::overrun and ::timeout (the host reads them
// after steps).
constexpr size_t kBatchOverrunOffset = 12 * sizeof(unsigned int);
constexpr size_t kBatchTimeoutOffset = 13 * sizeof(unsigned int);

}  // namespace strm
