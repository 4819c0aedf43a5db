/*
 * stroemung_gpu.h — C ABI of the GB300-native NaSt2D timestep.
 *
 * Drop-in for the timestep surface of the Rust crate wickedchicken/stroemung
 * (Simulation / SimulationGrid).  All fields live on one GPU; every entry point
 * takes plain pointers and sizes and returns an int status (STRM_OK = 0).
 *
 * Host arrays are [nx][ny] row-major with y the contiguous axis and the
 * one-cell ring included, exactly like the reference's GridArray
 * (src/types.rs:12-19); nx, ny are the reference's `size`.
 *
 * Threading: one simulation per handle, each with its own CUDA stream.  Calls
 * on one handle must not overlap; distinct handles are independent.
 */
#ifndef STROEMUNG_GPU_H
#define STROEMUNG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The first two mirror SimulationGridError
 * (src/grid/mod.rs:51-59): BoundaryTooThinError -> STRM_ERR_THIN_WALL,
 * BoundaryListIncorrectError -> STRM_ERR_BAD_BOUNDARY. */
enum {
    STRM_OK = 0,
    STRM_ERR_THIN_WALL = 1,    /* a boundary cell has fluid on opposite sides */
    STRM_ERR_BAD_BOUNDARY = 2, /* a cell code outside the five known kinds */
    STRM_ERR_NONFINITE = 3,    /* the step completed but its residual is NaN/Inf */
    STRM_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up */
    STRM_ERR_CUDA = 5,         /* a CUDA runtime call failed (see strm_last_error) */
    STRM_ERR_INVALID = 6,      /* bad argument */
    STRM_ERR_NO_DEVICE = 7     /* no usable sm_103 device */
};

/* Cell kinds (src/cell.rs:6-23).  STRM_MOVING_WALL is an extension (a wall
 * whose tangential velocity is the wall's, for the lid-driven cavity). */
enum {
    STRM_FLUID = 0,
    STRM_NO_SLIP = 1,
    STRM_OUTFLOW = 2,
    STRM_INFLOW = 3,
    STRM_MOVING_WALL = 4
};

/* Fields for strm_download / strm_upload. */
enum {
    STRM_FIELD_U = 0,
    STRM_FIELD_V = 1,
    STRM_FIELD_P = 2,  /* grid.pressure */
    STRM_FIELD_F = 3,
    STRM_FIELD_G = 4,
    STRM_FIELD_RHS = 5
};

/* Pressure-solve ordering. */
enum {
    STRM_SOR_RED_BLACK = 0,    /* (x+y) even cells, then odd: all SMs */
    STRM_SOR_LEXICOGRAPHIC = 1 /* the reference's x-major Gauss-Seidel order,
                                  run as anti-diagonal wavefronts in one CTA:
                                  bit-identical to the reference, for small grids */
};

/* Arithmetic of the FP64 step.  EXACT keeps the reference's operation order
 * everywhere (bit-identical boundary pass, F/G, RHS and velocity update).
 * FAST uses fused multiply-adds and reciprocal multiplies in the pressure
 * solve, F/G/RHS as face fluxes computed once per face, and a fused velocity
 * update: those pointwise kernels stay within 1e-12 relative of the
 * reference's; the boundary pass and classification stay exact. */
enum {
    STRM_ARITH_EXACT = 0, /* reference operation order, correctly rounded divisions */
    STRM_ARITH_FAST = 1   /* fused multiply-adds and reciprocal multiplies */
};

/* Precision of the pressure solve. */
enum {
    STRM_PREC_FP64 = 0,  /* plain FP64 SOR */
    STRM_PREC_MIXED = 1  /* FP32 red-black sweeps on the FP64 defect, FP64 refinement */
};

/* How a step is issued. */
enum {
    STRM_EXEC_GRAPH = 0, /* one CUDA graph launch per step (pressure loop as a
                            conditional WHILE node) */
    STRM_EXEC_EAGER = 1  /* the same kernels launched one by one, the loop driven
                            from the host; identical results, for profilers and
                            debugging */
};

/* Stop rules of the pressure solve (strm_mode.strict_eps). */
enum {
    STRM_STOP_REFERENCE = 0, /* ns < initial_norm_squared or ns < eps^2 (src/simulation.rs:276-281) */
    STRM_STOP_STRICT = 1,    /* ns < eps^2 */
    STRM_STOP_RELATIVE = 2   /* ns < eps^2 * the solve's starting norm */
};

/* FP32 sweep schedules of the mixed solve (strm_mode.sweep_schedule). */
enum {
    STRM_SWEEPS_DEFAULT = 0,    /* 48 x 112 blocked tiles, 4 sweeps per launch */
    STRM_SWEEPS_PER_COLOUR = 1, /* one launch per colour pass */
    /* 2..7: tiles (rows x columns) kept in shared memory for several sweeps
       (temporal blocking): 56x120 by 2, 48x112 by 4, 32x96 by 8, 80x112 by
       4, 112x112 by 4, 64x96 by 8 sweeps per launch */
    STRM_SWEEPS_COUNT = 8
};

/* Which cells the residual norm sums (strm_mode.norm_cells). */
enum {
    STRM_NORM_ALL_INTERIOR = 0,   /* the reference's sum (src/simulation.rs:216-227) */
    STRM_NORM_FLUID = 1,          /* fluid cells only */
    STRM_NORM_FLUID_MEAN_FREE = 2 /* fluid cells, residual mean removed: the
                                     pressure problem is pure Neumann, so the
                                     residual's fluid sum equals -sum rhs
                                     whatever p is; this part cannot be
                                     solved away and is left out */
};

/* Mirrors Simulation's parameters (src/simulation.rs:30-69). */
typedef struct {
    double dx, dy;            /* cell_size */
    double delt;              /* time step (the first step's, when tau > 0) */
    double gamma;             /* donor-cell blend */
    double reynolds;
    double eps;               /* sor_absolute_epsilon */
    double omega;
    uint32_t max_iterations;
    uint32_t iterations;
    double time;
    double initial_norm_squared; /* NaN: computed at creation, as the
                                    reference does for `None` */
    double tau;               /* > 0: adaptive time step, delt =
                                 tau*min(Re/2/(1/dx^2+1/dy^2), dx/max|u|, dy/max|v|)
                                 (extension; 0 keeps delt fixed as the reference) */
} strm_params;

typedef struct {
    int sor_order;    /* STRM_SOR_* */
    int arithmetic;   /* STRM_ARITH_* */
    int precision;    /* STRM_PREC_* */
    int strict_eps;   /* stop rule: 0 the reference's (ns < initial norm or
                         ns < eps^2); 1 only ns < eps^2; 2 relative,
                         ns < eps^2 * (norm the solve started from, before
                         its first sweep; red-black orders) */
    int inner_sweeps; /* mixed precision: FP32 sweeps per FP64 refinement (0 = 16) */
    int execution;    /* STRM_EXEC_* */
    int norm_cells;   /* STRM_NORM_ALL_INTERIOR: the residual norm sums every
                         interior cell, obstacles included, as the reference
                         does; STRM_NORM_FLUID(_MEAN_FREE): fluid cells only
                         (extension, red-black orders) -- on grids with
                         obstacles the reference sum has a floor that the
                         solve cannot lower.  Divided by fluid_cells. */
    int sweep_schedule; /* mixed precision: how the FP32 sweeps are issued
                           (STRM_SWEEPS_*; results are identical, only the
                           speed differs; strm_autotune_sweeps picks one) */
} strm_mode;

/* Scalar state readable after any call (pressure_range / speed_range are the
 * reference's grid fields, src/grid/mod.rs:121-124). */
typedef struct {
    double time;
    uint64_t iterations;
    double delt;                  /* the time step of the last step */
    double initial_norm_squared;
    double fluid_cells;           /* reference's BoundaryList::fluid_cells */
    double pressure_range[2];
    double speed_range[2];
    uint32_t last_sor_iterations;
    double last_norm_squared;
    uint32_t last_converged;
} strm_state;

typedef struct {
    uint32_t sor_iterations;
    uint32_t converged;
    double norm_squared;
    double delt;
} strm_step_stats;

typedef struct strm_sim strm_sim;

/* Creates a simulation and runs the construction-time passes of
 * Simulation::try_from (src/simulation.rs:71-99): classification
 * (SimulationGrid::try_from, src/grid/mod.rs:127-153), F, G, RHS and the
 * initial norm.  kinds[nx*ny] are STRM_* cell kinds; wall_uv[2*nx*ny] the
 * velocity of inflow / moving-wall cells (NULL when there are none); u, v, p
 * [nx*ny].  On STRM_ERR_THIN_WALL *bad_index (if given) is the first
 * offending cell x*ny+y in x-major order and *out is NULL. */
int strm_create(const strm_params *params, int nx, int ny, const uint8_t *kinds,
                const double *wall_uv, const double *u, const double *v, const double *p,
                strm_sim **out, int64_t *bad_index);

int strm_destroy(strm_sim *sim);

/* Selects ordering / arithmetic / precision; rebuilds the step graph. */
int strm_set_mode(strm_sim *sim, const strm_mode *mode);

/* Simulation::run_simulation_tick (src/simulation.rs:324-333): boundary
 * conditions, F/G, RHS, pressure solve, velocity update; time += delt;
 * iterations += 1.  Returns (sor_iterations, norm_squared).  One CUDA graph
 * launch and one 64-byte device-to-host read. */
int strm_tick(strm_sim *sim, uint32_t *sor_iterations, double *norm_squared);

/* run_simulation_tick in two halves, so that a predictor can replace the
 * pressure the solve starts from: strm_tick_prepare does the time step,
 * boundary pass, F/G and RHS; strm_tick_solve the pressure solve, the
 * velocity update and the time bookkeeping, returning what strm_tick does. */
int strm_tick_prepare(strm_sim *sim);
int strm_tick_solve(strm_sim *sim, uint32_t *sor_iterations, double *norm_squared);

/* Device-side plumbing for a pressure predictor: dense [nx][ny] FP32 copies
 * of RHS and pressure and the flag bytes (kind | edge << 3) into device
 * buffers (any may be NULL); p += scale * q on fluid interior cells (q a
 * device FP32 [nx-2][ny-2] array); and device-to-device copies of a whole
 * FP64 field to (to_sim = 0) or from (to_sim = 1) a dense [nx][ny] buffer
 * (u or v written refresh max|u|, max|v| as strm_upload does).  Each call
 * returns with its work finished; device inputs written on other streams
 * must be complete before the call. */
int strm_export_planes(strm_sim *sim, float *rhs, float *p, uint8_t *flags);
int strm_apply_correction(strm_sim *sim, const float *q, double scale);
int strm_copy_field_device(strm_sim *sim, int field, double *dense, int to_sim);

/* Judge of a predicted pressure correction (p += scale * q on fluid interior
 * cells, q as for strm_apply_correction), between strm_tick_prepare and
 * strm_tick_solve.  sweeps = 0: the correction is kept when it lowers the
 * residual norm of the pressure (after the boundary copy).  sweeps > 0: both
 * candidates first get `sweeps` FP64 red-black iterations and their norms
 * are compared then (a prediction that removes smooth error but adds a
 * little high-frequency error has a larger raw residual, which the first
 * sweeps remove).  Either way the pressure is left at the chosen candidate
 * without the judge's sweeps, boundary copy applied; ns_prev / ns_pred
 * receive the two norms, accepted 1 when the correction was kept (each may
 * be NULL).  The judge's launches run as one CUDA graph, recorded on the
 * first call for this q buffer and sweep count (and again after a mode
 * change or a cell edit).  No reference counterpart. */
int strm_judge_correction(strm_sim *sim, const float *q, double scale, int sweeps,
                          double *ns_prev, double *ns_pred, int *accepted);

/* n ticks back to back with a single host synchronisation; stats[n] (may be
 * NULL) receives each tick's results. */
int strm_step_n(strm_sim *sim, int n, strm_step_stats *stats);

/* Reads / writes a whole field ([nx*ny] host array) — the reference's public
 * fields grid.u, grid.v, grid.pressure, f, g, rhs (src/simulation.rs:50-69).
 * Writing u or v refreshes the max|u|, max|v| used by the adaptive step. */
int strm_download(strm_sim *sim, int field, double *host);
int strm_upload(strm_sim *sim, int field, const double *host);

/* Reads the cell kinds and the edge codes (0 none, 1 N, 2 NE, 3 E, 4 SE, 5 S,
 * 6 SW, 7 W, 8 NW — EdgeType, src/grid/mod.rs:19-49) of every cell. */
int strm_download_cells(strm_sim *sim, uint8_t *kinds, uint8_t *edges);

/* The GUI's paint path (src/lib.rs:38-78) followed by rebuild_boundary_list
 * (src/grid/mod.rs:202-235): for each of the n cells (xs[i], ys[i]) whose kind
 * differs from kinds[i], zero its u, v and pressure and set the new kind (and
 * wall velocity from wall_uv[2*i], may be NULL).  If the new layout has a thin
 * wall, every change is rolled back and STRM_ERR_THIN_WALL is returned. */
int strm_edit_cells(strm_sim *sim, int n, const int32_t *xs, const int32_t *ys,
                    const uint8_t *kinds, const double *wall_uv, int64_t *bad_index);

int strm_get_state(strm_sim *sim, strm_state *out);

/* Individual phases, for callers that drive the pipeline step by step. */
int strm_set_boundary_u_and_v(strm_sim *sim);      /* src/grid/mod.rs:414-651 */
int strm_calculate_f_g_rhs(strm_sim *sim);         /* src/simulation.rs:122-214 */
int strm_copy_pressure_to_boundaries(strm_sim *sim); /* src/grid/mod.rs:343-412 */
int strm_calculate_norm_squared(strm_sim *sim, double *norm_squared); /* src/simulation.rs:216-227 */
int strm_set_u_and_v(strm_sim *sim);               /* src/simulation.rs:287-322 */
int strm_calculate_pressure_range(strm_sim *sim);  /* src/grid/mod.rs:237-251 */
int strm_calculate_speed_range(strm_sim *sim);     /* src/grid/mod.rs:253-268 */

/* n red-black pressure iterations of the loop body of solve_sor
 * (src/simulation.rs:250-277: boundary pressure copy, sweep, residual norm)
 * with no stop test, on the current pressure and RHS, in the selected
 * arithmetic.  In STRM_PREC_MIXED it runs n FP32 red-black sweeps of the
 * correction equation on the current defect instead (the inner iteration of
 * the mixed solve; norm_squared then returns the last stored norm).
 * Asynchronous when norm_squared is NULL (see strm_synchronize); otherwise
 * waits and returns the last iteration's norm. */
int strm_sor_sweeps(strm_sim *sim, int n, double *norm_squared);

/* Batches (no reference counterpart): one CUDA graph steps several
 * simulations of any sizes and parameters together.  Each member's boundary
 * pass, F/G/RHS, pressure range and velocity update run as parallel graph
 * branches; the mixed-precision pressure solves of all members run as one
 * WHILE loop of table-driven kernels (every blocked sweep launch, refinement
 * and norm covers all members still solving).  Every member ends exactly
 * where stepping it alone (strm_tick, same schedule) ends.  Members must use
 * STRM_PREC_MIXED, a red-black order and graph execution, and have
 * max_iterations >= inner_sweeps (0 = 16); they stay owned by the caller and
 * must outlive the batch; their other entry points stay usable between
 * batch steps (a mode change needs a new batch). */
typedef struct strm_batch strm_batch;
int strm_batch_create(strm_sim *const *sims, int n, int inner_sweeps, strm_batch **out);
int strm_batch_destroy(strm_batch *batch);
/* n steps of every member, one host synchronisation; stats (may be NULL)
 * receives n entries per member, member-major. */
int strm_batch_step(strm_batch *batch, int n, strm_step_stats *stats);
/* One batch step in two halves, as strm_tick_prepare / strm_tick_solve for a
 * single simulation: prepare runs every member's boundary pass, time step,
 * F/G and RHS; between the halves the members' pressures may be changed
 * (strm_judge_correction, strm_upload); solve runs the pressure solves and
 * the second halves, and stats (may be NULL) receives one entry per member.
 * prepare followed by solve gives exactly the fields of strm_batch_step. */
int strm_batch_prepare(strm_batch *batch);
int strm_batch_solve(strm_batch *batch, strm_step_stats *stats);
/* Blocked sweep schedule of the batch (2..STRM_SWEEPS_COUNT-1). */
int strm_batch_set_schedule(strm_batch *batch, int schedule);
/* How a batch step issues the members' pressure solves (no reference
 * counterpart): STRM_BATCH_GRAPH_LOOP as a WHILE loop of table-driven graph
 * kernels (the default); STRM_BATCH_PERSISTENT as one persistent cooperative
 * kernel per step whose CTAs walk the members' tile tables phase by phase,
 * with a grid barrier between phases.  Results are identical.  A barrier
 * wait gives up after wait_limit polls (0: about a second or two); the CTA
 * then flags the step, every CTA returns, and the step returns
 * STRM_ERR_TIMEOUT with the members' fields partly solved (no fault, the
 * context stays usable). */
enum {
    STRM_BATCH_GRAPH_LOOP = 0,
    STRM_BATCH_PERSISTENT = 1
};
int strm_batch_set_solver(strm_batch *batch, int solver, uint64_t wait_limit);
/* Times `reps` whole batch steps under each blocked schedule (members'
 * u, v, p and step state restored afterwards), keeps the fastest; best and
 * ms_per_step[STRM_SWEEPS_COUNT] (per schedule, [0] the best) may be NULL. */
int strm_batch_autotune(strm_batch *batch, int reps, int *best, double *ms_per_step);

/* Residual history of the last pressure solve: (sweeps done, norm_squared)
 * pairs into out[2*cap], one per norm the solve took (every iteration in
 * FP64; the starting norm and one per inner_sweeps sweeps in mixed
 * precision); *n receives how many the solve recorded (at most 65536 are
 * kept).  Synchronises.  No reference counterpart. */
int strm_residual_history(strm_sim *sim, double *out, int cap, int *n);

/* Autotuner of the FP32 sweep schedule: times inner_sweeps sweeps `reps`
 * times under every schedule on this simulation's grid and defect (the
 * correction buffer is scratch between ticks), selects the fastest into the
 * mode and rebuilds the step graph.  best (may be NULL) receives its number;
 * ms_per_sweep (may be NULL, STRM_SWEEPS_COUNT entries) the measured
 * milliseconds per sweep of schedule v at [v], the best at [0].  Results do
 * not depend on the schedule.  No reference counterpart. */
int strm_autotune_sweeps(strm_sim *sim, int reps, int *best, double *ms_per_sweep);

/* Process-wide: whether the step graphs built from now on chain the colour
 * passes of the FAST red-black loop body by programmatic dependent launch
 * (on = 1, the default) or by plain graph edges (0); a graph that a driver
 * refuses to build with them is built without them.  Results do not depend
 * on it.  Returns the previous setting.  No reference counterpart. */
int strm_set_programmatic_launch(int on);

/* Residual norm that allocates nothing.  No counterpart in the reference.
 * For callers that must not allocate device memory once they are running:
 * host frameworks whose caching allocator owns the device budget (a
 * cudaMalloc beside that pool can fail or fragment it) and fixed-footprint
 * loops that reserve all memory at start-up (cudaMalloc may synchronise the
 * device and has no latency bound).  Computes the quantity that
 * strm_calculate_norm_squared returns under the default STRM_NORM_ALL_INTERIOR
 * (sum of squared residuals over every interior cell divided by fluid_cells,
 * reference operation order; the other norm_cells modes are not offered
 * here), equal to it within rounding: the partial sums are added in another
 * order.  p and rhs are caller-owned pitched fields ([nx][pitch], y
 * contiguous); the result is written to the device double *norm_squared,
 * asynchronously on `stream` (a cudaStream_t, NULL for the default stream).
 * fluid_cells must be positive and finite.
 * Its reduction scratch is a fixed __device__ array inside this library
 * (about 130 KB, held by every GPU that loads it until the process exits):
 * grids with more than STRM_NORM_NOALLOC_MAX_TILES interior tiles of 8 x 64
 * cells are rejected with STRM_ERR_INVALID.  The first call on a device looks
 * up that array's device address (cudaGetSymbolAddress) and keeps it for the
 * life of the process; make that first call before any stream capture, and
 * do not reset the device while the library is in use.  All calls share the
 * one array and it keeps the last call's contents: calls whose GPU work
 * overlaps (different streams or threads) race and must be serialised by
 * the caller. */
#define STRM_NORM_NOALLOC_MAX_TILES 16384
int strm_norm_squared_noalloc(const double *p, const double *rhs, int nx, int ny, int pitch,
                              double dx, double dy, double fluid_cells, double *norm_squared,
                              void *stream);

/* Waits until all work queued on the simulation's stream has finished. */
int strm_synchronize(strm_sim *sim);

/* Headless colour map of render_simulation (src/visualization.rs:79-105):
 * color_type 0 pressure, 1 speed, rendered on the GPU from the current
 * fields and ranges into rgba[ny][nx][4] (host), row y = image row, as the
 * reference's macroquad Image of width nx.  No graphics API involved. */
int strm_render_rgba(strm_sim *sim, int color_type, uint8_t *rgba);

/* Device pointers of the fields (pitch in elements) for zero-copy interop. */
typedef struct {
    double *u, *v, *p, *f, *g, *rhs;
    uint8_t *flags;
    int nx, ny, pitch;
    void *stream; /* cudaStream_t */
} strm_device_view;
int strm_device_view_get(strm_sim *sim, strm_device_view *out);

/* Host-side utilities (no GPU needed).  The same classification and
 * boundary-program compiler the device path uses, run on host arrays:
 * strm_host_classify is SimulationGrid::rebuild_boundary_list's edge
 * computation (src/grid/mod.rs:202-235, 270-332); strm_host_boundary_pass
 * applies set_boundary_u_and_v (src/grid/mod.rs:414-651) to u, v in place and
 * writes, for every boundary cell with an edge, the value set_u_and_v's
 * restore replay (src/simulation.rs:313-320) leaves in u, v. */
int strm_host_classify(int nx, int ny, const uint8_t *kinds, uint8_t *edges,
                       double *fluid_cells, int64_t *bad_index);
int strm_host_boundary_pass(int nx, int ny, const uint8_t *kinds, const double *wall_uv,
                            double *u, double *v, double *restore_u, double *restore_v);

/* Last error message of the calling thread. */
int strm_last_error(char *buf, size_t len);

/* Library version, for loaders that check the ABI. */
int strm_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
