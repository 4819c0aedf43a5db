/*
 * CPU oracle for the stroemung NaSt2D timestep — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP64 restatement of the reference solver's per-timestep pipeline
 * (src/math.rs, src/simulation.rs, src/grid/mod.rs of wickedchicken/stroemung)
 * with the reference's operation order and loop order, compiled with
 * -ffp-contract=off so that no multiply-add is fused (Rust does not contract).
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of bench.py
 * may call into this library.  The product path (stroemung_gb300) never
 * links, loads or falls back to it.
 *
 * Parity is pinned: the known-answer tests of src/math.rs:192-402 and
 * src/simulation.rs:449-569, the classification tests of
 * src/grid/mod.rs:683-801 and the tick snapshots of src/simulation.rs:571-618
 * are reproduced bit for bit (tests/test_oracle_golden.py).
 *
 * Layout: every field is [nx][ny] row-major, y the contiguous axis, exactly
 * like the reference's ndarray GridArray (src/types.rs:12-19); (0,0) is the
 * upper-left corner and "north" is y-1 (src/grid/mod.rs:168-170).
 */
#ifndef STROEMUNG_ORACLE_H
#define STROEMUNG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Cell kinds (src/cell.rs:6-23); ORC_MOVING_WALL is an extension used by the
 * lid-driven cavity, it has no reference counterpart. */
enum {
    ORC_FLUID = 0,
    ORC_NO_SLIP = 1,
    ORC_OUTFLOW = 2,
    ORC_INFLOW = 3,
    ORC_MOVING_WALL = 4
};

/* Edge codes, in the declaration order of EdgeType (src/grid/mod.rs:19-49). */
enum {
    ORC_EDGE_NONE = 0,
    ORC_EDGE_N = 1,
    ORC_EDGE_NE = 2,
    ORC_EDGE_E = 3,
    ORC_EDGE_SE = 4,
    ORC_EDGE_S = 5,
    ORC_EDGE_SW = 6,
    ORC_EDGE_W = 7,
    ORC_EDGE_NW = 8
};

/* Pressure-solve orderings. */
enum {
    ORC_SOR_LEXICOGRAPHIC = 0, /* the reference's Gauss-Seidel order */
    ORC_SOR_RED_BLACK = 1      /* (x+y) even first, then odd */
};

typedef struct orc_sim orc_sim;

typedef struct {
    int nx, ny;                    /* size, ring included */
    double dx, dy;                 /* cell_size */
    double delt, gamma, reynolds;
    double eps;                    /* sor_absolute_epsilon */
    double omega;
    uint32_t max_iterations;
    uint32_t iterations;
    double time;
    double initial_norm_squared;   /* used when has_initial_norm != 0 */
    int has_initial_norm;
    double tau;                    /* > 0: adaptive time step (extension) */
    int sor_order;                 /* ORC_SOR_* */
    int strict_eps;                /* 1: stop only when ns < eps^2 */
} orc_params;

/* ---- stencil primitives on 3x3 windows w[a*3+b] = f[i-1+a][j-1+b] ---- */
double orc_du2dx(const double *u, double delx, double gamma);
double orc_duvdx(const double *u, const double *v, double delx, double gamma);
double orc_duvdy(const double *u, const double *v, double dely, double gamma);
double orc_dv2dy(const double *v, double dely, double gamma);
double orc_laplacian(const double *e, double delx, double dely);
double orc_residual(const double *p, double delx, double dely, double rhs);
double orc_calculate_f(const double *u, const double *v, double delx, double dely,
                       double delt, double gamma, double reynolds);
double orc_calculate_g(const double *u, const double *v, double delx, double dely,
                       double delt, double gamma, double reynolds);

/* ---- classification ---- */
/* Fills edge[nx*ny] (ORC_EDGE_*; 0 for fluid cells) and *fluid_cells.
 * Returns 0, or 1 for "fluid on opposing sides" with *bad_index set to the
 * first offending cell in x-major order (x*ny+y). */
int orc_classify(int nx, int ny, const uint8_t *kind, uint8_t *edge,
                 double *fluid_cells, int64_t *bad_index);

/* ---- simulation ---- */
/* kind[nx*ny]; wall_uv[2*nx*ny] holds the velocity of inflow / moving-wall
 * cells (may be NULL when there are none); u, v, p are copied in.
 * Returns NULL and sets *status (1 = thin wall) on failure. */
orc_sim *orc_create(const orc_params *prm, const uint8_t *kind, const double *wall_uv,
                    const double *u, const double *v, const double *p, int *status,
                    int64_t *bad_index);
void orc_destroy(orc_sim *s);
void orc_tick(orc_sim *s, uint32_t *sor_iterations, double *norm_squared);
/* Whole-field accessors: which = 0 u, 1 v, 2 p, 3 f, 4 g, 5 rhs. */
void orc_get_field(const orc_sim *s, int which, double *out);
void orc_set_field(orc_sim *s, int which, const double *in);
void orc_get_edges(const orc_sim *s, uint8_t *out);
void orc_get_state(const orc_sim *s, double *out8);
/* out8 = {time, iterations, initial_norm_squared, delt, p_min, p_max, s_min, s_max} */

/* The individual phases, for phase-level parity tests. */
void orc_set_boundary_u_and_v(orc_sim *s);
void orc_calculate_f_and_g(orc_sim *s);
void orc_calculate_rhs(orc_sim *s);
void orc_copy_pressure_to_boundaries(orc_sim *s);
double orc_calculate_norm_squared(const orc_sim *s);
void orc_solve_sor(orc_sim *s, uint32_t *iters, double *ns);
void orc_set_u_and_v(orc_sim *s);
void orc_adapt_dt(orc_sim *s);
void orc_calculate_pressure_range(orc_sim *s);
void orc_calculate_speed_range(orc_sim *s);
/* Colour map of src/visualization.rs:79-105 into rgba[ny][nx][4]
 * (0 pressure, 1 speed). */
void orc_render(const orc_sim *s, int color_type, uint8_t *rgba);
/* A tick with its phases timed, for the CPU baseline (see the .c file). */
void orc_tick_timed(orc_sim *s, uint32_t max_iterations_cap, double *out4);
/* Threads of the red-black sweeps and the norm (1 = serial, the default). */
void orc_set_threads(orc_sim *s, int threads);

#ifdef __cplusplus
}
#endif
#endif
