/*
 * CPU oracle for the stroemung NaSt2D timestep — TEST INFRASTRUCTURE ONLY.
 * See stroemung_oracle.h for the contract.  Every routine cites the reference
 * function it restates (paths relative to the wickedchicken/stroemung tree).
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (oracle/Makefile).  The
 * contract flag matters: the reference is Rust, which never fuses a*b+c, so
 * fusing here would change the last bit of F, G, RHS, p and u/v.
 */
#define _POSIX_C_SOURCE 199309L
#include "stroemung_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* Rust's x.powi(2) lowers to x*x. */
static inline double sq(double x) { return x * x; }

/* ------------------------------------------------------------------ */
/* Stencil primitives, src/math.rs                                    */
/* ------------------------------------------------------------------ */

/* src/math.rs:19-33 */
static inline double du2dx_s(double u_im1, double u_i, double u_ip1, double delx,
                             double gamma) {
    double inner_left1 = sq(u_i + u_ip1);
    double inner_right1 = sq(u_im1 + u_i);
    double left_side = inner_left1 - inner_right1;
    double inner_left2 = fabs(u_i + u_ip1) * (u_i - u_ip1);
    double inner_right2 = fabs(u_im1 + u_i) * (u_im1 - u_i);
    return (left_side + (gamma * (inner_left2 - inner_right2))) / (4.0 * delx);
}

/* src/math.rs:53-77 */
static inline double duvdx_s(double u_i_j, double u_i_j_p1, double u_i_m1_j,
                             double u_i_m1_j_p1, double v_i_j, double v_i_p1_j,
                             double v_i_m1_j, double delx, double gamma) {
    double inner_left1 = (u_i_j + u_i_j_p1) * (v_i_j + v_i_p1_j);
    double inner_right1 = (u_i_m1_j + u_i_m1_j_p1) * (v_i_m1_j + v_i_j);
    double left_side = inner_left1 - inner_right1;
    double inner_left2 = fabs(u_i_j + u_i_j_p1) * (v_i_j - v_i_p1_j);
    double inner_right2 = fabs(u_i_m1_j + u_i_m1_j_p1) * (v_i_m1_j - v_i_j);
    return (left_side + (gamma * (inner_left2 - inner_right2))) / (4.0 * delx);
}

/* src/math.rs:97-120 */
static inline double duvdy_s(double u_i_j, double u_i_j_m1, double u_i_j_p1,
                             double v_i_j, double v_i_j_m1, double v_i_p1_j,
                             double v_i_p1_j_m1, double dely, double gamma) {
    double inner_left1 = (v_i_j + v_i_p1_j) * (u_i_j + u_i_j_p1);
    double inner_right1 = (v_i_j_m1 + v_i_p1_j_m1) * (u_i_j_m1 + u_i_j);
    double left_side = inner_left1 - inner_right1;
    double inner_left2 = fabs(v_i_j + v_i_p1_j) * (u_i_j - u_i_j_p1);
    double inner_right2 = fabs(v_i_j_m1 + v_i_p1_j_m1) * (u_i_j_m1 - u_i_j);
    return (left_side + (gamma * (inner_left2 - inner_right2))) / (4.0 * dely);
}

/* src/math.rs:136-150 */
static inline double dv2dy_s(double v_i_j_m1, double v_i_j, double v_i_j_p1,
                             double dely, double gamma) {
    double inner_left1 = sq(v_i_j + v_i_j_p1);
    double inner_right1 = sq(v_i_j_m1 + v_i_j);
    double left_side = inner_left1 - inner_right1;
    double inner_left2 = fabs(v_i_j + v_i_j_p1) * (v_i_j - v_i_j_p1);
    double inner_right2 = fabs(v_i_j_m1 + v_i_j) * (v_i_j_m1 - v_i_j);
    return (left_side + (gamma * (inner_left2 - inner_right2))) / (4.0 * dely);
}

/* src/math.rs:162-174 */
static inline double laplacian_s(double e_i_j, double e_i_j_m1, double e_i_j_p1,
                                 double e_i_m1_j, double e_i_p1_j, double delx,
                                 double dely) {
    double d2edx2 = (e_i_p1_j - (2. * e_i_j) + e_i_m1_j) / sq(delx);
    double d2edy2 = (e_i_j_p1 - (2. * e_i_j) + e_i_j_m1) / sq(dely);
    return d2edx2 + d2edy2;
}

/* src/math.rs:176-186 */
static inline double residual_s(double p_i_p1_j, double p_i_j, double p_i_m1_j,
                                double p_i_j_p1, double p_i_j_m1, double delx,
                                double dely, double rhs) {
    double part1 = ((p_i_p1_j - p_i_j) - (p_i_j - p_i_m1_j)) / sq(delx);
    double part2 = ((p_i_j_p1 - p_i_j) - (p_i_j - p_i_j_m1)) / sq(dely);
    return part1 + part2 - rhs;
}

/* src/simulation.rs:349-363 on the 3x3 windows of u and v at (i, j). */
static inline double calc_f_s(double u00, double u01, double u02, double u10,
                              double u11, double u12, double u20, double u21,
                              double v10, double v11, double v20, double v21,
                              double delx, double dely, double delt, double gamma,
                              double reynolds) {
    (void)u00; (void)u02; (void)u20;
    double lap = laplacian_s(u11, u10, u12, u01, u21, delx, dely);
    double a = du2dx_s(u01, u11, u21, delx, gamma);
    double b = duvdy_s(u11, u10, u12, v11, v10, v21, v20, dely, gamma);
    return u11 + (delt * ((lap / reynolds) - a - b));
}

/* src/simulation.rs:378-392 */
static inline double calc_g_s(double u01, double u02, double u11, double u12,
                              double v01, double v10, double v11, double v12,
                              double v21, double delx, double dely, double delt,
                              double gamma, double reynolds) {
    double lap = laplacian_s(v11, v10, v12, v01, v21, delx, dely);
    double a = duvdx_s(u11, u12, u01, u02, v11, v21, v01, delx, gamma);
    double b = dv2dy_s(v10, v11, v12, dely, gamma);
    return v11 + (delt * ((lap / reynolds) - a - b));
}

double orc_du2dx(const double *u, double delx, double gamma) {
    return du2dx_s(u[1], u[4], u[7], delx, gamma);
}
double orc_duvdx(const double *u, const double *v, double delx, double gamma) {
    return duvdx_s(u[4], u[5], u[1], u[2], v[4], v[7], v[1], delx, gamma);
}
double orc_duvdy(const double *u, const double *v, double dely, double gamma) {
    return duvdy_s(u[4], u[3], u[5], v[4], v[3], v[7], v[6], dely, gamma);
}
double orc_dv2dy(const double *v, double dely, double gamma) {
    return dv2dy_s(v[3], v[4], v[5], dely, gamma);
}
double orc_laplacian(const double *e, double delx, double dely) {
    return laplacian_s(e[4], e[3], e[5], e[1], e[7], delx, dely);
}
double orc_residual(const double *p, double delx, double dely, double rhs) {
    return residual_s(p[7], p[4], p[1], p[5], p[3], delx, dely, rhs);
}
double orc_calculate_f(const double *u, const double *v, double delx, double dely,
                       double delt, double gamma, double reynolds) {
    return calc_f_s(u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7], v[3], v[4], v[6],
                    v[7], delx, dely, delt, gamma, reynolds);
}
double orc_calculate_g(const double *u, const double *v, double delx, double dely,
                       double delt, double gamma, double reynolds) {
    return calc_g_s(u[1], u[2], u[4], u[5], v[1], v[3], v[4], v[5], v[7], delx, dely,
                    delt, gamma, reynolds);
}

/* ------------------------------------------------------------------ */
/* Grid: classification, src/grid/mod.rs:167-332                      */
/* ------------------------------------------------------------------ */

/* src/grid/mod.rs:270-332: which 4-neighbours are fluid decides the edge;
 * fluid on opposite sides is an error.  The neighbour test of
 * src/grid/mod.rs:167-200 treats cells outside the grid as "not fluid". */
static int edge_of(int nx, int ny, const uint8_t *kind, int x, int y, uint8_t *edge) {
    int left = x > 0 && kind[(size_t)(x - 1) * ny + y] == ORC_FLUID;
    int right = x < nx - 1 && kind[(size_t)(x + 1) * ny + y] == ORC_FLUID;
    int up = y > 0 && kind[(size_t)x * ny + (y - 1)] == ORC_FLUID;
    int down = y < ny - 1 && kind[(size_t)x * ny + (y + 1)] == ORC_FLUID;
    int code = (left << 3) | (right << 2) | (up << 1) | down;
    switch (code) {
    case 0x0: *edge = ORC_EDGE_NONE; return 0;
    case 0x8: *edge = ORC_EDGE_W; return 0;
    case 0xA: *edge = ORC_EDGE_NW; return 0;
    case 0x2: *edge = ORC_EDGE_N; return 0;
    case 0x6: *edge = ORC_EDGE_NE; return 0;
    case 0x4: *edge = ORC_EDGE_E; return 0;
    case 0x5: *edge = ORC_EDGE_SE; return 0;
    case 0x1: *edge = ORC_EDGE_S; return 0;
    case 0x9: *edge = ORC_EDGE_SW; return 0;
    default: return 1;
    }
}

/* src/grid/mod.rs:202-235: boundary cells in x-major (BTreeSet) order; the
 * first error in that order wins; fluid_cells counts every non-boundary cell. */
int orc_classify(int nx, int ny, const uint8_t *kind, uint8_t *edge,
                 double *fluid_cells, int64_t *bad_index) {
    int64_t fluid = 0;
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            size_t i = (size_t)x * ny + y;
            edge[i] = 0;
            if (kind[i] == ORC_FLUID) fluid++;
        }
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            size_t i = (size_t)x * ny + y;
            if (kind[i] == ORC_FLUID) continue;
            if (edge_of(nx, ny, kind, x, y, &edge[i])) {
                if (bad_index) *bad_index = (int64_t)i;
                return 1;
            }
        }
    if (fluid_cells) *fluid_cells = (double)fluid;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Simulation state                                                   */
/* ------------------------------------------------------------------ */

typedef struct {
    int64_t idx;
    int has_u, has_v;
    double u, v;
} restore_t;

struct orc_sim {
    orc_params prm;
    int nx, ny;
    double *u, *v, *p, *f, *g, *rhs;
    uint8_t *kind, *edge;
    double *wall;          /* 2 per cell */
    int64_t *bnd;          /* boundary indices, x-major */
    int64_t nbnd;
    double fluid_cells;
    restore_t *restore;    /* u_v_restore, src/grid/mod.rs:68 */
    int64_t nrestore;
    double pressure_range[2], speed_range[2];
    int threads;           /* > 1: red-black sweeps and norm on that many threads */
};

#define AT(a, x, y) (a)[(size_t)(x) * ny + (y)]

/* src/grid/mod.rs:237-251 (note the max starts at 0.0) */
void orc_calculate_pressure_range(orc_sim *s) {
    double mn = DBL_MAX, mx = 0.0;
    size_t n = (size_t)s->nx * s->ny;
    for (size_t i = 0; i < n; i++)
        if (s->kind[i] == ORC_FLUID) {
            mn = fmin(mn, s->p[i]);
            mx = fmax(mx, s->p[i]);
        }
    s->pressure_range[0] = mn;
    s->pressure_range[1] = mx;
}

/* src/grid/mod.rs:253-268 */
void orc_calculate_speed_range(orc_sim *s) {
    double mn = DBL_MAX, mx = 0.0;
    size_t n = (size_t)s->nx * s->ny;
    for (size_t i = 0; i < n; i++)
        if (s->kind[i] == ORC_FLUID) {
            double s2 = sq(s->u[i]) + sq(s->v[i]);
            mn = fmin(mn, s2);
            mx = fmax(mx, s2);
        }
    s->speed_range[0] = sqrt(mn);
    s->speed_range[1] = sqrt(mx);
}

/* src/simulation.rs:122-202 */
void orc_calculate_f_and_g(orc_sim *s) {
    const int nx = s->nx, ny = s->ny;
    const double dx = s->prm.dx, dy = s->prm.dy, dt = s->prm.delt;
    const double gm = s->prm.gamma, re = s->prm.reynolds;
    double *u = s->u, *v = s->v;
    for (int x = 1; x < nx - 1; x++)
        for (int y = 1; y < ny - 1; y++) {
            AT(s->f, x, y) = calc_f_s(AT(u, x - 1, y - 1), AT(u, x - 1, y), AT(u, x - 1, y + 1),
                                      AT(u, x, y - 1), AT(u, x, y), AT(u, x, y + 1),
                                      AT(u, x + 1, y - 1), AT(u, x + 1, y), AT(v, x, y - 1),
                                      AT(v, x, y), AT(v, x + 1, y - 1), AT(v, x + 1, y), dx,
                                      dy, dt, gm, re);
            AT(s->g, x, y) = calc_g_s(AT(u, x - 1, y), AT(u, x - 1, y + 1), AT(u, x, y),
                                      AT(u, x, y + 1), AT(v, x - 1, y), AT(v, x, y - 1),
                                      AT(v, x, y), AT(v, x, y + 1), AT(v, x + 1, y), dx, dy,
                                      dt, gm, re);
        }
    /* restore F and G on boundary cells and on the fluid cells west / north
     * of West- and North-facing edges (src/simulation.rs:167-201) */
    for (int64_t k = 0; k < s->nbnd; k++) {
        int64_t b = s->bnd[k];
        int x = (int)(b / ny), y = (int)(b % ny);
        s->f[b] = u[b];
        s->g[b] = v[b];
        switch (s->edge[b]) {
        case ORC_EDGE_N: AT(s->g, x, y - 1) = AT(v, x, y - 1); break;
        case ORC_EDGE_NW:
            AT(s->f, x - 1, y) = AT(u, x - 1, y);
            AT(s->g, x, y - 1) = AT(v, x, y - 1);
            break;
        case ORC_EDGE_W: AT(s->f, x - 1, y) = AT(u, x - 1, y); break;
        case ORC_EDGE_SW: AT(s->f, x - 1, y) = AT(u, x - 1, y); break;
        case ORC_EDGE_NE: AT(s->g, x, y - 1) = AT(v, x, y - 1); break;
        default: break;
        }
    }
}

/* src/simulation.rs:204-214 — over [1..nx, 1..ny], ring included */
void orc_calculate_rhs(orc_sim *s) {
    const int nx = s->nx, ny = s->ny;
    const double dx = s->prm.dx, dy = s->prm.dy, dt = s->prm.delt;
    for (int x = 1; x < nx; x++)
        for (int y = 1; y < ny; y++)
            AT(s->rhs, x, y) = (((AT(s->f, x, y) - AT(s->f, x - 1, y)) / dx) +
                                ((AT(s->g, x, y) - AT(s->g, x, y - 1)) / dy)) /
                               dt;
}

/* src/simulation.rs:216-227 — every interior cell, divided by fluid_cells */
double orc_calculate_norm_squared(const orc_sim *s) {
    const int nx = s->nx, ny = s->ny;
    const double dx = s->prm.dx, dy = s->prm.dy;
    const double *p = s->p;
    double acc = 0.0;
#ifdef _OPENMP
    if (s->threads > 1) {
        /* timing only: the threads' partial sums are added in another order */
#pragma omp parallel for schedule(static) num_threads(s->threads) reduction(+ : acc)
        for (int x = 1; x < nx - 1; x++)
            for (int y = 1; y < ny - 1; y++)
                acc = acc + sq(residual_s(AT(p, x + 1, y), AT(p, x, y), AT(p, x - 1, y),
                                          AT(p, x, y + 1), AT(p, x, y - 1), dx, dy,
                                          AT(s->rhs, x, y)));
        return acc / s->fluid_cells;
    }
#endif
    for (int x = 1; x < nx - 1; x++)
        for (int y = 1; y < ny - 1; y++)
            acc = acc + sq(residual_s(AT(p, x + 1, y), AT(p, x, y), AT(p, x - 1, y),
                                      AT(p, x, y + 1), AT(p, x, y - 1), dx, dy,
                                      AT(s->rhs, x, y)));
    return acc / s->fluid_cells;
}

/* src/grid/mod.rs:343-412 */
void orc_copy_pressure_to_boundaries(orc_sim *s) {
    const int ny = s->ny;
    double *p = s->p;
    for (int64_t k = 0; k < s->nbnd; k++) {
        int64_t b = s->bnd[k];
        int x = (int)(b / ny), y = (int)(b % ny);
        switch (s->edge[b]) {
        case ORC_EDGE_N: p[b] = AT(p, x, y - 1); break;
        case ORC_EDGE_NE: p[b] = (AT(p, x, y - 1) + AT(p, x + 1, y)) / 2.0; break;
        case ORC_EDGE_E: p[b] = AT(p, x + 1, y); break;
        case ORC_EDGE_SE: p[b] = (AT(p, x, y + 1) + AT(p, x + 1, y)) / 2.0; break;
        case ORC_EDGE_S: p[b] = AT(p, x, y + 1); break;
        case ORC_EDGE_SW: p[b] = (AT(p, x, y + 1) + AT(p, x - 1, y)) / 2.0; break;
        case ORC_EDGE_W: p[b] = AT(p, x - 1, y); break;
        case ORC_EDGE_NW: p[b] = (AT(p, x, y - 1) + AT(p, x - 1, y)) / 2.0; break;
        default: break;
        }
    }
}

static void push_restore(orc_sim *s, int64_t idx, int has_u, double u, int has_v,
                         double v) {
    restore_t *r = &s->restore[s->nrestore++];
    r->idx = idx;
    r->has_u = has_u;
    r->u = u;
    r->has_v = has_v;
    r->v = v;
}

/* src/grid/mod.rs:414-651.  The moving wall is the no-slip rule with the
 * wall's velocity (Uw, Vw): face-normal components take the wall value and
 * mirrored tangential components become 2W - (fluid neighbour). */
void orc_set_boundary_u_and_v(orc_sim *s) {
    const int ny = s->ny;
    double *u = s->u, *v = s->v;
    s->nrestore = 0;
    for (int64_t k = 0; k < s->nbnd; k++) {
        int64_t b = s->bnd[k];
        int x = (int)(b / ny), y = (int)(b % ny);
        int e = s->edge[b];
        if (e == ORC_EDGE_NONE) {
            push_restore(s, b, 1, u[b], 1, v[b]);
            continue;
        }
        int64_t n = (int64_t)x * ny + (y - 1), so = (int64_t)x * ny + (y + 1);
        int64_t ea = (int64_t)(x + 1) * ny + y, w = (int64_t)(x - 1) * ny + y;
        int kd = s->kind[b];
        if (kd == ORC_NO_SLIP || kd == ORC_INFLOW || kd == ORC_MOVING_WALL) {
            double bu = 0.0, bv = 0.0;
            if (kd != ORC_NO_SLIP) {
                bu = s->wall[2 * b];
                bv = s->wall[2 * b + 1];
            }
            /* mirror(a) = -a for no-slip / inflow, 2W - a for a moving wall */
#define MIR_U(a) (kd == ORC_MOVING_WALL ? (2.0 * bu) - (a) : -(a))
#define MIR_V(a) (kd == ORC_MOVING_WALL ? (2.0 * bv) - (a) : -(a))
            switch (e) {
            case ORC_EDGE_N: u[b] = MIR_U(u[n]); v[n] = bv; break;
            case ORC_EDGE_NE: u[b] = bu; v[n] = bv; v[b] = MIR_V(v[ea]); break;
            case ORC_EDGE_E: u[b] = bu; v[b] = MIR_V(v[ea]); break;
            case ORC_EDGE_SE: u[b] = bu; v[b] = bv; break;
            case ORC_EDGE_S: u[b] = MIR_U(u[so]); v[b] = bv; break;
            case ORC_EDGE_SW: u[w] = bu; u[b] = MIR_U(u[so]); v[b] = bv; break;
            case ORC_EDGE_W: u[w] = bu; v[b] = MIR_V(v[w]); break;
            case ORC_EDGE_NW:
                u[w] = bu;
                u[b] = MIR_U(u[n]);
                v[n] = bv;
                v[b] = MIR_V(v[w]);
                break;
            }
#undef MIR_U
#undef MIR_V
        } else { /* outflow: src/grid/mod.rs:489-536 */
            switch (e) {
            case ORC_EDGE_N: u[b] = u[n]; v[b] = v[n]; break;
            case ORC_EDGE_NE: u[b] = u[n]; v[b] = v[ea]; break;
            case ORC_EDGE_E: u[b] = u[ea]; v[b] = v[ea]; break;
            case ORC_EDGE_SE: u[b] = u[ea]; v[b] = v[so]; break;
            case ORC_EDGE_S: u[b] = u[so]; v[b] = v[so]; break;
            case ORC_EDGE_SW: u[b] = u[w]; v[b] = v[so]; break;
            case ORC_EDGE_W: u[b] = u[w]; v[b] = v[w]; break;
            case ORC_EDGE_NW: u[b] = u[n]; v[b] = v[w]; break;
            }
        }
        push_restore(s, b, 1, u[b], 1, v[b]);
        /* src/grid/mod.rs:602-648: keyed at b, valued at the neighbour */
        switch (e) {
        case ORC_EDGE_N: push_restore(s, b, 0, 0.0, 1, v[n]); break;
        case ORC_EDGE_NE: push_restore(s, b, 0, 0.0, 1, v[n]); break;
        case ORC_EDGE_SW: push_restore(s, b, 1, u[w], 0, 0.0); break;
        case ORC_EDGE_W: push_restore(s, b, 1, u[w], 0, 0.0); break;
        case ORC_EDGE_NW: push_restore(s, b, 1, u[w], 1, v[n]); break;
        default: break;
        }
    }
}

/* Adaptive step (extension; the reference keeps delt fixed, src/simulation.rs:330):
 * delt = tau * min(Re/2 / (1/dx^2 + 1/dy^2), dx/umax, dy/vmax), with umax and
 * vmax the largest |u| and |v| over every cell (floor 1e-10).  This is the
 * textbook step-size rule of Griebel, Dornseifer and Neunhoeffer. */
void orc_adapt_dt(orc_sim *s) {
    if (!(s->prm.tau > 0.0)) return;
    double umax = 1.0e-10, vmax = 1.0e-10;
    size_t n = (size_t)s->nx * s->ny;
    for (size_t i = 0; i < n; i++) {
        umax = fmax(umax, fabs(s->u[i]));
        vmax = fmax(vmax, fabs(s->v[i]));
    }
    const double dx = s->prm.dx, dy = s->prm.dy;
    double dt_re = (0.5 * s->prm.reynolds) / ((1.0 / (dx * dx)) + (1.0 / (dy * dy)));
    double dt_u = dx / umax, dt_v = dy / vmax;
    double m = fmin(dt_re, fmin(dt_u, dt_v));
    s->prm.delt = s->prm.tau * m;
}

static inline void sor_cell(orc_sim *s, int x, int y, double one_minus_w, double middle,
                            double delx2, double dely2) {
    const int ny = s->ny;
    double *p = s->p;
    double p_i_j = AT(p, x, y), p_i_m1_j = AT(p, x - 1, y), p_i_p1_j = AT(p, x + 1, y);
    double p_i_j_m1 = AT(p, x, y - 1), p_i_j_p1 = AT(p, x, y + 1);
    double rhs = AT(s->rhs, x, y);
    AT(p, x, y) = (one_minus_w * p_i_j) +
                  middle * (((p_i_p1_j + p_i_m1_j) / delx2) + ((p_i_j_p1 + p_i_j_m1) / dely2) -
                            rhs);
}

/* src/simulation.rs:239-285, with an optional red-black ordering and an
 * optional strict-eps stop (both extensions). */
void orc_solve_sor(orc_sim *s, uint32_t *iters, double *ns_out) {
    const int nx = s->nx, ny = s->ny;
    const double delx2 = sq(s->prm.dx), dely2 = sq(s->prm.dy);
    const double one_minus_w = 1.0 - s->prm.omega;
    const double middle = s->prm.omega / ((2.0 / delx2) + (2.0 / dely2));
    const double eps2 = sq(s->prm.eps);
    double ns = 0.0;
    for (uint32_t i = 0; i < s->prm.max_iterations; i++) {
        orc_copy_pressure_to_boundaries(s);
        if (s->prm.sor_order == ORC_SOR_RED_BLACK) {
            for (int color = 0; color < 2; color++) {
#ifdef _OPENMP
                /* the cells of one colour are independent: any thread count
                   gives the same fields */
#pragma omp parallel for schedule(static) num_threads(s->threads) if (s->threads > 1)
#endif
                for (int x = 1; x < nx - 1; x++)
                    for (int y = 1 + ((x + 1 + color) & 1); y < ny - 1; y += 2)
                        if (AT(s->kind, x, y) == ORC_FLUID)
                            sor_cell(s, x, y, one_minus_w, middle, delx2, dely2);
            }
        } else {
            for (int x = 1; x < nx - 1; x++)
                for (int y = 1; y < ny - 1; y++)
                    if (AT(s->kind, x, y) == ORC_FLUID)
                        sor_cell(s, x, y, one_minus_w, middle, delx2, dely2);
        }
        double ns0 = s->prm.initial_norm_squared;
        ns = orc_calculate_norm_squared(s);
        int done = s->prm.strict_eps ? (ns < eps2) : ((ns < ns0) || (ns < eps2));
        if (done) {
            *iters = i + 1;
            *ns_out = ns;
            return;
        }
    }
    orc_calculate_pressure_range(s);
    *iters = s->prm.max_iterations;
    *ns_out = ns;
}

/* Threads of the red-black sweeps and the norm (1, the default, runs the
 * reference's serial loops; more is for timing a multi-core CPU: the sweeps
 * give the same fields, the norm's sum is added in another order).  No
 * reference counterpart: the crate is single-threaded. */
void orc_set_threads(orc_sim *s, int threads) { s->threads = threads > 1 ? threads : 1; }

/* src/simulation.rs:287-322 */
void orc_set_u_and_v(orc_sim *s) {
    const int nx = s->nx, ny = s->ny;
    const double cu = s->prm.delt / s->prm.dx, cv = s->prm.delt / s->prm.dy;
    double *p = s->p;
    for (int x = 0; x < nx - 1; x++)
        for (int y = 0; y < ny - 1; y++) {
            double p_i_j = AT(p, x, y), p_i_p1_j = AT(p, x + 1, y), p_i_j_p1 = AT(p, x, y + 1);
            AT(s->u, x, y) = AT(s->f, x, y) - cu * (p_i_p1_j - p_i_j);
            AT(s->v, x, y) = AT(s->g, x, y) - cv * (p_i_j_p1 - p_i_j);
        }
    for (int64_t k = 0; k < s->nrestore; k++) {
        restore_t *r = &s->restore[k];
        if (r->has_u) s->u[r->idx] = r->u;
        if (r->has_v) s->v[r->idx] = r->v;
    }
    orc_calculate_speed_range(s);
}

/* src/simulation.rs:324-333 */
void orc_tick(orc_sim *s, uint32_t *sor_iterations, double *norm_squared) {
    orc_adapt_dt(s);
    orc_set_boundary_u_and_v(s);
    orc_calculate_f_and_g(s);
    orc_calculate_rhs(s);
    orc_solve_sor(s, sor_iterations, norm_squared);
    orc_set_u_and_v(s);
    s->prm.time += s->prm.delt;
    s->prm.iterations += 1;
}

/* src/simulation.rs:71-99 and src/grid/mod.rs:127-153 */
orc_sim *orc_create(const orc_params *prm, const uint8_t *kind, const double *wall_uv,
                    const double *u, const double *v, const double *p, int *status,
                    int64_t *bad_index) {
    const int nx = prm->nx, ny = prm->ny;
    size_t n = (size_t)nx * ny;
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    if (s) s->threads = 1;
    s->prm = *prm;
    s->nx = nx;
    s->ny = ny;
    s->u = (double *)malloc(n * sizeof(double));
    s->v = (double *)malloc(n * sizeof(double));
    s->p = (double *)malloc(n * sizeof(double));
    s->f = (double *)calloc(n, sizeof(double));
    s->g = (double *)calloc(n, sizeof(double));
    s->rhs = (double *)calloc(n, sizeof(double));
    s->kind = (uint8_t *)malloc(n);
    s->edge = (uint8_t *)malloc(n);
    s->wall = (double *)calloc(2 * n, sizeof(double));
    memcpy(s->u, u, n * sizeof(double));
    memcpy(s->v, v, n * sizeof(double));
    memcpy(s->p, p, n * sizeof(double));
    memcpy(s->kind, kind, n);
    if (wall_uv) memcpy(s->wall, wall_uv, 2 * n * sizeof(double));
    if (orc_classify(nx, ny, s->kind, s->edge, &s->fluid_cells, bad_index)) {
        if (status) *status = 1;
        orc_destroy(s);
        return NULL;
    }
    s->nbnd = 0;
    for (size_t i = 0; i < n; i++)
        if (s->kind[i] != ORC_FLUID) s->nbnd++;
    s->bnd = (int64_t *)malloc((s->nbnd + 1) * sizeof(int64_t));
    s->restore = (restore_t *)malloc((2 * s->nbnd + 1) * sizeof(restore_t));
    int64_t k = 0;
    for (size_t i = 0; i < n; i++)
        if (s->kind[i] != ORC_FLUID) s->bnd[k++] = (int64_t)i;
    orc_calculate_pressure_range(s);
    orc_calculate_speed_range(s);
    orc_calculate_f_and_g(s);
    orc_calculate_rhs(s);
    if (!s->prm.has_initial_norm) {
        s->prm.initial_norm_squared = orc_calculate_norm_squared(s);
        s->prm.has_initial_norm = 1;
    }
    if (status) *status = 0;
    return s;
}

void orc_destroy(orc_sim *s) {
    if (!s) return;
    free(s->u); free(s->v); free(s->p); free(s->f); free(s->g); free(s->rhs);
    free(s->kind); free(s->edge); free(s->wall); free(s->bnd); free(s->restore);
    free(s);
}

static double *field_ptr(const orc_sim *s, int which) {
    switch (which) {
    case 0: return s->u;
    case 1: return s->v;
    case 2: return s->p;
    case 3: return s->f;
    case 4: return s->g;
    default: return s->rhs;
    }
}

void orc_get_field(const orc_sim *s, int which, double *out) {
    memcpy(out, field_ptr(s, which), (size_t)s->nx * s->ny * sizeof(double));
}

void orc_set_field(orc_sim *s, int which, const double *in) {
    memcpy(field_ptr(s, which), in, (size_t)s->nx * s->ny * sizeof(double));
}

void orc_get_edges(const orc_sim *s, uint8_t *out) {
    memcpy(out, s->edge, (size_t)s->nx * s->ny);
}

void orc_get_state(const orc_sim *s, double *out8) {
    out8[0] = s->prm.time;
    out8[1] = (double)s->prm.iterations;
    out8[2] = s->prm.initial_norm_squared;
    out8[3] = s->prm.delt;
    out8[4] = s->pressure_range[0];
    out8[5] = s->pressure_range[1];
    out8[6] = s->speed_range[0];
    out8[7] = s->speed_range[1];
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* One tick with its phases timed (CPU-baseline sampling): out4 = {seconds
 * before the pressure solve (dt, boundary pass, F/G, RHS), seconds in the
 * solve, iterations run, seconds after it (velocity update)}.  A
 * max_iterations_cap > 0 bounds the solve for this tick only. */
void orc_tick_timed(orc_sim *s, uint32_t max_iterations_cap, double *out4) {
    uint32_t saved = s->prm.max_iterations, it = 0;
    double ns = 0.0;
    if (max_iterations_cap > 0 && max_iterations_cap < saved) s->prm.max_iterations = max_iterations_cap;
    double t0 = now_s();
    orc_adapt_dt(s);
    orc_set_boundary_u_and_v(s);
    orc_calculate_f_and_g(s);
    orc_calculate_rhs(s);
    double t1 = now_s();
    orc_solve_sor(s, &it, &ns);
    double t2 = now_s();
    orc_set_u_and_v(s);
    s->prm.time += s->prm.delt;
    s->prm.iterations += 1;
    double t3 = now_s();
    s->prm.max_iterations = saved;
    out4[0] = t1 - t0;
    out4[1] = t2 - t1;
    out4[2] = (double)it;
    out4[3] = t3 - t2;
}

/* ------------------------------------------------------------------ */
/* Colour map, src/visualization.rs:7-105                              */
/* ------------------------------------------------------------------ */

/* src/visualization.rs:7-27, in f32 */
static void hsl_to_rgb(float hue, float saturation, float lightness, float *r, float *g,
                       float *b) {
    float c = (1.0f - fabsf(2.0f * lightness - 1.0f)) * saturation;
    float x = c * (1.0f - fabsf(fmodf(hue / 60.0f, 2.0f) - 1.0f));
    float m = lightness - c / 2.0f;
    float rr, gg, bb;
    if (hue < 60.0f) { rr = c; gg = x; bb = 0.0f; }
    else if (hue < 120.0f) { rr = x; gg = c; bb = 0.0f; }
    else if (hue < 180.0f) { rr = 0.0f; gg = c; bb = x; }
    else if (hue < 240.0f) { rr = 0.0f; gg = x; bb = c; }
    else if (hue < 300.0f) { rr = x; gg = 0.0f; bb = c; }
    else { rr = c; gg = 0.0f; bb = x; }
    *r = rr + m;
    *g = gg + m;
    *b = bb + m;
}

/* Rust's `f as u8`: NaN -> 0, saturating, truncating; the colour channel is
 * scaled by 255 first (macroquad's Color -> [u8; 4] conversion). */
static uint8_t channel_u8(float c) {
    float v = c * 255.0f;
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}

/* render_simulation (src/visualization.rs:79-105) into rgba[ny][nx][4]:
 * color_type 0 pressure (:49-70), 1 speed (:29-47). */
void orc_render(const orc_sim *s, int color_type, uint8_t *rgba) {
    const int nx = s->nx, ny = s->ny;
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            size_t i = (size_t)x * ny + y;
            float r, g, b, a = 1.0f;
            if (s->kind[i] != ORC_FLUID) {
                if (color_type == 1) { r = 0.5f; g = 0.5f; b = 0.5f; }
                else { r = 0.5f; g = 0.0f; b = 0.0f; }
            } else {
                double hue_d;
                if (color_type == 1) {
                    double speed = sqrt(sq(s->u[i]) + sq(s->v[i]));
                    hue_d = 240.0 - (speed - s->speed_range[0]) * 240.0 /
                                        (s->speed_range[1] - s->speed_range[0]);
                } else {
                    double offset = 240.0;
                    hue_d = offset - (s->p[i] - s->pressure_range[0]) * offset /
                                         (s->pressure_range[1] - s->pressure_range[0]);
                }
                hsl_to_rgb((float)hue_d, 1.0f, 0.5f, &r, &g, &b);
            }
            uint8_t *px = rgba + ((size_t)y * nx + x) * 4;
            px[0] = channel_u8(r);
            px[1] = channel_u8(g);
            px[2] = channel_u8(b);
            px[3] = channel_u8(a);
        }
}
