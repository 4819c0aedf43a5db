// Host-side compiler of the boundary-condition pass.
//
// The reference applies its boundary conditions cell by cell in x-major order
// (SimulationGrid::set_boundary_u_and_v, src/grid/mod.rs:414-651), and a
// later cell can read a value an earlier cell wrote (at the domain corners a
// North-edged wall cell zeroes v of a fluid cell whose value an East-edged
// inflow cell copied just before).  It also records, per boundary cell, the
// values that set_u_and_v restores after the velocity update
// (src/grid/mod.rs:595-648; src/simulation.rs:313-320), keyed at the boundary
// cell even where the value is the neighbour's.
//
// This file executes that pass once, symbolically: every value is either a
// constant, a pre-pass value of some cell, its negation, or (moving walls)
// c minus a pre-pass value.  What remains is a set of independent
// (target <- expression) entries that the device evaluates in parallel,
// reading pre-pass values only.  The same symbolic pass is exported for the
// host (strm_host_boundary_pass) so that tests can compare it with the
// oracle without a GPU.
#include <map>
#include <stdexcept>
#include <vector>

#include "strm_bcprog.h"

namespace strm {

namespace {

struct Sym {
  int op;      // 0 const, 1 +src, 2 -src, 3 c - src
  long long src;
  double c;
};

struct Pass {
  int nx, ny, pitch;
  std::map<long long, Sym> written[2];  // u, v by dense index
  long long idx(int x, int y) const { return (long long)x * ny + y; }

  Sym read(int f, long long i) const {
    auto it = written[f].find(i);
    if (it != written[f].end()) return it->second;
    return Sym{1, i, 0.0};
  }
  void set(int f, long long i, Sym s) { written[f][i] = s; }
  static Sym cst(double c) { return Sym{0, 0, c}; }
  // -a: sources are fluid cells, which only ever hold a pre-pass value or a constant.
  static Sym neg(const Sym &a) {
    if (a.op == 0) return cst(-a.c);
    if (a.op == 1) return Sym{2, a.src, 0.0};
    throw std::logic_error("negation of a derived value");
  }
  static Sym csub(double c, const Sym &a) {
    if (a.op == 0) return cst(c - a.c);
    if (a.op == 1) return Sym{3, a.src, c};
    throw std::logic_error("moving-wall mirror of a derived value");
  }
};

}  // namespace

// Classification on the host (src/grid/mod.rs:270-332); returns false on a
// thin wall with *bad the first offending x*ny+y.
bool classify_host(int nx, int ny, const uint8_t *kind, uint8_t *edge, double *fluid_cells,
                   long long *bad) {
  long long fluid = 0;
  for (long long i = 0; i < (long long)nx * ny; ++i) {
    edge[i] = 0;
    if (kind[i] == K_FLUID) ++fluid;
  }
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y) {
      const long long i = (long long)x * ny + y;
      if (kind[i] == K_FLUID) continue;
      const int left = x > 0 && kind[i - ny] == K_FLUID;
      const int right = x < nx - 1 && kind[i + ny] == K_FLUID;
      const int up = y > 0 && kind[i - 1] == K_FLUID;
      const int down = y < ny - 1 && kind[i + 1] == K_FLUID;
      const int code = (left << 3) | (right << 2) | (up << 1) | down;
      int e;
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
        default:
          if (bad) *bad = i;
          return false;
      }
      edge[i] = (uint8_t)e;
    }
  if (fluid_cells) *fluid_cells = (double)fluid;
  return true;
}

void compile_boundary_program(int nx, int ny, int pitch, const uint8_t *kind,
                              const uint8_t *edge, const double *wall_uv,
                              std::vector<BcEntry> &prog, std::vector<PCopy> &pcopy) {
  Pass P{nx, ny, pitch, {}};
  struct Restore {
    long long b;
    Sym u, v;
  };
  std::vector<Restore> restore;
  prog.clear();
  pcopy.clear();
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y) {
      const long long b = P.idx(x, y);
      const int kd = kind[b];
      if (kd == K_FLUID) continue;
      const int e = edge[b];
      if (e == E_NONE) continue;  // its u, v are left alone and restored to themselves
      pcopy.push_back(PCopy{(long long)x * pitch + y, e, 0});
      const long long n = b - 1, s = b + 1, ea = b + ny, w = b - ny;
      const int U = 0, V = 1;
      if (kd == K_NO_SLIP || kd == K_INFLOW || kd == K_MOVING) {
        double bu = 0.0, bv = 0.0;
        if (kd != K_NO_SLIP && wall_uv) {
          bu = wall_uv[2 * b];
          bv = wall_uv[2 * b + 1];
        }
        const bool moving = kd == K_MOVING;
        auto mir_u = [&](const Sym &a) { return moving ? Pass::csub(2.0 * bu, a) : Pass::neg(a); };
        auto mir_v = [&](const Sym &a) { return moving ? Pass::csub(2.0 * bv, a) : Pass::neg(a); };
        switch (e) {
          case E_N:
            P.set(U, b, mir_u(P.read(U, n)));
            P.set(V, n, Pass::cst(bv));
            break;
          case E_NE:
            P.set(U, b, Pass::cst(bu));
            P.set(V, n, Pass::cst(bv));
            P.set(V, b, mir_v(P.read(V, ea)));
            break;
          case E_E:
            P.set(U, b, Pass::cst(bu));
            P.set(V, b, mir_v(P.read(V, ea)));
            break;
          case E_SE:
            P.set(U, b, Pass::cst(bu));
            P.set(V, b, Pass::cst(bv));
            break;
          case E_S:
            P.set(U, b, mir_u(P.read(U, s)));
            P.set(V, b, Pass::cst(bv));
            break;
          case E_SW:
            P.set(U, w, Pass::cst(bu));
            P.set(U, b, mir_u(P.read(U, s)));
            P.set(V, b, Pass::cst(bv));
            break;
          case E_W:
            P.set(U, w, Pass::cst(bu));
            P.set(V, b, mir_v(P.read(V, w)));
            break;
          case E_NW:
            P.set(U, w, Pass::cst(bu));
            P.set(U, b, mir_u(P.read(U, n)));
            P.set(V, n, Pass::cst(bv));
            P.set(V, b, mir_v(P.read(V, w)));
            break;
        }
      } else {  // outflow: copies, src/grid/mod.rs:489-536
        switch (e) {
          case E_N: P.set(U, b, P.read(U, n)); P.set(V, b, P.read(V, n)); break;
          case E_NE: P.set(U, b, P.read(U, n)); P.set(V, b, P.read(V, ea)); break;
          case E_E: P.set(U, b, P.read(U, ea)); P.set(V, b, P.read(V, ea)); break;
          case E_SE: P.set(U, b, P.read(U, ea)); P.set(V, b, P.read(V, s)); break;
          case E_S: P.set(U, b, P.read(U, s)); P.set(V, b, P.read(V, s)); break;
          case E_SW: P.set(U, b, P.read(U, w)); P.set(V, b, P.read(V, s)); break;
          case E_W: P.set(U, b, P.read(U, w)); P.set(V, b, P.read(V, w)); break;
          case E_NW: P.set(U, b, P.read(U, n)); P.set(V, b, P.read(V, w)); break;
        }
      }
      // The restore list: (b, u[b], v[b]), then for N/NE/NW v of the north
      // neighbour and for W/SW/NW u of the west neighbour, keyed at b.
      Restore r{b, P.read(U, b), P.read(V, b)};
      if (e == E_N || e == E_NE || e == E_NW) r.v = P.read(V, n);
      if (e == E_W || e == E_SW || e == E_NW) r.u = P.read(U, w);
      restore.push_back(r);
    }
  auto to_off = [&](long long dense) {
    return (dense / ny) * (long long)pitch + (dense % ny);
  };
  auto emit = [&](int field, long long dense_target, const Sym &s) {
    BcEntry en{};
    en.target = ((long long)field << 56) | to_off(dense_target);
    en.src = s.op == 0 ? 0 : to_off(s.src);
    en.c = s.c;
    en.op = s.op;
    prog.push_back(en);
  };
  for (int f = 0; f < 2; ++f)
    for (const auto &kv : P.written[f]) emit(f, kv.first, kv.second);
  for (const auto &r : restore) {
    emit(2, r.b, r.u);
    emit(3, r.b, r.v);
  }
}

void apply_boundary_program_host(const std::vector<BcEntry> &prog, double *u, double *v,
                                 double *ru, double *rv) {
  std::vector<double> val(prog.size());
  for (size_t k = 0; k < prog.size(); ++k) {
    const BcEntry &e = prog[k];
    const int field = (int)(e.target >> 56);
    const double s = e.op == 0 ? 0.0 : ((field & 1) ? v : u)[e.src];
    switch (e.op) {
      case 0: val[k] = e.c; break;
      case 1: val[k] = s; break;
      case 2: val[k] = -s; break;
      default: val[k] = e.c - s; break;
    }
  }
  for (size_t k = 0; k < prog.size(); ++k) {
    const long long t = prog[k].target;
    const int field = (int)(t >> 56);
    const long long off = t & ((1LL << 56) - 1);
    double *dst = field == 0 ? u : field == 1 ? v : field == 2 ? ru : rv;
    dst[off] = val[k];
  }
}

}  // namespace strm
