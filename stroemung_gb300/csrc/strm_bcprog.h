// Host-side boundary-program compiler (see strm_bcprog.cpp).
#pragma once

#include <stdint.h>

#include <vector>

#include "strm_internal.cuh"

namespace strm {

bool classify_host(int nx, int ny, const uint8_t *kind, uint8_t *edge, double *fluid_cells,
                   long long *bad);

// kind/edge/wall_uv are dense [nx][ny] host arrays; offsets in the emitted
// entries use `pitch`.
void compile_boundary_program(int nx, int ny, int pitch, const uint8_t *kind,
                              const uint8_t *edge, const double *wall_uv,
                              std::vector<BcEntry> &prog, std::vector<PCopy> &pcopy);

// Gather-then-scatter evaluation of a program on host arrays.
void apply_boundary_program_host(const std::vector<BcEntry> &prog, double *u, double *v,
                                 double *ru, double *rv);

}  // namespace strm
