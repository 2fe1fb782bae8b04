// Internal interface of the serving pools: on-device assembly into one slot
// of a batched hierarchy (gmg_assemble.cu), used by gmg_serve.cpp.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "gmg_internal.h"

#define GMG_FIELD_MAX_M 256  // random Fourier features of the coefficient field

namespace gmg {

// one slot's rows on one level of a pool
struct SlotLevel {
  int N = 0;              // points per axis of the cube grid on this level
  int off = 0;            // first union list position of the slot
  int nrows = 0;          // rows of the slot (N^3)
  const int *rows = nullptr;  // device: the slot's rows (processing order)
  const uint8_t *masks = nullptr;  // device: UG's mesh, the tetrahedra of every cell (nullptr: Freudenthal)
};

// field features of LogNormalField(seed, 3, corr, var) for a level with h =
// 2^-level, as (phi, theta_x, theta_y, theta_z) in 2^-32 turns per h/4
void cube_field_params(uint64_t seed, double corr, double var, int level, std::vector<uint32_t> &prm, float *amp,
                       int *M);
// k of every tetrahedron of a level with Nc cells per axis
// (masks: UG's mesh, every cell's six tetrahedra as corner masks; nullptr:
// the Freudenthal triangulation)
int k_cube_field(gmg_mg *mg, int Nc, const uint32_t *prm_dev, int M, float amp, float *kelem,
                 const uint8_t *masks = nullptr);
// the FP64 field of a level with Nc cells per axis from the features w (M x 3)
// and phi (M) of LogNormalField: tables (M (3 Nc + 30) double2) of per-axis and
// per-tetrahedron phase factors, then k of every tetrahedron
int k_cube_field64(gmg_mg *mg, int Nc, const double *w_dev, const double *phi_dev, int M, double amp,
                   double2 *tables, double *kelem, const uint8_t *masks = nullptr);
// the tetrahedra of every cell of a UG-refined cube level (generator kind 3),
// host memory owned by the generator; nullptr for the other kinds
const uint8_t *gen_cell_masks(const gmg_gen *g, int level);
int gen_kind(const gmg_gen *g);
// ... assembly from an FP64 field
int k_cube_assemble64(gmg_mg *mg, const Level &L, const SlotLevel &sl, const double *kelem, double h,
                      const int *c2s);
// the slot's rows of level L from k (kelem == nullptr: k = 1); c2s maps CSR
// entries to sliced-ELLPACK entries (nullptr if the level has none)
int k_cube_assemble(gmg_mg *mg, const Level &L, const SlotLevel &sl, const float *kelem, double h, const int *c2s);
// right-hand side of the slot (finest level), x = 0 there
int k_cube_rhs(gmg_mg *mg, const Level &L, const SlotLevel &sl, uint64_t seed, double *b, double *x);
// per-component norms of b over the slot's NEW_DEFECT rows into out[0..s);
// scratch holds SLOT_NORM_BLOCKS * GMG_MAX_S doubles and a zeroed ticket
constexpr int SLOT_NORM_BLOCKS = 304;
int k_slot_norm(gmg_mg *mg, const Level &L, const SlotLevel &sl, const double *b, double *scratch, double *out);

}  // namespace gmg
