// Device tables of a batch of scenes (batch.cu, batch_step_*.cu): per-lattice geometry,
// rates and storage shift; launch tiles; per-scene solid parameters.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "coupling_core.cuh"
#include "fsi_common.cuh"
#include "lbm_core.cuh"
#include "mpm_core.cuh"

namespace fsi {
namespace {

constexpr int kTileCells = 256;

struct BatchLattice {
  LbmGeom g;
  long long off;  // first cell in the concatenated arrays
  float s[19];
  float sg[19];  // 1 - s_k / 2
  float shift[19];
  float rho0;
  float base[3];
};

struct Tile {
  int lattice;
  int first;  // first cell (lattice tiles), particle block or node block (solid tiles)
};

struct BatchSolid {
  Mpm m;                  // n = end of the scene's particle range, cap = batch capacity
  long long block_off;    // first 4^3 node block of the scene in the dirty map
  fsi_coupling_desc c;
};

__device__ __forceinline__ void cell_ijk(const LbmGeom& g, int c, int& i, int& j, int& k) {
  const int nyz = g.ny * g.nz;
  i = c / nyz;
  const int r = c - i * nyz;
  j = r / g.nz;
  k = r - j * g.nz;
}

}  // namespace

// Launches the batched lattice step for one storage form (batch_step_{f32,f16,bf16}.cu).
// lat / tiles: device tables; tile_cells: cells per step tile (a multiple of 128, or of 256
// for the fast forms); variant: register-cap variant 0..2.
int batch_step_launch_f32(const void* lat, const void* tiles, int ntiles, int tile_cells,
                          int variant, bool fast, bool odd, bool recompute, void* pops,
                          float* macro, const float* force, const float* force_prev,
                          const uint32_t* flags, cudaStream_t stream);
int batch_step_launch_f16(const void* lat, const void* tiles, int ntiles, int tile_cells,
                          int variant, bool fast, bool odd, bool recompute, void* pops,
                          float* macro, const float* force, const float* force_prev,
                          const uint32_t* flags, cudaStream_t stream);
int batch_step_launch_bf16(const void* lat, const void* tiles, int ntiles, int tile_cells,
                           int variant, bool fast, bool odd, bool recompute, void* pops,
                           float* macro, const float* force, const float* force_prev,
                           const uint32_t* flags, cudaStream_t stream);

}  // namespace fsi
