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

// The lattice of a tile as the argument type of step_cells.
struct LatticeView {
  LbmGeom g;
  void* __restrict__ pops;
  float4* __restrict__ macro;
  const float* FSI_LAUNCH_RO force;
  const float* FSI_LAUNCH_RO force_prev;
  const uint32_t* __restrict__ flags;
  const float* s;
  const float* sg;
  const float* shift;
  int write_faces;
};

template <int kStore>
__device__ __forceinline__ LatticeView view_of(const BatchLattice& L, void* pops, float* macro,
                                               const float* force, const float* force_prev,
                                               const uint32_t* flags) {
  using T = typename Store<kStore>::T;
  LatticeView v;
  v.g = L.g;
  v.pops = reinterpret_cast<T*>(pops) + 19 * L.off;
  v.macro = reinterpret_cast<float4*>(macro) + L.off;
  v.force = force + 3 * L.off;
  v.force_prev = force_prev ? force_prev + 3 * L.off : nullptr;
  v.flags = flags + L.off;
  v.s = L.s;
  v.sg = L.sg;
  v.shift = L.shift;
  v.write_faces = 0;
  return v;
}

// update_macro of cell c of lattice L (lbm3d.py:409-425) in the concatenated arrays; returns
// the cell's fluid rho (0 on solid cells) and |u| in mass / vmax.
template <int kStore, bool kFast>
__device__ __forceinline__ void batch_macro_cell(const BatchLattice& L, int c, const void* pops_v,
                                                 const float* FSI_LAUNCH_RO force_all,
                                                 const uint32_t* __restrict__ flags_all,
                                                 int parity, float* macro_all, float& mass,
                                                 float& vmax) {
  int i, j, k;
  cell_ijk(L.g, c, i, j, k);
  const Deltas d(L.g, i, j, k);
  const uint32_t fl = flags_all[L.off + c];
  float4* macro = reinterpret_cast<float4*>(macro_all) + L.off;
  mass = 0.f;
  vmax = 0.f;
  if (fl & kFlagSolid) {
    macro[c] = make_float4(0.f, 0.f, 0.f, L.rho0);
    return;
  }
  const uint32_t n = (uint32_t)L.g.n;
  const auto* pops = reinterpret_cast<const typename Store<kStore>::T*>(pops_v) + 19 * L.off;
  const float* force = force_all + 3 * L.off;
  float F[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) F[q] = gather32<kStore>(pops, n, d, fl, q, parity, L.shift[q]);
  float rho, ux, uy, uz;
  macro_any<kFast>(F, force[c], force[n + c], force[2 * n + c], rho, ux, uy, uz);
  macro[c] = make_float4(ux, uy, uz, rho);
  mass = rho;
  vmax = norm3_ref(ux, uy, uz);
}

// The coupling arguments of scene `lattice` of a batch: the scene's coupling descriptor and
// lattice block, the batch's particle arrays and the scene's counters.
__device__ __forceinline__ ForceArgs scene_force_args(const ForceArgs& base, const BatchLattice& L,
                                                      const BatchSolid& S, int lattice,
                                                      float dt_ratio, int build_fraction) {
  ForceArgs a = base;
  a.c = S.c;
  a.c.dt_ratio = dt_ratio;
  a.c.build_fraction = build_fraction;
  a.g = Geo{L.g.nx, L.g.ny, L.g.nz, L.g.n};
  a.n = S.m.n;
  a.macro = base.macro + L.off;
  a.flags = base.flags + L.off;
  a.accum = base.accum + L.off;
  a.cnt = base.cnt + lattice;
  return a;
}

// The force-assembly arguments of scene `lattice` of a batch.
__device__ __forceinline__ AssembleArgs scene_assemble_args(const AssembleArgs& base,
                                                            const BatchLattice& L,
                                                            const BatchSolid& S, int lattice) {
  AssembleArgs a = base;
  a.c = S.c;
  a.g = Geo{L.g.nx, L.g.ny, L.g.nz, L.g.n};
  a.flags = base.flags + L.off;
#pragma unroll
  for (int i = 0; i < 3; ++i) a.base[i] = L.base[i];
  a.accum = base.accum + L.off;
  a.macro = base.macro ? base.macro + L.off : nullptr;
  a.force = base.force ? base.force + 3 * L.off : nullptr;
  a.ib = base.ib ? base.ib + 3 * L.off : nullptr;
  a.cnt = base.cnt + lattice;
  return a;
}

// Arguments of the persistent coupled-step kernel (batch_persistent.cuh).
struct PersistArgs {
  const BatchLattice* lat;
  const BatchSolid* sol;
  const Tile* cell_tiles;  // kTileCells consecutive cells of one lattice each
  int ncell_tiles;
  const Tile* step_tiles;  // step_tile_cells cells each
  int nstep_tiles;
  int step_tile_cells;
  const Tile* ptiles;  // kBlock particles of one scene each
  int nptiles;
  const Tile* ctiles;  // kBlock / 32 node blocks of one scene each
  int nctiles;
  int count;
  PView P;
  ForceArgs fa;        // batch-wide particle and coupling arrays
  AssembleArgs aa;     // batch-wide assembly arrays (force set per step)
  void* pops;
  float* macro;
  float* force[2];
  const uint32_t* flags;
  float4* grid;
  uint8_t* dirty;
  unsigned* sync;  // barrier arrival counter, zero at launch
  int* err;        // 0, or FSI_ERR_TIMEOUT after a wait gave up
  long long steps_done;
  int steps;
  int substeps;
  float dt_ratio;
  int build_fraction;
  int prev;         // force buffer of the step before the first (the first refresh reads it)
  int macro_fresh;  // rho, u of the initial state are already in macro
  long long wait_cycles;
};

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

// Launches the persistent coupled-step kernel of a batch for one storage form
// (batch_persist_{f32,f16,bf16}.cu); args points to a PersistArgs.
int batch_persist_launch_f32(const void* args, bool fast, cudaStream_t stream);
int batch_persist_launch_f16(const void* args, bool fast, cudaStream_t stream);
int batch_persist_launch_bf16(const void* args, bool fast, cudaStream_t stream);

}  // namespace fsi
