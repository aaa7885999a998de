// Batches of independent scenes: one launch per phase over every lattice of the batch.
//
// A launch walks the batch's tiles of kTileCells consecutive cells of one lattice each
// (tile = one thread block). Every lattice keeps its own geometry, relaxation rates and
// storage shift in a device table; the per-cell work is the single-lattice code
// (lbm_core.cuh) applied to that lattice's block of the concatenated arrays, so a batch
// reproduces each lattice's standalone run bit for bit.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "batch_types.cuh"

struct fsi_batch;

namespace fsi {
namespace {

}  // namespace
}  // namespace fsi

struct fsi_batch {
  fsi::BatchLattice* lat = nullptr;  // device
  fsi::Tile* tiles = nullptr;        // device
  int count = 0;
  int ntiles = 0;
  int storage = 0;
  int arithmetic = 0;
  long long cells = 0;
  std::vector<fsi::BatchLattice> host;
  // solids (fsi_batch_set_solids)
  fsi::Tile* step_tiles = nullptr;  // device: tiles of the step kernel (fsi_batch_tune)
  int nstep_tiles = 0;
  int step_tile_cells = 0;
  int variant = 1;
  fsi::BatchSolid* sol = nullptr;   // device
  fsi::Tile* ptiles = nullptr;      // device: (scene, particle block of kBlock particles)
  fsi::Tile* ctiles = nullptr;      // device: (scene, first node block of 8)
  int nptiles = 0;
  int nctiles = 0;
  long long capacity = 0;
  std::vector<fsi::BatchSolid> host_sol;
};

namespace fsi {
namespace {

// update_macro of every lattice (lbm3d.py:409-425), optionally with each lattice's sum of
// rho over fluid cells and max |u| (lbm3d.py:450-457) in diag[2 * lattice + {0, 1}].
template <int kStore, bool kFast>
__global__ void __launch_bounds__(kTileCells)
    batch_macro_kernel(const BatchLattice* __restrict__ lat, const Tile* __restrict__ tiles,
                       const void* pops_v, const float* __restrict__ force_all,
                       const uint32_t* __restrict__ flags_all, int parity, float* macro_all,
                       double* __restrict__ diag) {
  const Tile t = tiles[blockIdx.x];
  const BatchLattice& L = lat[t.lattice];
  const int c = t.first + threadIdx.x;
  float mass = 0.f, vmax = 0.f;
  if (c < L.g.n)
    batch_macro_cell<kStore, kFast>(L, c, pops_v, force_all, flags_all, parity, macro_all, mass,
                                    vmax);
  if (diag) {
    const float s[1] = {mass};
    block_accumulate<1>(diag + 2 * t.lattice, s, diag + 2 * t.lattice + 1, vmax);
  }
}

template <int kStore>
__global__ void __launch_bounds__(kTileCells)
    batch_distribution_kernel(const BatchLattice* __restrict__ lat, const Tile* __restrict__ tiles,
                              const void* pops_v, const uint32_t* __restrict__ flags_all,
                              int parity, float* __restrict__ out) {
  const Tile t = tiles[blockIdx.x];
  const BatchLattice& L = lat[t.lattice];
  const int c = t.first + threadIdx.x;
  if (c >= L.g.n) return;
  int i, j, k;
  cell_ijk(L.g, c, i, j, k);
  const Deltas d(L.g, i, j, k);
  const uint32_t fl = flags_all[L.off + c];
  const int p = (fl & kFlagSolid) ? 0 : parity;
  const auto* pops = reinterpret_cast<const typename Store<kStore>::T*>(pops_v) + 19 * L.off;
#pragma unroll
  for (int q = 0; q < 19; ++q)
    out[(size_t)(L.off + c) * 19 + q] = gather32<kStore>(pops, (uint32_t)L.g.n, d, fl, q, p, L.shift[q]);
}

__global__ void __launch_bounds__(kTileCells)
    batch_flags_kernel(const BatchLattice* __restrict__ lat, const Tile* __restrict__ tiles,
                       const int32_t* __restrict__ solid_all, uint32_t* __restrict__ flags_all) {
  const Tile t = tiles[blockIdx.x];
  const BatchLattice& L = lat[t.lattice];
  const int c = t.first + threadIdx.x;
  if (c >= L.g.n) return;
  int i, j, k;
  cell_ijk(L.g, c, i, j, k);
  const Deltas d(L.g, i, j, k);
  const int32_t* solid = solid_all + L.off;
  uint32_t f = solid[d.c] != 0 ? kFlagSolid : 0u;
#pragma unroll
  for (int q = 1; q < 19; ++q)
    if (solid[d.nb(q, +1)] != 0) f |= 1u << q;
  f |= corner_flag_bits(solid, d);
  if (i == 0) f |= kFlagFaceLeft;
  if (i == L.g.nx - 1) f |= kFlagFaceRight;
  flags_all[L.off + c] = f;
}

template <int kStore>
__global__ void __launch_bounds__(kTileCells)
    batch_init_kernel(const BatchLattice* __restrict__ lat, const Tile* __restrict__ tiles,
                      const float* __restrict__ u0, const uint32_t* __restrict__ flags_all,
                      void* pops_v, float* macro_all) {
  const Tile t = tiles[blockIdx.x];
  const BatchLattice& L = lat[t.lattice];
  const int c = t.first + threadIdx.x;
  if (c >= L.g.n) return;
  const bool solid = flags_all[L.off + c] & kFlagSolid;
  const float* u = u0 + 3 * t.lattice;
  const float ux = solid ? 0.f : u[0], uy = solid ? 0.f : u[1], uz = solid ? 0.f : u[2];
  reinterpret_cast<float4*>(macro_all)[L.off + c] = make_float4(ux, uy, uz, L.rho0);
  auto* pops = reinterpret_cast<typename Store<kStore>::T*>(pops_v) + 19 * L.off;
#pragma unroll
  for (int q = 0; q < 19; ++q)
    Store<kStore>::st(pops, (uint32_t)(q * L.g.n + c), feq_ref(q, L.rho0, ux, uy, uz), L.shift[q]);
}

__global__ void __launch_bounds__(kTileCells)
    batch_base_force_kernel(const BatchLattice* __restrict__ lat, const Tile* __restrict__ tiles,
                            const uint32_t* __restrict__ flags_all, float* __restrict__ force_all) {
  const Tile t = tiles[blockIdx.x];
  const BatchLattice& L = lat[t.lattice];
  const int c = t.first + threadIdx.x;
  if (c >= L.g.n) return;
  const bool fluid = !(flags_all[L.off + c] & kFlagSolid);
  float* force = force_all + 3 * L.off;
#pragma unroll
  for (int a = 0; a < 3; ++a) force[a * L.g.n + c] = fluid ? L.base[a] : 0.f;
}

template <int S, bool F>
struct BatchMacroLauncher {
  static void run(const fsi_batch* b, const void* pops, const float* force, const uint32_t* flags,
                  int parity, float* macro, double* diag, cudaStream_t s) {
    batch_macro_kernel<S, F><<<b->ntiles, kTileCells, 0, s>>>(b->lat, b->tiles, pops, force, flags,
                                                              parity, macro, diag);
  }
};

template <int S, bool F>
struct BatchDistLauncher {
  static void run(const fsi_batch* b, const void* pops, const uint32_t* flags, int parity,
                  float* out, cudaStream_t s) {
    batch_distribution_kernel<S><<<b->ntiles, kTileCells, 0, s>>>(b->lat, b->tiles, pops, flags,
                                                                  parity, out);
  }
};

template <int S, bool F>
struct BatchInitLauncher {
  static void run(const fsi_batch* b, const float* u0, const uint32_t* flags, void* pops,
                  float* macro, cudaStream_t s) {
    batch_init_kernel<S><<<b->ntiles, kTileCells, 0, s>>>(b->lat, b->tiles, u0, flags, pops, macro);
  }
};

template <template <int, bool> class Launcher, class... Args>
void dispatch_batch(const fsi_batch* b, Args&&... args) {
  switch (b->storage) {
    case FSI_STORAGE_F16: Launcher<FSI_STORAGE_F16, true>::run(b, args...); break;
    case FSI_STORAGE_BF16: Launcher<FSI_STORAGE_BF16, true>::run(b, args...); break;
    default:
      if (b->arithmetic == FSI_ARITH_FAST) Launcher<FSI_STORAGE_F32, true>::run(b, args...);
      else Launcher<FSI_STORAGE_F32, false>::run(b, args...);
  }
}

int check_batch(const fsi_batch* b) {
  FSI_REQUIRE(b != nullptr && b->lat != nullptr && b->ntiles > 0, "invalid batch handle");
  return FSI_OK;
}

// ------------------------------------------------------------------ solids

// One CTA per (scene, block of kBlock particles): the single-solver P2G / G2P bodies on the
// scene's grid block.
__global__ void __launch_bounds__(kBlock)
    batch_p2g_kernel(const BatchLattice* __restrict__ lat, const BatchSolid* __restrict__ sol,
                     const Tile* __restrict__ ptiles, PView P, float4* grid_all, uint8_t* dirty_all) {
  const Tile t = ptiles[blockIdx.x];
  const Mpm m = sol[t.lattice].m;
  p2g_body(m, P, grid_all + lat[t.lattice].off, dirty_all + sol[t.lattice].block_off,
           t.first * kBlock + threadIdx.x);
}

__global__ void __launch_bounds__(kBlock)
    batch_g2p_kernel(const BatchLattice* __restrict__ lat, const BatchSolid* __restrict__ sol,
                     const Tile* __restrict__ ptiles, PView P, const float4* grid_all) {
  const Tile t = ptiles[blockIdx.x];
  const Mpm m = sol[t.lattice].m;
  g2p_body(m, P, grid_all + lat[t.lattice].off, t.first * kBlock + threadIdx.x);
}

// One warp per node block: CTA (scene, first block) covers kBlock / 32 blocks.
__global__ void __launch_bounds__(kBlock)
    batch_clear_kernel(const BatchLattice* __restrict__ lat, const BatchSolid* __restrict__ sol,
                       const Tile* __restrict__ ctiles, float4* grid_all, uint8_t* dirty_all) {
  const Tile t = ctiles[blockIdx.x];
  const Mpm m = sol[t.lattice].m;
  clear_body(m, grid_all + lat[t.lattice].off, dirty_all + sol[t.lattice].block_off,
             (long long)t.first + (threadIdx.x >> 5));
}

__global__ void __launch_bounds__(kBlock)
    batch_coupling_forces_kernel(const BatchLattice* __restrict__ lat,
                                 const BatchSolid* __restrict__ sol, const Tile* __restrict__ ptiles,
                                 ForceArgs base, float dt_ratio, int build_fraction) {
  const Tile t = ptiles[blockIdx.x];
  const ForceArgs a = scene_force_args(base, lat[t.lattice], sol[t.lattice], t.lattice, dt_ratio,
                                       build_fraction);
  coupling_forces_body<false>(a, t.first * kBlock + threadIdx.x);
}

__global__ void __launch_bounds__(kTileCells)
    batch_assemble_kernel(const BatchLattice* __restrict__ lat, const BatchSolid* __restrict__ sol,
                          const Tile* __restrict__ tiles, AssembleArgs base) {
  const Tile t = tiles[blockIdx.x];
  const AssembleArgs a = scene_assemble_args(base, lat[t.lattice], sol[t.lattice], t.lattice);
  assemble_body(a, (long long)t.first + threadIdx.x);
}

int check_solids(const fsi_batch* b) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(b->sol != nullptr, "the batch has no solids (fsi_batch_set_solids)");
  return FSI_OK;
}

}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_batch_create(const fsi_batch_lattice* lattices, int32_t count, int32_t storage,
                                int32_t arithmetic, fsi_batch** out) {
  FSI_REQUIRE(out != nullptr, "NULL output handle");
  *out = nullptr;
  FSI_REQUIRE(lattices != nullptr && count > 0, "empty batch");
  FSI_REQUIRE(storage >= FSI_STORAGE_F32 && storage <= FSI_STORAGE_BF16, "unknown storage %d",
              storage);
  FSI_REQUIRE(arithmetic == FSI_ARITH_EXACT || arithmetic == FSI_ARITH_FAST,
              "unknown arithmetic form %d", arithmetic);
  FSI_REQUIRE(storage == FSI_STORAGE_F32 || arithmetic == FSI_ARITH_FAST,
              "FP16/BF16 population storage uses the fast arithmetic form");
  std::vector<BatchLattice> host(count);
  std::vector<Tile> tiles;
  long long off = 0;
  for (int s = 0; s < count; ++s) {
    const fsi_batch_lattice& in = lattices[s];
    FSI_REQUIRE(in.nx > 4 && in.ny > 4 && in.nz > 4, "lattice %d: %dx%dx%d too small", s, in.nx,
                in.ny, in.nz);
    const long long n = (long long)in.nx * in.ny * in.nz;
    FSI_REQUIRE(19ll * n < (1ll << 31), "lattice %d too large for a batch", s);
    FSI_REQUIRE(in.cell_offset == off, "lattice %d: cell_offset %lld, expected %lld", s,
                (long long)in.cell_offset, off);
    FSI_REQUIRE(in.s[0] == 0.f && in.s[3] == 0.f && in.s[5] == 0.f && in.s[7] == 0.f,
                "lattice %d: conserved moments must have zero relaxation rate", s);
    BatchLattice& L = host[s];
    L.g = LbmGeom{in.nx, in.ny, in.nz, n};
    L.off = off;
    for (int q = 0; q < 19; ++q) {
      L.s[q] = in.s[q];
      L.sg[q] = 1.0f - 0.5f * in.s[q];
      L.shift[q] = storage == FSI_STORAGE_F32 ? 0.f : weight_of(q) * in.rho0;
    }
    L.rho0 = in.rho0;
    for (int a = 0; a < 3; ++a) L.base[a] = in.base_force[a];
    for (long long c = 0; c < n; c += kTileCells) tiles.push_back(Tile{s, (int)c});
    off += n;
  }
  FSI_REQUIRE(tiles.size() < (1u << 31), "batch has too many tiles");
  fsi_batch* b = new fsi_batch;
  b->host = host;
  b->count = count;
  b->ntiles = (int)tiles.size();
  b->storage = storage;
  b->arithmetic = arithmetic;
  b->cells = off;
  if (cudaMalloc(&b->lat, sizeof(BatchLattice) * count) != cudaSuccess ||
      cudaMalloc(&b->tiles, sizeof(Tile) * tiles.size()) != cudaSuccess ||
      cudaMemcpy(b->lat, host.data(), sizeof(BatchLattice) * count, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(b->tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    const int e = check_launch("fsi_batch_create");
    cudaFree(b->lat);
    cudaFree(b->tiles);
    delete b;
    return e ? e : FSI_ERR_CUDA;
  }
  b->step_tiles = b->tiles;
  b->nstep_tiles = b->ntiles;
  b->step_tile_cells = kTileCells;
  *out = b;
  return FSI_OK;
}

extern "C" int fsi_batch_destroy(fsi_batch* b) {
  if (!b) return FSI_OK;
  cudaFree(b->lat);
  cudaFree(b->tiles);
  if (b->step_tiles != b->tiles) cudaFree(b->step_tiles);
  cudaFree(b->sol);
  cudaFree(b->ptiles);
  cudaFree(b->ctiles);
  delete b;
  return check_launch("fsi_batch_destroy");
}

extern "C" int fsi_batch_cells(const fsi_batch* b, int64_t* cells) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(cells != nullptr, "NULL output");
  *cells = b->cells;
  return FSI_OK;
}

extern "C" int fsi_batch_lbm_flags(const fsi_batch* b, const int32_t* solid, uint32_t* flags,
                                   void* stream) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(solid && flags, "NULL array");
  batch_flags_kernel<<<b->ntiles, kTileCells, 0, as_stream(stream)>>>(b->lat, b->tiles, solid, flags);
  return check_launch("batch_flags_kernel");
}

extern "C" int fsi_batch_lbm_init(const fsi_batch* b, const float* u0, const uint32_t* flags,
                                  void* pops, float* macro, void* stream) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(u0 && flags && pops && macro, "NULL array");
  dispatch_batch<BatchInitLauncher>(b, u0, flags, pops, macro, as_stream(stream));
  return check_launch("batch_init_kernel");
}

extern "C" int fsi_batch_lbm_step(const fsi_batch* b, void* pops, float* macro, const float* force,
                                  const float* force_prev, const uint32_t* flags,
                                  int64_t steps_done, void* stream) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(pops && macro && force && flags, "NULL array");
  FSI_REQUIRE(steps_done >= 0, "steps_done must be non-negative");
  const bool fast = b->arithmetic == FSI_ARITH_FAST, odd = (steps_done & 1) != 0;
  const bool recompute = force_prev != nullptr;
  cudaStream_t s = as_stream(stream);
  switch (b->storage) {
    case FSI_STORAGE_F16:
      return batch_step_launch_f16(b->lat, b->step_tiles, b->nstep_tiles, b->step_tile_cells,
                                   b->variant, fast, odd, recompute, pops, macro, force,
                                   force_prev, flags, s);
    case FSI_STORAGE_BF16:
      return batch_step_launch_bf16(b->lat, b->step_tiles, b->nstep_tiles, b->step_tile_cells,
                                    b->variant, fast, odd, recompute, pops, macro, force,
                                    force_prev, flags, s);
    default:
      return batch_step_launch_f32(b->lat, b->step_tiles, b->nstep_tiles, b->step_tile_cells,
                                   b->variant, fast, odd, recompute, pops, macro, force,
                                   force_prev, flags, s);
  }
}

extern "C" int fsi_batch_tune(fsi_batch* b, int32_t step_tile_cells, int32_t variant) {
  if (int e = check_batch(b)) return e;
  const int lanes = b->arithmetic == FSI_ARITH_FAST ? 2 : 1;
  FSI_REQUIRE(step_tile_cells > 0 && step_tile_cells % (kStepBlock * lanes) == 0 &&
                  step_tile_cells <= 8192,
              "step tile of %d cells is not a multiple of %d (at most 8192)", step_tile_cells,
              kStepBlock * lanes);
  FSI_REQUIRE(variant >= 0 && variant <= 2, "unknown variant %d", variant);
  std::vector<Tile> tiles;
  for (int s = 0; s < b->count; ++s)
    for (long long c = 0; c < b->host[s].g.n; c += step_tile_cells) tiles.push_back(Tile{s, (int)c});
  Tile* dev = nullptr;
  if (cudaMalloc(&dev, sizeof(Tile) * tiles.size()) != cudaSuccess ||
      cudaMemcpy(dev, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    cudaFree(dev);
    return check_launch("fsi_batch_tune");
  }
  if (b->step_tiles != b->tiles) cudaFree(b->step_tiles);
  b->step_tiles = dev;
  b->nstep_tiles = (int)tiles.size();
  b->step_tile_cells = step_tile_cells;
  b->variant = variant;
  return FSI_OK;
}

extern "C" int fsi_batch_lbm_macro(const fsi_batch* b, const void* pops, const float* force,
                                   const uint32_t* flags, int64_t steps_done, float* macro,
                                   double* diag, void* stream) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(pops && force && flags && macro, "NULL array");
  cudaStream_t s = as_stream(stream);
  if (diag && cudaMemsetAsync(diag, 0, 2 * sizeof(double) * b->count, s) != cudaSuccess)
    return check_launch("memset");
  dispatch_batch<BatchMacroLauncher>(b, pops, force, flags, (int)(steps_done & 1), macro, diag, s);
  return check_launch("batch_macro_kernel");
}

extern "C" int fsi_batch_lbm_distribution(const fsi_batch* b, const void* pops,
                                          const uint32_t* flags, int64_t steps_done, float* out,
                                          void* stream) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(pops && flags && out, "NULL array");
  dispatch_batch<BatchDistLauncher>(b, pops, flags, (int)(steps_done & 1), out, as_stream(stream));
  return check_launch("batch_distribution_kernel");
}

extern "C" int fsi_batch_lbm_base_force(const fsi_batch* b, const uint32_t* flags, float* force,
                                        void* stream) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(flags && force, "NULL array");
  batch_base_force_kernel<<<b->ntiles, kTileCells, 0, as_stream(stream)>>>(b->lat, b->tiles, flags,
                                                                           force);
  return check_launch("batch_base_force_kernel");
}

extern "C" int fsi_batch_set_solids(fsi_batch* b, const fsi_batch_solid* solids, int64_t capacity,
                                    int64_t* dirty_blocks) {
  if (int e = check_batch(b)) return e;
  FSI_REQUIRE(solids != nullptr && dirty_blocks != nullptr, "NULL argument");
  FSI_REQUIRE(capacity > 0 && capacity < (1ll << 31), "capacity %lld out of range",
              (long long)capacity);
  std::vector<BatchSolid> host(b->count);
  std::vector<Tile> ptiles, ctiles;
  long long next = 0, block_off = 0;
  // make_mpm validates a descriptor against particle arrays; the batch's arrays are checked
  // per call, so stand-in (never dereferenced) pointers satisfy its NULL checks here.
  fsi_particles dummy{};
  float stand_in = 0.f;
  int32_t stand_in_i = 0;
  dummy.x = dummy.v = dummy.C = dummy.F = dummy.force = dummy.mass = dummy.volume = &stand_in;
  dummy.active = &stand_in_i;
  dummy.capacity = capacity;
  for (int s = 0; s < b->count; ++s) {
    const fsi_batch_solid& in = solids[s];
    const BatchLattice& L = b->host[s];
    FSI_REQUIRE(in.mpm.nx == L.g.nx && in.mpm.ny == L.g.ny && in.mpm.nz == L.g.nz,
                "scene %d: MPM grid differs from its lattice", s);
    FSI_REQUIRE(in.particle_offset >= next && in.particle_offset % FSI_BATCH_PARTICLE_ALIGN == 0,
                "scene %d: particle_offset %lld not aligned or overlapping", s,
                (long long)in.particle_offset);
    FSI_REQUIRE(in.particle_offset + in.mpm.num_particles <= capacity,
                "scene %d: particles beyond the capacity", s);
    BatchSolid& S = host[s];
    PView unused;
    fsi_mpm_desc d = in.mpm;
    d.num_particles = 0;
    if (int e = make_mpm(&d, &dummy, S.m, unused)) return e;
    S.m.n = (int)(in.particle_offset + in.mpm.num_particles);
    S.m.cap = capacity;
    S.block_off = block_off;
    S.c = in.coupling;
    for (long long p = in.particle_offset; p < S.m.n; p += kBlock)
      ptiles.push_back(Tile{s, (int)(p / kBlock)});
    const long long nb = (long long)S.m.nbx * S.m.nby * S.m.nbz;
    for (long long q = 0; q < nb; q += kBlock / 32) ctiles.push_back(Tile{s, (int)q});
    block_off += nb;
    next = S.m.n;
  }
  cudaFree(b->sol); cudaFree(b->ptiles); cudaFree(b->ctiles);
  b->sol = nullptr; b->ptiles = b->ctiles = nullptr;
  const size_t np = ptiles.size() ? ptiles.size() : 1;
  if (cudaMalloc(&b->sol, sizeof(BatchSolid) * b->count) != cudaSuccess ||
      cudaMalloc(&b->ptiles, sizeof(Tile) * np) != cudaSuccess ||
      cudaMalloc(&b->ctiles, sizeof(Tile) * ctiles.size()) != cudaSuccess ||
      cudaMemcpy(b->sol, host.data(), sizeof(BatchSolid) * b->count, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      (ptiles.size() && cudaMemcpy(b->ptiles, ptiles.data(), sizeof(Tile) * ptiles.size(),
                                   cudaMemcpyHostToDevice) != cudaSuccess) ||
      cudaMemcpy(b->ctiles, ctiles.data(), sizeof(Tile) * ctiles.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    const int e = check_launch("fsi_batch_set_solids");
    cudaFree(b->sol); cudaFree(b->ptiles); cudaFree(b->ctiles);
    b->sol = nullptr; b->ptiles = b->ctiles = nullptr;
    return e ? e : FSI_ERR_CUDA;
  }
  b->host_sol = host;
  b->nptiles = (int)ptiles.size();
  b->nctiles = (int)ctiles.size();
  b->capacity = capacity;
  *dirty_blocks = block_off;
  return FSI_OK;
}

extern "C" int fsi_batch_set_gamma(fsi_batch* b, const float* gamma_eff) {
  if (int e = check_solids(b)) return e;
  FSI_REQUIRE(gamma_eff != nullptr, "NULL gamma");
  for (int s = 0; s < b->count; ++s) b->host_sol[s].c.gamma_eff = gamma_eff[s];
  if (cudaMemcpy(b->sol, b->host_sol.data(), sizeof(BatchSolid) * b->count,
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return check_launch("fsi_batch_set_gamma");
  return FSI_OK;
}

namespace {
int particle_view(const fsi_batch* b, const fsi_particles* p, PView& v) {
  FSI_REQUIRE(p != nullptr, "NULL particles");
  FSI_REQUIRE(p->capacity == b->capacity, "particle capacity %lld differs from the batch's %lld",
              (long long)p->capacity, b->capacity);
  FSI_REQUIRE(p->x && p->v && p->C && p->F && p->mass && p->volume && p->active && p->force,
              "NULL particle array");
  FSI_REQUIRE((p->mu == nullptr) == (p->lam == nullptr), "per-particle mu and lam go together");
  v.x = p->x; v.v = p->v; v.C = p->C; v.F = p->F; v.mass = p->mass; v.vol = p->volume;
  v.active = p->active; v.fp = p->force; v.mu = p->mu; v.lam = p->lam;
  return FSI_OK;
}
}  // namespace

extern "C" int fsi_batch_mpm_substep(const fsi_batch* b, const fsi_particles* particles,
                                     float* grid, uint8_t* dirty, void* stream) {
  if (int e = check_solids(b)) return e;
  FSI_REQUIRE(grid && dirty, "NULL array");
  FSI_REQUIRE(((uintptr_t)grid & 15) == 0, "grid must be 16-byte aligned");
  PView P;
  if (int e = particle_view(b, particles, P)) return e;
  if (b->nptiles == 0) return FSI_OK;
  cudaStream_t s = as_stream(stream);
  float4* g4 = reinterpret_cast<float4*>(grid);
  batch_p2g_kernel<<<b->nptiles, kBlock, 0, s>>>(b->lat, b->sol, b->ptiles, P, g4, dirty);
  if (int e = check_launch("batch_p2g_kernel")) return e;
  batch_g2p_kernel<<<b->nptiles, kBlock, 0, s>>>(b->lat, b->sol, b->ptiles, P, g4);
  if (int e = check_launch("batch_g2p_kernel")) return e;
  batch_clear_kernel<<<b->nctiles, kBlock, 0, s>>>(b->lat, b->sol, b->ctiles, g4, dirty);
  return check_launch("batch_clear_kernel");
}

extern "C" int fsi_batch_coupling_forces(const fsi_batch* b, const fsi_particles* particles,
                                         const float* macro, const uint32_t* flags, float* accum,
                                         float* valid_weight, int32_t* coupling_mask,
                                         void* counters, float dt_ratio, int32_t build_fraction,
                                         void* stream) {
  if (int e = check_solids(b)) return e;
  FSI_REQUIRE(macro && flags && accum && valid_weight && coupling_mask && counters, "NULL array");
  PView P;
  if (int e = particle_view(b, particles, P)) return e;
  if (b->nptiles == 0) return FSI_OK;
  ForceArgs a{};
  a.cap = b->capacity;
  a.x = P.x; a.v = P.v; a.mass = P.mass; a.vol = P.vol; a.active = P.active; a.fp = P.fp;
  a.macro = reinterpret_cast<const float4*>(macro);
  a.flags = flags;
  a.accum = reinterpret_cast<float4*>(accum);
  a.valid_out = valid_weight;
  a.mask_out = coupling_mask;
  a.cnt = reinterpret_cast<Cnt*>(counters);
  batch_coupling_forces_kernel<<<b->nptiles, kBlock, 0, as_stream(stream)>>>(
      b->lat, b->sol, b->ptiles, a, dt_ratio, build_fraction);
  return check_launch("batch_coupling_forces_kernel");
}

extern "C" int fsi_batch_coupling_assemble(const fsi_batch* b, const uint32_t* flags, int32_t mode,
                                           float* accum, const float* macro, float* force,
                                           float* ib_force, void* counters, void* stream) {
  if (int e = check_solids(b)) return e;
  FSI_REQUIRE(flags && accum && counters, "NULL array");
  FSI_REQUIRE(!(mode & FSI_ASSEMBLE_IB) || (macro && ib_force), "IB needs macro and ib_force");
  AssembleArgs a{};
  a.flags = flags;
  a.mode = mode;
  a.accum = reinterpret_cast<float4*>(accum);
  a.macro = reinterpret_cast<const float4*>(macro);
  a.force = force;
  a.ib = ib_force;
  a.cnt = reinterpret_cast<Cnt*>(counters);
  batch_assemble_kernel<<<b->ntiles, kTileCells, 0, as_stream(stream)>>>(b->lat, b->sol, b->tiles, a);
  return check_launch("batch_assemble_kernel");
}

extern "C" int fsi_batch_run_persistent(const fsi_batch* b, const fsi_particles* particles,
                                        const fsi_batch_state* st, int64_t steps_done,
                                        int32_t steps, int32_t substeps, float dt_ratio,
                                        int32_t build_fraction, int32_t assemble_mode,
                                        int32_t prev_force, int32_t macro_fresh,
                                        int64_t wait_cycles, void* stream) {
  if (int e = check_solids(b)) return e;
  FSI_REQUIRE(st != nullptr, "NULL state");
  FSI_REQUIRE(st->pops && st->macro && st->force[0] && st->force[1] && st->flags && st->accum &&
                  st->valid_weight && st->coupling_mask && st->counters && st->grid &&
                  st->dirty && st->sync && st->error,
              "NULL array in the batch state");
  FSI_REQUIRE(((uintptr_t)st->grid & 15) == 0 && ((uintptr_t)st->accum & 15) == 0 &&
                  ((uintptr_t)st->macro & 15) == 0,
              "grid, accum and macro must be 16-byte aligned");
  FSI_REQUIRE(steps_done >= 0 && steps >= 0 && substeps > 0, "bad step counts");
  FSI_REQUIRE(prev_force == 0 || prev_force == 1, "prev_force must be 0 or 1");
  FSI_REQUIRE(!(assemble_mode & FSI_ASSEMBLE_IB) || st->ib_force, "IB needs ib_force");
  PView P;
  if (int e = particle_view(b, particles, P)) return e;
  if (steps == 0) return FSI_OK;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(st->sync, 0, sizeof(uint32_t), s) != cudaSuccess) return check_launch("memset");
  PersistArgs a{};
  a.lat = b->lat;
  a.sol = b->sol;
  a.cell_tiles = b->tiles;
  a.ncell_tiles = b->ntiles;
  a.step_tiles = b->step_tiles;
  a.nstep_tiles = b->nstep_tiles;
  a.step_tile_cells = b->step_tile_cells;
  a.ptiles = b->ptiles;
  a.nptiles = b->nptiles;
  a.ctiles = b->ctiles;
  a.nctiles = b->nctiles;
  a.count = b->count;
  a.P = P;
  a.fa.cap = b->capacity;
  a.fa.x = P.x; a.fa.v = P.v; a.fa.mass = P.mass; a.fa.vol = P.vol; a.fa.active = P.active;
  a.fa.fp = P.fp;
  a.fa.macro = reinterpret_cast<const float4*>(st->macro);
  a.fa.flags = st->flags;
  a.fa.accum = reinterpret_cast<float4*>(st->accum);
  a.fa.valid_out = st->valid_weight;
  a.fa.mask_out = st->coupling_mask;
  a.fa.cnt = reinterpret_cast<Cnt*>(st->counters);
  a.aa.flags = st->flags;
  a.aa.mode = assemble_mode;
  a.aa.accum = reinterpret_cast<float4*>(st->accum);
  a.aa.macro = reinterpret_cast<const float4*>(st->macro);
  a.aa.force = nullptr;  // the step's buffer, set in the kernel
  a.aa.ib = st->ib_force;
  a.aa.cnt = reinterpret_cast<Cnt*>(st->counters);
  a.pops = st->pops;
  a.macro = st->macro;
  a.force[0] = st->force[0];
  a.force[1] = st->force[1];
  a.flags = st->flags;
  a.grid = reinterpret_cast<float4*>(st->grid);
  a.dirty = st->dirty;
  a.sync = st->sync;
  a.err = st->error;
  a.steps_done = steps_done;
  a.steps = steps;
  a.substeps = substeps;
  a.dt_ratio = dt_ratio;
  a.build_fraction = build_fraction;
  a.prev = prev_force;
  a.macro_fresh = macro_fresh;
  FSI_REQUIRE(wait_cycles >= 0, "wait_cycles must be non-negative");
  a.wait_cycles = wait_cycles > 0 ? wait_cycles : (1ll << 31);  // about a second
  const bool fast = b->arithmetic == FSI_ARITH_FAST;
  switch (b->storage) {
    case FSI_STORAGE_F16: return batch_persist_launch_f16(&a, fast, s);
    case FSI_STORAGE_BF16: return batch_persist_launch_bf16(&a, fast, s);
    default: return batch_persist_launch_f32(&a, fast, s);
  }
}
