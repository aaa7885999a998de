// Cell-sorted, atomic-free MLS-MPM substep on sm_103a, with the penalty coupling's spread
// folded into the scatter (reference: fsi/mpm3d.py:189-328, fsi/coupling.py:332-406).
//
// Every substep re-sorts the particles by base cell b = trunc(x / dx - 0.5) and then sums
// each grid node's contributions in one fixed order, so the result does not depend on
// thread scheduling:
//   1. count:   per particle, its base cell's slot (atomic) and its 8^3 cell tile's count.
//   2. tiles:   one block scans the tile counts (tile starts), lists the non-empty cell tiles
//               and the node tiles they touch, and resets the counters for the next substep.
//   3. cells:   per non-empty tile, a block scans its 512 cell counts (cell starts).
//   4. scatter: per particle, its index into its cell's range (arrival order).
//   5. prepare: per particle, its rank in the cell (ascending particle index) gives its
//               sorted position; the coupling force (interpolated fluid velocity, penalty,
//               clipping), F <- (I + dt C) F, the stress and the affine term are computed
//               and the particle's terms (weights, affine, momentum, force, valid weight)
//               are written to the payload at the sorted position.
//   6. tile:    one block per 8^3 node tile streams the 10 x-planes of its 10^3-cell region
//               (the tile's cells and two layers below it). For each non-empty cell a warp
//               forms the 27 cell partials S_b(o), lane o summing the cell's particles in
//               ascending index; then each tile node adds its partials in ascending cell
//               index into a ring of three node planes in shared memory. A completed node
//               plane is stored with plain stores: momentum/mass to the grid and the
//               reaction force / solid fraction to the lattice accumulator. No atomics, and
//               no grid clear: the tiles write every node any stencil touches.
//   7. g2p:     grid update and G2P per particle in sorted order (compact CTA boxes).
// The contributions are the reference's expressions term for term; only the order of the
// additions is fixed, and the oracle restates it (oracle/fsi_oracle.cpp, p2g_cell_order).
#include <cuda_runtime.h>

#include <cstdint>

#include "coupling_core.cuh"
#include "fsi_common.cuh"
#include "mpm_core.cuh"

namespace fsi {
namespace {

constexpr int kT = 8;                  // tile edge (cells and nodes)
constexpr int kTC = kT * kT * kT;      // cells per cell tile
constexpr int kRE = kT + 2;            // region edge of a node tile, in cells
constexpr int kRP = kRE * kRE;         // region cells per x-plane
constexpr int kTN = kT * kT;           // nodes per x-plane of a node tile
constexpr int kPay = 8;                // payload float4 per particle
constexpr int kTileThreads = 256;
constexpr int kScanThreads = 1024;

struct SortGeo {
  int ctx, cty, ctz;  // cell tiles per axis over base cells [-2, n-1] (shifted by +2)
  int ntiles;
  int ntx, nty, ntz;  // node tiles per axis over nodes [0, n)
  int nntiles;
};

struct Work {
  int32_t* cell_count;  // [ntiles * 512], zero between substeps
  int32_t* cell_start;  // [ntiles * 512]
  int32_t* tile_count;  // [ntiles], zero between substeps
  int32_t* tile_start;  // [ntiles + 1]
  int32_t* cell_tiles;  // [ntiles] non-empty cell tiles
  int32_t* node_tiles;  // [nntiles] node tiles touched by some stencil
  int32_t* header;      // [0] cell tiles, [1] node tiles, [2] particles outside, [3] tile cursor
  int32_t* key;         // [cap] tile * 512 + local cell, or -1
  int32_t* slot;        // [cap]
  int32_t* unsorted;    // [cap]
  int32_t* sorted;      // [cap]
  float4* payload;      // [cap * kPay]
};

SortGeo sort_geo(int nx, int ny, int nz) {
  SortGeo g;
  g.ctx = (nx + 2 + kT - 1) / kT;
  g.cty = (ny + 2 + kT - 1) / kT;
  g.ctz = (nz + 2 + kT - 1) / kT;
  g.ntiles = g.ctx * g.cty * g.ctz;
  g.ntx = (nx + kT - 1) / kT;
  g.nty = (ny + kT - 1) / kT;
  g.ntz = (nz + kT - 1) / kT;
  g.nntiles = g.ntx * g.nty * g.ntz;
  return g;
}

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Carves the workspace (base may be NULL to size it); returns the bytes needed.
size_t carve(const SortGeo& g, long long cap, char* base, Work& w) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  w.cell_count = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * kTC * 4));
  w.cell_start = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * kTC * 4));
  w.tile_count = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * 4));
  w.tile_start = reinterpret_cast<int32_t*>(take((size_t)(g.ntiles + 1) * 4));
  w.cell_tiles = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * 4));
  w.node_tiles = reinterpret_cast<int32_t*>(take((size_t)g.nntiles * 4));
  w.header = reinterpret_cast<int32_t*>(take(64));
  w.key = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.slot = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.unsorted = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.sorted = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.payload = reinterpret_cast<float4*>(take((size_t)cap * kPay * sizeof(float4)));
  return off;
}

// ------------------------------------------------------------------ scans --
// Exclusive scan over the block (blockDim.x a multiple of 32, at most 1024 threads).
// `ws` is 32 ints of shared scratch; *total receives the block's sum.
__device__ int block_excl_scan(int v, int* ws, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int s = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    ws[lane] = s;
  }
  __syncthreads();
  const int excl = incl - v + (wid > 0 ? ws[wid - 1] : 0);
  *total = ws[nw - 1];
  __syncthreads();
  return excl;
}

// 1. Base cell slot and tile count of every active particle; zeroes the step counters.
__global__ void __launch_bounds__(kBlock) sort_count_kernel(Mpm m, PView P, SortGeo g, Work w,
                                                            Cnt* cnt) {
  const int p = blockIdx.x * kBlock + threadIdx.x;
  if (p == 0) {
    w.header[2] = 0;
    if (cnt) { cnt->unsupported = 0; cnt->partial = 0; cnt->clipped = 0; }
  }
  int key = -1, tile = -1, slot = 0;
  if (p < m.n && P.active[p] != 0) {
    float x[3];
    load_particle_x(P, m.cap, p, x);
    int base[3];
    float fx[3];
    base_fx(m, x, base, fx);
    if (base[0] >= -2 && base[0] < m.nx && base[1] >= -2 && base[1] < m.ny && base[2] >= -2 &&
        base[2] < m.nz) {
      const int s0 = base[0] + 2, s1 = base[1] + 2, s2 = base[2] + 2;
      tile = ((s0 >> 3) * g.cty + (s1 >> 3)) * g.ctz + (s2 >> 3);
      key = tile * kTC + (((s0 & 7) << 6) | ((s1 & 7) << 3) | (s2 & 7));
      slot = atomicAdd(&w.cell_count[key], 1);
    }
  }
  const unsigned peers = __match_any_sync(0xffffffffu, tile);
  if (tile >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&w.tile_count[tile], __popc(peers));
  if (p < m.n) {
    w.key[p] = key;
    w.slot[p] = slot;
  }
}

// 2. Tile starts, the lists of non-empty cell tiles and touched node tiles (ascending), and
// the reset of the tile counts and the tile cursor. One block.
__global__ void __launch_bounds__(kScanThreads) sort_tile_scan_kernel(SortGeo g, Work w) {
  __shared__ int ws[32];
  __shared__ int carry[2];
  const int t = threadIdx.x;
  if (t == 0) { carry[0] = 0; carry[1] = 0; }
  __syncthreads();
  // Cell tiles, in chunks of one entry per thread.
  for (int base = 0; base < g.ntiles; base += kScanThreads) {
    const int i = base + t;
    const int c = i < g.ntiles ? w.tile_count[i] : 0;
    int tot, tot_a;
    const int ex = block_excl_scan(c, ws, &tot);
    const int ea = block_excl_scan(c > 0 ? 1 : 0, ws, &tot_a);
    if (i < g.ntiles) {
      w.tile_start[i] = carry[0] + ex;
      if (c > 0) w.cell_tiles[carry[1] + ea] = i;
      w.tile_count[i] = 0;
    }
    __syncthreads();
    if (t == 0) { carry[0] += tot; carry[1] += tot_a; }
    __syncthreads();
  }
  if (t == 0) {
    w.tile_start[g.ntiles] = carry[0];
    w.header[0] = carry[1];
    w.header[3] = 0;
    carry[1] = 0;
  }
  __syncthreads();
  // Node tile (a, b, c) receives from cell tiles (a..a+1, b..b+1, c..c+1).
  for (int base = 0; base < g.nntiles; base += kScanThreads) {
    const int i = base + t;
    int act = 0;
    if (i < g.nntiles) {
      const int a = i / (g.nty * g.ntz), b = (i / g.ntz) % g.nty, c = i % g.ntz;
      for (int da = 0; da < 2; ++da)
        for (int db = 0; db < 2; ++db)
          for (int dc = 0; dc < 2; ++dc) {
            const int ta = a + da, tb = b + db, tc = c + dc;
            if (ta >= g.ctx || tb >= g.cty || tc >= g.ctz) continue;
            const int ti = (ta * g.cty + tb) * g.ctz + tc;
            act |= w.tile_start[ti + 1] > w.tile_start[ti];
          }
    }
    int tot;
    const int ex = block_excl_scan(act, ws, &tot);
    if (act) w.node_tiles[carry[1] + ex] = i;
    __syncthreads();
    if (t == 0) carry[1] += tot;
    __syncthreads();
  }
  if (t == 0) w.header[1] = carry[1];
}

// 3. Cell starts of each non-empty cell tile (one block of 512 threads per tile); the cell
// counts are reset for the next substep.
__global__ void __launch_bounds__(kTC) sort_cell_scan_kernel(Work w) {
  __shared__ int ws[32];
  const int n = w.header[0];
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const int t = w.cell_tiles[i];
    const long long idx = (long long)t * kTC + threadIdx.x;
    const int c = w.cell_count[idx];
    int tot;
    const int ex = block_excl_scan(c, ws, &tot);
    w.cell_start[idx] = w.tile_start[t] + ex;
    w.cell_count[idx] = 0;
  }
}

// 4. Each particle into its cell's range, in arrival order.
__global__ void __launch_bounds__(kBlock) sort_scatter_kernel(int n, Work w) {
  const int p = blockIdx.x * kBlock + threadIdx.x;
  if (p >= n) return;
  const int key = w.key[p];
  if (key >= 0) w.unsorted[w.cell_start[key] + w.slot[p]] = p;
}

__device__ __forceinline__ int cell_end(const Work& w, int key) {
  return (key & (kTC - 1)) < kTC - 1 ? w.cell_start[key + 1] : w.tile_start[(key >> 9) + 1];
}

// 5. Sorted position, coupling force, stress and payload of every active particle.
// Payload (float4 x 8): (wx0 wx1 wx2 wy0) (wy1 wy2 wz0 wz1) (wz2 fx0 fx1 fx2) (A0..A3)
// (A4..A7) (A8 mv0 mv1 mv2) (f0 f1 f2 m) (valid vol coupled 0).
template <bool kCoupled, bool kGatherAhead>
__global__ void __launch_bounds__(kBlock) sorted_prepare_kernel(Mpm m, PView P, SortGeo g, Work w,
                                                                ForceArgs fa) {
  const int p = blockIdx.x * kBlock + threadIdx.x;
  const long long cap = m.cap;
  bool partial = false, clipped = false, unsupported = false;
  if (p < m.n) {
    if (P.active[p] == 0) {
      if (kCoupled) { P.fp[p] = 0.f; P.fp[cap + p] = 0.f; P.fp[2 * cap + p] = 0.f; }
    } else {
      const int key = w.key[p];
      int pos;
      if (key >= 0) {
        const int start = w.cell_start[key], end = cell_end(w, key);
        int rank = 0;
        for (int s = start; s < end; ++s) rank += w.unsorted[s] < p;
        pos = start + rank;
      } else {
        pos = w.tile_start[g.ntiles] + atomicAdd(&w.header[2], 1);
      }
      w.sorted[pos] = p;
      float pf[3], valid = 0.f;
      bool coupled = false;
      if (kCoupled) {
        int cb[3];
        float wv[3][3];
        uint32_t usable;
        coupled = coupling_particle<kGatherAhead>(fa, p, cb, wv, usable, valid, pf, partial,
                                                  clipped, unsupported);
        if (!coupled) pf[0] = pf[1] = pf[2] = 0.f;
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) pf[a] = P.fp[a * cap + p];
      }
      float affine[9], mass;
      p2g_stress_affine(m, P, p, affine, mass);
      if (key >= 0) {
        float x[3];
        load_particle_x(P, cap, p, x);
        int base[3];
        float fx[3];
        base_fx(m, x, base, fx);
        float wv[3][3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
#pragma unroll
          for (int i = 0; i < 3; ++i) wv[ax][i] = bspline_w(fx[ax], i);
        float mv[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) mv[a] = __fmul_rn(mass, P.v[a * cap + p]);
        float4* o = w.payload + (long long)pos * kPay;
        o[0] = make_float4(wv[0][0], wv[0][1], wv[0][2], wv[1][0]);
        o[1] = make_float4(wv[1][1], wv[1][2], wv[2][0], wv[2][1]);
        o[2] = make_float4(wv[2][2], fx[0], fx[1], fx[2]);
        o[3] = make_float4(affine[0], affine[1], affine[2], affine[3]);
        o[4] = make_float4(affine[4], affine[5], affine[6], affine[7]);
        o[5] = make_float4(affine[8], mv[0], mv[1], mv[2]);
        o[6] = make_float4(pf[0], pf[1], pf[2], mass);
        o[7] = make_float4(valid, P.vol[p], coupled ? 1.f : 0.f, 0.f);
      }
    }
  }
  if (kCoupled) {
    warp_count(&fa.cnt->unsupported, unsupported);
    warp_count(&fa.cnt->partial, partial);
    warp_count(&fa.cnt->clipped, clipped);
  }
}

template <bool kCoupled>
struct TileSmem {
  static constexpr int kNC = kCoupled ? 2 : 1;  // float4 per partial: grid (+ coupling)
  static constexpr size_t kBytes =
      (size_t)(kRP * 27 + 3 * kTN) * kNC * sizeof(float4) + (3 * kRP + 4) * sizeof(int);
};

__device__ __forceinline__ float sel3(int i, float a, float b, float c) {
  return i == 0 ? a : (i == 1 ? b : c);
}

// 6. The scatter of one 8^3 node tile per loop iteration (tiles taken from a cursor).
template <bool kCoupled>
__global__ void __launch_bounds__(kTileThreads, 2) sorted_tile_kernel(Mpm m, SortGeo g, Work w,
                                                                      float4* __restrict__ grid,
                                                                      fsi_coupling_desc cd,
                                                                      const uint32_t* __restrict__ flags,
                                                                      float4* __restrict__ accum) {
  constexpr int NC = TileSmem<kCoupled>::kNC;
  extern __shared__ float4 smem[];
  float4* S = smem;                                            // [kRP * 27][NC]
  float4* ring = S + kRP * 27 * NC;                            // [3 * kTN][NC]
  int* cstart = reinterpret_cast<int*>(ring + 3 * kTN * NC);   // [kRP]
  int* ccount = cstart + kRP;                                  // [kRP]
  int* cflag = ccount + kRP;                                   // [kRP]
  int* cursor = cflag + kRP;                                   // [1]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (;;) {
    if (tid == 0) cursor[0] = atomicAdd(&w.header[3], 1);
    __syncthreads();
    const int it = cursor[0];
    if (it >= w.header[1]) break;
    const int t = w.node_tiles[it];
    const int n0x = (t / (g.nty * g.ntz)) * kT, n0y = ((t / g.ntz) % g.nty) * kT,
              n0z = (t % g.ntz) * kT;
    // This thread's node column (Phase B / init / flush): yz = tid % 64.
    const int yz = tid & (kTN - 1);
    const int nj = n0y + (yz >> 3), nk = n0z + (yz & 7);
    const bool col_in = nj < m.ny && nk < m.nz;
    for (int ci = n0x - 2; ci <= n0x + kT - 1; ++ci) {
      // Node plane ci + 2 receives its first partials from cell plane ci.
      if (tid < kTN) {
        const int ni = ci + 2;
        if (ni >= n0x && ni < n0x + kT && ni < m.nx && col_in) {
          float4* r = ring + ((ni % 3) * kTN + yz) * NC;
          r[0] = zero4;
          if (kCoupled) r[1] = accum[node_index(m, ni, nj, nk)];
        }
      }
      // Particle ranges of the region's cells in this plane.
      if (tid < kRP) {
        const int cj = n0y - 2 + tid / kRE, ck = n0z - 2 + tid % kRE;
        int start = 0, count = 0;
        const int s0 = ci + 2, s1 = cj + 2, s2 = ck + 2;
        if (s0 < m.nx + 2 && s1 < m.ny + 2 && s2 < m.nz + 2) {
          const int tile = ((s0 >> 3) * g.cty + (s1 >> 3)) * g.ctz + (s2 >> 3);
          if (w.tile_start[tile + 1] > w.tile_start[tile]) {
            const int key = tile * kTC + (((s0 & 7) << 6) | ((s1 & 7) << 3) | (s2 & 7));
            start = w.cell_start[key];
            count = cell_end(w, key) - start;
          }
        }
        cstart[tid] = start;
        ccount[tid] = count;
        cflag[tid] = 0;
      }
      __syncthreads();
      // Phase A: cell partials, one warp per cell, lane o = 9 ox + 3 oy + oz.
      {
        const int ox = lane / 9, oy = (lane / 3) % 3, oz = lane % 3;
        const int ni = ci + ox;
        const bool ni_in = lane < 27 && ni >= n0x && ni < n0x + kT && ni < m.nx;
        for (int q = warp; q < kRP; q += kTileThreads / 32) {
          const int cnt = ccount[q];
          if (cnt == 0) continue;
          const int cj = n0y - 2 + q / kRE, ck = n0z - 2 + q % kRE;
          const int nnj = cj + oy, nnk = ck + oz;
          const bool in_tile = ni_in && nnj >= n0y && nnj < n0y + kT && nnj < m.ny &&
                               nnk >= n0z && nnk < n0z + kT && nnk < m.nz;
          bool fluid = false;
          if (kCoupled && in_tile) fluid = !(flags[node_index(m, ni, nnj, nnk)] & kFlagSolid);
          float am[4] = {0.f, 0.f, 0.f, 0.f}, ac[4] = {0.f, 0.f, 0.f, 0.f};
          bool any_coupled = false;
          const float4* pl = w.payload + (long long)cstart[q] * kPay;
          for (int s = 0; s < cnt; ++s, pl += kPay) {
            float4 r[kPay];
#pragma unroll
            for (int c = 0; c < kPay; ++c) r[c] = pl[c];
            const bool coupled = kCoupled && r[7].z != 0.f;
            any_coupled |= coupled;
            if (!in_tile) continue;
            const float wx = sel3(ox, r[0].x, r[0].y, r[0].z);
            const float wy = sel3(oy, r[0].w, r[1].x, r[1].y);
            const float wz = sel3(oz, r[1].z, r[1].w, r[2].x);
            const float wgt = __fmul_rn(__fmul_rn(wx, wy), wz);
            const float d0 = __fmul_rn(__fsub_rn((float)ox, r[2].y), m.dx);
            const float d1 = __fmul_rn(__fsub_rn((float)oy, r[2].z), m.dx);
            const float d2 = __fmul_rn(__fsub_rn((float)oz, r[2].w), m.dx);
            const float A[9] = {r[3].x, r[3].y, r[3].z, r[3].w, r[4].x, r[4].y, r[4].z, r[4].w, r[5].x};
            const float mv[3] = {r[5].y, r[5].z, r[5].w};
            const float pf[3] = {r[6].x, r[6].y, r[6].z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              const float ad = dot3r(A[3 * a], A[3 * a + 1], A[3 * a + 2], d0, d1, d2);
              const float dtf = __fmul_rn(m.dt, pf[a]);
              am[a] = __fadd_rn(am[a], __fmul_rn(wgt, __fadd_rn(__fadd_rn(mv[a], ad), dtf)));
            }
            am[3] = __fadd_rn(am[3], __fmul_rn(wgt, r[6].w));
            if (kCoupled && coupled && fluid) {
              const float4 tc = coupling_spread_terms(cd, wgt, r[7].x, pf, r[7].y);
              ac[0] = __fadd_rn(ac[0], tc.x);
              ac[1] = __fadd_rn(ac[1], tc.y);
              ac[2] = __fadd_rn(ac[2], tc.z);
              if (cd.build_fraction) ac[3] = __fadd_rn(ac[3], tc.w);
            }
          }
          if (in_tile) {
            S[(q * 27 + lane) * NC] = make_float4(am[0], am[1], am[2], am[3]);
            if (kCoupled) S[(q * 27 + lane) * NC + 1] = make_float4(ac[0], ac[1], ac[2], ac[3]);
          }
          if (lane == 0 && any_coupled) cflag[q] = 1;
        }
      }
      __syncthreads();
      // Phase B: node (ci + ox, nj, nk) adds the partials of its 9 cells in plane ci in
      // ascending cell index, i.e. (oy, oz) from (2, 2) down to (0, 0).
      if (tid < 3 * kTN) {
        const int ox = tid / kTN, ni = ci + ox;
        if (ni >= n0x && ni < n0x + kT && ni < m.nx && col_in) {
          float4* r = ring + ((ni % 3) * kTN + yz) * NC;
          float4 rm = r[0], rc = kCoupled ? r[1] : zero4;
          const bool nfluid = kCoupled && !(flags[node_index(m, ni, nj, nk)] & kFlagSolid);
          for (int oy = 2; oy >= 0; --oy)
            for (int oz = 2; oz >= 0; --oz) {
              const int q = ((yz >> 3) + 2 - oy) * kRE + ((yz & 7) + 2 - oz);
              const int o = ox * 9 + oy * 3 + oz;
              if (ccount[q] > 0) {
                const float4 sm = S[(q * 27 + o) * NC];
                rm.x = __fadd_rn(rm.x, sm.x);
                rm.y = __fadd_rn(rm.y, sm.y);
                rm.z = __fadd_rn(rm.z, sm.z);
                rm.w = __fadd_rn(rm.w, sm.w);
              }
              if (kCoupled && nfluid && cflag[q] != 0) {
                const float4 sc = S[(q * 27 + o) * NC + 1];
                rc.x = __fadd_rn(rc.x, sc.x);
                rc.y = __fadd_rn(rc.y, sc.y);
                rc.z = __fadd_rn(rc.z, sc.z);
                if (cd.build_fraction) rc.w = __fadd_rn(rc.w, sc.w);
              }
            }
          r[0] = rm;
          if (kCoupled) r[1] = rc;
        }
      }
      __syncthreads();
      // Node plane ci is complete: store it.
      if (tid < kTN && ci >= n0x && ci < m.nx && col_in) {
        const float4* r = ring + ((ci % 3) * kTN + yz) * NC;
        const long long node = node_index(m, ci, nj, nk);
        grid[node] = r[0];
        if (kCoupled) accum[node] = r[1];
      }
    }
    __syncthreads();
  }
}

// 7. Grid update + G2P of the particles in sorted order.
__global__ void __launch_bounds__(kBlock) sorted_g2p_kernel(Mpm m, PView P, SortGeo g, Work w,
                                                            const float4* __restrict__ grid) {
  const int s = blockIdx.x * kBlock + threadIdx.x;
  const int total = w.tile_start[g.ntiles] + w.header[2];
  const int p = s < total ? w.sorted[s] : m.n;  // m.n: no particle
  g2p_body(m, P, grid, p);
}

int num_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      sms = v;
    else
      sms = 152;
  }
  return sms;
}

// Opts the tile kernel into its dynamic shared memory, once per device.
template <bool kCoupled>
int tile_smem_attr() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("cudaGetDevice");
  if (dev < 0 || dev >= 64 || !done[dev]) {
    if (cudaFuncSetAttribute(sorted_tile_kernel<kCoupled>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)TileSmem<kCoupled>::kBytes) != cudaSuccess)
      return check_launch("cudaFuncSetAttribute(sorted_tile_kernel)");
    if (dev >= 0 && dev < 64) done[dev] = true;
  }
  return FSI_OK;
}

int check_workspace(const Mpm& m, void* work, int64_t work_bytes, SortGeo& g, Work& w) {
  FSI_REQUIRE(work, "NULL workspace");
  FSI_REQUIRE(((uintptr_t)work & 255) == 0, "workspace must be 256-byte aligned");
  g = sort_geo(m.nx, m.ny, m.nz);
  FSI_REQUIRE((long long)g.ntiles * kTC < (1ll << 31), "grid %dx%dx%d too large for the sort",
              m.nx, m.ny, m.nz);
  const size_t need = carve(g, m.cap, reinterpret_cast<char*>(work), w);
  FSI_REQUIRE(work_bytes >= (int64_t)need, "workspace of %lld bytes, %lld needed",
              (long long)work_bytes, (long long)need);
  return FSI_OK;
}

// The seven launches of a sorted substep (kCoupled: with the coupling folded in).
template <bool kCoupled>
int sorted_substep(const Mpm& m, const PView& P, const SortGeo& g, const Work& w, float4* grid,
                   const ForceArgs& fa, cudaStream_t s) {
  if (int e = tile_smem_attr<kCoupled>()) return e;
  const unsigned pg = grid_for(m.n, kBlock);
  sort_count_kernel<<<pg, kBlock, 0, s>>>(m, P, g, w, kCoupled ? fa.cnt : nullptr);
  if (int e = check_launch("sort_count_kernel")) return e;
  sort_tile_scan_kernel<<<1, kScanThreads, 0, s>>>(g, w);
  if (int e = check_launch("sort_tile_scan_kernel")) return e;
  const int sms = num_sms();
  sort_cell_scan_kernel<<<g.ntiles < 4 * sms ? g.ntiles : 4 * sms, kTC, 0, s>>>(w);
  if (int e = check_launch("sort_cell_scan_kernel")) return e;
  sort_scatter_kernel<<<pg, kBlock, 0, s>>>(m.n, w);
  if (int e = check_launch("sort_scatter_kernel")) return e;
  // Few particles (under two CTAs per SM): latency-bound, so the coupling's stencil loads go
  // out together.
  if (m.n < 2 * sms * kBlock)
    sorted_prepare_kernel<kCoupled, true><<<pg, kBlock, 0, s>>>(m, P, g, w, fa);
  else
    sorted_prepare_kernel<kCoupled, false><<<pg, kBlock, 0, s>>>(m, P, g, w, fa);
  if (int e = check_launch("sorted_prepare_kernel")) return e;
  const int tb = g.nntiles < 2 * sms ? g.nntiles : 2 * sms;
  sorted_tile_kernel<kCoupled><<<tb, kTileThreads, TileSmem<kCoupled>::kBytes, s>>>(
      m, g, w, grid, fa.c, fa.flags, fa.accum);
  if (int e = check_launch("sorted_tile_kernel")) return e;
  sorted_g2p_kernel<<<pg, kBlock, 0, s>>>(m, P, g, w, grid);
  return check_launch("sorted_g2p_kernel");
}

}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_mpm_workspace_bytes(const fsi_mpm_desc* d, int64_t capacity, int64_t* bytes) {
  FSI_REQUIRE(d && bytes, "NULL argument");
  FSI_REQUIRE(d->nx > 4 && d->ny > 4 && d->nz > 4, "grid %dx%dx%d too small", d->nx, d->ny, d->nz);
  FSI_REQUIRE(capacity >= 0 && capacity < (1ll << 31), "capacity %lld out of range",
              (long long)capacity);
  const SortGeo g = sort_geo(d->nx, d->ny, d->nz);
  FSI_REQUIRE((long long)g.ntiles * kTC < (1ll << 31), "grid %dx%dx%d too large for the sort",
              d->nx, d->ny, d->nz);
  Work w;
  *bytes = (int64_t)carve(g, capacity, nullptr, w);
  return FSI_OK;
}

extern "C" int fsi_mpm_substep_sorted(const fsi_mpm_desc* d, const fsi_particles* parts,
                                      float* grid, void* work, int64_t work_bytes, void* stream) {
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  FSI_REQUIRE(grid, "NULL grid");
  FSI_REQUIRE(((uintptr_t)grid & 15) == 0, "grid must be 16-byte aligned");
  SortGeo g;
  Work w;
  if (int e = check_workspace(m, work, work_bytes, g, w)) return e;
  if (m.n == 0) return FSI_OK;
  ForceArgs fa{};
  return sorted_substep<false>(m, P, g, w, reinterpret_cast<float4*>(grid), fa, as_stream(stream));
}

extern "C" int fsi_coupled_substep(const fsi_coupling_desc* c, const fsi_mpm_desc* d,
                                   const fsi_particles* parts, const float* macro,
                                   const uint32_t* flags, float* accum, float* valid_weight,
                                   int32_t* coupling_mask, void* counters, float* grid, void* work,
                                   int64_t work_bytes, void* stream) {
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  FSI_REQUIRE(c, "NULL coupling descriptor");
  FSI_REQUIRE(macro && flags && accum && valid_weight && coupling_mask && counters && grid,
              "NULL array");
  FSI_REQUIRE(((uintptr_t)grid & 15) == 0 && ((uintptr_t)accum & 15) == 0 &&
                  ((uintptr_t)macro & 15) == 0,
              "grid, accum and macro must be 16-byte aligned");
  SortGeo g;
  Work w;
  if (int e = check_workspace(m, work, work_bytes, g, w)) return e;
  if (m.n == 0) return FSI_OK;
  ForceArgs fa;
  fa.c = *c;
  fa.g = Geo{m.nx, m.ny, m.nz, (long long)m.nx * m.ny * m.nz};
  fa.n = m.n;
  fa.cap = m.cap;
  fa.x = P.x; fa.v = P.v; fa.mass = P.mass; fa.vol = P.vol; fa.active = P.active; fa.fp = P.fp;
  fa.macro = reinterpret_cast<const float4*>(macro);
  fa.flags = flags;
  fa.accum = reinterpret_cast<float4*>(accum);
  fa.valid_out = valid_weight;
  fa.mask_out = coupling_mask;
  fa.cnt = reinterpret_cast<Cnt*>(counters);
  return sorted_substep<true>(m, P, g, w, reinterpret_cast<float4*>(grid), fa, as_stream(stream));
}
