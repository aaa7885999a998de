// Cell-sorted, atomic-free MLS-MPM substep on sm_103a, with the penalty coupling's spread
// folded into the scatter (reference: fsi/mpm3d.py:189-328, fsi/coupling.py:332-406).
//
// Every substep re-sorts the particles by base cell b = trunc(x / dx - 0.5) and then sums
// each grid node's contributions in one fixed order, so the result does not depend on
// thread scheduling:
//   1. count:    per particle, its base cell's slot (atomic), its 8^3 cell tile's count and a
//                mark on the node tiles its stencil touches.
//   2. tiles:    a two-pass scan of the tile counts (tile starts); the non-empty cell tiles and
//                the marked node tiles are listed, and counts and marks reset for the next
//                substep.
//   3. cells:    per non-empty tile, a block scans its 512 cell counts (cell starts).
//   4. scatter:  per particle, its index into its cell's range (arrival order).
//   5. prepare:  per particle, its rank in the cell (ascending particle index) gives its
//                sorted position; the coupling force (interpolated fluid velocity, penalty,
//                clipping), F <- (I + dt C) F, the stress and the affine term are computed
//                and the particle's terms (weights, affine, momentum, force, valid weight)
//                are written to the payload at the sorted position.
//   6. partials: per non-empty cell b and stencil offset o, the sum of the cell's particles'
//                contributions to node b + o in ascending particle index (and, coupled, the
//                reaction / solid-fraction sum of its coupled particles): one block per
//                non-empty cell tile, a warp per z-run of three cells, particles staged in
//                shared memory by asynchronous copies one chunk ahead of the arithmetic.
//   7. nodes:    each node of a touched 8^3 node tile adds its cells' partials in ascending
//                cell index: momentum/mass into the grid from zero, the coupling partials onto
//                the lattice accumulator. Plain stores, no atomics, and no grid clear: the
//                node tiles cover every node a stencil touches.
//   8. g2p:      grid update and G2P per particle (storage order, coalesced).
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
  int32_t* cell_count;    // [ntiles * 512], zero between substeps
  int32_t* cell_start;    // [ntiles * 512]
  int32_t* cell_row;      // [ntiles * 512] first sorted position of a non-empty cell, else -1
  int32_t* tile_count;    // [ntiles], zero between substeps
  int32_t* tile_start;    // [ntiles + 1]
  int32_t* chunk_sum;     // [ntiles / 1024 + 1] tile counts per scan chunk
  int32_t* cell_tiles;    // [ntiles] non-empty cell tiles
  int32_t* node_tiles;    // [nntiles] node tiles touched by some stencil
  uint8_t* node_flag;     // [nntiles] touched this substep, zero between substeps
  int32_t* header;        // [0] cell tiles, [1] node tiles, [4] partials work cursor
  int32_t* key;           // [cap] tile * 512 + local cell, or -1
  int32_t* slot;          // [cap]
  int32_t* unsorted;      // [cap]
  float4* payload;        // [cap * kPay]
  float4* partial;        // [cap * 27 * 2] cell partials at the cell's first sorted position
  uint8_t* cell_coupled;  // [cap] the cell (at its first sorted position) has coupled particles
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
  w.cell_row = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * kTC * 4));
  w.tile_count = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * 4));
  w.tile_start = reinterpret_cast<int32_t*>(take((size_t)(g.ntiles + 1) * 4));
  w.chunk_sum = reinterpret_cast<int32_t*>(take((size_t)(g.ntiles / kScanThreads + 1) * 4));
  w.cell_tiles = reinterpret_cast<int32_t*>(take((size_t)g.ntiles * 4));
  w.node_tiles = reinterpret_cast<int32_t*>(take((size_t)g.nntiles * 4));
  w.node_flag = reinterpret_cast<uint8_t*>(take((size_t)g.nntiles));
  w.header = reinterpret_cast<int32_t*>(take(64));
  w.key = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.slot = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.unsorted = reinterpret_cast<int32_t*>(take((size_t)cap * 4));
  w.payload = reinterpret_cast<float4*>(take((size_t)cap * kPay * sizeof(float4)));
  w.partial = reinterpret_cast<float4*>(take((size_t)cap * 27 * 2 * sizeof(float4)));
  w.cell_coupled = reinterpret_cast<uint8_t*>(take((size_t)cap));
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

// 1. Base cell slot and tile count of every active particle, and the marks on the node tiles
// of its stencil; zeroes the step counters and the list lengths.
__global__ void __launch_bounds__(kBlock) sort_count_kernel(Mpm m, PView P, SortGeo g, Work w,
                                                            Cnt* cnt) {
  const int p = blockIdx.x * kBlock + threadIdx.x;
  if (p == 0) {
    w.header[0] = 0;
    w.header[1] = 0;
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
      // The node tiles of the stencil's in-grid nodes [max(b, 0), min(b + 2, n - 1)].
      const int n3[3] = {m.nx, m.ny, m.nz};
      int lo[3], hi[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        lo[a] = max(base[a], 0) >> 3;
        hi[a] = min(base[a] + 2, n3[a] - 1) >> 3;
      }
      for (int ta = lo[0]; ta <= hi[0]; ++ta)
        for (int tb = lo[1]; tb <= hi[1]; ++tb)
          for (int tc = lo[2]; tc <= hi[2]; ++tc) w.node_flag[(ta * g.nty + tb) * g.ntz + tc] = 1;
    }
  }
  const unsigned peers = __match_any_sync(0xffffffffu, tile);
  if (tile >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&w.tile_count[tile], __popc(peers));
  if (p < m.n) {
    w.key[p] = key;
    w.slot[p] = slot;
  }
}

// 2a. Per chunk of 1024 cell tiles: the exclusive prefix of the tile counts within the chunk
// (into tile_start) and the chunk's total (into chunk_sum).
__global__ void __launch_bounds__(kScanThreads) sort_tile_scan_local_kernel(SortGeo g, Work w) {
  __shared__ int ws[32];
  const int i = blockIdx.x * kScanThreads + threadIdx.x;
  const int c = i < g.ntiles ? w.tile_count[i] : 0;
  int tot;
  const int ex = block_excl_scan(c, ws, &tot);
  if (i < g.ntiles) w.tile_start[i] = ex;
  if (threadIdx.x == 0) w.chunk_sum[blockIdx.x] = tot;
}

// 2b. Tile starts = chunk offset + local prefix (the last block also writes the total); the
// non-empty cell tiles are listed in arrival order (the list only schedules work) and the
// tile counts reset.
__global__ void __launch_bounds__(kScanThreads) sort_tile_scan_global_kernel(SortGeo g, Work w) {
  __shared__ int off;
  if (threadIdx.x == 0) {
    int o = 0;
    for (int b = 0; b < (int)blockIdx.x; ++b) o += w.chunk_sum[b];
    off = o;
    if (blockIdx.x == gridDim.x - 1) w.tile_start[g.ntiles] = o + w.chunk_sum[blockIdx.x];
  }
  __syncthreads();
  const int i = blockIdx.x * kScanThreads + threadIdx.x;
  if (i >= g.ntiles) return;
  const int c = w.tile_count[i];
  w.tile_start[i] += off;
  if (c > 0) w.cell_tiles[atomicAdd(&w.header[0], 1)] = i;
  w.tile_count[i] = 0;
}

// 2c. The node tiles some stencil touched are listed (arrival order) and their marks reset;
// the partials kernel's work cursor is reset.
__global__ void __launch_bounds__(kBlock) sort_node_tiles_kernel(SortGeo g, Work w) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i == 0) w.header[4] = 0;
  if (i >= g.nntiles || w.node_flag[i] == 0) return;
  w.node_flag[i] = 0;
  w.node_tiles[atomicAdd(&w.header[1], 1)] = i;
}

// 3. Cell starts (and the first sorted position of each non-empty cell) of each non-empty
// cell tile, one block of 512 threads per tile; the cell counts are reset.
__global__ void __launch_bounds__(kTC) sort_cell_scan_kernel(Work w) {
  __shared__ int ws[32];
  const int n = w.header[0];
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const int t = w.cell_tiles[i];
    const long long idx = (long long)t * kTC + threadIdx.x;
    const int c = w.cell_count[idx];
    int tot;
    const int ex = block_excl_scan(c, ws, &tot);
    const int start = w.tile_start[t] + ex;
    w.cell_start[idx] = start;
    w.cell_row[idx] = c > 0 ? start : -1;
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
__global__ void __launch_bounds__(kBlock) sorted_prepare_kernel(Mpm m, PView P, Work w,
                                                                ForceArgs fa) {
  const int p = blockIdx.x * kBlock + threadIdx.x;
  const long long cap = m.cap;
  bool partial = false, clipped = false, unsupported = false;
  if (p < m.n) {
    if (P.active[p] == 0) {
      if (kCoupled) { P.fp[p] = 0.f; P.fp[cap + p] = 0.f; P.fp[2 * cap + p] = 0.f; }
    } else {
      const int key = w.key[p];
      int pos = -1;
      if (key >= 0) {
        const int start = w.cell_start[key], end = cell_end(w, key);
        int rank = 0;
        for (int s = start; s < end; ++s) rank += w.unsorted[s] < p;
        pos = start + rank;
      }
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

__device__ __forceinline__ float sel3(int i, float a, float b, float c) {
  return i == 0 ? a : (i == 1 ? b : c);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Particles per cell and chunk staged in shared memory by the partials kernel, and the
// float4 slots per staged particle (the payload's 8 plus one, which with the extra slot per
// cell area puts the three cells of a warp on different shared-memory banks).
constexpr int kChunk = 8;
constexpr int kSlot = kPay + 1;
constexpr int kGroupF4 = kChunk * kSlot + 1;  // one cell's staging area, in float4
constexpr int kWarpBufF4 = 3 * kGroupF4;      // three cells
constexpr int kPartialWarps = kTileThreads / 32;
constexpr size_t kPartialSmem =
    (size_t)2 * kPartialWarps * kWarpBufF4 * sizeof(float4) + kTC * sizeof(int2);

// One triple of cells of a cell tile: a z-run (cells lz = 3 r, 3 r + 1, 3 r + 2 of row
// (lx, ly)); the lanes 9 g .. 9 g + 8 of a warp serve cell g of the triple.
struct Triple {
  int start, count;  // this lane's cell (count 0: no cell or empty)
  int maxcount;      // warp-wide
};

// cells: the tile's (start, count) per local cell, staged in shared memory.
__device__ __forceinline__ Triple load_triple(const int2* cells, int tr, int grp) {
  Triple t;
  t.start = 0;
  t.count = 0;
  const int row = tr / 3, lz = 3 * (tr % 3) + grp;
  if (grp < 3 && lz < kT) {
    const int2 c = cells[row * kT + lz];
    t.start = c.x;
    t.count = c.y;
  }
  t.maxcount = __reduce_max_sync(0xffffffffu, t.count);
  return t;
}

// Stages particles [chunk * kChunk, ...) of the warp's three cells into buf (all lanes copy).
__device__ __forceinline__ void stage_chunk(const Work& w, float4* buf, int lane, int start,
                                            int count, int chunk) {
  const int lo = chunk * kChunk;
  const int n_own = max(0, min(count - lo, kChunk));
  int n[3], st[3];
#pragma unroll
  for (int g = 0; g < 3; ++g) {
    n[g] = __shfl_sync(0xffffffffu, n_own, 9 * g);
    st[g] = __shfl_sync(0xffffffffu, start, 9 * g) + lo;
  }
  const int total = (n[0] + n[1] + n[2]) * kPay;
  for (int i = lane; i < total; i += 32) {
    int g = 0, r = i;
    if (r >= n[0] * kPay) {
      r -= n[0] * kPay;
      g = 1;
      if (r >= n[1] * kPay) { r -= n[1] * kPay; g = 2; }
    }
    const int part = r / kPay, comp = r - part * kPay;
    cp_async16(buf + g * kGroupF4 + part * kSlot + comp,
               w.payload + (long long)(st[g] + part) * kPay + comp);
  }
  cp_async_commit();
}

// 6. Cell partials: for every non-empty cell b and stencil offset o, the sum over the cell's
// particles (ascending index, from zero) of their contribution to node b + o, written to
// partial[cell_row(b) * 27 + o]; the coupling partial (reaction, solid fraction) sums the
// cell's coupled particles. A block takes non-empty cell tiles from a cursor; a warp handles
// z-runs of three cells, their particles staged in shared memory with asynchronous copies one
// chunk ahead of the arithmetic. Lane (g, ox, oy) forms the partials of offsets (ox, oy, 0..2)
// of cell g, which share the x and y factors of the weight and the first two terms of the
// affine product.
template <bool kCoupled>
__global__ void __launch_bounds__(kTileThreads, kCoupled ? 2 : 3)
    sorted_partials_kernel(Mpm m, Work w, fsi_coupling_desc cd) {
  constexpr int NC = kCoupled ? 2 : 1;
  extern __shared__ float4 smem[];
  __shared__ int next_tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float4* bufs = smem + (size_t)warp * 2 * kWarpBufF4;
  int2* cells = reinterpret_cast<int2*>(smem + (size_t)2 * kPartialWarps * kWarpBufF4);
  const int grp = lane / 9, r9 = lane - 9 * grp;
  const int ox = r9 / 3, oy = r9 - 3 * ox;
  const int gsel = grp < 3 ? grp : 0;
  const int ntiles = w.header[0];
  constexpr int kTriples = kT * kT * 3;  // (lx, ly) rows x three z-runs
  for (;;) {
    __syncthreads();  // the previous tile's cell table and cursor are no longer read
    if (threadIdx.x == 0) next_tile = atomicAdd(&w.header[4], 1);
    __syncthreads();
    const int ti = next_tile;
    if (ti >= ntiles) break;
    const int tile = w.cell_tiles[ti];
    for (int c = threadIdx.x; c < kTC; c += kTileThreads) {
      const int key = tile * kTC + c;
      const int st = w.cell_start[key];
      cells[c] = make_int2(st, cell_end(w, key) - st);
    }
    __syncthreads();
    // Job sequence of this warp: (triple, chunk) pairs of its non-empty triples, in order.
    int tr = warp;
    Triple cur;
    for (; tr < kTriples; tr += kPartialWarps) {
      cur = load_triple(cells, tr, grp);
      if (cur.maxcount > 0) break;
    }
    if (tr >= kTriples) continue;
    int chunk = 0, slot = 0;
    stage_chunk(w, bufs, lane, cur.start, cur.count, 0);
    float am[3][4], ac[3][4];
#pragma unroll
    for (int oz = 0; oz < 3; ++oz)
#pragma unroll
      for (int a = 0; a < 4; ++a) { am[oz][a] = 0.f; ac[oz][a] = 0.f; }
    bool any_coupled = false;
    for (;;) {
      // The next job, whose copies go out before this job's arithmetic.
      int ntr = tr, nchunk = chunk + 1;
      Triple nxt = cur;
      if (nchunk * kChunk >= cur.maxcount) {
        nchunk = 0;
        for (ntr = tr + kPartialWarps; ntr < kTriples; ntr += kPartialWarps) {
          nxt = load_triple(cells, ntr, grp);
          if (nxt.maxcount > 0) break;
        }
      }
      const bool more = ntr < kTriples;
      if (more) stage_chunk(w, bufs + (slot ^ 1) * kWarpBufF4, lane, nxt.start, nxt.count, nchunk);
      if (more) cp_async_wait<1>(); else cp_async_wait<0>();
      __syncwarp();
      const float4* gb = bufs + slot * kWarpBufF4 + gsel * kGroupF4;
      const int n_own = grp < 3 ? max(0, min(cur.count - chunk * kChunk, kChunk)) : 0;
      for (int s = 0; s < n_own; ++s) {
        const float4* r = gb + s * kSlot;
        const float4 r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3], r4 = r[4], r5 = r[5], r6 = r[6];
        const float4 r7 = kCoupled ? r[7] : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool coupled = kCoupled && r7.z != 0.f;
        any_coupled |= coupled;
        const float wxy = __fmul_rn(sel3(ox, r0.x, r0.y, r0.z), sel3(oy, r0.w, r1.x, r1.y));
        const float wz[3] = {r1.z, r1.w, r2.x};
        const float d0 = __fmul_rn(__fsub_rn((float)ox, r2.y), m.dx);
        const float d1 = __fmul_rn(__fsub_rn((float)oy, r2.z), m.dx);
        const float A[9] = {r3.x, r3.y, r3.z, r3.w, r4.x, r4.y, r4.z, r4.w, r5.x};
        const float mv[3] = {r5.y, r5.z, r5.w};
        const float pf[3] = {r6.x, r6.y, r6.z};
        float pa[3], dtf[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          // dot3r's ((A0 d0 + A1 d1) + A2 d2): the first two terms are shared by the 3 oz.
          pa[a] = __fadd_rn(__fmul_rn(A[3 * a], d0), __fmul_rn(A[3 * a + 1], d1));
          dtf[a] = __fmul_rn(m.dt, pf[a]);
        }
#pragma unroll
        for (int oz = 0; oz < 3; ++oz) {
          const float wgt = __fmul_rn(wxy, wz[oz]);
          const float d2 = __fmul_rn(__fsub_rn((float)oz, r2.w), m.dx);
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float ad = __fadd_rn(pa[a], __fmul_rn(A[3 * a + 2], d2));
            am[oz][a] = __fadd_rn(am[oz][a], __fmul_rn(wgt, __fadd_rn(__fadd_rn(mv[a], ad), dtf[a])));
          }
          am[oz][3] = __fadd_rn(am[oz][3], __fmul_rn(wgt, r6.w));
          if (kCoupled && coupled) {
            const float4 tc = coupling_spread_terms(cd, wgt, r7.x, pf, r7.y);
            ac[oz][0] = __fadd_rn(ac[oz][0], tc.x);
            ac[oz][1] = __fadd_rn(ac[oz][1], tc.y);
            ac[oz][2] = __fadd_rn(ac[oz][2], tc.z);
            ac[oz][3] = __fadd_rn(ac[oz][3], tc.w);
          }
        }
      }
      __syncwarp();  // the slot is restaged two jobs from now
      if (nchunk == 0) {
        // Last chunk of this triple: store the partials of this lane's cell.
        if (grp < 3 && cur.count > 0) {
          float4* out = w.partial + ((long long)cur.start * 27 + 9 * ox + 3 * oy) * NC;
#pragma unroll
          for (int oz = 0; oz < 3; ++oz) {
            out[oz * NC] = make_float4(am[oz][0], am[oz][1], am[oz][2], am[oz][3]);
            if (kCoupled) out[oz * NC + 1] = make_float4(ac[oz][0], ac[oz][1], ac[oz][2], ac[oz][3]);
          }
          if (kCoupled && r9 == 0) w.cell_coupled[cur.start] = any_coupled ? 1 : 0;
        }
#pragma unroll
        for (int oz = 0; oz < 3; ++oz)
#pragma unroll
          for (int a = 0; a < 4; ++a) { am[oz][a] = 0.f; ac[oz][a] = 0.f; }
        any_coupled = false;
      }
      if (!more) break;
      tr = ntr;
      chunk = nchunk;
      cur = nxt;
      slot ^= 1;
    }
  }
}

// 7. Node sums: every node of a touched 8^3 node tile (one thread each) adds the partials of
// its non-empty cells b = node - o in ascending cell index (o from (2,2,2) down to (0,0,0)):
// momentum and mass from zero into the grid, and on fluid nodes the coupling partials of
// cells with coupled particles onto the accumulator's current value (the solid fraction
// only when it is being built). Plain stores: each node belongs to one block.
template <bool kCoupled>
__global__ void __launch_bounds__(kTC, 2) sorted_nodes_kernel(Mpm m, SortGeo g, Work w,
                                                              float4* __restrict__ grid,
                                                              fsi_coupling_desc cd,
                                                              const uint32_t* __restrict__ flags,
                                                              float4* __restrict__ accum) {
  constexpr int NC = kCoupled ? 2 : 1;
  constexpr int kRE = kT + 2;  // the region of a node tile: (kT + 2)^3 cells
  __shared__ int region[kRE * kRE * kRE];  // partial row of each region cell, or -1
  const int ntiles = w.header[1];
  for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const int t = w.node_tiles[it];
    const int a0 = (t / (g.nty * g.ntz)) * kT, b0 = ((t / g.ntz) % g.nty) * kT, c0 = (t % g.ntz) * kT;
    __syncthreads();  // the previous tile's region is no longer read
    // Region cell (x, y, z) has shifted coordinates (a0 + x, b0 + y, c0 + z): base cell
    // (a0 - 2 + x, ...).
    for (int r = threadIdx.x; r < kRE * kRE * kRE; r += kTC) {
      const int s0 = a0 + r / (kRE * kRE), s1 = b0 + (r / kRE) % kRE, s2 = c0 + r % kRE;
      int row = -1;
      if (s0 < m.nx + 2 && s1 < m.ny + 2 && s2 < m.nz + 2) {
        const int tile = ((s0 >> 3) * g.cty + (s1 >> 3)) * g.ctz + (s2 >> 3);
        if (w.tile_start[tile + 1] > w.tile_start[tile])
          row = w.cell_row[tile * kTC + (((s0 & 7) << 6) | ((s1 & 7) << 3) | (s2 & 7))];
      }
      region[r] = row;
    }
    __syncthreads();
    const int x = threadIdx.x >> 6, y = (threadIdx.x >> 3) & 7, z = threadIdx.x & 7;
    const int ni = a0 + x, nj = b0 + y, nk = c0 + z;
    if (ni >= m.nx || nj >= m.ny || nk >= m.nz) continue;
    const long long node = node_index(m, ni, nj, nk);
    float4 am = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 ac = make_float4(0.f, 0.f, 0.f, 0.f);
    bool fluid = false;
    if (kCoupled) {
      ac = accum[node];
      fluid = !(flags[node] & kFlagSolid);
    }
    // Cell node - o sits at region (x + 2 - i, y + 2 - j, z + 2 - k). The partials of a z-run
    // of three cells are loaded together, then added in order.
#pragma unroll
    for (int ij = 8; ij >= 0; --ij) {
      const int i = ij / 3, j = ij % 3;
      const int* rr = region + ((x + 2 - i) * kRE + (y + 2 - j)) * kRE + z;
      const int rows[3] = {rr[0], rr[1], rr[2]};  // k = 2, 1, 0
      float4 pm[3];
#pragma unroll
      for (int t3 = 0; t3 < 3; ++t3)
        pm[t3] = rows[t3] >= 0 ? w.partial[((long long)rows[t3] * 27 + 3 * ij + 2 - t3) * NC]
                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int t3 = 0; t3 < 3; ++t3) {
        if (rows[t3] < 0) continue;
        am.x = __fadd_rn(am.x, pm[t3].x);
        am.y = __fadd_rn(am.y, pm[t3].y);
        am.z = __fadd_rn(am.z, pm[t3].z);
        am.w = __fadd_rn(am.w, pm[t3].w);
        if (kCoupled && fluid && w.cell_coupled[rows[t3]]) {
          const float4 sc = w.partial[((long long)rows[t3] * 27 + 3 * ij + 2 - t3) * NC + 1];
          ac.x = __fadd_rn(ac.x, sc.x);
          ac.y = __fadd_rn(ac.y, sc.y);
          ac.z = __fadd_rn(ac.z, sc.z);
          if (cd.build_fraction) ac.w = __fadd_rn(ac.w, sc.w);
        }
      }
    }
    grid[node] = am;
    if (kCoupled) accum[node] = ac;
  }
}

// 8. Grid update + G2P per particle, in storage order (coalesced particle reads and writes;
// the CTA's stencil box is staged in shared memory when it fits).
__global__ void __launch_bounds__(kBlock) sorted_g2p_kernel(Mpm m, PView P,
                                                            const float4* __restrict__ grid) {
  g2p_body(m, P, grid, blockIdx.x * kBlock + threadIdx.x);
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

// Opts the partials kernel into its dynamic shared memory, once per device.
template <bool kCoupled>
int partials_smem_attr() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("cudaGetDevice");
  if (dev < 0 || dev >= 64 || !done[dev]) {
    if (cudaFuncSetAttribute(sorted_partials_kernel<kCoupled>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPartialSmem) !=
        cudaSuccess)
      return check_launch("cudaFuncSetAttribute(sorted_partials_kernel)");
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

// The ten launches of a sorted substep (kCoupled: with the coupling folded in).
template <bool kCoupled>
int sorted_substep(const Mpm& m, const PView& P, const SortGeo& g, const Work& w, float4* grid,
                   const ForceArgs& fa, cudaStream_t s) {
  if (int e = partials_smem_attr<kCoupled>()) return e;
  const unsigned pg = grid_for(m.n, kBlock);
  const int sms = num_sms();
  sort_count_kernel<<<pg, kBlock, 0, s>>>(m, P, g, w, kCoupled ? fa.cnt : nullptr);
  if (int e = check_launch("sort_count_kernel")) return e;
  const unsigned chunks = (unsigned)((g.ntiles + kScanThreads - 1) / kScanThreads);
  sort_tile_scan_local_kernel<<<chunks, kScanThreads, 0, s>>>(g, w);
  if (int e = check_launch("sort_tile_scan_local_kernel")) return e;
  sort_tile_scan_global_kernel<<<chunks, kScanThreads, 0, s>>>(g, w);
  if (int e = check_launch("sort_tile_scan_global_kernel")) return e;
  sort_node_tiles_kernel<<<grid_for(g.nntiles, kBlock), kBlock, 0, s>>>(g, w);
  if (int e = check_launch("sort_node_tiles_kernel")) return e;
  sort_cell_scan_kernel<<<g.ntiles < 4 * sms ? g.ntiles : 4 * sms, kTC, 0, s>>>(w);
  if (int e = check_launch("sort_cell_scan_kernel")) return e;
  sort_scatter_kernel<<<pg, kBlock, 0, s>>>(m.n, w);
  if (int e = check_launch("sort_scatter_kernel")) return e;
  // Few particles (under two CTAs per SM): latency-bound, so the coupling's stencil loads go
  // out together.
  if (m.n < 2 * sms * kBlock)
    sorted_prepare_kernel<kCoupled, true><<<pg, kBlock, 0, s>>>(m, P, w, fa);
  else
    sorted_prepare_kernel<kCoupled, false><<<pg, kBlock, 0, s>>>(m, P, w, fa);
  if (int e = check_launch("sorted_prepare_kernel")) return e;
  const int pb = g.ntiles < 3 * sms ? g.ntiles : 3 * sms;
  sorted_partials_kernel<kCoupled><<<pb, kTileThreads, kPartialSmem, s>>>(m, w, fa.c);
  if (int e = check_launch("sorted_partials_kernel")) return e;
  const int nb = g.nntiles < 4 * sms ? g.nntiles : 4 * sms;
  sorted_nodes_kernel<kCoupled><<<nb, kTC, 0, s>>>(m, g, w, grid, fa.c, fa.flags, fa.accum);
  if (int e = check_launch("sorted_nodes_kernel")) return e;
  sorted_g2p_kernel<<<pg, kBlock, 0, s>>>(m, P, grid);
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
