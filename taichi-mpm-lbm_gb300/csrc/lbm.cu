// D3Q19 MRT lattice Boltzmann on sm_103a: fused in-place AA-pattern step.
//
// One launch per lattice step performs the reference's collide + stream +
// bounce-back (fsi/lbm3d.py:314-361) on a single population array:
//   even steps: read the cell's own 19 slots, write post-collision f*_q into
//               slot opp(q) of the same cell;
//   odd steps:  read F_q from slot opp(q) of x - e_q (own slot q when x - e_q is
//               solid), write f*_q into slot q of x + e_q (own slot opp(q) when
//               x + e_q is solid: half-way bounce-back).
// Every slot is read and written by exactly one cell per step, so the update is
// race-free in place. After an odd number of steps the populations sit in the
// "AA-odd" arrangement that gather32() undoes.
//
// Two arithmetic forms:
//   exact (default, FP32 storage): the reference's float32 operations in the
//     reference's order (this file is compiled with -fmad=false and uses *_rn
//     intrinsics; the MRT transforms are generated formulas, lbm_formulas.cuh);
//   fast: the same collision operator with about 2.5x fewer operations
//     (parity-split moments, closed-form forcing moments, fused multiply-adds).
// Three storage forms: FP32 populations; FP16 or BF16 deviations from the rest
// equilibrium, f_q - w_q rho0 (FP16 scaled by 2^12 into its normal range). All
// arithmetic is FP32 in every form.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "fsi_common.cuh"
#include "lbm_formulas.cuh"
#include "lbm_vec.cuh"

#include "lbm_core.cuh"

namespace fsi {
namespace {

// x-face conditions applied to the post-stream state (lbm3d.py:363-407).
struct FaceArgs {
  LbmGeom g;
  void* __restrict__ pops;
  const float4* __restrict__ macro;  // u of the state before this step, on face cells
  const uint32_t* __restrict__ flags;
  int parity;  // of the state after the step
  int mode[2];
  float bc_rho[2];
  float bc_vel[2][3];
  float rho0;
  float shift[19];
};

template <int kStore>
__global__ void __launch_bounds__(kBlock) lbm_face_kernel(FaceArgs a) {
  using St = Store<kStore>;
  const int per_face = a.g.ny * a.g.nz;
  const int t = blockIdx.x * kBlock + threadIdx.x;
  if (t >= 2 * per_face) return;
  const int side = t / per_face;
  const int mode = a.mode[side];
  if (mode == 0) return;
  const int r = t - side * per_face;
  const Deltas d(a.g, side == 0 ? 0 : a.g.nx - 1, r / a.g.nz, r % a.g.nz);
  const uint32_t c = d.c;
  const uint32_t fl = a.flags[c];
  if (fl & kFlagSolid) return;
  const uint32_t n = (uint32_t)a.g.n;
  typename St::T* __restrict__ pops = reinterpret_cast<typename St::T*>(a.pops);
  float F[19];
  uint32_t slot[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    slot[q] = slot32(n, d, fl, q, a.parity);
    F[q] = St::ld(pops, slot[q], a.shift[q]);
  }
  if (mode == 1) {
    // Pressure: equilibrium at bc_rho with the velocity of this cell, or of the
    // inner neighbour when that one is solid (whose velocity is always 0).
    const bool inner_solid = (fl >> (side == 0 ? 1 : 2)) & 1u;
    float ux = 0.f, uy = 0.f, uz = 0.f;
    if (!inner_solid) {
      const float4 mc = a.macro[c];
      ux = mc.x; uy = mc.y; uz = mc.z;
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) F[q] = feq_ref(q, a.bc_rho[side], ux, uy, uz);
  } else if (mode == 2) {
    // Velocity: F_q = feq_opp - F_opp + feq_q, sequentially in q with the
    // already-updated F_opp (the reference updates the field in place).
    const float* v = a.bc_vel[side];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const int o = opp(q);
      float val = __fsub_rn(feq_ref(o, a.rho0, v[0], v[1], v[2]), F[o]);
      F[q] = __fadd_rn(val, feq_ref(q, a.rho0, v[0], v[1], v[2]));
    }
  } else {
    // Velocity, every F_opp read from before the update (mode 3, an extension).
    const float* v = a.bc_vel[side];
    float G[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const int o = opp(q);
      float val = __fsub_rn(feq_ref(o, a.rho0, v[0], v[1], v[2]), F[o]);
      G[q] = __fadd_rn(val, feq_ref(q, a.rho0, v[0], v[1], v[2]));
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) F[q] = G[q];
  }
#pragma unroll
  for (int q = 0; q < 19; ++q) St::st(pops, slot[q], F[q], a.shift[q]);
}

struct MacroArgs {
  LbmGeom g;
  const void* __restrict__ pops;
  const float* __restrict__ force;
  const uint32_t* __restrict__ flags;
  float4* __restrict__ macro;
  int parity;
  float rho0;
  float shift[19];
};

// update_macro (lbm3d.py:409-425) on the current state; with `diag` non-NULL it also adds
// sum(rho) over fluid cells to diag[0] and raises diag[1] to max |u| (lbm3d.py:450-457).
template <int kStore, bool kFast>
__global__ void __launch_bounds__(kBlock) lbm_macro_kernel(MacroArgs a, double* __restrict__ diag) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  float mass = 0.f, vmax = 0.f;
  if (k < a.g.nz && j < a.g.ny) {
    const Deltas d(a.g, i, j, k);
    const uint32_t c = d.c;
    const uint32_t fl = a.flags[c];
    if (fl & kFlagSolid) {
      a.macro[c] = make_float4(0.f, 0.f, 0.f, a.rho0);
    } else {
      const uint32_t n = (uint32_t)a.g.n;
      const auto* pops = reinterpret_cast<const typename Store<kStore>::T*>(a.pops);
      float F[19];
#pragma unroll
      for (int q = 0; q < 19; ++q) F[q] = gather32<kStore>(pops, n, d, fl, q, a.parity, a.shift[q]);
      float rho, ux, uy, uz;
      macro_any<kFast>(F, a.force[c], a.force[n + c], a.force[2 * n + c], rho, ux, uy, uz);
      a.macro[c] = make_float4(ux, uy, uz, rho);
      mass = rho;
      vmax = norm3_ref(ux, uy, uz);
    }
  }
  if (diag) {
    const float s[1] = {mass};
    block_accumulate<1>(diag, s, diag + 1, vmax);
  }
}

template <int kStore>
__global__ void __launch_bounds__(kBlock) lbm_distribution_kernel(LbmGeom g, const void* pops_v,
                                                                  const uint32_t* __restrict__ flags,
                                                                  int parity, float rho0,
                                                                  float* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= g.nz || j >= g.ny) return;
  const Deltas d(g, i, j, k);
  const uint32_t fl = flags[d.c];
  const int p = (fl & kFlagSolid) ? 0 : parity;
  const auto* pops = reinterpret_cast<const typename Store<kStore>::T*>(pops_v);
#pragma unroll
  for (int q = 0; q < 19; ++q)
    out[(size_t)d.c * 19 + q] =
        gather32<kStore>(pops, (uint32_t)g.n, d, fl, q, p, __fmul_rn(weight_of(q), rho0));
}

__global__ void __launch_bounds__(kBlock) lbm_flags_kernel(LbmGeom g,
                                                           const int32_t* __restrict__ solid,
                                                           uint32_t* __restrict__ flags) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= g.nz || j >= g.ny) return;
  const Deltas d(g, i, j, k);
  uint32_t f = solid[d.c] != 0 ? kFlagSolid : 0u;
#pragma unroll
  for (int q = 1; q < 19; ++q)
    if (solid[d.nb(q, +1)] != 0) f |= 1u << q;
  f |= corner_flag_bits(solid, d);
  if (i == 0) f |= kFlagFaceLeft;
  if (i == g.nx - 1) f |= kFlagFaceRight;
  flags[d.c] = f;
}

template <int kStore>
__global__ void __launch_bounds__(kBlock) lbm_init_kernel(LbmGeom g,
                                                          const uint32_t* __restrict__ flags,
                                                          float rho0, float u0x, float u0y,
                                                          float u0z, void* pops_v,
                                                          float4* __restrict__ macro) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= g.n) return;
  const bool solid = flags[c] & kFlagSolid;
  const float ux = solid ? 0.f : u0x, uy = solid ? 0.f : u0y, uz = solid ? 0.f : u0z;
  macro[c] = make_float4(ux, uy, uz, rho0);
  auto* pops = reinterpret_cast<typename Store<kStore>::T*>(pops_v);
#pragma unroll
  for (int q = 0; q < 19; ++q)
    Store<kStore>::st(pops, (uint32_t)(q * g.n + c), feq_ref(q, rho0, ux, uy, uz),
                      __fmul_rn(weight_of(q), rho0));
}

__global__ void __launch_bounds__(kBlock) lbm_force_kernel(LbmGeom g,
                                                           const uint32_t* __restrict__ flags,
                                                           int op, const float* __restrict__ in,
                                                           float vx, float vy, float vz,
                                                           float* __restrict__ out) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= g.n) return;
  const bool fluid = !(flags[c] & kFlagSolid);
  const float v[3] = {vx, vy, vz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float r;
    if (op == FSI_FORCE_CLEAR) r = 0.f;
    else if (op == FSI_FORCE_SET) r = fluid ? v[a] : 0.f;
    else if (op == FSI_FORCE_ADD) r = fluid ? __fadd_rn(in[a * g.n + c], v[a]) : 0.f;
    else r = fluid ? in[a * g.n + c] : 0.f;
    out[a * g.n + c] = r;
  }
}

// Lattice diagnostics of the current macro and force fields (lbm3d.py:450-483):
// out[0] += sum rho over fluid, out[1] = max |u| over all cells, out[2..4] += sum force over fluid.
// Sums over the lattice in warp tiles of 32 consecutive cells of a row (the same tiles as a
// one-thread-per-cell launch): each tile's fluid rho and force in float32 warp sums (a
// butterfly, so every lane holds the tile's sum), added in float64 per warp over its tiles,
// then per block, and once per block into out (out[0] sum of rho over fluid, out[1] max |u|,
// out[2..4] force sums). The float64 adds are this GPU's scarce pipe: lane j keeps the sum of
// the warp's j-th tile of each run of 32 and converts and adds it once per run, so one float64
// instruction serves 32 tiles. A bounded grid walks the tiles (a few atomics per block).
__global__ void __launch_bounds__(kBlock) lbm_reduce_kernel(LbmGeom g,
                                                            const float4* __restrict__ macro,
                                                            const float* __restrict__ force,
                                                            const uint32_t* __restrict__ flags,
                                                            double* __restrict__ out) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long tiles_per_row = (g.nz + 31) / 32;
  const long long tiles = (long long)g.nx * g.ny * tiles_per_row;
  const long long warps = (long long)gridDim.x * (kBlock / 32);
  const uint32_t n = (uint32_t)g.n;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  float hold[4] = {0.f, 0.f, 0.f, 0.f};
  int slot = 0;  // lane that keeps the next tile's sums
  float vmax = 0.f;
  // four tiles per pass, their loads issued together
  for (long long t0 = (long long)blockIdx.x * (kBlock / 32) + wib; t0 < tiles; t0 += 4 * warps) {
    float4 m[4];
    uint32_t fl[4];
    float fv[4][3];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const long long t = t0 + u * warps;
      const long long row = t / tiles_per_row;
      const int k = (int)(t - row * tiles_per_row) * 32 + lane;
      const bool in = t < tiles && k < g.nz;
      const uint32_t c = in ? (uint32_t)(row * g.nz + k) : 0u;
      m[u] = in ? macro[c] : make_float4(0.f, 0.f, 0.f, 0.f);
      fl[u] = in ? flags[c] : kFlagSolid;
#pragma unroll
      for (int a = 0; a < 3; ++a) fv[u][a] = (in && force) ? force[a * n + c] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      vmax = fmaxf(vmax, norm3_ref(m[u].x, m[u].y, m[u].z));
      if (!(fl[u] & kFlagSolid)) {
        v[0] = m[u].w;
        v[1] = fv[u][0]; v[2] = fv[u][1]; v[3] = fv[u][2];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < 4; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
      if (lane == slot)
#pragma unroll
        for (int i = 0; i < 4; ++i) hold[i] = v[i];
      if (++slot == 32) {
#pragma unroll
        for (int i = 0; i < 4; ++i) { acc[i] += (double)hold[i]; hold[i] = 0.f; }
        slot = 0;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[i] += (double)hold[i];
  // float64 warp sums, then block sums
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
    vmax = fmaxf(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
  }
  __shared__ double sh[4][kBlock / 32];
  __shared__ float shm[kBlock / 32];
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) sh[i][wib] = acc[i];
    shm[wib] = vmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s4[4] = {0.0, 0.0, 0.0, 0.0};
    float mx = 0.f;
    for (int w = 0; w < kBlock / 32; ++w) {
      for (int i = 0; i < 4; ++i) s4[i] += sh[i][w];
      mx = fmaxf(mx, shm[w]);
    }
    atomicAdd(out, s4[0]);
    atomic_max_nonneg(out + 1, (double)mx);
    for (int i = 0; i < 3; ++i) atomicAdd(out + 2 + i, s4[1 + i]);
  }
}

int check_desc(const fsi_lbm_desc* d) {
  FSI_REQUIRE(d != nullptr, "lbm descriptor is NULL");
  FSI_REQUIRE(d->nx > 4 && d->ny > 4 && d->nz > 4, "lattice %dx%dx%d too small", d->nx, d->ny, d->nz);
  FSI_REQUIRE(19ll * d->nx * d->ny * d->nz < (1ll << 32),
              "lattice of %lld cells too large for 32-bit population indexing",
              (long long)d->nx * d->ny * d->nz);
  FSI_REQUIRE(d->nx <= 65535, "nx must be at most 65535");
  FSI_REQUIRE(d->s[0] == 0.f && d->s[3] == 0.f && d->s[5] == 0.f && d->s[7] == 0.f,
              "conserved moments (0, 3, 5, 7) must have zero relaxation rate");
  for (int side = 0; side < 2; ++side) {
    int m = side == 0 ? d->bc_mode_left : d->bc_mode_right;
    FSI_REQUIRE(m >= 0 && m <= 3, "unknown x boundary mode %d", m);
  }
  FSI_REQUIRE(d->storage >= FSI_STORAGE_F32 && d->storage <= FSI_STORAGE_BF16,
              "unknown population storage %d", d->storage);
  FSI_REQUIRE(d->arithmetic == FSI_ARITH_EXACT || d->arithmetic == FSI_ARITH_FAST,
              "unknown arithmetic form %d", d->arithmetic);
  FSI_REQUIRE(d->storage == FSI_STORAGE_F32 || d->arithmetic == FSI_ARITH_FAST,
              "FP16/BF16 population storage uses the fast arithmetic form");
  return FSI_OK;
}

void fill_shift(const fsi_lbm_desc* d, float (&shift)[19]) {
  for (int q = 0; q < 19; ++q) shift[q] = d->storage == FSI_STORAGE_F32 ? 0.f : weight_of(q) * d->rho0;
}

// Launches kernel K<storage, fast, ...> for the descriptor's forms.
template <template <int, bool> class Launcher, class... Args>
void dispatch_forms(const fsi_lbm_desc* d, Args&&... args) {
  const bool fast = d->arithmetic == FSI_ARITH_FAST;
  switch (d->storage) {
    case FSI_STORAGE_F16: Launcher<FSI_STORAGE_F16, true>::run(args...); break;
    case FSI_STORAGE_BF16: Launcher<FSI_STORAGE_BF16, true>::run(args...); break;
    default:
      if (fast) Launcher<FSI_STORAGE_F32, true>::run(args...);
      else Launcher<FSI_STORAGE_F32, false>::run(args...);
  }
}

template <int S, bool F>
struct StepLauncher {
  static void run(const StepArgs& a, bool odd, bool recompute, const CellLaunch& L, cudaStream_t s) {
    if (recompute) {
      if (odd) lbm_step_kernel<S, F, true, true><<<L.grid, L.block, 0, s>>>(a);
      else lbm_step_kernel<S, F, false, true><<<L.grid, L.block, 0, s>>>(a);
    } else {
      if (odd) lbm_step_kernel<S, F, true, false><<<L.grid, L.block, 0, s>>>(a);
      else lbm_step_kernel<S, F, false, false><<<L.grid, L.block, 0, s>>>(a);
    }
  }
};

template <int S, bool F>
struct MacroLauncher {
  static void run(const MacroArgs& a, double* diag, cudaStream_t s) {
    const CellLaunch L = cell_launch(a.g);
    lbm_macro_kernel<S, F><<<L.grid, L.block, 0, s>>>(a, diag);
  }
};

template <int S, bool F>
struct FaceLauncher {
  static void run(const FaceArgs& f, cudaStream_t s) {
    const long long faces = 2ll * f.g.ny * f.g.nz;
    lbm_face_kernel<S><<<grid_for(faces, kBlock), kBlock, 0, s>>>(f);
  }
};

template <int S, bool F>
struct DistLauncher {
  static void run(const LbmGeom& g, const void* pops, const uint32_t* flags, int parity,
                  float rho0, float* out, cudaStream_t s) {
    const CellLaunch L = cell_launch(g);
    lbm_distribution_kernel<S><<<L.grid, L.block, 0, s>>>(g, pops, flags, parity, rho0, out);
  }
};

template <int S, bool F>
struct InitLauncher {
  static void run(const LbmGeom& g, const uint32_t* flags, float rho0, const float* u0, void* pops,
                  float4* macro, cudaStream_t s) {
    lbm_init_kernel<S><<<grid_for(g.n, kBlock), kBlock, 0, s>>>(g, flags, rho0, u0[0], u0[1],
                                                                 u0[2], pops, macro);
  }
};

MacroArgs macro_args(const fsi_lbm_desc* d, const void* pops, const float* force,
                     const uint32_t* flags, int64_t steps_done, float* macro) {
  MacroArgs a;
  a.g = geom_of(d);
  a.pops = pops;
  a.force = force;
  a.flags = flags;
  a.macro = reinterpret_cast<float4*>(macro);
  a.parity = (int)(steps_done & 1);
  a.rho0 = d->rho0;
  fill_shift(d, a.shift);
  return a;
}

}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_lbm_build_flags(const fsi_lbm_desc* d, const int32_t* solid, uint32_t* flags,
                                   void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(solid && flags, "NULL array");
  LbmGeom g = geom_of(d);
  const CellLaunch L = cell_launch(g);
  lbm_flags_kernel<<<L.grid, L.block, 0, as_stream(stream)>>>(g, solid, flags);
  return check_launch("lbm_flags_kernel");
}

extern "C" int fsi_lbm_init_fields(const fsi_lbm_desc* d, const uint32_t* flags, const float* u0,
                                   void* pops, float* macro, void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(flags && u0 && pops && macro, "NULL array");
  dispatch_forms<InitLauncher>(d, geom_of(d), flags, d->rho0, u0, pops,
                               reinterpret_cast<float4*>(macro), as_stream(stream));
  return check_launch("lbm_init_kernel");
}

extern "C" int fsi_lbm_step(const fsi_lbm_desc* d, void* pops, float* macro, const float* force,
                            const float* force_prev, const uint32_t* flags, int64_t steps_done,
                            void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(pops && macro && force && flags, "NULL array");
  FSI_REQUIRE(steps_done >= 0, "steps_done must be non-negative");
  StepArgs a;
  a.g = geom_of(d);
  a.pops = pops;
  a.macro = reinterpret_cast<float4*>(macro);
  a.force = force;
  a.force_prev = force_prev;
  a.flags = flags;
  for (int k = 0; k < 19; ++k) {
    a.s[k] = d->s[k];
    a.sg[k] = 1.0f - 0.5f * d->s[k];
  }
  fill_shift(d, a.shift);
  a.write_faces = (d->bc_mode_left != 0 || d->bc_mode_right != 0) ? 1 : 0;
  cudaStream_t s = as_stream(stream);
  const bool odd = (steps_done & 1) != 0;
  const int lanes = d->arithmetic == FSI_ARITH_FAST ? 2 : 1;
  dispatch_forms<StepLauncher>(d, a, odd, force_prev != nullptr, step_launch(a.g, lanes), s);
  if (int e = check_launch("lbm_step_kernel")) return e;
  if (a.write_faces) {
    FaceArgs f;
    f.g = a.g;
    f.pops = pops;
    f.macro = a.macro;
    f.flags = flags;
    f.parity = (int)((steps_done + 1) & 1);
    f.mode[0] = d->bc_mode_left;
    f.mode[1] = d->bc_mode_right;
    f.bc_rho[0] = d->bc_rho_left;
    f.bc_rho[1] = d->bc_rho_right;
    for (int i = 0; i < 3; ++i) {
      f.bc_vel[0][i] = d->bc_vel_left[i];
      f.bc_vel[1][i] = d->bc_vel_right[i];
    }
    f.rho0 = d->rho0;
    fill_shift(d, f.shift);
    dispatch_forms<FaceLauncher>(d, f, s);
    if (int e = check_launch("lbm_face_kernel")) return e;
  }
  return FSI_OK;
}

extern "C" int fsi_lbm_update_macro(const fsi_lbm_desc* d, const void* pops, const float* force,
                                    const uint32_t* flags, int64_t steps_done, float* macro,
                                    void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(pops && force && flags && macro, "NULL array");
  MacroArgs a = macro_args(d, pops, force, flags, steps_done, macro);
  dispatch_forms<MacroLauncher>(d, a, (double*)nullptr, as_stream(stream));
  return check_launch("lbm_macro_kernel");
}

extern "C" int fsi_lbm_distribution(const fsi_lbm_desc* d, const void* pops,
                                    const uint32_t* flags, int64_t steps_done, float* out,
                                    void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(pops && flags && out, "NULL array");
  dispatch_forms<DistLauncher>(d, geom_of(d), pops, flags, (int)(steps_done & 1), d->rho0, out,
                               as_stream(stream));
  return check_launch("lbm_distribution_kernel");
}

extern "C" int fsi_lbm_force_op(const fsi_lbm_desc* d, const uint32_t* flags, int op,
                                const float* in, const float* value, float* out, void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(flags && out, "NULL array");
  FSI_REQUIRE(op >= FSI_FORCE_CLEAR && op <= FSI_FORCE_ZERO_SOLID, "unknown force op %d", op);
  FSI_REQUIRE(in || op == FSI_FORCE_CLEAR || op == FSI_FORCE_SET, "force op %d needs an input", op);
  FSI_REQUIRE(value || (op != FSI_FORCE_SET && op != FSI_FORCE_ADD), "force op %d needs a value", op);
  LbmGeom g = geom_of(d);
  const float vx = value ? value[0] : 0.f, vy = value ? value[1] : 0.f, vz = value ? value[2] : 0.f;
  lbm_force_kernel<<<grid_for(g.n, kBlock), kBlock, 0, as_stream(stream)>>>(g, flags, op, in, vx,
                                                                             vy, vz, out);
  return check_launch("lbm_force_kernel");
}

extern "C" int fsi_lbm_reduce(const fsi_lbm_desc* d, const float* macro, const float* force,
                              const uint32_t* flags, double* out, void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(macro && flags && out, "NULL array");
  LbmGeom g = geom_of(d);
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out, 0, 8 * sizeof(double), s) != cudaSuccess) return check_launch("memset");
  const long long tiles = (long long)g.nx * g.ny * ((g.nz + 31) / 32);
  long long blocks = (tiles + kBlock / 32 - 1) / (kBlock / 32);
  if (blocks > 152 * 8) blocks = 152 * 8;
  lbm_reduce_kernel<<<(unsigned)blocks, kBlock, 0, s>>>(g, reinterpret_cast<const float4*>(macro),
                                                        force, flags, out);
  return check_launch("lbm_reduce_kernel");
}

extern "C" int fsi_lbm_macro_diagnostics(const fsi_lbm_desc* d, const void* pops,
                                         const float* force, const uint32_t* flags,
                                         int64_t steps_done, float* macro, double* out,
                                         void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(pops && force && flags && macro && out, "NULL array");
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out, 0, 2 * sizeof(double), s) != cudaSuccess) return check_launch("memset");
  MacroArgs a = macro_args(d, pops, force, flags, steps_done, macro);
  dispatch_forms<MacroLauncher>(d, a, out, s);
  return check_launch("lbm_macro_kernel (diagnostics)");
}
