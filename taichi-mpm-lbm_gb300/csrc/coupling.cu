// LBM-MPM coupling on sm_103a (reference: fsi/coupling.py:332-496).
//
//   coupling_forces: per particle, interpolate the fluid velocity over the
//     non-solid in-grid nodes of its 27-node stencil, form the penalty force
//     gamma m (u_f - v_p) with optional clipping, and spread the reaction
//     -(w/W) f dt_ratio / V_cell (plus the occupancy (w/W) V_p / V_cell on the
//     first substep) into a float4 accumulator (force xyz, solid fraction) with
//     vector reductions.
//   assemble: per cell, clamp the solid fraction, rebuild the LBM force as
//     base + coupling (+ Brinkman immersed-boundary drag), zero on solid cells.
//   contact: per particle, static/dynamic support test and velocity damping.
#include <cuda_runtime.h>

#include <cstdint>

#include "fsi_common.cuh"
#include "coupling_core.cuh"

namespace fsi {
namespace {

constexpr int kGatherAheadMax = 2 * 152 * kBlock;

template <bool kGatherAhead>
__global__ void __launch_bounds__(kBlock) coupling_forces_kernel(ForceArgs a) {
  coupling_forces_body<kGatherAhead>(a, blockIdx.x * kBlock + threadIdx.x);
}

__global__ void __launch_bounds__(kBlock) assemble_kernel(AssembleArgs a) {
  assemble_body(a, (long long)blockIdx.x * kBlock + threadIdx.x);
}

struct ContactArgs {
  fsi_coupling_desc c;
  Geo g;
  int n;
  long long cap;
  const float* __restrict__ x;
  float* __restrict__ v;
  const int32_t* __restrict__ active;
  const float4* __restrict__ accum;
  const uint32_t* __restrict__ flags;
  int32_t* __restrict__ mask;
  Cnt* __restrict__ cnt;
};

// _compute_contact_diagnostics_kernel, fsi/coupling.py:463-496.
__global__ void __launch_bounds__(kBlock) contact_kernel(ContactArgs a) {
  const int p = blockIdx.x * kBlock + threadIdx.x;
  bool cand = false, damped = false;
  if (p < a.n) {
    a.mask[p] = 0;
    if (a.c.contact_enabled && a.active[p] != 0) {
      const long long cap = a.cap;
      const float x[3] = {a.x[p], a.x[cap + p], a.x[2 * cap + p]};
      int base[3];
      float fx[3];
      stencil_base(a.c.inv_dx, x, base, fx);
      float dyn = 0.f, stat = 0.f;
#pragma unroll
      for (int s = 0; s < 27; ++s) {
        const int i = s / 9, j = (s / 3) % 3, k = s % 3;
        const int ni = base[0] + i, nj = base[1] + j, nk = base[2] + k;
        if (ni < 0 || ni >= a.g.nx || nj < 0 || nj >= a.g.ny || nk < 0 || nk >= a.g.nz) continue;
        const long long c = ((long long)ni * a.g.ny + nj) * a.g.nz + nk;
        const float w = __fmul_rn(__fmul_rn(bspline_w(fx[0], i), bspline_w(fx[1], j)), bspline_w(fx[2], k));
        dyn = __fadd_rn(dyn, __fmul_rn(w, a.accum[c].w));
        if (a.flags[c] & kFlagSolid) stat = __fadd_rn(stat, w);
      }
      if (dyn >= a.c.contact_threshold || stat >= a.c.contact_threshold) {
        a.mask[p] = 1;
        cand = true;
        if (a.c.contact_damping > 0.f) {
          const float s = __fsub_rn(1.0f, a.c.contact_damping);
          a.v[p] = __fmul_rn(a.v[p], s);
          a.v[cap + p] = __fmul_rn(a.v[cap + p], s);
          a.v[2 * cap + p] = __fmul_rn(a.v[2 * cap + p], s);
          damped = true;
        }
      }
    }
  }
  warp_count(&a.cnt->contact_candidates, cand);
  warp_count(&a.cnt->contact_damped, damped);
}

// Sum of the coupling force density over fluid cells (coupling.py:229-232).
__global__ void __launch_bounds__(kBlock) accum_reduce_kernel(Geo g, const float4* __restrict__ accum,
                                                              const uint32_t* __restrict__ flags,
                                                              double* __restrict__ out) {
  double s[3] = {0, 0, 0};
  for (long long c = (long long)blockIdx.x * kBlock + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * kBlock) {
    if (flags[c] & kFlagSolid) continue;
    const float4 v = accum[c];
    s[0] += v.x; s[1] += v.y; s[2] += v.z;
  }
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[ax] += __shfl_down_sync(0xffffffffu, s[ax], o);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out + 0, s[0]);
    atomicAdd(out + 1, s[1]);
    atomicAdd(out + 2, s[2]);
  }
}

// The per-step diagnostics of the coupled runner in one pass (FSISimulation.diagnostics,
// simulation.py:117-147): blocks [0, pblocks) reduce the particles, the rest the lattice
// accumulator over fluid cells; block 0 also copies the counters. out (zeroed by the caller):
// [0] sum m, [1..3] sum m x, [4] max |v|, [5..7] sum particle force, [8..10] sum of the fluid
// reaction over fluid cells, [11..18] the eight counters, [19..21] the IB force totals.
struct RunnerDiagArgs {
  int n;
  long long cap;
  const float* __restrict__ x;
  const float* __restrict__ v;
  const float* __restrict__ mass;
  const float* __restrict__ fp;
  Geo g;
  const float4* __restrict__ accum;
  const uint32_t* __restrict__ flags;
  const Cnt* __restrict__ cnt;
  int pblocks;
};


// hi + lo += x with hi + lo kept as an unevaluated float32 pair (Knuth's TwoSum), so a thread
// sums its particles to about 48 bits without float64 instructions.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

// Adds the block's per-thread float64 values v[0..NV) into out[dst[i]]: the threads' values go
// to shared memory, warp 0 adds them column by column and in a shuffle tree, one atomic each.
// Float64 instructions are this GPU's scarcest: 13 warp instructions per value and block.
template <int NV>
__device__ __forceinline__ void block_add(const double (&v)[NV], double* __restrict__ out,
                                          const int (&dst)[NV]) {
  __shared__ double sh[NV][kBlock];
#pragma unroll
  for (int i = 0; i < NV; ++i) sh[i][threadIdx.x] = v[i];
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double t = 0.0;
#pragma unroll
      for (int r = 0; r < kBlock / 32; ++r) t += sh[i][threadIdx.x + 32 * r];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (threadIdx.x == 0) atomicAdd(out + dst[i], t);
    }
  }
}

// The force assembly with the sum of the fluid reaction over fluid cells read in the same pass
// (the accumulator is read once for both). Warps walk 32-cell tiles grid-stride; each thread
// keeps its running sum as a float32 pair, and each block adds its threads' sums in float64.
constexpr int kAssembleSumPerSm = 6;
__global__ void __launch_bounds__(kBlock, kAssembleSumPerSm)
    assemble_sum_kernel(AssembleArgs a, double* __restrict__ reaction) {
  float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
  const long long tiles = (a.g.n + 31) / 32;
  const long long warps = (long long)gridDim.x * (kBlock / 32);
  for (long long t = (long long)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); t < tiles;
       t += warps) {
    float r[3];
    assemble_body(a, t * 32 + (threadIdx.x & 31), r);
#pragma unroll
    for (int i = 0; i < 3; ++i) ff_add(hi[i], lo[i], r[i]);
  }
  double s3[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) s3[i] = (double)hi[i] + (double)lo[i];
  const int dst[3] = {0, 1, 2};
  block_add<3>(s3, reaction, dst);
}

__global__ void __launch_bounds__(kBlock) runner_diag_kernel(RunnerDiagArgs a, double* __restrict__ out) {
  if (blockIdx.x == 0 && threadIdx.x < 12) {
    if (a.cnt) {
      if (threadIdx.x < 8) {
        const int32_t* c = &a.cnt->unsupported;
        out[11 + threadIdx.x] = (double)c[threadIdx.x];
      } else if (threadIdx.x < 11) {
        out[19 + threadIdx.x - 8] = (double)a.cnt->ib_total[threadIdx.x - 8];
      }
    }
  }
  if ((int)blockIdx.x < a.pblocks) {
    // Sum m, sum m x (exact products split into a rounded part and its remainder), sum f_p:
    // per-thread float32 pairs, one conversion to float64 per thread.
    float hi[7] = {0, 0, 0, 0, 0, 0, 0}, lo[7] = {0, 0, 0, 0, 0, 0, 0};
    float vmax = 0.f;
    for (int p = blockIdx.x * kBlock + threadIdx.x; p < a.n; p += a.pblocks * kBlock) {
      const float ms = a.mass[p];
      ff_add(hi[0], lo[0], ms);
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        const float xa = a.x[ax * a.cap + p];
        const float pr = __fmul_rn(ms, xa);
        ff_add(hi[1 + ax], lo[1 + ax], pr);
        lo[1 + ax] = __fadd_rn(lo[1 + ax], fmaf(ms, xa, -pr));
      }
      const float vx = a.v[p], vy = a.v[a.cap + p], vz = a.v[2 * a.cap + p];
      vmax = fmaxf(vmax, norm3(vx, vy, vz));
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) ff_add(hi[4 + ax], lo[4 + ax], a.fp[ax * a.cap + p]);
    }
    double acc[7];
#pragma unroll
    for (int i = 0; i < 7; ++i) acc[i] = (double)hi[i] + (double)lo[i];
    const int dst[7] = {0, 1, 2, 3, 5, 6, 7};
    block_add<7>(acc, out, dst);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0)
      atomicMax(reinterpret_cast<unsigned long long*>(out + 4),
                (unsigned long long)__double_as_longlong((double)vmax));
  } else if (a.accum) {
    // Fluid-cell sums of the reaction field: each lane adds its cells in float32 for 64 cells
    // and then into float64 (a few float64 instructions per 2,048 cells of a warp), four cells
    // per lane and pass with their loads issued together; no per-cell shuffles.
    double s3[3] = {0, 0, 0};
    float f3[3] = {0.f, 0.f, 0.f};
    int run = 0;
    const int lane = threadIdx.x & 31;
    const long long tiles = (a.g.n + 31) / 32;
    const long long warps = (long long)(gridDim.x - a.pblocks) * (kBlock / 32);
    for (long long t0 = (long long)(blockIdx.x - a.pblocks) * (kBlock / 32) + (threadIdx.x >> 5);
         t0 < tiles; t0 += 4 * warps) {
      uint32_t fl[4];
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const long long c = (t0 + u * warps) * 32 + lane;
        const bool in = c < a.g.n;
        fl[u] = in ? a.flags[c] : kFlagSolid;
        v[u] = in ? a.accum[c] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (!(fl[u] & kFlagSolid)) {
          f3[0] = __fadd_rn(f3[0], v[u].x);
          f3[1] = __fadd_rn(f3[1], v[u].y);
          f3[2] = __fadd_rn(f3[2], v[u].z);
        }
      if (++run == 16) {
#pragma unroll
        for (int i = 0; i < 3; ++i) { s3[i] += (double)f3[i]; f3[i] = 0.f; }
        run = 0;
      }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) s3[i] += (double)f3[i];
    const int dst[3] = {8, 9, 10};
    block_add<3>(s3, out, dst);
  }
}

Geo geo_of(const fsi_lbm_desc* d) { return Geo{d->nx, d->ny, d->nz, (long long)d->nx * d->ny * d->nz}; }
Geo geo_of(const fsi_mpm_desc* d) { return Geo{d->nx, d->ny, d->nz, (long long)d->nx * d->ny * d->nz}; }

}  // namespace
}  // namespace fsi

using namespace fsi;

static_assert(sizeof(Cnt) == sizeof(fsi_coupling_counters), "counter layout");

extern "C" int fsi_coupling_forces(const fsi_coupling_desc* c, const fsi_mpm_desc* m,
                                   const fsi_particles* p, const float* macro,
                                   const uint32_t* flags, float* accum, float* valid_weight,
                                   int32_t* coupling_mask, void* counters, void* stream) {
  FSI_REQUIRE(c && m && p, "NULL descriptor");
  FSI_REQUIRE(macro && flags && accum && valid_weight && coupling_mask && counters, "NULL array");
  FSI_REQUIRE(m->num_particles >= 0 && m->num_particles <= p->capacity, "bad particle count");
  if (m->num_particles == 0) return FSI_OK;
  ForceArgs a;
  a.c = *c;
  a.g = geo_of(m);
  a.n = m->num_particles;
  a.cap = p->capacity;
  a.x = p->x; a.v = p->v; a.mass = p->mass; a.vol = p->volume; a.active = p->active; a.fp = p->force;
  a.macro = reinterpret_cast<const float4*>(macro);
  a.flags = flags;
  a.accum = reinterpret_cast<float4*>(accum);
  a.valid_out = valid_weight;
  a.mask_out = coupling_mask;
  a.cnt = reinterpret_cast<Cnt*>(counters);
  // Few particles (under two CTAs per SM): latency-bound, so the stencil loads go out
  // together; otherwise the lower register count keeps more warps resident.
  if (a.n < kGatherAheadMax)
    coupling_forces_kernel<true><<<grid_for(a.n, kBlock), kBlock, 0, as_stream(stream)>>>(a);
  else
    coupling_forces_kernel<false><<<grid_for(a.n, kBlock), kBlock, 0, as_stream(stream)>>>(a);
  return check_launch("coupling_forces_kernel");
}

namespace fsi {
namespace {
int assemble_launch(const fsi_coupling_desc* c, const fsi_lbm_desc* l, const uint32_t* flags,
                    const float* base_force, int mode, float* accum, const float* macro,
                    float* force, float* ib_force, void* counters, double* reaction,
                    void* stream) {
  FSI_REQUIRE(c && l && base_force, "NULL descriptor");
  FSI_REQUIRE(flags && accum && counters, "NULL array");
  FSI_REQUIRE(!(mode & FSI_ASSEMBLE_IB) || (macro && ib_force), "IB needs macro and ib_force");
  AssembleArgs a;
  a.c = *c;
  a.g = geo_of(l);
  a.flags = flags;
  a.base_dev = nullptr;
  if (mode & FSI_ASSEMBLE_BASE_ON_DEVICE) {
    a.base_dev = base_force;
    for (int i = 0; i < 3; ++i) a.base[i] = 0.f;
  } else {
    for (int i = 0; i < 3; ++i) a.base[i] = base_force[i];
  }
  a.mode = mode;
  a.accum = reinterpret_cast<float4*>(accum);
  a.macro = reinterpret_cast<const float4*>(macro);
  a.force = force;
  a.ib = ib_force;
  a.cnt = reinterpret_cast<Cnt*>(counters);
  cudaStream_t s = as_stream(stream);
  if (!reaction) {
    assemble_kernel<<<grid_for(a.g.n, kBlock), kBlock, 0, s>>>(a);
    return check_launch("assemble_kernel");
  }
  if (cudaMemsetAsync(reaction, 0, 3 * sizeof(double), s) != cudaSuccess)
    return check_launch("memset");
  // one wave of resident blocks (the kernel's launch bounds guarantee kAssembleSumPerSm per
  // SM); the warps walk the tiles grid-stride
  long long blocks = grid_for((a.g.n + 31) / 32, kBlock / 32);
  if (blocks > 152ll * kAssembleSumPerSm) blocks = 152ll * kAssembleSumPerSm;
  assemble_sum_kernel<<<(unsigned)blocks, kBlock, 0, s>>>(a, reaction);
  return check_launch("assemble_sum_kernel");
}
}  // namespace
}  // namespace fsi

extern "C" int fsi_coupling_assemble(const fsi_coupling_desc* c, const fsi_lbm_desc* l,
                                     const uint32_t* flags, const float* base_force, int mode,
                                     float* accum, const float* macro, float* force,
                                     float* ib_force, void* counters, void* stream) {
  return fsi::assemble_launch(c, l, flags, base_force, mode, accum, macro, force, ib_force,
                              counters, nullptr, stream);
}

extern "C" int fsi_coupling_assemble_sum(const fsi_coupling_desc* c, const fsi_lbm_desc* l,
                                         const uint32_t* flags, const float* base_force,
                                         int mode, float* accum, const float* macro,
                                         float* force, float* ib_force, void* counters,
                                         double* reaction, void* stream) {
  FSI_REQUIRE(reaction, "NULL reaction");
  return fsi::assemble_launch(c, l, flags, base_force, mode, accum, macro, force, ib_force,
                              counters, reaction, stream);
}

extern "C" int fsi_contact(const fsi_coupling_desc* c, const fsi_mpm_desc* m,
                           const fsi_particles* p, const float* accum, const uint32_t* flags,
                           int32_t* contact_mask, void* counters, void* stream) {
  FSI_REQUIRE(c && m && p, "NULL descriptor");
  FSI_REQUIRE(accum && flags && contact_mask && counters, "NULL array");
  cudaStream_t s = as_stream(stream);
  Cnt* cnt = reinterpret_cast<Cnt*>(counters);
  if (cudaMemsetAsync(&cnt->contact_candidates, 0, 2 * sizeof(int32_t), s) != cudaSuccess)
    return check_launch("memset");
  if (m->num_particles == 0) return FSI_OK;
  ContactArgs a;
  a.c = *c;
  a.g = geo_of(m);
  a.n = m->num_particles;
  a.cap = p->capacity;
  a.x = p->x; a.v = p->v; a.active = p->active;
  a.accum = reinterpret_cast<const float4*>(accum);
  a.flags = flags;
  a.mask = contact_mask;
  a.cnt = cnt;
  contact_kernel<<<grid_for(a.n, kBlock), kBlock, 0, s>>>(a);
  return check_launch("contact_kernel");
}

extern "C" int fsi_coupling_reduce(const fsi_lbm_desc* l, const float* accum,
                                   const uint32_t* flags, double* out, void* stream) {
  FSI_REQUIRE(l && accum && flags && out, "NULL argument");
  Geo g = geo_of(l);
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out, 0, 4 * sizeof(double), s) != cudaSuccess) return check_launch("memset");
  int blocks = (int)grid_for(g.n, kBlock);
  if (blocks > 152 * 4) blocks = 152 * 4;
  accum_reduce_kernel<<<blocks, kBlock, 0, s>>>(g, reinterpret_cast<const float4*>(accum), flags, out);
  return check_launch("accum_reduce_kernel");
}

extern "C" int fsi_coupled_diagnostics(const fsi_mpm_desc* m, const fsi_particles* p,
                                       const fsi_lbm_desc* l, const float* accum,
                                       const uint32_t* flags, const void* counters, double* out,
                                       void* stream) {
  FSI_REQUIRE(m && p && l && out, "NULL argument");
  FSI_REQUIRE(!accum || flags, "accum needs flags");
  FSI_REQUIRE(m->num_particles >= 0 && m->num_particles <= p->capacity, "bad particle count");
  FSI_REQUIRE(m->nx == l->nx && m->ny == l->ny && m->nz == l->nz, "grids differ");
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out, 0, 22 * sizeof(double), s) != cudaSuccess) return check_launch("memset");
  RunnerDiagArgs a;
  a.n = m->num_particles;
  a.cap = p->capacity;
  a.x = p->x; a.v = p->v; a.mass = p->mass; a.fp = p->force;
  a.g = geo_of(l);
  a.accum = reinterpret_cast<const float4*>(accum);
  a.flags = flags;
  a.cnt = reinterpret_cast<const Cnt*>(counters);
  int pb = (int)grid_for(a.n, kBlock);
  if (pb > 152 * 2) pb = 152 * 2;
  int cb = accum ? (int)grid_for(a.g.n, kBlock) : 0;
  if (cb > 152 * 4) cb = 152 * 4;
  a.pblocks = pb;
  runner_diag_kernel<<<pb + cb, kBlock, 0, s>>>(a, out);
  return check_launch("runner_diag_kernel");
}
