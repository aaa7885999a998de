// Coupling building blocks shared by the single-scene kernels (coupling.cu) and the batched
// kernels (batch.cu): counters, stencil weights, and the per-particle coupling-force and
// per-cell force-assembly bodies.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "fsi_common.cuh"

namespace fsi {
namespace {


struct Cnt {
  int32_t unsupported, partial, clipped, contact_candidates, contact_damped, ib_active, ib_clipped,
      pad;
  float ib_total[4];
};

struct Geo {
  int nx, ny, nz;
  long long n;
};


__device__ __forceinline__ float norm3(float a, float b, float c) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c)));
}

__device__ __forceinline__ void stencil_base(float inv_dx, const float x[3], int base[3],
                                             float fx[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float g = __fmul_rn(x[a], inv_dx);
    base[a] = (int)__fsub_rn(g, 0.5f);
    fx[a] = __fsub_rn(g, (float)base[a]);
  }
}

struct ForceArgs {
  fsi_coupling_desc c;
  Geo g;
  int n;
  long long cap;
  const float* FSI_LAUNCH_RO x;
  const float* FSI_LAUNCH_RO v;
  const float* __restrict__ mass;
  const float* __restrict__ vol;
  const int32_t* __restrict__ active;
  float* __restrict__ fp;
  const float4* FSI_LAUNCH_RO macro;
  const uint32_t* __restrict__ flags;
  float4* __restrict__ accum;
  float* __restrict__ valid_out;
  int32_t* __restrict__ mask_out;
  Cnt* __restrict__ cnt;
};

// Flag bit that records whether node s = 9i + 3j + k of a stencil is solid, in the flag word
// of the stencil's centre node (offset (i-1, j-1, k-1) from it): bit 0 for the centre, bit q
// for the neighbour e_q, a corner bit for the 8 corners.
__host__ __device__ constexpr int stencil_flag_bit(int s) {
  const int di = s / 9 - 1, dj = (s / 3) % 3 - 1, dk = s % 3 - 1;
  if (di == 0 && dj == 0 && dk == 0) return 0;
  if (di != 0 && dj != 0 && dk != 0)
    return kFlagCornerShift + 4 * (di > 0) + 2 * (dj > 0) + (dk > 0);
  for (int q = 1; q < 19; ++q)
    if (ex(q) == di && ey(q) == dj && ez(q) == dk) return q;
  return -1;
}

// The per-particle part of _compute_coupling_forces_kernel (fsi/coupling.py:336-387) for
// active particle p: interpolates the fluid velocity over the in-grid fluid nodes of its
// stencil, and if the valid weight exceeds min_valid_weight computes the penalty force with
// its clipping. Writes the particle force, valid weight and coupling mask; returns true for
// a coupled particle, whose force, valid weight, stencil weights and usable-node mask (bit s:
// node s = 9i + 3j + k is in-grid and fluid) the spread needs. A stencil inside the lattice
// takes the fluid state of its 27 nodes from the centre node's flag word; one that reaches
// past the lattice's faces tests node by node, where kGatherAhead issues the stencil's loads
// up front (fewer dependent round trips, more registers: for launches with few particles,
// where latency and not occupancy bounds the kernel). Every path sums the same values in the
// same order.
template <bool kGatherAhead>
__device__ __forceinline__ bool coupling_particle(const ForceArgs& a, int p, int base[3],
                                                  float wv[3][3], uint32_t& usable, float& valid,
                                                  float pf[3], bool& partial, bool& clipped,
                                                  bool& unsupported) {
  const long long cap = a.cap;
  const float x[3] = {a.x[p], a.x[cap + p], a.x[2 * cap + p]};
  float fx[3];
  stencil_base(a.c.inv_dx, x, base, fx);
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
#pragma unroll
    for (int i = 0; i < 3; ++i) wv[ax][i] = bspline_w(fx[ax], i);
  valid = 0.f;
  float uf[3] = {0.f, 0.f, 0.f};
  usable = 0;
  const bool interior = base[0] >= 0 && base[0] + 2 < a.g.nx && base[1] >= 0 &&
                        base[1] + 2 < a.g.ny && base[2] >= 0 && base[2] + 2 < a.g.nz;
  if (interior) {
    // The whole stencil lies in the lattice: the flag word of its centre node says which of
    // the 27 nodes are fluid, so the lattice-velocity loads go out together (an x-plane of 9
    // nodes at a time) after one dependent load; the sums run in stencil order.
    const long long sx = (long long)a.g.ny * a.g.nz, sy = a.g.nz;
    const long long c1 = (base[0] + 1) * sx + (base[1] + 1) * sy + (base[2] + 1);
    const uint32_t fl = a.flags[c1];
#pragma unroll
    for (int s = 0; s < 27; ++s) usable |= ((~fl >> stencil_flag_bit(s)) & 1u) << s;
    constexpr int kB = 9;
    const float4* FSI_LAUNCH_RO m0 = a.macro + (c1 - sx - sy - 1);
#pragma unroll
    for (int b = 0; b < 27 / kB; ++b) {
      float4 mc[kB];
#pragma unroll
      for (int t = 0; t < kB; ++t) {
        const int s = kB * b + t, i = s / 9, j = (s / 3) % 3, k = s % 3;
        if ((usable >> s) & 1u) mc[t] = m0[i * sx + j * sy + k];
      }
#pragma unroll
      for (int t = 0; t < kB; ++t) {
        const int s = kB * b + t, i = s / 9, j = (s / 3) % 3, k = s % 3;
        if (!((usable >> s) & 1u)) continue;
        const float w = __fmul_rn(__fmul_rn(wv[0][i], wv[1][j]), wv[2][k]);
        valid = __fadd_rn(valid, w);
        uf[0] = __fadd_rn(uf[0], __fmul_rn(w, mc[t].x));
        uf[1] = __fadd_rn(uf[1], __fmul_rn(w, mc[t].y));
        uf[2] = __fadd_rn(uf[2], __fmul_rn(w, mc[t].z));
      }
    }
  } else if (!kGatherAhead) {
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int i = s / 9, j = (s / 3) % 3, k = s % 3;
      const int ni = base[0] + i, nj = base[1] + j, nk = base[2] + k;
      if (ni < 0 || ni >= a.g.nx || nj < 0 || nj >= a.g.ny || nk < 0 || nk >= a.g.nz) continue;
      const long long c = ((long long)ni * a.g.ny + nj) * a.g.nz + nk;
      if (a.flags[c] & kFlagSolid) continue;
      usable |= 1u << s;
      const float w = __fmul_rn(__fmul_rn(wv[0][i], wv[1][j]), wv[2][k]);
      valid = __fadd_rn(valid, w);
      const float4 mc = a.macro[c];
      uf[0] = __fadd_rn(uf[0], __fmul_rn(w, mc.x));
      uf[1] = __fadd_rn(uf[1], __fmul_rn(w, mc.y));
      uf[2] = __fadd_rn(uf[2], __fmul_rn(w, mc.z));
    }
  } else {
    // All loads go out before the first is needed: the 27 flags together, then the lattice
    // velocities of the usable nodes in three batches of 9; the sums still run in stencil
    // order (s = 0..26), so the result is that of the node-by-node loop.
    uint32_t inside = 0;  // bit s: node s of the stencil lies in the lattice
    uint32_t fl[27];
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int i = s / 9, j = (s / 3) % 3, k = s % 3;
      const int ni = base[0] + i, nj = base[1] + j, nk = base[2] + k;
      const bool in = ni >= 0 && ni < a.g.nx && nj >= 0 && nj < a.g.ny && nk >= 0 && nk < a.g.nz;
      inside |= (uint32_t)in << s;
      fl[s] = in ? a.flags[((long long)ni * a.g.ny + nj) * a.g.nz + nk] : kFlagSolid;
    }
#pragma unroll
    for (int s = 0; s < 27; ++s)
      if (((inside >> s) & 1u) && !(fl[s] & kFlagSolid)) usable |= 1u << s;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      float4 mc[9];
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int s = 9 * b + t, j = t / 3, k = t % 3;
        if ((usable >> s) & 1u)
          mc[t] = a.macro[((long long)(base[0] + b) * a.g.ny + (base[1] + j)) * a.g.nz + (base[2] + k)];
      }
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int s = 9 * b + t, j = t / 3, k = t % 3;
        if (!((usable >> s) & 1u)) continue;
        const float w = __fmul_rn(__fmul_rn(wv[0][b], wv[1][j]), wv[2][k]);
        valid = __fadd_rn(valid, w);
        uf[0] = __fadd_rn(uf[0], __fmul_rn(w, mc[t].x));
        uf[1] = __fadd_rn(uf[1], __fmul_rn(w, mc[t].y));
        uf[2] = __fadd_rn(uf[2], __fmul_rn(w, mc[t].z));
      }
    }
  }
  a.valid_out[p] = valid;
  if (!(valid > a.c.min_valid_weight)) {
    a.fp[p] = 0.f; a.fp[cap + p] = 0.f; a.fp[2 * cap + p] = 0.f;
    a.mask_out[p] = 0;
    unsupported = true;
    return false;
  }
  partial = valid < __fsub_rn(1.0f, 1.0e-5f);
  float dv[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    uf[ax] = __fdiv_rn(uf[ax], valid);
    dv[ax] = __fsub_rn(uf[ax], a.v[ax * cap + p]);
  }
  if (a.c.use_rel_limit) {
    const float nrm = norm3(dv[0], dv[1], dv[2]);
    if (nrm > a.c.rel_limit && nrm > 0.f) {
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) dv[ax] = __fmul_rn(__fdiv_rn(dv[ax], nrm), a.c.rel_limit);
      clipped = true;
    }
  }
  const float gm = __fmul_rn(a.c.gamma_eff, a.mass[p]);
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) pf[ax] = __fmul_rn(gm, dv[ax]);
  if (a.c.use_force_limit) {
    const float nrm = norm3(pf[0], pf[1], pf[2]);
    if (nrm > a.c.force_limit && nrm > 0.f) {
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) pf[ax] = __fmul_rn(__fdiv_rn(pf[ax], nrm), a.c.force_limit);
      clipped = true;
    }
  }
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) a.fp[ax * cap + p] = pf[ax];
  a.mask_out[p] = 1;
  return true;
}

// Reaction force xyz and solid-fraction term (w) that a coupled particle with stencil weight
// w, valid weight `valid` and force pf spreads into one fluid node (coupling.py:389-400).
__device__ __forceinline__ float4 coupling_spread_terms(const fsi_coupling_desc& c, float w,
                                                        float valid, const float pf[3], float vp) {
  // x / 1 is exactly x: the divisions by the cell volume are skipped for unit cells (dx = 1).
  const bool unit_cell = c.cell_volume == 1.0f;
  const float nw = __fdiv_rn(w, valid);
  float add[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    add[ax] = __fmul_rn(__fmul_rn(-nw, pf[ax]), c.dt_ratio);
    if (!unit_cell) add[ax] = __fdiv_rn(add[ax], c.cell_volume);
  }
  float ph = __fmul_rn(nw, vp);
  if (!unit_cell) ph = __fdiv_rn(ph, c.cell_volume);
  return make_float4(add[0], add[1], add[2], ph);
}

// _compute_coupling_forces_kernel, fsi/coupling.py:332-406, for particle p (this thread);
// every lane of the warp calls it (warp-aggregated counters). The reaction and solid
// fraction are spread with vector atomics (order of arrival).
template <bool kGatherAhead>
__device__ __forceinline__ void coupling_forces_body(const ForceArgs& a, int p) {
  const bool live = p < a.n;
  const long long cap = a.cap;
  bool partial = false, clipped = false, unsupported = false;
  if (live) {
    if (a.active[p] == 0) {
      a.fp[p] = 0.f; a.fp[cap + p] = 0.f; a.fp[2 * cap + p] = 0.f;
    } else {
      int base[3];
      float wv[3][3], valid, pf[3];
      uint32_t usable;
      if (coupling_particle<kGatherAhead>(a, p, base, wv, usable, valid, pf, partial, clipped,
                                          unsupported)) {
        const float vp = a.vol[p];
#pragma unroll
        for (int s = 0; s < 27; ++s) {
          if (!(usable & (1u << s))) continue;
          const int i = s / 9, j = (s / 3) % 3, k = s % 3;
          const long long c =
              ((long long)(base[0] + i) * a.g.ny + (base[1] + j)) * a.g.nz + (base[2] + k);
          const float w = __fmul_rn(__fmul_rn(wv[0][i], wv[1][j]), wv[2][k]);
          float4 t = coupling_spread_terms(a.c, w, valid, pf, vp);
          if (!a.c.build_fraction) t.w = 0.f;
          red_add_v4(a.accum + c, t.x, t.y, t.z, t.w);
        }
      }
    }
  }
  warp_count(&a.cnt->unsupported, unsupported);
  warp_count(&a.cnt->partial, partial);
  warp_count(&a.cnt->clipped, clipped);
}

// The coupling force alone (the first half of coupling_forces_body): force, valid weight and
// mask of particle p, counters; the spread is left to coupling_spread_body.
__device__ __forceinline__ void coupling_gather_body(const ForceArgs& a, int p) {
  const bool live = p < a.n;
  const long long cap = a.cap;
  bool partial = false, clipped = false, unsupported = false;
  if (live) {
    if (a.active[p] == 0) {
      a.fp[p] = 0.f; a.fp[cap + p] = 0.f; a.fp[2 * cap + p] = 0.f;
    } else {
      int base[3];
      float wv[3][3], valid, pf[3];
      uint32_t usable;
      coupling_particle<false>(a, p, base, wv, usable, valid, pf, partial, clipped, unsupported);
    }
  }
  warp_count(&a.cnt->unsupported, unsupported);
  warp_count(&a.cnt->partial, partial);
  warp_count(&a.cnt->clipped, clipped);
}

// The fluid reaction and solid-fraction spread of a particle that coupling_gather_body coupled
// (mask 1), from its position, stored force and valid weight: the same weights, usable nodes
// and terms as the spread loop of coupling_forces_body.
__device__ __forceinline__ void coupling_spread_body(const ForceArgs& a, int p) {
  if (p >= a.n || a.active[p] == 0 || a.mask_out[p] == 0) return;
  const long long cap = a.cap;
  const float x[3] = {a.x[p], a.x[cap + p], a.x[2 * cap + p]};
  int base[3];
  float fx[3], wv[3][3];
  stencil_base(a.c.inv_dx, x, base, fx);
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
#pragma unroll
    for (int i = 0; i < 3; ++i) wv[ax][i] = bspline_w(fx[ax], i);
  uint32_t usable = 0;
  const long long sx = (long long)a.g.ny * a.g.nz, sy = a.g.nz;
  if (base[0] >= 0 && base[0] + 2 < a.g.nx && base[1] >= 0 && base[1] + 2 < a.g.ny &&
      base[2] >= 0 && base[2] + 2 < a.g.nz) {
    const uint32_t fl = a.flags[(base[0] + 1) * sx + (base[1] + 1) * sy + (base[2] + 1)];
#pragma unroll
    for (int s = 0; s < 27; ++s) usable |= ((~fl >> stencil_flag_bit(s)) & 1u) << s;
  } else {
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int ni = base[0] + s / 9, nj = base[1] + (s / 3) % 3, nk = base[2] + s % 3;
      if (ni < 0 || ni >= a.g.nx || nj < 0 || nj >= a.g.ny || nk < 0 || nk >= a.g.nz) continue;
      if (!(a.flags[ni * sx + nj * sy + nk] & kFlagSolid)) usable |= 1u << s;
    }
  }
  const float valid = a.valid_out[p];
  const float pf[3] = {a.fp[p], a.fp[cap + p], a.fp[2 * cap + p]};
  const float vp = a.vol[p];
#pragma unroll
  for (int s = 0; s < 27; ++s) {
    if (!(usable & (1u << s))) continue;
    const int i = s / 9, j = (s / 3) % 3, k = s % 3;
    const long long c = (base[0] + i) * sx + (base[1] + j) * sy + (base[2] + k);
    const float w = __fmul_rn(__fmul_rn(wv[0][i], wv[1][j]), wv[2][k]);
    float4 t = coupling_spread_terms(a.c, w, valid, pf, vp);
    if (!a.c.build_fraction) t.w = 0.f;
    red_add_v4(a.accum + c, t.x, t.y, t.z, t.w);
  }
}

struct AssembleArgs {
  fsi_coupling_desc c;
  Geo g;
  const uint32_t* __restrict__ flags;
  float base[3];
  const float* base_dev;  // device float[3] read in place of base, or NULL
  int mode;
  float4* __restrict__ accum;
  const float4* FSI_LAUNCH_RO macro;
  float* __restrict__ force;
  float* __restrict__ ib;
  Cnt* __restrict__ cnt;
};

// _clamp_solid_volume_fraction_kernel + reset_force + _apply_coupling_force_to_lbm_kernel +
// _compute/_apply_immersed_boundary_force_kernel (coupling.py:408-461, lbm3d.py:504-510).
// Cell c (this thread); every lane of the warp calls it. With `reaction` non-NULL it also
// returns the cell's fluid reaction (accum.xyz on a fluid cell, else 0), the term that
// total_fluid_coupling_force (coupling.py:229-232) sums.
__device__ __forceinline__ void assemble_body(const AssembleArgs& a, long long c,
                                              float* reaction = nullptr) {
  bool ib_active = false, ib_clipped = false;
  float ibf[3] = {0.f, 0.f, 0.f};
  if (reaction) reaction[0] = reaction[1] = reaction[2] = 0.f;
  if (c < a.g.n) {
    const bool fluid = !(a.flags[c] & kFlagSolid);
    float4 acc = a.accum[c];
    if (reaction && fluid) {
      reaction[0] = acc.x;
      reaction[1] = acc.y;
      reaction[2] = acc.z;
    }
    if ((a.mode & FSI_ASSEMBLE_CLAMP_FRACTION) && !(acc.w <= 1.0f)) {
      // min(phi, 1): only cells above one (or NaN) change, so only they are written back
      acc.w = fminf(acc.w, 1.0f);
      a.accum[c].w = acc.w;
    }
    const float b0 = a.base_dev ? a.base_dev[0] : a.base[0];
    const float b1 = a.base_dev ? a.base_dev[1] : a.base[1];
    const float b2 = a.base_dev ? a.base_dev[2] : a.base[2];
    float f[3] = {fluid ? b0 : 0.f, fluid ? b1 : 0.f, fluid ? b2 : 0.f};
    if (a.mode & FSI_ASSEMBLE_COUPLING) {
      f[0] = fluid ? __fadd_rn(f[0], acc.x) : 0.f;
      f[1] = fluid ? __fadd_rn(f[1], acc.y) : 0.f;
      f[2] = fluid ? __fadd_rn(f[2], acc.z) : 0.f;
    }
    if (a.mode & FSI_ASSEMBLE_IB) {
      if (a.c.ib_enabled && a.c.ib_drag > 0.f && fluid) {
        const float phi = acc.w;
        if (phi > 0.f && phi >= a.c.ib_threshold) {
          const float4 mc = a.macro[c];
          const float s = __fmul_rn(__fmul_rn(-a.c.ib_drag, phi), mc.w);
          ibf[0] = __fmul_rn(s, mc.x); ibf[1] = __fmul_rn(s, mc.y); ibf[2] = __fmul_rn(s, mc.z);
          const float nrm = norm3(ibf[0], ibf[1], ibf[2]);
          if (a.c.ib_use_max && nrm > a.c.ib_max_force && nrm > 0.f) {
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) ibf[ax] = __fmul_rn(__fdiv_rn(ibf[ax], nrm), a.c.ib_max_force);
            ib_clipped = true;
          }
          ib_active = true;
        }
      }
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        a.ib[ax * a.g.n + c] = ibf[ax];
        f[ax] = fluid ? __fadd_rn(f[ax], ibf[ax]) : 0.f;
      }
    }
    if (a.force) {
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) a.force[ax * a.g.n + c] = f[ax];
    }
  }
  if (a.mode & FSI_ASSEMBLE_IB) {
    warp_count(&a.cnt->ib_active, ib_active);
    warp_count(&a.cnt->ib_clipped, ib_clipped);
    float t[3] = {ibf[0], ibf[1], ibf[2]};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t[ax] += __shfl_down_sync(0xffffffffu, t[ax], o);
    }
    const bool warp_active = __any_sync(0xffffffffu, ib_active);
    if ((threadIdx.x & 31) == 0 && warp_active) {
      atomicAdd(&a.cnt->ib_total[0], t[0]);
      atomicAdd(&a.cnt->ib_total[1], t[1]);
      atomicAdd(&a.cnt->ib_total[2], t[2]);
    }
  }
}

}  // namespace
}  // namespace fsi
