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
// "AA-odd" arrangement that gather_post_stream() undoes.
//
// The collision reproduces the reference's float32 arithmetic operation for
// operation (the kernel is compiled with -fmad=false and uses *_rn intrinsics):
// the MRT transforms are generated register formulas (lbm_formulas.cuh).
#include <cuda_runtime.h>

#include <cstdint>

#include "fsi_common.cuh"
#include "lbm_formulas.cuh"

namespace fsi {
namespace {

constexpr int kBlock = 256;

struct LbmGeom {
  int nx, ny, nz;
  long long n;  // cells
};

__host__ LbmGeom geom_of(const fsi_lbm_desc* d) {
  return LbmGeom{d->nx, d->ny, d->nz, (long long)d->nx * d->ny * d->nz};
}

// Wrapped neighbour coordinates of a cell for offsets -1, 0, +1 on each axis.
struct Nbr {
  int i[3], j[3], k[3];
  int ny, nz;
  __device__ Nbr(long long c, const LbmGeom& g) : ny(g.ny), nz(g.nz) {
    int kk = (int)(c % g.nz);
    long long r = c / g.nz;
    int jj = (int)(r % g.ny);
    int ii = (int)(r / g.ny);
    i[1] = ii; j[1] = jj; k[1] = kk;
    i[0] = ii == 0 ? g.nx - 1 : ii - 1; i[2] = ii == g.nx - 1 ? 0 : ii + 1;
    j[0] = jj == 0 ? g.ny - 1 : jj - 1; j[2] = jj == g.ny - 1 ? 0 : jj + 1;
    k[0] = kk == 0 ? g.nz - 1 : kk - 1; k[2] = kk == g.nz - 1 ? 0 : kk + 1;
  }
  // Linear index of x + s*e_q (s = +1 or -1), periodic in all axes (lbm3d.py:335-350).
  __device__ __forceinline__ long long at(int q, int s) const {
    int I = i[1 + s * ex(q)], J = j[1 + s * ey(q)], K = k[1 + s * ez(q)];
    return ((long long)I * ny + J) * nz + K;
  }
};

// Post-stream population F_q(x) of the current state (parity = steps done mod 2).
__device__ __forceinline__ float gather_post_stream(const float* __restrict__ pops, long long n,
                                                    long long c, const Nbr& nb, uint32_t fl,
                                                    int q, int parity) {
  if (parity == 0 || q == 0) return pops[(long long)q * n + c];
  const int o = opp(q);
  if (fl & (1u << o)) return pops[(long long)q * n + c];
  return pops[(long long)o * n + nb.at(q, -1)];
}

__device__ __forceinline__ float* post_stream_slot(float* pops, long long n, long long c,
                                                   const Nbr& nb, uint32_t fl, int q,
                                                   int parity) {
  if (parity == 0 || q == 0) return pops + (long long)q * n + c;
  const int o = opp(q);
  if (fl & (1u << o)) return pops + (long long)q * n + c;
  return pops + (long long)o * n + nb.at(q, -1);
}

// rho and u as update_macro computes them (lbm3d.py:409-425): sequential sums
// in q order, then u = u / rho, u = u + (force * 0.5) / rho.
__device__ __forceinline__ void macro_of(const float (&F)[19], float gx, float gy, float gz,
                                         float& rho, float& ux, float& uy, float& uz) {
  float r = F[0];
#pragma unroll
  for (int q = 1; q < 19; ++q) r = __fadd_rn(r, F[q]);
  float x = __fsub_rn(F[1], F[2]);
  x = __fadd_rn(x, F[7]); x = __fsub_rn(x, F[8]); x = __fadd_rn(x, F[9]); x = __fsub_rn(x, F[10]);
  x = __fadd_rn(x, F[11]); x = __fsub_rn(x, F[12]); x = __fadd_rn(x, F[13]); x = __fsub_rn(x, F[14]);
  float y = __fsub_rn(F[3], F[4]);
  y = __fadd_rn(y, F[7]); y = __fsub_rn(y, F[8]); y = __fsub_rn(y, F[9]); y = __fadd_rn(y, F[10]);
  y = __fadd_rn(y, F[15]); y = __fsub_rn(y, F[16]); y = __fadd_rn(y, F[17]); y = __fsub_rn(y, F[18]);
  float z = __fsub_rn(F[5], F[6]);
  z = __fadd_rn(z, F[11]); z = __fsub_rn(z, F[12]); z = __fsub_rn(z, F[13]); z = __fadd_rn(z, F[14]);
  z = __fadd_rn(z, F[15]); z = __fsub_rn(z, F[16]); z = __fsub_rn(z, F[17]); z = __fadd_rn(z, F[18]);
  x = __fdiv_rn(x, r); y = __fdiv_rn(y, r); z = __fdiv_rn(z, r);
  x = __fadd_rn(x, __fdiv_rn(__fmul_rn(gx, 0.5f), r));
  y = __fadd_rn(y, __fdiv_rn(__fmul_rn(gy, 0.5f), r));
  z = __fadd_rn(z, __fdiv_rn(__fmul_rn(gz, 0.5f), r));
  rho = r; ux = x; uy = y; uz = z;
}

// Sum of the non-zero terms e_c * v_c in x, y, z order (Taichi Vector.dot with
// exact zero products dropped).
__device__ __forceinline__ float edot(int q, float vx, float vy, float vz) {
  float s = 0.0f;
  bool first = true;
  if (ex(q) != 0) { s = ex(q) > 0 ? vx : -vx; first = false; }
  if (ey(q) != 0) { float t = ey(q) > 0 ? vy : -vy; s = first ? t : __fadd_rn(s, t); first = false; }
  if (ez(q) != 0) { float t = ez(q) > 0 ? vz : -vz; s = first ? t : __fadd_rn(s, t); }
  return s;
}

// MRT collision with Guo forcing of one fluid cell (lbm3d.py:276-333).
__device__ __forceinline__ void collide_cell(const float (&F)[19], float rho, float ux, float uy,
                                             float uz, float gx, float gy, float gz,
                                             const float* __restrict__ S, float (&out)[19]) {
  // Guo source terms t_q = w_q ((e_q - u).G + (e_q.u)(e_q.G)) (lbm3d.py:276-283).
  // (e - u_c) G_c takes three values per axis, for e = -1, 0, +1.
  const float dx[3] = {__fmul_rn(__fsub_rn(-1.0f, ux), gx), __fmul_rn(-ux, gx),
                       __fmul_rn(__fsub_rn(1.0f, ux), gx)};
  const float dy[3] = {__fmul_rn(__fsub_rn(-1.0f, uy), gy), __fmul_rn(-uy, gy),
                       __fmul_rn(__fsub_rn(1.0f, uy), gy)};
  const float dz[3] = {__fmul_rn(__fsub_rn(-1.0f, uz), gz), __fmul_rn(-uz, gz),
                       __fmul_rn(__fsub_rn(1.0f, uz), gz)};
  float t[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    float a = __fadd_rn(__fadd_rn(dx[ex(q) + 1], dy[ey(q) + 1]), dz[ez(q) + 1]);
    float b = q == 0 ? 0.0f : __fmul_rn(edot(q, ux, uy, uz), edot(q, gx, gy, gz));
    t[q] = __fmul_rn(weight_of(q), q == 0 ? a : __fadd_rn(a, b));
  }
  float g[19], m[19];
  mrt_forward(t, g);
  mrt_forward(F, m);
  // Relaxation towards meq (lbm3d.py:285-326). S_0 = S_3 = S_5 = S_7 = 0: those
  // moments only receive the forcing term.
  const float uu = __fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)), __fmul_rn(uz, uz));
  float meq[19];
#pragma unroll
  for (int k = 0; k < 19; ++k) meq[k] = 0.0f;
  meq[1] = uu;
  meq[9] = __fsub_rn(__fsub_rn(__fmul_rn(__fmul_rn(2.0f, ux), ux), __fmul_rn(uy, uy)),
                     __fmul_rn(uz, uz));
  meq[11] = __fsub_rn(__fmul_rn(uy, uy), __fmul_rn(uz, uz));
  meq[13] = __fmul_rn(ux, uy);
  meq[14] = __fmul_rn(uy, uz);
  meq[15] = __fmul_rn(ux, uz);
  (void)rho;
#pragma unroll
  for (int k = 0; k < 19; ++k) {
    if (k == 0 || k == 3 || k == 5 || k == 7) {
      m[k] = __fadd_rn(m[k], g[k]);
    } else {
      const bool has_eq = (k == 1 || k == 9 || k == 11 || k == 13 || k == 14 || k == 15);
      float d = has_eq ? __fsub_rn(m[k], meq[k]) : m[k];
      m[k] = __fsub_rn(m[k], __fmul_rn(S[k], d));
      m[k] = __fadd_rn(m[k], __fmul_rn(__fsub_rn(1.0f, __fmul_rn(0.5f, S[k])), g[k]));
    }
  }
  mrt_inverse(m, out);
}

struct StepArgs {
  LbmGeom g;
  float* __restrict__ pops;
  float4* __restrict__ macro;
  const float* __restrict__ force;
  const float* __restrict__ force_prev;
  const uint32_t* __restrict__ flags;
  float s[19];
  int write_faces;
};

template <bool kOdd, bool kRecompute>
__global__ void __launch_bounds__(kBlock) lbm_step_kernel(StepArgs a) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= a.g.n) return;
  const uint32_t fl = a.flags[c];
  if (fl & kFlagSolid) return;
  const long long n = a.g.n;
  const Nbr nb(c, a.g);

  float F[19];
  if (!kOdd) {
#pragma unroll
    for (int q = 0; q < 19; ++q) F[q] = a.pops[(long long)q * n + c];
  } else {
#pragma unroll
    for (int q = 0; q < 19; ++q) F[q] = gather_post_stream(a.pops, n, c, nb, fl, q, 1);
  }

  const float gx = a.force[c], gy = a.force[n + c], gz = a.force[2 * n + c];
  float rho, ux, uy, uz;
  if (kRecompute) {
    macro_of(F, a.force_prev[c], a.force_prev[n + c], a.force_prev[2 * n + c], rho, ux, uy, uz);
    if (a.write_faces && (fl & (kFlagFaceLeft | kFlagFaceRight)))
      a.macro[c] = make_float4(ux, uy, uz, rho);
  } else {
    const float4 mc = a.macro[c];
    ux = mc.x; uy = mc.y; uz = mc.z; rho = mc.w;
  }

  float out[19];
  collide_cell(F, rho, ux, uy, uz, gx, gy, gz, a.s, out);

  if (!kOdd) {
#pragma unroll
    for (int q = 0; q < 19; ++q) a.pops[(long long)opp(q) * n + c] = out[q];
  } else {
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      if (q == 0 || (fl & (1u << q)))
        a.pops[(long long)opp(q) * n + c] = out[q];
      else
        a.pops[(long long)q * n + nb.at(q, +1)] = out[q];
    }
  }
}

// x-face conditions applied to the post-stream state (lbm3d.py:363-407).
struct FaceArgs {
  LbmGeom g;
  float* __restrict__ pops;
  const float4* __restrict__ macro;  // u of the state before this step, on face cells
  const uint32_t* __restrict__ flags;
  int parity;  // of the state after the step
  int mode[2];
  float bc_rho[2];
  float bc_vel[2][3];
  float rho0;
};

__global__ void __launch_bounds__(kBlock) lbm_face_kernel(FaceArgs a) {
  const long long per_face = (long long)a.g.ny * a.g.nz;
  const long long t = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (t >= 2 * per_face) return;
  const int side = (int)(t / per_face);
  const int mode = a.mode[side];
  if (mode == 0) return;
  const long long c = (side == 0 ? 0 : (long long)(a.g.nx - 1) * per_face) + (t % per_face);
  const uint32_t fl = a.flags[c];
  if (fl & kFlagSolid) return;
  const long long n = a.g.n;
  const Nbr nb(c, a.g);
  float F[19];
  float* slot[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    slot[q] = post_stream_slot(a.pops, n, c, nb, fl, q, a.parity);
    F[q] = *slot[q];
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
  } else {
    // Velocity: F_q = feq_opp - F_opp + feq_q, sequentially in q with the
    // already-updated F_opp (the reference updates the field in place).
    const float* v = a.bc_vel[side];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const int o = opp(q);
      float val = __fsub_rn(feq_ref(o, a.rho0, v[0], v[1], v[2]), F[o]);
      F[q] = __fadd_rn(val, feq_ref(q, a.rho0, v[0], v[1], v[2]));
    }
  }
#pragma unroll
  for (int q = 0; q < 19; ++q) *slot[q] = F[q];
}

struct MacroArgs {
  LbmGeom g;
  const float* __restrict__ pops;
  const float* __restrict__ force;
  const uint32_t* __restrict__ flags;
  float4* __restrict__ macro;
  int parity;
  float rho0;
};

__global__ void __launch_bounds__(kBlock) lbm_macro_kernel(MacroArgs a) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= a.g.n) return;
  const uint32_t fl = a.flags[c];
  if (fl & kFlagSolid) {
    a.macro[c] = make_float4(0.f, 0.f, 0.f, a.rho0);
    return;
  }
  const long long n = a.g.n;
  const Nbr nb(c, a.g);
  float F[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) F[q] = gather_post_stream(a.pops, n, c, nb, fl, q, a.parity);
  float rho, ux, uy, uz;
  macro_of(F, a.force[c], a.force[n + c], a.force[2 * n + c], rho, ux, uy, uz);
  a.macro[c] = make_float4(ux, uy, uz, rho);
}

__global__ void __launch_bounds__(kBlock) lbm_distribution_kernel(LbmGeom g,
                                                                  const float* __restrict__ pops,
                                                                  const uint32_t* __restrict__ flags,
                                                                  int parity,
                                                                  float* __restrict__ out) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= g.n) return;
  const uint32_t fl = flags[c];
  const Nbr nb(c, g);
  const int p = (fl & kFlagSolid) ? 0 : parity;
#pragma unroll
  for (int q = 0; q < 19; ++q) out[c * 19 + q] = gather_post_stream(pops, g.n, c, nb, fl, q, p);
}

__global__ void __launch_bounds__(kBlock) lbm_flags_kernel(LbmGeom g,
                                                           const int32_t* __restrict__ solid,
                                                           uint32_t* __restrict__ flags) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= g.n) return;
  const Nbr nb(c, g);
  uint32_t f = solid[c] != 0 ? kFlagSolid : 0u;
#pragma unroll
  for (int q = 1; q < 19; ++q)
    if (solid[nb.at(q, +1)] != 0) f |= 1u << q;
  if (nb.i[1] == 0) f |= kFlagFaceLeft;
  if (nb.i[1] == g.nx - 1) f |= kFlagFaceRight;
  flags[c] = f;
}

__global__ void __launch_bounds__(kBlock) lbm_init_kernel(LbmGeom g,
                                                          const uint32_t* __restrict__ flags,
                                                          float rho0, float u0x, float u0y,
                                                          float u0z, float* __restrict__ pops,
                                                          float4* __restrict__ macro) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= g.n) return;
  const bool solid = flags[c] & kFlagSolid;
  const float ux = solid ? 0.f : u0x, uy = solid ? 0.f : u0y, uz = solid ? 0.f : u0z;
  macro[c] = make_float4(ux, uy, uz, rho0);
#pragma unroll
  for (int q = 0; q < 19; ++q) pops[(long long)q * g.n + c] = feq_ref(q, rho0, ux, uy, uz);
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

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

__global__ void __launch_bounds__(kBlock) lbm_reduce_kernel(LbmGeom g,
                                                            const float4* __restrict__ macro,
                                                            const float* __restrict__ force,
                                                            const uint32_t* __restrict__ flags,
                                                            double* __restrict__ out) {
  double mass = 0, fx = 0, fy = 0, fz = 0;
  float vmax = 0.f;
  for (long long c = (long long)blockIdx.x * kBlock + threadIdx.x; c < g.n;
       c += (long long)gridDim.x * kBlock) {
    const float4 m = macro[c];
    // numpy float32 norm of a length-3 vector: sqrt((x*x + y*y) + z*z).
    const float nrm = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(m.x, m.x), __fmul_rn(m.y, m.y)), __fmul_rn(m.z, m.z)));
    vmax = fmaxf(vmax, nrm);
    if (!(flags[c] & kFlagSolid)) {
      mass += (double)m.w;
      if (force) {
        fx += (double)force[c];
        fy += (double)force[g.n + c];
        fz += (double)force[2 * g.n + c];
      }
    }
  }
  __shared__ double sh[4][kBlock / 32];
  __shared__ float shm[kBlock / 32];
  mass = warp_sum(mass); fx = warp_sum(fx); fy = warp_sum(fy); fz = warp_sum(fz);
  vmax = warp_max(vmax);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[0][wid] = mass; sh[1][wid] = fx; sh[2][wid] = fy; sh[3][wid] = fz; shm[wid] = vmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[4] = {0, 0, 0, 0};
    float mx = 0.f;
    for (int w = 0; w < kBlock / 32; ++w) {
      for (int i = 0; i < 4; ++i) s[i] += sh[i][w];
      mx = fmaxf(mx, shm[w]);
    }
    atomicAdd(out + 0, s[0]);
    atomic_max_nonneg(out + 1, (double)mx);
    atomicAdd(out + 2, s[1]);
    atomicAdd(out + 3, s[2]);
    atomicAdd(out + 4, s[3]);
  }
}

int check_desc(const fsi_lbm_desc* d) {
  FSI_REQUIRE(d != nullptr, "lbm descriptor is NULL");
  FSI_REQUIRE(d->nx > 4 && d->ny > 4 && d->nz > 4, "lattice %dx%dx%d too small", d->nx, d->ny, d->nz);
  FSI_REQUIRE((long long)d->nx * d->ny * d->nz < (1ll << 40), "lattice too large");
  FSI_REQUIRE(d->s[0] == 0.f && d->s[3] == 0.f && d->s[5] == 0.f && d->s[7] == 0.f,
              "conserved moments (0, 3, 5, 7) must have zero relaxation rate");
  for (int side = 0; side < 2; ++side) {
    int m = side == 0 ? d->bc_mode_left : d->bc_mode_right;
    FSI_REQUIRE(m >= 0 && m <= 2, "unknown x boundary mode %d", m);
  }
  return FSI_OK;
}

}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_lbm_build_flags(const fsi_lbm_desc* d, const int32_t* solid, uint32_t* flags,
                                   void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(solid && flags, "NULL array");
  LbmGeom g = geom_of(d);
  lbm_flags_kernel<<<grid_for(g.n, kBlock), kBlock, 0, as_stream(stream)>>>(g, solid, flags);
  return check_launch("lbm_flags_kernel");
}

extern "C" int fsi_lbm_init_fields(const fsi_lbm_desc* d, const uint32_t* flags, const float* u0,
                                   float* pops, float* macro, void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(flags && u0 && pops && macro, "NULL array");
  LbmGeom g = geom_of(d);
  lbm_init_kernel<<<grid_for(g.n, kBlock), kBlock, 0, as_stream(stream)>>>(
      g, flags, d->rho0, u0[0], u0[1], u0[2], pops, reinterpret_cast<float4*>(macro));
  return check_launch("lbm_init_kernel");
}

extern "C" int fsi_lbm_step(const fsi_lbm_desc* d, float* pops, float* macro, const float* force,
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
  for (int k = 0; k < 19; ++k) a.s[k] = d->s[k];
  a.write_faces = (d->bc_mode_left != 0 || d->bc_mode_right != 0) ? 1 : 0;
  cudaStream_t s = as_stream(stream);
  const unsigned grid = grid_for(a.g.n, kBlock);
  const bool odd = (steps_done & 1) != 0;
  if (force_prev) {
    if (odd) lbm_step_kernel<true, true><<<grid, kBlock, 0, s>>>(a);
    else lbm_step_kernel<false, true><<<grid, kBlock, 0, s>>>(a);
  } else {
    if (odd) lbm_step_kernel<true, false><<<grid, kBlock, 0, s>>>(a);
    else lbm_step_kernel<false, false><<<grid, kBlock, 0, s>>>(a);
  }
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
    const long long faces = 2ll * d->ny * d->nz;
    lbm_face_kernel<<<grid_for(faces, kBlock), kBlock, 0, s>>>(f);
    if (int e = check_launch("lbm_face_kernel")) return e;
  }
  return FSI_OK;
}

extern "C" int fsi_lbm_update_macro(const fsi_lbm_desc* d, const float* pops, const float* force,
                                    const uint32_t* flags, int64_t steps_done, float* macro,
                                    void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(pops && force && flags && macro, "NULL array");
  MacroArgs a{geom_of(d), pops, force, flags, reinterpret_cast<float4*>(macro),
              (int)(steps_done & 1), d->rho0};
  lbm_macro_kernel<<<grid_for(a.g.n, kBlock), kBlock, 0, as_stream(stream)>>>(a);
  return check_launch("lbm_macro_kernel");
}

extern "C" int fsi_lbm_distribution(const fsi_lbm_desc* d, const float* pops,
                                    const uint32_t* flags, int64_t steps_done, float* out,
                                    void* stream) {
  if (int e = check_desc(d)) return e;
  FSI_REQUIRE(pops && flags && out, "NULL array");
  LbmGeom g = geom_of(d);
  lbm_distribution_kernel<<<grid_for(g.n, kBlock), kBlock, 0, as_stream(stream)>>>(
      g, pops, flags, (int)(steps_done & 1), out);
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
  int blocks = (int)grid_for(g.n, kBlock);
  if (blocks > 152 * 8) blocks = 152 * 8;
  lbm_reduce_kernel<<<blocks, kBlock, 0, s>>>(g, reinterpret_cast<const float4*>(macro), force,
                                              flags, out);
  return check_launch("lbm_reduce_kernel");
}
