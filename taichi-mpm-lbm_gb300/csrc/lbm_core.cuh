// Lattice Boltzmann building blocks shared by the single-lattice kernels (lbm.cu) and the
// batched kernels (batch.cu): geometry, storage forms, macroscopic fields, the MRT
// collision in the exact and fast forms, and the fused AA-pattern step of a thread's cells.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include "fsi_common.cuh"
#include "lbm_formulas.cuh"
#include "lbm_vec.cuh"

namespace fsi {
namespace {


struct LbmGeom {
  int nx, ny, nz;
  long long n;  // cells
};

__host__ LbmGeom geom_of(const fsi_lbm_desc* d) {
  return LbmGeom{d->nx, d->ny, d->nz, (long long)d->nx * d->ny * d->nz};
}

// Launch shape of the cell kernels: x = z (contiguous, coalesced), y = y rows, z = x planes,
// so a thread knows (i, j, k) without integer division.
struct CellLaunch {
  dim3 grid, block;
};

CellLaunch cell_launch(const LbmGeom& g) {
  int bz = ((g.nz + 31) / 32) * 32;
  if (bz > kBlock) bz = kBlock;
  int by = kBlock / bz;
  if (by > g.ny) by = g.ny;
  return CellLaunch{dim3((g.nz + bz - 1) / bz, (g.ny + by - 1) / by, g.nx), dim3(bz, by, 1)};
}

// Signed 32-bit offsets from a cell to its +-1 neighbours on each axis, periodic wrap included
// (lbm3d.py:335-350). A neighbour index is then one three-operand add.
struct Deltas {
  uint32_t c;
  int xp, xm, yp, ym, zp, zm;
  __device__ __forceinline__ Deltas() {}
  __device__ __forceinline__ Deltas(const LbmGeom& g, int i, int j, int k) {
    const int nyz = g.ny * g.nz;
    c = (uint32_t)((i * g.ny + j) * g.nz + k);
    xp = i == g.nx - 1 ? -(g.nx - 1) * nyz : nyz;
    xm = i == 0 ? (g.nx - 1) * nyz : -nyz;
    yp = j == g.ny - 1 ? -(g.ny - 1) * g.nz : g.nz;
    ym = j == 0 ? (g.ny - 1) * g.nz : -g.nz;
    zp = k == g.nz - 1 ? -(g.nz - 1) : 1;
    zm = k == 0 ? g.nz - 1 : -1;
  }
  // Index of x + s * e_q.
  __device__ __forceinline__ uint32_t nb(int q, int s) const {
    const int dx = s * ex(q), dy = s * ey(q), dz = s * ez(q);
    const int ox = dx > 0 ? xp : (dx < 0 ? xm : 0);
    const int oy = dy > 0 ? yp : (dy < 0 ? ym : 0);
    const int oz = dz > 0 ? zp : (dz < 0 ? zm : 0);
    return c + (uint32_t)(ox + oy + oz);
  }
};

// Flag bits of the 8 corner neighbours x + (+-1, +-1, +-1) of the cell of d (periodic wrap),
// from the 0/1 solid mask.
__device__ __forceinline__ uint32_t corner_flag_bits(const int32_t* __restrict__ solid,
                                                     const Deltas& d) {
  uint32_t f = 0;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const uint32_t nb = d.c + (uint32_t)((a ? d.xp : d.xm) + (b ? d.yp : d.ym) + (c ? d.zp : d.zm));
        if (solid[nb] != 0) f |= 1u << (kFlagCornerShift + 4 * a + 2 * b + c);
      }
  return f;
}

// ------------------------------------------------------------- storage forms
// ld(p, i, s) returns population i as float given its rest-equilibrium shift s = w_q rho0;
// st(p, i, v, s) stores population value v.
template <int kStore>
struct Store;

template <>
struct Store<FSI_STORAGE_F32> {
  using T = float;
  static __device__ __forceinline__ float ld(const T* p, uint32_t i, float) { return p[i]; }
  static __device__ __forceinline__ void st(T* p, uint32_t i, float v, float) { p[i] = v; }
  static __device__ __forceinline__ float2 ld2(const T* p, uint32_t i0, uint32_t i1, float) {
    return make_float2(p[i0], p[i1]);
  }
  static __device__ __forceinline__ void st2(T* p, uint32_t i0, uint32_t i1, float2 v, float) {
    p[i0] = v.x;
    p[i1] = v.y;
  }
};

constexpr float kF16Scale = 4096.0f;  // deviations of order 1e-8..1e-1 map into FP16's normal range

template <>
struct Store<FSI_STORAGE_F16> {
  using T = __half;
  static __device__ __forceinline__ float ld(const T* p, uint32_t i, float s) {
    return fmaf(__half2float(p[i]), 1.0f / kF16Scale, s);
  }
  static __device__ __forceinline__ void st(T* p, uint32_t i, float v, float s) {
    p[i] = __float2half_rn((v - s) * kF16Scale);
  }
  // Two values at once: one packed conversion and one packed fma / sub+mul per pair.
  static __device__ __forceinline__ float2 ld2(const T* p, uint32_t i0, uint32_t i1, float s) {
    const float2 h = __half22float2(__halves2half2(p[i0], p[i1]));
    return vfma(h, make_float2(1.0f / kF16Scale, 1.0f / kF16Scale), make_float2(s, s));
  }
  static __device__ __forceinline__ void st2(T* p, uint32_t i0, uint32_t i1, float2 v, float s) {
    const __half2 h = __float22half2_rn(vmul(vsub(v, s), kF16Scale));
    p[i0] = __low2half(h);
    p[i1] = __high2half(h);
  }
};

template <>
struct Store<FSI_STORAGE_BF16> {
  using T = __nv_bfloat16;
  static __device__ __forceinline__ float ld(const T* p, uint32_t i, float s) {
    return __bfloat162float(p[i]) + s;
  }
  static __device__ __forceinline__ void st(T* p, uint32_t i, float v, float s) {
    p[i] = __float2bfloat16_rn(v - s);
  }
  static __device__ __forceinline__ float2 ld2(const T* p, uint32_t i0, uint32_t i1, float s) {
    return vadd(__bfloat1622float2(__halves2bfloat162(p[i0], p[i1])), s);
  }
  static __device__ __forceinline__ void st2(T* p, uint32_t i0, uint32_t i1, float2 v, float s) {
    const __nv_bfloat162 h = __float22bfloat162_rn(vsub(v, s));
    p[i0] = __low2bfloat16(h);
    p[i1] = __high2bfloat16(h);
  }
};

// Post-stream F_q(x) of a fluid cell in a state of the given parity.
template <int kStore>
__device__ __forceinline__ float gather32(const typename Store<kStore>::T* FSI_LAUNCH_RO pops,
                                          uint32_t n, const Deltas& d, uint32_t fl, int q,
                                          int parity, float shift) {
  if (parity == 0 || q == 0 || ((fl >> opp(q)) & 1u)) return Store<kStore>::ld(pops, q * n + d.c, shift);
  return Store<kStore>::ld(pops, opp(q) * n + d.nb(q, -1), shift);
}

// Storage index of F_q(x) in a state of the given parity (the slot a gather reads).
__device__ __forceinline__ uint32_t slot32(uint32_t n, const Deltas& d, uint32_t fl, int q,
                                           int parity) {
  if (parity == 0 || q == 0 || ((fl >> opp(q)) & 1u)) return q * n + d.c;
  return opp(q) * n + d.nb(q, -1);
}

// ---------------------------------------------------------------- macro fields
// rho and u as update_macro computes them (lbm3d.py:409-425): sequential sums
// in q order, then u = u / rho, u = u + (force * 0.5) / rho.
template <class V>
__device__ __forceinline__ void macro_of(const V (&F)[19], V gx, V gy, V gz, V& rho, V& ux, V& uy,
                                         V& uz) {
  V r = F[0];
#pragma unroll
  for (int q = 1; q < 19; ++q) r = vadd(r, F[q]);
  V x = vsub(F[1], F[2]);
  x = vadd(x, F[7]); x = vsub(x, F[8]); x = vadd(x, F[9]); x = vsub(x, F[10]);
  x = vadd(x, F[11]); x = vsub(x, F[12]); x = vadd(x, F[13]); x = vsub(x, F[14]);
  V y = vsub(F[3], F[4]);
  y = vadd(y, F[7]); y = vsub(y, F[8]); y = vsub(y, F[9]); y = vadd(y, F[10]);
  y = vadd(y, F[15]); y = vsub(y, F[16]); y = vadd(y, F[17]); y = vsub(y, F[18]);
  V z = vsub(F[5], F[6]);
  z = vadd(z, F[11]); z = vsub(z, F[12]); z = vsub(z, F[13]); z = vadd(z, F[14]);
  z = vadd(z, F[15]); z = vsub(z, F[16]); z = vsub(z, F[17]); z = vadd(z, F[18]);
  x = vdiv(x, r); y = vdiv(y, r); z = vdiv(z, r);
  x = vadd(x, vdiv(vmul(gx, 0.5f), r));
  y = vadd(y, vdiv(vmul(gy, 0.5f), r));
  z = vadd(z, vdiv(vmul(gz, 0.5f), r));
  rho = r; ux = x; uy = y; uz = z;
}

// The same quantities from the moments m = M F of mrt_forward: its rows 0, 3, 5 and 7 are
// update_macro's sums of f, e_x f, e_y f and e_z f, term for term in q order (the formula
// generator's self-check asserts it), so rho and j are the same values.
template <class V>
__device__ __forceinline__ void macro_of_moments(const V (&m)[19], V gx, V gy, V gz, V& rho,
                                                 V& ux, V& uy, V& uz) {
  const V r = m[0];
  V x = vdiv(m[3], r), y = vdiv(m[5], r), z = vdiv(m[7], r);
  x = vadd(x, vdiv(vmul(gx, 0.5f), r));
  y = vadd(y, vdiv(vmul(gy, 0.5f), r));
  z = vadd(z, vdiv(vmul(gz, 0.5f), r));
  rho = r; ux = x; uy = y; uz = z;
}

// The same quantities with fused operations and one reciprocal (fast forms).
template <class V>
__device__ __forceinline__ void macro_fast(const V (&F)[19], V gx, V gy, V gz, V& rho, V& ux,
                                           V& uy, V& uz) {
  const V P0 = vadd(F[1], F[2]), P1 = vadd(F[3], F[4]), P2 = vadd(F[5], F[6]);
  const V P3 = vadd(F[7], F[8]), P4 = vadd(F[9], F[10]), P5 = vadd(F[11], F[12]);
  const V P6 = vadd(F[13], F[14]), P7 = vadd(F[15], F[16]), P8 = vadd(F[17], F[18]);
  const V r = vadd(vadd(vadd(vadd(F[0], P0), vadd(P1, P2)), vadd(vadd(P3, P4), vadd(P5, P6))),
                   vadd(P7, P8));
  const V D3 = vsub(F[7], F[8]), D4 = vsub(F[9], F[10]), D5 = vsub(F[11], F[12]);
  const V D6 = vsub(F[13], F[14]), D7 = vsub(F[15], F[16]), D8 = vsub(F[17], F[18]);
  const V jx = vadd(vadd(vsub(F[1], F[2]), vadd(D3, D4)), vadd(D5, D6));
  const V jy = vadd(vadd(vsub(F[3], F[4]), vsub(D3, D4)), vadd(D7, D8));
  const V jz = vadd(vadd(vsub(F[5], F[6]), vsub(D5, D6)), vsub(D7, D8));
  const V inv = vrcp(r);
  rho = r;
  ux = vmul(vfma(0.5f, gx, jx), inv);
  uy = vmul(vfma(0.5f, gy, jy), inv);
  uz = vmul(vfma(0.5f, gz, jz), inv);
}

template <bool kFast, class V>
__device__ __forceinline__ void macro_any(const V (&F)[19], V gx, V gy, V gz, V& rho, V& ux,
                                          V& uy, V& uz) {
  if (kFast) macro_fast(F, gx, gy, gz, rho, ux, uy, uz);
  else macro_of(F, gx, gy, gz, rho, ux, uy, uz);
}

// Sum of the non-zero terms e_c * v_c in x, y, z order (Taichi Vector.dot with
// exact zero products dropped).
template <class V>
__device__ __forceinline__ V edot(int q, V vx, V vy, V vz) {
  V s = splat<V>(0.0f);
  bool first = true;
  if (ex(q) != 0) { s = ex(q) > 0 ? vx : vneg(vx); first = false; }
  if (ey(q) != 0) { V t = ey(q) > 0 ? vy : vneg(vy); s = first ? t : vadd(s, t); first = false; }
  if (ez(q) != 0) { V t = ez(q) > 0 ? vz : vneg(vz); s = first ? t : vadd(s, t); }
  return s;
}

// MRT collision with Guo forcing of one fluid cell (or two, V = float2) in the reference's
// order (lbm3d.py:276-333), given the moments mF = M F of its populations (mrt_forward, which
// the caller also reads rho and j from). SG[k] is the forcing weight 1 - 0.5 S[k] of the reference,
// evaluated once per launch: 0.5 S[k] is an exact scaling, so 1 - 0.5 S[k] has a single
// rounding wherever it is computed.
template <class V>
__device__ __forceinline__ void collide_cell(const V (&mF)[19], V ux, V uy, V uz, V gx, V gy, V gz,
                                             const float* __restrict__ S,
                                             const float* __restrict__ SG, V (&out)[19]) {
  // Guo source terms t_q = w_q ((e_q - u).G + (e_q.u)(e_q.G)) (lbm3d.py:276-283).
  // (e - u_c) G_c takes three values per axis, for e = -1, 0, +1.
  const V dx[3] = {vmul(vsub(-1.0f, ux), gx), vmul(vneg(ux), gx), vmul(vsub(1.0f, ux), gx)};
  const V dy[3] = {vmul(vsub(-1.0f, uy), gy), vmul(vneg(uy), gy), vmul(vsub(1.0f, uy), gy)};
  const V dz[3] = {vmul(vsub(-1.0f, uz), gz), vmul(vneg(uz), gz), vmul(vsub(1.0f, uz), gz)};
  // (e.u)(e.G) of q and of opp(q) are the same rounded product: both dot products change
  // sign together and (-x)(-y) = xy. They can differ only in the sign of an exact zero,
  // which the forcing moments g = M t then carry only into sums that are non-zero or +0.
  V t[19], b[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const V a = vadd(vadd(dx[ex(q) + 1], dy[ey(q) + 1]), dz[ez(q) + 1]);
    if (q == 0) {
      t[q] = vmul(weight_of(q), a);
    } else {
      b[q] = (q & 1) ? vmul(edot(q, ux, uy, uz), edot(q, gx, gy, gz)) : b[q - 1];
      t[q] = vmul(weight_of(q), vadd(a, b[q]));
    }
  }
  V g[19], m[19];
  mrt_forward(t, g);
#pragma unroll
  for (int k = 0; k < 19; ++k) m[k] = mF[k];
  // Relaxation towards meq (lbm3d.py:285-326). S_0 = S_3 = S_5 = S_7 = 0: those
  // moments only receive the forcing term.
  const V uxx = vmul(ux, ux), uyy = vmul(uy, uy), uzz = vmul(uz, uz);
  V meq[19];
#pragma unroll
  for (int k = 0; k < 19; ++k) meq[k] = splat<V>(0.0f);
  meq[1] = vadd(vadd(uxx, uyy), uzz);
  meq[9] = vsub(vsub(vmul(vmul(2.0f, ux), ux), uyy), uzz);
  meq[11] = vsub(uyy, uzz);
  meq[13] = vmul(ux, uy);
  meq[14] = vmul(uy, uz);
  meq[15] = vmul(ux, uz);
#pragma unroll
  for (int k = 0; k < 19; ++k) {
    if (k == 0 || k == 3 || k == 5 || k == 7) {
      m[k] = vadd(m[k], g[k]);
    } else {
      const bool has_eq = (k == 1 || k == 9 || k == 11 || k == 13 || k == 14 || k == 15);
      const V d = has_eq ? vsub(m[k], meq[k]) : m[k];
      m[k] = vsub(m[k], vmul(S[k], d));
      m[k] = vadd(m[k], vmul(SG[k], g[k]));  // SG[k] = 1 - S[k]/2, rounded once
    }
  }
  mrt_inverse(m, out);
}

struct StepArgs {
  LbmGeom g;
  void* __restrict__ pops;
  float4* __restrict__ macro;
  const float* __restrict__ force;
  const float* __restrict__ force_prev;
  const uint32_t* __restrict__ flags;
  float s[19];
  float sg[19];     // 1 - s_k / 2, the weight of the forcing moment g_k (host-rounded once)
  float shift[19];  // w_q rho0, the storage offset of the deviation forms
  int write_faces;
};

// Cells per thread of the step kernel: the exact form evaluates one cell per thread in
// scalar float arithmetic; the fast forms evaluate the two cells (i, j, k) and (i, j + 1, k)
// of a thread together in packed float2 arithmetic (half the floating-point instructions).
// The exact form stays scalar because the assembler's optimisation of packed f32x2 code
// was observed to change rounding (a single-use product merged into the following
// subtraction), which would break bit-identity with the reference's float32 operations.
template <bool kFast>
struct StepLanes {
  static constexpr int n = kFast ? 2 : 1;
  using V = typename std::conditional<kFast, float2, float>::type;
};

// Minimum resident 128-thread blocks per SM of the step kernel (caps its registers at
// 65536 / (128 * n)): scalar exact form by parity, then the packed forms.
#ifndef FSI_LBM_MIN_BLOCKS_EXACT_EVEN
#define FSI_LBM_MIN_BLOCKS_EXACT_EVEN 6
#endif
#ifndef FSI_LBM_MIN_BLOCKS_EXACT_ODD
#define FSI_LBM_MIN_BLOCKS_EXACT_ODD 8
#endif
#ifndef FSI_LBM_MIN_BLOCKS_FAST
#define FSI_LBM_MIN_BLOCKS_FAST 6
#endif
constexpr int kStepBlock = 128;

template <bool kFast, bool kOdd>
constexpr int step_min_blocks() {
  return kFast ? FSI_LBM_MIN_BLOCKS_FAST
               : (kOdd ? FSI_LBM_MIN_BLOCKS_EXACT_ODD : FSI_LBM_MIN_BLOCKS_EXACT_EVEN);
}

// Launch shape of the step kernel: x = z (contiguous), y = groups of `lanes` rows, z = x planes.
CellLaunch step_launch(const LbmGeom& g, int lanes) {
  int bz = ((g.nz + 31) / 32) * 32;
  if (bz > kStepBlock) bz = kStepBlock;
  const int rows = (g.ny + lanes - 1) / lanes;
  int by = kStepBlock / bz;
  if (by > rows) by = rows;
  return CellLaunch{dim3((g.nz + bz - 1) / bz, (rows + by - 1) / by, g.nx), dim3(bz, by, 1)};
}

// Storage index that the odd step reads F_q(x) from, and that it writes f*_q(x) to.
__device__ __forceinline__ uint32_t odd_src(const Deltas& d, uint32_t fl, int q, uint32_t n) {
  return ((fl >> opp(q)) & 1u) ? q * n + d.c : opp(q) * n + d.nb(q, -1);
}
__device__ __forceinline__ uint32_t odd_dst(const Deltas& d, uint32_t fl, int q, uint32_t n) {
  return ((fl >> q) & 1u) ? opp(q) * n + d.c : q * n + d.nb(q, +1);
}

// One step of the cells (ci[l], cj[l], ck[l]) of the lanes of one thread; a lane with
// has[l] false is treated like a solid cell (read from another lane, never stored).
// Args is StepArgs (one lattice, parameters in the kernel's parameter space) or any type
// with the same members (a lattice of a batch, whose rates and shifts are pointers).
template <int kStore, bool kFast, bool kOdd, bool kRecompute, class Args>
__device__ __forceinline__ void step_cells(const Args& a,
                                           const int (&ci)[StepLanes<kFast>::n],
                                           const int (&cj)[StepLanes<kFast>::n],
                                           const int (&ck)[StepLanes<kFast>::n],
                                           const bool (&has)[StepLanes<kFast>::n]) {
  using St = Store<kStore>;
  constexpr int L = StepLanes<kFast>::n;
  using V = typename StepLanes<kFast>::V;
  using Ln = Lanes<V>;
  Deltas d[L];
  uint32_t fl[L];
  bool live[L];
  bool any = false;
#pragma unroll
  for (int l = 0; l < L; ++l) {
    const int o = has[l] ? l : 0;
    d[l] = Deltas(a.g, ci[o], cj[o], ck[o]);
    fl[l] = has[l] ? a.flags[d[l].c] : kFlagSolid;
    live[l] = !(fl[l] & kFlagSolid);
    any = any || live[l];
  }
  if (!any) return;
  // A solid (or missing) lane reads the cells of a live lane and is never stored.
  const int src = live[0] ? 0 : L - 1;
  const uint32_t n = (uint32_t)a.g.n;
  typename St::T* __restrict__ pops = reinterpret_cast<typename St::T*>(a.pops);

  V F[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    uint32_t sl[L];
#pragma unroll
    for (int l = 0; l < L; ++l) {
      const int ll = live[l] ? l : src;
      // F_q(x) = f*_q(x - e_q) in slot opp(q) there, or f*_opp(q)(x) in slot q here when
      // x - e_q is solid (half-way bounce-back).
      sl[l] = (!kOdd || q == 0) ? q * n + d[ll].c : odd_src(d[ll], fl[ll], q, n);
    }
    if constexpr (L == 2) {
      F[q] = St::ld2(pops, sl[0], sl[1], a.shift[q]);
    } else {
      F[q] = St::ld(pops, sl[0], a.shift[q]);
    }
  }
  // Exact form: the moments M F, from which both rho, j and the collision start.
  V mF[19];
  if (!kFast) mrt_forward(F, mF);

  uint32_t c[L];
#pragma unroll
  for (int l = 0; l < L; ++l) c[l] = d[live[l] ? l : src].c;
  V gx, gy, gz, rho, ux, uy, uz;
#pragma unroll
  for (int l = 0; l < L; ++l) {
    Ln::set(gx, l, a.force[c[l]]);
    Ln::set(gy, l, a.force[n + c[l]]);
    Ln::set(gz, l, a.force[2 * n + c[l]]);
  }
  if (kRecompute) {
    V px, py, pz;
#pragma unroll
    for (int l = 0; l < L; ++l) {
      Ln::set(px, l, a.force_prev[c[l]]);
      Ln::set(py, l, a.force_prev[n + c[l]]);
      Ln::set(pz, l, a.force_prev[2 * n + c[l]]);
    }
    if (kFast) macro_fast(F, px, py, pz, rho, ux, uy, uz);
    else macro_of_moments(mF, px, py, pz, rho, ux, uy, uz);
    if (a.write_faces) {
#pragma unroll
      for (int l = 0; l < L; ++l)
        if (live[l] && (fl[l] & (kFlagFaceLeft | kFlagFaceRight)))
          a.macro[d[l].c] = make_float4(Ln::get(ux, l), Ln::get(uy, l), Ln::get(uz, l),
                                        Ln::get(rho, l));
    }
  } else {
#pragma unroll
    for (int l = 0; l < L; ++l) {
      const float4 m = a.macro[c[l]];
      Ln::set(ux, l, m.x); Ln::set(uy, l, m.y); Ln::set(uz, l, m.z); Ln::set(rho, l, m.w);
    }
  }

  V out[19];
  if (kFast) mrt_collide_fast(F, rho, ux, uy, uz, gx, gy, gz, a.s, out);
  else collide_cell(mF, ux, uy, uz, gx, gy, gz, a.s, a.sg, out);

#pragma unroll
  for (int q = 0; q < 19; ++q) {
    // f*_q goes to slot opp(q) of this cell (even step, or odd-step bounce-back) or to slot q
    // of x + e_q (odd step). w_q = w_opp(q), so either slot's storage shift is shift[q].
    uint32_t t[L];
#pragma unroll
    for (int l = 0; l < L; ++l)
      t[l] = (!kOdd || q == 0) ? opp(q) * n + d[l].c : odd_dst(d[l], fl[l], q, n);
    if constexpr (L == 2) {
      if (live[0] && live[1]) {
        St::st2(pops, t[0], t[1], out[q], a.shift[q]);
        continue;
      }
    }
#pragma unroll
    for (int l = 0; l < L; ++l)
      if (live[l]) St::st(pops, t[l], Ln::get(out[q], l), a.shift[q]);
  }
}

template <int kStore, bool kFast, bool kOdd, bool kRecompute>
__global__ void __launch_bounds__(kStepBlock, (step_min_blocks<kFast, kOdd>()))
    lbm_step_kernel(StepArgs a) {
  constexpr int L = StepLanes<kFast>::n;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = L * (blockIdx.y * blockDim.y + threadIdx.y);
  const int i = blockIdx.z;
  if (k >= a.g.nz || j >= a.g.ny) return;
  int ci[L], cj[L], ck[L];
  bool has[L];
#pragma unroll
  for (int l = 0; l < L; ++l) {
    ci[l] = i; cj[l] = j + l; ck[l] = k;
    has[l] = j + l < a.g.ny;
  }
  step_cells<kStore, kFast, kOdd, kRecompute, StepArgs>(a, ci, cj, ck, has);
}

// numpy float32 norm of a 3-vector: sqrt((x*x + y*y) + z*z).
__device__ __forceinline__ float norm3_ref(float x, float y, float z) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// Adds this block's sums of `s` (float32 within a warp, float64 across warps) into
// sums[0..NS) and, when max_out is not NULL, raises *max_out to the block maximum of `mx`.
// Every thread of the block must call it; each instantiation owns its shared scratch.
template <int NS>
__device__ void block_accumulate(double* __restrict__ sums, const float (&s)[NS],
                                 double* __restrict__ max_out, float mx) {
  float v[NS];
#pragma unroll
  for (int i = 0; i < NS; ++i) v[i] = s[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int i = 0; i < NS; ++i) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  __shared__ double sh[NS][kBlock / 32];
  __shared__ float shm[kBlock / 32];
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  const int nwarps = (blockDim.x * blockDim.y + 31) / 32;
  if ((t & 31) == 0) {
#pragma unroll
    for (int i = 0; i < NS; ++i) sh[i][t >> 5] = (double)v[i];
    shm[t >> 5] = mx;
  }
  __syncthreads();
  if (t == 0) {
    float m = 0.f;
    for (int w = 0; w < nwarps; ++w) m = fmaxf(m, shm[w]);
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      double acc = 0.0;
      for (int w = 0; w < nwarps; ++w) acc += sh[i][w];
      atomicAdd(sums + i, acc);
    }
    if (max_out) atomic_max_nonneg(max_out, (double)m);
  }
}

}  // namespace
}  // namespace fsi
