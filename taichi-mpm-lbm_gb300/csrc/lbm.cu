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
__device__ __forceinline__ float gather32(const typename Store<kStore>::T* __restrict__ pops,
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
// order (lbm3d.py:276-333).
template <class V>
__device__ __forceinline__ void collide_cell(const V (&F)[19], V ux, V uy, V uz, V gx, V gy, V gz,
                                             const float* __restrict__ S, V (&out)[19]) {
  // Guo source terms t_q = w_q ((e_q - u).G + (e_q.u)(e_q.G)) (lbm3d.py:276-283).
  // (e - u_c) G_c takes three values per axis, for e = -1, 0, +1.
  const V dx[3] = {vmul(vsub(-1.0f, ux), gx), vmul(vneg(ux), gx), vmul(vsub(1.0f, ux), gx)};
  const V dy[3] = {vmul(vsub(-1.0f, uy), gy), vmul(vneg(uy), gy), vmul(vsub(1.0f, uy), gy)};
  const V dz[3] = {vmul(vsub(-1.0f, uz), gz), vmul(vneg(uz), gz), vmul(vsub(1.0f, uz), gz)};
  V t[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const V a = vadd(vadd(dx[ex(q) + 1], dy[ey(q) + 1]), dz[ez(q) + 1]);
    if (q == 0) {
      t[q] = vmul(weight_of(q), a);
    } else {
      const V b = vmul(edot(q, ux, uy, uz), edot(q, gx, gy, gz));
      t[q] = vmul(weight_of(q), vadd(a, b));
    }
  }
  V g[19], m[19];
  mrt_forward(t, g);
  mrt_forward(F, m);
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
      m[k] = vadd(m[k], vmul(__fsub_rn(1.0f, __fmul_rn(0.5f, S[k])), g[k]));
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

template <int kStore, bool kFast, bool kOdd, bool kRecompute>
__global__ void __launch_bounds__(kStepBlock, (step_min_blocks<kFast, kOdd>()))
    lbm_step_kernel(StepArgs a) {
  using St = Store<kStore>;
  constexpr int L = StepLanes<kFast>::n;
  using V = typename StepLanes<kFast>::V;
  using Ln = Lanes<V>;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = L * (blockIdx.y * blockDim.y + threadIdx.y);
  const int i = blockIdx.z;
  if (k >= a.g.nz || j >= a.g.ny) return;
  Deltas d[L];
  uint32_t fl[L];
  bool live[L];
  bool any = false;
#pragma unroll
  for (int l = 0; l < L; ++l) {
    const bool has = j + l < a.g.ny;
    d[l] = Deltas(a.g, i, has ? j + l : j, k);
    fl[l] = has ? a.flags[d[l].c] : kFlagSolid;
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
    macro_any<kFast>(F, px, py, pz, rho, ux, uy, uz);
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
  else collide_cell(F, ux, uy, uz, gx, gy, gz, a.s, out);

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
__global__ void __launch_bounds__(kBlock) lbm_reduce_kernel(LbmGeom g,
                                                            const float4* __restrict__ macro,
                                                            const float* __restrict__ force,
                                                            const uint32_t* __restrict__ flags,
                                                            double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  float mass = 0.f, vmax = 0.f, f[3] = {0.f, 0.f, 0.f};
  if (k < g.nz && j < g.ny) {
    const uint32_t c = (uint32_t)((i * g.ny + j) * g.nz + k);
    const uint32_t n = (uint32_t)g.n;
    const float4 m = macro[c];
    vmax = norm3_ref(m.x, m.y, m.z);
    if (!(flags[c] & kFlagSolid)) {
      mass = m.w;
      if (force) { f[0] = force[c]; f[1] = force[n + c]; f[2] = force[2 * n + c]; }
    }
  }
  const float s1[1] = {mass};
  block_accumulate<1>(out, s1, out + 1, vmax);
  block_accumulate<3>(out + 2, f, nullptr, 0.f);
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
    FSI_REQUIRE(m >= 0 && m <= 2, "unknown x boundary mode %d", m);
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
  for (int k = 0; k < 19; ++k) a.s[k] = d->s[k];
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
  const CellLaunch L = cell_launch(g);
  lbm_reduce_kernel<<<L.grid, L.block, 0, s>>>(g, reinterpret_cast<const float4*>(macro), force,
                                               flags, out);
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
