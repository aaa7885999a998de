// MLS-MPM building blocks shared by the single-solver kernels (mpm.cu) and the batched
// kernels (batch.cu): solver parameters, particle views, B-spline weights, the polar
// rotation, and the per-CTA bodies of P2G (optionally with the penalty coupling folded in),
// grid update + G2P and the block clear.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "coupling_core.cuh"
#include "fsi_common.cuh"

namespace fsi {
namespace {

constexpr int kTileCap = 2048;  // nodes per shared tile

struct Mpm {
  int nx, ny, nz;
  int n;  // particles
  float dt, dx, inv_dx, mu, lam, g[3], damping;
  int bw, apic;
  float lower, upper[3];
  long long cap;
  int nbx, nby, nbz;  // 4^3 block grid
  int material;       // FSI_MATERIAL_*
  int threads;        // threads per block of the tiled P2G / G2P (128, 256 or 512)
  int fold;           // coupled tiled substep: 0 by particle count, 1 in P2G, 2 separate,
                      // 3 separate force and spread kernels
};

struct PView {
  float* __restrict__ x;
  float* __restrict__ v;
  float* __restrict__ C;
  float* __restrict__ F;
  const float* __restrict__ mass;
  const float* __restrict__ vol;
  const int32_t* __restrict__ active;
  float* __restrict__ fp;
  const float* __restrict__ mu;   // per-particle Lame parameters, or NULL
  const float* __restrict__ lam;
};

__device__ __forceinline__ void base_fx(const Mpm& m, const float x[3], int base[3], float fx[3]) {
  // base = trunc(x * inv_dx - 0.5) (cast toward zero), fx = x * inv_dx - base (mpm3d.py:239-240).
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float gpos = __fmul_rn(x[a], m.inv_dx);
    base[a] = (int)__fsub_rn(gpos, 0.5f);
    fx[a] = __fsub_rn(gpos, (float)base[a]);
  }
}


__device__ __forceinline__ float dot3r(float a0, float a1, float a2, float b0, float b1, float b2) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

// out = A B for row-major 3x3, sequential sum over k.
__device__ __forceinline__ void matmul3(const float* A, const float* B, float* out) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      out[3 * a + b] = dot3r(A[3 * a], A[3 * a + 1], A[3 * a + 2], B[b], B[3 + b], B[6 + b]);
}

__device__ __forceinline__ float det3(const float* a) {
  const float t0 = __fsub_rn(__fmul_rn(a[4], a[8]), __fmul_rn(a[7], a[5]));
  const float t1 = __fsub_rn(__fmul_rn(a[1], a[8]), __fmul_rn(a[7], a[2]));
  const float t2 = __fsub_rn(__fmul_rn(a[1], a[5]), __fmul_rn(a[4], a[2]));
  float d = __fsub_rn(__fmul_rn(a[0], t0), __fmul_rn(a[3], t1));
  return __fadd_rn(d, __fmul_rn(a[6], t2));
}

// Rotation of the polar decomposition by one-sided Jacobi SVD (Hestenes 1958):
// orthogonalise the columns of A = F V by plane rotations; R = U V^T with
// U = A column-normalised, the smallest column flipped if U V^T is improper.
__device__ void polar_jacobi(const float* F, float* R) {
  float A[9], V[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
#pragma unroll
  for (int i = 0; i < 9; ++i) A[i] = F[i];
  for (int sweep = 0; sweep < 8; ++sweep) {
    float off = 0.f;
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const float alpha = dot3r(A[p], A[3 + p], A[6 + p], A[p], A[3 + p], A[6 + p]);
      const float beta = dot3r(A[q], A[3 + q], A[6 + q], A[q], A[3 + q], A[6 + q]);
      const float gamma = dot3r(A[p], A[3 + p], A[6 + p], A[q], A[3 + q], A[6 + q]);
      if (gamma == 0.f) continue;
      off = fmaxf(off, fabsf(gamma) / sqrtf(alpha * beta));
      const float zeta = (beta - alpha) / (2.f * gamma);
      const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
      const float c = 1.f / sqrtf(1.f + t * t), s = c * t;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float ap = A[3 * r + p], aq = A[3 * r + q];
        A[3 * r + p] = c * ap - s * aq;
        A[3 * r + q] = s * ap + c * aq;
        const float vp = V[3 * r + p], vq = V[3 * r + q];
        V[3 * r + p] = c * vp - s * vq;
        V[3 * r + q] = s * vp + c * vq;
      }
    }
    if (off < 1e-7f) break;
  }
  float nrm[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) nrm[c] = sqrtf(A[c] * A[c] + A[3 + c] * A[3 + c] + A[6 + c] * A[6 + c]);
  float U[9];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) U[3 * r + c] = nrm[c] > 0.f ? A[3 * r + c] / nrm[c] : (r == c ? 1.f : 0.f);
  if (det3(U) * det3(V) < 0.f) {
    int cmin = 0;
    if (nrm[1] < nrm[cmin]) cmin = 1;
    if (nrm[2] < nrm[cmin]) cmin = 2;
#pragma unroll
    for (int r = 0; r < 3; ++r) U[3 * r + cmin] = -U[3 * r + cmin];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      R[3 * a + b] = U[3 * a] * V[3 * b] + U[3 * a + 1] * V[3 * b + 1] + U[3 * a + 2] * V[3 * b + 2];
}

// Rotation of F = R S by Newton's iteration X <- (z X + X^{-T}/z)/2 with
// Frobenius-norm scaling z = (|X^{-1}|_F / |X|_F)^{1/2} (Higham, SIAM J. Sci.
// Stat. Comput. 7, 1986). Used for det F > 0, where R is the unique rotation
// the reference obtains as U V^T from ti.svd (mpm3d.py:245-246); inverted or
// degenerate F fall back to the Jacobi SVD.
__device__ void polar_rotation(const float* F, float* R) {
  float X[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) X[i] = F[i];
  if (!(det3(F) > 1e-20f)) {
    polar_jacobi(F, R);
    return;
  }
  bool scale = true;
  for (int it = 0; it < 16; ++it) {
    float Cf[9];
    Cf[0] = X[4] * X[8] - X[5] * X[7];
    Cf[1] = X[5] * X[6] - X[3] * X[8];
    Cf[2] = X[3] * X[7] - X[4] * X[6];
    Cf[3] = X[2] * X[7] - X[1] * X[8];
    Cf[4] = X[0] * X[8] - X[2] * X[6];
    Cf[5] = X[1] * X[6] - X[0] * X[7];
    Cf[6] = X[1] * X[5] - X[2] * X[4];
    Cf[7] = X[2] * X[3] - X[0] * X[5];
    Cf[8] = X[0] * X[4] - X[1] * X[3];
    const float det = X[0] * Cf[0] + X[1] * Cf[1] + X[2] * Cf[2];
    float z = 1.f;
    if (scale) {
      float nx2 = 0.f, nc2 = 0.f;
#pragma unroll
      for (int i = 0; i < 9; ++i) { nx2 += X[i] * X[i]; nc2 += Cf[i] * Cf[i]; }
      z = sqrtf(sqrtf(nc2 / nx2) / fabsf(det));
    }
    const float a = 0.5f * z, b = 0.5f / (z * det);
    float d2 = 0.f, n2 = 0.f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const float xn = a * X[i] + b * Cf[i];
      const float dd = xn - X[i];
      d2 += dd * dd;
      n2 += xn * xn;
      X[i] = xn;
    }
    if (d2 < 1e-4f * n2) scale = false;
    if (d2 <= 1e-13f * n2) break;
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = X[i];
}

__device__ __forceinline__ bool inside(const Mpm& m, int i, int j, int k) {
  return 0 <= i && i < m.nx && 0 <= j && j < m.ny && 0 <= k && k < m.nz;
}

__device__ __forceinline__ long long node_index(const Mpm& m, int i, int j, int k) {
  return ((long long)i * m.ny + j) * m.nz + k;
}

__device__ __forceinline__ void mark_block(const Mpm& m, uint8_t* dirty, int i, int j, int k) {
  dirty[((long long)(i >> 2) * m.nby + (j >> 2)) * m.nbz + (k >> 2)] = 1;
}

// Block-wide bounding box of the stencils of this CTA's active particles.
struct Box {
  int lo[3], ext[3];
  int vol;
};

__device__ bool cta_box(const Mpm& m, bool act, const int base[3], Box& box, int* sh) {
  // sh: 6 ints of shared scratch
  if (threadIdx.x < 3) { sh[threadIdx.x] = 0x7fffffff; sh[3 + threadIdx.x] = -0x7fffffff; }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int lo = act ? base[a] : 0x7fffffff;
    int hi = act ? base[a] + 2 : -0x7fffffff;
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if ((threadIdx.x & 31) == 0) { atomicMin(&sh[a], lo); atomicMax(&sh[3 + a], hi); }
  }
  __syncthreads();
  if (sh[0] == 0x7fffffff) return false;  // no active particle
  const int n[3] = {m.nx, m.ny, m.nz};
  long long vol = 1;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int lo = max(sh[a], 0), hi = min(sh[3 + a], n[a] - 1);
    box.lo[a] = lo;
    box.ext[a] = hi >= lo ? hi - lo + 1 : 0;
    vol *= box.ext[a];
  }
  box.vol = vol > (long long)kTileCap ? kTileCap + 1 : (int)vol;
  return true;
}

__device__ __forceinline__ void load_particle_x(const PView& P, long long cap, int p, float x[3]) {
  x[0] = P.x[p]; x[1] = P.x[cap + p]; x[2] = P.x[2 * cap + p];
}

// The once-per-particle part of P2G for active particle p (mpm3d.py:242-252):
// F <- (I + dt C) F (written back), the stress, and affine = stress term + m C.
__device__ __forceinline__ void p2g_stress_affine(const Mpm& m, const PView& P, int p,
                                                  float affine[9], float& mass) {
  const long long cap = m.cap;
  float Cp[9], Fp[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) { Cp[i] = P.C[i * cap + p]; Fp[i] = P.F[i * cap + p]; }
  // F <- (I + dt C) F (mpm3d.py:243)
  float A[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) A[i] = __fadd_rn((i % 4 == 0) ? 1.f : 0.f, __fmul_rn(m.dt, Cp[i]));
  float Fn[9];
  matmul3(A, Fp, Fn);
#pragma unroll
  for (int i = 0; i < 9; ++i) P.F[i * cap + p] = Fn[i];
  const float J = det3(Fn);
  const float mu = P.mu ? P.mu[p] : m.mu;
  const float lam = P.lam ? P.lam[p] : m.lam;
  float Ft[9], S[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) Ft[3 * a + b] = Fn[3 * b + a];
  if (m.material == FSI_MATERIAL_NEO_HOOKEAN) {
    // Kirchhoff stress of compressible Neo-Hookean: mu (F F^T - I) + lam ln(J) I.
    matmul3(Fn, Ft, S);
#pragma unroll
    for (int i = 0; i < 9; ++i) S[i] = __fmul_rn(mu, __fsub_rn(S[i], (i % 4 == 0) ? 1.f : 0.f));
    const float ll = __fmul_rn(lam, logf(J));
    S[0] = __fadd_rn(S[0], ll); S[4] = __fadd_rn(S[4], ll); S[8] = __fadd_rn(S[8], ll);
  } else {
    // Fixed-corotated: 2 mu (F - R) F^T + lam J (J - 1) I (mpm3d.py:247-251)
    float R[9];
    polar_rotation(Fn, R);
    const float twomu = __fmul_rn(2.f, mu);
    float Pm[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Pm[i] = __fmul_rn(twomu, __fsub_rn(Fn[i], R[i]));
    matmul3(Pm, Ft, S);
    const float lj = __fmul_rn(__fmul_rn(lam, J), __fsub_rn(J, 1.f));
    S[0] = __fadd_rn(S[0], lj); S[4] = __fadd_rn(S[4], lj); S[8] = __fadd_rn(S[8], lj);
  }
  float coef = __fmul_rn(__fmul_rn(__fmul_rn(-m.dt, P.vol[p]), 4.f), m.inv_dx);
  coef = __fmul_rn(coef, m.inv_dx);
  mass = P.mass[p];
#pragma unroll
  for (int i = 0; i < 9; ++i) affine[i] = __fadd_rn(__fmul_rn(coef, S[i]), __fmul_rn(mass, Cp[i]));
}

// P2G of particle p (this thread) within its CTA; every thread of the CTA calls it.
// kCoupled folds _compute_coupling_forces_kernel (fsi/coupling.py:332-406) in front of the
// scatter: the particle's coupling force is formed first (it is P2G's dt f term) and the
// fluid reaction and solid fraction are spread into fa.accum beside the grid scatter.
// kExtTile: the tile is the caller's shared memory `ext` (4 x kTileCap floats) instead of a
// static array of its own (a kernel that also runs g2p_body then holds one tile, not two).
template <bool kCoupled = false, bool kExtTile = false>
__device__ __forceinline__ void p2g_body(const Mpm& m, const PView& P, float4* __restrict__ grid,
                                         uint8_t* __restrict__ dirty, int p,
                                         const ForceArgs* fa = nullptr,
                                         float (*ext)[kTileCap] = nullptr) {
  __shared__ float own[kExtTile ? 1 : 4][kExtTile ? 1 : kTileCap];
  float (*tile)[kTileCap] = kExtTile ? ext : reinterpret_cast<float (*)[kTileCap]>(own);
  __shared__ int sh[8];
  const long long cap = m.cap;
  const bool act = p < m.n && P.active[p] != 0;

  int base[3] = {0, 0, 0};
  float fx[3] = {0.f, 0.f, 0.f};
  float affine[9], mv[3], dtf[3], mass = 0.f;
  // coupling: in-grid fluid stencil nodes (bit 9i + 3j + k), valid weight, force, volume
  uint32_t usable = 0;
  float valid = 0.f, pf[3] = {0.f, 0.f, 0.f}, vp = 0.f;
  if (kCoupled) {
    bool partial = false, clipped = false, unsupported = false;
    if (act) {
      int cb[3];
      float cw[3][3];
      if (!coupling_particle<false>(*fa, p, cb, cw, usable, valid, pf, partial, clipped,
                                    unsupported)) {
        usable = 0;
        pf[0] = pf[1] = pf[2] = 0.f;
      }
      vp = P.vol[p];
    } else if (p < m.n) {
      P.fp[p] = 0.f; P.fp[cap + p] = 0.f; P.fp[2 * cap + p] = 0.f;
    }
    warp_count(&fa->cnt->unsupported, unsupported);
    warp_count(&fa->cnt->partial, partial);
    warp_count(&fa->cnt->clipped, clipped);
  }
  if (act) {
    float x[3];
    load_particle_x(P, cap, p, x);
    base_fx(m, x, base, fx);
    p2g_stress_affine(m, P, p, affine, mass);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      mv[a] = __fmul_rn(mass, P.v[a * cap + p]);
      dtf[a] = __fmul_rn(m.dt, kCoupled ? pf[a] : P.fp[a * cap + p]);
    }
  }

  Box box;
  if (!cta_box(m, act, base, box, sh)) return;
  const bool use_tile = box.vol <= kTileCap;
  if (use_tile) {
    for (int t = threadIdx.x; t < box.vol; t += blockDim.x) {
      tile[0][t] = 0.f; tile[1][t] = 0.f; tile[2][t] = 0.f; tile[3][t] = 0.f;
    }
    __syncthreads();
  }

  if (act) {
    // Per-axis stencil terms, once per particle: weights, offsets (i - fx) dx, in-grid tests
    // and the node's place in the tile (or grid). Odd lanes walk the stencil backwards (their
    // axis terms are stored reversed), so the two particles of a sub-cell pair, which share a
    // base cell, add into different nodes at each step.
    const bool rev = (threadIdx.x & 1) != 0;
    float wa[3][3], da[3][3];
    bool ina[3][3];
    int oa[3][3];  // axis offset of stencil step s: the node index is base + oa
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int s3 = 0; s3 < 3; ++s3) {
        const int o = rev ? 2 - s3 : s3;
        oa[a][s3] = o;
        wa[a][s3] = bspline_w(fx[a], o);
        da[a][s3] = __fmul_rn(__fsub_rn((float)o, fx[a]), m.dx);
        const int n = base[a] + o;
        ina[a][s3] = n >= 0 && n < (a == 0 ? m.nx : (a == 1 ? m.ny : m.nz));
      }
    const int st1 = use_tile ? box.ext[2] : m.nz;
    const long long st0 = use_tile ? (long long)box.ext[1] * box.ext[2] : (long long)m.ny * m.nz;
    const long long t0 = use_tile
        ? ((long long)(base[0] - box.lo[0]) * box.ext[1] + (base[1] - box.lo[1])) * box.ext[2] + (base[2] - box.lo[2])
        : ((long long)base[0] * m.ny + base[1]) * m.nz + base[2];
    const long long g0 = ((long long)base[0] * m.ny + base[1]) * m.nz + base[2];  // lattice node
    const long long gs0 = (long long)m.ny * m.nz;
#pragma unroll
    for (int si = 0; si < 3; ++si) {
      if (!ina[0][si]) continue;
#pragma unroll
      for (int sj = 0; sj < 3; ++sj) {
        if (!ina[1][sj]) continue;
        const float wxy = __fmul_rn(wa[0][si], wa[1][sj]);
        // dot3r's ((A0 d0 + A1 d1) + A2 d2): the first two terms are shared by the 3 k.
        float pa[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
          pa[a] = __fadd_rn(__fmul_rn(affine[3 * a], da[0][si]), __fmul_rn(affine[3 * a + 1], da[1][sj]));
#pragma unroll
        for (int sk = 0; sk < 3; ++sk) {
          if (!ina[2][sk]) continue;
          const float w = __fmul_rn(wxy, wa[2][sk]);
          float add[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float ad = __fadd_rn(pa[a], __fmul_rn(affine[3 * a + 2], da[2][sk]));
            add[a] = __fmul_rn(w, __fadd_rn(__fadd_rn(mv[a], ad), dtf[a]));
          }
          const float addm = __fmul_rn(w, mass);
          const long long t = t0 + oa[0][si] * st0 + oa[1][sj] * st1 + oa[2][sk];
          if (kCoupled && ((usable >> (9 * oa[0][si] + 3 * oa[1][sj] + oa[2][sk])) & 1u)) {
            float4 c = coupling_spread_terms(fa->c, w, valid, pf, vp);
            if (!fa->c.build_fraction) c.w = 0.f;
            red_add_v4(fa->accum + g0 + oa[0][si] * gs0 + oa[1][sj] * m.nz + oa[2][sk],
                       c.x, c.y, c.z, c.w);
          }
          if (use_tile) {
            atomicAdd(&tile[0][t], add[0]);
            atomicAdd(&tile[1][t], add[1]);
            atomicAdd(&tile[2][t], add[2]);
            atomicAdd(&tile[3][t], addm);
          } else {
            red_add_v4(grid + t, add[0], add[1], add[2], addm);
            mark_block(m, dirty, base[0] + oa[0][si], base[1] + oa[1][sj], base[2] + oa[2][sk]);
          }
        }
      }
    }
  }

  if (use_tile) {
    __syncthreads();
    if (box.vol == 0) return;  // every stencil node lies outside the grid
    const int e12 = box.ext[1] * box.ext[2];
    for (int t = threadIdx.x; t < box.vol; t += blockDim.x) {
      const float a = tile[0][t], b = tile[1][t], c = tile[2][t], d = tile[3][t];
      if (a == 0.f && b == 0.f && c == 0.f && d == 0.f) continue;
      const int ti = t / e12, r = t - ti * e12, tj = r / box.ext[2], tk = r - tj * box.ext[2];
      red_add_v4(grid + node_index(m, box.lo[0] + ti, box.lo[1] + tj, box.lo[2] + tk), a, b, c, d);
    }
    // Mark the 4^3 blocks overlapped by the box.
    const int b0[3] = {box.lo[0] >> 2, box.lo[1] >> 2, box.lo[2] >> 2};
    const int b1[3] = {(box.lo[0] + box.ext[0] - 1) >> 2, (box.lo[1] + box.ext[1] - 1) >> 2,
                       (box.lo[2] + box.ext[2] - 1) >> 2};
    const int nbx = b1[0] - b0[0] + 1, nby = b1[1] - b0[1] + 1, nbz = b1[2] - b0[2] + 1;
    for (int t = threadIdx.x; t < nbx * nby * nbz; t += blockDim.x) {
      const int bi = b0[0] + t / (nby * nbz), bj = b0[1] + (t / nbz) % nby, bk = b0[2] + t % nbz;
      dirty[((long long)bi * m.nby + bj) * m.nbz + bk] = 1;
    }
  }
}

// Grid update of one node (mpm3d.py:268-288): v = p/m + dt g, then per-axis
// walls within boundary_width: outward velocity becomes -damping * v.
__device__ __forceinline__ void grid_op(const Mpm& m, float4 node, int i, int j, int k, float v[3]) {
  v[0] = node.x; v[1] = node.y; v[2] = node.z;
  if (!(node.w > 0.f)) return;
#pragma unroll
  for (int a = 0; a < 3; ++a) v[a] = __fdiv_rn(v[a], node.w);
#pragma unroll
  for (int a = 0; a < 3; ++a) v[a] = __fadd_rn(v[a], __fmul_rn(m.dt, m.g[a]));
  const int idx[3] = {i, j, k};
  const int n[3] = {m.nx, m.ny, m.nz};
  const float nd = -m.damping;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (idx[a] < m.bw && v[a] < 0.f) v[a] = __fmul_rn(nd, v[a]);
    if (idx[a] >= n[a] - m.bw && v[a] > 0.f) v[a] = __fmul_rn(nd, v[a]);
  }
}

// Grid update + G2P of particle p (this thread) within its CTA; every thread calls it.
// kExtTile as for p2g_body (3 x kTileCap floats of the caller's shared memory).
template <bool kExtTile = false>
__device__ __forceinline__ void g2p_body(const Mpm& m, const PView& P,
                                         const float4* FSI_LAUNCH_RO grid, int p,
                                         float (*ext)[kTileCap] = nullptr) {
  __shared__ float own[kExtTile ? 1 : 3][kExtTile ? 1 : kTileCap];
  float (*tile)[kTileCap] = kExtTile ? ext : reinterpret_cast<float (*)[kTileCap]>(own);
  __shared__ int sh[8];
  const long long cap = m.cap;
  const bool act = p < m.n && P.active[p] != 0;
  int base[3] = {0, 0, 0};
  float fx[3] = {0.f, 0.f, 0.f}, x[3] = {0.f, 0.f, 0.f};
  if (act) {
    load_particle_x(P, cap, p, x);
    base_fx(m, x, base, fx);
  }
  Box box;
  if (!cta_box(m, act, base, box, sh)) return;
  const bool use_tile = box.vol <= kTileCap;
  if (use_tile) {
    const int e12 = box.ext[1] * box.ext[2];
    for (int t = threadIdx.x; t < box.vol; t += blockDim.x) {
      const int ti = t / e12, r = t - ti * e12, tj = r / box.ext[2], tk = r - tj * box.ext[2];
      const int i = box.lo[0] + ti, j = box.lo[1] + tj, k = box.lo[2] + tk;
      float v[3];
      grid_op(m, grid[node_index(m, i, j, k)], i, j, k, v);
      tile[0][t] = v[0]; tile[1][t] = v[1]; tile[2][t] = v[2];
    }
    __syncthreads();
  }
  if (!act) return;
  float nv[3] = {0.f, 0.f, 0.f};
  float nc[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const float four_inv_dx = __fmul_rn(4.f, m.inv_dx);
  // Per-axis stencil terms, once per particle; the sums run in the reference's node order.
  float wa[3][3], dp[3][3];
  bool ina[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int o = 0; o < 3; ++o) {
      wa[a][o] = bspline_w(fx[a], o);
      dp[a][o] = __fsub_rn((float)o, fx[a]);
      const int n = base[a] + o;
      ina[a][o] = n >= 0 && n < (a == 0 ? m.nx : (a == 1 ? m.ny : m.nz));
    }
  const int st1 = use_tile ? box.ext[2] : m.nz;
  const long long st0 = use_tile ? (long long)box.ext[1] * box.ext[2] : (long long)m.ny * m.nz;
  const long long t0 = use_tile
      ? ((long long)(base[0] - box.lo[0]) * box.ext[1] + (base[1] - box.lo[1])) * box.ext[2] + (base[2] - box.lo[2])
      : ((long long)base[0] * m.ny + base[1]) * m.nz + base[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (!ina[0][i]) continue;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (!ina[1][j]) continue;
      const float wxy = __fmul_rn(wa[0][i], wa[1][j]);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (!ina[2][k]) continue;
        const float w = __fmul_rn(wxy, wa[2][k]);
        const long long t = t0 + i * st0 + j * st1 + k;
        float gv[3];
        if (use_tile) {
          gv[0] = tile[0][t]; gv[1] = tile[1][t]; gv[2] = tile[2][t];
        } else {
          grid_op(m, grid[t], base[0] + i, base[1] + j, base[2] + k, gv);
        }
        const float dpos[3] = {dp[0][i], dp[1][j], dp[2][k]};
#pragma unroll
        for (int a = 0; a < 3; ++a) nv[a] = __fadd_rn(nv[a], __fmul_rn(w, gv[a]));
        const float s = __fmul_rn(four_inv_dx, w);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b)
            nc[3 * a + b] = __fadd_rn(nc[3 * a + b], __fmul_rn(s, __fmul_rn(gv[a], dpos[b])));
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) P.v[a * cap + p] = nv[a];
#pragma unroll
  for (int i = 0; i < 9; ++i) P.C[i * cap + p] = m.apic ? nc[i] : 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float xa = __fadd_rn(x[a], __fmul_rn(m.dt, nv[a]));
    xa = fminf(fmaxf(xa, m.lower), m.upper[a]);
    P.x[a * cap + p] = xa;
  }
}

// Zero every dirty 4^3 node block and reset its flag (one warp per block).
// Clears node block b when dirty (one warp per block; the warp's lanes all call it).
__device__ __forceinline__ void clear_body(const Mpm& m, float4* __restrict__ grid,
                                           uint8_t* __restrict__ dirty, long long b) {
  const long long nblocks = (long long)m.nbx * m.nby * m.nbz;
  if (b >= nblocks || dirty[b] == 0) return;
  const int lane = threadIdx.x & 31;
  const int bi = (int)(b / ((long long)m.nby * m.nbz));
  const int bj = (int)((b / m.nbz) % m.nby);
  const int bk = (int)(b % m.nbz);
  for (int t = lane; t < 64; t += 32) {
    const int i = bi * 4 + (t >> 4), j = bj * 4 + ((t >> 2) & 3), k = bk * 4 + (t & 3);
    if (i < m.nx && j < m.ny && k < m.nz) grid[node_index(m, i, j, k)] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncwarp();
  if (lane == 0) dirty[b] = 0;
}


// Host-side validation of a solver descriptor and its particle arrays.
int make_mpm(const fsi_mpm_desc* d, const fsi_particles* p, Mpm& m, PView& v) {
  FSI_REQUIRE(d && p, "NULL descriptor");
  FSI_REQUIRE(d->nx > 4 && d->ny > 4 && d->nz > 4, "grid %dx%dx%d too small", d->nx, d->ny, d->nz);
  FSI_REQUIRE(d->num_particles >= 0 && d->num_particles <= p->capacity,
              "num_particles %d outside [0, capacity %lld]", d->num_particles,
              (long long)p->capacity);
  FSI_REQUIRE(p->x && p->v && p->C && p->F && p->mass && p->volume && p->active && p->force,
              "NULL particle array");
  m.nx = d->nx; m.ny = d->ny; m.nz = d->nz;
  m.n = d->num_particles;
  m.dt = d->dt; m.dx = d->dx; m.inv_dx = d->inv_dx; m.mu = d->mu; m.lam = d->lam;
  for (int a = 0; a < 3; ++a) { m.g[a] = d->gravity[a]; m.upper[a] = d->clamp_upper[a]; }
  m.damping = d->boundary_damping; m.bw = d->boundary_width; m.apic = d->apic;
  m.lower = d->clamp_lower;
  m.cap = p->capacity;
  m.nbx = (d->nx + 3) / 4; m.nby = (d->ny + 3) / 4; m.nbz = (d->nz + 3) / 4;
  FSI_REQUIRE(d->material == FSI_MATERIAL_FIXED_COROTATED || d->material == FSI_MATERIAL_NEO_HOOKEAN,
              "unknown material %d", d->material);
  FSI_REQUIRE((p->mu == nullptr) == (p->lam == nullptr), "per-particle mu and lam go together");
  m.material = d->material;
  FSI_REQUIRE(d->launch_threads == 0 || d->launch_threads == 128 || d->launch_threads == 256 ||
                  d->launch_threads == 512,
              "launch_threads %d is not 0, 128, 256 or 512", d->launch_threads);
  FSI_REQUIRE(d->coupling_fold >= 0 && d->coupling_fold <= 3, "coupling_fold %d outside 0..3",
              d->coupling_fold);
  m.threads = d->launch_threads ? d->launch_threads : kBlock;
  m.fold = d->coupling_fold;
  v.x = p->x; v.v = p->v; v.C = p->C; v.F = p->F; v.mass = p->mass; v.vol = p->volume;
  v.active = p->active; v.fp = p->force; v.mu = p->mu; v.lam = p->lam;
  return FSI_OK;
}

}  // namespace
}  // namespace fsi
