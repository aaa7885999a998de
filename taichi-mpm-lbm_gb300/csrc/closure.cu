// Learned coarse-grid closure: a per-cell MLP (656 -> 64 -> 64 -> 64 -> 19, GELU) that
// corrects the populations of a lattice running on a 2x coarser grid, on the fifth-
// generation tensor cores (tcgen05, BF16 operands, FP32 accumulation in tensor memory).
// No reference counterpart.
//
// Features of a cell x: for each of the 27 cells y of its 3^3 neighbourhood (periodic wrap,
// offsets in (dx, dy, dz) order, dz fastest) the 19 post-stream populations as scaled
// deviations (f_q(y) - w_q rho0) * pop_scale, the occupancy of y (1 solid, 0 fluid) and the
// 3 force components of y * force_scale: 27 * 23 = 621 values. Column layout: neighbour o's
// 23 values in columns [24 o, 24 o + 23), column 24 o + 23 zero, columns 648..655 zero
// (K = 656), so every neighbour group is three aligned 16-byte pieces.
//
// Kernels:
//   closure_features_kernel: the feature rows of a list of cells, BF16 [M][656] (training).
//   gemm_kernel: C = A B^T for K-major BF16 A [M][K], B [N][K] (row-major in global memory),
//     128-row tiles, split-K over blockIdx.y, two-stage cp.async pipeline into shared memory
//     (canonical no-swizzle core-matrix layout), tcgen05.mma into tensor memory, and a fused
//     epilogue: store FP32 / add FP32 atomically / bias + GELU forward (BF16 activations,
//     their transpose and the FP32 pre-activation) / GELU backward (BF16 gradient and its
//     transpose).
//   closure_infer_kernel: the fused inference pass: features built by the threads straight
//     into shared memory, the four layers on the tensor cores with the weights resident in
//     shared memory, and the 19 outputs written as corrections per cell.
//   closure_apply_kernel: f_q(x) += correction, mass-conserving (sum_q w-weighted projection).
//   loss / Adam kernels for training.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "fsi_common.cuh"
#include "lbm_core.cuh"
#include "tc_gemm.cuh"

namespace fsi {
namespace {

constexpr int kGroup = 24;           // columns per neighbour (23 values + 1 zero)
constexpr int kK1 = 27 * kGroup + 8;  // 656
constexpr int kOut = 19;
constexpr int kOutPad = 32;

// GELU, tanh form of Hendrycks & Gimpel (2016): 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))).
constexpr float kGeluC0 = 0.7978845608028654f;
constexpr float kGeluC1 = 0.044715f;
__device__ __forceinline__ float gelu(float z) {
  const float t = tanhf(kGeluC0 * (z + kGeluC1 * z * z * z));
  return 0.5f * z * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float t = tanhf(kGeluC0 * (z + kGeluC1 * z * z * z));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * kGeluC0 * (1.0f + 3.0f * kGeluC1 * z * z);
}

struct FeatArgs {
  LbmGeom g;
  const float* __restrict__ pops;  // FP32 populations [19][N], AA layout of `parity`
  const uint32_t* __restrict__ flags;
  const float* __restrict__ force;  // [3][N]
  int parity;
  float rho0, pop_scale, force_scale;
};

// The 23 feature values of neighbour y of a cell (populations, occupancy, force).
__device__ __forceinline__ void neighbour_features(const FeatArgs& a, int i, int j, int k,
                                                   float (&v)[23]) {
  const Deltas d(a.g, i, j, k);
  const uint32_t fl = a.flags[d.c];
  const uint32_t n = (uint32_t)a.g.n;
  const bool solid = fl & kFlagSolid;
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const float f = gather32<FSI_STORAGE_F32>(a.pops, n, d, fl, q, solid ? 0 : a.parity, 0.f);
    v[q] = solid ? 0.f : (f - weight_of(q) * a.rho0) * a.pop_scale;
  }
  v[19] = solid ? 1.f : 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) v[20 + c] = a.force[c * n + d.c] * a.force_scale;
}

__device__ __forceinline__ void wrap_neighbour(const LbmGeom& g, int i, int j, int k, int o,
                                               int& ni, int& nj, int& nk) {
  const int dx = o / 9 - 1, dy = (o / 3) % 3 - 1, dz = o % 3 - 1;
  ni = i + dx; nj = j + dy; nk = k + dz;
  ni = ni < 0 ? ni + g.nx : (ni >= g.nx ? ni - g.nx : ni);
  nj = nj < 0 ? nj + g.ny : (nj >= g.ny ? nj - g.ny : nj);
  nk = nk < 0 ? nk + g.nz : (nk >= g.nz ? nk - g.nz : nk);
}

// Feature rows of cells[m] (BF16, [M][656]); one thread per (row, neighbour).
__global__ void __launch_bounds__(256) closure_features_kernel(FeatArgs a,
                                                                const int32_t* __restrict__ cells,
                                                                int m, __nv_bfloat16* __restrict__ x) {
  const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
  if (t >= (long long)m * 28) return;
  const int row = (int)(t / 28), o = (int)(t % 28);
  __nv_bfloat16* out = x + (size_t)row * kK1;
  if (o == 27) {  // padding columns
    for (int c = 27 * kGroup; c < kK1; ++c) out[c] = __float2bfloat16(0.f);
    return;
  }
  const int c = cells[row];
  const int nyz = a.g.ny * a.g.nz;
  const int i = c / nyz, j = (c / a.g.nz) % a.g.ny, k = c % a.g.nz;
  int ni, nj, nk;
  wrap_neighbour(a.g, i, j, k, o, ni, nj, nk);
  float v[23];
  neighbour_features(a, ni, nj, nk, v);
#pragma unroll
  for (int f = 0; f < 23; ++f) out[o * kGroup + f] = __float2bfloat16_rn(v[f]);
  out[o * kGroup + 23] = __float2bfloat16_rn(0.f);
}

// ------------------------------------------------------------------ GEMM
enum Epilogue { kStoreF32 = 0, kAtomicF32 = 1, kGeluFwd = 2, kGeluBwd = 3 };

struct GemmArgs {
  const __nv_bfloat16* __restrict__ A;  // [M][lda]
  const __nv_bfloat16* __restrict__ B;  // [N][ldb]
  int lda, ldb;
  int m, n, k;        // rows of A (>= m valid rows are zero), columns of C, reduction length
  int k_chunk;        // K per blockIdx.y (multiple of 64)
  int mode;           // Epilogue
  float* C;           // f32 out [m][ldc] (store / atomic)
  int ldc;
  const float* bias;  // [n] (GELU forward)
  __nv_bfloat16* H;   // bf16 out [m][n] (GELU fwd: activation; bwd: gradient)
  __nv_bfloat16* HT;  // bf16 out [n][ldht] transposed, or NULL
  int ldht;
  float* Zout;        // f32 pre-activation [m][n] (GELU fwd), or NULL
  const float* Zin;   // f32 pre-activation [m][n] (GELU bwd)
  int* err;
};

constexpr int kBM = 128, kBK = 64;

template <int BN>
__global__ void __launch_bounds__(128) gemm_kernel(GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sa[2] = {smem, smem + kBM * kBK * 2};
  unsigned char* sb[2] = {smem + 2 * kBM * kBK * 2, smem + 2 * kBM * kBK * 2 + BN * kBK * 2};
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tbase;
  const int t = threadIdx.x, warp = t >> 5;
  const int row0 = blockIdx.x * kBM, col0 = blockIdx.z * BN;
  const int kbeg = blockIdx.y * g.k_chunk;
  const int kend = min(g.k, kbeg + g.k_chunk);
  const int nk = (kend - kbeg + kBK - 1) / kBK;

  if (warp == 0) tc::tmem_alloc(&tbase, BN < 32 ? 32 : BN);
  if (t == 0) { tc::mbar_init(&bar[0], 1); tc::mbar_init(&bar[1], 1); }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tbase;

  // Copies K chunk `c` of A and B into stage s (16-byte pieces; zero-fill outside).
  auto load = [&](int c, int s) {
    const int k0 = kbeg + c * kBK;
    const uint32_t a0 = tc::smem_addr(sa[s]), b0 = tc::smem_addr(sb[s]);
    for (int p = t; p < kBM * (kBK / 8); p += 128) {
      const int r = p / (kBK / 8), kk = (p % (kBK / 8)) * 8;
      const bool ok = row0 + r < g.m && k0 + kk < kend;
      const __nv_bfloat16* src = g.A + (size_t)(ok ? row0 + r : 0) * g.lda + (ok ? k0 + kk : 0);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(a0 + tc::kmajor_offset(r, kk, kBK)),
                   "l"(src), "r"(ok ? 16 : 0));
    }
    for (int p = t; p < BN * (kBK / 8); p += 128) {
      const int r = p / (kBK / 8), kk = (p % (kBK / 8)) * 8;
      const bool ok = col0 + r < g.n && k0 + kk < kend;
      const __nv_bfloat16* src = g.B + (size_t)(ok ? col0 + r : 0) * g.ldb + (ok ? k0 + kk : 0);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(b0 + tc::kmajor_offset(r, kk, kBK)),
                   "l"(src), "r"(ok ? 16 : 0));
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };

  bool ok = true;
  uint32_t uses[2] = {0, 0};
  if (nk > 0) load(0, 0);
  for (int c = 0; c < nk && ok; ++c) {
    const int s = c & 1;
    if (c + 1 < nk) {
      const int s2 = (c + 1) & 1;
      if (c + 1 >= 2) {  // the MMAs that read stage s2 (chunk c - 1) must be done
        // One decision for the whole CTA: the loop body holds block-wide barriers.
        ok = __syncthreads_and(tc::mbar_wait(&bar[s2], (uses[s2] - 1) & 1, g.err, 1)) != 0;
        if (!ok) break;
      }
      load(c + 1, s2);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    tc::fence_smem_for_async();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_addr(sa[s]), b0 = tc::smem_addr(sb[s]);
#pragma unroll
      for (int q = 0; q < kBK / 16; ++q)
        tc::mma_bf16(tmem, tc::tile_desc(a0, kBK, q), tc::tile_desc(b0, kBK, q),
                     tc::idesc_bf16(kBM, BN), c > 0 || q > 0);
      tc::mma_commit(&bar[s]);
    }
    ++uses[s];
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // All MMAs were committed in order: the last commit completes after all of them.
  if (ok && nk > 0) {
    const int s = (nk - 1) & 1;
    ok = tc::mbar_wait(&bar[s], (uses[s] - 1) & 1, g.err, 2);
  }
  ok = __syncthreads_and(ok) != 0;  // the epilogue's TMEM loads are warp-collective
  tc::fence_after_sync();
  const int r = row0 + 32 * warp + (t & 31);
  if (ok && nk > 0) {
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + c0, v);  // whole warp
      if (r >= g.m) continue;
      for (int i = 0; i < 16; ++i) {
        const int col = col0 + c0 + i;
        if (col >= g.n) break;
        const float a = v[i];
        switch (g.mode) {
          case kStoreF32: g.C[(size_t)r * g.ldc + col] = a; break;
          case kAtomicF32: atomicAdd(g.C + (size_t)r * g.ldc + col, a); break;
          case kGeluFwd: {
            const float z = a + g.bias[col];
            if (g.Zout) g.Zout[(size_t)r * g.n + col] = z;
            const __nv_bfloat16 h = __float2bfloat16_rn(gelu(z));
            g.H[(size_t)r * g.n + col] = h;
            if (g.HT) g.HT[(size_t)col * g.ldht + r] = h;
            break;
          }
          default: {  // kGeluBwd
            const __nv_bfloat16 h = __float2bfloat16_rn(a * gelu_grad(g.Zin[(size_t)r * g.n + col]));
            g.H[(size_t)r * g.n + col] = h;
            if (g.HT) g.HT[(size_t)col * g.ldht + r] = h;
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, BN < 32 ? 32 : BN);
}


// ------------------------------------------------------------ fused inference
struct InferArgs {
  FeatArgs f;
  const __nv_bfloat16* __restrict__ w1;  // [64][656]
  const __nv_bfloat16* __restrict__ w2;  // [64][64]
  const __nv_bfloat16* __restrict__ w3;  // [64][64]
  const __nv_bfloat16* __restrict__ w4;  // [32][64], rows >= 19 zero
  const float* __restrict__ b;           // b1[64] b2[64] b3[64] b4[32]
  float out_scale;                       // correction = y / out_scale
  float* __restrict__ corr;              // [19][N]
  int* err;
};

constexpr int kInferThreads = 512;
// Layer 1 runs in three passes over neighbour groups 0-9, 10-19 and 20-26 (+ 8 zero columns):
// 240, 240 and 176 columns of the A tile.
constexpr int kPassCols = 240;
// A tile is a 2 x 8 x 8 block of cells (128 rows); its 3^3 neighbourhoods lie in a
// 4 x 10 x 10 halo block whose feature groups are staged in shared memory once.
constexpr int kTX = 2, kTY = 8, kTZ = 8;
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2;
constexpr int kHalo = kHX * kHY * kHZ;
constexpr size_t kOffW1 = 0;
constexpr size_t kOffW2 = kOffW1 + 64 * kK1 * 2;
constexpr size_t kOffW3 = kOffW2 + 64 * 64 * 2;
constexpr size_t kOffW4 = kOffW3 + 64 * 64 * 2;
constexpr size_t kOffA = kOffW4 + kOutPad * 64 * 2;
constexpr size_t kOffH = kOffA + 128 * kPassCols * 2;
constexpr size_t kOffHalo = kOffH + 128 * 64 * 2;
constexpr size_t kInferSmem = kOffHalo + (kHalo + 1) * kGroup * 2;  // + one zero group
static_assert(kInferSmem <= 227 * 1024 - 2048, "fused inference tile exceeds shared memory");

__device__ __forceinline__ void stage_weights(unsigned char* dst, const __nv_bfloat16* src, int rows,
                                              int kc) {
  for (int p = threadIdx.x; p < rows * (kc / 8); p += blockDim.x) {
    const int r = p / (kc / 8), k = (p % (kc / 8)) * 8;
    *reinterpret_cast<uint4*>(dst + tc::kmajor_offset(r, k, kc)) =
        *reinterpret_cast<const uint4*>(src + (size_t)r * kc + k);
  }
}

// Bias + GELU of TMEM columns [quarter * 16, quarter * 16 + 16) of this warp's 32 rows into H.
__device__ __forceinline__ void hidden_epilogue(uint32_t taddr, const float* bias, int quarter,
                                                unsigned char* h, int row) {
  float v[16];
  tc::tmem_ld16(taddr + quarter * 16, v);
  uint32_t w[8];
#pragma unroll
  for (int i = 0; i < 16; i += 2) {
    const int col = quarter * 16 + i;
    const __nv_bfloat162 pr = __floats2bfloat162_rn(gelu(v[i] + bias[col]), gelu(v[i + 1] + bias[col + 1]));
    w[i / 2] = *reinterpret_cast<const uint32_t*>(&pr);
  }
  *reinterpret_cast<uint4*>(h + tc::kmajor_offset(row, quarter * 16, 64)) = make_uint4(w[0], w[1], w[2], w[3]);
  *reinterpret_cast<uint4*>(h + tc::kmajor_offset(row, quarter * 16 + 8, 64)) = make_uint4(w[4], w[5], w[6], w[7]);
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__global__ void __launch_bounds__(kInferThreads, 1) closure_infer_kernel(InferArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ float sb[64 * 3 + kOutPad];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  stage_weights(smem + kOffW1, a.w1, 64, kK1);
  stage_weights(smem + kOffW2, a.w2, 64, 64);
  stage_weights(smem + kOffW3, a.w3, 64, 64);
  stage_weights(smem + kOffW4, a.w4, kOutPad, 64);
  for (int i = t; i < 64 * 3 + kOutPad; i += kInferThreads) sb[i] = a.b[i];
  if (warp == 0) tc::tmem_alloc(&tbase, 256);
  if (t == 0) tc::mbar_init(&bar, 1);
  tc::fence_smem_for_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tbase;
  const uint32_t sA = tc::smem_addr(smem + kOffA), sH = tc::smem_addr(smem + kOffH);
  const uint32_t sW1 = tc::smem_addr(smem + kOffW1), sW2 = tc::smem_addr(smem + kOffW2);
  const uint32_t sW3 = tc::smem_addr(smem + kOffW3), sW4 = tc::smem_addr(smem + kOffW4);
  __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(smem + kOffHalo);
  const LbmGeom& g = a.f.g;
  const int ntx = (g.nx + kTX - 1) / kTX, nty = (g.ny + kTY - 1) / kTY, ntz = (g.nz + kTZ - 1) / kTZ;
  const long long ntiles = (long long)ntx * nty * ntz;
  uint32_t phase = 0;
  bool ok = true;
  const int lrow = 32 * (warp & 3) + lane, lq = warp >> 2;     // epilogue role (TMEM lane)
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;

  // Issues the MMAs of one layer and waits for them; false on timeout (CTA-uniform).
  auto run_layer = [&](uint32_t dcol, uint32_t a_addr, int akc, uint32_t b_addr, int bkc,
                       int kslice0, int nsl, int n, bool accumulate) -> bool {
    tc::fence_smem_for_async();
    tc::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      for (int s = 0; s < nsl; ++s)
        tc::mma_bf16(tmem + dcol, tc::tile_desc(a_addr, akc, s), tc::tile_desc(b_addr, bkc, kslice0 + s),
                     tc::idesc_bf16(128, n), accumulate || s > 0);
      tc::mma_commit(&bar);
    }
    const bool r = tc::mbar_wait(&bar, phase & 1, a.err, 3);
    ++phase;
    tc::fence_after_sync();
    return __syncthreads_and(r) != 0;
  };

  if (t < 3) reinterpret_cast<uint4*>(halo + kHalo * kGroup)[t] = make_uint4(0, 0, 0, 0);  // zero group
  for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int tx = (int)(tile / ((long long)nty * ntz)), ty = (int)((tile / ntz) % nty), tz = (int)(tile % ntz);
    const int x0 = tx * kTX, y0 = ty * kTY, z0 = tz * kTZ;
    // Stage the halo block's feature vectors (the previous tile's reads of the halo are
    // complete: its last layer waited on the tensor cores and synchronised the CTA).
    for (int h = t; h < kHalo; h += kInferThreads) {
      const int hx = h / (kHY * kHZ), hy = (h / kHZ) % kHY, hz = h % kHZ;
      float v[23];
      neighbour_features(a.f, wrap(x0 + hx - 1, g.nx), wrap(y0 + hy - 1, g.ny), wrap(z0 + hz - 1, g.nz), v);
      uint32_t w[12];
#pragma unroll
      for (int f = 0; f < 22; f += 2) {
        const __nv_bfloat162 pr = __floats2bfloat162_rn(v[f], v[f + 1]);
        w[f / 2] = *reinterpret_cast<const uint32_t*>(&pr);
      }
      {
        const __nv_bfloat162 pr = __floats2bfloat162_rn(v[22], 0.f);
        w[11] = *reinterpret_cast<const uint32_t*>(&pr);
      }
      uint4* dst = reinterpret_cast<uint4*>(halo + h * kGroup);
      dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
      dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
      dst[2] = make_uint4(w[8], w[9], w[10], w[11]);
    }
    __syncthreads();
    // Layer 1 in three passes of neighbour groups: each group is three 16-byte pieces.
    for (int p = 0; p < 3 && ok; ++p) {
      unsigned char* A = smem + kOffA;
      const int o0 = p * 10, ng = p < 2 ? 10 : 7;
      const int cols = p < 2 ? kPassCols : 7 * kGroup + 8;
      const int pieces = cols / 8;  // ng groups x 3 pieces (+1 zero piece in the last pass)
      for (int it = t; it < 128 * pieces; it += kInferThreads) {
        const int r = it & 127, pc = it >> 7;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (pc < ng * 3) {
          const int o = o0 + pc / 3;
          const int rrx = r / (kTY * kTZ), rry = (r / kTZ) % kTY, rrz = r % kTZ;
          const int hc = ((rrx + o / 9) * kHY + rry + (o / 3) % 3) * kHZ + rrz + o % 3;
          val = reinterpret_cast<const uint4*>(halo + hc * kGroup)[pc % 3];
        }
        *reinterpret_cast<uint4*>(A + tc::kmajor_offset(r, pc * 8, cols)) = val;
      }
      ok = run_layer(0, sA, cols, sW1, kK1, o0 * kGroup / 16, cols / 16, 64, p > 0);
    }
    if (!ok) break;
    hidden_epilogue(tmem + lane_base, sb, lq, smem + kOffH, lrow);
    ok = run_layer(64, sH, 64, sW2, 64, 0, 4, 64, false);
    if (!ok) break;
    hidden_epilogue(tmem + lane_base + 64, sb + 64, lq, smem + kOffH, lrow);
    ok = run_layer(128, sH, 64, sW3, 64, 0, 4, 64, false);
    if (!ok) break;
    hidden_epilogue(tmem + lane_base + 128, sb + 128, lq, smem + kOffH, lrow);
    ok = run_layer(192, sH, 64, sW4, 64, 0, 4, kOutPad, false);
    if (!ok) break;
    // Output layer: warps 0-3 own the 128 rows; 19 of the 32 columns are used.
    if (warp < 4) {
      float y[32];
      tc::tmem_ld16(tmem + lane_base + 192, *reinterpret_cast<float(*)[16]>(y));
      tc::tmem_ld16(tmem + lane_base + 208, *reinterpret_cast<float(*)[16]>(y + 16));
      const int ox = x0 + lrow / (kTY * kTZ), oy = y0 + (lrow / kTZ) % kTY, oz = z0 + lrow % kTZ;
      if (ox < g.nx && oy < g.ny && oz < g.nz) {
        const long long cc = ((long long)ox * g.ny + oy) * g.nz + oz;
        const bool fluid = !(a.f.flags[cc] & kFlagSolid);
#pragma unroll
        for (int q = 0; q < kOut; ++q)
          a.corr[(size_t)q * g.n + cc] = fluid ? (y[q] + sb[192 + q]) / a.out_scale : 0.f;
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

// f_q(x) += c_q - w_q sum_p c_p on fluid cells (the correction moves no mass).
__global__ void __launch_bounds__(kBlock) closure_apply_kernel(LbmGeom g, float* __restrict__ pops,
                                                               const uint32_t* __restrict__ flags,
                                                               int parity, const float* __restrict__ corr) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= g.n) return;
  const uint32_t fl = flags[c];
  if (fl & kFlagSolid) return;
  const int nyz = g.ny * g.nz;
  const Deltas d(g, (int)(c / nyz), (int)((c / g.nz) % g.ny), (int)(c % g.nz));
  float cq[19], sum = 0.f;
#pragma unroll
  for (int q = 0; q < 19; ++q) { cq[q] = corr[(size_t)q * g.n + c]; sum += cq[q]; }
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    const uint32_t s = slot32((uint32_t)g.n, d, fl, q, parity);
    pops[s] += cq[q] - weight_of(q) * sum;
  }
}

// Restriction of a fine lattice (2nx x 2ny x 2nz) onto the coarse one: mean post-stream
// populations of the fluid children (reference layout out[Nc][19]); a coarse cell whose
// children are all solid gets the rest equilibrium w_q rho0.
__global__ void __launch_bounds__(kBlock) closure_restrict_kernel(LbmGeom fg, const float* __restrict__ fpops,
                                                                  const uint32_t* __restrict__ fflags,
                                                                  int parity, LbmGeom cg, float rho0,
                                                                  float* __restrict__ out) {
  const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (c >= cg.n) return;
  const int nyz = cg.ny * cg.nz;
  const int I = (int)(c / nyz), J = (int)((c / cg.nz) % cg.ny), K = (int)(c % cg.nz);
  float acc[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) acc[q] = 0.f;
  int nf = 0;
  for (int ch = 0; ch < 8; ++ch) {
    const int i = 2 * I + (ch >> 2), j = 2 * J + ((ch >> 1) & 1), k = 2 * K + (ch & 1);
    const Deltas d(fg, i, j, k);
    const uint32_t fl = fflags[d.c];
    if (fl & kFlagSolid) continue;
    ++nf;
#pragma unroll
    for (int q = 0; q < 19; ++q) acc[q] += gather32<FSI_STORAGE_F32>(fpops, (uint32_t)fg.n, d, fl, q, parity, 0.f);
  }
#pragma unroll
  for (int q = 0; q < 19; ++q) out[(size_t)c * 19 + q] = nf ? acc[q] / (float)nf : weight_of(q) * rho0;
}

// dY = 2 (Y + b4 - T) / (m * 19) on the 19 outputs (0 on padding), BF16 [m][32] and its
// transpose [32][ldt]; loss += sum (Y + b4 - T)^2 / (m * 19).
__global__ void __launch_bounds__(kBlock) closure_loss_kernel(const float* __restrict__ y,
                                                              const float* __restrict__ target,
                                                              const float* __restrict__ b4, int m,
                                                              __nv_bfloat16* __restrict__ dy,
                                                              __nv_bfloat16* __restrict__ dyt, int ldt,
                                                              double* __restrict__ loss) {
  const long long t = (long long)blockIdx.x * kBlock + threadIdx.x;
  float e2 = 0.f;
  if (t < (long long)m * kOutPad) {
    const int r = (int)(t / kOutPad), q = (int)(t % kOutPad);
    float gq = 0.f;
    if (q < kOut) {
      const float e = y[t] + b4[q] - target[(size_t)r * kOut + q];
      e2 = e * e;
      gq = 2.f * e / ((float)m * kOut);
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(gq);
    dy[t] = h;
    dyt[(size_t)q * ldt + r] = h;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e2 += __shfl_down_sync(0xffffffffu, e2, o);
  if ((threadIdx.x & 31) == 0 && e2 != 0.f) atomicAdd(loss, (double)e2 / ((double)m * kOut));
}

// out[c] += sum over rows of g[r][c] (bias gradients), g BF16 [m][n].
__global__ void __launch_bounds__(kBlock) closure_colsum_kernel(const __nv_bfloat16* __restrict__ g,
                                                                int m, int n, float* __restrict__ out) {
  const int col = blockIdx.y;
  float s = 0.f;
  for (long long r = (long long)blockIdx.x * kBlock + threadIdx.x; r < m; r += (long long)gridDim.x * kBlock)
    s += __bfloat162float(g[(size_t)r * n + col]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out + col, s);
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void __launch_bounds__(kBlock) closure_adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                                                              float* __restrict__ m, float* __restrict__ v,
                                                              long long n, float lr, float b1, float b2,
                                                              float eps, float c1, float c2) {
  const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

FeatArgs feat_args(const fsi_lbm_desc* d, const float* pops, const uint32_t* flags,
                   const float* force, int64_t steps_done, float pop_scale, float force_scale) {
  FeatArgs f;
  f.g = geom_of(d);
  f.pops = pops;
  f.flags = flags;
  f.force = force;
  f.parity = (int)(steps_done & 1);
  f.rho0 = d->rho0;
  f.pop_scale = pop_scale;
  f.force_scale = force_scale;
  return f;
}

int check_closure_lattice(const fsi_lbm_desc* d) {
  FSI_REQUIRE(d != nullptr, "NULL lattice descriptor");
  FSI_REQUIRE(d->storage == FSI_STORAGE_F32, "the closure runs on FP32 populations");
  FSI_REQUIRE(d->nx > 4 && d->ny > 4 && d->nz > 4, "lattice too small");
  FSI_REQUIRE(19ll * d->nx * d->ny * d->nz < (1ll << 32), "lattice too large");
  return FSI_OK;
}

}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_closure_features(const fsi_lbm_desc* d, const float* pops, const uint32_t* flags,
                                    const float* force, int64_t steps_done, const int32_t* cells,
                                    int32_t m, float pop_scale, float force_scale, void* x,
                                    void* stream) {
  if (int e = check_closure_lattice(d)) return e;
  FSI_REQUIRE(pops && flags && force && cells && x && m > 0, "NULL array or empty cell list");
  const FeatArgs f = feat_args(d, pops, flags, force, steps_done, pop_scale, force_scale);
  closure_features_kernel<<<grid_for(28ll * m, 256), 256, 0, as_stream(stream)>>>(
      f, cells, m, reinterpret_cast<__nv_bfloat16*>(x));
  return check_launch("closure_features_kernel");
}

extern "C" int fsi_closure_gemm(const fsi_closure_gemm_desc* d, void* stream) {
  FSI_REQUIRE(d && d->a && d->b && d->err, "NULL GEMM operand");
  FSI_REQUIRE(d->m > 0 && d->n > 0 && d->k > 0, "empty GEMM");
  FSI_REQUIRE(d->lda % 8 == 0 && d->ldb % 8 == 0, "leading dimensions must be multiples of 8");
  FSI_REQUIRE(((uintptr_t)d->a & 15) == 0 && ((uintptr_t)d->b & 15) == 0, "operands must be 16-byte aligned");
  FSI_REQUIRE(d->k_chunk > 0 && d->k_chunk % kBK == 0, "k_chunk must be a positive multiple of 64");
  FSI_REQUIRE(d->mode >= 0 && d->mode <= 3, "unknown epilogue %d", d->mode);
  FSI_REQUIRE(d->mode > 1 || d->c, "FP32 output missing");
  FSI_REQUIRE(d->mode < 2 || d->h, "BF16 output missing");
  FSI_REQUIRE(d->mode != 2 || d->bias, "bias missing");
  FSI_REQUIRE(d->mode != 3 || d->zin, "pre-activation missing");
  GemmArgs g{};
  g.A = reinterpret_cast<const __nv_bfloat16*>(d->a);
  g.B = reinterpret_cast<const __nv_bfloat16*>(d->b);
  g.lda = d->lda; g.ldb = d->ldb;
  g.m = d->m; g.n = d->n; g.k = d->k; g.k_chunk = d->k_chunk; g.mode = d->mode;
  g.C = d->c; g.ldc = d->ldc; g.bias = d->bias;
  g.H = reinterpret_cast<__nv_bfloat16*>(d->h);
  g.HT = reinterpret_cast<__nv_bfloat16*>(d->ht);
  g.ldht = d->ldht; g.Zout = d->zout; g.Zin = d->zin; g.err = d->err;
  const int bn = d->n <= 32 ? 32 : (d->n <= 64 ? 64 : 128);
  const dim3 grid((d->m + kBM - 1) / kBM, (d->k + d->k_chunk - 1) / d->k_chunk, (d->n + bn - 1) / bn);
  FSI_REQUIRE(grid.y <= 65535 && grid.z <= 65535, "GEMM grid too large");
  cudaStream_t s = as_stream(stream);
  const int smem = (2 * kBM * kBK + 2 * bn * kBK) * 2;
  if (bn == 32) {
    cudaFuncSetAttribute(gemm_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    gemm_kernel<32><<<grid, 128, smem, s>>>(g);
  } else if (bn == 64) {
    cudaFuncSetAttribute(gemm_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    gemm_kernel<64><<<grid, 128, smem, s>>>(g);
  } else {
    cudaFuncSetAttribute(gemm_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    gemm_kernel<128><<<grid, 128, smem, s>>>(g);
  }
  return check_launch("gemm_kernel");
}

extern "C" int fsi_closure_infer(const fsi_lbm_desc* d, const float* pops, const uint32_t* flags,
                                 const float* force, int64_t steps_done,
                                 const fsi_closure_weights* w, float* corr, int32_t* err,
                                 void* stream) {
  if (int e = check_closure_lattice(d)) return e;
  FSI_REQUIRE(pops && flags && force && w && corr && err, "NULL array");
  FSI_REQUIRE(w->w1 && w->w2 && w->w3 && w->w4 && w->bias, "NULL weights");
  FSI_REQUIRE(w->out_scale != 0.f, "out_scale must be non-zero");
  InferArgs a;
  a.f = feat_args(d, pops, flags, force, steps_done, w->pop_scale, w->force_scale);
  a.w1 = reinterpret_cast<const __nv_bfloat16*>(w->w1);
  a.w2 = reinterpret_cast<const __nv_bfloat16*>(w->w2);
  a.w3 = reinterpret_cast<const __nv_bfloat16*>(w->w3);
  a.w4 = reinterpret_cast<const __nv_bfloat16*>(w->w4);
  a.b = w->bias;
  a.out_scale = w->out_scale;
  a.corr = corr;
  a.err = err;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (long long)((a.f.g.nx + kTX - 1) / kTX) * ((a.f.g.ny + kTY - 1) / kTY) *
                          ((a.f.g.nz + kTZ - 1) / kTZ);
  const int grid = (int)(tiles < sms ? tiles : sms);
  cudaFuncSetAttribute(closure_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kInferSmem);
  closure_infer_kernel<<<grid, kInferThreads, kInferSmem, as_stream(stream)>>>(a);
  return check_launch("closure_infer_kernel");
}

extern "C" int fsi_closure_apply(const fsi_lbm_desc* d, float* pops, const uint32_t* flags,
                                 int64_t steps_done, const float* corr, void* stream) {
  if (int e = check_closure_lattice(d)) return e;
  FSI_REQUIRE(pops && flags && corr, "NULL array");
  const LbmGeom g = geom_of(d);
  closure_apply_kernel<<<grid_for(g.n, kBlock), kBlock, 0, as_stream(stream)>>>(
      g, pops, flags, (int)(steps_done & 1), corr);
  return check_launch("closure_apply_kernel");
}

extern "C" int fsi_closure_restrict(const fsi_lbm_desc* fine, const float* pops, const uint32_t* flags,
                                    int64_t steps_done, const fsi_lbm_desc* coarse, float* out,
                                    void* stream) {
  if (int e = check_closure_lattice(fine)) return e;
  if (int e = check_closure_lattice(coarse)) return e;
  FSI_REQUIRE(pops && flags && out, "NULL array");
  FSI_REQUIRE(fine->nx == 2 * coarse->nx && fine->ny == 2 * coarse->ny && fine->nz == 2 * coarse->nz,
              "fine lattice must be twice the coarse one on every axis");
  const LbmGeom cg = geom_of(coarse);
  closure_restrict_kernel<<<grid_for(cg.n, kBlock), kBlock, 0, as_stream(stream)>>>(
      geom_of(fine), pops, flags, (int)(steps_done & 1), cg, coarse->rho0, out);
  return check_launch("closure_restrict_kernel");
}

extern "C" int fsi_closure_loss(const float* y, const float* target, const float* b4, int32_t m,
                                void* dy, void* dyt, int32_t ldt, double* loss, void* stream) {
  FSI_REQUIRE(y && target && b4 && dy && dyt && loss && m > 0 && ldt >= m, "bad loss arguments");
  closure_loss_kernel<<<grid_for((long long)m * kOutPad, kBlock), kBlock, 0, as_stream(stream)>>>(
      y, target, b4, m, reinterpret_cast<__nv_bfloat16*>(dy), reinterpret_cast<__nv_bfloat16*>(dyt),
      ldt, loss);
  return check_launch("closure_loss_kernel");
}

extern "C" int fsi_closure_colsum(const void* g, int32_t m, int32_t n, float* out, void* stream) {
  FSI_REQUIRE(g && out && m > 0 && n > 0 && n <= 65535, "bad column-sum arguments");
  int blocks = (int)((m + kBlock - 1) / kBlock);
  if (blocks > 64) blocks = 64;
  closure_colsum_kernel<<<dim3(blocks, n), kBlock, 0, as_stream(stream)>>>(
      reinterpret_cast<const __nv_bfloat16*>(g), m, n, out);
  return check_launch("closure_colsum_kernel");
}

extern "C" int fsi_closure_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr,
                                float beta1, float beta2, float eps, int32_t step, void* stream) {
  FSI_REQUIRE(p && g && m && v && n > 0 && step > 0, "bad Adam arguments");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  closure_adam_kernel<<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(p, g, m, v, n, lr, beta1,
                                                                              beta2, eps, c1, c2);
  return check_launch("closure_adam_kernel");
}
