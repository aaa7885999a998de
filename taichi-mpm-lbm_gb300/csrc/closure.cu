// Learned coarse-grid closure: a per-cell MLP (656 -> 64 -> 64 -> 64 -> 19, GELU) that
// corrects the populations of a lattice running on a 2x coarser grid, on the fifth-
// generation tensor cores (tcgen05, BF16 operands, FP32 accumulation in tensor memory).
// No reference counterpart.
//
// Features of a cell x: for each of the 27 cells y of its 3^3 neighbourhood (periodic wrap,
// offsets in (dx, dy, dz) order, dz fastest) the 19 post-stream populations as scaled
// deviations (f_q(y) - w_q rho0) * pop_scale, the occupancy of y (its solid fraction when
// given -- the share of a coarse cell's fine children that are solid --, else 1 solid /
// 0 fluid) and the
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
//   closure_infer_kernel: the fused inference pass: layer 1 as an implicit 3x3x3
//     convolution over per-cell feature rows staged once in shared memory, the four layers
//     on the tensor cores with the weights resident in shared memory, two tiles in flight,
//     and the 19 outputs written as corrections per cell.
//   closure_apply_kernel: f_q(x) += correction, mass-conserving (sum_q w-weighted projection).
//   loss / Adam kernels for training.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

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

// GELU, tanh form of Hendrycks & Gimpel (2016): 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))),
// with tanh from the hardware approximation (tanh.approx.f32, relative error about 2^-11,
// below the BF16 rounding of the activations). Training and inference use the same form.
constexpr float kGeluC0 = 0.7978845608028654f;
constexpr float kGeluC1 = 0.044715f;
constexpr float kGeluC01 = kGeluC0 * kGeluC1;
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float z) {
  const float t = tanh_approx(z * fmaf(kGeluC01, z * z, kGeluC0));
  const float hz = 0.5f * z;
  return fmaf(hz, t, hz);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float t = tanh_approx(z * fmaf(kGeluC01, z * z, kGeluC0));
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * kGeluC0 * (1.0f + 3.0f * kGeluC1 * z * z);
}

struct FeatArgs {
  LbmGeom g;
  const float* __restrict__ pops;  // FP32 populations [19][N], AA layout of `parity`
  const uint32_t* __restrict__ flags;
  const float* __restrict__ force;  // [3][N]
  const float* __restrict__ frac;   // [N] solid fraction of each cell, or NULL (occupancy 0/1)
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
  v[19] = a.frac ? a.frac[d.c] : (solid ? 1.f : 0.f);
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
//
// Layer 1 is a 3 x 3 x 3 convolution of per-cell vectors of 24 channels (the 23 feature
// values of a cell + one zero), so it runs as an implicit GEMM: the 24-channel rows of a
// block of cells are staged in shared memory once, and each of the 27 neighbour offsets is
// an MMA whose A operand is the same rows shifted by that offset.
//
// Rows are laid out for this: three channel chunks (channels 0-7, 8-15, 16-23), each an
// array of rows at a 16-byte stride, so the core matrices of 8 rows x 16 bytes follow one
// another (stride byte offset 128) and chunk c + 1 lies kChunkBytes after chunk c (leading
// byte offset). A row shift is a start-address shift of 16 bytes. Per offset o, one K = 16
// MMA covers channels 0-15; channels 16-23 of two offsets a < b of the same x-plane share
// one MMA whose second K half starts (row_b - row_a) * 16 bytes after the first. That is
// 27 + 3 * 5 = 42 MMAs of M = 128, N = 64, K = 16 per tile of 128 rows.
//
// closure_rows_kernel first writes every cell's 24 BF16 channels to global memory in the
// same chunked layout, on a lattice padded by one periodic image in y and z (and to whole
// columns). Cells are walked in columns: 32 cells along z x 11 lines along y, streamed
// along x. An x-plane of a column is a 34 x 13 halo block (442 rows, z fastest), fetched
// into a ring of four slots (x - 1, x, x + 1 in use, x + 2 in flight) by three TMA tensor
// copies (one box of 8 channels x 34 x 13 per chunk) that complete on the slot's mbarrier. The output rows of a plane are the
// 374 rows of lines 1..11, covered by three M tiles of 128 consecutive rows; rows on the z
// halo (and past line 11) are computed and discarded.
//
// Each CTA (one per SM) takes a contiguous range of (column, x) plane steps. Warps 0-15 run
// the epilogues (warp w reads TMEM lanes 32 (w % 4) .. + 31 and columns 16 (w / 4) .. + 15);
// one thread of warp 16 issues the plane copies and layers 2-4 of each tile as its layer-1,
// -2 and -3 epilogues finish; one thread of warp 17 issues layer 1 (42 MMAs) of the tiles
// ahead, as soon as the tensor-memory half and the planes a tile needs are free and loaded.
// Two tiles are in flight (TMEM halves 0 and 256): the tensor cores run layer 1 of tile
// t + 1 while the epilogues of tile t run on the CUDA cores, and the small layers of tile t
// never queue behind a thread that is blocked issuing layer 1. Every hand-over is an
// mbarrier, so no CTA-wide barrier sits inside the loop; barriers written more than once
// per tile by a role that can run ahead (layer-1 commits, layer-1 epilogue arrivals) come
// in pairs indexed by the TMEM half, so a waiter is never two phases behind.
constexpr int kLine = 34;                             // halo line along z: 32 cells + 2
constexpr int kLineCells = 32;
constexpr int kLines = 11;                            // output lines along y per column
constexpr int kPlaneRows = kLine * (kLines + 2);      // 442
constexpr int kPlaneTiles = (kLine * kLines + 127) / 128;  // 3
constexpr int kSlots = 4;
constexpr int kSlotRows = 448;                        // a plane, padded to 128-byte boundaries
constexpr int kPadLo = 8, kPadHi = 48;
constexpr int kChunkRows = kPadLo + kSlots * kSlotRows + kPadHi;
constexpr int kChunkBytes = kChunkRows * 16;
constexpr int kL1Mmas = 27 + 3 * 5;                   // 42
constexpr int kL1Chunk = kL1Mmas / 3;                 // 14 MMAs per issue
constexpr int kEpiWarps = 16;                         // epilogue warps (4 per TMEM lane quarter)
constexpr int kWorkers = 32 * kEpiWarps;
constexpr int kGroupWarps = kEpiWarps / 2;            // two epilogue groups, alternate tiles
constexpr size_t kHBytes = 128 * 64 * 2;              // one activation tile
constexpr int kChainWarp = kEpiWarps, kL1Warp = kEpiWarps + 1;
constexpr int kInferThreads = kWorkers + 64;          // + the two MMA-issuing warps
constexpr uint32_t kPlaneBytes = 3u * kPlaneRows * 16u;  // one plane: three tensor-copy boxes
static_assert(kL1Chunk * 3 == kL1Mmas, "layer 1 is issued in three equal chunks");
// Highest row read: the last tile's last row, offset +35, and the +16-byte second half of
// the unpaired offset of a plane.
static_assert(kLine + 128 * kPlaneTiles + kLine + 2 <= kSlotRows + kPadHi, "row padding");
static_assert(kSlotRows >= kPlaneRows && (kSlotRows * 16) % 128 == 0 && (kPadLo * 16) % 128 == 0 &&
                  kChunkBytes % 128 == 0,
              "tensor-copy destinations are 128-byte aligned");
static_assert(kChunkBytes < (1 << 18), "leading byte offset field");

constexpr size_t kOffW1 = 0;                                  // 42 slices of 64 x 16
constexpr size_t kOffW2 = kOffW1 + (size_t)kL1Mmas * 64 * 16 * 2;
constexpr size_t kOffW3 = kOffW2 + 64 * 64 * 2;
constexpr size_t kOffW4 = kOffW3 + 64 * 64 * 2;
constexpr size_t kOffH = kOffW4 + kOutPad * 64 * 2;
constexpr size_t kOffRows = kOffH + 2 * kHBytes;     // an activation tile per group
constexpr size_t kInferSmem = kOffRows + 3 * (size_t)kChunkBytes;
static_assert(kInferSmem <= 227 * 1024 - 2048, "fused inference exceeds shared memory");

// Padded row lattice of the inference: nx x ny_pad x nz_pad rows per chunk; padded row
// (x, jp, kp) holds cell (x, (jp - 1) mod ny, (kp - 1) mod nz).
struct RowGeom {
  int nyb, nzb;           // columns: ceil(ny / 11) x ceil(nz / 32)
  int ny_pad, nz_pad;     // 11 nyb + 2, 32 nzb + 2
  long long chunk_rows;   // nx * ny_pad * nz_pad
};

inline RowGeom row_geom(const LbmGeom& g) {
  RowGeom r;
  r.nyb = (g.ny + kLines - 1) / kLines;
  r.nzb = (g.nz + kLineCells - 1) / kLineCells;
  r.ny_pad = kLines * r.nyb + 2;
  r.nz_pad = kLineCells * r.nzb + 2;
  r.chunk_rows = (long long)g.nx * r.ny_pad * r.nz_pad;
  return r;
}

struct InferArgs {
  FeatArgs f;
  RowGeom rg;
  const unsigned char* __restrict__ grows;  // [3][chunk_rows][16 B] from closure_rows_kernel
  const __nv_bfloat16* __restrict__ w1;     // [64][656]
  const __nv_bfloat16* __restrict__ w2;     // [64][64]
  const __nv_bfloat16* __restrict__ w3;     // [64][64]
  const __nv_bfloat16* __restrict__ w4;     // [32][64], rows >= 19 zero
  const float* __restrict__ b;              // b1[64] b2[64] b3[64] b4[32]
  float out_scale;                          // correction = y / out_scale
  float* __restrict__ corr;                 // [19][N] (kApply = false)
  float* __restrict__ pops;                 // populations corrected in place (kApply = true)
  int* err;
  long long work;                           // plane steps: columns * nx
};

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }
__device__ __forceinline__ int wrap_any(int v, int n) {
  const int m = v % n;
  return m < 0 ? m + n : m;
}

// The 24 BF16 channels of every padded row: thread (kp, jp, x) of a grid of 128-thread
// blocks over (z, y, x). All loads are issued before the flags are needed: the populations
// are gathered from the slots a fluid neighbourhood uses, and only the few directions whose
// upwind neighbour is solid (bounce-back) read their own slot afterwards.
__global__ void __launch_bounds__(128) closure_rows_kernel(FeatArgs a, RowGeom rg,
                                                           unsigned char* __restrict__ grows) {
  const int kp = blockIdx.x * 128 + threadIdx.x;
  if (kp >= rg.nz_pad) return;
  const int jp = blockIdx.y, x = blockIdx.z;
  const LbmGeom& g = a.g;
  const Deltas d(g, x, wrap_any(jp - 1, g.ny), wrap_any(kp - 1, g.nz));
  const uint32_t n = (uint32_t)g.n;
  const uint32_t fl = a.flags[d.c];
  float f[19], frc[3];
  f[0] = a.pops[d.c];
  if (a.parity == 0) {
#pragma unroll
    for (int q = 1; q < 19; ++q) f[q] = a.pops[q * n + d.c];
  } else {
#pragma unroll
    for (int q = 1; q < 19; ++q) f[q] = a.pops[opp(q) * n + d.nb(q, -1)];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) frc[c] = a.force[c * n + d.c];
  const bool solid = fl & kFlagSolid;
  if (a.parity != 0 && !solid && (fl & ~kFlagSolid)) {
#pragma unroll
    for (int q = 1; q < 19; ++q)
      if ((fl >> opp(q)) & 1u) f[q] = a.pops[q * n + d.c];
  }
  float v[24];
#pragma unroll
  for (int q = 0; q < 19; ++q) v[q] = solid ? 0.f : (f[q] - weight_of(q) * a.rho0) * a.pop_scale;
  v[19] = a.frac ? a.frac[d.c] : (solid ? 1.f : 0.f);
#pragma unroll
  for (int c = 0; c < 3; ++c) v[20 + c] = frc[c] * a.force_scale;
  v[23] = 0.f;
  uint32_t w[12];
#pragma unroll
  for (int i = 0; i < 24; i += 2) {
    const __nv_bfloat162 pr = __floats2bfloat162_rn(v[i], v[i + 1]);
    w[i / 2] = *reinterpret_cast<const uint32_t*>(&pr);
  }
  const size_t r = ((size_t)x * rg.ny_pad + jp) * rg.nz_pad + kp;
#pragma unroll
  for (int c = 0; c < 3; ++c)
    *reinterpret_cast<uint4*>(grows + ((size_t)c * rg.chunk_rows + r) * 16) =
        make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
}

__device__ __forceinline__ void stage_weights(unsigned char* dst, const __nv_bfloat16* src, int rows,
                                              int kc) {
  for (int p = threadIdx.x; p < rows * (kc / 8); p += blockDim.x) {
    const int r = p / (kc / 8), k = (p % (kc / 8)) * 8;
    *reinterpret_cast<uint4*>(dst + tc::kmajor_offset(r, k, kc)) =
        *reinterpret_cast<const uint4*>(src + (size_t)r * kc + k);
  }
}

// Row offset of neighbour o (dx, dy, dz in {-1, 0, 1}, o = 9 (dx+1) + 3 (dy+1) + dz + 1)
// within its x-plane.
__host__ __device__ constexpr int tap_dy(int o) { return (o / 3) % 3 - 1; }
__host__ __device__ constexpr int tap_dz(int o) { return o % 3 - 1; }
__host__ __device__ constexpr int tap_off(int o) { return kLine * tap_dy(o) + tap_dz(o); }

// Layer-1 weight slices: slice s < 27 holds W1 columns [24 s, 24 s + 16) (channels 0-15 of
// neighbour s); slice 27 + 5 p + j holds channels 16-23 of neighbours 9 p + 2 j and
// 9 p + 2 j + 1 (j < 4), or of neighbour 9 p + 8 and zeros (j = 4).
__device__ __forceinline__ void stage_w1(unsigned char* dst, const __nv_bfloat16* w1) {
  for (int p = threadIdx.x; p < kL1Mmas * 64 * 2; p += blockDim.x) {
    const int s = p >> 7, r = (p >> 1) & 63, half = p & 1;
    int col;
    if (s < 27) {
      col = kGroup * s + 8 * half;
    } else {
      const int u = s - 27, plane = u / 5, j = u % 5;
      col = (j == 4 && half) ? -1 : kGroup * (9 * plane + 2 * j + half) + 16;
    }
    const uint4 v = col < 0 ? make_uint4(0, 0, 0, 0)
                            : *reinterpret_cast<const uint4*>(w1 + (size_t)r * kK1 + col);
    *reinterpret_cast<uint4*>(dst + (size_t)s * 2048 + tc::kmajor_offset(r, 8 * half, 16)) = v;
  }
}

__device__ __forceinline__ float2 gelu2(float2 z) {
  const float2 z2 = vmul(z, z);
  const float2 u = vmul(z, vfma(z2, splat<float2>(kGeluC01), splat<float2>(kGeluC0)));
  const float2 t = make_float2(tanh_approx(u.x), tanh_approx(u.y));
  const float2 hz = vmul(z, splat<float2>(0.5f));
  return vfma(hz, t, hz);
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
    const float2 g = gelu2(vadd(make_float2(v[i], v[i + 1]), make_float2(bias[col], bias[col + 1])));
    const __nv_bfloat162 pr = __floats2bfloat162_rn(g.x, g.y);
    w[i / 2] = *reinterpret_cast<const uint32_t*>(&pr);
  }
  *reinterpret_cast<uint4*>(h + tc::kmajor_offset(row, quarter * 16, 64)) = make_uint4(w[0], w[1], w[2], w[3]);
  *reinterpret_cast<uint4*>(h + tc::kmajor_offset(row, quarter * 16 + 8, 64)) = make_uint4(w[4], w[5], w[6], w[7]);
}

constexpr uint32_t kIdesc64 = tc::idesc_bf16(128, 64), kIdesc32 = tc::idesc_bf16(128, kOutPad);

__device__ __forceinline__ uint64_t opaque(uint64_t v) {
  asm volatile("mov.b64 %0, %0;" : "+l"(v));
  return v;
}

// Layer-1 MMAs [14 C, 14 C + 14) of one tile, into TMEM column d. Descriptors are built by
// adding compile-time offsets to base descriptors: `rows` addresses row 0 of channel chunk 0
// (leading byte offset 0, stride byte offset 128), `w1` weight slice 0; the start-address
// field counts 16-byte units, so a row shift adds the row count. r0, r1, r2: the tile's first
// output row in the x-planes dx = -1, 0, +1.
template <int C>
__device__ __forceinline__ void issue_l1_chunk(uint32_t d, uint64_t rows, int r0, int r1, int r2,
                                               uint64_t w1) {
#pragma unroll
  for (int s = kL1Chunk * C; s < kL1Chunk * (C + 1); ++s) {
    // Each descriptor is derived from an opaque copy of the bases right before its MMA, so
    // the compiler does not compute all of them ahead (they would not fit in registers).
    const uint64_t rows_s = opaque(rows), w1_s = opaque(w1);
    uint64_t a;
    if (s < 27) {
      const int rp = s < 9 ? r0 : (s < 18 ? r1 : r2);
      a = rows_s + ((uint64_t)(kChunkBytes >> 4) << 16) + (uint64_t)(rp + tap_off(s));
    } else {
      const int u = s - 27, plane = u / 5, j = u % 5, o = 9 * plane + 2 * j;
      const int rp = plane == 0 ? r0 : (plane == 1 ? r1 : r2);
      const uint64_t lbo = j < 4 ? (uint64_t)(tap_off(o + 1) - tap_off(o)) : 1u;  // 16-byte units
      a = rows_s + (lbo << 16) + (uint64_t)((2 * kChunkBytes) >> 4) + (uint64_t)(rp + tap_off(o));
    }
    tc::mma_bf16(d, a, w1_s + (uint64_t)(s * (2048 >> 4)), kIdesc64, s > 0);
  }
}

// One hidden or output layer: A = H (128 x 64, K-major), B = the layer's weights.
__device__ __forceinline__ void issue_layer(uint32_t d, uint64_t h, uint64_t w, uint32_t idesc) {
#pragma unroll
  for (int s = 0; s < 4; ++s) tc::mma_bf16(d, h + (uint64_t)(16 * s), w + (uint64_t)(16 * s), idesc, s > 0);
}

__device__ __forceinline__ void expect_bytes(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Plane x of the column at (y0, z0) into ring slot `slot`: one tensor copy per channel chunk
// (box: 8 channels x 34 rows along z x 13 lines along y) completing on `bar`.
__device__ __forceinline__ void fill_plane(const CUtensorMap* map, uint32_t s_rows, uint64_t* bar, int slot,
                                           int x, int y0, int z0) {
  expect_bytes(bar, kPlaneBytes);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const uint32_t dst = s_rows + (uint32_t)c * kChunkBytes + (uint32_t)(kPadLo + slot * kSlotRows) * 16u;
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(z0), "r"(y0), "r"(x), "r"(c), "r"(tc::smem_addr(bar))
        : "memory");
  }
}

// The tiles of one CTA, by segment: a segment is a run of plane steps within one column.
struct Segment {
  int p0;                 // first plane step
  int xs, nq, y0, z0;     // first x, plane steps, column origin
  uint32_t first, ntile;  // CTA tile index of the first tile, tiles
};

__device__ __forceinline__ Segment segment_at(int p0, int w1, uint32_t first, const LbmGeom& g, const RowGeom& rg) {
  Segment s;
  s.p0 = p0;
  const int col = p0 / g.nx;
  s.xs = p0 - col * g.nx;
  s.nq = min(g.nx - s.xs, w1 - p0);
  const int yb = col / rg.nzb, zb = col - yb * rg.nzb;
  s.y0 = yb * kLines;
  s.z0 = zb * kLineCells;
  s.first = first;
  s.ntile = (uint32_t)(kPlaneTiles * s.nq);
  return s;
}

// Moves s forward to the segment holding CTA tile t.
__device__ __forceinline__ void seek(Segment& s, uint32_t t, int w1, const LbmGeom& g, const RowGeom& rg) {
  while (t >= s.first + s.ntile) s = segment_at(s.p0 + s.nq, w1, s.first + s.ntile, g, rg);
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;}"
      : "=r"(done)
      : "r"(tc::smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Chain-issuer state of one epilogue group: its next tile, the epilogue of that tile it
// waits for (0-2), phases of its hand-over barrier waited and commits to its layer barrier.
struct Group {
  uint32_t tile, stage = 0, n_h = 0, c_l = 0;
  Segment seg;
};

struct ChainCtx {
  const CUtensorMap* map;
  uint32_t s_rows;
  uint64_t* bar_rows;
  uint32_t tmem;
  uint64_t w2, w3, w4;
  int w1;
  uint32_t ntiles;
};

// The first planes of segment s (ordinal u = plane xs - 1 + u, slot u & 3).
__device__ __forceinline__ void fill_segment_start(const CUtensorMap* map, uint32_t s_rows, uint64_t* bar_rows,
                                                   uint32_t& fills, const Segment& s, int nx) {
  for (int u = 0; u < 3; ++u) {
    fill_plane(map, s_rows, &bar_rows[u], u, wrap(s.xs - 1 + u, nx), s.y0, s.z0);
    fills ^= 1u << u;
  }
  if (s.nq > 1) {
    fill_plane(map, s_rows, &bar_rows[3], 3, wrap(s.xs + 2, nx), s.y0, s.z0);
    fills ^= 1u << 3;
  }
}

// If group H has handed over its next epilogue, issues the layer that follows it (and, after
// a layer-1 epilogue, the plane copies that tile frees); returns whether it did.
template <int H>
__device__ __forceinline__ bool serve(Group& gr, uint64_t& bar_h, uint64_t& bar_l, uint64_t dh, const ChainCtx& cx,
                                      uint32_t& fills, const LbmGeom& g, const RowGeom& rg) {
  if (gr.tile >= cx.ntiles || !mbar_test(&bar_h, gr.n_h & 1)) return false;
  ++gr.n_h;
  tc::fence_after_sync();
  const uint32_t tb = cx.tmem + ((uint32_t)H << 8);
  if (gr.stage == 0) {  // layer-1 epilogue done: layer 2, plane copies
    issue_layer(tb + 64, dh, cx.w2, kIdesc64);
    tc::mma_commit(&bar_l);
    ++gr.c_l;
    seek(gr.seg, gr.tile, cx.w1, g, rg);
    const Segment& s = gr.seg;
    const int ti = (int)(gr.tile - s.first), q = ti / kPlaneTiles, m = ti - q * kPlaneTiles;
    // Layer 1 of this tile is complete, so is every earlier one: plane step q - 1's oldest
    // plane gives its slot to plane xs + q + 2; after a segment's last tile, the next
    // segment's first planes go in.
    if (m == 0 && q >= 1 && q + 1 < s.nq) {
      const int sl = (q + 3) & 3;
      fill_plane(cx.map, cx.s_rows, &cx.bar_rows[sl], sl, wrap(s.xs + q + 2, g.nx), s.y0, s.z0);
      fills ^= 1u << sl;
    }
    if ((uint32_t)ti + 1 == s.ntile && s.p0 + s.nq < cx.w1)
      fill_segment_start(cx.map, cx.s_rows, cx.bar_rows, fills, segment_at(s.p0 + s.nq, cx.w1, s.first + s.ntile, g, rg),
                         g.nx);
    gr.stage = 1;
  } else if (gr.stage == 1) {
    issue_layer(tb + 128, dh, cx.w3, kIdesc64);
    tc::mma_commit(&bar_l);
    ++gr.c_l;
    gr.stage = 2;
  } else {
    issue_layer(tb + 192, dh, cx.w4, kIdesc32);
    tc::mma_commit(&bar_l);
    ++gr.c_l;
    gr.stage = 0;
    gr.tile += 2;
  }
  return true;
}

// kApply = false: corrections to a.corr. kApply = true: each cell's mass-conserving correction
// f_q += c_q - w_q sum_p c_p added to its populations in place (the arithmetic of
// closure_apply_kernel); the kernel reads only the staged rows, never the populations, so
// no other cell's inputs change.
template <bool kApply>
__global__ void __launch_bounds__(kInferThreads, 1) closure_infer_kernel(InferArgs a,
                                                                        const __grid_constant__ CUtensorMap rows_map) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ float sb[64 * 3 + kOutPad];
  // Per epilogue group / TMEM half h: bar_l1[h] layer 1 done, bar_e1[h] its accumulator read,
  // bar_h[h] an epilogue handed over, bar_l[h] a layer 2-4 done.
  __shared__ __align__(8) uint64_t bar_l1[2], bar_e1[2], bar_h[2], bar_l[2], bar_rows[kSlots];
  __shared__ uint32_t tbase;
  __shared__ int abort_flag;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  stage_w1(smem + kOffW1, a.w1);
  stage_weights(smem + kOffW2, a.w2, 64, 64);
  stage_weights(smem + kOffW3, a.w3, 64, 64);
  stage_weights(smem + kOffW4, a.w4, kOutPad, 64);
  for (int i = t; i < 64 * 3 + kOutPad; i += kInferThreads) sb[i] = a.b[i];
  // Rows no copy writes (padding) stay zero: they feed discarded rows only, but must be finite.
  constexpr int kGap = kSlotRows - kPlaneRows;
  for (int i = t; i < 3 * (kPadLo + kPadHi + kSlots * kGap); i += kInferThreads) {
    const int c = i / (kPadLo + kPadHi + kSlots * kGap), p = i % (kPadLo + kPadHi + kSlots * kGap);
    int row;
    if (p < kPadLo) row = p;
    else if (p < kPadLo + kPadHi) row = kPadLo + kSlots * kSlotRows + (p - kPadLo);
    else row = kPadLo + ((p - kPadLo - kPadHi) / kGap) * kSlotRows + kPlaneRows + (p - kPadLo - kPadHi) % kGap;
    *reinterpret_cast<uint4*>(smem + kOffRows + (size_t)c * kChunkBytes + (size_t)row * 16) =
        make_uint4(0, 0, 0, 0);
  }
  if (warp == 0) tc::tmem_alloc(&tbase, 512);
  if (t == 0) {
    for (int h = 0; h < 2; ++h) {
      tc::mbar_init(&bar_l1[h], 1);
      tc::mbar_init(&bar_e1[h], kGroupWarps);
      tc::mbar_init(&bar_h[h], kGroupWarps);
      tc::mbar_init(&bar_l[h], 1);
    }
    for (int s = 0; s < kSlots; ++s) tc::mbar_init(&bar_rows[s], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_smem_for_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tbase;
  volatile int* abort = &abort_flag;
  const LbmGeom& g = a.f.g;
  const RowGeom& rg = a.rg;
  // This CTA's plane steps [w0, w1) (the host keeps the count below 2^31 / 3).
  const int w0 = (int)((long long)a.work * blockIdx.x / gridDim.x);
  const int w1 = (int)((long long)a.work * (blockIdx.x + 1) / gridDim.x);
  const uint32_t ntiles = (uint32_t)(kPlaneTiles * (w1 - w0));

  const uint32_t sRows = tc::smem_addr(smem + kOffRows);
  if (warp == kChainWarp) {
    // ------------------------------------------------ plane copies, layers 2-4
    if (lane == 0) {
      const uint64_t dH0 = tc::tile_desc(tc::smem_addr(smem + kOffH), 64, 0);
      const uint64_t dH1 = tc::tile_desc(tc::smem_addr(smem + kOffH + kHBytes), 64, 0);
      const uint64_t dW2 = tc::tile_desc(tc::smem_addr(smem + kOffW2), 64, 0);
      const uint64_t dW3 = tc::tile_desc(tc::smem_addr(smem + kOffW3), 64, 0);
      const uint64_t dW4 = tc::tile_desc(tc::smem_addr(smem + kOffW4), 64, 0);
      uint32_t fills = 0;  // parity of the copies issued per slot
      bool ok = true;
      Group gr0, gr1;
      gr0.tile = 0;
      gr1.tile = 1;
      if (ntiles > 0) {
        // The first segment's planes: ordinal u is plane xs - 1 + u, in slot u & 3.
        const Segment s0 = segment_at(w0, w1, 0, g, rg);
        fill_segment_start(&rows_map, sRows, bar_rows, fills, s0, g.nx);
        gr0.seg = s0;
        gr1.seg = s0;
      }
      const ChainCtx cx{&rows_map, sRows, bar_rows, tmem, dW2, dW3, dW4, w1, ntiles};
      long long t_idle = clock64();
      // Serve the two epilogue groups in the order their hand-overs arrive.
      while (gr0.tile < ntiles || gr1.tile < ntiles) {
        const bool p0 = serve<0>(gr0, bar_h[0], bar_l[0], dH0, cx, fills, g, rg);
        const bool p1 = serve<1>(gr1, bar_h[1], bar_l[1], dH1, cx, fills, g, rg);
        if (p0 || p1) {
          t_idle = clock64();
        } else if (*abort) {
          ok = false;
          break;
        } else if (clock64() - t_idle > tc::kWaitCycles) {
          *abort = 1;
          atomicExch(a.err, 9);
          ok = false;
          break;
        } else {
          __nanosleep(20);
        }
      }
      if (!ok) {
        // Let the copies and MMAs this thread issued finish before the CTA exits (bounded).
        for (int sl = 0; sl < kSlots; ++sl) tc::mbar_wait(&bar_rows[sl], ((fills >> sl) & 1u) ^ 1u, nullptr, 0);
        if (gr0.c_l > 0) tc::mbar_wait(&bar_l[0], (gr0.c_l - 1) & 1, nullptr, 0);
        if (gr1.c_l > 0) tc::mbar_wait(&bar_l[1], (gr1.c_l - 1) & 1, nullptr, 0);
      }
    }
  } else if (warp == kL1Warp) {
    // ------------------------------------------------------------------ layer 1
    if (lane == 0) {
      const uint64_t dRows = tc::smem_desc(sRows, 0u, 128u);
      const uint64_t dW1 = tc::smem_desc(tc::smem_addr(smem + kOffW1), 128u, 256u);
      uint32_t tile = 0, rows_phase = 0, issued = 0;
      bool ok = true;
#define FSI_WAIT_ROWS(sl) (ok = tc::mbar_wait_abortable(&bar_rows[(sl)], (rows_phase >> (sl)) & 1u, abort, a.err, 12), rows_phase ^= 1u << (sl), ok)
      for (int p0 = w0; p0 < w1 && ok;) {
        const int nq = min(g.nx - p0 % g.nx, w1 - p0);
        const int ntile = kPlaneTiles * nq;
        for (int ti = 0; ti < ntile; ++ti, ++tile) {
          const int q = ti / kPlaneTiles, m = ti - q * kPlaneTiles;
          const uint32_t h = tile & 1;
          // The TMEM half's previous tile (tile - 2) has been read by its layer-1 epilogue.
          if (tile >= 2 && !(ok = tc::mbar_wait_abortable(&bar_e1[h], ((tile - 2) >> 1) & 1u, abort, a.err, 14))) break;
          // The planes of this plane step are loaded.
          if (ti == 0) {
            if (!FSI_WAIT_ROWS(0) || !FSI_WAIT_ROWS(1) || !FSI_WAIT_ROWS(2)) break;
          } else if (m == 0 && !FSI_WAIT_ROWS((q + 2) & 3)) {
            break;
          }
          tc::fence_after_sync();
          const int base = kPadLo + kLine + 128 * m;
          const int r0 = base + (q & 3) * kSlotRows, r1 = base + ((q + 1) & 3) * kSlotRows,
                    r2 = base + ((q + 2) & 3) * kSlotRows;
          const uint32_t d = tmem + (h << 8);
          issue_l1_chunk<0>(d, dRows, r0, r1, r2, dW1);
          issue_l1_chunk<1>(d, dRows, r0, r1, r2, dW1);
          issue_l1_chunk<2>(d, dRows, r0, r1, r2, dW1);
          tc::mma_commit(&bar_l1[h]);
          ++issued;
        }
        p0 += nq;
      }
      if (!ok && issued > 0) {
        // Let the last layer 1 issued (tile issued - 1; tiles go in order) finish (bounded).
        const uint32_t lt = issued - 1;
        tc::mbar_wait(&bar_l1[lt & 1], (lt >> 1) & 1u, nullptr, 0);
      }
#undef FSI_WAIT_ROWS
    }
  } else {
    // ------------------------------------------------------------------ epilogues
    // Group h = warp / 8 takes the tiles of parity h (TMEM half h, its own H tile); within
    // a group, warp w reads TMEM lanes 32 (w % 4) .. + 31 and columns 32 cb .. + 31,
    // cb = (w % 8) / 4.
    const int h = warp / kGroupWarps, cb = (warp % kGroupWarps) >> 2;
    const int lrow = 32 * (warp & 3) + lane;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    unsigned char* H = smem + kOffH + h * kHBytes;
    const float inv_out = 1.0f / a.out_scale;
    uint32_t n_l1 = 0, n_l = 0;
    bool ok = true;
    // Warp-uniform bounded wait (every lane takes the same branch afterwards), and the hand-over
    // of this warp's H rows (and TMEM reads) to the issuer.
#define FSI_WWAIT(bar, parity, code) (__all_sync(0xffffffffu, tc::mbar_wait_abortable((bar), (parity), abort, a.err, (code))) != 0)
#define FSI_HAND_OVER()                              \
  do {                                                \
    tc::fence_smem_for_async();                       \
    tc::fence_before_sync();                          \
    __syncwarp();                                     \
    if (lane == 0) tc::mbar_arrive(&bar_h[h]);        \
  } while (0)
    Segment s = segment_at(w0, w1, 0, g, rg);
    for (uint32_t tt = (uint32_t)h; tt < ntiles && ok; tt += 2) {
      seek(s, tt, w1, g, rg);
      const int ti = (int)(tt - s.first), q = ti / kPlaneTiles, m = ti - q * kPlaneTiles;
      // This thread's output cell (if its row is one) and its occupancy, fetched early.
      const int pr = kLine + 128 * m + lrow;
      const int hy = pr / kLine, hz = pr - hy * kLine;
      const int oy = s.y0 + hy - 1, oz = s.z0 + hz - 1;
      const bool valid = (kApply ? cb == 0 : true) && hy <= kLines && hz >= 1 && hz <= kLineCells &&
                         oy < g.ny && oz < g.nz;
      const long long cc = ((long long)(s.xs + q) * g.ny + oy) * g.nz + oz;
      const uint32_t fl = valid ? a.f.flags[cc] : kFlagSolid;
      // In place: the cell's 19 populations, loaded now so the output epilogue only adds.
      float fq[kApply ? kOut : 1];
      if (kApply && valid) {
        const Deltas dc(g, s.xs + q, oy, oz);
#pragma unroll
        for (int qo = 0; qo < kOut; ++qo) fq[qo] = a.pops[slot32((uint32_t)g.n, dc, fl, qo, a.f.parity)];
      }
      const uint32_t tb = tmem + ((uint32_t)h << 8) + lane_base;
      if (!(ok = FSI_WWAIT(&bar_l1[h], n_l1 & 1u, 3))) break;
      ++n_l1;
      tc::fence_after_sync();
      hidden_epilogue(tb, sb, 2 * cb, H, lrow);
      hidden_epilogue(tb, sb, 2 * cb + 1, H, lrow);
      FSI_HAND_OVER();
      if (lane == 0) tc::mbar_arrive(&bar_e1[h]);  // this half's layer-1 accumulator is free
      if (!(ok = FSI_WWAIT(&bar_l[h], n_l & 1, 4))) break;
      ++n_l;
      tc::fence_after_sync();
      hidden_epilogue(tb + 64, sb + 64, 2 * cb, H, lrow);
      hidden_epilogue(tb + 64, sb + 64, 2 * cb + 1, H, lrow);
      FSI_HAND_OVER();
      if (!(ok = FSI_WWAIT(&bar_l[h], n_l & 1, 5))) break;
      ++n_l;
      tc::fence_after_sync();
      hidden_epilogue(tb + 128, sb + 128, 2 * cb, H, lrow);
      hidden_epilogue(tb + 128, sb + 128, 2 * cb + 1, H, lrow);
      FSI_HAND_OVER();
      if (!(ok = FSI_WWAIT(&bar_l[h], n_l & 1, 6))) break;
      ++n_l;
      tc::fence_after_sync();
      // Outputs: columns 0-31, 19 used. Corrections: 16 per warp (cb); in place: the warps
      // with cb == 0 take all 32 columns of their rows.
      if (!kApply) {
        float y[16];
        tc::tmem_ld16(tb + 192 + 16 * cb, y);
        if (valid) {
          const float keep = (fl & kFlagSolid) ? 0.f : inv_out;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int qo = 16 * cb + i;
            if (qo < kOut) a.corr[(size_t)qo * g.n + cc] = (y[i] + sb[192 + qo]) * keep;
          }
        }
      } else if (cb == 0) {
        float y[32];
        tc::tmem_ld16(tb + 192, *reinterpret_cast<float(*)[16]>(y));
        tc::tmem_ld16(tb + 208, *reinterpret_cast<float(*)[16]>(y + 16));
        if (valid && !(fl & kFlagSolid)) {
          float cq[kOut], sum = 0.f;
#pragma unroll
          for (int qo = 0; qo < kOut; ++qo) {
            cq[qo] = (y[qo] + sb[192 + qo]) * inv_out;
            sum += cq[qo];
          }
          const Deltas dc(g, s.xs + q, oy, oz);
#pragma unroll
          for (int qo = 0; qo < kOut; ++qo)
            a.pops[slot32((uint32_t)g.n, dc, fl, qo, a.f.parity)] = fq[qo] + (cq[qo] - weight_of(qo) * sum);
        }
      }
    }
#undef FSI_WWAIT
#undef FSI_HAND_OVER
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
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
                   const float* force, const float* frac, int64_t steps_done, float pop_scale,
                   float force_scale) {
  FeatArgs f;
  f.frac = frac;
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
                                    const float* force, const float* solid_fraction, int64_t steps_done,
                                    const int32_t* cells,
                                    int32_t m, float pop_scale, float force_scale, void* x,
                                    void* stream) {
  if (int e = check_closure_lattice(d)) return e;
  FSI_REQUIRE(pops && flags && force && cells && x && m > 0, "NULL array or empty cell list");
  const FeatArgs f = feat_args(d, pops, flags, force, solid_fraction, steps_done, pop_scale, force_scale);
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

extern "C" int64_t fsi_closure_rows_bytes(const fsi_lbm_desc* d) {
  if (check_closure_lattice(d)) return -1;
  return 3 * row_geom(geom_of(d)).chunk_rows * 16;
}

namespace fsi {
namespace {

// The row pass, then the fused inference (corrections to corr, or applied to pops_out).
template <bool kApply>
int launch_infer(const fsi_lbm_desc* d, const float* pops, const uint32_t* flags, const float* force,
                 const float* frac, int64_t steps_done, const fsi_closure_weights* w, void* rows, float* corr, float* pops_out,
                 int32_t* err, void* stream) {
  if (int e = check_closure_lattice(d)) return e;
  FSI_REQUIRE(pops && flags && force && w && rows && err && (kApply || corr), "NULL array");
  FSI_REQUIRE(((uintptr_t)rows & 15) == 0, "rows must be 16-byte aligned");
  FSI_REQUIRE(w->w1 && w->w2 && w->w3 && w->w4 && w->bias, "NULL weights");
  FSI_REQUIRE(w->out_scale != 0.f, "out_scale must be non-zero");
  InferArgs a;
  a.f = feat_args(d, pops, flags, force, frac, steps_done, w->pop_scale, w->force_scale);
  a.rg = row_geom(a.f.g);
  a.grows = reinterpret_cast<const unsigned char*>(rows);
  a.w1 = reinterpret_cast<const __nv_bfloat16*>(w->w1);
  a.w2 = reinterpret_cast<const __nv_bfloat16*>(w->w2);
  a.w3 = reinterpret_cast<const __nv_bfloat16*>(w->w3);
  a.w4 = reinterpret_cast<const __nv_bfloat16*>(w->w4);
  a.b = w->bias;
  a.out_scale = w->out_scale;
  a.corr = corr;
  a.pops = pops_out;
  a.err = err;
  a.work = (long long)a.rg.nyb * a.rg.nzb * a.f.g.nx;
  FSI_REQUIRE(a.work < (1ll << 31) / kPlaneTiles, "lattice too large for the closure inference");
  cudaStream_t s = as_stream(stream);
  FSI_REQUIRE(a.rg.ny_pad <= 65535 && a.f.g.nx <= 65535, "lattice too large for the row pass");
  closure_rows_kernel<<<dim3((a.rg.nz_pad + 127) / 128, a.rg.ny_pad, a.f.g.nx), 128, 0, s>>>(
      a.f, a.rg, reinterpret_cast<unsigned char*>(rows));
  if (int e = check_launch("closure_rows_kernel")) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)(a.work < sms ? a.work : sms);
  // Tensor map of the padded rows: dims (8 channels, nz_pad, ny_pad, nx, 3 chunks).
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", reinterpret_cast<void**>(&encode),
                                                           12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !encode) {
      encode = nullptr;
      set_error("cuTensorMapEncodeTiled unavailable (%s)", cudaGetErrorString(e));
      return FSI_ERR_CUDA;
    }
  }
  CUtensorMap map;
  const cuuint64_t dims[5] = {8, (cuuint64_t)a.rg.nz_pad, (cuuint64_t)a.rg.ny_pad, (cuuint64_t)a.f.g.nx, 3};
  const cuuint64_t strides[4] = {16, (cuuint64_t)a.rg.nz_pad * 16, (cuuint64_t)a.rg.ny_pad * a.rg.nz_pad * 16,
                                 (cuuint64_t)a.rg.chunk_rows * 16};
  const cuuint32_t box[5] = {8, kLine, kLines + 2, 1, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult cr = encode(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, rows, dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FSI_REQUIRE(cr == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d)", (int)cr);
  cudaFuncSetAttribute(closure_infer_kernel<kApply>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kInferSmem);
  closure_infer_kernel<kApply><<<grid, kInferThreads, kInferSmem, s>>>(a, map);
  return check_launch("closure_infer_kernel");
}


}  // namespace
}  // namespace fsi

extern "C" int fsi_closure_infer(const fsi_lbm_desc* d, const float* pops, const uint32_t* flags,
                                 const float* force, const float* solid_fraction, int64_t steps_done,
                                 const fsi_closure_weights* w, void* rows, float* corr, int32_t* err,
                                 void* stream) {
  return launch_infer<false>(d, pops, flags, force, solid_fraction, steps_done, w, rows, corr, nullptr, err,
                             stream);
}

extern "C" int fsi_closure_infer_apply(const fsi_lbm_desc* d, float* pops, const uint32_t* flags,
                                       const float* force, const float* solid_fraction, int64_t steps_done,
                                       const fsi_closure_weights* w, void* rows, int32_t* err,
                                       void* stream) {
  return launch_infer<true>(d, pops, flags, force, solid_fraction, steps_done, w, rows, nullptr, pops, err,
                            stream);
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

namespace fsi {
namespace {

// Self-test of the bounded waits (no reference counterpart): one CTA, two roles, one mbarrier
// that nothing arrives on. Role A (thread 0) waits with tc::mbar_wait: after tc::kWaitCycles it
// records kWaitSelfTestCode and raises the abort flag. Role B (thread 32) first sleeps for
// kWaitSelfTestDelay cycles, so that its own limit falls well after A's, then waits with
// tc::mbar_wait_abortable and returns on A's abort without recording its code. Both loops
// end by the clock whatever happens.
constexpr int kWaitSelfTestCode = 7;
constexpr long long kWaitSelfTestDelay = 1ll << 29;  // a quarter of the wait limit

__global__ void wait_limit_selftest_kernel(int* __restrict__ err, int* __restrict__ out) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
  }
  __syncthreads();
  volatile int* abort = &abort_flag;
  if (threadIdx.x == 0) {
    const bool ok = tc::mbar_wait(&bar, 0, err, kWaitSelfTestCode);
    if (!ok) *abort = 1;
    out[0] = ok ? 1 : 0;
  } else if (threadIdx.x == 32) {
    const long long t0 = clock64();
    while (clock64() - t0 < kWaitSelfTestDelay) __nanosleep(100000);
    const bool ok = tc::mbar_wait_abortable(&bar, 0, abort, err, kWaitSelfTestCode + 1);
    out[1] = ok ? 1 : 0;
  }
}

}  // namespace
}  // namespace fsi

extern "C" int fsi_selftest_wait_limit(int32_t* err, int32_t* out, void* stream) {
  FSI_REQUIRE(err && out, "NULL array");
  wait_limit_selftest_kernel<<<1, 64, 0, as_stream(stream)>>>(err, out);
  return check_launch("wait_limit_selftest_kernel");
}
