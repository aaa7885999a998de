// MLS-MPM / APIC substep on sm_103a (reference: fsi/mpm3d.py:189-328).
//
// A substep is three launches on a grid buffer of float4 nodes (momentum xyz,
// mass) that is all-zero on entry and left all-zero on exit:
//   1. p2g:   one thread per particle. Deformation update, fixed-corotated
//             stress (polar rotation by Newton iteration), then the 27-node
//             quadratic B-spline scatter, unrolled with the per-axis weights and
//             offsets formed once. A CTA first bounds its particles' stencils; if
//             the box fits in shared memory the scatter goes to a shared tile (odd
//             lanes walk the stencil backwards, so the two particles of a sub-cell
//             pair add into different nodes) and the tile is flushed with one
//             vector reduction per touched node. Otherwise each particle reduces
//             straight into global memory. Touched 4^3 node blocks are marked dirty.
//             The coupled substep forms each particle's penalty force in the same
//             pass on small launches, or in a separate kernel before it.
//   2. g2p:   grid update (p/m + dt g, sticky/damped walls) fused into the
//             gather: a CTA stages the grid-updated velocities of its stencil box
//             in shared memory, then each particle gathers v and the APIC C,
//             advects and clamps.
//   3. clear: zeroes the dirty blocks, restoring the all-zero grid.
// Arithmetic follows the reference's float32 operation order (no contraction).
#include <cuda_runtime.h>

#include <cstdint>

#include "fsi_common.cuh"
#include "mpm_core.cuh"

namespace fsi {
namespace {

// P2G and G2P are capped at 64 registers (4 CTAs, 32 warps per SM, against 3 CTAs at their
// natural 75-80): the extra resident warps hide more of the tile-atomic and gather latency
// (measured: 2,097,152-particle substep 0.475 -> 0.450 ms with P2G capped, 0.454 ms with G2P
// capped; no spills in P2G, 8 bytes in G2P).
// Threads per block kT (m.threads): 128, 256 or 512, each at the same 64-register cap.
template <int kT>
__global__ void __launch_bounds__(kT, 1024 / kT) p2g_kernel(Mpm m, PView P,
                                                            float4* __restrict__ grid,
                                                            uint8_t* __restrict__ dirty) {
  p2g_body(m, P, grid, dirty, blockIdx.x * kT + threadIdx.x);
}

// The penalty coupling alone (one thread per particle), before p2g_kernel on large launches.
__global__ void __launch_bounds__(kBlock) coupling_only_kernel(ForceArgs fa) {
  coupling_forces_body<false>(fa, blockIdx.x * kBlock + threadIdx.x);
}

// The coupling split in two lighter kernels: the force (gathers), then the spread (vector
// reductions), each at its own register count (coupling_fold 3).
#ifndef FSI_GATHER_MIN_BLOCKS
#define FSI_GATHER_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(kBlock, FSI_GATHER_MIN_BLOCKS) coupling_gather_kernel(ForceArgs fa) {
  coupling_gather_body(fa, blockIdx.x * kBlock + threadIdx.x);
}
__global__ void __launch_bounds__(kBlock) coupling_spread_kernel(ForceArgs fa) {
  coupling_spread_body(fa, blockIdx.x * kBlock + threadIdx.x);
}

// P2G with the penalty coupling folded in (one thread per particle).
template <int kT>
__global__ void __launch_bounds__(kT) coupled_p2g_kernel(Mpm m, PView P, float4* __restrict__ grid,
                                                         uint8_t* __restrict__ dirty, ForceArgs fa) {
  p2g_body<true>(m, P, grid, dirty, blockIdx.x * kT + threadIdx.x, &fa);
}

template <int kT>
__global__ void __launch_bounds__(kT, 1024 / kT) g2p_kernel(Mpm m, PView P,
                                                            const float4* __restrict__ grid) {
  g2p_body(m, P, grid, blockIdx.x * kT + threadIdx.x);
}

// Launches K<m.threads> over the particles.
template <template <int> class K, class... Args>
int launch_tiled(const Mpm& m, cudaStream_t s, const char* what, Args... args) {
  switch (m.threads) {
    case 128: K<128>::run(grid_for(m.n, 128), s, args...); break;
    case 512: K<512>::run(grid_for(m.n, 512), s, args...); break;
    default: K<256>::run(grid_for(m.n, 256), s, args...); break;
  }
  return check_launch(what);
}
template <int kT>
struct P2G {
  static void run(unsigned g, cudaStream_t s, Mpm m, PView P, float4* grid, uint8_t* dirty) {
    p2g_kernel<kT><<<g, kT, 0, s>>>(m, P, grid, dirty);
  }
};
template <int kT>
struct CoupledP2G {
  static void run(unsigned g, cudaStream_t s, Mpm m, PView P, float4* grid, uint8_t* dirty,
                  ForceArgs fa) {
    coupled_p2g_kernel<kT><<<g, kT, 0, s>>>(m, P, grid, dirty, fa);
  }
};
template <int kT>
struct G2P {
  static void run(unsigned g, cudaStream_t s, Mpm m, PView P, const float4* grid) {
    g2p_kernel<kT><<<g, kT, 0, s>>>(m, P, grid);
  }
};

__global__ void __launch_bounds__(kBlock) clear_kernel(Mpm m, float4* __restrict__ grid,
                                                       uint8_t* __restrict__ dirty) {
  clear_body(m, grid, dirty, ((long long)blockIdx.x * kBlock + threadIdx.x) >> 5);
}

// Zeroes the dirty 4^3 node blocks: each warp reads the flags of 32 consecutive blocks with
// one load, then zeroes the dirty ones together (two nodes per lane) and resets their flags.
// Launches one warp per 32 blocks instead of one per block.
__global__ void __launch_bounds__(kBlock) clear_dirty_kernel(Mpm m, float4* __restrict__ grid,
                                                             uint8_t* __restrict__ dirty) {
  const long long nblocks = (long long)m.nbx * m.nby * m.nbz;
  const int lane = threadIdx.x & 31;
  const long long b0 = (((long long)blockIdx.x * kBlock + threadIdx.x) >> 5) << 5;
  const long long mine = b0 + lane;
  const bool d = mine < nblocks && dirty[mine] != 0;
  unsigned todo = __ballot_sync(0xffffffffu, d);
  while (todo) {
    const int l = __ffs(todo) - 1;
    todo &= todo - 1;
    const long long b = b0 + l;
    const int bi = (int)(b / ((long long)m.nby * m.nbz));
    const int bj = (int)((b / m.nbz) % m.nby);
    const int bk = (int)(b % m.nbz);
#pragma unroll
    for (int t = lane; t < 64; t += 32) {
      const int i = bi * 4 + (t >> 4), j = bj * 4 + ((t >> 2) & 3), k = bk * 4 + (t & 3);
      if (i < m.nx && j < m.ny && k < m.nz) grid[node_index(m, i, j, k)] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  if (d) dirty[mine] = 0;
}

__global__ void polar_kernel(const float* __restrict__ F, float* __restrict__ R, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float f[9], r[9];
#pragma unroll
  for (int a = 0; a < 9; ++a) f[a] = F[9 * i + a];
  polar_rotation(f, r);
#pragma unroll
  for (int a = 0; a < 9; ++a) R[9 * i + a] = r[a];
}

__global__ void base_cells_kernel(Mpm m, PView P, int32_t* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m.n) return;
  float x[3];
  load_particle_x(P, m.cap, p, x);
  int base[3];
  float fx[3];
  base_fx(m, x, base, fx);
  out[3 * p] = base[0]; out[3 * p + 1] = base[1]; out[3 * p + 2] = base[2];
}

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Particle diagnostics: [0] sum m, [1..3] sum m x, [4] max |v|, [5..7] sum f_p.
__global__ void __launch_bounds__(kBlock) particle_reduce_kernel(Mpm m, PView P,
                                                                 double* __restrict__ out) {
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  float vmax = 0.f;
  const long long cap = m.cap;
  for (int p = blockIdx.x * kBlock + threadIdx.x; p < m.n; p += gridDim.x * kBlock) {
    const double ms = P.mass[p];
    acc[0] += ms;
    for (int a = 0; a < 3; ++a) acc[1 + a] += ms * (double)P.x[a * cap + p];
    const float vx = P.v[p], vy = P.v[cap + p], vz = P.v[2 * cap + p];
    vmax = fmaxf(vmax, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)),
                                            __fmul_rn(vz, vz))));
    for (int a = 0; a < 3; ++a) acc[4 + a] += (double)P.fp[a * cap + p];
  }
  __shared__ double sh[7][kBlock / 32];
  __shared__ float shm[kBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = 0; i < 7; ++i) acc[i] = wsum(acc[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
  if (lane == 0) { for (int i = 0; i < 7; ++i) sh[i][wid] = acc[i]; shm[wid] = vmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    float mx = 0.f;
    for (int w = 0; w < kBlock / 32; ++w) {
      for (int i = 0; i < 7; ++i) s[i] += sh[i][w];
      mx = fmaxf(mx, shm[w]);
    }
    for (int i = 0; i < 4; ++i) atomicAdd(out + i, s[i]);
    atomicMax(reinterpret_cast<unsigned long long*>(out + 4),
              (unsigned long long)__double_as_longlong((double)mx));
    for (int i = 0; i < 3; ++i) atomicAdd(out + 5 + i, s[4 + i]);
  }
}


}  // namespace
}  // namespace fsi

using namespace fsi;

extern "C" int fsi_mpm_substep(const fsi_mpm_desc* d, const fsi_particles* parts, float* grid,
                               uint8_t* dirty, void* stream) {
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  FSI_REQUIRE(grid && dirty, "NULL grid or dirty map");
  FSI_REQUIRE(((uintptr_t)grid & 15) == 0, "grid must be 16-byte aligned");
  if (m.n == 0) return FSI_OK;
  cudaStream_t s = as_stream(stream);
  float4* g4 = reinterpret_cast<float4*>(grid);
  if (int e = launch_tiled<P2G>(m, s, "p2g_kernel", m, P, g4, dirty)) return e;
  if (int e = launch_tiled<G2P>(m, s, "g2p_kernel", m, P, (const float4*)g4)) return e;
  const long long nblocks = (long long)m.nbx * m.nby * m.nbz;
  clear_dirty_kernel<<<grid_for(nblocks, kBlock), kBlock, 0, s>>>(m, g4, dirty);
  return check_launch("clear_dirty_kernel");
}

extern "C" int fsi_mpm_polar(const float* F, float* R, int64_t n, void* stream) {
  FSI_REQUIRE(F && R && n >= 0, "bad arguments");
  if (n == 0) return FSI_OK;
  polar_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(F, R, n);
  return check_launch("polar_kernel");
}

extern "C" int fsi_mpm_base_cells(const fsi_mpm_desc* d, const fsi_particles* parts, int32_t* out,
                                  void* stream) {
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  FSI_REQUIRE(out, "NULL output");
  if (m.n == 0) return FSI_OK;
  base_cells_kernel<<<grid_for(m.n, 128), 128, 0, as_stream(stream)>>>(m, P, out);
  return check_launch("base_cells_kernel");
}

extern "C" int fsi_mpm_reduce(const fsi_mpm_desc* d, const fsi_particles* parts, double* out,
                              void* reserved, void* stream) {
  (void)reserved;
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  FSI_REQUIRE(out, "NULL output");
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out, 0, 8 * sizeof(double), s) != cudaSuccess) return check_launch("memset");
  if (m.n == 0) return FSI_OK;
  int blocks = (int)grid_for(m.n, kBlock);
  if (blocks > 152 * 4) blocks = 152 * 4;
  particle_reduce_kernel<<<blocks, kBlock, 0, s>>>(m, P, out);
  return check_launch("particle_reduce_kernel");
}

// ----------------------------------------------------------------------------
// Substep for callers that cannot allocate device memory.
//
// Some hosts of this library may not call cudaMalloc: a real-time loop in which
// the implicit device synchronisation of an allocation is not allowed, a plugin
// inside an application that owns the device memory pool, or a plain FFI caller
// with no device allocator of its own. For them the grid and the dirty-block map
// of fsi_mpm_substep live in one library-owned array of static device memory,
// sized for grids of at most FSI_NOALLOC_MAX_NODES nodes. Every GPU that loads
// the library holds this array (about 4 MB) until the process exits.
// ----------------------------------------------------------------------------
#include <mutex>

namespace fsi {
namespace {

constexpr long long kNoAllocGridBytes = (long long)FSI_NOALLOC_MAX_NODES * 16;
constexpr long long kNoAllocBytes = kNoAllocGridBytes + FSI_NOALLOC_MAX_BLOCKS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxContexts = 64;
std::mutex g_noalloc_mutex;
// Cache of the array's device address per CUDA context (identified by its driver-assigned
// context ID, which is never reused: a context re-created after cudaDeviceReset, or another
// context of the same device made current by a driver-API host, gets its own lookup).
unsigned long long g_noalloc_ctx[kMaxContexts] = {};
void* g_noalloc_ptr[kMaxContexts] = {};
int g_noalloc_used = 0;

typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

// The driver's cuCtxGetCurrent / cuCtxGetId, reached through the runtime (the library does
// not link the driver library); NULL when unavailable.
template <class Fn>
Fn driver_fn(const char* name) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<Fn>(fn);
}

// ID of the current context (0 when it cannot be read or no context is current yet).
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
  static CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || ctx == nullptr) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != 0) return 0;
  return id + 1;  // 0 stays "unknown"
}

// Device address of the static array in the current context. Host code cannot use the
// symbol itself (it names a host-side stand-in), so the address is looked up with
// cudaGetSymbolAddress, once per context, and cached under that context's ID.
int noalloc_scratch(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("cudaGetDevice: %s", cudaGetErrorString(e));
    return FSI_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  unsigned long long id = current_context_id();
  for (int i = 0; id != 0 && i < g_noalloc_used; ++i)
    if (g_noalloc_ctx[i] == id) {
      *out = g_noalloc_ptr[i];
      return FSI_OK;
    }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the primary context current if none is
  if (e != cudaSuccess || p == nullptr) {
    set_error("cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
    return FSI_ERR_CUDA;
  }
  if (id == 0) id = current_context_id();
  if (id != 0 && g_noalloc_used < kMaxContexts) {
    g_noalloc_ctx[g_noalloc_used] = id;
    g_noalloc_ptr[g_noalloc_used] = p;
    ++g_noalloc_used;
  }
  *out = p;
  return FSI_OK;
}

}  // namespace
}  // namespace fsi

extern "C" int fsi_mpm_substep_noalloc(const fsi_mpm_desc* d, const fsi_particles* parts,
                                       void* stream) {
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  const long long nodes = (long long)m.nx * m.ny * m.nz;
  const long long nblocks = (long long)m.nbx * m.nby * m.nbz;
  FSI_REQUIRE(nodes <= FSI_NOALLOC_MAX_NODES,
              "grid %dx%dx%d has %lld nodes; fsi_mpm_substep_noalloc supports at most %d "
              "(use fsi_mpm_substep with a caller-allocated grid)",
              m.nx, m.ny, m.nz, nodes, FSI_NOALLOC_MAX_NODES);
  FSI_REQUIRE(nblocks <= FSI_NOALLOC_MAX_BLOCKS,
              "grid %dx%dx%d has %lld 4^3 node blocks; fsi_mpm_substep_noalloc supports at most %d",
              m.nx, m.ny, m.nz, nblocks, FSI_NOALLOC_MAX_BLOCKS);
  if (m.n == 0) return FSI_OK;
  void* base = nullptr;
  if (int e = noalloc_scratch(&base)) return e;
  float4* g4 = reinterpret_cast<float4*>(base);
  uint8_t* dirty = reinterpret_cast<uint8_t*>(base) + kNoAllocGridBytes;
  cudaStream_t s = as_stream(stream);
  // The array keeps whatever the previous call left; the part this call uses must start at 0.
  if (cudaMemsetAsync(g4, 0, (size_t)nodes * sizeof(float4), s) != cudaSuccess ||
      cudaMemsetAsync(dirty, 0, (size_t)nblocks, s) != cudaSuccess)
    return check_launch("no-alloc scratch clear");
  if (int e = launch_tiled<P2G>(m, s, "p2g_kernel (no-alloc)", m, P, g4, dirty)) return e;
  if (int e = launch_tiled<G2P>(m, s, "g2p_kernel (no-alloc)", m, P, (const float4*)g4)) return e;
  clear_kernel<<<grid_for(nblocks * 32, kBlock), kBlock, 0, s>>>(m, g4, dirty);
  return check_launch("clear_kernel (no-alloc)");
}

extern "C" int fsi_coupled_substep_tiled(const fsi_coupling_desc* c, const fsi_mpm_desc* d,
                                         const fsi_particles* parts, const float* macro,
                                         const uint32_t* flags, float* accum, float* valid_weight,
                                         int32_t* coupling_mask, void* counters, float* grid,
                                         uint8_t* dirty, void* stream) {
  Mpm m;
  PView P;
  if (int e = make_mpm(d, parts, m, P)) return e;
  FSI_REQUIRE(c, "NULL coupling descriptor");
  FSI_REQUIRE(macro && flags && accum && valid_weight && coupling_mask && counters && grid && dirty,
              "NULL array");
  FSI_REQUIRE(((uintptr_t)grid & 15) == 0 && ((uintptr_t)accum & 15) == 0 &&
                  ((uintptr_t)macro & 15) == 0,
              "grid, accum and macro must be 16-byte aligned");
  cudaStream_t s = as_stream(stream);
  // unsupported / partial / clipped of this substep start from zero (coupling.py:147)
  if (cudaMemsetAsync(counters, 0, 3 * sizeof(int32_t), s) != cudaSuccess) return check_launch("memset");
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
  float4* g4 = reinterpret_cast<float4*>(grid);
  // Few particles (under two CTAs per SM): launch- and latency-bound, so the coupling runs
  // inside P2G (one launch less per substep). Many particles: the coupling's 27 lattice
  // gathers and reductions run better in a separate lighter kernel than at P2G's occupancy,
  // so the coupling runs first on its own (measured on the 384x192x192 coupled step: 3.71 ms
  // separate against 3.93 ms fused). m.fold overrides the choice.
  const bool fold = m.fold == 1 || (m.fold == 0 && m.n < 2 * 152 * kBlock);
  if (fold) {
    if (int e = launch_tiled<CoupledP2G>(m, s, "coupled_p2g_kernel", m, P, g4, dirty, fa)) return e;
  } else if (m.fold == 3) {
    coupling_gather_kernel<<<grid_for(m.n, kBlock), kBlock, 0, s>>>(fa);
    if (int e = check_launch("coupling_gather_kernel")) return e;
    coupling_spread_kernel<<<grid_for(m.n, kBlock), kBlock, 0, s>>>(fa);
    if (int e = check_launch("coupling_spread_kernel")) return e;
    if (int e = launch_tiled<P2G>(m, s, "p2g_kernel", m, P, g4, dirty)) return e;
  } else {
    coupling_only_kernel<<<grid_for(m.n, kBlock), kBlock, 0, s>>>(fa);
    if (int e = check_launch("coupling_only_kernel")) return e;
    if (int e = launch_tiled<P2G>(m, s, "p2g_kernel", m, P, g4, dirty)) return e;
  }
  if (int e = launch_tiled<G2P>(m, s, "g2p_kernel", m, P, (const float4*)g4)) return e;
  const long long nblocks = (long long)m.nbx * m.nby * m.nbz;
  clear_dirty_kernel<<<grid_for(nblocks, kBlock), kBlock, 0, s>>>(m, g4, dirty);
  return check_launch("clear_dirty_kernel");
}
