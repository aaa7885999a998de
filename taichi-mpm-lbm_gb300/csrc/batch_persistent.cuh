// Coupled steps of a scene batch in one persistent launch, instantiated per storage form in
// batch_persist_{f32,f16,bf16}.cu (FSI_BATCH_STEP_STORAGE, FSI_BATCH_PERSIST_NAME). Those
// units define FSI_LAUNCH_RO empty: the kernel's phases write what later phases read.
//
// One cooperative launch of as many 256-thread blocks as fit on the GPU at once runs `steps`
// coupled steps of every scene. Each phase of a step is a loop of the blocks over that phase's
// work items (cell tiles, particle tiles, node-block tiles or step tiles of every scene),
// running the per-item code of the one-launch-per-phase batch kernels; phases are separated by
// grid-wide barriers. Per step (coupling.py:135-173 per scene, SceneBatch.step's order):
//   1. rho, u of every cell (stale after the previous lattice step), the coupling accumulator
//      and immersed-boundary field zeroed, particle valid weights / masks and the counters
//      zeroed;
//   2. per substep: coupling forces | P2G | grid update + G2P | block clear (and the next
//      substep's coupling counters zeroed);
//   3. force assembly into the step's force buffer;
//   4. the lattice step (AA parity of the step) with that force.
// Every barrier wait is bounded by a clock limit: a block that gives up records FSI_ERR_TIMEOUT
// in the error word, and every block leaves at its next barrier once the word is set, so the
// launch ends with an error status instead of hanging.
#pragma once
#include "batch_types.cuh"

namespace fsi {
namespace {

// Grid-wide barrier of a cooperative launch: every block arrives once per barrier on a
// monotonically increasing counter and waits until all gridDim.x blocks of this epoch have.
// Returns false (for every thread of the block) when the launch is being abandoned.
__device__ __forceinline__ bool grid_barrier(const PersistArgs& a, unsigned& epoch) {
  __shared__ int ok;
  __syncthreads();
  ++epoch;
  if (threadIdx.x == 0) {
    const unsigned target = epoch * gridDim.x;
    __threadfence();
    atomicAdd(a.sync, 1u);
    int good = 1;
    const long long t0 = clock64();
    while (true) {
      const unsigned v = *reinterpret_cast<volatile unsigned*>(a.sync);
      if (v >= target) break;
      if (*reinterpret_cast<volatile int*>(a.err) != 0) { good = 0; break; }
      if (clock64() - t0 > a.wait_cycles) {
        atomicCAS(a.err, 0, FSI_ERR_TIMEOUT);
        good = 0;
        break;
      }
      __nanosleep(128);
    }
    __threadfence();
    ok = good && *reinterpret_cast<volatile int*>(a.err) == 0;
  }
  __syncthreads();
  return ok != 0;
}

template <int kStore, bool kFast, bool kOdd>
__device__ __forceinline__ void persist_step_tiles(const PersistArgs& a, float* force) {
  constexpr int NL = StepLanes<kFast>::n;
  for (int ti = blockIdx.x; ti < a.nstep_tiles; ti += gridDim.x) {
    const Tile t = a.step_tiles[ti];
    const BatchLattice& L = a.lat[t.lattice];
    const LatticeView v = view_of<kStore>(L, a.pops, a.macro, force, nullptr, a.flags);
    const int n = (int)L.g.n;
    for (int base = 0; base < a.step_tile_cells; base += kBlock * NL) {
      int ci[NL], cj[NL], ck[NL];
      bool has[NL];
      bool any = false;
#pragma unroll
      for (int l = 0; l < NL; ++l) {
        const int off = base + threadIdx.x + l * kBlock;
        const int c = t.first + off;
        has[l] = off < a.step_tile_cells && c < n;
        any = any || has[l];
        cell_ijk(L.g, has[l] ? c : t.first, ci[l], cj[l], ck[l]);
      }
      if (any) step_cells<kStore, kFast, kOdd, false, LatticeView>(v, ci, cj, ck, has);
    }
  }
}

// Resident 256-thread blocks per SM the kernel is compiled for (caps its registers).
#ifndef FSI_PERSIST_MIN_BLOCKS
#define FSI_PERSIST_MIN_BLOCKS 3
#endif

template <int kStore, bool kFast>
__global__ void __launch_bounds__(kBlock, FSI_PERSIST_MIN_BLOCKS) batch_persistent_kernel(PersistArgs a) {
  extern __shared__ float4 persist_smem[];
  float (*tile)[kTileCap] = reinterpret_cast<float (*)[kTileCap]>(persist_smem);
  unsigned epoch = 0;
  int prev = a.prev;
  int* const words = reinterpret_cast<int*>(a.fa.cnt);  // [count][12] counter words
  for (int step = 0; step < a.steps; ++step) {
    const int parity = (int)((a.steps_done + step) & 1);
    const bool refresh = step > 0 || !a.macro_fresh;
    float* const fprev = a.force[prev];
    float* const fnext = a.force[1 - prev];
    // 1. rho, u of the current state; zero the step's accumulators and counters
    for (int ti = blockIdx.x; ti < a.ncell_tiles; ti += gridDim.x) {
      const Tile t = a.cell_tiles[ti];
      const BatchLattice& L = a.lat[t.lattice];
      const int c = t.first + threadIdx.x;
      if (c >= L.g.n) continue;
      if (refresh) {
        float mass, vmax;
        batch_macro_cell<kStore, kFast>(L, c, a.pops, fprev, a.flags, parity, a.macro, mass, vmax);
      }
      a.fa.accum[L.off + c] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (a.aa.ib) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) a.aa.ib[3 * L.off + ax * L.g.n + c] = 0.f;
      }
    }
    for (int ti = blockIdx.x; ti < a.nptiles; ti += gridDim.x) {
      const Tile t = a.ptiles[ti];
      const int p = t.first * kBlock + threadIdx.x;
      if (p < a.sol[t.lattice].m.n) {
        a.fa.valid_out[p] = 0.f;
        a.fa.mask_out[p] = 0;
      }
    }
    if (blockIdx.x == 0)
      for (int w = threadIdx.x; w < 12 * a.count; w += kBlock) words[w] = 0;
    if (!grid_barrier(a, epoch)) return;
    // 2. substeps
    for (int sub = 0; sub < a.substeps; ++sub) {
      const int build = sub == 0 ? a.build_fraction : 0;
      for (int ti = blockIdx.x; ti < a.nptiles; ti += gridDim.x) {
        const Tile t = a.ptiles[ti];
        const ForceArgs f = scene_force_args(a.fa, a.lat[t.lattice], a.sol[t.lattice], t.lattice,
                                             a.dt_ratio, build);
        coupling_forces_body<false>(f, t.first * kBlock + threadIdx.x);
      }
      if (!grid_barrier(a, epoch)) return;
      for (int ti = blockIdx.x; ti < a.nptiles; ti += gridDim.x) {
        const Tile t = a.ptiles[ti];
        const BatchSolid& S = a.sol[t.lattice];
        p2g_body<false, true>(S.m, a.P, a.grid + a.lat[t.lattice].off, a.dirty + S.block_off,
                              t.first * kBlock + threadIdx.x, nullptr, tile);
      }
      if (!grid_barrier(a, epoch)) return;
      for (int ti = blockIdx.x; ti < a.nptiles; ti += gridDim.x) {
        const Tile t = a.ptiles[ti];
        g2p_body<true>(a.sol[t.lattice].m, a.P, a.grid + a.lat[t.lattice].off,
                       t.first * kBlock + threadIdx.x, tile);
      }
      if (!grid_barrier(a, epoch)) return;
      for (int ti = blockIdx.x; ti < a.nctiles; ti += gridDim.x) {
        const Tile t = a.ctiles[ti];
        const BatchSolid& S = a.sol[t.lattice];
        clear_body(S.m, a.grid + a.lat[t.lattice].off, a.dirty + S.block_off,
                   (long long)t.first + (threadIdx.x >> 5));
      }
      // the next substep's unsupported / partial / clipped counts start from zero
      if (blockIdx.x == 0 && sub + 1 < a.substeps)
        for (int w = threadIdx.x; w < 12 * a.count; w += kBlock)
          if (w % 12 < 5) words[w] = 0;
      if (!grid_barrier(a, epoch)) return;
    }
    // 3. force assembly into the step's force buffer
    for (int ti = blockIdx.x; ti < a.ncell_tiles; ti += gridDim.x) {
      const Tile t = a.cell_tiles[ti];
      AssembleArgs base = a.aa;
      base.force = fnext;
      const AssembleArgs as = scene_assemble_args(base, a.lat[t.lattice], a.sol[t.lattice], t.lattice);
      assemble_body(as, (long long)t.first + threadIdx.x);
    }
    if (!grid_barrier(a, epoch)) return;
    // 4. the lattice step with that force (rho, u are fresh: no recomputation)
    if (parity) persist_step_tiles<kStore, kFast, true>(a, fnext);
    else persist_step_tiles<kStore, kFast, false>(a, fnext);
    prev = 1 - prev;
    if (step + 1 < a.steps && !grid_barrier(a, epoch)) return;
  }
}

}  // namespace

// Launches batch_persistent_kernel for this storage form (FSI_BATCH_STEP_STORAGE): the fast
// arithmetic form for FP16/BF16 storage, either form for FP32. Returns FSI_OK, or an error
// when the launch could not be made (the kernel's own timeout shows in a->err).
int FSI_BATCH_PERSIST_NAME(const void* args, bool fast, cudaStream_t stream) {
  const PersistArgs& a = *static_cast<const PersistArgs*>(args);
  const size_t smem = sizeof(float) * 4 * kTileCap;
  auto launch = [&](auto kernel) -> int {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return check_launch("cudaFuncSetAttribute(batch_persistent_kernel)");
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem) != cudaSuccess)
      return check_launch("batch_persistent_kernel occupancy");
    FSI_REQUIRE(per_sm > 0, "batch_persistent_kernel does not fit on a multiprocessor");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(per_sm * sms));
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, kernel, a) != cudaSuccess)
      return check_launch("batch_persistent_kernel");
    return FSI_OK;
  };
#if FSI_BATCH_STEP_STORAGE == FSI_STORAGE_F32
  if (!fast) return launch(batch_persistent_kernel<FSI_STORAGE_F32, false>);
  return launch(batch_persistent_kernel<FSI_STORAGE_F32, true>);
#else
  (void)fast;
  return launch(batch_persistent_kernel<FSI_BATCH_STEP_STORAGE, true>);
#endif
}

}  // namespace fsi
