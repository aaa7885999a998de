// The batched lattice step kernel, instantiated per storage form in batch_step_f32.cu,
// batch_step_f16.cu and batch_step_bf16.cu (FSI_BATCH_STEP_STORAGE, FSI_BATCH_STEP_NAME),
// so that the forms' many template instances compile in parallel.
#include "batch_types.cuh"

namespace fsi {
namespace {

struct BatchStepArgs {
  const BatchLattice* lat;
  const Tile* tiles;
  int reps;  // passes of kStepBlock * lanes cells over the tile
  void* pops;
  float* macro;
  const float* force;
  const float* force_prev;
  const uint32_t* flags;
};

// Minimum resident blocks per SM of register-cap variant kVar (0..2).
template <bool kFast, bool kOdd, int kVar>
constexpr int batch_min_blocks() {
  return (kFast || !kOdd) ? (kVar == 0 ? 4 : kVar == 1 ? 6 : 8) : (kVar == 0 ? 6 : 8);
}

// kStepBlock threads cover a tile of reps * kStepBlock * lanes cells: the exact form takes
// one cell per thread and pass, the fast forms two (the packed lanes).
template <int kStore, bool kFast, bool kOdd, bool kRecompute, int kVar>
__global__ void __launch_bounds__(kStepBlock, (batch_min_blocks<kFast, kOdd, kVar>()))
    batch_step_kernel(BatchStepArgs b) {
  constexpr int NL = StepLanes<kFast>::n;
  const int kReps = b.reps;
  const Tile t = b.tiles[blockIdx.x];
  const BatchLattice& L = b.lat[t.lattice];
  const LatticeView v = view_of<kStore>(L, b.pops, b.macro, b.force, b.force_prev, b.flags);
  const int n = (int)L.g.n;
  for (int r = 0; r < kReps; ++r) {
    int ci[NL], cj[NL], ck[NL];
    bool has[NL];
    bool any = false;
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const int c = t.first + threadIdx.x + (r * NL + l) * kStepBlock;
      has[l] = c < n;
      any = any || has[l];
      cell_ijk(L.g, has[l] ? c : t.first, ci[l], cj[l], ck[l]);
    }
    if (any) step_cells<kStore, kFast, kOdd, kRecompute, LatticeView>(v, ci, cj, ck, has);
  }
}

template <int S, bool F, int V>
void launch_variant(const BatchStepArgs& a, int ntiles, bool odd, bool recompute, cudaStream_t s) {
  if (recompute) {
    if (odd) batch_step_kernel<S, F, true, true, V><<<ntiles, kStepBlock, 0, s>>>(a);
    else batch_step_kernel<S, F, false, true, V><<<ntiles, kStepBlock, 0, s>>>(a);
  } else {
    if (odd) batch_step_kernel<S, F, true, false, V><<<ntiles, kStepBlock, 0, s>>>(a);
    else batch_step_kernel<S, F, false, false, V><<<ntiles, kStepBlock, 0, s>>>(a);
  }
}

template <int S, bool F>
void launch_form(const BatchStepArgs& a, int ntiles, int variant, bool odd, bool recompute,
                 cudaStream_t s) {
  if (variant == 0) launch_variant<S, F, 0>(a, ntiles, odd, recompute, s);
  else if (variant == 2) launch_variant<S, F, 2>(a, ntiles, odd, recompute, s);
  else launch_variant<S, F, 1>(a, ntiles, odd, recompute, s);
}

}  // namespace

int FSI_BATCH_STEP_NAME(const void* lat, const void* tiles, int ntiles, int tile_cells,
                        int variant, bool fast, bool odd, bool recompute, void* pops,
                        float* macro, const float* force, const float* force_prev,
                        const uint32_t* flags, cudaStream_t stream) {
  BatchStepArgs a{static_cast<const BatchLattice*>(lat), static_cast<const Tile*>(tiles), 0,
                  pops, macro, force, force_prev, flags};
  a.reps = tile_cells / (kStepBlock * (fast ? 2 : 1));
#if FSI_BATCH_STEP_STORAGE == FSI_STORAGE_F32
  if (fast) launch_form<FSI_STORAGE_F32, true>(a, ntiles, variant, odd, recompute, stream);
  else launch_form<FSI_STORAGE_F32, false>(a, ntiles, variant, odd, recompute, stream);
#else
  launch_form<FSI_BATCH_STEP_STORAGE, true>(a, ntiles, variant, odd, recompute, stream);
#endif
  return check_launch("batch_step_kernel");
}

}  // namespace fsi
