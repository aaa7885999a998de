// Shared device/host helpers of the GB300 LBM-MPM library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "../../include/fsi_gb300.h"

// Qualifier of device pointers that a kernel only reads but that another phase of the same
// launch may write (particle positions, rho / u, the force field, the grid, populations).
// __restrict__ (the default) lets the compiler serve such reads from the read-only data
// path, which is only valid when the data does not change during the launch; the translation
// units of the persistent batch kernel, whose phases write what later phases read, define it
// empty.
#ifndef FSI_LAUNCH_RO
#define FSI_LAUNCH_RO __restrict__
#endif

namespace fsi {

// ------------------------------------------------------------ errors -------
void set_error(const char* fmt, ...);
int check_launch(const char* what);

#define FSI_REQUIRE(cond, ...)                 \
  do {                                         \
    if (!(cond)) {                             \
      ::fsi::set_error(__VA_ARGS__);           \
      return FSI_ERR_INVALID_ARG;              \
    }                                          \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (unsigned)(g < 1 ? 1 : g);
}

// D3Q19 velocities in the reference's order (fsi/lbm3d.py:221-239) and opposites (lbm3d.py:171-174).
__host__ __device__ constexpr int ex(int q) {
  return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int ey(int q) {
  return (q == 3 || q == 7 || q == 10 || q == 15 || q == 17) ? 1
         : (q == 4 || q == 8 || q == 9 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ez(int q) {
  return (q == 5 || q == 11 || q == 14 || q == 15 || q == 18) ? 1
         : (q == 6 || q == 12 || q == 13 || q == 16 || q == 17) ? -1 : 0;
}
// Threads per block of the one-thread-per-item kernels.
constexpr int kBlock = 256;

// Quadratic B-spline weight of offset i (mpm3d.py:227-232).
__device__ __forceinline__ float bspline_w(float fx, int i) {
  if (i == 0) { float a = __fsub_rn(1.5f, fx); return __fmul_rn(0.5f, __fmul_rn(a, a)); }
  if (i == 1) { float b = __fsub_rn(fx, 1.0f); return __fsub_rn(0.75f, __fmul_rn(b, b)); }
  float c = __fsub_rn(fx, 0.5f);
  return __fmul_rn(0.5f, __fmul_rn(c, c));
}

__host__ __device__ constexpr int opp(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }

// Lattice weights as the reference stores them: float32(1/3), float32(1/18), float32(1/36).
constexpr float kW0 = 0x1.555556p-2f;
constexpr float kW1 = 0x1.c71c72p-5f;
constexpr float kW2 = 0x1.c71c72p-6f;
__host__ __device__ constexpr float weight_of(int q) { return q == 0 ? kW0 : (q < 7 ? kW1 : kW2); }

// Per-cell flag word of the lattice (built once from the solid mask):
//   bit 0       this cell is solid
//   bit q 1..18 neighbour x + e_q (periodic wrap) is solid
//   bit 20/21   cell lies on the x = 0 / x = nx-1 face
//   bit 22 + 4a + 2b + c   corner neighbour x + (2a-1, 2b-1, 2c-1) (periodic wrap) is solid
// With the cell's own bit and the 18 neighbour bits, the corner bits give the solid state of
// the whole 3^3 block around the cell from one word (the coupling's stencil).
constexpr uint32_t kFlagSolid = 1u;
constexpr uint32_t kFlagFaceLeft = 1u << 20;
constexpr uint32_t kFlagFaceRight = 1u << 21;
constexpr int kFlagCornerShift = 22;

// ------------------------------------------------------------ atomics ------
// Vector reduction into global memory (no return value), 16-byte aligned address.
__device__ __forceinline__ void red_add_v4(float4* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}

// Warp-aggregated integer counter increment (one atomic per warp).
__device__ __forceinline__ void warp_count(int* counter, bool pred) {
  unsigned mask = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0 && mask) atomicAdd(counter, __popc(mask));
}

// Reference float32 feq (fsi/lbm3d.py:250-254), rounding each operation.
__device__ __forceinline__ float feq_ref(int q, float rho, float ux, float uy, float uz) {
  float eu;
  {
    // e.u with Taichi's Vector.dot order ((ex*ux + ey*uy) + ez*uz).
    float a = __fmul_rn((float)ex(q), ux);
    a = __fadd_rn(a, __fmul_rn((float)ey(q), uy));
    eu = __fadd_rn(a, __fmul_rn((float)ez(q), uz));
  }
  float uv = __fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)), __fmul_rn(uz, uz));
  float inner = __fadd_rn(1.0f, __fmul_rn(3.0f, eu));
  inner = __fadd_rn(inner, __fmul_rn(__fmul_rn(4.5f, eu), eu));
  inner = __fsub_rn(inner, __fmul_rn(1.5f, uv));
  return __fmul_rn(__fmul_rn(weight_of(q), rho), inner);
}

}  // namespace fsi
