// GENERATED by gen_lbm_formulas.py -- do not edit by hand.
// D3Q19 MRT collision of the reference (fsi/lbm3d.py:269-333) as explicit
// register formulas with the reference's float32 operation order.
#pragma once

#include "lbm_vec.cuh"

namespace fsi {

// m[k] = sum_q M[k][q] * X[q], sequential in q (lbm3d.py:269-274).
template <class V>
__device__ __forceinline__ void mrt_forward(const V (&X)[19], V (&m)[19]) {
  V two[19];
  two[1] = vadd(X[1], X[1]);
  two[2] = vadd(X[2], X[2]);
  two[3] = vadd(X[3], X[3]);
  two[4] = vadd(X[4], X[4]);
  two[5] = vadd(X[5], X[5]);
  two[6] = vadd(X[6], X[6]);
  two[15] = vadd(X[15], X[15]);
  two[16] = vadd(X[16], X[16]);
  two[17] = vadd(X[17], X[17]);
  two[18] = vadd(X[18], X[18]);
  m[0] = X[0]; m[0] = vadd(m[0], X[1]); m[0] = vadd(m[0], X[2]); m[0] = vadd(m[0], X[3]); m[0] = vadd(m[0], X[4]); m[0] = vadd(m[0], X[5]); m[0] = vadd(m[0], X[6]); m[0] = vadd(m[0], X[7]); m[0] = vadd(m[0], X[8]); m[0] = vadd(m[0], X[9]); m[0] = vadd(m[0], X[10]); m[0] = vadd(m[0], X[11]); m[0] = vadd(m[0], X[12]); m[0] = vadd(m[0], X[13]); m[0] = vadd(m[0], X[14]); m[0] = vadd(m[0], X[15]); m[0] = vadd(m[0], X[16]); m[0] = vadd(m[0], X[17]); m[0] = vadd(m[0], X[18]);
  m[1] = vneg(X[0]); m[1] = vadd(m[1], X[7]); m[1] = vadd(m[1], X[8]); m[1] = vadd(m[1], X[9]); m[1] = vadd(m[1], X[10]); m[1] = vadd(m[1], X[11]); m[1] = vadd(m[1], X[12]); m[1] = vadd(m[1], X[13]); m[1] = vadd(m[1], X[14]); m[1] = vadd(m[1], X[15]); m[1] = vadd(m[1], X[16]); m[1] = vadd(m[1], X[17]); m[1] = vadd(m[1], X[18]);
  m[2] = X[0]; m[2] = vsub(m[2], two[1]); m[2] = vsub(m[2], two[2]); m[2] = vsub(m[2], two[3]); m[2] = vsub(m[2], two[4]); m[2] = vsub(m[2], two[5]); m[2] = vsub(m[2], two[6]); m[2] = vadd(m[2], X[7]); m[2] = vadd(m[2], X[8]); m[2] = vadd(m[2], X[9]); m[2] = vadd(m[2], X[10]); m[2] = vadd(m[2], X[11]); m[2] = vadd(m[2], X[12]); m[2] = vadd(m[2], X[13]); m[2] = vadd(m[2], X[14]); m[2] = vadd(m[2], X[15]); m[2] = vadd(m[2], X[16]); m[2] = vadd(m[2], X[17]); m[2] = vadd(m[2], X[18]);
  m[3] = X[1]; m[3] = vsub(m[3], X[2]); m[3] = vadd(m[3], X[7]); m[3] = vsub(m[3], X[8]); m[3] = vadd(m[3], X[9]); m[3] = vsub(m[3], X[10]); m[3] = vadd(m[3], X[11]); m[3] = vsub(m[3], X[12]); m[3] = vadd(m[3], X[13]); m[3] = vsub(m[3], X[14]);
  m[4] = vneg(two[1]); m[4] = vadd(m[4], two[2]); m[4] = vadd(m[4], X[7]); m[4] = vsub(m[4], X[8]); m[4] = vadd(m[4], X[9]); m[4] = vsub(m[4], X[10]); m[4] = vadd(m[4], X[11]); m[4] = vsub(m[4], X[12]); m[4] = vadd(m[4], X[13]); m[4] = vsub(m[4], X[14]);
  m[5] = X[3]; m[5] = vsub(m[5], X[4]); m[5] = vadd(m[5], X[7]); m[5] = vsub(m[5], X[8]); m[5] = vsub(m[5], X[9]); m[5] = vadd(m[5], X[10]); m[5] = vadd(m[5], X[15]); m[5] = vsub(m[5], X[16]); m[5] = vadd(m[5], X[17]); m[5] = vsub(m[5], X[18]);
  m[6] = vneg(two[3]); m[6] = vadd(m[6], two[4]); m[6] = vadd(m[6], X[7]); m[6] = vsub(m[6], X[8]); m[6] = vsub(m[6], X[9]); m[6] = vadd(m[6], X[10]); m[6] = vadd(m[6], X[15]); m[6] = vsub(m[6], X[16]); m[6] = vadd(m[6], X[17]); m[6] = vsub(m[6], X[18]);
  m[7] = X[5]; m[7] = vsub(m[7], X[6]); m[7] = vadd(m[7], X[11]); m[7] = vsub(m[7], X[12]); m[7] = vsub(m[7], X[13]); m[7] = vadd(m[7], X[14]); m[7] = vadd(m[7], X[15]); m[7] = vsub(m[7], X[16]); m[7] = vsub(m[7], X[17]); m[7] = vadd(m[7], X[18]);
  m[8] = vneg(two[5]); m[8] = vadd(m[8], two[6]); m[8] = vadd(m[8], X[11]); m[8] = vsub(m[8], X[12]); m[8] = vsub(m[8], X[13]); m[8] = vadd(m[8], X[14]); m[8] = vadd(m[8], X[15]); m[8] = vsub(m[8], X[16]); m[8] = vsub(m[8], X[17]); m[8] = vadd(m[8], X[18]);
  m[9] = two[1]; m[9] = vadd(m[9], two[2]); m[9] = vsub(m[9], X[3]); m[9] = vsub(m[9], X[4]); m[9] = vsub(m[9], X[5]); m[9] = vsub(m[9], X[6]); const V pre9_6 = m[9]; m[9] = vadd(m[9], X[7]); m[9] = vadd(m[9], X[8]); m[9] = vadd(m[9], X[9]); m[9] = vadd(m[9], X[10]); m[9] = vadd(m[9], X[11]); m[9] = vadd(m[9], X[12]); m[9] = vadd(m[9], X[13]); m[9] = vadd(m[9], X[14]); m[9] = vsub(m[9], two[15]); m[9] = vsub(m[9], two[16]); m[9] = vsub(m[9], two[17]); m[9] = vsub(m[9], two[18]);
  m[10] = vsub(X[7], pre9_6); m[10] = vadd(m[10], X[8]); m[10] = vadd(m[10], X[9]); m[10] = vadd(m[10], X[10]); m[10] = vadd(m[10], X[11]); m[10] = vadd(m[10], X[12]); m[10] = vadd(m[10], X[13]); m[10] = vadd(m[10], X[14]); m[10] = vsub(m[10], two[15]); m[10] = vsub(m[10], two[16]); m[10] = vsub(m[10], two[17]); m[10] = vsub(m[10], two[18]);
  m[11] = X[3]; m[11] = vadd(m[11], X[4]); m[11] = vsub(m[11], X[5]); m[11] = vsub(m[11], X[6]); const V pre11_4 = m[11]; m[11] = vadd(m[11], X[7]); m[11] = vadd(m[11], X[8]); m[11] = vadd(m[11], X[9]); m[11] = vadd(m[11], X[10]); m[11] = vsub(m[11], X[11]); m[11] = vsub(m[11], X[12]); m[11] = vsub(m[11], X[13]); m[11] = vsub(m[11], X[14]);
  m[12] = vsub(X[7], pre11_4); m[12] = vadd(m[12], X[8]); m[12] = vadd(m[12], X[9]); m[12] = vadd(m[12], X[10]); m[12] = vsub(m[12], X[11]); m[12] = vsub(m[12], X[12]); m[12] = vsub(m[12], X[13]); m[12] = vsub(m[12], X[14]);
  m[13] = X[7]; m[13] = vadd(m[13], X[8]); m[13] = vsub(m[13], X[9]); m[13] = vsub(m[13], X[10]);
  m[14] = X[15]; m[14] = vadd(m[14], X[16]); m[14] = vsub(m[14], X[17]); m[14] = vsub(m[14], X[18]);
  m[15] = X[11]; m[15] = vadd(m[15], X[12]); m[15] = vsub(m[15], X[13]); m[15] = vsub(m[15], X[14]);
  m[16] = X[7]; m[16] = vsub(m[16], X[8]); const V pre16_2 = m[16]; m[16] = vadd(m[16], X[9]); m[16] = vsub(m[16], X[10]); m[16] = vsub(m[16], X[11]); m[16] = vadd(m[16], X[12]); m[16] = vsub(m[16], X[13]); m[16] = vadd(m[16], X[14]);
  m[17] = vsub(X[9], pre16_2); m[17] = vsub(m[17], X[10]); m[17] = vadd(m[17], X[15]); m[17] = vsub(m[17], X[16]); m[17] = vadd(m[17], X[17]); m[17] = vsub(m[17], X[18]);
  m[18] = X[11]; m[18] = vsub(m[18], X[12]); m[18] = vsub(m[18], X[13]); m[18] = vadd(m[18], X[14]); m[18] = vsub(m[18], X[15]); m[18] = vadd(m[18], X[16]); m[18] = vadd(m[18], X[17]); m[18] = vsub(m[18], X[18]);
}

// f[q] = sum_k inv(M)[q][k] * m[k], sequential in k (lbm3d.py:328-333).
// 22 rounded products; every other product is an exact power-of-two scaling.
template <class V>
__device__ __forceinline__ void mrt_inverse(const V (&m)[19], V (&f)[19]) {
  const V p0_0 = vmul(m[0], 0x1.5555560000000p-2f);
  const V p0_1 = vmul(m[0], 0x1.c71c720000000p-5f);
  const V p1_0 = vmul(m[1], 0x1.0000000000000p-1f);
  const V p1_1 = vmul(m[1], 0x1.5555560000000p-5f);
  const V p2_0 = vmul(m[2], 0x1.5555560000000p-3f);
  const V p2_1 = vmul(m[2], 0x1.c71c720000000p-5f);
  const V p3_0 = vmul(m[3], 0x1.5555560000000p-3f);
  const V p4_0 = vmul(m[4], 0x1.5555560000000p-3f);
  const V p5_0 = vmul(m[5], 0x1.5555560000000p-3f);
  const V p6_0 = vmul(m[6], 0x1.5555560000000p-3f);
  const V p7_0 = vmul(m[7], 0x1.5555560000000p-3f);
  const V p8_0 = vmul(m[8], 0x1.5555560000000p-3f);
  const V p9_0 = vmul(m[9], 0x1.5555560000000p-4f);
  const V p10_0 = vmul(m[10], 0x1.5555560000000p-4f);
  const V p11_0 = vmul(m[11], 0x1.0000000000000p-3f);
  const V p12_0 = vmul(m[12], 0x1.0000000000000p-3f);
  const V p13_0 = vmul(m[13], 0x1.0000000000000p-2f);
  const V p14_0 = vmul(m[14], 0x1.0000000000000p-2f);
  const V p15_0 = vmul(m[15], 0x1.0000000000000p-2f);
  const V p16_0 = vmul(m[16], 0x1.0000000000000p-3f);
  const V p17_0 = vmul(m[17], 0x1.0000000000000p-3f);
  const V p18_0 = vmul(m[18], 0x1.0000000000000p-3f);
  const V p9_0_s0 = vmul(p9_0, 0x1.0000000000000p-1f);
  const V p10_0_s1 = vmul(p10_0, 0x1.0000000000000p-1f);
  const V p0_1_s2 = vmul(p0_1, 0x1.0000000000000p-1f);
  const V p2_1_s3 = vmul(p2_1, 0x1.0000000000000p-2f);
  const V p3_0_s4 = vmul(p3_0, 0x1.0000000000000p-1f);
  const V p4_0_s5 = vmul(p4_0, 0x1.0000000000000p-2f);
  const V p5_0_s6 = vmul(p5_0, 0x1.0000000000000p-1f);
  const V p6_0_s7 = vmul(p6_0, 0x1.0000000000000p-2f);
  const V p9_0_s8 = vmul(p9_0, 0x1.0000000000000p-2f);
  const V p10_0_s9 = vmul(p10_0, 0x1.0000000000000p-2f);
  const V p11_0_s10 = vmul(p11_0, 0x1.0000000000000p-1f);
  const V p12_0_s11 = vmul(p12_0, 0x1.0000000000000p-1f);
  const V p7_0_s12 = vmul(p7_0, 0x1.0000000000000p-1f);
  const V p8_0_s13 = vmul(p8_0, 0x1.0000000000000p-2f);
  f[0] = p0_0; f[0] = vsub(f[0], p1_0); f[0] = vadd(f[0], p2_0);
  f[1] = p0_1; f[1] = vsub(f[1], p2_1); const V r0 = f[1]; f[1] = vadd(f[1], p3_0); f[1] = vsub(f[1], p4_0); f[1] = vadd(f[1], p9_0); f[1] = vsub(f[1], p10_0);
  f[2] = r0; f[2] = vsub(f[2], p3_0); f[2] = vadd(f[2], p4_0); f[2] = vadd(f[2], p9_0); f[2] = vsub(f[2], p10_0);
  f[3] = r0; f[3] = vadd(f[3], p5_0); f[3] = vsub(f[3], p6_0); f[3] = vsub(f[3], p9_0_s0); f[3] = vadd(f[3], p10_0_s1); f[3] = vadd(f[3], p11_0); f[3] = vsub(f[3], p12_0);
  f[4] = r0; f[4] = vsub(f[4], p5_0); f[4] = vadd(f[4], p6_0); f[4] = vsub(f[4], p9_0_s0); f[4] = vadd(f[4], p10_0_s1); f[4] = vadd(f[4], p11_0); f[4] = vsub(f[4], p12_0);
  f[5] = r0; f[5] = vadd(f[5], p7_0); f[5] = vsub(f[5], p8_0); f[5] = vsub(f[5], p9_0_s0); f[5] = vadd(f[5], p10_0_s1); f[5] = vsub(f[5], p11_0); f[5] = vadd(f[5], p12_0);
  f[6] = r0; f[6] = vsub(f[6], p7_0); f[6] = vadd(f[6], p8_0); f[6] = vsub(f[6], p9_0_s0); f[6] = vadd(f[6], p10_0_s1); f[6] = vsub(f[6], p11_0); f[6] = vadd(f[6], p12_0);
  f[7] = p0_1_s2; f[7] = vadd(f[7], p1_1); f[7] = vadd(f[7], p2_1_s3); const V r1 = f[7]; f[7] = vadd(f[7], p3_0_s4); f[7] = vadd(f[7], p4_0_s5); const V r2 = f[7]; f[7] = vadd(f[7], p5_0_s6); f[7] = vadd(f[7], p6_0_s7); f[7] = vadd(f[7], p9_0_s8); f[7] = vadd(f[7], p10_0_s9); f[7] = vadd(f[7], p11_0_s10); f[7] = vadd(f[7], p12_0_s11); f[7] = vadd(f[7], p13_0); f[7] = vadd(f[7], p16_0); f[7] = vsub(f[7], p17_0);
  f[8] = r1; f[8] = vsub(f[8], p3_0_s4); f[8] = vsub(f[8], p4_0_s5); const V r3 = f[8]; f[8] = vsub(f[8], p5_0_s6); f[8] = vsub(f[8], p6_0_s7); f[8] = vadd(f[8], p9_0_s8); f[8] = vadd(f[8], p10_0_s9); f[8] = vadd(f[8], p11_0_s10); f[8] = vadd(f[8], p12_0_s11); f[8] = vadd(f[8], p13_0); f[8] = vsub(f[8], p16_0); f[8] = vadd(f[8], p17_0);
  f[9] = r2; f[9] = vsub(f[9], p5_0_s6); f[9] = vsub(f[9], p6_0_s7); f[9] = vadd(f[9], p9_0_s8); f[9] = vadd(f[9], p10_0_s9); f[9] = vadd(f[9], p11_0_s10); f[9] = vadd(f[9], p12_0_s11); f[9] = vsub(f[9], p13_0); f[9] = vadd(f[9], p16_0); f[9] = vadd(f[9], p17_0);
  f[10] = r3; f[10] = vadd(f[10], p5_0_s6); f[10] = vadd(f[10], p6_0_s7); f[10] = vadd(f[10], p9_0_s8); f[10] = vadd(f[10], p10_0_s9); f[10] = vadd(f[10], p11_0_s10); f[10] = vadd(f[10], p12_0_s11); f[10] = vsub(f[10], p13_0); f[10] = vsub(f[10], p16_0); f[10] = vsub(f[10], p17_0);
  f[11] = r2; f[11] = vadd(f[11], p7_0_s12); f[11] = vadd(f[11], p8_0_s13); f[11] = vadd(f[11], p9_0_s8); f[11] = vadd(f[11], p10_0_s9); f[11] = vsub(f[11], p11_0_s10); f[11] = vsub(f[11], p12_0_s11); f[11] = vadd(f[11], p15_0); f[11] = vsub(f[11], p16_0); f[11] = vadd(f[11], p18_0);
  f[12] = r3; f[12] = vsub(f[12], p7_0_s12); f[12] = vsub(f[12], p8_0_s13); f[12] = vadd(f[12], p9_0_s8); f[12] = vadd(f[12], p10_0_s9); f[12] = vsub(f[12], p11_0_s10); f[12] = vsub(f[12], p12_0_s11); f[12] = vadd(f[12], p15_0); f[12] = vadd(f[12], p16_0); f[12] = vsub(f[12], p18_0);
  f[13] = r2; f[13] = vsub(f[13], p7_0_s12); f[13] = vsub(f[13], p8_0_s13); f[13] = vadd(f[13], p9_0_s8); f[13] = vadd(f[13], p10_0_s9); f[13] = vsub(f[13], p11_0_s10); f[13] = vsub(f[13], p12_0_s11); f[13] = vsub(f[13], p15_0); f[13] = vsub(f[13], p16_0); f[13] = vsub(f[13], p18_0);
  f[14] = r3; f[14] = vadd(f[14], p7_0_s12); f[14] = vadd(f[14], p8_0_s13); f[14] = vadd(f[14], p9_0_s8); f[14] = vadd(f[14], p10_0_s9); f[14] = vsub(f[14], p11_0_s10); f[14] = vsub(f[14], p12_0_s11); f[14] = vsub(f[14], p15_0); f[14] = vadd(f[14], p16_0); f[14] = vadd(f[14], p18_0);
  f[15] = r1; f[15] = vadd(f[15], p5_0_s6); f[15] = vadd(f[15], p6_0_s7); const V r4 = f[15]; f[15] = vadd(f[15], p7_0_s12); f[15] = vadd(f[15], p8_0_s13); f[15] = vsub(f[15], p9_0_s0); f[15] = vsub(f[15], p10_0_s1); f[15] = vadd(f[15], p14_0); f[15] = vadd(f[15], p17_0); f[15] = vsub(f[15], p18_0);
  f[16] = r1; f[16] = vsub(f[16], p5_0_s6); f[16] = vsub(f[16], p6_0_s7); const V r5 = f[16]; f[16] = vsub(f[16], p7_0_s12); f[16] = vsub(f[16], p8_0_s13); f[16] = vsub(f[16], p9_0_s0); f[16] = vsub(f[16], p10_0_s1); f[16] = vadd(f[16], p14_0); f[16] = vsub(f[16], p17_0); f[16] = vadd(f[16], p18_0);
  f[17] = r4; f[17] = vsub(f[17], p7_0_s12); f[17] = vsub(f[17], p8_0_s13); f[17] = vsub(f[17], p9_0_s0); f[17] = vsub(f[17], p10_0_s1); f[17] = vsub(f[17], p14_0); f[17] = vadd(f[17], p17_0); f[17] = vadd(f[17], p18_0);
  f[18] = r5; f[18] = vadd(f[18], p7_0_s12); f[18] = vadd(f[18], p8_0_s13); f[18] = vsub(f[18], p9_0_s0); f[18] = vsub(f[18], p10_0_s1); f[18] = vsub(f[18], p14_0); f[18] = vsub(f[18], p17_0); f[18] = vsub(f[18], p18_0);
}


// Reduced-operation MRT + Guo collision (same operator, not the reference's rounding):
// parity-split moments from pair sums/differences, closed-form forcing moments
// g_k = A_k.G - B_k (u.G) + u^T C_k G, parity-split inverse. Used by the FP16/BF16
// storage forms and the FP32 fast form.
template <class V>
__device__ __forceinline__ void mrt_collide_fast(const V (&F)[19], V rho, V ux, V uy, V uz,
    V gx, V gy, V gz, const float* __restrict__ S, V (&out)[19]) {
  const V P0 = vadd(F[1], F[2]), D0 = vsub(F[1], F[2]);
  const V P1 = vadd(F[3], F[4]), D1 = vsub(F[3], F[4]);
  const V P2 = vadd(F[5], F[6]), D2 = vsub(F[5], F[6]);
  const V P3 = vadd(F[7], F[8]), D3 = vsub(F[7], F[8]);
  const V P4 = vadd(F[9], F[10]), D4 = vsub(F[9], F[10]);
  const V P5 = vadd(F[11], F[12]), D5 = vsub(F[11], F[12]);
  const V P6 = vadd(F[13], F[14]), D6 = vsub(F[13], F[14]);
  const V P7 = vadd(F[15], F[16]), D7 = vsub(F[15], F[16]);
  const V P8 = vadd(F[17], F[18]), D8 = vsub(F[17], F[18]);
  V m0 = vadd(vadd(vadd(vadd(vadd(vadd(vadd(vadd(vadd(F[0], P0), P1), P2), P3), P4), P5), P6), P7), P8);
  V m1 = vadd(vadd(vadd(vadd(vadd(vadd(vneg(F[0]), P3), P4), P5), P6), P7), P8);
  V m2 = vadd(vadd(vadd(vadd(vadd(vadd(vfma(-0x1.0000000000000p+1f, P2, vfma(-0x1.0000000000000p+1f, P1, vfma(-0x1.0000000000000p+1f, P0, F[0]))), P3), P4), P5), P6), P7), P8);
  V m9 = vfma(-0x1.0000000000000p+1f, P8, vfma(-0x1.0000000000000p+1f, P7, vadd(vadd(vadd(vadd(vsub(vsub(vmul(P0, 0x1.0000000000000p+1f), P1), P2), P3), P4), P5), P6)));
  V m10 = vfma(-0x1.0000000000000p+1f, P8, vfma(-0x1.0000000000000p+1f, P7, vadd(vadd(vadd(vadd(vadd(vadd(vmul(P0, -0x1.0000000000000p+1f), P1), P2), P3), P4), P5), P6)));
  V m11 = vsub(vsub(vadd(vadd(vsub(P1, P2), P3), P4), P5), P6);
  V m12 = vsub(vsub(vadd(vadd(vadd(vneg(P1), P2), P3), P4), P5), P6);
  V m13 = vsub(P3, P4);
  V m14 = vsub(P7, P8);
  V m15 = vsub(P5, P6);
  V m3 = vadd(vadd(vadd(vadd(D0, D3), D4), D5), D6);
  V m4 = vadd(vadd(vadd(vadd(vmul(D0, -0x1.0000000000000p+1f), D3), D4), D5), D6);
  V m5 = vadd(vadd(vsub(vadd(D1, D3), D4), D7), D8);
  V m6 = vadd(vadd(vsub(vadd(vmul(D1, -0x1.0000000000000p+1f), D3), D4), D7), D8);
  V m7 = vsub(vadd(vsub(vadd(D2, D5), D6), D7), D8);
  V m8 = vsub(vadd(vsub(vadd(vmul(D2, -0x1.0000000000000p+1f), D5), D6), D7), D8);
  V m16 = vsub(vsub(vadd(D3, D4), D5), D6);
  V m17 = vadd(vadd(vadd(vneg(D3), D4), D7), D8);
  V m18 = vadd(vsub(vsub(D5, D6), D7), D8);
  const V uG = vfma(ux, gx, vfma(uy, gy, vmul(uz, gz)));
  const V pxx = vmul(ux, gx), pyy = vmul(uy, gy), pzz = vmul(uz, gz);
  const V sxy = vfma(ux, gy, vmul(uy, gx)), syz = vfma(uy, gz, vmul(uz, gy)), sxz = vfma(ux, gz, vmul(uz, gx));
  const V g0 = vfma(0x1.5555560000000p-2f, pzz, vfma(0x1.5555560000000p-2f, pyy, vfma(0x1.5555560000000p-2f, pxx, vneg(uG))));
  const V g1 = vfma(0x1.c71c720000000p-3f, pzz, vfma(0x1.c71c720000000p-3f, pyy, vmul(pxx, 0x1.c71c720000000p-3f)));
  const V g3 = vmul(gx, 0x1.5555560000000p-2f);
  const V g5 = vmul(gy, 0x1.5555560000000p-2f);
  const V g7 = vmul(gz, 0x1.5555560000000p-2f);
  const V g9 = vfma(-0x1.c71c720000000p-3f, pzz, vfma(-0x1.c71c720000000p-3f, pyy, vmul(pxx, 0x1.c71c720000000p-2f)));
  const V g11 = vfma(-0x1.c71c720000000p-3f, pzz, vmul(pyy, 0x1.c71c720000000p-3f));
  const V g13 = vmul(sxy, 0x1.c71c720000000p-4f);
  const V g14 = vmul(syz, 0x1.c71c720000000p-4f);
  const V g15 = vmul(sxz, 0x1.c71c720000000p-4f);
  const V uu = vfma(ux, ux, vfma(uy, uy, vmul(uz, uz)));
  m0 = vadd(m0, g0);
  m1 = vfma(fmaf(-0.5f, S[1], 1.0f), g1, vfma(-S[1], vsub(m1, uu), m1));
  m2 = vfma(-S[2], m2, m2);
  m3 = vadd(m3, g3);
  m4 = vfma(-S[4], m4, m4);
  m5 = vadd(m5, g5);
  m6 = vfma(-S[6], m6, m6);
  m7 = vadd(m7, g7);
  m8 = vfma(-S[8], m8, m8);
  m9 = vfma(fmaf(-0.5f, S[9], 1.0f), g9, vfma(-S[9], vsub(m9, vfma(vadd(ux, ux), ux, vneg(vfma(uy, uy, vmul(uz, uz))))), m9));
  m10 = vfma(-S[10], m10, m10);
  m11 = vfma(fmaf(-0.5f, S[11], 1.0f), g11, vfma(-S[11], vsub(m11, vfma(uy, uy, vneg(vmul(uz, uz)))), m11));
  m12 = vfma(-S[12], m12, m12);
  m13 = vfma(fmaf(-0.5f, S[13], 1.0f), g13, vfma(-S[13], vsub(m13, vmul(ux, uy)), m13));
  m14 = vfma(fmaf(-0.5f, S[14], 1.0f), g14, vfma(-S[14], vsub(m14, vmul(uy, uz)), m14));
  m15 = vfma(fmaf(-0.5f, S[15], 1.0f), g15, vfma(-S[15], vsub(m15, vmul(ux, uz)), m15));
  m16 = vfma(-S[16], m16, m16);
  m17 = vfma(-S[17], m17, m17);
  m18 = vfma(-S[18], m18, m18);
  out[0] = vfma(0x1.5555560000000p-3f, m2, vfma(-0x1.0000000000000p-1f, m1, vmul(m0, 0x1.5555560000000p-2f)));
  { const V e = vfma(-0x1.5555560000000p-4f, m10, vfma(0x1.5555560000000p-4f, m9, vfma(-0x1.c71c720000000p-5f, m2, vmul(m0, 0x1.c71c720000000p-5f)))), o = vfma(-0x1.5555560000000p-3f, m4, vmul(m3, 0x1.5555560000000p-3f)); out[1] = vadd(e, o); out[2] = vsub(e, o); }
  { const V e = vfma(-0x1.0000000000000p-3f, m12, vfma(0x1.0000000000000p-3f, m11, vfma(0x1.5555560000000p-5f, m10, vfma(-0x1.5555560000000p-5f, m9, vfma(-0x1.c71c720000000p-5f, m2, vmul(m0, 0x1.c71c720000000p-5f)))))), o = vfma(-0x1.5555560000000p-3f, m6, vmul(m5, 0x1.5555560000000p-3f)); out[3] = vadd(e, o); out[4] = vsub(e, o); }
  { const V e = vfma(0x1.0000000000000p-3f, m12, vfma(-0x1.0000000000000p-3f, m11, vfma(0x1.5555560000000p-5f, m10, vfma(-0x1.5555560000000p-5f, m9, vfma(-0x1.c71c720000000p-5f, m2, vmul(m0, 0x1.c71c720000000p-5f)))))), o = vfma(-0x1.5555560000000p-3f, m8, vmul(m7, 0x1.5555560000000p-3f)); out[5] = vadd(e, o); out[6] = vsub(e, o); }
  { const V e = vfma(0x1.0000000000000p-2f, m13, vfma(0x1.0000000000000p-4f, m12, vfma(0x1.0000000000000p-4f, m11, vfma(0x1.5555560000000p-6f, m10, vfma(0x1.5555560000000p-6f, m9, vfma(0x1.c71c720000000p-7f, m2, vfma(0x1.5555560000000p-5f, m1, vmul(m0, 0x1.c71c720000000p-6f)))))))), o = vfma(-0x1.0000000000000p-3f, m17, vfma(0x1.0000000000000p-3f, m16, vfma(0x1.5555560000000p-5f, m6, vfma(0x1.5555560000000p-4f, m5, vfma(0x1.5555560000000p-5f, m4, vmul(m3, 0x1.5555560000000p-4f)))))); out[7] = vadd(e, o); out[8] = vsub(e, o); }
  { const V e = vfma(-0x1.0000000000000p-2f, m13, vfma(0x1.0000000000000p-4f, m12, vfma(0x1.0000000000000p-4f, m11, vfma(0x1.5555560000000p-6f, m10, vfma(0x1.5555560000000p-6f, m9, vfma(0x1.c71c720000000p-7f, m2, vfma(0x1.5555560000000p-5f, m1, vmul(m0, 0x1.c71c720000000p-6f)))))))), o = vfma(0x1.0000000000000p-3f, m17, vfma(0x1.0000000000000p-3f, m16, vfma(-0x1.5555560000000p-5f, m6, vfma(-0x1.5555560000000p-4f, m5, vfma(0x1.5555560000000p-5f, m4, vmul(m3, 0x1.5555560000000p-4f)))))); out[9] = vadd(e, o); out[10] = vsub(e, o); }
  { const V e = vfma(0x1.0000000000000p-2f, m15, vfma(-0x1.0000000000000p-4f, m12, vfma(-0x1.0000000000000p-4f, m11, vfma(0x1.5555560000000p-6f, m10, vfma(0x1.5555560000000p-6f, m9, vfma(0x1.c71c720000000p-7f, m2, vfma(0x1.5555560000000p-5f, m1, vmul(m0, 0x1.c71c720000000p-6f)))))))), o = vfma(0x1.0000000000000p-3f, m18, vfma(-0x1.0000000000000p-3f, m16, vfma(0x1.5555560000000p-5f, m8, vfma(0x1.5555560000000p-4f, m7, vfma(0x1.5555560000000p-5f, m4, vmul(m3, 0x1.5555560000000p-4f)))))); out[11] = vadd(e, o); out[12] = vsub(e, o); }
  { const V e = vfma(-0x1.0000000000000p-2f, m15, vfma(-0x1.0000000000000p-4f, m12, vfma(-0x1.0000000000000p-4f, m11, vfma(0x1.5555560000000p-6f, m10, vfma(0x1.5555560000000p-6f, m9, vfma(0x1.c71c720000000p-7f, m2, vfma(0x1.5555560000000p-5f, m1, vmul(m0, 0x1.c71c720000000p-6f)))))))), o = vfma(-0x1.0000000000000p-3f, m18, vfma(-0x1.0000000000000p-3f, m16, vfma(-0x1.5555560000000p-5f, m8, vfma(-0x1.5555560000000p-4f, m7, vfma(0x1.5555560000000p-5f, m4, vmul(m3, 0x1.5555560000000p-4f)))))); out[13] = vadd(e, o); out[14] = vsub(e, o); }
  { const V e = vfma(0x1.0000000000000p-2f, m14, vfma(-0x1.5555560000000p-5f, m10, vfma(-0x1.5555560000000p-5f, m9, vfma(0x1.c71c720000000p-7f, m2, vfma(0x1.5555560000000p-5f, m1, vmul(m0, 0x1.c71c720000000p-6f)))))), o = vfma(-0x1.0000000000000p-3f, m18, vfma(0x1.0000000000000p-3f, m17, vfma(0x1.5555560000000p-5f, m8, vfma(0x1.5555560000000p-4f, m7, vfma(0x1.5555560000000p-5f, m6, vmul(m5, 0x1.5555560000000p-4f)))))); out[15] = vadd(e, o); out[16] = vsub(e, o); }
  { const V e = vfma(-0x1.0000000000000p-2f, m14, vfma(-0x1.5555560000000p-5f, m10, vfma(-0x1.5555560000000p-5f, m9, vfma(0x1.c71c720000000p-7f, m2, vfma(0x1.5555560000000p-5f, m1, vmul(m0, 0x1.c71c720000000p-6f)))))), o = vfma(0x1.0000000000000p-3f, m18, vfma(0x1.0000000000000p-3f, m17, vfma(-0x1.5555560000000p-5f, m8, vfma(-0x1.5555560000000p-4f, m7, vfma(0x1.5555560000000p-5f, m6, vmul(m5, 0x1.5555560000000p-4f)))))); out[17] = vadd(e, o); out[18] = vsub(e, o); }
}
}  // namespace fsi
