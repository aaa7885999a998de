// GENERATED by gen_lbm_formulas.py -- do not edit by hand.
// D3Q19 MRT collision of the reference (fsi/lbm3d.py:269-333) as explicit
// register formulas with the reference's float32 operation order.
#pragma once

namespace fsi {

// m[k] = sum_q M[k][q] * X[q], sequential in q (lbm3d.py:269-274).
__device__ __forceinline__ void mrt_forward(const float (&X)[19], float (&m)[19]) {
  float two[19];
  two[1] = __fadd_rn(X[1], X[1]);
  two[2] = __fadd_rn(X[2], X[2]);
  two[3] = __fadd_rn(X[3], X[3]);
  two[4] = __fadd_rn(X[4], X[4]);
  two[5] = __fadd_rn(X[5], X[5]);
  two[6] = __fadd_rn(X[6], X[6]);
  two[15] = __fadd_rn(X[15], X[15]);
  two[16] = __fadd_rn(X[16], X[16]);
  two[17] = __fadd_rn(X[17], X[17]);
  two[18] = __fadd_rn(X[18], X[18]);
  m[0] = X[0]; m[0] = __fadd_rn(m[0], X[1]); m[0] = __fadd_rn(m[0], X[2]); m[0] = __fadd_rn(m[0], X[3]); m[0] = __fadd_rn(m[0], X[4]); m[0] = __fadd_rn(m[0], X[5]); m[0] = __fadd_rn(m[0], X[6]); m[0] = __fadd_rn(m[0], X[7]); m[0] = __fadd_rn(m[0], X[8]); m[0] = __fadd_rn(m[0], X[9]); m[0] = __fadd_rn(m[0], X[10]); m[0] = __fadd_rn(m[0], X[11]); m[0] = __fadd_rn(m[0], X[12]); m[0] = __fadd_rn(m[0], X[13]); m[0] = __fadd_rn(m[0], X[14]); m[0] = __fadd_rn(m[0], X[15]); m[0] = __fadd_rn(m[0], X[16]); m[0] = __fadd_rn(m[0], X[17]); m[0] = __fadd_rn(m[0], X[18]);
  m[1] = -X[0]; m[1] = __fadd_rn(m[1], X[7]); m[1] = __fadd_rn(m[1], X[8]); m[1] = __fadd_rn(m[1], X[9]); m[1] = __fadd_rn(m[1], X[10]); m[1] = __fadd_rn(m[1], X[11]); m[1] = __fadd_rn(m[1], X[12]); m[1] = __fadd_rn(m[1], X[13]); m[1] = __fadd_rn(m[1], X[14]); m[1] = __fadd_rn(m[1], X[15]); m[1] = __fadd_rn(m[1], X[16]); m[1] = __fadd_rn(m[1], X[17]); m[1] = __fadd_rn(m[1], X[18]);
  m[2] = X[0]; m[2] = __fsub_rn(m[2], two[1]); m[2] = __fsub_rn(m[2], two[2]); m[2] = __fsub_rn(m[2], two[3]); m[2] = __fsub_rn(m[2], two[4]); m[2] = __fsub_rn(m[2], two[5]); m[2] = __fsub_rn(m[2], two[6]); m[2] = __fadd_rn(m[2], X[7]); m[2] = __fadd_rn(m[2], X[8]); m[2] = __fadd_rn(m[2], X[9]); m[2] = __fadd_rn(m[2], X[10]); m[2] = __fadd_rn(m[2], X[11]); m[2] = __fadd_rn(m[2], X[12]); m[2] = __fadd_rn(m[2], X[13]); m[2] = __fadd_rn(m[2], X[14]); m[2] = __fadd_rn(m[2], X[15]); m[2] = __fadd_rn(m[2], X[16]); m[2] = __fadd_rn(m[2], X[17]); m[2] = __fadd_rn(m[2], X[18]);
  m[3] = X[1]; m[3] = __fsub_rn(m[3], X[2]); m[3] = __fadd_rn(m[3], X[7]); m[3] = __fsub_rn(m[3], X[8]); m[3] = __fadd_rn(m[3], X[9]); m[3] = __fsub_rn(m[3], X[10]); m[3] = __fadd_rn(m[3], X[11]); m[3] = __fsub_rn(m[3], X[12]); m[3] = __fadd_rn(m[3], X[13]); m[3] = __fsub_rn(m[3], X[14]);
  m[4] = -two[1]; m[4] = __fadd_rn(m[4], two[2]); m[4] = __fadd_rn(m[4], X[7]); m[4] = __fsub_rn(m[4], X[8]); m[4] = __fadd_rn(m[4], X[9]); m[4] = __fsub_rn(m[4], X[10]); m[4] = __fadd_rn(m[4], X[11]); m[4] = __fsub_rn(m[4], X[12]); m[4] = __fadd_rn(m[4], X[13]); m[4] = __fsub_rn(m[4], X[14]);
  m[5] = X[3]; m[5] = __fsub_rn(m[5], X[4]); m[5] = __fadd_rn(m[5], X[7]); m[5] = __fsub_rn(m[5], X[8]); m[5] = __fsub_rn(m[5], X[9]); m[5] = __fadd_rn(m[5], X[10]); m[5] = __fadd_rn(m[5], X[15]); m[5] = __fsub_rn(m[5], X[16]); m[5] = __fadd_rn(m[5], X[17]); m[5] = __fsub_rn(m[5], X[18]);
  m[6] = -two[3]; m[6] = __fadd_rn(m[6], two[4]); m[6] = __fadd_rn(m[6], X[7]); m[6] = __fsub_rn(m[6], X[8]); m[6] = __fsub_rn(m[6], X[9]); m[6] = __fadd_rn(m[6], X[10]); m[6] = __fadd_rn(m[6], X[15]); m[6] = __fsub_rn(m[6], X[16]); m[6] = __fadd_rn(m[6], X[17]); m[6] = __fsub_rn(m[6], X[18]);
  m[7] = X[5]; m[7] = __fsub_rn(m[7], X[6]); m[7] = __fadd_rn(m[7], X[11]); m[7] = __fsub_rn(m[7], X[12]); m[7] = __fsub_rn(m[7], X[13]); m[7] = __fadd_rn(m[7], X[14]); m[7] = __fadd_rn(m[7], X[15]); m[7] = __fsub_rn(m[7], X[16]); m[7] = __fsub_rn(m[7], X[17]); m[7] = __fadd_rn(m[7], X[18]);
  m[8] = -two[5]; m[8] = __fadd_rn(m[8], two[6]); m[8] = __fadd_rn(m[8], X[11]); m[8] = __fsub_rn(m[8], X[12]); m[8] = __fsub_rn(m[8], X[13]); m[8] = __fadd_rn(m[8], X[14]); m[8] = __fadd_rn(m[8], X[15]); m[8] = __fsub_rn(m[8], X[16]); m[8] = __fsub_rn(m[8], X[17]); m[8] = __fadd_rn(m[8], X[18]);
  m[9] = two[1]; m[9] = __fadd_rn(m[9], two[2]); m[9] = __fsub_rn(m[9], X[3]); m[9] = __fsub_rn(m[9], X[4]); m[9] = __fsub_rn(m[9], X[5]); m[9] = __fsub_rn(m[9], X[6]); m[9] = __fadd_rn(m[9], X[7]); m[9] = __fadd_rn(m[9], X[8]); m[9] = __fadd_rn(m[9], X[9]); m[9] = __fadd_rn(m[9], X[10]); m[9] = __fadd_rn(m[9], X[11]); m[9] = __fadd_rn(m[9], X[12]); m[9] = __fadd_rn(m[9], X[13]); m[9] = __fadd_rn(m[9], X[14]); m[9] = __fsub_rn(m[9], two[15]); m[9] = __fsub_rn(m[9], two[16]); m[9] = __fsub_rn(m[9], two[17]); m[9] = __fsub_rn(m[9], two[18]);
  m[10] = -two[1]; m[10] = __fsub_rn(m[10], two[2]); m[10] = __fadd_rn(m[10], X[3]); m[10] = __fadd_rn(m[10], X[4]); m[10] = __fadd_rn(m[10], X[5]); m[10] = __fadd_rn(m[10], X[6]); m[10] = __fadd_rn(m[10], X[7]); m[10] = __fadd_rn(m[10], X[8]); m[10] = __fadd_rn(m[10], X[9]); m[10] = __fadd_rn(m[10], X[10]); m[10] = __fadd_rn(m[10], X[11]); m[10] = __fadd_rn(m[10], X[12]); m[10] = __fadd_rn(m[10], X[13]); m[10] = __fadd_rn(m[10], X[14]); m[10] = __fsub_rn(m[10], two[15]); m[10] = __fsub_rn(m[10], two[16]); m[10] = __fsub_rn(m[10], two[17]); m[10] = __fsub_rn(m[10], two[18]);
  m[11] = X[3]; m[11] = __fadd_rn(m[11], X[4]); m[11] = __fsub_rn(m[11], X[5]); m[11] = __fsub_rn(m[11], X[6]); m[11] = __fadd_rn(m[11], X[7]); m[11] = __fadd_rn(m[11], X[8]); m[11] = __fadd_rn(m[11], X[9]); m[11] = __fadd_rn(m[11], X[10]); m[11] = __fsub_rn(m[11], X[11]); m[11] = __fsub_rn(m[11], X[12]); m[11] = __fsub_rn(m[11], X[13]); m[11] = __fsub_rn(m[11], X[14]);
  m[12] = -X[3]; m[12] = __fsub_rn(m[12], X[4]); m[12] = __fadd_rn(m[12], X[5]); m[12] = __fadd_rn(m[12], X[6]); m[12] = __fadd_rn(m[12], X[7]); m[12] = __fadd_rn(m[12], X[8]); m[12] = __fadd_rn(m[12], X[9]); m[12] = __fadd_rn(m[12], X[10]); m[12] = __fsub_rn(m[12], X[11]); m[12] = __fsub_rn(m[12], X[12]); m[12] = __fsub_rn(m[12], X[13]); m[12] = __fsub_rn(m[12], X[14]);
  m[13] = X[7]; m[13] = __fadd_rn(m[13], X[8]); m[13] = __fsub_rn(m[13], X[9]); m[13] = __fsub_rn(m[13], X[10]);
  m[14] = X[15]; m[14] = __fadd_rn(m[14], X[16]); m[14] = __fsub_rn(m[14], X[17]); m[14] = __fsub_rn(m[14], X[18]);
  m[15] = X[11]; m[15] = __fadd_rn(m[15], X[12]); m[15] = __fsub_rn(m[15], X[13]); m[15] = __fsub_rn(m[15], X[14]);
  m[16] = X[7]; m[16] = __fsub_rn(m[16], X[8]); m[16] = __fadd_rn(m[16], X[9]); m[16] = __fsub_rn(m[16], X[10]); m[16] = __fsub_rn(m[16], X[11]); m[16] = __fadd_rn(m[16], X[12]); m[16] = __fsub_rn(m[16], X[13]); m[16] = __fadd_rn(m[16], X[14]);
  m[17] = -X[7]; m[17] = __fadd_rn(m[17], X[8]); m[17] = __fadd_rn(m[17], X[9]); m[17] = __fsub_rn(m[17], X[10]); m[17] = __fadd_rn(m[17], X[15]); m[17] = __fsub_rn(m[17], X[16]); m[17] = __fadd_rn(m[17], X[17]); m[17] = __fsub_rn(m[17], X[18]);
  m[18] = X[11]; m[18] = __fsub_rn(m[18], X[12]); m[18] = __fsub_rn(m[18], X[13]); m[18] = __fadd_rn(m[18], X[14]); m[18] = __fsub_rn(m[18], X[15]); m[18] = __fadd_rn(m[18], X[16]); m[18] = __fadd_rn(m[18], X[17]); m[18] = __fsub_rn(m[18], X[18]);
}

// f[q] = sum_k inv(M)[q][k] * m[k], sequential in k (lbm3d.py:328-333).
// 22 rounded products; every other product is an exact power-of-two scaling.
__device__ __forceinline__ void mrt_inverse(const float (&m)[19], float (&f)[19]) {
  const float p0_0 = __fmul_rn(0x1.5555560000000p-2f, m[0]);
  const float p0_1 = __fmul_rn(0x1.c71c720000000p-5f, m[0]);
  const float p1_0 = __fmul_rn(0x1.0000000000000p-1f, m[1]);
  const float p1_1 = __fmul_rn(0x1.5555560000000p-5f, m[1]);
  const float p2_0 = __fmul_rn(0x1.5555560000000p-3f, m[2]);
  const float p2_1 = __fmul_rn(0x1.c71c720000000p-5f, m[2]);
  const float p3_0 = __fmul_rn(0x1.5555560000000p-3f, m[3]);
  const float p4_0 = __fmul_rn(0x1.5555560000000p-3f, m[4]);
  const float p5_0 = __fmul_rn(0x1.5555560000000p-3f, m[5]);
  const float p6_0 = __fmul_rn(0x1.5555560000000p-3f, m[6]);
  const float p7_0 = __fmul_rn(0x1.5555560000000p-3f, m[7]);
  const float p8_0 = __fmul_rn(0x1.5555560000000p-3f, m[8]);
  const float p9_0 = __fmul_rn(0x1.5555560000000p-4f, m[9]);
  const float p10_0 = __fmul_rn(0x1.5555560000000p-4f, m[10]);
  const float p11_0 = __fmul_rn(0x1.0000000000000p-3f, m[11]);
  const float p12_0 = __fmul_rn(0x1.0000000000000p-3f, m[12]);
  const float p13_0 = __fmul_rn(0x1.0000000000000p-2f, m[13]);
  const float p14_0 = __fmul_rn(0x1.0000000000000p-2f, m[14]);
  const float p15_0 = __fmul_rn(0x1.0000000000000p-2f, m[15]);
  const float p16_0 = __fmul_rn(0x1.0000000000000p-3f, m[16]);
  const float p17_0 = __fmul_rn(0x1.0000000000000p-3f, m[17]);
  const float p18_0 = __fmul_rn(0x1.0000000000000p-3f, m[18]);
  { float a; a = p0_0; a = __fsub_rn(a, p1_0); a = __fadd_rn(a, p2_0); f[0] = a; }
  { float a; a = p0_1; a = __fsub_rn(a, p2_1); a = __fadd_rn(a, p3_0); a = __fsub_rn(a, p4_0); a = __fadd_rn(a, p9_0); a = __fsub_rn(a, p10_0); f[1] = a; }
  { float a; a = p0_1; a = __fsub_rn(a, p2_1); a = __fsub_rn(a, p3_0); a = __fadd_rn(a, p4_0); a = __fadd_rn(a, p9_0); a = __fsub_rn(a, p10_0); f[2] = a; }
  { float a; a = p0_1; a = __fsub_rn(a, p2_1); a = __fadd_rn(a, p5_0); a = __fsub_rn(a, p6_0); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p11_0); a = __fsub_rn(a, p12_0); f[3] = a; }
  { float a; a = p0_1; a = __fsub_rn(a, p2_1); a = __fsub_rn(a, p5_0); a = __fadd_rn(a, p6_0); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p11_0); a = __fsub_rn(a, p12_0); f[4] = a; }
  { float a; a = p0_1; a = __fsub_rn(a, p2_1); a = __fadd_rn(a, p7_0); a = __fsub_rn(a, p8_0); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p11_0); a = __fadd_rn(a, p12_0); f[5] = a; }
  { float a; a = p0_1; a = __fsub_rn(a, p2_1); a = __fsub_rn(a, p7_0); a = __fadd_rn(a, p8_0); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p11_0); a = __fadd_rn(a, p12_0); f[6] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p13_0); a = __fadd_rn(a, p16_0); a = __fsub_rn(a, p17_0); f[7] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p13_0); a = __fsub_rn(a, p16_0); a = __fadd_rn(a, p17_0); f[8] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p13_0); a = __fadd_rn(a, p16_0); a = __fadd_rn(a, p17_0); f[9] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p13_0); a = __fsub_rn(a, p16_0); a = __fsub_rn(a, p17_0); f[10] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p15_0); a = __fsub_rn(a, p16_0); a = __fadd_rn(a, p18_0); f[11] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p15_0); a = __fadd_rn(a, p16_0); a = __fsub_rn(a, p18_0); f[12] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p15_0); a = __fsub_rn(a, p16_0); a = __fsub_rn(a, p18_0); f[13] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p3_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p4_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p11_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p12_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p15_0); a = __fadd_rn(a, p16_0); a = __fadd_rn(a, p18_0); f[14] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p14_0); a = __fadd_rn(a, p17_0); a = __fsub_rn(a, p18_0); f[15] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, p14_0); a = __fsub_rn(a, p17_0); a = __fadd_rn(a, p18_0); f[16] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p14_0); a = __fadd_rn(a, p17_0); a = __fadd_rn(a, p18_0); f[17] = a; }
  { float a; a = __fmul_rn(p0_1, 0x1.0000000000000p-1f); a = __fadd_rn(a, p1_1); a = __fadd_rn(a, __fmul_rn(p2_1, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p5_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p6_0, 0x1.0000000000000p-2f)); a = __fadd_rn(a, __fmul_rn(p7_0, 0x1.0000000000000p-1f)); a = __fadd_rn(a, __fmul_rn(p8_0, 0x1.0000000000000p-2f)); a = __fsub_rn(a, __fmul_rn(p9_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, __fmul_rn(p10_0, 0x1.0000000000000p-1f)); a = __fsub_rn(a, p14_0); a = __fsub_rn(a, p17_0); a = __fsub_rn(a, p18_0); f[18] = a; }
}


// Reduced-operation MRT + Guo collision (same operator, not the reference's rounding):
// parity-split moments from pair sums/differences, closed-form forcing moments
// g_k = A_k.G - B_k (u.G) + u^T C_k G, parity-split inverse. Used by the FP16/BF16
// storage forms and the FP32 fast form.
__device__ __forceinline__ void mrt_collide_fast(const float (&F)[19], float rho, float ux,
    float uy, float uz, float gx, float gy, float gz, const float* __restrict__ S,
    float (&out)[19]) {
  const float P0 = F[1] + F[2], D0 = F[1] - F[2];
  const float P1 = F[3] + F[4], D1 = F[3] - F[4];
  const float P2 = F[5] + F[6], D2 = F[5] - F[6];
  const float P3 = F[7] + F[8], D3 = F[7] - F[8];
  const float P4 = F[9] + F[10], D4 = F[9] - F[10];
  const float P5 = F[11] + F[12], D5 = F[11] - F[12];
  const float P6 = F[13] + F[14], D6 = F[13] - F[14];
  const float P7 = F[15] + F[16], D7 = F[15] - F[16];
  const float P8 = F[17] + F[18], D8 = F[17] - F[18];
  float m0 = (((((((((F[0] + P0) + P1) + P2) + P3) + P4) + P5) + P6) + P7) + P8);
  float m1 = ((((((-F[0] + P3) + P4) + P5) + P6) + P7) + P8);
  float m2 = ((((((fmaf(-0x1.0000000000000p+1f, P2, fmaf(-0x1.0000000000000p+1f, P1, fmaf(-0x1.0000000000000p+1f, P0, F[0]))) + P3) + P4) + P5) + P6) + P7) + P8);
  float m9 = fmaf(-0x1.0000000000000p+1f, P8, fmaf(-0x1.0000000000000p+1f, P7, (((((((0x1.0000000000000p+1f * P0) - P1) - P2) + P3) + P4) + P5) + P6)));
  float m10 = fmaf(-0x1.0000000000000p+1f, P8, fmaf(-0x1.0000000000000p+1f, P7, (((((((-0x1.0000000000000p+1f * P0) + P1) + P2) + P3) + P4) + P5) + P6)));
  float m11 = (((((P1 - P2) + P3) + P4) - P5) - P6);
  float m12 = (((((-P1 + P2) + P3) + P4) - P5) - P6);
  float m13 = (P3 - P4);
  float m14 = (P7 - P8);
  float m15 = (P5 - P6);
  float m3 = ((((D0 + D3) + D4) + D5) + D6);
  float m4 = (((((-0x1.0000000000000p+1f * D0) + D3) + D4) + D5) + D6);
  float m5 = ((((D1 + D3) - D4) + D7) + D8);
  float m6 = (((((-0x1.0000000000000p+1f * D1) + D3) - D4) + D7) + D8);
  float m7 = ((((D2 + D5) - D6) + D7) - D8);
  float m8 = (((((-0x1.0000000000000p+1f * D2) + D5) - D6) + D7) - D8);
  float m16 = (((D3 + D4) - D5) - D6);
  float m17 = (((-D3 + D4) + D7) + D8);
  float m18 = (((D5 - D6) - D7) + D8);
  const float uG = fmaf(ux, gx, fmaf(uy, gy, uz * gz));
  const float pxx = ux * gx, pyy = uy * gy, pzz = uz * gz;
  const float sxy = fmaf(ux, gy, uy * gx), syz = fmaf(uy, gz, uz * gy), sxz = fmaf(ux, gz, uz * gx);
  const float g0 = fmaf(0x1.5555560000000p-2f, pzz, fmaf(0x1.5555560000000p-2f, pyy, fmaf(0x1.5555560000000p-2f, pxx, -uG)));
  const float g1 = fmaf(0x1.c71c720000000p-3f, pzz, fmaf(0x1.c71c720000000p-3f, pyy, (0x1.c71c720000000p-3f * pxx)));
  const float g3 = (0x1.5555560000000p-2f * gx);
  const float g5 = (0x1.5555560000000p-2f * gy);
  const float g7 = (0x1.5555560000000p-2f * gz);
  const float g9 = fmaf(-0x1.c71c720000000p-3f, pzz, fmaf(-0x1.c71c720000000p-3f, pyy, (0x1.c71c720000000p-2f * pxx)));
  const float g11 = fmaf(-0x1.c71c720000000p-3f, pzz, (0x1.c71c720000000p-3f * pyy));
  const float g13 = (0x1.c71c720000000p-4f * sxy);
  const float g14 = (0x1.c71c720000000p-4f * syz);
  const float g15 = (0x1.c71c720000000p-4f * sxz);
  const float uu = fmaf(ux, ux, fmaf(uy, uy, uz * uz));
  m0 = m0 + g0;
  m1 = fmaf(fmaf(-0.5f, S[1], 1.0f), g1, fmaf(-S[1], (m1 - (uu)), m1));
  m2 = fmaf(-S[2], m2, m2);
  m3 = m3 + g3;
  m4 = fmaf(-S[4], m4, m4);
  m5 = m5 + g5;
  m6 = fmaf(-S[6], m6, m6);
  m7 = m7 + g7;
  m8 = fmaf(-S[8], m8, m8);
  m9 = fmaf(fmaf(-0.5f, S[9], 1.0f), g9, fmaf(-S[9], (m9 - (fmaf(2.0f * ux, ux, -fmaf(uy, uy, uz * uz)))), m9));
  m10 = fmaf(-S[10], m10, m10);
  m11 = fmaf(fmaf(-0.5f, S[11], 1.0f), g11, fmaf(-S[11], (m11 - (fmaf(uy, uy, -(uz * uz)))), m11));
  m12 = fmaf(-S[12], m12, m12);
  m13 = fmaf(fmaf(-0.5f, S[13], 1.0f), g13, fmaf(-S[13], (m13 - (ux * uy)), m13));
  m14 = fmaf(fmaf(-0.5f, S[14], 1.0f), g14, fmaf(-S[14], (m14 - (uy * uz)), m14));
  m15 = fmaf(fmaf(-0.5f, S[15], 1.0f), g15, fmaf(-S[15], (m15 - (ux * uz)), m15));
  m16 = fmaf(-S[16], m16, m16);
  m17 = fmaf(-S[17], m17, m17);
  m18 = fmaf(-S[18], m18, m18);
  out[0] = fmaf(0x1.5555560000000p-3f, m2, fmaf(-0x1.0000000000000p-1f, m1, (0x1.5555560000000p-2f * m0)));
  { const float e = fmaf(-0x1.5555560000000p-4f, m10, fmaf(0x1.5555560000000p-4f, m9, fmaf(-0x1.c71c720000000p-5f, m2, (0x1.c71c720000000p-5f * m0)))), o = fmaf(-0x1.5555560000000p-3f, m4, (0x1.5555560000000p-3f * m3)); out[1] = e + o; out[2] = e - o; }
  { const float e = fmaf(-0x1.0000000000000p-3f, m12, fmaf(0x1.0000000000000p-3f, m11, fmaf(0x1.5555560000000p-5f, m10, fmaf(-0x1.5555560000000p-5f, m9, fmaf(-0x1.c71c720000000p-5f, m2, (0x1.c71c720000000p-5f * m0)))))), o = fmaf(-0x1.5555560000000p-3f, m6, (0x1.5555560000000p-3f * m5)); out[3] = e + o; out[4] = e - o; }
  { const float e = fmaf(0x1.0000000000000p-3f, m12, fmaf(-0x1.0000000000000p-3f, m11, fmaf(0x1.5555560000000p-5f, m10, fmaf(-0x1.5555560000000p-5f, m9, fmaf(-0x1.c71c720000000p-5f, m2, (0x1.c71c720000000p-5f * m0)))))), o = fmaf(-0x1.5555560000000p-3f, m8, (0x1.5555560000000p-3f * m7)); out[5] = e + o; out[6] = e - o; }
  { const float e = fmaf(0x1.0000000000000p-2f, m13, fmaf(0x1.0000000000000p-4f, m12, fmaf(0x1.0000000000000p-4f, m11, fmaf(0x1.5555560000000p-6f, m10, fmaf(0x1.5555560000000p-6f, m9, fmaf(0x1.c71c720000000p-7f, m2, fmaf(0x1.5555560000000p-5f, m1, (0x1.c71c720000000p-6f * m0)))))))), o = fmaf(-0x1.0000000000000p-3f, m17, fmaf(0x1.0000000000000p-3f, m16, fmaf(0x1.5555560000000p-5f, m6, fmaf(0x1.5555560000000p-4f, m5, fmaf(0x1.5555560000000p-5f, m4, (0x1.5555560000000p-4f * m3)))))); out[7] = e + o; out[8] = e - o; }
  { const float e = fmaf(-0x1.0000000000000p-2f, m13, fmaf(0x1.0000000000000p-4f, m12, fmaf(0x1.0000000000000p-4f, m11, fmaf(0x1.5555560000000p-6f, m10, fmaf(0x1.5555560000000p-6f, m9, fmaf(0x1.c71c720000000p-7f, m2, fmaf(0x1.5555560000000p-5f, m1, (0x1.c71c720000000p-6f * m0)))))))), o = fmaf(0x1.0000000000000p-3f, m17, fmaf(0x1.0000000000000p-3f, m16, fmaf(-0x1.5555560000000p-5f, m6, fmaf(-0x1.5555560000000p-4f, m5, fmaf(0x1.5555560000000p-5f, m4, (0x1.5555560000000p-4f * m3)))))); out[9] = e + o; out[10] = e - o; }
  { const float e = fmaf(0x1.0000000000000p-2f, m15, fmaf(-0x1.0000000000000p-4f, m12, fmaf(-0x1.0000000000000p-4f, m11, fmaf(0x1.5555560000000p-6f, m10, fmaf(0x1.5555560000000p-6f, m9, fmaf(0x1.c71c720000000p-7f, m2, fmaf(0x1.5555560000000p-5f, m1, (0x1.c71c720000000p-6f * m0)))))))), o = fmaf(0x1.0000000000000p-3f, m18, fmaf(-0x1.0000000000000p-3f, m16, fmaf(0x1.5555560000000p-5f, m8, fmaf(0x1.5555560000000p-4f, m7, fmaf(0x1.5555560000000p-5f, m4, (0x1.5555560000000p-4f * m3)))))); out[11] = e + o; out[12] = e - o; }
  { const float e = fmaf(-0x1.0000000000000p-2f, m15, fmaf(-0x1.0000000000000p-4f, m12, fmaf(-0x1.0000000000000p-4f, m11, fmaf(0x1.5555560000000p-6f, m10, fmaf(0x1.5555560000000p-6f, m9, fmaf(0x1.c71c720000000p-7f, m2, fmaf(0x1.5555560000000p-5f, m1, (0x1.c71c720000000p-6f * m0)))))))), o = fmaf(-0x1.0000000000000p-3f, m18, fmaf(-0x1.0000000000000p-3f, m16, fmaf(-0x1.5555560000000p-5f, m8, fmaf(-0x1.5555560000000p-4f, m7, fmaf(0x1.5555560000000p-5f, m4, (0x1.5555560000000p-4f * m3)))))); out[13] = e + o; out[14] = e - o; }
  { const float e = fmaf(0x1.0000000000000p-2f, m14, fmaf(-0x1.5555560000000p-5f, m10, fmaf(-0x1.5555560000000p-5f, m9, fmaf(0x1.c71c720000000p-7f, m2, fmaf(0x1.5555560000000p-5f, m1, (0x1.c71c720000000p-6f * m0)))))), o = fmaf(-0x1.0000000000000p-3f, m18, fmaf(0x1.0000000000000p-3f, m17, fmaf(0x1.5555560000000p-5f, m8, fmaf(0x1.5555560000000p-4f, m7, fmaf(0x1.5555560000000p-5f, m6, (0x1.5555560000000p-4f * m5)))))); out[15] = e + o; out[16] = e - o; }
  { const float e = fmaf(-0x1.0000000000000p-2f, m14, fmaf(-0x1.5555560000000p-5f, m10, fmaf(-0x1.5555560000000p-5f, m9, fmaf(0x1.c71c720000000p-7f, m2, fmaf(0x1.5555560000000p-5f, m1, (0x1.c71c720000000p-6f * m0)))))), o = fmaf(0x1.0000000000000p-3f, m18, fmaf(0x1.0000000000000p-3f, m17, fmaf(-0x1.5555560000000p-5f, m8, fmaf(-0x1.5555560000000p-4f, m7, fmaf(0x1.5555560000000p-5f, m6, (0x1.5555560000000p-4f * m5)))))); out[17] = e + o; out[18] = e - o; }
}
}  // namespace fsi
