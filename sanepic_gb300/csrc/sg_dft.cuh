// Generated by gen_dft.py -- do not edit.
// In-register unnormalised DFTs of size 2..32 (radix-2 DIT, literal twiddles).
#pragma once
#include "sg_cplx.cuh"

template <typename T>
__device__ __forceinline__ void sg_dft2_fwd(cplx<T> (&a)[2]) {
  cplx<T> b[2];
  b[0] = a[0];
  b[1] = a[1];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  a[0] = b[0];
  a[1] = b[1];
}

template <typename T>
__device__ __forceinline__ void sg_dft2_bwd(cplx<T> (&a)[2]) {
  cplx<T> b[2];
  b[0] = a[0];
  b[1] = a[1];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  a[0] = b[0];
  a[1] = b[1];
}

template <typename T>
__device__ __forceinline__ void sg_dft4_fwd(cplx<T> (&a)[4]) {
  cplx<T> b[4];
  b[0] = a[0];
  b[1] = a[2];
  b[2] = a[1];
  b[3] = a[3];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{b[3].y, -b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
}

template <typename T>
__device__ __forceinline__ void sg_dft4_bwd(cplx<T> (&a)[4]) {
  cplx<T> b[4];
  b[0] = a[0];
  b[1] = a[2];
  b[2] = a[1];
  b[3] = a[3];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{-b[3].y, b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
}

template <typename T>
__device__ __forceinline__ void sg_dft8_fwd(cplx<T> (&a)[8]) {
  cplx<T> b[8];
  b[0] = a[0];
  b[1] = a[4];
  b[2] = a[2];
  b[3] = a[6];
  b[4] = a[1];
  b[5] = a[5];
  b[6] = a[3];
  b[7] = a[7];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[5]; b[5] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = b[7]; b[7] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{b[3].y, -b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = b[6]; b[6] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cplx<T>{b[7].y, -b[7].x}; b[7] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = b[4]; b[4] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[5], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[5] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cplx<T>{b[6].y, -b[6].x}; b[6] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[7], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[7] = b[3] - t; b[3] = b[3] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
  a[4] = b[4];
  a[5] = b[5];
  a[6] = b[6];
  a[7] = b[7];
}

template <typename T>
__device__ __forceinline__ void sg_dft8_bwd(cplx<T> (&a)[8]) {
  cplx<T> b[8];
  b[0] = a[0];
  b[1] = a[4];
  b[2] = a[2];
  b[3] = a[6];
  b[4] = a[1];
  b[5] = a[5];
  b[6] = a[3];
  b[7] = a[7];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[5]; b[5] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = b[7]; b[7] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{-b[3].y, b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = b[6]; b[6] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cplx<T>{-b[7].y, b[7].x}; b[7] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = b[4]; b[4] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[5], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[5] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cplx<T>{-b[6].y, b[6].x}; b[6] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[7], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[7] = b[3] - t; b[3] = b[3] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
  a[4] = b[4];
  a[5] = b[5];
  a[6] = b[6];
  a[7] = b[7];
}

template <typename T>
__device__ __forceinline__ void sg_dft16_fwd(cplx<T> (&a)[16]) {
  cplx<T> b[16];
  b[0] = a[0];
  b[1] = a[8];
  b[2] = a[4];
  b[3] = a[12];
  b[4] = a[2];
  b[5] = a[10];
  b[6] = a[6];
  b[7] = a[14];
  b[8] = a[1];
  b[9] = a[9];
  b[10] = a[5];
  b[11] = a[13];
  b[12] = a[3];
  b[13] = a[11];
  b[14] = a[7];
  b[15] = a[15];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[5]; b[5] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = b[7]; b[7] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = b[9]; b[9] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = b[11]; b[11] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = b[13]; b[13] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = b[15]; b[15] = b[14] - t; b[14] = b[14] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{b[3].y, -b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = b[6]; b[6] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cplx<T>{b[7].y, -b[7].x}; b[7] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = b[10]; b[10] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cplx<T>{b[11].y, -b[11].x}; b[11] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = b[14]; b[14] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = cplx<T>{b[15].y, -b[15].x}; b[15] = b[13] - t; b[13] = b[13] + t; }
  { cplx<T> t = b[4]; b[4] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[5], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[5] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cplx<T>{b[6].y, -b[6].x}; b[6] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[7], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[7] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = b[12]; b[12] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[13] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = cplx<T>{b[14].y, -b[14].x}; b[14] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[15] = b[11] - t; b[11] = b[11] + t; }
  { cplx<T> t = b[8]; b[8] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[9], cplx<T>{T(0.9238795325112867), T(-0.3826834323650898)}); b[9] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cmul(b[10], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[10] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[11], cplx<T>{T(0.38268343236508984), T(-0.9238795325112867)}); b[11] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = cplx<T>{b[12].y, -b[12].x}; b[12] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(-0.3826834323650897), T(-0.9238795325112867)}); b[13] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = cmul(b[14], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[14] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.9238795325112867), T(-0.3826834323650899)}); b[15] = b[7] - t; b[7] = b[7] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
  a[4] = b[4];
  a[5] = b[5];
  a[6] = b[6];
  a[7] = b[7];
  a[8] = b[8];
  a[9] = b[9];
  a[10] = b[10];
  a[11] = b[11];
  a[12] = b[12];
  a[13] = b[13];
  a[14] = b[14];
  a[15] = b[15];
}

template <typename T>
__device__ __forceinline__ void sg_dft16_bwd(cplx<T> (&a)[16]) {
  cplx<T> b[16];
  b[0] = a[0];
  b[1] = a[8];
  b[2] = a[4];
  b[3] = a[12];
  b[4] = a[2];
  b[5] = a[10];
  b[6] = a[6];
  b[7] = a[14];
  b[8] = a[1];
  b[9] = a[9];
  b[10] = a[5];
  b[11] = a[13];
  b[12] = a[3];
  b[13] = a[11];
  b[14] = a[7];
  b[15] = a[15];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[5]; b[5] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = b[7]; b[7] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = b[9]; b[9] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = b[11]; b[11] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = b[13]; b[13] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = b[15]; b[15] = b[14] - t; b[14] = b[14] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{-b[3].y, b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = b[6]; b[6] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cplx<T>{-b[7].y, b[7].x}; b[7] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = b[10]; b[10] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cplx<T>{-b[11].y, b[11].x}; b[11] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = b[14]; b[14] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = cplx<T>{-b[15].y, b[15].x}; b[15] = b[13] - t; b[13] = b[13] + t; }
  { cplx<T> t = b[4]; b[4] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[5], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[5] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cplx<T>{-b[6].y, b[6].x}; b[6] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[7], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[7] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = b[12]; b[12] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[13] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = cplx<T>{-b[14].y, b[14].x}; b[14] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[15] = b[11] - t; b[11] = b[11] + t; }
  { cplx<T> t = b[8]; b[8] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[9], cplx<T>{T(0.9238795325112867), T(0.3826834323650898)}); b[9] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cmul(b[10], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[10] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[11], cplx<T>{T(0.38268343236508984), T(0.9238795325112867)}); b[11] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = cplx<T>{-b[12].y, b[12].x}; b[12] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(-0.3826834323650897), T(0.9238795325112867)}); b[13] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = cmul(b[14], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[14] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.9238795325112867), T(0.3826834323650899)}); b[15] = b[7] - t; b[7] = b[7] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
  a[4] = b[4];
  a[5] = b[5];
  a[6] = b[6];
  a[7] = b[7];
  a[8] = b[8];
  a[9] = b[9];
  a[10] = b[10];
  a[11] = b[11];
  a[12] = b[12];
  a[13] = b[13];
  a[14] = b[14];
  a[15] = b[15];
}

template <typename T>
__device__ __forceinline__ void sg_dft32_fwd(cplx<T> (&a)[32]) {
  cplx<T> b[32];
  b[0] = a[0];
  b[1] = a[16];
  b[2] = a[8];
  b[3] = a[24];
  b[4] = a[4];
  b[5] = a[20];
  b[6] = a[12];
  b[7] = a[28];
  b[8] = a[2];
  b[9] = a[18];
  b[10] = a[10];
  b[11] = a[26];
  b[12] = a[6];
  b[13] = a[22];
  b[14] = a[14];
  b[15] = a[30];
  b[16] = a[1];
  b[17] = a[17];
  b[18] = a[9];
  b[19] = a[25];
  b[20] = a[5];
  b[21] = a[21];
  b[22] = a[13];
  b[23] = a[29];
  b[24] = a[3];
  b[25] = a[19];
  b[26] = a[11];
  b[27] = a[27];
  b[28] = a[7];
  b[29] = a[23];
  b[30] = a[15];
  b[31] = a[31];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[5]; b[5] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = b[7]; b[7] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = b[9]; b[9] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = b[11]; b[11] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = b[13]; b[13] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = b[15]; b[15] = b[14] - t; b[14] = b[14] + t; }
  { cplx<T> t = b[17]; b[17] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = b[19]; b[19] = b[18] - t; b[18] = b[18] + t; }
  { cplx<T> t = b[21]; b[21] = b[20] - t; b[20] = b[20] + t; }
  { cplx<T> t = b[23]; b[23] = b[22] - t; b[22] = b[22] + t; }
  { cplx<T> t = b[25]; b[25] = b[24] - t; b[24] = b[24] + t; }
  { cplx<T> t = b[27]; b[27] = b[26] - t; b[26] = b[26] + t; }
  { cplx<T> t = b[29]; b[29] = b[28] - t; b[28] = b[28] + t; }
  { cplx<T> t = b[31]; b[31] = b[30] - t; b[30] = b[30] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{b[3].y, -b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = b[6]; b[6] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cplx<T>{b[7].y, -b[7].x}; b[7] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = b[10]; b[10] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cplx<T>{b[11].y, -b[11].x}; b[11] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = b[14]; b[14] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = cplx<T>{b[15].y, -b[15].x}; b[15] = b[13] - t; b[13] = b[13] + t; }
  { cplx<T> t = b[18]; b[18] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = cplx<T>{b[19].y, -b[19].x}; b[19] = b[17] - t; b[17] = b[17] + t; }
  { cplx<T> t = b[22]; b[22] = b[20] - t; b[20] = b[20] + t; }
  { cplx<T> t = cplx<T>{b[23].y, -b[23].x}; b[23] = b[21] - t; b[21] = b[21] + t; }
  { cplx<T> t = b[26]; b[26] = b[24] - t; b[24] = b[24] + t; }
  { cplx<T> t = cplx<T>{b[27].y, -b[27].x}; b[27] = b[25] - t; b[25] = b[25] + t; }
  { cplx<T> t = b[30]; b[30] = b[28] - t; b[28] = b[28] + t; }
  { cplx<T> t = cplx<T>{b[31].y, -b[31].x}; b[31] = b[29] - t; b[29] = b[29] + t; }
  { cplx<T> t = b[4]; b[4] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[5], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[5] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cplx<T>{b[6].y, -b[6].x}; b[6] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[7], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[7] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = b[12]; b[12] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[13] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = cplx<T>{b[14].y, -b[14].x}; b[14] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[15] = b[11] - t; b[11] = b[11] + t; }
  { cplx<T> t = b[20]; b[20] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = cmul(b[21], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[21] = b[17] - t; b[17] = b[17] + t; }
  { cplx<T> t = cplx<T>{b[22].y, -b[22].x}; b[22] = b[18] - t; b[18] = b[18] + t; }
  { cplx<T> t = cmul(b[23], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[23] = b[19] - t; b[19] = b[19] + t; }
  { cplx<T> t = b[28]; b[28] = b[24] - t; b[24] = b[24] + t; }
  { cplx<T> t = cmul(b[29], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[29] = b[25] - t; b[25] = b[25] + t; }
  { cplx<T> t = cplx<T>{b[30].y, -b[30].x}; b[30] = b[26] - t; b[26] = b[26] + t; }
  { cplx<T> t = cmul(b[31], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[31] = b[27] - t; b[27] = b[27] + t; }
  { cplx<T> t = b[8]; b[8] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[9], cplx<T>{T(0.9238795325112867), T(-0.3826834323650898)}); b[9] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cmul(b[10], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[10] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[11], cplx<T>{T(0.38268343236508984), T(-0.9238795325112867)}); b[11] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = cplx<T>{b[12].y, -b[12].x}; b[12] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(-0.3826834323650897), T(-0.9238795325112867)}); b[13] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = cmul(b[14], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[14] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.9238795325112867), T(-0.3826834323650899)}); b[15] = b[7] - t; b[7] = b[7] + t; }
  { cplx<T> t = b[24]; b[24] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = cmul(b[25], cplx<T>{T(0.9238795325112867), T(-0.3826834323650898)}); b[25] = b[17] - t; b[17] = b[17] + t; }
  { cplx<T> t = cmul(b[26], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[26] = b[18] - t; b[18] = b[18] + t; }
  { cplx<T> t = cmul(b[27], cplx<T>{T(0.38268343236508984), T(-0.9238795325112867)}); b[27] = b[19] - t; b[19] = b[19] + t; }
  { cplx<T> t = cplx<T>{b[28].y, -b[28].x}; b[28] = b[20] - t; b[20] = b[20] + t; }
  { cplx<T> t = cmul(b[29], cplx<T>{T(-0.3826834323650897), T(-0.9238795325112867)}); b[29] = b[21] - t; b[21] = b[21] + t; }
  { cplx<T> t = cmul(b[30], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[30] = b[22] - t; b[22] = b[22] + t; }
  { cplx<T> t = cmul(b[31], cplx<T>{T(-0.9238795325112867), T(-0.3826834323650899)}); b[31] = b[23] - t; b[23] = b[23] + t; }
  { cplx<T> t = b[16]; b[16] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[17], cplx<T>{T(0.9807852804032304), T(-0.19509032201612825)}); b[17] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cmul(b[18], cplx<T>{T(0.9238795325112867), T(-0.3826834323650898)}); b[18] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[19], cplx<T>{T(0.8314696123025452), T(-0.5555702330196022)}); b[19] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = cmul(b[20], cplx<T>{T(0.7071067811865476), T(-0.7071067811865475)}); b[20] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cmul(b[21], cplx<T>{T(0.5555702330196023), T(-0.8314696123025452)}); b[21] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = cmul(b[22], cplx<T>{T(0.38268343236508984), T(-0.9238795325112867)}); b[22] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = cmul(b[23], cplx<T>{T(0.19509032201612833), T(-0.9807852804032304)}); b[23] = b[7] - t; b[7] = b[7] + t; }
  { cplx<T> t = cplx<T>{b[24].y, -b[24].x}; b[24] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cmul(b[25], cplx<T>{T(-0.1950903220161282), T(-0.9807852804032304)}); b[25] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = cmul(b[26], cplx<T>{T(-0.3826834323650897), T(-0.9238795325112867)}); b[26] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = cmul(b[27], cplx<T>{T(-0.555570233019602), T(-0.8314696123025455)}); b[27] = b[11] - t; b[11] = b[11] + t; }
  { cplx<T> t = cmul(b[28], cplx<T>{T(-0.7071067811865475), T(-0.7071067811865476)}); b[28] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = cmul(b[29], cplx<T>{T(-0.8314696123025453), T(-0.5555702330196022)}); b[29] = b[13] - t; b[13] = b[13] + t; }
  { cplx<T> t = cmul(b[30], cplx<T>{T(-0.9238795325112867), T(-0.3826834323650899)}); b[30] = b[14] - t; b[14] = b[14] + t; }
  { cplx<T> t = cmul(b[31], cplx<T>{T(-0.9807852804032304), T(-0.1950903220161286)}); b[31] = b[15] - t; b[15] = b[15] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
  a[4] = b[4];
  a[5] = b[5];
  a[6] = b[6];
  a[7] = b[7];
  a[8] = b[8];
  a[9] = b[9];
  a[10] = b[10];
  a[11] = b[11];
  a[12] = b[12];
  a[13] = b[13];
  a[14] = b[14];
  a[15] = b[15];
  a[16] = b[16];
  a[17] = b[17];
  a[18] = b[18];
  a[19] = b[19];
  a[20] = b[20];
  a[21] = b[21];
  a[22] = b[22];
  a[23] = b[23];
  a[24] = b[24];
  a[25] = b[25];
  a[26] = b[26];
  a[27] = b[27];
  a[28] = b[28];
  a[29] = b[29];
  a[30] = b[30];
  a[31] = b[31];
}

template <typename T>
__device__ __forceinline__ void sg_dft32_bwd(cplx<T> (&a)[32]) {
  cplx<T> b[32];
  b[0] = a[0];
  b[1] = a[16];
  b[2] = a[8];
  b[3] = a[24];
  b[4] = a[4];
  b[5] = a[20];
  b[6] = a[12];
  b[7] = a[28];
  b[8] = a[2];
  b[9] = a[18];
  b[10] = a[10];
  b[11] = a[26];
  b[12] = a[6];
  b[13] = a[22];
  b[14] = a[14];
  b[15] = a[30];
  b[16] = a[1];
  b[17] = a[17];
  b[18] = a[9];
  b[19] = a[25];
  b[20] = a[5];
  b[21] = a[21];
  b[22] = a[13];
  b[23] = a[29];
  b[24] = a[3];
  b[25] = a[19];
  b[26] = a[11];
  b[27] = a[27];
  b[28] = a[7];
  b[29] = a[23];
  b[30] = a[15];
  b[31] = a[31];
  { cplx<T> t = b[1]; b[1] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = b[3]; b[3] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = b[5]; b[5] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = b[7]; b[7] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = b[9]; b[9] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = b[11]; b[11] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = b[13]; b[13] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = b[15]; b[15] = b[14] - t; b[14] = b[14] + t; }
  { cplx<T> t = b[17]; b[17] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = b[19]; b[19] = b[18] - t; b[18] = b[18] + t; }
  { cplx<T> t = b[21]; b[21] = b[20] - t; b[20] = b[20] + t; }
  { cplx<T> t = b[23]; b[23] = b[22] - t; b[22] = b[22] + t; }
  { cplx<T> t = b[25]; b[25] = b[24] - t; b[24] = b[24] + t; }
  { cplx<T> t = b[27]; b[27] = b[26] - t; b[26] = b[26] + t; }
  { cplx<T> t = b[29]; b[29] = b[28] - t; b[28] = b[28] + t; }
  { cplx<T> t = b[31]; b[31] = b[30] - t; b[30] = b[30] + t; }
  { cplx<T> t = b[2]; b[2] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cplx<T>{-b[3].y, b[3].x}; b[3] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = b[6]; b[6] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cplx<T>{-b[7].y, b[7].x}; b[7] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = b[10]; b[10] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cplx<T>{-b[11].y, b[11].x}; b[11] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = b[14]; b[14] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = cplx<T>{-b[15].y, b[15].x}; b[15] = b[13] - t; b[13] = b[13] + t; }
  { cplx<T> t = b[18]; b[18] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = cplx<T>{-b[19].y, b[19].x}; b[19] = b[17] - t; b[17] = b[17] + t; }
  { cplx<T> t = b[22]; b[22] = b[20] - t; b[20] = b[20] + t; }
  { cplx<T> t = cplx<T>{-b[23].y, b[23].x}; b[23] = b[21] - t; b[21] = b[21] + t; }
  { cplx<T> t = b[26]; b[26] = b[24] - t; b[24] = b[24] + t; }
  { cplx<T> t = cplx<T>{-b[27].y, b[27].x}; b[27] = b[25] - t; b[25] = b[25] + t; }
  { cplx<T> t = b[30]; b[30] = b[28] - t; b[28] = b[28] + t; }
  { cplx<T> t = cplx<T>{-b[31].y, b[31].x}; b[31] = b[29] - t; b[29] = b[29] + t; }
  { cplx<T> t = b[4]; b[4] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[5], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[5] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cplx<T>{-b[6].y, b[6].x}; b[6] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[7], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[7] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = b[12]; b[12] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[13] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = cplx<T>{-b[14].y, b[14].x}; b[14] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[15] = b[11] - t; b[11] = b[11] + t; }
  { cplx<T> t = b[20]; b[20] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = cmul(b[21], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[21] = b[17] - t; b[17] = b[17] + t; }
  { cplx<T> t = cplx<T>{-b[22].y, b[22].x}; b[22] = b[18] - t; b[18] = b[18] + t; }
  { cplx<T> t = cmul(b[23], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[23] = b[19] - t; b[19] = b[19] + t; }
  { cplx<T> t = b[28]; b[28] = b[24] - t; b[24] = b[24] + t; }
  { cplx<T> t = cmul(b[29], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[29] = b[25] - t; b[25] = b[25] + t; }
  { cplx<T> t = cplx<T>{-b[30].y, b[30].x}; b[30] = b[26] - t; b[26] = b[26] + t; }
  { cplx<T> t = cmul(b[31], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[31] = b[27] - t; b[27] = b[27] + t; }
  { cplx<T> t = b[8]; b[8] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[9], cplx<T>{T(0.9238795325112867), T(0.3826834323650898)}); b[9] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cmul(b[10], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[10] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[11], cplx<T>{T(0.38268343236508984), T(0.9238795325112867)}); b[11] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = cplx<T>{-b[12].y, b[12].x}; b[12] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cmul(b[13], cplx<T>{T(-0.3826834323650897), T(0.9238795325112867)}); b[13] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = cmul(b[14], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[14] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = cmul(b[15], cplx<T>{T(-0.9238795325112867), T(0.3826834323650899)}); b[15] = b[7] - t; b[7] = b[7] + t; }
  { cplx<T> t = b[24]; b[24] = b[16] - t; b[16] = b[16] + t; }
  { cplx<T> t = cmul(b[25], cplx<T>{T(0.9238795325112867), T(0.3826834323650898)}); b[25] = b[17] - t; b[17] = b[17] + t; }
  { cplx<T> t = cmul(b[26], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[26] = b[18] - t; b[18] = b[18] + t; }
  { cplx<T> t = cmul(b[27], cplx<T>{T(0.38268343236508984), T(0.9238795325112867)}); b[27] = b[19] - t; b[19] = b[19] + t; }
  { cplx<T> t = cplx<T>{-b[28].y, b[28].x}; b[28] = b[20] - t; b[20] = b[20] + t; }
  { cplx<T> t = cmul(b[29], cplx<T>{T(-0.3826834323650897), T(0.9238795325112867)}); b[29] = b[21] - t; b[21] = b[21] + t; }
  { cplx<T> t = cmul(b[30], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[30] = b[22] - t; b[22] = b[22] + t; }
  { cplx<T> t = cmul(b[31], cplx<T>{T(-0.9238795325112867), T(0.3826834323650899)}); b[31] = b[23] - t; b[23] = b[23] + t; }
  { cplx<T> t = b[16]; b[16] = b[0] - t; b[0] = b[0] + t; }
  { cplx<T> t = cmul(b[17], cplx<T>{T(0.9807852804032304), T(0.19509032201612825)}); b[17] = b[1] - t; b[1] = b[1] + t; }
  { cplx<T> t = cmul(b[18], cplx<T>{T(0.9238795325112867), T(0.3826834323650898)}); b[18] = b[2] - t; b[2] = b[2] + t; }
  { cplx<T> t = cmul(b[19], cplx<T>{T(0.8314696123025452), T(0.5555702330196022)}); b[19] = b[3] - t; b[3] = b[3] + t; }
  { cplx<T> t = cmul(b[20], cplx<T>{T(0.7071067811865476), T(0.7071067811865475)}); b[20] = b[4] - t; b[4] = b[4] + t; }
  { cplx<T> t = cmul(b[21], cplx<T>{T(0.5555702330196023), T(0.8314696123025452)}); b[21] = b[5] - t; b[5] = b[5] + t; }
  { cplx<T> t = cmul(b[22], cplx<T>{T(0.38268343236508984), T(0.9238795325112867)}); b[22] = b[6] - t; b[6] = b[6] + t; }
  { cplx<T> t = cmul(b[23], cplx<T>{T(0.19509032201612833), T(0.9807852804032304)}); b[23] = b[7] - t; b[7] = b[7] + t; }
  { cplx<T> t = cplx<T>{-b[24].y, b[24].x}; b[24] = b[8] - t; b[8] = b[8] + t; }
  { cplx<T> t = cmul(b[25], cplx<T>{T(-0.1950903220161282), T(0.9807852804032304)}); b[25] = b[9] - t; b[9] = b[9] + t; }
  { cplx<T> t = cmul(b[26], cplx<T>{T(-0.3826834323650897), T(0.9238795325112867)}); b[26] = b[10] - t; b[10] = b[10] + t; }
  { cplx<T> t = cmul(b[27], cplx<T>{T(-0.555570233019602), T(0.8314696123025455)}); b[27] = b[11] - t; b[11] = b[11] + t; }
  { cplx<T> t = cmul(b[28], cplx<T>{T(-0.7071067811865475), T(0.7071067811865476)}); b[28] = b[12] - t; b[12] = b[12] + t; }
  { cplx<T> t = cmul(b[29], cplx<T>{T(-0.8314696123025453), T(0.5555702330196022)}); b[29] = b[13] - t; b[13] = b[13] + t; }
  { cplx<T> t = cmul(b[30], cplx<T>{T(-0.9238795325112867), T(0.3826834323650899)}); b[30] = b[14] - t; b[14] = b[14] + t; }
  { cplx<T> t = cmul(b[31], cplx<T>{T(-0.9807852804032304), T(0.1950903220161286)}); b[31] = b[15] - t; b[15] = b[15] + t; }
  a[0] = b[0];
  a[1] = b[1];
  a[2] = b[2];
  a[3] = b[3];
  a[4] = b[4];
  a[5] = b[5];
  a[6] = b[6];
  a[7] = b[7];
  a[8] = b[8];
  a[9] = b[9];
  a[10] = b[10];
  a[11] = b[11];
  a[12] = b[12];
  a[13] = b[13];
  a[14] = b[14];
  a[15] = b[15];
  a[16] = b[16];
  a[17] = b[17];
  a[18] = b[18];
  a[19] = b[19];
  a[20] = b[20];
  a[21] = b[21];
  a[22] = b[22];
  a[23] = b[23];
  a[24] = b[24];
  a[25] = b[25];
  a[26] = b[26];
  a[27] = b[27];
  a[28] = b[28];
  a[29] = b[29];
  a[30] = b[30];
  a[31] = b[31];
}

template <int P, bool INV, typename T> struct SgDft;
template <typename T> struct SgDft<2, false, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[2]) { sg_dft2_fwd(a); } };
template <typename T> struct SgDft<2, true, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[2]) { sg_dft2_bwd(a); } };
template <typename T> struct SgDft<4, false, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[4]) { sg_dft4_fwd(a); } };
template <typename T> struct SgDft<4, true, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[4]) { sg_dft4_bwd(a); } };
template <typename T> struct SgDft<8, false, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[8]) { sg_dft8_fwd(a); } };
template <typename T> struct SgDft<8, true, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[8]) { sg_dft8_bwd(a); } };
template <typename T> struct SgDft<16, false, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[16]) { sg_dft16_fwd(a); } };
template <typename T> struct SgDft<16, true, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[16]) { sg_dft16_bwd(a); } };
template <typename T> struct SgDft<32, false, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[32]) { sg_dft32_fwd(a); } };
template <typename T> struct SgDft<32, true, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[32]) { sg_dft32_bwd(a); } };
