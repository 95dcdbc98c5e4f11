// cell_math.cuh -- the per-cell arithmetic of the compact forms, shared by
// every kernel that updates them (the z-marching single-solve and batched
// kernels and the strip kernel), so that all of them give the same bits.
//
// Every operation is an explicit intrinsic: which products the compiler
// would contract into fused multiply-adds can differ between two kernels
// that inline the same expression, explicit roundings cannot.
//
// H update (updateHField, fdtd_calculations.cu:43-76), one component:
//   h' = h - k1 (a1 - b1) + k2 (a2 - b2)
// D increment of the compact form, one component (updateDField,
// fdtd_calculations.cu:96-121, without D^n):
//   dD = t1 (a1 - b1) - t2 (a2 - b2)
// E and recursion variable of the compact form (updateEField,
// fdtd_calculations.cu:146-183, rearranged with R = -a E^{n-1} - 2 tau
// (D^n - D^{n-1})):
//   E^{n+1} = c (d E^n + ((2 dt + 2 tau) dD + R^n)),  R^{n+1} = -a E^n - 2 tau dD
#pragma once

#include "fdtd_internal.h"

namespace fdtd {

__device__ __forceinline__ float cm_h(float h, float k1, float a1, float b1, float k2, float a2, float b2)
{
    return __fmaf_rn(k2, __fsub_rn(a2, b2), __fmaf_rn(-k1, __fsub_rn(a1, b1), h));
}

__device__ __forceinline__ float cm_dinc(float t1, float a1, float b1, float t2, float a2, float b2)
{
    return __fmaf_rn(t1, __fsub_rn(a1, b1), -__fmul_rn(t2, __fsub_rn(a2, b2)));
}

// 2 dt + 2 tau of a class
__device__ __forceinline__ float cm_k12(const DebyeCoef &k) { return __fadd_rn(k.two_dt, k.two_tau); }

__device__ __forceinline__ float cm_e_next(const DebyeCoef &k, float k12, float e, float g, float r)
{
    return __fmul_rn(k.c, __fmaf_rn(k.d, e, __fmaf_rn(k12, g, r)));
}

// The sum with +0 turns a zero of either sign into +0 (and changes no other
// value): in a class without relaxation (tau = 0, so a = 0) R stays +0 on
// every step, the value zeroed memory starts with, so a kernel may leave R of
// such cells unread and unwritten and still give the same bits.
__device__ __forceinline__ float cm_r_next(const DebyeCoef &k, float e, float g)
{
    return __fadd_rn(__fmaf_rn(-k.two_tau, g, __fmul_rn(-k.a, e)), 0.0f);
}

// ---- 16-bit R: the residual rho = R^{n+1} + a E^{n+1} as FP16 bits times a
// power-of-two scale 2^(b - 127) shared by the three components of a 32-cell
// row segment (b in the low byte of the segment's word).

// The scale of word w (w = 0 gives 0).
__device__ __forceinline__ float cm_r16_scale(uint32_t w) { return __uint_as_float(w << 23); }

// R^n = rho - a E^n from the stored bits h (exact decode: an FP16 value has
// 11 significant bits and the scale is a power of two).
__device__ __forceinline__ float cm_r16_r(unsigned short h, float scale, float a, float e)
{
    float f;
    asm("cvt.f32.f16 %0, %1;" : "=f"(f) : "h"(h));
    return __fmaf_rn(-a, e, __fmul_rn(f, scale));
}

// rho = R^{n+1} + a E^{n+1}
__device__ __forceinline__ float cm_r16_rho(float a, float en, float rn) { return __fmaf_rn(a, en, rn); }

// Warp-collective (every lane of the warp calls it; one warp is one row
// segment): b = e - 14, at least 1, for the largest |r0|, |r1|, |r2| of the
// segment with biased exponent e; returns b and sets each hk to the FP16
// bits of rk 2^(127-b) rounded to nearest even.  The scaling by a power of
// two is exact and puts the segment's largest value in [2^14, 2^15), below
// the FP16 maximum; every value above 2^-29 of it keeps FP16's 11
// significant bits, so the three components share one scale.  Lanes that
// hold no updated cell pass zeros.
__device__ __forceinline__ uint32_t cm_r16_encode(float r0, float r1, float r2, unsigned short &h0, unsigned short &h1,
                                                  unsigned short &h2)
{
    const float a = fmaxf(fmaxf(fabsf(r0), fabsf(r1)), fabsf(r2));
    const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(a));
    const uint32_t b = (uint32_t)max((int)(m >> 23) - 14, 1);
    const float mult = __uint_as_float((254u - b) << 23);
    asm("cvt.rn.f16.f32 %0, %1;" : "=h"(h0) : "f"(__fmul_rn(r0, mult)));
    asm("cvt.rn.f16.f32 %0, %1;" : "=h"(h1) : "f"(__fmul_rn(r1, mult)));
    asm("cvt.rn.f16.f32 %0, %1;" : "=h"(h2) : "f"(__fmul_rn(r2, mult)));
    return b;
}

}  // namespace fdtd
