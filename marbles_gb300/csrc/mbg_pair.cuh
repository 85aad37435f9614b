// mbg_pair.cuh -- paired FP32 arithmetic: F2 holds one quantity of two cells
// and maps + - * and fused multiply-add onto Blackwell's two-lane FP32
// instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn: one instruction for both
// cells), so that the per-cell templates of mbg_physics.cuh (MomentAcc,
// Macro, build_equilibrium, Equilibrium) run on two cells at once when
// instantiated with R = F2.  Each lane is rounded as the scalar FP32
// operation; a * b + c is two roundings (no contraction), division is two
// scalar IEEE divisions.
#pragma once

#include <cuda_runtime.h>

namespace mbg {

struct F2 {
    float2 v;
    F2() = default;
    __device__ __forceinline__ F2(float2 a) : v(a) {}
    __device__ __forceinline__ F2(float a, float b) : v(make_float2(a, b)) {}
    // broadcast of a scalar (literals and per-level constants)
    __device__ __forceinline__ F2(float s) : v(make_float2(s, s)) {}
    __device__ __forceinline__ F2(double s) : v(make_float2((float)s, (float)s)) {}
    __device__ __forceinline__ F2(int s) : v(make_float2((float)s, (float)s)) {}
};

__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 operator-(F2 a) { return F2(-a.v.x, -a.v.y); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2(__fadd2_rn(a.v, make_float2(-b.v.x, -b.v.y))); }
__device__ __forceinline__ F2 operator/(F2 a, F2 b) { return F2(a.v.x / b.v.x, a.v.y / b.v.y); }
__device__ __forceinline__ F2& operator+=(F2& a, F2 b) { return a = a + b; }
__device__ __forceinline__ F2& operator-=(F2& a, F2 b) { return a = a - b; }
__device__ __forceinline__ F2& operator*=(F2& a, F2 b) { return a = a * b; }
// a * b + c rounded once per lane
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return F2(__ffma2_rn(a.v, b.v, c.v)); }

}  // namespace mbg
