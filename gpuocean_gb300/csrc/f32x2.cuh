// Paired float32 arithmetic (.f32x2, sm_100 and later): one instruction
// applies the same operation to two independent values, each rounded exactly
// as the scalar instruction is in the step kernels (round to nearest even,
// subnormals flushed to zero).  Code that pairs independent operations this
// way gives the scalar code's bits with fewer instructions issued - the step
// is bound by instruction issue.
//
// ptxas contracts a paired multiply whose result feeds a paired add or
// subtract into a paired fused multiply-add, even in code built without
// contraction (--fmad=false) and with explicit round-to-nearest modifiers.
// The sums below are therefore fused multiply-adds themselves, a * u + b with
// a unit factor u that is 1 at run time but unknown to the compiler: a
// multiply by exactly 1 followed by one rounding gives the plain sum's bits
// (signed zeros included), and an instruction that already is a fused
// multiply-add cannot absorb another multiply.  Callers pass u from a kernel
// parameter or from memory (StepConst::one).
#pragma once

namespace goc {

__device__ __forceinline__ unsigned long long pack2(float2 v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}

__device__ __forceinline__ float2 unpack2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}

__device__ __forceinline__ float2 pr(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 pr(float a) { return make_float2(a, a); }

__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)), "l"(pack2(c)));
    return unpack2(r);
}

// a + b (u = 1 at run time)
__device__ __forceinline__ float2 add2(float2 a, float2 b, float u) { return fma2(a, pr(u), b); }

// a - b (u = 1 at run time): b * (-1) + a
__device__ __forceinline__ float2 sub2(float2 a, float2 b, float u) { return fma2(b, pr(-u), a); }

// The same with the unit factor given as a pair, u2 = (u, u) and
// nu2 = (-u, -u), read from memory as one 64-bit operand.
__device__ __forceinline__ float2 add2(float2 a, float2 b, float2 u2) { return fma2(a, u2, b); }
__device__ __forceinline__ float2 sub2n(float2 a, float2 b, float2 nu2) { return fma2(b, nu2, a); }

}  // namespace goc
