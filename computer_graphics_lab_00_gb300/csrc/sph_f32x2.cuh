// sph_f32x2.cuh — two FP32 values in one 64-bit register pair for the packed
// FP32 pipe (add/mul/fma.rn.f32x2), in half the issue slots of scalar code.
//
// One packed add, sub or mul rounds each lane as the scalar instruction does
// (the division self-test's modes 2-4 compare them lane by lane). A chain of
// them does not have to: ptxas contracts a packed mul whose result feeds a
// packed add into one packed FMA even under --fmad=false (self-test mode 5,
// a squared distance, differs from the scalar chain). So the exact passes
// use scalar arithmetic, and these helpers serve only code whose results are
// not held to the scalar bits: the MLP epilogue (bias add and GELU, rounded
// to BF16 and checked against the oracle with a tolerance).
#pragma once

namespace sph {

using f32x2 = unsigned long long;

__device__ __forceinline__ f32x2 pack2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ void unpack2(f32x2 r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}

__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

}  // namespace sph
