// lbm_f32x2.cuh - a pair of FP32 values in one 64-bit register, with the
// packed f32x2 arithmetic of sm_100-class GPUs (one instruction operates on
// both halves).  Used to collide two neighbouring x nodes per thread in the
// FP32 stream+collide kernel: the same per-node arithmetic as the scalar
// code, in about half the instructions.
//
// F2 supports + - * and a product proxy P2 so that a*b + c and c - a*b
// become one fused multiply-add, as the scalar code's contraction would.
// Constants (F2(double)) are splatted at compile time; negating a constant
// folds away.
#pragma once
#include <cstdint>
#include <cstring>

namespace lbm {
namespace {

struct F2 {
  unsigned long long v;
  F2() = default;
  __host__ __device__ explicit constexpr F2(unsigned long long bits, int) : v(bits) {}
  __host__ __device__ F2(double c) : v(splat_bits(static_cast<float>(c))) {}
  __host__ __device__ static unsigned long long splat_bits(float f) {
    uint32_t u;
    memcpy(&u, &f, sizeof u);
    return (static_cast<unsigned long long>(u) << 32) | u;
  }
};

__device__ __forceinline__ F2 pack2(float lo, float hi) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ F2 splat2(float a) { return pack2(a, a); }
__device__ __forceinline__ void unpack2(F2 a, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
// sign flip of both halves (exact)
__device__ __forceinline__ F2 neg2(F2 a) { return F2(a.v ^ 0x8000000080000000ull, 0); }

struct P2 {  // a * b, not yet rounded
  F2 a, b;
  __device__ __forceinline__ operator F2() const { return mul2(a, b); }
};

__device__ __forceinline__ P2 operator*(F2 a, F2 b) { return P2{a, b}; }
__device__ __forceinline__ P2 operator*(P2 p, F2 b) { return P2{F2(p), b}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return add2(a, b); }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return sub2(a, b); }
__device__ __forceinline__ F2 operator+(F2 c, P2 p) { return fma2(p.a, p.b, c); }
__device__ __forceinline__ F2 operator+(P2 p, F2 c) { return fma2(p.a, p.b, c); }
__device__ __forceinline__ F2 operator+(P2 p, P2 q) { return fma2(p.a, p.b, F2(q)); }
__device__ __forceinline__ F2 operator-(F2 c, P2 p) { return fma2(neg2(p.a), p.b, c); }
__device__ __forceinline__ F2 operator-(P2 p, F2 c) { return fma2(p.a, p.b, neg2(c)); }
__device__ __forceinline__ F2 operator-(P2 p, P2 q) { return fma2(neg2(q.a), q.b, F2(p)); }

}  // namespace
}  // namespace lbm
