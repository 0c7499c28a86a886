// Forward-mode (tangent) arithmetic for second-order products of the score.
//
// Dual holds a value and its directional derivative along one tangent direction. Code
// written over a scalar type S (float or Dual) and the vector type Vec<S>::type (float3
// or D3) computes, when run on Dual inputs carrying a direction v, the derivative along v
// of everything it computes; run on the score's gradient code this is the
// Hessian-vector product (forward over reverse). Comparisons and branches use values:
// the derivative is that of the branch taken, i.e. the derivative almost everywhere of a
// piecewise-smooth function (ramps and clamps contribute their constant slopes).
#pragma once

#include "device_eval.cuh"

namespace pxd {

struct Dual {
    float v, t;
};
struct D3 {
    Dual x, y, z;
};

template <class S>
struct IsDual {
    static constexpr bool value = false;
};
template <>
struct IsDual<Dual> {
    static constexpr bool value = true;
};

template <class S>
struct Vec;
template <>
struct Vec<float> {
    using type = float3;
};
template <>
struct Vec<Dual> {
    using type = D3;
};

__device__ __forceinline__ Dual dual(float v, float t = 0.f) { return Dual{v, t}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.t + b.t}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.t - b.t}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, fmaf(a.t, b.v, a.v * b.t)}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const float q = a.v / b.v;
    return {q, (a.t - q * b.t) / b.v};
}
__device__ __forceinline__ Dual operator+(Dual a, float b) { return {a.v + b, a.t}; }
__device__ __forceinline__ Dual operator+(float a, Dual b) { return {a + b.v, b.t}; }
__device__ __forceinline__ Dual operator-(Dual a, float b) { return {a.v - b, a.t}; }
__device__ __forceinline__ Dual operator-(float a, Dual b) { return {a - b.v, -b.t}; }
__device__ __forceinline__ Dual operator*(Dual a, float b) { return {a.v * b, a.t * b}; }
__device__ __forceinline__ Dual operator*(float a, Dual b) { return {a * b.v, a * b.t}; }
__device__ __forceinline__ Dual operator/(Dual a, float b) { return {a.v / b, a.t / b}; }
__device__ __forceinline__ Dual operator/(float a, Dual b) {
    const float q = a / b.v;
    return {q, -q * b.t / b.v};
}
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.t}; }

// value / tangent parts, and lifting constants
__device__ __forceinline__ float val(float a) { return a; }
__device__ __forceinline__ float val(Dual a) { return a.v; }
__device__ __forceinline__ float part(float a) { return a; }   // what a float run outputs
__device__ __forceinline__ float part(Dual a) { return a.t; }  // what a Dual run outputs
template <class S>
__device__ __forceinline__ S lift(float a);
template <>
__device__ __forceinline__ float lift<float>(float a) { return a; }
template <>
__device__ __forceinline__ Dual lift<Dual>(float a) { return Dual{a, 0.f}; }

// math: float versions are the intrinsics the float code used
__device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
__device__ __forceinline__ Dual sqrt_(Dual a) {
    const float s = sqrtf(a.v);
    return {s, s > 0.f ? 0.5f * a.t / s : 0.f};
}
__device__ __forceinline__ float rsqrt_(float a) { return rsqrtf(a); }
__device__ __forceinline__ Dual rsqrt_(Dual a) {
    const float r = rsqrtf(a.v);
    return {r, -0.5f * r * r * r * a.t};
}
__device__ __forceinline__ float acos_(float a) { return acosf(a); }
__device__ __forceinline__ Dual acos_(Dual a) {
    const float d = 1.f - a.v * a.v;
    return {acosf(a.v), d > 0.f ? -a.t * rsqrtf(d) : 0.f};
}
__device__ __forceinline__ float cos_(float a) { return cosf(a); }
__device__ __forceinline__ Dual cos_(Dual a) { return {cosf(a.v), -sinf(a.v) * a.t}; }
__device__ __forceinline__ float sin_(float a) { return sinf(a); }
__device__ __forceinline__ Dual sin_(Dual a) { return {sinf(a.v), cosf(a.v) * a.t}; }
__device__ __forceinline__ float atan2_(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ Dual atan2_(Dual y, Dual x) {
    const float r2 = x.v * x.v + y.v * y.v;
    return {atan2f(y.v, x.v), r2 > 0.f ? (x.v * y.t - y.v * x.t) / r2 : 0.f};
}
__device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ Dual fma_(Dual a, Dual b, Dual c) { return a * b + c; }
__device__ __forceinline__ Dual fma_(Dual a, float b, Dual c) { return a * b + c; }
__device__ __forceinline__ float min_(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ Dual min_(Dual a, float b) { return a.v <= b ? a : Dual{b, 0.f}; }
__device__ __forceinline__ float max_(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ Dual max_(Dual a, float b) { return a.v >= b ? a : Dual{b, 0.f}; }

// D3 vector helpers (float3 versions live in device_eval.cuh)
__device__ __forceinline__ D3 sub3(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 add3(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 mul3(D3 a, Dual s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ D3 mul3(D3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ Dual dot3(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross3(D3 a, D3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// constants as vectors of S, vectors of float3 parts
template <class S>
__device__ __forceinline__ typename Vec<S>::type lift3(float3 a);
template <>
__device__ __forceinline__ float3 lift3<float>(float3 a) { return a; }
template <>
__device__ __forceinline__ D3 lift3<Dual>(float3 a) { return {dual(a.x), dual(a.y), dual(a.z)}; }
__device__ __forceinline__ float3 part3(float3 a) { return a; }
__device__ __forceinline__ float3 part3(D3 a) { return make_float3(a.x.t, a.y.t, a.z.t); }
__device__ __forceinline__ float3 val3(float3 a) { return a; }
__device__ __forceinline__ float3 val3(D3 a) { return make_float3(a.x.v, a.y.v, a.z.v); }
__device__ __forceinline__ float3 zero3f() { return make_float3(0.f, 0.f, 0.f); }
template <class S>
__device__ __forceinline__ typename Vec<S>::type zero3() { return lift3<S>(zero3f()); }

// Atom i of a pose held as values X (and, for Dual, tangents XT) in shared memory.
template <class S>
__device__ __forceinline__ typename Vec<S>::type atom3(const float4* X, const float4* XT, int i);
template <>
__device__ __forceinline__ float3 atom3<float>(const float4* X, const float4*, int i) { return xyz(X[i]); }
template <>
__device__ __forceinline__ D3 atom3<Dual>(const float4* X, const float4* XT, int i) {
    const float4 a = X[i], b = XT[i];
    return {Dual{a.x, b.x}, Dual{a.y, b.y}, Dual{a.z, b.z}};
}

// Butterfly sums of one part (all lanes end with the same bits).
__device__ __forceinline__ float3 warp_sum3(float3 v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        v.x += __shfl_xor_sync(kFull, v.x, off);
        v.y += __shfl_xor_sync(kFull, v.y, off);
        v.z += __shfl_xor_sync(kFull, v.z, off);
    }
    return v;
}

}  // namespace pxd
