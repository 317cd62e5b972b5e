// pn_vjp2.cuh -- the mixed-precision adjoint pair sweep on packed FP32x2 instructions.
//
// The scalar sweep k_pair_vjp<float> (pn_adjoint.cu) issues one instruction per operation of
// its ~154 per pair and is bound by the issue slots (83 % busy, FMA pipe 71 %).  Here each
// thread holds TWO rows p (lane 0: p0, lane 1: p0 + 128) in f32x2 registers and every j value
// is stored duplicated in both lanes of its pack entry, so the same arithmetic (the vjp_pair
// template, instantiated on V2) runs one instruction for two pairs.
//
// j data: the "duplicated" adjoint pack, 13 float4 groups per star ([g][npad]), each group
// (a, a, b, b) so that one 128-bit shared load yields two broadcast operands:
//   g0 (ex ey) g1 (ez m) g2 (lx ly) g3 (lz mu3) g4 (vx vy) g5 (vz qe) g6 (c1 c3) g7 (k35 vi2)
//   g8 (Gx Gy) g9 (Gz Phi) g10 (Wx Wy) g11 (Wz S0) g12 (U cW)
// (positions hi/lo relative to the tile origin, as in the forward FP32 pack; adjoint state
// from k_finish_vjp).  Built by k_vjp_dup from the forward pack and the adjoint pack.
#pragma once

#include "pn_pair2.cuh"

namespace pn {

// Two FP32 lanes in one 64-bit register pair, with the arithmetic of the vjp_pair template.
struct V2 {
    f2 v;
    __device__ __forceinline__ V2() {}
    __device__ __forceinline__ V2(float a) : v(f2_bcast(a)) {}
    __device__ __forceinline__ V2(double a) : v(f2_bcast((float)a)) {}
    __device__ __forceinline__ V2(int a) : v(f2_bcast((float)a)) {}
    __device__ __forceinline__ static V2 raw(f2 x) {
        V2 r;
        r.v = x;
        return r;
    }
    __device__ __forceinline__ V2 &operator+=(V2 b) {
        v = add2(v, b.v);
        return *this;
    }
};
__device__ __forceinline__ V2 operator+(V2 a, V2 b) { return V2::raw(add2(a.v, b.v)); }
__device__ __forceinline__ V2 operator-(V2 a, V2 b) { return V2::raw(sub2(a.v, b.v)); }
__device__ __forceinline__ V2 operator*(V2 a, V2 b) { return V2::raw(mul2(a.v, b.v)); }
__device__ __forceinline__ V2 operator-(V2 a) { return V2::raw(mul2(a.v, f2_bcast(-1.f))); }
template <> __device__ __forceinline__ V2 pn_fma<V2>(V2 a, V2 b, V2 c) { return V2::raw(fma2(a.v, b.v, c.v)); }
// MUFU rsqrt per lane refined by one Newton-Raphson step y (1.5 - 0.5 x y^2), as rsqrt_mufu_nr.
template <> __device__ __forceinline__ V2 pn_rsqrt<V2>(V2 x) {
    float a, b;
    f2_unpack(x.v, a, b);
    float ya, yb;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(ya) : "f"(a));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(yb) : "f"(b));
    const f2 y = f2_pack(ya, yb);
    const f2 r = fma2(mul2(x.v, f2_bcast(-0.5f)), mul2(y, y), f2_bcast(1.5f));
    return V2::raw(mul2(y, r));
}
// the self pair's mask: lane k keeps its pair unless it is row k's own star
__device__ __forceinline__ V2 vjp_self_mask(V2 Q, V2 keep) { return Q * keep; }
__device__ __forceinline__ V2 vjp_self_mask(V2 Q, bool self) { return self ? V2(0.f) : Q; }

__device__ __forceinline__ float lane(V2 x, int k) {
    float a, b;
    f2_unpack(x.v, a, b);
    return k ? b : a;
}

}  // namespace pn
