// ncg_dw.cuh — double-word (float-float) arithmetic on the FP32 pipes.
//
// GB300 executes FP64 at a small fraction of its FP32 rate: one warp-wide f64
// instruction occupies the FP64 pipe for tens of cycles even with one active
// lane.  The FP64-class parts of the narrow phase (simplex sub-solve, EPA face
// normals, distances and termination tests) therefore run on a pair of floats
// hi + lo (|lo| <= ulp(hi)/2, ~48-bit significand) built from error-free
// transformations:
//   2Sum (Knuth), Fast2Sum (Dekker), Fast2Mult with FMA;
//   AccurateDWPlusDW (Alg. 6), DWTimesDW3 (Alg. 12), DWTimesFP3 (Alg. 9) and
//   DWDivDW2 (Alg. 17) of Joldes, Muller, Popescu, "Tight and rigorous error
//   bounds for basic building blocks of double-word arithmetic", ACM TOMS 2017;
//   square root: one Newton correction of sqrtf(hi) (Karp & Markstein).
// The library is compiled with -fmad=false so that only the explicit fmaf
// calls fuse; every other single-precision operation rounds to nearest.
#pragma once

#include <cfloat>
#include <cstdint>

#ifndef NCG_DEV
#define NCG_DEV __device__ __forceinline__
#endif

// NCG_DW_OUTLINE, defined by a translation unit before its includes: 1 keeps
// the double-word sum, quotient and square root out of line (one shared copy
// each: the GJK-type loops are bound by instruction fetch), 2 also the
// product.  Unset, everything is inlined (the EPA stages are latency-bound).
#if defined(NCG_DW_OUTLINE) && NCG_DW_OUTLINE >= 1
#define NCG_DW_BIG static __device__ __noinline__
#else
#define NCG_DW_BIG NCG_DEV
#endif
#if defined(NCG_DW_OUTLINE) && NCG_DW_OUTLINE >= 2
#define NCG_DW_MUL static __device__ __noinline__
#else
#define NCG_DW_MUL NCG_DEV
#endif

namespace ncg {

struct dw {
    float h, l;
    NCG_DEV dw() : h(0.0f), l(0.0f) {}
    NCG_DEV dw(float a) : h(a), l(0.0f) {}
    NCG_DEV dw(float a, float b) : h(a), l(b) {}
    NCG_DEV explicit operator float() const { return h; }
};

// Host-side split of an f64 constant (tolerances, parameters).
struct dw_host {
    float h, l;
};
inline dw_host dw_split(double d) {
    float h = (float)d;
    return dw_host{h, (float)(d - (double)h)};
}

NCG_DEV dw two_sum(float a, float b) {
    float s = a + b;
    float ap = s - b;
    float bp = s - ap;
    float da = a - ap;
    float db = b - bp;
    return dw(s, da + db);
}
NCG_DEV dw fast_two_sum(float a, float b) {
    float s = a + b;
    float z = s - a;
    return dw(s, b - z);
}
NCG_DEV dw two_prod(float a, float b) {
    float p = a * b;
    return dw(p, __fmaf_rn(a, b, -p));
}
NCG_DW_BIG dw operator+(dw x, dw y) {
    dw s = two_sum(x.h, y.h);
    dw t = two_sum(x.l, y.l);
    float c = s.l + t.h;
    dw v = fast_two_sum(s.h, c);
    float w = t.l + v.l;
    return fast_two_sum(v.h, w);
}
NCG_DEV dw operator-(dw x) { return dw(-x.h, -x.l); }
NCG_DEV dw operator-(dw x, dw y) { return x + (-y); }
NCG_DW_MUL dw operator*(dw x, dw y) {
    dw c = two_prod(x.h, y.h);
    float tl0 = x.l * y.l;
    float tl1 = __fmaf_rn(x.h, y.l, tl0);
    float cl2 = __fmaf_rn(x.l, y.h, tl1);
    float cl3 = c.l + cl2;
    return fast_two_sum(c.h, cl3);
}
NCG_DEV dw mul_fp(dw x, float y) {
    dw c = two_prod(x.h, y);
    float cl3 = __fmaf_rn(x.l, y, c.l);
    return fast_two_sum(c.h, cl3);
}
NCG_DW_BIG dw operator/(dw x, dw y) {
    float th = __fdiv_rn(x.h, y.h);
    dw r = mul_fp(y, th);
    float ph = x.h - r.h;
    float dl = x.l - r.l;
    float d = ph + dl;
    float tl = __fdiv_rn(d, y.h);
    return fast_two_sum(th, tl);
}
NCG_DW_BIG dw sqrt(dw x) {
    if (!(x.h > 0.0f)) return x.h == 0.0f ? dw(0.0f) : dw(__int_as_float(0x7fc00000));
    float s = __fsqrt_rn(x.h);
    dw p = two_prod(s, s);
    float r = ((x.h - p.h) - p.l) + x.l;
    float e = __fdiv_rn(r, 2.0f * s);
    return fast_two_sum(s, e);
}
NCG_DEV dw fabs(dw x) { return (x.h < 0.0f || (x.h == 0.0f && x.l < 0.0f)) ? -x : x; }
NCG_DEV bool operator<(dw a, dw b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
NCG_DEV bool operator<=(dw a, dw b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); }
NCG_DEV bool operator>(dw a, dw b) { return b < a; }
NCG_DEV bool operator>=(dw a, dw b) { return b <= a; }
NCG_DEV bool operator==(dw a, dw b) { return a.h == b.h && a.l == b.l; }
NCG_DEV bool operator!=(dw a, dw b) { return !(a == b); }

// ---------------------------------------------------------------- f32r
// Plain f32 arithmetic behind the same interface: the reference's f32 path
// (every sub-solve, bound and EPA distance in f32), used by the translation
// units built with NCG_REAL_F32.  `l` is always zero, so records laid out
// for double-words (heap keys, spill headers) hold the same bits.
struct f32r {
    float h, l;
    NCG_DEV f32r() : h(0.0f), l(0.0f) {}
    NCG_DEV f32r(float a) : h(a), l(0.0f) {}
    NCG_DEV f32r(float a, float) : h(a), l(0.0f) {}
    NCG_DEV explicit operator float() const { return h; }
};
NCG_DEV f32r operator+(f32r x, f32r y) { return f32r(__fadd_rn(x.h, y.h)); }
NCG_DEV f32r operator-(f32r x) { return f32r(-x.h); }
NCG_DEV f32r operator-(f32r x, f32r y) { return f32r(__fsub_rn(x.h, y.h)); }
NCG_DEV f32r operator*(f32r x, f32r y) { return f32r(__fmul_rn(x.h, y.h)); }
NCG_DEV f32r operator/(f32r x, f32r y) { return f32r(__fdiv_rn(x.h, y.h)); }
NCG_DEV f32r sqrt(f32r x) { return f32r(__fsqrt_rn(x.h)); }
NCG_DEV f32r fabs(f32r x) { return f32r(fabsf(x.h)); }
NCG_DEV bool operator<(f32r a, f32r b) { return a.h < b.h; }
NCG_DEV bool operator<=(f32r a, f32r b) { return a.h <= b.h; }
NCG_DEV bool operator>(f32r a, f32r b) { return a.h > b.h; }
NCG_DEV bool operator>=(f32r a, f32r b) { return a.h >= b.h; }
NCG_DEV bool operator==(f32r a, f32r b) { return a.h == b.h; }
NCG_DEV bool operator!=(f32r a, f32r b) { return a.h != b.h; }

}  // namespace ncg
