// dw.hpp — TEST INFRASTRUCTURE ONLY: double-word (float-float) arithmetic for
// the oracle's MIXED instantiation, i.e. the arithmetic the GPU kernels use
// for their FP64-class sub-solve.  A value is hi + lo with |lo| <= ulp(hi)/2.
//
// Algorithms (the oracle and the kernels implement the same published
// sequences independently; results are bit-identical when both round each
// single-precision operation to nearest and fmaf is fused):
//   2Sum (Knuth), Fast2Sum (Dekker), Fast2Mult with FMA;
//   AccurateDWPlusDW (Alg. 6), DWTimesDW3 (Alg. 12), DWTimesFP3 (Alg. 9) and
//   DWDivDW2 (Alg. 17) of Joldes, Muller, Popescu, "Tight and rigorous error
//   bounds for basic building blocks of double-word arithmetic", ACM TOMS 2017;
//   square root: one Newton correction of sqrtf(hi) (Karp & Markstein).
// Build with -ffp-contract=off.
#pragma once

#include <cfloat>
#include <cmath>
#include <limits>

namespace ncgo {

struct dw {
    float h, l;
    dw() : h(0.0f), l(0.0f) {}
    dw(float a) : h(a), l(0.0f) {}  // exact
    dw(float a, float b) : h(a), l(b) {}
    static dw from_double(double d) {
        float h = (float)d;
        return dw(h, (float)(d - (double)h));
    }
    explicit dw(double d) { *this = from_double(d); }
    explicit dw(int i) : h((float)i), l(0.0f) {}
    explicit operator float() const { return h; }
    explicit operator double() const { return (double)h; }
};

inline dw two_sum(float a, float b) {
    float s = a + b;
    float ap = s - b;
    float bp = s - ap;
    float da = a - ap;
    float db = b - bp;
    return dw(s, da + db);
}
inline dw fast_two_sum(float a, float b) {
    float s = a + b;
    float z = s - a;
    return dw(s, b - z);
}
inline dw two_prod(float a, float b) {
    float p = a * b;
    return dw(p, std::fmaf(a, b, -p));
}
inline dw operator+(dw x, dw y) {
    dw s = two_sum(x.h, y.h);
    dw t = two_sum(x.l, y.l);
    float c = s.l + t.h;
    dw v = fast_two_sum(s.h, c);
    float w = t.l + v.l;
    return fast_two_sum(v.h, w);
}
inline dw operator-(dw x) { return dw(-x.h, -x.l); }
inline dw operator-(dw x, dw y) { return x + (-y); }
inline dw operator*(dw x, dw y) {
    dw c = two_prod(x.h, y.h);
    float tl0 = x.l * y.l;
    float tl1 = std::fmaf(x.h, y.l, tl0);
    float cl2 = std::fmaf(x.l, y.h, tl1);
    float cl3 = c.l + cl2;
    return fast_two_sum(c.h, cl3);
}
inline dw mul_fp(dw x, float y) {
    dw c = two_prod(x.h, y);
    float cl3 = std::fmaf(x.l, y, c.l);
    return fast_two_sum(c.h, cl3);
}
inline dw operator/(dw x, dw y) {
    float th = x.h / y.h;
    dw r = mul_fp(y, th);
    float ph = x.h - r.h;
    float dl = x.l - r.l;
    float d = ph + dl;
    float tl = d / y.h;
    return fast_two_sum(th, tl);
}
inline dw sqrt(dw x) {
    if (!(x.h > 0.0f)) return x.h == 0.0f ? dw(0.0f) : dw(std::numeric_limits<float>::quiet_NaN());
    float s = std::sqrt(x.h);
    dw p = two_prod(s, s);
    float r = ((x.h - p.h) - p.l) + x.l;
    float e = r / (2.0f * s);
    return fast_two_sum(s, e);
}
inline dw fabs(dw x) { return (x.h < 0.0f || (x.h == 0.0f && x.l < 0.0f)) ? -x : x; }
inline bool operator<(dw a, dw b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
inline bool operator<=(dw a, dw b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); }
inline bool operator>(dw a, dw b) { return b < a; }
inline bool operator>=(dw a, dw b) { return b <= a; }
inline bool operator==(dw a, dw b) { return a.h == b.h && a.l == b.l; }
inline bool operator!=(dw a, dw b) { return !(a == b); }

}  // namespace ncgo

namespace std {
template <> struct numeric_limits<ncgo::dw> {
    static ncgo::dw max() { return ncgo::dw(FLT_MAX); }
    static ncgo::dw epsilon() { return ncgo::dw(FLT_EPSILON); }
};
}  // namespace std
