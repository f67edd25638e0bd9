// Double-single arithmetic on the FP32 pipes: a value is hi + lo with |lo| <= ulp(hi) / 2
// (Dekker, "A floating-point technique for extending the available precision", 1971; Knuth's
// two-sum). About 48 significant bits; GB300's FP32 rate is 64 times its FP64 rate, so a
// double-single operation (6 to 20 FP32 operations) still runs several times faster than
// the FP64 one. Used where FP64 accuracy is needed in bulk (the element integrals of the
// FP32 + refinement path).
#pragma once

namespace fg {

struct dsf {
    float h, l;
};

__device__ __forceinline__ dsf ds_make(float h, float l) { return {h, l}; }

// exact sum a + b = s + e
__device__ __forceinline__ dsf ds_two_sum_f(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
// renormalise, |a| >= |b|
__device__ __forceinline__ dsf ds_quick(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dsf ds_add(dsf x, dsf y) {
    dsf s = ds_two_sum_f(x.h, y.h);
    s.l += x.l + y.l;
    return ds_quick(s.h, s.l);
}
__device__ __forceinline__ dsf ds_neg(dsf x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dsf ds_sub(dsf x, dsf y) { return ds_add(x, ds_neg(y)); }
__device__ __forceinline__ dsf ds_mul(dsf x, dsf y) {
    const float p = x.h * y.h;
    float e = fmaf(x.h, y.h, -p);
    e = fmaf(x.h, y.l, e);
    e = fmaf(x.l, y.h, e);
    return ds_quick(p, e);
}
__device__ __forceinline__ dsf ds_fma(dsf x, dsf y, dsf z) { return ds_add(ds_mul(x, y), z); }
// x / y: quotient estimate from the FP32 parts, one correction from the double-single remainder
__device__ __forceinline__ dsf ds_div(dsf x, dsf y) {
    const float q1 = x.h / y.h;
    const dsf r = ds_sub(x, ds_mul(y, dsf{q1, 0.f}));
    const float q2 = r.h / y.h;
    return ds_quick(q1, q2);
}
__device__ __forceinline__ bool ds_gt(dsf x, dsf y) { return x.h > y.h || (x.h == y.h && x.l > y.l); }
__device__ __forceinline__ dsf ds_from(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double ds_to(dsf x) { return (double)x.h + (double)x.l; }

}  // namespace fg
