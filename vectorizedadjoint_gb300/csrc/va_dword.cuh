// Double-word ("float-float") arithmetic: a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi)/2, about 48 significant bits.
// On this GPU FP64 issues at 1/61 of the FP32 rate, so double-word
// arithmetic, which runs entirely on the FP32 pipe, is the cheaper way to
// carry near-FP64 precision through the stage and VJP arithmetic.
//
// Algorithms (with FMA) from M. Joldes, J.-M. Muller, V. Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 44(2), 2017:
//   Fast2Sum, 2Sum, 2Prod (Algorithms 1-3), accurate DWPlusDW (Alg. 6,
//   relative error <= 3u^2), DWTimesFP (Alg. 9, <= 2u^2) and DWTimesDW
//   (Alg. 12, <= 5u^2), u = 2^-24.
// Sums of products use a compensated accumulator (dacc below): Dot2 of
// T. Ogita, S. M. Rump, S. Oishi, "Accurate sum and dot product", SIAM J.
// Sci. Comput. 26(6), 2005 (Algorithm 5.3), with double-word factors.
//
// Every leading product goes through fmul_rn, so no translation unit can
// contract it into the following add: the error-free transformations need
// the product rounded on its own, and the sweeps that re-run a segment need
// the same bits from every kernel that inlines these functions.
#pragma once

#include <cstring>

namespace va {

__host__ __device__ __forceinline__ float fmul_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

struct dword {
    float hi, lo;

    dword() = default;
    __host__ __device__ constexpr dword(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr dword(int v) : hi((float)v), lo(0.0f) {}
    // split of a double: hi = RN(d), lo = RN(d - hi)
    __host__ __device__ constexpr dword(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__host__ __device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &t)
{
    s = a + b;
    const float z = s - a;
    t = b - z;
}

__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &t)
{
    s = a + b;
    const float ap = s - b;
    const float bp = s - ap;
    t = (a - ap) + (b - bp);
}

__host__ __device__ __forceinline__ dword operator+(dword x, dword y)
{
    float sh, sl, th, tl;
    two_sum(x.hi, y.hi, sh, sl);
    two_sum(x.lo, y.lo, th, tl);
    const float c = sl + th;
    float vh, vl;
    fast_two_sum(sh, c, vh, vl);
    const float w = tl + vl;
    dword z;
    fast_two_sum(vh, w, z.hi, z.lo);
    return z;
}

__host__ __device__ __forceinline__ dword operator-(dword x) { return dword(-x.hi, -x.lo); }
__host__ __device__ __forceinline__ dword operator-(dword x, dword y) { return x + (-y); }

__host__ __device__ __forceinline__ dword operator*(dword x, dword y)
{
    const float ch = fmul_rn(x.hi, y.hi);
    const float cl1 = fmaf(x.hi, y.hi, -ch);
    const float tl0 = x.lo * y.lo;
    const float tl1 = fmaf(x.hi, y.lo, tl0);
    const float cl2 = fmaf(x.lo, y.hi, tl1);
    const float cl3 = cl1 + cl2;
    dword z;
    fast_two_sum(ch, cl3, z.hi, z.lo);
    return z;
}

__host__ __device__ __forceinline__ dword operator*(dword x, float y)
{
    const float ch = fmul_rn(x.hi, y);
    const float cl1 = fmaf(x.hi, y, -ch);
    const float cl3 = fmaf(x.lo, y, cl1);
    dword z;
    fast_two_sum(ch, cl3, z.hi, z.lo);
    return z;
}

__host__ __device__ __forceinline__ dword &operator+=(dword &x, dword y) { return x = x + y; }

__host__ __device__ __forceinline__ dword dabs(dword x) { return x.hi < 0.0f ? -x : x; }

// x / y: one long-division step on the leading words (DWDivDW2 of the same
// paper: t = xh / yh, remainder x - t y by DWTimesFP, correction / yh,
// Fast2Sum), relative error O(u^2).
__host__ __device__ __forceinline__ dword operator/(dword x, dword y)
{
    const float th = x.hi / y.hi;
    const dword r = y * th;
    // (r = t y by DWTimesFP; the remainder x - r is exact to O(u^2))
    const float ph = x.hi - r.hi;
    const float dl = x.lo - r.lo;
    const float d = ph + dl;
    const float tl = d / y.hi;
    dword z;
    fast_two_sum(th, tl, z.hi, z.lo);
    return z;
}

// x > y for normalized double-words (leading words first)
__host__ __device__ __forceinline__ bool dw_greater(dword x, dword y)
{
    return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo);
}
__host__ __device__ __forceinline__ bool dw_less(dword x, dword y) { return dw_greater(y, x); }

// ------------------------------------------------ compensated sums (Dot2)

// Running sum s + c: s carries the float sum, c the accumulated rounding
// errors of the sum and of the products plus the products' low-order terms.
struct dacc {
    float s, c;
};

__host__ __device__ __forceinline__ dacc dacc_of(dword v) { return dacc{v.hi, v.lo}; }

// the sum as a normalized double-word (2Sum: after cancellation |c| may
// exceed |s|)
__host__ __device__ __forceinline__ dword dacc_get(dacc r)
{
    dword z;
    two_sum(r.s, r.c, z.hi, z.lo);
    return z;
}

// r += a b for double-words a, b: 2Prod of the leading words, its error and
// the cross terms a.hi b.lo + a.lo b.hi into c (a.lo b.lo, ~u^2 of the
// product's low part, is dropped), 2Sum of the leading product into s.
__host__ __device__ __forceinline__ void dacc_fma(dacc &r, dword a, dword b)
{
    const float p = fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s, se;
    two_sum(r.s, p, s, se);
    r.s = s;
    r.c = r.c + (se + e);
}

// r += k b for a coefficient k known at compile time: its split into
// kh + kl folds, and the kl term vanishes for coefficients exact in FP32.
__host__ __device__ __forceinline__ void dacc_fma_k(dacc &r, double k, dword b)
{
    const float kh = (float)k;
    const float kl = (float)(k - (double)kh);
    const float p = fmul_rn(kh, b.hi);
    float e = fmaf(kh, b.hi, -p);
    e = fmaf(kh, b.lo, e);
    if (kl != 0.0f)
        e = fmaf(kl, b.hi, e);
    float s, se;
    two_sum(r.s, p, s, se);
    r.s = s;
    r.c = r.c + (se + e);
}

// the product k b alone (first term of a sum)
__host__ __device__ __forceinline__ dacc dacc_mul_k(double k, dword b)
{
    const float kh = (float)k;
    const float kl = (float)(k - (double)kh);
    const float p = fmul_rn(kh, b.hi);
    float e = fmaf(kh, b.hi, -p);
    e = fmaf(kh, b.lo, e);
    if (kl != 0.0f)
        e = fmaf(kl, b.hi, e);
    return dacc{p, e};
}
__host__ __device__ __forceinline__ dacc dacc_mul(dword a, dword b)
{
    const float p = fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return dacc{p, e};
}

// r += v
__host__ __device__ __forceinline__ void dacc_add(dacc &r, dword v)
{
    float s, se;
    two_sum(r.s, v.hi, s, se);
    r.s = s;
    r.c = r.c + (se + v.lo);
}

// A double-word in one 8-byte slot (a checkpoint record field): the leading
// float in the low word, so the slot reads as float[2] = {hi, lo}.
__host__ __device__ __forceinline__ double dw_pack(dword v)
{
#ifdef __CUDA_ARCH__
    return __hiloint2double(__float_as_int(v.lo), __float_as_int(v.hi));
#else
    const float f[2] = {v.hi, v.lo};
    double d;
    memcpy(&d, f, sizeof d);
    return d;
#endif
}
__host__ __device__ __forceinline__ dword dw_unpack(double d)
{
#ifdef __CUDA_ARCH__
    return dword(__int_as_float(__double2loint(d)), __int_as_float(__double2hiint(d)));
#else
    float f[2];
    memcpy(f, &d, sizeof f);
    return dword(f[0], f[1]);
#endif
}

} // namespace va
