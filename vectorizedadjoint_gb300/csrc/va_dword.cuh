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
#pragma once

namespace va {

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
    const float ch = x.hi * y.hi;
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
    const float ch = x.hi * y;
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

} // namespace va
