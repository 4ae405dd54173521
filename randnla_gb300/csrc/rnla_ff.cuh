// Float-float ("double-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats, about 48 significant
// bits.  The building blocks are the classical error-free transformations:
// TwoSum (Knuth: s + e = a + b exactly, any magnitudes), FastTwoSum (Dekker:
// the same when |a| >= |b|) and TwoProduct through one FMA (p + e = a b
// exactly).  Products drop the lo*lo term.
//
// GB300 executes FP64 at 1/64 of the FP32 rate and a dependent FP64
// operation costs ~64 cycles (a divide or square root several hundred), so
// vector arithmetic that needs more than FP32 runs in this form instead.
#pragma once
#include <cstdint>

namespace rnla {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}

// (sh, sl) += (ah + al)(bh + bl): exact product of the high parts (FMA error
// term), TwoSum into the running high part, every low-order term into sl.
// The accumulator is left unnormalised; ff_norm() renormalises it.
__device__ __forceinline__ void ff_madd(float ah, float al, float bh, float bl, float& sh, float& sl) {
    const float p = __fmul_rn(ah, bh);
    const float e = __fmaf_rn(ah, bh, -p);
    const float c = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
    float t;
    two_sum(sh, p, sh, t);
    sl += t + c;
}

// (h, l) += (oh, ol) for unnormalised accumulators
__device__ __forceinline__ void ff_acc(float& h, float& l, float oh, float ol) {
    float t;
    two_sum(h, oh, h, t);
    l = l + ol + t;
}

__device__ __forceinline__ float2 ff_norm(float h, float l) {
    float s, e;
    fast_two_sum(h, l, s, e);
    return make_float2(s, e);
}

__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    float s, e;
    two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    return ff_norm(s, e);
}

__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e));
    return ff_norm(p, e);
}

// a b + c
__device__ __forceinline__ float2 ff_fma(float2 a, float2 b, float2 c) { return ff_add(ff_mul(a, b), c); }

__device__ __forceinline__ double ff_to_double(float2 a) { return (double)a.x + (double)a.y; }

// a / b: two-term long division (Dekker): q1 ~ a.hi / b.hi, q2 from the
// float-float remainder a - q1 b (formed exactly), so q1 needs only FP32
// accuracy and comes from the fast approximate divide; relative error
// ~2^-44.  b must be a normal, nonzero number.
__device__ __forceinline__ float2 ff_div(float2 a, float2 b) {
    const float q1 = __fdividef(a.x, b.x);
    const float2 r = ff_add(a, ff_neg(ff_mul(make_float2(q1, 0.f), b)));
    const float q2 = __fdividef(r.x, b.x);
    return ff_norm(q1, q2);
}

// sqrt(a), a >= 0 (Karp and Markstein): y = a.hi rsqrt(a.hi), then two
// Newton corrections y + (a - y^2) / (2 y), the residual a - y^2 formed in
// float-float each time.
__device__ __forceinline__ float2 ff_sqrt(float2 a) {
    if (!(a.x > 0.f)) return make_float2(0.f, 0.f);
    const float x = rsqrtf(a.x);
    const float hx = __fmul_rn(x, 0.5f);
    const float y = __fmul_rn(a.x, x);
    const float p = __fmul_rn(y, y);
    const float e = __fmaf_rn(y, y, -p);
    const float2 r = ff_add(a, make_float2(-p, -e));
    const float2 y2 = ff_norm(y, __fmul_rn(r.x, hx));
    const float2 r2 = ff_add(a, ff_neg(ff_mul(y2, y2)));
    return ff_add(y2, make_float2(__fmul_rn(r2.x, hx), 0.f));
}

// FP64 -> (hi, lo) with integer operations only (no FP64 pipe): hi = v
// rounded to 24 bits (half up in magnitude), lo = the remainder rounded to
// 24 bits, so hi + lo carries 48 bits of v.  Values outside 2^+-100 take the
// conversion route.
__device__ __forceinline__ float2 ff_split(double v) {
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 100 || e > 1023 + 100) {
        if (e == 0 && (b << 1) == 0) return make_float2(__uint_as_float((uint32_t)(b >> 32) & 0x80000000u), 0.f);
        const float h = __double2float_rn(v);
        return make_float2(h, __double2float_rn(v - (double)h));
    }
    const uint32_t sign = (uint32_t)(b >> 63);
    const uint64_t M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    uint64_t Mh = (M + (1ull << 28)) >> 29;
    int eh = e;
    if (Mh >> 24) { Mh >>= 1; ++eh; }
    const uint32_t hb = (sign << 31) | ((uint32_t)(eh - 896) << 23) | ((uint32_t)Mh & 0x7FFFFFu);
    const long long rem = (long long)M - (long long)(Mh << (29 + (eh - e)));   // |rem| <= 2^28
    float lo = 0.f;
    if (rem != 0) {
        const float rf = (float)(sign ? -rem : rem);
        const int be = (int)((__float_as_uint(rf) >> 23) & 0xff) + (e - 1075);
        if (be > 0) lo = __uint_as_float((__float_as_uint(rf) & 0x807FFFFFu) | ((uint32_t)be << 23));
    }
    return make_float2(__uint_as_float(hb), lo);
}

// Butterfly sum over the warp of an unnormalised accumulator; every lane
// receives lane 0's result, so all lanes hold identical bits.
__device__ __forceinline__ float2 ff_warp_sum(float h, float l) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, o);
        const float ol = __shfl_xor_sync(0xffffffffu, l, o);
        ff_acc(h, l, oh, ol);
    }
    h = __shfl_sync(0xffffffffu, h, 0);
    l = __shfl_sync(0xffffffffu, l, 0);
    return ff_norm(h, l);
}

}  // namespace rnla

// ---------------------------------------------------------------------------
// Packed pairs: two independent FP32 values in one 64-bit register pair,
// operated on by the sm_100+ .f32x2 instructions (one instruction, two
// IEEE round-to-nearest results).  ff2_* apply the float-float operations
// above to two independent lanes at once.
// ---------------------------------------------------------------------------
namespace rnla {

typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 upk2(f32x2 r) {
    float a, b;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
    return make_float2(a, b);
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f32x2 neg2(f32x2 a) { return a ^ 0x8000000080000000ull; }

// (sh, sl) += (ah + al)(bh + bl) on both lanes (see ff_madd); nbh = -bh is
// passed in (b is reused across many a, so the negation is hoisted) and the
// TwoSum is written around -p: 12 instructions for two multiply-adds.
__device__ __forceinline__ void ff2_madd(f32x2 ah, f32x2 al, f32x2 bh, f32x2 nbh, f32x2 bl, f32x2& sh,
                                         f32x2& sl) {
    const f32x2 np = mul2(ah, nbh);                        // -p, p = ah bh
    const f32x2 e = fma2(ah, bh, np);                      // ah bh - p, exact
    const f32x2 c = fma2(ah, bl, fma2(al, bh, e));
    const f32x2 s = sub2(sh, np);                          // sh + p
    const f32x2 bp = sub2(s, sh);
    const f32x2 t = sub2(sub2(sh, sub2(s, bp)), add2(np, bp));
    sh = s;
    sl = add2(sl, add2(t, c));
}

// (sh, sl) += a (bh + bl) on both lanes for an exact FP32 pair a (a value
// with no low part): ff2_madd without the al bh term, 11 instructions.
__device__ __forceinline__ void ff2_madd_x(f32x2 a, f32x2 bh, f32x2 nbh, f32x2 bl, f32x2& sh, f32x2& sl) {
    const f32x2 np = mul2(a, nbh);                         // -p, p = a bh
    const f32x2 e = fma2(a, bh, np);                       // a bh - p, exact
    const f32x2 c = fma2(a, bl, e);
    const f32x2 s = sub2(sh, np);                          // sh + p
    const f32x2 bp = sub2(s, sh);
    const f32x2 t = sub2(sub2(sh, sub2(s, bp)), add2(np, bp));
    sh = s;
    sl = add2(sl, add2(t, c));
}

// The same with -bh formed on the fly (one integer sign flip instead of a
// register pair holding -bh).
__device__ __forceinline__ void ff2_madd_xp(f32x2 a, f32x2 bh, f32x2 bl, f32x2& sh, f32x2& sl) {
    const f32x2 p = mul2(a, bh);
    const f32x2 np = neg2(p);
    const f32x2 e = fma2(a, bh, np);                       // a bh - p, exact
    const f32x2 c = fma2(a, bl, e);
    const f32x2 s = add2(sh, p);                           // sh + p
    const f32x2 bp = sub2(s, sh);
    const f32x2 t = add2(sub2(sh, sub2(s, bp)), sub2(p, bp));
    sh = s;
    sl = add2(sl, add2(t, c));
}

// (h, l) += (oh, ol) on both lanes (see ff_acc)
__device__ __forceinline__ void ff2_acc(f32x2& h, f32x2& l, f32x2 oh, f32x2 ol) {
    const f32x2 s = add2(h, oh);
    const f32x2 bp = sub2(s, h);
    const f32x2 t = add2(sub2(h, sub2(s, bp)), sub2(oh, bp));
    h = s;
    l = add2(add2(l, ol), t);
}

}  // namespace rnla
