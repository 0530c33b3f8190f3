// gray_device.cuh -- device-side arithmetic shared by the gray_gb300 kernels.
//
// Every expression here is evaluated exactly as written: the library is compiled with
// -fmad=false (no implicit FMA contraction) and without --use_fast_math, and fmaf appears
// only where an FMA is intended.  Together with the project's own exp/log below this makes
// hit lists, fp16 keys and composited transmittance reproducible bit-for-bit on the CPU.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/gray_gb300.h"

#define GRAY_LEAF_BIT 0x80000000u
#define GRAY_NULL 0xFFFFFFFFu

namespace gray {

// ---------------------------------------------------------------------------------------------
// exp: Cody & Waite argument reduction (x = k ln2 + r, |r| <= ln2/2, ln2 carried as two floats)
// and the degree-7 Taylor polynomial of e^r in Horner form; 2^k applied through the exponent
// field (two steps for results in the subnormal range).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float exp_poly(float x, int &ki) {
    float k = rintf(x * 0x1.715476p+0f);
    float r = fmaf(-k, 0x1.62ep-1f, x);
    r = fmaf(-k, 0x1.0bfbe8p-15f, r);
    float p = 0x1.a01a02p-13f;
    p = fmaf(p, r, 0x1.6c16c2p-10f);
    p = fmaf(p, r, 0x1.111112p-7f);
    p = fmaf(p, r, 0x1.555556p-5f);
    p = fmaf(p, r, 0x1.555556p-3f);
    p = fmaf(p, r, 0x1.0p-1f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    ki = (int)k;
    return p;
}

__device__ __forceinline__ float gexp(float x) {
    int ki;
    // |x| <= 87: k in [-126, 126], 2^k a normal float (the hit loop's case: one test)
    if (fabsf(x) <= 87.0f) {
        float p = exp_poly(x, ki);
        return p * __int_as_float((ki + 127) << 23);
    }
    if (x != x) return x;
    if (x > 89.0f) return __int_as_float(0x7f800000);
    if (x < -104.0f) return 0.0f;
    float p = exp_poly(x, ki);
    if (ki > 127) {
        p = p * 2.0f;
        ki -= 1;
    }
    if (ki < -126) {
        p = p * __int_as_float((ki + 64 + 127) << 23);
        return p * 0x1.0p-64f;
    }
    return p * __int_as_float((ki + 127) << 23);
}

// log: x = m 2^e, m in [sqrt(1/2), sqrt(2)]; log m = 2 atanh(s), s = (m-1)/(m+1), series to s^11.
__device__ __forceinline__ float log_poly(float m, int e) {
    if (m > 0x1.6a09e6p+0f) {
        m = m * 0.5f;
        e += 1;
    }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float q = 0x1.745d18p-4f;
    q = fmaf(q, z, 0x1.c71c72p-4f);
    q = fmaf(q, z, 0x1.24924ap-3f);
    q = fmaf(q, z, 0x1.99999ap-3f);
    q = fmaf(q, z, 0x1.555556p-2f);
    float two_s = 2.0f * s;
    float lm = fmaf(two_s * z, q, two_s);
    float ef = (float)e;
    return fmaf(ef, 0x1.62ep-1f, fmaf(ef, 0x1.0bfbe8p-15f, lm));
}

__device__ __forceinline__ float glog(float x) {
    uint32_t u = __float_as_uint(x);
    // positive normal x (the hit loop's case: one test)
    if (u - 0x00800000u < 0x7f000000u)
        return log_poly(__uint_as_float((u & 0x007fffffu) | 0x3f800000u), (int)(u >> 23) - 127);
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    x = x * 0x1.0p23f;  // positive subnormal
    u = __float_as_uint(x);
    return log_poly(__uint_as_float((u & 0x007fffffu) | 0x3f800000u), (int)(u >> 23) - 127 - 23);
}

__device__ __forceinline__ float gpow(float a, float b) { return gexp(b * glog(a)); }

__device__ __forceinline__ float sigmoid_act(float x) { return 1.0f / (1.0f + gexp(-x)); }

// MAX_ALPHA (the double 0.9999) * a * b with a single final rounding: a*b split exactly by an
// FMA, 0.9999 carried as a float pair.
__device__ __forceinline__ float maxalpha_mul(float a, float b) {
    const float c_hi = 0x1.fff2e4p-1f, c_lo = 0x1.1d14e4p-26f;
    float p = a * b;
    float e = fmaf(a, b, -p);
    return fmaf(c_hi, p, fmaf(c_hi, e, c_lo * p));
}

// Scaling factor that clips the Gaussian where its alpha falls to alpha_threshold
// (reference: cuda/utils/kernel.cu:3-22).
__device__ __forceinline__ float scaling_factor(float opacity, float alpha_threshold, float exp_power) {
    if (opacity <= alpha_threshold) return 0.0f;
    float log_ratio = glog(opacity / alpha_threshold);
    if (exp_power == 1.0f) return sqrtf(2.0f * log_ratio);
    if (exp_power == 2.0f) return sqrtf(sqrtf(4.0f * log_ratio));
    if (exp_power == 3.0f) {
        float v = sqrtf(6.0f * log_ratio);
        return v == 0.0f ? 0.0f : gexp(glog(v) * 0x1.555556p-2f);
    }
    float k = 2.0f * exp_power;
    return gpow(k * log_ratio, 1.0f / k);
}

// Gaussian response at squared local radius d (reference: cuda/utils/kernel.cu:24-38).
__device__ __forceinline__ float eval_gaussian(float d, float exp_power) {
    if (exp_power == 1.0f) return gexp(-0.5f * d);
    if (exp_power == 2.0f) return gexp(-0.25f * d * d);
    if (exp_power == 3.0f) return gexp(-(d * d * d) / 6.0f);
    float k = 2.0f * exp_power;
    return gexp(-gpow(d, exp_power) / k);
}

// beta^n rounded to float (binary exponentiation in double), for Adam's bias correction.
__device__ __forceinline__ float adam_pow(float beta, int n) {
    double b = (double)beta, r = 1.0;
    unsigned int k = (unsigned int)(n < 0 ? 0 : n);
    while (k) {
        if (k & 1u) r *= b;
        b *= b;
        k >>= 1;
    }
    return (float)r;
}

// Fixed-point form of one all-hit sum term: v * scale (scale a power of two) truncated toward
// zero, clamped to +-2^62, NaN -> 0.  Decoded from the float's bits with integer operations only
// (a float-to-int64 conversion would go through the FP64 unit, which is narrow on GB300):
// |t| = m 2^(e-150) with m the 24-bit significand, so trunc(|t|) = m << (e-150) or m >> (150-e).
__device__ __forceinline__ long long to_fixed(float v, float scale) {
    const uint32_t b = __float_as_uint(v * scale);
    const uint32_t e = (b >> 23) & 0xFFu;
    if (e < 127u) return 0;                                // |t| < 1 (zero, subnormal)
    if (e == 0xFFu && (b & 0x7FFFFFu)) return 0;           // NaN
    unsigned long long mag;
    if (e >= 189u) {
        mag = 1ull << 62;                                  // |t| >= 2^62 (inf included)
    } else {
        const unsigned long long m = (unsigned long long)((b & 0x7FFFFFu) | 0x800000u);
        mag = e >= 150u ? m << (e - 150u) : m >> (150u - e);
    }
    return (b >> 31) ? -(long long)mag : (long long)mag;
}

__device__ __forceinline__ uint16_t f2h_bits(float f) { return __half_as_ushort(__float2half_rn(f)); }
__device__ __forceinline__ float h2f_bits(uint16_t h) { return __half2float(__ushort_as_half(h)); }

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// a.b as an FMA chain: fma(a.z, b.z, fma(a.y, b.y, a.x * b.x))
__device__ __forceinline__ float fdot3(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ float fdot3(float4 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }

// Object-space ray of one Gaussian and its max-density point (reference: cuda/shaders.cu:17-49).
// g0..g2 = rows (M | mu) of the snapshot.  With lo = M (o - mu) and ld = M d (d a unit world
// direction), the max-density point is at world distance t = -<lo,ld> / <ld,ld> (the reference
// normalises ld and divides by its length twice; the value is the same) and u = lo + t ld.
struct LocalHit {
    f3 lo, ld;  // object-space origin and direction
    float b;    // <lo, ld>
    float t;    // world distance of the max-density point
    f3 u;       // max-density point in the unit-sphere frame
};

__device__ __forceinline__ void local_ray(const float4 g0, const float4 g1, const float4 g2, f3 ro, f3 rd,
                                          LocalHit &h) {
    f3 rel = mk3(ro.x - g0.w, ro.y - g1.w, ro.z - g2.w);
    h.lo = mk3(fdot3(g0, rel), fdot3(g1, rel), fdot3(g2, rel));
    h.ld = mk3(fdot3(g0, rd), fdot3(g1, rd), fdot3(g2, rd));
    h.b = fdot3(h.lo, h.ld);
}

__device__ __forceinline__ void closest_point(LocalHit &h) {
    h.t = -h.b / fdot3(h.ld, h.ld);
    h.u = mk3(fmaf(h.t, h.ld.x, h.lo.x), fmaf(h.t, h.ld.y, h.lo.y), fmaf(h.t, h.ld.z, h.lo.z));
}

// Segment [znear, zfar] of the object-space ray against the instance's unit box [-1, 1]^3 (the
// candidate test OptiX applies before the intersection program).
__device__ __forceinline__ bool unit_box_overlap(const LocalHit &h, float znear, float zfar) {
    float t0 = znear, t1 = zfar;
    const float lo[3] = {h.lo.x, h.lo.y, h.lo.z}, ld[3] = {h.ld.x, h.ld.y, h.ld.z};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float inv = 1.0f / ld[k];
        float ta = (-1.0f - lo[k]) * inv, tb = (1.0f - lo[k]) * inv;
        t0 = fmaxf(t0, fminf(ta, tb));
        t1 = fminf(t1, fmaxf(ta, tb));
    }
    return t0 <= t1;
}

// Intersection program (reference: cuda/shaders.cu:10-67) for one (ray, Gaussian) pair.
// o = live opacity (or -inf if the snapshot marked the Gaussian invisible), sf = live scaling
// factor.  Returns true on a hit with the world distance and fp32 alpha.
__device__ __forceinline__ bool intersect(const float4 g0, const float4 g1, const float4 g2, float o, float sf, f3 ro,
                                          f3 rd, float alpha_threshold, float exp_power, float znear, float zfar,
                                          float &dist, float &alpha) {
    if (o <= alpha_threshold) return false;
    LocalHit h;
    local_ray(g0, g1, g2, ro, rd, h);
    if (h.b > 0.0f) return false;
    closest_point(h);
    float sq = fdot3(h.u, h.u);
    if (sq > 1.0f) return false;
    dist = h.t;
    if (!(dist >= znear && dist <= zfar)) {
        if (!unit_box_overlap(h, znear, zfar)) return false;
    }
    f3 x = mk3(h.u.x * sf, h.u.y * sf, h.u.z * sf);
    float gv = eval_gaussian(fdot3(x, x), exp_power);
    alpha = maxalpha_mul(gv, o);
    return true;
}

// Full transmittance prod(1 - alpha) over all hits of a ray, kept order-independent: the sum of
// log(1 - alpha) in 2^-40 fixed point, exponentiated once at the end.  Terms are <= 0; once the sum
// is below -105 (exp underflows to 0 in fp32) further terms are not added, which bounds it for any
// number of hits.
constexpr long long kLogFixFloor = -105LL * (1LL << 40);
__device__ __forceinline__ void add_log_transmittance(long long &s, float alpha) {
    if (s > kLogFixFloor) s += to_fixed(glog(1.0f - alpha), 0x1.0p40f);
}
__device__ __forceinline__ float full_transmittance(long long s) { return gexp(__ll2float_rn(s) * 0x1.0p-40f); }

// Object-space origin lo = M (o - mu) of a snapshot (rows g0..g2 = (M | mu)), as local_ray computes it.
__device__ __forceinline__ f3 local_origin(const float4 g0, const float4 g1, const float4 g2, f3 ro) {
    const f3 rel = mk3(ro.x - g0.w, ro.y - g1.w, ro.z - g2.w);
    return mk3(fdot3(g0, rel), fdot3(g1, rel), fdot3(g2, rel));
}

// local_ray for rows whose w column already holds the object-space origin lo (rays that share one
// origin: lo is computed once per Gaussian with local_origin, the same arithmetic).
__device__ __forceinline__ void local_ray_lo(const float4 m0, const float4 m1, const float4 m2, f3 rd, LocalHit &h) {
    h.lo = mk3(m0.w, m1.w, m2.w);
    h.ld = mk3(fdot3(m0, rd), fdot3(m1, rd), fdot3(m2, rd));
    h.b = fdot3(h.lo, h.ld);
}

// intersect() for rows (M | lo) from local_origin: the same arithmetic, so the same answer.
__device__ __forceinline__ bool intersect_lo(const float4 m0, const float4 m1, const float4 m2, float o, float sf,
                                             f3 rd, float alpha_threshold, float exp_power, float znear, float zfar,
                                             float &dist, float &alpha) {
    if (o <= alpha_threshold) return false;
    LocalHit h;
    local_ray_lo(m0, m1, m2, rd, h);
    if (h.b > 0.0f) return false;
    closest_point(h);
    float sq = fdot3(h.u, h.u);
    if (sq > 1.0f) return false;
    dist = h.t;
    if (!(dist >= znear && dist <= zfar)) {
        if (!unit_box_overlap(h, znear, zfar)) return false;
    }
    f3 x = mk3(h.u.x * sf, h.u.y * sf, h.u.z * sf);
    float gv = eval_gaussian(fdot3(x, x), exp_power);
    alpha = maxalpha_mul(gv, o);
    return true;
}

// Division-free, conservative form of the hit decision of intersect() for the object-space ray
// (lo, ld) with b = <lo, ld> as local_ray computes them: false only when intersect() on the same
// lo, ld and b reports no hit (b > 0, or the max-density point outside the unit sphere); a true
// may still be a miss.  The line's squared distance from the centre is |lo x ld|^2 / |ld|^2, and a
// hit of intersect() puts it at most 1 + 5 ulp: its u is lo + t ld rounded, a point of the line.
// The cross product's roundings are relative to |lo|_inf |ld| (linear, not quadratic, in |lo|), so
// with q = 2^-24 |lo|_inf the computed C = |c|^2 stays below |ld|^2 (1 + 64 ulp + 4q + 4q^2) for
// every hit; the range conditions keep every product finite and away from subnormals (outside them
// the answer is true).  The all-pairs hit test of a packet runs this; the intersection program
// (intersect, intersect_lo) decides, so results do not depend on it.
__device__ __forceinline__ bool may_hit_local(f3 lo, f3 ld, float b) {
    if (b > 0.0f) return false;
    const float L = fdot3(ld, ld);
    const float p0 = lo.z * ld.y, p1 = lo.x * ld.z, p2 = lo.y * ld.x;
    const f3 c = mk3(fmaf(lo.y, ld.z, -p0), fmaf(lo.z, ld.x, -p1), fmaf(lo.x, ld.y, -p2));
    const float C = fdot3(c, c);
    const float li = fmaxf(fabsf(lo.x), fmaxf(fabsf(lo.y), fabsf(lo.z)));
    const float q4 = li * 0x1.0p-22f;
    const float k = fmaf(q4, fmaf(q4, 0.25f, 1.0f), 1.0f + 0x1.0p-18f);
    return !(C > L * k && li <= 0x1.0p40f && L >= 0x1.0p-60f && L <= 0x1.0p40f);
}

// may_hit_local() for rows (M | lo) from local_origin, with the opacity test of intersect_lo().
__device__ __forceinline__ bool may_hit_lo(const float4 m0, const float4 m1, const float4 m2, float o, f3 rd,
                                           float alpha_threshold) {
    if (o <= alpha_threshold) return false;
    LocalHit h;
    local_ray_lo(m0, m1, m2, rd, h);
    return may_hit_local(h.lo, h.ld, h.b);
}

// Colour in 2^-24 fixed point (clamped to [-64, 64], so it fits 31 bits): the tail sums add
// alpha16_fixed(a) * colour_fixed(c), an exact 64-bit product in 2^-48 units.
__device__ __forceinline__ int colour_fixed(float c) {
    return (int)to_fixed(fminf(fmaxf(c, -64.0f), 64.0f), 0x1.0p24f);
}
__device__ __forceinline__ long long mul_fixed(long long a16fix, int cfix) {
    return (long long)(int)a16fix * (long long)cfix;
}

// alpha * 2^24 for an fp16 alpha in [0, 1): an exact integer, from the half's bits
__device__ __forceinline__ long long alpha16_fixed(uint16_t a16) {
    const uint32_t e = (a16 >> 10) & 0x1fu, m = a16 & 0x3ffu;
    return e ? (long long)((1024u + m) << (e - 1u)) : (long long)m;
}

// Device-side error reporting: bits are OR-ed into a status word; the host reads it later.
__device__ __forceinline__ void raise_status(int32_t *status, int32_t bits) {
    if (status) atomicOr(status, bits);
}

}  // namespace gray
