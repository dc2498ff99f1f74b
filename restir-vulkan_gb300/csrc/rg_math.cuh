// rg_math.cuh -- arithmetic of the ReSTIR hot path, shared by the CUDA
// kernels and the host-side G-buffer tracer.
//
// Every function fixes one operation order, and every translation unit that
// includes this header is compiled without FMA contraction (nvcc -fmad=false,
// g++ -ffp-contract=off) and with IEEE division and square root, so the same
// inputs give the same bits on the host and on the GPU.  The GLSL built-ins
// the reference shaders rely on are given these meanings:
//   min(x,y) = y<x ? y : x, max(x,y) = x<y ? y : x  (GLSL 4.50 section 8.3)
//   clamp(x,a,b) = min(max(x,a),b), mix(x,y,a) = x*(1-a) + y*a
//   dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, normalize(v) = v / sqrt(dot(v,v))
//   pow(r, 2.0) = r*r, round() half away from zero
//   cos/sin: Cody-Waite reduction by pi/2 plus Taylor polynomials (sincos_cw)
// Reference paths are relative to the reference project root.
#pragma once
#include <stdint.h>
#include <math.h>

#ifdef __CUDACC__
#define RG_HD __host__ __device__ __forceinline__
#else
#define RG_HD inline
#endif

namespace rgm {

constexpr float kPi = 3.14159274101257324f;        // (float)M_PI, disneyBRDF.glsl:1 (GLSL float literal)
constexpr float kDeg2Rad = 0.0174532923847436905f; // (float)(pi/180), GLSL radians()

struct f3 { float x, y, z; };
RG_HD f3 mk(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
RG_HD f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
RG_HD f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
RG_HD f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
RG_HD f3 scale(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
RG_HD f3 divs(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
RG_HD float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
RG_HD f3 cross(f3 a, f3 b) { return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
RG_HD f3 normalize(f3 a) { return divs(a, sqrtf(dot(a, a))); }
RG_HD float gmin(float x, float y) { return y < x ? y : x; }
RG_HD float gmax(float x, float y) { return x < y ? y : x; }
RG_HD float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
RG_HD float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
RG_HD int imin(int a, int b) { return b < a ? b : a; }
RG_HD int imax(int a, int b) { return a < b ? b : a; }
RG_HD int iclamp(int x, int lo, int hi) { return imin(imax(x, lo), hi); }

// ---------------------------------------------------------------- PCG32 (rand.glsl:7-32)
struct Pcg { uint64_t state, inc; };
RG_HD uint32_t pcg_next(Pcg &r) {
    uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + r.inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
RG_HD Pcg pcg_seed(uint64_t seed, uint64_t seq) {
    Pcg r;
    r.state = 0;
    r.inc = (seq << 1u) | 1u;
    pcg_next(r);
    r.state += seed;
    pcg_next(r);
    return r;
}
// uint -> float rounds to nearest, then an exact scaling by 2^-32; may be 1.0.
RG_HD float rand_float(Pcg &r) { return (float)pcg_next(r) / 4294967296.0f; }

// ---------------------------------------------------------------- sin / cos
// x = k*(pi/2) + y, pi/2 = C1 + C2 + C3 with C1 (8 bits) and C2 (12 bits)
// short enough that k*C1, k*C2 are exact for |k| < 2^12; Taylor series of sin
// to y^9 and cos to y^10 on |y| <= pi/4 (truncation error < 2e-9).
RG_HD void sincos_cw(float x, float &s, float &c) {
    const float k = rintf(x * 0.636619746685028076f);
    const float y = ((x - k * 1.5703125f) - k * 4.83870506286621094e-4f) - k * -4.37113882867379300e-8f;
    const float y2 = y * y;
    const float ps = ((2.75573188446287531e-6f * y2 - 1.98412701138295233e-4f) * y2 + 8.33333376795053482e-3f) * y2
                     - 0.166666671633720398f;
    const float sy = y + (y * y2) * ps;
    const float pc = ((2.48015876422869042e-5f - 2.75573199814971304e-7f * y2) * y2 - 1.38888892251998186e-3f) * y2
                     + 4.16666679084300995e-2f;
    const float cy = (1.0f - 0.5f * y2) + (y2 * y2) * pc;
    const int q = ((int)k) & 3;
    if (q == 0) { s = sy; c = cy; }
    else if (q == 1) { s = cy; c = -sy; }
    else if (q == 2) { s = -sy; c = -cy; }
    else { s = -cy; c = sy; }
}
RG_HD float cos_cw(float x) { float s, c; sincos_cw(x, s, c); return c; }

RG_HD float luminance(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; } // common.glsl:7-9

// ---------------------------------------------------------------- Disney BRDF (disneyBRDF.glsl:5-90)
RG_HD float schlick_fresnel(float c) {
    const float m = gclamp(1.0f - c, 0.0f, 1.0f);
    const float sm = m * m;
    return sm * sm * m;
}
RG_HD float gtr2(float ndoth, float a) {
    const float a2 = a * a;
    const float t = 1.0f + (a2 - 1.0f) * ndoth * ndoth;
    return a2 / (kPi * t * t);
}
RG_HD float smith_g_ggx(float ndotv, float alpha_g) {
    const float a = alpha_g * alpha_g;
    const float b = ndotv * ndotv;
    return 1.0f / (fabsf(ndotv) + gmax(sqrtf(a + b - a * b), 0.0001f));
}
RG_HD float diffuse_factor(float cos_in, float cos_out, float cos_in_half, float roughness, float metallic) {
    const float f_in = schlick_fresnel(cos_in);
    const float f_out = schlick_fresnel(cos_out);
    const float fd90 = 0.5f + 2.0f * cos_in_half * cos_in_half * roughness;
    const float fd = gmix(1.0f, fd90, f_in) * gmix(1.0f, fd90, f_out);
    return fd * (1.0f - metallic) / kPi;
}
RG_HD void specular_factors(float cos_in, float cos_out, float cos_half, float cos_in_half, float roughness,
                            float &fresnel, float &gd) {
    fresnel = schlick_fresnel(cos_in_half);
    const float a = gmax(0.001f, roughness * roughness);
    const float ds = gtr2(cos_half, a);
    float gs = smith_g_ggx(cos_in, a);
    gs *= smith_g_ggx(cos_out, a);
    gd = gs * ds;
}
RG_HD float brdf_lum(float cos_in, float cos_out, float cos_half, float cos_in_half, float lum, float roughness,
                     float metallic) {
    if (cos_in < 0.0f) return 0.0f;
    const float diffuse = lum * diffuse_factor(cos_in, cos_out, cos_in_half, roughness, metallic);
    float fr, gd;
    specular_factors(cos_in, cos_out, cos_half, cos_in_half, roughness, fr, gd);
    const float fs = gmix(gmix(0.04f, lum, metallic), 1.0f, fr);
    return diffuse + fs * gd;
}
RG_HD f3 brdf_color(float cos_in, float cos_out, float cos_half, float cos_in_half, f3 albedo, float roughness,
                    float metallic) {
    if (cos_in < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    const float df = diffuse_factor(cos_in, cos_out, cos_in_half, roughness, metallic);
    const f3 diffuse = mk(albedo.x * df, albedo.y * df, albedo.z * df);
    float fr, gd;
    specular_factors(cos_in, cos_out, cos_half, cos_in_half, roughness, fr, gd);
    const f3 fs = mk(gmix(gmix(0.04f, albedo.x, metallic), 1.0f, fr), gmix(gmix(0.04f, albedo.y, metallic), 1.0f, fr),
                     gmix(gmix(0.04f, albedo.z, metallic), 1.0f, fr));
    return diffuse + mk(fs.x * gd, fs.y * gd, fs.z * gd);
}

// ---------------------------------------------------------------- target function (restirUtils.glsl:3-55)
// wo = normalize(cam - worldPos) depends on the pixel only; callers in loops
// compute it once (the value is the same as computing it per call).
RG_HD f3 view_dir(f3 cam, f3 wpos) { return normalize(cam - wpos); }

RG_HD float eval_phat_wo(f3 wpos, f3 lpos, f3 wo, f3 n, f3 ln, bool use_ln, float albedo_lum, float emission_lum,
                         float roughness, float metallic) {
    f3 wi = lpos - wpos;
    if (dot(wi, n) < 0.0f) return 0.0f;
    const float sqr_dist = dot(wi, wi);
    wi = divs(wi, sqrtf(sqr_dist));
    const float cos_in = dot(n, wi);
    const float cos_out = dot(n, wo);
    const f3 h = normalize(wi + wo);
    const float cos_half = dot(n, h);
    const float cos_in_half = dot(wi, h);
    float geometry = cos_in / sqr_dist;
    if (use_ln) geometry *= fabsf(dot(wi, ln));
    return emission_lum * brdf_lum(cos_in, cos_out, cos_half, cos_in_half, albedo_lum, roughness, metallic) * geometry;
}
// eval_phat_wo with the terms that depend on the shading point only (the
// view-side cosine, Fresnel and Smith term, alpha, the specular base)
// computed once per pixel: the same operations on the same values, so the
// same result.
struct PhatPx {
    f3 wpos, wo, n;
    float lum, roughness, metallic;
    float cos_out, f_out, a, g_out, spec0;
};
RG_HD PhatPx phat_px(f3 wpos, f3 wo, f3 n, float albedo_lum, float roughness, float metallic) {
    PhatPx p;
    p.wpos = wpos;
    p.wo = wo;
    p.n = n;
    p.lum = albedo_lum;
    p.roughness = roughness;
    p.metallic = metallic;
    p.cos_out = dot(n, wo);
    p.f_out = schlick_fresnel(p.cos_out);
    p.a = gmax(0.001f, roughness * roughness);
    p.g_out = smith_g_ggx(p.cos_out, p.a);
    p.spec0 = gmix(0.04f, albedo_lum, metallic);
    return p;
}
RG_HD float eval_phat_px(const PhatPx &p, f3 lpos, f3 ln, bool use_ln, float emission_lum) {
    f3 wi = lpos - p.wpos;
    if (dot(wi, p.n) < 0.0f) return 0.0f;
    const float sqr_dist = dot(wi, wi);
    wi = divs(wi, sqrtf(sqr_dist));
    const float cos_in = dot(p.n, wi);
    const f3 h = normalize(wi + p.wo);
    const float cos_half = dot(p.n, h);
    const float cos_in_half = dot(wi, h);
    float geometry = cos_in / sqr_dist;
    if (use_ln) geometry *= fabsf(dot(wi, ln));
    float b = 0.0f;  // brdf_lum
    if (!(cos_in < 0.0f)) {
        const float f_in = schlick_fresnel(cos_in);
        const float fd90 = 0.5f + 2.0f * cos_in_half * cos_in_half * p.roughness;
        const float fd = gmix(1.0f, fd90, f_in) * gmix(1.0f, fd90, p.f_out);
        const float diffuse = p.lum * (fd * (1.0f - p.metallic) / kPi);
        const float fr = schlick_fresnel(cos_in_half);
        const float ds = gtr2(cos_half, p.a);
        float gs = smith_g_ggx(cos_in, p.a);
        gs *= p.g_out;
        const float gd = gs * ds;
        const float fs = gmix(p.spec0, 1.0f, fr);
        b = diffuse + fs * gd;
    }
    return emission_lum * b * geometry;
}
RG_HD f3 eval_phat_full(f3 wpos, f3 lpos, f3 cam, f3 n, f3 ln, bool use_ln, f3 albedo, f3 emission, float roughness,
                        float metallic) {
    f3 wi = lpos - wpos;
    if (dot(wi, n) < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    const float sqr_dist = dot(wi, wi);
    wi = divs(wi, sqrtf(sqr_dist));
    const f3 wo = normalize(cam - wpos);
    const float cos_in = dot(n, wi);
    const float cos_out = dot(n, wo);
    const f3 h = normalize(wi + wo);
    const float cos_half = dot(n, h);
    const float cos_in_half = dot(wi, h);
    float geometry = cos_in / sqr_dist;
    if (use_ln) geometry *= fabsf(dot(wi, ln));
    const f3 e = emission * brdf_color(cos_in, cos_out, cos_half, cos_in_half, albedo, roughness, metallic);
    return mk(e.x * geometry, e.y * geometry, e.z * geometry);
}

// ---------------------------------------------------------------- intersection (softwareRaytracing.glsl:3-37)
RG_HD bool ray_aabb(f3 o, f3 d, f3 bmin, f3 bmax) {
    const float t0x = (bmin.x - o.x) / d.x, t1x = (bmax.x - o.x) / d.x;
    const float t0y = (bmin.y - o.y) / d.y, t1y = (bmax.y - o.y) / d.y;
    const float t0z = (bmin.z - o.z) / d.z, t1z = (bmax.z - o.z) / d.z;
    const float rmin = gmax(gmin(t0x, t1x), gmax(gmin(t0y, t1y), gmin(t0z, t1z)));
    const float rmax = gmin(gmax(t0x, t1x), gmin(gmax(t0y, t1y), gmax(t0z, t1z)));
    return rmin < 1.0f && rmax >= rmin && rmax > 0.0f;
}
// Moeller-Trumbore segment test with e1 = p2-p1, e2 = p3-p1 precomputed (the
// same single subtractions the reference performs per test).
RG_HD bool ray_tri(f3 p1, f3 e1, f3 e2, f3 o, f3 d) {
    const f3 p = cross(d, e2);
    float f = 1.0f / dot(e1, p);
    const f3 s = o - p1;
    const float bx = f * dot(s, p);
    if (bx < 0.0f || bx > 1.0f) return false;
    const f3 q = cross(s, e1);
    const float by = f * dot(d, q);
    if (by < 0.0f || by + bx > 1.0f) return false;
    f *= dot(e2, q);
    return f > 0.0f && f < 1.0f;
}
// Shadow segment of testVisibility (visibilityTest.glsl:1-4,26-29).
RG_HD void shadow_segment(f3 p1, f3 p2, f3 &o, f3 &d) {
    const float tmin = 0.001f;
    const f3 dir = p2 - p1;
    const f3 off = scale(tmin, normalize(dir));
    o = p1 + off;
    d = dir - scale(2.0f, off);
}

// ---------------------------------------------------------------- G-buffer decoding
RG_HD float half_bits_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t ex = (h >> 10) & 0x1fu;
    uint32_t man = h & 0x3ffu;
    uint32_t bits;
    if (ex == 0) {
        if (man == 0) {
            bits = sign;
        } else {
            int e = -1;
            do { ++e; man <<= 1; } while (!(man & 0x400u));
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3ffu) << 13);
        }
    } else if (ex == 31) {
        bits = sign | 0x7f800000u | (man << 13);
    } else {
        bits = sign | ((ex + 112u) << 23) | (man << 13);
    }
    union { uint32_t u; float f; } cv;
    cv.u = bits;
    return cv.f;
}
// float -> half, round to nearest even (used to write the G-buffer normal).
RG_HD uint16_t float_to_half_bits(float f) {
    union { float f; uint32_t u; } cv;
    cv.f = f;
    const uint32_t x = cv.u;
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); // rounds to >= 65520 -> inf
    if (ax < 0x38800000u) {                                    // below 2^-14: subnormal half or zero
        if (ax < 0x33000000u) return (uint16_t)sign;           // < 2^-25 rounds to 0
        const uint32_t e = ax >> 23;
        const uint32_t m = (ax & 0x7fffffu) | 0x800000u;       // value = m * 2^(e-150)
        const uint32_t sh = 126u - e;                          // value / 2^-24 = m >> (126-e), 14 <= sh <= 24
        uint32_t v = m >> sh;
        const uint32_t rem = m & ((1u << sh) - 1u);
        const uint32_t halfway = 1u << (sh - 1u);
        if (rem > halfway || (rem == halfway && (v & 1u))) ++v;
        return (uint16_t)(sign | v);
    }
    uint32_t v = ((ax >> 13) - (112u << 10));
    const uint32_t rem = ax & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (v & 1u))) ++v;
    return (uint16_t)(sign | v);
}

}  // namespace rgm
