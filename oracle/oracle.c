/*
 * oracle.c -- CPU oracle for the ReSTIR direct-lighting hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker.  Only tests/, the smoke()
 * entry and bench.py's CPU-baseline leg load this library; the product path
 * never does.
 *
 * Single precision throughout (except the FP64 judge at the end), compiled
 * with -ffp-contract=off so every a*b+c is two rounded operations, exactly as
 * the CUDA kernels (built with -fmad=false) compute it.  GLSL built-ins are
 * given one fixed meaning shared with the CUDA path:
 *   min(x,y) = y<x ? y : x          max(x,y) = x<y ? y : x   (GLSL 4.50 8.3)
 *   clamp(x,a,b) = min(max(x,a),b)  mix(x,y,a) = x*(1-a) + y*a
 *   dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z
 *   normalize(v) = v / sqrt(dot(v,v)) (component-wise IEEE division)
 *   pow(r, 2.0) = r*r               round() = half away from zero
 *   sin/cos: Cody-Waite reduction by pi/2 + Taylor polynomials (or_sinf/or_cosf)
 *   M*v = ((m0*x + m1*y) + m2*z) + m3*w   (column-major)
 * Reference paths below are relative to the reference project root.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_F 3.14159274101257324f          /* (float)M_PI, disneyBRDF.glsl:1 as a GLSL float literal */
#define DEG2RAD_F 0.0174532923847436905f    /* (float)(pi/180): GLSL radians() */
#define PI_D 3.14159265358979323846
#define STACK_SIZE 64                        /* reference: 32 (softwareRaytracing.glsl:40), UB on overflow */

/* ------------------------------------------------------------------ vec3 */
typedef struct { float x, y, z; } v3;
static inline v3 V(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmuls(float s, v3 a) { return V(s * a.x, s * a.y, s * a.z); }
static inline v3 vmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vdivs(v3 a, float s) { return V(a.x / s, a.y / s, a.z / s); }
static inline v3 vdiv(v3 a, v3 b) { return V(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
    return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline v3 vnormalize(v3 a) { return vdivs(a, sqrtf(vdot(a, a))); }
static inline float gmin(float x, float y) { return y < x ? y : x; }
static inline float gmax(float x, float y) { return x < y ? y : x; }
static inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
static inline float gmix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
static inline v3 f4xyz(or_f4 f) { return V(f.x, f.y, f.z); }
static inline int imin(int a, int b) { return b < a ? b : a; }
static inline int imax(int a, int b) { return a < b ? b : a; }
static inline int iclamp(int x, int lo, int hi) { return imin(imax(x, lo), hi); }

/* ------------------------------------------------------------------ PCG32 (rand.glsl:7-32) */
typedef struct { uint64_t state, inc; } pcg_t;
static inline uint32_t pcg_next(pcg_t *r) {
    uint64_t old = r->state;
    r->state = old * 6364136223846793005ULL + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
static inline pcg_t pcg_seed(uint64_t seed, uint64_t seq) {
    pcg_t r;
    r.state = 0;
    r.inc = (seq << 1u) | 1u;
    pcg_next(&r);
    r.state += seed;
    pcg_next(&r);
    return r;
}
/* rand.glsl:30-32: uint -> float (round to nearest) / 2^32; may return exactly 1.0 */
static inline float rand_float(pcg_t *r) { return (float)pcg_next(r) / 4294967296.0f; }

void or_pcg_stream(uint64_t seed, uint64_t seq, int32_t n, uint32_t *out) {
    pcg_t r = pcg_seed(seed, seq);
    for (int32_t i = 0; i < n; ++i) out[i] = pcg_next(&r);
}
void or_rand_floats(uint64_t seed, uint64_t seq, int32_t n, float *out) {
    pcg_t r = pcg_seed(seed, seq);
    for (int32_t i = 0; i < n; ++i) out[i] = rand_float(&r);
}

/* ------------------------------------------------------------------ sin / cos
 * Cody-Waite reduction x = k*pi/2 + y with pi/2 = C1 + C2 + C3 (C1 8 bits,
 * C2 12 bits, so k*C1 and k*C2 are exact for |k| < 2^12), then Taylor
 * polynomials of sin (to y^9) and cos (to y^10) on |y| <= pi/4, Horner form.
 * Same constants and operation order as the CUDA kernels. */
#define CW_2_OVER_PI 0.636619746685028076f
#define CW_C1 1.5703125f
#define CW_C2 4.83870506286621094e-4f
#define CW_C3 -4.37113882867379300e-8f
#define TS3 0.166666671633720398f
#define TS5 8.33333376795053482e-3f
#define TS7 1.98412701138295233e-4f
#define TS9 2.75573188446287531e-6f
#define TC4 4.16666679084300995e-2f
#define TC6 1.38888892251998186e-3f
#define TC8 2.48015876422869042e-5f
#define TC10 2.75573199814971304e-7f

static inline void or_sincos(float x, float *s, float *c) {
    float k = rintf(x * CW_2_OVER_PI);
    float y = ((x - k * CW_C1) - k * CW_C2) - k * CW_C3;
    float y2 = y * y;
    float ps = ((TS9 * y2 - TS7) * y2 + TS5) * y2 - TS3;
    float sy = y + (y * y2) * ps;
    float pc = ((TC8 - TC10 * y2) * y2 - TC6) * y2 + TC4;
    float cy = (1.0f - 0.5f * y2) + (y2 * y2) * pc;
    int q = ((int)k) & 3;
    switch (q) {
    case 0: *s = sy; *c = cy; break;
    case 1: *s = cy; *c = -sy; break;
    case 2: *s = -sy; *c = -cy; break;
    default: *s = -cy; *c = sy; break;
    }
}
static inline float or_cosf(float x) { float s, c; or_sincos(x, &s, &c); return c; }

void or_sincos_batch(int32_t n, const float *x, float *s, float *c) {
    for (int32_t i = 0; i < n; ++i) or_sincos(x[i], &s[i], &c[i]);
}

/* ------------------------------------------------------------------ G-buffer decoding
 * albedo is R8G8B8A8_SRGB (gBufferPass.cpp:75-79): sampling decodes the sRGB
 * transfer function; the table is evaluated in double and rounded once. */
static float g_srgb[256];
static int g_srgb_ready = 0;
static void srgb_init(void) {
    if (g_srgb_ready) return;
    for (int i = 0; i < 256; ++i) {
        double c = (double)i / 255.0;
        double l = c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
        g_srgb[i] = (float)l;
    }
    g_srgb_ready = 1;
}
void or_srgb_lut(float *out256) { srgb_init(); memcpy(out256, g_srgb, sizeof(g_srgb)); }

float or_half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1fu;
    uint32_t man = h & 0x3ffu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {           /* subnormal half -> normal float */
            int e = -1;
            do { ++e; man <<= 1; } while (!(man & 0x400u));
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3ffu) << 13);
        }
    } else if (exp == 31) {
        bits = sign | 0x7f800000u | (man << 13);
    } else {
        bits = sign | ((exp + 112u) << 23) | (man << 13);
    }
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

typedef struct {
    v3 albedo; float albedo_a;
    v3 normal;
    float roughness, metallic;
    v3 wpos;
    float depth;
} texel_t;

/* G-buffer attachment formats: the VkFormat numbers of the reference's
 * candidates (src/passes/gBufferPass.cpp:81-101); 0 is the default layout. */
#define OR_R16G16B16_SNORM 85
#define OR_R16G16B16_SFLOAT 90
#define OR_R16G16B16A16_SNORM 92
#define OR_R16G16B16A16_SFLOAT 97
#define OR_R32G32B32_SFLOAT 106
#define OR_R32G32B32A32_SFLOAT 109
#define OR_D32_SFLOAT 126
#define OR_D24_UNORM_S8_UINT 129
#define OR_D32_SFLOAT_S8_UINT 130

/* Vulkan's conversion from normalized fixed point: max(c / (2^15 - 1), -1) */
static inline float snorm16(uint16_t c) {
    const float v = (float)(int16_t)c / 32767.0f;
    return v < -1.0f ? -1.0f : v;
}
static v3 g_normal(const or_gbuffer *g, size_t i) {
    switch (g->normal_format) {
        case OR_R16G16B16A16_SNORM: {
            const uint16_t *n = g->normal + 4 * i;
            return V(snorm16(n[0]), snorm16(n[1]), snorm16(n[2]));
        }
        case OR_R16G16B16_SNORM: {
            const uint16_t *n = g->normal + 3 * i;
            return V(snorm16(n[0]), snorm16(n[1]), snorm16(n[2]));
        }
        case OR_R16G16B16_SFLOAT: {
            const uint16_t *n = g->normal + 3 * i;
            return V(or_half_to_float(n[0]), or_half_to_float(n[1]), or_half_to_float(n[2]));
        }
        case OR_R32G32B32_SFLOAT: {
            const float *n = (const float *)(const void *)g->normal + 3 * i;
            return V(n[0], n[1], n[2]);
        }
        default: {   /* R16G16B16A16_SFLOAT */
            const uint16_t *n = g->normal + 4 * i;
            return V(or_half_to_float(n[0]), or_half_to_float(n[1]), or_half_to_float(n[2]));
        }
    }
}
static inline v3 g_wpos(const or_gbuffer *g, size_t i) {
    const float *p = g->world_pos + (g->world_pos_format == OR_R32G32B32_SFLOAT ? 3 : 4) * i;
    return V(p[0], p[1], p[2]);
}
/* D32F (also the depth plane of D32_SFLOAT_S8_UINT), or D24_UNORM_S8_UINT:
 * the low 24 bits of each 32-bit word over 2^24 - 1 */
static inline float g_depth(const or_gbuffer *g, size_t i) {
    if (g->depth_format == OR_D24_UNORM_S8_UINT) {
        uint32_t w;
        memcpy(&w, g->depth + i, 4);
        return (float)(w & 0xffffffu) / 16777215.0f;
    }
    return g->depth[i];
}

static inline void fetch_texel(const or_gbuffer *g, int x, int y, texel_t *t) {
    size_t i = (size_t)y * (size_t)g->width + (size_t)x;
    const uint8_t *a = g->albedo + 4 * i;
    t->albedo = V(g_srgb[a[0]], g_srgb[a[1]], g_srgb[a[2]]);
    t->albedo_a = (float)a[3] / 255.0f;
    t->normal = g_normal(g, i);
    const uint16_t *m = g->material + 2 * i;
    t->roughness = (float)m[0] / 65535.0f;
    t->metallic = (float)m[1] / 65535.0f;
    t->wpos = g_wpos(g, i);
    t->depth = g_depth(g, i);
}

/* ------------------------------------------------------------------ BRDF (disneyBRDF.glsl:5-90) */
static inline float luminance(float r, float g, float b) { /* common.glsl:7-9 */
    return 0.2126f * r + 0.7152f * g + 0.0722f * b;
}
static inline float schlick_fresnel(float c) { /* :5-10 */
    float m = gclamp(1.0f - c, 0.0f, 1.0f);
    float sm = m * m;
    return sm * sm * m;
}
static inline float gtr2(float ndoth, float a) { /* :13-18 */
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * ndoth * ndoth;
    return a2 / (PI_F * t * t);
}
static inline float smith_g_ggx(float ndotv, float alpha_g) { /* :20-25 */
    float a = alpha_g * alpha_g;
    float b = ndotv * ndotv;
    return 1.0f / (fabsf(ndotv) + gmax(sqrtf(a + b - a * b), 0.0001f));
}
static inline float diffuse_factor(float cos_in, float cos_out, float cos_in_half, float roughness, float metallic) { /* :27-33 */
    float f_in = schlick_fresnel(cos_in);
    float f_out = schlick_fresnel(cos_out);
    float fd90 = 0.5f + 2.0f * cos_in_half * cos_in_half * roughness;
    float fd = gmix(1.0f, fd90, f_in) * gmix(1.0f, fd90, f_out);
    return fd * (1.0f - metallic) / PI_F;
}
static inline void specular_factors(float cos_in, float cos_out, float cos_half, float cos_in_half,
                                    float roughness, float *fresnel, float *gd) { /* :42-55 */
    *fresnel = schlick_fresnel(cos_in_half);
    float a = gmax(0.001f, roughness * roughness);
    float ds = gtr2(cos_half, a);
    float gs = smith_g_ggx(cos_in, a);
    gs *= smith_g_ggx(cos_out, a);
    *gd = gs * ds;
}
static inline float brdf_lum(float cos_in, float cos_out, float cos_half, float cos_in_half,
                             float lum, float roughness, float metallic) { /* :82-90 */
    if (cos_in < 0.0f) return 0.0f;
    float diffuse = lum * diffuse_factor(cos_in, cos_out, cos_in_half, roughness, metallic);
    float fr, gd;
    specular_factors(cos_in, cos_out, cos_half, cos_in_half, roughness, &fr, &gd);
    float spec_lum = gmix(0.04f, lum, metallic);
    float fs = gmix(spec_lum, 1.0f, fr);
    return diffuse + fs * gd;
}
static inline v3 brdf_color(float cos_in, float cos_out, float cos_half, float cos_in_half,
                            v3 albedo, float roughness, float metallic) { /* :73-81 */
    if (cos_in < 0.0f) return V(0.0f, 0.0f, 0.0f);
    float df = diffuse_factor(cos_in, cos_out, cos_in_half, roughness, metallic);
    v3 diffuse = V(albedo.x * df, albedo.y * df, albedo.z * df);
    float fr, gd;
    specular_factors(cos_in, cos_out, cos_half, cos_in_half, roughness, &fr, &gd);
    v3 sc = V(gmix(0.04f, albedo.x, metallic), gmix(0.04f, albedo.y, metallic), gmix(0.04f, albedo.z, metallic));
    v3 fs = V(gmix(sc.x, 1.0f, fr), gmix(sc.y, 1.0f, fr), gmix(sc.z, 1.0f, fr));
    return vadd(diffuse, V(fs.x * gd, fs.y * gd, fs.z * gd));
}

/* ------------------------------------------------------------------ p-hat (restirUtils.glsl:3-55) */
static float eval_phat(v3 wpos, v3 lpos, v3 cam, v3 n, v3 ln, int use_ln,
                       float albedo_lum, float emission_lum, float roughness, float metallic) {
    v3 wi = vsub(lpos, wpos);
    if (vdot(wi, n) < 0.0f) return 0.0f;
    float sqr_dist = vdot(wi, wi);
    wi = vdivs(wi, sqrtf(sqr_dist));
    v3 wo = vnormalize(vsub(cam, wpos));
    float cos_in = vdot(n, wi);
    float cos_out = vdot(n, wo);
    v3 h = vnormalize(vadd(wi, wo));
    float cos_half = vdot(n, h);
    float cos_in_half = vdot(wi, h);
    float geometry = cos_in / sqr_dist;
    if (use_ln) geometry *= fabsf(vdot(wi, ln));
    return emission_lum * brdf_lum(cos_in, cos_out, cos_half, cos_in_half, albedo_lum, roughness, metallic) * geometry;
}
static v3 eval_phat_full(v3 wpos, v3 lpos, v3 cam, v3 n, v3 ln, int use_ln,
                         v3 albedo, v3 emission, float roughness, float metallic) {
    v3 wi = vsub(lpos, wpos);
    if (vdot(wi, n) < 0.0f) return V(0.0f, 0.0f, 0.0f);
    float sqr_dist = vdot(wi, wi);
    wi = vdivs(wi, sqrtf(sqr_dist));
    v3 wo = vnormalize(vsub(cam, wpos));
    float cos_in = vdot(n, wi);
    float cos_out = vdot(n, wo);
    v3 h = vnormalize(vadd(wi, wo));
    float cos_half = vdot(n, h);
    float cos_in_half = vdot(wi, h);
    float geometry = cos_in / sqr_dist;
    if (use_ln) geometry *= fabsf(vdot(wi, ln));
    v3 f = brdf_color(cos_in, cos_out, cos_half, cos_in_half, albedo, roughness, metallic);
    v3 e = vmul(emission, f);
    return V(e.x * geometry, e.y * geometry, e.z * geometry);
}

void or_eval_phat_batch(int32_t n, const float *a, float *out) {
    for (int32_t i = 0; i < n; ++i, a += 20)
        out[i] = eval_phat(V(a[0], a[1], a[2]), V(a[3], a[4], a[5]), V(a[6], a[7], a[8]), V(a[9], a[10], a[11]),
                           V(a[12], a[13], a[14]), a[15] > 0.5f, a[16], a[17], a[18], a[19]);
}
void or_eval_phat_full_batch(int32_t n, const float *a, float *out) {
    for (int32_t i = 0; i < n; ++i, a += 24) {
        v3 r = eval_phat_full(V(a[0], a[1], a[2]), V(a[3], a[4], a[5]), V(a[6], a[7], a[8]), V(a[9], a[10], a[11]),
                              V(a[12], a[13], a[14]), a[15] > 0.5f, V(a[16], a[17], a[18]), V(a[19], a[20], a[21]),
                              a[22], a[23]);
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
}

/* ------------------------------------------------------------------ traversal (softwareRaytracing.glsl) */
static inline float max3(v3 v) { return gmax(v.x, gmax(v.y, v.z)); }
static inline float min3(v3 v) { return gmin(v.x, gmin(v.y, v.z)); }
static inline int ray_aabb(v3 o, v3 d, v3 bmin, v3 bmax) { /* :9-14 */
    v3 t0 = vdiv(vsub(bmin, o), d);
    v3 t1 = vdiv(vsub(bmax, o), d);
    float rmin = max3(V(gmin(t0.x, t1.x), gmin(t0.y, t1.y), gmin(t0.z, t1.z)));
    float rmax = min3(V(gmax(t0.x, t1.x), gmax(t0.y, t1.y), gmax(t0.z, t1.z)));
    return rmin < 1.0f && rmax >= rmin && rmax > 0.0f;
}
static inline int ray_tri(v3 p1, v3 p2, v3 p3, v3 o, v3 d) { /* :15-37 */
    v3 e1 = vsub(p2, p1);
    v3 e2 = vsub(p3, p1);
    v3 p = vcross(d, e2);
    float f = 1.0f / vdot(e1, p);
    v3 s = vsub(o, p1);
    float bx = f * vdot(s, p);
    if (bx < 0.0f || bx > 1.0f) return 0;
    v3 q = vcross(s, e1);
    float by = f * vdot(d, q);
    if (by < 0.0f || by + bx > 1.0f) return 0;
    f *= vdot(e2, q);
    return f > 0.0f && f < 1.0f;
}

typedef struct { uint64_t node_visits, box_tests, tri_tests, overflows; } trav_count;

/* :42-85, same stack discipline and 8-pop batched leaf tests; returns 1 when
 * the segment origin..origin+dir is unoccluded.  The stack is stack_size deep
 * (the reference's 32 entries overflow on deep trees); an overflow is counted. */
static int raytrace(const or_scene *sc, v3 o, v3 d, int stack_size, trav_count *tc) {
    int stack[256], top = 1;
    int cand[16], ncand = 0, counter = 0;
    if (stack_size > 256) stack_size = 256;
    stack[0] = 0;
    if (sc->n_nodes <= 0) return 1;
    while (top > 0) {
        const or_node *nd = &sc->nodes[stack[--top]];
        tc->node_visits++;
        tc->box_tests += 2;
        int li = ray_aabb(o, d, f4xyz(nd->lmin), f4xyz(nd->lmax));
        int ri = ray_aabb(o, d, f4xyz(nd->rmin), f4xyz(nd->rmax));
        if (li) {
            if (nd->left < 0) cand[ncand++] = ~nd->left;
            else if (top < stack_size) stack[top++] = nd->left;
            else tc->overflows++;
        }
        if (ri) {
            if (nd->right < 0) cand[ncand++] = ~nd->right;
            else if (top < stack_size) stack[top++] = nd->right;
            else tc->overflows++;
        }
        if (++counter == 8) {
            for (int i = 0; i < ncand; ++i) {
                const or_tri *t = &sc->tris[cand[i]];
                tc->tri_tests++;
                if (ray_tri(f4xyz(t->p1), f4xyz(t->p2), f4xyz(t->p3), o, d)) return 0;
            }
            ncand = 0;
            counter = 0;
        }
    }
    for (int i = 0; i < ncand; ++i) {
        const or_tri *t = &sc->tris[cand[i]];
        tc->tri_tests++;
        if (ray_tri(f4xyz(t->p1), f4xyz(t->p2), f4xyz(t->p3), o, d)) return 0;
    }
    return 1;
}

/* visibilityTest.glsl:1-4,26-29: returns 1 when p1 -> p2 is shadowed */
static int test_visibility(const or_scene *sc, v3 p1, v3 p2, trav_count *tc) {
    const float tmin = 0.001f;
    v3 dir = vsub(p2, p1);
    v3 off = vmuls(tmin, vnormalize(dir));
    return !raytrace(sc, vadd(p1, off), vsub(dir, vmuls(2.0f, off)), STACK_SIZE, tc);
}

static void stats_add(or_stats *st, const trav_count *tc, uint64_t rays) {
    if (!st) return;
#pragma omp atomic
    st->rays += rays;
#pragma omp atomic
    st->node_visits += tc->node_visits;
#pragma omp atomic
    st->box_tests += tc->box_tests;
#pragma omp atomic
    st->tri_tests += tc->tri_tests;
#pragma omp atomic
    st->stack_overflows += tc->overflows;
}

void or_ray_aabb_batch(int32_t n, const float *a, uint8_t *out) {
    for (int32_t i = 0; i < n; ++i, a += 12)
        out[i] = (uint8_t)ray_aabb(V(a[0], a[1], a[2]), V(a[3], a[4], a[5]), V(a[6], a[7], a[8]), V(a[9], a[10], a[11]));
}
void or_ray_tri_batch(int32_t n, const float *a, uint8_t *out) {
    for (int32_t i = 0; i < n; ++i, a += 15)
        out[i] = (uint8_t)ray_tri(V(a[6], a[7], a[8]), V(a[9], a[10], a[11]), V(a[12], a[13], a[14]),
                                  V(a[0], a[1], a[2]), V(a[3], a[4], a[5]));
}
void or_raytrace_batch(const or_scene *sc, int32_t n, const float *rays, uint8_t *out, int32_t stack_size, or_stats *st) {
    trav_count tot = {0, 0, 0, 0};
#pragma omp parallel
    {
        trav_count tc = {0, 0, 0, 0};
#pragma omp for schedule(dynamic, 256)
        for (int32_t i = 0; i < n; ++i) {
            const float *r = rays + 6 * (size_t)i;
            out[i] = (uint8_t)raytrace(sc, V(r[0], r[1], r[2]), V(r[3], r[4], r[5]), stack_size, &tc);
        }
#pragma omp critical
        {
            tot.node_visits += tc.node_visits; tot.box_tests += tc.box_tests;
            tot.tri_tests += tc.tri_tests; tot.overflows += tc.overflows;
        }
    }
    stats_add(st, &tot, (uint64_t)n);
}
void or_test_visibility_batch(const or_scene *sc, int32_t n, const float *p1, const float *p2, uint8_t *out, or_stats *st) {
    trav_count tot = {0, 0, 0, 0};
#pragma omp parallel
    {
        trav_count tc = {0, 0, 0, 0};
#pragma omp for schedule(dynamic, 256)
        for (int32_t i = 0; i < n; ++i) {
            const float *a = p1 + 3 * (size_t)i, *b = p2 + 3 * (size_t)i;
            out[i] = (uint8_t)test_visibility(sc, V(a[0], a[1], a[2]), V(b[0], b[1], b[2]), &tc);
        }
#pragma omp critical
        {
            tot.node_visits += tc.node_visits; tot.box_tests += tc.box_tests;
            tot.tri_tests += tc.tri_tests; tot.overflows += tc.overflows;
        }
    }
    stats_add(st, &tot, (uint64_t)n);
}

/* ------------------------------------------------------------------ alias table */
/* restirOmni.glsl:73-83 */
static inline void alias_sample(const or_alias *tab, int32_t count, float r1, float r2, int *idx, float *prob) {
    int col = imin((int)((float)count * r1), count - 1);
    const or_alias *c = &tab[col];
    if (c->prob > r2) { *idx = col; *prob = c->ori_prob; }
    else { *idx = c->alias; *prob = c->alias_ori_prob; }
}
void or_alias_sample_batch(const or_alias *tab, int32_t count, int32_t n, const float *r, int32_t *idx, float *prob) {
    for (int32_t i = 0; i < n; ++i) { int k; float p; alias_sample(tab, count, r[2 * i], r[2 * i + 1], &k, &p); idx[i] = k; prob[i] = p; }
}

/* misc.cpp:418-497: Vose's method with FIFO work lists, float arithmetic. */
void or_build_alias_table(const or_point_light *pl, int32_t n_pl, const or_tri_light *tl, int32_t n_tl, or_alias *out) {
    int32_t n = n_pl > 0 ? n_pl : n_tl;
    if (n <= 0) return;
    float *p = (float *)malloc(sizeof(float) * (size_t)n);
    int32_t *big = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * 2);
    int32_t *small = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * 2);
    size_t bh = 0, bt = 0, sh = 0, st = 0; /* FIFO heads / tails; each index is pushed at most n times in total */
    float sum = 0.0f;
    for (int32_t i = 0; i < n; ++i) {
        float v = n_pl > 0 ? pl[i].color_lum.w : tl[i].emission_lum.w * tl[i].normal_area.w;
        sum += v;
        p[i] = v;
    }
    for (int32_t i = 0; i < n; ++i) {
        out[i].prob = 0.0f;
        out[i].alias = -1;
        out[i].ori_prob = p[i] / sum;
        p[i] = (float)n * p[i] / sum;
        if (p[i] >= 1.0f) big[bt++] = i; else small[st++] = i;
    }
    while (bh < bt && sh < st) {
        int32_t g = big[bh++], l = small[sh++];
        out[l].prob = p[l];
        out[l].alias = g;
        p[g] = (p[g] + p[l]) - 1.0f;
        if (p[g] < 1.0f) small[st++] = g; else big[bt++] = g;
    }
    while (bh < bt) { int32_t g = big[bh++]; out[g].prob = 1.0f; out[g].alias = g; }
    while (sh < st) { int32_t l = small[sh++]; out[l].prob = 1.0f; out[l].alias = l; }
    for (int32_t i = 0; i < n; ++i) out[i].alias_ori_prob = out[out[i].alias].ori_prob;
    free(p); free(big); free(small);
}

/* ------------------------------------------------------------------ reservoirs (reservoir.glsl:6-76) */
static inline void update_reservoir_at(or_reservoir *r, int i, float weight, v3 pos, or_f4 nrm, float lum,
                                       int32_t idx, float p_hat, float w, float sum_phat, pcg_t *rng) { /* :6-26 */
    or_sample *s = &r->s[i];
    s->sum_weights += weight;
    float replace = weight / s->sum_weights;
    if (rand_float(rng) < replace) {
        s->pos_lum.x = pos.x; s->pos_lum.y = pos.y; s->pos_lum.z = pos.z; s->pos_lum.w = lum;
        s->normal = nrm;
        s->light_index = idx;
        s->p_hat = p_hat;
        s->w = w;
#if OR_MIS
        s->sum_phat += sum_phat;
#else
        (void)sum_phat;
#endif
    }
}
static inline void add_sample(or_reservoir *r, v3 pos, or_f4 nrm, float lum, int32_t idx, float p_hat,
                              float sample_p, pcg_t *rng) { /* :28-42 */
    float weight = p_hat / sample_p;
    r->m += 1;
    for (int i = 0; i < OR_RS; ++i) {
        float w = (r->s[i].sum_weights + weight) / ((float)r->m * p_hat);
        update_reservoir_at(r, i, weight, pos, nrm, lum, idx, p_hat, w, p_hat, rng);
    }
}
/* :44-64.  With UNBIASED_MIS the reference passes other's sumPHat where
 * updateReservoirAt takes w and other's w where it takes sumPHat (:55-60);
 * that is kept unless swap_fix. */
static inline void combine_reservoirs(or_reservoir *self, const or_reservoir *other, const float *p_hat,
                                      int swap_fix, pcg_t *rng) {
    self->m += other->m;
    for (int i = 0; i < OR_RS; ++i) {
        const or_sample *o = &other->s[i];
        float weight = p_hat[i] * o->w * (float)other->m;
        if (weight > 0.0f) {
#if OR_MIS
            const float wv = swap_fix ? o->w : o->sum_phat;
            const float sp = swap_fix ? o->sum_phat : o->w;
#else
            const float wv = o->w, sp = 0.0f;
            (void)swap_fix;
#endif
            update_reservoir_at(self, i, weight, f4xyz(o->pos_lum), o->normal, o->pos_lum.w, o->light_index, p_hat[i],
                                wv, sp, rng);
        }
        if (self->s[i].w > 0.0f) self->s[i].w = self->s[i].sum_weights / ((float)self->m * self->s[i].p_hat);
    }
}
/* :66-76; the fields the reference leaves uninitialised are defined as zero */
static inline void new_reservoir(or_reservoir *r) { memset(r, 0, sizeof(*r)); }

void or_reservoir_layout(int32_t *rs, int32_t *mis, int32_t *bytes) {
    if (rs) *rs = OR_RS;
    if (mis) *mis = OR_MIS;
    if (bytes) *bytes = (int32_t)sizeof(or_reservoir);
}

void or_reservoir_script(const float *cand, int32_t n, const or_reservoir *other, const float *other_phat,
                         uint64_t seed, uint64_t seq, int32_t swap_fix, or_reservoir *out) {
    pcg_t rng = pcg_seed(seed, seq);
    or_reservoir r;
    new_reservoir(&r);
    for (int32_t k = 0; k < n; ++k) {
        const float *c = cand + 12 * (size_t)k;
        or_f4 nrm;
        nrm.x = c[3]; nrm.y = c[4]; nrm.z = c[5]; nrm.w = c[6];
        int32_t idx;
        memcpy(&idx, &c[8], 4);
        add_sample(&r, V(c[0], c[1], c[2]), nrm, c[7], idx, c[9], c[10], &rng);
    }
    if (other) combine_reservoirs(&r, other, other_phat, swap_fix, &rng);
    *out = r;
}

static int crop_ok(const int32_t *crop, int W, int H, int *x0, int *y0, int *cw, int *ch) {
    if (!crop) { *x0 = 0; *y0 = 0; *cw = W; *ch = H; return 1; }
    *x0 = crop[0]; *y0 = crop[1]; *cw = crop[2]; *ch = crop[3];
    return *x0 >= 0 && *y0 >= 0 && *cw >= 0 && *ch >= 0 && *x0 + *cw <= W && *y0 + *ch <= H;
}

/* ------------------------------------------------------------------ RIS + visibility + temporal (restirOmni.glsl:86-212) */
int or_initial_temporal(const or_scene *sc, const or_gbuffer *cur, const or_gbuffer *prev,
                        const or_reservoir *prev_res, or_reservoir *out, const or_uniforms *u,
                        const int32_t *crop, or_stats *st) {
    return or_initial_temporal_learned(sc, cur, prev, prev_res, out, u, NULL, crop, st);
}

/* With l != NULL (point lights only), candidate i of pixel p is l->cand[p*32+i]
 * of the learned proposal: key < 0 names a cluster whose light is drawn from
 * the cluster's alias table with r1, r2; key >= 0 is a light; the source pdf
 * is mix * q * p(light | cluster) + uniform_pdf.  Everything else is the
 * reference's pass. */
int or_initial_temporal_learned(const or_scene *sc, const or_gbuffer *cur, const or_gbuffer *prev,
                                const or_reservoir *prev_res, or_reservoir *out, const or_uniforms *u,
                                const or_learned *l, const int32_t *crop, or_stats *st) {
    srgb_init();
    if (l && sc->n_point_lights == 0) return -3;
    int W = (int)u->size[0], H = (int)u->size[1];
    int x0, y0, cw, ch;
    if (W != cur->width || H != cur->height) return -1;
    if (!crop_ok(crop, W, H, &x0, &y0, &cw, &ch)) return -2;
    const int use_point = sc->n_point_lights != 0;
    const v3 cam = f4xyz(u->camera_pos);
    trav_count tot = {0, 0, 0, 0};
    uint64_t rays = 0;
#pragma omp parallel
    {
        trav_count tc = {0, 0, 0, 0};
        uint64_t my_rays = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t pi = 0; pi < (int64_t)cw * ch; ++pi) {
            int x = x0 + (int)(pi % cw), y = y0 + (int)(pi / cw);
            texel_t t;
            fetch_texel(cur, x, y, &t);
            float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
            or_reservoir res;
            new_reservoir(&res);
            pcg_t rng = pcg_seed((uint64_t)u->frame, (uint64_t)((uint32_t)y * 10007u + (uint32_t)x));
            int zero_normal = !(vdot(t.normal, t.normal) != 0.0f);
            if (!zero_normal) {
                for (int i = 0; (uint32_t)i < u->initial_light_sample_count; ++i) {
                    int sel; float prob;
                    float r1 = rand_float(&rng), r2 = rand_float(&rng);
                    if (l) {
                        const or_candidate cd = l->cand[((size_t)y * (size_t)W + (size_t)x) * 32 + (size_t)i];
                        float pl;
                        if (cd.key < 0) {
                            const int32_t cl = -1 - cd.key;
                            const int32_t b = l->offset[cl], m = l->offset[cl + 1] - b;
                            const int32_t pos = b + imin((int)((float)m * r1), m - 1);
                            const or_alias *c = &l->col[pos];
                            if (c->prob > r2) { sel = l->order[pos]; pl = c->ori_prob; }
                            else { sel = l->order[c->alias]; pl = c->alias_ori_prob; }
                        } else {
                            sel = cd.key;
                            pl = l->within[sel];
                        }
                        prob = l->mix * cd.q * pl + l->uniform_pdf;
                    } else {
                        alias_sample(sc->alias, sc->n_alias, r1, r2, &sel, &prob);
                    }
                    v3 lpos; or_f4 ln; float llum; int32_t lidx;
                    if (use_point) {
                        const or_point_light *L = &sc->point_lights[sel];
                        lpos = f4xyz(L->pos);
                        llum = L->color_lum.w;
                        lidx = sel;
                        ln.x = ln.y = ln.z = ln.w = 0.0f;
                    } else {
                        const or_tri_light *L = &sc->tri_lights[sel];
                        float a = rand_float(&rng), b = rand_float(&rng);
                        /* pickPointOnTriangle, restirOmni.glsl:68-71 */
                        float sa = sqrtf(a);
                        v3 q1 = vmuls(1.0f - sa, f4xyz(L->p1));
                        v3 q2 = vmuls(sa * (1.0f - b), f4xyz(L->p2));
                        v3 q3 = vmuls(b * sa, f4xyz(L->p3));
                        lpos = vadd(vadd(q1, q2), q3);
                        llum = L->emission_lum.w;
                        lidx = -1 - sel;
                        v3 wi = vnormalize(vsub(t.wpos, lpos));
                        v3 nn = f4xyz(L->normal_area);
                        prob /= fabsf(vdot(wi, nn)) * L->normal_area.w;
                        ln.x = nn.x; ln.y = nn.y; ln.z = nn.z; ln.w = 1.0f;
                    }
                    float ph = eval_phat(t.wpos, lpos, cam, t.normal, f4xyz(ln), ln.w > 0.5f, albedo_lum, llum,
                                         t.roughness, t.metallic);
                    add_sample(&res, lpos, ln, llum, lidx, ph, prob, &rng);
                }
                if (u->flags & OR_FLAG_FINAL_RIS_WEIGHT)
                    for (int i = 0; i < OR_RS; ++i)
                        if (res.s[i].sum_weights > 0.0f)
                            res.s[i].w = res.s[i].sum_weights / ((float)res.m * res.s[i].p_hat);
            }
            /* visibility reuse :147-160 -- a background pixel's (zero normal) sample is
             * undefined in the reference; here it is the zero sample, for which zeroing
             * w and sumWeights changes nothing, so no ray is traced for it. */
            if ((u->flags & OR_FLAG_VISIBILITY) && !zero_normal) {
                for (int i = 0; i < OR_RS; ++i) {
                    ++my_rays;
                    if (test_visibility(sc, t.wpos, f4xyz(res.s[i].pos_lum), &tc)) {
                        res.s[i].w = 0.0f;
                        res.s[i].sum_weights = 0.0f;
#if OR_MIS
                        res.s[i].sum_phat = 0.0f;
#endif
                    }
                }
            }
            /* temporal reuse :162-209 */
            if ((u->flags & OR_FLAG_TEMPORAL) && prev != NULL && prev_res != NULL) {
                const float *m = u->prev_pv;
                float px = ((m[0] * t.wpos.x + m[4] * t.wpos.y) + m[8] * t.wpos.z) + m[12] * 1.0f;
                float py = ((m[1] * t.wpos.x + m[5] * t.wpos.y) + m[9] * t.wpos.z) + m[13] * 1.0f;
                float pw = ((m[3] * t.wpos.x + m[7] * t.wpos.y) + m[11] * t.wpos.z) + m[15] * 1.0f;
                px /= pw;
                py /= pw;
                px = (px + 1.0f) * 0.5f * (float)u->size[0];
                py = (py + 1.0f) * 0.5f * (float)u->size[1];
                if (px > 0.0f && py > 0.0f && px < (float)u->size[0] && py < (float)u->size[1]) {
                    int fx = (int)px, fy = (int)py;
                    texel_t pt;
                    fetch_texel(prev, fx, fy, &pt);
                    v3 dp = vsub(t.wpos, pt.wpos);
                    if (vdot(dp, dp) < 0.01f) {
                        v3 da = vsub(t.albedo, pt.albedo);
                        if (vdot(da, da) < 0.01f) {
                            if (vdot(t.normal, pt.normal) > 0.5f) {
                                or_reservoir pr = prev_res[(size_t)fy * u->size[0] + (size_t)fx];
                                uint32_t cap = u->temporal_mult * res.m;
                                pr.m = pr.m < cap ? pr.m : cap;
                                float ph[OR_RS];
                                for (int i = 0; i < OR_RS; ++i)
                                    ph[i] = eval_phat(t.wpos, f4xyz(pr.s[i].pos_lum), cam, t.normal,
                                                      f4xyz(pr.s[i].normal), pr.s[i].normal.w > 0.5f, albedo_lum,
                                                      pr.s[i].pos_lum.w, t.roughness, t.metallic);
                                combine_reservoirs(&res, &pr, ph, (u->flags & OR_FLAG_MIS_SWAP_FIX) != 0, &rng);
                            }
                        }
                    }
                }
            }
            out[(size_t)y * (size_t)W + (size_t)x] = res;
        }
#pragma omp critical
        {
            tot.node_visits += tc.node_visits; tot.box_tests += tc.box_tests;
            tot.tri_tests += tc.tri_tests; tot.overflows += tc.overflows;
            rays += my_rays;
        }
    }
    stats_add(st, &tot, rays);
    return 0;
}

/* ------------------------------------------------------------------ biased spatial (spatialReuse.comp:30-86) */
int or_spatial_biased(const or_scene *sc, const or_gbuffer *g, const or_reservoir *in, or_reservoir *out,
                      const or_uniforms *u, int32_t iter, const int32_t *crop) {
    (void)sc;
    srgb_init();
    int W = (int)u->size[0], H = (int)u->size[1];
    int x0, y0, cw, ch;
    if (W != g->width || H != g->height) return -1;
    if (!crop_ok(crop, W, H, &x0, &y0, &cw, &ch)) return -2;
    const v3 cam = f4xyz(u->camera_pos);
    const float cos_thr = or_cosf(u->normal_threshold * DEG2RAD_F);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t pi = 0; pi < (int64_t)cw * ch; ++pi) {
        int x = x0 + (int)(pi % cw), y = y0 + (int)(pi / cw);
        texel_t t;
        fetch_texel(g, x, y, &t);
        float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
        size_t ri = (size_t)y * (size_t)W + (size_t)x;
        or_reservoir res = in[ri];
        pcg_t rng = pcg_seed((uint64_t)(u->frame * 31u + (uint32_t)iter), (uint64_t)((uint32_t)y * 10007u + (uint32_t)x));
        for (uint32_t i = 0; i < u->spatial_neighbors; ++i) {
            float angle = rand_float(&rng) * 2.0f * PI_F;
            float radius = sqrtf(rand_float(&rng)) * u->spatial_radius;
            float s, c;
            or_sincos(angle, &s, &c);
            int ox = (int)floorf(c * radius), oy = (int)floorf(s * radius);
            int nx = iclamp(x + ox, 0, W - 1), ny = iclamp(y + oy, 0, H - 1);
            size_t ni = (size_t)ny * (size_t)W + (size_t)nx;
            float nd = g_depth(g, ni);
            v3 nnor = g_normal(g, ni);
            if (fabsf(nd - t.depth) > u->pos_threshold * fabsf(t.depth) || vdot(nnor, t.normal) < cos_thr) continue;
            const or_reservoir *rr = &in[ni];
            float ph[OR_RS];
            for (int j = 0; j < OR_RS; ++j)
                ph[j] = eval_phat(t.wpos, f4xyz(rr->s[j].pos_lum), cam, t.normal, f4xyz(rr->s[j].normal),
                                  rr->s[j].normal.w > 0.5f, albedo_lum, rr->s[j].pos_lum.w, t.roughness, t.metallic);
            combine_reservoirs(&res, rr, ph, (u->flags & OR_FLAG_MIS_SWAP_FIX) != 0, &rng);
        }
        out[ri] = res;
    }
    return 0;
}

/* ------------------------------------------------------------------ unbiased spatial (unbiasedReuse.glsl:50-185)
 * num_neighbors is NUM_NEIGHBORS (the reference hard-codes 3, :48).  The
 * reference seeds with frame*17 (:72); pass_index p seeds with frame*17 + p
 * so chained passes draw fresh neighbours (p = 0 is the reference). */
int or_spatial_unbiased(const or_scene *sc, const or_gbuffer *g, const or_reservoir *in, or_reservoir *out,
                        const or_uniforms *u, int32_t num_neighbors, int32_t pass_index, const int32_t *crop, or_stats *st) {
    srgb_init();
    int W = (int)u->size[0], H = (int)u->size[1];
    int x0, y0, cw, ch;
    if (W != g->width || H != g->height) return -1;
    if (!crop_ok(crop, W, H, &x0, &y0, &cw, &ch)) return -2;
    if (num_neighbors < 0 || num_neighbors > 64) return -3;
    const v3 cam = f4xyz(u->camera_pos);
    const int vis = (u->flags & OR_FLAG_VISIBILITY) != 0;
    trav_count tot = {0, 0, 0, 0};
    uint64_t rays = 0, unobs = 0;
#pragma omp parallel
    {
        trav_count tc = {0, 0, 0, 0};
        uint64_t my_rays = 0, my_unobs = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t pi = 0; pi < (int64_t)cw * ch; ++pi) {
            int x = x0 + (int)(pi % cw), y = y0 + (int)(pi / cw);
            texel_t t;
            fetch_texel(g, x, y, &t);
            float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
            size_t ri = (size_t)y * (size_t)W + (size_t)x;
            or_reservoir res = in[ri];
            pcg_t rng = pcg_seed((uint64_t)(u->frame * 17u + (uint32_t)pass_index), (uint64_t)((uint32_t)y * 10007u + (uint32_t)x));
            int npx[64], npy[64];
            uint32_t nm[64];
#if OR_MIS
            float nsp[OR_RS][64], orig_sp[OR_RS];
            for (int i = 0; i < OR_RS; ++i) orig_sp[i] = res.s[i].sum_phat;
#endif
            for (int i = 0; i < num_neighbors; ++i) {
                float angle = rand_float(&rng) * 2.0f * PI_F;
                float radius = sqrtf(rand_float(&rng)) * u->spatial_radius;
                float s, c;
                or_sincos(angle, &s, &c);
                int ox = (int)roundf(c * radius), oy = (int)roundf(s * radius);
                int nx = iclamp(x + ox, 0, (int)(u->size[0] - 1u)), ny = iclamp(y + oy, 0, (int)(u->size[1] - 1u));
                const or_reservoir *rr = &in[(size_t)ny * (size_t)W + (size_t)nx];
                npx[i] = nx; npy[i] = ny;
                nm[i] = rr->m;
#if OR_MIS
                for (int j = 0; j < OR_RS; ++j) nsp[j][i] = rr->s[j].sum_phat;
#endif
                res.m += rr->m;
                for (int j = 0; j < OR_RS; ++j) {
                    const or_sample *o = &rr->s[j];
                    float ph = eval_phat(t.wpos, f4xyz(o->pos_lum), cam, t.normal, f4xyz(o->normal),
                                         o->normal.w > 0.5f, albedo_lum, o->pos_lum.w, t.roughness, t.metallic);
                    float weight = ph * o->w * (float)rr->m;
#if OR_MIS
                    const float sp = o->sum_phat;
#else
                    const float sp = 0.0f;
#endif
                    if (weight > 0.0f)
                        update_reservoir_at(&res, j, weight, f4xyz(o->pos_lum), o->normal, o->pos_lum.w,
                                            o->light_index, ph, o->w, sp, &rng);
                }
            }
            texel_t nt[64];
            for (int j = 0; j < num_neighbors; ++j) fetch_texel(g, npx[j], npy[j], &nt[j]);
            for (int i = 0; i < OR_RS; ++i) {
                v3 lpos = f4xyz(res.s[i].pos_lum);
#if OR_MIS
                float sum_phat = orig_sp[i];
#else
                uint32_t ns = in[ri].m;  /* the reservoir's own count before the merges */
#endif
                uint64_t neighbour_rays = 0;
                for (int j = 0; j < num_neighbors; ++j) {
                    if (vdot(vsub(lpos, nt[j].wpos), nt[j].normal) < 0.0f) continue;
                    if (vis) {
                        ++my_rays;
                        ++neighbour_rays;
                        if (test_visibility(sc, nt[j].wpos, lpos, &tc)) continue;
                    }
#if OR_MIS
                    sum_phat += nsp[i][j];
#else
                    ns += nm[j];
#endif
                }
                if (vis) {
                    ++my_rays;
                    if (test_visibility(sc, t.wpos, lpos, &tc)) {
                        my_unobs += neighbour_rays;
#if OR_MIS
                        sum_phat = 0.0f;
#else
                        ns = 0;
#endif
                    }
                }
#if OR_MIS
                if (sum_phat > 0.0f) {
                    res.s[i].w = res.s[i].sum_weights * res.s[i].p_hat / (sum_phat * res.s[i].p_hat);
                } else {
                    res.s[i].w = 0.0f;
                    res.s[i].sum_weights = 0.0f;
                    res.s[i].sum_phat = 0.0f;
                }
#else
                if (ns > 0) {
                    res.s[i].w = res.s[i].sum_weights / ((float)ns * res.s[i].p_hat);
                } else {
                    res.s[i].w = 0.0f;
                    res.s[i].sum_weights = 0.0f;
                }
#endif
            }
            (void)nm;
            out[ri] = res;
        }
#pragma omp critical
        {
            tot.node_visits += tc.node_visits; tot.box_tests += tc.box_tests;
            tot.tri_tests += tc.tri_tests; tot.overflows += tc.overflows;
            rays += my_rays;
            unobs += my_unobs;
        }
    }
    stats_add(st, &tot, rays);
    if (st) st->rays_unobservable += unobs;
    return 0;
}

/* ------------------------------------------------------------------ shading (lighting.frag:43-71,103) */
int or_shade(const or_scene *sc, const or_gbuffer *g, const or_reservoir *resv, const or_lighting_uniforms *u,
             float *rgba, const int32_t *crop) {
    srgb_init();
    int W = (int)u->size[0], H = (int)u->size[1];
    int x0, y0, cw, ch;
    if (W != g->width || H != g->height) return -1;
    if (!crop_ok(crop, W, H, &x0, &y0, &cw, &ch)) return -2;
    const v3 cam = f4xyz(u->camera_pos);
    const float inv_gamma = 1.0f / u->gamma;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t pi = 0; pi < (int64_t)cw * ch; ++pi) {
        int x = x0 + (int)(pi % cw), y = y0 + (int)(pi / cw);
        texel_t t;
        fetch_texel(g, x, y, &t);
        size_t ri = (size_t)y * (size_t)W + (size_t)x;
        const or_reservoir *r = &resv[ri];
        v3 col = V(0.0f, 0.0f, 0.0f);
        for (int i = 0; i < OR_RS; ++i) {
            const or_sample *sm = &r->s[i];
            v3 emission;
            if (sm->light_index < 0) {
                int k = -1 - sm->light_index;
                emission = (k < sc->n_tri_lights) ? f4xyz(sc->tri_lights[k].emission_lum) : V(0.0f, 0.0f, 0.0f);
            } else {
                int k = sm->light_index;
                emission = (k < sc->n_point_lights) ? f4xyz(sc->point_lights[k].color_lum) : V(0.0f, 0.0f, 0.0f);
            }
            v3 ph = eval_phat_full(t.wpos, f4xyz(sm->pos_lum), cam, t.normal, f4xyz(sm->normal), sm->normal.w > 0.5f,
                                   t.albedo, emission, t.roughness, t.metallic);
            col = V(col.x + ph.x * sm->w, col.y + ph.y * sm->w, col.z + ph.z * sm->w);
        }
        col = vdivs(col, (float)OR_RS); /* RESERVOIR_SIZE */
        if (t.albedo_a > 0.5f) col = t.albedo;
        if (u->gamma != 1.0f) col = V(powf(col.x, inv_gamma), powf(col.y, inv_gamma), powf(col.z, inv_gamma));
        rgba[4 * ri] = col.x; rgba[4 * ri + 1] = col.y; rgba[4 * ri + 2] = col.z; rgba[4 * ri + 3] = 1.0f;
    }
    return 0;
}

/* ------------------------------------------------------------------ FP64 brute-force judge
 * L(x) = sum over every light of emission * BRDF * cos / d^2 * V, with the
 * reference's BRDF and the reference's shadow segment, both in double, on
 * the same BVH.  Emissive pixels return their albedo (lighting.frag:69-71). */
typedef struct { double x, y, z; } d3;
static inline d3 D(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline d3 dsub(d3 a, d3 b) { return D(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 dadd(d3 a, d3 b) { return D(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 dmuls(double s, d3 a) { return D(s * a.x, s * a.y, s * a.z); }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 dcross(d3 a, d3 b) { return D(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
static inline d3 dnorm(d3 a) { double l = sqrt(ddot(a, a)); return D(a.x / l, a.y / l, a.z / l); }
static inline d3 df4(or_f4 f) { return D(f.x, f.y, f.z); }
static inline double dmin(double a, double b) { return b < a ? b : a; }
static inline double dmax(double a, double b) { return a < b ? b : a; }

static int d_ray_aabb(d3 o, d3 d, or_f4 bmin, or_f4 bmax) {
    double t0x = (bmin.x - o.x) / d.x, t1x = (bmax.x - o.x) / d.x;
    double t0y = (bmin.y - o.y) / d.y, t1y = (bmax.y - o.y) / d.y;
    double t0z = (bmin.z - o.z) / d.z, t1z = (bmax.z - o.z) / d.z;
    double rmin = dmax(dmin(t0x, t1x), dmax(dmin(t0y, t1y), dmin(t0z, t1z)));
    double rmax = dmin(dmax(t0x, t1x), dmin(dmax(t0y, t1y), dmax(t0z, t1z)));
    return rmin < 1.0 && rmax >= rmin && rmax > 0.0;
}
static int d_ray_tri(const or_tri *t, d3 o, d3 d) {
    d3 p1 = df4(t->p1);
    d3 e1 = dsub(df4(t->p2), p1), e2 = dsub(df4(t->p3), p1);
    d3 p = dcross(d, e2);
    double f = 1.0 / ddot(e1, p);
    d3 s = dsub(o, p1);
    double bx = f * ddot(s, p);
    if (bx < 0.0 || bx > 1.0) return 0;
    d3 q = dcross(s, e1);
    double by = f * ddot(d, q);
    if (by < 0.0 || by + bx > 1.0) return 0;
    f *= ddot(e2, q);
    return f > 0.0 && f < 1.0;
}
static int d_shadowed(const or_scene *sc, d3 p1, d3 p2) {
    d3 dir = dsub(p2, p1);
    d3 off = dmuls(0.001, dnorm(dir));
    d3 o = dadd(p1, off), d = dsub(dir, dmuls(2.0, off));
    int stack[256], top = 1;
    stack[0] = 0;
    if (sc->n_nodes <= 0) return 0;
    while (top > 0) {
        const or_node *nd = &sc->nodes[stack[--top]];
        if (d_ray_aabb(o, d, nd->lmin, nd->lmax)) {
            if (nd->left < 0) { if (d_ray_tri(&sc->tris[~nd->left], o, d)) return 1; }
            else if (top < 256) stack[top++] = nd->left;
        }
        if (d_ray_aabb(o, d, nd->rmin, nd->rmax)) {
            if (nd->right < 0) { if (d_ray_tri(&sc->tris[~nd->right], o, d)) return 1; }
            else if (top < 256) stack[top++] = nd->right;
        }
    }
    return 0;
}
static double d_schlick(double c) { double m = dmin(dmax(1.0 - c, 0.0), 1.0); double sm = m * m; return sm * sm * m; }
static double d_smith(double ndotv, double ag) { double a = ag * ag, b = ndotv * ndotv; return 1.0 / (fabs(ndotv) + dmax(sqrt(a + b - a * b), 0.0001)); }

int or_brute_force_fp64(const or_scene *sc, const or_gbuffer *g, const float *cam3, double *rgb_out, const int32_t *crop) {
    srgb_init();
    int W = g->width, H = g->height;
    int x0, y0, cw, ch;
    if (!crop_ok(crop, W, H, &x0, &y0, &cw, &ch)) return -2;
    const d3 cam = D(cam3[0], cam3[1], cam3[2]);
    const int use_point = sc->n_point_lights != 0;
    const int nl = use_point ? sc->n_point_lights : sc->n_tri_lights;
    if (!use_point && nl > 0) return -4; /* triangle lights need an area integral; not part of the judge */
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t pi = 0; pi < (int64_t)cw * ch; ++pi) {
        int x = x0 + (int)(pi % cw), y = y0 + (int)(pi / cw);
        texel_t t;
        fetch_texel(g, x, y, &t);
        double acc[3] = {0.0, 0.0, 0.0};
        size_t oi = (size_t)(pi) * 3;
        if (t.albedo_a > 0.5f) {
            rgb_out[oi] = t.albedo.x; rgb_out[oi + 1] = t.albedo.y; rgb_out[oi + 2] = t.albedo.z;
            continue;
        }
        d3 n = D(t.normal.x, t.normal.y, t.normal.z);
        d3 wp = D(t.wpos.x, t.wpos.y, t.wpos.z);
        if (ddot(n, n) == 0.0) { rgb_out[oi] = rgb_out[oi + 1] = rgb_out[oi + 2] = 0.0; continue; }
        double rough = t.roughness, metal = t.metallic;
        double alb[3] = {t.albedo.x, t.albedo.y, t.albedo.z};
        d3 wo = dnorm(dsub(cam, wp));
        double cos_out = ddot(n, wo);
        for (int l = 0; l < nl; ++l) {
            const or_point_light *L = &sc->point_lights[l];
            d3 lp = df4(L->pos);
            d3 wi = dsub(lp, wp);
            if (ddot(wi, n) < 0.0) continue;
            double sq = ddot(wi, wi);
            wi = dmuls(1.0 / sqrt(sq), wi);
            double cos_in = ddot(n, wi);
            if (cos_in < 0.0) continue;
            d3 h = dnorm(dadd(wi, wo));
            double cos_half = ddot(n, h), cos_in_half = ddot(wi, h);
            double fi = d_schlick(cos_in), fo = d_schlick(cos_out);
            double fd90 = 0.5 + 2.0 * cos_in_half * cos_in_half * rough;
            double fd = (1.0 * (1.0 - fi) + fd90 * fi) * (1.0 * (1.0 - fo) + fd90 * fo);
            double dfac = fd * (1.0 - metal) / PI_D;
            double fr = d_schlick(cos_in_half);
            double a = dmax(0.001, rough * rough);
            double a2 = a * a, tt = 1.0 + (a2 - 1.0) * cos_half * cos_half;
            double ds = a2 / (PI_D * tt * tt);
            double gd = d_smith(cos_in, a) * d_smith(cos_out, a) * ds;
            double geometry = cos_in / sq;
            if (geometry == 0.0) continue;
            if (d_shadowed(sc, wp, lp)) continue;
            double em[3] = {L->color_lum.x, L->color_lum.y, L->color_lum.z};
            for (int c = 0; c < 3; ++c) {
                double sc_ = 0.04 * (1.0 - metal) + alb[c] * metal;
                double fs = sc_ * (1.0 - fr) + 1.0 * fr;
                acc[c] += em[c] * (alb[c] * dfac + fs * gd) * geometry;
            }
        }
        rgb_out[oi] = acc[0]; rgb_out[oi + 1] = acc[1]; rgb_out[oi + 2] = acc[2];
    }
    return 0;
}

/* ------------------------------------------------------------------ tree builder
 * AabbTree::build (src/aabbTreeBuilder.cpp:52-214) restated in C, operation
 * for operation, so the node and triangle buffers come out byte-identical:
 *   - triangles pass through the node's world matrix (identity here), which
 *     turns a -0 coordinate into +0 and keeps every other value;
 *   - a leaf's box is the component-wise nvmath min/max of its vertices
 *     (nv_min(a, b) = a < b ? a : b, nv_max(a, b) = a > b ? a : b), its
 *     centroid 0.5f * (min + max);
 *   - ranges are split breadth first (a FIFO queue; nodes are numbered in pop
 *     order, the root is node 0): 1 triangle = a leaf link ~index, 2 = a node
 *     with both leaves; otherwise 12 buckets over the widest centroid axis
 *     (x > y ? x : y, then z if larger), bucket = (size_t)clamp((c - cmin) /
 *     (span / 12), 0.5, 11.5), the split minimising
 *     0.125 + (nL * SA(L) + nR * SA(R)) / SA(range) over the 11 split points
 *     (SA = sx*sy + sx*sz + sy*sz; the right-side bounds accumulated from
 *     the top bucket down), an in-place swap partition, and the median split
 *     with recomputed bounds when one side is empty. */
typedef struct { float c[3], mn[3], mx[3]; int32_t geom; size_t bucket; } bl_leaf;
typedef struct { float mn[3], mx[3]; size_t count; } bl_bucket;
typedef struct { int32_t *parent; size_t beg, end; } bl_step;

static inline float nvmn(float a, float b) { return a < b ? a : b; }
static inline float nvmx(float a, float b) { return a > b ? a : b; }
static float bl_sah(const float mn[3], const float mx[3]) {
    const float sx = mx[0] - mn[0], sy = mx[1] - mn[1], sz = mx[2] - mn[2];
    return (sx * sy + sx * sz) + sy * sz;
}
static void bl_bucket_init(bl_bucket *b) {
    for (int a = 0; a < 3; ++a) { b->mn[a] = 3.402823466e38f; b->mx[a] = -3.402823466e38f; }
    b->count = 0;
}
static bl_bucket bl_merge(bl_bucket l, const bl_bucket *r) {
    l.count += r->count;
    for (int a = 0; a < 3; ++a) { l.mn[a] = nvmn(l.mn[a], r->mn[a]); l.mx[a] = nvmx(l.mx[a], r->mx[a]); }
    return l;
}
static float bl_heur(const bl_bucket *b) { return (float)b->count * bl_sah(b->mn, b->mx); }
static void bl_set(or_f4 *dst, const float v[3]) { dst->x = v[0]; dst->y = v[1]; dst->z = v[2]; dst->w = 1.0f; }

int32_t or_build_bvh(const float *xyz, int32_t n, or_node *nodes, or_tri *tris) {
    enum { NB = 12 };
    if (n < 2) return -1;
    bl_leaf *leaves = (bl_leaf *)malloc(sizeof(bl_leaf) * (size_t)n);
    bl_step *q = (bl_step *)malloc(sizeof(bl_step) * (size_t)(2 * n));
    if (!leaves || !q) { free(leaves); free(q); return -2; }
    for (int32_t i = 0; i < n; ++i) {
        float p[3][3];
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) p[k][a] = xyz[(size_t)i * 9 + 3 * k + a] + 0.0f;  /* -0 -> +0 */
        or_tri *t = &tris[i];
        t->p1.x = p[0][0]; t->p1.y = p[0][1]; t->p1.z = p[0][2]; t->p1.w = 1.0f;
        t->p2.x = p[1][0]; t->p2.y = p[1][1]; t->p2.z = p[1][2]; t->p2.w = 1.0f;
        t->p3.x = p[2][0]; t->p3.y = p[2][1]; t->p3.z = p[2][2]; t->p3.w = 1.0f;
        bl_leaf *L = &leaves[i];
        for (int a = 0; a < 3; ++a) {
            L->mn[a] = L->mx[a] = p[0][a];
            L->mn[a] = nvmn(L->mn[a], p[1][a]);
            L->mx[a] = nvmx(L->mx[a], p[1][a]);
            L->mn[a] = nvmn(L->mn[a], p[2][a]);
            L->mx[a] = nvmx(L->mx[a], p[2][a]);
            L->c[a] = 0.5f * (L->mn[a] + L->mx[a]);
        }
        L->geom = i;
        L->bucket = 0;
    }
    memset(nodes, 0, sizeof(or_node) * (size_t)(n - 1));
    int32_t alloc = 0, dummy_root = -1, rc = n - 1;
    size_t qh = 0, qt = 0;
    q[qt].parent = &dummy_root; q[qt].beg = 0; q[qt].end = (size_t)n; ++qt;
    while (qh < qt) {
        const bl_step st = q[qh++];
        const size_t cnt = st.end - st.beg;
        if (cnt == 1) {
            *st.parent = ~leaves[st.beg].geom;
            continue;
        }
        if (cnt == 2) {
            const bl_leaf *l = &leaves[st.beg], *r = &leaves[st.beg + 1];
            const int32_t ni = alloc++;
            *st.parent = ni;
            or_node *nd = &nodes[ni];
            nd->left = ~l->geom;
            nd->right = ~r->geom;
            bl_set(&nd->lmin, l->mn); bl_set(&nd->lmax, l->mx);
            bl_set(&nd->rmin, r->mn); bl_set(&nd->rmax, r->mx);
            continue;
        }
        float cmin[3], cmax[3], bmin[3], bmax[3];
        for (int a = 0; a < 3; ++a) {
            cmin[a] = cmax[a] = leaves[st.beg].c[a];
            bmin[a] = leaves[st.beg].mn[a];
            bmax[a] = leaves[st.beg].mx[a];
        }
        for (size_t i = st.beg + 1; i < st.end; ++i)
            for (int a = 0; a < 3; ++a) {
                cmin[a] = nvmn(cmin[a], leaves[i].c[a]);
                cmax[a] = nvmx(cmax[a], leaves[i].c[a]);
                bmin[a] = nvmn(bmin[a], leaves[i].mn[a]);
                bmax[a] = nvmx(bmax[a], leaves[i].mx[a]);
            }
        const float outer = bl_sah(bmin, bmax);
        const float span[3] = {cmax[0] - cmin[0], cmax[1] - cmin[1], cmax[2] - cmin[2]};
        int dim = span[0] > span[1] ? 0 : 1;
        if (span[2] > span[dim]) dim = 2;
        if (!(span[dim] > 0.0f)) { rc = -3; break; }   /* (c - cmin) / 0: undefined in the reference */
        bl_bucket bk[NB];
        for (int b = 0; b < NB; ++b) bl_bucket_init(&bk[b]);
        const float range = span[dim] / (float)NB;
        for (size_t i = st.beg; i < st.end; ++i) {
            float u = (leaves[i].c[dim] - cmin[dim]) / range;
            u = u < 0.5f ? 0.5f : u;
            u = u > (float)NB - 0.5f ? (float)NB - 0.5f : u;
            leaves[i].bucket = (size_t)u;
            bl_bucket *b = &bk[leaves[i].bucket];
            for (int a = 0; a < 3; ++a) { b->mn[a] = nvmn(b->mn[a], leaves[i].mn[a]); b->mx[a] = nvmx(b->mx[a], leaves[i].mx[a]); }
            ++b->count;
        }
        bl_bucket cache[NB - 1];
        {
            bl_bucket cur = bk[NB - 1];
            for (size_t i = NB - 1; i > 0;) {
                cache[--i] = cur;
                cur = bl_merge(cur, &bk[i]);
            }
        }
        size_t opt = 0;
        int found = 0;
        float lmn[3] = {0, 0, 0}, lmx[3] = {0, 0, 0}, rmn[3] = {0, 0, 0}, rmx[3] = {0, 0, 0};
        {
            float best = 3.402823466e38f;
            bl_bucket left;
            bl_bucket_init(&left);
            for (size_t sp = 0; sp < NB - 1; ++sp) {
                left = bl_merge(left, &bk[sp]);
                const bl_bucket *right = &cache[sp];
                const float h = 0.125f + (bl_heur(&left) + bl_heur(right)) / outer;
                if (h < best) {
                    best = h;
                    opt = sp;
                    found = 1;
                    memcpy(lmn, left.mn, sizeof(lmn)); memcpy(lmx, left.mx, sizeof(lmx));
                    memcpy(rmn, right->mn, sizeof(rmn)); memcpy(rmx, right->mx, sizeof(rmx));
                }
            }
        }
        size_t pivot = st.beg;
        for (size_t i = st.beg; i < st.end; ++i)
            if (leaves[i].bucket <= opt) {
                const bl_leaf tmp = leaves[i];
                leaves[i] = leaves[pivot];
                leaves[pivot] = tmp;
                ++pivot;
            }
        if (pivot == st.beg || pivot == st.end) {
            pivot = (st.beg + st.end) / 2;
            for (int a = 0; a < 3; ++a) { lmn[a] = leaves[st.beg].mn[a]; lmx[a] = leaves[st.beg].mx[a]; }
            for (size_t i = st.beg + 1; i < pivot; ++i)
                for (int a = 0; a < 3; ++a) { lmn[a] = nvmn(lmn[a], leaves[i].mn[a]); lmx[a] = nvmx(lmx[a], leaves[i].mx[a]); }
            for (int a = 0; a < 3; ++a) { rmn[a] = leaves[pivot].mn[a]; rmx[a] = leaves[pivot].mx[a]; }
            for (size_t i = pivot; i < st.end; ++i)
                for (int a = 0; a < 3; ++a) { rmn[a] = nvmn(rmn[a], leaves[i].mn[a]); rmx[a] = nvmx(rmx[a], leaves[i].mx[a]); }
        } else if (!found) {
            rc = -3;   /* no finite heuristic: the reference's bounds stay uninitialised */
            break;
        }
        const int32_t ni = alloc++;
        *st.parent = ni;
        or_node *nd = &nodes[ni];
        bl_set(&nd->lmin, lmn); bl_set(&nd->lmax, lmx);
        bl_set(&nd->rmin, rmn); bl_set(&nd->rmax, rmx);
        q[qt].parent = &nd->left; q[qt].beg = st.beg; q[qt].end = pivot; ++qt;
        q[qt].parent = &nd->right; q[qt].beg = pivot; q[qt].end = st.end; ++qt;
    }
    free(leaves);
    free(q);
    return rc;
}

/* ------------------------------------------------------------------ primary-ray G-buffer
 * The reference rasterises its G-buffer (src/passes/gBufferPass.cpp:75-108,
 * src/shaders/gBuffer.vert, src/shaders/gBuffer.frag:27-79); headless, the
 * same planes come from one closest-hit ray per pixel centre:
 *   - the camera of src/camera.h:25-50: view rows (right, -up, forward), clip
 *     x = f/aspect * view x, clip y = f * view y, clip w = view z, so the
 *     pixel centre (px + 0.5, py + 0.5) at NDC (nx, ny) looks along
 *     right * (nx * aspect * tan(fov/2)) - up * (ny * tan(fov/2)) + forward
 *     (NDC y grows downwards in Vulkan, the view's y axis is -up);
 *   - the visible surface is the triangle with the smallest ray parameter t > 0
 *     of the Moller-Trumbore test of softwareRaytracing.glsl:15-37 (float, same
 *     operation order; 0 <= b1, 0 <= b2, b1 + b2 <= 1, NaN = miss, no upper
 *     bound on t), ties to the smaller triangle index -- the depth test's
 *     nearest fragment;
 *   - outputs as gBuffer.frag writes them for a flat, untextured triangle:
 *     albedo RGBA8 sRGB with alpha 255 for emissive surfaces (:73-79), normal
 *     = the face normal normalize(cross(p2 - p1, p3 - p1)) turned towards the
 *     viewer (gBuffer.frag:40-43 writes the interpolated vertex normal as it
 *     is; the generated scenes carry no vertex normals, so the face normal of
 *     the side the camera sees stands for it) as RGBA16F (w = 0), material
 *     RG16 unorm (roughness, metallic), world position o + t*d as RGBA32F
 *     (w = 1), depth = clip z / clip w of P*V times that position (the
 *     rasteriser's depth);
 *   - a ray that hits nothing leaves zero planes and depth 1 (the clear
 *     values).
 * The walk over the reference's tree is conservative: every box is grown by
 * 1e-5 (absolute) plus 1e-5 of its coordinates and tested in double, and a
 * box is skipped only when it starts beyond the best t found so far plus a
 * margin of the same size, so no triangle the float test hits in front of the
 * current best is missed; nearer children are walked first.
 * Triangles without a material take albedo (180, 180, 180), roughness 1. */
uint16_t or_float_to_half(float f) {
    /* IEEE 754 binary16, round to nearest even: the value scaled by the
     * spacing of halves at its exponent is rounded by nearbyint (exact in
     * double: a float has 24 significant bits). */
    uint32_t x;
    memcpy(&x, &f, 4);
    const uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
    const float a = fabsf(f);
    if (a != a) return (uint16_t)(sign | 0x7e00u);
    if (a >= 65520.0f) return (uint16_t)(sign | 0x7c00u);        /* rounds to infinity */
    if (a < 6.103515625e-05f) {                                  /* below 2^-14: spacing 2^-24 */
        const double m = nearbyint((double)a * 16777216.0);      /* m = 1024 is the smallest normal */
        return (uint16_t)(sign | (uint16_t)m);
    }
    int e;
    frexp((double)a, &e);                                        /* a in [2^(e-1), 2^e) */
    int E = e - 1;
    double m = nearbyint((double)a / ldexp(1.0, E - 10));        /* in [1024, 2048] */
    if (m >= 2048.0) { m = 1024.0; E += 1; }
    return (uint16_t)(sign | (uint16_t)(((E + 15) << 10) | ((int)m - 1024)));
}

/* ray parameter of the float Moller-Trumbore test, or -1 on a miss */
static float gb_tri_t(const or_tri *tr, v3 o, v3 d) {
    const v3 p1 = f4xyz(tr->p1);
    const v3 e1 = vsub(f4xyz(tr->p2), p1), e2 = vsub(f4xyz(tr->p3), p1);
    const v3 p = vcross(d, e2);
    const float f = 1.0f / vdot(e1, p);
    const v3 s = vsub(o, p1);
    const float bx = f * vdot(s, p);
    if (!(bx >= 0.0f && bx <= 1.0f)) return -1.0f;
    const v3 q = vcross(s, e1);
    const float by = f * vdot(d, q);
    if (!(by >= 0.0f && by + bx <= 1.0f)) return -1.0f;
    const float t = f * vdot(e2, q);
    return t > 0.0f ? t : -1.0f;
}

/* entry parameter of the grown box along o + t d in double, or +inf when the
 * line misses it or it lies behind the origin */
static double gb_box_entry(const double o[3], const double d[3], or_f4 bmin, or_f4 bmax) {
    const float lo3[3] = {bmin.x, bmin.y, bmin.z}, hi3[3] = {bmax.x, bmax.y, bmax.z};
    double lo = -INFINITY, hi = INFINITY;
    for (int a = 0; a < 3; ++a) {
        const double m = 1e-5 + 1e-5 * fmax(fabs((double)lo3[a]), fabs((double)hi3[a]));
        const double b0 = (double)lo3[a] - m, b1 = (double)hi3[a] + m;
        if (!(b0 <= b1)) return INFINITY;   /* NaN box */
        if (d[a] == 0.0) {
            if (o[a] < b0 || o[a] > b1) return INFINITY;
            continue;
        }
        double t0 = (b0 - o[a]) / d[a], t1 = (b1 - o[a]) / d[a];
        if (t0 > t1) { const double tt = t0; t0 = t1; t1 = tt; }
        if (t0 > lo) lo = t0;
        if (t1 < hi) hi = t1;
    }
    if (!(lo <= hi) || hi < 0.0) return INFINITY;
    return lo;
}

typedef struct { float t; int tri; } gb_hit;

static int gb_closest(const or_scene *sc, v3 o, v3 d, gb_hit *best) {
    best->t = INFINITY;
    best->tri = -1;
    if (sc->n_nodes <= 0) {
        for (int i = 0; i < sc->n_tris; ++i) {
            const float t = gb_tri_t(&sc->tris[i], o, d);
            if (t > 0.0f && (t < best->t || (t == best->t && i < best->tri))) { best->t = t; best->tri = i; }
        }
        return 0;
    }
    const double od[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    int stack[256], top = 0, node = 0;
    double stack_t[256];
    int64_t visits = 0;
    for (;;) {
        if (++visits > (int64_t)sc->n_nodes) return -5;
        const or_node *nd = &sc->nodes[node];
        const int child[2] = {nd->left, nd->right};
        const or_f4 mn[2] = {nd->lmin, nd->rmin}, mx[2] = {nd->lmax, nd->rmax};
        double te[2];
        for (int k = 0; k < 2; ++k) {
            te[k] = gb_box_entry(od, dd, mn[k], mx[k]);
            const double limit = best->tri < 0 ? INFINITY : (double)best->t + 1e-5 * (1.0 + (double)best->t);
            if (!(te[k] <= limit)) te[k] = INFINITY;
            if (te[k] != INFINITY && child[k] < 0) {   /* a leaf: its triangle now */
                const int i = ~child[k];
                const float t = gb_tri_t(&sc->tris[i], o, d);
                if (t > 0.0f && (t < best->t || (t == best->t && i < best->tri))) { best->t = t; best->tri = i; }
                te[k] = INFINITY;
            }
        }
        /* inner children: the nearer one is walked first (pushed last) */
        const int near = te[1] < te[0] ? 1 : 0;
        for (int j = 0; j < 2; ++j) {
            const int k = j == 0 ? 1 - near : near;
            if (te[k] == INFINITY) continue;
            if (top >= 256) return -5;
            stack[top] = child[k];
            stack_t[top++] = te[k];
        }
        node = -1;
        while (top > 0) {
            --top;
            const double limit = best->tri < 0 ? INFINITY : (double)best->t + 1e-5 * (1.0 + (double)best->t);
            if (stack_t[top] <= limit) { node = stack[top]; break; }
        }
        if (node < 0) return 0;
    }
}

int or_trace_gbuffer(const or_scene *sc, const or_material *mats, int32_t n_mats, const or_camera *c, int32_t W,
                     int32_t H, const int32_t *crop, uint8_t *albedo, uint16_t *normal, uint16_t *material,
                     float *world_pos, float *depth) {
    int x0, y0, cw, ch;
    if (!crop_ok(crop, W, H, &x0, &y0, &cw, &ch)) return -2;
    int err = 0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t pi = 0; pi < (int64_t)cw * ch; ++pi) {
        const int px = x0 + (int)(pi % cw), py = y0 + (int)(pi / cw);
        const float ndc_x = (((float)px + 0.5f) / (float)W) * 2.0f - 1.0f;
        const float ndc_y = (((float)py + 0.5f) / (float)H) * 2.0f - 1.0f;
        const float vx = ndc_x * c->aspect * c->tan_half_fov_y;
        const float vy = ndc_y * c->tan_half_fov_y;
        const v3 right = V(c->right[0], c->right[1], c->right[2]);
        const v3 up = V(c->up[0], c->up[1], c->up[2]);
        const v3 fwd = V(c->forward[0], c->forward[1], c->forward[2]);
        const v3 o = V(c->position[0], c->position[1], c->position[2]);
        const v3 d = vadd(vsub(vmuls(vx, right), vmuls(vy, up)), fwd);
        gb_hit hit;
        const int rc = gb_closest(sc, o, d, &hit);
        const size_t i = (size_t)py * (size_t)W + (size_t)px;
        if (rc != 0) {
#pragma omp atomic write
            err = rc;
        }
        if (rc != 0 || hit.tri < 0) {
            memset(albedo + 4 * i, 0, 4);
            memset(normal + 4 * i, 0, 8);
            memset(material + 2 * i, 0, 4);
            memset(world_pos + 4 * i, 0, 16);
            depth[i] = 1.0f;
            continue;
        }
        const or_tri *tr = &sc->tris[hit.tri];
        const v3 p1 = f4xyz(tr->p1);
        v3 n = vnormalize(vcross(vsub(f4xyz(tr->p2), p1), vsub(f4xyz(tr->p3), p1)));
        if (vdot(n, d) > 0.0f) n = V(-n.x, -n.y, -n.z);
        const v3 p = vadd(o, vmuls(hit.t, d));
        if (mats && hit.tri < n_mats) {
            memcpy(albedo + 4 * i, mats[hit.tri].albedo_srgb, 4);
            material[2 * i] = mats[hit.tri].roughness;
            material[2 * i + 1] = mats[hit.tri].metallic;
        } else {
            albedo[4 * i] = albedo[4 * i + 1] = albedo[4 * i + 2] = 180;
            albedo[4 * i + 3] = 0;
            material[2 * i] = 65535;
            material[2 * i + 1] = 0;
        }
        normal[4 * i] = or_float_to_half(n.x);
        normal[4 * i + 1] = or_float_to_half(n.y);
        normal[4 * i + 2] = or_float_to_half(n.z);
        normal[4 * i + 3] = 0;
        world_pos[4 * i] = p.x;
        world_pos[4 * i + 1] = p.y;
        world_pos[4 * i + 2] = p.z;
        world_pos[4 * i + 3] = 1.0f;
        const float *m = c->projection_view;
        const float cz = ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14] * 1.0f;
        const float cwv = ((m[3] * p.x + m[7] * p.y) + m[11] * p.z) + m[15] * 1.0f;
        depth[i] = cz / cwv;
    }
    return err;
}

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void or_set_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ learned light-cluster proposal
 * No reference counterpart: the CPU statement of the product's learned
 * proposal (network, sampling rule and training loss), used to check its
 * tensor-core kernels.  Layout of the packed parameters: W1 16x64, b1, W2
 * 64x64, b2, W3 64x64, b3, W4 64xC, b4 (matrices row-major, one row per
 * input).  Forward: h = bf16(relu(W^T h_prev + b)) per hidden layer with bf16
 * weights, z = W4^T h3 + b4, sums accumulated in double here (FP32 on the
 * tensor cores). */
#define MLP_IN 16
#define MLP_IN_USED 9
#define MLP_H 64
#define MLP_CAND 32
#define MLP_SEED_MUL 0x9E3779B97F4A7C15ULL
#define MLP_SEED_ADD 0x2545F4914F6CDD1DULL

/* round to nearest even on the upper 16 bits of the binary32 pattern */
float or_bf16_round(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) {
        if (u & 0x007fffffu) u |= 0x00400000u;  /* quiet NaN */
        u &= 0xffff0000u;
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);
        u &= 0xffff0000u;
    }
    float r;
    memcpy(&r, &u, 4);
    return r;
}

typedef struct { size_t w1, b1, w2, b2, w3, b3, w4, b4, total; } mlp_layout;
static mlp_layout mlp_layout_of(int32_t c) {
    mlp_layout L;
    size_t o = 0;
    L.w1 = o; o += (size_t)MLP_IN * MLP_H;
    L.b1 = o; o += MLP_H;
    L.w2 = o; o += (size_t)MLP_H * MLP_H;
    L.b2 = o; o += MLP_H;
    L.w3 = o; o += (size_t)MLP_H * MLP_H;
    L.b3 = o; o += MLP_H;
    L.w4 = o; o += (size_t)MLP_H * c;
    L.b4 = o; o += (size_t)c;
    L.total = o;
    return L;
}
int64_t or_mlp_param_count(int32_t clusters) { return (int64_t)mlp_layout_of(clusters).total; }

void or_mlp_features(const or_mlp *m, const or_gbuffer *g, const float cam[3], int32_t px, float x[16]) {
    const float *p = g->world_pos + 4 * (size_t)px;
    const uint16_t *nb = g->normal + 4 * (size_t)px;
    const v3 wpos = V(p[0], p[1], p[2]);
    const v3 n = V(or_half_to_float(nb[0]), or_half_to_float(nb[1]), or_half_to_float(nb[2]));
    const v3 v = vnormalize(vsub(V(cam[0], cam[1], cam[2]), wpos));
    float t[16] = {0};
    t[0] = (wpos.x - m->box_center[0]) * m->box_inv_half[0];
    t[1] = (wpos.y - m->box_center[1]) * m->box_inv_half[1];
    t[2] = (wpos.z - m->box_center[2]) * m->box_inv_half[2];
    t[3] = n.x; t[4] = n.y; t[5] = n.z;
    t[6] = v.x; t[7] = v.y; t[8] = v.z;
    for (int i = 0; i < MLP_IN; ++i) x[i] = (i < MLP_IN_USED && isfinite(t[i])) ? or_bf16_round(t[i]) : 0.0f;
}

/* weights as double: bf16-rounded (emulate) or exact */
static void mlp_weights(const or_mlp *m, const double *p64, int emulate, double *w) {
    const mlp_layout L = mlp_layout_of(m->clusters);
    for (size_t i = 0; i < L.total; ++i) {
        double v = p64 ? p64[i] : (double)m->params[i];
        const int is_weight = (i < L.b1) || (i >= L.w2 && i < L.b2) || (i >= L.w3 && i < L.b3) ||
                              (i >= L.w4 && i < L.b4);
        if (emulate && is_weight) v = (double)or_bf16_round((float)v);
        w[i] = v;
    }
}

/* forward of one row; h* as double (bf16 values when emulating); z with -inf for empty clusters */
static void mlp_forward_row(const or_mlp *m, const double *w, int emulate, const float *x, double *h1, double *h2,
                            double *h3, double *z) {
    const mlp_layout L = mlp_layout_of(m->clusters);
    const double *layer_w[3] = {w + L.w1, w + L.w2, w + L.w3};
    const double *layer_b[3] = {w + L.b1, w + L.b2, w + L.b3};
    double xin[MLP_H];
    double *outs[3] = {h1, h2, h3};
    for (int i = 0; i < MLP_IN; ++i) xin[i] = x[i];
    int nin = MLP_IN;
    const double *in = xin;
    for (int l = 0; l < 3; ++l) {
        for (int j = 0; j < MLP_H; ++j) {
            double acc = 0.0;
            for (int k = 0; k < nin; ++k) acc += in[k] * layer_w[l][(size_t)k * MLP_H + j];
            double v = acc + layer_b[l][j];
            v = v > 0.0 ? v : 0.0;
            outs[l][j] = emulate ? (double)or_bf16_round((float)v) : v;
        }
        in = outs[l];
        nin = MLP_H;
    }
    for (int c = 0; c < m->clusters; ++c) {
        if (!m->cluster_valid[c]) { z[c] = -INFINITY; continue; }
        double acc = 0.0;
        for (int k = 0; k < MLP_H; ++k) acc += h3[k] * w[L.w4 + (size_t)k * m->clusters + c];
        z[c] = acc + w[L.b4 + c];
    }
}

static double mlp_lse(const double *z, int32_t c, int32_t *amax) {
    double mx = -INFINITY;
    int32_t a = 0;
    for (int32_t i = 0; i < c; ++i)
        if (z[i] > mx) { mx = z[i]; a = i; }
    double s = 0.0;
    for (int32_t i = 0; i < c; ++i) s += exp(z[i] - mx);
    if (amax) *amax = a;
    return mx + log(s);
}

void or_mlp_row_stats(const or_mlp *m, const or_gbuffer *g, const float cam[3], int32_t n, const int32_t *rows,
                      double *lse, int32_t *amax, double *z_out) {
    const mlp_layout L = mlp_layout_of(m->clusters);
    double *w = (double *)malloc(L.total * sizeof(double));
    mlp_weights(m, NULL, 1, w);
#pragma omp parallel
    {
        double *z = (double *)malloc((size_t)m->clusters * sizeof(double));
        double h1[MLP_H], h2[MLP_H], h3[MLP_H];
        float x[MLP_IN];
#pragma omp for schedule(dynamic, 16)
        for (int32_t r = 0; r < n; ++r) {
            or_mlp_features(m, g, cam, rows ? rows[r] : r, x);
            mlp_forward_row(m, w, 1, x, h1, h2, h3, z);
            lse[r] = mlp_lse(z, m->clusters, amax ? amax + r : NULL);
            if (z_out) memcpy(z_out + (size_t)r * m->clusters, z, (size_t)m->clusters * sizeof(double));
        }
        free(z);
    }
    free(w);
}

/* The proposal's candidates of pixel rows[r] (keys/q: [n x n_cand]), drawn
 * from the pixel's PCG stream (seed frame*MUL+ADD, sequence pixel):
 *   per slot j two draws u0, u1: u0 < mix makes j a learned slot, otherwise
 *   the slot holds light min(floor(N*u1), N-1) with q of its cluster;
 *   then the n learned slots' uniforms as ascending order statistics,
 *   u_k = 1 - (1 - u_{k-1}) * V^(1/(n-k)) with one draw V each, the k-th going
 *   to the k-th learned slot and placed on the double-precision softmax CDF
 *   (a uniform at or beyond the total takes the most probable cluster). */
void or_mlp_sample(const or_mlp *m, const or_gbuffer *g, const float cam[3], uint32_t frame, int32_t n_cand,
                   int32_t n, const int32_t *rows, int32_t *keys, float *qs) {
    const mlp_layout L = mlp_layout_of(m->clusters);
    double *w = (double *)malloc(L.total * sizeof(double));
    mlp_weights(m, NULL, 1, w);
#pragma omp parallel
    {
        double *z = (double *)malloc((size_t)m->clusters * sizeof(double));
        double h1[MLP_H], h2[MLP_H], h3[MLP_H];
        float x[MLP_IN];
#pragma omp for schedule(dynamic, 16)
        for (int32_t r = 0; r < n; ++r) {
            const int32_t px = rows ? rows[r] : r;
            or_mlp_features(m, g, cam, px, x);
            mlp_forward_row(m, w, 1, x, h1, h2, h3, z);
            int32_t amax = 0;
            const double lse = mlp_lse(z, m->clusters, &amax);
            pcg_t rng = pcg_seed((uint64_t)frame * MLP_SEED_MUL + MLP_SEED_ADD, (uint64_t)px);
            int32_t learned[MLP_CAND];
            int32_t n_u = 0;
            for (int32_t j = 0; j < n_cand; ++j) {
                const float u0 = rand_float(&rng);
                const float u1 = rand_float(&rng);
                if (u0 < m->mix) {
                    learned[n_u++] = j;
                } else {
                    const int32_t l = imin((int)((float)m->n_lights * u1), m->n_lights - 1);
                    keys[(size_t)r * n_cand + j] = l;
                    qs[(size_t)r * n_cand + j] = (float)exp(z[m->cluster_of[l]] - lse);
                }
            }
            float u = 0.0f;
            int32_t c = 0;
            double cum = exp(z[0] - lse);
            for (int32_t k = 0; k < n_u; ++k) {
                const float v = rand_float(&rng);
                u = 1.0f - (1.0f - u) * powf(v, 1.0f / (float)(n_u - k));
                while (c < m->clusters && !((double)u < cum)) {
                    ++c;
                    if (c < m->clusters) cum += exp(z[c] - lse);
                }
                const int32_t col = c < m->clusters ? c : amax;
                keys[(size_t)r * n_cand + learned[k]] = -1 - col;
                qs[(size_t)r * n_cand + learned[k]] = (float)exp(z[col] - lse);
            }
        }
        free(z);
    }
    free(w);
}

/* Summed cross-entropy over the rows with a target (target -1: no loss) and
 * its gradient divided by n, i.e. the gradient of the mean over all n rows.
 * emulate = 1 rounds to bf16 where the product does (weights, activations,
 * the logit gradient and the hidden pre-activation gradients entering the
 * weight products); emulate = 0 is plain double arithmetic (params64, when
 * given, replaces the FP32 parameters). */
double or_mlp_loss_grad(const or_mlp *m, const double *params64, const or_gbuffer *g, const float cam[3], int32_t n,
                        const int32_t *rows, const int32_t *target, int32_t emulate, double *grad) {
    const mlp_layout L = mlp_layout_of(m->clusters);
    const int32_t C = m->clusters;
    double *w = (double *)malloc(L.total * sizeof(double));
    mlp_weights(m, params64, emulate, w);
    memset(grad, 0, L.total * sizeof(double));
    double loss = 0.0;
    const double inv_n = 1.0 / (double)n;
    double *z = (double *)malloc((size_t)C * sizeof(double));
    double *dz = (double *)malloc((size_t)C * sizeof(double));
    for (int32_t r = 0; r < n; ++r) {
        const int32_t t = target[r];
        if (t < 0) continue;
        float x[MLP_IN];
        double h1[MLP_H], h2[MLP_H], h3[MLP_H];
        or_mlp_features(m, g, cam, rows[r], x);
        mlp_forward_row(m, w, emulate, x, h1, h2, h3, z);
        const double lse = mlp_lse(z, C, NULL);
        loss += lse - z[t];
        for (int32_t c = 0; c < C; ++c) {
            double d = (exp(z[c] - lse) - (c == t ? 1.0 : 0.0)) * inv_n;
            if (emulate) d = (double)or_bf16_round((float)d);
            dz[c] = d;
        }
        double dh3[MLP_H], da3[MLP_H], da2[MLP_H], da1[MLP_H];
        for (int k = 0; k < MLP_H; ++k) {
            double acc = 0.0;
            const double *wr = w + L.w4 + (size_t)k * C;
            double *gr = grad + L.w4 + (size_t)k * C;
            for (int32_t c = 0; c < C; ++c) {
                acc += dz[c] * wr[c];
                gr[c] += h3[k] * dz[c];
            }
            dh3[k] = acc;
        }
        for (int32_t c = 0; c < C; ++c) grad[L.b4 + c] += dz[c];
        for (int k = 0; k < MLP_H; ++k) da3[k] = h3[k] > 0.0 ? dh3[k] : 0.0;
        for (int i = 0; i < MLP_H; ++i) {
            double acc = 0.0;
            for (int k = 0; k < MLP_H; ++k) acc += w[L.w3 + (size_t)i * MLP_H + k] * da3[k];
            da2[i] = h2[i] > 0.0 ? acc : 0.0;
        }
        for (int i = 0; i < MLP_H; ++i) {
            double acc = 0.0;
            for (int k = 0; k < MLP_H; ++k) acc += w[L.w2 + (size_t)i * MLP_H + k] * da2[k];
            da1[i] = h1[i] > 0.0 ? acc : 0.0;
        }
        for (int j = 0; j < MLP_H; ++j) {
            const double r3 = emulate ? (double)or_bf16_round((float)da3[j]) : da3[j];
            const double r2 = emulate ? (double)or_bf16_round((float)da2[j]) : da2[j];
            const double r1 = emulate ? (double)or_bf16_round((float)da1[j]) : da1[j];
            for (int i = 0; i < MLP_H; ++i) {
                grad[L.w3 + (size_t)i * MLP_H + j] += h2[i] * r3;
                grad[L.w2 + (size_t)i * MLP_H + j] += h1[i] * r2;
            }
            for (int i = 0; i < MLP_IN; ++i) grad[L.w1 + (size_t)i * MLP_H + j] += (double)x[i] * r1;
            grad[L.b3 + j] += da3[j];
            grad[L.b2 + j] += da2[j];
            grad[L.b1 + j] += da1[j];
        }
    }
    free(z);
    free(dz);
    free(w);
    return loss;
}

/* Lights grouped by cluster (stable by index) with one alias table per cluster
 * over its members (createAliasTable, src/misc.cpp:418-497, on the subset):
 * order[pos] light at grouped position pos, offset[c] first position of
 * cluster c (offset[k] = n), col[pos] the column with its alias as a grouped
 * position, within[light] p(light | its cluster). */
int or_cluster_tables(const or_point_light *pl, int32_t n, const int32_t *cluster_of, int32_t k, int32_t *order,
                      int32_t *offset, or_alias *col, float *within) {
    int32_t *cnt = (int32_t *)calloc((size_t)k + 1, sizeof(int32_t));
    for (int32_t i = 0; i < n; ++i) {
        if (cluster_of[i] < 0 || cluster_of[i] >= k) { free(cnt); return -1; }
        ++cnt[cluster_of[i] + 1];
    }
    offset[0] = 0;
    for (int32_t c = 0; c < k; ++c) offset[c + 1] = offset[c] + cnt[c + 1];
    int32_t *fill = (int32_t *)malloc((size_t)k * sizeof(int32_t));
    memcpy(fill, offset, (size_t)k * sizeof(int32_t));
    for (int32_t i = 0; i < n; ++i) order[fill[cluster_of[i]]++] = i;
    or_point_light *sub = (or_point_light *)malloc((size_t)n * sizeof(or_point_light));
    for (int32_t c = 0; c < k; ++c) {
        const int32_t b = offset[c], m = offset[c + 1] - b;
        if (m <= 0) continue;
        for (int32_t j = 0; j < m; ++j) sub[j] = pl[order[b + j]];
        or_build_alias_table(sub, m, NULL, 0, col + b);
        for (int32_t j = 0; j < m; ++j) {
            col[b + j].alias += b;
            within[order[b + j]] = col[b + j].ori_prob;
        }
    }
    free(sub);
    free(fill);
    free(cnt);
    return 0;
}

/* collectTriangleLightsFromScene (src/misc.cpp:380-414): every triangle of an
 * instance whose material's emissiveFactor.sq_norm() > 1e-6 (a float compared
 * with a double literal); vertices are node.worldMatrix * vec4(pos, 1)
 * (nvmath.inl:491-499, sums left to right, matrix column-major), normal =
 * cross(p2 - p1, p3 - p1) (nvmath.inl:254-261), area = normal.norm()
 * (sqrtf of x*x + y*y + z*z), normal /= area, area *= 0.5f; emission =
 * (emissiveFactor, luminance) with luminance of common.glsl:7-9. */
int64_t or_collect_tri_lights(const or_mesh_instance *inst, int32_t n, or_tri_light *out, int64_t cap) {
    int64_t count = 0;
    for (int32_t k = 0; k < n; ++k) {
        const float *ef = inst[k].emissive_factor;
        float sq = ef[0] * ef[0];
        sq = sq + ef[1] * ef[1];
        sq = sq + ef[2] * ef[2];
        if (!((double)sq > 1e-6)) continue;
        const float *w = inst[k].world_matrix;
        float lum = 0.2126f * ef[0];
        lum = lum + 0.7152f * ef[1];
        lum = lum + 0.0722f * ef[2];
        for (uint32_t t = 0; t + 2 < inst[k].index_count; t += 3) {
            float v[3][4];
            for (int c = 0; c < 3; ++c) {
                const float *pos = inst[k].positions + 3 * (size_t)inst[k].indices[t + c];
                for (int row = 0; row < 4; ++row) {
                    float acc = w[0 * 4 + row] * pos[0];
                    acc = acc + w[1 * 4 + row] * pos[1];
                    acc = acc + w[2 * 4 + row] * pos[2];
                    acc = acc + w[3 * 4 + row] * 1.0f;
                    v[c][row] = acc;
                }
            }
            float e1[3], e2[3], nrm[3];
            for (int c = 0; c < 3; ++c) {
                e1[c] = v[1][c] - v[0][c];
                e2[c] = v[2][c] - v[0][c];
            }
            nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
            nrm[1] = e1[2] * e2[0] - e1[0] * e2[2];
            nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
            float len2 = nrm[0] * nrm[0];
            len2 = len2 + nrm[1] * nrm[1];
            len2 = len2 + nrm[2] * nrm[2];
            float area = sqrtf(len2);
            for (int c = 0; c < 3; ++c) nrm[c] = nrm[c] / area;
            area = area * 0.5f;
            if (out && count < cap) {
                or_tri_light *o = &out[count];
                o->p1 = (or_f4){v[0][0], v[0][1], v[0][2], v[0][3]};
                o->p2 = (or_f4){v[1][0], v[1][1], v[1][2], v[1][3]};
                o->p3 = (or_f4){v[2][0], v[2][1], v[2][2], v[2][3]};
                o->emission_lum = (or_f4){ef[0], ef[1], ef[2], lum};
                o->normal_area = (or_f4){nrm[0], nrm[1], nrm[2], area};
            }
            ++count;
        }
    }
    return count;
}
