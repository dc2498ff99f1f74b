// ref_reservoir_bridge.cpp -- compiles the reference's reservoir operations
// (src/shaders/include/reservoir.glsl, rand.glsl, structs/restirStructs.glsl)
// as C++ for one RESERVOIR_SIZE / UNBIASED_MIS variant, from copies that
// oracle/Makefile derives into oracle/_ref/res_<variant>/ with three textual
// changes: `inout T x` becomes `T &x`, the `#extension` line is dropped, and
// the two variant #defines of restirStructs.glsl:16-17 are set.  Exports one
// scripted sequence of operations so the tests can pin the oracle's variant
// builds against the reference's own code.
//
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/; nothing here is shipped.
#include <cstdint>
#include <cstring>

#include "refshim/glsl_shim.hpp"

namespace refres {
using namespace glsl;
using uint = unsigned;
struct mat4 { gfloat m[16]; };
struct uvec2 { unsigned x, y; };
#define float gfloat
#include "reservoir.glsl"
#undef float
}  // namespace refres

extern "C" {

// Interchange layout: per sample 16 floats (position xyz + emission luminance,
// normal xyzw, light index (int bits), p-hat, sumWeights, w, sumPHat, 3
// unused), then numStreamSamples (uint bits) and 3 unused: RS * 16 + 4 floats.
int32_t ref_reservoir_size(int32_t *mis) {
#ifdef UNBIASED_MIS
    *mis = 1;
#else
    *mis = 0;
#endif
    return RESERVOIR_SIZE;
}

static void to_flat(const refres::Reservoir &r, float *o) {
    for (int i = 0; i < RESERVOIR_SIZE; ++i) {
        const refres::LightSample &s = r.samples[i];
        float *p = o + 16 * i;
        p[0] = s.position_emissionLum.xyz.x.v; p[1] = s.position_emissionLum.xyz.y.v;
        p[2] = s.position_emissionLum.xyz.z.v; p[3] = s.position_emissionLum.w.v;
        p[4] = s.normal.xyz.x.v; p[5] = s.normal.xyz.y.v; p[6] = s.normal.xyz.z.v; p[7] = s.normal.w.v;
        std::memcpy(&p[8], &s.lightIndex, 4);
        p[9] = s.pHat.v; p[10] = s.sumWeights.v; p[11] = s.w.v;
#ifdef UNBIASED_MIS
        p[12] = s.sumPHat.v;
#else
        p[12] = 0.0f;
#endif
        p[13] = p[14] = p[15] = 0.0f;
    }
    std::memcpy(o + 16 * RESERVOIR_SIZE, &r.numStreamSamples, 4);
    o[16 * RESERVOIR_SIZE + 1] = o[16 * RESERVOIR_SIZE + 2] = o[16 * RESERVOIR_SIZE + 3] = 0.0f;
}

static refres::Reservoir from_flat(const float *o) {
    refres::Reservoir r = refres::newReservoir();
    for (int i = 0; i < RESERVOIR_SIZE; ++i) {
        refres::LightSample &s = r.samples[i];
        const float *p = o + 16 * i;
        s.position_emissionLum = refres::vec4(p[0], p[1], p[2], p[3]);
        s.normal = refres::vec4(p[4], p[5], p[6], p[7]);
        std::memcpy(&s.lightIndex, &p[8], 4);
        s.pHat = p[9]; s.sumWeights = p[10]; s.w = p[11];
#ifdef UNBIASED_MIS
        s.sumPHat = p[12];
#endif
    }
    std::memcpy(&r.numStreamSamples, o + 16 * RESERVOIR_SIZE, 4);
    return r;
}

// newReservoir; addSampleToReservoir for each candidate (12 floats: position
// xyz, normal xyzw, emission luminance, light index bits, p-hat, source pdf,
// unused); then combineReservoirs(other, other_phat) if other != null.
void ref_reservoir_script(const float *cand, int32_t n, const float *other, const float *other_phat, uint64_t seed,
                          uint64_t seq, float *out) {
    refres::Rand rng = refres::seedRand(seed, seq);
    refres::Reservoir r = refres::newReservoir();
    for (int i = 0; i < RESERVOIR_SIZE; ++i) {  // fields newReservoir leaves undefined: zero, as the oracle
        r.samples[i].position_emissionLum = refres::vec4(0.0f, 0.0f, 0.0f, 0.0f);
        r.samples[i].normal = refres::vec4(0.0f, 0.0f, 0.0f, 0.0f);
        r.samples[i].lightIndex = 0;
        r.samples[i].pHat = 0.0f;
        r.samples[i].w = 0.0f;
    }
    for (int32_t k = 0; k < n; ++k) {
        const float *c = cand + 12 * (size_t)k;
        int32_t idx;
        std::memcpy(&idx, &c[8], 4);
        refres::addSampleToReservoir(r, refres::vec3(c[0], c[1], c[2]), refres::vec4(c[3], c[4], c[5], c[6]), c[7],
                                     idx, c[9], c[10], rng);
    }
    if (other) {
        refres::gfloat ph[RESERVOIR_SIZE];
        for (int i = 0; i < RESERVOIR_SIZE; ++i) ph[i] = other_phat[i];
        refres::combineReservoirs(r, from_flat(other), ph, rng);
    }
    to_flat(r, out);
}

}  // extern "C"
