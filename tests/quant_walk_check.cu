// Host-side check of the quantized 4-wide copy of the tree (host_pack_quant),
// built by tests/test_quant_tree.py and run on the CPU.
//
// For seeded scenes (an axis-aligned floor grid, random small triangles,
// axis-aligned quads; optionally shifted far from the origin) it builds the
// reference's tree (host_build_bvh), packs the quantized copy and checks:
//  - every decoded child box contains the child's exact box;
//  - for segments aimed at triangle edges, nearly axis-aligned segments and
//    random ones, the set of triangles the quantized walk tests (the decoded
//    boxes' sure-miss test of trace_pool.cuh, near/far code words by the ray's
//    direction signs, constant difference margin; each reached triangle gated
//    by its exact box) equals the set whose whole box path passes the
//    reference's slab test (softwareRaytracing.glsl:9-14), and the any-hit
//    answers agree.
// Prints one line of counts; exit status 0 when every check holds.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <set>
#include <vector>

#include "host_internal.h"
#include "rg_math.cuh"

using rgm::f3;
using rgm::mk;

namespace {

float f_of(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// The filtered decision of trace_pool.cuh (hit / miss margins).
void filtered_decision(float rmin, float rmax, bool &hit, bool &miss) {
    const float kEps = 1.9073486328125e-6f, kTiny = 8.0779356694631609e-28f;
    const float dd = rmax - rmin;
    const float ss = fmaf(kEps, fabsf(rmin) + fabsf(rmax), kTiny);
    hit = rmin < 1.0f - kEps && rmax > kTiny && dd > ss;
    miss = rmin > 1.0f + kEps || rmax < -kTiny || dd < -ss;
}

struct Scene {
    std::vector<rg_aabb_tree_node> nodes;
    std::vector<rg_triangle> tris;
    std::vector<float> t12;
    std::vector<uint32_t> q;
    std::vector<float> ql;
};

// Triangles tested by the reference's walk (every box on the path passes).
void binary_set(const Scene &s, f3 o, f3 d, std::set<int> &tested, bool &any) {
    std::vector<int> st{0};
    while (!st.empty()) {
        const int x = st.back();
        st.pop_back();
        const rg_aabb_tree_node &nd = s.nodes[(size_t)x];
        for (int side = 0; side < 2; ++side) {
            const float *lo = side ? nd.right_aabb_min : nd.left_aabb_min;
            const float *hi = side ? nd.right_aabb_max : nd.left_aabb_max;
            if (!rgm::ray_aabb(o, d, mk(lo[0], lo[1], lo[2]), mk(hi[0], hi[1], hi[2]))) continue;
            const int c = side ? nd.right_child : nd.left_child;
            if (c >= 0) {
                st.push_back(c);
            } else {
                tested.insert(~c);
                const float *p = &s.t12[12 * (size_t)(~c)];
                any = any || rgm::ray_tri(mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8]), o, d);
            }
        }
    }
}

// Leaf records gated by the quantized walk (the device arithmetic).
void quant_set(const Scene &s, f3 o, f3 d, f3 inv, std::set<int> &gated, bool &any, long &visits) {
    std::vector<int> st{0};
    const float iv[3] = {inv.x, inv.y, inv.z}, oo[3] = {o.x, o.y, o.z};
    while (!st.empty()) {
        const int x = st.back();
        st.pop_back();
        ++visits;
        const uint32_t *w = &s.q[16 * (size_t)x];
        const float base[3] = {f_of(w[0]), f_of(w[1]), f_of(w[2])};
        const int eb[3] = {(int)(w[3] & 255u), (int)((w[3] >> 8) & 255u), (int)((w[3] >> 16) & 255u)};
        const unsigned meta = w[3] >> 24;
        int32_t links[4];
        memcpy(links, &w[12], sizeof(links));
        // the walk reads the x and y scales as floats from words 10 and 11
        const float scale[3] = {f_of(w[10]), f_of(w[11]), f_of((uint32_t)eb[2] << 23)};
        if (w[10] != ((uint32_t)eb[0] << 23) || w[11] != ((uint32_t)eb[1] << 23)) {
            printf("scale words differ from the exponent bytes\n");
            exit(4);
        }
        for (int k = 0; k < 4; ++k) {
            const bool leaf = ((meta >> k) & 1u) != 0, inner = ((meta >> (4 + k)) & 1u) != 0;
            if (!leaf && !inner) continue;
            float tn[3], tf[3];
            for (int a = 0; a < 3; ++a) {
                const float sc = scale[a];
                const unsigned ql = (w[4 + 2 * a] >> (8 * k)) & 255u, qh = (w[5 + 2 * a] >> (8 * k)) & 255u;
                const float lo = fmaf(f_of(0x4B000000u | ql), sc, base[a]);
                const float hi = fmaf(f_of(0x4B000000u | qh), sc, base[a]);
                const float n_ = iv[a] < 0.0f ? hi : lo, f_ = iv[a] < 0.0f ? lo : hi;
                tn[a] = (n_ + (-oo[a])) * iv[a];
                tf[a] = (f_ + (-oo[a])) * iv[a];
            }
            const float rmin = fmaxf(fmaxf(tn[0], tn[1]), tn[2]), rmax = fminf(fminf(tf[0], tf[1]), tf[2]);
            const float a1 = fmaf(rmin, -1.0f, 1.0000019073486328125f), b1 = rmax + 8.0779356694631609e-28f;
            const float c1 = fmaf(rmin, -1.0f, rmax) + 7.62939453125e-6f;
            if (fminf(fminf(a1, b1), c1) < 0.0f) continue;
            if (inner) {
                st.push_back(links[k]);
                continue;
            }
            const float *r = &s.ql[16 * (size_t)(~links[k])];
            float gn[3], gf[3];
            for (int a = 0; a < 3; ++a) {
                const float t0 = (r[a] + (-oo[a])) * iv[a], t1 = (r[3 + a] + (-oo[a])) * iv[a];
                gn[a] = fminf(t0, t1);
                gf[a] = fmaxf(t0, t1);
            }
            bool h, m;
            filtered_decision(fmaxf(fmaxf(gn[0], gn[1]), gn[2]), fminf(fminf(gf[0], gf[1]), gf[2]), h, m);
            if (!h && !m) h = rgm::ray_aabb(o, d, mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]));
            if (!h) continue;
            gated.insert(~links[k]);
            any = any || rgm::ray_tri(mk(r[6], r[7], r[8]), mk(r[9], r[10], r[11]), mk(r[12], r[13], r[14]), o, d);
        }
    }
}

// Every decoded child box contains the exact boxes of all leaves below that
// child (a leaf slot: its own record's box).  Returns the node's leaf-box
// union through lo/hi.
long containment_failures(const Scene &s, int x, float lo[3], float hi[3]) {
    long bad = 0;
    const uint32_t *w = &s.q[16 * (size_t)x];
    const unsigned meta = w[3] >> 24;
    int32_t links[4];
    memcpy(links, &w[12], sizeof(links));
    for (int a = 0; a < 3; ++a) { lo[a] = INFINITY; hi[a] = -INFINITY; }
    for (int k = 0; k < 4; ++k) {
        const bool leaf = ((meta >> k) & 1u) != 0, inner = ((meta >> (4 + k)) & 1u) != 0;
        if (!leaf && !inner) continue;
        float clo[3], chi[3];
        if (leaf) {
            const float *r = &s.ql[16 * (size_t)(~links[k])];
            for (int a = 0; a < 3; ++a) { clo[a] = r[a]; chi[a] = r[3 + a]; }
        } else {
            bad += containment_failures(s, links[k], clo, chi);
        }
        for (int a = 0; a < 3; ++a) {
            const float sc = f_of((uint32_t)((w[3] >> (8 * a)) & 255u) << 23);
            const float base = f_of(w[a]);
            const float dlo = fmaf(f_of(0x4B000000u | ((w[4 + 2 * a] >> (8 * k)) & 255u)), sc, base);
            const float dhi = fmaf(f_of(0x4B000000u | ((w[5 + 2 * a] >> (8 * k)) & 255u)), sc, base);
            if (!(dlo <= clo[a]) || !(dhi >= chi[a])) ++bad;
            lo[a] = fminf(lo[a], clo[a]);
            hi[a] = fmaxf(hi[a], chi[a]);
        }
    }
    return bad;
}

}  // namespace

int main(int argc, char **argv) {
    const int ntri = argc > 1 ? atoi(argv[1]) : 20000;
    const int nrays = argc > 2 ? atoi(argv[2]) : 10000;
    const float off = argc > 3 ? (float)atof(argv[3]) : 0.0f;
    const unsigned seed = argc > 4 ? (unsigned)atoi(argv[4]) : 7u;
    std::mt19937 rng(seed);
    std::uniform_real_distribution<float> U(-10.f, 10.f), S(0.f, 1.f);
    std::vector<float> xyz;
    const int g = 40;  // floor grid: flat boxes
    for (int i = 0; i < g; ++i)
        for (int j = 0; j < g; ++j) {
            const float x0 = -10 + 20.f * i / g, x1 = -10 + 20.f * (i + 1) / g;
            const float z0 = -10 + 20.f * j / g, z1 = -10 + 20.f * (j + 1) / g;
            const float a[18] = {x0, 0, z0, x1, 0, z0, x1, 0, z1, x0, 0, z0, x1, 0, z1, x0, 0, z1};
            xyz.insert(xyz.end(), a, a + 18);
        }
    while ((int)xyz.size() / 9 < ntri) {
        const float cx = U(rng), cy = 5 + 0.5f * U(rng), cz = U(rng), sz = 0.05f + 0.5f * S(rng);
        if (S(rng) < 0.2f) {  // axis-aligned quad
            float a[9] = {cx, cy, cz, cx + sz, cy, cz, cx, cy, cz + sz};
            if (S(rng) < 0.5f) { a[3] = cx; a[4] = cy + sz; a[6] = cx; a[7] = cy; a[8] = cz + sz; }
            xyz.insert(xyz.end(), a, a + 9);
        } else {
            for (int k = 0; k < 3; ++k) {
                xyz.push_back(cx + sz * (S(rng) - 0.5f));
                xyz.push_back(cy + sz * (S(rng) - 0.5f));
                xyz.push_back(cz + sz * (S(rng) - 0.5f));
            }
        }
    }
    for (size_t i = 0; i < xyz.size(); i += 3) xyz[i] += off;
    const int n = (int)xyz.size() / 9;
    Scene s;
    s.nodes.resize((size_t)n - 1);
    s.tris.resize((size_t)n);
    int undefined = 0;
    if (host_build_bvh(xyz.data(), n, s.nodes.data(), s.tris.data(), &undefined) < 0) {
        printf("tree build failed\n");
        return 1;
    }
    s.t12.resize(12 * (size_t)n);
    host_pack_tris(s.tris.data(), n, s.t12.data());
    int depth = 0;
    const int nq = host_pack_quant(s.nodes.data(), n - 1, s.t12.data(), s.q, s.ql, &depth);
    if (nq <= 0 || (int)(s.ql.size() / 16) != n) {
        printf("quantized copy not built (%d)\n", nq);
        return 1;
    }
    float rlo[3], rhi[3];
    const long contain = containment_failures(s, 0, rlo, rhi);
    long fast = 0, set_mismatch = 0, any_mismatch = 0, visits = 0;
    std::uniform_int_distribution<int> T(0, n - 1);
    for (int i = 0; i < nrays; ++i) {
        f3 p1, p2;
        const int kind = i % 4;
        if (kind == 0) {
            p1 = mk(U(rng), 0.0f, U(rng));
            p2 = mk(U(rng), 8 + U(rng) * 0.3f, U(rng));
        } else if (kind == 1) {  // through a point of a triangle edge
            const rg_triangle &t = s.tris[(size_t)T(rng)];
            const float u = S(rng);
            const f3 m = mk(t.p1[0] + u * (t.p2[0] - t.p1[0]), t.p1[1] + u * (t.p2[1] - t.p1[1]),
                            t.p1[2] + u * (t.p2[2] - t.p1[2]));
            p1 = mk(U(rng) + off, 0.0f, U(rng));
            p2 = mk(m.x + (m.x - p1.x), m.y + (m.y - p1.y), m.z + (m.z - p1.z));
            p1.x -= off;
            p2.x -= off;
        } else if (kind == 2) {  // nearly axis-aligned
            p1 = mk(U(rng), 0.0f, U(rng));
            p2 = mk(p1.x + 1e-4f * U(rng), 9.0f, p1.z + 1e-4f * U(rng));
        } else {
            p1 = mk(U(rng), 5 + U(rng) * 0.3f, U(rng));
            p2 = mk(U(rng), 5 + U(rng) * 0.3f, U(rng));
        }
        p1.x += off;
        p2.x += off;
        f3 o, d;
        rgm::shadow_segment(p1, p2, o, d);
        const float lo = 7.8886090522101181e-31f, hi = 1.2676506002282294e30f;
        if (!(fabsf(d.x) >= lo && fabsf(d.x) <= hi && fabsf(d.y) >= lo && fabsf(d.y) <= hi && fabsf(d.z) >= lo &&
              fabsf(d.z) <= hi))
            continue;  // off the fast path: those rays walk the reference's tree
        ++fast;
        const f3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        std::set<int> bt, qg;
        bool ba = false, qa = false;
        binary_set(s, o, d, bt, ba);
        quant_set(s, o, d, inv, qg, qa, visits);
        // leaf records hold the triangles' own fields: compare the sets by them
        std::set<int> qg_tri;
        for (int r : qg) {
            const float *rp = &s.ql[16 * (size_t)r];
            int found = -1;
            for (int t : bt)
                if (!memcmp(&s.t12[12 * (size_t)t], rp + 6, 36)) { found = t; break; }
            qg_tri.insert(found);
        }
        if (qg_tri != bt || qg.size() != bt.size()) ++set_mismatch;
        if (ba != qa) ++any_mismatch;
    }
    printf("triangles %d quantized_nodes %d containment_failures %ld fast_rays %ld set_mismatches %ld "
           "answer_mismatches %ld visits_per_ray %.2f\n",
           n, nq, contain, fast, set_mismatch, any_mismatch, fast ? (double)visits / fast : 0.0);
    return (contain || set_mismatch || any_mismatch || fast < nrays / 2) ? 2 : 0;
}
