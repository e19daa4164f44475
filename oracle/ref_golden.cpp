// ref_golden.cpp — TEST INFRASTRUCTURE ONLY.  Emits golden vectors computed by the
// reference's own header-only math (include/axiom/math/{vec3,aabb,random}.hpp of
// itsakeyfut/axiom-physics-engine), compiled where those headers lie by
// oracle/build_ref.sh into oracle/_ref/ref_golden.  Nothing of the reference is copied:
// this program only includes its headers and prints what they compute, as JSON, for
// tests/golden/make_golden.py to freeze into tests/golden/ref_math.json.
//
// Quaternion and transform code (src/math/quat.cpp, transform.cpp) needs GLM, which is
// not available here; those semantics are pinned by restated reference test cases
// instead (tests/test_oracle_math.py).
#include <cinttypes>
#include <cstdio>
#include <vector>

#include "axiom/math/aabb.hpp"
#include "axiom/math/random.hpp"
#include "axiom/math/vec3.hpp"

using axiom::math::AABB;
using axiom::math::DeterministicRNG;
using axiom::math::Vec3;

static void printFloat(float f) { std::printf("%.9g", (double)f); }

int main() {
    std::printf("{\n");
    // ---- DeterministicRNG (random.hpp:19-64) ----
    const uint64_t seeds[] = {0ull, 1ull, 42ull, 12345ull, 54321ull, 0x8000000000000005ull};
    std::printf("\"rng\": [\n");
    for (size_t s = 0; s < sizeof(seeds) / sizeof(seeds[0]); ++s) {
        DeterministicRNG a(seeds[s]), b(seeds[s]), c(seeds[s]), d(seeds[s]);
        std::printf("  {\"seed\": %" PRIu64 ", \"u32\": [", seeds[s]);
        for (int i = 0; i < 64; ++i) std::printf("%s%u", i ? ", " : "", a.next());
        std::printf("], \"float\": [");
        for (int i = 0; i < 64; ++i) {
            std::printf("%s", i ? ", " : "");
            printFloat(b.nextFloat());
        }
        std::printf("], \"float_jitter\": [");
        for (int i = 0; i < 32; ++i) {
            std::printf("%s", i ? ", " : "");
            printFloat(c.nextFloat(-0.002f, 0.002f));
        }
        std::printf("], \"float_10_20\": [");
        for (int i = 0; i < 32; ++i) {
            std::printf("%s", i ? ", " : "");
            printFloat(d.nextFloat(10.0f, 20.0f));
        }
        std::printf("]}%s\n", s + 1 < sizeof(seeds) / sizeof(seeds[0]) ? "," : "");
    }
    std::printf("],\n");

    // ---- AABB::intersects / fromCenterExtents / expand(margin) (aabb.hpp:132-215) ----
    // Boxes on a coarse 0.25 grid so that exact touching happens often.
    DeterministicRNG rng(7);
    auto q = [&](void) { return (float)(int)(rng.next() % 17u) * 0.25f; };
    std::printf("\"aabb\": [\n");
    const int nCases = 400;
    for (int k = 0; k < nCases; ++k) {
        Vec3 ca(q(), q(), q()), ea(0.25f + q() * 0.25f, 0.25f + q() * 0.25f, 0.25f + q() * 0.25f);
        Vec3 cb(q(), q(), q()), eb(0.25f + q() * 0.25f, 0.25f + q() * 0.25f, 0.25f + q() * 0.25f);
        AABB a = AABB::fromCenterExtents(ca, ea);
        AABB b = AABB::fromCenterExtents(cb, eb);
        float margin = (float)(k % 3) * 0.125f;
        AABB am = a;
        am.expand(margin);
        std::printf("  {\"ca\": [%.9g, %.9g, %.9g], \"ea\": [%.9g, %.9g, %.9g], ", ca.x, ca.y, ca.z,
                    ea.x, ea.y, ea.z);
        std::printf("\"cb\": [%.9g, %.9g, %.9g], \"eb\": [%.9g, %.9g, %.9g], ", cb.x, cb.y, cb.z,
                    eb.x, eb.y, eb.z);
        std::printf("\"amin\": [%.9g, %.9g, %.9g], \"amax\": [%.9g, %.9g, %.9g], ", a.min.x,
                    a.min.y, a.min.z, a.max.x, a.max.y, a.max.z);
        std::printf("\"margin\": %.9g, \"am_min\": [%.9g, %.9g, %.9g], \"am_max\": [%.9g, %.9g, %.9g], ",
                    margin, am.min.x, am.min.y, am.min.z, am.max.x, am.max.y, am.max.z);
        std::printf("\"ab\": %s, \"ba\": %s}%s\n", a.intersects(b) ? "true" : "false",
                    b.intersects(a) ? "true" : "false", k + 1 < nCases ? "," : "");
    }
    std::printf("],\n");

    // ---- Vec3 dot / cross / normalized (vec3.hpp:179-215) ----
    DeterministicRNG vr(99);
    std::printf("\"vec3\": [\n");
    const int nVec = 64;
    for (int k = 0; k < nVec; ++k) {
        Vec3 a = k == 0 ? Vec3(0.0f, 0.0f, 0.0f)
                        : Vec3(vr.nextFloat(-5.0f, 5.0f), vr.nextFloat(-5.0f, 5.0f), vr.nextFloat(-5.0f, 5.0f));
        Vec3 b(vr.nextFloat(-5.0f, 5.0f), vr.nextFloat(-5.0f, 5.0f), vr.nextFloat(-5.0f, 5.0f));
        Vec3 n = a.normalized();
        Vec3 c = a.cross(b);
        std::printf("  {\"a\": [%.9g, %.9g, %.9g], \"b\": [%.9g, %.9g, %.9g], \"dot\": %.9g, ", a.x,
                    a.y, a.z, b.x, b.y, b.z, a.dot(b));
        std::printf("\"cross\": [%.9g, %.9g, %.9g], \"normalized\": [%.9g, %.9g, %.9g]}%s\n", c.x, c.y,
                    c.z, n.x, n.y, n.z, k + 1 < nVec ? "," : "");
    }
    std::printf("]\n}\n");
    return 0;
}
