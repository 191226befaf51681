// The integer-pipe reciprocal of csrc/khs_device_math.cuh (dm::recip_rn),
// compiled for the host, against the IEEE division 1.0 / x on random
// doubles over the whole exponent range, mantissas next to powers of two,
// and inputs whose reciprocal is below the normal range.  The device seed
// (rcp.approx.ftz.f32) differs from the host's correctly rounded float
// reciprocal by at most an ulp; the algorithm is also run with the seed
// perturbed by up to 3 ulps.  Built and run by tests/test_recip.py.
#include <cstdint>
#include <cstring>

// The seed with an offset of g_seed_ulps units in its last place.
static int g_seed_ulps = 0;
static float perturbed_seed(float m)
{
    float r = 1.0f / m;
    uint32_t b;
    std::memcpy(&b, &r, 4);
    b = uint32_t(int64_t(b) + g_seed_ulps);
    std::memcpy(&r, &b, 4);
    return r;
}
#define KHS_RECIP_SEED_HOST(m) perturbed_seed(m)
#include "khs_device_math.cuh"

#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace dm = khs::dm;

static uint64_t mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

int main(int argc, char **argv)
{
    const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : (1ull << 24);
    uint64_t bad = 0, checked = 0;
    for (int ulps = -3; ulps <= 3; ++ulps)
    for (uint64_t i = 0; i < n; ++i) {
        g_seed_ulps = ulps;
        const uint64_t z = mix64(i);
        uint64_t mant = z & 0xfffffffffffffull;
        if ((i & 7) == 0) mant = (i >> 3) & 0xffff;                       // just above a power of two
        if ((i & 7) == 1) mant = 0xfffffffffffffull - ((i >> 3) & 0xffff); // just below
        uint64_t ex = 1 + (z >> 52) % 2046;
        if ((i & 15) == 3) ex = 2040 + (z >> 52) % 7;                      // reciprocal subnormal or near it
        const double x = dm::double_of(((z >> 63) << 63) | (ex << 52) | mant);
        const double got = dm::recip_rn(x), want = 1.0 / x;
        ++checked;
        if (dm::bits_of(got) != dm::bits_of(want)) {
            if (bad < 5) std::printf("mismatch x=%a got=%a want=%a seed offset %d\n", x, got, want, ulps);
            ++bad;
        }
    }
    std::printf("%llu values, %llu mismatches\n", (unsigned long long)checked, (unsigned long long)bad);
    if (bad == 0) std::printf("PASS\n");
    return bad != 0;
}
