// Seeded synthetic molecules for benchmarks and tests (no public dataset is involved).
//
// Generators follow the workload definitions used for the SES benchmarks:
//   * ball   - N heavy atoms uniform in a ball of radius (3N / (4 pi rho))^(1/3)
//   * shell  - N heavy atoms uniform in volume in a spherical shell [r_in, r_in + t]
//   * jitter - i.i.d. Gaussian displacement of a base frame (trajectory frames)
// with rejection of any atom closer than `min_dist` to an accepted one, and the element
// mix C 62% / N 17% / O 19% / S 2% with radii 1.70 / 1.55 / 1.52 / 1.80 A.
//
// The random stream is std::mt19937_64 (fully specified by the C++ standard) with our own
// uniform/normal transforms, so the same seed gives the same molecule on every host.
#include <cmath>
#include <cstdint>
#include <random>
#include <unordered_map>
#include <vector>

#include "qses_internal.h"

namespace {

struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t seed) : g(seed) {}
    double uni() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
    double normal() {  // Box-Muller, one value per call
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

// Hash grid for the minimum-distance rejection.
struct Reject {
    double cell, md2;
    std::unordered_map<uint64_t, std::vector<uint32_t>> bins;
    const std::vector<double> &pts;
    Reject(double min_dist, const std::vector<double> &p) : cell(min_dist > 0 ? min_dist : 1.0),
                                                          md2(min_dist * min_dist), pts(p) {}
    static uint64_t key(int64_t a, int64_t b, int64_t c) {
        return ((uint64_t)(a & 0x1fffff) << 42) | ((uint64_t)(b & 0x1fffff) << 21) | (uint64_t)(c & 0x1fffff);
    }
    bool ok(double x, double y, double z) const {
        if (md2 <= 0) return true;
        int64_t a = (int64_t)std::floor(x / cell), b = (int64_t)std::floor(y / cell), c = (int64_t)std::floor(z / cell);
        for (int i = -1; i <= 1; i++)
            for (int j = -1; j <= 1; j++)
                for (int k = -1; k <= 1; k++) {
                    auto it = bins.find(key(a + i, b + j, c + k));
                    if (it == bins.end()) continue;
                    for (uint32_t q : it->second) {
                        double dx = pts[3 * q] - x, dy = pts[3 * q + 1] - y, dz = pts[3 * q + 2] - z;
                        if (dx * dx + dy * dy + dz * dz < md2) return false;
                    }
                }
        return true;
    }
    void add(uint32_t id, double x, double y, double z) {
        if (md2 <= 0) return;
        bins[key((int64_t)std::floor(x / cell), (int64_t)std::floor(y / cell), (int64_t)std::floor(z / cell))].push_back(id);
    }
};

void element(Rng &rng, float *rad, unsigned char *elem, unsigned a) {
    double u = rng.uni();
    unsigned char e;
    float r;
    if (u < 0.62) { e = 'C'; r = 1.70f; }
    else if (u < 0.79) { e = 'N'; r = 1.55f; }
    else if (u < 0.98) { e = 'O'; r = 1.52f; }
    else { e = 'S'; r = 1.80f; }
    rad[a] = r;
    if (elem) elem[a] = e;
}

template <class Sampler>
int generate(unsigned N, uint64_t seed, double min_dist, Sampler sample, float *xyz, float *rad,
             unsigned char *elem) {
    Rng rng(seed);
    std::vector<double> pts;
    pts.reserve((size_t)N * 3);
    Reject rej(min_dist, pts);
    const uint64_t max_tries = 2000000ull + 1000ull * N;
    uint64_t tries = 0;
    for (unsigned a = 0; a < N; a++) {
        double p[3];
        for (;;) {
            if (++tries > max_tries) return QSES_ERR_INVALID_ARG;  // packing too dense
            sample(rng, p);
            if (rej.ok(p[0], p[1], p[2])) break;
        }
        rej.add(a, p[0], p[1], p[2]);
        pts.push_back(p[0]); pts.push_back(p[1]); pts.push_back(p[2]);
        xyz[3 * a] = (float)p[0]; xyz[3 * a + 1] = (float)p[1]; xyz[3 * a + 2] = (float)p[2];
        element(rng, rad, elem, a);
    }
    return QSES_OK;
}

}  // namespace

extern "C" {

QSES_API int qses_synth_ball(unsigned N, uint64_t seed, float density, float min_dist, float *xyz, float *rad,
                             unsigned char *elem) {
    if (!xyz || !rad || density <= 0) return QSES_ERR_INVALID_ARG;
    const double Rb = std::cbrt(3.0 * N / (4.0 * 3.141592653589793 * density));
    auto sample = [Rb](Rng &rng, double *p) {
        for (;;) {
            double x = (2 * rng.uni() - 1) * Rb, y = (2 * rng.uni() - 1) * Rb, z = (2 * rng.uni() - 1) * Rb;
            if (x * x + y * y + z * z <= Rb * Rb) { p[0] = x; p[1] = y; p[2] = z; return; }
        }
    };
    return generate(N, seed, min_dist, sample, xyz, rad, elem);
}

QSES_API int qses_synth_shell(unsigned N, uint64_t seed, float r_in, float thickness, float min_dist, float *xyz,
                              float *rad, unsigned char *elem) {
    if (!xyz || !rad || r_in < 0 || thickness <= 0) return QSES_ERR_INVALID_ARG;
    const double ri3 = (double)r_in * r_in * r_in, ro = (double)r_in + thickness, ro3 = ro * ro * ro;
    auto sample = [ri3, ro3](Rng &rng, double *p) {
        double r = std::cbrt(rng.uni() * (ro3 - ri3) + ri3);
        for (;;) {
            double x = 2 * rng.uni() - 1, y = 2 * rng.uni() - 1, z = 2 * rng.uni() - 1;
            double n2 = x * x + y * y + z * z;
            if (n2 > 1e-12 && n2 <= 1.0) {
                double s = r / std::sqrt(n2);
                p[0] = x * s; p[1] = y * s; p[2] = z * s;
                return;
            }
        }
    };
    return generate(N, seed, min_dist, sample, xyz, rad, elem);
}

QSES_API int qses_synth_jitter(const float *base_xyz, unsigned N, float sigma, uint64_t seed, float *out_xyz) {
    if (!base_xyz || !out_xyz) return QSES_ERR_INVALID_ARG;
    Rng rng(seed);
    for (size_t q = 0; q < (size_t)N * 3; q++) out_xyz[q] = (float)((double)base_xyz[q] + sigma * rng.normal());
    return QSES_OK;
}

}  // extern "C"
