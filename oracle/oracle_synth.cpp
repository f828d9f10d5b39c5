// Seeded synthetic molecules on the oracle side.  TEST INFRASTRUCTURE ONLY: the benchmark's
// CPU legs (the reference arm and the CPU baseline) build their inputs with these, so they
// never load the product library, and the tests check that every atom equals the library
// generator's (same seed, same bits).
//
// Workload definitions (no public dataset is involved):
//   ball  - N atoms uniform in a ball of radius (3N / (4 pi rho))^(1/3)
//   shell - N atoms uniform in volume in the shell r_in <= r <= r_in + t
// Candidates closer than `min_dist` to an accepted atom are rejected; each accepted atom
// then draws its element: C 62 % (1.70 A), N 17 % (1.55 A), O 19 % (1.52 A), S 2 % (1.80 A).
//
// Random stream: std::mt19937_64 (its output sequence is fixed by the C++ standard), a
// double in [0, 1) from the top 53 bits of each output.  Draw order per candidate: x, y, z
// for the ball (redrawn until inside); for the shell the radius from one draw by the
// inverse CDF of r^3, then direction draws x, y, z until 0 < |d|^2 <= 1.
#include <cmath>
#include <cstdint>
#include <random>
#include <unordered_map>
#include <vector>

namespace {

double unit(std::mt19937_64 &g) { return (double)(g() >> 11) * 0x1.0p-53; }

// Exact minimum-distance test: accepted atoms binned in cubes of edge min_dist, so every
// atom within min_dist of a candidate lies in the candidate's cube or one of its 26
// neighbours.  Bins are keyed by the cube's integer coordinates.
class Spacing {
  public:
    explicit Spacing(double min_dist) : edge_(min_dist > 0 ? min_dist : 1.0), limit2_(min_dist * min_dist) {}
    bool far_enough(const double *p) const {
        if (limit2_ <= 0) return true;
        long long c[3];
        cube(p, c);
        for (int i = -1; i <= 1; i++)
            for (int j = -1; j <= 1; j++)
                for (int k = -1; k <= 1; k++) {
                    auto it = bins_.find(pack(c[0] + i, c[1] + j, c[2] + k));
                    if (it == bins_.end()) continue;
                    for (size_t q : it->second) {
                        const double *a = &pos_[3 * q];
                        const double d0 = a[0] - p[0], d1 = a[1] - p[1], d2 = a[2] - p[2];
                        if (d0 * d0 + d1 * d1 + d2 * d2 < limit2_) return false;
                    }
                }
        return true;
    }
    void accept(const double *p) {
        if (limit2_ <= 0) return;
        long long c[3];
        cube(p, c);
        bins_[pack(c[0], c[1], c[2])].push_back(pos_.size() / 3);
        pos_.insert(pos_.end(), p, p + 3);
    }

  private:
    void cube(const double *p, long long *c) const {
        for (int q = 0; q < 3; q++) c[q] = (long long)std::floor(p[q] / edge_);
    }
    static unsigned long long pack(long long a, long long b, long long c) {
        const unsigned long long m = (1ull << 21) - 1;
        return (((unsigned long long)a & m) << 42) | (((unsigned long long)b & m) << 21) | ((unsigned long long)c & m);
    }
    double edge_, limit2_;
    std::vector<double> pos_;
    std::unordered_map<unsigned long long, std::vector<size_t>> bins_;
};

template <class Draw>
int place(unsigned N, uint64_t seed, float min_dist, Draw draw, float *xyz, float *rad) {
    std::mt19937_64 g(seed);
    Spacing sp((double)min_dist);
    const unsigned long long budget = 2000000ull + 1000ull * N;  // candidates before giving up
    unsigned long long used = 0;
    for (unsigned a = 0; a < N; a++) {
        double p[3];
        do {
            if (++used > budget) return 1;  // too dense to place N atoms
            draw(g, p);
        } while (!sp.far_enough(p));
        sp.accept(p);
        for (int q = 0; q < 3; q++) xyz[3 * a + q] = (float)p[q];
        const double u = unit(g);
        rad[a] = u < 0.62 ? 1.70f : u < 0.79 ? 1.55f : u < 0.98 ? 1.52f : 1.80f;
    }
    return 0;
}

}  // namespace

extern "C" {

int oracle_synth_ball(unsigned N, uint64_t seed, float density, float min_dist, float *xyz, float *rad) {
    if (!xyz || !rad || !(density > 0)) return 1;
    const double rb = std::cbrt(3.0 * N / (4.0 * 3.141592653589793 * (double)density));
    return place(N, seed, min_dist, [rb](std::mt19937_64 &g, double *p) {
        for (;;) {
            for (int q = 0; q < 3; q++) p[q] = (2 * unit(g) - 1) * rb;
            if (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] <= rb * rb) return;
        }
    }, xyz, rad);
}

int oracle_synth_shell(unsigned N, uint64_t seed, float r_in, float thickness, float min_dist, float *xyz,
                       float *rad) {
    if (!xyz || !rad || r_in < 0 || !(thickness > 0)) return 1;
    const double in3 = (double)r_in * r_in * r_in, out = (double)r_in + thickness, out3 = out * out * out;
    return place(N, seed, min_dist, [in3, out3](std::mt19937_64 &g, double *p) {
        const double r = std::cbrt(unit(g) * (out3 - in3) + in3);
        for (;;) {
            double d[3];
            for (int q = 0; q < 3; q++) d[q] = 2 * unit(g) - 1;
            const double n2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (n2 > 1e-12 && n2 <= 1.0) {
                const double s = r / std::sqrt(n2);
                for (int q = 0; q < 3; q++) p[q] = d[q] * s;
                return;
            }
        }
    }, xyz, rad);
}

}  // extern "C"
