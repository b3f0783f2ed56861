// The C++ drop-in's exchange arrays: Particle -> structure of arrays ->
// Particle against a plain one-thread conversion, bit for bit, for a count
// that is split over host threads and for small ones that are not.  Needs no
// GPU and no library (only the header's free functions are used).
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "rd_lagrange_euler_view.hpp"

using MaterialPointMethod::Particle;
namespace mpd = MaterialPointMethod::detail;

static bool same(float a, float b) { return std::memcmp(&a, &b, sizeof a) == 0; }

static int check(int n) {
    std::mt19937 rng(static_cast<unsigned>(n) + 1u);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    std::vector<Particle> ps(n);
    for (auto& p : ps) {
        for (int a = 0; a < 3; ++a) { p.pos[a] = U(rng); p.velocity[a] = U(rng); }
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) {
                p.B[c][r] = U(rng);
                p.FElastic[c][r] = U(rng);
                p.FPlastic[c][r] = U(rng);
            }
        p.mass = U(rng);
        p.volume = U(rng);
    }
    const size_t N = static_cast<size_t>(n);
    std::vector<float> soa(36 * N + 1, 0.0f), ref(36 * N + 1, 0.0f);
    mpd::particles_to_soa(ps.data(), n, soa.data());
    for (size_t i = 0; i < N; ++i) {
        const Particle& p = ps[i];
        for (int a = 0; a < 3; ++a) { ref[3 * i + a] = p.pos[a]; ref[3 * N + 3 * i + a] = p.velocity[a]; }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                ref[6 * N + 9 * i + 3 * r + c] = p.B[c][r];
                ref[15 * N + 9 * i + 3 * r + c] = p.FElastic[c][r];
                ref[24 * N + 9 * i + 3 * r + c] = p.FPlastic[c][r];
            }
        ref[33 * N + i] = p.mass;
        ref[34 * N + i] = p.volume;
    }
    if (std::memcmp(soa.data(), ref.data(), soa.size() * sizeof(float)) != 0) return 1;
    std::vector<Particle> back(n);
    mpd::soa_to_particles(soa.data(), n, back.data());
    for (size_t i = 0; i < N; ++i) {
        const Particle &p = ps[i], &q = back[i];
        for (int a = 0; a < 3; ++a)
            if (!same(p.pos[a], q.pos[a]) || !same(p.velocity[a], q.velocity[a])) return 2;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                if (!same(p.B[c][r], q.B[c][r]) || !same(p.FElastic[c][r], q.FElastic[c][r]) ||
                    !same(p.FPlastic[c][r], q.FPlastic[c][r]))
                    return 3;
        if (!same(p.mass, q.mass) || !same(p.volume, q.volume)) return 4;
    }
    return 0;
}

int main() {
    const int counts[] = {0, 1, 2147, 300001};
    for (int k = 0; k < 4; ++k) {
        const int r = check(counts[k]);
        if (r) {
            std::printf("mismatch %d at n = %d\n", r, counts[k]);
            return 10 * (k + 1) + r;
        }
    }
    std::printf("ok\n");
    return 0;
}
