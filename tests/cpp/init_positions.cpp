// Writes the reference's initial particle positions (initializeParticles,
// material_point_method.cpp:18-63, rand() seed 1 as main.cpp:52 runs it) as
// produced by the C++ drop-in header, for comparison with the reference's own.
#include <cstdio>
#include <cstdlib>
#include "rd_lagrange_euler_view.hpp"
int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::vector<MaterialPointMethod::Particle> ps(2147);
    std::srand(1);
    const int more = MaterialPointMethod::reference_initial_particles(0.05f, {0.5f, 0.6f, 0.5f}, {0.f, -200.f, 0.f}, ps);
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    for (auto& p : ps) {
        const float v[4] = {p.pos.x, p.pos.y, p.pos.z, p.mass};
        std::fwrite(v, sizeof(float), 4, f);
    }
    std::fclose(f);
    std::printf("%d\n", more);
    return 0;
}
