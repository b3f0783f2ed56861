// A headless copy of the reference's driver sequence (main.cpp:48-54 and one
// pass of main.cpp:192-218 with dt = 1e-5 and no colliders) over the C++
// drop-in header; writes x, v, B, F_E, F_P (row-major) and volume per particle.
// argv[2] = "stages" runs the seven stage calls, "fused" calls step(dt);
// argv[3] = "info" lowers the log level to INFO after main.cpp's own setLevel.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "rd_lagrange_euler_view.hpp"
#if !__has_include(<glm/glm.hpp>)
namespace glm {
using vec3 = rd_facade::vec3;  // glm is not on this driver's include path
}
#endif
int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const bool fused = std::strcmp(argv[2], "fused") == 0;
    MaterialPointMethod::WeightCalculator::h = 0.05f;
    std::srand(1);
    // main.cpp:48-54, line for line
    const auto numParticles = 270 + 1877;
    const glm::vec3 particlesOrigin(0.5f, 0.6f, 0.5f);
    MaterialPointMethod::LagrangeEulerView MPM{ 20, 20, 20, numParticles };
    MPM.setLevel(MaterialPointMethod::DEFAULT_LOG_LEVEL_MPM);
    if (argc > 3 && std::strcmp(argv[3], "info") == 0) MPM.setLevel(Logger::LogLevel::INFO);
    MPM.initializeParticles(particlesOrigin, { 0.0f, -200.0f, 0.0f });
    MPM.rasterizeParticlesToGrid();
    MPM.computeParticleVolumesAndDensities();
    const float delta = 1e-5f;
    // the shape of the reference's MeshCollider (mesh transform + velocity);
    // this scene has none, as the golden fixture was made without them
    struct Box {
        struct {
            float translation[3], scale[3];
            struct { float w, x, y, z; } rotation;
        } mesh;
        float velocity[3];
    };
    const std::vector<Box> solidObjects;
    if (fused) {
        MPM.step(delta);
    } else {
        MPM.rasterizeParticlesToGrid();
        MPM.computeExplicitGridForces();
        MPM.gridVelocitiesUpdate(delta);
        MPM.gridBasedCollisions(delta, solidObjects);
        MPM.updateDeformationGradient(delta);
        MPM.updateParticleVelocities();
        MPM.updateParticlePositions(delta);
    }
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 3;
    const MaterialPointMethod::Particle* ps = MPM.getParticles();
    for (int i = 0; i < MPM.getNumParticles(); ++i) {
        const auto& p = ps[i];
        float rec[3 + 3 + 27 + 1];
        for (int a = 0; a < 3; ++a) { rec[a] = p.pos[a]; rec[3 + a] = p.velocity[a]; }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                rec[6 + 3 * r + c] = p.B[c][r];
                rec[15 + 3 * r + c] = p.FElastic[c][r];
                rec[24 + 3 * r + c] = p.FPlastic[c][r];
            }
        rec[33] = p.volume;
        std::fwrite(rec, sizeof(float), 34, f);
    }
    std::fclose(f);
    // the drop-in's exchange arrays are page-locked: no byte went through staging
    uint64_t in_place = 0, staged = 0;
    if (rd_io_bytes(MPM.handle(), &in_place, &staged) != RD_OK || staged != 0 || in_place == 0) return 4;
    return 0;
}
