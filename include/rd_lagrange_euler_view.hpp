// rd_lagrange_euler_view.hpp - C++ drop-in for the simulation class of
// brocbyte/realtime-deformations, MaterialPointMethod::LagrangeEulerView
// (realtime-deformations/material_point_method.hpp:174-233), implemented over
// the C ABI of rd_mpm.h.  Header only; link against librd_mpm.so.
//
// A main.cpp-style driver keeps its calls (main.cpp:48-54,192-218):
//
//     MaterialPointMethod::WeightCalculator::h = 0.05f;      // before construction
//     MaterialPointMethod::LagrangeEulerView MPM{20, 20, 20, 2147};
//     MPM.initializeParticles({0.5f, 0.6f, 0.5f}, {0.0f, -200.0f, 0.0f});
//     MPM.rasterizeParticlesToGrid();
//     MPM.computeParticleVolumesAndDensities();
//     for (;;) { MPM.rasterizeParticlesToGrid(); ...; MPM.updateParticlePositions(dt); }
//
// or replaces the seven stage calls by MPM.step(dt), the fused path.
// getParticles() returns a host array of Particle synchronised from the device
// on each call; writes through it reach the device only through
// syncParticlesToDevice().  Errors throw rd::Error (a std::runtime_error).
//
// With glm on the include path the vector and matrix members are glm::vec3 and
// glm::mat3 as in the reference (material_point_method.hpp:96-110); otherwise
// small stand-ins with the same member access (x/y/z, m[col][row]) are used.
//
// Logging follows the reference's Logger / Loggable (logger.hpp:7-43): the
// class derives from Loggable, so MPM.setLevel(MaterialPointMethod::
// DEFAULT_LOG_LEVEL_MPM) (main.cpp:51) compiles unchanged, and the stage calls
// print the reference's diagnostics at its levels (see LagrangeEulerView).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "rd_mpm.h"

#if defined(RD_WITH_GLM) || __has_include(<glm/glm.hpp>)
#include <glm/glm.hpp>
namespace rd_facade {
using vec3 = glm::vec3;
using mat3 = glm::mat3;
}  // namespace rd_facade
#else
namespace rd_facade {
struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct mat3 {  // column-major like glm: m[col][row]
    vec3 c[3];
    explicit mat3(float d = 1.0f) { c[0] = {d, 0, 0}; c[1] = {0, d, 0}; c[2] = {0, 0, d}; }
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
}  // namespace rd_facade
#endif

// logger.hpp:7-33: messages at or above the level go to std::cout, one per
// line; "<name> is: <value>" with std::to_string for numbers, vectors as
// "x y z" and matrices as three lines, one per glm column.
class Logger {
public:
    enum class LogLevel { INFO, WARNING, ERROR };
    void log(LogLevel level, const std::string& iMessage) {
        if (level >= level_) std::cout << iMessage << "\n";
    }
    void log(LogLevel level, const std::string& iName, float iValue) {
        log(level, iName + " is: " + std::to_string(iValue));
    }
    void log(LogLevel level, const std::string& iName, int iValue) {
        log(level, iName + " is: " + std::to_string(iValue));
    }
    void log(LogLevel level, const std::string& iName, const rd_facade::vec3& v) {
        log(level, iName + " is: " + std::to_string(v[0]) + " " + std::to_string(v[1]) + " " + std::to_string(v[2]));
    }
    void log(LogLevel level, const std::string& iName, const rd_facade::mat3& m) {
        std::string s;
        for (int c = 0; c < 3; ++c) {
            if (c) s += "\n";
            for (int r = 0; r < 3; ++r) s += (r ? " " : "") + std::to_string(m[c][r]);
        }
        log(level, iName + " is: " + s);
    }
    void setLevel(LogLevel level) { level_ = level; }
    // Whether a message at `level` would be printed (lets a caller skip the
    // work of computing a value nobody sees).
    bool enabled(LogLevel level) const { return level >= level_; }

private:
    LogLevel level_ = LogLevel::INFO;
};

// logger.hpp:36-43.
class Loggable {
public:
    void setLevel(Logger::LogLevel level) { logger.setLevel(level); }

protected:
    Logger logger;
};

namespace rd {
struct Error : std::runtime_error {
    rd_status status;
    Error(rd_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};
}  // namespace rd

namespace MaterialPointMethod {

// material_point_method.hpp:15-16.
const auto DEFAULT_LOG_LEVEL_OPTIMIZER = Logger::LogLevel::WARNING;
const auto DEFAULT_LOG_LEVEL_MPM = Logger::LogLevel::WARNING;

namespace WeightCalculator {
// The reference's global cell size (material_point_method.cpp:17); read when a
// LagrangeEulerView is constructed.
inline float h = 0.05f;
}  // namespace WeightCalculator

// material_point_method.hpp:96-110 without the per-step neighbour list.
struct Particle {
    float mass = 0;
    rd_facade::vec3 velocity;
    float volume = 0;
    rd_facade::vec3 pos;
    rd_facade::mat3 FElastic{1.0f};
    rd_facade::mat3 FPlastic{1.0f};
    rd_facade::mat3 B{0.0f};
    unsigned char r = 255, g = 255, b = 255, a = 255;  // colour (viewer only)
    float size = 0.02f;
};

// material_point_method.cpp:18-63 with utils.h:110-127: 8 quarter-offset
// points per cell of a cube around the origin, each jittered inside a ball of
// a quarter cell drawn with the C library's rand(), kept within 0.2 of the
// origin, mass 6e-5, filled from the last particle down; accepted points also
// draw three colour values.  The types follow the reference's (randFloat
// returns float, cos theta is double) so the same rand() sequence gives the
// same positions.  Returns how many accepted points did not fit.
inline int reference_initial_particles(float h, const rd_facade::vec3& origin, const rd_facade::vec3& velocity,
                                       std::vector<Particle>& particles) {
    const float width = 0.2f;
    const int cx = static_cast<int>(origin.x / h), cy = static_cast<int>(origin.y / h),
              cz = static_cast<int>(origin.z / h);
    const int wic = static_cast<int>(width / h);
    static const float ds[8][3] = {{1, 1, 1}, {1, 1, 3}, {1, 3, 1}, {1, 3, 3},
                                   {3, 1, 1}, {3, 1, 3}, {3, 3, 1}, {3, 3, 3}};
    int left = static_cast<int>(particles.size()), need_more = 0;
    auto rand_float = [](float lo, float hi) -> float { return lo + (std::rand() % 2000) / 2000.0 * (hi - lo); };
    for (int i = cx - wic; i < cx + wic; ++i)
        for (int j = cy - wic; j < cy + wic; ++j)
            for (int k = cz - wic; k < cz + wic; ++k)
                for (int d = 0; d < 8; ++d) {
                    const float phi = rand_float(0.0f, 2.0 * 3.1415);
                    const double costheta = rand_float(0.0, 2.0) - 1.0;
                    const float u = rand_float(0.0, 1.0);
                    const double theta = std::acos(costheta);
                    const float r = 0.25f * std::cbrt(u);
                    const float jx = r * std::sin(theta) * std::cos((double)phi);
                    const float jy = r * std::sin(theta) * std::sin((double)phi);
                    const float jz = r * std::cos(theta);
                    const float px = (i + ds[d][0] * (1 / 4.0f) + jx) * h;
                    const float py = (j + ds[d][1] * (1 / 4.0f) + jy) * h;
                    const float pz = (k + ds[d][2] * (1 / 4.0f) + jz) * h;
                    const float dx = px - origin.x, dy = py - origin.y, dz = pz - origin.z;
                    if (std::sqrt(dx * dx + dy * dy + dz * dz) > width) continue;
                    if (!left) { ++need_more; continue; }
                    Particle& p = particles[--left];
                    p.pos = rd_facade::vec3(px, py, pz);
                    p.velocity = velocity;
                    for (int c = 0; c < 3; ++c) (void)std::rand();  // colour draws, overwritten with white
                    p.mass = 0.00006f;
                }
    return need_more;
}

namespace detail {
// f(begin, end) over [0, n): in one call for small n, else split over the
// host's cores (at least 32,768 particles a thread).
template <typename F>
inline void parallel_ranges(int n, F&& f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = static_cast<int>(std::min<unsigned>(hw, static_cast<unsigned>(std::max(1, n / 32768))));
    if (nt <= 1) {
        f(0, n);
        return;
    }
    const int per = (n + nt - 1) / nt;
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    int next = 1;  // first range not handed to a thread
    try {
        for (; next < nt; ++next) {
            const int b = next * per, e = std::min(n, b + per);
            if (b < e) pool.emplace_back([&f, b, e] { f(b, e); });
        }
    } catch (const std::system_error&) {
        // no more threads could be started: the ranges from `next` on run on
        // this thread below, after the ones already running are joined
    }
    f(0, std::min(n, per));
    for (auto& t : pool) t.join();
    for (; next < nt; ++next) {
        const int b = next * per, e = std::min(n, b + per);
        if (b < e) f(b, e);
    }
}

// The exchange arrays of rd_set_particles / rd_get_particles, structure of
// arrays of n particles: x 3n | v 3n | B 9n | FE 9n | FP 9n | mass n | vol n
// (| Jp n, filled by the library); matrices row-major, glm's m[col][row].
inline size_t soa_offset(int k, int n) {
    static const size_t off[] = {0, 3, 6, 15, 24, 33, 34, 35};
    return off[k] * static_cast<size_t>(n);
}

inline void particles_to_soa(const Particle* ps, int n, float* soa) {
    parallel_ranges(n, [=](int b, int e) {
        float *x = soa + soa_offset(0, n), *v = soa + soa_offset(1, n), *B = soa + soa_offset(2, n),
              *FE = soa + soa_offset(3, n), *FP = soa + soa_offset(4, n), *m = soa + soa_offset(5, n),
              *vol = soa + soa_offset(6, n);
        for (int i = b; i < e; ++i) {
            const Particle& p = ps[i];
            for (int a = 0; a < 3; ++a) { x[3 * i + a] = p.pos[a]; v[3 * i + a] = p.velocity[a]; }
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    B[9 * i + 3 * r + c] = p.B[c][r];
                    FE[9 * i + 3 * r + c] = p.FElastic[c][r];
                    FP[9 * i + 3 * r + c] = p.FPlastic[c][r];
                }
            m[i] = p.mass;
            vol[i] = p.volume;
        }
    });
}

inline void soa_to_particles(const float* soa, int n, Particle* ps) {
    parallel_ranges(n, [=](int b, int e) {
        const float *x = soa + soa_offset(0, n), *v = soa + soa_offset(1, n), *B = soa + soa_offset(2, n),
                    *FE = soa + soa_offset(3, n), *FP = soa + soa_offset(4, n), *m = soa + soa_offset(5, n),
                    *vol = soa + soa_offset(6, n);
        for (int i = b; i < e; ++i) {
            Particle& p = ps[i];
            for (int a = 0; a < 3; ++a) { p.pos[a] = x[3 * i + a]; p.velocity[a] = v[3 * i + a]; }
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    p.B[c][r] = B[9 * i + 3 * r + c];
                    p.FElastic[c][r] = FE[9 * i + 3 * r + c];
                    p.FPlastic[c][r] = FP[9 * i + 3 * r + c];
                }
            p.mass = m[i];
            p.volume = vol[i];
        }
    });
}
}  // namespace detail

// Logging (Loggable, material_point_method.hpp:174): at INFO the stage calls
// print what the reference's print - initializeParticles the particle momentum
// and the average particles per occupied cell (material_point_method.cpp:61-62),
// rasterizeParticlesToGrid the particle and grid momentum (:122-125),
// computeParticleVolumesAndDensities the average cell and particle densities
// (:140-141), updateDeformationGradient the average of F_E F_P (:329) - and at
// WARNING (the default level, DEFAULT_LOG_LEVEL_MPM) rasterizeParticlesToGrid
// warns when the two momenta differ by more than 1% (:126-128).  The values come
// from device reductions (rd_get_diagnostics), which wait for the stream, so
// they are computed only at a level that prints them: setLevel(ERROR) skips all
// of it.  The reference's per-particle "SVD Singular" line (:318) is not
// printed.  step() logs nothing.
class LagrangeEulerView : public Loggable {
public:
    const int MAX_I, MAX_J, MAX_K;

    // material_point_method.cpp:144-154.  Extra parameters are optional and
    // default to the reference's constants.
    LagrangeEulerView(int max_i, int max_j, int max_k, int particlesNum, const rd_params* extra = nullptr)
        : MAX_I(max_i), MAX_J(max_j), MAX_K(max_k), n_(particlesNum), particles_(particlesNum) {
        rd_params p;
        if (extra) p = *extra; else rd_default_params(&p);
        p.max_i = max_i; p.max_j = max_j; p.max_k = max_k; p.num_particles = particlesNum;
        p.h = WeightCalculator::h;
        p.track_fp = 1;
        h_ = p.h;
        check(rd_create(&p, &sim_), "rd_create");
        // page-locked, so rd_set_particles / rd_get_particles move it in place
        void* buf = nullptr;
        const rd_status s = rd_host_alloc(static_cast<size_t>(n_) * 36 * sizeof(float), &buf);
        if (s != RD_OK) {
            rd_destroy(sim_);
            sim_ = nullptr;
            throw rd::Error(s, "rd_host_alloc: page-locked exchange arrays");
        }
        host_ = static_cast<float*>(buf);
    }
    ~LagrangeEulerView() {
        if (sim_) rd_destroy(sim_);
        rd_host_free(host_);
    }
    LagrangeEulerView(const LagrangeEulerView&) = delete;
    LagrangeEulerView& operator=(const LagrangeEulerView&) = delete;

    int getNumParticles() const { return n_; }

    // The reference's initialiser (see reference_initial_particles), then upload.
    void initializeParticles(const rd_facade::vec3& origin, const rd_facade::vec3& velocity) {
        reference_initial_particles(h_, origin, velocity, particles_);
        syncParticlesToDevice();
        if (logger.enabled(Logger::LogLevel::INFO)) {
            rd_diagnostics d = diagnostics();
            logger.log(Logger::LogLevel::INFO, "Particles momentum", vec(d.particle_momentum));
            logger.log(Logger::LogLevel::INFO, "Average PPC", averagePPC());
        }
    }

    // Returns the host copy, synchronised from the device (material_point_method.hpp:181-183).
    Particle* getParticles() {
        if (dirty_host_) download();
        return particles_.data();
    }
    // Uploads the host copy after the caller changed particles through getParticles().
    void syncParticlesToDevice() { upload(); }

    void rasterizeParticlesToGrid() {
        stage(RD_STAGE_RASTERIZE, 0.0);
        if (logger.enabled(Logger::LogLevel::WARNING)) {
            const rd_diagnostics d = diagnostics();
            logger.log(Logger::LogLevel::INFO, "ParticlesMomentum", vec(d.particle_momentum));
            logger.log(Logger::LogLevel::INFO, "GridMomentum", vec(d.grid_momentum));
            double diff = 0, gn = 0;
            for (int a = 0; a < 3; ++a) {
                diff += (d.particle_momentum[a] - d.grid_momentum[a]) * (d.particle_momentum[a] - d.grid_momentum[a]);
                gn += d.grid_momentum[a] * d.grid_momentum[a];
            }
            if (std::sqrt(diff) / std::sqrt(gn) > 1e-2)  // NaN (no grid momentum) does not warn, as in the reference
                logger.log(Logger::LogLevel::WARNING, "GridMomentum != ParticlesMomentum after rasterization");
        }
    }
    void computeParticleVolumesAndDensities() {
        stage(RD_STAGE_VOLUMES, 0.0);
        if (logger.enabled(Logger::LogLevel::INFO)) {
            const rd_diagnostics d = diagnostics();
            const double cell = static_cast<double>(h_) * h_ * h_;
            logger.log(Logger::LogLevel::INFO, "Average cell density",
                       static_cast<float>(d.grid_mass / static_cast<double>(d.used_cells) / cell));
            logger.log(Logger::LogLevel::INFO, "Average particle density",
                       static_cast<float>(d.average_particle_density));
        }
    }
    void computeExplicitGridForces() { stage(RD_STAGE_FORCES, 0.0); }
    void gridVelocitiesUpdate(float timeDelta) { stage(RD_STAGE_GRID_VELOCITIES, timeDelta); }
    // material_point_method.cpp:264-304.  The colliders are the reference's
    // MeshColliders (or anything with mesh.translation, mesh.rotation (w, x, y, z),
    // mesh.scale and velocity); they are uploaded when they changed since the
    // last call, and rd_step applies the last set too.
    template <typename Colliders>
    void gridBasedCollisions(float timeDelta, const Colliders& objects) {
        std::vector<rd_collider> cs;
        for (const auto& o : objects) {
            rd_collider c{};
            for (int a = 0; a < 3; ++a) {
                c.translation[a] = o.mesh.translation[a];
                c.scale[a] = o.mesh.scale[a];
                c.velocity[a] = o.velocity[a];
            }
            c.rotation[0] = o.mesh.rotation.w; c.rotation[1] = o.mesh.rotation.x;
            c.rotation[2] = o.mesh.rotation.y; c.rotation[3] = o.mesh.rotation.z;
            cs.push_back(c);
        }
        if (cs.size() != colliders_.size() ||
            (!cs.empty() && std::memcmp(cs.data(), colliders_.data(), cs.size() * sizeof(rd_collider)) != 0)) {
            check(rd_set_colliders(sim_, cs.data(), static_cast<int32_t>(cs.size()), RD_COLLIDE_REFERENCE, 0.5),
                  "rd_set_colliders");
            colliders_ = cs;
        }
        stage(RD_STAGE_COLLISIONS, timeDelta);
    }
    // material_point_method.cpp:212-233 (rd_time_integration): the grid
    // velocities become the minimiser of the reference's implicit energy, with
    // its L-BFGS settings unless opts says otherwise.
    rd_implicit_result timeIntegration(float timeDelta, const rd_implicit_opts* opts = nullptr) {
        rd_implicit_result r{};
        check(rd_time_integration(sim_, timeDelta, opts, &r), "rd_time_integration");
        return r;
    }
    void updateDeformationGradient(float timeDelta) {
        stage(RD_STAGE_DEFORMATION, timeDelta);
        if (logger.enabled(Logger::LogLevel::INFO)) {
            const rd_diagnostics d = diagnostics();
            rd_facade::mat3 m(0.0f);
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) m[c][r] = static_cast<float>(d.average_deformation_gradient[3 * r + c]);
            logger.log(Logger::LogLevel::INFO, "Average deformation gradient", m);
        }
    }
    void updateParticleVelocities() { stage(RD_STAGE_PARTICLE_VELOCITIES, 0.0); }
    void updateParticlePositions(float timeDelta) { stage(RD_STAGE_POSITIONS, timeDelta); }

    // The seven stage calls of main.cpp:192-218, fused (rd_step).
    void step(float timeDelta, int nsteps = 1) {
        check(rd_step(sim_, timeDelta, nsteps), "rd_step");
        dirty_host_ = true;
    }

    rd_handle* handle() { return sim_; }

private:
    void check(rd_status s, const char* what) {
        if (s == RD_OK) return;
        char buf[256] = {0};
        if (sim_) rd_last_error(sim_, buf, sizeof buf);
        throw rd::Error(s, std::string(what) + ": " + buf);
    }
    void stage(int id, double dt) {
        check(rd_stage(sim_, id, dt), "rd_stage");
        dirty_host_ = true;
    }
    rd_diagnostics diagnostics() {
        rd_diagnostics d;
        check(rd_get_diagnostics(sim_, 0, &d), "rd_get_diagnostics");
        return d;
    }
    static rd_facade::vec3 vec(const double* v) {
        return rd_facade::vec3(static_cast<float>(v[0]), static_cast<float>(v[1]), static_cast<float>(v[2]));
    }
    // averagePPC (material_point_method.cpp:396-414): particles per cell
    // ivec3(pos / h), averaged over the cells holding any, from the host copy.
    float averagePPC() {
        const Particle* ps = getParticles();
        std::vector<int> cnt(static_cast<size_t>(MAX_I) * MAX_J * MAX_K, 0);
        for (int i = 0; i < n_; ++i) {
            const int a = static_cast<int>(ps[i].pos[0] / h_), b = static_cast<int>(ps[i].pos[1] / h_),
                      c = static_cast<int>(ps[i].pos[2] / h_);
            if (a < 0 || b < 0 || c < 0 || a >= MAX_I || b >= MAX_J || c >= MAX_K) continue;
            ++cnt[(static_cast<size_t>(a) * MAX_J + b) * MAX_K + c];
        }
        long sum = 0, occupied = 0;
        for (int v : cnt)
            if (v > 0) { sum += v; ++occupied; }
        return static_cast<float>(sum) / static_cast<float>(occupied);
    }
    // host_ holds the exchange arrays (detail::soa_offset)
    float* soa(int k) { return host_ + detail::soa_offset(k, n_); }
    rd_particles views() {
        rd_particles v;
        v.x = soa(0); v.v = soa(1); v.B = soa(2); v.FE = soa(3); v.FP = soa(4); v.mass = soa(5);
        v.volume = soa(6); v.Jp = soa(7);
        return v;
    }
    void upload() {
        detail::particles_to_soa(particles_.data(), n_, host_);
        rd_particles v = views();
        v.Jp = nullptr;  // det F_P from FP
        check(rd_set_particles(sim_, &v, RD_HOST), "rd_set_particles");
        dirty_host_ = false;
    }
    void download() {
        rd_particles v = views();
        check(rd_get_particles(sim_, &v, RD_HOST), "rd_get_particles");
        detail::soa_to_particles(host_, n_, particles_.data());
        dirty_host_ = false;
    }

    int n_;
    float h_ = 0.05f;
    rd_handle* sim_ = nullptr;
    std::vector<Particle> particles_;
    float* host_ = nullptr;  // page-locked (rd_host_alloc), 36 n floats
    std::vector<rd_collider> colliders_;
    bool dirty_host_ = false;
};

}  // namespace MaterialPointMethod
