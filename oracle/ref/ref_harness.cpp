// Headless C harness around the reference's own MaterialPointMethod::
// LagrangeEulerView (material_point_method.hpp:174-233).  Test infrastructure:
// it drives the unmodified step methods in the order main.cpp:192-218 calls
// them, with the reference's own MeshCollider boxes (none unless set), and
// copies state in and out.
//
// Exchange layout: x, v are n x 3; B, FE, FP are n x 9 row-major in the math
// sense (M[3*r + c] = M(r, c)); glm stores m[c][r] = M(r, c) (column-major).
// Grid arrays are dense MAX_I*MAX_J*MAX_K in the reference's own index order
// i*MAX_J*MAX_K + j*MAX_K + k (material_point_method.hpp:129-131).
#include "material_point_method.hpp"
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

float rd_ref_E = 1.4e5f;
float rd_ref_nu = 0.2f;
float rd_ref_xi = 10.0f;
float rd_ref_gy = (float)-9.8;
double rd_ref_theta_c = 2.5f * 1e-2;
double rd_ref_theta_s = 5.0f * 1e-3;
int rd_ref_p4 = 0;

// cudaCalc.cuh symbols referenced by the (never called) precalculateWeights.
ftype devH;
void cuP2G(MaterialPointMethod::Particle*, MaterialPointMethod::Cell*, int, int, int, int, ftype*) {}
// mesh.hpp declares Mesh::draw without defining it outside the GL build.
void Mesh::draw() {}

using MaterialPointMethod::LagrangeEulerView;
using MaterialPointMethod::MeshCollider;

namespace {
// MeshCollider's sdf captures `this`: the objects live here (stable
// addresses) and the list passed to gridBasedCollisions holds copies whose
// sdf still reads these objects' meshes, as main.cpp's solidObjects does.
std::vector<std::unique_ptr<MeshCollider>> g_objects;
std::vector<MeshCollider> g_colliders;
glm::mat4 g_vp(1.0f);
}  // namespace

namespace {
inline void to_glm(glm::mat3& g, const float* m) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) g[c][r] = m[3 * r + c];
}
inline void from_glm(float* m, const glm::mat3& g) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) m[3 * r + c] = g[c][r];
}
}  // namespace

extern "C" {

void rdref_set_params(float E, float nu, float xi, float gy, double theta_c, double theta_s, int p4) {
    rd_ref_E = E;
    rd_ref_nu = nu;
    rd_ref_xi = xi;
    rd_ref_gy = gy;
    rd_ref_theta_c = theta_c;
    rd_ref_theta_s = theta_s;
    rd_ref_p4 = p4;
}

// h must be set before construction: DpInverse is initialised from it
// (material_point_method.hpp:177).
void* rdref_create(int mi, int mj, int mk, int n, float h) {
    MaterialPointMethod::WeightCalculator::h = h;
    auto* s = new LagrangeEulerView(mi, mj, mk, n);
    s->setLevel(Logger::LogLevel::ERROR);
    return s;
}

void rdref_destroy(void* p) { delete static_cast<LagrangeEulerView*>(p); }

float rdref_dp_inverse(void* p) { return static_cast<LagrangeEulerView*>(p)->DpInverse[0][0]; }

void rdref_set_particles(void* p, const float* x, const float* v, const float* mass,
                         const float* B, const float* FE, const float* FP, const float* vol) {
    auto* s = static_cast<LagrangeEulerView*>(p);
    auto* ps = s->getParticles();
    for (int i = 0; i < s->getNumParticles(); ++i) {
        auto& q = ps[i];
        q.pos = glm::vec3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        q.velocity = glm::vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        q.mass = mass[i];
        if (B) to_glm(q.B, B + 9 * i); else q.B = glm::mat3(0.0f);
        if (FE) to_glm(q.FElastic, FE + 9 * i); else q.FElastic = glm::mat3(1.0f);
        if (FP) to_glm(q.FPlastic, FP + 9 * i); else q.FPlastic = glm::mat3(1.0f);
        q.volume = vol ? vol[i] : 0.0f;
    }
}

void rdref_get_particles(void* p, float* x, float* v, float* B, float* FE, float* FP, float* vol) {
    auto* s = static_cast<LagrangeEulerView*>(p);
    const auto* ps = s->getParticles();
    for (int i = 0; i < s->getNumParticles(); ++i) {
        const auto& q = ps[i];
        for (int a = 0; a < 3; ++a) {
            if (x) x[3 * i + a] = q.pos[a];
            if (v) v[3 * i + a] = q.velocity[a];
        }
        if (B) from_glm(B + 9 * i, q.B);
        if (FE) from_glm(FE + 9 * i, q.FElastic);
        if (FP) from_glm(FP + 9 * i, q.FPlastic);
        if (vol) vol[i] = q.volume;
    }
}

void rdref_get_mass(void* p, float* mass) {
    auto* s = static_cast<LagrangeEulerView*>(p);
    const auto* ps = s->getParticles();
    for (int i = 0; i < s->getNumParticles(); ++i) mass[i] = ps[i].mass;
}

// Cell fields as the reference holds them at the time of the call.
void rdref_get_grid(void* p, float* mass, float* vel, float* force) {
    auto* s = static_cast<LagrangeEulerView*>(p);
    const size_t n = s->grid.grid.size();
    for (size_t c = 0; c < n; ++c) {
        const auto& cell = s->grid.grid[c];
        if (mass) mass[c] = cell.mass;
        for (int a = 0; a < 3; ++a) {
            if (vel) vel[3 * c + a] = cell.velocity[a];
            if (force) force[3 * c + a] = cell.force[a];
        }
    }
}

// Stage ids follow main.cpp:192-218; 0 = rasterize, 1 = forces, 2 = grid
// velocities, 3 = collisions (empty list), 4 = deformation gradient,
// 5 = particle velocities, 6 = positions, 7 = volumes (main.cpp:54).
void rdref_stage(void* p, int stage, float dt) {
    auto* s = static_cast<LagrangeEulerView*>(p);

    switch (stage) {
        case 0: s->rasterizeParticlesToGrid(); break;
        case 1: s->computeExplicitGridForces(); break;
        case 2: s->gridVelocitiesUpdate(dt); break;
        case 3: s->gridBasedCollisions(dt, g_colliders); break;
        case 4: s->updateDeformationGradient(dt); break;
        case 5: s->updateParticleVelocities(); break;
        case 6: s->updateParticlePositions(dt); break;
        case 7: s->computeParticleVolumesAndDensities(); break;
        default: break;
    }
}

// The reference's own particle initialiser (material_point_method.cpp:18-63):
// a jittered 8-per-cell sphere drawn with the C library's rand(); main.cpp:52
// runs it before seeding, i.e. with seed 1.
void rdref_initialize_particles(void* p, unsigned seed, float ox, float oy, float oz, float vx, float vy, float vz) {
    srand(seed);
    static_cast<LagrangeEulerView*>(p)->initializeParticles(glm::vec3(ox, oy, oz), glm::vec3(vx, vy, vz));
}

// Box colliders placed as main.cpp:119-160 places them: applyMatrix4(T R S)
// on a box mesh, with a velocity.  spec: 13 doubles per box, translation (3),
// rotation quaternion (w, x, y, z), scale (3), velocity (3).
void rdref_set_colliders(int n, const double* spec) {
    g_colliders.clear();
    g_objects.clear();
    for (int k = 0; k < n; ++k) {
        const double* c = spec + 13 * k;
        auto obj = std::make_unique<MeshCollider>(0u, g_vp, std::vector<GLfloat>{}, std::vector<GLfloat>{},
                                                  glm::vec3((float)c[10], (float)c[11], (float)c[12]));
        const glm::quat q((float)c[3], (float)c[4], (float)c[5], (float)c[6]);
        obj->mesh.applyMatrix4(glm::translate(glm::mat4(), glm::vec3((float)c[0], (float)c[1], (float)c[2])) *
                               glm::toMat4(q) *
                               glm::scale(glm::mat4(), glm::vec3((float)c[7], (float)c[8], (float)c[9])));
        g_objects.push_back(std::move(obj));
    }
    for (auto& o : g_objects) g_colliders.push_back(*o);
}

// main.cpp:188: box.move(delta) for every box.
void rdref_move_colliders(float dt) {
    for (auto& o : g_objects) o->move(dt);
}

// The reference's implicit energy (material_point_method.cpp:160-173, a
// private method made reachable by the build's P2 patch) at grid velocities
// given densely, cells x 3: the entries of its used cells, in their order,
// form the VectorXf it takes.
float rdref_energy(void* p, const float* vel, float dt) {
    auto* s = static_cast<LagrangeEulerView*>(p);
    Eigen::VectorXf v(s->used_cells.size() * 3);
    for (size_t u = 0; u < s->used_cells.size(); ++u) {
        const auto& c = s->used_cells[u];
        const size_t idx = ((size_t)c.x * s->MAX_J + c.y) * s->MAX_K + c.z;
        for (int a = 0; a < 3; ++a) v[3 * u + a] = vel[3 * idx + a];
    }
    return s->Energy(v, dt);
}

// timeIntegration (material_point_method.cpp:212-233): LBFGS over the used
// cells' velocities; the grid then holds the minimiser it found.
void rdref_time_integration(void* p, float dt) { static_cast<LagrangeEulerView*>(p)->timeIntegration(dt); }

// main.cpp:53-54
void rdref_init(void* p) {
    rdref_stage(p, 0, 0.0f);
    rdref_stage(p, 7, 0.0f);
}

// main.cpp:192-218, nsteps times.
void rdref_step(void* p, float dt, int nsteps) {
    for (int s = 0; s < nsteps; ++s)
        for (int st = 0; st <= 6; ++st) rdref_stage(p, st, dt);
}

}  // extern "C"
