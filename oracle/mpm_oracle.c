/*
 * CPU restatement of the reference's explicit APIC / MLS-MPM snow step
 * (brocbyte/realtime-deformations).  TEST INFRASTRUCTURE ONLY: this file is the
 * oracle that the CUDA path is checked against and the "port" CPU baseline; the
 * product never links or calls it.
 *
 * Compiled twice: -DORC_REAL=float gives the FP32 oracle, which follows the
 * reference's own arithmetic (FP32 state, the FP64 literals inside the B-spline,
 * glm's evaluation order for products, determinants and inverses);
 * -DORC_REAL=double gives the FP64 oracle for the FP64 build of the kernels.
 *
 * Parity is pinned by tests against the reference itself, built headless from
 * its sources (oracle/ref/build_ref.sh) and by the committed fixtures in
 * tests/golden/.  Deliberate departures, each documented where it happens:
 *   - the plastic split uses W clamp(S) Z^T for F_E = W S Z^T (the reference
 *     decomposes F_E^T and transposes U and V back, which scrambles F_E: see
 *     orc_update_F); the headless build's switch rd_ref_p4 = 1 gives the same;
 *   - the rotation R of F_E = R S comes from the same SVD instead of the
 *     Higham-Noferini iteration the reference vendors;
 *   - an optional sticky-wall boundary (bc = 1) the reference does not have.
 *
 * Matrices are row-major in the math sense: M[3*r + c] = M(r, c).  glm stores
 * m[c][r] = M(r, c); the comments give the reference's expressions.
 * The dense grid index is i*MJ*MK + j*MK + k (material_point_method.hpp:129-131).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL real;
#define ORC_IS_FLOAT (sizeof(real) == sizeof(float))
/* glm::exp on a float calls the C library's expf */
static real orc_exp(real x) { return ORC_IS_FLOAT ? (real)expf((float)x) : (real)exp((double)x); }

typedef struct orc_params {
    int mi, mj, mk;      /* MAX_I, MAX_J, MAX_K */
    double h;            /* WeightCalculator::h (material_point_method.cpp:17) */
    double dinv;         /* DpInverse diagonal (material_point_method.hpp:177) */
    double E, nu, xi;    /* material_point_method.cpp:237-238, .hpp:213 */
    double theta_c, theta_s; /* material_point_method.cpp:320 */
    double gravity[3];   /* material_point_method.cpp:260 */
    int bc;              /* 0: none (reference); 1: sticky walls, width bc_width */
    int bc_width;
    int lagged_c;        /* 1: F update uses B of the previous G2P (main.cpp:209-214) */
} orc_params;

typedef struct orc_state {
    int n;
    real *x, *v;         /* n x 3 */
    real *B;             /* n x 9, APIC B (C = B * DpInverse) */
    real *FE, *FP;       /* n x 9 */
    real *mass, *vol;    /* n */
} orc_state;

typedef struct orc_grid {
    real *mass;          /* cells */
    real *vel;           /* cells x 3 */
    real *force;         /* cells x 3 */
} orc_grid;

static size_t ncells(const orc_params* P) { return (size_t)P->mi * P->mj * P->mk; }
static size_t cidx(const orc_params* P, int i, int j, int k) {
    return ((size_t)i * P->mj + j) * P->mk + k;
}

/* WeightCalculator::weightNx (material_point_method.hpp:20-31): FP32 powers,
 * FP64 polynomial (the literals are double), rounded to FP32 on return. */
static real weight_nx(real x) {
    const real a = (real)fabs((double)x);
    const real a2 = a * a;
    const real a3 = a * a * a;
    if (a < 1.0) return (real)(0.5 * (double)a3 - (double)a2 + 2.0 / 3.0);
    if (a < 2.0) {
        const real t = (real)2 - a;
        return (real)((1.0 / 6.0) * (double)t * (double)t * (double)t);
    }
    return (real)0;
}

/* WeightCalculator::wipHost (material_point_method.hpp:53-58). */
static real wip(const orc_params* P, int i, int j, int k, const real* pos) {
    const real h = (real)P->h;
    const real xc = pos[0] / h - (real)i;
    const real yc = pos[1] / h - (real)j;
    const real zc = pos[2] / h - (real)k;
    return weight_nx(xc) * weight_nx(yc) * weight_nx(zc);
}

/* getParticleNeighs (material_point_method.cpp:80-93): ivec3(pos / h), i.e. a
 * component-wise FP32 divide truncated toward zero. */
static void base_cell(const orc_params* P, const real* pos, int* b) {
    const real h = (real)P->h;
    b[0] = (int)(pos[0] / h);
    b[1] = (int)(pos[1] / h);
    b[2] = (int)(pos[2] / h);
}

/* ---- 3x3 helpers in glm's evaluation order ------------------------------ */
static void mat_mul(real* R, const real* A, const real* B) {
    /* glm type_mat3x3.inl operator*(mat3, mat3): sum over k in order 0,1,2 */
    real T[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            T[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
    memcpy(R, T, sizeof T);
}
static void mat_vec(real* y, const real* A, const real* x) {
    real t[3];
    for (int r = 0; r < 3; ++r) t[r] = A[3 * r] * x[0] + A[3 * r + 1] * x[1] + A[3 * r + 2] * x[2];
    y[0] = t[0]; y[1] = t[1]; y[2] = t[2];
}
static real mat_det(const real* M) {
    /* glm compute_determinant<tmat3x3> in row-major terms */
    return +M[0] * (M[4] * M[8] - M[5] * M[7])
           - M[1] * (M[3] * M[8] - M[5] * M[6])
           + M[2] * (M[3] * M[7] - M[4] * M[6]);
}
static void mat_inv(real* R, const real* M) {
    /* glm compute_inverse<tmat3x3>: cofactors times 1/det */
    const real od = (real)1 / mat_det(M);
    real T[9];
    T[0] = +(M[4] * M[8] - M[5] * M[7]) * od;
    T[1] = -(M[1] * M[8] - M[2] * M[7]) * od;
    T[2] = +(M[1] * M[5] - M[2] * M[4]) * od;
    T[3] = -(M[3] * M[8] - M[5] * M[6]) * od;
    T[4] = +(M[0] * M[8] - M[2] * M[6]) * od;
    T[5] = -(M[0] * M[5] - M[2] * M[3]) * od;
    T[6] = +(M[3] * M[7] - M[4] * M[6]) * od;
    T[7] = -(M[0] * M[7] - M[1] * M[6]) * od;
    T[8] = +(M[0] * M[4] - M[1] * M[3]) * od;
    memcpy(R, T, sizeof T);
}
static void mat_transpose(real* R, const real* M) {
    real T[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) T[3 * c + r] = M[3 * r + c];
    memcpy(R, T, sizeof T);
}

/* ---- FP64 SVD (test oracle only) ---------------------------------------
 * F = W diag(s) Z^T with s >= 0 sorted descending, W and Z orthogonal (either
 * may be a reflection), the convention of Eigen's JacobiSVD that the reference
 * calls (material_point_method.cpp:312).  Method: cyclic Jacobi
 * eigen-decomposition of F^T F (Golub & Van Loan, Matrix Computations, 8.5),
 * Z = eigenvectors, W = F Z / s completed by Gram-Schmidt where s vanishes.
 * Deliberately a different algorithm from the one in the CUDA kernels. */
static void svd3_f64(const double* F, double* W, double* s, double* Z) {
    double A[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            A[3 * r + c] = F[r] * F[c] + F[3 + r] * F[3 + c] + F[6 + r] * F[6 + c];
    double V[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int sweep = 0; sweep < 60; ++sweep) {
        const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
        const double dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
        if (off <= 1e-34 * dia || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const double apq = A[3 * p + q];
                if (apq == 0.0) continue;
                const double theta = (A[3 * q + q] - A[3 * p + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; ++k) { /* A <- J^T A J, J rotates (p, q) */
                    const double akp = A[3 * k + p], akq = A[3 * k + q];
                    A[3 * k + p] = c * akp - sn * akq;
                    A[3 * k + q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    const double apk = A[3 * p + k], aqk = A[3 * q + k];
                    A[3 * p + k] = c * apk - sn * aqk;
                    A[3 * q + k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const double vkp = V[3 * k + p], vkq = V[3 * k + q];
                    V[3 * k + p] = c * vkp - sn * vkq;
                    V[3 * k + q] = sn * vkp + c * vkq;
                }
            }
    }
    double ev[3] = {A[0], A[4], A[8]};
    int ord[3] = {0, 1, 2};
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (ev[ord[b]] > ev[ord[a]]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Z[3 * r + c] = V[3 * r + ord[c]];
    /* W columns: F z_c / |F z_c|, orthogonalised against earlier columns. */
    for (int c = 0; c < 3; ++c) {
        double u[3];
        for (int r = 0; r < 3; ++r)
            u[r] = F[3 * r] * Z[c] + F[3 * r + 1] * Z[3 + c] + F[3 * r + 2] * Z[6 + c];
        double nrm = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        s[c] = nrm;
        for (int e = 0; e < c; ++e) {
            const double d = u[0] * W[e] + u[1] * W[3 + e] + u[2] * W[6 + e];
            for (int r = 0; r < 3; ++r) u[r] -= d * W[3 * r + e];
        }
        double n2 = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (n2 <= 1e-300 || nrm <= 1e-150) {
            /* complete the basis: the unit axis least aligned with earlier columns */
            int best = 0; double bestv = 1e300;
            for (int ax = 0; ax < 3; ++ax) {
                double m = 0;
                for (int e = 0; e < c; ++e) m += fabs(W[3 * ax + e]);
                if (m < bestv) { bestv = m; best = ax; }
            }
            u[0] = u[1] = u[2] = 0; u[best] = 1;
            for (int e = 0; e < c; ++e) {
                const double d = u[0] * W[e] + u[1] * W[3 + e] + u[2] * W[6 + e];
                for (int r = 0; r < 3; ++r) u[r] -= d * W[3 * r + e];
            }
            n2 = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        }
        for (int r = 0; r < 3; ++r) W[3 * r + c] = u[r] / n2;
    }
}

/* Rotation R of F = R S, computed as W D Z^T with D = diag(1, 1, det(W Z^T)) so
 * that R is a proper rotation like the reference's polar decomposition
 * (utils.h:55-75, polar_decomposition_3x3_impl.h:1355-1356). */
static void polar_rotation(real* R, const real* F) {
    double Fd[9], W[9], s[3], Z[9];
    for (int e = 0; e < 9; ++e) Fd[e] = (double)F[e];
    svd3_f64(Fd, W, s, Z);
    double Rd[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            Rd[3 * r + c] = W[3 * r] * Z[3 * c] + W[3 * r + 1] * Z[3 * c + 1] + W[3 * r + 2] * Z[3 * c + 2];
    const double d = Rd[0] * (Rd[4] * Rd[8] - Rd[5] * Rd[7]) - Rd[1] * (Rd[3] * Rd[8] - Rd[5] * Rd[6]) +
                     Rd[2] * (Rd[3] * Rd[7] - Rd[4] * Rd[6]);
    if (d < 0)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Rd[3 * r + c] -= 2.0 * W[3 * r + 2] * Z[3 * c + 2];
    for (int e = 0; e < 9; ++e) R[e] = (real)Rd[e];
}

/* ---- stages -------------------------------------------------------------- */

/* rasterizeParticlesToGrid (material_point_method.cpp:94-129): clear, mass
 * scatter over the 125-node stencil, APIC momentum scatter, v = (m v) / m on
 * cells with m != 0. */
void orc_rasterize(const orc_params* P, const orc_state* S, orc_grid* G) {
    const size_t nc = ncells(P);
    memset(G->mass, 0, nc * sizeof(real));
    memset(G->vel, 0, 3 * nc * sizeof(real));
    memset(G->force, 0, 3 * nc * sizeof(real));
    const real h = (real)P->h, dinv = (real)P->dinv;
    for (int p = 0; p < S->n; ++p) {
        const real* pos = S->x + 3 * p;
        int b[3];
        base_cell(P, pos, b);
        for (int dx = 0; dx <= 4; ++dx)
            for (int dy = 0; dy <= 4; ++dy)
                for (int dz = 0; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    G->mass[cidx(P, i, j, k)] += S->mass[p] * wip(P, i, j, k, pos);
                }
    }
    for (int p = 0; p < S->n; ++p) {
        const real* pos = S->x + 3 * p;
        real C[9];
        for (int e = 0; e < 9; ++e) C[e] = S->B[9 * p + e] * dinv; /* p.B * DpInverse */
        int b[3];
        base_cell(P, pos, b);
        for (int dx = 0; dx <= 4; ++dx)
            for (int dy = 0; dy <= 4; ++dy)
                for (int dz = 0; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    const real d[3] = {(real)i * h - pos[0], (real)j * h - pos[1], (real)k * h - pos[2]};
                    real cd[3];
                    mat_vec(cd, C, d);
                    const real s = wip(P, i, j, k, pos) * S->mass[p];
                    real* gv = G->vel + 3 * cidx(P, i, j, k);
                    for (int a = 0; a < 3; ++a) gv[a] += s * (S->v[3 * p + a] + cd[a]);
                }
    }
    for (size_t c = 0; c < nc; ++c)
        if (G->mass[c] != (real)0)
            for (int a = 0; a < 3; ++a) G->vel[3 * c + a] /= G->mass[c];
}

/* computeParticleVolumesAndDensities (material_point_method.cpp:131-142). */
void orc_volumes(const orc_params* P, orc_state* S, const orc_grid* G) {
    const real h = (real)P->h;
    for (int p = 0; p < S->n; ++p) {
        const real* pos = S->x + 3 * p;
        int b[3];
        base_cell(P, pos, b);
        real density = 0;
        for (int dx = 0; dx <= 4; ++dx)
            for (int dy = 0; dy <= 4; ++dy)
                for (int dz = 0; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    density += G->mass[cidx(P, i, j, k)] * wip(P, i, j, k, pos);
                }
        density /= (h * h * h);
        S->vol[p] = density != (real)0 ? (S->mass[p] / density) : (real)0;
    }
}

/* computeExplicitGridForces (material_point_method.cpp:235-254):
 * P = 2 mu (F - R) + lambda (J - 1) J F^-T with mu, lambda scaled by
 * exp(xi (1 - det F_P)); f_i -= V D^-1 P F^T w_ip (x_i - x_p). */
void orc_forces(const orc_params* P, const orc_state* S, orc_grid* G) {
    const real h = (real)P->h, dinv = (real)P->dinv;
    const real E = (real)P->E, nu = (real)P->nu, xi = (real)P->xi;
    const real mu0 = E / ((real)2 * ((real)1 + nu));
    const real lambda0 = (E * nu) / (((real)1 + nu) * ((real)1 - (real)2 * nu));
    for (int p = 0; p < S->n; ++p) {
        const real* pos = S->x + 3 * p;
        const real* F = S->FE + 9 * p;
        const real jp = mat_det(S->FP + 9 * p);
        const real hard = orc_exp(xi * ((real)1 - jp));
        const real mu = mu0 * hard, lambda = lambda0 * hard;
        real R[9], Finv[9], FinvT[9], Pm[9], FT[9], Gm[9];
        polar_rotation(R, F);
        const real J = mat_det(F);
        mat_inv(Finv, F);
        mat_transpose(FinvT, Finv);
        const real a = (real)2 * mu, bcoef = lambda * (J - (real)1) * J;
        for (int e = 0; e < 9; ++e) Pm[e] = a * (F[e] - R[e]) + bcoef * FinvT[e];
        /* (((V * DpInverse) * P) * F^T): DpInverse is diagonal */
        const real vd = S->vol[p] * dinv;
        for (int e = 0; e < 9; ++e) Gm[e] = vd * Pm[e];
        mat_transpose(FT, F);
        mat_mul(Gm, Gm, FT);
        int b[3];
        base_cell(P, pos, b);
        for (int dx = 0; dx <= 4; ++dx)
            for (int dy = 0; dy <= 4; ++dy)
                for (int dz = 0; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    const real w = wip(P, i, j, k, pos);
                    real Gw[9];
                    for (int e = 0; e < 9; ++e) Gw[e] = Gm[e] * w;
                    const real d[3] = {(real)i * h - pos[0], (real)j * h - pos[1], (real)k * h - pos[2]};
                    real fd[3];
                    mat_vec(fd, Gw, d);
                    real* gf = G->force + 3 * cidx(P, i, j, k);
                    for (int q = 0; q < 3; ++q) gf[q] -= fd[q];
                }
    }
}

/* gridVelocitiesUpdate (material_point_method.cpp:256-262) on cells with
 * m != 0, then the optional sticky walls (not in the reference). */
void orc_grid_velocities(const orc_params* P, real dt, orc_grid* G) {
    const real g[3] = {(real)P->gravity[0], (real)P->gravity[1], (real)P->gravity[2]};
    for (int i = 0; i < P->mi; ++i)
        for (int j = 0; j < P->mj; ++j)
            for (int k = 0; k < P->mk; ++k) {
                const size_t c = cidx(P, i, j, k);
                if (G->mass[c] == (real)0) continue;
                for (int a = 0; a < 3; ++a)
                    G->vel[3 * c + a] += dt * (G->force[3 * c + a] / G->mass[c] + g[a]);
                if (P->bc == 1) {
                    const int w = P->bc_width;
                    if (i < w || j < w || k < w || i >= P->mi - w || j >= P->mj - w || k >= P->mk - w)
                        G->vel[3 * c] = G->vel[3 * c + 1] = G->vel[3 * c + 2] = (real)0;
                }
            }
}

/* Box colliders of gridBasedCollisions (material_point_method.cpp:264-304),
 * the MeshCollider of material_point_method.hpp:74-93: per collider the
 * world-from-box rotation R (row-major), the centre t, the half extents s and
 * the velocity v.  Mode 0 follows the reference (finite-difference normal,
 * glm's vec3::length() = 3 in the friction law), mode 1 the Coulomb law with
 * the face normal. */
#define ORC_MAX_COLLIDERS 16
static int orc_ncol = 0, orc_col_mode = 0;
static double orc_mu = 0.5;
static double orc_cols[ORC_MAX_COLLIDERS][18]; /* R 9 | t 3 | s 3 | v 3 */

/* spec: per collider t (3), unit quaternion (w, x, y, z), s (3), v (3). */
void orc_set_colliders(int n, const double* spec, int mode, double mu) {
    orc_ncol = n < 0 ? 0 : (n > ORC_MAX_COLLIDERS ? ORC_MAX_COLLIDERS : n);
    orc_col_mode = mode;
    orc_mu = mu;
    for (int k = 0; k < orc_ncol; ++k) {
        const double* c = spec + 13 * k;
        double w = c[3], x = c[4], y = c[5], z = c[6];
        const double nn = sqrt(w * w + x * x + y * y + z * z);
        if (nn > 0) { w /= nn; x /= nn; y /= nn; z /= nn; }
        double* o = orc_cols[k];
        o[0] = 1 - 2 * (y * y + z * z); o[1] = 2 * (x * y - w * z);     o[2] = 2 * (x * z + w * y);
        o[3] = 2 * (x * y + w * z);     o[4] = 1 - 2 * (x * x + z * z); o[5] = 2 * (y * z - w * x);
        o[6] = 2 * (x * z - w * y);     o[7] = 2 * (y * z + w * x);     o[8] = 1 - 2 * (x * x + y * y);
        for (int a = 0; a < 3; ++a) { o[9 + a] = c[a]; o[12 + a] = c[7 + a]; o[15 + a] = c[10 + a]; }
    }
}

/* MeshCollider::move (material_point_method.hpp:89-91) */
void orc_move_colliders(double dt) {
    for (int k = 0; k < orc_ncol; ++k)
        for (int a = 0; a < 3; ++a) orc_cols[k][9 + a] += dt * orc_cols[k][15 + a];
}

/* MeshCollider::sdf: |max(q, 0)| + min(max(q), 0) with q = |R^T (x - t)| - s. */
static real box_sdf(const double* c, real x0, real x1, real x2) {
    const real d[3] = {x0 - (real)c[9], x1 - (real)c[10], x2 - (real)c[11]};
    real q[3];
    for (int a = 0; a < 3; ++a) {
        const real p = (real)c[a] * d[0] + (real)c[3 + a] * d[1] + (real)c[6 + a] * d[2];
        q[a] = (real)fabs((double)p) - (real)c[12 + a];
    }
    real qm = q[0];
    if (q[1] > qm) qm = q[1];
    if (q[2] > qm) qm = q[2];
    return (real)fabs((double)(qm > 0 ? qm : (real)0)) + (qm < 0 ? qm : (real)0);
}

/* gridBasedCollisions / bodyCollision on every node with mass. */
void orc_collisions(const orc_params* P, orc_grid* G) {
    if (!orc_ncol) return;
    const real h = (real)P->h, mu = (real)orc_mu;
    for (int i = 0; i < P->mi; ++i)
        for (int j = 0; j < P->mj; ++j)
            for (int k = 0; k < P->mk; ++k) {
                const size_t cc = cidx(P, i, j, k);
                if (G->mass[cc] == (real)0) continue;
                const real x[3] = {(real)i * h, (real)j * h, (real)k * h};
                real* v = G->vel + 3 * cc;
                for (int o = 0; o < orc_ncol; ++o) {
                    const double* c = orc_cols[o];
                    if (box_sdf(c, x[0], x[1], x[2]) > 0) continue;
                    real n[3];
                    if (orc_col_mode == 0) { /* gradient(phi, pos, 3), delta 0.001 (mathy.hpp:40-56) */
                        const real dl = (real)0.001f;
                        for (int a = 0; a < 3; ++a) {
                            real xp[3] = {x[0], x[1], x[2]}, xm[3] = {x[0], x[1], x[2]};
                            xp[a] += dl;
                            xm[a] -= dl;
                            n[a] = (box_sdf(c, xp[0], xp[1], xp[2]) - box_sdf(c, xm[0], xm[1], xm[2])) / ((real)2 * dl);
                        }
                    } else { /* outward normal of the face of largest q */
                        const real d[3] = {x[0] - (real)c[9], x[1] - (real)c[10], x[2] - (real)c[11]};
                        real p[3], q[3];
                        for (int a = 0; a < 3; ++a) {
                            p[a] = (real)c[a] * d[0] + (real)c[3 + a] * d[1] + (real)c[6 + a] * d[2];
                            q[a] = (real)fabs((double)p[a]) - (real)c[12 + a];
                        }
                        int f = 0;
                        if (q[1] > q[f]) f = 1;
                        if (q[2] > q[f]) f = 2;
                        const real sg = p[f] < 0 ? (real)-1 : (real)1;
                        for (int a = 0; a < 3; ++a) n[a] = sg * (real)c[3 * a + f];
                    }
                    const real rel[3] = {v[0] - (real)c[15], v[1] - (real)c[16], v[2] - (real)c[17]};
                    const real vn = rel[0] * n[0] + rel[1] * n[1] + rel[2] * n[2];
                    if (vn >= 0) continue;
                    const real vt[3] = {rel[0] - n[0] * vn, rel[1] - n[1] * vn, rel[2] - n[2] * vn};
                    const real len = orc_col_mode == 0 ? (real)3
                                                       : (real)sqrt((double)(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]));
                    real f = 0;
                    if (len > -mu * vn && len > 0) f = (real)1 + mu * vn / len;
                    for (int a = 0; a < 3; ++a) v[a] = vt[a] * f + (real)c[15 + a];
                }
            }
}

/* updateDeformationGradient (material_point_method.cpp:306-330):
 * Fhat = (I + dt B D^-1) F_E F_P; F_E* = Fhat F_P^-1 = W S Z^T;
 * F_E <- W clamp(S, 1 - theta_c, 1 + theta_s) Z^T; F_P <- F_E^-1 Fhat.
 * The reference converts glm -> Eigen transposing, so it decomposes F_E*^T =
 * U S V^T and sets F_E <- U^T clamp(S) V (utils.h:15-33); that is not a
 * function of F_E* alone.  Here, as with the headless build's rd_ref_p4 = 1,
 * F_E* itself is decomposed.  Both keep Fhat = F_E F_P and det F_P. */
void orc_update_F(const orc_params* P, real dt, orc_state* S) {
    const real dinv = (real)P->dinv;
    const real lo = (real)(1 - P->theta_c), hi = (real)(1 + P->theta_s);
    for (int p = 0; p < S->n; ++p) {
        real* FE = S->FE + 9 * p;
        real* FP = S->FP + 9 * p;
        real A[9], Fhat[9], FPinv[9], Fst[9];
        for (int e = 0; e < 9; ++e) A[e] = S->B[9 * p + e] * dinv * dt;
        A[0] += 1; A[4] += 1; A[8] += 1;
        mat_mul(Fhat, A, FE);
        mat_mul(Fhat, Fhat, FP);
        mat_inv(FPinv, FP);
        mat_mul(Fst, Fhat, FPinv);
        double Fd[9], W[9], s[3], Z[9];
        for (int e = 0; e < 9; ++e) Fd[e] = (double)Fst[e];
        svd3_f64(Fd, W, s, Z);
        real sc[3];
        for (int a = 0; a < 3; ++a) {
            real sv = (real)s[a];
            sc[a] = sv < lo ? lo : (sv > hi ? hi : sv);
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double acc = 0;
                for (int a = 0; a < 3; ++a) acc += W[3 * r + a] * (double)sc[a] * Z[3 * c + a];
                FE[3 * r + c] = (real)acc;
            }
        real FEinv[9];
        mat_inv(FEinv, FE);
        mat_mul(FP, FEinv, Fhat);
    }
}

/* updateParticleVelocities (material_point_method.cpp:332-342):
 * v_p = sum w v_i; B_p = sum w v_i (x_i - x_p)^T. */
void orc_g2p(const orc_params* P, orc_state* S, const orc_grid* G) {
    const real h = (real)P->h;
    for (int p = 0; p < S->n; ++p) {
        const real* pos = S->x + 3 * p;
        real vp[3] = {0, 0, 0}, Bp[9] = {0};
        int b[3];
        base_cell(P, pos, b);
        for (int dx = 0; dx <= 4; ++dx)
            for (int dy = 0; dy <= 4; ++dy)
                for (int dz = 0; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    const real* gv = G->vel + 3 * cidx(P, i, j, k);
                    const real w = wip(P, i, j, k, pos);
                    for (int a = 0; a < 3; ++a) vp[a] += gv[a] * w;
                    const real d[3] = {(real)i * h - pos[0], (real)j * h - pos[1], (real)k * h - pos[2]};
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) Bp[3 * r + c] += w * (gv[r] * d[c]);
                }
        memcpy(S->v + 3 * p, vp, sizeof vp);
        memcpy(S->B + 9 * p, Bp, sizeof Bp);
    }
}

/* updateParticlePositions + clampPosition (material_point_method.cpp:344-350,
 * 381-388): x += v dt, each axis clamped to [3h, (MAX - 3) h]. */
void orc_advect(const orc_params* P, real dt, orc_state* S) {
    const real h = (real)P->h;
    const real lo = (real)3 * h;
    const real hi[3] = {(real)(P->mi - 3) * h, (real)(P->mj - 3) * h, (real)(P->mk - 3) * h};
    for (int p = 0; p < S->n; ++p)
        for (int a = 0; a < 3; ++a) {
            real x = S->x[3 * p + a] + S->v[3 * p + a] * dt;
            x = x < lo ? lo : (x > hi[a] ? hi[a] : x);
            S->x[3 * p + a] = x;
        }
}

/* ---- implicit time integration (material_point_method.cpp:160-233) --------
 * Dead code in the reference (nothing calls timeIntegration), restated for the
 * GPU's rd_time_integration: the energy of the grid velocities v of the cells
 * with mass,
 *   E(v) = sum_i 1/2 m_i |v_i - v*_i|^2 + sum_p V_p Psi(Fhat_p(v), F_P,p),
 *   Fhat_p = (I + dt sum_i v_i grad w_ip^T) F_E,p,
 *   Psi = mu ||Fhat - R||^2 + lambda / 2 (J - 1)^2,  R = polar rotation of Fhat,
 * with v* the grid velocities at the call, and mu = mu0 h, lambda = lambda0 h
 * where, as the reference writes it (:194-199), h = exp(xi * 1 - det F_P)
 * (mode 0; mode 1 is the intended exp(xi (1 - det F_P))).  The reference's
 * own constants are mu0 = lambda0 = 1, xi = 10 (material_point_method.hpp:
 * 213-216).  The reference minimises E with LBFGS on finite differences; here
 * the gradient is analytic:
 *   dE/dv_i = m_i (v_i - v*_i) + dt sum_p V_p P_p F_E,p^T grad w_ip,
 *   P = 2 mu (Fhat - R) + lambda (J - 1) J Fhat^-T. */

/* WeightCalculator::weightNxDerivative (material_point_method.hpp:32-51): the
 * literals are double, the argument float. */
static real weight_nx_derivative(real x) {
    const real a = (real)fabs((double)x);
    const double xd = (double)x;
    if (a < 1.0f) {
        if (x >= 0) return (real)(3.0 / 2.0 * xd * xd - (double)((real)2 * x));
        return (real)(-3.0 / 2.0 * xd * xd - (double)((real)2 * x));
    }
    if (a < 2.0) {
        if (x >= 0) {
            const double t = (double)((real)2 - x);
            return (real)(-0.5 * t * t);
        }
        const double t = (double)((real)2 + x);
        return (real)(0.5 * t * t);
    }
    return (real)0;
}

/* WeightCalculator::wipGrad (material_point_method.hpp:59-70). */
static void wip_grad(const orc_params* P, int i, int j, int k, const real* pos, real* g) {
    const real h = (real)P->h;
    const real xc = (pos[0] - (real)i * h) / h;
    const real yc = (pos[1] - (real)j * h) / h;
    const real zc = (pos[2] - (real)k * h) / h;
    const real nx = weight_nx(xc), ny = weight_nx(yc), nz = weight_nx(zc);
    const double ih = 1.0 / (double)h;
    g[0] = (real)(ih * (double)weight_nx_derivative(xc) * (double)ny * (double)nz);
    g[1] = (real)(ih * (double)nx * (double)weight_nx_derivative(yc) * (double)nz);
    g[2] = (real)(ih * (double)nx * (double)ny * (double)weight_nx_derivative(zc));
}

/* The polar rotation R, the energy density and, when Pout is given, its
 * derivative P (ElasticPlasticEnergyDensity, material_point_method.cpp:
 * 192-210; fNorm2 sums in double). */
static real implicit_density(const real* F, real mu, real lambda, real* Pout) {
    real R[9];
    polar_rotation(R, F);
    double n2 = 0.0;
    for (int e = 0; e < 9; ++e) {
        const real d = F[e] - R[e];
        n2 += (double)(d * d);
    }
    const real J = mat_det(F);
    if (Pout) {
        /* (J - 1) J F^-T = (J - 1) cof(F) */
        const real cof[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                             F[2] * F[7] - F[1] * F[8], F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                             F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
        for (int e = 0; e < 9; ++e) Pout[e] = (real)2 * mu * (F[e] - R[e]) + lambda * (J - (real)1) * cof[e];
    }
    return mu * (real)n2 + lambda / (real)2 * (J - (real)1) * (J - (real)1);
}

/* Energy (material_point_method.cpp:160-173) at the dense velocity field vel
 * (cells x 3; only cells with mass count), ElasticPotential (:175-190) summed
 * in `real` over the particles in order; the gradient (dense, cells x 3, zero
 * where there is no mass) when grad is given.  G holds the masses and the
 * grid velocities v* of the call. */
double orc_implicit_energy(const orc_params* P, const orc_state* S, const orc_grid* G, real dt, double mu0,
                           double lambda0, double xi, int mode, const real* vel, real* grad) {
    const size_t nc = ncells(P);
    double kinetic = 0.0;
    if (grad) memset(grad, 0, 3 * nc * sizeof(real));
    for (size_t c = 0; c < nc; ++c) {
        if (G->mass[c] == (real)0) continue;
        const real d[3] = {vel[3 * c] - G->vel[3 * c], vel[3 * c + 1] - G->vel[3 * c + 1],
                           vel[3 * c + 2] - G->vel[3 * c + 2]};
        const real len = (real)sqrt((double)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
        kinetic += 0.5 * (double)G->mass[c] * (double)len * (double)len;
        if (grad)
            for (int a = 0; a < 3; ++a) grad[3 * c + a] = G->mass[c] * d[a];
    }
    real acc = 0;
    for (int p = 0; p < S->n; ++p) {
        const real* pos = S->x + 3 * p;
        real Fh[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        int b[3];
        base_cell(P, pos, b);
        /* the nodes with a non-zero weight gradient, in the reference's
         * (x-major) order of its used cells */
        for (int dx = 1; dx <= 4; ++dx)
            for (int dy = 1; dy <= 4; ++dy)
                for (int dz = 1; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    const size_t c = cidx(P, i, j, k);
                    if (G->mass[c] == (real)0) continue;
                    real g[3];
                    wip_grad(P, i, j, k, pos, g);
                    const real vd[3] = {vel[3 * c] * dt, vel[3 * c + 1] * dt, vel[3 * c + 2] * dt};
                    for (int r = 0; r < 3; ++r)
                        for (int q = 0; q < 3; ++q) Fh[3 * r + q] += vd[r] * g[q]; /* outerProduct(v dt, grad w) */
                }
        mat_mul(Fh, Fh, S->FE + 9 * p);
        const real jp = mat_det(S->FP + 9 * p);
        const real e = mode == 0 ? (real)xi * (real)1 - jp : (real)xi * ((real)1 - jp);
        const real hard = orc_exp(e);
        const real mu = (real)mu0 * hard, lambda = (real)lambda0 * hard;
        real Pm[9];
        acc += S->vol[p] * implicit_density(Fh, mu, lambda, grad ? Pm : NULL);
        if (!grad) continue;
        /* dt V P F_E^T, applied to each node's weight gradient */
        real FT[9], A[9];
        mat_transpose(FT, S->FE + 9 * p);
        mat_mul(A, Pm, FT);
        const real s = dt * S->vol[p];
        for (int e2 = 0; e2 < 9; ++e2) A[e2] *= s;
        for (int dx = 1; dx <= 4; ++dx)
            for (int dy = 1; dy <= 4; ++dy)
                for (int dz = 1; dz <= 4; ++dz) {
                    const int i = b[0] + dx - 2, j = b[1] + dy - 2, k = b[2] + dz - 2;
                    const size_t c = cidx(P, i, j, k);
                    if (G->mass[c] == (real)0) continue;
                    real g[3], Ag[3];
                    wip_grad(P, i, j, k, pos, g);
                    mat_vec(Ag, A, g);
                    for (int a = 0; a < 3; ++a) grad[3 * c + a] += Ag[a];
                }
    }
    return kinetic + (double)acc;
}

/* main.cpp:53-54 */
void orc_init(const orc_params* P, orc_state* S, orc_grid* G) {
    orc_rasterize(P, S, G);
    orc_volumes(P, S, G);
}

/* main.cpp:192-218 with the colliders of orc_set_colliders (none by default);
 * lagged_c = 0 swaps the F update after G2P (the textbook order). */
void orc_step(const orc_params* P, real dt, int nsteps, orc_state* S, orc_grid* G) {
    for (int s = 0; s < nsteps; ++s) {
        orc_rasterize(P, S, G);
        orc_forces(P, S, G);
        orc_grid_velocities(P, dt, G);
        orc_collisions(P, G);
        if (P->lagged_c) {
            orc_update_F(P, dt, S);
            orc_g2p(P, S, G);
        } else {
            orc_g2p(P, S, G);
            orc_update_F(P, dt, S);
        }
        orc_advect(P, dt, S);
    }
}

/* Exposed for the oracle's own tests. */
void orc_svd3(const double* F, double* W, double* s, double* Z) { svd3_f64(F, W, s, Z); }
real orc_weight(real x) { return weight_nx(x); }
