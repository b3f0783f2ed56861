/* Switches that the patched reference reads (oracle/ref/build_ref.sh, patches
 * P3 and P4).  Defaults reproduce the reference's hard-coded values exactly:
 *   E, nu        material_point_method.cpp:237-238
 *   xi           material_point_method.hpp:213
 *   gravity y    material_point_method.cpp:260
 *   theta_c/s    material_point_method.cpp:320 (kept as double, as there)
 * rd_ref_p4 = 0 keeps the reference's transposing glm<->Eigen conversion
 * around the plastic SVD (utils.h:15-33, material_point_method.cpp:311-326);
 * rd_ref_p4 = 1 decomposes F_E itself, so F_E <- W clamp(S) Z^T. */
#pragma once
#include <glm/glm.hpp>
#include <Eigen/Dense>
extern float rd_ref_E, rd_ref_nu, rd_ref_xi, rd_ref_gy;
extern double rd_ref_theta_c, rd_ref_theta_s;
extern int rd_ref_p4;
inline Eigen::MatrixXf rd_ref_toEigen(const glm::mat3& mat) {
    Eigen::MatrixXf m{ 3, 3 };
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) {
            if (rd_ref_p4) m(r, c) = mat[c][r];   // math orientation
            else m(c, r) = mat[c][r];             // utils.h:15-23 (transposes)
        }
    return m;
}
inline glm::mat3 rd_ref_toGlm(const Eigen::MatrixXf& mat) {
    glm::mat3 m;
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) {
            if (rd_ref_p4) m[c][r] = mat(r, c);
            else m[c][r] = mat(c, r);             // utils.h:25-33 (transposes)
        }
    return m;
}
