"""The fused step's stress without an SVD (stress_direct, inside_clamp in
rd_kernels.cuh), checked on the CPU as mathematics: the same series, summed
through the same Cayley-Hamilton recurrences in float64, against the SVD form
the reference's fixed-corotated stress takes (material_point_method.cpp:
235-254: 2 mu (F - R) F^T + lambda (J - 1) J I), and the positive-definiteness
test against the singular values it stands for.  The GPU path itself is
checked against the oracle in tests/test_gpu_parity.py."""
import numpy as np

Q = [0.0, 1 / 2, -3 / 8, 5 / 16, -35 / 128, 63 / 256, -231 / 1024, 429 / 2048]


def strain_of(F):
    G = F - np.eye(3)
    S = G + G.T + G.T @ G
    jm1 = np.trace(G) + (G[0, 0] * G[1, 1] - G[0, 1] * G[1, 0] + G[0, 0] * G[2, 2] - G[0, 2] * G[2, 0] +
                         G[1, 1] * G[2, 2] - G[1, 2] * G[2, 1]) + np.linalg.det(G)
    return S, jm1


def pos_def(M):
    d2 = M[0, 0] * M[1, 1] - M[0, 1] ** 2
    return M[0, 0] > 0 and d2 > 0 and np.linalg.det(M) > 0


def inside_clamp(S, jm1, elo, ehi):
    return jm1 > -1 and pos_def(S - elo * np.eye(3)) and pos_def(ehi * np.eye(3) - S)


def q_of(S):
    I1 = np.trace(S)
    I2 = 0.5 * (I1 ** 2 - np.trace(S @ S))
    I3 = np.linalg.det(S)
    a, b, c = 0.0, 0.0, 1.0
    al, be, ga = 0.0, Q[1], Q[2]
    for k in range(3, 8):
        a, b, c = c * I3, a - c * I2, b + c * I1
        al += Q[k] * a
        be += Q[k] * b
        ga += Q[k] * c
    return al * np.eye(3) + be * S + ga * S @ S


def rotation(rng):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q * np.sign(np.linalg.det(q))


def test_series_matches_the_polar_form():
    rng = np.random.default_rng(0)
    for spread in (1e-6, 1e-3, 1e-2, 0.04):
        for _ in range(200):
            U, V = rotation(rng), rotation(rng)
            s = np.clip(1 + rng.normal(0, spread, 3), np.sqrt(0.9), np.sqrt(1.1))
            F = U @ np.diag(s) @ V.T
            S, jm1 = strain_of(F)
            dev = F @ q_of(S) @ F.T
            ref = U @ np.diag(s * (s - 1)) @ U.T  # (F - R) F^T with R = U V^T
            # the first term left out, q_8 e^8, is below 4e-8 of Q's eigenvalue
            # (~ e / 2) at |e| = 0.1; FP32 rounds at 6e-8
            assert np.abs(dev - ref).max() <= 6e-8 * np.abs(s - 1).max() + 1e-13
            assert abs(jm1 - (np.prod(s) - 1)) <= 1e-14


def test_positive_definite_test_matches_singular_values():
    rng = np.random.default_rng(1)
    lo, hi = 1 - 2.5e-2, 1 + 7.5e-3
    elo, ehi = lo * lo - 1 + 1e-5, hi * hi - 1 - 1e-5
    seen = {True: 0, False: 0}
    for _ in range(2000):
        U, V = rotation(rng), rotation(rng)
        s = 1 + rng.uniform(-0.03, 0.01, 3)
        F = U @ np.diag(s) @ V.T
        S, jm1 = strain_of(F)
        e = s * s - 1
        want = bool(np.all((e > elo) & (e < ehi)))
        assert inside_clamp(S, jm1, elo, ehi) == want
        seen[want] += 1
    assert min(seen.values()) > 100
    # an inverted F is never accepted
    F = np.diag([1.0, 1.0, -1.0])
    assert not inside_clamp(*strain_of(F), elo, ehi)
