/* The C ABI example of the integration guide as a program: a single scene,
 * page-locked particle arrays, init, steps and positions read back each
 * frame.  tests/test_abi.py compiles and links it (C99, no CUDA headers).
 * Usage: abi_example N FRAMES. */
#include <stdio.h>
#include <stdlib.h>

#include "rd_mpm.h"

int main(int argc, char** argv) {
    const int n = argc > 1 ? atoi(argv[1]) : 8192;
    const int frames = argc > 2 ? atoi(argv[2]) : 10;
    rd_params p;
    rd_default_params(&p); /* the reference's constants */
    p.max_i = p.max_j = p.max_k = 64;
    p.num_particles = n;
    p.h = 1.0 / 64;
    rd_handle* h = NULL;
    if (rd_create(&p, &h) != RD_OK) return 1; /* allocates everything once */
    float *x = NULL, *v = NULL, *mass = NULL; /* page-locked: moved in place */
    if (rd_host_alloc(3 * (size_t)n * sizeof(float), (void**)&x) != RD_OK ||
        rd_host_alloc(3 * (size_t)n * sizeof(float), (void**)&v) != RD_OK ||
        rd_host_alloc((size_t)n * sizeof(float), (void**)&mass) != RD_OK)
        return 2;
    srand(1);
    for (int i = 0; i < n; ++i) { /* a cube of snow falling at 2 m/s */
        for (int a = 0; a < 3; ++a) {
            x[3 * i + a] = 0.4f + 0.2f * (float)rand() / (float)RAND_MAX;
            v[3 * i + a] = a == 1 ? -2.0f : 0.0f;
        }
        mass[i] = 400.0f * 0.008f / (float)n;
    }
    rd_particles in = {x, v, NULL, NULL, NULL, NULL, mass, NULL};
    if (rd_set_particles(h, &in, RD_HOST) != RD_OK) return 3;
    if (rd_init_volumes(h) != RD_OK) return 4; /* main.cpp:53-54 */
    for (int f = 0; f < frames; ++f) {
        if (rd_step(h, 1e-4, 1) != RD_OK) return 5; /* main.cpp:192-218 */
        rd_particles out = {x, NULL, NULL, NULL, NULL, NULL, NULL, NULL};
        if (rd_get_particles(h, &out, RD_HOST) != RD_OK) return 6; /* drawParticles' positions */
    }
    uint32_t flags = 0;
    rd_get_flags(h, &flags);
    printf("%d particles, %d frames, flags %u, x0 = (%g, %g, %g)\n", n, frames, flags, x[0], x[1], x[2]);
    rd_destroy(h);
    rd_host_free(x);
    rd_host_free(v);
    rd_host_free(mass);
    return flags == 0 ? 0 : 7;
}
