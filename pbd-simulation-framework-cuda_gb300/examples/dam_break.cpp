// dam_break.cpp -- a C++ host driving the step through the C ABI alone, the way the reference's
// application drives Fluid::compute (Simulation::step + cudaDeviceSynchronize,
// Simulation.cu:16-19; particles spawned on a lattice as Particles.cc:189-222 does).
//
//   dam_break (--config config.txt | --params params.bin) [--lattice nx ny nz spacing]
//             [--frames F] [--out state.bin]
//
// --config reads the reference's config grammar over the defaults; --params reads a raw
// pbd_params struct (struct_size must match).  The lattice starts at (2.5, 2.5, 2.5), x outer
// and z inner, at rest.  --out writes x then v of the final state (N float4 each).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pbd.h"

static int fail(const char* what) {
    std::fprintf(stderr, "%s: %s\n", what, pbd_last_error());
    return 1;
}

int main(int argc, char** argv) {
    const char *config = nullptr, *params_bin = nullptr, *out = nullptr;
    int nx = 16, ny = 16, nz = 16, frames = 60;
    float spacing = 1.0f;
    for (int a = 1; a < argc; ++a) {
        if (!std::strcmp(argv[a], "--config") && a + 1 < argc) config = argv[++a];
        else if (!std::strcmp(argv[a], "--params") && a + 1 < argc) params_bin = argv[++a];
        else if (!std::strcmp(argv[a], "--out") && a + 1 < argc) out = argv[++a];
        else if (!std::strcmp(argv[a], "--frames") && a + 1 < argc) frames = std::atoi(argv[++a]);
        else if (!std::strcmp(argv[a], "--lattice") && a + 4 < argc) {
            nx = std::atoi(argv[++a]); ny = std::atoi(argv[++a]); nz = std::atoi(argv[++a]);
            spacing = (float)std::atof(argv[++a]);
        } else {
            std::fprintf(stderr, "usage: %s (--config FILE | --params FILE) [--lattice nx ny nz spacing] "
                                 "[--frames F] [--out FILE]\n", argv[0]);
            return 2;
        }
    }
    pbd_params p;
    if (pbd_params_default(&p)) return fail("pbd_params_default");
    if (config && pbd_load_config(&p, config)) return fail("pbd_load_config");
    if (params_bin) {
        FILE* f = std::fopen(params_bin, "rb");
        if (!f || std::fread(&p, sizeof(p), 1, f) != 1) { std::fprintf(stderr, "cannot read %s\n", params_bin); return 1; }
        std::fclose(f);
    }
    const uint32_t n = (uint32_t)nx * (uint32_t)ny * (uint32_t)nz;
    std::vector<float> pos(4 * (size_t)n, 0.0f), vel(4 * (size_t)n, 0.0f);
    size_t k = 0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int l = 0; l < nz; ++l, ++k) {
                pos[4 * k + 0] = 2.5f + (float)i * spacing;
                pos[4 * k + 1] = 2.5f + (float)j * spacing;
                pos[4 * k + 2] = 2.5f + (float)l * spacing;
            }
    pbd_sim* sim = nullptr;
    if (pbd_create(&p, n, &sim)) return fail("pbd_create");
    if (pbd_add_particles(sim, n, pos.data(), vel.data(), nullptr)) return fail("pbd_add_particles");
    for (int f = 0; f < frames; ++f)
        if (pbd_step(sim, 1, nullptr)) return fail("pbd_step");
    if (pbd_sync(sim)) return fail("pbd_sync");
    std::vector<float> x(4 * (size_t)n), v(4 * (size_t)n);
    if (pbd_get_state(sim, x.data(), v.data(), nullptr, nullptr)) return fail("pbd_get_state");
    double ymean = 0.0, vmax = 0.0;
    for (size_t q = 0; q < n; ++q) {
        ymean += x[4 * q + 1];
        vmax = std::fmax(vmax, std::sqrt((double)v[4 * q] * v[4 * q] + (double)v[4 * q + 1] * v[4 * q + 1] +
                                         (double)v[4 * q + 2] * v[4 * q + 2]));
    }
    std::printf("%u particles, %d frames: mean y %.6f, max |v| %.6f\n", n, frames, ymean / n, vmax);
    if (out) {
        FILE* f = std::fopen(out, "wb");
        if (!f || std::fwrite(x.data(), 4, x.size(), f) != x.size() || std::fwrite(v.data(), 4, v.size(), f) != v.size()) {
            std::fprintf(stderr, "cannot write %s\n", out);
            return 1;
        }
        std::fclose(f);
    }
    return pbd_destroy(sim) ? fail("pbd_destroy") : 0;
}
