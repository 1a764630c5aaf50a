// A C++ caller of the libnyxpm C ABI, written the way a Nyx-side shim would use
// it: create a context, one FP64 box, upload a particle file's worth of
// particles, the post_init solve, then PM steps with dt from computeNewDt;
// finally the particle state is written as an AsciiFile.
//
// usage: pm_driver <in.ascii> <n> <L> <a0> <steps> <out.ascii>
#include "nyxpm.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

static int check(nyxpm_ctx* c, nyxpm_status st, const char* what)
{
    if (st == NYXPM_OK) return 0;
    std::fprintf(stderr, "%s failed (%d): %s\n", what, (int)st, c ? nyxpm_last_error(c) : "");
    return 1;
}

int main(int argc, char** argv)
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s in.ascii n L a0 steps out.ascii\n", argv[0]);
        return 2;
    }
    const char* in = argv[1];
    const int n = std::atoi(argv[2]);
    const double L = std::atof(argv[3]);
    double a = std::atof(argv[4]);
    const int steps = std::atoi(argv[5]);
    char err[256];
    int64_t np = 0;
    if (nyxpm_particle_file_count(in, NYXPM_FILE_ASCII, &np, err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    std::vector<double> pos(3 * np), vel(3 * np), mass(np);
    int64_t got = 0;
    if (nyxpm_particle_file_read(in, NYXPM_FILE_ASCII, np, pos.data(), vel.data(), mass.data(), &got,
                                 err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    nyxpm_params p;
    nyxpm_default_params(&p);
    nyxpm_ctx* c = nullptr;
    if (check(nullptr, nyxpm_create(&p, &c), "nyxpm_create")) return 1;
    nyxpm_box* b = nullptr;
    if (check(c, nyxpm_box_create(c, n, L, np, NYXPM_FP64, &b), "nyxpm_box_create")) return 1;
    if (check(c, nyxpm_box_upload(c, b, pos.data(), vel.data(), nullptr, mass[0]), "upload")) return 1;
    nyxpm_solve_info si;
    if (check(c, nyxpm_init_field(c, b, a, &si), "nyxpm_init_field")) return 1;
    nyxpm_dt_params dp;
    nyxpm_default_dt_params(&dp);
    double t = 0.0, dt_old = -1.0;
    for (int s = 0; s < steps; ++s) {
        double dt = 0.0, a_new = 0.0;
        if (check(c, nyxpm_compute_new_dt(c, b, &dp, t, a, dt_old, &dt, &a_new), "compute_new_dt"))
            return 1;
        nyxpm_step_info info;
        if (check(c, nyxpm_step(c, b, a, a_new, dt, 0, &info), "nyxpm_step")) return 1;
        std::printf("step %d a %.17g dt %.17g vcycles %d %d\n", s + 1, a_new, dt, info.old_solve.vcycles,
                    info.new_solve.vcycles);
        t += dt;
        dt_old = dt;
        a = a_new;
    }
    if (check(c, nyxpm_box_download(c, b, pos.data(), vel.data()), "download")) return 1;
    if (nyxpm_particle_file_write(argv[6], NYXPM_FILE_ASCII, np, pos.data(), vel.data(), nullptr, mass[0],
                                  err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    nyxpm_box_destroy(c, b);
    nyxpm_destroy(c);
    return 0;
}
