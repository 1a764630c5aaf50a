// A C++ caller of the libnyxpm C ABI, written the way a Nyx-side shim would use
// it: create a context, one FP64 box, upload a particle file's worth of
// particles, the post_init solve, then PM steps with dt from computeNewDt;
// finally the particle state is written as an AsciiFile.
//
// A second mode kicks with an acceleration the caller computed, as a Nyx shim
// hands moveKickDrift the acc MultiFab of its own Gravity object: upload, the
// field from a raw float64 file (3 n^3 values, component-major, x fastest) by
// nyxpm_set_grav_vector, one moveKickDrift, then the AsciiFile out.
//
// A third mode takes multilevel steps without subcycling on fixed grids, as
// Nyx::advance_particles_only at level 0 would through the shim: the boxes of
// levels 1 .. nlev-1 on the command line (6 ints each, in each level's own index
// space), steps at constant a with a given dt, then the AsciiFile out.
//
// usage: pm_driver <in.ascii> <n> <L> <a0> <steps> <out.ascii>
//        pm_driver kick <in.ascii> <n> <L> <acc.f64> <dt> <a_old> <a_half> <out.ascii>
//        pm_driver amr <in.ascii> <n0> <L> <a> <dt> <steps> <out.ascii> <nlev>
//                  <boxes on level 1> ... <boxes on level nlev-1> <6 ints per box ...>
#include "nyxpm.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

static int check(nyxpm_ctx* c, nyxpm_status st, const char* what)
{
    if (st == NYXPM_OK) return 0;
    std::fprintf(stderr, "%s failed (%d): %s\n", what, (int)st, c ? nyxpm_last_error(c) : "");
    return 1;
}

static int read_particles(const char* in, std::vector<double>& pos, std::vector<double>& vel,
                          std::vector<double>& mass, int64_t* np)
{
    char err[256];
    if (nyxpm_particle_file_count(in, NYXPM_FILE_ASCII, np, err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    pos.resize(3 * *np);
    vel.resize(3 * *np);
    mass.resize(*np);
    int64_t got = 0;
    if (nyxpm_particle_file_read(in, NYXPM_FILE_ASCII, *np, pos.data(), vel.data(), mass.data(), &got,
                                 err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    return 0;
}

static int kick_with_callers_field(char** argv)
{
    const int n = std::atoi(argv[3]);
    const double L = std::atof(argv[4]);
    const double dt = std::atof(argv[6]), a_old = std::atof(argv[7]), a_half = std::atof(argv[8]);
    std::vector<double> pos, vel, mass;
    int64_t np = 0;
    if (read_particles(argv[2], pos, vel, mass, &np)) return 1;
    const size_t count = 3 * (size_t)n * n * n;
    std::vector<double> acc(count);
    FILE* f = std::fopen(argv[5], "rb");
    if (!f || std::fread(acc.data(), sizeof(double), count, f) != count) {
        std::fprintf(stderr, "cannot read %zu doubles from %s\n", count, argv[5]);
        if (f) std::fclose(f);
        return 1;
    }
    std::fclose(f);
    nyxpm_params p;
    nyxpm_default_params(&p);
    nyxpm_ctx* c = nullptr;
    if (check(nullptr, nyxpm_create(&p, &c), "nyxpm_create")) return 1;
    nyxpm_box* b = nullptr;
    if (check(c, nyxpm_box_create(c, n, L, np, NYXPM_FP64, &b), "nyxpm_box_create")) return 1;
    if (check(c, nyxpm_box_upload(c, b, pos.data(), vel.data(), nullptr, mass[0]), "upload")) return 1;
    if (check(c, nyxpm_set_grav_vector(c, b, acc.data(), 0), "nyxpm_set_grav_vector")) return 1;
    if (check(c, nyxpm_kick_drift(c, b, dt, a_old, a_half), "nyxpm_kick_drift")) return 1;
    if (check(c, nyxpm_box_download(c, b, pos.data(), vel.data()), "download")) return 1;
    char err[256];
    if (nyxpm_particle_file_write(argv[9], NYXPM_FILE_ASCII, np, pos.data(), vel.data(), nullptr, mass[0],
                                  err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    nyxpm_box_destroy(c, b);
    nyxpm_destroy(c);
    return 0;
}

static int amr_steps(int argc, char** argv)
{
    const int n0 = std::atoi(argv[3]);
    const double L = std::atof(argv[4]), a = std::atof(argv[5]), dt = std::atof(argv[6]);
    const int steps = std::atoi(argv[7]);
    const int nlev = std::atoi(argv[9]);
    if (nlev < 1 || argc < 10 + nlev - 1) return 2;
    std::vector<int> nbox(nlev > 1 ? nlev - 1 : 1, 0), boxes;
    int total = 0;
    for (int l = 1; l < nlev; ++l) total += (nbox[l - 1] = std::atoi(argv[9 + l]));
    if (argc != 10 + (nlev - 1) + 6 * total) return 2;
    for (int t = 0; t < 6 * total; ++t) boxes.push_back(std::atoi(argv[9 + nlev + t]));
    std::vector<double> pos, vel, mass;
    int64_t np = 0;
    if (read_particles(argv[2], pos, vel, mass, &np)) return 1;
    nyxpm_params p;
    nyxpm_default_params(&p);
    nyxpm_ctx* c = nullptr;
    if (check(nullptr, nyxpm_create(&p, &c), "nyxpm_create")) return 1;
    nyxpm_amr* h = nullptr;
    if (check(c, nyxpm_amr_create(c, n0, L, nlev, nbox.data(), boxes.empty() ? nullptr : boxes.data(), np, &h),
              "nyxpm_amr_create"))
        return 1;
    if (check(c, nyxpm_amr_upload(c, h, pos.data(), vel.data(), mass.data(), 0.0), "nyxpm_amr_upload")) return 1;
    for (int s = 0; s < steps; ++s) {
        nyxpm_step_info info;
        if (check(c, nyxpm_amr_step(c, h, a, a, dt, &info), "nyxpm_amr_step")) return 1;
        std::printf("step %d vcycles %d %d\n", s + 1, info.old_solve.vcycles, info.new_solve.vcycles);
    }
    if (check(c, nyxpm_amr_download(c, h, pos.data(), vel.data()), "nyxpm_amr_download")) return 1;
    nyxpm_amr_destroy(c, h);
    nyxpm_destroy(c);
    char err[256];
    if (nyxpm_particle_file_write(argv[8], NYXPM_FILE_ASCII, np, pos.data(), vel.data(), mass.data(), 0.0,
                                  err, sizeof(err)) != NYXPM_OK) {
        std::fprintf(stderr, "%s\n", err);
        return 1;
    }
    return 0;
}

int main(int argc, char** argv)
{
    if (argc >= 10 && std::strcmp(argv[1], "amr") == 0) return amr_steps(argc, argv);
    if (argc == 10 && std::strcmp(argv[1], "kick") == 0) return kick_with_callers_field(argv);
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s in.ascii n L a0 steps out.ascii\n"
                             "       %s kick in.ascii n L acc.f64 dt a_old a_half out.ascii\n",
                     argv[0], argv[0]);
        return 2;
    }
    const char* in = argv[1];
    const int n = std::atoi(argv[2]);
    const double L = std::atof(argv[3]);
    double a = std::atof(argv[4]);
    const int steps = std::atoi(argv[5]);
    char err[256];
    int64_t np = 0;
    std::vector<double> pos, vel, mass;
    if (read_particles(in, pos, vel, mass, &np)) return 1;
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
