// Host side of libnyxpm: the C ABI of include/nyxpm.h, box memory, the step
// orchestration of Nyx::advance_particles_only, launch profiling and the FP64
// a(t) integrators of Source/Driver/comoving.cpp.
#include "pm_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

using namespace nyxpm;

namespace nyxpm {

void prof_begin(Ctx& c)
{
    c.launches += 1;
    if (!c.prof_on) return;
    if (c.recs.size() >= c.ev_a.size()) {
        // pool full: fold what was recorded, then reuse the events
        nyxpm_profile tmp;
        nyxpm_get_profile(static_cast<nyxpm_ctx*>(&c), &tmp, 0);
    }
    cudaEventRecord(c.ev_a[c.recs.size()], c.stream);
}

void prof_end(Ctx& c, int stage, double bytes, int fine)
{
    if (!c.prof_on) return;
    cudaEventRecord(c.ev_b[c.recs.size()], c.stream);
    c.recs.push_back(ProfRec{stage, fine, bytes});
}

nyxpm_status check_launch(Ctx& c, const char* what)
{
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = c.launch_error;
    c.launch_error = cudaSuccess;
    if (e == cudaSuccess) return NYXPM_OK;
    c.err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? NYXPM_OOM : NYXPM_CUDA_ERROR;
}

nyxpm_status run_iteration(Ctx& c, IterGraph& g, const std::function<nyxpm_status()>& body)
{
    if (c.prof_on || g.failed) return body();
    if (!g.exec) {
        const int64_t l0 = c.launches;
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            g.failed = 1;
            return body();
        }
        const nyxpm_status st = body();
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
        const int64_t n = c.launches - l0;
        c.launches = l0;
        if (st != NYXPM_OK) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return st;
        }
        cudaError_t ei = e;
        if (ei == cudaSuccess && graph) ei = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ei != cudaSuccess || !graph) {
            // the stream would not capture (e.g. a caller's stream in another
            // capture): the same launches, eagerly, from now on
            cudaGetLastError();
            g.exec = nullptr;
            g.failed = 1;
            return body();
        }
        g.launches = n;
    }
    c.launches += g.launches;
    if (cudaGraphLaunch(g.exec, c.stream) != cudaSuccess) return check_launch(c, "solver iteration graph");
    return NYXPM_OK;
}

}  // namespace nyxpm

namespace {

constexpr int kProfEvents = 8192;

nyxpm_status fail(Ctx* c, nyxpm_status st, const std::string& msg)
{
    if (c) c->err = msg;
    return st;
}

template <typename T>
nyxpm_status dalloc(Ctx& c, Box& b, T** p, size_t count)
{
    if (count == 0) count = 1;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c.err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return NYXPM_OOM;
    }
    b.allocs.push_back(q);
    *p = static_cast<T*>(q);
    return NYXPM_OK;
}

int bottom_edge(int n)
{
    int m = n;
    while (m % 2 == 0 && m > kCoarsenAbove) m /= 2;
    return m;
}

// Green's function of the periodic 7-point Laplacian on nb^3 with spacing h,
// without the constant mode, in smoother units (applied to beta = h^2 rhs / 6):
// the exact coarsest-level solve.
void bottom_green(int nb, double h, double* G)
{
    const long nc = (long)nb * nb * nb;
    const double twopi = 2.0 * std::acos(-1.0);
    std::vector<double> lam(nc);
    for (int kz = 0; kz < nb; ++kz)
        for (int ky = 0; ky < nb; ++ky)
            for (int kx = 0; kx < nb; ++kx) {
                double l = (2.0 * std::cos(twopi * kx / nb) - 2.0) + (2.0 * std::cos(twopi * ky / nb) - 2.0)
                         + (2.0 * std::cos(twopi * kz / nb) - 2.0);
                lam[kx + nb * (ky + (long)nb * kz)] = l / (h * h);
            }
    const double scale = 6.0 / (h * h);
    for (int dz = 0; dz < nb; ++dz)
        for (int dy = 0; dy < nb; ++dy)
            for (int dxx = 0; dxx < nb; ++dxx) {
                double s = 0.0;
                for (int kz = 0; kz < nb; ++kz)
                    for (int ky = 0; ky < nb; ++ky)
                        for (int kx = 0; kx < nb; ++kx) {
                            if (kx == 0 && ky == 0 && kz == 0) continue;
                            const long ph = ((long)kx * dxx + (long)ky * dy + (long)kz * dz) % nb;
                            s += std::cos(twopi * (double)ph / nb) / lam[kx + nb * (ky + (long)nb * kz)];
                        }
                G[dxx + nb * (dy + (long)nb * dz)] = (s / (double)nc) * scale;
            }
}

double adot(double H0, double OmM, double OmR, double OmL, double a)
{
    return H0 * std::sqrt(OmM / a + OmR / (a * a) + OmL * a * a);
}

nyxpm_status ensure_sorted(Ctx& c, Box& b)
{
    if (b.sorted) return NYXPM_OK;
    return b.prec == NYXPM_MIXED ? mixed_sort(c, b) : launch_sort(c, b);
}

nyxpm_status do_deposit(Ctx& c, Box& b)
{
    nyxpm_status st = ensure_sorted(c, b);
    if (st != NYXPM_OK) return st;
    return b.prec == NYXPM_MIXED ? mixed_deposit(c, b) : launch_deposit(c, b);
}

// RHS, V-cycles, then the cell-centred gravity vector of the new phi
nyxpm_status do_solve(Ctx& c, Box& b, double a, int zero_guess, nyxpm_solve_info* info)
{
    nyxpm_status st;
    const bool mixed = b.prec == NYXPM_MIXED;
    if ((st = mixed ? mixed_make_rhs(c, b, a) : launch_make_rhs(c, b, a)) != NYXPM_OK) return st;
    if (zero_guess && (st = launch_zero_phi(c, b)) != NYXPM_OK) return st;
    nyxpm_status solved = mixed ? mixed_solve(c, b, zero_guess, info) : mg_solve(c, b, info);
    if (solved != NYXPM_OK && solved != NYXPM_NOT_CONVERGED) return solved;
    b.g_from_caller = 0;   // the gravity vector follows the new phi from here on
    // the mixed solve leaves its FP32 gravity vector in g32 itself
    if (!mixed && (st = launch_grav_vector(c, b)) != NYXPM_OK) return st;
    return solved;
}

nyxpm_status do_kick(Ctx& c, Box& b, double dt, double a_prev, double a_cur, int do_move, int do_wrap)
{
    if (b.prec == NYXPM_MIXED) {
        // mixed positions are cell-relative: always in the box, no wrap needed
        return mixed_kick(c, b, dt, a_prev, a_cur, do_move);
    }
    return launch_kick(c, b, dt, a_prev, a_cur, do_move, do_wrap);
}

#define CHECK_CTX(ctx)                                                                       \
    do {                                                                                     \
        if (!(ctx)) return NYXPM_INVALID_ARG;                                                \
    } while (0)
#define CHECK_BOX(ctx, box)                                                                  \
    do {                                                                                     \
        CHECK_CTX(ctx);                                                                      \
        if (!(box)) return fail(ctx, NYXPM_INVALID_ARG, "null box");                         \
    } while (0)
#define TRY(expr)                                                                            \
    do {                                                                                     \
        nyxpm_status _st = (expr);                                                           \
        if (_st != NYXPM_OK) return _st;                                                     \
    } while (0)

}  // namespace

extern "C" {

int nyxpm_abi_version(void) { return NYXPM_ABI_VERSION; }

void nyxpm_default_params(nyxpm_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->device = 0;
    p->stream = nullptr;
    p->comoving_OmM = 1.0;
    p->comoving_OmR = 0.0;
    p->comoving_h = 0.675;
    {
        const double M_unit = 1.98848e33;
        const double L_unit = 3.0856776e24;
        const double V_unit = 1.e5;
        const double T_unit = L_unit / V_unit;
        p->gconst = 6.67408e-8 * M_unit * T_unit * T_unit / (L_unit * L_unit * L_unit);
    }
    p->rel_tol = 1e-10;
    p->max_vcycles = 100;
    p->nu1 = 2;
    p->nu2 = 2;
    p->verbose = 0;
    p->mixed_inner_vcycles = 2;
    p->mg_fused_edge = 16;
}

nyxpm_status nyxpm_create(const nyxpm_params* p, nyxpm_ctx** out)
{
    if (!p || !out) return NYXPM_INVALID_ARG;
    *out = nullptr;
    if (p->nu1 < 0 || p->nu2 < 0 || p->max_vcycles < 1 || !(p->rel_tol > 0) ||
        p->mixed_inner_vcycles < 1 || p->mg_fused_edge < 0)
        return NYXPM_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return NYXPM_NO_DEVICE;
    }
    if (p->device < 0 || p->device >= ndev) return NYXPM_INVALID_ARG;
    if (cudaSetDevice(p->device) != cudaSuccess) return NYXPM_CUDA_ERROR;
    nyxpm_ctx* c = new (std::nothrow) nyxpm_ctx();
    if (!c) return NYXPM_OOM;
    c->p = *p;
    if (p->stream) {
        c->stream = static_cast<cudaStream_t>(p->stream);
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return NYXPM_CUDA_ERROR;
        }
        c->own_stream = 1;
    }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, p->device);
    const char* no_pdl = std::getenv("NYXPM_NO_PDL");
    c->pdl = (no_pdl && no_pdl[0] && no_pdl[0] != '0') ? 0 : 1;
    *out = c;
    return NYXPM_OK;
}

void nyxpm_destroy(nyxpm_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->p.device);
    cudaStreamSynchronize(c->stream);
    for (auto e : c->ev_a) cudaEventDestroy(e);
    for (auto e : c->ev_b) cudaEventDestroy(e);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaEventDestroy(c->ev_copy_in);
        cudaEventDestroy(c->ev_copy_out);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* nyxpm_last_error(const nyxpm_ctx* c) { return c ? c->err.c_str() : "null context"; }

void* nyxpm_stream(nyxpm_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

nyxpm_status nyxpm_synchronize(nyxpm_ctx* c)
{
    CHECK_CTX(c);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(c, NYXPM_CUDA_ERROR, cudaGetErrorString(e));
    return NYXPM_OK;
}

int64_t nyxpm_launch_count(const nyxpm_ctx* c) { return c ? c->launches : 0; }

size_t nyxpm_box_bytes(int n, int64_t np, nyxpm_precision prec)
{
    const double nc = (double)n * n * n;
    double per_particle, per_cell;
    if (prec == NYXPM_MIXED) {
        // cell + 3 offsets + 3 vel + mass + id, double-buffered; key, perm; staging
        per_particle = 2.0 * (4 + 12 + 12 + 4 + 4) + 8 + 56 + 2;
        per_cell = 4 + 4 + 4 + 4 + 8 + 24 + 8 + 16 + 4 + 16.0 * 8 / 7 + 8.0 * 8 / 7;
    } else {
        per_particle = 2.0 * (7 * 8 + 4) + 8 + 56 + 2;
        per_cell = 4 + 4 + 4 + 8 + 24 + 8 + 64 + 4 + 16.0 * 8 / 7;
    }
    return (size_t)(per_particle * (double)np + per_cell * nc + 8.0 * n * n + (1 << 20));
}

nyxpm_status nyxpm_box_create(nyxpm_ctx* c, int n, double L, int64_t np, nyxpm_precision prec,
                              nyxpm_box** out)
{
    CHECK_CTX(c);
    if (!out) return fail(c, NYXPM_INVALID_ARG, "null output");
    *out = nullptr;
    if (n < 2 || n > 1024) return fail(c, NYXPM_INVALID_ARG, "n must be in [2, 1024]");
    if (bottom_edge(n) > kMaxBottom)
        return fail(c, NYXPM_INVALID_ARG, "n must be m * 2^k with m <= 8");
    if (!(L > 0)) return fail(c, NYXPM_INVALID_ARG, "L must be positive");
    if (np < 1 || np > (int64_t)0x7fffffff) return fail(c, NYXPM_INVALID_ARG, "np out of range");
    if (prec != NYXPM_FP64 && prec != NYXPM_MIXED) return fail(c, NYXPM_INVALID_ARG, "precision");
    cudaSetDevice(c->p.device);
    nyxpm_box* b = new (std::nothrow) nyxpm_box();
    if (!b) return NYXPM_OOM;
    b->n = n;
    b->L = L;
    b->dx = L / n;
    b->dxi = (double)n / L;
    b->np = np;
    b->prec = prec;
    const size_t nc = (size_t)n * n * n;
    auto cleanup = [&](nyxpm_status st) {
        for (void* q : b->allocs) cudaFree(q);
        if (b->h_norms) cudaFreeHost(b->h_norms);
        delete b;
        return st;
    };
#define ALLOC(ptr, cnt)                                                                      \
    do {                                                                                     \
        nyxpm_status _s = dalloc(*c, *b, &(ptr), (cnt));                                     \
        if (_s != NYXPM_OK) return cleanup(_s);                                              \
    } while (0)
    if (prec == NYXPM_FP64) {
        ALLOC(b->x, np); ALLOC(b->y, np); ALLOC(b->z, np);
        ALLOC(b->vx, np); ALLOC(b->vy, np); ALLOC(b->vz, np); ALLOC(b->m, np); ALLOC(b->id, np);
        ALLOC(b->x2, np); ALLOC(b->y2, np); ALLOC(b->z2, np);
        ALLOC(b->vx2, np); ALLOC(b->vy2, np); ALLOC(b->vz2, np); ALLOC(b->m2, np); ALLOC(b->id2, np);
        ALLOC(b->key_part, 8 * nc);
    } else {
        ALLOC(b->cell, np); ALLOC(b->ox, np); ALLOC(b->oy, np); ALLOC(b->oz, np);
        ALLOC(b->fvx, np); ALLOC(b->fvy, np); ALLOC(b->fvz, np); ALLOC(b->fm, np); ALLOC(b->id, np);
        ALLOC(b->cell2, np); ALLOC(b->ox2, np); ALLOC(b->oy2, np); ALLOC(b->oz2, np);
        ALLOC(b->fvx2, np); ALLOC(b->fvy2, np); ALLOC(b->fvz2, np); ALLOC(b->fm2, np); ALLOC(b->id2, np);
        ALLOC(b->frho, nc);
        ALLOC(b->g32, 4 * nc);
        ALLOC(b->r_lo, nc);
    }
    ALLOC(b->key, np);
    ALLOC(b->perm, np);
    ALLOC(b->cell_count, nc);
    ALLOC(b->cell_start, nc + 1);
    b->ntiles = (int)((nc + 4095) / 4096);
    ALLOC(b->tile_sums, b->ntiles);
    ALLOC(b->long_list, nc);
    ALLOC(b->long_count, 1);
    ALLOC(b->heavy_part, 8 * (size_t)(np / (kDepositLanes + 1) + 1));
    ALLOC(b->key_slot, nc);
    ALLOC(b->rho, nc);
    ALLOC(b->g, 3 * nc);
    ALLOC(b->nat, nc);
    ALLOC(b->rows, (size_t)n * n);
    ALLOC(b->planes, n);
    ALLOC(b->scal, 4);
    ALLOC(b->norms, 8);
    ALLOC(b->staging, 7 * (size_t)np + 1);
    if (cudaMallocHost(&b->h_norms, 8 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        b->h_norms = nullptr;
        return cleanup(fail(c, NYXPM_OOM, "cudaMallocHost"));
    }
    // multigrid hierarchy: split levels while n > 8, natural bottom
    const int nbot = bottom_edge(n);
    for (int nl = n;; nl /= 2) {
        Level l;
        l.n = nl;
        l.split = nl > nbot ? 1 : 0;
        const size_t cnt = (size_t)nl * nl * nl;
        if (l.split) {
            ALLOC(l.phi_r, cnt / 2); ALLOC(l.phi_b, cnt / 2);
            ALLOC(l.beta_r, cnt / 2); ALLOC(l.beta_b, cnt / 2);
            if (prec == NYXPM_MIXED) {
                ALLOC(l.fphi_r, cnt / 2); ALLOC(l.fphi_b, cnt / 2);
                ALLOC(l.fbeta_r, cnt / 2); ALLOC(l.fbeta_b, cnt / 2);
            }
        } else {
            ALLOC(l.phi_r, cnt); ALLOC(l.beta_r, cnt);
            if (prec == NYXPM_MIXED) { ALLOC(l.fphi_r, cnt); ALLOC(l.fbeta_r, cnt); }
        }
        b->levels.push_back(l);
        if (nl == nbot) break;
    }
    b->nb = nbot;
    if (prec == NYXPM_FP64 && b->levels[0].split) {
        b->phi_r_alloc = b->levels[0].phi_r;
        ALLOC(b->phi_r_spare, nc / 2);
    }
    ALLOC(b->G, (size_t)nbot * nbot * nbot);
    ALLOC(b->Gf, (size_t)nbot * nbot * nbot);
#undef ALLOC
    std::vector<double> G((size_t)nbot * nbot * nbot);
    std::vector<float> Gf(G.size());
    bottom_green(nbot, L / nbot, G.data());
    for (size_t t = 0; t < G.size(); ++t) Gf[t] = (float)G[t];
    cudaMemcpyAsync(b->G, G.data(), sizeof(double) * G.size(), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(b->Gf, Gf.data(), sizeof(float) * Gf.size(), cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(b->cell_count, 0, sizeof(int) * nc, c->stream);
    for (const Level& l : b->levels) {
        const size_t cnt = (size_t)l.n * l.n * l.n;
        if (l.split) {
            cudaMemsetAsync(l.phi_r, 0, sizeof(double) * cnt / 2, c->stream);
            cudaMemsetAsync(l.phi_b, 0, sizeof(double) * cnt / 2, c->stream);
            if (l.fphi_r) {
                cudaMemsetAsync(l.fphi_r, 0, sizeof(float) * cnt / 2, c->stream);
                cudaMemsetAsync(l.fphi_b, 0, sizeof(float) * cnt / 2, c->stream);
            }
        } else {
            cudaMemsetAsync(l.phi_r, 0, sizeof(double) * cnt, c->stream);
            if (l.fphi_r) cudaMemsetAsync(l.fphi_r, 0, sizeof(float) * cnt, c->stream);
        }
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        nyxpm_status st = check_launch(*c, "box init");
        return cleanup(st == NYXPM_OK ? NYXPM_CUDA_ERROR : st);
    }
    *out = b;
    return NYXPM_OK;
}

nyxpm_status nyxpm_box_destroy(nyxpm_ctx* c, nyxpm_box* b)
{
    CHECK_BOX(c, b);
    cudaSetDevice(c->p.device);
    cudaStreamSynchronize(c->stream);
    for (IterGraph& g : b->iter_graph)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (void* q : b->allocs) cudaFree(q);
    if (b->h_norms) cudaFreeHost(b->h_norms);
    delete b;
    return NYXPM_OK;
}

nyxpm_status nyxpm_box_upload(nyxpm_ctx* c, nyxpm_box* b, const double* pos, const double* vel,
                              const double* mass, double mass_scalar)
{
    CHECK_BOX(c, b);
    if (!pos || !vel) return fail(c, NYXPM_INVALID_ARG, "null pos/vel");
    const int64_t np = b->np;
    double total = 0.0;
    if (mass) {
        for (int64_t q = 0; q < np; ++q) {
            if (!(mass[q] >= 0) || !std::isfinite(mass[q])) return fail(c, NYXPM_INVALID_ARG, "bad mass");
            total = total + mass[q];
        }
    } else {
        if (!(mass_scalar >= 0) || !std::isfinite(mass_scalar)) return fail(c, NYXPM_INVALID_ARG, "bad mass");
        total = mass_scalar * (double)np;
    }
    b->uniform_mass = mass ? 0 : 1;
    b->mscalar = mass ? 0.0 : mass_scalar;
    b->mass_offset = total / (b->L * b->L * b->L);
    double* d_pos = b->staging;
    double* d_vel = b->staging + 3 * np;
    cudaMemcpyAsync(d_pos, pos, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_vel, vel, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream);
    const double* d_mass = nullptr;
    if (mass) {
        double* dm = b->staging + 6 * np;
        cudaMemcpyAsync(dm, mass, sizeof(double) * np, cudaMemcpyHostToDevice, c->stream);
        d_mass = dm;
    }
    TRY(check_launch(*c, "upload copy"));
    cudaMemsetAsync(b->norms + 2, 0, sizeof(unsigned long long), c->stream);
    if (b->prec == NYXPM_MIXED) TRY(mixed_unpack(*c, *b, d_pos, d_vel, d_mass));
    else TRY(launch_unpack(*c, *b, d_pos, d_vel, d_mass));
    // the unpack kernels count non-finite positions/velocities into norms[2]
    cudaMemcpyAsync(b->h_norms + 2, b->norms + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                    c->stream);
    TRY(nyxpm_synchronize(c));
    b->sorted = 0;
    if (b->h_norms[2] != 0) {
        b->uploaded = 0;
        return fail(c, NYXPM_INVALID_ARG, "non-finite particle position or velocity");
    }
    b->uploaded = 1;
    return NYXPM_OK;
}

nyxpm_status nyxpm_box_init_cosmo_1ppc(nyxpm_ctx* c, nyxpm_box* b, const double* disp,
                                       const double* vel, const double* disp_fac,
                                       const double* vel_fac, double particle_mass)
{
    CHECK_BOX(c, b);
    const int64_t nc = (int64_t)b->n * b->n * b->n;
    if (b->np != nc) return fail(c, NYXPM_INVALID_ARG, "one particle per cell needs np = n^3");
    std::vector<double> pos(3 * (size_t)nc), v(3 * (size_t)nc);
    if (nyxpm_cosmo_1ppc_particles(b->n, b->L, disp, vel, disp_fac, vel_fac, pos.data(), v.data()) !=
        NYXPM_OK)
        return fail(c, NYXPM_INVALID_ARG, "null displacement/velocity field or factors");
    return nyxpm_box_upload(c, b, pos.data(), v.data(), nullptr, particle_mass);
}

nyxpm_status nyxpm_box_download(nyxpm_ctx* c, nyxpm_box* b, double* pos, double* vel)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (!pos || !vel) return fail(c, NYXPM_INVALID_ARG, "null pos/vel");
    const int64_t np = b->np;
    double* d_pos = b->staging;
    double* d_vel = b->staging + 3 * np;
    if (b->prec == NYXPM_MIXED) TRY(mixed_pack(*c, *b, d_pos, d_vel));
    else TRY(launch_pack(*c, *b, d_pos, d_vel));
    cudaMemcpyAsync(pos, d_pos, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(vel, d_vel, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c->stream);
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_set_mass_offset(nyxpm_ctx* c, nyxpm_box* b, double* mass_offset)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (mass_offset) *mass_offset = b->mass_offset;
    return NYXPM_OK;
}

nyxpm_status nyxpm_redistribute(nyxpm_ctx* c, nyxpm_box* b)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (b->prec == NYXPM_FP64) TRY(launch_wrap(*c, *b));
    b->sorted = 0;
    return ensure_sorted(*c, *b);
}

nyxpm_status nyxpm_deposit(nyxpm_ctx* c, nyxpm_box* b, double* rho_out)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    TRY(do_deposit(*c, *b));
    if (rho_out) {
        const size_t nc = (size_t)b->n * b->n * b->n;
        if (b->prec == NYXPM_MIXED) TRY(mixed_rho_to_double(*c, *b));
        cudaMemcpyAsync(rho_out, b->rho, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream);
        TRY(check_launch(*c, "rho copy"));
        return nyxpm_synchronize(c);
    }
    return NYXPM_OK;
}

nyxpm_status nyxpm_solve_phi(nyxpm_ctx* c, nyxpm_box* b, double a, int zero_guess,
                             nyxpm_solve_info* info)
{
    CHECK_BOX(c, b);
    if (!(a > 0)) return fail(c, NYXPM_INVALID_ARG, "a must be positive");
    return do_solve(*c, *b, a, zero_guess, info);
}

nyxpm_status nyxpm_get_phi(nyxpm_ctx* c, nyxpm_box* b, double* phi)
{
    CHECK_BOX(c, b);
    if (!phi) return fail(c, NYXPM_INVALID_ARG, "null phi");
    const size_t nc = (size_t)b->n * b->n * b->n;
    TRY(launch_phi_to_natural(*c, *b, b->nat));
    cudaMemcpyAsync(phi, b->nat, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream);
    TRY(check_launch(*c, "phi copy"));
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_set_phi(nyxpm_ctx* c, nyxpm_box* b, const double* phi)
{
    CHECK_BOX(c, b);
    if (!phi) return fail(c, NYXPM_INVALID_ARG, "null phi");
    const size_t nc = (size_t)b->n * b->n * b->n;
    cudaMemcpyAsync(b->nat, phi, sizeof(double) * nc, cudaMemcpyHostToDevice, c->stream);
    TRY(check_launch(*c, "phi copy"));
    TRY(launch_phi_from_natural(*c, *b, b->nat));
    TRY(launch_grav_vector(*c, *b));
    if (b->prec == NYXPM_MIXED) TRY(mixed_grav32(*c, *b));
    b->have_phi = 1;
    b->g_from_caller = 0;
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_set_grav_vector(nyxpm_ctx* c, nyxpm_box* b, const double* g, int on_device)
{
    CHECK_BOX(c, b);
    if (!g) return fail(c, NYXPM_INVALID_ARG, "null g");
    const size_t nc = (size_t)b->n * b->n * b->n;
    cudaMemcpyAsync(b->g, g, sizeof(double) * 3 * nc,
                    on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream);
    TRY(check_launch(*c, "caller gravity copy"));
    if (b->prec == NYXPM_MIXED) TRY(mixed_g32_from_g(*c, *b));
    b->g_from_caller = 1;
    // a host buffer may be reused as soon as the call returns
    return on_device ? NYXPM_OK : nyxpm_synchronize(c);
}

nyxpm_status nyxpm_grav_vector(nyxpm_ctx* c, nyxpm_box* b, double* g_out)
{
    CHECK_BOX(c, b);
    if (!b->have_phi && !b->g_from_caller)
        return fail(c, NYXPM_INVALID_ARG, "no field: solve, set phi or set the gravity vector first");
    if (b->prec == NYXPM_MIXED && !b->g_from_caller) TRY(launch_grav_vector(*c, *b));
    if (g_out) {
        const size_t nc = (size_t)b->n * b->n * b->n;
        cudaMemcpyAsync(g_out, b->g, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream);
        TRY(check_launch(*c, "g copy"));
        return nyxpm_synchronize(c);
    }
    return NYXPM_OK;
}

nyxpm_status nyxpm_kick_drift(nyxpm_ctx* c, nyxpm_box* b, double dt, double a_old, double a_half)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (!b->have_phi && !b->g_from_caller)
        return fail(c, NYXPM_INVALID_ARG, "no field: solve, set phi or set the gravity vector first");
    if (!(a_half > 0) || !std::isfinite(dt)) return fail(c, NYXPM_INVALID_ARG, "bad dt / a");
    return do_kick(*c, *b, dt, a_old, a_half, 1, 0);
}

nyxpm_status nyxpm_kick(nyxpm_ctx* c, nyxpm_box* b, double dt, double a_new, double a_half)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (!b->have_phi && !b->g_from_caller)
        return fail(c, NYXPM_INVALID_ARG, "no field: solve, set phi or set the gravity vector first");
    if (!(a_new > 0) || !std::isfinite(dt)) return fail(c, NYXPM_INVALID_ARG, "bad dt / a");
    return do_kick(*c, *b, dt, a_half, a_new, 0, 0);
}

nyxpm_status nyxpm_init_field(nyxpm_ctx* c, nyxpm_box* b, double a, nyxpm_solve_info* info)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (!(a > 0)) return fail(c, NYXPM_INVALID_ARG, "a must be positive");
    if (b->prec == NYXPM_FP64) TRY(launch_wrap(*c, *b));
    b->sorted = 0;
    TRY(do_deposit(*c, *b));
    return do_solve(*c, *b, a, 1, info);
}

nyxpm_status nyxpm_step(nyxpm_ctx* c, nyxpm_box* b, double a_old, double a_new, double dt,
                        unsigned flags, nyxpm_step_info* info)
{
    CHECK_BOX(c, b);
    if (!b->uploaded) return fail(c, NYXPM_INVALID_ARG, "box has no particles");
    if (!(a_old > 0) || !(a_new > 0) || !std::isfinite(dt))
        return fail(c, NYXPM_INVALID_ARG, "bad a / dt");
    const double a_half = 0.5 * (a_old + a_new);
    nyxpm_step_info local;
    std::memset(&local, 0, sizeof(local));
    const bool reuse = (flags & NYXPM_STEP_REUSE_FIELD) != 0;
    if (reuse && !b->have_phi) return fail(c, NYXPM_INVALID_ARG, "no field to reuse: call nyxpm_init_field");
    nyxpm_status st_old = NYXPM_OK, st_new;
    if (!reuse) {
        // old-time solve from the start-of-step positions, phi = 0 guess
        TRY(do_deposit(*c, *b));
        st_old = do_solve(*c, *b, a_old, 1, &local.old_solve);
        if (st_old != NYXPM_OK && st_old != NYXPM_NOT_CONVERGED) return st_old;
    }
    TRY(do_kick(*c, *b, dt, a_old, a_half, 1, 0));
    // new-time solve, the old phi as the initial guess
    TRY(do_deposit(*c, *b));
    st_new = do_solve(*c, *b, a_new, 0, &local.new_solve);
    if (st_new != NYXPM_OK && st_new != NYXPM_NOT_CONVERGED) return st_new;
    TRY(do_kick(*c, *b, dt, a_half, a_new, 0, 1));
    if (info) *info = local;
    return st_old != NYXPM_OK ? st_old : st_new;
}

nyxpm_status nyxpm_step_host(nyxpm_ctx* c, nyxpm_box* b, double* pos, double* vel,
                             const double* mass, double mass_scalar, double a_old, double a_new,
                             double dt, unsigned flags, nyxpm_step_info* info)
{
    CHECK_BOX(c, b);
    if (!pos || !vel) return fail(c, NYXPM_INVALID_ARG, "null pos/vel");
    if (!(a_old > 0) || !(a_new > 0) || !std::isfinite(dt)) return fail(c, NYXPM_INVALID_ARG, "bad a / dt");
    const bool reuse = (flags & NYXPM_STEP_REUSE_FIELD) != 0;
    const bool mixed = b->prec == NYXPM_MIXED;
    if (reuse && !b->have_phi) return fail(c, NYXPM_INVALID_ARG, "no field to reuse: call nyxpm_init_field");
    const int64_t np = b->np;
    double total = 0.0;
    if (mass) {
        for (int64_t q = 0; q < np; ++q) {
            if (!(mass[q] >= 0) || !std::isfinite(mass[q])) return fail(c, NYXPM_INVALID_ARG, "bad mass");
            total = total + mass[q];
        }
    } else {
        if (!(mass_scalar >= 0) || !std::isfinite(mass_scalar)) return fail(c, NYXPM_INVALID_ARG, "bad mass");
        total = mass_scalar * (double)np;
    }
    if (!c->copy_stream) {
        if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_copy_in, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_copy_out, cudaEventDisableTiming) != cudaSuccess)
            return check_launch(*c, "copy stream");
    }
    b->uniform_mass = mass ? 0 : 1;
    b->mscalar = mass ? 0.0 : mass_scalar;
    b->mass_offset = total / (b->L * b->L * b->L);
    double* s_pos = b->staging;
    double* s_vel = b->staging + 3 * np;
    double* s_mass = b->staging + 6 * np;
    // positions (and masses) first, on the step's stream ...
    cudaMemsetAsync(b->norms + 2, 0, sizeof(unsigned long long), c->stream);
    cudaMemcpyAsync(s_pos, pos, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->stream);
    if (mass) cudaMemcpyAsync(s_mass, mass, sizeof(double) * np, cudaMemcpyHostToDevice, c->stream);
    // (the velocity copy starts after them: run at the same time, the two would
    // share the host link and the positions, on the critical path, would take
    // twice as long)
    cudaEventRecord(c->ev_copy_out, c->stream);
    TRY(mixed ? mixed_unpack_pos(*c, *b, s_pos, mass ? s_mass : nullptr)
              : launch_unpack_pos(*c, *b, s_pos, mass ? s_mass : nullptr));
    // ... the velocities on the copy stream, under the sort, deposit and old-time solve
    cudaStreamWaitEvent(c->copy_stream, c->ev_copy_out, 0);
    cudaMemcpyAsync(s_vel, vel, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, c->copy_stream);
    cudaEventRecord(c->ev_copy_in, c->copy_stream);
    TRY(check_launch(*c, "host step input copies"));
    b->uploaded = 1;
    b->sorted = 0;
    const double a_half = 0.5 * (a_old + a_new);
    nyxpm_step_info local;
    std::memset(&local, 0, sizeof(local));
    nyxpm_status st_old = NYXPM_OK, st_new;
    bool sorted_since = false;
    if (!reuse) {
        // nyxpm_step's old-time part, the sort leaving the velocities for later
        TRY(mixed ? mixed_sort(*c, *b, true) : launch_sort(*c, *b, true));
        sorted_since = true;
        TRY(mixed ? mixed_deposit(*c, *b) : launch_deposit(*c, *b));
        st_old = do_solve(*c, *b, a_old, 1, &local.old_solve);
        if (st_old != NYXPM_OK && st_old != NYXPM_NOT_CONVERGED) return st_old;
    }
    cudaStreamWaitEvent(c->stream, c->ev_copy_in, 0);
    TRY(mixed ? mixed_unpack_vel(*c, *b, s_vel, sorted_since)
              : launch_unpack_gather_vel(*c, *b, s_vel, sorted_since));
    TRY(do_kick(*c, *b, dt, a_old, a_half, 1, 0));
    // the positions are final now (the closing kick only wraps them, and not at
    // all in the mixed form): out on the copy stream under the new-time deposit
    // and solve
    TRY(mixed ? mixed_pack_pos(*c, *b, s_pos) : launch_pack_pos_wrapped(*c, *b, s_pos));
    cudaEventRecord(c->ev_copy_out, c->stream);
    cudaStreamWaitEvent(c->copy_stream, c->ev_copy_out, 0);
    cudaMemcpyAsync(pos, s_pos, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c->copy_stream);
    TRY(do_deposit(*c, *b));
    st_new = do_solve(*c, *b, a_new, 0, &local.new_solve);
    if (st_new != NYXPM_OK && st_new != NYXPM_NOT_CONVERGED) return st_new;
    TRY(do_kick(*c, *b, dt, a_half, a_new, 0, 1));
    TRY(mixed ? mixed_pack_vel(*c, *b, s_vel) : launch_pack_vel(*c, *b, s_vel));
    cudaMemcpyAsync(vel, s_vel, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(b->h_norms + 2, b->norms + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                    c->stream);
    TRY(check_launch(*c, "host step output copies"));
    const cudaError_t e1 = cudaStreamSynchronize(c->copy_stream);
    const cudaError_t e2 = cudaStreamSynchronize(c->stream);
    if (e1 != cudaSuccess || e2 != cudaSuccess)
        return fail(c, NYXPM_CUDA_ERROR, cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    if (b->h_norms[2] != 0) {
        b->uploaded = 0;
        return fail(c, NYXPM_INVALID_ARG, "non-finite particle position or velocity");
    }
    if (info) *info = local;
    return st_old != NYXPM_OK ? st_old : st_new;
}

double nyxpm_integrate_a(const nyxpm_params* p, double a_old, double dt)
{
    if (!p || p->comoving_h == 0.0) return a_old;
    const double H0 = p->comoving_h * 100.0;
    const double OmM = p->comoving_OmM, OmR = p->comoving_OmR;
    const double OmL = 1.0 - OmM - OmR;
    double prev = 2.0, a_new = a_old;
    for (int iter = 1; iter <= 11; ++iter) {
        const int nsteps = 1 << (iter - 1);
        const double Dt = dt / nsteps;
        double end_a = a_old;
        for (int j = 1; j <= nsteps; ++j) {
            const double start_a = end_a;
            const double s0 = adot(H0, OmM, OmR, OmL, start_a);
            end_a = start_a + s0 * Dt;
            const double s1 = adot(H0, OmM, OmR, OmL, end_a);
            end_a = start_a + 0.5 * (s0 + s1) * Dt;
        }
        a_new = end_a;
        if (std::fabs(1.0 - a_new / prev) <= 1.0e-8) return a_new;
        prev = a_new;
    }
    return a_new;
}

double nyxpm_dt_for_da(const nyxpm_params* p, double a_old, double a_value, double dt)
{
    if (!p) return dt;
    const double H0 = p->comoving_h * 100.0;
    const double OmM = p->comoving_OmM, OmR = p->comoving_OmR;
    const double OmL = 1.0 - OmM - OmR;
    const int nsteps = 2048;
    const double Dt = dt / nsteps;
    double end_a = a_old;
    for (int j = 1; j <= nsteps; ++j) {
        const double start_a = end_a;
        const double s0 = adot(H0, OmM, OmR, OmL, start_a);
        end_a = start_a + s0 * Dt;
        const double s1 = adot(H0, OmM, OmR, OmL, end_a);
        end_a = start_a + 0.5 * (s0 + s1) * Dt;
        if ((end_a - a_value) * (start_a - a_value) < 0)
            return ((end_a - a_value) * double(j) + (a_value - start_a) * double(j + 1)) /
                   (end_a - start_a) * Dt;
    }
    return dt;
}

// ---------------------------------------------------------------------------
// time-step control
// ---------------------------------------------------------------------------
void nyxpm_default_dt_params(nyxpm_dt_params* dp)
{
    if (!dp) return;
    dp->cfl = 0.5;
    dp->change_max = 1.1;
    dp->relative_max_change_a = 0.01;
    dp->absolute_max_change_a = -1.0;
    dp->final_a = -1.0;
    dp->stop_time = -1.0;
    dp->dt_binpow = -1.0;
}

nyxpm_status nyxpm_est_time_step(nyxpm_ctx* c, nyxpm_box* b, double cfl, double a, double* dt)
{
    CHECK_BOX(c, b);
    if (!dt) return fail(c, NYXPM_INVALID_ARG, "null dt");
    if (!(cfl > 0) || !(a > 0)) return fail(c, NYXPM_INVALID_ARG, "cfl and a must be positive");
    if (!b->uploaded || b->np == 0) {
        *dt = -1.0e50;  // no particles at this level (NyxParticleContainer.H:455)
        return NYXPM_OK;
    }
    if (!b->have_phi && !b->g_from_caller)
        return fail(c, NYXPM_INVALID_ARG, "no field: solve, step, set phi or set the gravity vector first");
    TRY(b->prec == NYXPM_MIXED ? mixed_est_dt(*c, *b, cfl, a) : launch_est_dt(*c, *b, cfl, a));
    cudaMemcpyAsync(b->h_norms + 3, b->norms + 3, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                    c->stream);
    TRY(check_launch(*c, "time-step readback"));
    TRY(nyxpm_synchronize(c));
    const unsigned long long bits = ~b->h_norms[3];
    std::memcpy(dt, &bits, sizeof(double));
    return NYXPM_OK;
}

namespace {

// est_maxdt_comoving_a (comoving.cpp:191-215): at most a 5% change of a per
// forward-Euler step
double cap_dt_by_hubble(const nyxpm_params* p, double a, double dt)
{
    const double H0 = p->comoving_h * 100.0;
    if (H0 == 0.0) return dt;
    const double OmL = 1.0 - p->comoving_OmM - p->comoving_OmR;
    const double a3 = a * a * a;
    const double lim = 0.05 / H0 / std::sqrt(p->comoving_OmM / a3 + p->comoving_OmR / (a3 * a) + OmL);
    return std::min(dt, lim);
}

// est_lindt_comoving_a (comoving.cpp:217-237)
double linear_dt_guess(const nyxpm_params* p, double a_from, double a_to, double dt)
{
    const double H0 = p->comoving_h * 100.0;
    if (H0 == 0.0) return dt;
    const double s = std::pow(0.75, 2.0 / 3.0);
    return (std::pow(a_to / s, 0.75) - std::pow(a_from / s, 0.75)) / H0;
}

}  // namespace

nyxpm_status nyxpm_comoving_est_dt(const nyxpm_params* p, double a, double estdt,
                                   const nyxpm_dt_params* dp, double* out)
{
    if (!p || !dp || !out) return NYXPM_INVALID_ARG;
    if (p->comoving_h == 0.0) {
        *out = estdt;
        return NYXPM_OK;
    }
    // estdt_comoving_a (comoving.cpp:239-280)
    double dt = estdt, a_next;
    if (dp->absolute_max_change_a <= 0.0) {
        dt = cap_dt_by_hubble(p, a, dt);
        a_next = nyxpm_integrate_a(p, a, dt);
        // enforce_percent_change (comoving.cpp:282-317)
        if (((a_next - a) / a) / dp->relative_max_change_a > 1.0) {
            for (int it = 1; it <= 100; ++it) {
                const double factor = ((a_next - a) / a) / dp->relative_max_change_a;
                if (factor > 1.0) {
                    dt = (1.0 / factor) * dt * 0.99;
                    a_next = nyxpm_integrate_a(p, a, dt);
                } else if (it < 100) {
                    a_next = nyxpm_integrate_a(p, a, dt);
                    break;
                } else {
                    return NYXPM_INVALID_ARG;  // the reference aborts here
                }
            }
        }
    } else {
        a_next = a + dp->absolute_max_change_a;
        dt = linear_dt_guess(p, a, a_next, dt);
        dt = cap_dt_by_hubble(p, a, dt);
        dt = nyxpm_dt_for_da(p, a, a_next, dt);
    }
    // enforce_final_a (comoving.cpp:319-350)
    if (dp->final_a > 0.0) {
        if (a > dp->final_a) return NYXPM_INVALID_ARG;
        if (a_next > dp->final_a) {
            for (int it = 1; it <= 100; ++it) {
                if (a_next > dp->final_a + 1.0e-10 || a_next < dp->final_a) {
                    dt = dt * ((dp->final_a - a) / (a_next - a));
                    a_next = nyxpm_integrate_a(p, a, dt);
                } else if (it < 100) {
                    break;
                } else {
                    return NYXPM_INVALID_ARG;  // the reference aborts here
                }
            }
        }
    }
    // comoving_est_time_step (comoving.cpp:353-483): power-of-two binning or min
    if (dp->dt_binpow >= 0) {
        if (estdt >= dt) {
            estdt = dt;
        } else {
            double frac = 0.5;
            for (; frac >= 0.0625; frac *= 0.5)
                if (estdt > frac * dt) break;
            estdt = frac >= 0.0625 ? frac * dt : dt * std::pow(2.0, -std::ceil(std::log2(dt / estdt)));
        }
    } else {
        estdt = std::min(estdt, dt);
    }
    *out = estdt;
    return NYXPM_OK;
}

nyxpm_status nyxpm_compute_new_dt(nyxpm_ctx* c, nyxpm_box* b, const nyxpm_dt_params* dp,
                                  double time, double a, double dt_old, double* dt_new,
                                  double* a_new)
{
    CHECK_BOX(c, b);
    if (!dp || !dt_new) return fail(c, NYXPM_INVALID_ARG, "null argument");
    // Nyx::est_time_step (Nyx.cpp:912-1020): particles, then the a-change limit
    double est = 1.0e200;
    double part = 0;
    TRY(nyxpm_est_time_step(c, b, dp->cfl, a, &part));
    if (part > 0) est = std::min(est, part);
    if (nyxpm_comoving_est_dt(&c->p, a, est, dp, &est) != NYXPM_OK)
        return fail(c, NYXPM_INVALID_ARG, "comoving time-step limit did not converge or a > final_a");
    // computeNewDt (Nyx.cpp:1023-1208), one level, no subcycling
    if (dt_old > 0) est = std::min(est, dp->change_max * dt_old);
    if (dp->stop_time >= 0.0) {
        const double eps = 0.001 * est;
        if (time + est > dp->stop_time - eps) est = dp->stop_time - time;
    }
    *dt_new = est;
    if (a_new) *a_new = nyxpm_integrate_a(&c->p, a, est);
    return NYXPM_OK;
}

nyxpm_status nyxpm_set_profiling(nyxpm_ctx* c, int on)
{
    CHECK_CTX(c);
    if (on && c->ev_a.empty()) {
        c->ev_a.resize(kProfEvents);
        c->ev_b.resize(kProfEvents);
        for (int i = 0; i < kProfEvents; ++i) {
            if (cudaEventCreate(&c->ev_a[i]) != cudaSuccess || cudaEventCreate(&c->ev_b[i]) != cudaSuccess)
                return fail(c, NYXPM_CUDA_ERROR, "cudaEventCreate");
        }
    }
    c->prof_on = on ? 1 : 0;
    return NYXPM_OK;
}

nyxpm_status nyxpm_get_profile(nyxpm_ctx* c, nyxpm_profile* out, int reset)
{
    CHECK_CTX(c);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(c, NYXPM_CUDA_ERROR, cudaGetErrorString(e));
    for (size_t i = 0; i < c->recs.size(); ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev_a[i], c->ev_b[i]);
        const ProfRec& r = c->recs[i];
        c->acc.launches[r.stage] += 1;
        c->acc.ms[r.stage] += ms;
        c->acc.bytes[r.stage] += r.bytes;
        if (r.fine && r.stage == NYXPM_ST_SMOOTH) {
            c->acc.fine_smooth_launches += 1;
            c->acc.fine_smooth_ms += ms;
            c->acc.fine_smooth_bytes += r.bytes;
        }
    }
    c->recs.clear();
    if (out) *out = c->acc;
    if (reset) std::memset(&c->acc, 0, sizeof(c->acc));
    return NYXPM_OK;
}

}  // extern "C"
