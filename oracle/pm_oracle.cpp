// CPU FP64 oracle for the Nyx particle-mesh (PM) gravity step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library's
// results are compared against, and the CPU baseline that bench.py times.  The
// product (nyx_gb300/libnyxpm.so) never links, loads or calls it.
//
// It restates, in plain C++ with OpenMP, the single-level periodic
// dark-matter-only PM step of Nyx (reference tree paths, no prefix):
//   * counting sort by deposit cell      -- stands in for RedistributeLocal,
//                                           Source/Driver/Nyx.cpp:1421-1437
//   * CIC deposit                        -- Source/Particle/NeutrinoParticleContainer.cpp:209-302
//                                           with the weights of NeutrinoParticles_K.H:16-45
//                                           (gamma = 1: the non-relativistic deposit)
//   * RHS = -4 pi G (rho - rho_bar - mean) / a
//                                        -- Source/Gravity/Gravity.cpp:267-315, 1207-1244,
//                                           705-753, Source/Driver/sum_utils.cpp:21-97
//   * periodic Poisson solve             -- geometric multigrid V-cycles with red-black
//                                           Gauss-Seidel; Gravity.cpp:1318-1416 hands this to
//                                           AMReX MLMG, whose source is not in the tree
//   * cell-centred gravity vector        -- face gradient averaged to cell centres,
//                                           Gravity.cpp:781-850
//   * CIC interpolation + kick (+ drift) -- Source/Particle/DarkMatterParticleContainer.cpp:250-306
//   * step order                         -- Source/TimeStep/Nyx_advance_particles.cpp:137-268
//   * a(t)                               -- Source/Driver/comoving.cpp:74-130, 629-688
//
// The AMReX pieces (deposit summation order, the MLMG schedule) cannot be read
// in the reference tree.  The oracle fixes them to one deterministic definition
// that the GPU library implements as well:
//   * deposit: rho(c) = inv_vol * sum over the 8 deposit keys K of c, in the
//     order (dk,dj,di) = (0,0,0),(0,0,1),...,(1,1,1), of the sum over the
//     particles of K of ((sx*sy)*sz)*m -- sequential in sorted order for up to
//     32 particles, else 32 lane-strided sequential partials combined by an
//     xor butterfly (the order one warp sums a long key in);
//   * mean: row sums by 32 strided lane partials and a halving tree, then a
//     sequential sum over rows of a plane, then over planes;
//   * MG: V(nu1,nu2) cycles, red then black, full-weighting (8-cell average)
//     restriction, trilinear cell-centred prolongation, exact bottom solve by the
//     circulant pseudo-inverse on the coarsest grid (n <= 8), stop when
//     ||r||_inf <= rel_tol * max(||rhs||_inf, ||r0||_inf).
//
// All floating-point expressions are written out in a fixed order and the file
// is built with -ffp-contract=off so that no multiply-add is fused.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// ----------------------------------------------------------------------------
// constants (Source/Driver/constants_cosmo.H:7-16, 38)
// ----------------------------------------------------------------------------
double orc_gconst(void)
{
    const double M_unit = 1.98848e33;
    const double L_unit = 3.0856776e24;
    const double V_unit = 1.e5;
    const double T_unit = L_unit / V_unit;
    return 6.67408e-8 * M_unit * T_unit * T_unit / (L_unit * L_unit * L_unit);
}

double orc_hubble_const(void) { return 100.0; }

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int t)
{
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

} // extern "C"

namespace {

inline int wrapi(int i, int n) { i %= n; return i < 0 ? i + n : i; }

inline long cidx(int i, int j, int k, int n) { return (long)i + (long)n * ((long)j + (long)n * k); }

// keys with more particles than this sum them in lane-strided partials
constexpr int kDepositLanes = 32;

// deposit key of one coordinate: floor((x - plo) * dxi + 0.5), plo = 0
// (NeutrinoParticles_K.H:15-21, DarkMatterParticleContainer.cpp:263-269),
// the product and the sum fused into one multiply-add
inline int key1(double x, double dxi, int n, double* frac)
{
    double l = std::fma(x, dxi, 0.5);
    int i = (int)std::floor(l);
    *frac = l - i;
    return wrapi(i, n);
}

} // namespace

extern "C" {

// ----------------------------------------------------------------------------
// periodic shift of positions into [0, L)  (AMReX periodic shift in
// RedistributeLocal, called from Nyx.cpp:1426)
// ----------------------------------------------------------------------------
void orc_wrap(double L, long np, double* x, double* y, double* z)
{
    double* c[3] = {x, y, z};
    for (int d = 0; d < 3; ++d) {
        double* p = c[d];
#pragma omp parallel for schedule(static)
        for (long q = 0; q < np; ++q) {
            double v = p[q];
            if (v >= L) v = v - L; else if (v < 0.0) v = v + L;
            if (v >= L) v = 0.0;
            p[q] = v;
        }
    }
}

// ----------------------------------------------------------------------------
// stable counting sort of the particles by deposit key.
// cell_start has n^3 + 1 entries; particles of key K occupy
// [cell_start[K], cell_start[K+1]).  Stable: equal keys keep their order.
// ----------------------------------------------------------------------------
int orc_sort(int n, double L, long np, double* x, double* y, double* z,
             double* vx, double* vy, double* vz, double* m, int* id, int* cell_start)
{
    const long nc = (long)n * n * n;
    const double dxi = (double)n / L;
    std::vector<int> key(np);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < np; ++q) {
        double f;
        int i = key1(x[q], dxi, n, &f);
        int j = key1(y[q], dxi, n, &f);
        int k = key1(z[q], dxi, n, &f);
        key[q] = (int)cidx(i, j, k, n);
    }
    std::vector<long> cnt(nc + 1, 0);
    for (long q = 0; q < np; ++q) cnt[key[q] + 1]++;
    for (long c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    for (long c = 0; c <= nc; ++c) cell_start[c] = (int)cnt[c];
    std::vector<long> perm(np);
    for (long q = 0; q < np; ++q) perm[cnt[key[q]]++] = q;
    double* arrs[7] = {x, y, z, vx, vy, vz, m};
    std::vector<double> tmp(np);
    for (int a = 0; a < 7; ++a) {
        if (!arrs[a]) continue;
        double* p = arrs[a];
#pragma omp parallel for schedule(static)
        for (long q = 0; q < np; ++q) tmp[q] = p[perm[q]];
        std::memcpy(p, tmp.data(), sizeof(double) * np);
    }
    if (id) {
        std::vector<int> t(np);
        for (long q = 0; q < np; ++q) t[q] = id[perm[q]];
        std::memcpy(id, t.data(), sizeof(int) * np);
    }
    return 0;
}

// ----------------------------------------------------------------------------
// CIC deposit (AssignDensitySingleLevel).  Particles must be sorted by key
// (orc_sort).  m == NULL means every particle has mass mscalar.
// Per particle: l = x*dxi + 0.5, i = floor(l), f = l - i, weights
// sx = {1-f, f} on cells {i-1, i}, w = (sx*sy)*sz (NeutrinoParticles_K.H:15-45).
// Per-particle masses: the key sums w*m (fused), the cell sum is scaled by
// 1/dx^3 (NeutrinoParticleContainer.cpp:300-302).  Uniform mass: the key sums w
// and the cell sum is scaled once by m/dx^3.
// ----------------------------------------------------------------------------
void orc_deposit(int n, double L, long np, const double* x, const double* y, const double* z,
                 const double* m, double mscalar, const int* cell_start, double* rho)
{
    (void)np;
    const long nc = (long)n * n * n;
    const double dx = L / n;
    const double dxi = (double)n / L;
    const double inv_vol = 1.0 / (dx * dx * dx);
    const double scale = m ? inv_vol : mscalar * inv_vol;
    // per-key partial sums: part[K*8 + corner], corner = cx + 2*cy + 4*cz where
    // cx = 0 is the cell i-1 (weight 1-f) and cx = 1 the cell i (weight f).
    // A key of at most kDepositLanes particles sums them in sorted order.  A
    // longer key sums in kDepositLanes lane partials -- lane l takes particles
    // l, l + 32, l + 64, ... in order -- combined by the xor butterfly: for
    // off = 16, 8, 4, 2, 1 every lane adds the partial of lane l ^ off.
    std::vector<double> part(nc * 8);
    auto accumulate = [&](int q, double* s) {
        double fx, fy, fz;
        key1(x[q], dxi, n, &fx);
        key1(y[q], dxi, n, &fy);
        key1(z[q], dxi, n, &fz);
        const double sx[2] = {1.0 - fx, fx};
        const double sy[2] = {1.0 - fy, fy};
        const double sz[2] = {1.0 - fz, fz};
        for (int cz = 0; cz < 2; ++cz)
            for (int cy = 0; cy < 2; ++cy)
                for (int cx = 0; cx < 2; ++cx) {
                    const double w = (sx[cx] * sy[cy]) * sz[cz];
                    double& a = s[cx + 2 * cy + 4 * cz];
                    a = m ? std::fma(w, m[q], a) : a + w;
                }
    };
#pragma omp parallel for schedule(dynamic, 64)
    for (long K = 0; K < nc; ++K) {
        const int s0 = cell_start[K], e = cell_start[K + 1];
        double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (e - s0 <= kDepositLanes) {
            for (int q = s0; q < e; ++q) accumulate(q, s);
        } else {
            double lane[kDepositLanes][8] = {};
            for (int l = 0; l < kDepositLanes; ++l)
                for (int q = s0 + l; q < e; q += kDepositLanes) accumulate(q, lane[l]);
            for (int off = kDepositLanes / 2; off >= 1; off >>= 1) {
                double nxt[kDepositLanes][8];
                for (int l = 0; l < kDepositLanes; ++l)
                    for (int c = 0; c < 8; ++c) nxt[l][c] = lane[l][c] + lane[l ^ off][c];
                std::memcpy(lane, nxt, sizeof(lane));
            }
            for (int c = 0; c < 8; ++c) s[c] = lane[0][c];
        }
        for (int c = 0; c < 8; ++c) part[K * 8 + c] = s[c];
    }
    // cell c receives from key K = c + d (d in {0,1}^3) the corner (1-dx, 1-dy, 1-dz)
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                double acc = 0.0;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di) {
                            long K = cidx(wrapi(i + di, n), wrapi(j + dj, n), wrapi(k + dk, n), n);
                            int corner = (1 - di) + 2 * (1 - dj) + 4 * (1 - dk);
                            acc = acc + part[K * 8 + corner];
                        }
                rho[cidx(i, j, k, n)] = acc * scale;
            }
}

// ----------------------------------------------------------------------------
// canonical sum of a cell field (the fixed reduction tree shared with the GPU)
// ----------------------------------------------------------------------------
double orc_canonical_sum(int n, const double* f)
{
    std::vector<double> rows((long)n * n);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)n * n; ++r) {
        double p[32];
        for (int l = 0; l < 32; ++l) {
            double s = 0.0;
            for (int i = l; i < n; i += 32) s = s + f[r * n + i];
            p[l] = s;
        }
        for (int off = 16; off >= 1; off >>= 1)
            for (int l = 0; l < off; ++l) p[l] = p[l] + p[l + off];
        rows[r] = p[0];
    }
    std::vector<double> planes(n);
    for (int k = 0; k < n; ++k) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s = s + rows[(long)k * n + j];
        planes[k] = s;
    }
    double s = 0.0;
    for (int k = 0; k < n; ++k) s = s + planes[k];
    return s;
}

// ----------------------------------------------------------------------------
// RHS of the comoving Poisson equation (Gravity.cpp:267-290, 1207-1244):
// rhs = (((rho - mass_offset) - mean) * Ggravity) * (1/a),
// mean = (S * dx^3) / L^3, S the canonical sum of (rho - mass_offset).
// Returns the mean that was subtracted.
// ----------------------------------------------------------------------------
double orc_make_rhs(int n, double L, const double* rho, double mass_offset, double ggrav,
                    double a, double* rhs)
{
    const long nc = (long)n * n * n;
    const double dx = L / n;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c) rhs[c] = rho[c] - mass_offset;
    const double S = orc_canonical_sum(n, rhs);
    const double mean = (S * (dx * dx * dx)) / (L * L * L);
    const double ainv = 1.0 / a;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c) rhs[c] = ((rhs[c] - mean) * ggrav) * ainv;
    return mean;
}

} // extern "C"

// ----------------------------------------------------------------------------
// multigrid
// ----------------------------------------------------------------------------
namespace {

struct Level {
    int n;
    std::vector<double> phi;
    std::vector<double> beta;   // right-hand side in smoother units: h^2 rhs / 6
};

inline double nbr_sum(const double* p, int i, int j, int k, int n)
{
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    double s = p[cidx(im, j, k, n)] + p[cidx(ip, j, k, n)];
    s = s + p[cidx(i, jm, k, n)];
    s = s + p[cidx(i, jp, k, n)];
    s = s + p[cidx(i, j, km, n)];
    s = s + p[cidx(i, j, kp, n)];
    return s;
}

const double kSixth = 1.0 / 6.0;

// one red-black sweep: red cells ((i+j+k) even) then black;
// phi = s/6 - beta with s the sum of the 6 neighbours (one fused multiply-add)
void gsrb(Level& lv)
{
    const int n = lv.n;
    double* p = lv.phi.data();
    const double* b = lv.beta.data();
    for (int color = 0; color < 2; ++color) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j)
                for (int i = (j + k + color) & 1; i < n; i += 2) {
                    const double s = nbr_sum(p, i, j, k, n);
                    p[cidx(i, j, k, n)] = std::fma(s, kSixth, -b[cidx(i, j, k, n)]);
                }
    }
}

// residual in smoother units: beta - (s/6 - phi)  ( = h^2/6 (rhs - lap phi) )
inline double resid_at(const Level& lv, int i, int j, int k)
{
    const int n = lv.n;
    const double* p = lv.phi.data();
    const double s = nbr_sum(p, i, j, k, n);
    return lv.beta[cidx(i, j, k, n)] - std::fma(s, kSixth, -p[cidx(i, j, k, n)]);
}

// ||r_beta||_inf over all cells (red_only = 0) or over the red cells only
// (red_only = 1: after a V-cycle that ends with a black half sweep the black
// residuals are round-off by construction and are not scanned)
double resid_norm(const Level& lv, int red_only)
{
    const int n = lv.n;
    double mx = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mx)
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = red_only ? ((j + k) & 1) : 0; i < n; i += red_only ? 2 : 1) {
                double v = std::fabs(resid_at(lv, i, j, k));
                if (v > mx) mx = v;
            }
    return mx;
}

double inf_norm(const double* f, long nc)
{
    double mx = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mx)
    for (long c = 0; c < nc; ++c) {
        double v = std::fabs(f[c]);
        if (v > mx) mx = v;
    }
    return mx;
}

// coarse beta = 1/2 of the sum of the 8 fine residuals (summed dk, dj, di):
// the 8-cell average of rhs - lap phi, rescaled by h_c^2/6 = 4 h_f^2/6.
// red_only = 1 (the level was just pre-smoothed, ending with a black half
// sweep): the black children's residuals are round-off by construction and are
// taken as 0, so only the 4 red children (di + dj + dk even) are summed, in the
// same (dk, dj, di) order.
void restrict_resid(const Level& f, Level& c, int red_only)
{
    const int nc = c.n;
#pragma omp parallel for schedule(static)
    for (int K = 0; K < nc; ++K)
        for (int J = 0; J < nc; ++J)
            for (int I = 0; I < nc; ++I) {
                double s = 0.0;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di)
                            if (!red_only || ((di + dj + dk) & 1) == 0)
                                s = s + resid_at(f, 2 * I + di, 2 * J + dj, 2 * K + dk);
                c.beta[cidx(I, J, K, nc)] = s * 0.5;
            }
}

// trilinear cell-centred prolongation weights (3/4, 1/4 per axis; exact in binary),
// indexed t + 2a + 4b with t, a, b selecting (parent, neighbour) along x, y, z
const double kProlongW[8] = {0.421875, 0.140625, 0.140625, 0.046875,
                             0.140625, 0.046875, 0.046875, 0.015625};

void prolong_add(const Level& c, Level& f)
{
    const int n = f.n, nc = c.n;
    const double* e = c.phi.data();
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int I = i >> 1, J = j >> 1, K = k >> 1;
                const int I1 = wrapi((i & 1) ? I + 1 : I - 1, nc);
                const int J1 = wrapi((j & 1) ? J + 1 : J - 1, nc);
                const int K1 = wrapi((k & 1) ? K + 1 : K - 1, nc);
                const int Is[2] = {I, I1}, Js[2] = {J, J1}, Ks[2] = {K, K1};
                double s = 0.0;
                for (int b = 0; b < 2; ++b)
                    for (int a = 0; a < 2; ++a)
                        for (int t = 0; t < 2; ++t)
                            s = std::fma(kProlongW[t + 2 * a + 4 * b], e[cidx(Is[t], Js[a], Ks[b], nc)], s);
                f.phi[cidx(i, j, k, n)] = f.phi[cidx(i, j, k, n)] + s;
            }
}

} // namespace

extern "C" {

// Green's function of the periodic 7-point Laplacian on an nb^3 grid with
// spacing h, projected off the constant mode, in smoother units (applied to
// beta = h^2 rhs / 6):
// G(d) = (6/h^2) (1/nb^3) sum_{kappa != 0} cos(2 pi kappa.d / nb) / lambda(kappa),
// lambda = sum_d (2 cos(2 pi kappa_d / nb) - 2) / h^2.
void orc_bottom_green(int nb, double h, double* G)
{
    const long nc = (long)nb * nb * nb;
    const double twopi = 2.0 * std::acos(-1.0);
    std::vector<double> lam(nc);
    for (int kz = 0; kz < nb; ++kz)
        for (int ky = 0; ky < nb; ++ky)
            for (int kx = 0; kx < nb; ++kx) {
                double l = (2.0 * std::cos(twopi * kx / nb) - 2.0) + (2.0 * std::cos(twopi * ky / nb) - 2.0)
                         + (2.0 * std::cos(twopi * kz / nb) - 2.0);
                lam[cidx(kx, ky, kz, nb)] = l / (h * h);
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
                            s += std::cos(twopi * (double)ph / nb) / lam[cidx(kx, ky, kz, nb)];
                        }
                G[cidx(dxx, dy, dz, nb)] = (s / (double)nc) * scale;
            }
}

} // extern "C"

namespace {

// exact coarsest solve: phi = G * beta (cyclic convolution, y in storage order)
void bottom_solve(Level& lv, const std::vector<double>& G)
{
    const int n = lv.n;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                double s = 0.0;
                for (int yk = 0; yk < n; ++yk)
                    for (int yj = 0; yj < n; ++yj)
                        for (int yi = 0; yi < n; ++yi) {
                            const long d = cidx(wrapi(i - yi, n), wrapi(j - yj, n), wrapi(k - yk, n), n);
                            s = std::fma(G[d], lv.beta[cidx(yi, yj, yk, n)], s);
                        }
                lv.phi[cidx(i, j, k, n)] = s;
            }
}

struct Hierarchy {
    std::vector<Level> lv;
    std::vector<double> G;
};

bool build_hierarchy(int n, double L, Hierarchy& H)
{
    int m = n;
    while (m % 2 == 0 && m > 4) m /= 2;
    if (m > 8 || n < 2) return false;
    for (int nl = n;; nl /= 2) {
        Level l;
        l.n = nl;
        l.phi.assign((long)nl * nl * nl, 0.0);
        l.beta.assign((long)nl * nl * nl, 0.0);
        H.lv.push_back(std::move(l));
        if (nl == m) break;
    }
    H.G.resize((long)m * m * m);
    orc_bottom_green(m, L / m, H.G.data());
    return true;
}

void vcycle(Hierarchy& H, size_t l, int nu1, int nu2)
{
    Level& f = H.lv[l];
    if (l + 1 == H.lv.size()) { bottom_solve(f, H.G); return; }
    for (int s = 0; s < nu1; ++s) gsrb(f);
    Level& c = H.lv[l + 1];
    restrict_resid(f, c, nu1 > 0 ? 1 : 0);
    std::fill(c.phi.begin(), c.phi.end(), 0.0);
    vcycle(H, l + 1, nu1, nu2);
    prolong_add(c, f);
    for (int s = 0; s < nu2; ++s) gsrb(f);
}

} // namespace

extern "C" {

// Number of levels of the hierarchy for an n^3 grid: halve while the edge is even
// and above 4; the coarsest edge must be <= 8 (0 if n is not m*2^k with m <= 8).
int orc_mg_levels(int n)
{
    int m = n, L = 1;
    while (m % 2 == 0 && m > 4) { m /= 2; ++L; }
    return (m > 8 || n < 2) ? 0 : L;
}

// Scale factor from rhs to smoother units on an n^3 grid of side L: (h*h)*(1/6).
double orc_beta_scale(int n, double L)
{
    const double h = L / n;
    return (h * h) * kSixth;
}

// Solve lap(phi) = rhs (periodic, 7-point) by V-cycles from the initial guess in
// phi.  The convergence test is done in smoother units,
// ||r_beta||_inf <= rel_tol * max(||beta||_inf, ||r_beta0||_inf), the norm after
// each cycle taken over the red cells (see resid_norm); the norms are reported
// in rhs units (divided by the scale).  Returns 0 when converged, 4 when
// max_cycles was reached, 1 on bad n.
int orc_mg_solve(int n, double L, const double* rhs, double* phi, double rel_tol, int max_cycles,
                 int nu1, int nu2, int* ncycles, double* resnorm0, double* resnorm)
{
    Hierarchy H;
    if (!build_hierarchy(n, L, H)) return 1;
    const long nc = (long)n * n * n;
    Level& f = H.lv[0];
    const double k0 = orc_beta_scale(n, L);
    const double inv_k0 = 1.0 / k0;
    for (long c = 0; c < nc; ++c) f.beta[c] = rhs[c] * k0;
    std::memcpy(f.phi.data(), phi, sizeof(double) * nc);
    const double bnorm = inf_norm(f.beta.data(), nc);
    const double r0 = resid_norm(f, 0);
    // post-cycle norms scan the red cells when the cycle ends with a black half
    // sweep on a smoothed (even) finest level
    const int red_only = (nu2 > 0 && H.lv.size() > 1) ? 1 : 0;
    const double target = rel_tol * std::max(bnorm, r0);
    double r = r0;
    int it = 0;
    int status = 0;
    if (r0 > target) {
        for (it = 1; it <= max_cycles; ++it) {
            vcycle(H, 0, nu1, nu2);
            r = resid_norm(f, red_only);
            if (r <= target) break;
        }
        if (it > max_cycles) { it = max_cycles; status = 4; }
    }
    std::memcpy(phi, f.phi.data(), sizeof(double) * nc);
    if (ncycles) *ncycles = it;
    if (resnorm0) *resnorm0 = r0 * inv_k0;
    if (resnorm) *resnorm = r * inv_k0;
    return status;
}

// One V(nu1,nu2) cycle of the periodic hierarchy from a zero initial guess for
// the right-hand side beta given in smoother units (n^3, natural order); the
// result in e.  The base level's correction solve of the multilevel (AMR)
// composite V-cycle.  Returns 1 on bad n.
int orc_mg_vcycle_zero(int n, double L, const double* beta, double* e, int nu1, int nu2)
{
    // the hierarchy of the last (n, L), kept between calls (one V-cycle per call)
    static Hierarchy H;
    static int Hn = 0;
    static double HL = 0.0;
    if (Hn != n || HL != L) {
        H = Hierarchy();
        Hn = 0;
        if (!build_hierarchy(n, L, H)) return 1;
        Hn = n;
        HL = L;
    }
    const long nc = (long)n * n * n;
    std::memcpy(H.lv[0].beta.data(), beta, sizeof(double) * nc);
    std::fill(H.lv[0].phi.begin(), H.lv[0].phi.end(), 0.0);
    vcycle(H, 0, nu1, nu2);
    std::memcpy(e, H.lv[0].phi.data(), sizeof(double) * nc);
    return 0;
}

// Cell-centred gravity vector g = average of the two face gradients
// (Gravity.cpp:817-850): g_d(c) = 0.5*((phi_c - phi_{c-e_d})*dxi + (phi_{c+e_d} - phi_c)*dxi),
// the second product fused with the sum.  g holds the three components one
// after another (component-major).
void orc_grav_vector(int n, double L, const double* phi, double* g)
{
    const long nc = (long)n * n * n;
    const double dxi = (double)n / L;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const long c = cidx(i, j, k, n);
                const double pc = phi[c];
                const long xm = cidx(wrapi(i - 1, n), j, k, n), xp = cidx(wrapi(i + 1, n), j, k, n);
                const long ym = cidx(i, wrapi(j - 1, n), k, n), yp = cidx(i, wrapi(j + 1, n), k, n);
                const long zm = cidx(i, j, wrapi(k - 1, n), n), zp = cidx(i, j, wrapi(k + 1, n), n);
                g[c] = 0.5 * std::fma(phi[xp] - pc, dxi, (pc - phi[xm]) * dxi);
                g[nc + c] = 0.5 * std::fma(phi[yp] - pc, dxi, (pc - phi[ym]) * dxi);
                g[2 * nc + c] = 0.5 * std::fma(phi[zp] - pc, dxi, (pc - phi[zm]) * dxi);
            }
}

// update_dm_particle_single (DarkMatterParticleContainer.cpp:250-306) over all
// particles, with the acceleration field g (component-major, periodic):
// l = x*dxi + 1/2 (fused), i = floor(l), weights w = (sx*sy)*sz of the 8 cells
// (i-ii, j-jj, k-kk) in the order kk, jj, ii; val_d = sum w*g_d (fused);
// v = (a_prev*v + dt/2*val) / a_cur (the first product fused); x += dt/a_cur*v (fused).
void orc_move(int n, double L, long np, double* x, double* y, double* z, double* vx, double* vy,
              double* vz, const double* g, double dt, double a_prev, double a_cur, int do_move)
{
    const long nc = (long)n * n * n;
    const double dxi = (double)n / L;
    const double half_dt = 0.5 * dt;
    const double a_cur_inv = 1.0 / a_cur;
    const double dt_a_cur_inv = dt * a_cur_inv;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < np; ++q) {
        const double lx = std::fma(x[q], dxi, 0.5);
        const double ly = std::fma(y[q], dxi, 0.5);
        const double lz = std::fma(z[q], dxi, 0.5);
        const double fi = std::floor(lx), fj = std::floor(ly), fk = std::floor(lz);
        const int i = (int)fi, j = (int)fj, k = (int)fk;
        const double xint = lx - fi, yint = ly - fj, zint = lz - fk;
        const double sx[2] = {1.0 - xint, xint};
        const double sy[2] = {1.0 - yint, yint};
        const double sz[2] = {1.0 - zint, zint};
        double w[8];
        long cells[8];
        for (int kk = 0; kk <= 1; ++kk)
            for (int jj = 0; jj <= 1; ++jj)
                for (int ii = 0; ii <= 1; ++ii) {
                    const int t = ii + 2 * jj + 4 * kk;
                    w[t] = (sx[1 - ii] * sy[1 - jj]) * sz[1 - kk];
                    cells[t] = cidx(wrapi(i - ii, n), wrapi(j - jj, n), wrapi(k - kk, n), n);
                }
        double* v[3] = {vx + q, vy + q, vz + q};
        for (int d = 0; d < 3; ++d) {
            double val = 0.0;
            for (int t = 0; t < 8; ++t) val = std::fma(w[t], g[d * nc + cells[t]], val);
            const double u = std::fma(a_prev, *v[d], half_dt * val);
            *v[d] = u * a_cur_inv;
        }
        if (do_move == 1) {
            x[q] = std::fma(dt_a_cur_inv, vx[q], x[q]);
            y[q] = std::fma(dt_a_cur_inv, vy[q], y[q]);
            z[q] = std::fma(dt_a_cur_inv, vz[q], z[q]);
        }
    }
}

// ----------------------------------------------------------------------------
// a(t) (comoving.cpp).  comoving_type > 0 (the cosmological branch).
// ----------------------------------------------------------------------------
static inline double adot(double H0, double OmM, double OmR, double OmL, double a)
{
    return H0 * std::sqrt(OmM / a + OmR / (a * a) + OmL * a * a);
}

// integrate_comoving_a(old_a, new_a, dt): RK2 with step doubling to 1e-8
// (comoving.cpp:629-688)
double orc_integrate_a(double OmM, double OmR, double h, double a_old, double dt)
{
    if (h == 0.0) return a_old;
    const double H0 = h * 100.0;
    const double OmL = 1.0 - OmM - OmR;
    double prev = 2.0, a_new = a_old;
    for (int iter = 1; iter <= 11; ++iter) {
        const int nsteps = (int)std::lround(std::pow(2.0, iter - 1));
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

// integrate_comoving_a_to_a(old_a, a_value, dt): 2048 RK2 substeps of dt/2048,
// dt interpolated where a crosses a_value (comoving.cpp:74-130).  dt is the
// search window; it is returned unchanged if a_value is not reached.
double orc_dt_for_da(double OmM, double OmR, double h, double a_old, double a_value, double dt)
{
    const double H0 = h * 100.0;
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
        if ((end_a - a_value) * (start_a - a_value) < 0) {
            return ((end_a - a_value) * double(j) + (a_value - start_a) * double(j + 1)) / (end_a - start_a) * Dt;
        }
    }
    return dt;
}

// ----------------------------------------------------------------------------
// one-particle-per-cell cosmological ICs, InitCosmo1ppcMultiLevel on one level
// (DarkMatterParticleContainer.cpp:309-450): the particle of cell (i,j,k) at
// the cell centre plus disp * disp_fac (positions :376-386), shifted
// periodically into [0, L); velocity vel * vel_fac.  disp, vel: 3 n^3,
// component-major, x fastest.  pos/vel out: n^3 x 3.
// ----------------------------------------------------------------------------
void orc_cosmo_1ppc(int n, double L, const double* disp, const double* vel, const double* disp_fac,
                    const double* vel_fac, double* pos, double* velo)
{
    const long nc = (long)n * n * n;
    const double dx = L / n;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const long c = cidx(i, j, k, n);
                const int ijk[3] = {i, j, k};
                for (int d = 0; d < 3; ++d) {
                    double x = (ijk[d] + 0.5) * dx;
                    x = x + disp[d * nc + c] * disp_fac[d];
                    if (x >= L) x = x - L; else if (x < 0.0) x = x + L;
                    if (x >= L || x < 0.0) x = x - L * std::floor(x / L);
                    if (x >= L) x = 0.0;
                    pos[3 * c + d] = x;
                    velo[3 * c + d] = vel[d * nc + c] * vel_fac[d];
                }
            }
}

// ----------------------------------------------------------------------------
// time-step control
// ----------------------------------------------------------------------------

// Particle time-step limit, NyxParticleContainer::estTimestep
// (NyxParticleContainer.H:329-465): per particle
//   dt_p = cfl / max_d(|v_d| * (dxi / a))     (1e50 when all components are 0),
//   dt_p = min(dt_p, 1 / sqrt(|g| * dxi))    when |g| > 0,
// with |g| = sqrt((gx*gx + gy*gy) + gz*gz) taken at the cell floor(x * dxi)
// (no interpolation; the index wraps periodically, as the ghost cells of the
// reference's field do).  Returns the minimum over particles, 1e50 when no
// particle limits it and -1e50 when there are no particles.
double orc_est_time_step(int n, double L, long np, const double* x, const double* y,
                         const double* z, const double* vx, const double* vy, const double* vz,
                         const double* g, double cfl, double a)
{
    if (np <= 0) return -1.0e50;
    const long nc = (long)n * n * n;
    const double dxi = (double)n / L;
    const double adxi = dxi / a;
    double dt = 1.0e50;
#pragma omp parallel for schedule(static) reduction(min : dt)
    for (long q = 0; q < np; ++q) {
        const int i = wrapi((int)std::floor(x[q] * dxi), n);
        const int j = wrapi((int)std::floor(y[q] * dxi), n);
        const int k = wrapi((int)std::floor(z[q] * dxi), n);
        const double ux = std::fabs(vx[q]) * adxi;
        const double uy = std::fabs(vy[q]) * adxi;
        const double uz = std::fabs(vz[q]) * adxi;
        const double um = std::max(std::max(ux, uy), uz);
        double dtp = (um > 0) ? (cfl / um) : 1.0e50;
        const long c = cidx(i, j, k, n);
        const double gx = g[c], gy = g[nc + c], gz = g[2 * nc + c];
        const double ga = std::sqrt((gx * gx + gy * gy) + gz * gz);
        if (ga > 0) dtp = std::min(dtp, 1.0 / std::sqrt(ga * dxi));
        dt = std::min(dt, dtp);
    }
    return dt;
}

// est_maxdt_comoving_a (comoving.cpp:191-215): a must not change by more than
// 5% in one forward-Euler step.
static double est_maxdt_a(double OmM, double OmR, double h, double a, double dt)
{
    const double H0 = h * 100.0;
    const double OmL = 1.0 - OmM - OmR;
    if (H0 != 0.0) {
        const double max_dt = 0.05 / H0 / std::sqrt(OmM / (a * a * a) + OmR / (a * a * a * a) + OmL);
        dt = std::min(dt, max_dt);
    }
    return dt;
}

// est_lindt_comoving_a (comoving.cpp:217-237): the EdS-like first guess of the
// dt that takes a_old to a_new.
static double est_lindt_a(double h, double a_old, double a_new, double dt)
{
    const double H0 = h * 100.0;
    if (H0 != 0.0) {
        const double s = std::pow(0.75, 2.0 / 3.0);
        dt = (std::pow(a_new / s, 0.75) - std::pow(a_old / s, 0.75)) / H0;
    }
    return dt;
}

// Nyx::comoving_est_time_step (comoving.cpp:353-483) from the current a (its
// new-a and old-a branches differ only in which a they pass), through
// estdt_comoving_a (:239-280), enforce_percent_change (:282-317) and
// enforce_final_a (:319-350).  estdt is
// the estimate so far (particles); relative_max_change_a bounds da/a when
// absolute_max_change_a <= 0, otherwise a steps by absolute_max_change_a;
// final_a > 0 stops a there; dt_binpow >= 0 snaps the estimate to the a-limited
// dt divided by a power of two.  Returns the new estimate; *status = 1 where
// the reference aborts (a past final_a, no convergence in 100 iterations).
double orc_comoving_est_dt(double OmM, double OmR, double h, double a, double estdt,
                           double relative_max_change_a, double absolute_max_change_a,
                           double final_a, double dt_binpow, int* status)
{
    *status = 0;
    if (h == 0.0) return estdt;
    double dt = estdt;
    double new_a;
    if (absolute_max_change_a <= 0.0) {
        dt = est_maxdt_a(OmM, OmR, h, a, dt);
        new_a = orc_integrate_a(OmM, OmR, h, a, dt);
        double factor = ((new_a - a) / a) / relative_max_change_a;
        if (factor > 1.0) {
            for (int i = 1; i <= 100; ++i) {
                factor = ((new_a - a) / a) / relative_max_change_a;
                if (factor > 1.0) {
                    dt = (1.0 / factor) * dt * 0.99;
                    new_a = orc_integrate_a(OmM, OmR, h, a, dt);
                } else if (i < 100) {
                    new_a = orc_integrate_a(OmM, OmR, h, a, dt);
                    break;
                } else {
                    *status = 1;
                    return dt;
                }
            }
        }
    } else {
        new_a = a + absolute_max_change_a;
        dt = est_lindt_a(h, a, new_a, dt);
        dt = est_maxdt_a(OmM, OmR, h, a, dt);
        dt = orc_dt_for_da(OmM, OmR, h, a, new_a, dt);
    }
    if (final_a > 0.0) {
        const double eps = 1.0e-10;
        if (a > final_a) {
            *status = 1;
            return dt;
        }
        if (new_a > final_a) {
            for (int i = 1; i <= 100; ++i) {
                if (new_a > final_a + eps || new_a < final_a) {
                    const double factor = (final_a - a) / (new_a - a);
                    dt = dt * factor;
                    new_a = orc_integrate_a(OmM, OmR, h, a, dt);
                } else if (i < 100) {
                    break;
                } else {
                    *status = 1;
                    return dt;
                }
            }
        }
    }
    if (dt_binpow >= 0) {
        if (estdt >= dt)
            estdt = dt;
        else if (estdt > 0.5 * dt)
            estdt = 0.5 * dt;
        else if (estdt > 0.25 * dt)
            estdt = 0.25 * dt;
        else if (estdt > 0.125 * dt)
            estdt = 0.125 * dt;
        else if (estdt > 0.0625 * dt)
            estdt = 0.0625 * dt;
        else
            estdt = dt * std::pow(2.0, -std::ceil(std::log2(dt / estdt)));
    } else {
        estdt = std::min(estdt, dt);
    }
    return estdt;
}

// ----------------------------------------------------------------------------
// one PM step (Nyx_advance_particles.cpp:137-268 + the periodic shift of
// Nyx::post_timestep, Nyx.cpp:1421-1437).
//
// reuse_field = 0: the reference schedule -- the old-time field is recomputed
//   from the positions at the start of the step with a zero initial guess
//   (Gravity.cpp:665-666), then the new-time field after the drift with the
//   old phi as the guess (Nyx_advance_particles.cpp:216-221).
// reuse_field = 1: the old-time field is taken from phi/g as passed in (the
//   previous step's new-time solution), so one deposit and one solve per step.
//
// phi (n^3) is in/out: on entry the previous new-time phi (used when
// reuse_field = 1), on exit the new-time phi.  g (3 n^3) likewise.
// rho_out (n^3, nullable) receives the new-time density.  cycles[2] receives
// the V-cycle counts of the old and new solves (0 for a reused field).
// ----------------------------------------------------------------------------
typedef struct {
    int n;
    double L;
    double mass_offset;
    double ggrav;      // -4 pi G
    double rel_tol;
    int max_cycles;
    int nu1, nu2;
    int reuse_field;
} orc_cfg;

int orc_step(const orc_cfg* cfg, long np, double* x, double* y, double* z, double* vx, double* vy,
             double* vz, double* m, double mscalar, int* id, double a_old, double a_new, double dt,
             double* phi, double* g, double* rho_out, int* cycles)
{
    const int n = cfg->n;
    const double L = cfg->L;
    const long nc = (long)n * n * n;
    std::vector<int> cs(nc + 1);
    std::vector<double> rho(nc), rhs(nc);
    int st = 0;
    double r0, r;
    const double a_half = 0.5 * (a_old + a_new);
    cycles[0] = cycles[1] = 0;
    if (!cfg->reuse_field) {
        orc_sort(n, L, np, x, y, z, vx, vy, vz, m, id, cs.data());
        orc_deposit(n, L, np, x, y, z, m, mscalar, cs.data(), rho.data());
        orc_make_rhs(n, L, rho.data(), cfg->mass_offset, cfg->ggrav, a_old, rhs.data());
        std::fill(phi, phi + nc, 0.0);
        st = orc_mg_solve(n, L, rhs.data(), phi, cfg->rel_tol, cfg->max_cycles, cfg->nu1, cfg->nu2,
                          &cycles[0], &r0, &r);
        if (st == 1) return st;
        orc_grav_vector(n, L, phi, g);
    }
    orc_move(n, L, np, x, y, z, vx, vy, vz, g, dt, a_old, a_half, 1);
    orc_sort(n, L, np, x, y, z, vx, vy, vz, m, id, cs.data());
    orc_deposit(n, L, np, x, y, z, m, mscalar, cs.data(), rho.data());
    orc_make_rhs(n, L, rho.data(), cfg->mass_offset, cfg->ggrav, a_new, rhs.data());
    int st2 = orc_mg_solve(n, L, rhs.data(), phi, cfg->rel_tol, cfg->max_cycles, cfg->nu1, cfg->nu2,
                           &cycles[1], &r0, &r);
    if (st2 == 1) return st2;
    orc_grav_vector(n, L, phi, g);
    orc_move(n, L, np, x, y, z, vx, vy, vz, g, dt, a_half, a_new, 0);
    orc_wrap(L, np, x, y, z);
    if (rho_out) std::memcpy(rho_out, rho.data(), sizeof(double) * nc);
    return st ? st : st2;
}

} // extern "C"
