// CPU FP64 oracle of the multilevel (AMR) particle-mesh step without subcycling.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library's
// multilevel step (nyx_gb300/csrc/pm_amr.cu) is compared against.  The product
// never links, loads or calls it.
//
// It restates Nyx::advance_particles_only for finest_level > 0 with
// amr.subcycling_mode = None (Source/TimeStep/Nyx_advance_particles.cpp:9-272:
// the multilevel old-time solve, moveKickDrift level by level, the multilevel
// new-time solve, moveKick level by level) and Gravity::actual_multilevel_solve
// (Source/Gravity/Gravity.cpp:602-779: the particle density of every level with
// the fine density averaged onto the covered coarse cells, minus mass_offset,
// the solvability correction summed over the uncovered cells, times
// Ggravity / a, a composite solve from a zero guess -- both multilevel solves
// are called without use_previous_phi_as_guess, Nyx_advance_particles.cpp:171,
// 213, and Gravity.H:64-69 default it to 0).  The multilevel deposit (AMReX
// AssignDensity) and the composite MLMG solve are AMReX's, which the reference
// tree does not hold; this file fixes them to one definition that the GPU
// library implements as well:
//   * grids: level l has n0 2^l cells per side; every level above 0 is a list of
//     boxes (inclusive lo/hi in the level's own index space) with even lo and odd
//     hi, disjoint, and nested in the coarser level with one coarse cell to spare;
//   * particle level: the finest level whose boxes hold the particle's cell
//     floor(x / h_l), fixed at the start of the step (AMReX's particle-to-grid
//     assignment, redone by Redistribute after every step);
//   * deposit: the 8 CIC corner masses of a particle (the single-level weights
//     at its level's spacing) go to the corner cell if that cell is valid on the
//     particle's level, else to its parent on the next coarser level (repeated);
//     a corner that lands on a cell covered by a finer level goes in equal eighths
//     to its 8 children (repeated).  Mass is conserved exactly; density = mass /
//     h^3, and a covered cell takes the average of its 8 children;
//   * composite operator: the 7-point Laplacian on every level; a ghost cell of a
//     fine box takes the value of the same-level cell valid there, else the
//     trilinear interpolation of the next coarser level at the ghost's centre
//     (recursively, weights exact in binary); at a face between an uncovered
//     coarse cell and a covered one the coarse flux is replaced by the mean of the
//     4 fine fluxes through it (refluxing);
//   * composite V-cycle, a correction scheme after Martin & Cartwright (1996),
//     "Solving Poisson's equation using adaptive mesh refinement": from the
//     finest level down, nu1 red-black Gauss-Seidel sweeps of the level's
//     correction (ghosts from the coarser correction, zero on the way down), its
//     residual restricted (8-cell sum x 1/2 in smoother units) onto the covered
//     cells below and the change of the fine flux refluxed into the coarse cells
//     beside them; one V-cycle of the periodic single-level hierarchy on level 0;
//     back up, the trilinear prolongation of the coarser correction and nu2
//     sweeps; then phi += e and the fine phi averaged onto the covered cells;
//   * convergence: max over levels of the uncovered composite residual in rhs
//     units <= rel_tol * max(||rhs||, ||r0||), the single-level criterion;
//   * gravity: the single-level cell-centred difference on each level; the 3
//     ghost rings of a fine box's g interpolated from the coarser g as above;
//     each particle kicked (and drifted) with its own level's g.
// Built with -ffp-contract=off: only the explicit std::fma calls fuse.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

extern "C" int orc_mg_vcycle_zero(int n, double L, const double* beta, double* e, int nu1, int nu2);
extern "C" int orc_mg_levels(int n);

namespace {

constexpr int kGW = 3;   // ghost rings of a fine box
const double kSixth = 1.0 / 6.0;
const double kPW[8] = {0.421875, 0.140625, 0.140625, 0.046875,
                       0.140625, 0.046875, 0.046875, 0.015625};

inline int wrapi(int i, int n) { i %= n; return i < 0 ? i + n : i; }
inline long cidx(int i, int j, int k, int n) { return (long)i + (long)n * ((long)j + (long)n * k); }

struct ABox {
    int lev;
    int lo[3], hi[3];
    int d[3];        // padded extents
    long off;        // first padded cell in the composite layout
};

struct Cell {
    long q;
    int box;
    int i, j, k;
};

struct Entry {
    long src;
    double w;
};

struct Ghost {
    long dst;
    int first, count;
};

struct RRec {
    long P, c0;
    long sx, sxy;
};

struct Face {
    long N;
    long f[4], g[4];
};

struct FRec {
    long C;
    std::vector<Face> faces;
};

struct Amr {
    int n0 = 0, nlev = 1;
    double L = 0;
    std::vector<ABox> box;
    std::vector<int> first, count;                 // boxes of each level
    std::vector<std::vector<int>> owner;           // level >= 1: n_l^3 -> box or -1
    long ntot = 0;
    std::vector<std::vector<Cell>> cells;          // level >= 1: valid cells, box/k/j/i order
    std::vector<std::vector<Cell>> color[2];       // the same split by (i+j+k) parity
    std::vector<std::vector<Ghost>> ghost1, ghost23;   // per level: ring 1, rings 2-3
    std::vector<Entry> ent;
    std::vector<std::vector<RRec>> rrec;           // level l >= 1: covered cells of l-1
    std::vector<std::vector<FRec>> frec;           // level l >= 1: c/f faces of l-1
    std::vector<char> cov;                         // 1 on covered valid cells
    std::vector<double> mass, rho, beta, phi, R, e, T, g[3];
    std::vector<int> plev, pbox;
    std::string err;
};

inline int nl(const Amr& A, int l) { return A.n0 << l; }
inline double hl(const Amr& A, int l) { return A.L / nl(A, l); }
inline double scale_l(const Amr& A, int l) { const double h = hl(A, l); return (h * h) * kSixth; }

inline long gidx(const ABox& b, int i, int j, int k)
{
    return b.off + (long)(i - b.lo[0] + kGW) +
           (long)b.d[0] * ((long)(j - b.lo[1] + kGW) + (long)b.d[1] * (k - b.lo[2] + kGW));
}

int owner_of(const Amr& A, int l, int i, int j, int k)
{
    const int n = nl(A, l);
    return A.owner[l][cidx(wrapi(i, n), wrapi(j, n), wrapi(k, n), n)];
}

// composite index of the valid cell (i,j,k) of level l (wrapped), or -1
long vidx(const Amr& A, int l, int i, int j, int k)
{
    const int n = nl(A, l);
    i = wrapi(i, n); j = wrapi(j, n); k = wrapi(k, n);
    if (l == 0) return cidx(i, j, k, n);
    const int o = A.owner[l][cidx(i, j, k, n)];
    return o < 0 ? -1 : gidx(A.box[o], i, j, k);
}

bool covered(const Amr& A, int l, int i, int j, int k)
{
    return l + 1 < A.nlev && owner_of(A, l + 1, 2 * wrapi(i, nl(A, l)), 2 * wrapi(j, nl(A, l)),
                                      2 * wrapi(k, nl(A, l))) >= 0;
}

// the source cells and weights of the value of level l at cell (i,j,k)
void gen(const Amr& A, int l, int i, int j, int k, double w, std::vector<Entry>& out)
{
    const long v = vidx(A, l, i, j, k);
    if (v >= 0) { out.push_back({v, w}); return; }
    const int n = nl(A, l);
    const int c[3] = {wrapi(i, n), wrapi(j, n), wrapi(k, n)};
    int I0[3];
    double t[3];
    for (int d = 0; d < 3; ++d) {
        if (c[d] & 1) { I0[d] = (c[d] - 1) / 2; t[d] = 0.25; }
        else { I0[d] = c[d] / 2 - 1; t[d] = 0.75; }
    }
    for (int dk = 0; dk < 2; ++dk)
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di) {
                const double wx = di ? t[0] : 1.0 - t[0];
                const double wy = dj ? t[1] : 1.0 - t[1];
                const double wz = dk ? t[2] : 1.0 - t[2];
                gen(A, l - 1, I0[0] + di, I0[1] + dj, I0[2] + dk, w * ((wx * wy) * wz), out);
            }
}

bool build(Amr& A, int n0, double L, int nlev, const int* nbox, const int* boxes)
{
    A.n0 = n0; A.L = L; A.nlev = nlev;
    if (nlev < 1 || orc_mg_levels(n0) == 0) { A.err = "bad n0 or level count"; return false; }
    A.first.assign(nlev, 0); A.count.assign(nlev, 0);
    A.owner.assign(nlev, {});
    long off = (long)n0 * n0 * n0;
    int q = 0;
    for (int l = 1; l < nlev; ++l) {
        const int n = nl(A, l);
        A.owner[l].assign((size_t)n * n * n, -1);
        A.first[l] = (int)A.box.size();
        A.count[l] = nbox[l - 1];
        if (nbox[l - 1] < 1) { A.err = "a level without boxes"; return false; }
        for (int b = 0; b < nbox[l - 1]; ++b, ++q) {
            ABox B;
            B.lev = l;
            for (int d = 0; d < 3; ++d) {
                B.lo[d] = boxes[6 * q + d];
                B.hi[d] = boxes[6 * q + 3 + d];
                if (B.lo[d] < 0 || B.hi[d] >= n || B.lo[d] > B.hi[d] || (B.lo[d] & 1) || !(B.hi[d] & 1)) {
                    A.err = "box outside its level, empty, or not aligned to the refinement ratio";
                    return false;
                }
                B.d[d] = B.hi[d] - B.lo[d] + 1 + 2 * kGW;
            }
            B.off = off;
            off += (long)B.d[0] * B.d[1] * B.d[2];
            const int id = (int)A.box.size();
            for (int k = B.lo[2]; k <= B.hi[2]; ++k)
                for (int j = B.lo[1]; j <= B.hi[1]; ++j)
                    for (int i = B.lo[0]; i <= B.hi[0]; ++i) {
                        int& o = A.owner[l][cidx(i, j, k, n)];
                        if (o >= 0) { A.err = "boxes of one level overlap"; return false; }
                        o = id;
                    }
            A.box.push_back(B);
        }
    }
    A.ntot = off;
    // nesting: the coarsened box grown by one cell is valid on the coarser level
    for (const ABox& B : A.box) {
        if (B.lev < 2) continue;
        for (int K = B.lo[2] / 2 - 1; K <= B.hi[2] / 2 + 1; ++K)
            for (int J = B.lo[1] / 2 - 1; J <= B.hi[1] / 2 + 1; ++J)
                for (int I = B.lo[0] / 2 - 1; I <= B.hi[0] / 2 + 1; ++I)
                    if (vidx(A, B.lev - 1, I, J, K) < 0) {
                        A.err = "a box is not nested in the coarser level with one cell to spare";
                        return false;
                    }
    }
    // cell lists
    A.cells.assign(nlev, {});
    A.color[0].assign(nlev, {});
    A.color[1].assign(nlev, {});
    for (int l = 1; l < nlev; ++l)
        for (int b = A.first[l]; b < A.first[l] + A.count[l]; ++b) {
            const ABox& B = A.box[b];
            for (int k = B.lo[2]; k <= B.hi[2]; ++k)
                for (int j = B.lo[1]; j <= B.hi[1]; ++j)
                    for (int i = B.lo[0]; i <= B.hi[0]; ++i) {
                        Cell c{gidx(B, i, j, k), b, i, j, k};
                        A.cells[l].push_back(c);
                        A.color[(i + j + k) & 1][l].push_back(c);
                    }
        }
    // covered flags
    A.cov.assign(A.ntot, 0);
    for (int k = 0; k < n0; ++k)
        for (int j = 0; j < n0; ++j)
            for (int i = 0; i < n0; ++i)
                if (covered(A, 0, i, j, k)) A.cov[cidx(i, j, k, n0)] = 1;
    for (int l = 1; l < nlev; ++l)
        for (const Cell& c : A.cells[l])
            if (covered(A, l, c.i, c.j, c.k)) A.cov[c.q] = 1;
    // ghost lists: ring 1, then rings 2 and 3
    A.ghost1.assign(nlev, {});
    A.ghost23.assign(nlev, {});
    for (int l = 1; l < nlev; ++l)
        for (int b = A.first[l]; b < A.first[l] + A.count[l]; ++b) {
            const ABox& B = A.box[b];
            for (int k = B.lo[2] - kGW; k <= B.hi[2] + kGW; ++k)
                for (int j = B.lo[1] - kGW; j <= B.hi[1] + kGW; ++j)
                    for (int i = B.lo[0] - kGW; i <= B.hi[0] + kGW; ++i) {
                        const int dist = std::max({B.lo[0] - i, i - B.hi[0], B.lo[1] - j, j - B.hi[1],
                                                   B.lo[2] - k, k - B.hi[2], 0});
                        if (dist == 0) continue;
                        Ghost gh{gidx(B, i, j, k), (int)A.ent.size(), 0};
                        gen(A, l, i, j, k, 1.0, A.ent);
                        gh.count = (int)A.ent.size() - gh.first;
                        (dist == 1 ? A.ghost1 : A.ghost23)[l].push_back(gh);
                    }
        }
    // restriction records and coarse/fine faces of every level pair
    A.rrec.assign(nlev, {});
    A.frec.assign(nlev, {});
    for (int l = 1; l < nlev; ++l) {
        for (int b = A.first[l]; b < A.first[l] + A.count[l]; ++b) {
            const ABox& B = A.box[b];
            for (int K = B.lo[2] / 2; K <= B.hi[2] / 2; ++K)
                for (int J = B.lo[1] / 2; J <= B.hi[1] / 2; ++J)
                    for (int I = B.lo[0] / 2; I <= B.hi[0] / 2; ++I)
                        A.rrec[l].push_back({vidx(A, l - 1, I, J, K), gidx(B, 2 * I, 2 * J, 2 * K),
                                             (long)B.d[0], (long)B.d[0] * B.d[1]});
        }
        auto faces_of = [&](int i, int j, int k, long C) {
            if (covered(A, l - 1, i, j, k)) return;
            FRec r;
            r.C = C;
            for (int d = 0; d < 3; ++d)
                for (int s = -1; s <= 1; s += 2) {
                    int nb[3] = {i, j, k};
                    nb[d] += s;
                    if (!covered(A, l - 1, nb[0], nb[1], nb[2])) continue;
                    const int n = nl(A, l - 1);
                    for (int t = 0; t < 3; ++t) nb[t] = wrapi(nb[t], n);
                    Face f;
                    f.N = vidx(A, l - 1, nb[0], nb[1], nb[2]);
                    const int ta = d == 0 ? 1 : 0, tb = d == 2 ? 1 : 2;   // tangential axes, tb outer
                    int kk = 0;
                    for (int ob = 0; ob < 2; ++ob)
                        for (int oa = 0; oa < 2; ++oa, ++kk) {
                            int fc[3];
                            fc[d] = 2 * nb[d] + (s > 0 ? 0 : 1);
                            fc[ta] = 2 * nb[ta] + oa;
                            fc[tb] = 2 * nb[tb] + ob;
                            const int o = owner_of(A, l, fc[0], fc[1], fc[2]);
                            const ABox& FB = A.box[o];
                            f.f[kk] = gidx(FB, fc[0], fc[1], fc[2]);
                            int gc[3] = {fc[0], fc[1], fc[2]};
                            gc[d] -= s;
                            f.g[kk] = gidx(FB, gc[0], gc[1], gc[2]);
                        }
                    r.faces.push_back(f);
                }
            if (!r.faces.empty()) A.frec[l].push_back(r);
        };
        if (l - 1 == 0) {
            for (int k = 0; k < n0; ++k)
                for (int j = 0; j < n0; ++j)
                    for (int i = 0; i < n0; ++i) faces_of(i, j, k, cidx(i, j, k, n0));
        } else {
            for (const Cell& c : A.cells[l - 1]) faces_of(c.i, c.j, c.k, c.q);
        }
    }
    for (auto* v : {&A.mass, &A.rho, &A.beta, &A.phi, &A.R, &A.e, &A.T, &A.g[0], &A.g[1], &A.g[2]})
        v->assign(A.ntot, 0.0);
    return true;
}

void ghost_fill(Amr& A, std::vector<double>& f, const std::vector<Ghost>& gl)
{
    // sources are valid cells, destinations ghost cells: the ghosts are independent
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)gl.size(); ++t) {
        const Ghost& gh = gl[t];
        double v = 0.0;
        for (int t = 0; t < gh.count; ++t) v = std::fma(A.ent[gh.first + t].w, f[A.ent[gh.first + t].src], v);
        f[gh.dst] = v;
    }
}

void ghost_fill_level(Amr& A, std::vector<double>& f, int l) { ghost_fill(A, f, A.ghost1[l]); }

void ghost_fill_all(Amr& A, std::vector<double>& f, int rings3)
{
    for (int l = 1; l < A.nlev; ++l) {
        ghost_fill(A, f, A.ghost1[l]);
        if (rings3) ghost_fill(A, f, A.ghost23[l]);
    }
}

// the covered cells of level l-1 take the average of their 8 children
void avg_down(Amr& A, std::vector<double>& f, int l)
{
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)A.rrec[l].size(); ++t) {
        const RRec& r = A.rrec[l][t];
        double s = 0.0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) s = s + f[r.c0 + di + dj * r.sx + dk * r.sxy];
        f[r.P] = s * 0.125;
    }
}

inline double nbr0(const std::vector<double>& f, int i, int j, int k, int n)
{
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    double s = f[cidx(im, j, k, n)] + f[cidx(ip, j, k, n)];
    s = s + f[cidx(i, jm, k, n)];
    s = s + f[cidx(i, jp, k, n)];
    s = s + f[cidx(i, j, km, n)];
    s = s + f[cidx(i, j, kp, n)];
    return s;
}

inline double nbrf(const Amr& A, const std::vector<double>& f, const Cell& c)
{
    const ABox& B = A.box[c.box];
    const long sx = B.d[0], sxy = (long)B.d[0] * B.d[1];
    double s = f[c.q - 1] + f[c.q + 1];
    s = s + f[c.q - sx];
    s = s + f[c.q + sx];
    s = s + f[c.q - sxy];
    s = s + f[c.q + sxy];
    return s;
}

// out = rhs - (s/6 - u) on every valid cell of level l (smoother units)
void resid_level(Amr& A, const std::vector<double>& u, const std::vector<double>& rhs,
                 std::vector<double>& out, int l)
{
    if (l == 0) {
        const int n = A.n0;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    const long q = cidx(i, j, k, n);
                    out[q] = rhs[q] - std::fma(nbr0(u, i, j, k, n), kSixth, -u[q]);
                }
        return;
    }
    const std::vector<Cell>& cl = A.cells[l];
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)cl.size(); ++t)
        out[cl[t].q] = rhs[cl[t].q] - std::fma(nbrf(A, u, cl[t]), kSixth, -u[cl[t].q]);
}

// refluxing at the faces between the uncovered cells of level l-1 and level l
void reflux(Amr& A, const std::vector<double>& u, std::vector<double>& R, int l)
{
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)A.frec[l].size(); ++t) {
        const FRec& r = A.frec[l][t];
        double v = R[r.C];
        for (const Face& f : r.faces) {
            double s = u[f.f[0]] - u[f.g[0]];
            s = s + (u[f.f[1]] - u[f.g[1]]);
            s = s + (u[f.f[2]] - u[f.g[2]]);
            s = s + (u[f.f[3]] - u[f.g[3]]);
            v = v - (((s * 0.5) - (u[f.N] - u[r.C])) * kSixth);
        }
        R[r.C] = v;
    }
}

double level_absmax(const Amr& A, const std::vector<double>& f, int l)
{
    double mx = 0.0;
    if (l == 0) {
        const long nc = (long)A.n0 * A.n0 * A.n0;
#pragma omp parallel for schedule(static) reduction(max : mx)
        for (long q = 0; q < nc; ++q)
            if (!A.cov[q]) mx = std::max(mx, std::fabs(f[q]));
    } else {
        const std::vector<Cell>& cl = A.cells[l];
#pragma omp parallel for schedule(static) reduction(max : mx)
        for (long t = 0; t < (long)cl.size(); ++t)
            if (!A.cov[cl[t].q]) mx = std::max(mx, std::fabs(f[cl[t].q]));
    }
    return mx;
}

double comp_norm(const Amr& A, const std::vector<double>& f)
{
    double mx = 0.0;
    for (int l = 0; l < A.nlev; ++l) mx = std::max(mx, level_absmax(A, f, l) * (1.0 / scale_l(A, l)));
    return mx;
}

// composite residual of phi into R; phi's covered cells averaged and its ghosts
// filled on the way
double comp_resid(Amr& A)
{
    for (int l = A.nlev - 1; l >= 1; --l) avg_down(A, A.phi, l);
    ghost_fill_all(A, A.phi, 0);
    for (int l = 0; l < A.nlev; ++l) resid_level(A, A.phi, A.beta, A.R, l);
    for (int l = 1; l < A.nlev; ++l) reflux(A, A.phi, A.R, l);
    return comp_norm(A, A.R);
}

void gsrb_level(Amr& A, int l)
{
    for (int col = 0; col < 2; ++col) {
        ghost_fill_level(A, A.e, l);
        const std::vector<Cell>& cl = A.color[col][l];
#pragma omp parallel for schedule(static)
        for (long t = 0; t < (long)cl.size(); ++t)
            A.e[cl[t].q] = std::fma(nbrf(A, A.e, cl[t]), kSixth, -A.R[cl[t].q]);
    }
}

void prolong_level(Amr& A, int l)
{
#pragma omp parallel for schedule(static)
    for (long ci = 0; ci < (long)A.cells[l].size(); ++ci) {
        const Cell& c = A.cells[l][ci];
        const int I = c.i >> 1, J = c.j >> 1, K = c.k >> 1;
        const int Is[2] = {I, (c.i & 1) ? I + 1 : I - 1};
        const int Js[2] = {J, (c.j & 1) ? J + 1 : J - 1};
        const int Ks[2] = {K, (c.k & 1) ? K + 1 : K - 1};
        double s = 0.0;
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a)
                for (int t = 0; t < 2; ++t)
                    s = std::fma(kPW[t + 2 * a + 4 * b], A.e[vidx(A, l - 1, Is[t], Js[a], Ks[b])], s);
        A.e[c.q] = A.e[c.q] + s;
    }
}

int vcycle(Amr& A, int nu1, int nu2)
{
    std::fill(A.e.begin(), A.e.end(), 0.0);
    for (int l = A.nlev - 1; l >= 1; --l) {
        for (int s = 0; s < nu1; ++s) gsrb_level(A, l);
        ghost_fill_level(A, A.e, l);
        resid_level(A, A.e, A.R, A.T, l);
#pragma omp parallel for schedule(static)
        for (long t = 0; t < (long)A.rrec[l].size(); ++t) {
            const RRec& r = A.rrec[l][t];
            double s = 0.0;
            for (int dk = 0; dk < 2; ++dk)
                for (int dj = 0; dj < 2; ++dj)
                    for (int di = 0; di < 2; ++di) s = s + A.T[r.c0 + di + dj * r.sx + dk * r.sxy];
            A.R[r.P] = s * 0.5;
        }
        reflux(A, A.e, A.R, l);
    }
    const long n3 = (long)A.n0 * A.n0 * A.n0;
    std::vector<double> e0(n3);
    if (orc_mg_vcycle_zero(A.n0, A.L, A.R.data(), e0.data(), nu1, nu2)) return 1;
    std::memcpy(A.e.data(), e0.data(), sizeof(double) * n3);
    for (int l = 1; l < A.nlev; ++l) {
        if (l - 1 >= 1) ghost_fill_level(A, A.e, l - 1);
        prolong_level(A, l);
        for (int s = 0; s < nu2; ++s) gsrb_level(A, l);
    }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < A.ntot; ++q) A.phi[q] = A.phi[q] + A.e[q];
    return 0;
}

}  // namespace

extern "C" {

typedef struct {
    double mass_offset;
    double ggrav;      // -4 pi G
    double rel_tol;
    int max_cycles;
    int nu1, nu2;
} orc_amr_cfg;

// nbox[l-1] boxes on level l = 1 .. nlev-1; boxes: 6 ints each (lo xyz, hi xyz),
// level by level.  Returns null on invalid grids, with the reason in err.
void* orc_amr_create(int n0, double L, int nlev, const int* nbox, const int* boxes, char* err, int errlen)
{
    Amr* A = new Amr;
    if (!build(*A, n0, L, nlev, nbox, boxes)) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", A->err.c_str());
        delete A;
        return nullptr;
    }
    return A;
}

void orc_amr_destroy(void* h) { delete static_cast<Amr*>(h); }

// particle level and box: the finest level whose boxes hold floor(x / h_l)
// (box -1 on level 0)
void orc_amr_assign(void* h, long np, const double* x, const double* y, const double* z, int* lev,
                    int* box)
{
    Amr& A = *static_cast<Amr*>(h);
    for (long p = 0; p < np; ++p) {
        lev[p] = 0;
        box[p] = -1;
        for (int l = A.nlev - 1; l >= 1; --l) {
            const double dxi = (double)nl(A, l) / A.L;
            const int o = owner_of(A, l, (int)std::floor(x[p] * dxi), (int)std::floor(y[p] * dxi),
                                   (int)std::floor(z[p] * dxi));
            if (o >= 0) { lev[p] = l; box[p] = o; break; }
        }
    }
}

// multilevel CIC deposit into the composite density (covered cells averaged)
void orc_amr_deposit(void* h, long np, const double* x, const double* y, const double* z,
                     const double* m, double mscalar, const int* lev)
{
    Amr& A = *static_cast<Amr*>(h);
    std::fill(A.mass.begin(), A.mass.end(), 0.0);
    // the corner mass q lands on cell c of level l: coarser while not valid,
    // then finer in eighths while covered
    struct Put {
        Amr& A;
        void up(int l, int i, int j, int k, double q)
        {
            if (covered(A, l, i, j, k)) {
                const int n = nl(A, l);
                i = wrapi(i, n); j = wrapi(j, n); k = wrapi(k, n);
                const double q8 = q * 0.125;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di) up(l + 1, 2 * i + di, 2 * j + dj, 2 * k + dk, q8);
                return;
            }
            const long v = vidx(A, l, i, j, k);
            A.mass[v] = A.mass[v] + q;
        }
        void put(int l, int i, int j, int k, double q)
        {
            while (vidx(A, l, i, j, k) < 0) {
                const int n = nl(A, l);
                i = wrapi(i, n) >> 1; j = wrapi(j, n) >> 1; k = wrapi(k, n) >> 1;
                --l;
            }
            up(l, i, j, k, q);
        }
    } put{A};
    for (long p = 0; p < np; ++p) {
        const int l = lev[p];
        const double dxi = (double)nl(A, l) / A.L;
        const double lx = std::fma(x[p], dxi, 0.5), ly = std::fma(y[p], dxi, 0.5), lz = std::fma(z[p], dxi, 0.5);
        const double fi = std::floor(lx), fj = std::floor(ly), fk = std::floor(lz);
        const int i = (int)fi, j = (int)fj, k = (int)fk;
        const double fx = lx - fi, fy = ly - fj, fz = lz - fk;
        const double sx[2] = {1.0 - fx, fx}, sy[2] = {1.0 - fy, fy}, sz[2] = {1.0 - fz, fz};
        const double mp = m ? m[p] : mscalar;
        for (int cz = 0; cz < 2; ++cz)
            for (int cy = 0; cy < 2; ++cy)
                for (int cx = 0; cx < 2; ++cx)
                    put.put(l, i - 1 + cx, j - 1 + cy, k - 1 + cz, ((sx[cx] * sy[cy]) * sz[cz]) * mp);
    }
    for (int l = 0; l < A.nlev; ++l) {
        const double h = hl(A, l);
        const double inv_vol = 1.0 / ((h * h) * h);
        if (l == 0) {
            const long nc = (long)A.n0 * A.n0 * A.n0;
            for (long q = 0; q < nc; ++q) A.rho[q] = A.mass[q] * inv_vol;
        } else {
            for (const Cell& c : A.cells[l]) A.rho[c.q] = A.mass[c.q] * inv_vol;
        }
    }
    for (int l = A.nlev - 1; l >= 1; --l) avg_down(A, A.rho, l);
}

// rhs from the composite density and the composite solve from a zero guess.
// Returns 0 converged, 4 max_cycles reached, 1 bad hierarchy.
int orc_amr_solve(void* h, const orc_amr_cfg* cfg, double a, int* ncycles, double* resnorm0,
                  double* resnorm)
{
    Amr& A = *static_cast<Amr*>(h);
    // solvability: the mean of rho - mass_offset over the uncovered cells, volume weighted
    double S = 0.0;
    for (int l = 0; l < A.nlev; ++l) {
        const double h = hl(A, l);
        double s = 0.0;
        if (l == 0) {
            const long nc = (long)A.n0 * A.n0 * A.n0;
            for (long q = 0; q < nc; ++q)
                if (!A.cov[q]) s = s + (A.rho[q] - cfg->mass_offset);
        } else {
            for (const Cell& c : A.cells[l])
                if (!A.cov[c.q]) s = s + (A.rho[c.q] - cfg->mass_offset);
        }
        S = S + s * ((h * h) * h);
    }
    const double mean = S / ((A.L * A.L) * A.L);
    const double ainv = 1.0 / a;
    for (int l = 0; l < A.nlev; ++l) {
        const double k0 = scale_l(A, l);
        auto rhs = [&](long q) {
            A.beta[q] = ((((A.rho[q] - cfg->mass_offset) - mean) * cfg->ggrav) * ainv) * k0;
        };
        if (l == 0) {
            const long nc = (long)A.n0 * A.n0 * A.n0;
            for (long q = 0; q < nc; ++q) rhs(q);
        } else {
            for (const Cell& c : A.cells[l]) rhs(c.q);
        }
    }
    std::fill(A.phi.begin(), A.phi.end(), 0.0);
    const double bnorm = comp_norm(A, A.beta);
    const double r0 = comp_resid(A);
    const double target = cfg->rel_tol * std::max(bnorm, r0);
    double r = r0;
    int it = 0, st = 0;
    if (r0 > target) {
        for (it = 1; it <= cfg->max_cycles; ++it) {
            if (vcycle(A, cfg->nu1, cfg->nu2)) return 1;
            r = comp_resid(A);
            if (r <= target) break;
        }
        if (it > cfg->max_cycles) { it = cfg->max_cycles; st = 4; }
    }
    if (ncycles) *ncycles = it;
    if (resnorm0) *resnorm0 = r0;
    if (resnorm) *resnorm = r;
    return st;
}

// the cell-centred gravity vector of every level (the single-level difference),
// the fine boxes' 3 ghost rings interpolated from the coarser g
void orc_amr_grav(void* h)
{
    Amr& A = *static_cast<Amr*>(h);
    for (int l = 0; l < A.nlev; ++l) {
        const double dxi = (double)nl(A, l) / A.L;
        auto one = [&](long q, long xm, long xp, long ym, long yp, long zm, long zp) {
            const double pc = A.phi[q];
            A.g[0][q] = 0.5 * std::fma(A.phi[xp] - pc, dxi, (pc - A.phi[xm]) * dxi);
            A.g[1][q] = 0.5 * std::fma(A.phi[yp] - pc, dxi, (pc - A.phi[ym]) * dxi);
            A.g[2][q] = 0.5 * std::fma(A.phi[zp] - pc, dxi, (pc - A.phi[zm]) * dxi);
        };
        if (l == 0) {
            const int n = A.n0;
            for (int k = 0; k < n; ++k)
                for (int j = 0; j < n; ++j)
                    for (int i = 0; i < n; ++i)
                        one(cidx(i, j, k, n), cidx(wrapi(i - 1, n), j, k, n), cidx(wrapi(i + 1, n), j, k, n),
                            cidx(i, wrapi(j - 1, n), k, n), cidx(i, wrapi(j + 1, n), k, n),
                            cidx(i, j, wrapi(k - 1, n), n), cidx(i, j, wrapi(k + 1, n), n));
        } else {
            for (const Cell& c : A.cells[l]) {
                const ABox& B = A.box[c.box];
                const long sx = B.d[0], sxy = (long)B.d[0] * B.d[1];
                one(c.q, c.q - 1, c.q + 1, c.q - sx, c.q + sx, c.q - sxy, c.q + sxy);
            }
        }
    }
    for (int d = 0; d < 3; ++d) ghost_fill_all(A, A.g[d], 1);
}

// update_dm_particle_single (DarkMatterParticleContainer.cpp:250-306) of every
// particle with its own level's g.  Returns 5 if a particle's stencil leaves its
// box's ghost rings.
int orc_amr_move(void* h, long np, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                 const int* lev, const int* box, double dt, double a_prev, double a_cur, int do_move)
{
    Amr& A = *static_cast<Amr*>(h);
    const double half_dt = 0.5 * dt;
    const double a_cur_inv = 1.0 / a_cur;
    const double dt_a_cur_inv = dt * a_cur_inv;
    int st = 0;
    for (long p = 0; p < np; ++p) {
        const int l = lev[p];
        const double dxi = (double)nl(A, l) / A.L;
        const double lx = std::fma(x[p], dxi, 0.5), ly = std::fma(y[p], dxi, 0.5), lz = std::fma(z[p], dxi, 0.5);
        const double fi = std::floor(lx), fj = std::floor(ly), fk = std::floor(lz);
        const int i = (int)fi, j = (int)fj, k = (int)fk;
        const double xint = lx - fi, yint = ly - fj, zint = lz - fk;
        const double sx[2] = {1.0 - xint, xint}, sy[2] = {1.0 - yint, yint}, sz[2] = {1.0 - zint, zint};
        double w[8];
        long cells[8];
        bool ok = true;
        for (int kk = 0; kk <= 1; ++kk)
            for (int jj = 0; jj <= 1; ++jj)
                for (int ii = 0; ii <= 1; ++ii) {
                    const int t = ii + 2 * jj + 4 * kk;
                    w[t] = (sx[1 - ii] * sy[1 - jj]) * sz[1 - kk];
                    if (l == 0) {
                        const int n = A.n0;
                        cells[t] = cidx(wrapi(i - ii, n), wrapi(j - jj, n), wrapi(k - kk, n), n);
                    } else {
                        const ABox& B = A.box[box[p]];
                        const int ci = i - ii, cj = j - jj, ck = k - kk;
                        if (ci < B.lo[0] - kGW || ci > B.hi[0] + kGW || cj < B.lo[1] - kGW || cj > B.hi[1] + kGW ||
                            ck < B.lo[2] - kGW || ck > B.hi[2] + kGW) { ok = false; cells[t] = B.off; }
                        else cells[t] = gidx(B, ci, cj, ck);
                    }
                }
        if (!ok) st = 5;
        double* v[3] = {vx + p, vy + p, vz + p};
        for (int d = 0; d < 3; ++d) {
            double val = 0.0;
            for (int t = 0; t < 8; ++t) val = std::fma(w[t], A.g[d][cells[t]], val);
            const double u = std::fma(a_prev, *v[d], half_dt * val);
            *v[d] = u * a_cur_inv;
        }
        if (do_move == 1) {
            x[p] = std::fma(dt_a_cur_inv, vx[p], x[p]);
            y[p] = std::fma(dt_a_cur_inv, vy[p], y[p]);
            z[p] = std::fma(dt_a_cur_inv, vz[p], z[p]);
        }
    }
    return st;
}

// one multilevel step (positions wrapped into [0, L) on entry and on exit):
// levels assigned, old-time deposit and solve, kick-drift, new-time deposit and
// solve, kick.  cycles[2]: the V-cycle counts of the two solves; lev/box
// (nullable) receive the particle levels and boxes of the step.
int orc_amr_step(void* h, const orc_amr_cfg* cfg, long np, double* x, double* y, double* z, double* vx,
                 double* vy, double* vz, const double* m, double mscalar, double a_old, double a_new,
                 double dt, int* cycles, int* lev_out, int* box_out)
{
    Amr& A = *static_cast<Amr*>(h);
    std::vector<int> lev(np), box(np);
    orc_amr_assign(h, np, x, y, z, lev.data(), box.data());
    const double a_half = 0.5 * (a_old + a_new);
    double r0, r;
    orc_amr_deposit(h, np, x, y, z, m, mscalar, lev.data());
    int st = orc_amr_solve(h, cfg, a_old, &cycles[0], &r0, &r);
    if (st == 1) return st;
    orc_amr_grav(h);
    int sm = orc_amr_move(h, np, x, y, z, vx, vy, vz, lev.data(), box.data(), dt, a_old, a_half, 1);
    orc_amr_deposit(h, np, x, y, z, m, mscalar, lev.data());
    int st2 = orc_amr_solve(h, cfg, a_new, &cycles[1], &r0, &r);
    if (st2 == 1) return st2;
    orc_amr_grav(h);
    int sm2 = orc_amr_move(h, np, x, y, z, vx, vy, vz, lev.data(), box.data(), dt, a_half, a_new, 0);
    double* c[3] = {x, y, z};
    for (int d = 0; d < 3; ++d)
        for (long p = 0; p < np; ++p) {
            double v = c[d][p];
            if (v >= A.L) v = v - A.L; else if (v < 0.0) v = v + A.L;
            if (v >= A.L) v = 0.0;
            c[d][p] = v;
        }
    if (lev_out) std::memcpy(lev_out, lev.data(), sizeof(int) * np);
    if (box_out) std::memcpy(box_out, box.data(), sizeof(int) * np);
    if (sm || sm2) return 5;
    return st ? st : st2;
}

// a field of one level (box -1: level 0, n0^3) or one box (its valid cells,
// x fastest): which = 0 density, 1 phi, 2..4 g_x, g_y, g_z, 5 mass
int orc_amr_field(void* h, int which, int box, double* out)
{
    Amr& A = *static_cast<Amr*>(h);
    const std::vector<double>* f[6] = {&A.rho, &A.phi, &A.g[0], &A.g[1], &A.g[2], &A.mass};
    if (which < 0 || which > 5) return 1;
    const std::vector<double>& v = *f[which];
    if (box < 0) {
        std::memcpy(out, v.data(), sizeof(double) * (size_t)A.n0 * A.n0 * A.n0);
        return 0;
    }
    if (box >= (int)A.box.size()) return 1;
    const ABox& B = A.box[box];
    long t = 0;
    for (int k = B.lo[2]; k <= B.hi[2]; ++k)
        for (int j = B.lo[1]; j <= B.hi[1]; ++j)
            for (int i = B.lo[0]; i <= B.hi[0]; ++i) out[t++] = v[gidx(B, i, j, k)];
    return 0;
}

// the composite mass on the uncovered valid cells (the deposited total)
double orc_amr_total_mass(void* h)
{
    Amr& A = *static_cast<Amr*>(h);
    double s = 0.0;
    for (int l = 0; l < A.nlev; ++l) {
        if (l == 0) {
            const long nc = (long)A.n0 * A.n0 * A.n0;
            for (long q = 0; q < nc; ++q)
                if (!A.cov[q]) s += A.mass[q];
        } else {
            for (const Cell& c : A.cells[l])
                if (!A.cov[c.q]) s += A.mass[c.q];
        }
    }
    return s;
}

}  // extern "C"
