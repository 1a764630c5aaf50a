// Multilevel (AMR) particle-mesh step without subcycling, FP64: the GB300 form
// of Nyx::advance_particles_only for finest_level > 0 with amr.subcycling_mode =
// None (Source/TimeStep/Nyx_advance_particles.cpp:9-272: the multilevel
// old-time solve, moveKickDrift level by level, the multilevel new-time solve,
// moveKick level by level) and of Gravity::actual_multilevel_solve
// (Source/Gravity/Gravity.cpp:602-779: particle density on every level with
// the fine density averaged onto the covered coarse cells, minus mass_offset,
// the solvability correction over the uncovered cells, times Ggravity / a, a
// composite solve from a zero guess).
//
// The multilevel deposit (AMReX AssignDensity) and the composite MLMG solve
// are AMReX's, which the reference tree does not hold.  This file implements
// one definition of them:
//   * level l has n0 2^l cells per side; the levels above 0 are lists of boxes
//     (even lo, odd hi, disjoint, nested in the coarser level with one coarse
//     cell to spare), each stored with 3 ghost rings in one composite array
//     after level 0's n0^3 cells;
//   * a particle belongs to the finest level whose boxes hold its cell;
//   * its 8 CIC corner masses go to the corner cell if that is valid on its
//     level, else to the parent on the next coarser level (repeated); a corner on
//     a cell covered by a finer level goes in eighths to the children (repeated);
//   * the composite operator is the 7-point Laplacian on every level, fine ghost
//     cells from the same level where valid, else the trilinear interpolation of
//     the coarser level (recursively); coarse fluxes through coarse/fine faces
//     replaced by the mean of the 4 fine fluxes (refluxing);
//   * the solve is the composite V-cycle (a correction scheme after Martin &
//     Cartwright 1996): red-black Gauss-Seidel on each fine level, the fine
//     residual restricted onto covered coarse cells and the fine flux change
//     refluxed, one V-cycle of the periodic single-level hierarchy on level 0
//     (mg_vcycle_zero), trilinear prolongation back up.
// Every index structure (ghost stencils with the same-level copies first,
// restriction and coarse/fine face records, per-cell parents, a prefix of fine
// cells per box) is built once on the host when the hierarchy is created.  The
// smoother, residual and norms number the fine cells box by box (a binary search
// over the prefix finds the box); the other kernels walk flat lists, one thread
// per cell, ghost cell, record or particle.
// Built with --fmad=false: only the explicit fma() calls fuse.
#include "pm_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace nyxpm;

namespace {

constexpr int kGW = 3;          // ghost rings of a fine box
constexpr int kMaxLevels = 4;   // level 0 and up to 3 refined levels
constexpr int kT = 256;
constexpr double kSixth = 1.0 / 6.0;

__constant__ double kAmrProlongW[8] = {0.421875, 0.140625, 0.140625, 0.046875,
                                       0.140625, 0.046875, 0.046875, 0.015625};

struct ABox {
    int lev;
    int lo[3], hi[3];
    int d[3];          // padded extents
    int pbox;          // the coarser box holding this box's parents (-1: level 0; -2: several)
    long long off;     // first padded cell in the composite layout
};

struct ACell {
    long long q;
    int i, j, k, box;
};

struct AGhost {
    long long dst;
    int first, count;
};

struct AEnt {
    long long src;
    double w;
};

struct ARRec {
    long long P, c0;
    int sx, sxy;
};

struct AFace {
    long long N;
    long long f[4], g[4];
};

struct AFRec {
    long long C;
    int first, count;
};

struct APar {
    long long pc;      // parent's composite index
    int sx, sxy;       // strides of the parent's box (0: the parent is on level 0)
};

struct BoxTab {
    const ABox* box;
    int nlev, n0;
    int first[kMaxLevels], count[kMaxLevels];
    double dxi[kMaxLevels];
};

struct Range {
    long long first = 0, count = 0;
};

inline unsigned nblk(long long n) { return (unsigned)std::max<long long>(1, (n + kT - 1) / kT); }

// grid-stride reductions: at most 4 blocks per SM
inline unsigned norm_grid(const Ctx& c, long long n)
{
    return (unsigned)std::min<long long>(nblk(n), (long long)std::max(1, c.sm_count) * 4);
}

__host__ __device__ inline long long box_idx(const ABox& B, int i, int j, int k)
{
    return B.off + (long long)(i - B.lo[0] + kGW) +
           (long long)B.d[0] * ((long long)(j - B.lo[1] + kGW) + (long long)B.d[1] * (k - B.lo[2] + kGW));
}

__host__ __device__ inline bool box_has(const ABox& B, int i, int j, int k)
{
    return i >= B.lo[0] && i <= B.hi[0] && j >= B.lo[1] && j <= B.hi[1] && k >= B.lo[2] && k <= B.hi[2];
}

// composite index of the valid cell (i,j,k) (wrapped) of level l, or -1
__host__ __device__ inline long long tab_vidx(const BoxTab& T, int l, int i, int j, int k)
{
    const int n = T.n0 << l;
    i = wrapi(i, n);
    j = wrapi(j, n);
    k = wrapi(k, n);
    if (l == 0) return cidx(i, j, k, n);
    for (int b = T.first[l]; b < T.first[l] + T.count[l]; ++b)
        if (box_has(T.box[b], i, j, k)) return box_idx(T.box[b], i, j, k);
    return -1;
}

__host__ __device__ inline bool tab_covered(const BoxTab& T, int l, int i, int j, int k)
{
    if (l + 1 >= T.nlev) return false;
    const int n = T.n0 << l;
    return tab_vidx(T, l + 1, 2 * wrapi(i, n), 2 * wrapi(j, n), 2 * wrapi(k, n)) >= 0;
}

// ---------------------------------------------------------------------------
// particles
// ---------------------------------------------------------------------------
__global__ void k_amr_assign(BoxTab T, long long np, const double* __restrict__ x,
                             const double* __restrict__ y, const double* __restrict__ z, int* lev,
                             int* box)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int L = 0, B = -1;
    for (int l = T.nlev - 1; l >= 1 && B < 0; --l) {
        const double dxi = T.dxi[l];
        const int n = T.n0 << l;
        const int i = wrapi((int)floor(x[p] * dxi), n);
        const int j = wrapi((int)floor(y[p] * dxi), n);
        const int k = wrapi((int)floor(z[p] * dxi), n);
        for (int b = T.first[l]; b < T.first[l] + T.count[l]; ++b)
            if (box_has(T.box[b], i, j, k)) { L = l; B = b; break; }
    }
    lev[p] = L;
    box[p] = B;
}

struct PutItem {
    int l, i, j, k;
    double q;
};

// the corner mass q of level l at cell (i,j,k): coarser while not valid, then
// finer in eighths while covered
__device__ void amr_put(const BoxTab& T, int l, int i, int j, int k, double q, double* mass)
{
    while (tab_vidx(T, l, i, j, k) < 0) {
        const int n = T.n0 << l;
        i = wrapi(i, n) >> 1;
        j = wrapi(j, n) >> 1;
        k = wrapi(k, n) >> 1;
        --l;
    }
    PutItem st[8 * (kMaxLevels - 1) + 1];
    int top = 0;
    st[top++] = PutItem{l, i, j, k, q};
    while (top > 0) {
        const PutItem s = st[--top];
        if (tab_covered(T, s.l, s.i, s.j, s.k)) {
            const int n = T.n0 << s.l;
            const int ci = 2 * wrapi(s.i, n), cj = 2 * wrapi(s.j, n), ck = 2 * wrapi(s.k, n);
            const double q8 = s.q * 0.125;
            for (int c = 0; c < 8; ++c)
                st[top++] = PutItem{s.l + 1, ci + (c & 1), cj + ((c >> 1) & 1), ck + (c >> 2), q8};
        } else {
            atomicAdd(mass + tab_vidx(T, s.l, s.i, s.j, s.k), s.q);
        }
    }
}

__global__ void k_amr_deposit(BoxTab T, long long np, const double* __restrict__ x,
                              const double* __restrict__ y, const double* __restrict__ z,
                              const double* __restrict__ m, double mscalar, const int* __restrict__ lev,
                              double* mass)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int l = lev[p];
    const double dxi = T.dxi[l];
    const double lx = fma(x[p], dxi, 0.5), ly = fma(y[p], dxi, 0.5), lz = fma(z[p], dxi, 0.5);
    const double fi = floor(lx), fj = floor(ly), fk = floor(lz);
    const int i = (int)fi, j = (int)fj, k = (int)fk;
    const double fx = lx - fi, fy = ly - fj, fz = lz - fk;
    const double sx[2] = {1.0 - fx, fx}, sy[2] = {1.0 - fy, fy}, sz[2] = {1.0 - fz, fz};
    const double mp = m ? m[p] : mscalar;
    for (int cz = 0; cz < 2; ++cz)
        for (int cy = 0; cy < 2; ++cy)
            for (int cx = 0; cx < 2; ++cx)
                amr_put(T, l, i - 1 + cx, j - 1 + cy, k - 1 + cz, ((sx[cx] * sy[cy]) * sz[cz]) * mp, mass);
}

// update_dm_particle_single (DarkMatterParticleContainer.cpp:250-306) with the
// particle's own level's g; err counts stencils outside the box's ghost rings
__global__ void k_amr_move(BoxTab T, long long np, double* x, double* y, double* z, double* vx, double* vy,
                           double* vz, const int* __restrict__ lev, const int* __restrict__ box,
                           const double* __restrict__ g0, const double* __restrict__ g1,
                           const double* __restrict__ g2, double dt, double a_prev, double a_cur,
                           int do_move, unsigned long long* err)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const double half_dt = 0.5 * dt;
    const double a_cur_inv = 1.0 / a_cur;
    const double dt_a_cur_inv = dt * a_cur_inv;
    const int l = lev[p];
    const double dxi = T.dxi[l];
    const double lx = fma(x[p], dxi, 0.5), ly = fma(y[p], dxi, 0.5), lz = fma(z[p], dxi, 0.5);
    const double fi = floor(lx), fj = floor(ly), fk = floor(lz);
    const int i = (int)fi, j = (int)fj, k = (int)fk;
    const double xint = lx - fi, yint = ly - fj, zint = lz - fk;
    const double sx[2] = {1.0 - xint, xint}, sy[2] = {1.0 - yint, yint}, sz[2] = {1.0 - zint, zint};
    double w[8];
    long long cells[8];
    bool ok = true;
    for (int kk = 0; kk <= 1; ++kk)
        for (int jj = 0; jj <= 1; ++jj)
            for (int ii = 0; ii <= 1; ++ii) {
                const int t = ii + 2 * jj + 4 * kk;
                w[t] = (sx[1 - ii] * sy[1 - jj]) * sz[1 - kk];
                if (l == 0) {
                    const int n = T.n0;
                    cells[t] = cidx(wrapi(i - ii, n), wrapi(j - jj, n), wrapi(k - kk, n), n);
                } else {
                    const ABox& B = T.box[box[p]];
                    const int ci = i - ii, cj = j - jj, ck = k - kk;
                    if (ci < B.lo[0] - kGW || ci > B.hi[0] + kGW || cj < B.lo[1] - kGW || cj > B.hi[1] + kGW ||
                        ck < B.lo[2] - kGW || ck > B.hi[2] + kGW) {
                        ok = false;
                        cells[t] = B.off;
                    } else {
                        cells[t] = box_idx(B, ci, cj, ck);
                    }
                }
            }
    if (!ok) atomicAdd(err, 1ULL);
    const double* g[3] = {g0, g1, g2};
    double* v[3] = {vx + p, vy + p, vz + p};
    for (int d = 0; d < 3; ++d) {
        double val = 0.0;
        for (int t = 0; t < 8; ++t) val = fma(w[t], g[d][cells[t]], val);
        const double u = fma(a_prev, *v[d], half_dt * val);
        *v[d] = u * a_cur_inv;
    }
    if (do_move == 1) {
        x[p] = fma(dt_a_cur_inv, vx[p], x[p]);
        y[p] = fma(dt_a_cur_inv, vy[p], y[p]);
        z[p] = fma(dt_a_cur_inv, vz[p], z[p]);
    }
}

__global__ void k_amr_wrap(long long np, double L, double* x, double* y, double* z)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double* c[3] = {x, y, z};
    for (int d = 0; d < 3; ++d) {
        double v = c[d][p];
        if (v >= L) v = v - L;
        else if (v < 0.0) v = v + L;
        if (v >= L) v = 0.0;
        c[d][p] = v;
    }
}

__global__ void k_amr_unpack(long long np, const double* __restrict__ pos, const double* __restrict__ vel,
                             double* x, double* y, double* z, double* vx, double* vy, double* vz)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    x[p] = pos[3 * p];
    y[p] = pos[3 * p + 1];
    z[p] = pos[3 * p + 2];
    vx[p] = vel[3 * p];
    vy[p] = vel[3 * p + 1];
    vz[p] = vel[3 * p + 2];
}

__global__ void k_amr_pack(long long np, const double* x, const double* y, const double* z, const double* vx,
                           const double* vy, const double* vz, double* pos, double* vel)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    pos[3 * p] = x[p];
    pos[3 * p + 1] = y[p];
    pos[3 * p + 2] = z[p];
    vel[3 * p] = vx[p];
    vel[3 * p + 1] = vy[p];
    vel[3 * p + 2] = vz[p];
}

// ---------------------------------------------------------------------------
// fields
// ---------------------------------------------------------------------------
// dst = src * s on level 0 (q < n3) or on a list of fine cells
__global__ void k_amr_scale0(long long n3, const double* __restrict__ src, double s, double* dst)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n3) dst[q] = src[q] * s;
}

__global__ void k_amr_scalef(long long nc, const ACell* __restrict__ cells, const double* __restrict__ src,
                             double s, double* dst)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nc) dst[cells[t].q] = src[cells[t].q] * s;
}

// dst[P] = (sum of the 8 children of P in src, dk dj di order) * s
__global__ void k_amr_sum8(long long nr, const ARRec* __restrict__ r, const double* __restrict__ src, double s,
                           double* dst)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nr) return;
    const ARRec R = r[t];
    double v = 0.0;
    for (int dk = 0; dk < 2; ++dk)
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di) v = v + src[R.c0 + di + (long long)dj * R.sx + (long long)dk * R.sxy];
    dst[R.P] = v * s;
}

__device__ inline void block_add(double v, double* out)
{
    __shared__ double part[kT / 32];
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) part[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += part[i];
        atomicAdd(out, s);
    }
}

// sum of (rho - mass_offset) over the uncovered cells of level 0 / of a fine level
__global__ void k_amr_usum0(long long n3, const double* __restrict__ rho, const unsigned char* __restrict__ cov,
                            double mo, double* out)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double v = (q < n3 && !cov[q]) ? rho[q] - mo : 0.0;
    block_add(v, out);
}

__global__ void k_amr_usumf(long long nc, const ACell* __restrict__ cells, const double* __restrict__ rho,
                            const unsigned char* __restrict__ cov, double mo, double* out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (t < nc && !cov[cells[t].q]) v = rho[cells[t].q] - mo;
    block_add(v, out);
}

// mean = (sum over levels of S_l h_l^3) / L^3, levels in order
__global__ void k_amr_mean(int nlev, const double* __restrict__ S, const double* __restrict__ hcube, double L3,
                           double* mean)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int l = 0; l < nlev; ++l) s = s + S[l] * hcube[l];
    *mean = s / L3;
}

__device__ __forceinline__ double amr_beta(double rho, double mo, double mean, double ggrav, double ainv, double k0)
{
    return ((((rho - mo) - mean) * ggrav) * ainv) * k0;
}

__global__ void k_amr_beta0(long long n3, const double* __restrict__ rho, double mo, const double* __restrict__ mean,
                            double ggrav, double ainv, double k0, double* beta)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n3) beta[q] = amr_beta(rho[q], mo, *mean, ggrav, ainv, k0);
}

__global__ void k_amr_betaf(long long nc, const ACell* __restrict__ cells, const double* __restrict__ rho,
                            double mo, const double* __restrict__ mean, double ggrav, double ainv, double k0,
                            double* beta)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nc) beta[cells[t].q] = amr_beta(rho[cells[t].q], mo, *mean, ggrav, ainv, k0);
}

// ghost cells: f[dst] = sum of w * f[src] over the ghost's stencil (sources are valid cells)
__global__ void k_amr_ghost(long long ng, const AGhost* __restrict__ gh, const AEnt* __restrict__ ent, double* f)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ng) return;
    const AGhost G = gh[t];
    double v = 0.0;
    for (int e = 0; e < G.count; ++e) v = fma(ent[G.first + e].w, f[ent[G.first + e].src], v);
    f[G.dst] = v;
}

__global__ void k_amr_ghost3(long long ng, const AGhost* __restrict__ gh, const AEnt* __restrict__ ent, double* f0,
                             double* f1, double* f2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ng) return;
    const AGhost G = gh[t];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (int e = 0; e < G.count; ++e) {
        const AEnt E = ent[G.first + e];
        v0 = fma(E.w, f0[E.src], v0);
        v1 = fma(E.w, f1[E.src], v1);
        v2 = fma(E.w, f2[E.src], v2);
    }
    f0[G.dst] = v0;
    f1[G.dst] = v1;
    f2[G.dst] = v2;
}

// out = rhs - (s/6 - u), s the 6 neighbours in the order xm + xp, ym, yp, zm, zp
__global__ void k_amr_resid0(int n, const double* __restrict__ u, const double* __restrict__ rhs, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    double s = u[cidx(im, j, k, n)] + u[cidx(ip, j, k, n)];
    s = s + u[cidx(i, jm, k, n)];
    s = s + u[cidx(i, jp, k, n)];
    s = s + u[cidx(i, j, km, n)];
    s = s + u[cidx(i, j, kp, n)];
    const long long q = cidx(i, j, k, n);
    out[q] = rhs[q] - fma(s, kSixth, -u[q]);
}

__device__ __forceinline__ double nbr_fine(const double* __restrict__ u, long long q, long long sx, long long sxy)
{
    double s = u[q - 1] + u[q + 1];
    s = s + u[q - sx];
    s = s + u[q + sx];
    s = s + u[q - sxy];
    s = s + u[q + sxy];
    return s;
}

// Fine cells are numbered box by box (x fastest), boxes in level order;
// pref[b] is the number of fine cells in the boxes before b (every box has an
// even number of cells per row, so each colour holds half of each row and
// pref[b] / 2 numbers the cells of one colour).  find_box: the box of fine cell
// (or colour cell) g among the boxes [b0, b0 + nb).
__device__ __forceinline__ int find_box(const long long* __restrict__ pref, int b0, int nb, long long g, int half)
{
    int lo = b0, hi = b0 + nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const long long pm = half ? (pref[mid] >> 1) : pref[mid];
        if (pm <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// composite index of fine cell g (numbered from the first cell of box b0)
__device__ __forceinline__ long long fine_cell(const ABox* __restrict__ boxes, const long long* __restrict__ pref,
                                              int b0, int nb, long long t, int& b)
{
    const long long g = pref[b0] + t;
    b = find_box(pref, b0, nb, g, 0);
    const ABox& B = boxes[b];
    // a box holds fewer than 2^31 cells: 32-bit index arithmetic
    const unsigned r = (unsigned)(g - pref[b]);
    const unsigned nx = (unsigned)(B.hi[0] - B.lo[0] + 1), ny = (unsigned)(B.hi[1] - B.lo[1] + 1);
    const unsigned row = r / nx;
    const int u = (int)(r - row * nx);
    const unsigned k = row / ny;
    const int j = (int)(row - k * ny);
    return box_idx(B, B.lo[0] + u, B.lo[1] + j, B.lo[2] + (int)k);
}

// composite index of the t-th cell of colour col (numbered from box b0)
__device__ __forceinline__ long long fine_color_cell(const ABox* __restrict__ boxes, const long long* __restrict__ pref,
                                                    int b0, int nb, long long t, int col, int& b, int* ijk = nullptr)
{
    const long long g = (pref[b0] >> 1) + t;
    b = find_box(pref, b0, nb, g, 1);
    const ABox& B = boxes[b];
    const unsigned r = (unsigned)(g - (pref[b] >> 1));
    const unsigned hx = (unsigned)(B.hi[0] - B.lo[0] + 1) >> 1, ny = (unsigned)(B.hi[1] - B.lo[1] + 1);
    const unsigned row = r / hx;
    const int tp = (int)(r - row * hx);
    const unsigned kk = row / ny;
    const int j = B.lo[1] + (int)(row - kk * ny), k = B.lo[2] + (int)kk;
    const int i = B.lo[0] + 2 * tp + ((col - B.lo[0] - j - k) & 1);
    if (ijk) {
        ijk[0] = i;
        ijk[1] = j;
        ijk[2] = k;
    }
    return box_idx(B, i, j, k);
}

// out = rhs - (s/6 - u) on the n fine cells from box b0
__global__ void k_amr_residf(long long n, int b0, int nb, const long long* __restrict__ pref,
                             const ABox* __restrict__ boxes, const double* __restrict__ u,
                             const double* __restrict__ rhs, double* out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int b;
    const long long q = fine_cell(boxes, pref, b0, nb, t, b);
    const long long sx = boxes[b].d[0], sxy = (long long)boxes[b].d[0] * boxes[b].d[1];
    out[q] = rhs[q] - fma(nbr_fine(u, q, sx, sxy), kSixth, -u[q]);
}

// one colour of a Gauss-Seidel sweep on the n colour cells from box b0
__global__ void k_amr_gsrbf(long long n, int b0, int nb, const long long* __restrict__ pref,
                            const ABox* __restrict__ boxes, int col, double* e, const double* __restrict__ R)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int b;
    const long long q = fine_color_cell(boxes, pref, b0, nb, t, col, b);
    const long long sx = boxes[b].d[0], sxy = (long long)boxes[b].d[0] * boxes[b].d[1];
    e[q] = fma(nbr_fine(e, q, sx, sxy), kSixth, -R[q]);
}

// R(C) -= ((sum_k (u(f_k) - u(g_k))) / 2 - (u(N) - u(C))) / 6 at each coarse/fine face of C
__global__ void k_amr_reflux(long long nr, const AFRec* __restrict__ recs, const AFace* __restrict__ faces,
                             const double* __restrict__ u, double* R)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nr) return;
    const AFRec r = recs[t];
    double v = R[r.C];
    for (int f = r.first; f < r.first + r.count; ++f) {
        const AFace& F = faces[f];
        double s = u[F.f[0]] - u[F.g[0]];
        s = s + (u[F.f[1]] - u[F.g[1]]);
        s = s + (u[F.f[2]] - u[F.g[2]]);
        s = s + (u[F.f[3]] - u[F.g[3]]);
        v = v - (((s * 0.5) - (u[F.N] - u[r.C])) * kSixth);
    }
    R[r.C] = v;
}

// e += the trilinear prolongation of the coarser level's e
__global__ void k_amr_prolong(long long nc, const ACell* __restrict__ cells, const APar* __restrict__ par, int n0,
                              double* e)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc) return;
    const ACell c = cells[t];
    const APar P = par[t];
    const int I = c.i >> 1, J = c.j >> 1, K = c.k >> 1;
    const int di = (c.i & 1) ? 1 : -1, dj = (c.j & 1) ? 1 : -1, dk = (c.k & 1) ? 1 : -1;
    double s = 0.0;
    for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a)
            for (int u = 0; u < 2; ++u) {
                long long src;
                if (P.sx == 0) {
                    src = cidx(wrapi(I + u * di, n0), wrapi(J + a * dj, n0), wrapi(K + b * dk, n0), n0);
                } else {
                    src = P.pc + (long long)(u * di) + (long long)(a * dj) * P.sx + (long long)(b * dk) * P.sxy;
                }
                s = fma(kAmrProlongW[u + 2 * a + 4 * b], e[src], s);
            }
    e[c.q] = e[c.q] + s;
}

// the same on the black cells only (the red ones are overwritten by the red half
// sweep that follows), for levels whose boxes each have their parents in one
// coarser box (or on level 0)
__global__ void k_amr_prolong_black(long long n, int b0, int nb, const long long* __restrict__ pref,
                                    const ABox* __restrict__ boxes, int n0, double* e)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int b, c[3];
    const long long q = fine_color_cell(boxes, pref, b0, nb, t, 1, b, c);
    const ABox& B = boxes[b];
    const int I = c[0] >> 1, J = c[1] >> 1, K = c[2] >> 1;
    const int di = (c[0] & 1) ? 1 : -1, dj = (c[1] & 1) ? 1 : -1, dk = (c[2] & 1) ? 1 : -1;
    long long pc = 0, sx = 0, sxy = 0;
    if (B.pbox >= 0) {
        const ABox& P = boxes[B.pbox];
        pc = box_idx(P, I, J, K);
        sx = P.d[0];
        sxy = (long long)P.d[0] * P.d[1];
    }
    double s = 0.0;
    for (int bz = 0; bz < 2; ++bz)
        for (int a = 0; a < 2; ++a)
            for (int u = 0; u < 2; ++u) {
                const long long src = B.pbox < 0
                    ? cidx(wrapi(I + u * di, n0), wrapi(J + a * dj, n0), wrapi(K + bz * dk, n0), n0)
                    : pc + (long long)(u * di) + (long long)(a * dj) * sx + (long long)(bz * dk) * sxy;
                s = fma(kAmrProlongW[u + 2 * a + 4 * bz], e[src], s);
            }
    e[q] = e[q] + s;
}

__global__ void k_amr_add(long long n, double* phi, const double* __restrict__ e)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) phi[q] = phi[q] + e[q];
}

// max |f| * inv_scale over the uncovered cells into out (as the bits of a
// non-negative double): a block maximum, then one atomic per block
__device__ __forceinline__ void block_umax(unsigned long long v, unsigned long long* out)
{
    __shared__ unsigned long long part[kT / 32];
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = part[w] > v ? part[w] : v;
        if (v != 0ULL) atomicMax(out, v);
    }
}

// (the maximum is taken over the bit patterns: equal to the maximum of the
// non-negative values, and a NaN, whose bits are above every number's, wins)
__device__ __forceinline__ unsigned long long umax_bits(unsigned long long v, double x)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return u > v ? u : v;
}

__global__ void k_amr_absmax0(long long n3, const double* __restrict__ f, const unsigned char* __restrict__ cov,
                              double inv_scale, unsigned long long* out)
{
    unsigned long long v = 0ULL;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (long long)gridDim.x * blockDim.x)
        if (!cov[q]) v = umax_bits(v, fabs(f[q]) * inv_scale);
    block_umax(v, out);
}

__global__ void k_amr_absmaxf(long long n, int b0, int nb, const long long* __restrict__ pref,
                              const ABox* __restrict__ boxes, const double* __restrict__ f,
                              const unsigned char* __restrict__ cov, const double* __restrict__ inv_scale,
                              unsigned long long* out)
{
    unsigned long long v = 0ULL;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int b;
        const long long q = fine_cell(boxes, pref, b0, nb, t, b);
        if (!cov[q]) v = umax_bits(v, fabs(f[q]) * inv_scale[boxes[b].lev]);
    }
    block_umax(v, out);
}

// the single-level cell-centred gravity vector on level 0 / on fine cells
__device__ __forceinline__ void grav_one(const double* __restrict__ phi, long long q, long long xm, long long xp,
                                         long long ym, long long yp, long long zm, long long zp, double dxi,
                                         double* g0, double* g1, double* g2)
{
    const double pc = phi[q];
    g0[q] = 0.5 * fma(phi[xp] - pc, dxi, (pc - phi[xm]) * dxi);
    g1[q] = 0.5 * fma(phi[yp] - pc, dxi, (pc - phi[ym]) * dxi);
    g2[q] = 0.5 * fma(phi[zp] - pc, dxi, (pc - phi[zm]) * dxi);
}

__global__ void k_amr_grav0(int n, double dxi, const double* __restrict__ phi, double* g0, double* g1, double* g2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    grav_one(phi, cidx(i, j, k, n), cidx(wrapi(i - 1, n), j, k, n), cidx(wrapi(i + 1, n), j, k, n),
             cidx(i, wrapi(j - 1, n), k, n), cidx(i, wrapi(j + 1, n), k, n), cidx(i, j, wrapi(k - 1, n), n),
             cidx(i, j, wrapi(k + 1, n), n), dxi, g0, g1, g2);
}

__global__ void k_amr_gravf(long long nc, const ACell* __restrict__ cells, const ABox* __restrict__ boxes,
                            const double* __restrict__ dxi_l, const double* __restrict__ phi, double* g0, double* g1,
                            double* g2)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc) return;
    const ACell c = cells[t];
    const ABox& B = boxes[c.box];
    const long long sx = B.d[0], sxy = (long long)B.d[0] * B.d[1];
    grav_one(phi, c.q, c.q - 1, c.q + 1, c.q - sx, c.q + sx, c.q - sxy, c.q + sxy, dxi_l[B.lev], g0, g1, g2);
}

// a valid field of level 0 or of one box into natural order
__global__ void k_amr_box_out(ABox B, const double* __restrict__ f, double* out)
{
    const int nx = B.hi[0] - B.lo[0] + 1, ny = B.hi[1] - B.lo[1] + 1, nz = B.hi[2] - B.lo[2] + 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nx * ny * nz) return;
    const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((long long)nx * ny));
    out[t] = f[box_idx(B, B.lo[0] + i, B.lo[1] + j, B.lo[2] + k)];
}

}  // namespace

// ---------------------------------------------------------------------------
// the hierarchy
// ---------------------------------------------------------------------------
struct nyxpm_amr {
    int n0 = 0, nlev = 1;
    double L = 0;
    int64_t np = 0;
    int uploaded = 0;
    int uniform_mass = 1;
    double mscalar = 0, mass_offset = 0;
    std::vector<ABox> boxes;
    BoxTab tab{};                       // device pointer to the box table
    long long ntot = 0;
    // per level: ranges in the device lists
    // ghost1[l]: the ring-1 ghosts of level l, its copies of same-level cells first
    // (ghost1_same[l]), then the ones interpolated from coarser levels
    Range cells[kMaxLevels], ghost1[kMaxLevels], ghost1_same[kMaxLevels], ghost23[kMaxLevels], rrec[kMaxLevels],
        frec[kMaxLevels];
    int prolong_black_ok[kMaxLevels] = {0, 0, 0, 0};
    Range fine_cells, all_ghost1, all_ghost23, all_frec;
    double scale[kMaxLevels], inv_scale[kMaxLevels], hcube[kMaxLevels], dxi[kMaxLevels];
    // device lists
    ABox* d_boxes = nullptr;
    ACell* d_cells = nullptr;      // every fine cell, level by level
    long long* d_pref = nullptr;   // fine cells in the boxes before box b (b = 0 .. nboxes)
    APar* d_par = nullptr;         // aligned with d_cells
    AGhost* d_ghost = nullptr;
    AEnt* d_ent = nullptr;
    ARRec* d_rrec = nullptr;
    AFRec* d_frec = nullptr;
    AFace* d_face = nullptr;
    unsigned char* d_cov = nullptr;
    double* d_level = nullptr;     // [0..3] usum, [4..7] hcube, [8..11] inv_scale, [12..15] dxi, [16] mean
    // composite fields
    double *mass = nullptr, *rho = nullptr, *beta = nullptr, *phi = nullptr, *R = nullptr, *e = nullptr,
           *T = nullptr, *g[3] = {nullptr, nullptr, nullptr};
    // particles
    double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr, *m = nullptr;
    int *lev = nullptr, *box = nullptr;
    double* staging = nullptr;
    unsigned long long* norms = nullptr;     // [0] ||beta||, [1] ||r||, [2] move errors
    unsigned long long* h_norms = nullptr;
    nyxpm_box* mg = nullptr;                 // level 0's multigrid hierarchy
    std::vector<void*> allocs;
};

namespace {

nyxpm_status afail(nyxpm_ctx* c, nyxpm_status st, const std::string& msg)
{
    if (c) c->err = msg;
    return st;
}

template <typename T>
nyxpm_status aalloc(nyxpm_ctx* c, nyxpm_amr* a, T** p, size_t count)
{
    if (count == 0) count = 1;
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, sizeof(T) * count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return afail(c, NYXPM_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    a->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return NYXPM_OK;
}

template <typename T>
nyxpm_status upload_vec(nyxpm_ctx* c, nyxpm_amr* a, T** p, const std::vector<T>& v)
{
    nyxpm_status st = aalloc(c, a, p, v.size());
    if (st != NYXPM_OK) return st;
    if (!v.empty()) cudaMemcpyAsync(*p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->stream);
    return NYXPM_OK;
}

// host builder of the index structures
struct Builder {
    nyxpm_amr& A;
    BoxTab H;   // host copy of the table (box points at A.boxes)

    explicit Builder(nyxpm_amr& a) : A(a)
    {
        H = A.tab;
        H.box = A.boxes.data();
    }

    long long vidx(int l, int i, int j, int k) const { return tab_vidx(H, l, i, j, k); }
    bool covered(int l, int i, int j, int k) const { return tab_covered(H, l, i, j, k); }
    int owner(int l, int i, int j, int k) const
    {
        const int n = A.n0 << l;
        i = wrapi(i, n);
        j = wrapi(j, n);
        k = wrapi(k, n);
        for (int b = H.first[l]; b < H.first[l] + H.count[l]; ++b)
            if (box_has(A.boxes[b], i, j, k)) return b;
        return -1;
    }

    // the sources and weights of level l's value at cell (i,j,k)
    void gen(int l, int i, int j, int k, double w, std::vector<AEnt>& out) const
    {
        const long long v = vidx(l, i, j, k);
        if (v >= 0) {
            out.push_back(AEnt{v, w});
            return;
        }
        const int n = A.n0 << l;
        const int c[3] = {wrapi(i, n), wrapi(j, n), wrapi(k, n)};
        int I0[3];
        double t[3];
        for (int d = 0; d < 3; ++d) {
            if (c[d] & 1) {
                I0[d] = (c[d] - 1) / 2;
                t[d] = 0.25;
            } else {
                I0[d] = c[d] / 2 - 1;
                t[d] = 0.75;
            }
        }
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    const double wx = di ? t[0] : 1.0 - t[0];
                    const double wy = dj ? t[1] : 1.0 - t[1];
                    const double wz = dk ? t[2] : 1.0 - t[2];
                    gen(l - 1, I0[0] + di, I0[1] + dj, I0[2] + dk, w * ((wx * wy) * wz), out);
                }
    }
};

nyxpm_status build_lists(nyxpm_ctx* c, nyxpm_amr* a)
{
    nyxpm_amr& A = *a;
    Builder Bd(A);
    const int n0 = A.n0;
    std::vector<ACell> cells;
    std::vector<long long> pref(1, 0);
    std::vector<APar> par;
    std::vector<AGhost> ghost;
    std::vector<AEnt> ent;
    std::vector<ARRec> rrec;
    std::vector<AFRec> frec;
    std::vector<AFace> face;
    std::vector<unsigned char> cov((size_t)A.ntot, 0);
    // fine cells, level by level, and their parents
    for (int l = 1; l < A.nlev; ++l) {
        A.cells[l].first = (long long)cells.size();
        for (int b = A.tab.first[l]; b < A.tab.first[l] + A.tab.count[l]; ++b) {
            const ABox& B = A.boxes[b];
            for (int k = B.lo[2]; k <= B.hi[2]; ++k)
                for (int j = B.lo[1]; j <= B.hi[1]; ++j)
                    for (int i = B.lo[0]; i <= B.hi[0]; ++i) {
                        cells.push_back(ACell{box_idx(B, i, j, k), i, j, k, b});
                        APar P{};
                        if (l - 1 == 0) {
                            P.pc = cidx(i >> 1, j >> 1, k >> 1, n0);
                        } else {
                            const int o = Bd.owner(l - 1, i >> 1, j >> 1, k >> 1);
                            const ABox& PB = A.boxes[o];
                            P.pc = box_idx(PB, i >> 1, j >> 1, k >> 1);
                            P.sx = PB.d[0];
                            P.sxy = PB.d[0] * PB.d[1];
                        }
                        par.push_back(P);
                    }
            pref.push_back((long long)cells.size());
        }
        A.cells[l].count = (long long)cells.size() - A.cells[l].first;
    }
    A.fine_cells = Range{0, (long long)cells.size()};
    // covered flags
    for (int k = 0; k < n0; ++k)
        for (int j = 0; j < n0; ++j)
            for (int i = 0; i < n0; ++i)
                if (Bd.covered(0, i, j, k)) cov[cidx(i, j, k, n0)] = 1;
    for (const ACell& cl : cells)
        if (Bd.covered(A.boxes[cl.box].lev, cl.i, cl.j, cl.k)) cov[cl.q] = 1;
    // ghost stencils: all ring-1 ghosts level by level, then rings 2-3
    for (int pass = 0; pass < 2; ++pass)
        for (int l = 1; l < A.nlev; ++l) {
            Range& R = pass == 0 ? A.ghost1[l] : A.ghost23[l];
            R.first = (long long)ghost.size();
            std::vector<AGhost> same, interp;
            for (int b = A.tab.first[l]; b < A.tab.first[l] + A.tab.count[l]; ++b) {
                const ABox& B = A.boxes[b];
                for (int k = B.lo[2] - kGW; k <= B.hi[2] + kGW; ++k)
                    for (int j = B.lo[1] - kGW; j <= B.hi[1] + kGW; ++j)
                        for (int i = B.lo[0] - kGW; i <= B.hi[0] + kGW; ++i) {
                            const int dist = std::max({B.lo[0] - i, i - B.hi[0], B.lo[1] - j, j - B.hi[1],
                                                       B.lo[2] - k, k - B.hi[2], 0});
                            if (dist == 0 || (pass == 0) != (dist == 1)) continue;
                            AGhost G{box_idx(B, i, j, k), (int)ent.size(), 0};
                            Bd.gen(l, i, j, k, 1.0, ent);
                            G.count = (int)ent.size() - G.first;
                            (Bd.vidx(l, i, j, k) >= 0 ? same : interp).push_back(G);
                        }
            }
            if (pass == 0) A.ghost1_same[l] = Range{(long long)ghost.size(), (long long)same.size()};
            ghost.insert(ghost.end(), same.begin(), same.end());
            ghost.insert(ghost.end(), interp.begin(), interp.end());
            R.count = (long long)ghost.size() - R.first;
        }
    A.all_ghost1 = Range{0, A.nlev > 1 ? A.ghost1[A.nlev - 1].first + A.ghost1[A.nlev - 1].count : 0};
    A.all_ghost23 = Range{A.all_ghost1.count, (long long)ghost.size() - A.all_ghost1.count};
    // restriction records and coarse/fine faces
    for (int l = 1; l < A.nlev; ++l) {
        A.rrec[l].first = (long long)rrec.size();
        for (int b = A.tab.first[l]; b < A.tab.first[l] + A.tab.count[l]; ++b) {
            const ABox& B = A.boxes[b];
            for (int K = B.lo[2] / 2; K <= B.hi[2] / 2; ++K)
                for (int J = B.lo[1] / 2; J <= B.hi[1] / 2; ++J)
                    for (int I = B.lo[0] / 2; I <= B.hi[0] / 2; ++I)
                        rrec.push_back(ARRec{Bd.vidx(l - 1, I, J, K), box_idx(B, 2 * I, 2 * J, 2 * K), B.d[0],
                                             B.d[0] * B.d[1]});
        }
        A.rrec[l].count = (long long)rrec.size() - A.rrec[l].first;
        A.frec[l].first = (long long)frec.size();
        auto faces_of = [&](int i, int j, int k, long long C) {
            if (Bd.covered(l - 1, i, j, k)) return;
            AFRec r{C, (int)face.size(), 0};
            const int n = A.n0 << (l - 1);
            for (int d = 0; d < 3; ++d)
                for (int s = -1; s <= 1; s += 2) {
                    int nb[3] = {i, j, k};
                    nb[d] += s;
                    if (!Bd.covered(l - 1, nb[0], nb[1], nb[2])) continue;
                    for (int t = 0; t < 3; ++t) nb[t] = wrapi(nb[t], n);
                    AFace F{};
                    F.N = Bd.vidx(l - 1, nb[0], nb[1], nb[2]);
                    const int ta = d == 0 ? 1 : 0, tb = d == 2 ? 1 : 2;
                    int kk = 0;
                    for (int ob = 0; ob < 2; ++ob)
                        for (int oa = 0; oa < 2; ++oa, ++kk) {
                            int fc[3];
                            fc[d] = 2 * nb[d] + (s > 0 ? 0 : 1);
                            fc[ta] = 2 * nb[ta] + oa;
                            fc[tb] = 2 * nb[tb] + ob;
                            const ABox& FB = A.boxes[Bd.owner(l, fc[0], fc[1], fc[2])];
                            F.f[kk] = box_idx(FB, fc[0], fc[1], fc[2]);
                            int gc[3] = {fc[0], fc[1], fc[2]};
                            gc[d] -= s;
                            F.g[kk] = box_idx(FB, gc[0], gc[1], gc[2]);
                        }
                    face.push_back(F);
                    r.count += 1;
                }
            if (r.count > 0) frec.push_back(r);
        };
        if (l - 1 == 0) {
            for (int k = 0; k < n0; ++k)
                for (int j = 0; j < n0; ++j)
                    for (int i = 0; i < n0; ++i) faces_of(i, j, k, cidx(i, j, k, n0));
        } else {
            for (long long t = A.cells[l - 1].first; t < A.cells[l - 1].first + A.cells[l - 1].count; ++t)
                faces_of(cells[t].i, cells[t].j, cells[t].k, cells[t].q);
        }
        A.frec[l].count = (long long)frec.size() - A.frec[l].first;
    }
    A.all_frec = Range{0, (long long)frec.size()};
    nyxpm_status st;
    if ((st = upload_vec(c, a, &A.d_cells, cells)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_pref, pref)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_par, par)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_ghost, ghost)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_ent, ent)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_rrec, rrec)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_frec, frec)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_face, face)) != NYXPM_OK) return st;
    if ((st = upload_vec(c, a, &A.d_cov, cov)) != NYXPM_OK) return st;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return check_launch(*c, "hierarchy lists");
    return NYXPM_OK;
}

// ---------------------------------------------------------------------------
// launch sequences
// ---------------------------------------------------------------------------
nyxpm_status ghost_fill(Ctx& c, nyxpm_amr& A, double* f, const Range& r)
{
    if (r.count == 0) return NYXPM_OK;
    prof_begin(c);
    k_amr_ghost<<<nblk(r.count), kT, 0, c.stream>>>(r.count, A.d_ghost + r.first, A.d_ent, f);
    prof_end(c, NYXPM_ST_SMOOTH, 40.0 * r.count);
    return check_launch(c, "ghost fill");
}

nyxpm_status avg_down(Ctx& c, nyxpm_amr& A, double* f)
{
    for (int l = A.nlev - 1; l >= 1; --l) {
        prof_begin(c);
        k_amr_sum8<<<nblk(A.rrec[l].count), kT, 0, c.stream>>>(A.rrec[l].count, A.d_rrec + A.rrec[l].first, f,
                                                                 0.125, f);
        prof_end(c, NYXPM_ST_RESTRICT, 96.0 * A.rrec[l].count);
    }
    return check_launch(c, "average down");
}

nyxpm_status deposit(Ctx& c, nyxpm_amr& A)
{
    const long long n3 = (long long)A.n0 * A.n0 * A.n0;
    cudaMemsetAsync(A.mass, 0, sizeof(double) * A.ntot, c.stream);
    prof_begin(c);
    k_amr_deposit<<<nblk(A.np), kT, 0, c.stream>>>(A.tab, A.np, A.x, A.y, A.z, A.uniform_mass ? nullptr : A.m,
                                                   A.mscalar, A.lev, A.mass);
    prof_end(c, NYXPM_ST_DEPOSIT, 36.0 * A.np);
    const double h0 = A.L / A.n0;
    prof_begin(c);
    k_amr_scale0<<<nblk(n3), kT, 0, c.stream>>>(n3, A.mass, 1.0 / ((h0 * h0) * h0), A.rho);
    prof_end(c, NYXPM_ST_DEPOSIT, 16.0 * n3);
    for (int l = 1; l < A.nlev; ++l) {
        const double h = A.L / (A.n0 << l);
        const Range& r = A.cells[l];
        prof_begin(c);
        k_amr_scalef<<<nblk(r.count), kT, 0, c.stream>>>(r.count, A.d_cells + r.first, A.mass,
                                                         1.0 / ((h * h) * h), A.rho);
        prof_end(c, NYXPM_ST_DEPOSIT, 40.0 * r.count);
    }
    nyxpm_status st = check_launch(c, "multilevel deposit");
    if (st != NYXPM_OK) return st;
    return avg_down(c, A, A.rho);
}

// the composite residual of phi into R (phi's covered cells averaged and ghosts
// filled first); its norm into norms[slot]
nyxpm_status comp_resid(Ctx& c, nyxpm_amr& A, int slot)
{
    nyxpm_status st;
    const long long n3 = (long long)A.n0 * A.n0 * A.n0;
    if ((st = avg_down(c, A, A.phi)) != NYXPM_OK) return st;
    if ((st = ghost_fill(c, A, A.phi, A.all_ghost1)) != NYXPM_OK) return st;
    const Geo g = geo3(A.n0, A.n0, A.n0);
    prof_begin(c);
    k_amr_resid0<<<g.grid, g.block, 0, c.stream>>>(A.n0, A.phi, A.beta, A.R);
    prof_end(c, NYXPM_ST_NORM, 24.0 * n3);
    if (A.fine_cells.count) {
        prof_begin(c);
        k_amr_residf<<<nblk(A.fine_cells.count), kT, 0, c.stream>>>(A.fine_cells.count, 0, (int)A.boxes.size(),
                                                                     A.d_pref, A.d_boxes, A.phi, A.beta, A.R);
        prof_end(c, NYXPM_ST_NORM, 48.0 * A.fine_cells.count);
    }
    if (A.all_frec.count) {
        prof_begin(c);
        k_amr_reflux<<<nblk(A.all_frec.count), kT, 0, c.stream>>>(A.all_frec.count, A.d_frec, A.d_face, A.phi,
                                                                   A.R);
        prof_end(c, NYXPM_ST_NORM, 96.0 * A.all_frec.count);
    }
    cudaMemsetAsync(A.norms + slot, 0, sizeof(unsigned long long), c.stream);
    prof_begin(c);
    k_amr_absmax0<<<norm_grid(c, n3), kT, 0, c.stream>>>(n3, A.R, A.d_cov, A.inv_scale[0], A.norms + slot);
    prof_end(c, NYXPM_ST_NORM, 9.0 * n3);
    if (A.fine_cells.count) {
        prof_begin(c);
        k_amr_absmaxf<<<norm_grid(c, A.fine_cells.count), kT, 0, c.stream>>>(
            A.fine_cells.count, 0, (int)A.boxes.size(), A.d_pref, A.d_boxes, A.R, A.d_cov, A.d_level + 8,
            A.norms + slot);
        prof_end(c, NYXPM_ST_NORM, 33.0 * A.fine_cells.count);
    }
    return check_launch(c, "composite residual");
}

// nsweeps red-black sweeps of level l's correction.  A ring-1 ghost is either a
// copy of a same-level cell or an interpolation of coarser levels, and those do
// not change while level l smooths: the interpolated ghosts are filled once, at
// the start (fill_interp; not on the way down, where every coarser correction
// and so every such ghost is still zero), the copies before each colour.
nyxpm_status smooth_level(Ctx& c, nyxpm_amr& A, int l, int nsweeps, int fill_interp)
{
    nyxpm_status st;
    const long long half = A.cells[l].count / 2;
    for (int s = 0; s < nsweeps; ++s)
        for (int col = 0; col < 2; ++col) {
            const bool all = fill_interp && s == 0 && col == 0;
            if ((st = ghost_fill(c, A, A.e, all ? A.ghost1[l] : A.ghost1_same[l])) != NYXPM_OK) return st;
            prof_begin(c);
            k_amr_gsrbf<<<nblk(half), kT, 0, c.stream>>>(half, A.tab.first[l], A.tab.count[l], A.d_pref, A.d_boxes,
                                                         col, A.e, A.R);
            prof_end(c, NYXPM_ST_SMOOTH, 24.0 * half, 1);
        }
    return check_launch(c, "fine smoother");
}

nyxpm_status vcycle(nyxpm_ctx* cx, nyxpm_amr& A)
{
    Ctx& c = *cx;
    nyxpm_status st;
    const int nu1 = c.p.nu1, nu2 = c.p.nu2;
    cudaMemsetAsync(A.e, 0, sizeof(double) * A.ntot, c.stream);
    for (int l = A.nlev - 1; l >= 1; --l) {
        if ((st = smooth_level(c, A, l, nu1, 0)) != NYXPM_OK) return st;
        if ((st = ghost_fill(c, A, A.e, A.ghost1_same[l])) != NYXPM_OK) return st;
        const Range& r = A.cells[l];
        prof_begin(c);
        k_amr_residf<<<nblk(r.count), kT, 0, c.stream>>>(r.count, A.tab.first[l], A.tab.count[l], A.d_pref,
                                                         A.d_boxes, A.e, A.R, A.T);
        prof_end(c, NYXPM_ST_RESTRICT, 48.0 * r.count);
        prof_begin(c);
        k_amr_sum8<<<nblk(A.rrec[l].count), kT, 0, c.stream>>>(A.rrec[l].count, A.d_rrec + A.rrec[l].first, A.T,
                                                                 0.5, A.R);
        prof_end(c, NYXPM_ST_RESTRICT, 96.0 * A.rrec[l].count);
        if (A.frec[l].count) {
            prof_begin(c);
            k_amr_reflux<<<nblk(A.frec[l].count), kT, 0, c.stream>>>(A.frec[l].count, A.d_frec + A.frec[l].first,
                                                                      A.d_face, A.e, A.R);
            prof_end(c, NYXPM_ST_RESTRICT, 96.0 * A.frec[l].count);
        }
        if ((st = check_launch(c, "composite restriction")) != NYXPM_OK) return st;
    }
    if ((st = mg_vcycle_zero(c, *A.mg, A.R, A.e)) != NYXPM_OK) return st;
    for (int l = 1; l < A.nlev; ++l) {
        // the parents' neighbours are valid coarser cells: in the parent's box or
        // in the copies of its ring
        if (l - 1 >= 1 && (st = ghost_fill(c, A, A.e, A.ghost1_same[l - 1])) != NYXPM_OK) return st;
        const Range& r = A.cells[l];
        prof_begin(c);
        if (nu2 > 0 && A.prolong_black_ok[l]) {
            k_amr_prolong_black<<<nblk(r.count / 2), kT, 0, c.stream>>>(r.count / 2, A.tab.first[l], A.tab.count[l],
                                                                       A.d_pref, A.d_boxes, A.n0, A.e);
            prof_end(c, NYXPM_ST_PROLONG, 48.0 * r.count);
        } else {
            k_amr_prolong<<<nblk(r.count), kT, 0, c.stream>>>(r.count, A.d_cells + r.first, A.d_par + r.first, A.n0,
                                                              A.e);
            prof_end(c, NYXPM_ST_PROLONG, 96.0 * r.count);
        }
        if ((st = check_launch(c, "composite prolongation")) != NYXPM_OK) return st;
        if ((st = smooth_level(c, A, l, nu2, 1)) != NYXPM_OK) return st;
    }
    prof_begin(c);
    k_amr_add<<<nblk(A.ntot), kT, 0, c.stream>>>(A.ntot, A.phi, A.e);
    prof_end(c, NYXPM_ST_PROLONG, 24.0 * A.ntot);
    return check_launch(c, "composite update");
}

double read_bits(const unsigned long long* h, int slot)
{
    double v;
    std::memcpy(&v, h + slot, sizeof(v));
    return v;
}

nyxpm_status solve(nyxpm_ctx* cx, nyxpm_amr& A, double a, nyxpm_solve_info* info)
{
    Ctx& c = *cx;
    nyxpm_status st;
    const long long n3 = (long long)A.n0 * A.n0 * A.n0;
    // right-hand side with the solvability correction over the uncovered cells
    cudaMemsetAsync(A.d_level, 0, sizeof(double) * kMaxLevels, c.stream);
    prof_begin(c);
    k_amr_usum0<<<nblk(n3), kT, 0, c.stream>>>(n3, A.rho, A.d_cov, A.mass_offset, A.d_level);
    prof_end(c, NYXPM_ST_RHS, 9.0 * n3);
    for (int l = 1; l < A.nlev; ++l) {
        const Range& r = A.cells[l];
        prof_begin(c);
        k_amr_usumf<<<nblk(r.count), kT, 0, c.stream>>>(r.count, A.d_cells + r.first, A.rho, A.d_cov,
                                                        A.mass_offset, A.d_level + l);
        prof_end(c, NYXPM_ST_RHS, 33.0 * r.count);
    }
    prof_begin(c);
    k_amr_mean<<<1, 32, 0, c.stream>>>(A.nlev, A.d_level, A.d_level + 4, (A.L * A.L) * A.L, A.d_level + 16);
    prof_end(c, NYXPM_ST_RHS, 0);
    const double ggrav = -4.0 * M_PI * c.p.gconst, ainv = 1.0 / a;
    prof_begin(c);
    k_amr_beta0<<<nblk(n3), kT, 0, c.stream>>>(n3, A.rho, A.mass_offset, A.d_level + 16, ggrav, ainv, A.scale[0],
                                               A.beta);
    prof_end(c, NYXPM_ST_RHS, 16.0 * n3);
    for (int l = 1; l < A.nlev; ++l) {
        const Range& r = A.cells[l];
        prof_begin(c);
        k_amr_betaf<<<nblk(r.count), kT, 0, c.stream>>>(r.count, A.d_cells + r.first, A.rho, A.mass_offset,
                                                        A.d_level + 16, ggrav, ainv, A.scale[l], A.beta);
        prof_end(c, NYXPM_ST_RHS, 40.0 * r.count);
    }
    if ((st = check_launch(c, "multilevel rhs")) != NYXPM_OK) return st;
    cudaMemsetAsync(A.phi, 0, sizeof(double) * A.ntot, c.stream);
    cudaMemsetAsync(A.norms, 0, sizeof(unsigned long long), c.stream);
    prof_begin(c);
    k_amr_absmax0<<<norm_grid(c, n3), kT, 0, c.stream>>>(n3, A.beta, A.d_cov, A.inv_scale[0], A.norms);
    prof_end(c, NYXPM_ST_NORM, 9.0 * n3);
    if (A.fine_cells.count) {
        prof_begin(c);
        k_amr_absmaxf<<<norm_grid(c, A.fine_cells.count), kT, 0, c.stream>>>(
            A.fine_cells.count, 0, (int)A.boxes.size(), A.d_pref, A.d_boxes, A.beta, A.d_cov, A.d_level + 8,
            A.norms);
        prof_end(c, NYXPM_ST_NORM, 33.0 * A.fine_cells.count);
    }
    if ((st = comp_resid(c, A, 1)) != NYXPM_OK) return st;
    cudaMemcpyAsync(A.h_norms, A.norms, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c.stream);
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return check_launch(c, "multilevel solve sync");
    const double bnorm = read_bits(A.h_norms, 0), r0 = read_bits(A.h_norms, 1);
    const double target = c.p.rel_tol * std::max(bnorm, r0);
    double r = r0;
    int it = 0;
    nyxpm_status result = NYXPM_OK;
    if (r0 > target) {
        for (it = 1; it <= c.p.max_vcycles; ++it) {
            if ((st = vcycle(cx, A)) != NYXPM_OK) return st;
            if ((st = comp_resid(c, A, 1)) != NYXPM_OK) return st;
            cudaMemcpyAsync(A.h_norms + 1, A.norms + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            c.stream);
            if (cudaStreamSynchronize(c.stream) != cudaSuccess) return check_launch(c, "multilevel solve sync");
            r = read_bits(A.h_norms, 1);
            if (r != r) {
                c.err = "multilevel residual is NaN";
                return NYXPM_NOT_CONVERGED;
            }
            if (r <= target) break;
        }
        if (it > c.p.max_vcycles) {
            it = c.p.max_vcycles;
            result = NYXPM_NOT_CONVERGED;
            c.err = "multilevel solve reached max_vcycles above tolerance";
        }
    }
    if (info) {
        info->vcycles = it;
        info->inner_vcycles = 0;
        info->resnorm0 = r0;
        info->resnorm = r;
        info->bnorm = bnorm;
    }
    return result;
}

nyxpm_status grav(Ctx& c, nyxpm_amr& A)
{
    const long long n3 = (long long)A.n0 * A.n0 * A.n0;
    const Geo g = geo3(A.n0, A.n0, A.n0);
    prof_begin(c);
    k_amr_grav0<<<g.grid, g.block, 0, c.stream>>>(A.n0, A.dxi[0], A.phi, A.g[0], A.g[1], A.g[2]);
    prof_end(c, NYXPM_ST_KICK, 32.0 * n3);
    if (A.fine_cells.count) {
        prof_begin(c);
        k_amr_gravf<<<nblk(A.fine_cells.count), kT, 0, c.stream>>>(A.fine_cells.count, A.d_cells, A.d_boxes,
                                                                    A.d_level + 12, A.phi, A.g[0], A.g[1], A.g[2]);
        prof_end(c, NYXPM_ST_KICK, 56.0 * A.fine_cells.count);
    }
    for (const Range* r : {&A.all_ghost1, &A.all_ghost23}) {
        if (r->count == 0) continue;
        prof_begin(c);
        k_amr_ghost3<<<nblk(r->count), kT, 0, c.stream>>>(r->count, A.d_ghost + r->first, A.d_ent, A.g[0], A.g[1],
                                                          A.g[2]);
        prof_end(c, NYXPM_ST_KICK, 64.0 * r->count);
    }
    return check_launch(c, "multilevel gravity");
}

nyxpm_status move(Ctx& c, nyxpm_amr& A, double dt, double a_prev, double a_cur, int do_move)
{
    prof_begin(c);
    k_amr_move<<<nblk(A.np), kT, 0, c.stream>>>(A.tab, A.np, A.x, A.y, A.z, A.vx, A.vy, A.vz, A.lev, A.box, A.g[0],
                                                A.g[1], A.g[2], dt, a_prev, a_cur, do_move, A.norms + 2);
    prof_end(c, NYXPM_ST_KICK, 120.0 * A.np);
    return check_launch(c, "multilevel kick");
}

nyxpm_status assign(Ctx& c, nyxpm_amr& A)
{
    prof_begin(c);
    k_amr_assign<<<nblk(A.np), kT, 0, c.stream>>>(A.tab, A.np, A.x, A.y, A.z, A.lev, A.box);
    prof_end(c, NYXPM_ST_KEYS, 32.0 * A.np);
    return check_launch(c, "particle levels");
}

nyxpm_status move_errors(nyxpm_ctx* c, nyxpm_amr& A)
{
    cudaMemcpyAsync(A.h_norms + 2, A.norms + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return check_launch(*c, "multilevel kick sync");
    if (A.h_norms[2] != 0) {
        c->err = "a particle's stencil left its box's ghost cells (more than 2 cells of motion in one step)";
        cudaMemsetAsync(A.norms + 2, 0, sizeof(unsigned long long), c->stream);
        return NYXPM_INVALID_ARG;
    }
    return NYXPM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define AMR_CHECK(ctx, amr)                                                                  \
    do {                                                                                     \
        if (!(ctx)) return NYXPM_INVALID_ARG;                                                \
        if (!(amr)) return afail(ctx, NYXPM_INVALID_ARG, "null hierarchy");                  \
    } while (0)
#define ATRY(expr)                                                                           \
    do {                                                                                     \
        nyxpm_status st_ = (expr);                                                           \
        if (st_ != NYXPM_OK) return st_;                                                     \
    } while (0)

extern "C" {

nyxpm_status nyxpm_amr_create(nyxpm_ctx* c, int n0, double L, int nlev, const int* nbox, const int* boxes,
                              int64_t np, nyxpm_amr** out)
{
    if (!c) return NYXPM_INVALID_ARG;
    if (!out) return afail(c, NYXPM_INVALID_ARG, "null output");
    *out = nullptr;
    if (nlev < 1 || nlev > kMaxLevels) return afail(c, NYXPM_INVALID_ARG, "nlev must be in [1, 4]");
    if (nlev > 1 && (!nbox || !boxes)) return afail(c, NYXPM_INVALID_ARG, "null boxes");
    if (np < 1 || np > (int64_t)0x7fffffff) return afail(c, NYXPM_INVALID_ARG, "np out of range");
    if (!(L > 0)) return afail(c, NYXPM_INVALID_ARG, "L must be positive");
    if (n0 < 2 || ((long long)n0 << (nlev - 1)) > (1LL << 20))
        return afail(c, NYXPM_INVALID_ARG, "n0 out of range");
    nyxpm_amr* a = new (std::nothrow) nyxpm_amr();
    if (!a) return NYXPM_OOM;
    auto cleanup = [&](nyxpm_status st) {
        for (void* q : a->allocs) cudaFree(q);
        if (a->h_norms) cudaFreeHost(a->h_norms);
        if (a->mg) nyxpm_box_destroy(c, a->mg);
        delete a;
        return st;
    };
    a->n0 = n0;
    a->L = L;
    a->nlev = nlev;
    a->np = np;
    // boxes: validated, laid out after level 0
    long long off = (long long)n0 * n0 * n0;
    int q = 0;
    a->tab.nlev = nlev;
    a->tab.n0 = n0;
    for (int l = 1; l < nlev; ++l) {
        const int n = n0 << l;
        if (nbox[l - 1] < 1) return cleanup(afail(c, NYXPM_INVALID_ARG, "a level without boxes"));
        a->tab.first[l] = (int)a->boxes.size();
        a->tab.count[l] = nbox[l - 1];
        for (int b = 0; b < nbox[l - 1]; ++b, ++q) {
            ABox B{};
            B.lev = l;
            for (int d = 0; d < 3; ++d) {
                B.lo[d] = boxes[6 * q + d];
                B.hi[d] = boxes[6 * q + 3 + d];
                if (B.lo[d] < 0 || B.hi[d] >= n || B.lo[d] > B.hi[d] || (B.lo[d] & 1) || !(B.hi[d] & 1))
                    return cleanup(afail(c, NYXPM_INVALID_ARG,
                                         "box outside its level, empty, or not aligned to the refinement ratio"));
                B.d[d] = B.hi[d] - B.lo[d] + 1 + 2 * kGW;
            }
            if ((long long)B.d[0] * B.d[1] * B.d[2] >= (1LL << 31))
                return cleanup(afail(c, NYXPM_INVALID_ARG, "a box of 2^31 cells or more"));
            for (int o = a->tab.first[l]; o < (int)a->boxes.size(); ++o) {
                const ABox& O = a->boxes[o];
                bool sep = false;
                for (int d = 0; d < 3; ++d) sep = sep || B.hi[d] < O.lo[d] || O.hi[d] < B.lo[d];
                if (!sep) return cleanup(afail(c, NYXPM_INVALID_ARG, "boxes of one level overlap"));
            }
            B.off = off;
            off += (long long)B.d[0] * B.d[1] * B.d[2];
            a->boxes.push_back(B);
        }
    }
    a->ntot = off;
    {
        Builder Bd(*a);
        for (const ABox& B : a->boxes) {
            if (B.lev < 2) continue;
            for (int K = B.lo[2] / 2 - 1; K <= B.hi[2] / 2 + 1; ++K)
                for (int J = B.lo[1] / 2 - 1; J <= B.hi[1] / 2 + 1; ++J)
                    for (int I = B.lo[0] / 2 - 1; I <= B.hi[0] / 2 + 1; ++I)
                        if (Bd.vidx(B.lev - 1, I, J, K) < 0)
                            return cleanup(afail(c, NYXPM_INVALID_ARG,
                                                 "a box is not nested in the coarser level with one cell to spare"));
        }
    }
    for (ABox& B : a->boxes) {
        B.pbox = -1;
        if (B.lev < 2) continue;
        B.pbox = -2;
        for (int o = a->tab.first[B.lev - 1]; o < a->tab.first[B.lev - 1] + a->tab.count[B.lev - 1]; ++o) {
            const ABox& P = a->boxes[o];
            if (box_has(P, B.lo[0] / 2, B.lo[1] / 2, B.lo[2] / 2) && box_has(P, B.hi[0] / 2, B.hi[1] / 2, B.hi[2] / 2))
                B.pbox = o;
        }
    }
    for (int l = 1; l < nlev; ++l) {
        a->prolong_black_ok[l] = 1;
        for (int b = a->tab.first[l]; b < a->tab.first[l] + a->tab.count[l]; ++b)
            if (a->boxes[b].pbox == -2) a->prolong_black_ok[l] = 0;
    }
    for (int l = 0; l < nlev; ++l) {
        const double h = L / (n0 << l);
        a->scale[l] = (h * h) * kSixth;
        a->inv_scale[l] = 1.0 / a->scale[l];
        a->hcube[l] = (h * h) * h;
        a->dxi[l] = (double)(n0 << l) / L;
        a->tab.dxi[l] = a->dxi[l];
    }
    cudaSetDevice(c->p.device);
    {
        // level 0's multigrid hierarchy (validates n0)
        const nyxpm_status st = nyxpm_box_create(c, n0, L, 1, NYXPM_FP64, &a->mg);
        if (st != NYXPM_OK) {
            a->mg = nullptr;
            return cleanup(st);
        }
    }
    nyxpm_status st;
#define AALLOC(p, cnt)                                                                       \
    if ((st = aalloc(c, a, &(p), (cnt))) != NYXPM_OK) return cleanup(st)
    AALLOC(a->d_boxes, a->boxes.size());
    if (!a->boxes.empty())
        cudaMemcpyAsync(a->d_boxes, a->boxes.data(), sizeof(ABox) * a->boxes.size(), cudaMemcpyHostToDevice,
                        c->stream);
    a->tab.box = a->d_boxes;
    AALLOC(a->d_level, 32);
    std::vector<double> lv(32, 0.0);
    for (int l = 0; l < nlev; ++l) {
        lv[4 + l] = a->hcube[l];
        lv[8 + l] = a->inv_scale[l];
        lv[12 + l] = a->dxi[l];
    }
    cudaMemcpyAsync(a->d_level, lv.data(), sizeof(double) * 32, cudaMemcpyHostToDevice, c->stream);
    if ((st = build_lists(c, a)) != NYXPM_OK) return cleanup(st);
    for (double** f : {&a->mass, &a->rho, &a->beta, &a->phi, &a->R, &a->e, &a->T, &a->g[0], &a->g[1], &a->g[2]}) {
        AALLOC(*f, (size_t)a->ntot);
        cudaMemsetAsync(*f, 0, sizeof(double) * a->ntot, c->stream);
    }
    for (double** f : {&a->x, &a->y, &a->z, &a->vx, &a->vy, &a->vz, &a->m}) AALLOC(*f, (size_t)np);
    AALLOC(a->lev, (size_t)np);
    AALLOC(a->box, (size_t)np);
    AALLOC(a->staging, (size_t)6 * np);
    AALLOC(a->norms, 4);
    cudaMemsetAsync(a->norms, 0, 4 * sizeof(unsigned long long), c->stream);
#undef AALLOC
    if (cudaMallocHost(&a->h_norms, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        a->h_norms = nullptr;
        return cleanup(afail(c, NYXPM_OOM, "pinned norms"));
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return cleanup(check_launch(*c, "hierarchy create"));
    *out = a;
    return NYXPM_OK;
}

nyxpm_status nyxpm_amr_destroy(nyxpm_ctx* c, nyxpm_amr* a)
{
    if (!c) return NYXPM_INVALID_ARG;
    if (!a) return NYXPM_OK;
    cudaStreamSynchronize(c->stream);
    for (void* q : a->allocs) cudaFree(q);
    if (a->h_norms) cudaFreeHost(a->h_norms);
    if (a->mg) nyxpm_box_destroy(c, a->mg);
    delete a;
    return NYXPM_OK;
}

nyxpm_status nyxpm_amr_upload(nyxpm_ctx* c, nyxpm_amr* a, const double* pos, const double* vel,
                              const double* mass, double mass_scalar)
{
    AMR_CHECK(c, a);
    if (!pos || !vel) return afail(c, NYXPM_INVALID_ARG, "null pos/vel");
    double total = 0.0;
    for (int64_t p = 0; p < a->np; ++p) {
        for (int d = 0; d < 3; ++d)
            if (!std::isfinite(pos[3 * p + d]) || !std::isfinite(vel[3 * p + d]))
                return afail(c, NYXPM_INVALID_ARG, "non-finite particle position or velocity");
        if (mass) {
            if (!(mass[p] >= 0) || !std::isfinite(mass[p])) return afail(c, NYXPM_INVALID_ARG, "bad mass");
            total = total + mass[p];
        }
    }
    if (!mass) {
        if (!(mass_scalar >= 0) || !std::isfinite(mass_scalar)) return afail(c, NYXPM_INVALID_ARG, "bad mass");
        total = mass_scalar * (double)a->np;
    }
    a->uniform_mass = mass ? 0 : 1;
    a->mscalar = mass ? 0.0 : mass_scalar;
    a->mass_offset = total / (a->L * a->L * a->L);
    cudaMemcpyAsync(a->staging, pos, sizeof(double) * 3 * a->np, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(a->staging + 3 * a->np, vel, sizeof(double) * 3 * a->np, cudaMemcpyHostToDevice, c->stream);
    if (mass) cudaMemcpyAsync(a->m, mass, sizeof(double) * a->np, cudaMemcpyHostToDevice, c->stream);
    prof_begin(*c);
    k_amr_unpack<<<nblk(a->np), kT, 0, c->stream>>>(a->np, a->staging, a->staging + 3 * a->np, a->x, a->y, a->z,
                                                     a->vx, a->vy, a->vz);
    prof_end(*c, NYXPM_ST_GATHER, 96.0 * a->np);
    prof_begin(*c);
    k_amr_wrap<<<nblk(a->np), kT, 0, c->stream>>>(a->np, a->L, a->x, a->y, a->z);
    prof_end(*c, NYXPM_ST_KICK, 48.0 * a->np);
    ATRY(check_launch(*c, "hierarchy upload"));
    ATRY(nyxpm_synchronize(c));
    a->uploaded = 1;
    return NYXPM_OK;
}

nyxpm_status nyxpm_amr_download(nyxpm_ctx* c, nyxpm_amr* a, double* pos, double* vel)
{
    AMR_CHECK(c, a);
    if (!pos || !vel) return afail(c, NYXPM_INVALID_ARG, "null pos/vel");
    prof_begin(*c);
    k_amr_pack<<<nblk(a->np), kT, 0, c->stream>>>(a->np, a->x, a->y, a->z, a->vx, a->vy, a->vz, a->staging,
                                                   a->staging + 3 * a->np);
    prof_end(*c, NYXPM_ST_GATHER, 96.0 * a->np);
    ATRY(check_launch(*c, "hierarchy download"));
    cudaMemcpyAsync(pos, a->staging, sizeof(double) * 3 * a->np, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(vel, a->staging + 3 * a->np, sizeof(double) * 3 * a->np, cudaMemcpyDeviceToHost, c->stream);
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_amr_assign(nyxpm_ctx* c, nyxpm_amr* a, int* lev, int* box)
{
    AMR_CHECK(c, a);
    if (!a->uploaded) return afail(c, NYXPM_INVALID_ARG, "no particles uploaded");
    ATRY(assign(*c, *a));
    if (lev) cudaMemcpyAsync(lev, a->lev, sizeof(int) * a->np, cudaMemcpyDeviceToHost, c->stream);
    if (box) cudaMemcpyAsync(box, a->box, sizeof(int) * a->np, cudaMemcpyDeviceToHost, c->stream);
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_amr_deposit(nyxpm_ctx* c, nyxpm_amr* a)
{
    AMR_CHECK(c, a);
    if (!a->uploaded) return afail(c, NYXPM_INVALID_ARG, "no particles uploaded");
    ATRY(deposit(*c, *a));
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_amr_solve(nyxpm_ctx* c, nyxpm_amr* a, double comoving_a, nyxpm_solve_info* info)
{
    AMR_CHECK(c, a);
    if (!(comoving_a > 0)) return afail(c, NYXPM_INVALID_ARG, "a must be positive");
    return solve(c, *a, comoving_a, info);
}

nyxpm_status nyxpm_amr_grav_vector(nyxpm_ctx* c, nyxpm_amr* a)
{
    AMR_CHECK(c, a);
    ATRY(grav(*c, *a));
    return nyxpm_synchronize(c);
}

nyxpm_status nyxpm_amr_kick(nyxpm_ctx* c, nyxpm_amr* a, double dt, double a_prev, double a_cur, int do_move)
{
    AMR_CHECK(c, a);
    if (!a->uploaded) return afail(c, NYXPM_INVALID_ARG, "no particles uploaded");
    if (!(a_cur > 0)) return afail(c, NYXPM_INVALID_ARG, "a must be positive");
    ATRY(move(*c, *a, dt, a_prev, a_cur, do_move ? 1 : 0));
    return move_errors(c, *a);
}

nyxpm_status nyxpm_amr_step(nyxpm_ctx* c, nyxpm_amr* a, double a_old, double a_new, double dt,
                            nyxpm_step_info* info)
{
    AMR_CHECK(c, a);
    if (!a->uploaded) return afail(c, NYXPM_INVALID_ARG, "no particles uploaded");
    if (!(a_old > 0) || !(a_new > 0)) return afail(c, NYXPM_INVALID_ARG, "a must be positive");
    const double a_half = 0.5 * (a_old + a_new);
    nyxpm_solve_info s0{}, s1{};
    ATRY(assign(*c, *a));
    ATRY(deposit(*c, *a));
    nyxpm_status st = solve(c, *a, a_old, &s0);
    if (st != NYXPM_OK && st != NYXPM_NOT_CONVERGED) return st;
    ATRY(grav(*c, *a));
    ATRY(move(*c, *a, dt, a_old, a_half, 1));
    ATRY(deposit(*c, *a));
    nyxpm_status st2 = solve(c, *a, a_new, &s1);
    if (st2 != NYXPM_OK && st2 != NYXPM_NOT_CONVERGED) return st2;
    ATRY(grav(*c, *a));
    ATRY(move(*c, *a, dt, a_half, a_new, 0));
    prof_begin(*c);
    k_amr_wrap<<<nblk(a->np), kT, 0, c->stream>>>(a->np, a->L, a->x, a->y, a->z);
    prof_end(*c, NYXPM_ST_KICK, 48.0 * a->np);
    ATRY(check_launch(*c, "multilevel wrap"));
    ATRY(move_errors(c, *a));
    if (info) {
        info->old_solve = s0;
        info->new_solve = s1;
    }
    return st != NYXPM_OK ? st : st2;
}

nyxpm_status nyxpm_amr_field(nyxpm_ctx* c, nyxpm_amr* a, int which, int box, double* out)
{
    AMR_CHECK(c, a);
    if (!out) return afail(c, NYXPM_INVALID_ARG, "null output");
    double* f[6] = {a->rho, a->phi, a->g[0], a->g[1], a->g[2], a->mass};
    if (which < 0 || which > 5) return afail(c, NYXPM_INVALID_ARG, "bad field");
    if (box < -1 || box >= (int)a->boxes.size()) return afail(c, NYXPM_INVALID_ARG, "bad box");
    if (box < 0) {
        cudaMemcpyAsync(out, f[which], sizeof(double) * a->n0 * a->n0 * a->n0, cudaMemcpyDeviceToHost, c->stream);
        return nyxpm_synchronize(c);
    }
    const ABox& B = a->boxes[box];
    const long long cnt = (long long)(B.hi[0] - B.lo[0] + 1) * (B.hi[1] - B.lo[1] + 1) * (B.hi[2] - B.lo[2] + 1);
    prof_begin(*c);
    k_amr_box_out<<<nblk(cnt), kT, 0, c->stream>>>(B, f[which], a->T);
    prof_end(*c, NYXPM_ST_GATHER, 16.0 * cnt);
    ATRY(check_launch(*c, "box field"));
    cudaMemcpyAsync(out, a->T, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream);
    return nyxpm_synchronize(c);
}

int64_t nyxpm_amr_cells(const nyxpm_amr* a, int box)
{
    if (!a) return -1;
    if (box < 0) return (int64_t)a->n0 * a->n0 * a->n0;
    if (box >= (int)a->boxes.size()) return -1;
    const ABox& B = a->boxes[box];
    return (int64_t)(B.hi[0] - B.lo[0] + 1) * (B.hi[1] - B.lo[1] + 1) * (B.hi[2] - B.lo[2] + 1);
}

}  // extern "C"
