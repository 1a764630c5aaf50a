// Comoving Poisson solve of the FP64 PM step: RHS assembly with the mean
// density removed (Gravity::solve_for_phi + CorrectRhsUsingOffset,
// Source/Gravity/Gravity.cpp:267-315, 1207-1244) and a geometric multigrid
// V-cycle with red-black Gauss-Seidel smoothing on the red-black split layout,
// the GB300-native replacement of the AMReX MLMG solve that
// Gravity::solve_with_MLMG (Gravity.cpp:1318-1416) calls.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so these kernels
// are written for the fewest FP64 instructions: the right-hand side is kept in
// smoother units (beta = h^2 rhs / 6, one fused multiply-add per Gauss-Seidel
// update), the trilinear prolongation weights are exact constants, and index
// arithmetic uses 3-D launch geometry instead of integer division.  Built with
// --fmad=false: only the explicit fma() calls fuse, in the same places the CPU
// oracle fuses, so both round identically.
#include "pm_common.cuh"
#include "pm_tail.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace nyxpm {

namespace {

constexpr int kThreads = 256;
constexpr double kSixth = 1.0 / 6.0;

__constant__ double kProlongW[8] = {0.421875, 0.140625, 0.140625, 0.046875,
                                    0.140625, 0.046875, 0.046875, 0.015625};

inline unsigned blocks_for(long long n, int t = kThreads)
{
    long long b = (n + t - 1) / t;
    return (unsigned)(b < 1 ? 1 : b);
}

__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ---------------------------------------------------------------------------
// RHS: canonical sum of (rho - mass_offset), then
// beta = ((((rho - mass_offset) - mean) * ggrav) * (1/a)) * (h^2/6)
// ---------------------------------------------------------------------------
// one warp per row: 32 strided lane partials, then a halving tree
__global__ void k_rowsum(int n, const double* __restrict__ rho, double mo, double* rows)
{
    const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= (long long)n * n) return;
    const double* r = rho + row * n;
    double s = 0.0;
    for (int i = lane; i < n; i += 32) s = s + (r[i] - mo);
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const double t = __shfl_down_sync(0xffffffffu, s, off);
        if (lane < off) s = s + t;
    }
    if (lane == 0) rows[row] = s;
}

__global__ void k_planesum(int n, const double* __restrict__ rows, double* planes)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double s = 0.0;
    for (int j = 0; j < n; ++j) s = s + rows[(long long)k * n + j];
    planes[k] = s;
}

__global__ void k_mean(int n, double dx, double L, const double* __restrict__ planes, double* scal)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int k = 0; k < n; ++k) s = s + planes[k];
    scal[0] = (s * (dx * dx * dx)) / (L * L * L);
}

__global__ void k_make_beta(int n, int split, const double* __restrict__ rho, double mo,
                            const double* __restrict__ scal, double ggrav, double ainv, double k0,
                            double* beta_r, double* beta_b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    const double mean = scal[0];
    const double v = rho[cidx(i, j, k, n)];
    *lv_ptr<double>(beta_r, beta_b, n, split, i, j, k) = ((((v - mo) - mean) * ggrav) * ainv) * k0;
}

// ---------------------------------------------------------------------------
// norms (max is order independent; non-negative doubles compare as their bits)
// ---------------------------------------------------------------------------
__global__ void k_absmax(long long cnt, const double* __restrict__ a, unsigned long long* out)
{
    unsigned long long v = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < cnt;
         t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long u = absbits(a[t]);
        v = u > v ? u : v;
    }
    block_umax_store(v, out);
}

// neighbour sum in the oracle's order: x-, x+, y-, y+, z-, z+
__device__ __forceinline__ double nbr_sum(const LevelView& L, int i, int j, int k)
{
    const int n = L.n;
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    double s = *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, im, j, k) +
               *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, ip, j, k);
    s = s + *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, i, jm, k);
    s = s + *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, i, jp, k);
    s = s + *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, i, j, km);
    s = s + *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, i, j, kp);
    return s;
}

// residual in smoother units: beta - (s/6 - phi)
__device__ __forceinline__ double resid_at(const LevelView& L, int i, int j, int k)
{
    const double s = nbr_sum(L, i, j, k);
    const double c = *lv_ptr<double>(L.phi_r, L.phi_b, L.n, L.split, i, j, k);
    const double b = *lv_ptr<double>(L.beta_r, L.beta_b, L.n, L.split, i, j, k);
    return b - fma(s, kSixth, -c);
}

// ||r_beta||_inf of a split level: one thread per (ih, j, k), both cells of the pair
__global__ void k_resnorm_split(LevelView L, unsigned long long* out)
{
    const int half = L.n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (ih < half && j < L.n) {
        const unsigned long long a = absbits(resid_at(L, 2 * ih, j, k));
        const unsigned long long b = absbits(resid_at(L, 2 * ih + 1, j, k));
        v = a > b ? a : b;
    }
    block_umax_store(v, out);
}

// the same over the red cells only: one thread per red cell of the split level
__global__ void k_resnorm_red(int n, const double* __restrict__ phi_r, const double* __restrict__ phi_b,
                              const double* __restrict__ beta_r, unsigned long long* out)
{
    const int half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (ih < half && j < n) {
        const int q = (j + k) & 1;  // the red cell of this pair is i = 2*ih + q
        const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
        const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        const long long row = (long long)j + (long long)n * k;
        const long long t = row * half + ih;
        double s = phi_b[row * half + ihm] + phi_b[row * half + ihp];
        s = s + phi_b[((long long)jm + (long long)n * k) * half + ih];
        s = s + phi_b[((long long)jp + (long long)n * k) * half + ih];
        s = s + phi_b[((long long)j + (long long)n * km) * half + ih];
        s = s + phi_b[((long long)j + (long long)n * kp) * half + ih];
        v = absbits(beta_r[t] - fma(s, kSixth, -phi_r[t]));
    }
    block_umax_store(v, out);
}

// k_resnorm_red fused with the red half sweep that opens the next V-cycle: both
// need the same neighbour sum s of each red cell, so one pass gives the norm of
// beta - (s/6 - phi_red) and the next red value fma(s, 1/6, -beta), written to a
// spare red array (adopted only if the solve goes on) -- the same bits as the
// norm pass followed by the sweep
__global__ void k_resnorm_red_sweep(int n, const double* __restrict__ phi_r,
                                    const double* __restrict__ phi_b,
                                    const double* __restrict__ beta_r, double* __restrict__ next_r,
                                    unsigned long long* out)
{
    pdl_wait();
    pdl_trigger();
    const int half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (ih < half && j < n) {
        const int q = (j + k) & 1;
        const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
        const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        const long long row = (long long)j + (long long)n * k;
        const long long t = row * half + ih;
        double s = phi_b[row * half + ihm] + phi_b[row * half + ihp];
        s = s + phi_b[((long long)jm + (long long)n * k) * half + ih];
        s = s + phi_b[((long long)jp + (long long)n * k) * half + ih];
        s = s + phi_b[((long long)j + (long long)n * km) * half + ih];
        s = s + phi_b[((long long)j + (long long)n * kp) * half + ih];
        const double b = beta_r[t];
        v = absbits(b - fma(s, kSixth, -phi_r[t]));
        next_r[t] = fma(s, kSixth, -b);
    }
    block_umax_store(v, out);
}

__global__ void k_resnorm_nat(LevelView L, unsigned long long* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (i < L.n && j < L.n) v = absbits(resid_at(L, i, j, k));
    block_umax_store(v, out);
}

// ---------------------------------------------------------------------------
// red-black Gauss-Seidel half sweep on a split level: one thread per cell of
// the colour being updated; reads the other colour's array, writes this one.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gsrb(int n, int color, double* __restrict__ mine,
                                              const double* __restrict__ other,
                                              const double* __restrict__ beta)
{
    pdl_wait();
    pdl_trigger();
    const int half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (ih >= half || j >= n) return;
    const int q = (j + k + color) & 1;  // this cell is i = 2*ih + q
    const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
    const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    const long long row = (long long)j + (long long)n * k;
    const long long t = row * half + ih;
    double s = other[row * half + ihm] + other[row * half + ihp];
    s = s + other[((long long)jm + (long long)n * k) * half + ih];
    s = s + other[((long long)jp + (long long)n * k) * half + ih];
    s = s + other[((long long)j + (long long)n * km) * half + ih];
    s = s + other[((long long)j + (long long)n * kp) * half + ih];
    mine[t] = fma(s, kSixth, -beta[t]);
}

// coarse beta = 1/2 of the 8 fine residuals (summed dk, dj, di); coarse phi = 0
// RED = 1 after pre-smoothing (the last half sweep was black): the black
// children's residuals are round-off by construction and count as 0, so the 4 red
// children (di + dj + dk even) are summed in the same (dk, dj, di) order -- half
// the FP64 residual work
template <int RED>
__global__ void k_restrict(LevelView F, LevelView Cv)
{
    pdl_wait();
    pdl_trigger();
    const int nc = Cv.n;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= nc || J >= nc) return;
    double s = 0.0;
#pragma unroll
    for (int dk = 0; dk < 2; ++dk)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
            for (int di = 0; di < 2; ++di)
                if (!RED || ((di + dj + dk) & 1) == 0)
                    s = s + resid_at(F, 2 * I + di, 2 * J + dj, 2 * K + dk);
    *lv_ptr<double>(Cv.beta_r, Cv.beta_b, nc, Cv.split, I, J, K) = s * 0.5;
    *lv_ptr<double>(Cv.phi_r, Cv.phi_b, nc, Cv.split, I, J, K) = 0.0;
}

// k_prolong for a split fine level over a split coarse level with
// half % 4 == 0: four compact columns (eight fine cells) per thread.  The six
// coarse x-neighbours ih0-1 .. ih0+4 of each (J', K') row are a pair plus one
// in each colour array.  Same weighted sums in the same order.
// BLACK = 1 when post-smoothing follows (nu2 > 0): its first half sweep
// overwrites every red cell without reading it, so only the black fine cells take
// the correction -- the same bits as correcting all cells, for half the FP64 work
template <int BLACK>
__global__ void k_prolong4(LevelView Cv, LevelView F)
{
    pdl_wait();
    pdl_trigger();
    const int n = F.n, nc = Cv.n;
    const unsigned half = (unsigned)n >> 1, chalf = (unsigned)nc >> 1, h4 = half >> 2;
    const unsigned t4 = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (t4 >= h4 || j >= n) return;
    const int J = j >> 1, K = k >> 1;
    const int Js[2] = {J, wrap1((j & 1) ? J + 1 : J - 1, nc)};
    const int Ks[2] = {K, wrap1((k & 1) ? K + 1 : K - 1, nc)};
    const unsigned c2 = 2 * t4;
    double v[2][2][6];
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const unsigned row = ((unsigned)Js[a] + (unsigned)nc * (unsigned)Ks[b]) * chalf;
            const bool even_red = ((Js[a] + Ks[b]) & 1) == 0;
            const double* ev = even_red ? Cv.phi_r : Cv.phi_b;
            const double* od = even_red ? Cv.phi_b : Cv.phi_r;
            const double2 e01 = __ldg(reinterpret_cast<const double2*>(ev + row + c2));
            const double e2 = __ldg(ev + row + (c2 + 2 == chalf ? 0u : c2 + 2));
            const double2 o01 = __ldg(reinterpret_cast<const double2*>(od + row + c2));
            const double om = __ldg(od + row + (c2 == 0 ? chalf - 1 : c2 - 1));
            v[b][a][0] = om;
            v[b][a][1] = e01.x;
            v[b][a][2] = o01.x;
            v[b][a][3] = e01.y;
            v[b][a][4] = o01.y;
            v[b][a][5] = e2;
        }
    const unsigned t = ((unsigned)j + (unsigned)n * (unsigned)k) * half + 4 * t4;
    const bool even_fine_red = ((j + k) & 1) == 0;
    double* fe = (even_fine_red ? F.phi_r : F.phi_b) + t;
    double* fo = (even_fine_red ? F.phi_b : F.phi_r) + t;
    if (!BLACK || !even_fine_red) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            double se = 0.0;
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    se = fma(kProlongW[0 + 2 * a + 4 * b], v[b][a][r + 1], se);
                    se = fma(kProlongW[1 + 2 * a + 4 * b], v[b][a][r], se);
                }
            fe[r] = fe[r] + se;
        }
    }
    if (!BLACK || even_fine_red) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            double so = 0.0;
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    so = fma(kProlongW[0 + 2 * a + 4 * b], v[b][a][r + 1], so);
                    so = fma(kProlongW[1 + 2 * a + 4 * b], v[b][a][r + 2], so);
                }
            fo[r] = fo[r] + so;
        }
    }
}

// trilinear cell-centred prolongation of the coarse correction, added to the
// fine phi; one thread per fine pair (2ih, 2ih+1) of a split level (BLACK: the
// black cell of the pair only, as in k_prolong4)
template <int BLACK>
__global__ void k_prolong(LevelView Cv, LevelView F)
{
    pdl_wait();
    pdl_trigger();
    const int n = F.n, nc = Cv.n, half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (ih >= half || j >= n) return;
    const int J = j >> 1, K = k >> 1;
    const int Js[2] = {J, wrap1((j & 1) ? J + 1 : J - 1, nc)};
    const int Ks[2] = {K, wrap1((k & 1) ? K + 1 : K - 1, nc)};
    const long long t = ((long long)j + (long long)n * k) * half + ih;
#pragma unroll
    for (int odd = 0; odd < 2; ++odd) {
        const int i = 2 * ih + odd;
        if (BLACK && ((i + j + k) & 1) == 0) continue;
        const int I = ih;
        const int Is[2] = {I, wrap1(odd ? I + 1 : I - 1, nc)};
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int tt = 0; tt < 2; ++tt)
                    s = fma(kProlongW[tt + 2 * a + 4 * b],
                            *lv_ptr<const double>(Cv.phi_r, Cv.phi_b, nc, Cv.split, Is[tt], Js[a], Ks[b]), s);
        double* p = (((i + j + k) & 1) ? F.phi_b : F.phi_r) + t;
        *p = *p + s;
    }
}

// exact coarsest solve: phi = G * beta (cyclic convolution, y in storage order), one block
__global__ void k_bottom(int nb, const double* __restrict__ G, const double* __restrict__ beta,
                         double* phi)
{
    pdl_wait();
    pdl_trigger();
    __shared__ double r[kMaxBottom * kMaxBottom * kMaxBottom];
    __shared__ double g[kMaxBottom * kMaxBottom * kMaxBottom];
    const int nc = nb * nb * nb;
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
        r[t] = beta[t];
        g[t] = G[t];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int i = c % nb, j = (c / nb) % nb, k = c / (nb * nb);
        double s = 0.0;
        int y = 0;
        for (int yk = 0; yk < nb; ++yk) {
            const int dk = wrap1(k - yk, nb) * nb * nb;
            for (int yj = 0; yj < nb; ++yj) {
                const int djk = dk + wrap1(j - yj, nb) * nb;
                for (int yi = 0; yi < nb; ++yi, ++y) s = fma(g[djk + wrap1(i - yi, nb)], r[y], s);
            }
        }
        phi[c] = s;
    }
}

// the coarse end of an FP64 V-cycle by one CTA (pm_tail.cuh): the arithmetic of
// k_gsrb, k_restrict, k_bottom and k_prolong in the same order, so the same bits
struct TailD {
    int nl;                  // levels in the tail; the last is the bottom (natural layout)
    int nu1, nu2, nb;
    const double* G;
    LevelView lv[kMaxTail];
};

__global__ void __launch_bounds__(kTailThreadsD) k_vcycle_tail_d(TailD A)
{
    pdl_wait();
    pdl_trigger();
    __shared__ double r[kMaxBottom * kMaxBottom * kMaxBottom];
    __shared__ double g[kMaxBottom * kMaxBottom * kMaxBottom];
    vcycle_tail<double>(A.lv, A.nl, A.nu1, A.nu2, A.G, A.nb, r, g, A.nu1 > 0);
}

// g_d(c) = 0.5*((phi_c - phi_{c-e_d})*dxi + (phi_{c+e_d} - phi_c)*dxi), second product fused;
// component-major output
__global__ void k_grav(LevelView L, double dxi, double* g)
{
    const int n = L.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    const long long nc = (long long)n * n * n;
    const long long c = cidx(i, j, k, n);
    auto P = [&](int a, int b, int d) {
        return *lv_ptr<const double>(L.phi_r, L.phi_b, n, L.split, a, b, d);
    };
    const double pc = P(i, j, k);
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    g[c] = 0.5 * fma(P(ip, j, k) - pc, dxi, (pc - P(im, j, k)) * dxi);
    g[nc + c] = 0.5 * fma(P(i, jp, k) - pc, dxi, (pc - P(i, jm, k)) * dxi);
    g[2 * nc + c] = 0.5 * fma(P(i, j, kp) - pc, dxi, (pc - P(i, j, km)) * dxi);
}

__global__ void k_to_natural(LevelView L, double* out)
{
    const int n = L.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    out[cidx(i, j, k, n)] = *lv_ptr<const double>(L.phi_r, L.phi_b, n, L.split, i, j, k);
}

__global__ void k_from_natural(LevelView L, const double* __restrict__ in)
{
    const int n = L.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    *lv_ptr<double>(L.phi_r, L.phi_b, n, L.split, i, j, k) = in[cidx(i, j, k, n)];
}

__global__ void k_beta_from_natural(LevelView L, const double* __restrict__ in)
{
    const int n = L.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    *lv_ptr<double>(L.beta_r, L.beta_b, n, L.split, i, j, k) = in[cidx(i, j, k, n)];
}

inline unsigned norm_blocks(Ctx& c, long long cnt)
{
    long long b = (cnt + kThreads - 1) / kThreads;
    long long cap = (long long)c.sm_count * 8;
    return (unsigned)std::max<long long>(1, std::min(b, cap));
}

nyxpm_status gsrb_sweep(Ctx& c, const Level& l, int fine, int black_only = 0)
{
    const long long half_cells = (long long)l.n * l.n * l.n / 2;
    const Geo g = geo3(l.n / 2, l.n, l.n);
    for (int color = black_only ? 1 : 0; color < 2; ++color) {
        double* mine = color ? l.phi_b : l.phi_r;
        const double* other = color ? l.phi_r : l.phi_b;
        const double* beta = color ? l.beta_b : l.beta_r;
        prof_begin(c);
        launch_pdl(c, k_gsrb, dim3(g.grid), dim3(g.block), l.n, color, mine, other, beta);
        prof_end(c, NYXPM_ST_SMOOTH, 24.0 * half_cells, fine);
    }
    return check_launch(c, "gsrb");
}

// One SM issues FP64 at 1/64 of its FP32 rate, so the FP64 form fuses only the
// levels of at most half the FP32 edge (8^3 cells at the default 16): there a
// level's half sweep is a few hundred cells, cheaper on one SM than a launch.
bool tail_fits_d(const Ctx& c, const Box& b, size_t li)
{
    const int edge = c.p.mg_fused_edge / 2;
    return li > 0 && edge > 0 && b.levels[li].n <= edge && b.levels.size() - li >= 2 &&
           b.levels.size() - li <= (size_t)kMaxTail;
}

nyxpm_status vcycle_tail_d(Ctx& c, Box& b, size_t li)
{
    TailD A;
    A.nl = (int)(b.levels.size() - li);
    A.nu1 = c.p.nu1;
    A.nu2 = c.p.nu2;
    A.nb = b.nb;
    A.G = b.G;
    double bytes = 0;
    for (int l = 0; l < A.nl; ++l) {
        const Level& lv = b.levels[li + l];
        A.lv[l] = view(lv);
        const double cells = (double)lv.n * lv.n * lv.n;
        bytes += (l + 1 < A.nl) ? 12.0 * cells * 2 * (c.p.nu1 + c.p.nu2) + 32.0 * cells : 16.0 * cells;
    }
    prof_begin(c);
    launch_pdl(c, k_vcycle_tail_d, dim3(1), dim3(kTailThreadsD), A);
    prof_end(c, NYXPM_ST_SMOOTH, bytes);
    return check_launch(c, "fused coarse V-cycle");
}

// red_done: the opening red half sweep of this level was already made (by
// k_resnorm_red_sweep)
nyxpm_status vcycle(Ctx& c, Box& b, size_t li, int red_done = 0)
{
    nyxpm_status st;
    const Level& f = b.levels[li];
    if (tail_fits_d(c, b, li)) return vcycle_tail_d(c, b, li);
    if (li + 1 == b.levels.size()) {
        prof_begin(c);
        launch_pdl(c, k_bottom, dim3(1), dim3(512), b.nb, b.G, f.beta_r, f.phi_r);
        prof_end(c, NYXPM_ST_BOTTOM, 16.0 * f.n * f.n * f.n);
        return check_launch(c, "bottom");
    }
    const int nu1 = c.p.nu1, nu2 = c.p.nu2;
    for (int s = 0; s < nu1; ++s)
        if ((st = gsrb_sweep(c, f, li == 0, s == 0 && red_done)) != NYXPM_OK) return st;
    const Level& cl = b.levels[li + 1];
    const long long ncc = (long long)cl.n * cl.n * cl.n;
    const long long ncf = (long long)f.n * f.n * f.n;
    const bool quads = f.split && (f.n / 2) % 4 == 0;
    {
        const Geo g = geo3(cl.n, cl.n, cl.n);
        prof_begin(c);
        if (c.p.nu1 > 0)
            launch_pdl(c, k_restrict<1>, dim3(g.grid), dim3(g.block), view(f), view(cl));
        else
            launch_pdl(c, k_restrict<0>, dim3(g.grid), dim3(g.block), view(f), view(cl));
        prof_end(c, NYXPM_ST_RESTRICT, 16.0 * ncf + 16.0 * ncc);
    }
    if ((st = check_launch(c, "restrict")) != NYXPM_OK) return st;
    if ((st = vcycle(c, b, li + 1)) != NYXPM_OK) return st;
    {
        prof_begin(c);
        const bool black = nu2 > 0;
        if (quads && cl.split) {
            const Geo g = geo3(f.n / 8, f.n, f.n);
            if (black) launch_pdl(c, k_prolong4<1>, dim3(g.grid), dim3(g.block), view(cl), view(f));
            else launch_pdl(c, k_prolong4<0>, dim3(g.grid), dim3(g.block), view(cl), view(f));
        } else {
            const Geo g = geo3(f.n / 2, f.n, f.n);
            if (black) launch_pdl(c, k_prolong<1>, dim3(g.grid), dim3(g.block), view(cl), view(f));
            else launch_pdl(c, k_prolong<0>, dim3(g.grid), dim3(g.block), view(cl), view(f));
        }
        prof_end(c, NYXPM_ST_PROLONG, 16.0 * ncf + 8.0 * ncc);
    }
    if ((st = check_launch(c, "prolong")) != NYXPM_OK) return st;
    for (int s = 0; s < nu2; ++s)
        if ((st = gsrb_sweep(c, f, li == 0)) != NYXPM_OK) return st;
    return NYXPM_OK;
}

// launch ||r_beta||_inf of level 0 into norms[slot]: all cells, or the red
// cells only after a cycle that ended with a black half sweep
nyxpm_status launch_resnorm(Ctx& c, Box& b, int slot, int red_only)
{
    const Level& l = b.levels[0];
    const long long nc = (long long)l.n * l.n * l.n;
    prof_begin(c);
    cudaMemsetAsync(b.norms + slot, 0, sizeof(unsigned long long), c.stream);
    if (l.split && red_only) {
        const Geo g = geo3(l.n / 2, l.n, l.n);
        k_resnorm_red<<<g.grid, g.block, 0, c.stream>>>(l.n, l.phi_r, l.phi_b, l.beta_r, b.norms + slot);
    } else if (l.split) {
        const Geo g = geo3(l.n / 2, l.n, l.n);
        k_resnorm_split<<<g.grid, g.block, 0, c.stream>>>(view(l), b.norms + slot);
    } else {
        const Geo g = geo3(l.n, l.n, l.n);
        k_resnorm_nat<<<g.grid, g.block, 0, c.stream>>>(view(l), b.norms + slot);
    }
    prof_end(c, NYXPM_ST_NORM, (red_only ? 12.0 : 16.0) * nc);
    return check_launch(c, "resnorm");
}

double read_norm(Box& b, int slot)
{
    double v;
    std::memcpy(&v, &b.h_norms[slot], sizeof(v));
    return v;
}

}  // namespace

double beta_scale(const Box& b)
{
    const double h = b.L / b.n;
    return (h * h) * kSixth;
}

nyxpm_status launch_make_rhs(Ctx& c, Box& b, double a)
{
    const int n = b.n;
    const long long nc = (long long)n * n * n;
    const Level& l0 = b.levels[0];
    const double dx = b.L / n;
    const Geo g = geo3(n, n, n);
    prof_begin(c);
    k_rowsum<<<blocks_for((long long)n * n * 32), kThreads, 0, c.stream>>>(n, b.rho, b.mass_offset,
                                                                          b.rows);
    k_planesum<<<blocks_for(n, 128), 128, 0, c.stream>>>(n, b.rows, b.planes);
    k_mean<<<1, 32, 0, c.stream>>>(n, dx, b.L, b.planes, b.scal);
    k_make_beta<<<g.grid, g.block, 0, c.stream>>>(n, l0.split, b.rho, b.mass_offset, b.scal,
                                                  -4.0 * M_PI * c.p.gconst, 1.0 / a, beta_scale(b),
                                                  l0.beta_r, l0.beta_b);
    prof_end(c, NYXPM_ST_RHS, 24.0 * nc);
    c.launches += 3;
    return check_launch(c, "make rhs");
}

nyxpm_status launch_zero_phi(Ctx& c, Box& b)
{
    const Level& l0 = b.levels[0];
    const size_t nc = (size_t)l0.n * l0.n * l0.n;
    if (l0.split) {
        cudaMemsetAsync(l0.phi_r, 0, sizeof(double) * nc / 2, c.stream);
        cudaMemsetAsync(l0.phi_b, 0, sizeof(double) * nc / 2, c.stream);
    } else {
        cudaMemsetAsync(l0.phi_r, 0, sizeof(double) * nc, c.stream);
    }
    return check_launch(c, "zero phi");
}

nyxpm_status mg_solve(Ctx& c, Box& b, nyxpm_solve_info* info)
{
    nyxpm_status st;
    const Level& l0 = b.levels[0];
    const long long nc = (long long)l0.n * l0.n * l0.n;
    // ||beta||_inf and ||r0||_inf
    prof_begin(c);
    cudaMemsetAsync(b.norms, 0, sizeof(unsigned long long), c.stream);
    if (l0.split) {
        k_absmax<<<norm_blocks(c, nc / 2), kThreads, 0, c.stream>>>(nc / 2, l0.beta_r, b.norms);
        k_absmax<<<norm_blocks(c, nc / 2), kThreads, 0, c.stream>>>(nc / 2, l0.beta_b, b.norms);
        c.launches += 1;
    } else {
        k_absmax<<<norm_blocks(c, nc), kThreads, 0, c.stream>>>(nc, l0.beta_r, b.norms);
    }
    prof_end(c, NYXPM_ST_NORM, 8.0 * nc);
    if ((st = check_launch(c, "rhs norm")) != NYXPM_OK) return st;
    if ((st = launch_resnorm(c, b, 1, 0)) != NYXPM_OK) return st;
    cudaMemcpyAsync(b.h_norms, b.norms, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                    c.stream);
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return check_launch(c, "solve sync");
    const double bnorm = read_norm(b, 0);
    const double r0 = read_norm(b, 1);
    const double target = c.p.rel_tol * std::max(bnorm, r0);
    double r = r0;
    int it = 0;
    nyxpm_status result = NYXPM_OK;
    const int red_only = (c.p.nu2 > 0 && b.levels.size() > 1) ? 1 : 0;
    // The red-cell norm after a V-cycle and the red half sweep that opens the next
    // one share their neighbour sums: k_resnorm_red_sweep makes both, the sweep into
    // the spare red array, which becomes level 0's red array only if the solve
    // goes on (the next V-cycle then starts at its black half sweep).
    Level& L0 = b.levels[0];
    const bool fuse = red_only && c.p.nu1 > 0 && L0.split && b.phi_r_spare;
    if (!(r0 <= target)) {
        bool first = true;
        auto iteration = [&]() -> nyxpm_status {
            nyxpm_status s;
            if ((s = vcycle(c, b, 0, fuse && !first ? 1 : 0)) != NYXPM_OK) return s;
            if (fuse) {
                const Geo g = geo3(L0.n / 2, L0.n, L0.n);
                prof_begin(c);
                cudaMemsetAsync(b.norms + 1, 0, sizeof(unsigned long long), c.stream);
                launch_pdl(c, k_resnorm_red_sweep, dim3(g.grid), dim3(g.block), L0.n, L0.phi_r, L0.phi_b, L0.beta_r,
                                                                      b.phi_r_spare, b.norms + 1);
                prof_end(c, NYXPM_ST_NORM, 16.0 * nc);
                if ((s = check_launch(c, "red norm + sweep")) != NYXPM_OK) return s;
            } else if ((s = launch_resnorm(c, b, 1, red_only)) != NYXPM_OK) {
                return s;
            }
            cudaMemcpyAsync(b.h_norms + 1, b.norms + 1, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, c.stream);
            return check_launch(c, "norm copy");
        };
        for (it = 1; it <= c.p.max_vcycles; ++it) {
            // one graph per (opening or later iteration, physical red array)
            const int gi = (first ? 0 : 2) + (L0.phi_r == b.phi_r_alloc ? 0 : 1);
            if ((st = run_iteration(c, b.iter_graph[gi], iteration)) != NYXPM_OK) return st;
            if (cudaStreamSynchronize(c.stream) != cudaSuccess) return check_launch(c, "solve sync");
            r = read_norm(b, 1);
            if (r != r) {
                c.err = "multigrid residual is NaN";
                return NYXPM_NOT_CONVERGED;
            }
            if (r <= target) break;
            if (fuse && it < c.p.max_vcycles) {
                std::swap(L0.phi_r, b.phi_r_spare);
                first = false;
            }
        }
        if (it > c.p.max_vcycles) {
            it = c.p.max_vcycles;
            result = NYXPM_NOT_CONVERGED;
            c.err = "multigrid reached max_vcycles above tolerance";
        }
    }
    b.have_phi = 1;
    if (info) {
        const double inv_k0 = 1.0 / beta_scale(b);
        info->vcycles = it;
        info->inner_vcycles = 0;
        info->resnorm0 = r0 * inv_k0;
        info->resnorm = r * inv_k0;
        info->bnorm = bnorm * inv_k0;
    }
    return result;
}

nyxpm_status launch_grav_vector(Ctx& c, Box& b)
{
    const long long nc = (long long)b.n * b.n * b.n;
    const Geo g = geo3(b.n, b.n, b.n);
    prof_begin(c);
    k_grav<<<g.grid, g.block, 0, c.stream>>>(view(b.levels[0]), b.dxi, b.g);
    prof_end(c, NYXPM_ST_KICK, 32.0 * nc);
    return check_launch(c, "grav vector");
}

nyxpm_status launch_phi_to_natural(Ctx& c, Box& b, double* d_out)
{
    const long long nc = (long long)b.n * b.n * b.n;
    const Geo g = geo3(b.n, b.n, b.n);
    prof_begin(c);
    k_to_natural<<<g.grid, g.block, 0, c.stream>>>(view(b.levels[0]), d_out);
    prof_end(c, NYXPM_ST_GATHER, 16.0 * nc);
    return check_launch(c, "phi to natural");
}

nyxpm_status launch_phi_from_natural(Ctx& c, Box& b, const double* d_in)
{
    const long long nc = (long long)b.n * b.n * b.n;
    const Geo g = geo3(b.n, b.n, b.n);
    prof_begin(c);
    k_from_natural<<<g.grid, g.block, 0, c.stream>>>(view(b.levels[0]), d_in);
    prof_end(c, NYXPM_ST_GATHER, 16.0 * nc);
    return check_launch(c, "phi from natural");
}

nyxpm_status mg_vcycle_zero(Ctx& c, Box& b, const double* beta_nat, double* e_nat)
{
    nyxpm_status st;
    const long long nc = (long long)b.n * b.n * b.n;
    const Geo g = geo3(b.n, b.n, b.n);
    prof_begin(c);
    k_beta_from_natural<<<g.grid, g.block, 0, c.stream>>>(view(b.levels[0]), beta_nat);
    prof_end(c, NYXPM_ST_RHS, 16.0 * nc);
    if ((st = launch_zero_phi(c, b)) != NYXPM_OK) return st;
    if ((st = vcycle(c, b, 0)) != NYXPM_OK) return st;
    return launch_phi_to_natural(c, b, e_nat);
}

}  // namespace nyxpm
