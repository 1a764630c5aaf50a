// The coarse end of a V-cycle run by one CTA: every level from the first one of
// at most mg_fused_edge cells per edge (half that in FP64) down to the bottom is smoothed,
// restricted, solved exactly and prolonged by the block, with a block barrier
// between the passes.  It replaces some 20 dependent launches of a few hundred
// to a few thousand cells each per V-cycle.  (One SM is slower than a
// grid-wide launch from 32^3 cells up: 16 is the default edge.)
//
// Each cell's arithmetic is the one of the per-pass kernels (red-black
// Gauss-Seidel, residual + restriction, circulant bottom solve, trilinear
// prolongation + correction), in the same order, so a fused V-cycle gives the
// same bits as the launches it replaces.  The code is templated on the scalar:
// float for the mixed form's inner V-cycles, double for the coarsest levels of
// the FP64 form (whose restriction sums the red children only, as k_restrict<1>).  Loads are plain (not the read-only
// path): the block writes what it reads.
#pragma once

#include "pm_common.cuh"

namespace nyxpm {

constexpr int kMaxTail = 8;
constexpr int kTailThreads = 1024;   // FP32 tail: levels up to 16^3
constexpr int kTailThreadsD = 256;   // FP64 tail: levels up to 8^3 (256 cells per half sweep)

__device__ __forceinline__ int tail_wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// t -> (x, y, z) with x < nx, y < ny: shifts when both are powers of two
__device__ __forceinline__ void tail_split3(int t, int nx, int ny, int& x, int& y, int& z)
{
    if (((nx & (nx - 1)) | (ny & (ny - 1))) == 0) {
        const int sx = __ffs(nx) - 1, sy = __ffs(ny) - 1;
        x = t & (nx - 1);
        y = (t >> sx) & (ny - 1);
        z = t >> (sx + sy);
    } else {
        const int r = t / nx;
        x = t - r * nx;
        z = r / ny;
        y = r - z * ny;
    }
}

// trilinear weights 27/64, 9/64, 9/64, 3/64, 9/64, 3/64, 3/64, 1/64 at index tt + 2a + 4b
template <typename T>
__device__ __forceinline__ T tail_prolong_w(int idx)
{
    constexpr T w[8] = {T(0.421875), T(0.140625), T(0.140625), T(0.046875),
                        T(0.140625), T(0.046875), T(0.046875), T(0.015625)};
    return w[idx];
}

__device__ __forceinline__ float tail_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double tail_fma(double a, double b, double c) { return fma(a, b, c); }
template <typename T>
__device__ __forceinline__ T tail_sixth() { return T(1) / T(6); }

// one red (color 0) or black (1) half sweep of a split level
template <typename T, typename LV>
__device__ __forceinline__ void tail_gsrb(const LV& F, int color)
{
    const int n = F.n, half = n >> 1;
    const int total = half * n * n;
    T* mine = color ? F.phi_b : F.phi_r;
    const T* other = color ? F.phi_r : F.phi_b;
    const T* beta = color ? F.beta_b : F.beta_r;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int ih, j, k;
        tail_split3(t, half, n, ih, j, k);
        const int q = (j + k + color) & 1;
        const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
        const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        const int row = j + n * k;
        T s = other[row * half + ihm] + other[row * half + ihp];
        s = s + other[(jm + n * k) * half + ih];
        s = s + other[(jp + n * k) * half + ih];
        s = s + other[(j + n * km) * half + ih];
        s = s + other[(j + n * kp) * half + ih];
        mine[t] = tail_fma(s, tail_sixth<T>(), -beta[t]);
    }
}

template <typename T, typename LV>
__device__ __forceinline__ T tail_resid(const LV& L, int i, int j, int k)
{
    const int n = L.n;
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    T s = *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, im, j, k) +
          *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, ip, j, k);
    s = s + *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, i, jm, k);
    s = s + *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, i, jp, k);
    s = s + *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, i, j, km);
    s = s + *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, i, j, kp);
    const T c = *lv_ptr<T>(L.phi_r, L.phi_b, n, L.split, i, j, k);
    return *lv_ptr<T>(L.beta_r, L.beta_b, n, L.split, i, j, k) - tail_fma(s, tail_sixth<T>(), -c);
}

// residual of F restricted to the coarse right-hand side; coarse phi = 0.
// red_only: the children with di + dj + dk even only (F ends its pre-smoothing
// with a black half sweep, so the black residuals are round-off)
template <typename T, typename LV>
__device__ __forceinline__ void tail_restrict(const LV& F, const LV& Cv, bool red_only)
{
    const int nc = Cv.n;
    const int total = nc * nc * nc;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int I, J, K;
        tail_split3(t, nc, nc, I, J, K);
        T s = T(0);
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int di = 0; di < 2; ++di)
                    if (!red_only || ((di + dj + dk) & 1) == 0)
                        s = s + tail_resid<T>(F, 2 * I + di, 2 * J + dj, 2 * K + dk);
        *lv_ptr<T>(Cv.beta_r, Cv.beta_b, nc, Cv.split, I, J, K) = s * T(0.5);
        *lv_ptr<T>(Cv.phi_r, Cv.phi_b, nc, Cv.split, I, J, K) = T(0);
    }
}

// fine phi += trilinear interpolation of the coarse phi (black: the black fine
// cells only -- the post-smoothing's first half sweep overwrites the red ones
// unread)
template <typename T, typename LV>
__device__ __forceinline__ void tail_prolong(const LV& Cv, const LV& F, bool black)
{
    const int n = F.n, nc = Cv.n, half = n >> 1;
    const int total = half * n * n;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int ih, j, k;
        tail_split3(t, half, n, ih, j, k);
        const int J = j >> 1, K = k >> 1;
        const int Js[2] = {J, tail_wrap((j & 1) ? J + 1 : J - 1, nc)};
        const int Ks[2] = {K, tail_wrap((k & 1) ? K + 1 : K - 1, nc)};
#pragma unroll
        for (int odd = 0; odd < 2; ++odd) {
            const int i = 2 * ih + odd;
            if (black && ((i + j + k) & 1) == 0) continue;
            const int Is[2] = {ih, tail_wrap(odd ? ih + 1 : ih - 1, nc)};
            T s = T(0);
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int tt = 0; tt < 2; ++tt)
                        s = tail_fma(tail_prolong_w<T>(tt + 2 * a + 4 * b),
                                     *lv_ptr<const T>(Cv.phi_r, Cv.phi_b, nc, Cv.split, Is[tt], Js[a], Ks[b]),
                                     s);
            T* p = (((i + j + k) & 1) ? F.phi_b : F.phi_r) + t;
            *p = *p + s;
        }
    }
}

// exact bottom solve phi = G (*) beta on the natural nb^3 level (cyclic
// convolution, y in storage order); r and g are kMaxBottom^3 shared arrays
template <typename T, typename LV>
__device__ __forceinline__ void tail_bottom(const LV& B, const T* Gf, int nb, T* r, T* g)
{
    const int nc = nb * nb * nb;
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
        r[t] = B.beta_r[t];
        g[t] = Gf[t];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int i = c % nb, j = (c / nb) % nb, k = c / (nb * nb);
        T s = T(0);
        int y = 0;
        for (int yk = 0; yk < nb; ++yk) {
            const int dk = tail_wrap(k - yk, nb) * nb * nb;
            for (int yj = 0; yj < nb; ++yj) {
                const int djk = dk + tail_wrap(j - yj, nb) * nb;
                for (int yi = 0; yi < nb; ++yi, ++y) s = tail_fma(g[djk + tail_wrap(i - yi, nb)], r[y], s);
            }
        }
        B.phi_r[c] = s;
    }
}

// the V-cycle over lv[0 .. nl-1] (lv[nl-1] the natural bottom) by the calling
// block; lv[0]'s right-hand side is in place and its phi is the initial guess
// red_restrict: restrictions after pre-smoothing sum the red children only
template <typename T, typename LV>
__device__ __forceinline__ void vcycle_tail(const LV* lv, int nl, int nu1, int nu2, const T* Gf,
                                            int nb, T* r, T* g, bool red_restrict)
{
    for (int l = 0; l + 1 < nl; ++l) {
        for (int sw = 0; sw < nu1; ++sw) {
            tail_gsrb<T>(lv[l], 0);
            __syncthreads();
            tail_gsrb<T>(lv[l], 1);
            __syncthreads();
        }
        tail_restrict<T>(lv[l], lv[l + 1], red_restrict && nu1 > 0);
        __syncthreads();
    }
    tail_bottom<T>(lv[nl - 1], Gf, nb, r, g);
    __syncthreads();
    for (int l = nl - 2; l >= 0; --l) {
        tail_prolong<T>(lv[l + 1], lv[l], nu2 > 0);
        __syncthreads();
        for (int sw = 0; sw < nu2; ++sw) {
            tail_gsrb<T>(lv[l], 0);
            __syncthreads();
            tail_gsrb<T>(lv[l], 1);
            __syncthreads();
        }
    }
}

}  // namespace nyxpm
