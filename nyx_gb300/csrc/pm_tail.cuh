// The coarse end of an FP32 V-cycle run by one CTA: every level from the first
// one of at most mg_fused_edge cells per edge down to the bottom is smoothed,
// restricted, solved exactly and prolonged by the block, with a block barrier
// between the passes.  It replaces some 20 dependent launches of a few hundred
// to a few thousand cells each per V-cycle.  (One SM is slower than a
// grid-wide launch from 32^3 cells up: 16 is the default edge.)
//
// Each cell's arithmetic is the one of the per-pass FP32 kernels (red-black
// Gauss-Seidel, residual + restriction, circulant bottom solve, trilinear
// prolongation + correction), in the same order, so a fused V-cycle gives the
// same bits as the launches it replaces.  Loads are plain (not the read-only
// path): the block writes what it reads.
#pragma once

#include "pm_common.cuh"

namespace nyxpm {

constexpr int kMaxTail = 8;
constexpr int kTailThreads = 1024;

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
__device__ __forceinline__ float tail_prolong_w(int idx)
{
    constexpr float w[8] = {0.421875f, 0.140625f, 0.140625f, 0.046875f,
                            0.140625f, 0.046875f, 0.046875f, 0.015625f};
    return w[idx];
}

// one red (color 0) or black (1) half sweep of a split level
__device__ __forceinline__ void tail_gsrb(const LevelViewF& F, int color)
{
    const int n = F.n, half = n >> 1;
    const int total = half * n * n;
    float* mine = color ? F.phi_b : F.phi_r;
    const float* other = color ? F.phi_r : F.phi_b;
    const float* beta = color ? F.beta_b : F.beta_r;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int ih, j, k;
        tail_split3(t, half, n, ih, j, k);
        const int q = (j + k + color) & 1;
        const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
        const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        const int row = j + n * k;
        float s = other[row * half + ihm] + other[row * half + ihp];
        s = s + other[(jm + n * k) * half + ih];
        s = s + other[(jp + n * k) * half + ih];
        s = s + other[(j + n * km) * half + ih];
        s = s + other[(j + n * kp) * half + ih];
        mine[t] = fmaf(s, 1.0f / 6.0f, -beta[t]);
    }
}

__device__ __forceinline__ float tail_resid(const LevelViewF& L, int i, int j, int k)
{
    const int n = L.n;
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    float s = *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, im, j, k) +
              *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, ip, j, k);
    s += *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, i, jm, k);
    s += *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, i, jp, k);
    s += *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, i, j, km);
    s += *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, i, j, kp);
    const float c = *lv_ptr<float>(L.phi_r, L.phi_b, n, L.split, i, j, k);
    return *lv_ptr<float>(L.beta_r, L.beta_b, n, L.split, i, j, k) - fmaf(s, 1.0f / 6.0f, -c);
}

// residual of F restricted to the coarse right-hand side; coarse phi = 0
__device__ __forceinline__ void tail_restrict(const LevelViewF& F, const LevelViewF& Cv)
{
    const int nc = Cv.n;
    const int total = nc * nc * nc;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int I, J, K;
        tail_split3(t, nc, nc, I, J, K);
        float s = 0.f;
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int di = 0; di < 2; ++di) s += tail_resid(F, 2 * I + di, 2 * J + dj, 2 * K + dk);
        *lv_ptr<float>(Cv.beta_r, Cv.beta_b, nc, Cv.split, I, J, K) = s * 0.5f;
        *lv_ptr<float>(Cv.phi_r, Cv.phi_b, nc, Cv.split, I, J, K) = 0.f;
    }
}

// fine phi += trilinear interpolation of the coarse phi (black: the black fine
// cells only -- the post-smoothing's first half sweep overwrites the red ones
// unread)
__device__ __forceinline__ void tail_prolong(const LevelViewF& Cv, const LevelViewF& F, bool black)
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
            float s = 0.f;
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int tt = 0; tt < 2; ++tt)
                        s = fmaf(tail_prolong_w(tt + 2 * a + 4 * b),
                                 *lv_ptr<const float>(Cv.phi_r, Cv.phi_b, nc, Cv.split, Is[tt], Js[a], Ks[b]),
                                 s);
            float* p = (((i + j + k) & 1) ? F.phi_b : F.phi_r) + t;
            *p += s;
        }
    }
}

// exact bottom solve phi = G (*) beta on the natural nb^3 level (cyclic
// convolution, y in storage order); r and g are kMaxBottom^3 shared arrays
__device__ __forceinline__ void tail_bottom(const LevelViewF& B, const float* Gf, int nb, float* r,
                                            float* g)
{
    const int nc = nb * nb * nb;
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
        r[t] = B.beta_r[t];
        g[t] = Gf[t];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int i = c % nb, j = (c / nb) % nb, k = c / (nb * nb);
        float s = 0.f;
        int y = 0;
        for (int yk = 0; yk < nb; ++yk) {
            const int dk = tail_wrap(k - yk, nb) * nb * nb;
            for (int yj = 0; yj < nb; ++yj) {
                const int djk = dk + tail_wrap(j - yj, nb) * nb;
                for (int yi = 0; yi < nb; ++yi, ++y) s = fmaf(g[djk + tail_wrap(i - yi, nb)], r[y], s);
            }
        }
        B.phi_r[c] = s;
    }
}

// the V-cycle over lv[0 .. nl-1] (lv[nl-1] the natural bottom) by the calling
// block; lv[0]'s right-hand side is in place and its phi is the initial guess
__device__ __forceinline__ void vcycle_tail(const LevelViewF* lv, int nl, int nu1, int nu2,
                                            const float* Gf, int nb, float* r, float* g)
{
    for (int l = 0; l + 1 < nl; ++l) {
        for (int sw = 0; sw < nu1; ++sw) {
            tail_gsrb(lv[l], 0);
            __syncthreads();
            tail_gsrb(lv[l], 1);
            __syncthreads();
        }
        tail_restrict(lv[l], lv[l + 1]);
        __syncthreads();
    }
    tail_bottom(lv[nl - 1], Gf, nb, r, g);
    __syncthreads();
    for (int l = nl - 2; l >= 0; --l) {
        tail_prolong(lv[l + 1], lv[l], nu2 > 0);
        __syncthreads();
        for (int sw = 0; sw < nu2; ++sw) {
            tail_gsrb(lv[l], 0);
            __syncthreads();
            tail_gsrb(lv[l], 1);
            __syncthreads();
        }
    }
}

}  // namespace nyxpm
