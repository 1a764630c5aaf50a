// Mixed-precision form of the PM step.
//
// Particles are stored cell-relative: the cell of floor(x/dx) packed as
// i | j << 10 | k << 20 and the offset inside it as three FP32 values in [0, 1),
// so a position keeps 24 bits relative to its cell anywhere in the box.
// Velocities are FP32.  The deposit and the multigrid V-cycles run in FP32; the
// solution phi, the right-hand side and the outer residual stay FP64 and the
// FP32 V-cycles are used as the inner solver of an FP64 defect correction
// (r = rhs - L phi in FP64; L e = r by FP32 V-cycles; phi += e in FP64) until
// the FP64 residual meets the same relative tolerance as the FP64 form.  The
// global mean density is a compensated FP64 sum; a(t) stays FP64 on the host.
//
// FP32 arithmetic is compiled with multiply-add contraction (the default): this
// form is checked against the FP64 oracle by a stated tolerance, not bitwise.
#include "pm_common.cuh"
#include "pm_prolong.cuh"
#include "pm_restrict.cuh"
#include "pm_tail.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace nyxpm {

namespace {

constexpr int kThreads = 256;
constexpr float kSixthF = 1.0f / 6.0f;
constexpr double kSixth = 1.0 / 6.0;

__constant__ float kProlongWF[8] = {0.421875f, 0.140625f, 0.140625f, 0.046875f,
                                    0.140625f, 0.046875f, 0.046875f, 0.015625f};

inline unsigned blocks_for(long long n, int t = kThreads)
{
    long long b = (n + t - 1) / t;
    return (unsigned)(b < 1 ? 1 : b);
}

__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

__device__ __forceinline__ int pack_cell(int i, int j, int k) { return i | (j << 10) | (k << 20); }
__device__ __forceinline__ int cell_i(int c) { return c & 1023; }
__device__ __forceinline__ int cell_j(int c) { return (c >> 10) & 1023; }
__device__ __forceinline__ int cell_k(int c) { return (c >> 20) & 1023; }

// split x = (i + o) dx with i = floor(x/dx) wrapped, o in [0, 1)
__device__ __forceinline__ void to_cell(double x, double dxi, int n, int* i, float* o)
{
    const double l = x * dxi;
    int il;
    const double fl = floor_int(l, &il);
    float f = f64_to_f32_rn(l - fl);
    if (f >= 1.0f) {  // rounding up to 1 moves the particle to the next cell's origin
        f = 0.0f;
        il += 1;
    }
    *i = wrapi(il, n);
    *o = f;
}

// deposit key along one axis and the CIC fraction: floor(o + 1/2) relative to the cell
__device__ __forceinline__ int key_frac(int ci, float o, int n, float* f)
{
    if (o >= 0.5f) {
        *f = o - 0.5f;
        return ci + 1 == n ? 0 : ci + 1;
    }
    *f = o + 0.5f;
    return ci;
}

// ---------------------------------------------------------------------------
// upload / download
// ---------------------------------------------------------------------------
__global__ void k_mx_unpack(long long np, int n, double dxi, const double* __restrict__ pos,
                            const double* __restrict__ vel, const double* __restrict__ mass,
                            int* cell, float* ox, float* oy, float* oz, float* vx, float* vy,
                            float* vz, float* m, int* id, unsigned long long* bad)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) ok = ok && isfinite(pos[3 * q + d]) && isfinite(vel[3 * q + d]);
    if (!ok) {
        atomicAdd(bad, 1ULL);
        cell[q] = 0;
        ox[q] = oy[q] = oz[q] = 0.f;
        vx[q] = vy[q] = vz[q] = 0.f;
        id[q] = (int)q;
        return;
    }
    int i, j, k;
    float a, b, c;
    to_cell(pos[3 * q], dxi, n, &i, &a);
    to_cell(pos[3 * q + 1], dxi, n, &j, &b);
    to_cell(pos[3 * q + 2], dxi, n, &k, &c);
    cell[q] = pack_cell(i, j, k);
    ox[q] = a;
    oy[q] = b;
    oz[q] = c;
    vx[q] = f64_to_f32_rn(vel[3 * q]);
    vy[q] = f64_to_f32_rn(vel[3 * q + 1]);
    vz[q] = f64_to_f32_rn(vel[3 * q + 2]);
    if (m) m[q] = f64_to_f32_rn(mass[q]);
    id[q] = (int)q;
}

// The host-buffer step's split transfers (nyxpm_step_host): positions (and
// masses) first, velocities later; positions out as soon as the drift made them
// final (the mixed closing kick does not move particles).  Together these give
// exactly what k_mx_unpack and k_mx_pack give.
__global__ void k_mx_unpack_pos(long long np, int n, double dxi, const double* __restrict__ pos,
                                const double* __restrict__ mass, int* cell, float* ox, float* oy,
                                float* oz, float* m, int* id, unsigned long long* bad)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    id[q] = (int)q;
    if (m) m[q] = f64_to_f32_rn(mass[q]);
    const double px = pos[3 * q], py = pos[3 * q + 1], pz = pos[3 * q + 2];
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) {
        atomicAdd(bad, 1ULL);
        cell[q] = 0;
        ox[q] = oy[q] = oz[q] = 0.f;
        return;
    }
    int i, j, k;
    float a, b, c;
    to_cell(px, dxi, n, &i, &a);
    to_cell(py, dxi, n, &j, &b);
    to_cell(pz, dxi, n, &k, &c);
    cell[q] = pack_cell(i, j, k);
    ox[q] = a;
    oy[q] = b;
    oz[q] = c;
}

// velocities in upload order; with perm, permuted by the sort that ran without
// them (vx[s] = vel[perm[s]]), else in place (vx[q] = vel[q])
__global__ void k_mx_unpack_vel(long long np, const double* __restrict__ vel,
                                const int* __restrict__ perm, float* vx, float* vy, float* vz,
                                unsigned long long* bad)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    const long long q = perm ? (long long)perm[s] : s;
    const double ux = vel[3 * q], uy = vel[3 * q + 1], uz = vel[3 * q + 2];
    if (!(isfinite(ux) && isfinite(uy) && isfinite(uz))) {
        atomicAdd(bad, 1ULL);
        vx[s] = vy[s] = vz[s] = 0.f;
        return;
    }
    vx[s] = f64_to_f32_rn(ux);
    vy[s] = f64_to_f32_rn(uy);
    vz[s] = f64_to_f32_rn(uz);
}

__global__ void k_mx_pack_pos(long long np, double dx, const int* __restrict__ cell,
                              const float* __restrict__ ox, const float* __restrict__ oy,
                              const float* __restrict__ oz, const int* __restrict__ id, double* pos)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int c = cell[q];
    const long long o = 3LL * id[q];
    pos[o] = ((double)cell_i(c) + f32_to_f64(ox[q])) * dx;
    pos[o + 1] = ((double)cell_j(c) + f32_to_f64(oy[q])) * dx;
    pos[o + 2] = ((double)cell_k(c) + f32_to_f64(oz[q])) * dx;
}

__global__ void k_mx_pack_vel(long long np, const float* __restrict__ vx, const float* __restrict__ vy,
                              const float* __restrict__ vz, const int* __restrict__ id, double* vel)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const long long o = 3LL * id[q];
    vel[o] = f32_to_f64(vx[q]);
    vel[o + 1] = f32_to_f64(vy[q]);
    vel[o + 2] = f32_to_f64(vz[q]);
}

__global__ void k_mx_pack(long long np, double dx, const int* __restrict__ cell,
                          const float* __restrict__ ox, const float* __restrict__ oy,
                          const float* __restrict__ oz, const float* __restrict__ vx,
                          const float* __restrict__ vy, const float* __restrict__ vz,
                          const int* __restrict__ id, double* pos, double* vel)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int c = cell[q];
    const long long o = 3LL * id[q];
    pos[o] = ((double)cell_i(c) + f32_to_f64(ox[q])) * dx;
    pos[o + 1] = ((double)cell_j(c) + f32_to_f64(oy[q])) * dx;
    pos[o + 2] = ((double)cell_k(c) + f32_to_f64(oz[q])) * dx;
    vel[o] = f32_to_f64(vx[q]);
    vel[o + 1] = f32_to_f64(vy[q]);
    vel[o + 2] = f32_to_f64(vz[q]);
}

// ---------------------------------------------------------------------------
// sort
// ---------------------------------------------------------------------------
__global__ void k_mx_keys(long long np, int n, const int* __restrict__ cell,
                          const float* __restrict__ ox, const float* __restrict__ oy,
                          const float* __restrict__ oz, int* key, int* count)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int c = cell[q];
    float f;
    const int i = key_frac(cell_i(c), ox[q], n, &f);
    const int j = key_frac(cell_j(c), oy[q], n, &f);
    const int k = key_frac(cell_k(c), oz[q], n, &f);
    const int K = (int)cidx(i, j, k, n);
    key[q] = K;
    atomicAdd(count + K, 1);
}

__global__ void k_mx_gather(long long np, const int* __restrict__ perm, const int* __restrict__ cell,
                            const float* __restrict__ ox, const float* __restrict__ oy,
                            const float* __restrict__ oz, const float* __restrict__ vx,
                            const float* __restrict__ vy, const float* __restrict__ vz,
                            const float* __restrict__ m, const int* __restrict__ id, int* cell2,
                            float* ox2, float* oy2, float* oz2, float* vx2, float* vy2, float* vz2,
                            float* m2, int* id2)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    const int q = perm[s];
    cell2[s] = cell[q];
    ox2[s] = ox[q];
    oy2[s] = oy[q];
    oz2[s] = oz[q];
    if (vx) {   // null: the velocities follow later (k_mx_unpack_vel with perm)
        vx2[s] = vx[q];
        vy2[s] = vy[q];
        vz2[s] = vz[q];
    }
    if (m) m2[s] = m[q];
    id2[s] = id[q];
}

// ---------------------------------------------------------------------------
// FP32 deposit (same tiling as the FP64 form: per-key partials in shared
// memory, cells add their 8 key partials in a fixed order)
// ---------------------------------------------------------------------------

// adds particle q's eight CIC weights (times its mass, if m) to s
__device__ __forceinline__ void mx_add_weights(int q, int n, const int* __restrict__ cell,
                                               const float* __restrict__ ox,
                                               const float* __restrict__ oy,
                                               const float* __restrict__ oz,
                                               const float* __restrict__ m, float s[8])
{
    const int c = cell[q];
    float fx, fy, fz;
    key_frac(cell_i(c), ox[q], n, &fx);
    key_frac(cell_j(c), oy[q], n, &fy);
    key_frac(cell_k(c), oz[q], n, &fz);
    const float sx[2] = {1.f - fx, fx};
    const float sy[2] = {1.f - fy, fy};
    const float sz[2] = {1.f - fz, fz};
    const float mq = m ? m[q] : 1.f;
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
            for (int cx = 0; cx < 2; ++cx)
                s[cx + 2 * cy + 4 * cz] += (sx[cx] * sy[cy]) * sz[cz] * mq;
}

// keys longer than a warp (the sort's long_list), one warp each: lane-strided
// partials and an xor butterfly, as the FP64 deposit sums them
__global__ void __launch_bounds__(256) k_mx_deposit_heavy(int n, const int* __restrict__ cell,
                                                          const float* __restrict__ ox,
                                                          const float* __restrict__ oy,
                                                          const float* __restrict__ oz,
                                                          const float* __restrict__ m,
                                                          const int* __restrict__ start,
                                                          const int* __restrict__ long_list,
                                                          const int* __restrict__ long_count,
                                                          int* key_slot, float* heavy_part)
{
    const int lane = threadIdx.x & 31;
    const int total = *long_count;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < total; li += nwarps) {
        const int K = long_list[li];
        const int e = start[K + 1];
        float s[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) s[c] = 0.f;
        for (int q = start[K] + lane; q < e; q += 32) mx_add_weights(q, n, cell, ox, oy, oz, m, s);
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c] += __shfl_xor_sync(0xffffffffu, s[c], off);
        if (lane < 8) {
            float v = s[0];
#pragma unroll
            for (int c = 1; c < 8; ++c)
                if (lane == c) v = s[c];
            heavy_part[8LL * li + lane] = v;
        }
        if (lane == 0) key_slot[K] = li;
    }
}

// One CTA per tile of 8 x 8 x 8 cells.  Phase 1: one thread per key of the
// 9 x 9 x 9 key window (cells of floor(x/dx + 1/2), from the tile's corner to one
// past its far corner) sums its segment's 8 corner weights in sorted order (keys
// longer than a warp take their sums from k_mx_deposit_heavy).  Phase 2: each
// cell adds the 8 corner sums of its keys in a fixed (dk, dj, di) order.  No
// atomics: the order of every sum is fixed, so the density is bitwise
// reproducible.  (Measured against it at 256^3, one particle per cell, on
// GB300, and slower: a 16 x 8 x 8 tile whose warps number the window's particles
// densely and stage their weights in shared memory, 382-384 us against 233 us;
// cell sums by shared-memory fixed-point atomics, 270 us with 32-bit and 464 us
// and more with 64-bit accumulators.)
constexpr int kDepTx = 8, kDepTy = 8, kDepTz = 8;
constexpr int kDepKx = kDepTx + 1, kDepKy = kDepTy + 1, kDepKz = kDepTz + 1;
constexpr int kDepKeys = kDepKx * kDepKy * kDepKz;   // 729
constexpr int kDepThreads = 256;

__device__ __forceinline__ int wrap_up(int i, int n)
{
    while (i >= n) i -= n;   // i < n + 9: at most one pass unless n < 9
    return i;
}

__global__ void __launch_bounds__(kDepThreads) k_mx_deposit(
    int n, float scale, const int* __restrict__ cell, const float* __restrict__ ox,
    const float* __restrict__ oy, const float* __restrict__ oz, const float* __restrict__ m,
    const int* __restrict__ start, const int* __restrict__ key_slot,
    const float* __restrict__ heavy_part, float* rho)
{
    // corner-major: a warp's 32 consecutive keys (or cells) touch 32 banks
    __shared__ float part[8 * kDepKeys];
    const int i0 = blockIdx.x * kDepTx, j0 = blockIdx.y * kDepTy, k0 = blockIdx.z * kDepTz;
    for (int kl = threadIdx.x; kl < kDepKeys; kl += blockDim.x) {
        const int ki = kl % kDepKx, kj = (kl / kDepKx) % kDepKy, kk = kl / (kDepKx * kDepKy);
        const long long K = cidx(wrap_up(i0 + ki, n), wrap_up(j0 + kj, n), wrap_up(k0 + kk, n), n);
        float s[8];
        const int b0 = start[K], e = start[K + 1];
        if (e - b0 > kDepositLanes) {
            const float* hp = heavy_part + 8LL * key_slot[K];
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c] = hp[c];
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c] = 0.f;
            for (int q = b0; q < e; ++q) mx_add_weights(q, n, cell, ox, oy, oz, m, s);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) part[c * kDepKeys + kl] = s[c];
    }
    __syncthreads();
    for (int cl = threadIdx.x; cl < kDepTx * kDepTy * kDepTz; cl += blockDim.x) {
        const int ci = cl % kDepTx, cj = (cl / kDepTx) % kDepTy, ck = cl / (kDepTx * kDepTy);
        const int i = i0 + ci, j = j0 + cj, k = k0 + ck;
        if (i >= n || j >= n || k >= n) continue;
        float acc = 0.f;
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int di = 0; di < 2; ++di) {
                    const int kl = (ci + di) + kDepKx * ((cj + dj) + kDepKy * (ck + dk));
                    acc += part[((1 - di) + 2 * (1 - dj) + 4 * (1 - dk)) * kDepKeys + kl];
                }
        rho[cidx(i, j, k, n)] = acc * scale;
    }
}

__global__ void k_f2d(long long cnt, const float* __restrict__ a, double* b)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) b[t] = a[t];
}

// ---------------------------------------------------------------------------
// compensated FP64 mean of (rho - mass_offset) and the FP64 right-hand side
// ---------------------------------------------------------------------------
__device__ __forceinline__ void kahan_add(double& s, double& c, double v)
{
    const double y = v - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
}

// one warp per plane row: each lane sums its FP32 densities as a double-float
// pair (TwoSum on the FP32 pipe, exact to ~2^-48), the lanes' pairs are added in
// FP64 and n * mass_offset is taken off once per row
__global__ void k_mx_rowsum(int n, const float* __restrict__ rho, double mo, double* rows)
{
    const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= (long long)n * n) return;
    const float* r = rho + row * n;
    float sh = 0.f, sl = 0.f;
    for (int i = lane; i < n; i += 32) {
        float err;
        df_two_sum(sh, r[i], sh, err);
        sl = __fadd_rn(sl, err);
    }
    double s = f32_to_f64(sh) + f32_to_f64(sl);
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const double t = __shfl_down_sync(0xffffffffu, s, off);
        if (lane < off) s = s + t;
    }
    if (lane == 0) rows[row] = s - (double)n * mo;
}

__global__ void k_mx_mean(int n, double dx, double L, const double* __restrict__ rows, double* scal)
{
    // one block: compensated sum of the n^2 row sums
    __shared__ double ss[32];
    double s = 0.0, c = 0.0;
    for (long long r = threadIdx.x; r < (long long)n * n; r += blockDim.x) kahan_add(s, c, rows[r]);
    s -= c;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) ss[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, tc = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) kahan_add(t, tc, ss[q]);
        t -= tc;
        scal[0] = (t * (dx * dx * dx)) / (L * L * L);
    }
}

// beta = (rho - mass_offset - mean) * (-4 pi G / a) * h^2/6: one FP64 subtraction
// and one product per cell (offset and scale folded once)
__global__ void k_mx_make_beta(int n, int split, const float* __restrict__ rho, double mo,
                               const double* __restrict__ scal, double scale, double* beta_r,
                               double* beta_b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    const double off = mo + scal[0];
    const double v = f32_to_f64(rho[cidx(i, j, k, n)]);
    *lv_ptr<double>(beta_r, beta_b, n, split, i, j, k) = (v - off) * scale;
}

// ---------------------------------------------------------------------------
// norms (max over |v| bits on the integer pipe)
// ---------------------------------------------------------------------------
__global__ void k_mx_absmax(long long cnt, const double* __restrict__ a, unsigned long long* out)
{
    unsigned long long v = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < cnt;
         t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long u = absbits(a[t]);
        v = u > v ? u : v;
    }
    block_umax_store(v, out);
}

// ---------------------------------------------------------------------------
// outer FP64 residual -> FP32 inner right-hand side (+ its max norm)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T nbr_sum_split(const T* other, int n, int half, int ih, int j, int k,
                                           int q)
{
    const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
    const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    const long long row = (long long)j + (long long)n * k;
    T s = other[row * half + ihm] + other[row * half + ihp];
    s = s + other[((long long)jm + (long long)n * k) * half + ih];
    s = s + other[((long long)jp + (long long)n * k) * half + ih];
    s = s + other[((long long)j + (long long)n * km) * half + ih];
    s = s + other[((long long)j + (long long)n * kp) * half + ih];
    return s;
}

// residual of both colours of a split level 0: r = beta - (s/6 - phi), one thread per (ih, j, k)
__global__ void k_mx_resid(int n, const double* __restrict__ phi_r, const double* __restrict__ phi_b,
                           const double* __restrict__ beta_r, const double* __restrict__ beta_b,
                           float* r_r, float* r_b, float* rl_r, float* rl_b,
                           unsigned long long* norm)
{
    const int half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (ih < half && j < n) {
        const long long t = ((long long)j + (long long)n * k) * half + ih;
#pragma unroll
        for (int color = 0; color < 2; ++color) {
            const int q = (j + k + color) & 1;
            const double* other = color ? phi_r : phi_b;
            const double* mine = color ? phi_b : phi_r;
            const double* beta = color ? beta_b : beta_r;
            const double s = nbr_sum_split<double>(other, n, half, ih, j, k, q);
            const double r = beta[t] - fma(s, kSixth, -mine[t]);
            const float h = f64_to_f32_rn(r);
            (color ? r_b : r_r)[t] = h;
            if (rl_r) (color ? rl_b : rl_r)[t] = f64_to_f32_rn(r - f32_to_f64(h));
            const unsigned long long u = absbits(r);
            v = u > v ? u : v;
        }
    }
    block_umax_store(v, norm);
}

// The same residual, two compact cells of each colour per thread (16-byte
// loads of FP64 pairs) for rows of an even number of compact cells.  Every
// residual is k_mx_resid's, term for term.
__global__ void k_mx_resid2(int n, const double* __restrict__ phi_r, const double* __restrict__ phi_b,
                            const double* __restrict__ beta_r, const double* __restrict__ beta_b,
                            float* r_r, float* r_b, float* rl_r, float* rl_b,
                            unsigned long long* norm)
{
    const unsigned half = (unsigned)n >> 1;
    const unsigned t2 = blockIdx.x * blockDim.x + threadIdx.x;   // compact cells 2 t2, 2 t2 + 1
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (t2 < half / 2 && j < n) {
        const unsigned ih = 2 * t2;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
        const unsigned r0 = row(j, k);
        const unsigned t = r0 + ih;
#pragma unroll
        for (int color = 0; color < 2; ++color) {
            const int q = (j + k + color) & 1;
            const double* other = color ? phi_r : phi_b;
            const double* mine = color ? phi_b : phi_r;
            const double* beta = color ? beta_b : beta_r;
            const double2 c = __ldg(reinterpret_cast<const double2*>(other + t));
            double xm0, xm1, xp0, xp1;
            if (q) {   // neighbours ih, ih + 1
                const double e = __ldg(other + r0 + (ih + 2 == half ? 0u : ih + 2));
                xm0 = c.x; xp0 = c.y; xm1 = c.y; xp1 = e;
            } else {   // neighbours ih - 1, ih
                const double e = __ldg(other + r0 + (ih == 0 ? half - 1 : ih - 1));
                xm0 = e; xp0 = c.x; xm1 = c.x; xp1 = c.y;
            }
            const double2 ym = __ldg(reinterpret_cast<const double2*>(other + row(jm, k) + ih));
            const double2 yp = __ldg(reinterpret_cast<const double2*>(other + row(jp, k) + ih));
            const double2 zm = __ldg(reinterpret_cast<const double2*>(other + row(j, km) + ih));
            const double2 zp = __ldg(reinterpret_cast<const double2*>(other + row(j, kp) + ih));
            const double2 b = __ldg(reinterpret_cast<const double2*>(beta + t));
            const double2 m = __ldg(reinterpret_cast<const double2*>(mine + t));
            double s0 = xm0 + xp0;
            s0 = s0 + ym.x;
            s0 = s0 + yp.x;
            s0 = s0 + zm.x;
            s0 = s0 + zp.x;
            double s1 = xm1 + xp1;
            s1 = s1 + ym.y;
            s1 = s1 + yp.y;
            s1 = s1 + zm.y;
            s1 = s1 + zp.y;
            const double r0v = b.x - fma(s0, kSixth, -m.x);
            const double r1v = b.y - fma(s1, kSixth, -m.y);
            const float h0 = f64_to_f32_rn(r0v), h1 = f64_to_f32_rn(r1v);
            reinterpret_cast<float2*>(color ? r_b : r_r)[t >> 1] = make_float2(h0, h1);
            if (rl_r)
                reinterpret_cast<float2*>(color ? rl_b : rl_r)[t >> 1] =
                    make_float2(f64_to_f32_rn(r0v - f32_to_f64(h0)), f64_to_f32_rn(r1v - f32_to_f64(h1)));
            const unsigned long long u0 = absbits(r0v), u1 = absbits(r1v);
            v = u0 > v ? u0 : v;
            v = u1 > v ? u1 : v;
        }
    }
    block_umax_store(v, norm);
}

// the same for a natural-layout level 0 (n <= 8)
__global__ void k_mx_resid_nat(int n, const double* __restrict__ phi, const double* __restrict__ beta,
                               float* r, unsigned long long* norm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long v = 0;
    if (i < n && j < n) {
        const int im = wrap1(i - 1, n), ip = wrap1(i + 1, n), jm = wrap1(j - 1, n), jp = wrap1(j + 1, n);
        const int km = wrap1(k - 1, n), kp = wrap1(k + 1, n);
        double s = phi[cidx(im, j, k, n)] + phi[cidx(ip, j, k, n)];
        s = s + phi[cidx(i, jm, k, n)];
        s = s + phi[cidx(i, jp, k, n)];
        s = s + phi[cidx(i, j, km, n)];
        s = s + phi[cidx(i, j, kp, n)];
        const long long c = cidx(i, j, k, n);
        const double rr = beta[c] - fma(s, kSixth, -phi[c]);
        r[c] = f64_to_f32_rn(rr);
        v = absbits(rr);
    }
    block_umax_store(v, norm);
}

// phi += e (FP64 update with the FP32 correction)
__global__ void k_mx_update(long long cnt, double* phi, const float* __restrict__ e)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) phi[t] = phi[t] + f32_to_f64(e[t]);
}

// Defect-correction step without an FP64 stencil: phi += e (FP64) and the
// residual r = beta - L phi, kept as a double-float (r_hi = the FP32 inner
// right-hand side, r_lo), is updated by r -= L e with L e = s(e)/6 - e formed in
// double-float from the FP32 correction e.  The error this adds is at most
// kDfUpdateErr * max|e|; the kernel reports max|e| (enorm) so that the solve can
// bound the difference between the tracked residual and the residual of phi,
// and recompute r with the FP64 stencil when the bound could matter.  One
// thread per compact cell of each colour of a split level 0.
__global__ void k_mx_correct(int n, float c_hi, float c_lo, const float* __restrict__ e_r,
                             const float* __restrict__ e_b, double* phi_r, double* phi_b,
                             float* r_r, float* r_b, float* rl_r, float* rl_b,
                             unsigned long long* norm, unsigned long long* enorm)
{
    const int half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    float vmax = 0.f, emax = 0.f;
    if (ih < half && j < n) {
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        const long long row = (long long)j + (long long)n * k;
        const long long t = row * half + ih;
#pragma unroll
        for (int color = 0; color < 2; ++color) {
            const int q = (j + k + color) & 1;
            const float* other = color ? e_r : e_b;
            const float em = (color ? e_b : e_r)[t];
            const int ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
            const int ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
            const float v[6] = {other[row * half + ihm], other[row * half + ihp],
                                other[((long long)jm + (long long)n * k) * half + ih],
                                other[((long long)jp + (long long)n * k) * half + ih],
                                other[((long long)j + (long long)n * km) * half + ih],
                                other[((long long)j + (long long)n * kp) * half + ih]};
            float* rh_p = color ? r_b : r_r;
            float* rl_p = color ? rl_b : rl_r;
            float rh = rh_p[t], rl = rl_p[t];
            df_residual_update(v, em, c_hi, c_lo, rh, rl);
            rh_p[t] = rh;
            rl_p[t] = rl;
            double* pp = color ? phi_b : phi_r;
            pp[t] = pp[t] + f32_to_f64(em);
            vmax = fmaxf(vmax, fabsf(rh));
            emax = fmaxf(emax, fabsf(em));
        }
    }
    block_umax_store(absbits(f32_to_f64(vmax)), norm);
    block_umax_store(absbits(f32_to_f64(emax)), enorm);
}

// k_mx_correct with two compact cells of each colour per thread (8- and 16-byte
// accesses) for rows of an even number of compact cells; every cell's update is
// k_mx_correct's, term for term.
__global__ void k_mx_correct2(int n, float c_hi, float c_lo, const float* __restrict__ e_r,
                              const float* __restrict__ e_b, double* phi_r, double* phi_b,
                              float* r_r, float* r_b, float* rl_r, float* rl_b,
                              unsigned long long* norm, unsigned long long* enorm)
{
    const unsigned half = (unsigned)n >> 1;
    const unsigned t2 = blockIdx.x * blockDim.x + threadIdx.x;   // compact cells 2 t2, 2 t2 + 1
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    float vmax = 0.f, emax = 0.f;
    if (t2 < half / 2 && j < n) {
        const unsigned ih = 2 * t2;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
        const unsigned r0 = row(j, k);
        const unsigned t = r0 + ih;
#pragma unroll
        for (int color = 0; color < 2; ++color) {
            const int q = (j + k + color) & 1;
            const float* other = color ? e_r : e_b;
            const float2 em = __ldg(reinterpret_cast<const float2*>((color ? e_b : e_r) + t));
            const float2 c = __ldg(reinterpret_cast<const float2*>(other + t));
            float xm0, xm1, xp0, xp1;
            if (q) {   // neighbours ih, ih + 1
                const float e = __ldg(other + r0 + (ih + 2 == half ? 0u : ih + 2));
                xm0 = c.x; xp0 = c.y; xm1 = c.y; xp1 = e;
            } else {   // neighbours ih - 1, ih
                const float e = __ldg(other + r0 + (ih == 0 ? half - 1 : ih - 1));
                xm0 = e; xp0 = c.x; xm1 = c.x; xp1 = c.y;
            }
            const float2 ym = __ldg(reinterpret_cast<const float2*>(other + row(jm, k) + ih));
            const float2 yp = __ldg(reinterpret_cast<const float2*>(other + row(jp, k) + ih));
            const float2 zm = __ldg(reinterpret_cast<const float2*>(other + row(j, km) + ih));
            const float2 zp = __ldg(reinterpret_cast<const float2*>(other + row(j, kp) + ih));
            float2* rh_p = reinterpret_cast<float2*>((color ? r_b : r_r) + t);
            float2* rl_p = reinterpret_cast<float2*>((color ? rl_b : rl_r) + t);
            float2 rh = *rh_p, rl = *rl_p;
            const float v0[6] = {xm0, xp0, ym.x, yp.x, zm.x, zp.x};
            const float v1[6] = {xm1, xp1, ym.y, yp.y, zm.y, zp.y};
            df_residual_update(v0, em.x, c_hi, c_lo, rh.x, rl.x);
            df_residual_update(v1, em.y, c_hi, c_lo, rh.y, rl.y);
            *rh_p = rh;
            *rl_p = rl;
            double2* pp = reinterpret_cast<double2*>((color ? phi_b : phi_r) + t);
            double2 ph = *pp;
            ph.x = ph.x + f32_to_f64(em.x);
            ph.y = ph.y + f32_to_f64(em.y);
            *pp = ph;
            vmax = fmaxf(vmax, fmaxf(fabsf(rh.x), fabsf(rh.y)));
            emax = fmaxf(emax, fmaxf(fabsf(em.x), fabsf(em.y)));
        }
    }
    block_umax_store(absbits(f32_to_f64(vmax)), norm);
    block_umax_store(absbits(f32_to_f64(emax)), enorm);
}

// r0 = beta of a split level 0 as its two words (the residual of phi = 0)
__global__ void k_mx_split_beta(long long cnt, const double* __restrict__ beta_r,
                                const double* __restrict__ beta_b, float* r_r, float* r_b,
                                float* rl_r, float* rl_b)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const double br = beta_r[t], bb = beta_b[t];
    const float hr = f64_to_f32_rn(br), hb = f64_to_f32_rn(bb);
    r_r[t] = hr;
    r_b[t] = hb;
    rl_r[t] = f64_to_f32_rn(br - f32_to_f64(hr));
    rl_b[t] = f64_to_f32_rn(bb - f32_to_f64(hb));
}

// ---------------------------------------------------------------------------
// FP32 V-cycle kernels (smoother units, same structure as the FP64 form)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gsrb_f(int n, int color, float* __restrict__ mine,
                                                const float* __restrict__ other,
                                                const float* __restrict__ beta)
{
    pdl_wait();
    pdl_trigger();
    const int half = n >> 1;
    const int ih = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (ih >= half || j >= n) return;
    const int q = (j + k + color) & 1;
    const long long t = ((long long)j + (long long)n * k) * half + ih;
    const float s = nbr_sum_split<float>(other, n, half, ih, j, k, q);
    mine[t] = fmaf(s, kSixthF, -beta[t]);
}

// The same half sweep, four cells of a row per thread (one 16-byte load per
// neighbour row) marching over kMarchZ consecutive planes: the row of the plane
// above becomes the row of this plane and the one below it, so each plane
// loads three neighbour rows (y-1, y+1, z+1), the right-hand side and one edge
// value for the x neighbours.  The sums are the scalar kernel's, term for term.
// Needs half % 4 == 0 (rows start on 16 bytes).
// 2 planes: at 256^3 a block marching 4 planes leaves 2048 blocks, 2.25 waves
// at 6 blocks per SM, and the last wave's tail costs a quarter of the launch
// (measured 20.6 us per half sweep; 2 planes 19.1 us, 1 plane 19.4 us)
constexpr int kMarchZ = 2;
constexpr int kMarchMinEdge = 256;

template <int MZ>
__global__ void __launch_bounds__(256) k_gsrb_f4(int n, int color, float* __restrict__ mine,
                                                 const float* __restrict__ other,
                                                 const float* __restrict__ beta)
{
    pdl_wait();
    pdl_trigger();
    // 32-bit offsets: a level holds at most 1024^3 / 2 cells of a colour
    const unsigned half = (unsigned)n >> 1, h4 = half >> 2;
    const unsigned t4 = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k0 = blockIdx.z * MZ;
    if (t4 >= h4 || j >= n) return;
    const unsigned ih = 4 * t4;
    const unsigned plane = (unsigned)n * half;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const unsigned rj = (unsigned)j * half + ih, rjm = (unsigned)jm * half + ih,
                   rjp = (unsigned)jp * half + ih;
    const float4* o4 = reinterpret_cast<const float4*>(other);
    const float4* b4 = reinterpret_cast<const float4*>(beta);
    float4* m4 = reinterpret_cast<float4*>(mine);
    const int kfirst = k0 == 0 ? n - 1 : k0 - 1;
    float4 zm = __ldg(o4 + (((unsigned)kfirst * plane + rj) >> 2));
    float4 c = __ldg(o4 + (((unsigned)k0 * plane + rj) >> 2));
    // the levels this kernel runs on have n % 8 == 0: every block marches MZ planes
#pragma unroll
    for (int kk = 0; kk < MZ; ++kk) {
        const int k = k0 + kk;
        const int kp = k == n - 1 ? 0 : k + 1;
        const unsigned pk = (unsigned)k * plane;
        const float4 zp = __ldg(o4 + (((unsigned)kp * plane + rj) >> 2));
        const float4 ym = __ldg(o4 + ((pk + rjm) >> 2));
        const float4 yp = __ldg(o4 + ((pk + rjp) >> 2));
        const unsigned t = pk + rj;
        const float4 b = __ldg(b4 + (t >> 2));
        const int q = (j + k + color) & 1;
        // x neighbours: q = 1 -> (ih, ih+1), q = 0 -> (ih-1, ih) of the other colour
        const unsigned rowbase = t - ih;
        float xm0, xm1, xm2, xm3, xp0, xp1, xp2, xp3;
        if (q) {
            const float edge = __ldg(other + rowbase + (ih + 4 == half ? 0u : ih + 4));
            xm0 = c.x; xm1 = c.y; xm2 = c.z; xm3 = c.w;
            xp0 = c.y; xp1 = c.z; xp2 = c.w; xp3 = edge;
        } else {
            const float edge = __ldg(other + rowbase + (ih == 0 ? half - 1 : ih - 1));
            xm0 = edge; xm1 = c.x; xm2 = c.y; xm3 = c.z;
            xp0 = c.x; xp1 = c.y; xp2 = c.z; xp3 = c.w;
        }
        float4 r;
        r.x = fmaf(((((xm0 + xp0) + ym.x) + yp.x) + zm.x) + zp.x, kSixthF, -b.x);
        r.y = fmaf(((((xm1 + xp1) + ym.y) + yp.y) + zm.y) + zp.y, kSixthF, -b.y);
        r.z = fmaf(((((xm2 + xp2) + ym.z) + yp.z) + zm.z) + zp.z, kSixthF, -b.z);
        r.w = fmaf(((((xm3 + xp3) + ym.w) + yp.w) + zm.w) + zp.w, kSixthF, -b.w);
        m4[t >> 2] = r;
        zm = c;
        c = zp;
    }
}

// The opening red half sweep of an inner solve, whose correction starts at 0:
// every black neighbour is 0, so each red cell gets fmaf(0, 1/6, -beta) -- the
// general sweep's value, without the loads, and without zeroing e beforehand
// (the black half sweep after it reads only the red cells it overwrote).
__global__ void k_gsrb_f_zero(long long cnt, float* __restrict__ mine, const float* __restrict__ beta)
{
    pdl_wait();
    pdl_trigger();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) mine[t] = fmaf(0.f, kSixthF, -beta[t]);
}

__device__ __forceinline__ float resid_f(const LevelViewF& L, int i, int j, int k)
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
    return *lv_ptr<float>(L.beta_r, L.beta_b, n, L.split, i, j, k) - fmaf(s, kSixthF, -c);
}

// RED = 1 after pre-smoothing (it ends with a black half sweep): the red
// children only, as k_restrict_f4_red and the fused coarse V-cycle take them
template <int RED>
__global__ void k_restrict_f(LevelViewF F, LevelViewF Cv)
{
    pdl_wait();
    pdl_trigger();
    const int nc = Cv.n;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= nc || J >= nc) return;
    float s = 0.f;
#pragma unroll
    for (int dk = 0; dk < 2; ++dk)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
            for (int di = 0; di < 2; ++di)
                if (!RED || ((di + dj + dk) & 1) == 0) s += resid_f(F, 2 * I + di, 2 * J + dj, 2 * K + dk);
    *lv_ptr<float>(Cv.beta_r, Cv.beta_b, nc, Cv.split, I, J, K) = s * 0.5f;
    *lv_ptr<float>(Cv.phi_r, Cv.phi_b, nc, Cv.split, I, J, K) = 0.f;
}

// The residual + restriction for a split fine level with half % 4 == 0: two
// coarse cells (four fine cells of each of their four fine rows) per thread.
// In a fine row of parity p = (j + k) & 1 the cells i = 4t .. 4t+3 are, in
// order, colour p at compact 2t, colour 1-p at 2t, colour p at 2t+1, colour
// 1-p at 2t+1: one 8-byte pair per colour array and row.  Every fine residual
// is resid_f's, term for term, and the coarse sums add them in the same
// (dk, dj, di) order.
__device__ __forceinline__ void fine_row_resid(const LevelViewF& F, int j, int k, unsigned t,
                                               float r[4])
{
    const int n = F.n;
    const unsigned half = (unsigned)n >> 1;
    const int p = (j + k) & 1;
    const float* Pp = p ? F.phi_b : F.phi_r;      // colour of even i in this row
    const float* Pq = p ? F.phi_r : F.phi_b;
    const float* Bp = p ? F.beta_b : F.beta_r;
    const float* Bq = p ? F.beta_r : F.beta_b;
    const unsigned c2 = 2 * t;
    auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
    const unsigned r0 = row(j, k);
    const float2 ep = __ldg(reinterpret_cast<const float2*>(Pp + r0 + c2));   // phi(4t), phi(4t+2)
    const float2 eq = __ldg(reinterpret_cast<const float2*>(Pq + r0 + c2));   // phi(4t+1), phi(4t+3)
    const float left = __ldg(Pq + r0 + (c2 == 0 ? half - 1 : c2 - 1));        // phi(4t-1)
    const float right = __ldg(Pp + r0 + (c2 + 2 == half ? 0u : c2 + 2));      // phi(4t+4)
    const float2 bp = __ldg(reinterpret_cast<const float2*>(Bp + r0 + c2));
    const float2 bq = __ldg(reinterpret_cast<const float2*>(Bq + r0 + c2));
    // neighbour rows have the other parity: even i there is colour 1-p
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    const unsigned nr[4] = {row(jm, k), row(jp, k), row(j, km), row(j, kp)};
    float2 ne[4], no[4];   // neighbour rows: values at even i (colour 1-p), odd i (colour p)
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ne[a] = __ldg(reinterpret_cast<const float2*>(Pq + nr[a] + c2));
        no[a] = __ldg(reinterpret_cast<const float2*>(Pp + nr[a] + c2));
    }
    const float self[4] = {ep.x, eq.x, ep.y, eq.y};
    const float xm[4] = {left, ep.x, eq.x, ep.y};
    const float xp[4] = {eq.x, ep.y, eq.y, right};
    const float beta[4] = {bp.x, bq.x, bp.y, bq.y};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const bool even = (c & 1) == 0;
        const int h = c >> 1;
        float s = xm[c] + xp[c];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const float2 v = even ? ne[a] : no[a];
            s += h ? v.y : v.x;
        }
        r[c] = beta[c] - fmaf(s, kSixthF, -self[c]);
    }
}


// The restriction after pre-smoothing: the coarse right-hand side from the red
// children only (the black ones' residuals are round-off), summed in (dk, dj)
// order; half the loads of k_restrict_f4.
__global__ void __launch_bounds__(256) k_restrict_f4_red(LevelViewF F, LevelViewF Cv)
{
    pdl_wait();
    pdl_trigger();
    const int nc = Cv.n;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // coarse cells 2t, 2t+1
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (t >= (unsigned)nc / 2 || J >= nc) return;
    float r[2][2][2];
#pragma unroll
    for (int dk = 0; dk < 2; ++dk)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) fine_row_resid_red(F, 2 * J + dj, 2 * K + dk, t, r[dk][dj]);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        float s = 0.f;
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj) s += r[dk][dj][u];
        const int I = 2 * (int)t + u;
        *lv_ptr<float>(Cv.beta_r, Cv.beta_b, nc, Cv.split, I, J, K) = s * 0.5f;
        *lv_ptr<float>(Cv.phi_r, Cv.phi_b, nc, Cv.split, I, J, K) = 0.f;
    }
}

__global__ void __launch_bounds__(256) k_restrict_f4(LevelViewF F, LevelViewF Cv)
{
    pdl_wait();
    pdl_trigger();
    const int nc = Cv.n;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // coarse cells 2t, 2t+1
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (t >= (unsigned)nc / 2 || J >= nc) return;
    float r[2][2][4];
#pragma unroll
    for (int dk = 0; dk < 2; ++dk)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj) fine_row_resid(F, 2 * J + dj, 2 * K + dk, t, r[dk][dj]);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        float s = 0.f;
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int di = 0; di < 2; ++di) s += r[dk][dj][2 * u + di];
        const int I = 2 * (int)t + u;
        *lv_ptr<float>(Cv.beta_r, Cv.beta_b, nc, Cv.split, I, J, K) = s * 0.5f;
        *lv_ptr<float>(Cv.phi_r, Cv.phi_b, nc, Cv.split, I, J, K) = 0.f;
    }
}

// BLACK = 1 when post-smoothing follows: its first half sweep overwrites the red
// cells unread, so only the black fine cells take the correction (same bits)
template <int BLACK>
__global__ void k_prolong_f(LevelViewF Cv, LevelViewF F)
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
        const int Is[2] = {ih, wrap1(odd ? ih + 1 : ih - 1, nc)};
        float s = 0.f;
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int tt = 0; tt < 2; ++tt)
                    s = fmaf(kProlongWF[tt + 2 * a + 4 * b],
                             *lv_ptr<const float>(Cv.phi_r, Cv.phi_b, nc, Cv.split, Is[tt], Js[a], Ks[b]), s);
        float* p = (((i + j + k) & 1) ? F.phi_b : F.phi_r) + t;
        *p += s;
    }
}

// The same prolongation for a split fine level over a split coarse level with
// half % 4 == 0: four compact columns (eight fine cells of a row) per thread.
// The coarse neighbours of those cells along x are the six coarse cells
// ih0-1 .. ih0+4 of each of the four (J', K') rows; in the split layout the
// even ones are three consecutive values of one colour array and the odd ones
// three of the other, loaded as a pair plus one.  Each fine cell sums its
// eight weighted coarse values in e_prolong's order, so the results are the
// scalar kernel's; the corrections go to two float4 of the fine arrays.
template <int BLACK>
__global__ void __launch_bounds__(256) k_prolong_f4(LevelViewF Cv, LevelViewF F)
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
    const unsigned c2 = 2 * t4;                       // compact index of coarse I = ih0 (even)
    // v[b][a][0..5] = coarse values at I = ih0-1 .. ih0+4 of row (Js[a], Ks[b])
    float v[2][2][6];
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const unsigned row = ((unsigned)Js[a] + (unsigned)nc * (unsigned)Ks[b]) * chalf;
            const bool even_red = ((Js[a] + Ks[b]) & 1) == 0;   // colour of an even I
            const float* ev = even_red ? Cv.phi_r : Cv.phi_b;
            const float* od = even_red ? Cv.phi_b : Cv.phi_r;
            const float2 e01 = __ldg(reinterpret_cast<const float2*>(ev + row + c2));
            const float e2 = __ldg(ev + row + (c2 + 2 == chalf ? 0u : c2 + 2));
            const float2 o01 = __ldg(reinterpret_cast<const float2*>(od + row + c2));
            const float om = __ldg(od + row + (c2 == 0 ? chalf - 1 : c2 - 1));
            v[b][a][0] = om;       // I = ih0 - 1
            v[b][a][1] = e01.x;    // ih0
            v[b][a][2] = o01.x;    // ih0 + 1
            v[b][a][3] = e01.y;    // ih0 + 2
            v[b][a][4] = o01.y;    // ih0 + 3
            v[b][a][5] = e2;       // ih0 + 4
        }
    float s0[4], s1[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float se = 0.f, so = 0.f;   // fine i = 2 ih (tt1: I - 1) and 2 ih + 1 (tt1: I + 1)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                se = fmaf(kProlongWF[0 + 2 * a + 4 * b], v[b][a][r + 1], se);
                se = fmaf(kProlongWF[1 + 2 * a + 4 * b], v[b][a][r], se);
                so = fmaf(kProlongWF[0 + 2 * a + 4 * b], v[b][a][r + 1], so);
                so = fmaf(kProlongWF[1 + 2 * a + 4 * b], v[b][a][r + 2], so);
            }
        s0[r] = se;
        s1[r] = so;
    }
    const unsigned t = ((unsigned)j + (unsigned)n * (unsigned)k) * half + 4 * t4;
    const bool even_fine_red = ((j + k) & 1) == 0;   // colour of fine i = 2 ih
    float4* fe = reinterpret_cast<float4*>(even_fine_red ? F.phi_r : F.phi_b) + (t >> 2);
    float4* fo = reinterpret_cast<float4*>(even_fine_red ? F.phi_b : F.phi_r) + (t >> 2);
    if (!BLACK || !even_fine_red) {
        float4 pe = *fe;
        pe.x += s0[0]; pe.y += s0[1]; pe.z += s0[2]; pe.w += s0[3];
        *fe = pe;
    }
    if (!BLACK || even_fine_red) {
        float4 po = *fo;
        po.x += s1[0]; po.y += s1[1]; po.z += s1[2]; po.w += s1[3];
        *fo = po;
    }
}

// The black-only prolongation (post-smoothing follows) with four fine rows per
// thread (pm_prolong.cuh): nine coarse row segments for four fine rows, the same
// bits as k_prolong_f4<1>.
__global__ void __launch_bounds__(256, 5) k_prolong_f4_black(LevelViewF Cv, LevelViewF F)
{
    pdl_wait();
    pdl_trigger();
    const unsigned h4 = (unsigned)F.n >> 3;
    const unsigned t4 = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (t4 >= h4 || J >= Cv.n) return;
    prolong_black_quad(Cv, F, J, K, t4);
}

__global__ void k_bottom_f(int nb, const float* __restrict__ G, const float* __restrict__ beta, float* phi)
{
    pdl_wait();
    pdl_trigger();
    __shared__ float r[kMaxBottom * kMaxBottom * kMaxBottom];
    __shared__ float g[kMaxBottom * kMaxBottom * kMaxBottom];
    const int nc = nb * nb * nb;
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
        r[t] = beta[t];
        g[t] = G[t];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int i = c % nb, j = (c / nb) % nb, k = c / (nb * nb);
        float s = 0.f;
        int y = 0;
        for (int yk = 0; yk < nb; ++yk) {
            const int dk = wrap1(k - yk, nb) * nb * nb;
            for (int yj = 0; yj < nb; ++yj) {
                const int djk = dk + wrap1(j - yj, nb) * nb;
                for (int yi = 0; yi < nb; ++yi, ++y) s = fmaf(g[djk + wrap1(i - yi, nb)], r[y], s);
            }
        }
        phi[c] = s;
    }
}

// the coarse end of a V-cycle (levels of at most mg_fused_edge cells per edge
// down to the bottom) by one CTA; the arithmetic of the per-pass kernels
struct TailF {
    int nl;                  // levels in the tail; the last is the bottom (natural layout)
    int nu1, nu2, nb;
    const float* Gf;
    LevelViewF lv[kMaxTail];
};

__global__ void __launch_bounds__(kTailThreads) k_vcycle_tail_f(TailF A)
{
    pdl_wait();
    pdl_trigger();
    __shared__ float r[kMaxBottom * kMaxBottom * kMaxBottom];
    __shared__ float g[kMaxBottom * kMaxBottom * kMaxBottom];
    vcycle_tail<float>(A.lv, A.nl, A.nu1, A.nu2, A.Gf, A.nb, r, g, A.nu1 > 0);
}

// FP32 gravity vector from the FP64 phi: the difference in FP64, the scaling in FP32
// (one float4 {gx, gy, gz, 0} per cell: a CIC corner is one 16-byte load)
__global__ void k_mx_grav(LevelView L, float half_dxi, float* g)
{
    const int n = L.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    const long long c = cidx(i, j, k, n);
    auto P = [&](int a, int b, int d) {
        return *lv_ptr<const double>(L.phi_r, L.phi_b, n, L.split, a, b, d);
    };
    const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    reinterpret_cast<float4*>(g)[c] = make_float4(f64_to_f32_rn(P(ip, j, k) - P(im, j, k)) * half_dxi,
                                                  f64_to_f32_rn(P(i, jp, k) - P(i, jm, k)) * half_dxi,
                                                  f64_to_f32_rn(P(i, j, kp) - P(i, j, km)) * half_dxi, 0.f);
}

// a caller's FP64 gravity vector (3 n^3, component-major) as the kicks' float4 per cell
__global__ void k_mx_g32_from_g(long long nc, const double* __restrict__ g, float* g32)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    reinterpret_cast<float4*>(g32)[c] =
        make_float4(f64_to_f32_rn(g[c]), f64_to_f32_rn(g[nc + c]), f64_to_f32_rn(g[2 * nc + c]), 0.f);
}

// ---------------------------------------------------------------------------
// FP32 CIC interpolation + kick (+ drift in cell units with re-binning)
// ---------------------------------------------------------------------------
struct MxKickArgs {
    int n;
    const float* g;
    float half_dt, a_prev, a_cur_inv, drift;  // drift = dt / a_cur / dx (cell units)
    int do_move;
};

__global__ void __launch_bounds__(256, 6) k_mx_kick(long long np, MxKickArgs A, int* cell, float* ox,
                                                 float* oy, float* oz, float* vx, float* vy, float* vz)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int n = A.n;
    const int c = cell[q];
    int ci = cell_i(c), cj = cell_j(c), ck = cell_k(c);
    float o[3] = {ox[q], oy[q], oz[q]};
    float fx, fy, fz;
    const int i = key_frac(ci, o[0], n, &fx);
    const int j = key_frac(cj, o[1], n, &fy);
    const int k = key_frac(ck, o[2], n, &fz);
    const float sx[2] = {1.f - fx, fx};
    const float sy[2] = {1.f - fy, fy};
    const float sz[2] = {1.f - fz, fz};
    float w[8];
    // 32-bit cell offsets (n <= 1024): the eight corners are a row pair, a plane
    // pair and a column pair around (i, j, k)
    const unsigned xs[2] = {(unsigned)i, (unsigned)wrap1(i - 1, n)};
    const unsigned ys[2] = {(unsigned)j * (unsigned)n, (unsigned)wrap1(j - 1, n) * (unsigned)n};
    const unsigned nn = (unsigned)n * (unsigned)n;
    const unsigned zs[2] = {(unsigned)k * nn, (unsigned)wrap1(k - 1, n) * nn};
    unsigned cc[8];
#pragma unroll
    for (int kk = 0; kk <= 1; ++kk)
#pragma unroll
        for (int jj = 0; jj <= 1; ++jj)
#pragma unroll
            for (int ii = 0; ii <= 1; ++ii) {
                const int t = ii + 2 * jj + 4 * kk;
                w[t] = (sx[1 - ii] * sy[1 - jj]) * sz[1 - kk];
                cc[t] = xs[ii] + ys[jj] + zs[kk];
            }
    float v[3] = {vx[q], vy[q], vz[q]};
    float val[3] = {0.f, 0.f, 0.f};
    const float4* g4 = reinterpret_cast<const float4*>(A.g);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const float4 gc = __ldg(g4 + cc[t]);
        val[0] = fmaf(w[t], gc.x, val[0]);
        val[1] = fmaf(w[t], gc.y, val[1]);
        val[2] = fmaf(w[t], gc.z, val[2]);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = fmaf(A.a_prev, v[d], A.half_dt * val[d]) * A.a_cur_inv;
    vx[q] = v[0];
    vy[q] = v[1];
    vz[q] = v[2];
    if (A.do_move) {
        int ic[3] = {ci, cj, ck};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float p = fmaf(A.drift, v[d], o[d]);
            float fl = floorf(p);
            p -= fl;
            if (p >= 1.f) {  // -tiny + 1 rounded up to 1: the particle sits at the next cell's origin
                p = 0.f;
                fl += 1.f;
            }
            int idx = ic[d] + (int)fl;
            if (idx >= n) idx -= n;       // a move of less than n cells: one step
            else if (idx < 0) idx += n;
            if ((unsigned)idx >= (unsigned)n) {   // further: the general wrap
                idx %= n;
                if (idx < 0) idx += n;
            }
            ic[d] = idx;
            o[d] = p;
        }
        cell[q] = pack_cell(ic[0], ic[1], ic[2]);
        ox[q] = o[0];
        oy[q] = o[1];
        oz[q] = o[2];
    }
}

inline unsigned norm_blocks(Ctx& c, long long cnt)
{
    long long b = (cnt + kThreads - 1) / kThreads;
    long long cap = (long long)c.sm_count * 8;
    return (unsigned)std::max<long long>(1, std::min(b, cap));
}

double read_norm(Box& b, int slot)
{
    double v;
    std::memcpy(&v, &b.h_norms[slot], sizeof(v));
    return v;
}

// zero_start: the level's correction is 0 on entry (an inner solve's first sweep
// on level 0): the red half sweep is k_gsrb_f_zero
nyxpm_status gsrb_sweep_f(Ctx& c, const Level& l, int fine, bool zero_start = false)
{
    const long long half_cells = (long long)l.n * l.n * l.n / 2;
    const int half = l.n / 2;
    const bool vec = half % 4 == 0;   // then n % 8 == 0, a whole number of kMarchZ planes
    // marching pays on the large levels; below, more threads hide more latency
    const bool march = vec && l.n >= kMarchMinEdge;
    Geo g;
    if (vec) {
        g = geo3(half / 4, l.n, 1);
        g.grid.z = march ? (l.n + kMarchZ - 1) / kMarchZ : l.n;
    } else {
        g = geo3(half, l.n, l.n);
    }
    for (int color = 0; color < 2; ++color) {
        float* mine = color ? l.fphi_b : l.fphi_r;
        const float* other = color ? l.fphi_r : l.fphi_b;
        const float* beta = color ? l.fbeta_b : l.fbeta_r;
        prof_begin(c);
        if (zero_start && color == 0)
            launch_pdl(c, k_gsrb_f_zero, dim3(blocks_for(half_cells)), dim3(kThreads), half_cells, mine, beta);
        else if (march)
            launch_pdl(c, k_gsrb_f4<kMarchZ>, dim3(g.grid), dim3(g.block), l.n, color, mine, other, beta);
        else if (vec)
            launch_pdl(c, k_gsrb_f4<1>, dim3(g.grid), dim3(g.block), l.n, color, mine, other, beta);
        else
            launch_pdl(c, k_gsrb_f, dim3(g.grid), dim3(g.block), l.n, color, mine, other, beta);
        prof_end(c, NYXPM_ST_SMOOTH, 12.0 * half_cells, fine);
    }
    return check_launch(c, "gsrb f32");
}

// levels li .. last in one k_vcycle_tail_f launch
nyxpm_status vcycle_tail_f(Ctx& c, Box& b, size_t li)
{
    TailF A;
    A.nl = (int)(b.levels.size() - li);
    A.nu1 = c.p.nu1;
    A.nu2 = c.p.nu2;
    A.nb = b.nb;
    A.Gf = b.Gf;
    double bytes = 0;
    for (int l = 0; l < A.nl; ++l) {
        const Level& lv = b.levels[li + l];
        A.lv[l] = viewf(lv);
        const double cells = (double)lv.n * lv.n * lv.n;
        bytes += (l + 1 < A.nl) ? 6.0 * cells * 2 * (c.p.nu1 + c.p.nu2) + 16.0 * cells : 8.0 * cells;
    }
    prof_begin(c);
    launch_pdl(c, k_vcycle_tail_f, dim3(1), dim3(kTailThreads), A);
    prof_end(c, NYXPM_ST_SMOOTH, bytes);
    return check_launch(c, "fused coarse V-cycle f32");
}

bool tail_fits(const Ctx& c, const Box& b, size_t li)
{
    return c.p.mg_fused_edge > 0 && b.levels[li].n <= c.p.mg_fused_edge &&
           b.levels.size() - li <= (size_t)kMaxTail;
}

// fresh: level li's correction is 0 on entry without having been zeroed (the
// first inner V-cycle of a defect-correction step)
nyxpm_status vcycle_f(Ctx& c, Box& b, size_t li, bool fresh = false)
{
    nyxpm_status st;
    const Level& f = b.levels[li];
    if (fresh && (tail_fits(c, b, li) || !f.split)) {
        // the fused tail and the bottom read the level as it is: zero it (a few
        // thousand cells at most)
        const size_t cnt = (size_t)f.n * f.n * f.n;
        if (f.split) {
            cudaMemsetAsync(f.fphi_r, 0, cnt / 2 * sizeof(float), c.stream);
            cudaMemsetAsync(f.fphi_b, 0, cnt / 2 * sizeof(float), c.stream);
        } else {
            cudaMemsetAsync(f.fphi_r, 0, cnt * sizeof(float), c.stream);
        }
        fresh = false;
    }
    if (tail_fits(c, b, li)) return vcycle_tail_f(c, b, li);
    if (li + 1 == b.levels.size()) {
        prof_begin(c);
        launch_pdl(c, k_bottom_f, dim3(1), dim3(512), b.nb, b.Gf, f.fbeta_r, f.fphi_r);
        prof_end(c, NYXPM_ST_BOTTOM, 8.0 * f.n * f.n * f.n);
        return check_launch(c, "bottom f32");
    }
    if (fresh && c.p.nu1 == 0) {
        const size_t half_bytes = (size_t)f.n * f.n * f.n / 2 * sizeof(float);
        cudaMemsetAsync(f.fphi_r, 0, half_bytes, c.stream);
        cudaMemsetAsync(f.fphi_b, 0, half_bytes, c.stream);
    }
    for (int s = 0; s < c.p.nu1; ++s)
        if ((st = gsrb_sweep_f(c, f, li == 0, fresh && s == 0)) != NYXPM_OK) return st;
    const Level& cl = b.levels[li + 1];
    const long long ncc = (long long)cl.n * cl.n * cl.n;
    const long long ncf = (long long)f.n * f.n * f.n;
    {
        prof_begin(c);
        if ((f.n / 2) % 4 == 0) {
            const Geo g = geo3(cl.n / 2, cl.n, cl.n);
            if (c.p.nu1 > 0) launch_pdl(c, k_restrict_f4_red, dim3(g.grid), dim3(g.block), viewf(f), viewf(cl));
            else launch_pdl(c, k_restrict_f4, dim3(g.grid), dim3(g.block), viewf(f), viewf(cl));
        } else {
            const Geo g = geo3(cl.n, cl.n, cl.n);
            if (c.p.nu1 > 0) launch_pdl(c, k_restrict_f<1>, dim3(g.grid), dim3(g.block), viewf(f), viewf(cl));
            else launch_pdl(c, k_restrict_f<0>, dim3(g.grid), dim3(g.block), viewf(f), viewf(cl));
        }
        // phi and beta read once, coarse beta and phi written; the red-only form reads
        // the black cells' beta not at all
        const bool red = c.p.nu1 > 0;
        prof_end(c, NYXPM_ST_RESTRICT, (red ? 6.0 : 8.0) * ncf + 8.0 * ncc);
    }
    if ((st = check_launch(c, "restrict f32")) != NYXPM_OK) return st;
    if ((st = vcycle_f(c, b, li + 1)) != NYXPM_OK) return st;
    {
        prof_begin(c);
        const bool black = c.p.nu2 > 0;
        if (cl.split && (f.n / 2) % 4 == 0 && black) {
            const Geo g = geo3(f.n / 8, cl.n, cl.n);
            launch_pdl(c, k_prolong_f4_black, dim3(g.grid), dim3(g.block), viewf(cl), viewf(f));
        } else if (cl.split && (f.n / 2) % 4 == 0) {
            const Geo g = geo3(f.n / 8, f.n, f.n);
            launch_pdl(c, k_prolong_f4<0>, dim3(g.grid), dim3(g.block), viewf(cl), viewf(f));
        } else {
            const Geo g = geo3(f.n / 2, f.n, f.n);
            if (black) launch_pdl(c, k_prolong_f<1>, dim3(g.grid), dim3(g.block), viewf(cl), viewf(f));
            else launch_pdl(c, k_prolong_f<0>, dim3(g.grid), dim3(g.block), viewf(cl), viewf(f));
        }
        // the fine corrections read and written (black cells only when post-smoothing
        // follows), the coarse level read once
        prof_end(c, NYXPM_ST_PROLONG, (black ? 4.0 : 8.0) * ncf + 4.0 * ncc);
    }
    if ((st = check_launch(c, "prolong f32")) != NYXPM_OK) return st;
    for (int s = 0; s < c.p.nu2; ++s)
        if ((st = gsrb_sweep_f(c, f, li == 0)) != NYXPM_OK) return st;
    return NYXPM_OK;
}

// FP64 residual of level 0 into the FP32 inner right-hand side, its norm into norms[1]
nyxpm_status launch_mx_resid(Ctx& c, Box& b, bool low_words)
{
    const Level& l = b.levels[0];
    const long long nc = (long long)l.n * l.n * l.n;
    float* rl_r = (low_words && l.split) ? b.r_lo : nullptr;
    float* rl_b = rl_r ? b.r_lo + nc / 2 : nullptr;
    prof_begin(c);
    cudaMemsetAsync(b.norms + 1, 0, sizeof(unsigned long long), c.stream);
    if (l.split) {
        const Geo g = geo3(l.n / 2, l.n, l.n);
        if ((l.n / 2) % 2 == 0) {
            const Geo g2 = geo3(l.n / 4, l.n, l.n);
            k_mx_resid2<<<g2.grid, g2.block, 0, c.stream>>>(l.n, l.phi_r, l.phi_b, l.beta_r,
                                                            l.beta_b, l.fbeta_r, l.fbeta_b, rl_r,
                                                            rl_b, b.norms + 1);
        } else {
            k_mx_resid<<<g.grid, g.block, 0, c.stream>>>(l.n, l.phi_r, l.phi_b, l.beta_r, l.beta_b,
                                                         l.fbeta_r, l.fbeta_b, rl_r, rl_b,
                                                         b.norms + 1);
        }
    } else {
        const Geo g = geo3(l.n, l.n, l.n);
        k_mx_resid_nat<<<g.grid, g.block, 0, c.stream>>>(l.n, l.phi_r, l.beta_r, l.fbeta_r,
                                                         b.norms + 1);
    }
    prof_end(c, NYXPM_ST_NORM, 20.0 * nc);
    return check_launch(c, "mixed residual");
}

// phi += e and the double-float residual update of a split level 0 (k_mx_correct)
nyxpm_status launch_mx_correct(Ctx& c, Box& b)
{
    const Level& l = b.levels[0];
    const long long nc = (long long)l.n * l.n * l.n;
    const float c_hi = (float)(1.0 / 6.0);
    const float c_lo = (float)(1.0 / 6.0 - (double)c_hi);
    prof_begin(c);
    cudaMemsetAsync(b.norms + 1, 0, sizeof(unsigned long long), c.stream);
    cudaMemsetAsync(b.norms + 4, 0, sizeof(unsigned long long), c.stream);
    if ((l.n / 2) % 2 == 0) {
        const Geo g = geo3(l.n / 4, l.n, l.n);
        k_mx_correct2<<<g.grid, g.block, 0, c.stream>>>(l.n, c_hi, c_lo, l.fphi_r, l.fphi_b,
                                                        l.phi_r, l.phi_b, l.fbeta_r, l.fbeta_b,
                                                        b.r_lo, b.r_lo + nc / 2, b.norms + 1,
                                                        b.norms + 4);
    } else {
        const Geo g = geo3(l.n / 2, l.n, l.n);
        k_mx_correct<<<g.grid, g.block, 0, c.stream>>>(l.n, c_hi, c_lo, l.fphi_r, l.fphi_b,
                                                       l.phi_r, l.phi_b, l.fbeta_r, l.fbeta_b,
                                                       b.r_lo, b.r_lo + nc / 2, b.norms + 1,
                                                       b.norms + 4);
    }
    prof_end(c, NYXPM_ST_NORM, 36.0 * nc);
    return check_launch(c, "mixed correction");
}

nyxpm_status launch_mx_split_beta(Ctx& c, Box& b)
{
    const Level& l = b.levels[0];
    const long long half_cells = (long long)l.n * l.n * l.n / 2;
    prof_begin(c);
    k_mx_split_beta<<<blocks_for(half_cells), kThreads, 0, c.stream>>>(
        half_cells, l.beta_r, l.beta_b, l.fbeta_r, l.fbeta_b, b.r_lo, b.r_lo + half_cells);
    prof_end(c, NYXPM_ST_NORM, 32.0 * half_cells);
    return check_launch(c, "mixed split beta");
}

nyxpm_status launch_mx_update(Ctx& c, Box& b)
{
    const Level& l = b.levels[0];
    const long long nc = (long long)l.n * l.n * l.n;
    prof_begin(c);
    if (l.split) {
        k_mx_update<<<blocks_for(nc / 2), kThreads, 0, c.stream>>>(nc / 2, l.phi_r, l.fphi_r);
        k_mx_update<<<blocks_for(nc / 2), kThreads, 0, c.stream>>>(nc / 2, l.phi_b, l.fphi_b);
        c.launches += 1;
    } else {
        k_mx_update<<<blocks_for(nc), kThreads, 0, c.stream>>>(nc, l.phi_r, l.fphi_r);
    }
    prof_end(c, NYXPM_ST_PROLONG, 20.0 * nc);
    return check_launch(c, "mixed update");
}

// particle time-step limit of the mixed form: the same formula as the FP64
// form (NyxParticleContainer.H:329-465), from the FP32 velocities and the FP32
// gravity vector the kicks use, evaluated in FP64; the cell is the particle's
// stored cell (floor(x*dxi)).  out must start at 0 (complemented-bits max).
__global__ void __launch_bounds__(256) k_mx_est_dt(long long np, int n, double dxi, double adxi,
                                                   double cfl, const int* __restrict__ cell,
                                                   const float* __restrict__ vx,
                                                   const float* __restrict__ vy,
                                                   const float* __restrict__ vz,
                                                   const float* __restrict__ g,
                                                   unsigned long long* out)
{
    double best = 1.0e50;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < np;
         q += (long long)gridDim.x * blockDim.x) {
        const int cq = cell[q];
        const double ux = fabs((double)vx[q]) * adxi, uy = fabs((double)vy[q]) * adxi,
                     uz = fabs((double)vz[q]) * adxi;
        const double um = fmax(fmax(ux, uy), uz);
        double dtp = um > 0 ? cfl / um : 1.0e50;
        const long long c = cidx(cell_i(cq), cell_j(cq), cell_k(cq), n);
        const float4 gc = __ldg(reinterpret_cast<const float4*>(g) + c);
        const double gx = gc.x, gy = gc.y, gz = gc.z;
        const double ga = sqrt((gx * gx + gy * gy) + gz * gz);
        if (ga > 0) dtp = fmin(dtp, 1.0 / sqrt(ga * dxi));
        best = fmin(best, dtp);
    }
    block_umax_store(~(unsigned long long)__double_as_longlong(best), out);
}

}  // namespace

nyxpm_status mixed_unpack(Ctx& c, Box& b, const double* d_pos, const double* d_vel,
                          const double* d_mass)
{
    prof_begin(c);
    k_mx_unpack<<<blocks_for(b.np), kThreads, 0, c.stream>>>(
        b.np, b.n, b.dxi, d_pos, d_vel, d_mass, b.cell, b.ox, b.oy, b.oz, b.fvx, b.fvy, b.fvz,
        d_mass ? b.fm : nullptr, b.id, b.norms + 2);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "mixed unpack");
}

nyxpm_status mixed_unpack_pos(Ctx& c, Box& b, const double* d_pos, const double* d_mass)
{
    prof_begin(c);
    k_mx_unpack_pos<<<blocks_for(b.np), kThreads, 0, c.stream>>>(
        b.np, b.n, b.dxi, d_pos, d_mass, b.cell, b.ox, b.oy, b.oz, d_mass ? b.fm : nullptr, b.id,
        b.norms + 2);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "mixed unpack positions");
}

nyxpm_status mixed_unpack_vel(Ctx& c, Box& b, const double* d_vel, bool sorted_since)
{
    prof_begin(c);
    k_mx_unpack_vel<<<blocks_for(b.np), kThreads, 0, c.stream>>>(
        b.np, d_vel, sorted_since ? b.perm : nullptr, b.fvx, b.fvy, b.fvz, b.norms + 2);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "mixed unpack velocities");
}

nyxpm_status mixed_pack_pos(Ctx& c, Box& b, double* d_pos)
{
    prof_begin(c);
    k_mx_pack_pos<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.dx, b.cell, b.ox, b.oy, b.oz,
                                                                b.id, d_pos);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "mixed pack positions");
}

nyxpm_status mixed_pack_vel(Ctx& c, Box& b, double* d_vel)
{
    prof_begin(c);
    k_mx_pack_vel<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.fvx, b.fvy, b.fvz, b.id, d_vel);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "mixed pack velocities");
}

nyxpm_status mixed_pack(Ctx& c, Box& b, double* d_pos, double* d_vel)
{
    prof_begin(c);
    k_mx_pack<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.dx, b.cell, b.ox, b.oy, b.oz,
                                                            b.fvx, b.fvy, b.fvz, b.id, d_pos, d_vel);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "mixed pack");
}

nyxpm_status mixed_sort(Ctx& c, Box& b, bool defer_vel)
{
    nyxpm_status st;
    cudaMemsetAsync(b.cell_count, 0, sizeof(int) * (size_t)b.n * b.n * b.n, c.stream);
    prof_begin(c);
    k_mx_keys<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.n, b.cell, b.ox, b.oy, b.oz,
                                                            b.key, b.cell_count);
    prof_end(c, NYXPM_ST_KEYS, 20.0 * b.np);
    if ((st = check_launch(c, "mixed keys")) != NYXPM_OK) return st;
    if ((st = sort_from_keys(c, b)) != NYXPM_OK) return st;
    const bool pm = !b.uniform_mass;
    prof_begin(c);
    k_mx_gather<<<blocks_for(b.np), kThreads, 0, c.stream>>>(
        b.np, b.perm, b.cell, b.ox, b.oy, b.oz, defer_vel ? nullptr : b.fvx, b.fvy, b.fvz,
        pm ? b.fm : nullptr, b.id, b.cell2, b.ox2, b.oy2, b.oz2, b.fvx2, b.fvy2, b.fvz2,
        pm ? b.fm2 : nullptr, b.id2);
    prof_end(c, NYXPM_ST_GATHER, ((pm ? 76.0 : 68.0) - (defer_vel ? 24.0 : 0.0)) * b.np);
    if ((st = check_launch(c, "mixed gather")) != NYXPM_OK) return st;
    std::swap(b.cell, b.cell2);
    std::swap(b.ox, b.ox2);
    std::swap(b.oy, b.oy2);
    std::swap(b.oz, b.oz2);
    if (!defer_vel) {
        std::swap(b.fvx, b.fvx2);
        std::swap(b.fvy, b.fvy2);
        std::swap(b.fvz, b.fvz2);
    }
    std::swap(b.fm, b.fm2);
    std::swap(b.id, b.id2);
    b.sorted = 1;
    return NYXPM_OK;
}

nyxpm_status mixed_deposit(Ctx& c, Box& b)
{
    const int n = b.n;
    dim3 grid((n + kDepTx - 1) / kDepTx, (n + kDepTy - 1) / kDepTy, (n + kDepTz - 1) / kDepTz);
    const double dx = b.L / n;
    const double inv_vol = 1.0 / (dx * dx * dx);
    const float scale = (float)(b.uniform_mass ? b.mscalar * inv_vol : inv_vol);
    const double nc = (double)n * n * n;
    const float* mq = b.uniform_mass ? nullptr : b.fm;
    // the FP32 partials of long keys live in the box's heavy-key array (8 floats
    // in the room of 8 doubles per slot)
    float* heavy = reinterpret_cast<float*>(b.heavy_part);
    prof_begin(c);
    k_mx_deposit_heavy<<<c.sm_count * 4, 256, 0, c.stream>>>(n, b.cell, b.ox, b.oy, b.oz, mq,
                                                             b.cell_start, b.long_list, b.long_count,
                                                             b.key_slot, heavy);
    k_mx_deposit<<<grid, kDepThreads, 0, c.stream>>>(n, scale, b.cell, b.ox, b.oy, b.oz, mq,
                                                     b.cell_start, b.key_slot, heavy, b.frho);
    c.launches += 1;
    prof_end(c, NYXPM_ST_DEPOSIT, (b.uniform_mass ? 16.0 : 20.0) * b.np + 8.0 * nc);
    return check_launch(c, "mixed deposit");
}

nyxpm_status mixed_rho_to_double(Ctx& c, Box& b)
{
    const long long nc = (long long)b.n * b.n * b.n;
    k_f2d<<<blocks_for(nc), kThreads, 0, c.stream>>>(nc, b.frho, b.rho);
    c.launches += 1;
    return check_launch(c, "rho to double");
}

nyxpm_status mixed_make_rhs(Ctx& c, Box& b, double a)
{
    const int n = b.n;
    const long long nc = (long long)n * n * n;
    const Level& l0 = b.levels[0];
    const double dx = b.L / n;
    const Geo g = geo3(n, n, n);
    prof_begin(c);
    k_mx_rowsum<<<blocks_for((long long)n * n * 32), kThreads, 0, c.stream>>>(n, b.frho,
                                                                             b.mass_offset, b.rows);
    k_mx_mean<<<1, 1024, 0, c.stream>>>(n, dx, b.L, b.rows, b.scal);
    const double scale = ((-4.0 * M_PI * c.p.gconst) * (1.0 / a)) * beta_scale(b);
    k_mx_make_beta<<<g.grid, g.block, 0, c.stream>>>(n, l0.split, b.frho, b.mass_offset, b.scal,
                                                     scale, l0.beta_r, l0.beta_b);
    prof_end(c, NYXPM_ST_RHS, 20.0 * nc);
    c.launches += 2;
    return check_launch(c, "mixed rhs");
}

nyxpm_status mixed_grav32(Ctx& c, Box& b)
{
    const long long nc = (long long)b.n * b.n * b.n;
    const Geo g = geo3(b.n, b.n, b.n);
    prof_begin(c);
    k_mx_grav<<<g.grid, g.block, 0, c.stream>>>(view(b.levels[0]), (float)(0.5 * b.dxi), b.g32);
    prof_end(c, NYXPM_ST_KICK, 20.0 * nc);
    return check_launch(c, "mixed grav");
}

nyxpm_status mixed_g32_from_g(Ctx& c, Box& b)
{
    const long long nc = (long long)b.n * b.n * b.n;
    prof_begin(c);
    k_mx_g32_from_g<<<blocks_for(nc), kThreads, 0, c.stream>>>(nc, b.g, b.g32);
    prof_end(c, NYXPM_ST_KICK, 40.0 * nc);
    return check_launch(c, "mixed caller gravity");
}

nyxpm_status mixed_solve(Ctx& c, Box& b, int zero_guess, nyxpm_solve_info* info)
{
    nyxpm_status st;
    const Level& l0 = b.levels[0];
    const long long nc = (long long)l0.n * l0.n * l0.n;
    // A split level 0 keeps its residual as a double-float pair (r_hi, the FP32
    // inner right-hand side, and r_lo) and updates it from each correction
    // (k_mx_correct) instead of applying the FP64 stencil to phi.
    const bool incremental = l0.split != 0;
    prof_begin(c);
    cudaMemsetAsync(b.norms, 0, sizeof(unsigned long long), c.stream);
    if (l0.split) {
        k_mx_absmax<<<norm_blocks(c, nc / 2), kThreads, 0, c.stream>>>(nc / 2, l0.beta_r, b.norms);
        k_mx_absmax<<<norm_blocks(c, nc / 2), kThreads, 0, c.stream>>>(nc / 2, l0.beta_b, b.norms);
        c.launches += 1;
    } else {
        k_mx_absmax<<<norm_blocks(c, nc), kThreads, 0, c.stream>>>(nc, l0.beta_r, b.norms);
    }
    prof_end(c, NYXPM_ST_NORM, 8.0 * nc);
    if ((st = check_launch(c, "mixed rhs norm")) != NYXPM_OK) return st;
    if (zero_guess && incremental) {
        // r0 = beta exactly: its two words, no stencil
        if ((st = launch_mx_split_beta(c, b)) != NYXPM_OK) return st;
        cudaMemcpyAsync(b.h_norms, b.norms, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        c.stream);
    } else {
        if ((st = launch_mx_resid(c, b, incremental)) != NYXPM_OK) return st;
        cudaMemcpyAsync(b.h_norms, b.norms, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        c.stream);
    }
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return check_launch(c, "mixed sync");
    const double bnorm = read_norm(b, 0);
    const double r0 = (zero_guess && incremental) ? bnorm : read_norm(b, 1);
    const double target = c.p.rel_tol * std::max(bnorm, r0);
    double r = r0;
    double err = 0.0;   // bound on |tracked residual - residual of phi|
    int it = 0, inner = 0;
    nyxpm_status result = NYXPM_OK;
    if (!(r0 <= target)) {
        auto iteration = [&]() -> nyxpm_status {
            // inner FP32 solve of L e = r from e = 0, phi += e, the new residual
            nyxpm_status s;
            // e starts at 0: the first V-cycle's opening sweep does not read it
            for (int v = 0; v < c.p.mixed_inner_vcycles; ++v)
                if ((s = vcycle_f(c, b, 0, v == 0)) != NYXPM_OK) return s;
            if (incremental) {
                if ((s = launch_mx_correct(c, b)) != NYXPM_OK) return s;
                cudaMemcpyAsync(b.h_norms + 4, b.norms + 4, sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, c.stream);
            } else {
                if ((s = launch_mx_update(c, b)) != NYXPM_OK) return s;
                if ((s = launch_mx_resid(c, b, false)) != NYXPM_OK) return s;
            }
            cudaMemcpyAsync(b.h_norms + 1, b.norms + 1, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, c.stream);
            return check_launch(c, "norm copy");
        };
        for (it = 1; it <= c.p.max_vcycles; ++it) {
            if ((st = run_iteration(c, b.iter_graph[0], iteration)) != NYXPM_OK) return st;
            inner += c.p.mixed_inner_vcycles;
            if (cudaStreamSynchronize(c.stream) != cudaSuccess) return check_launch(c, "mixed sync");
            r = read_norm(b, 1);
            if (incremental) {
                err += kDfUpdateErr * read_norm(b, 4);
                if (err > 0.5 * target && r == r) {
                    // the bound could hide the tolerance: recompute r from phi with
                    // the FP64 stencil (a zero-guess solve's first correction is as
                    // large as phi, so it always lands here once)
                    if ((st = launch_mx_resid(c, b, true)) != NYXPM_OK) return st;
                    cudaMemcpyAsync(b.h_norms + 1, b.norms + 1, sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, c.stream);
                    if (cudaStreamSynchronize(c.stream) != cudaSuccess)
                        return check_launch(c, "mixed sync");
                    r = read_norm(b, 1);
                    err = 0.0;
                }
            }
            if (r != r) {
                c.err = "mixed defect correction residual is NaN";
                return NYXPM_NOT_CONVERGED;
            }
            if (r + err <= target) break;
        }
        if (it > c.p.max_vcycles) {
            it = c.p.max_vcycles;
            result = NYXPM_NOT_CONVERGED;
            c.err = "defect correction reached max_vcycles above tolerance";
        }
    }
    b.have_phi = 1;
    if ((st = mixed_grav32(c, b)) != NYXPM_OK) return st;
    if (info) {
        const double inv_k0 = 1.0 / beta_scale(b);
        info->vcycles = it;
        info->inner_vcycles = inner;
        info->resnorm0 = r0 * inv_k0;
        info->resnorm = (r + err) * inv_k0;   // a bound on the residual of phi
        info->bnorm = bnorm * inv_k0;
    }
    return result;
}

nyxpm_status mixed_kick(Ctx& c, Box& b, double dt, double a_prev, double a_cur, int do_move)
{
    MxKickArgs A;
    A.n = b.n;
    A.g = b.g32;
    A.half_dt = (float)(0.5 * dt);
    A.a_prev = (float)a_prev;
    A.a_cur_inv = (float)(1.0 / a_cur);
    A.drift = (float)(dt / a_cur * b.dxi);
    A.do_move = do_move;
    prof_begin(c);
    k_mx_kick<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, A, b.cell, b.ox, b.oy, b.oz, b.fvx,
                                                            b.fvy, b.fvz);
    const double nc = (double)b.n * b.n * b.n;
    prof_end(c, NYXPM_ST_KICK, (do_move ? 56.0 : 40.0) * b.np + 12.0 * nc);
    if (do_move) b.sorted = 0;
    return check_launch(c, "mixed kick");
}

nyxpm_status mixed_est_dt(Ctx& c, Box& b, double cfl, double a)
{
    cudaMemsetAsync(b.norms + 3, 0, sizeof(unsigned long long), c.stream);
    const unsigned blocks = std::min(blocks_for(b.np), (unsigned)(c.sm_count * 8));
    k_mx_est_dt<<<blocks, kThreads, 0, c.stream>>>(b.np, b.n, b.dxi, b.dxi / a, cfl, b.cell, b.fvx,
                                                    b.fvy, b.fvz, b.g32, b.norms + 3);
    c.launches += 1;
    return check_launch(c, "mixed time-step estimate");
}

}  // namespace nyxpm
