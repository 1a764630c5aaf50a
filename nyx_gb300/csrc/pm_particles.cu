// Particle kernels of the FP64 PM step: upload/download, periodic wrap, the
// per-step counting sort by deposit cell, the atomic-free CIC deposit and the
// CIC interpolation + kick(-drift) (+ periodic wrap).
//
// Built with --fmad=false: every FP64 expression rounds exactly as written, in
// the order written, with explicit fma() only where the CPU oracle uses fma()
// too -- the arithmetic of update_dm_particle_single
// (Source/Particle/DarkMatterParticleContainer.cpp:250-306) and of the CIC
// weights (Source/Particle/NeutrinoParticles_K.H:15-45).  GB300 runs FP64 at a
// small fraction of its FP32 rate, so every FP64 instruction saved counts.
#include "pm_common.cuh"

#include <algorithm>
#include <cstdio>

namespace nyxpm {

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(long long n, int t = kThreads)
{
    long long b = (n + t - 1) / t;
    return (unsigned)(b < 1 ? 1 : b);
}

// deposit key along one axis: floor(x*dxi + 1/2) (product and sum fused)
// wrapped into [0, n)
__device__ __forceinline__ int key1(double x, double dxi, int n, double* frac)
{
    const double l = fma(x, dxi, 0.5);
    int il;
    const double fl = floor_int(l, &il);
    *frac = l - fl;
    return wrapi(il, n);
}

// ---------------------------------------------------------------------------
// upload / download (AoS host layout <-> SoA device layout)
// ---------------------------------------------------------------------------
__global__ void k_unpack(long long np, const double* __restrict__ pos, const double* __restrict__ vel,
                         const double* __restrict__ mass, double* x, double* y, double* z, double* vx,
                         double* vy, double* vz, double* m, int* id, unsigned long long* bad)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) ok = ok && isfinite(pos[3 * q + d]) && isfinite(vel[3 * q + d]);
    if (!ok) atomicAdd(bad, 1ULL);
    x[q] = pos[3 * q];
    y[q] = pos[3 * q + 1];
    z[q] = pos[3 * q + 2];
    vx[q] = vel[3 * q];
    vy[q] = vel[3 * q + 1];
    vz[q] = vel[3 * q + 2];
    if (m) m[q] = mass[q];
    id[q] = (int)q;
}

__global__ void k_pack(long long np, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ z, const double* __restrict__ vx,
                       const double* __restrict__ vy, const double* __restrict__ vz,
                       const int* __restrict__ id, double* pos, double* vel)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const long long o = 3LL * id[q];
    pos[o] = x[q];
    pos[o + 1] = y[q];
    pos[o + 2] = z[q];
    vel[o] = vx[q];
    vel[o + 1] = vy[q];
    vel[o + 2] = vz[q];
}


// The host-buffer step's split upload and download (nyxpm_step_host): positions
// (and masses) first, velocities later; positions out as soon as the drift made
// them final, already wrapped as the step's closing kick wraps them.
__global__ void k_unpack_pos(long long np, const double* __restrict__ pos,
                             const double* __restrict__ mass, double* x, double* y, double* z,
                             double* m, int* id, unsigned long long* bad)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const double px = pos[3 * q], py = pos[3 * q + 1], pz = pos[3 * q + 2];
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) atomicAdd(bad, 1ULL);
    x[q] = px;
    y[q] = py;
    z[q] = pz;
    if (m) m[q] = mass[q];
    id[q] = (int)q;
}

__global__ void k_unpack_vel(long long np, const double* __restrict__ vel, double* vx, double* vy,
                             double* vz, unsigned long long* bad)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const double ux = vel[3 * q], uy = vel[3 * q + 1], uz = vel[3 * q + 2];
    if (!(isfinite(ux) && isfinite(uy) && isfinite(uz))) atomicAdd(bad, 1ULL);
    vx[q] = ux;
    vy[q] = uy;
    vz[q] = uz;
}

__global__ void k_pack_pos_wrapped(long long np, double L, const double* __restrict__ x,
                                   const double* __restrict__ y, const double* __restrict__ z,
                                   const int* __restrict__ id, double* pos)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const long long o = 3LL * id[q];
    pos[o] = wrap_pos(x[q], L);
    pos[o + 1] = wrap_pos(y[q], L);
    pos[o + 2] = wrap_pos(z[q], L);
}

__global__ void k_pack_vel(long long np, const double* __restrict__ vx, const double* __restrict__ vy,
                           const double* __restrict__ vz, const int* __restrict__ id, double* vel)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const long long o = 3LL * id[q];
    vel[o] = vx[q];
    vel[o + 1] = vy[q];
    vel[o + 2] = vz[q];
}

// velocities permuted by the sort's perm (the position part of the sort ran
// without them)
__global__ void k_gather_vel(long long np, const int* __restrict__ perm,
                             const double* __restrict__ vx, const double* __restrict__ vy,
                             const double* __restrict__ vz, double* vx2, double* vy2, double* vz2)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    const int q = perm[s];
    vx2[s] = vx[q];
    vy2[s] = vy[q];
    vz2[s] = vz[q];
}

__global__ void k_wrap(long long np, double L, double* x, double* y, double* z)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    x[q] = wrap_pos(x[q], L);
    y[q] = wrap_pos(y[q], L);
    z[q] = wrap_pos(z[q], L);
}

// ---------------------------------------------------------------------------
// counting sort
// ---------------------------------------------------------------------------
__global__ void k_keys(long long np, int n, double dxi, const double* __restrict__ x,
                       const double* __restrict__ y, const double* __restrict__ z, int* key,
                       int* count)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    double f;
    const int i = key1(x[q], dxi, n, &f);
    const int j = key1(y[q], dxi, n, &f);
    const int k = key1(z[q], dxi, n, &f);
    const int K = (int)cidx(i, j, k, n);
    key[q] = K;
    atomicAdd(count + K, 1);
}

// slot = start[key] + (remaining count - 1); leaves count all zero
__global__ void k_scatter(long long np, const int* __restrict__ key, const int* __restrict__ start,
                          int* count, int* perm)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int K = key[q];
    const int slot = start[K] + atomicSub(count + K, 1) - 1;
    perm[slot] = (int)q;
}

// Sort every key segment by previous particle index so the result does not
// depend on the order the atomics above were served in.  Segments up to 32
// long are sorted by one thread in registers; longer ones are queued.
__global__ void k_fix_short(int nc, const int* __restrict__ start, int* perm, int* long_list,
                            int* long_count)
{
    int K = blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= nc) return;
    const int s = start[K], e = start[K + 1];
    const int len = e - s;
    if (len <= 1) return;
    if (len > 32) {
        long_list[atomicAdd(long_count, 1)] = K;
        return;
    }
    sort_short_segment(perm, s, len);
}

// long segments: rank sort by one block per segment (values are distinct)
constexpr int kLongSmem = 12288;

__global__ void k_fix_long(const int* __restrict__ start, const int* __restrict__ long_list,
                           const int* __restrict__ long_count, int* perm, int* tmp)
{
    __shared__ int sv[kLongSmem];
    const int total = *long_count;
    for (int li = blockIdx.x; li < total; li += gridDim.x) {
        const int K = long_list[li];
        const int s = start[K], len = start[K + 1] - s;
        const bool in_smem = len <= kLongSmem;
        __syncthreads();
        if (in_smem)
            for (int t = threadIdx.x; t < len; t += blockDim.x) sv[t] = perm[s + t];
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += blockDim.x) {
            const int v = in_smem ? sv[t] : perm[s + t];
            int rank = 0;
            if (in_smem) {
                for (int u = 0; u < len; ++u) rank += sv[u] < v;
            } else {
                for (int u = 0; u < len; ++u) rank += perm[s + u] < v;
            }
            tmp[s + rank] = v;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += blockDim.x) perm[s + t] = tmp[s + t];
    }
}

__global__ void k_gather(long long np, const int* __restrict__ perm, const double* __restrict__ x,
                         const double* __restrict__ y, const double* __restrict__ z,
                         const double* __restrict__ vx, const double* __restrict__ vy,
                         const double* __restrict__ vz, const double* __restrict__ m,
                         const int* __restrict__ id, double* x2, double* y2, double* z2,
                         double* vx2, double* vy2, double* vz2, double* m2, int* id2)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    const int q = perm[s];
    x2[s] = x[q];
    y2[s] = y[q];
    z2[s] = z[q];
    if (vx) {   // null: velocities follow later (k_gather_vel)
        vx2[s] = vx[q];
        vy2[s] = vy[q];
        vz2[s] = vz[q];
    }
    if (m) m2[s] = m[q];
    id2[s] = id[q];
}

// ---------------------------------------------------------------------------
// exclusive scan of the per-key counts (3 phases, 4096 keys per tile)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int warp_incl_scan(int v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one int per thread; returns the block total in *total
__device__ int block_excl_scan(int v, int* total)
{
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int inc = warp_incl_scan(v);
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        int s = lane < nw ? ws[lane] : 0;
        s = warp_incl_scan(s);
        ws[lane] = s;
    }
    __syncthreads();
    const int before = (w > 0 ? ws[w - 1] : 0) + inc - v;
    *total = ws[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void k_scan_reduce(const int* __restrict__ in, int n, int* tile_sums)
{
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t)
        if (base + t < n) s += in[base + t];
    int total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_scan_top(int* tile_sums, int ntiles)
{
    int carry = 0;
    for (int b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = i < ntiles ? tile_sums[i] : 0;
        int total;
        const int ex = block_excl_scan(v, &total);
        if (i < ntiles) tile_sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void k_scan_down(const int* __restrict__ in, int n, const int* __restrict__ tile_off,
                            int* out)
{
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        v[t] = base + t < n ? in[base + t] : 0;
        s += v[t];
    }
    int total;
    int run = block_excl_scan(s, &total) + tile_off[blockIdx.x];
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        if (base + t < n) out[base + t] = run;
        run += v[t];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = run;
}

// ---------------------------------------------------------------------------
// CIC deposit: one block per 8x8x8 tile of cells.  Phase 1: one thread per key of
// the 9x9x9 key window sums its segment's 8 corner weights sequentially (keys of
// one row are contiguous in the sorted particle array).  Phase 2: each cell adds
// the 8 corner partials of its keys in a fixed order.  No atomics; the order is
// fixed, so the density is bitwise reproducible.
// ---------------------------------------------------------------------------
static_assert(kDepositLanes == 32, "long keys are summed by one warp; the sort queues keys > 32");

// adds particle q's eight CIC weights (times its mass, fused, if m) to s
__device__ __forceinline__ void add_weights(int q, int n, double dxi, const double* __restrict__ x,
                                            const double* __restrict__ y,
                                            const double* __restrict__ z,
                                            const double* __restrict__ m, double s[8])
{
    double fx, fy, fz;
    key1(x[q], dxi, n, &fx);
    key1(y[q], dxi, n, &fy);
    key1(z[q], dxi, n, &fz);
    const double sx[2] = {1.0 - fx, fx};
    const double sy[2] = {1.0 - fy, fy};
    const double sz[2] = {1.0 - fz, fz};
    if (m) {
        const double mq = m[q];
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                for (int cx = 0; cx < 2; ++cx)
                    s[cx + 2 * cy + 4 * cz] = fma((sx[cx] * sy[cy]) * sz[cz], mq, s[cx + 2 * cy + 4 * cz]);
    } else {
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                for (int cx = 0; cx < 2; ++cx)
                    s[cx + 2 * cy + 4 * cz] = s[cx + 2 * cy + 4 * cz] + (sx[cx] * sy[cy]) * sz[cz];
    }
}

// Keys longer than a warp (the sort's long_list), one warp each: lane l sums
// particles l, l+32, l+64, ... of the key in order, then the xor butterfly
// (offsets 16, 8, 4, 2, 1) combines the lanes.  The eight corner sums go to
// heavy_part[slot], and key_slot[K] = slot tells the tile kernel where.
__global__ void __launch_bounds__(256) k_deposit_heavy(int n, double dxi,
                                                       const double* __restrict__ x,
                                                       const double* __restrict__ y,
                                                       const double* __restrict__ z,
                                                       const double* __restrict__ m,
                                                       const int* __restrict__ start,
                                                       const int* __restrict__ long_list,
                                                       const int* __restrict__ long_count,
                                                       int* key_slot, double* heavy_part)
{
    const int lane = threadIdx.x & 31;
    const int total = *long_count;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < total; li += nwarps) {
        const int K = long_list[li];
        const int e = start[K + 1];
        double s[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) s[c] = 0.0;
        for (int q = start[K] + lane; q < e; q += 32) add_weights(q, n, dxi, x, y, z, m, s);
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c] = s[c] + __shfl_xor_sync(0xffffffffu, s[c], off);
        if (lane < 8) {
            double v = s[0];
#pragma unroll
            for (int c = 1; c < 8; ++c)
                if (lane == c) v = s[c];
            heavy_part[8LL * li + lane] = v;
        }
        if (lane == 0) key_slot[K] = li;
    }
}

// Pass 1 of the FP64 deposit: the eight corner sums of every key into
// part[corner * nc + K].  One warp takes 32 consecutive keys.  Their particles
// (sorted, so contiguous) are numbered densely across the warp and each lane
// computes the CIC weights of one particle per batch of 32, into shared
// memory; then the adds run with eight lanes per key, one per corner, each
// adding its key's particles of the batch in sorted order.  So every key is
// summed in order, exactly as one thread would, while the expensive part (the
// weights) is spread evenly over the lanes whatever the keys' occupancy.
// Keys longer than a warp take their sums from k_deposit_heavy.
constexpr int kKeyWarps = 8;

__global__ void __launch_bounds__(32 * kKeyWarps) k_deposit_keys(long long nc, int n, double dxi,
                                                                 const double* __restrict__ x,
                                                                 const double* __restrict__ y,
                                                                 const double* __restrict__ z,
                                                                 const double* __restrict__ m,
                                                                 const int* __restrict__ start,
                                                                 const int* __restrict__ key_slot,
                                                                 const double* __restrict__ heavy_part,
                                                                 double* __restrict__ part)
{
    __shared__ double wbuf[kKeyWarps][32][9];   // a batch's weights (and masses)
    __shared__ double acc[kKeyWarps][32][8];    // the warp's 32 keys' corner sums
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long K0 = ((long long)blockIdx.x * kKeyWarps + wid) * 32;
    if (K0 >= nc) return;                        // the whole warp leaves together
    const long long K = K0 + lane;
    const bool valid = K < nc;
    int b0 = 0, cnt = 0;
    if (valid) {
        b0 = start[K];
        cnt = start[K + 1] - b0;
    }
    const bool heavy = cnt > kDepositLanes;
    const int ml = heavy ? 0 : cnt;
    int incl = ml;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int v = __shfl_up_sync(full, incl, off);
        if (lane >= off) incl += v;
    }
    const int excl = incl - ml;
    const int total = __shfl_sync(full, incl, 31);
    double* mine = acc[wid][lane];
    if (heavy) {
        const double* hp = heavy_part + 8LL * key_slot[K];
#pragma unroll
        for (int c = 0; c < 8; ++c) mine[c] = hp[c];
    } else {
#pragma unroll
        for (int c = 0; c < 8; ++c) mine[c] = 0.0;
    }
    __syncwarp();
    const int corner = lane & 7;
    for (int base = 0; base < total; base += 32) {
        // the lane owning particle number q: the first lane whose inclusive count exceeds q
        const int q = base + lane;
        int o = 0;
#pragma unroll
        for (int bit = 16; bit >= 1; bit >>= 1) {
            const int v = __shfl_sync(full, incl, o + bit - 1);
            if (v <= q) o += bit;
        }
        const int ob0 = __shfl_sync(full, b0, o & 31);
        const int oex = __shfl_sync(full, excl, o & 31);
        if (q < total) {
            const int p = ob0 + (q - oex);
            double fx, fy, fz;
            key1(x[p], dxi, n, &fx);
            key1(y[p], dxi, n, &fy);
            key1(z[p], dxi, n, &fz);
            const double sx[2] = {1.0 - fx, fx};
            const double sy[2] = {1.0 - fy, fy};
            const double sz[2] = {1.0 - fz, fz};
            double* w = wbuf[wid][lane];
#pragma unroll
            for (int cz = 0; cz < 2; ++cz)
#pragma unroll
                for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                    for (int cx = 0; cx < 2; ++cx) w[cx + 2 * cy + 4 * cz] = (sx[cx] * sy[cy]) * sz[cz];
            if (m) w[8] = m[p];
        }
        __syncwarp();
        // eight rounds of four keys x eight corners
#pragma unroll 1
        for (int r = 0; r < 8; ++r) {
            const int ow = 4 * r + (lane >> 3);
            const int oi = __shfl_sync(full, incl, ow);
            const int oe = __shfl_sync(full, excl, ow);
            const int lo = max(oe, base) - base, hi = min(oi, base + 32) - base;
            if (lo < hi) {
                double a = acc[wid][ow][corner];
                if (m) {
                    for (int t = lo; t < hi; ++t) a = fma(wbuf[wid][t][corner], wbuf[wid][t][8], a);
                } else {
                    for (int t = lo; t < hi; ++t) a = a + wbuf[wid][t][corner];
                }
                acc[wid][ow][corner] = a;
            }
        }
        __syncwarp();
    }
    if (valid) {
#pragma unroll
        for (int c = 0; c < 8; ++c) part[c * nc + K] = mine[c];
    }
}

// Pass 2, one thread per cell: the eight keys' corners in the fixed (dk, dj, di)
// order, times the scale -- the same sums as the tile kernel's, term for term.
__global__ void __launch_bounds__(256) k_deposit_cells(int n, double scale,
                                                       const double* __restrict__ part,
                                                       double* __restrict__ rho)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    const long long nc = (long long)n * n * n;
    const int ip = i == n - 1 ? 0 : i + 1, jp = j == n - 1 ? 0 : j + 1, kp = k == n - 1 ? 0 : k + 1;
    const int is[2] = {i, ip}, js[2] = {j, jp}, ks[2] = {k, kp};
    double acc = 0.0;
#pragma unroll
    for (int dk = 0; dk < 2; ++dk)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
            for (int di = 0; di < 2; ++di) {
                const int corner = (1 - di) + 2 * (1 - dj) + 4 * (1 - dk);
                acc = acc + __ldg(part + corner * nc + cidx(is[di], js[dj], ks[dk], n));
            }
    rho[cidx(i, j, k, n)] = acc * scale;
}

// ---------------------------------------------------------------------------
// CIC interpolation of the cell-centred gravity vector + kick (+ drift)
// (+ periodic wrap), update_dm_particle_single with the products of the
// reference fused where the oracle fuses them
// ---------------------------------------------------------------------------
struct KickArgs {
    int n;
    double dxi, L;
    const double* g;   // 3 n^3, component-major
    double half_dt, a_prev, a_cur_inv, dt_a_cur_inv;
    int do_move, do_wrap;
};

__global__ void __launch_bounds__(256) k_kick(long long np, KickArgs A, double* x, double* y,
                                              double* z, double* vx, double* vy, double* vz)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int n = A.n;
    const long long nc = (long long)n * n * n;
    const double lx = fma(x[q], A.dxi, 0.5);
    const double ly = fma(y[q], A.dxi, 0.5);
    const double lz = fma(z[q], A.dxi, 0.5);
    int i, j, k;
    const double fi = floor_int(lx, &i), fj = floor_int(ly, &j), fk = floor_int(lz, &k);
    const double xint = lx - fi, yint = ly - fj, zint = lz - fk;
    const double sx[2] = {1.0 - xint, xint};
    const double sy[2] = {1.0 - yint, yint};
    const double sz[2] = {1.0 - zint, zint};
    double w[8];
    long long cell[8];
#pragma unroll
    for (int kk = 0; kk <= 1; ++kk)
#pragma unroll
        for (int jj = 0; jj <= 1; ++jj)
#pragma unroll
            for (int ii = 0; ii <= 1; ++ii) {
                const int t = ii + 2 * jj + 4 * kk;
                w[t] = (sx[1 - ii] * sy[1 - jj]) * sz[1 - kk];
                cell[t] = cidx(wrapi(i - ii, n), wrapi(j - jj, n), wrapi(k - kk, n), n);
            }
    double v[3] = {vx[q], vy[q], vz[q]};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double* gd = A.g + d * nc;
        double val = 0.0;
#pragma unroll
        for (int t = 0; t < 8; ++t) val = fma(w[t], __ldg(gd + cell[t]), val);
        const double u = fma(A.a_prev, v[d], A.half_dt * val);
        v[d] = u * A.a_cur_inv;
    }
    vx[q] = v[0];
    vy[q] = v[1];
    vz[q] = v[2];
    if (A.do_move == 1) {
        double px = fma(A.dt_a_cur_inv, v[0], x[q]);
        double py = fma(A.dt_a_cur_inv, v[1], y[q]);
        double pz = fma(A.dt_a_cur_inv, v[2], z[q]);
        if (A.do_wrap) {
            px = wrap_pos(px, A.L);
            py = wrap_pos(py, A.L);
            pz = wrap_pos(pz, A.L);
        }
        x[q] = px;
        y[q] = py;
        z[q] = pz;
    } else if (A.do_wrap) {
        x[q] = wrap_pos(x[q], A.L);
        y[q] = wrap_pos(y[q], A.L);
        z[q] = wrap_pos(z[q], A.L);
    }
}

// ---------------------------------------------------------------------------
// particle time-step limit (NyxParticleContainer::estTimestep,
// NyxParticleContainer.H:329-465): per particle
//   dt_p = cfl / max_d(|v_d| * adxi)   (adxi = dxi / a; 1e50 when v = 0),
//   dt_p = min(dt_p, 1 / sqrt(|g| * dxi)) when |g| > 0,
// |g| = sqrt((gx*gx + gy*gy) + gz*gz) at the cell floor(x*dxi) (wrapped), and
// the minimum over particles.  A positive double orders like its bit pattern,
// so the minimum is an integer max of the complemented bits: the result does
// not depend on the order the blocks finish in.  out must start at 0.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_est_dt(long long np, int n, double dxi, double adxi,
                                                double cfl, const double* __restrict__ x,
                                                const double* __restrict__ y,
                                                const double* __restrict__ z,
                                                const double* __restrict__ vx,
                                                const double* __restrict__ vy,
                                                const double* __restrict__ vz,
                                                const double* __restrict__ g,
                                                unsigned long long* out)
{
    const long long nc = (long long)n * n * n;
    double best = 1.0e50;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < np;
         q += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        floor_int(x[q] * dxi, &i);
        floor_int(y[q] * dxi, &j);
        floor_int(z[q] * dxi, &k);
        i = wrapi(i, n);
        j = wrapi(j, n);
        k = wrapi(k, n);
        const double ux = fabs(vx[q]) * adxi, uy = fabs(vy[q]) * adxi, uz = fabs(vz[q]) * adxi;
        const double um = fmax(fmax(ux, uy), uz);
        double dtp = um > 0 ? cfl / um : 1.0e50;
        const long long c = cidx(i, j, k, n);
        const double gx = __ldg(g + c), gy = __ldg(g + nc + c), gz = __ldg(g + 2 * nc + c);
        const double ga = sqrt((gx * gx + gy * gy) + gz * gz);
        if (ga > 0) dtp = fmin(dtp, 1.0 / sqrt(ga * dxi));
        best = fmin(best, dtp);
    }
    block_umax_store(~(unsigned long long)__double_as_longlong(best), out);
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
nyxpm_status launch_unpack(Ctx& c, Box& b, const double* d_pos, const double* d_vel,
                           const double* d_mass)
{
    prof_begin(c);
    k_unpack<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, d_pos, d_vel, d_mass, b.x, b.y, b.z,
                                                           b.vx, b.vy, b.vz, d_mass ? b.m : nullptr,
                                                           b.id, b.norms + 2);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "unpack");
}

nyxpm_status launch_pack(Ctx& c, Box& b, double* d_pos, double* d_vel)
{
    prof_begin(c);
    k_pack<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.x, b.y, b.z, b.vx, b.vy, b.vz, b.id,
                                                         d_pos, d_vel);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "pack");
}

nyxpm_status launch_wrap(Ctx& c, Box& b)
{
    prof_begin(c);
    k_wrap<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.L, b.x, b.y, b.z);
    prof_end(c, NYXPM_ST_KICK, 48.0 * b.np);
    return check_launch(c, "wrap");
}

nyxpm_status scan_counts(Ctx& c, Box& b)
{
    const int nc = b.n * b.n * b.n;
    const int nt = b.ntiles;
    prof_begin(c);
    k_scan_reduce<<<nt, kScanThreads, 0, c.stream>>>(b.cell_count, nc, b.tile_sums);
    k_scan_top<<<1, 1024, 0, c.stream>>>(b.tile_sums, nt);
    k_scan_down<<<nt, kScanThreads, 0, c.stream>>>(b.cell_count, nc, b.tile_sums, b.cell_start);
    prof_end(c, NYXPM_ST_SCAN, 12.0 * nc);
    c.launches += 2;
    return check_launch(c, "scan");
}

nyxpm_status fix_segments(Ctx& c, Box& b)
{
    const int nc = b.n * b.n * b.n;
    prof_begin(c);
    cudaMemsetAsync(b.long_count, 0, sizeof(int), c.stream);
    k_fix_short<<<blocks_for(nc), kThreads, 0, c.stream>>>(nc, b.cell_start, b.perm, b.long_list,
                                                            b.long_count);
    k_fix_long<<<c.sm_count * 2, 512, 0, c.stream>>>(b.cell_start, b.long_list, b.long_count, b.perm,
                                                      b.key);
    prof_end(c, NYXPM_ST_SCATTER, 4.0 * nc + 8.0 * b.np);
    c.launches += 1;
    return check_launch(c, "fix segments");
}

nyxpm_status sort_from_keys(Ctx& c, Box& b)
{
    nyxpm_status st;
    if ((st = scan_counts(c, b)) != NYXPM_OK) return st;
    prof_begin(c);
    k_scatter<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.key, b.cell_start, b.cell_count,
                                                            b.perm);
    prof_end(c, NYXPM_ST_SCATTER, 12.0 * b.np);
    if ((st = check_launch(c, "scatter")) != NYXPM_OK) return st;
    return fix_segments(c, b);
}

nyxpm_status launch_sort(Ctx& c, Box& b, bool defer_vel)
{
    nyxpm_status st;
    // the scatter leaves the counts at zero, but an interrupted sort may not have
    cudaMemsetAsync(b.cell_count, 0, sizeof(int) * (size_t)b.n * b.n * b.n, c.stream);
    prof_begin(c);
    k_keys<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.n, b.dxi, b.x, b.y, b.z, b.key,
                                                         b.cell_count);
    prof_end(c, NYXPM_ST_KEYS, 32.0 * b.np);
    if ((st = check_launch(c, "keys")) != NYXPM_OK) return st;
    if ((st = sort_from_keys(c, b)) != NYXPM_OK) return st;
    const int nvals = (b.uniform_mass ? 6 : 7) - (defer_vel ? 3 : 0);
    prof_begin(c);
    // defer_vel: the velocities are not on the device yet; launch_gather_vel
    // permutes them by the same perm once they are
    k_gather<<<blocks_for(b.np), kThreads, 0, c.stream>>>(
        b.np, b.perm, b.x, b.y, b.z, defer_vel ? nullptr : b.vx, b.vy, b.vz,
        b.uniform_mass ? nullptr : b.m, b.id, b.x2, b.y2, b.z2, b.vx2, b.vy2, b.vz2,
        b.uniform_mass ? nullptr : b.m2, b.id2);
    prof_end(c, NYXPM_ST_GATHER, (16.0 * nvals + 12.0) * b.np);
    if ((st = check_launch(c, "gather")) != NYXPM_OK) return st;
    std::swap(b.x, b.x2);
    std::swap(b.y, b.y2);
    std::swap(b.z, b.z2);
    if (!defer_vel) {
        std::swap(b.vx, b.vx2);
        std::swap(b.vy, b.vy2);
        std::swap(b.vz, b.vz2);
    }
    std::swap(b.m, b.m2);
    std::swap(b.id, b.id2);
    b.sorted = 1;
    return NYXPM_OK;
}

nyxpm_status launch_unpack_pos(Ctx& c, Box& b, const double* d_pos, const double* d_mass)
{
    prof_begin(c);
    k_unpack_pos<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, d_pos, d_mass, b.x, b.y, b.z,
                                                               d_mass ? b.m : nullptr, b.id, b.norms + 2);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "unpack positions");
}

// the velocities, in the order the particles had before the last (deferred) sort,
// into the scratch arrays, then permuted into place by that sort's perm
nyxpm_status launch_unpack_gather_vel(Ctx& c, Box& b, const double* d_vel, bool sorted_since)
{
    prof_begin(c);
    if (sorted_since) {
        k_unpack_vel<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, d_vel, b.vx2, b.vy2, b.vz2,
                                                                   b.norms + 2);
        k_gather_vel<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.perm, b.vx2, b.vy2, b.vz2,
                                                                   b.vx, b.vy, b.vz);
        c.launches += 1;
    } else {
        k_unpack_vel<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, d_vel, b.vx, b.vy, b.vz,
                                                                   b.norms + 2);
    }
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "unpack velocities");
}

nyxpm_status launch_pack_pos_wrapped(Ctx& c, Box& b, double* d_pos)
{
    prof_begin(c);
    k_pack_pos_wrapped<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.L, b.x, b.y, b.z, b.id,
                                                                     d_pos);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "pack positions");
}

nyxpm_status launch_pack_vel(Ctx& c, Box& b, double* d_vel)
{
    prof_begin(c);
    k_pack_vel<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, b.vx, b.vy, b.vz, b.id, d_vel);
    prof_end(c, NYXPM_ST_GATHER, 0);
    return check_launch(c, "pack velocities");
}

nyxpm_status launch_deposit(Ctx& c, Box& b)
{
    const int n = b.n;
    const double dx = b.L / n;
    const double inv_vol = 1.0 / (dx * dx * dx);
    // per-particle masses: keys sum w*m, cells scale by 1/dx^3; uniform: keys sum w, cells by m/dx^3
    const double scale = b.uniform_mass ? b.mscalar * inv_vol : inv_vol;
    const double nc = (double)n * n * n;
    const double* mq = b.uniform_mass ? nullptr : b.m;
    prof_begin(c);
    k_deposit_heavy<<<c.sm_count * 4, 256, 0, c.stream>>>(n, b.dxi, b.x, b.y, b.z, mq, b.cell_start,
                                                          b.long_list, b.long_count, b.key_slot,
                                                          b.heavy_part);
    const long long ncl = (long long)n * n * n;
    const unsigned kb = (unsigned)((ncl + 32LL * kKeyWarps - 1) / (32LL * kKeyWarps));
    k_deposit_keys<<<kb, 32 * kKeyWarps, 0, c.stream>>>(ncl, n, b.dxi, b.x, b.y, b.z, mq,
                                                         b.cell_start, b.key_slot, b.heavy_part,
                                                         b.key_part);
    const Geo g = geo3(n, n, n);
    k_deposit_cells<<<g.grid, g.block, 0, c.stream>>>(n, scale, b.key_part, b.rho);
    c.launches += 2;
    prof_end(c, NYXPM_ST_DEPOSIT, (b.uniform_mass ? 24.0 : 32.0) * b.np + 12.0 * nc);
    return check_launch(c, "deposit");
}

nyxpm_status launch_kick(Ctx& c, Box& b, double dt, double a_prev, double a_cur, int do_move,
                         int do_wrap)
{
    KickArgs A;
    A.n = b.n;
    A.dxi = b.dxi;
    A.L = b.L;
    A.g = b.g;
    A.half_dt = 0.5 * dt;
    A.a_prev = a_prev;
    A.a_cur_inv = 1.0 / a_cur;
    A.dt_a_cur_inv = dt * A.a_cur_inv;
    A.do_move = do_move;
    A.do_wrap = do_wrap;
    prof_begin(c);
    k_kick<<<blocks_for(b.np), kThreads, 0, c.stream>>>(b.np, A, b.x, b.y, b.z, b.vx, b.vy, b.vz);
    const double nc = (double)b.n * b.n * b.n;
    prof_end(c, NYXPM_ST_KICK, (do_move ? 96.0 : 72.0) * b.np + 24.0 * nc);
    b.sorted = b.sorted && !do_move && !do_wrap;
    return check_launch(c, "kick");
}

nyxpm_status launch_est_dt(Ctx& c, Box& b, double cfl, double a)
{
    cudaMemsetAsync(b.norms + 3, 0, sizeof(unsigned long long), c.stream);
    const unsigned blocks = std::min(blocks_for(b.np), (unsigned)(c.sm_count * 8));
    k_est_dt<<<blocks, kThreads, 0, c.stream>>>(b.np, b.n, b.dxi, b.dxi / a, cfl, b.x, b.y, b.z,
                                                 b.vx, b.vy, b.vz, b.g, b.norms + 3);
    c.launches += 1;
    return check_launch(c, "time-step estimate");
}

}  // namespace nyxpm
