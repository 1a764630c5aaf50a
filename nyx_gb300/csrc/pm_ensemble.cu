// Batched ensemble of independent periodic PM boxes of uneven sizes, all in the
// mixed-precision form, advanced together: every stage of a step is ONE
// persistent launch over a work list that spans all boxes (particle chunks,
// plane rows of every multigrid level, deposit tiles, per-box items), and the
// step is captured in CUDA graphs and replayed.
//
// What a kernel needs about a box comes from two device arrays: a descriptor
// (sizes and array pointers; written by the host, read-only on the device) and
// a state record (current particle buffer, activity, step scalars, convergence;
// owned by the device).  The graphs therefore replay without host updates; the
// per-box step scalars are copied in from a pinned host buffer by the graph
// itself.  Box storage comes from a device arena (one cudaMalloc at creation,
// first-fit sub-allocation), so boxes join and leave without cudaMalloc.
//
// The arithmetic per box is that of the single-box mixed form (FP32
// cell-relative particles, FP32 deposit and V-cycles, FP64 defect correction to
// the context's relative tolerance, compensated FP64 mean, FP64 a(t) on the
// host).  Convergence is per box: a step is ONE graph -- the opening kick, the
// deposit and max_outer defect-correction iterations, then a conditional WHILE
// node that repeats one more iteration (the residual recomputed with the FP64
// stencil) while any box is above its tolerance, up to max_vcycles, then the
// gravity vector and the closing kick.  A box that has met its tolerance skips
// the remaining iterations' work, so a slow box never changes another box's
// result.
#include "pm_common.cuh"
#include "pm_prolong.cuh"
#include "pm_restrict.cuh"
#include "pm_tail.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <vector>

namespace nyxpm {

namespace {

constexpr int kMaxLev = 9;
constexpr int kPT = 256;             // threads of the particle kernels' blocks
// particles per particle work item (the sort's and the kicks' bucket): the
// nyxpm_tuning knob sort_bucket, a multiple of kPT
constexpr int kScanT = 512, kScanIPT = 8, kScanTile = kScanT * kScanIPT;
constexpr float kSixthF = 1.0f / 6.0f;
constexpr double kSixth = 1.0 / 6.0;

__constant__ float kProlongWE[8] = {0.421875f, 0.140625f, 0.140625f, 0.046875f,
                                    0.140625f, 0.046875f, 0.046875f, 0.015625f};

struct ELevel {
    int n, split;
    float* phi_r;
    float* phi_b;
    float* beta_r;
    float* beta_b;
};

// per-box descriptor: written by the host, read-only on the device
struct EDesc {
    int n, nlev, nb, used;
    long long np;
    double L, dx, dxi, mass_offset, mscalar, beta_scale;
    float dep_scale;                  // (float)(mscalar / dx^3), the FP32 deposit's cell scale
    int pad_scale;
    // particle arrays: buffer 0 and buffer 1 (the sort gathers from one into the other)
    int *cell0, *id0, *cell1, *id1;
    float *ox0, *oy0, *oz0, *vx0, *vy0, *vz0;
    float *ox1, *oy1, *oz1, *vx1, *vy1, *vz1;
    int *key, *perm, *cell_count, *cell_start, *tile_sums, *long_list, *long_count;
    float *frho, *g32;
    double *rows, *scal;              // scal[0] mean
    double *phi_r, *phi_b, *beta_r, *beta_b;   // level-0 FP64, split layout
    float* r_lo;                      // low words of the level-0 residual (red n^3/2, black n^3/2)
    int tail_l;                       // first level of the fused coarse V-cycle (e_tail)
    int pad_tail;
    float* Gf;
    unsigned long long* norms;        // [0] ||beta||, [1] ||r||, [2] bad uploads
    ELevel lv[kMaxLev];
};

// per-box state owned by the device (the host reads it, or resets it for a new box)
struct EState {
    int parity;                       // which particle buffer is current
    int active;                       // takes part in the current pass
    int solve_active;                 // still iterating in the current solve
    int outer, inner;                 // defect-correction / FP32 V-cycle counts of the last solve
    int pad;
    double target;                    // convergence target of the current solve (smoother units)
    double err;                       // bound on |tracked residual - residual of phi| (e_correct)
    double a_old, a_new, dt;
    // the kicks' FP32 scalars per phase (0: kick-drift to a_half, 1: kick to a_new):
    // a_prev, 1 / a_cur, dt / 2, drift in cells; formed once per box in FP64
    float kick[2][4];
};

// step scalars written by the host each step (pinned) and copied in by the graph
struct EStep {
    double a_old, a_new, dt;
    int active;
    int pad;
};

struct Item {
    int box, a, b, c;
};

// current particle arrays of a box
struct PArr {
    int* cell;
    int* id;
    float *ox, *oy, *oz, *vx, *vy, *vz;
};

__device__ __forceinline__ PArr parr(const EDesc& d, int parity)
{
    if (parity) return PArr{d.cell1, d.id1, d.ox1, d.oy1, d.oz1, d.vx1, d.vy1, d.vz1};
    return PArr{d.cell0, d.id0, d.ox0, d.oy0, d.oz0, d.vx0, d.vy0, d.vz0};
}

__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__device__ __forceinline__ int pack_cell(int i, int j, int k) { return i | (j << 10) | (k << 20); }
__device__ __forceinline__ int cell_i(int c) { return c & 1023; }
__device__ __forceinline__ int cell_j(int c) { return (c >> 10) & 1023; }
__device__ __forceinline__ int cell_k(int c) { return (c >> 20) & 1023; }

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
// step scalars
// ---------------------------------------------------------------------------
__global__ void e_load_step(int nbox, const EStep* __restrict__ st, const EDesc* __restrict__ D,
                            EState* S)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox) return;
    const double a_old = st[b].a_old, a_new = st[b].a_new, dt = st[b].dt;
    S[b].a_old = a_old;
    S[b].a_new = a_new;
    S[b].dt = dt;
    S[b].active = st[b].active;
    const double a_half = 0.5 * (a_old + a_new);
    for (int phase = 0; phase < 2; ++phase) {
        const double a_cur = phase == 0 ? a_half : a_new;
        S[b].kick[phase][0] = (float)(phase == 0 ? a_old : a_half);
        S[b].kick[phase][1] = (float)(1.0 / a_cur);
        S[b].kick[phase][2] = (float)(0.5 * dt);
        S[b].kick[phase][3] = (float)(dt / a_cur * D[b].dxi);
    }
}

// ---------------------------------------------------------------------------
// particle stages: item = (box, bucket of `bucket` consecutive particles), a
// block of kPT threads striding through the bucket
// ---------------------------------------------------------------------------
// phase 0: kick-drift (a_old -> a_half, move); phase 1: kick (a_half -> a_new)
__global__ void __launch_bounds__(kPT, 4) e_kick(const Item* __restrict__ items, int nitems,
                                               const EDesc* __restrict__ D, const EState* __restrict__ S,
                                               int phase, int bucket)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        // by reference: a copy indexed by the runtime phase would live in local memory
        const EState& st = S[it.box];
        if (!st.active) continue;
        const EDesc& d = D[it.box];
      for (int t = threadIdx.x; t < bucket; t += kPT) {
        const long long q = (long long)it.a * bucket + t;
        if (q >= d.np) break;
        const PArr P = parr(d, st.parity);
        const int n = d.n;
        const float a_prev = st.kick[phase][0];
        const float a_cur_inv = st.kick[phase][1];
        const float half_dt = st.kick[phase][2];
        const float drift = st.kick[phase][3];
        const int c = P.cell[q];
        const int ci = cell_i(c), cj = cell_j(c), ck = cell_k(c);
        float o[3] = {P.ox[q], P.oy[q], P.oz[q]};
        float fx, fy, fz;
        const int i = key_frac(ci, o[0], n, &fx);
        const int j = key_frac(cj, o[1], n, &fy);
        const int k = key_frac(ck, o[2], n, &fz);
        const float sx[2] = {1.f - fx, fx};
        const float sy[2] = {1.f - fy, fy};
        const float sz[2] = {1.f - fz, fz};
        float wgt[8];
        // 32-bit cell offsets (n <= 1024), as in k_mx_kick
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
                    wgt[t] = (sx[1 - ii] * sy[1 - jj]) * sz[1 - kk];
                    cc[t] = xs[ii] + ys[jj] + zs[kk];
                }
        float v[3] = {P.vx[q], P.vy[q], P.vz[q]};
        float val[3] = {0.f, 0.f, 0.f};
        const float4* g4 = reinterpret_cast<const float4*>(d.g32);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const float4 gc = __ldg(g4 + cc[t]);
            val[0] = fmaf(wgt[t], gc.x, val[0]);
            val[1] = fmaf(wgt[t], gc.y, val[1]);
            val[2] = fmaf(wgt[t], gc.z, val[2]);
        }
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) v[dd] = fmaf(a_prev, v[dd], half_dt * val[dd]) * a_cur_inv;
        P.vx[q] = v[0];
        P.vy[q] = v[1];
        P.vz[q] = v[2];
        if (phase == 0) {
            int ic[3] = {ci, cj, ck};
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) {
                float p = fmaf(drift, v[dd], o[dd]);
                float fl = floorf(p);
                p -= fl;
                if (p >= 1.f) {  // -tiny + 1 rounded up to 1: the next cell's origin
                    p = 0.f;
                    fl += 1.f;
                }
                int idx = ic[dd] + (int)fl;
                if (idx >= n) idx -= n;       // a move of less than n cells: one step
                else if (idx < 0) idx += n;
                if ((unsigned)idx >= (unsigned)n) {   // further: the general wrap
                    idx %= n;
                    if (idx < 0) idx += n;
                }
                ic[dd] = idx;
                o[dd] = p;
            }
            P.cell[q] = pack_cell(ic[0], ic[1], ic[2]);
            P.ox[q] = o[0];
            P.oy[q] = o[1];
            P.oz[q] = o[2];
        }
      }
    }
}

__global__ void __launch_bounds__(kPT) e_keys(const Item* __restrict__ items, int nitems,
                                               const EDesc* __restrict__ D, const EState* __restrict__ S,
                                               int bucket)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!st.active) continue;
        const EDesc& d = D[it.box];
        const PArr P = parr(d, st.parity);
        for (int t = threadIdx.x; t < bucket; t += kPT) {
            const long long q = (long long)it.a * bucket + t;
            if (q >= d.np) break;
            const int c = P.cell[q];
            float f;
            const int i = key_frac(cell_i(c), P.ox[q], d.n, &f);
            const int j = key_frac(cell_j(c), P.oy[q], d.n, &f);
            const int k = key_frac(cell_k(c), P.oz[q], d.n, &f);
            const int K = (int)cidx(i, j, k, d.n);
            d.key[q] = K;
            atomicAdd(d.cell_count + K, 1);
        }
    }
}

__global__ void __launch_bounds__(kPT) e_scatter(const Item* __restrict__ items, int nitems,
                                                  const EDesc* __restrict__ D, const EState* __restrict__ S,
                                                  int bucket)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        if (!S[it.box].active) continue;
        const EDesc& d = D[it.box];
        for (int t = threadIdx.x; t < bucket; t += kPT) {
            const long long q = (long long)it.a * bucket + t;
            if (q >= d.np) break;
            const int K = d.key[q];
            d.perm[d.cell_start[K] + atomicSub(d.cell_count + K, 1) - 1] = (int)q;
        }
    }
}

__global__ void __launch_bounds__(kPT, 8) e_gather(const Item* __restrict__ items, int nitems,
                                                 const EDesc* __restrict__ D, const EState* __restrict__ S,
                                                 int bucket)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!st.active) continue;
        const EDesc& d = D[it.box];
        const PArr A = parr(d, st.parity), B = parr(d, st.parity ^ 1);
        for (int t = threadIdx.x; t < bucket; t += kPT) {
            const long long s = (long long)it.a * bucket + t;
            if (s >= d.np) break;
            const int q = d.perm[s];
            B.cell[s] = A.cell[q];
            B.ox[s] = A.ox[q];
            B.oy[s] = A.oy[q];
            B.oz[s] = A.oz[q];
            B.vx[s] = A.vx[q];
            B.vy[s] = A.vy[q];
            B.vz[s] = A.vz[q];
            B.id[s] = A.id[q];
        }
    }
}

// flip the current particle buffer of every active box (after the gather)
__global__ void e_flip(int nbox, EState* S)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox || !S[b].active) return;
    S[b].parity ^= 1;
}

// ---------------------------------------------------------------------------
// per-box segmented scan of the key counts: item = (box, tile of 4096 keys)
// ---------------------------------------------------------------------------
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

__global__ void __launch_bounds__(kScanT) e_scan_reduce(const Item* __restrict__ items, int nitems,
                                                        const EDesc* __restrict__ D,
                                                        const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        if (!S[it.box].active) continue;  // uniform across the block
        const EDesc& d = D[it.box];
        const int nc = d.n * d.n * d.n;
        const long long base = (long long)it.a * kScanTile + (long long)threadIdx.x * kScanIPT;
        int s = 0;
#pragma unroll
        for (int t = 0; t < kScanIPT; ++t)
            if (base + t < nc) s += d.cell_count[base + t];
        int total;
        block_excl_scan(s, &total);
        if (threadIdx.x == 0) d.tile_sums[it.a] = total;
    }
}

__global__ void e_scan_top(int nbox, const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    const int b = blockIdx.x;
    if (b >= nbox || !S[b].active) return;
    const EDesc& d = D[b];
    const int nc = d.n * d.n * d.n;
    const int ntiles = (nc + kScanTile - 1) / kScanTile;
    int carry = 0;
    for (int b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = i < ntiles ? d.tile_sums[i] : 0;
        int total;
        const int ex = block_excl_scan(v, &total);
        if (i < ntiles) d.tile_sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanT) e_scan_down(const Item* __restrict__ items, int nitems,
                                                      const EDesc* __restrict__ D,
                                                      const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        if (!S[it.box].active) continue;
        const EDesc& d = D[it.box];
        const int nc = d.n * d.n * d.n;
        const long long base = (long long)it.a * kScanTile + (long long)threadIdx.x * kScanIPT;
        int v[kScanIPT];
        int s = 0;
#pragma unroll
        for (int t = 0; t < kScanIPT; ++t) {
            v[t] = base + t < nc ? d.cell_count[base + t] : 0;
            s += v[t];
        }
        int total;
        int run = block_excl_scan(s, &total) + d.tile_sums[it.a];
#pragma unroll
        for (int t = 0; t < kScanIPT; ++t) {
            if (base + t < nc) d.cell_start[base + t] = run;
            run += v[t];
        }
        if (base < nc && base + kScanIPT >= nc) d.cell_start[nc] = run;
    }
}

// deterministic order inside each key segment: item = (box, chunk of 256 keys)
__global__ void __launch_bounds__(256) e_fix_short(const Item* __restrict__ items, int nitems,
                                                    const EDesc* __restrict__ D,
                                                    const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        if (!S[it.box].active) continue;
        const EDesc& d = D[it.box];
        const int K = it.a * 256 + threadIdx.x;
        if (K >= d.n * d.n * d.n) continue;
        const int s = d.cell_start[K], len = d.cell_start[K + 1] - s;
        if (len <= 1) continue;
        if (len > 32) {
            d.long_list[atomicAdd(d.long_count, 1)] = K;
            continue;
        }
        sort_short_segment(d.perm, s, len);
    }
}

constexpr int kLongSmem = 12288;

__global__ void e_fix_long(int nbox, const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    __shared__ int sv[kLongSmem];
    for (int b = 0; b < nbox; ++b) {
        if (!S[b].active) continue;
        const EDesc& d = D[b];
        const int total = *d.long_count;
        for (int li = blockIdx.x; li < total; li += gridDim.x) {
            const int K = d.long_list[li];
            const int s = d.cell_start[K], len = d.cell_start[K + 1] - s;
            const bool in_smem = len <= kLongSmem;
            __syncthreads();
            if (in_smem)
                for (int t = threadIdx.x; t < len; t += blockDim.x) sv[t] = d.perm[s + t];
            __syncthreads();
            for (int t = threadIdx.x; t < len; t += blockDim.x) {
                const int v = in_smem ? sv[t] : d.perm[s + t];
                int rank = 0;
                if (in_smem) {
                    for (int u = 0; u < len; ++u) rank += sv[u] < v;
                } else {
                    for (int u = 0; u < len; ++u) rank += d.perm[s + u] < v;
                }
                d.key[s + rank] = v;
            }
            __syncthreads();
            for (int t = threadIdx.x; t < len; t += blockDim.x) d.perm[s + t] = d.key[s + t];
        }
    }
}

__global__ void e_sort_reset(int nbox, const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox || !S[b].active) return;
    *D[b].long_count = 0;
}

// ---------------------------------------------------------------------------
// FP32 deposit: item = (box, tile); tile shape from the template
// ---------------------------------------------------------------------------
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(256) e_deposit(const Item* __restrict__ items, int nitems,
                                                 const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    constexpr int KX = TX + 1, KY = TY + 1, KZ = TZ + 1, NK = KX * KY * KZ;
    // corner-major: a warp's consecutive keys (or cells) touch consecutive banks
    __shared__ float part[NK * 8];
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!st.active) continue;
        const EDesc& d = D[it.box];
        const PArr P = parr(d, st.parity);
        const int n = d.n;
        const int i0 = it.a * TX, j0 = it.b * TY, k0 = it.c * TZ;
        __syncthreads();
        for (int kl = threadIdx.x; kl < NK; kl += blockDim.x) {
            const int ki = kl % KX, kj = (kl / KX) % KY, kk = kl / (KX * KY);
            // window coordinates exceed n by less than a tile: wrap by subtraction
            int wi = i0 + ki, wj = j0 + kj, wk = k0 + kk;
            while (wi >= n) wi -= n;
            while (wj >= n) wj -= n;
            while (wk >= n) wk -= n;
            const unsigned K = (unsigned)wi + (unsigned)n * ((unsigned)wj + (unsigned)n * (unsigned)wk);
            float s[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) s[c] = 0.f;
            const int e = d.cell_start[K + 1];
            for (int q = d.cell_start[K]; q < e; ++q) {
                const int c = P.cell[q];
                float fx, fy, fz;
                key_frac(cell_i(c), P.ox[q], n, &fx);
                key_frac(cell_j(c), P.oy[q], n, &fy);
                key_frac(cell_k(c), P.oz[q], n, &fz);
                const float sx[2] = {1.f - fx, fx};
                const float sy[2] = {1.f - fy, fy};
                const float sz[2] = {1.f - fz, fz};
#pragma unroll
                for (int cz = 0; cz < 2; ++cz)
#pragma unroll
                    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                        for (int cx = 0; cx < 2; ++cx) s[cx + 2 * cy + 4 * cz] += (sx[cx] * sy[cy]) * sz[cz];
            }
#pragma unroll
            for (int c = 0; c < 8; ++c) part[c * NK + kl] = s[c];
        }
        __syncthreads();
        const float scale = d.dep_scale;
        for (int cl = threadIdx.x; cl < TX * TY * TZ; cl += blockDim.x) {
            const int ci = cl % TX, cj = (cl / TX) % TY, ck = cl / (TX * TY);
            const int i = i0 + ci, j = j0 + cj, k = k0 + ck;
            if (i >= n || j >= n || k >= n) continue;
            float acc = 0.f;
#pragma unroll
            for (int dk = 0; dk < 2; ++dk)
#pragma unroll
                for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                    for (int di = 0; di < 2; ++di) {
                        const int kl = (ci + di) + KX * ((cj + dj) + KY * (ck + dk));
                        acc += part[((1 - di) + 2 * (1 - dj) + 4 * (1 - dk)) * NK + kl];
                    }
            d.frho[cidx(i, j, k, n)] = acc * scale;
        }
    }
}

// ---------------------------------------------------------------------------
// RHS: item = (box, 8 rows); warp per row, compensated FP64 lane sums
// ---------------------------------------------------------------------------
__device__ __forceinline__ void kahan_add(double& s, double& c, double v)
{
    const double y = v - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
}

__global__ void __launch_bounds__(256) e_rowsum(const Item* __restrict__ items, int nitems,
                                                const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    const int lane = threadIdx.x & 31, wr = threadIdx.x >> 5;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        if (!S[it.box].active) continue;
        const EDesc& d = D[it.box];
        const int n = d.n;
        const long long row = (long long)it.a * 8 + wr;
        if (row >= (long long)n * n) continue;
        // double-float lane sums of the FP32 densities (k_mx_rowsum's scheme)
        const float* r = d.frho + row * n;
        float sh = 0.f, sl = 0.f;
        for (int i = lane; i < n; i += 32) {
            float err;
            df_two_sum(sh, r[i], sh, err);
            sl = __fadd_rn(sl, err);
        }
        double s = f32_to_f64(sh) + f32_to_f64(sl);
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) d.rows[row] = s - (double)n * d.mass_offset;
    }
}

// per-box mean (one block per box); also opens the solve of every active box
__global__ void e_mean(int nbox, const EDesc* __restrict__ D, EState* S, double ggrav)
{
    __shared__ double ss[32];
    const int b = blockIdx.x;
    if (b >= nbox || !S[b].active) return;
    const EDesc& d = D[b];
    const long long nr = (long long)d.n * d.n;
    double s = 0.0, c = 0.0;
    for (long long r = threadIdx.x; r < nr; r += blockDim.x) kahan_add(s, c, d.rows[r]);
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
        d.scal[0] = (t * (d.dx * d.dx * d.dx)) / (d.L * d.L * d.L);
        // e_make_beta's folded offset and scale for this solve
        d.scal[1] = d.mass_offset + d.scal[0];
        d.scal[2] = (ggrav * (1.0 / S[b].a_new)) * d.beta_scale;
        d.norms[0] = 0ULL;
        d.norms[1] = 0ULL;
        S[b].solve_active = 1;
    }
}

// beta (FP64, split) from the FP32 density; |beta| max into norms[0].
// item = (box, level 0, plane k, first row j0), block (32, R)
__global__ void __launch_bounds__(256) e_make_beta(const Item* __restrict__ items, int nitems,
                                                   const EDesc* __restrict__ D,
                                                   const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!st.active) continue;  // uniform across the block
        const EDesc& d = D[it.box];
        unsigned long long vmax = 0;
        const int n = d.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j < n) {
            const double off = d.scal[1], scale = d.scal[2];
            for (int ih = threadIdx.x; ih < half; ih += blockDim.x) {
                const long long t = ((long long)j + (long long)n * k) * half + ih;
#pragma unroll
                for (int odd = 0; odd < 2; ++odd) {
                    const int i = 2 * ih + odd;
                    const double v = f32_to_f64(d.frho[cidx(i, j, k, n)]);
                    const double bt = (v - off) * scale;
                    (((i + j + k) & 1) ? d.beta_b : d.beta_r)[t] = bt;
                    const unsigned long long u = absbits(bt);
                    vmax = u > vmax ? u : vmax;
                }
            }
        }
        warp_umax_atomic(vmax, d.norms + 0);
    }
}

// rows of level 0 per e_correct_v and e_resid_v item: enough (row, pair) tasks to fill a block
// of nthreads threads (n / 4 compact pairs per row)
__host__ __device__ inline int correct_rows(int n, int nthreads)
{
    const int pairs = n >> 2;
    const int r = pairs > 0 ? nthreads / pairs : n;
    return r < 1 ? 1 : (r > n ? n : r);
}

template <typename T>
__device__ __forceinline__ T nbr_sum_split(const T* other, int n, int half, int ih, int j, int k, int q)
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

// FP64 residual of level 0 -> FP32 inner rhs (level-0 FP32 beta) with e = 0;
// max |r| into norms[1]; boxes still iterating.  low_words: also the residual's
// low words (r - (float)r) for the double-float updates of e_correct
__global__ void __launch_bounds__(256) e_resid(const Item* __restrict__ items, int nitems,
                                               const EDesc* __restrict__ D, const EState* __restrict__ S,
                                               int low_words)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        unsigned long long vmax = 0;
        const int n = d.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j < n) {
            for (int ih = threadIdx.x; ih < half; ih += blockDim.x) {
                const long long t = ((long long)j + (long long)n * k) * half + ih;
#pragma unroll
                for (int color = 0; color < 2; ++color) {
                    const int q = (j + k + color) & 1;
                    const double* other = color ? d.phi_r : d.phi_b;
                    const double* mine = color ? d.phi_b : d.phi_r;
                    const double* beta = color ? d.beta_b : d.beta_r;
                    const double s = nbr_sum_split<double>(other, n, half, ih, j, k, q);
                    const double r = beta[t] - fma(s, kSixth, -mine[t]);
                    const float h = f64_to_f32_rn(r);
                    (color ? d.lv[0].beta_b : d.lv[0].beta_r)[t] = h;
                    if (low_words) d.r_lo[(color ? (long long)n * n * half : 0LL) + t] = f64_to_f32_rn(r - f32_to_f64(h));
                    (color ? d.lv[0].phi_b : d.lv[0].phi_r)[t] = 0.f;
                    const unsigned long long u = absbits(r);
                    vmax = u > vmax ? u : vmax;
                }
            }
        }
        warp_umax_atomic(vmax, d.norms + 1);
    }
}

// e_resid for boxes whose level-0 rows hold an even number of compact cells, on
// e_correct_v's items: one task per compact pair of one row (k_mx_resid2's
// pattern: paired FP64 loads, the neighbour sum in nbr_sum_split's order), so
// small boxes fill the block; the same bits as e_resid.
__global__ void __launch_bounds__(256, 5) e_resid_v(const Item* __restrict__ items, int nitems,
                                                 const EDesc* __restrict__ D, const EState* __restrict__ S,
                                                 int low_words)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;  // uniform across the block
        const EDesc& d = D[it.box];
        const int n = d.n, k = it.b;
        const unsigned half = (unsigned)n >> 1;
        const unsigned pairs = half >> 1;
        const unsigned nh = (unsigned)n * (unsigned)n * half;
        const int rows = correct_rows(n, nthreads);
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
        unsigned long long vmax = 0;
        for (unsigned task = tid; task < (unsigned)rows * pairs; task += nthreads) {
            const int j = it.c + (int)(task / pairs);
            if (j >= n) break;
            const unsigned ih = 2 * (task % pairs);
            const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
            const unsigned r0 = row(j, k);
            const unsigned t = r0 + ih;
#pragma unroll
            for (int color = 0; color < 2; ++color) {
                const int q = (j + k + color) & 1;
                const double* other = color ? d.phi_r : d.phi_b;
                const double* mine = color ? d.phi_b : d.phi_r;
                const double* beta = color ? d.beta_b : d.beta_r;
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
                reinterpret_cast<float2*>((color ? d.lv[0].beta_b : d.lv[0].beta_r) + t)[0] = make_float2(h0, h1);
                if (low_words)
                    reinterpret_cast<float2*>(d.r_lo + (color ? nh : 0u) + t)[0] =
                        make_float2(f64_to_f32_rn(r0v - f32_to_f64(h0)), f64_to_f32_rn(r1v - f32_to_f64(h1)));
                reinterpret_cast<float2*>((color ? d.lv[0].phi_b : d.lv[0].phi_r) + t)[0] = make_float2(0.f, 0.f);
                const unsigned long long u0 = absbits(r0v), u1 = absbits(r1v);
                vmax = u0 > vmax ? u0 : vmax;
                vmax = u1 > vmax ? u1 : vmax;
            }
        }
        warp_umax_atomic(vmax, d.norms + 1);
    }
}

// per-box convergence after a residual pass.  mode 1: after the solve's first
// residual -- set the target from ||beta|| and ||r0|| and start iterating if
// above it; 2: after a defect-correction step that recomputed r with the FP64
// stencil; 0: after a step that updated r in double-float (e_correct) -- the
// error bound grows by kDfUpdateErr * max|e| and the box stops when the tracked
// residual plus the bound meets the target
__global__ void e_flags(int nbox, const EDesc* __restrict__ D, EState* S, double rel_tol, int mode)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox) return;
    EState& st = S[b];
    if (!st.active) return;
    const EDesc& d = D[b];
    if (mode != 1 && !st.solve_active) return;
    auto bits = [](unsigned long long u) {
        double v;
        memcpy(&v, &u, sizeof(v));
        return v;
    };
    const double r = bits(d.norms[1]);
    if (mode == 1) {
        const double bn = bits(d.norms[0]);
        st.target = rel_tol * (bn > r ? bn : r);
        st.err = 0.0;
        st.outer = 0;
        st.inner = 0;
        st.solve_active = (r <= st.target) ? 0 : 1;
    } else {
        st.outer += 1;
        st.err = mode == 2 ? 0.0 : st.err + kDfUpdateErr * bits(d.norms[3]);
        if (r + st.err <= st.target) st.solve_active = 0;
    }
    d.norms[1] = 0ULL;
    d.norms[3] = 0ULL;
}

// The condition of the step graph's WHILE node: repeat while any active box is
// above its tolerance and fewer than `limit` extra iterations ran.  One block;
// inc: a loop body just ran (count it); else: the loop is about to start.
__global__ void e_loop_cond(int nbox, const EState* __restrict__ S, int* loop, int limit, int inc,
                            cudaGraphConditionalHandle h)
{
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int b = threadIdx.x; b < nbox; b += blockDim.x)
        if (S[b].active && S[b].solve_active) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        const int it = inc ? loop[0] + 1 : 0;
        loop[0] = it;
        cudaGraphSetConditional(h, (any && it < limit) ? 1u : 0u);
    }
}

__global__ void e_count_inner(int nbox, EState* S, int cycles)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox) return;
    if (S[b].active && S[b].solve_active) S[b].inner += cycles;
}

// phi += e and r -= L e in double-float on level 0 (the single-box k_mx_correct
// over item rows): the defect-correction steps after a solve's first, which
// refreshes r with the FP64 stencil (e_resid with low words); max |r| into
// norms[1]; boxes still iterating
__global__ void __launch_bounds__(256) e_correct(const Item* __restrict__ items, int nitems,
                                                 const EDesc* __restrict__ D,
                                                 const EState* __restrict__ S, float c_hi, float c_lo)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;  // uniform across the block
        const EDesc& d = D[it.box];
        const int n = d.n, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;                           // uniform across the warp
        const unsigned half = (unsigned)n >> 1;
        const unsigned nh = (unsigned)n * (unsigned)n * half;
        const float* e_r = d.lv[0].phi_r;
        const float* e_b = d.lv[0].phi_b;
        float* rh_r = d.lv[0].beta_r;
        float* rh_b = d.lv[0].beta_b;
        float* rl = d.r_lo;
        double* p_r = d.phi_r;
        double* p_b = d.phi_b;
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
        const unsigned r0 = row(j, k), rym = row(jm, k), ryp = row(jp, k), rzm = row(j, km),
                       rzp = row(j, kp);
        float vmax = 0.f, emax = 0.f;
        if ((half & 1u) == 0) {
            // two compact cells per thread: the k_mx_correct2 pattern
            for (unsigned ih = 2 * threadIdx.x; ih < half; ih += 2 * blockDim.x) {
                const unsigned t = r0 + ih;
#pragma unroll
                for (int color = 0; color < 2; ++color) {
                    const int q = (j + k + color) & 1;
                    const float* other = color ? e_r : e_b;
                    const float2 em = *reinterpret_cast<const float2*>((color ? e_b : e_r) + t);
                    const float2 cc = *reinterpret_cast<const float2*>(other + t);
                    float xm0, xm1, xp0, xp1;
                    if (q) {
                        const float e = other[r0 + (ih + 2 == half ? 0u : ih + 2)];
                        xm0 = cc.x; xp0 = cc.y; xm1 = cc.y; xp1 = e;
                    } else {
                        const float e = other[r0 + (ih == 0 ? half - 1 : ih - 1)];
                        xm0 = e; xp0 = cc.x; xm1 = cc.x; xp1 = cc.y;
                    }
                    const float2 ym = *reinterpret_cast<const float2*>(other + rym + ih);
                    const float2 yp = *reinterpret_cast<const float2*>(other + ryp + ih);
                    const float2 zm = *reinterpret_cast<const float2*>(other + rzm + ih);
                    const float2 zp = *reinterpret_cast<const float2*>(other + rzp + ih);
                    float2* rh_p = reinterpret_cast<float2*>((color ? rh_b : rh_r) + t);
                    float2* rl_p = reinterpret_cast<float2*>(rl + (color ? nh : 0u) + t);
                    float2 rh = *rh_p, rlo = *rl_p;
                    const float v0[6] = {xm0, xp0, ym.x, yp.x, zm.x, zp.x};
                    const float v1[6] = {xm1, xp1, ym.y, yp.y, zm.y, zp.y};
                    df_residual_update(v0, em.x, c_hi, c_lo, rh.x, rlo.x);
                    df_residual_update(v1, em.y, c_hi, c_lo, rh.y, rlo.y);
                    *rh_p = rh;
                    *rl_p = rlo;
                    double2* pp = reinterpret_cast<double2*>((color ? p_b : p_r) + t);
                    double2 ph = *pp;
                    ph.x = ph.x + f32_to_f64(em.x);
                    ph.y = ph.y + f32_to_f64(em.y);
                    *pp = ph;
                    vmax = fmaxf(vmax, fmaxf(fabsf(rh.x), fabsf(rh.y)));
                    emax = fmaxf(emax, fmaxf(fabsf(em.x), fabsf(em.y)));
                }
            }
        } else {
            for (unsigned ih = threadIdx.x; ih < half; ih += blockDim.x) {
                const unsigned t = r0 + ih;
#pragma unroll
                for (int color = 0; color < 2; ++color) {
                    const int q = (j + k + color) & 1;
                    const float* other = color ? e_r : e_b;
                    const float em = (color ? e_b : e_r)[t];
                    const unsigned ihm = q ? ih : (ih == 0 ? half - 1 : ih - 1);
                    const unsigned ihp = q ? (ih == half - 1 ? 0 : ih + 1) : ih;
                    const float v[6] = {other[r0 + ihm], other[r0 + ihp], other[rym + ih],
                                        other[ryp + ih], other[rzm + ih], other[rzp + ih]};
                    float* rh_p = (color ? rh_b : rh_r) + t;
                    float* rl_p = rl + (color ? nh : 0u) + t;
                    float rh = *rh_p, rlo = *rl_p;
                    df_residual_update(v, em, c_hi, c_lo, rh, rlo);
                    *rh_p = rh;
                    *rl_p = rlo;
                    double* pp = (color ? p_b : p_r) + t;
                    *pp = *pp + f32_to_f64(em);
                    vmax = fmaxf(vmax, fabsf(rh));
                    emax = fmaxf(emax, fabsf(em));
                }
            }
        }
        warp_umax_atomic(absbits(f32_to_f64(vmax)), d.norms + 1);
        warp_umax_atomic(absbits(f32_to_f64(emax)), d.norms + 3);
    }
}

// e_correct for boxes whose level-0 rows hold an even number of compact cells,
// on items {box, 0, plane k, first row j0} of correct_rows(n) rows: one task per
// compact pair of one row, so small boxes fill the block too.  The same
// arithmetic per cell as e_correct (the k_mx_correct2 pattern).
__global__ void __launch_bounds__(256) e_correct_v(const Item* __restrict__ items, int nitems,
                                                   const EDesc* __restrict__ D,
                                                   const EState* __restrict__ S, float c_hi, float c_lo)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;  // uniform across the block
        const EDesc& d = D[it.box];
        const int n = d.n, k = it.b;
        const unsigned half = (unsigned)n >> 1;
        const unsigned pairs = half >> 1;
        const unsigned nh = (unsigned)n * (unsigned)n * half;
        const int rows = correct_rows(n, nthreads);
        const float* e_r = d.lv[0].phi_r;
        const float* e_b = d.lv[0].phi_b;
        float* rh_r = d.lv[0].beta_r;
        float* rh_b = d.lv[0].beta_b;
        float* rl = d.r_lo;
        double* p_r = d.phi_r;
        double* p_b = d.phi_b;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
        float vmax = 0.f, emax = 0.f;
        for (unsigned task = tid; task < (unsigned)rows * pairs; task += nthreads) {
            const int j = it.c + (int)(task / pairs);
            if (j >= n) break;                           // later tasks lie further down
            const unsigned ih = 2 * (task % pairs);
            const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
            const unsigned r0 = row(j, k), rym = row(jm, k), ryp = row(jp, k), rzm = row(j, km),
                           rzp = row(j, kp);
            const unsigned t = r0 + ih;
#pragma unroll
            for (int color = 0; color < 2; ++color) {
                const int q = (j + k + color) & 1;
                const float* other = color ? e_r : e_b;
                const float2 em = *reinterpret_cast<const float2*>((color ? e_b : e_r) + t);
                const float2 cc = *reinterpret_cast<const float2*>(other + t);
                float xm0, xm1, xp0, xp1;
                if (q) {
                    const float e = other[r0 + (ih + 2 == half ? 0u : ih + 2)];
                    xm0 = cc.x; xp0 = cc.y; xm1 = cc.y; xp1 = e;
                } else {
                    const float e = other[r0 + (ih == 0 ? half - 1 : ih - 1)];
                    xm0 = e; xp0 = cc.x; xm1 = cc.x; xp1 = cc.y;
                }
                const float2 ym = *reinterpret_cast<const float2*>(other + rym + ih);
                const float2 yp = *reinterpret_cast<const float2*>(other + ryp + ih);
                const float2 zm = *reinterpret_cast<const float2*>(other + rzm + ih);
                const float2 zp = *reinterpret_cast<const float2*>(other + rzp + ih);
                float2* rh_p = reinterpret_cast<float2*>((color ? rh_b : rh_r) + t);
                float2* rl_p = reinterpret_cast<float2*>(rl + (color ? nh : 0u) + t);
                float2 rh = *rh_p, rlo = *rl_p;
                const float v0[6] = {xm0, xp0, ym.x, yp.x, zm.x, zp.x};
                const float v1[6] = {xm1, xp1, ym.y, yp.y, zm.y, zp.y};
                df_residual_update(v0, em.x, c_hi, c_lo, rh.x, rlo.x);
                df_residual_update(v1, em.y, c_hi, c_lo, rh.y, rlo.y);
                *rh_p = rh;
                *rl_p = rlo;
                double2* pp = reinterpret_cast<double2*>((color ? p_b : p_r) + t);
                double2 ph = *pp;
                ph.x = ph.x + f32_to_f64(em.x);
                ph.y = ph.y + f32_to_f64(em.y);
                *pp = ph;
                vmax = fmaxf(vmax, fmaxf(fabsf(rh.x), fabsf(rh.y)));
                emax = fmaxf(emax, fmaxf(fabsf(em.x), fabsf(em.y)));
            }
        }
        warp_umax_atomic(absbits(f32_to_f64(vmax)), d.norms + 1);
        warp_umax_atomic(absbits(f32_to_f64(emax)), d.norms + 3);
    }
}

// e = 0 on level 0 for the next inner solve (after e_correct), boxes still
// iterating whose level 0 is cycled by e_tail
__global__ void __launch_bounds__(256) e_zero_inner(const Item* __restrict__ items, int nitems,
                                                    const EDesc* __restrict__ D,
                                                    const EState* __restrict__ S, int all)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        if (!all && d.tail_l != 0) continue;   // the others start with e_gsrb_zero
        const int n = d.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;
        for (int ih = threadIdx.x; ih < half; ih += blockDim.x) {
            const long long t = ((long long)j + (long long)n * k) * half + ih;
            d.lv[0].phi_r[t] = 0.f;
            d.lv[0].phi_b[t] = 0.f;
        }
    }
}

// The opening red half sweep of an inner solve on level 0, whose correction
// starts at 0: fmaf(0, 1/6, -beta) per red cell (the general sweep's value with
// every black neighbour 0), so e needs no zeroing between defect-correction
// steps.  Boxes whose level 0 is cycled by e_tail are zeroed by e_zero_inner.
__global__ void __launch_bounds__(256) e_gsrb_zero(const Item* __restrict__ items, int nitems,
                                                   const EDesc* __restrict__ D,
                                                   const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState& st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        if (d.tail_l == 0) continue;
        const int n = d.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;
        const long long row = ((long long)j + (long long)n * k) * half;
        for (int ih = threadIdx.x; ih < half; ih += blockDim.x)
            d.lv[0].phi_r[row + ih] = fmaf(0.f, kSixthF, -d.lv[0].beta_r[row + ih]);
    }
}

// e_gsrb_zero on e_correct_v's items: the plane segment's red cells are one
// contiguous range of the level-0 red array, taken four at a time (level-0 rows
// of a multiple of four compact cells; else one at a time); the same values.
__global__ void __launch_bounds__(256) e_gsrb_zero_v(const Item* __restrict__ items, int nitems,
                                                     const EDesc* __restrict__ D,
                                                     const EState* __restrict__ S)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        if (d.tail_l == 0) continue;
        const int n = d.n, k = it.b;
        const unsigned half = (unsigned)n >> 1;
        const int rows = min(correct_rows(n, nthreads), n - it.c);
        const unsigned begin = ((unsigned)it.c + (unsigned)n * (unsigned)k) * half;
        const unsigned cnt = (unsigned)rows * half;
        float* phi = d.lv[0].phi_r + begin;
        const float* beta = d.lv[0].beta_r + begin;
        if ((half & 3u) == 0) {
            for (unsigned q = tid; q < cnt / 4; q += nthreads) {
                const float4 b = __ldg(reinterpret_cast<const float4*>(beta) + q);
                reinterpret_cast<float4*>(phi)[q] = make_float4(fmaf(0.f, kSixthF, -b.x), fmaf(0.f, kSixthF, -b.y),
                                                                fmaf(0.f, kSixthF, -b.z), fmaf(0.f, kSixthF, -b.w));
            }
        } else {
            for (unsigned q = tid; q < cnt; q += nthreads) phi[q] = fmaf(0.f, kSixthF, -beta[q]);
        }
    }
}

// phi += e on level 0 (split), boxes still iterating
__global__ void __launch_bounds__(256) e_update(const Item* __restrict__ items, int nitems,
                                                const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const int n = d.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;
        for (int ih = threadIdx.x; ih < half; ih += blockDim.x) {
            const long long t = ((long long)j + (long long)n * k) * half + ih;
            d.phi_r[t] = d.phi_r[t] + f32_to_f64(d.lv[0].phi_r[t]);
            d.phi_b[t] = d.phi_b[t] + f32_to_f64(d.lv[0].phi_b[t]);
        }
    }
}

// ---------------------------------------------------------------------------
// FP32 V-cycle kernels over level rows
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) e_gsrb(const Item* __restrict__ items, int nitems,
                                              const EDesc* __restrict__ D, const EState* __restrict__ S,
                                              int color)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& L = d.lv[it.a];
        const int n = L.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;
        float* mine = color ? L.phi_b : L.phi_r;
        const float* other = color ? L.phi_r : L.phi_b;
        const float* beta = color ? L.beta_b : L.beta_r;
        const int q = (j + k + color) & 1;
        for (int ih = threadIdx.x; ih < half; ih += blockDim.x) {
            const long long t = ((long long)j + (long long)n * k) * half + ih;
            const float s = nbr_sum_split<float>(other, n, half, ih, j, k, q);
            mine[t] = fmaf(s, kSixthF, -beta[t]);
        }
    }
}

// The same half sweep for levels whose compact rows hold a multiple of four
// cells: four cells per thread, one 16-byte load per neighbour row.  The
// item's rows are sized so that (rows x half/4) fills the block; the sums are
// e_gsrb's, term for term, so the results are bitwise the same.
__host__ __device__ inline int vec_rows(int n, int nthreads)
{
    const int h4 = (n >> 1) >> 2;
    const int r = nthreads / h4;
    return r < 1 ? 1 : (r > n ? n : r);
}

// Items of this kernel cover kMarchE consecutive planes (k0 = it.b): each task
// marches over them, so the row of the plane above becomes this plane's row and
// then the one below, and each plane loads three neighbour rows, the right-hand
// side and one edge value.  32-bit offsets (a level has at most 1024^3 / 2
// cells of a colour).  Levels with half % 4 == 0 have n % 8 == 0, so every item
// holds exactly kMarchE planes.
constexpr int kMarchE = 4;

__global__ void __launch_bounds__(256, 6) e_gsrb4(const Item* __restrict__ items, int nitems,
                                               const EDesc* __restrict__ D,
                                               const EState* __restrict__ S, int color)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& L = d.lv[it.a];
        const int n = L.n;
        const unsigned half = (unsigned)n >> 1, h4 = half >> 2, plane = (unsigned)n * half;
        const int k0 = it.b;
        const int rows = vec_rows(n, nthreads);
        float4* m4 = reinterpret_cast<float4*>(color ? L.phi_b : L.phi_r);
        const float* other = color ? L.phi_r : L.phi_b;
        const float4* o4 = reinterpret_cast<const float4*>(other);
        const float4* b4 = reinterpret_cast<const float4*>(color ? L.beta_b : L.beta_r);
        for (int task = tid; task < rows * (int)h4; task += nthreads) {
            const int r = task / (int)h4, t4 = task - r * (int)h4;
            const int j = it.c + r;
            if (j >= n) continue;
            const unsigned ih = 4 * (unsigned)t4;
            const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
            const unsigned rj = (unsigned)j * half + ih, rjm = (unsigned)jm * half + ih,
                           rjp = (unsigned)jp * half + ih;
            const int kfirst = k0 == 0 ? n - 1 : k0 - 1;
            float4 zm = __ldg(o4 + (((unsigned)kfirst * plane + rj) >> 2));
            float4 c = __ldg(o4 + (((unsigned)k0 * plane + rj) >> 2));
#pragma unroll
            for (int kk = 0; kk < kMarchE; ++kk) {
                const int k = k0 + kk;
                const int kp = k == n - 1 ? 0 : k + 1;
                const unsigned pk = (unsigned)k * plane;
                const float4 zp = __ldg(o4 + (((unsigned)kp * plane + rj) >> 2));
                const float4 ym = __ldg(o4 + ((pk + rjm) >> 2));
                const float4 yp = __ldg(o4 + ((pk + rjp) >> 2));
                const unsigned t = pk + rj;
                const float4 b = __ldg(b4 + (t >> 2));
                const int q = (j + k + color) & 1;
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
                float4 o;
                o.x = fmaf(((((xm0 + xp0) + ym.x) + yp.x) + zm.x) + zp.x, kSixthF, -b.x);
                o.y = fmaf(((((xm1 + xp1) + ym.y) + yp.y) + zm.y) + zp.y, kSixthF, -b.y);
                o.z = fmaf(((((xm2 + xp2) + ym.z) + yp.z) + zm.z) + zp.z, kSixthF, -b.z);
                o.w = fmaf(((((xm3 + xp3) + ym.w) + yp.w) + zm.w) + zp.w, kSixthF, -b.w);
                m4[t >> 2] = o;
                zm = c;
                c = zp;
            }
        }
    }
}

__device__ __forceinline__ float resid_f(const ELevel& L, int i, int j, int k)
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

// item level = the coarse level; rows of the coarse level (natural coordinates)
__global__ void __launch_bounds__(256) e_restrict(const Item* __restrict__ items, int nitems,
                                                  const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& F = d.lv[it.a - 1];
        const ELevel& C = d.lv[it.a];
        const int nc = C.n, K = it.b;
        const int J = it.c + threadIdx.y;
        if (J >= nc) continue;
        for (int I = threadIdx.x; I < nc; I += blockDim.x) {
            float s = 0.f;
#pragma unroll
            for (int dk = 0; dk < 2; ++dk)
#pragma unroll
                for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                    for (int di = 0; di < 2; ++di) s += resid_f(F, 2 * I + di, 2 * J + dj, 2 * K + dk);
            *lv_ptr<float>(C.beta_r, C.beta_b, nc, C.split, I, J, K) = s * 0.5f;
            *lv_ptr<float>(C.phi_r, C.phi_b, nc, C.split, I, J, K) = 0.f;
        }
    }
}

// The residual of four fine cells of one fine row (i = 4t .. 4t+3) of a split
// level with half % 4 == 0, as resid_f computes each of them: in a row of parity
// p the cells are colour p at compact 2t, colour 1-p at 2t, colour p at 2t+1 and
// colour 1-p at 2t+1, so each colour array gives an 8-byte pair per row.
__device__ __forceinline__ void fine_row_resid(const ELevel& F, int j, int k, unsigned t, float r[4])
{
    const int n = F.n;
    const unsigned half = (unsigned)n >> 1;
    const int p = (j + k) & 1;
    const float* Pp = p ? F.phi_b : F.phi_r;
    const float* Pq = p ? F.phi_r : F.phi_b;
    const float* Bp = p ? F.beta_b : F.beta_r;
    const float* Bq = p ? F.beta_r : F.beta_b;
    const unsigned c2 = 2 * t;
    auto row = [&](int jj, int kk) -> unsigned { return ((unsigned)jj + (unsigned)n * (unsigned)kk) * half; };
    const unsigned r0 = row(j, k);
    const float2 ep = __ldg(reinterpret_cast<const float2*>(Pp + r0 + c2));
    const float2 eq = __ldg(reinterpret_cast<const float2*>(Pq + r0 + c2));
    const float left = __ldg(Pq + r0 + (c2 == 0 ? half - 1 : c2 - 1));
    const float right = __ldg(Pp + r0 + (c2 + 2 == half ? 0u : c2 + 2));
    const float2 bp = __ldg(reinterpret_cast<const float2*>(Bp + r0 + c2));
    const float2 bq = __ldg(reinterpret_cast<const float2*>(Bq + r0 + c2));
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
    const unsigned nr[4] = {row(jm, k), row(jp, k), row(j, km), row(j, kp)};
    float2 ne[4], no[4];
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

// e_restrict for boxes whose fine level allows the paired loads (fine
// half % 4 == 0): two coarse cells per task, on e_restrict's row items.  The
// coarse sums add the fine residuals in e_restrict's order.
__global__ void __launch_bounds__(256) e_restrict4(const Item* __restrict__ items, int nitems,
                                                   const EDesc* __restrict__ D,
                                                   const EState* __restrict__ S)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int R = blockDim.y;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& F = d.lv[it.a - 1];
        const ELevel& C = d.lv[it.a];
        const int nc = C.n, K = it.b;
        const int npair = nc >> 1;
        for (int task = tid; task < R * npair; task += nthreads) {
            const int rr = task / npair, t = task - rr * npair;
            const int J = it.c + rr;
            if (J >= nc) continue;
            float r[2][2][4];
#pragma unroll
            for (int dk = 0; dk < 2; ++dk)
#pragma unroll
                for (int dj = 0; dj < 2; ++dj) fine_row_resid(F, 2 * J + dj, 2 * K + dk, (unsigned)t, r[dk][dj]);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                float s = 0.f;
#pragma unroll
                for (int dk = 0; dk < 2; ++dk)
#pragma unroll
                    for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                        for (int di = 0; di < 2; ++di) s += r[dk][dj][2 * u + di];
                const int I = 2 * t + u;
                *lv_ptr<float>(C.beta_r, C.beta_b, nc, C.split, I, J, K) = s * 0.5f;
                *lv_ptr<float>(C.phi_r, C.phi_b, nc, C.split, I, J, K) = 0.f;
            }
        }
    }
}

// e_restrict4 after pre-smoothing (the last half sweep black): the coarse
// right-hand side from the 4 red children of each coarse cell, whose residuals
// are the only ones above round-off (pm_restrict.cuh, as k_restrict_f4_red),
// summed in (dk, dj) order; half the loads and residual arithmetic.
__global__ void __launch_bounds__(256, 5) e_restrict4_red(const Item* __restrict__ items, int nitems,
                                                       const EDesc* __restrict__ D,
                                                       const EState* __restrict__ S)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int R = blockDim.y;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& F = d.lv[it.a - 1];
        const ELevel& C = d.lv[it.a];
        const int nc = C.n, K = it.b;
        const int npair = nc >> 1;
        for (int task = tid; task < R * npair; task += nthreads) {
            const int rr = task / npair, t = task - rr * npair;
            const int J = it.c + rr;
            if (J >= nc) continue;
            float r[2][2][2];
#pragma unroll
            for (int dk = 0; dk < 2; ++dk)
#pragma unroll
                for (int dj = 0; dj < 2; ++dj) fine_row_resid_red(F, 2 * J + dj, 2 * K + dk, (unsigned)t, r[dk][dj]);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                float s = 0.f;
#pragma unroll
                for (int dk = 0; dk < 2; ++dk)
#pragma unroll
                    for (int dj = 0; dj < 2; ++dj) s += r[dk][dj][u];
                const int I = 2 * t + u;
                *lv_ptr<float>(C.beta_r, C.beta_b, nc, C.split, I, J, K) = s * 0.5f;
                *lv_ptr<float>(C.phi_r, C.phi_b, nc, C.split, I, J, K) = 0.f;
            }
        }
    }
}

// item level = the fine level (split); rows of the fine level
// black: only the black fine cells take the correction (post-smoothing follows
// and overwrites the red ones unread; the same bits)
__global__ void __launch_bounds__(256) e_prolong(const Item* __restrict__ items, int nitems,
                                                 const EDesc* __restrict__ D, const EState* __restrict__ S,
                                                 int black)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& F = d.lv[it.a];
        const ELevel& C = d.lv[it.a + 1];
        const int n = F.n, nc = C.n, half = n >> 1, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;
        const int J = j >> 1, K = k >> 1;
        const int Js[2] = {J, wrap1((j & 1) ? J + 1 : J - 1, nc)};
        const int Ks[2] = {K, wrap1((k & 1) ? K + 1 : K - 1, nc)};
        for (int ih = threadIdx.x; ih < half; ih += blockDim.x) {
            const long long t = ((long long)j + (long long)n * k) * half + ih;
#pragma unroll
            for (int odd = 0; odd < 2; ++odd) {
                const int i = 2 * ih + odd;
                if (black && ((i + j + k) & 1) == 0) continue;
                const int Is[2] = {ih, wrap1(odd ? ih + 1 : ih - 1, nc)};
                float s = 0.f;
#pragma unroll
                for (int b = 0; b < 2; ++b)
#pragma unroll
                    for (int a = 0; a < 2; ++a)
#pragma unroll
                        for (int tt = 0; tt < 2; ++tt)
                            s = fmaf(kProlongWE[tt + 2 * a + 4 * b],
                                     *lv_ptr<const float>(C.phi_r, C.phi_b, nc, C.split, Is[tt], Js[a], Ks[b]), s);
                float* p = (((i + j + k) & 1) ? F.phi_b : F.phi_r) + t;
                *p += s;
            }
        }
    }
}

// The prolongation on the smoother's vectorised items: four compact columns
// (eight fine cells) per task where the coarse level is split too (the six
// coarse x-neighbours of each (J', K') row are a pair plus one in each colour
// array), otherwise one column per task as e_prolong.  Same sums, same order.
__global__ void __launch_bounds__(256) e_prolong4(const Item* __restrict__ items, int nitems,
                                                  const EDesc* __restrict__ D,
                                                  const EState* __restrict__ S, int black)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const EDesc& d = D[it.box];
        const ELevel& F = d.lv[it.a];
        const ELevel& C = d.lv[it.a + 1];
        const int n = F.n, nc = C.n, half = n >> 1, h4 = half >> 2, k = it.b;
        const int rows = vec_rows(n, nthreads);
        const int K = k >> 1;
        const int Ks[2] = {K, wrap1((k & 1) ? K + 1 : K - 1, nc)};
        if (!C.split) {
            for (int task = tid; task < rows * half; task += nthreads) {
                const int r = task / half, ih = task - r * half;
                const int j = it.c + r;
                if (j >= n) continue;
                const int J = j >> 1;
                const int Js[2] = {J, wrap1((j & 1) ? J + 1 : J - 1, nc)};
                const long long t = ((long long)j + (long long)n * k) * half + ih;
#pragma unroll
                for (int odd = 0; odd < 2; ++odd) {
                    const int i = 2 * ih + odd;
                    if (black && ((i + j + k) & 1) == 0) continue;
                    const int Is[2] = {ih, wrap1(odd ? ih + 1 : ih - 1, nc)};
                    float s = 0.f;
#pragma unroll
                    for (int b = 0; b < 2; ++b)
#pragma unroll
                        for (int a = 0; a < 2; ++a)
#pragma unroll
                            for (int tt = 0; tt < 2; ++tt)
                                s = fmaf(kProlongWE[tt + 2 * a + 4 * b],
                                         *lv_ptr<const float>(C.phi_r, C.phi_b, nc, C.split, Is[tt], Js[a],
                                                              Ks[b]),
                                         s);
                    float* p = (((i + j + k) & 1) ? F.phi_b : F.phi_r) + t;
                    *p += s;
                }
            }
            continue;
        }
        const unsigned chalf = (unsigned)nc >> 1;
        for (int task = tid; task < rows * h4; task += nthreads) {
            const int r = task / h4, t4 = task - r * h4;
            const int j = it.c + r;
            if (j >= n) continue;
            const int J = j >> 1;
            const int Js[2] = {J, wrap1((j & 1) ? J + 1 : J - 1, nc)};
            const unsigned c2 = 2 * (unsigned)t4;
            float v[2][2][6];
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const unsigned row = ((unsigned)Js[a] + (unsigned)nc * (unsigned)Ks[b]) * chalf;
                    const bool even_red = ((Js[a] + Ks[b]) & 1) == 0;
                    const float* ev = even_red ? C.phi_r : C.phi_b;
                    const float* od = even_red ? C.phi_b : C.phi_r;
                    const float2 e01 = __ldg(reinterpret_cast<const float2*>(ev + row + c2));
                    const float e2 = __ldg(ev + row + (c2 + 2 == chalf ? 0u : c2 + 2));
                    const float2 o01 = __ldg(reinterpret_cast<const float2*>(od + row + c2));
                    const float om = __ldg(od + row + (c2 == 0 ? chalf - 1 : c2 - 1));
                    v[b][a][0] = om;
                    v[b][a][1] = e01.x;
                    v[b][a][2] = o01.x;
                    v[b][a][3] = e01.y;
                    v[b][a][4] = o01.y;
                    v[b][a][5] = e2;
                }
            float s0[4], s1[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float se = 0.f, so = 0.f;
#pragma unroll
                for (int b = 0; b < 2; ++b)
#pragma unroll
                    for (int a = 0; a < 2; ++a) {
                        se = fmaf(kProlongWE[0 + 2 * a + 4 * b], v[b][a][q + 1], se);
                        se = fmaf(kProlongWE[1 + 2 * a + 4 * b], v[b][a][q], se);
                        so = fmaf(kProlongWE[0 + 2 * a + 4 * b], v[b][a][q + 1], so);
                        so = fmaf(kProlongWE[1 + 2 * a + 4 * b], v[b][a][q + 2], so);
                    }
                s0[q] = se;
                s1[q] = so;
            }
            const unsigned t = ((unsigned)j + (unsigned)n * (unsigned)k) * (unsigned)half + 4 * (unsigned)t4;
            const bool even_fine_red = ((j + k) & 1) == 0;
            float4* fe = reinterpret_cast<float4*>(even_fine_red ? F.phi_r : F.phi_b) + (t >> 2);
            float4* fo = reinterpret_cast<float4*>(even_fine_red ? F.phi_b : F.phi_r) + (t >> 2);
            if (!black || !even_fine_red) {
                float4 pe = *fe;
                pe.x += s0[0]; pe.y += s0[1]; pe.z += s0[2]; pe.w += s0[3];
                *fe = pe;
            }
            if (!black || even_fine_red) {
                float4 po = *fo;
                po.x += s1[0]; po.y += s1[1]; po.z += s1[2]; po.w += s1[3];
                *fo = po;
            }
        }
    }
}

// coarse rows per item of e_prolong4_black: rows x h4 tasks fill a 256-thread block
__host__ __device__ inline int quad_rows(int n)
{
    const int h4 = n >> 3;
    const int r = 256 / h4;
    return r < 1 ? 1 : (r > (n >> 1) ? (n >> 1) : r);
}

// The black-only prolongation (post-smoothing follows) with four fine rows per
// task (pm_prolong.cuh), on items {box, fine level a, coarse plane K = b, first
// coarse row J0 = c}: fine levels whose compact rows hold a multiple of four
// cells, over a split coarse level.  The same bits as e_prolong4.
__global__ void __launch_bounds__(256, 4) e_prolong4_black(const Item* __restrict__ items, int nitems,
                                                          const EDesc* __restrict__ D,
                                                          const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        const EState st = S[it.box];
        if (!(st.active && st.solve_active)) continue;
        const ELevel F = D[it.box].lv[it.a];
        const ELevel C = D[it.box].lv[it.a + 1];
        const int h4 = F.n >> 3, nc = C.n;
        const int rows = quad_rows(F.n);
        for (int task = threadIdx.x; task < rows * h4; task += blockDim.x) {
            const int r = task / h4, t4 = task - r * h4;
            const int J = it.c + r;
            if (J >= nc) continue;
            prolong_black_quad(C, F, J, it.b, (unsigned)t4);
        }
    }
}

// the coarse end of every box's V-cycle (levels tail_l .. bottom), one CTA per
// box: the per-pass kernels' arithmetic (pm_tail.cuh), so the same bits
__global__ void __launch_bounds__(kTailThreads) e_tail(int nbox, const EDesc* __restrict__ D,
                                                       const EState* __restrict__ S, int nu1, int nu2)
{
    __shared__ float r[kMaxBottom * kMaxBottom * kMaxBottom];
    __shared__ float g[kMaxBottom * kMaxBottom * kMaxBottom];
    const int b = blockIdx.x;
    if (b >= nbox) return;
    if (!(S[b].active && S[b].solve_active)) return;
    const EDesc& d = D[b];
    LevelViewF lv[kMaxTail];
    const int nl = d.nlev - d.tail_l;
    for (int l = 0; l < nl; ++l) {
        const ELevel& e = d.lv[d.tail_l + l];
        lv[l] = LevelViewF{e.n, e.split, e.phi_r, e.phi_b, e.beta_r, e.beta_b};
    }
    vcycle_tail<float>(lv, nl, nu1, nu2, d.Gf, d.nb, r, g, nu1 > 0);
}

// FP32 gravity vector from the FP64 phi (level-0 rows, natural coordinates)
__global__ void __launch_bounds__(256) e_grav(const Item* __restrict__ items, int nitems,
                                              const EDesc* __restrict__ D, const EState* __restrict__ S)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const Item it = items[w];
        if (!S[it.box].active) continue;
        const EDesc& d = D[it.box];
        const int n = d.n, k = it.b;
        const int j = it.c + threadIdx.y;
        if (j >= n) continue;
        const long long nc = (long long)n * n * n;
        const float hdxi = (float)(0.5 * d.dxi);
        const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
        const int km = k == 0 ? n - 1 : k - 1, kp = k == n - 1 ? 0 : k + 1;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int im = i == 0 ? n - 1 : i - 1, ip = i == n - 1 ? 0 : i + 1;
            auto P = [&](int a, int b2, int c2) {
                return *lv_ptr<const double>(d.phi_r, d.phi_b, n, 1, a, b2, c2);
            };
            const long long c = cidx(i, j, k, n);
            reinterpret_cast<float4*>(d.g32)[c] =
                make_float4(f64_to_f32_rn(P(ip, j, k) - P(im, j, k)) * hdxi,
                            f64_to_f32_rn(P(i, jp, k) - P(i, jm, k)) * hdxi,
                            f64_to_f32_rn(P(i, j, kp) - P(i, j, km)) * hdxi, 0.f);
        }
    }
}

__global__ void e_phi_to_natural(int n, const double* __restrict__ pr, const double* __restrict__ pb,
                                 double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    out[cidx(i, j, k, n)] = *lv_ptr<const double>(pr, pb, n, 1, i, j, k);
}

// the float4-per-cell FP32 gravity vector as 3 component-major FP64 arrays
__global__ void e_g32_to_double(long long nc, const float* __restrict__ a, double* b)
{
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc) return;
    const float4 g = reinterpret_cast<const float4*>(a)[t];
    b[t] = g.x;
    b[nc + t] = g.y;
    b[2 * nc + t] = g.z;
}

// ---------------------------------------------------------------------------
// device arena: first-fit sub-allocator over one cudaMalloc (256-byte granules)
// ---------------------------------------------------------------------------
class Arena {
public:
    void* base = nullptr;
    size_t bytes = 0;
    std::map<size_t, size_t> free_;   // offset -> size
    std::map<size_t, size_t> used_;   // offset -> size

    bool init(size_t b)
    {
        bytes = (b + 255) & ~size_t(255);
        if (bytes == 0 || cudaMalloc(&base, bytes) != cudaSuccess) {
            cudaGetLastError();
            base = nullptr;
            return false;
        }
        free_[0] = bytes;
        return true;
    }
    void* alloc(size_t b)
    {
        b = (b + 255) & ~size_t(255);
        if (b == 0) b = 256;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= b) {
                const size_t off = it->first, sz = it->second;
                free_.erase(it);
                if (sz > b) free_[off + b] = sz - b;
                used_[off] = b;
                return static_cast<char*>(base) + off;
            }
        }
        return nullptr;
    }
    void release(void* p)
    {
        if (!p) return;
        const size_t off = static_cast<char*>(p) - static_cast<char*>(base);
        auto u = used_.find(off);
        if (u == used_.end()) return;
        size_t sz = u->second, o = off;
        used_.erase(u);
        auto nx = free_.lower_bound(o);
        if (nx != free_.end() && o + sz == nx->first) {
            sz += nx->second;
            free_.erase(nx);
        }
        auto pv = free_.lower_bound(o);
        if (pv != free_.begin()) {
            --pv;
            if (pv->first + pv->second == o) {
                o = pv->first;
                sz += pv->second;
                free_.erase(pv);
            }
        }
        free_[o] = sz;
    }
    size_t used_bytes() const
    {
        size_t s = 0;
        for (auto& kv : used_) s += kv.second;
        return s;
    }
    void destroy()
    {
        if (base) cudaFree(base);
        base = nullptr;
    }
};

int ens_bottom_edge(int n)
{
    int m = n;
    while (m % 2 == 0 && m > kCoarsenAbove) m /= 2;
    return m;
}

int ens_levels(int n)
{
    int L = 1, m = n;
    while (m % 2 == 0 && m > kCoarsenAbove) {
        m /= 2;
        ++L;
    }
    return L;
}

}  // namespace

struct EnsSlot {
    int used = 0;
    int uploaded = 0;
    int init_pending = 0;
    int fresh = 1;                    // device state not yet reset
    std::vector<void*> blocks;
    EDesc desc{};
};

}  // namespace nyxpm

struct nyxpm_ensemble {
    nyxpm::Arena arena;
    std::vector<nyxpm::EnsSlot> slots;
    int dirty = 1;                    // membership or tuning changed: tables and graphs stale
    struct Range {
        int off = 0, cnt = 0;
    };
    nyxpm::Item* d_items = nullptr;
    size_t items_cap = 0;
    Range r_part, r_scan, r_keys, r_tile, r_rows_rho;
    Range r_rows_split[nyxpm::kMaxLev];   // rows of split levels (compact extent)
    Range r_rows_nat[nyxpm::kMaxLev];     // rows of levels >= 1 (natural coordinates)
    // the smoother's items: levels whose compact rows hold a multiple of four
    // cells take the vectorised kernel (row groups sized to fill a block), the
    // others the row items above
    Range r_smooth_vec[nyxpm::kMaxLev];
    Range r_smooth_row[nyxpm::kMaxLev];
    // the vectorised smoother's items: the same row groups, kMarchE planes each
    Range r_smooth_march[nyxpm::kMaxLev];
    // the restriction's coarse-row items, split the same way by the fine level
    Range r_restrict_vec[nyxpm::kMaxLev];
    Range r_restrict_row[nyxpm::kMaxLev];
    // the black-only prolongation's items (nyxpm_tuning.prolong_quad): four fine
    // rows per task where the coarse level is split, e_prolong4's items elsewhere
    Range r_prolong_quad[nyxpm::kMaxLev];
    Range r_prolong_rest[nyxpm::kMaxLev];
    // e_correct's items: level-0 plane segments of correct_rows rows for boxes
    // whose rows hold an even number of compact cells, rows of r_rows_split[0]
    // for the others
    Range r_correct_vec, r_correct_rest;
    nyxpm::EDesc* d_desc = nullptr;
    nyxpm::EState* d_state = nullptr;
    nyxpm::EStep* d_step = nullptr;
    nyxpm::EStep* h_step = nullptr;       // pinned, the step graph's source
    nyxpm::EStep* h_init = nullptr;       // pinned, the init pass's source
    nyxpm::EState* h_state = nullptr;     // pinned, state read back
    unsigned long long* h_scratch = nullptr;  // pinned
    int cap = 0;
    int max_lev = 0;
    nyxpm_tuning tune{};
    cudaGraphExec_t exec_solve = nullptr, exec_finish = nullptr;
    int sm = 0;
    int64_t graph_launches_solve = 0, graph_launches_finish = 0;
    // the whole step as one graph (conditional WHILE node for the extra iterations)
    cudaGraphExec_t exec_step = nullptr;
    int64_t graph_launches_step = 0;   // launches of the graph without the loop body's
    int64_t graph_launches_body = 0;   // launches of one loop body
    int single_graph_failed = 0;       // the runtime refused it: the two graphs from then on
    cudaStream_t body_stream = nullptr;// captures the loop body
    int* d_loop = nullptr;             // [0] loop iterations of the last step
};

using namespace nyxpm;

namespace {

nyxpm_status efail(nyxpm_ctx* c, nyxpm_status st, const char* msg)
{
    if (c) c->err = msg;
    return st;
}

nyxpm_status echeck(nyxpm_ctx* c, const char* what)
{
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return NYXPM_OK;
    c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return NYXPM_CUDA_ERROR;
}

#define ETRY(expr)                                                                           \
    do {                                                                                     \
        nyxpm_status _st = (expr);                                                           \
        if (_st != NYXPM_OK) return _st;                                                     \
    } while (0)

unsigned pgrid(nyxpm_ensemble* E, int nitems, int per_sm = 8)
{
    const int cap = E->sm * per_sm;
    return (unsigned)std::max(1, std::min(nitems, cap));
}

void invalidate_graphs(nyxpm_ensemble* E)
{
    if (E->exec_solve) cudaGraphExecDestroy(E->exec_solve);
    if (E->exec_finish) cudaGraphExecDestroy(E->exec_finish);
    if (E->exec_step) cudaGraphExecDestroy(E->exec_step);
    E->exec_solve = E->exec_finish = E->exec_step = nullptr;
}

bool slot_ok(nyxpm_ensemble* E, int slot)
{
    return slot >= 0 && slot < (int)E->slots.size() && E->slots[slot].used;
}

// rebuild work tables and push descriptors after a membership or tuning change
nyxpm_status rebuild(nyxpm_ctx* c, nyxpm_ensemble* E)
{
    std::vector<Item> items;
    const int nbox = (int)E->slots.size();
    const int R = E->tune.smooth_rows;
    E->max_lev = 0;
    for (auto& s : E->slots)
        if (s.used) E->max_lev = std::max(E->max_lev, s.desc.nlev);
    // first level of each box's fused coarse V-cycle: the first of at most
    // mg_fused_edge cells per edge (at most kMaxTail levels), else the bottom
    for (auto& s : E->slots) {
        if (!s.used) continue;
        EDesc& d = s.desc;
        d.tail_l = d.nlev - 1;
        if (c->p.mg_fused_edge > 0)
            for (int l = std::max(0, d.nlev - kMaxTail); l < d.nlev; ++l)
                if (d.lv[l].n <= c->p.mg_fused_edge) {
                    d.tail_l = l;
                    break;
                }
    }
    auto begin = [&](nyxpm_ensemble::Range& r) { r.off = (int)items.size(); };
    auto end = [&](nyxpm_ensemble::Range& r) { r.cnt = (int)items.size() - r.off; };
    begin(E->r_part);
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        if (!s.used) continue;
        const long long bk = E->tune.sort_bucket;
        for (long long ch = 0; ch < (s.desc.np + bk - 1) / bk; ++ch) items.push_back(Item{b, (int)ch, 0, 0});
    }
    end(E->r_part);
    begin(E->r_scan);
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        if (!s.used) continue;
        const long long nc = (long long)s.desc.n * s.desc.n * s.desc.n;
        for (long long t = 0; t < (nc + kScanTile - 1) / kScanTile; ++t) items.push_back(Item{b, (int)t, 0, 0});
    }
    end(E->r_scan);
    begin(E->r_keys);
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        if (!s.used) continue;
        const long long nc = (long long)s.desc.n * s.desc.n * s.desc.n;
        for (long long t = 0; t < (nc + 255) / 256; ++t) items.push_back(Item{b, (int)t, 0, 0});
    }
    end(E->r_keys);
    int TX = 8, TY = 8, TZ = 8;
    if (E->tune.deposit_tile == 1) TZ = 4;
    if (E->tune.deposit_tile == 2) {
        TX = 16;
        TZ = 4;
    }
    begin(E->r_tile);
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        if (!s.used) continue;
        const int n = s.desc.n;
        for (int tk = 0; tk < (n + TZ - 1) / TZ; ++tk)
            for (int tj = 0; tj < (n + TY - 1) / TY; ++tj)
                for (int ti = 0; ti < (n + TX - 1) / TX; ++ti) items.push_back(Item{b, ti, tj, tk});
    }
    end(E->r_tile);
    begin(E->r_rows_rho);
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        if (!s.used) continue;
        const long long nr = (long long)s.desc.n * s.desc.n;
        for (long long t = 0; t < (nr + 7) / 8; ++t) items.push_back(Item{b, (int)t, 0, 0});
    }
    end(E->r_rows_rho);
    for (int vec = 1; vec >= 0; --vec) {
        auto& rg = vec ? E->r_correct_vec : E->r_correct_rest;
        begin(rg);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || s.desc.nlev < 2) continue;
            const int n = s.desc.n;
            if ((((n >> 1) & 1) == 0) != (vec == 1)) continue;
            const int step = vec ? correct_rows(n, 32 * R) : R;
            for (int k = 0; k < n; ++k)
                for (int j0 = 0; j0 < n; j0 += step) items.push_back(Item{b, 0, k, j0});
        }
        end(rg);
    }
    for (int l = 0; l < kMaxLev; ++l) {
        begin(E->r_rows_split[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l >= s.desc.nlev - 1) continue;
            const int nl = s.desc.lv[l].n;
            for (int k = 0; k < nl; ++k)
                for (int j0 = 0; j0 < nl; j0 += R) items.push_back(Item{b, l, k, j0});
        }
        end(E->r_rows_split[l]);
        begin(E->r_smooth_vec[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l >= s.desc.tail_l) continue;
            const int nl = s.desc.lv[l].n;
            if ((nl / 2) % 4 != 0) continue;
            const int rv = vec_rows(nl, 32 * R);
            for (int k = 0; k < nl; ++k)
                for (int j0 = 0; j0 < nl; j0 += rv) items.push_back(Item{b, l, k, j0});
        }
        end(E->r_smooth_vec[l]);
        begin(E->r_smooth_march[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l >= s.desc.tail_l) continue;
            const int nl = s.desc.lv[l].n;
            if ((nl / 2) % 4 != 0) continue;
            const int rv = vec_rows(nl, 32 * R);
            for (int k = 0; k < nl; k += kMarchE)
                for (int j0 = 0; j0 < nl; j0 += rv) items.push_back(Item{b, l, k, j0});
        }
        end(E->r_smooth_march[l]);
        begin(E->r_smooth_row[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l >= s.desc.tail_l) continue;
            const int nl = s.desc.lv[l].n;
            if ((nl / 2) % 4 == 0) continue;
            for (int k = 0; k < nl; ++k)
                for (int j0 = 0; j0 < nl; j0 += R) items.push_back(Item{b, l, k, j0});
        }
        end(E->r_smooth_row[l]);
        begin(E->r_prolong_quad[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l >= s.desc.tail_l) continue;
            const int nl = s.desc.lv[l].n;
            if ((nl / 2) % 4 != 0 || !s.desc.lv[l + 1].split) continue;
            const int rq = quad_rows(nl);
            for (int K = 0; K < nl / 2; ++K)
                for (int J0 = 0; J0 < nl / 2; J0 += rq) items.push_back(Item{b, l, K, J0});
        }
        end(E->r_prolong_quad[l]);
        begin(E->r_prolong_rest[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l >= s.desc.tail_l) continue;
            const int nl = s.desc.lv[l].n;
            if ((nl / 2) % 4 != 0 || s.desc.lv[l + 1].split) continue;
            const int rv = vec_rows(nl, 32 * R);
            for (int k = 0; k < nl; ++k)
                for (int j0 = 0; j0 < nl; j0 += rv) items.push_back(Item{b, l, k, j0});
        }
        end(E->r_prolong_rest[l]);
        for (int vec = 1; vec >= 0; --vec) {
            auto& rg = vec ? E->r_restrict_vec[l] : E->r_restrict_row[l];
            begin(rg);
            for (int b = 0; b < nbox; ++b) {
                const EnsSlot& s = E->slots[b];
                if (!s.used || l == 0 || l > s.desc.tail_l) continue;
                if ((((s.desc.lv[l - 1].n / 2) % 4) == 0) != (vec == 1)) continue;
                const int nl = s.desc.lv[l].n;
                for (int k = 0; k < nl; ++k)
                    for (int j0 = 0; j0 < nl; j0 += R) items.push_back(Item{b, l, k, j0});
            }
            end(rg);
        }
        begin(E->r_rows_nat[l]);
        for (int b = 0; b < nbox; ++b) {
            const EnsSlot& s = E->slots[b];
            if (!s.used || l == 0 || l >= s.desc.nlev) continue;
            const int nl = s.desc.lv[l].n;
            for (int k = 0; k < nl; ++k)
                for (int j0 = 0; j0 < nl; j0 += R) items.push_back(Item{b, l, k, j0});
        }
        end(E->r_rows_nat[l]);
    }
    if (items.empty()) items.push_back(Item{0, 0, 0, 0});
    if (items.size() > E->items_cap) {
        if (E->d_items) cudaFree(E->d_items);
        E->items_cap = items.size() + items.size() / 4 + 1024;
        if (cudaMalloc(&E->d_items, E->items_cap * sizeof(Item)) != cudaSuccess) {
            cudaGetLastError();
            E->d_items = nullptr;
            E->items_cap = 0;
            return efail(c, NYXPM_OOM, "ensemble work tables");
        }
    }
    if (nbox > E->cap) {
        // grow the descriptor / state arrays, keeping the device state of existing boxes
        const int ncap = nbox + 16;
        EDesc* nd = nullptr;
        EState* ns = nullptr;
        EStep* nst = nullptr;
        EStep *hs = nullptr, *hi = nullptr;
        EState* hst = nullptr;
        if (cudaMalloc(&nd, ncap * sizeof(EDesc)) != cudaSuccess ||
            cudaMalloc(&ns, ncap * sizeof(EState)) != cudaSuccess ||
            cudaMalloc(&nst, ncap * sizeof(EStep)) != cudaSuccess ||
            cudaMallocHost(&hs, ncap * sizeof(EStep)) != cudaSuccess ||
            cudaMallocHost(&hi, ncap * sizeof(EStep)) != cudaSuccess ||
            cudaMallocHost(&hst, ncap * sizeof(EState)) != cudaSuccess) {
            cudaGetLastError();
            return efail(c, NYXPM_OOM, "ensemble descriptors");
        }
        cudaMemsetAsync(ns, 0, ncap * sizeof(EState), c->stream);
        if (E->d_state && E->cap > 0)
            cudaMemcpyAsync(ns, E->d_state, E->cap * sizeof(EState), cudaMemcpyDeviceToDevice, c->stream);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble grow");
        if (E->d_desc) cudaFree(E->d_desc);
        if (E->d_state) cudaFree(E->d_state);
        if (E->d_step) cudaFree(E->d_step);
        if (E->h_step) cudaFreeHost(E->h_step);
        if (E->h_init) cudaFreeHost(E->h_init);
        if (E->h_state) cudaFreeHost(E->h_state);
        E->d_desc = nd;
        E->d_state = ns;
        E->d_step = nst;
        E->h_step = hs;
        E->h_init = hi;
        E->h_state = hst;
        std::memset(E->h_step, 0, ncap * sizeof(EStep));
        std::memset(E->h_init, 0, ncap * sizeof(EStep));
        E->cap = ncap;
    }
    std::vector<EDesc> descs(nbox);
    for (int b = 0; b < nbox; ++b) {
        descs[b] = E->slots[b].desc;
        descs[b].used = E->slots[b].used;
        if (E->slots[b].used && E->slots[b].fresh) {
            cudaMemsetAsync(E->d_state + b, 0, sizeof(EState), c->stream);
            E->slots[b].fresh = 0;
        }
    }
    cudaMemcpyAsync(E->d_items, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(E->d_desc, descs.data(), nbox * sizeof(EDesc), cudaMemcpyHostToDevice, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble rebuild");
    invalidate_graphs(E);
    E->dirty = 0;
    return NYXPM_OK;
}

nyxpm_status pull_state(nyxpm_ctx* c, nyxpm_ensemble* E)
{
    const int nbox = (int)E->slots.size();
    if (!E->d_state || nbox == 0) return NYXPM_OK;
    cudaMemcpyAsync(E->h_state, E->d_state, nbox * sizeof(EState), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble state");
    return NYXPM_OK;
}

// Stage timing of the eager profiling step (nyxpm_set_profiling on): CUDA
// events around each group of launches.  Never active while a graph is being
// captured (the profiled step runs without graphs), and the launch counts are
// kept by the enqueue functions themselves.
inline void ep_begin(nyxpm_ctx* c)
{
    if (!c->prof_on) return;
    const int64_t l = c->launches;
    prof_begin(*c);
    c->launches = l;
}

inline void ep_end(nyxpm_ctx* c, int stage)
{
    if (c->prof_on) prof_end(*c, stage, 0.0);
}

// sort + deposit + RHS + first residual + targets of the active boxes
void enqueue_solve_head(nyxpm_ctx* c, nyxpm_ensemble* E)
{
    cudaStream_t s = c->stream;
    const int nbox = (int)E->slots.size();
    const Item* it = E->d_items;
    const EDesc* D = E->d_desc;
    EState* S = E->d_state;
    const unsigned bb = (unsigned)((nbox + 127) / 128);
    ep_begin(c);
    e_sort_reset<<<bb, 128, 0, s>>>(nbox, D, S);
    e_keys<<<pgrid(E, E->r_part.cnt), kPT, 0, s>>>(it + E->r_part.off, E->r_part.cnt, D, S,
                                                   E->tune.sort_bucket);
    ep_end(c, NYXPM_ST_KEYS);
    ep_begin(c);
    e_scan_reduce<<<pgrid(E, E->r_scan.cnt), kScanT, 0, s>>>(it + E->r_scan.off, E->r_scan.cnt, D, S);
    e_scan_top<<<nbox, 1024, 0, s>>>(nbox, D, S);
    e_scan_down<<<pgrid(E, E->r_scan.cnt), kScanT, 0, s>>>(it + E->r_scan.off, E->r_scan.cnt, D, S);
    ep_end(c, NYXPM_ST_SCAN);
    ep_begin(c);
    e_scatter<<<pgrid(E, E->r_part.cnt), kPT, 0, s>>>(it + E->r_part.off, E->r_part.cnt, D, S,
                                                      E->tune.sort_bucket);
    e_fix_short<<<pgrid(E, E->r_keys.cnt), 256, 0, s>>>(it + E->r_keys.off, E->r_keys.cnt, D, S);
    e_fix_long<<<E->sm * 2, 512, 0, s>>>(nbox, D, S);
    ep_end(c, NYXPM_ST_SCATTER);
    ep_begin(c);
    e_gather<<<pgrid(E, E->r_part.cnt), kPT, 0, s>>>(it + E->r_part.off, E->r_part.cnt, D, S,
                                                     E->tune.sort_bucket);
    e_flip<<<bb, 128, 0, s>>>(nbox, S);
    ep_end(c, NYXPM_ST_GATHER);
    ep_begin(c);
    const unsigned gt = pgrid(E, E->r_tile.cnt, 4);
    if (E->tune.deposit_tile == 1)
        e_deposit<8, 8, 4><<<gt, 256, 0, s>>>(it + E->r_tile.off, E->r_tile.cnt, D, S);
    else if (E->tune.deposit_tile == 2)
        e_deposit<16, 8, 4><<<gt, 256, 0, s>>>(it + E->r_tile.off, E->r_tile.cnt, D, S);
    else
        e_deposit<8, 8, 8><<<gt, 256, 0, s>>>(it + E->r_tile.off, E->r_tile.cnt, D, S);
    ep_end(c, NYXPM_ST_DEPOSIT);
    ep_begin(c);
    e_rowsum<<<pgrid(E, E->r_rows_rho.cnt), 256, 0, s>>>(it + E->r_rows_rho.off, E->r_rows_rho.cnt, D, S);
    const double ggrav = -4.0 * M_PI * c->p.gconst;
    e_mean<<<nbox, 512, 0, s>>>(nbox, D, S, ggrav);
    const dim3 rb(32, E->tune.smooth_rows);
    const auto& r0 = E->r_rows_split[0];
    e_make_beta<<<pgrid(E, r0.cnt), rb, 0, s>>>(it + r0.off, r0.cnt, D, S);
    {
        const auto& cv = E->r_correct_vec;
        const auto& cr = E->r_correct_rest;
        if (cv.cnt) e_resid_v<<<pgrid(E, cv.cnt), rb, 0, s>>>(it + cv.off, cv.cnt, D, S, 1);
        if (cr.cnt) e_resid<<<pgrid(E, cr.cnt), rb, 0, s>>>(it + cr.off, cr.cnt, D, S, 1);
        c->launches += (cv.cnt ? 1 : 0) + (cr.cnt ? 1 : 0) - 1;
    }
    e_flags<<<bb, 128, 0, s>>>(nbox, D, S, c->p.rel_tol, 1);
    ep_end(c, NYXPM_ST_RHS);
    c->launches += 16;
}

// `outer` defect-correction iterations (boxes that converged skip them).  With
// first = 1 the first of them recomputes the residual with the FP64 stencil (a
// zero-guess solve, whose first correction is as large as phi, or a retry of
// boxes whose error bound kept them from converging); the others update it in
// double-float from the correction.
void enqueue_iterations(nyxpm_ctx* c, nyxpm_ensemble* E, int outer, int first)
{
    cudaStream_t s = c->stream;
    const int nbox = (int)E->slots.size();
    const Item* it = E->d_items;
    const EDesc* D = E->d_desc;
    EState* S = E->d_state;
    const unsigned bb = (unsigned)((nbox + 127) / 128);
    const dim3 rb(32, E->tune.smooth_rows);
    // one red or black half sweep of level l over every box: the vectorised
    // kernel for the boxes whose level-l rows allow it, the row kernel for the rest
    auto smooth = [&](int l, int color, bool zero_start = false) {
        const auto& rv = E->r_smooth_march[l];
        const auto& rr = E->r_smooth_row[l];
        if (zero_start) {
            // the opening red half sweep of an inner solve on level 0
            const auto& cv = E->r_correct_vec;
            const auto& cr = E->r_correct_rest;
            ep_begin(c);
            if (cv.cnt) e_gsrb_zero_v<<<pgrid(E, cv.cnt), rb, 0, s>>>(it + cv.off, cv.cnt, D, S);
            if (cr.cnt) e_gsrb_zero<<<pgrid(E, cr.cnt), rb, 0, s>>>(it + cr.off, cr.cnt, D, S);
            c->launches += (cv.cnt ? 1 : 0) + (cr.cnt ? 1 : 0) - 1;
            ep_end(c, NYXPM_ST_SMOOTH);
            c->launches += 1;
            return;
        }
        ep_begin(c);
        if (rv.cnt) {
            e_gsrb4<<<pgrid(E, rv.cnt), rb, 0, s>>>(it + rv.off, rv.cnt, D, S, color);
            c->launches += 1;
        }
        if (rr.cnt) {
            e_gsrb<<<pgrid(E, rr.cnt), rb, 0, s>>>(it + rr.off, rr.cnt, D, S, color);
            c->launches += 1;
        }
        ep_end(c, NYXPM_ST_SMOOTH);
    };
    for (int o = 0; o < outer; ++o) {
        for (int v = 0; v < E->tune.inner_vcycles; ++v) {
            for (int l = 0; l < E->max_lev - 1; ++l) {
                const auto& rs = E->r_rows_split[l];
                if (rs.cnt == 0) continue;
                for (int sw = 0; sw < c->p.nu1; ++sw)
                    for (int color = 0; color < 2; ++color)
                        smooth(l, color, l == 0 && v == 0 && sw == 0 && color == 0);
                const auto& qv = E->r_restrict_vec[l + 1];
                const auto& qr = E->r_restrict_row[l + 1];
                ep_begin(c);
                if (qv.cnt && c->p.nu1 > 0)
                    e_restrict4_red<<<pgrid(E, qv.cnt), rb, 0, s>>>(it + qv.off, qv.cnt, D, S);
                else if (qv.cnt)
                    e_restrict4<<<pgrid(E, qv.cnt), rb, 0, s>>>(it + qv.off, qv.cnt, D, S);
                if (qr.cnt) e_restrict<<<pgrid(E, qr.cnt), rb, 0, s>>>(it + qr.off, qr.cnt, D, S);
                ep_end(c, NYXPM_ST_RESTRICT);
                c->launches += (qv.cnt ? 1 : 0) + (qr.cnt ? 1 : 0) - 1;
                c->launches += 1;
            }
            ep_begin(c);
            e_tail<<<nbox, kTailThreads, 0, s>>>(nbox, D, S, c->p.nu1, c->p.nu2);
            ep_end(c, NYXPM_ST_BOTTOM);
            c->launches += 1;
            for (int l = E->max_lev - 2; l >= 0; --l) {
                const auto& rs = E->r_rows_split[l];
                if (rs.cnt == 0) continue;
                const auto& pv = E->r_smooth_vec[l];
                const auto& pr = E->r_smooth_row[l];
                ep_begin(c);
                const int black = c->p.nu2 > 0 ? 1 : 0;
                int nk = 0;
                if (black && E->tune.prolong_quad) {
                    const auto& pq = E->r_prolong_quad[l];
                    const auto& pe = E->r_prolong_rest[l];
                    if (pq.cnt) e_prolong4_black<<<pgrid(E, pq.cnt, 4), 256, 0, s>>>(it + pq.off, pq.cnt, D, S);
                    if (pe.cnt) e_prolong4<<<pgrid(E, pe.cnt), rb, 0, s>>>(it + pe.off, pe.cnt, D, S, black);
                    nk += (pq.cnt ? 1 : 0) + (pe.cnt ? 1 : 0);
                } else {
                    if (pv.cnt) e_prolong4<<<pgrid(E, pv.cnt), rb, 0, s>>>(it + pv.off, pv.cnt, D, S, black);
                    nk += pv.cnt ? 1 : 0;
                }
                if (pr.cnt) e_prolong<<<pgrid(E, pr.cnt), rb, 0, s>>>(it + pr.off, pr.cnt, D, S, black);
                ep_end(c, NYXPM_ST_PROLONG);
                c->launches += nk + (pr.cnt ? 1 : 0) - 1;
                for (int sw = 0; sw < c->p.nu2; ++sw)
                    for (int color = 0; color < 2; ++color) smooth(l, color);
                c->launches += 1;
            }
        }
        const auto& r0 = E->r_rows_split[0];
        ep_begin(c);
        e_count_inner<<<bb, 128, 0, s>>>(nbox, S, E->tune.inner_vcycles);
        if (first && o == 0) {
            e_update<<<pgrid(E, r0.cnt), rb, 0, s>>>(it + r0.off, r0.cnt, D, S);
            const auto& cv = E->r_correct_vec;
            const auto& cr = E->r_correct_rest;
            if (cv.cnt) e_resid_v<<<pgrid(E, cv.cnt), rb, 0, s>>>(it + cv.off, cv.cnt, D, S, 1);
            if (cr.cnt) e_resid<<<pgrid(E, cr.cnt), rb, 0, s>>>(it + cr.off, cr.cnt, D, S, 1);
            c->launches += (cv.cnt ? 1 : 0) + (cr.cnt ? 1 : 0) - 1;
        } else {
            const float c_hi = (float)(1.0 / 6.0);
            const float c_lo = (float)(1.0 / 6.0 - (double)c_hi);
            const auto& cv = E->r_correct_vec;
            const auto& cr = E->r_correct_rest;
            if (cv.cnt) e_correct_v<<<pgrid(E, cv.cnt), rb, 0, s>>>(it + cv.off, cv.cnt, D, S, c_hi, c_lo);
            if (cr.cnt) e_correct<<<pgrid(E, cr.cnt), rb, 0, s>>>(it + cr.off, cr.cnt, D, S, c_hi, c_lo);
            c->launches += (cv.cnt ? 1 : 0) + (cr.cnt ? 1 : 0) - 1;
            e_zero_inner<<<pgrid(E, r0.cnt), rb, 0, s>>>(it + r0.off, r0.cnt, D, S,
                                                          c->p.nu1 > 0 ? 0 : 1);
        }
        e_flags<<<bb, 128, 0, s>>>(nbox, D, S, c->p.rel_tol, (first && o == 0) ? 2 : 0);
        ep_end(c, NYXPM_ST_NORM);
        c->launches += 4;
    }
}

void enqueue_grav(nyxpm_ctx* c, nyxpm_ensemble* E)
{
    const dim3 rb(32, E->tune.smooth_rows);
    const auto& r0 = E->r_rows_split[0];
    ep_begin(c);
    e_grav<<<pgrid(E, r0.cnt), rb, 0, c->stream>>>(E->d_items + r0.off, r0.cnt, E->d_desc, E->d_state);
    ep_end(c, NYXPM_ST_KICK);
    c->launches += 1;
}

void enqueue_kick(nyxpm_ctx* c, nyxpm_ensemble* E, int phase)
{
    ep_begin(c);
    e_kick<<<pgrid(E, E->r_part.cnt), kPT, 0, c->stream>>>(E->d_items + E->r_part.off, E->r_part.cnt,
                                                            E->d_desc, E->d_state, phase,
                                                            E->tune.sort_bucket);
    ep_end(c, NYXPM_ST_KICK);
    c->launches += 1;
}

void enqueue_load(nyxpm_ctx* c, nyxpm_ensemble* E, const EStep* host_src)
{
    const int nbox = (int)E->slots.size();
    cudaMemcpyAsync(E->d_step, host_src, nbox * sizeof(EStep), cudaMemcpyHostToDevice, c->stream);
    e_load_step<<<(nbox + 127) / 128, 128, 0, c->stream>>>(nbox, E->d_step, E->d_desc, E->d_state);
    c->launches += 1;
}

// iterate eagerly until every active box has converged
nyxpm_status finish_unconverged(nyxpm_ctx* c, nyxpm_ensemble* E, int* extra)
{
    *extra = 0;
    const int nbox = (int)E->slots.size();
    for (int guard = 0; guard <= c->p.max_vcycles; ++guard) {
        ETRY(pull_state(c, E));
        bool any = false;
        for (int b = 0; b < nbox; ++b)
            if (E->slots[b].used && E->h_state[b].active && E->h_state[b].solve_active) any = true;
        if (!any) return NYXPM_OK;
        if (guard == c->p.max_vcycles) break;
        // each extra iteration refreshes the residual with the FP64 stencil, as
        // the step graph's loop body does
        enqueue_iterations(c, E, 1, 1);
        ETRY(echeck(c, "ensemble iterations"));
        *extra += 1;
    }
    return efail(c, NYXPM_NOT_CONVERGED, "ensemble: a box did not converge");
}

// The whole step as one graph: load, kick-drift, deposit and solve head,
// max_outer iterations, then a WHILE node whose body is one more iteration (FP64
// residual refresh) and the loop condition, then gravity and the closing kick.
// The WHILE node is added to the graph under capture and its body captured on a
// second stream; any refusal by the runtime returns an error and the caller
// falls back to two graphs with the loop on the host.
nyxpm_status capture_step(nyxpm_ctx* c, nyxpm_ensemble* E)
{
    if (c->prof_on) return efail(c, NYXPM_INVALID_ARG, "ensemble graphs are not captured while profiling");
    const int nbox = (int)E->slots.size();
    const int64_t l0 = c->launches;
    cudaGraph_t g = nullptr;
    cudaStream_t main = c->stream;
    if (cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return echeck(c, "ensemble capture begin");
    bool ok = true;
    enqueue_load(c, E, E->h_step);
    enqueue_kick(c, E, 0);
    enqueue_solve_head(c, E);
    enqueue_iterations(c, E, E->tune.max_outer, 0);
    cudaGraph_t cg = nullptr;
    cudaStreamCaptureStatus cs;
    cudaGraphConditionalHandle h = 0;
    ok = cudaStreamGetCaptureInfo(main, &cs, nullptr, &cg, nullptr, nullptr, nullptr) == cudaSuccess &&
         cs == cudaStreamCaptureStatusActive &&
         cudaGraphConditionalHandleCreate(&h, cg, 0, 0) == cudaSuccess;
    int64_t body_launches = 0;
    if (ok) {
        e_loop_cond<<<1, 128, 0, main>>>(nbox, E->d_state, E->d_loop, c->p.max_vcycles, 0, h);
        c->launches += 1;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        ok = cudaStreamGetCaptureInfo(main, &cs, nullptr, &cg, &deps, nullptr, &ndeps) == cudaSuccess;
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t wn = nullptr;
        ok = ok && cudaGraphAddNode(&wn, cg, deps, nullptr, ndeps, &p) == cudaSuccess &&
             cudaStreamUpdateCaptureDependencies(main, &wn, nullptr, 1, cudaStreamSetCaptureDependencies) ==
                 cudaSuccess;
        if (ok) {
            // the loop body, captured into the WHILE node's graph on the second stream
            ok = cudaStreamBeginCaptureToGraph(E->body_stream, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                const int64_t lb = c->launches;
                c->stream = E->body_stream;
                enqueue_iterations(c, E, 1, 1);
                e_loop_cond<<<1, 128, 0, E->body_stream>>>(nbox, E->d_state, E->d_loop, c->p.max_vcycles, 1, h);
                c->launches += 1;
                c->stream = main;
                body_launches = c->launches - lb;
                c->launches = lb;
                cudaGraph_t bg = nullptr;
                ok = cudaStreamEndCapture(E->body_stream, &bg) == cudaSuccess;
            }
        }
    }
    if (ok) {
        enqueue_grav(c, E);
        enqueue_kick(c, E, 1);
    }
    const cudaError_t ce = cudaStreamEndCapture(main, &g);
    cudaError_t ie = cudaErrorUnknown;
    cudaGraphExec_t exec = nullptr;
    if (ok && ce == cudaSuccess && g) ie = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    const int64_t n = c->launches - l0;
    c->launches = l0;
    if (!ok || ce != cudaSuccess || ie != cudaSuccess) {
        cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        return efail(c, NYXPM_CUDA_ERROR, "ensemble: the one-graph step was refused by the runtime");
    }
    E->exec_step = exec;
    E->graph_launches_step = n;
    E->graph_launches_body = body_launches;
    return NYXPM_OK;
}

nyxpm_status capture(nyxpm_ctx* c, nyxpm_ensemble* E, cudaGraphExec_t* exec, int which)
{
    cudaGraph_t g = nullptr;
    const int64_t l0 = c->launches;
    if (c->prof_on) return efail(c, NYXPM_INVALID_ARG, "ensemble graphs are not captured while profiling");
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return echeck(c, "ensemble capture begin");
    if (which == 0) {
        enqueue_load(c, E, E->h_step);
        enqueue_kick(c, E, 0);
        enqueue_solve_head(c, E);
        enqueue_iterations(c, E, E->tune.max_outer, 0);
    } else {
        enqueue_grav(c, E);
        enqueue_kick(c, E, 1);
    }
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (ce != cudaSuccess) return echeck(c, "ensemble capture end");
    if (cudaGraphInstantiate(exec, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        return echeck(c, "ensemble graph instantiate");
    }
    cudaGraphDestroy(g);
    const int64_t n = c->launches - l0;
    c->launches = l0;
    if (which == 0) E->graph_launches_solve = n;
    else E->graph_launches_finish = n;
    return NYXPM_OK;
}

}  // namespace

extern "C" {

size_t nyxpm_ensemble_box_bytes(int n, int64_t np)
{
    const double nc = (double)n * n * n;
    // particles: 2 x (cell, id, 3 offsets, 3 velocities) + key + perm + staging for upload
    // cells: count, start, FP32 rho, FP32 g (float4), FP64 phi + beta, residual low
    // words, FP32 levels (phi + beta, 8/7)
    return (size_t)(np * (2.0 * 32 + 8) + nc * (4 + 4 + 4 + 16 + 16 + 4 + 16 + 8.0 * 8 / 7) + 8.0 * n * n +
                    4.0 * (np / 32 + 2) + 256.0 * 64 + 4.0 * nc / 4096);
}

nyxpm_status nyxpm_ensemble_create(nyxpm_ctx* c, size_t arena_bytes, nyxpm_ensemble** out)
{
    if (!c || !out) return NYXPM_INVALID_ARG;
    *out = nullptr;
    cudaSetDevice(c->p.device);
    nyxpm_ensemble* E = new (std::nothrow) nyxpm_ensemble();
    if (!E) return NYXPM_OOM;
    if (!E->arena.init(arena_bytes)) {
        delete E;
        return efail(c, NYXPM_OOM, "ensemble arena (memory budget) could not be allocated");
    }
    if (cudaMallocHost(&E->h_scratch, 64) != cudaSuccess || cudaMalloc(&E->d_loop, 64) != cudaSuccess ||
        cudaStreamCreateWithFlags(&E->body_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        if (E->h_scratch) cudaFreeHost(E->h_scratch);
        if (E->d_loop) cudaFree(E->d_loop);
        E->arena.destroy();
        delete E;
        return efail(c, NYXPM_OOM, "ensemble pinned scratch");
    }
    cudaMemset(E->d_loop, 0, 64);
    E->tune.deposit_tile = 0;
    E->tune.smooth_rows = 8;
    E->tune.inner_vcycles = c->p.mixed_inner_vcycles;
    E->tune.max_outer = 6;
    E->tune.sort_bucket = 256;
    E->tune.prolong_quad = 1;
    E->sm = c->sm_count;
    *out = E;
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_destroy(nyxpm_ctx* c, nyxpm_ensemble* E)
{
    if (!c || !E) return NYXPM_INVALID_ARG;
    cudaStreamSynchronize(c->stream);
    invalidate_graphs(E);
    if (E->d_items) cudaFree(E->d_items);
    if (E->d_desc) cudaFree(E->d_desc);
    if (E->d_state) cudaFree(E->d_state);
    if (E->d_step) cudaFree(E->d_step);
    if (E->h_step) cudaFreeHost(E->h_step);
    if (E->h_init) cudaFreeHost(E->h_init);
    if (E->h_state) cudaFreeHost(E->h_state);
    if (E->h_scratch) cudaFreeHost(E->h_scratch);
    if (E->d_loop) cudaFree(E->d_loop);
    if (E->body_stream) cudaStreamDestroy(E->body_stream);
    E->arena.destroy();
    delete E;
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_add(nyxpm_ctx* c, nyxpm_ensemble* E, int n, double L, int64_t np, int* slot)
{
    if (!c || !E || !slot) return NYXPM_INVALID_ARG;
    if (n < 16 || n > 1024 || ens_bottom_edge(n) > kMaxBottom)
        return efail(c, NYXPM_INVALID_ARG, "ensemble boxes need n >= 16 of the form m*2^k, m <= 8");
    if (!(L > 0) || np < 1 || np > 0x7fffffffLL) return efail(c, NYXPM_INVALID_ARG, "bad L / np");
    if (ens_levels(n) > kMaxLev) return efail(c, NYXPM_INVALID_ARG, "too many levels");
    int b = -1;
    for (int i = 0; i < (int)E->slots.size(); ++i)
        if (!E->slots[i].used) {
            b = i;
            break;
        }
    if (b < 0) {
        b = (int)E->slots.size();
        E->slots.emplace_back();
    }
    EnsSlot& s = E->slots[b];
    s = EnsSlot();
    const size_t nc = (size_t)n * n * n;
    bool ok = true;
    auto A = [&](size_t bytes) -> void* {
        void* p = E->arena.alloc(bytes);
        if (!p) ok = false;
        else s.blocks.push_back(p);
        return p;
    };
    EDesc& d = s.desc;
    std::memset(&d, 0, sizeof(d));
    d.n = n;
    d.nlev = ens_levels(n);
    d.nb = ens_bottom_edge(n);
    d.np = np;
    d.L = L;
    d.dx = L / n;
    d.dxi = (double)n / L;
    {
        const double h = L / n;
        d.beta_scale = (h * h) * kSixth;
    }
    d.cell0 = (int*)A(4 * np); d.id0 = (int*)A(4 * np); d.cell1 = (int*)A(4 * np); d.id1 = (int*)A(4 * np);
    d.ox0 = (float*)A(4 * np); d.oy0 = (float*)A(4 * np); d.oz0 = (float*)A(4 * np);
    d.vx0 = (float*)A(4 * np); d.vy0 = (float*)A(4 * np); d.vz0 = (float*)A(4 * np);
    d.ox1 = (float*)A(4 * np); d.oy1 = (float*)A(4 * np); d.oz1 = (float*)A(4 * np);
    d.vx1 = (float*)A(4 * np); d.vy1 = (float*)A(4 * np); d.vz1 = (float*)A(4 * np);
    d.key = (int*)A(4 * np); d.perm = (int*)A(4 * np);
    d.cell_count = (int*)A(4 * nc);
    d.cell_start = (int*)A(4 * (nc + 1));
    d.tile_sums = (int*)A(4 * ((nc + kScanTile - 1) / kScanTile + 1));
    d.long_list = (int*)A(4 * (np / 32 + 2));
    d.long_count = (int*)A(256);
    d.frho = (float*)A(4 * nc);
    d.g32 = (float*)A(16 * nc);
    d.rows = (double*)A(8 * (size_t)n * n);
    d.scal = (double*)A(256);
    d.norms = (unsigned long long*)A(256);
    d.phi_r = (double*)A(8 * nc / 2); d.phi_b = (double*)A(8 * nc / 2);
    d.beta_r = (double*)A(8 * nc / 2); d.beta_b = (double*)A(8 * nc / 2);
    d.r_lo = (float*)A(4 * nc);
    for (int l = 0, nl = n; l < d.nlev; ++l, nl /= 2) {
        ELevel& lv = d.lv[l];
        lv.n = nl;
        lv.split = (l < d.nlev - 1) ? 1 : 0;
        const size_t cnt = (size_t)nl * nl * nl;
        if (lv.split) {
            lv.phi_r = (float*)A(4 * cnt / 2); lv.phi_b = (float*)A(4 * cnt / 2);
            lv.beta_r = (float*)A(4 * cnt / 2); lv.beta_b = (float*)A(4 * cnt / 2);
        } else {
            lv.phi_r = (float*)A(4 * cnt); lv.beta_r = (float*)A(4 * cnt);
        }
    }
    d.Gf = (float*)A(4 * (size_t)d.nb * d.nb * d.nb);
    if (!ok) {
        for (void* p : s.blocks) E->arena.release(p);
        s = EnsSlot();
        s.used = 0;
        return efail(c, NYXPM_OOM, "ensemble arena exhausted (memory budget)");
    }
    {
        const int nb = d.nb;
        const long ncb = (long)nb * nb * nb;
        std::vector<float> Gf(ncb);
        const double h = L / nb, twopi = 2.0 * std::acos(-1.0);
        std::vector<double> lam(ncb);
        for (int kz = 0; kz < nb; ++kz)
            for (int ky = 0; ky < nb; ++ky)
                for (int kx = 0; kx < nb; ++kx)
                    lam[kx + nb * (ky + (long)nb * kz)] =
                        ((2.0 * std::cos(twopi * kx / nb) - 2.0) + (2.0 * std::cos(twopi * ky / nb) - 2.0) +
                         (2.0 * std::cos(twopi * kz / nb) - 2.0)) / (h * h);
        for (int dz = 0; dz < nb; ++dz)
            for (int dy = 0; dy < nb; ++dy)
                for (int dxx = 0; dxx < nb; ++dxx) {
                    double acc = 0.0;
                    for (int kz = 0; kz < nb; ++kz)
                        for (int ky = 0; ky < nb; ++ky)
                            for (int kx = 0; kx < nb; ++kx) {
                                if (kx == 0 && ky == 0 && kz == 0) continue;
                                const long ph = ((long)kx * dxx + (long)ky * dy + (long)kz * dz) % nb;
                                acc += std::cos(twopi * (double)ph / nb) / lam[kx + nb * (ky + (long)nb * kz)];
                            }
                    Gf[dxx + nb * (dy + (long)nb * dz)] = (float)((acc / (double)ncb) * (6.0 / (h * h)));
                }
        cudaMemcpyAsync(d.Gf, Gf.data(), sizeof(float) * Gf.size(), cudaMemcpyHostToDevice, c->stream);
        cudaMemsetAsync(d.cell_count, 0, 4 * nc, c->stream);
        cudaMemsetAsync(d.phi_r, 0, 8 * nc / 2, c->stream);
        cudaMemsetAsync(d.phi_b, 0, 8 * nc / 2, c->stream);
        cudaMemsetAsync(d.long_count, 0, 4, c->stream);
        cudaMemsetAsync(d.norms, 0, 32, c->stream);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble add");
    }
    s.used = 1;
    s.fresh = 1;
    E->dirty = 1;
    *slot = b;
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_remove(nyxpm_ctx* c, nyxpm_ensemble* E, int slot)
{
    if (!c || !E || !slot_ok(E, slot)) return NYXPM_INVALID_ARG;
    cudaStreamSynchronize(c->stream);
    EnsSlot& s = E->slots[slot];
    for (void* p : s.blocks) E->arena.release(p);
    s = EnsSlot();
    s.used = 0;
    E->dirty = 1;
    return NYXPM_OK;
}

size_t nyxpm_ensemble_arena_used(const nyxpm_ensemble* E) { return E ? E->arena.used_bytes() : 0; }

// host-side split x = (i + o) dx, the arithmetic of to_cell() (this file is
// compiled without host contraction)
static void host_to_cell(double x, double dxi, int n, int* i, float* o)
{
    const double l = x * dxi;
    double fl = std::floor(l);
    float f = (float)(l - fl);
    if (f >= 1.0f) {
        f = 0.0f;
        fl += 1.0;
    }
    *i = wrapi((int)fl, n);
    *o = f;
}

nyxpm_status nyxpm_ensemble_upload(nyxpm_ctx* c, nyxpm_ensemble* E, int slot, const double* pos,
                                   const double* vel, double mass)
{
    if (!c || !E || !slot_ok(E, slot) || !pos || !vel) return NYXPM_INVALID_ARG;
    if (!(mass >= 0) || !std::isfinite(mass)) return efail(c, NYXPM_INVALID_ARG, "bad mass");
    if (E->dirty) ETRY(rebuild(c, E));
    EnsSlot& s = E->slots[slot];
    EDesc& d = s.desc;
    const long long np = d.np;
    // convert on the host into the box's buffer-0 arrays: no device staging, so an
    // upload never needs arena space beyond the box itself
    std::vector<int> cell(np), id(np);
    std::vector<float> f[6];
    for (auto& a : f) a.resize(np);
    for (long long q = 0; q < np; ++q) {
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(pos[3 * q + k]) || !std::isfinite(vel[3 * q + k])) {
                s.uploaded = 0;
                return efail(c, NYXPM_INVALID_ARG, "non-finite particle position or velocity");
            }
        int ii[3];
        for (int k = 0; k < 3; ++k) host_to_cell(pos[3 * q + k], d.dxi, d.n, &ii[k], &f[k][q]);
        cell[q] = ii[0] | (ii[1] << 10) | (ii[2] << 20);
        for (int k = 0; k < 3; ++k) f[3 + k][q] = (float)vel[3 * q + k];
        id[q] = (int)q;
    }
    float* dst[6] = {d.ox0, d.oy0, d.oz0, d.vx0, d.vy0, d.vz0};
    cudaMemcpyAsync(d.cell0, cell.data(), 4 * np, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d.id0, id.data(), 4 * np, cudaMemcpyHostToDevice, c->stream);
    for (int k = 0; k < 6; ++k) cudaMemcpyAsync(dst[k], f[k].data(), 4 * np, cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(&E->d_state[slot].parity, 0, sizeof(int), c->stream);
    d.mscalar = mass;
    d.mass_offset = mass * (double)np / (d.L * d.L * d.L);
    d.dep_scale = (float)(d.mscalar / (d.dx * d.dx * d.dx));
    // the descriptor changed (mass): push it
    cudaMemcpyAsync(E->d_desc + slot, &d, sizeof(EDesc), cudaMemcpyHostToDevice, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble upload");
    s.uploaded = 1;
    s.init_pending = 1;
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_download(nyxpm_ctx* c, nyxpm_ensemble* E, int slot, double* pos, double* vel)
{
    if (!c || !E || !slot_ok(E, slot) || !pos || !vel) return NYXPM_INVALID_ARG;
    if (!E->slots[slot].uploaded) return efail(c, NYXPM_INVALID_ARG, "slot has no particles");
    ETRY(pull_state(c, E));
    const EDesc& d = E->slots[slot].desc;
    const int par = E->h_state[slot].parity;
    const long long np = d.np;
    std::vector<int> cell(np), id(np);
    std::vector<float> f[6];
    for (auto& a : f) a.resize(np);
    const float* src[6] = {par ? d.ox1 : d.ox0, par ? d.oy1 : d.oy0, par ? d.oz1 : d.oz0,
                           par ? d.vx1 : d.vx0, par ? d.vy1 : d.vy0, par ? d.vz1 : d.vz0};
    cudaMemcpyAsync(cell.data(), par ? d.cell1 : d.cell0, 4 * np, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(id.data(), par ? d.id1 : d.id0, 4 * np, cudaMemcpyDeviceToHost, c->stream);
    for (int k = 0; k < 6; ++k) cudaMemcpyAsync(f[k].data(), src[k], 4 * np, cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble download");
    for (long long q = 0; q < np; ++q) {
        const long long o = 3LL * id[q];
        if (id[q] < 0 || id[q] >= np) return efail(c, NYXPM_CUDA_ERROR, "corrupt particle id");
        const int cc = cell[q];
        const int ci[3] = {cc & 1023, (cc >> 10) & 1023, (cc >> 20) & 1023};
        for (int k = 0; k < 3; ++k) {
            pos[o + k] = ((double)ci[k] + (double)f[k][q]) * d.dx;
            vel[o + k] = f[3 + k][q];
        }
    }
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_get_phi(nyxpm_ctx* c, nyxpm_ensemble* E, int slot, double* phi)
{
    if (!c || !E || !slot_ok(E, slot) || !phi) return NYXPM_INVALID_ARG;
    const EDesc& d = E->slots[slot].desc;
    const size_t nc = (size_t)d.n * d.n * d.n;
    void* tmp = E->arena.alloc(8 * nc);
    if (!tmp) return efail(c, NYXPM_OOM, "ensemble phi staging");
    const Geo g = geo3(d.n, d.n, d.n);
    e_phi_to_natural<<<g.grid, g.block, 0, c->stream>>>(d.n, d.phi_r, d.phi_b, (double*)tmp);
    cudaMemcpyAsync(phi, tmp, 8 * nc, cudaMemcpyDeviceToHost, c->stream);
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    E->arena.release(tmp);
    return e == cudaSuccess ? NYXPM_OK : echeck(c, "ensemble get phi");
}

nyxpm_status nyxpm_ensemble_grav_vector(nyxpm_ctx* c, nyxpm_ensemble* E, int slot, double* g_out)
{
    if (!c || !E || !slot_ok(E, slot) || !g_out) return NYXPM_INVALID_ARG;
    const EDesc& d = E->slots[slot].desc;
    const long long ncell = (long long)d.n * d.n * d.n;
    const long long cnt = 3 * ncell;
    void* tmp = E->arena.alloc(8 * cnt);
    if (tmp) {
        e_g32_to_double<<<(unsigned)((ncell + 255) / 256), 256, 0, c->stream>>>(ncell, d.g32, (double*)tmp);
        cudaMemcpyAsync(g_out, tmp, 8 * cnt, cudaMemcpyDeviceToHost, c->stream);
        const cudaError_t e = cudaStreamSynchronize(c->stream);
        E->arena.release(tmp);
        return e == cudaSuccess ? NYXPM_OK : echeck(c, "ensemble grav");
    }
    // the arena is full: the FP32 float4 field to the host and widened there
    std::vector<float> h(4 * (size_t)ncell);
    cudaMemcpyAsync(h.data(), d.g32, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return echeck(c, "ensemble grav");
    for (long long t = 0; t < ncell; ++t)
        for (int comp = 0; comp < 3; ++comp) g_out[comp * ncell + t] = h[4 * t + comp];
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_set_tuning(nyxpm_ctx* c, nyxpm_ensemble* E, const nyxpm_tuning* t)
{
    if (!c || !E || !t) return NYXPM_INVALID_ARG;
    if (t->deposit_tile < 0 || t->deposit_tile > 2 ||
        (t->smooth_rows != 1 && t->smooth_rows != 2 && t->smooth_rows != 4 && t->smooth_rows != 8) ||
        t->inner_vcycles < 1 || t->inner_vcycles > 8 || t->max_outer < 1 || t->max_outer > 64 ||
        (t->sort_bucket != 256 && t->sort_bucket != 512 && t->sort_bucket != 1024) ||
        (t->prolong_quad != 0 && t->prolong_quad != 1))
        return efail(c, NYXPM_INVALID_ARG, "bad tuning");
    E->tune = *t;
    E->dirty = 1;
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_get_tuning(nyxpm_ctx* c, nyxpm_ensemble* E, nyxpm_tuning* t)
{
    if (!c || !E || !t) return NYXPM_INVALID_ARG;
    *t = E->tune;
    return NYXPM_OK;
}

nyxpm_status nyxpm_ensemble_step(nyxpm_ctx* c, nyxpm_ensemble* E, const double* a_old,
                                 const double* a_new, const double* dt, nyxpm_ensemble_info* info)
{
    if (!c || !E || !a_old || !a_new || !dt) return NYXPM_INVALID_ARG;
    const int nbox = (int)E->slots.size();
    if (info) std::memset(info, 0, sizeof(*info));
    if (nbox == 0) return NYXPM_OK;
    if (E->dirty) ETRY(rebuild(c, E));
    const int64_t launches0 = c->launches;
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, c->stream);
    int extra = 0;
    bool one_graph = false;
    // initial fields of boxes uploaded since their last step (an eager pass with
    // only those boxes active; the RHS of the init solve uses a_new = a_old)
    bool any_init = false;
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        const bool init = s.used && s.uploaded && s.init_pending && a_old[b] > 0;
        E->h_init[b].active = init ? 1 : 0;
        E->h_init[b].a_old = a_old[b];
        E->h_init[b].a_new = a_old[b];
        E->h_init[b].dt = 0.0;
        any_init = any_init || init;
    }
    if (any_init) {
        enqueue_load(c, E, E->h_init);
        enqueue_solve_head(c, E);
        enqueue_iterations(c, E, E->tune.max_outer, 1);
        ETRY(echeck(c, "ensemble init"));
        int more = 0;
        ETRY(finish_unconverged(c, E, &more));
        enqueue_grav(c, E);
        for (int b = 0; b < nbox; ++b)
            if (E->h_init[b].active) E->slots[b].init_pending = 0;
        extra += more;
    }
    for (int b = 0; b < nbox; ++b) {
        const EnsSlot& s = E->slots[b];
        const bool on = s.used && s.uploaded && !s.init_pending && a_old[b] > 0;
        E->h_step[b].active = on ? 1 : 0;
        E->h_step[b].a_old = a_old[b];
        E->h_step[b].a_new = a_new[b];
        E->h_step[b].dt = dt[b];
    }
    if (c->prof_on) {
        // profiling: the same launches eagerly, with stage events (no graphs)
        enqueue_load(c, E, E->h_step);
        enqueue_kick(c, E, 0);
        enqueue_solve_head(c, E);
        enqueue_iterations(c, E, E->tune.max_outer, 0);
        ETRY(echeck(c, "ensemble profiled step"));
        int more = 0;
        ETRY(finish_unconverged(c, E, &more));
        extra += more;
        enqueue_grav(c, E);
        enqueue_kick(c, E, 1);
    } else {
        if (!E->exec_step && !E->single_graph_failed && capture_step(c, E) != NYXPM_OK)
            E->single_graph_failed = 1;
        if (E->exec_step) {
            // the whole step: one graph launch
            if (cudaGraphLaunch(E->exec_step, c->stream) != cudaSuccess) return echeck(c, "ensemble step graph");
            cudaMemcpyAsync(E->h_scratch, E->d_loop, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
            one_graph = true;
        } else {
            if (!E->exec_solve) ETRY(capture(c, E, &E->exec_solve, 0));
            if (!E->exec_finish) ETRY(capture(c, E, &E->exec_finish, 1));
            if (cudaGraphLaunch(E->exec_solve, c->stream) != cudaSuccess)
                return echeck(c, "ensemble solve graph");
            c->launches += E->graph_launches_solve;
            int more = 0;
            ETRY(finish_unconverged(c, E, &more));
            extra += more;
            if (cudaGraphLaunch(E->exec_finish, c->stream) != cudaSuccess)
                return echeck(c, "ensemble finish graph");
            c->launches += E->graph_launches_finish;
        }
    }
    cudaEventRecord(ev1, c->stream);
    if (cudaEventSynchronize(ev1) != cudaSuccess) return echeck(c, "ensemble step");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    ETRY(pull_state(c, E));
    bool unconverged = false;
    if (one_graph) {
        int loops = 0;
        std::memcpy(&loops, E->h_scratch, sizeof(int));
        extra += loops;
        c->launches += E->graph_launches_step + loops * E->graph_launches_body;
        for (int b = 0; b < nbox; ++b)
            if (E->slots[b].used && E->h_state[b].active && E->h_state[b].solve_active) unconverged = true;
    }
    if (info) {
        int mx = 0, inner = 0, boxes = 0;
        for (int b = 0; b < nbox; ++b)
            if (E->slots[b].used && E->h_state[b].active) {
                mx = std::max(mx, E->h_state[b].outer);
                inner = std::max(inner, E->h_state[b].inner);
                ++boxes;
            }
        info->boxes = boxes;
        info->max_outer_used = mx;
        info->max_inner_used = inner;
        info->fallback_iters = extra;
        info->launches = (int)(c->launches - launches0);
        info->ms = ms;
    }
    if (unconverged) return efail(c, NYXPM_NOT_CONVERGED, "ensemble: a box did not converge");
    return NYXPM_OK;
}

}  // extern "C"
